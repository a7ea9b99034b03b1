// Cost-model state attached to a graph handle (filled in by the model module).
#include "accx_internal.h"

extern "C" int accx_model_table_stub(void) { return 0; }

int accx_model_table(accx_graph *g, uint8_t *table) {
  (void)g;
  (void)table;
  return ACCX_ERR_NOT_READY;
}

void accx_model_release(accx_graph *g) { g->model = nullptr; }
