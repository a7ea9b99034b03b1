/* Stand-in for the empty libpopcnt submodule: a portable popcount over a byte buffer. */
#pragma once
#include <stdint.h>
#include <string.h>
static inline uint64_t popcnt(const void *data, uint64_t size) {
  const unsigned char *p = (const unsigned char *)data;
  uint64_t total = 0;
  for (uint64_t i = 0; i < size; i++) total += (uint64_t)__builtin_popcount(p[i]);
  return total;
}
