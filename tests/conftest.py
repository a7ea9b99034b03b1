import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


NON_GRAPH_FIXTURES = {"edge_list_converter"}  # converter input/output, not a SCAN case


def golden_cases():
    return sorted(n for n in (os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
                  if n not in NON_GRAPH_FIXTURES)


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def quick_sched_file(tmp_path_factory):
    """A scheduler file trained on this GPU in quick mode by the library's own
    training CLI (accx-sched-train)."""
    import subprocess
    from acctricnt_gb300 import BUILD_DIR
    path = str(tmp_path_factory.mktemp("sched") / "quick.model")
    r = subprocess.run([os.path.join(BUILD_DIR, "accx-sched-train"), path, "quick"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return path


@pytest.fixture(scope="session")
def default_sched():
    """The full scheduler of the build folder (trained on this GPU when absent)."""
    from acctricnt_gb300 import sched
    s, _ = sched.default_scheduler()
    return s
