import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle.build import reference_root  # noqa: E402

REFERENCE = reference_root()
GOLDEN_CASE = REFERENCE / "sources" / "RRSPH_COMMON" / "tests" / "caseDamBreak"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the in-tree libraries once per session (incremental)."""
    from oracle import build as ob
    from sph2d_gb300 import build

    build.build_cuda()
    ob.build_oracle()
    ob.build_reference()
    yield


def has_reference_sources() -> bool:
    return GOLDEN_CASE.is_dir()


needs_reference = pytest.mark.skipif(not GOLDEN_CASE.is_dir(), reason="reference sources not present on this machine")


@pytest.fixture(scope="session")
def gpu_available():
    import ctypes

    try:
        import torch  # noqa: F401

        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    if not ok:
        pytest.skip("no CUDA device")
    return True


def rel_l2(a, b) -> float:
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)
