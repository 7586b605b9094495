import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
BOUNDS_CHECKED = os.environ.get("WOXEL_GB300_BOUNDS_CHECK") == "1"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Build libwoxel_gb300.so (or, under WOXEL_GB300_BOUNDS_CHECK=1, the bounds-checked
    build) and the oracle once per session (no-op when up to date)."""
    from woxel_gb300 import build as b

    b.build(checked=BOUNDS_CHECKED)
    b.build_oracle()
    yield


# The whole 4096^3 noise grid flattened by the oracle alone takes its single-threaded
# compute_sdf a few minutes and about 20 GB of host memory: it is built on a host thread
# from the first GPU test on (ctypes releases the interpreter lock during the oracle's
# calls), while the other GPU tests run, and joined by the test that needs it.
_NOISE_VIEW = {}


def pytest_collection_modifyitems(config, items):
    if any("oracle_noise_view" in getattr(i, "fixturenames", ()) for i in items):
        _NOISE_VIEW["wanted"] = True


def _start_noise_oracle_view():
    import threading

    if "thread" in _NOISE_VIEW or not _NOISE_VIEW.get("wanted"):
        return

    def work():
        try:
            import oracle as orc

            _NOISE_VIEW["view"] = orc.workload_view("noise")
        except BaseException as e:  # reported by the test that joins it
            _NOISE_VIEW["error"] = e

    t = threading.Thread(target=work, daemon=True)
    _NOISE_VIEW["thread"] = t
    t.start()


@pytest.fixture(scope="session")
def oracle_noise_view():
    """The benchmark's noise grid (2.68M leaves) flattened by the oracle alone: its
    restated generator, compute_sdf and atlas()."""
    _NOISE_VIEW["wanted"] = True
    _start_noise_oracle_view()
    _NOISE_VIEW["thread"].join()
    if "error" in _NOISE_VIEW:
        raise _NOISE_VIEW["error"]
    return _NOISE_VIEW["view"]


@pytest.fixture(scope="session")
def cuda_ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but CUDA is not available")
    import woxel_gb300 as wx

    _start_noise_oracle_view()

    ctx = wx.Context(int(os.environ.get("WX_TEST_DEVICE", "0")))
    yield ctx
    if BOUNDS_CHECKED:  # every index the session's kernels used was in range
        assert ctx.bounds_violations() == 0
    ctx.close()


@pytest.fixture(scope="session")
def oracle_spheres_view():
    """The 2000-sphere benchmark grid's flattened view with its level-set values, built by
    the oracle alone (restated generator, set_voxel, compute_sdf, atlas()): the view the
    full-size parity tests hand the oracle, independent of the product's generator and SDF."""
    import oracle as orc

    return orc.workload_view("spheres", values=True)
