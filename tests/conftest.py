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


@pytest.fixture(scope="session")
def cuda_ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but CUDA is not available")
    import woxel_gb300 as wx

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
