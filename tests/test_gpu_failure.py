"""Failure paths on the GPU without a GPU fault: a bounded device wait that nothing completes gives up
after its time limit and the call reports GBO_ERR_TIMEOUT; the context stays usable afterwards. Host-side
failures (bad handles, capacity, malformed batches) are covered by the CPU tests and the no-alloc test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402


def test_bounded_wait_times_out_and_the_context_survives(port):
    elapsed = C.c_double()
    for limit_ns in (2_000_000, 20_000_000):
        st = capi.lib().gbo_selftest_bounded_wait(limit_ns, C.byref(elapsed))
        assert st == capi.ERR_TIMEOUT
        assert limit_ns * 1e-6 <= elapsed.value < limit_ns * 1e-6 + 500.0
    # the same process keeps working: a validity batch against the oracle
    from oracle.oracle import CheckerDesc, SpaceDesc
    rng = np.random.default_rng(2)
    circles = np.c_[rng.uniform(0, 1, (50, 2)), rng.uniform(0.02, 0.06, 50)]
    sd = SpaceDesc(capi.SPACE_REAL_VECTOR, 2, np.zeros(2), np.ones(2))
    ckd = CheckerDesc(capi.CHECK_CIRCLES, circles)
    states = rng.uniform(0, 1, (5000, 2))
    s = B.RealVectorStateSpace(2, np.zeros(2), np.ones(2))
    ck = B.CirclesValidityChecker(s, circles)
    assert np.array_equal(ck.isValid(states), port.is_valid(sd, ckd, states).astype(bool))
