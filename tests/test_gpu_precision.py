"""The precision machinery on the GPU: the correctly rounded FP64 sin/cos of the FP64 forms against the
oracle's double-double evaluation (bitwise), the one-ulp hazard counters of the FP64 decisions, and the
FP32 forms' precision statistics (a flip, an FP32 verdict taken at face value that differs from the
FP64 one, can only occur in a state the guard band sends to the FP64 re-check)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402


def test_sincos_cr_matches_double_double_oracle(port):
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.uniform(-40, 40, 2_000_000), rng.uniform(-1e-4, 1e-4, 10_000),
                        np.arange(-50, 51) * (math.pi / 4), np.array([0.0, -0.0, 1e-300, 1e5, -3e5])])
    t = torch.as_tensor(x, device="cuda")
    s, c = torch.empty_like(t), torch.empty_like(t)
    capi.check(capi.lib().gbo_sincos_cr(B._ptr(t), len(x), B._ptr(s), B._ptr(c), B._stream(None)))
    port.set_threads(16)
    rs, rc, hard = port.sincos_rn(x)
    assert hard <= 1
    assert np.array_equal(s.cpu().numpy().view(np.uint64), rs.view(np.uint64))
    assert np.array_equal(c.cpu().numpy().view(np.uint64), rc.view(np.uint64))


def test_log_rn_matches_oracle(port):
    """The sampleGaussian log (a plain-FP64 evaluation with a rounding test, the double-double one when
    that cannot decide) against the oracle's double-double log, which the CPU suite pins against a 200-bit
    evaluation: bitwise on the polar method's arguments x^2 + y^2, arguments within 2^-53..2^-110 of 1,
    next to powers of two, and over the whole exponent range."""
    rng = np.random.default_rng(12)
    u = rng.random((3_000_000, 2)) * 2 - 1
    r2 = (u * u).sum(axis=1)
    r2 = r2[(r2 > 0) & (r2 <= 1)]
    k = rng.integers(1, 1 << 52, size=200_000).astype(np.float64)
    sh = rng.integers(53, 110, size=200_000)
    x = np.concatenate([r2, 1.0 - np.ldexp(k, -sh), 1.0 + np.ldexp(k, -sh),
                        np.ldexp(1.0 + rng.uniform(-0.3, 0.4, 200_000), -rng.integers(0, 1000, 200_000)),
                        np.exp(rng.uniform(-700, 700, 200_000)),
                        [1.0, 0.5, 0.25, 2.0, np.nextafter(1.0, 0.0), np.nextafter(1.0, 2.0), 2.0 ** -1022]])
    t = torch.as_tensor(x, device="cuda")
    out = torch.empty_like(t)
    capi.check(capi.lib().gbo_log_rn(B._ptr(t), len(x), B._ptr(out), B._stream(None)))
    want = port.log_rn(x)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want.view(np.uint64))


def test_glibc_trig_rounding_on_this_host(port):
    """Recorded on the GPU machine's C library (aarch64): how often sin/cos differ from the correctly
    rounded values; always by at most one ulp."""
    r = port.trig_rounding(np.random.default_rng(7).uniform(-40, 40, 400_000))
    print("C library sin/cos vs correctly rounded:", r)
    assert r["max_ulps"] <= 1


def _chain():
    w = W.config1(n_states=200_000, n_edges=10, n_queries=10)
    space = B.KinematicChainSpace(10, w.link_length)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    return w, space, B.KinematicChainValidityChecker(space, w.obstacles)


def _arm(n_world=4096):
    w = W.config2(n_edges=10, n_world=n_world)
    space = B.RealVectorStateSpace(7, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    return w, space, B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)


def test_chain_hazards_and_precision_stats():
    w, space, ck = _chain()
    st = torch.as_tensor(w.states.T.copy(), device="cuda")
    ck.setPrecision("fp64")
    ck.isValid(st, soa=True)
    assert ck.stats()["hazards"] == 0
    ps = ck.precisionStats(st, soa=True)
    assert ps["states"] == len(w.states)
    assert ps["flips"] <= ps["ambiguous"] < 0.05 * ps["states"]
    assert 0.0 < ps["max_abs_err"] < 1e-5


def test_arm_hazards_and_precision_stats():
    w, space, ck = _arm()
    q = np.random.default_rng(8).uniform(-math.pi, math.pi, size=(60_000, 7))
    ck.setPrecision("fp64")
    ck.isValid(q)
    assert ck.stats()["hazards"] == 0
    ps = ck.precisionStats(q)
    assert ps["states"] == len(q)
    assert ps["flips"] <= ps["ambiguous"] < 0.05 * ps["states"]
    assert 0.0 < ps["max_abs_err"] < 1e-4


def test_precision_stats_unsupported_for_circles():
    w = W.config0()
    space = B.RealVectorStateSpace(2, w.low, w.high)
    ck = B.CirclesValidityChecker(space, w.obstacles)
    with pytest.raises(capi.GboError):
        ck.precisionStats(w.states[:10])
