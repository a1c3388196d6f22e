"""Box obstacles: the DH arm's spheres against axis-aligned world boxes (GBO_CHECK_DH_BOXES; the
definition is oracle/dh_arm.h, dh_pair_hits) on the GPU through the C ABI, against the oracle: validity
and both precisions of DiscreteMotionValidator on every schedule, a world too large for shared memory,
the FP32 form's precision statistics and the trig hazard count."""
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
from oracle.oracle import CheckerDesc, SpaceDesc  # noqa: E402

SCHEDULES = [capi.SCHEDULE_PLAIN, capi.SCHEDULE_TILE, capi.SCHEDULE_WARP, capi.SCHEDULE_AUTO]


def _case(n_boxes, n_edges, seed):
    w = W.config2(n_edges=n_edges, n_world=16)
    boxes = W.box_world(np.random.default_rng(seed), n_boxes)
    sd = SpaceDesc(w.space_kind, 7, w.low, w.high, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(W.CHECK_DH_BOXES, boxes, w.dh, 8, 0.05)
    space = B.RealVectorStateSpace(7, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    ck = B.DHBoxArmValidityChecker(space, w.dh, boxes, 8, 0.05)
    return w, sd, cd, ck


@pytest.mark.parametrize("n_boxes", [2048, 16384])
def test_box_world_validity_and_motion_vs_oracle(port, n_boxes):
    w, sd, cd, ck = _case(n_boxes, 1500, n_boxes)
    port.set_threads(16)
    st = np.random.default_rng(5).uniform(-math.pi, math.pi, size=(20_000, 7))
    v_ref = port.is_valid(sd, cd, st).astype(bool)
    assert 0.02 < v_ref.mean() < 0.98
    m_ref = port.check_motion(sd, cd, w.s1, w.s2, want_state=False, want_bisect=False)
    mv = B.DiscreteMotionValidator(ck)
    for p in ("fp32_guarded", "fp64"):
        ck.setPrecision(p)
        assert np.array_equal(ck.isValid(st), v_ref), p
        assert ck.stats()["hazards"] == 0
        for sch in SCHEDULES:
            r = mv.checkMotions(w.s1, w.s2, schedule=sch)
            assert np.array_equal(r["ok"], m_ref["ok"]), (p, sch)
            assert np.array_equal(r["first_j"], m_ref["first_j"]) and np.array_equal(r["nd"], m_ref["nd"]), (p, sch)


def test_box_world_precision_stats():
    w, sd, cd, ck = _case(4096, 10, 7)
    q = np.random.default_rng(8).uniform(-math.pi, math.pi, size=(60_000, 7))
    ps = ck.precisionStats(q)
    assert ps["states"] == len(q)
    assert ps["flips"] <= ps["ambiguous"] < 0.05 * ps["states"]
    assert 0.0 < ps["max_abs_err"] < 1e-4
