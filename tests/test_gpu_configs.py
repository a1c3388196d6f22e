"""Parity at the workloads' stated sizes, through the C ABI, against the oracle (tests/golden for the
PRM digest):

  * circles in RealVector(2): 10,000 states, 10,000 edges at segment fraction 0.01, nearestK k = 10
    for 1,000 queries over the 10,000 states (the whole workload, every output bitwise);
  * the kinematic chain's nearestK through the cell search (an index of >= 65,536 chain states and
    a batch of >= 1,024 queries without prefix limits takes knn_ccell_warp_kernel);
  * the DH arm among 4,096 spheres: 3,000 edges of 2..2000 interpolation steps, every schedule and
    precision;
  * the PRM roadmap of the DH arm among 16,384 spheres from 200,000 and 2,000,000 samples, against the
    digest tests/golden/make_prm_digest.py computed with the oracle on the CPU."""
import json
import math
import os

import numpy as np
import pytest

from helpers import same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402
from ompl_gb300 import prm  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402
from oracle.oracle import CheckerDesc, SpaceDesc  # noqa: E402

SCHEDULES = [capi.SCHEDULE_PLAIN, capi.SCHEDULE_TILE, capi.SCHEDULE_WARP, capi.SCHEDULE_AUTO]
HERE = os.path.dirname(os.path.abspath(__file__))


def ulp_close(a, b, rel=1e-12):
    """Chain-metric distances: the GPU's FP64 sin/cos and the C library's may differ in the last bit,
    magnified to ~1e-13 relative by the metric's cancellations. Tolerance: relative 1e-12."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return bool(np.all((np.abs(a - b) <= rel * np.maximum(np.abs(a), np.abs(b))) | (a == b)))


def test_circles_workload_full_size(port):
    w = W.config0()
    assert (len(w.states), len(w.s1), len(w.queries)) == (10_000, 10_000, 1_000)
    sd = SpaceDesc(w.space_kind, 2, w.low, w.high, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles)
    port.set_threads(16)
    v_ref = port.is_valid(sd, cd, w.states).astype(bool)
    m_ref = port.check_motion(sd, cd, w.s1, w.s2, want_state=True, want_bisect=True)
    space = B.RealVectorStateSpace(2, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    ck = B.CirclesValidityChecker(space, w.obstacles)
    assert np.array_equal(ck.isValid(w.states), v_ref)
    mv = B.DiscreteMotionValidator(ck)
    for sch in SCHEDULES:
        r = mv.checkMotions(w.s1, w.s2, schedule=sch)
        assert np.array_equal(r["ok"], m_ref["ok"]), sch
        assert np.array_equal(r["first_j"], m_ref["first_j"]) and np.array_equal(r["nd"], m_ref["nd"]), sch
    lt = mv.checkMotions(w.s1, w.s2, schedule=capi.SCHEDULE_AUTO, last_valid=True)
    bad = lt["ok"] == 0
    assert same_bits(lt["last_t"][bad], m_ref["last_t"][bad])
    assert same_bits(lt["last_state"][bad], m_ref["last_state"][bad])
    # the bisection overload (DiscreteMotionValidator.cpp:93-145) evaluates the same states
    assert np.array_equal(lt["ok"], m_ref["ok_bisect"])
    i_ref, d_ref = port.knn(sd, w.states, w.queries, 10)
    for precision in ("fp64", "fp32_guarded"):
        nn = B.NearestNeighborsGPU(space, capacity=len(w.states), precision=precision)
        nn.add(w.states)
        idx, dist = nn.nearestK(w.queries, 10)
        assert np.array_equal(idx, i_ref) and same_bits(dist, d_ref), precision


def test_chain_cell_search_knn_vs_oracle(port):
    """100,000 chain states, 2,048 queries (1,024 of them states of the index), k = 16 and k = 20: the
    batch takes the chain cell search (index >= 65,536, batch >= 1,024, no prefix limits, k <= 20)."""
    w = W.config1(n_states=100_000, n_edges=10, n_queries=10)
    rng = np.random.default_rng(5)
    q = np.concatenate([w.states[rng.integers(0, len(w.states), 1024)],
                        rng.uniform(-math.pi, math.pi, size=(1024, 10))])
    sd = SpaceDesc(w.space_kind, 10, link_length=w.link_length, lvs_fraction=w.lvs_fraction)
    port.set_threads(16)
    space = B.KinematicChainSpace(10, w.link_length)
    nn = B.NearestNeighborsGPU(space, capacity=len(w.states))
    nn.add(torch.as_tensor(w.states.T.copy(), device="cuda"), soa=True)
    for k in (16, 20):
        i_ref, d_ref = port.knn(sd, w.states, q, k)
        idx, dist = nn.nearestK(q, k)
        assert np.array_equal(idx, i_ref), k
        assert ulp_close(dist, d_ref), k


def test_dh_arm_4096_spheres_vs_oracle(port):
    w = W.config2(n_edges=3000)
    assert w.obstacles.shape[0] == 4096
    sd = SpaceDesc(w.space_kind, 7, w.low, w.high, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, dh=w.dh, spheres_per_link=8, sphere_radius=0.05)
    port.set_threads(16)
    ref = port.check_motion(sd, cd, w.s1, w.s2, want_state=False, want_bisect=False)
    assert ref["nd"].min() >= 2 and ref["nd"].max() >= 1000
    space = B.RealVectorStateSpace(7, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    ck = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    mv = B.DiscreteMotionValidator(ck)
    for p in ("fp32_guarded", "fp64"):
        ck.setPrecision(p)
        for sch in SCHEDULES:
            r = mv.checkMotions(w.s1, w.s2, schedule=sch)
            assert np.array_equal(r["ok"], ref["ok"]), (p, sch)
            assert np.array_equal(r["first_j"], ref["first_j"]) and np.array_equal(r["nd"], ref["nd"]), (p, sch)


@pytest.mark.parametrize("n_samples", [200_000, 2_000_000])
def test_prm_roadmap_digest(n_samples):
    with open(os.path.join(HERE, "golden", "prm_dh_arm7_digest.json")) as f:
        ref = json.load(f)["sizes"][str(n_samples)]
    from golden.make_prm_digest import roadmap_digest
    w = W.config4()
    space = B.WrapL2StateSpace(7)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    ck = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    ck.setPrecision("fp32_guarded")
    rm = prm.construct_roadmap(space, ck, w.extra["sampler_seed"], n_samples)
    got = roadmap_digest(rm.sample_index.cpu().numpy(), rm.edge_src.cpu().numpy(), rm.edge_dst.cpu().numpy(),
                         rm.candidate_edges)
    assert got == ref
