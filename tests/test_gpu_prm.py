"""Batched PRM roadmap (PRM.cpp:364-385, 570-604 semantics) on the GPU path against the same
construction done step by step with the oracle: identical milestones (bitwise), identical neighbour
lists (prefix nearestK, k = 10) and an identical edge set (checkMotion(n, m) valid)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import prm  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402
from oracle.oracle import CheckerDesc, SpaceDesc  # noqa: E402


@pytest.mark.parametrize("precision", ["fp32_guarded", "fp64"])
def test_prm_roadmap_matches_sequential_prm(port, precision):
    n_samples, k = 2500, 10
    w = W.config4(n_samples=n_samples, n_world=1024)
    seed = w.extra["sampler_seed"]
    space = B.WrapL2StateSpace(7)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    checker.setPrecision(precision)
    rm = prm.construct_roadmap(space, checker, seed, n_samples, k=k)

    port.set_threads(16)
    sd = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, dh=w.dh, spheres_per_link=8, sphere_radius=0.05)
    samples = port.sample_uniform(sd, seed, n_samples)
    valid = port.is_valid(sd, cd, samples).astype(bool)
    M = samples[valid]
    assert np.array_equal(rm.sample_index.cpu().numpy(), np.flatnonzero(valid))
    assert np.array_equal(rm.milestones.cpu().numpy().T.view(np.uint64), M.view(np.uint64))
    nbr, _ = port.knn_prefix(sd, M, M, np.arange(len(M)), k)
    dst = np.repeat(np.arange(len(M)), k)
    src = nbr.reshape(-1)
    have = src >= 0
    src, dst = src[have], dst[have]
    assert rm.candidate_edges == len(src)
    ok = port.check_motion(sd, cd, M[src], M[dst], want_state=False, want_bisect=False)["ok"].astype(bool)
    ref_edges = set(zip(src[ok].tolist(), dst[ok].tolist()))
    got_edges = set(zip(rm.edge_src.cpu().tolist(), rm.edge_dst.cpu().tolist()))
    assert got_edges == ref_edges
    assert prm.connected_components(len(M), rm.edge_src.cpu().numpy(), rm.edge_dst.cpu().numpy()) == \
        prm.connected_components(len(M), src[ok], dst[ok])


def test_prm_star_roadmap_matches_sequential_prm(port):
    """PRM* (KStarStrategy): milestone m connects to its ceil((e + e/7) log(m + 1)) nearest
    predecessors (22 at the last of ~900 milestones, so the kNN keeps 48-entry lists)."""
    n_samples = 2500
    w = W.config4(n_samples=n_samples, n_world=1024)
    seed = w.extra["sampler_seed"]
    space = B.WrapL2StateSpace(7)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    rm = prm.construct_roadmap(space, checker, seed, n_samples, star=True)

    port.set_threads(16)
    sd = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, dh=w.dh, spheres_per_link=8, sphere_radius=0.05)
    samples = port.sample_uniform(sd, seed, n_samples)
    M = samples[port.is_valid(sd, cd, samples).astype(bool)]
    ks = prm.kstar_counts(len(M), 7)
    kmax = int(ks[-1])
    assert kmax > 20
    nbr, _ = port.knn_prefix(sd, M, M, np.arange(len(M)), kmax)
    src, dst = [], []
    for m in range(len(M)):
        row = nbr[m, :ks[m]]
        row = row[row >= 0]
        src.extend(row.tolist())
        dst.extend([m] * len(row))
    src, dst = np.array(src, dtype=np.int64), np.array(dst, dtype=np.int64)
    assert rm.candidate_edges == len(src)
    ok = port.check_motion(sd, cd, M[src], M[dst], want_state=False, want_bisect=False)["ok"].astype(bool)
    assert set(zip(rm.edge_src.cpu().tolist(), rm.edge_dst.cpu().tolist())) == \
        set(zip(src[ok].tolist(), dst[ok].tolist()))


def test_prm_planner_data_archive(port, tmp_path):
    """PRM::getPlannerData of the GPU roadmap equals the oracle replay of PRM's edge sequence (vertex
    order, tags, out-edge lists), and PlannerDataStorage's archive of it reads back unchanged."""
    from ompl_gb300 import plannerdata as PD
    from oracle.planner_data import prm_planner_data
    n_samples, k = 2500, 10
    w = W.config4(n_samples=n_samples, n_world=1024)
    seed = w.extra["sampler_seed"]
    space = B.WrapL2StateSpace(7)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    rm = prm.construct_roadmap(space, checker, seed, n_samples, k=k)
    pd = PD.planner_data(rm, space)
    ref = port.prm_roadmap(SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction),
                           CheckerDesc(w.checker_kind, w.obstacles, dh=w.dh, spheres_per_link=8, sphere_radius=0.05),
                           seed, n_samples, k)
    vertices, tags, out = prm_planner_data(len(rm.sample_index), list(zip(ref["edge_src"].tolist(),
                                                                        ref["edge_dst"].tolist())))
    assert pd.milestone.tolist() == vertices and pd.tags.tolist() == tags
    assert [pd.targets[pd.offsets[v]:pd.offsets[v + 1]].tolist() for v in range(pd.num_vertices)] == out
    path = tmp_path / "prm.pdam"
    PD.store(pd, path)
    back = PD.load(path, signature=PD.space_signature(space))
    assert np.array_equal(back.states.view(np.uint64), pd.states.view(np.uint64))
    assert np.array_equal(back.targets, pd.targets) and np.array_equal(back.tags, pd.tags)
