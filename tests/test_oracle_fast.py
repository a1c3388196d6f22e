"""The oracle's faster exact forms against its direct forms (CPU only):

  * the DH arm checker's grid broad phase against the all-pairs definition (oracle/dh_arm.h), on
    uniform states and on states next to contact;
  * the chain metric's kNN with per-row precomputed link directions against distance() per pair;
  * the blocked prefix kNN against a per-query sort by (distance, index);
  * the PRM roadmap builder against the same construction composed from the oracle's single steps;
  * the double-double sin/cos: its constants and results against 200-bit arithmetic (mpmath, where
    installed), and how often the C library's sin/cos differ from the correctly rounded values."""
import math

import numpy as np
import pytest

from ompl_gb300 import workloads as W
from oracle.oracle import CheckerDesc, SpaceDesc


@pytest.mark.parametrize("n_world", [4096, 16384])
def test_dh_grid_equals_all_pairs(port, n_world):
    w = W.config4(n_world=n_world)
    sd = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, w.dh, 8, 0.05)
    rng = np.random.default_rng(n_world)
    st = rng.uniform(-math.pi, math.pi, size=(1500, 7))
    port.set_threads(8)
    a = port.is_valid(sd, cd, st)
    assert np.array_equal(a, port.is_valid_brute(sd, cd, st))
    # states along edges that cross contact: the first invalid states of motions are next to contact
    s1 = st[a == 1][:40]
    s2 = rng.uniform(-math.pi, math.pi, size=(len(s1), 7))
    r = port.check_motion(sd, cd, s1, s2, want_state=True, want_bisect=False)
    bad = r["ok"] == 0
    near = np.concatenate([r["last_state"][bad], port.interpolate(sd, s1[bad], s2[bad],
                                                                 r["first_j"][bad] / np.maximum(r["nd"][bad], 1))])
    assert np.array_equal(port.is_valid(sd, cd, near), port.is_valid_brute(sd, cd, near))


def test_chain_knn_precomputed_directions(port):
    w = W.config1(n_states=3000, n_edges=10, n_queries=40)
    sd = SpaceDesc(w.space_kind, 10, link_length=0.1, lvs_fraction=0.005)
    idx, dist = port.knn(sd, w.states, w.queries, 12)
    n, q = len(w.states), len(w.queries)
    d = port.distance(sd, np.tile(w.states, (q, 1)), np.repeat(w.queries, n, axis=0)).reshape(q, n)
    for i in range(q):
        order = np.lexsort((np.arange(n), d[i]))[:12]
        assert np.array_equal(idx[i], order)
        assert np.array_equal(dist[i].view(np.uint64), d[i][order].view(np.uint64))


@pytest.mark.parametrize("kind", [3, 0])
def test_blocked_prefix_knn(port, kind):
    rng = np.random.default_rng(kind)
    pts = rng.uniform(-math.pi, math.pi, size=(5000, 7))
    pts[100] = pts[50]  # an exact tie: the earlier index wins
    sd = SpaceDesc(kind, 7, np.full(7, -math.pi), np.full(7, math.pi), lvs_fraction=0.01)
    limit = np.minimum(np.arange(200) * 37, 5000)
    q = pts[rng.integers(0, 5000, 200)]
    q[7] = pts[50]
    limit[7] = 4000
    idx, dist = port.knn_prefix(sd, pts, q, limit, 10)
    for i in range(200):
        m = int(limit[i])
        d = port.distance(sd, pts[:m], np.repeat(q[i:i + 1], m, axis=0)) if m else np.zeros(0)
        order = np.lexsort((np.arange(m), d))[:10]
        assert np.array_equal(idx[i, :len(order)], order) and np.all(idx[i, len(order):] == -1)
        assert np.array_equal(dist[i, :len(order)], d[order])
    assert idx[7, 0] == 50 and idx[7, 1] == 100


def test_prm_roadmap_equals_composed_steps(port):
    n, k = 3000, 10
    w = W.config4(n_samples=n, n_world=1024)
    sd = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, w.dh, 8, 0.05)
    port.set_threads(8)
    r = port.prm_roadmap(sd, cd, w.extra["sampler_seed"], n, k)
    samples = port.sample_uniform(sd, w.extra["sampler_seed"], n)
    valid = port.is_valid(sd, cd, samples).astype(bool)
    assert np.array_equal(r["sample_index"], np.flatnonzero(valid))
    M = samples[valid]
    nbr, _ = port.knn_prefix(sd, M, M, np.arange(len(M)), k)
    dst = np.repeat(np.arange(len(M)), k)
    src = nbr.reshape(-1)
    have = src >= 0
    src, dst = src[have], dst[have]
    assert r["candidates"] == len(src)
    ok = port.check_motion(sd, cd, M[src], M[dst], want_state=False, want_bisect=False)["ok"].astype(bool)
    assert np.array_equal(r["edge_src"], src[ok]) and np.array_equal(r["edge_dst"], dst[ok])


def test_double_double_sincos_constants_and_values(port):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 200
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-40, 40, 3000), rng.uniform(-1e-3, 1e-3, 300), np.arange(-25, 26) * math.pi / 4,
                        np.array([0.0, -0.0, 1e-300, math.pi / 2, 1e5, -3e5])])
    s, c, hard = port.sincos_rn(x)
    assert hard <= 1  # at most the subnormal-scale argument, whose rounding needs no series
    for i in range(len(x)):
        xs = mp.mpf(float(x[i]))
        assert s[i] == float(mp.sin(xs)) and c[i] == float(mp.cos(xs)), x[i]


def test_c_library_trig_rounding_rate(port):
    """Recorded, not required: glibc's sin/cos are not correctly rounded on every argument (about 0.14% of
    arguments in [-40, 40] on glibc 2.39, one ulp each). The one-ulp hazard counters of the GPU's FP64
    forms exist because of this."""
    x = np.random.default_rng(4).uniform(-40, 40, 400_000)
    r = port.trig_rounding(x)
    assert r["undecided"] == 0 and r["max_ulps"] <= 1
    assert (r["sin_misrounded"] + r["cos_misrounded"]) / (2 * len(x)) < 0.01


@pytest.mark.parametrize("n_world", [1000, 8000])
def test_dh_grid_equals_all_pairs_boxes(port, n_world):
    w = W.config4(n_world=16)
    boxes = W.box_world(np.random.default_rng(n_world), n_world)
    sd = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(W.CHECK_DH_BOXES, boxes, w.dh, 8, 0.05)
    st = np.random.default_rng(n_world + 1).uniform(-math.pi, math.pi, size=(1500, 7))
    port.set_threads(8)
    a = port.is_valid(sd, cd, st)
    assert 0.05 < a.mean() < 0.95
    assert np.array_equal(a, port.is_valid_brute(sd, cd, st))
    s1 = st[a == 1][:40]
    s2 = np.random.default_rng(3).uniform(-math.pi, math.pi, size=(len(s1), 7))
    r = port.check_motion(sd, cd, s1, s2, want_state=True, want_bisect=False)
    bad = r["ok"] == 0
    near = np.concatenate([r["last_state"][bad], port.interpolate(sd, s1[bad], s2[bad],
                                                                 r["first_j"][bad] / np.maximum(r["nd"][bad], 1))])
    assert np.array_equal(port.is_valid(sd, cd, near), port.is_valid_brute(sd, cd, near))
