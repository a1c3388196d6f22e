"""The CPU restatement (oracle/liboracle.so) against fixtures produced by OMPL's own code.

Every comparison is exact (bitwise for FP64): the restatement must reproduce OMPL's arithmetic
operation for operation, because it is the checker for the GPU path on machines without OMPL.
"""
import math

import numpy as np
import pytest

from helpers import checker_of, same_bits, space_of
from oracle.oracle import NN_EXACT

SPACES = ["rv2", "rv7", "so2", "chain10", "wrap7"]


def test_rng_uniform_streams(port, golden):
    # RandomNumbers.h:66-76 over libstdc++ mt19937 / generate_canonical
    g = golden("rng")
    for i, s in enumerate(g["seeds"]):
        assert same_bits(port.rng_uniform(int(s), 2000), g["u01"][i])
        assert same_bits(port.rng_uniform(int(s), 2000, -math.pi, math.pi), g["upi"][i])


@pytest.mark.parametrize("name", SPACES)
def test_space_metric_interpolation(port, golden, name):
    g = golden(f"space_{name}")
    sp = space_of(g)
    assert port.extent(sp) == g["extent"]
    assert port.lvs(sp) == g["lvs"]
    assert same_bits(port.distance(sp, g["a"], g["b"]), g["distance"])
    assert same_bits(port.interpolate(sp, g["a"], g["b"], g["t"]), g["interpolate"])
    assert np.array_equal(port.valid_segment_count(sp, g["a"], g["b"]), g["valid_segment_count"])
    assert same_bits(port.enforce_bounds(sp, g["oob"]), g["enforce"])


@pytest.mark.parametrize("name", SPACES)
def test_state_samplers(port, golden, name):
    g = golden(f"space_{name}")
    sp = space_of(g)
    assert same_bits(port.sample_uniform(sp, int(g["sample_seed"]), 700), g["sample"])
    assert same_bits(port.sample_uniform_near(sp, 11, g["near"], float(g["near_distance"])), g["sample_near"])


GAUSS_NAMES = {0: "uniform", 1: "gaussian"}


def gauss_script(g):
    return [(GAUSS_NAMES[int(k)], int(c)) for k, c in zip(g["gauss_kinds"], g["gauss_counts"])]


@pytest.mark.parametrize("name", SPACES)
def test_state_sampler_gaussian(port, golden, name):
    # sampleGaussian (RealVectorStateSpace.cpp:67-82, SO2StateSpace.cpp:58-62) interleaved with
    # sampleUniform on one RNG; std::normal_distribution's cached value carries across calls
    g = golden(f"space_{name}")
    sp = space_of(g)
    out = port.sample_script(sp, int(g["gauss_seed"]), gauss_script(g), g["gauss_mean"], float(g["gauss_stddev"]))
    assert same_bits(out, g["gauss_out"])


def test_log_rounded_to_nearest(port):
    """ora_log_rn against a 200-bit evaluation (mpmath), on the arguments the polar method feeds it
    (x^2 + y^2 in (0, 1]) and on arguments next to 1 and to powers of two."""
    mpmath = pytest.importorskip("mpmath")
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, size=(6000, 2))
    r2 = (x * x).sum(axis=1)
    r2 = r2[(r2 > 0) & (r2 <= 1)]
    near1 = 1.0 - np.ldexp(rng.integers(1, 1 << 52, size=1000).astype(np.float64), -rng.integers(53, 110, size=1000))
    pow2 = np.ldexp(1.0 + rng.uniform(-0.3, 0.4, size=1000), -rng.integers(0, 200, size=1000))
    args = np.concatenate([r2, near1, pow2, [1.0, 0.5, 0.25, np.nextafter(1.0, 0.0), 2.0 ** -1000]])
    got = port.log_rn(args)
    mpmath.mp.prec = 200
    want = np.array([float(mpmath.log(mpmath.mpf(float(v)))) for v in args])
    assert same_bits(got, want)


@pytest.mark.parametrize("name", ["circles_seeded", "circles_ompl_tests", "chain_seeded", "chain_horn", "dh_arm"])
def test_validity_and_discrete_motion(port, golden, name):
    g = golden(name)
    sp, ck = space_of(g), checker_of(g)
    assert np.array_equal(port.is_valid(sp, ck, g["states"]), g["valid"])
    m = port.check_motion(sp, ck, g["s1"], g["s2"])
    for key in ("ok", "ok_bisect", "nd", "first_j"):
        assert np.array_equal(m[key], g[key]), key
    assert same_bits(m["last_t"], g["last_t"])
    assert same_bits(m["last_state"], g["last_state"])
    # both DiscreteMotionValidator variants check the same state set
    assert np.array_equal(m["ok"], m["ok_bisect"])


@pytest.mark.parametrize("name", ["rv2", "chain10", "wrap7"])
def test_nearest_neighbors(port, golden, name):
    g = golden(f"knn_{name}")
    sp = space_of(g)
    k = int(g["k"])
    idx, dist = port.knn(sp, g["pts"], g["q"], k, NN_EXACT)
    # seeded inputs have no distance ties, so OMPL's partial_sort order is the (distance, index) order
    assert np.array_equal(idx, g["linear_idx"])
    assert same_bits(dist, g["linear_dist"])
    # every OMPL structure returns the same distances (nearestneighbors.cpp:154-180 compares at 1e-6)
    for key in ("gnat_dist", "gnat_nts_dist", "sqrt_dist"):
        assert same_bits(dist, g[key]), key
    assert np.array_equal(g["gnat_idx"], idx)
    bi, bd = port.knn(sp, g["pts"][:50], g["q"][:10], 80, NN_EXACT)
    assert np.array_equal(bi, g["big_idx"]) and same_bits(bd, g["big_dist"])
    counts, ri, rd = port.radius(sp, g["pts"], g["q"], float(g["r"]))
    assert np.array_equal(counts, g["radius_counts"]) and np.array_equal(counts, g["gnat_radius_counts"])
    assert np.array_equal(ri, g["radius_idx"]) and same_bits(rd, g["radius_dist"])
    assert same_bits(rd, g["gnat_radius_dist"])
    pi_, pd_ = port.knn_prefix(sp, g["pts"], g["q"], g["prefix_limit"], k)
    assert np.array_equal(pi_, g["prefix_idx"]) and same_bits(pd_, g["prefix_dist"])


def test_motion_states(port, golden):
    g = golden("motion_states")
    sp, ck = space_of(g), checker_of(g)
    off = 0
    for i in range(len(g["count"])):
        n = int(g["lengths"][i])
        st = port.get_motion_states(sp, g["a"][i], g["b"][i], int(g["count"][i]), int(g["endpoints"][i]))
        assert same_bits(st, g["states"][off:off + n])
        ok, fi, okb = port.check_motion_states(sp, ck, st)
        assert ok == bool(g["ok"][i]) and okb == bool(g["ok_bisect"][i])
        if not ok:
            assert fi == g["first_invalid"][i]
        off += n


def test_so2_known_answers(port):
    # tests/base/state_spaces.cpp:169-215 (SO2_Simple)
    from oracle.oracle import SPACE_SO2, SpaceDesc
    sp = SpaceDesc(SPACE_SO2, 1)
    pi = math.pi
    assert port.extent(sp) == pi
    assert abs(port.distance(sp, [pi - 0.1], [-pi + 0.1])[0] - 0.2) < 1e-3
    assert abs(port.distance(sp, [-pi + 0.1], [pi - 0.1])[0] - 0.2) < 1e-3
    assert abs(port.interpolate(sp, [pi - 0.08], [-pi + 0.1], 0.5)[0, 0] - (-pi + 0.01)) < 1e-3
    assert abs(port.distance(sp, [0.1], [pi - 0.1])[0] - (pi - 0.2)) < 1e-3
    assert abs(port.interpolate(sp, [pi - 0.1], [0.1], 0.5)[0, 0] - pi / 2) < 1e-3
    assert port.interpolate(sp, [0.5], [1.5], 0.0)[0, 0] == 0.5
    assert abs(port.interpolate(sp, [0.5], [1.5], 1.0)[0, 0] - 1.5) < 1e-3


def test_real_vector_known_answers(port):
    # tests/base/state_spaces.cpp:291-354 (RealVector_Bounds / _Simple): extent sqrt(3), midpoint 0.5
    from oracle.oracle import SPACE_REAL_VECTOR, SpaceDesc
    sp = SpaceDesc(SPACE_REAL_VECTOR, 3, np.zeros(3), np.ones(3))
    assert abs(port.extent(sp) - math.sqrt(3.0)) < 1e-12
    assert np.allclose(port.interpolate(sp, np.zeros(3), np.ones(3), 0.5), 0.5)


SQRT_CASES = {"rv2": (0, 2, 0.0), "chain10": (2, 10, 0.1), "wrap7": (3, 7, 0.0)}


def sqrt_space(kind, dim, link):
    from oracle.oracle import SpaceDesc
    if kind == 0:
        return SpaceDesc(kind, dim, np.zeros(dim), np.ones(dim))
    if kind == 2:
        return SpaceDesc(kind, dim, link_length=link)
    return SpaceDesc(kind, dim)


@pytest.mark.parametrize("name", list(SQRT_CASES))
def test_sqrt_approx_nearest(port, golden, name):
    # NearestNeighborsSqrtApprox.h:91-125 after add(all) and removals, queries in order
    g = golden("sqrt_approx")
    idx, dist, off = port.nn_sqrt_approx(sqrt_space(*SQRT_CASES[name]), g[f"{name}_pts"], g[f"{name}_q"],
                                         g[f"{name}_remove"])
    assert np.array_equal(idx, g[f"{name}_idx"])
    assert same_bits(dist, g[f"{name}_dist"])
    assert off == int(g[f"{name}_offset"])
