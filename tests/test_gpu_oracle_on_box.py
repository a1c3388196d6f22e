"""The oracle restatement, compiled on the GPU machine (aarch64, its own C library), against the fixtures
OMPL's own code produced on the x86 build machine. The CPU suite pins the restatement on x86; this
module repeats the pin where the GPU tests actually use it as the checker, so that the chain parity
there rests on a pinned oracle. Everything that does not call sin/cos is compared bit for bit; chain
distances, whose sin/cos come from the local C library, must agree to 1e-12 relative (the same bound
as the GPU's kNN distances), and the number that differ at all is reported."""
import numpy as np
import pytest

from helpers import checker_of, same_bits, space_of
from oracle.oracle import NN_EXACT

pytestmark = pytest.mark.gpu


def close(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and bool(np.all(np.abs(a - b) <= 1e-12 * np.maximum(np.abs(a), np.abs(b))))


@pytest.mark.parametrize("name", ["rv2", "rv7", "so2", "wrap7"])
def test_spaces_without_trig_bitwise(port, golden, name):
    g = golden(f"space_{name}")
    sp = space_of(g)
    assert same_bits(port.distance(sp, g["a"], g["b"]), g["distance"])
    assert same_bits(port.interpolate(sp, g["a"], g["b"], g["t"]), g["interpolate"])
    assert np.array_equal(port.valid_segment_count(sp, g["a"], g["b"]), g["valid_segment_count"])
    assert same_bits(port.sample_uniform(sp, int(g["sample_seed"]), 700), g["sample"])


def test_chain_space_on_this_c_library(port, golden):
    g = golden("space_chain10")
    sp = space_of(g)
    d = port.distance(sp, g["a"], g["b"])
    assert close(d, g["distance"])
    print("chain distances differing in any bit from x86 glibc:", int(np.count_nonzero(d != g["distance"])),
          "of", d.size)
    assert same_bits(port.interpolate(sp, g["a"], g["b"], g["t"]), g["interpolate"])
    # segment counts come from the distances; equal on every fixture edge
    assert np.array_equal(port.valid_segment_count(sp, g["a"], g["b"]), g["valid_segment_count"])


@pytest.mark.parametrize("name", ["circles_seeded", "circles_ompl_tests", "chain_seeded", "chain_horn", "dh_arm"])
def test_validity_and_motion_on_this_c_library(port, golden, name):
    g = golden(name)
    sp, ck = space_of(g), checker_of(g)
    assert np.array_equal(port.is_valid(sp, ck, g["states"]), g["valid"])
    m = port.check_motion(sp, ck, g["s1"], g["s2"])
    for key in ("ok", "ok_bisect", "nd", "first_j"):
        assert np.array_equal(m[key], g[key]), key
    assert same_bits(m["last_t"], g["last_t"])


@pytest.mark.parametrize("name", ["rv2", "chain10", "wrap7"])
def test_nearest_neighbors_on_this_c_library(port, golden, name):
    g = golden(f"knn_{name}")
    sp = space_of(g)
    idx, dist = port.knn(sp, g["pts"], g["q"], int(g["k"]), NN_EXACT)
    assert np.array_equal(idx, g["linear_idx"])
    assert (close if name == "chain10" else same_bits)(dist, g["linear_dist"])
