"""NearestNeighborsSqrtApprox::nearest on the GPU index (gbo_nn_nearest_sqrt_approx): the same elements,
in the same round-robin subsets, as OMPL's class, call after call. Against the fixture OMPL's own
class produced (tests/golden/sqrt_approx.npz) and against the oracle restatement at larger sizes, with
removals, several calls carrying the offset, and the offset restarting at clear()."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402
from oracle.oracle import SpaceDesc  # noqa: E402

CASES = {"rv2": (capi.SPACE_REAL_VECTOR, 2, 0.0), "chain10": (capi.SPACE_KINEMATIC_CHAIN, 10, 0.1),
         "wrap7": (capi.SPACE_WRAP_L2, 7, 0.0)}


def spaces(kind, dim, link):
    if kind == capi.SPACE_REAL_VECTOR:
        return SpaceDesc(kind, dim, np.zeros(dim), np.ones(dim)), B.RealVectorStateSpace(dim, 0.0, 1.0)
    if kind == capi.SPACE_KINEMATIC_CHAIN:
        return SpaceDesc(kind, dim, link_length=link), B.KinematicChainSpace(dim, link)
    return SpaceDesc(kind, dim), B.WrapL2StateSpace(dim)


def close(a, b, chain):
    if not chain:
        return np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return np.all(np.abs(a - b) <= 1e-12 * np.maximum(np.abs(a), np.abs(b)))  # FP64 sin/cos vs the C library


@pytest.mark.parametrize("name", list(CASES))
def test_sqrt_approx_vs_ompl_fixture(golden, name):
    g = golden("sqrt_approx")
    kind, dim, link = CASES[name]
    _, space = spaces(kind, dim, link)
    nn = B.NearestNeighborsGPU(space, capacity=2000)
    nn.add(g[f"{name}_pts"])
    nn.remove(g[f"{name}_remove"])
    idx, dist = nn.nearestSqrtApprox(g[f"{name}_q"])
    assert np.array_equal(idx, g[f"{name}_idx"])
    assert close(dist, g[f"{name}_dist"], kind == capi.SPACE_KINEMATIC_CHAIN)
    assert nn._sqrt_offset == int(g[f"{name}_offset"])


@pytest.mark.parametrize("name", list(CASES))
def test_sqrt_approx_large_calls_carry_the_offset(port, name):
    kind, dim, link = CASES[name]
    sd, space = spaces(kind, dim, link)
    rng = np.random.default_rng(9)
    lo, hi = (0.0, 1.0) if kind == capi.SPACE_REAL_VECTOR else (-math.pi, math.pi)
    pts = rng.uniform(lo, hi, size=(70_000, dim))
    q = rng.uniform(lo, hi, size=(3001, dim))
    rem = rng.choice(70_000, size=2_500, replace=False)
    ref_idx, ref_dist, ref_off = port.nn_sqrt_approx(sd, pts, q, rem)
    nn = B.NearestNeighborsGPU(space, capacity=70_000)
    nn.add(torch.as_tensor(pts, device="cuda"))
    nn.remove(rem)
    parts = [nn.nearestSqrtApprox(q[a:b]) for a, b in ((0, 1), (1, 1200), (1200, 3001))]
    idx = np.concatenate([p[0] for p in parts])
    dist = np.concatenate([p[1] for p in parts])
    assert np.array_equal(idx, ref_idx)
    assert close(dist, ref_dist, kind == capi.SPACE_KINEMATIC_CHAIN)
    assert nn._sqrt_offset == ref_off
    # without removals the positions are the keys; clear() restarts the offset
    nn.clear()
    nn.add(pts[:5000])
    i2, _ = nn.nearestSqrtApprox(q[:300])
    r2, _, _ = port.nn_sqrt_approx(sd, pts[:5000], q[:300])
    assert np.array_equal(i2, r2)


def test_sqrt_approx_on_an_empty_index_fails():
    nn = B.NearestNeighborsGPU(B.RealVectorStateSpace(2, 0.0, 1.0), capacity=10)
    with pytest.raises(capi.GboError):
        nn.nearestSqrtApprox(np.zeros((1, 2)))
