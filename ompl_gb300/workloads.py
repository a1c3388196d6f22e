"""Seeded synthetic workloads for the sampling / validity / motion / kNN path.

No public dataset is named for this path, so every input is synthetic and generated here from a
seed with numpy's PCG64 (identical on x86 and Arm). States are returned row-major (n, dim) FP64,
the layout OMPL keeps inside each RealVectorStateSpace::StateType.

Workloads (index = configuration number):
  0  point robot in RealVector(2) on [0,1]^2, 100 circles (centre U[0,1]^2, r U(0.02,0.06)),
     10,000 states, 10,000 edges between random state pairs at segment fraction 0.01,
     kNN k=10 for 1,000 uniform queries over the 10,000 states.
  1  planar kinematic chain: 10 links of length 0.1, joints U[-pi,pi], 32 world segments with
     endpoints U[-1,1]^2, 1M states, 100k edges at segment fraction 0.005, kNN k=16 over the 1M
     states for 100k queries drawn from the set.
  2  7-DoF DH arm (a, d ~ U(0,0.4), alpha in {0, +pi/2, -pi/2}), 8 spheres of radius 0.05 per link,
     4,096 world spheres (centre uniform in [-1,1]^3 outside a 0.8 m ball around the base,
     r U(0.02,0.1)), 256k edges whose lengths give log-uniform 2..2000 interpolation steps.
  3  serving: per-client worlds of 1,024..8,192 spheres with the workload-2 arm.
  4  PRM roadmap for the workload-2 arm among 16,384 spheres in the wrap-L2 joint space.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

PI = np.pi

SPACE_REAL_VECTOR, SPACE_SO2, SPACE_KINEMATIC_CHAIN, SPACE_WRAP_L2 = 0, 1, 2, 3
CHECK_ALL_VALID, CHECK_CIRCLES, CHECK_CHAIN_SEGMENTS, CHECK_DH_SPHERES, CHECK_DH_BOXES = 0, 1, 2, 3, 4


@dataclass
class Workload:
    name: str
    space_kind: int
    dim: int
    low: np.ndarray
    high: np.ndarray
    link_length: float
    lvs_fraction: float
    checker_kind: int
    obstacles: np.ndarray
    dh: np.ndarray | None = None
    spheres_per_link: int = 0
    sphere_radius: float = 0.0
    states: np.ndarray | None = None
    s1: np.ndarray | None = None
    s2: np.ndarray | None = None
    queries: np.ndarray | None = None
    k: int = 10
    extra: dict = field(default_factory=dict)


def circles_world(rng, n=100, rmin=0.02, rmax=0.06):
    c = rng.uniform(0.0, 1.0, size=(n, 2))
    r = rng.uniform(rmin, rmax, size=(n, 1))
    return np.ascontiguousarray(np.hstack([c, r]))


def segment_world(rng, n=32):
    return np.ascontiguousarray(rng.uniform(-1.0, 1.0, size=(n, 4)))


def dh_arm(rng, joints=7):
    a = rng.uniform(0.0, 0.4, size=joints)
    d = rng.uniform(0.0, 0.4, size=joints)
    code = rng.integers(-1, 2, size=joints).astype(np.float64)
    return np.ascontiguousarray(np.stack([a, d, code], axis=1))


FREE_RADIUS = 0.8


def sphere_world(rng, n, rmin=0.02, rmax=0.1, free_radius=FREE_RADIUS):
    """n spheres, centres uniform in [-1,1]^3 outside a ball of radius `free_radius` around the arm
    base, radii U(rmin, rmax). With the whole cube filled no arm state is collision-free (0 of 400
    sampled states for 1,024..16,384 spheres); the empty ball leaves 30-36% of states valid."""
    out = np.empty((0, 3))
    while out.shape[0] < n:
        c = rng.uniform(-1.0, 1.0, size=(2 * n, 3))
        out = np.vstack([out, c[np.linalg.norm(c, axis=1) >= free_radius]])
    r = rng.uniform(rmin, rmax, size=(n, 1))
    return np.ascontiguousarray(np.hstack([out[:n], r]))


def box_world(rng, n, hmin=0.02, hmax=0.1, free_radius=FREE_RADIUS):
    """n axis-aligned boxes, rows (cx, cy, cz, hx, hy, hz): centres uniform in [-1,1]^3 outside a ball of
    radius `free_radius` around the arm base (as sphere_world), half extents U(hmin, hmax) per axis."""
    out = np.empty((0, 3))
    while out.shape[0] < n:
        c = rng.uniform(-1.0, 1.0, size=(2 * n, 3))
        out = np.vstack([out, c[np.linalg.norm(c, axis=1) >= free_radius]])
    h = rng.uniform(hmin, hmax, size=(n, 3))
    return np.ascontiguousarray(np.hstack([out[:n], h]))


def random_pairs(rng, states, n_edges):
    i = rng.integers(0, states.shape[0], size=n_edges)
    j = rng.integers(0, states.shape[0], size=n_edges)
    return np.ascontiguousarray(states[i]), np.ascontiguousarray(states[j])


def config0(seed=0, n_states=10_000, n_edges=10_000, n_queries=1_000):
    rng = np.random.default_rng(seed)
    world = circles_world(rng)
    states = rng.uniform(0.0, 1.0, size=(n_states, 2))
    s1, s2 = random_pairs(rng, states, n_edges)
    queries = rng.uniform(0.0, 1.0, size=(n_queries, 2))
    return Workload("circles2d", SPACE_REAL_VECTOR, 2, np.zeros(2), np.ones(2), 0.0, 0.01, CHECK_CIRCLES, world,
                    states=states, s1=s1, s2=s2, queries=queries, k=10)


def config1(seed=1, n_states=1_000_000, n_edges=100_000, n_queries=100_000, links=10):
    rng = np.random.default_rng(seed)
    world = segment_world(rng)
    states = rng.uniform(-PI, PI, size=(n_states, links))
    s1, s2 = random_pairs(rng, states, n_edges)
    qi = rng.integers(0, n_states, size=n_queries)
    return Workload("kinematic_chain10", SPACE_KINEMATIC_CHAIN, links, np.full(links, -PI), np.full(links, PI), 0.1,
                    0.005, CHECK_CHAIN_SEGMENTS, world, states=states, s1=s1, s2=s2,
                    queries=np.ascontiguousarray(states[qi]), k=16, extra={"query_index": qi})


def arm_edges(rng, n_edges, lvs, low, high, nmin=2, nmax=2000):
    """Edges with log-uniform step counts: length (n - 0.5) * lvs along a uniform direction, s1 drawn
    uniformly from the positions that keep s2 inside the bounds (direction redrawn when none fit)."""
    dim = low.shape[0]
    n = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=n_edges))
    n = np.floor(n).astype(np.int64)
    length = (n - 0.5) * lvs
    s1 = np.empty((n_edges, dim))
    s2 = np.empty((n_edges, dim))
    todo = np.arange(n_edges)
    span = high - low
    while todo.size:
        u = rng.normal(size=(todo.size, dim))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        step = u * length[todo, None]
        fit = np.all(np.abs(step) < span, axis=1)
        idx = todo[fit]
        st = step[fit]
        lo = low - np.minimum(st, 0.0)
        hi = high - np.maximum(st, 0.0)
        a = lo + (hi - lo) * rng.uniform(size=st.shape)
        s1[idx] = a
        s2[idx] = np.clip(a + st, low, high)
        todo = todo[~fit]
    return s1, s2


def config2(seed=2, n_edges=256_000, n_world=4096, lvs_fraction=1.0 / 2500.0):
    rng = np.random.default_rng(seed)
    dh = dh_arm(rng)
    world = sphere_world(rng, n_world)
    low, high = np.full(7, -PI), np.full(7, PI)
    extent = np.sqrt(np.sum((high - low) ** 2))
    s1, s2 = arm_edges(rng, n_edges, extent * lvs_fraction, low, high)
    return Workload("dh_arm7", SPACE_REAL_VECTOR, 7, low, high, 0.0, lvs_fraction, CHECK_DH_SPHERES, world, dh=dh,
                    spheres_per_link=8, sphere_radius=0.05, s1=s1, s2=s2, k=10)


def config4(seed=4, n_samples=2_000_000, n_world=16_384):
    rng = np.random.default_rng(seed)
    dh = dh_arm(np.random.default_rng(2))  # the workload-2 arm
    world = sphere_world(rng, n_world)
    low, high = np.full(7, -PI), np.full(7, PI)
    extent = np.sqrt(7 * PI * PI)
    return Workload("prm_dh_arm7", SPACE_WRAP_L2, 7, low, high, 0.0, 0.01 / extent, CHECK_DH_SPHERES, world, dh=dh,
                    spheres_per_link=8, sphere_radius=0.05, k=10, extra={"n_samples": n_samples, "sampler_seed": seed})
