"""The request loop: requests from many clients, submitted together so that they are admitted while
others run and overlap on the device, return exactly what the same request returns alone."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402
from ompl_gb300 import serve  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402


def _clients(n_clients, rng):
    dh = W.dh_arm(np.random.default_rng(2))
    clients = []
    for c in range(n_clients):
        world = W.sphere_world(np.random.default_rng(1000 + c), int(rng.integers(1024, 4096)))
        space = B.RealVectorStateSpace(7, -math.pi, math.pi)
        space.setLongestValidSegmentFraction(1.0 / 1500)
        ck = B.DHSphereArmValidityChecker(space, dh, world, 8, 0.05)
        ck.setPrecision("fp32_guarded")
        wspace = B.WrapL2StateSpace(7)
        nn = B.NearestNeighborsGPU(wspace, capacity=20_000)
        nn.add(rng.uniform(-math.pi, math.pi, size=(int(rng.integers(2000, 20_000)), 7)))
        clients.append((ck, nn))
    return clients


def test_results_alone_equal_results_in_the_mix():
    rng = np.random.default_rng(77)
    clients = _clients(12, rng)
    reqs = []
    for i in range(60):
        c = int(rng.integers(0, len(clients)))
        kind = i % 3
        if kind == 0:
            n = int(rng.integers(16, 3000))
            s1, s2 = W.arm_edges(rng, n, 2 * math.pi * math.sqrt(7) / 1500, np.full(7, -math.pi),
                                 np.full(7, math.pi), nmax=300)
            reqs.append(("motion", c, s1, s2))
        elif kind == 1:
            reqs.append(("validity", c, rng.uniform(-math.pi, math.pi, size=(int(rng.integers(1, 5000)), 7)), None))
        else:
            reqs.append(("knn", c, rng.uniform(-math.pi, math.pi, size=(int(rng.integers(1, 2000)), 7)), None))

    def submit(srv, r):
        kind, c, a, b = r
        ck, nn = clients[c]
        if kind == "motion":
            return srv.submit_motion(ck, a, b, schedule=capi.SCHEDULE_TILE)
        if kind == "validity":
            return srv.submit_validity(ck, a)
        return srv.submit_knn(nn, a, 10)

    srv = serve.Server(n_streams=8, arena_bytes=256 << 20)
    alone = []
    for r in reqs:  # one at a time
        res, _ = srv.wait(submit(srv, r))
        alone.append(res)
    tickets = [submit(srv, r) for r in reqs]  # all at once: admitted as slots free, overlapping
    mixed = [srv.wait(t)[0] for t in tickets]
    assert srv.stats()["max_concurrent"] > 1
    for r, x, y in zip(reqs, alone, mixed):
        keys = ("ok", "first_j", "nd") if r[0] == "motion" else (("ok",) if r[0] == "validity" else ("idx", "dist"))
        for key in keys:
            assert np.array_equal(x[key], y[key]), (r[0], key)
    # and the mix equals the direct (non-served) API
    for r, y in zip(reqs[:9], mixed[:9]):
        kind, c, a, b = r
        ck, nn = clients[c]
        if kind == "motion":
            d = B.DiscreteMotionValidator(ck).checkMotions(a, b, schedule=capi.SCHEDULE_TILE)
            assert np.array_equal(d["ok"], y["ok"]) and np.array_equal(d["first_j"], y["first_j"])
        elif kind == "validity":
            assert np.array_equal(ck.isValid(a).astype(np.uint8), y["ok"])
        else:
            idx, dist = nn.nearestK(a, 10)
            assert np.array_equal(idx, y["idx"])
    srv.close()


def test_admission_by_footprint():
    rng = np.random.default_rng(5)
    (ck, nn), = _clients(1, rng)
    srv = serve.Server(n_streams=4, arena_bytes=1 << 20)
    big = rng.uniform(-math.pi, math.pi, size=(40_000, 7))  # 2.2 MB of states: never fits
    with pytest.raises(capi.GboError):
        srv.submit_validity(ck, big)
    # the host staging arena (as large as the 1 MiB device arena) holds three of these at a time, so the
    # later submissions use the caller's arrays directly: both paths must return the direct API's results
    batches = [rng.uniform(-math.pi, math.pi, size=(5000, 7)) for _ in range(10)]
    small = [srv.submit_validity(ck, b) for b in batches]
    for t, b in zip(small, batches):
        res, lat = srv.wait(t)
        assert lat >= 0.0 and res["ok"].shape == (5000,)
        assert np.array_equal(res["ok"], ck.isValid(b).astype(np.uint8))
    srv.close()
