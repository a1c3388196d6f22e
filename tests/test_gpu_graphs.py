"""CUDA-graph capture of the path. Once a checker's schedule is tuned (the autotuner synchronises, so
it runs before any capture), DiscreteMotionValidator batches (the persistent kernels and the counter
reset are plain stream work) and validity batches capture into a CUDA graph, and so does the
allocation-free nearestK; replays over new inputs copied into the captured buffers must equal direct
calls."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402


def _same(a, b):
    return all(torch.equal(a[k], b[k]) for k in ("ok", "first_j", "nd"))


def test_motion_and_validity_replay_from_graph():
    w = W.config1(n_states=60_000, n_edges=10, n_queries=10)
    space = B.KinematicChainSpace(w.dim, w.link_length)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    ck = B.KinematicChainValidityChecker(space, w.obstacles)
    ck.setPrecision("fp32_guarded")
    mv = B.DiscreteMotionValidator(ck)
    st = torch.as_tensor(w.states.T.copy(), device="cuda")
    vs = st[:, ck.isValid(st, soa=True).bool()]
    g = torch.Generator(device="cpu").manual_seed(4)
    n = 20_000
    pick = lambda: vs[:, torch.randint(0, vs.shape[1], (n,), generator=g)].contiguous()  # noqa: E731
    a1, a2, b1, b2 = pick(), pick(), pick(), pick()
    ref_a = mv.checkMotions(a1, a2, schedule=capi.SCHEDULE_AUTO, soa=True)
    ref_b = mv.checkMotions(b1, b2, schedule=capi.SCHEDULE_AUTO, soa=True)
    val_a, val_b = ck.isValid(a1, soa=True), ck.isValid(b1, soa=True)
    s1, s2 = a1.clone(), a2.clone()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):  # warm-up on the capture stream's kind of stream
        mv.checkMotions(s1, s2, schedule=capi.SCHEDULE_AUTO, soa=True)
        ck.isValid(s1, soa=True)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        out = mv.checkMotions(s1, s2, schedule=capi.SCHEDULE_AUTO, soa=True)
        val = ck.isValid(s1, soa=True)
    for (x1, x2, ref, rv) in ((b1, b2, ref_b, val_b), (a1, a2, ref_a, val_a), (b1, b2, ref_b, val_b)):
        s1.copy_(x1)
        s2.copy_(x2)
        graph.replay()
        torch.cuda.synchronize()
        assert _same(out, ref)
        assert torch.equal(val, rv)


def test_noalloc_nearest_k_replay_from_graph():
    rng = np.random.default_rng(8)
    space = B.WrapL2StateSpace(7)
    pts = torch.as_tensor(rng.uniform(-np.pi, np.pi, size=(7, 50_000)), device="cuda")
    nn = B.NearestNeighborsGPU(space, capacity=50_000)
    nn.add(pts, soa=True)
    L = capi.lib()
    nq, k = 2048, 10
    qa = torch.as_tensor(rng.uniform(-np.pi, np.pi, size=(7, nq)), device="cuda")
    qb = torch.as_tensor(rng.uniform(-np.pi, np.pi, size=(7, nq)), device="cuda")
    ref_a, _ = nn.nearestK(qa, k, soa=True)
    ref_b, _ = nn.nearestK(qb, k, soa=True)
    q = qa.clone()
    idx = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dist = torch.empty((nq, k), dtype=torch.float64, device="cuda")

    def call():
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        return L.gbo_nn_nearest_k_noalloc(nn._h, C.c_void_p(q.data_ptr()), nq, nq, capi.LAYOUT_SOA, k, None,
                                          C.c_void_p(idx.data_ptr()), C.c_void_p(dist.data_ptr()), st)

    assert call() == capi.OK  # first call on the device looks the scratch array up, before capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        assert call() == capi.OK
    for qq, ref in ((qb, ref_b), (qa, ref_a)):
        q.copy_(qq)
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(idx, ref)
