"""gbo_nn_nearest_k_noalloc, the nearestK entry point that allocates no device memory during the call
(for callers that cannot allocate once set up: CUDA-graph capture, real-time planning loops, GPU
memory owned by another allocator). It must return exactly what gbo_nn_nearest_k returns, on
consecutive calls that reuse its fixed scratch array, and reject batches larger than that array.
Collected last (file name) so that a run stopping at the first failure has run everything else."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402


def _call(fn, nn, q, k, idx, dist, prefix=None, sync=True):
    nq = q.shape[1]
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    pre = C.c_void_p(prefix.data_ptr()) if prefix is not None else None
    status = fn(nn._h, C.c_void_p(q.data_ptr()), nq, nq, capi.LAYOUT_SOA, k, pre, C.c_void_p(idx.data_ptr()),
                C.c_void_p(dist.data_ptr()), st)
    if sync:
        torch.cuda.synchronize()
    return status


def _knn(fn, nn, q, k, prefix=None):
    nq = q.shape[1]
    idx = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dist = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    status = _call(fn, nn, q, k, idx, dist, prefix)
    return status, idx.cpu().numpy(), dist.cpu().numpy()


def _space(space_kind):
    if space_kind == "chain10":
        return B.KinematicChainSpace(10, 0.1), 10, 16
    return B.WrapL2StateSpace(7), 7, 10


def _index(space_kind, n, rng):
    space, dim, k = _space(space_kind)
    pts = torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, n)), device="cuda")
    nn = B.NearestNeighborsGPU(space, capacity=n)
    nn.add(pts, soa=True)
    torch.cuda.synchronize()
    return nn, dim, k


@pytest.mark.parametrize("space_kind", ["chain10", "wrap7"])
@pytest.mark.parametrize("n_points", [60_000, 70_000])
def test_noalloc_nearest_k_matches_regular(space_kind, n_points):
    L = capi.lib()
    rng = np.random.default_rng(31)
    nn, dim, k = _index(space_kind, n_points, rng)
    for call in range(3):  # calls in a row share the scratch array; the third restricts to a prefix
        nq = 3000 + 1000 * call if n_points < 65_536 else 1024 + 2048 * call
        q = torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, nq)), device="cuda")
        prefix = None
        if call == 2:
            prefix = torch.as_tensor(rng.integers(0, n_points + 1, size=nq), device="cuda")
        s0, i0, d0 = _knn(L.gbo_nn_nearest_k, nn, q, k, prefix)
        s1, i1, d1 = _knn(L.gbo_nn_nearest_k_noalloc, nn, q, k, prefix)
        assert s0 == capi.OK and s1 == capi.OK
        assert np.array_equal(i0, i1)
        assert np.array_equal(d0.view(np.uint64), d1.view(np.uint64))


def _cudart():
    """The CUDA runtime (for the default memory pool's reserved size), or None."""
    import glob
    import os
    for cand in ["libcudart.so"] + sorted(glob.glob(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                                                                 "lib64", "libcudart.so*"))):
        try:
            return C.CDLL(cand)
        except OSError:
            continue
    return None


def _pool_reserved(rt):
    pool = C.c_void_p()
    if rt is None or rt.cudaDeviceGetDefaultMemPool(C.byref(pool), torch.cuda.current_device()) != 0:
        return None
    v = C.c_uint64()
    reserved_mem_current = 5  # cudaMemPoolAttrReservedMemCurrent
    if rt.cudaMemPoolGetAttribute(pool, reserved_mem_current, C.byref(v)) != 0:
        return None
    return v.value


@pytest.mark.parametrize("space_kind", ["chain10", "wrap7"])
def test_noalloc_captures_in_a_cuda_graph_and_allocates_nothing(space_kind):
    """The call recorded in a CUDA graph and replayed on new query values gives the regular call's
    results; a burst of calls (batches up to the largest the scratch takes) changes neither the
    device's free memory, the default memory pool's reservation nor torch's."""
    L = capi.lib()
    rng = np.random.default_rng(47)
    nn, dim, k = _index(space_kind, 70_000, rng)
    nq = 4096
    q = torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, nq)), device="cuda")
    idx = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dist = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    assert _call(L.gbo_nn_nearest_k_noalloc, nn, q, k, idx, dist) == capi.OK  # looks the scratch up
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            status = _call(L.gbo_nn_nearest_k_noalloc, nn, q, k, idx, dist, sync=False)
    torch.cuda.synchronize()
    assert status == capi.OK
    for rep in range(3):
        q.copy_(torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, nq)), device="cuda"))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        s0, i0, d0 = _knn(L.gbo_nn_nearest_k, nn, q, k)
        assert s0 == capi.OK
        assert np.array_equal(idx.cpu().numpy(), i0), rep
        assert np.array_equal(dist.cpu().numpy().view(np.uint64), d0.view(np.uint64)), rep
    del g
    # allocation-free: sizes up to the largest batch, warmed first (module loading is not counted)
    big = 16_384
    qb = torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, big)), device="cuda")
    ib = torch.empty((big, k), dtype=torch.int64, device="cuda")
    db = torch.empty((big, k), dtype=torch.float64, device="cuda")
    sizes = [big, 1, 100, 5000, big // 2, big]
    for n in sizes:
        assert _call(L.gbo_nn_nearest_k_noalloc, nn, qb[:, :n].contiguous(), k, ib, db) == capi.OK
    views = [qb[:, :n].contiguous() for n in sizes]
    torch.cuda.synchronize()
    rt = _cudart()
    free0, pool0, torch0 = torch.cuda.mem_get_info()[0], _pool_reserved(rt), torch.cuda.memory_reserved()
    for _ in range(5):
        for v in views:
            assert _call(L.gbo_nn_nearest_k_noalloc, nn, v, k, ib, db, sync=False) == capi.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert _pool_reserved(rt) == pool0
    assert torch.cuda.memory_reserved() == torch0


def test_noalloc_rejects_batches_beyond_its_scratch():
    L = capi.lib()
    space = B.KinematicChainSpace(10, 0.1)
    nn = B.NearestNeighborsGPU(space, capacity=1000)
    nn.add(np.zeros((1000, 10)))
    q = torch.zeros((10, 200_000), dtype=torch.float64, device="cuda")
    s, _, _ = _knn(L.gbo_nn_nearest_k_noalloc, nn, q, 16)
    assert s == capi.ERR_OUT_OF_MEMORY
    assert b"scratch" in L.gbo_last_error()
