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


def _knn(fn, nn, q, k):
    nq = q.shape[1]
    idx = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dist = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = fn(nn._h, C.c_void_p(q.data_ptr()), nq, nq, capi.LAYOUT_SOA, k, None, C.c_void_p(idx.data_ptr()),
                C.c_void_p(dist.data_ptr()), st)
    torch.cuda.synchronize()
    return status, idx.cpu().numpy(), dist.cpu().numpy()


@pytest.mark.parametrize("space_kind", ["chain10", "wrap7"])
def test_noalloc_nearest_k_matches_regular(space_kind):
    L = capi.lib()
    rng = np.random.default_rng(31)
    if space_kind == "chain10":
        space = B.KinematicChainSpace(10, 0.1)
        dim, k = 10, 16
    else:
        space = B.WrapL2StateSpace(7)
        dim, k = 7, 10
    pts = torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, 60_000)), device="cuda")
    nn = B.NearestNeighborsGPU(space, capacity=60_000)
    nn.add(pts, soa=True)
    torch.cuda.synchronize()
    for call in range(2):  # two calls in a row share the scratch array
        nq = 3000 + 1000 * call
        q = torch.as_tensor(rng.uniform(-math.pi, math.pi, size=(dim, nq)), device="cuda")
        s0, i0, d0 = _knn(L.gbo_nn_nearest_k, nn, q, k)
        s1, i1, d1 = _knn(L.gbo_nn_nearest_k_noalloc, nn, q, k)
        assert s0 == capi.OK and s1 == capi.OK
        assert np.array_equal(i0, i1)
        assert np.array_equal(d0.view(np.uint64), d1.view(np.uint64))


def test_noalloc_rejects_batches_beyond_its_scratch():
    L = capi.lib()
    space = B.KinematicChainSpace(10, 0.1)
    nn = B.NearestNeighborsGPU(space, capacity=1000)
    nn.add(np.zeros((1000, 10)))
    q = torch.zeros((10, 200_000), dtype=torch.float64, device="cuda")
    s, _, _ = _knn(L.gbo_nn_nearest_k_noalloc, nn, q, 16)
    assert s == capi.ERR_OUT_OF_MEMORY
    assert b"scratch" in L.gbo_last_error()
