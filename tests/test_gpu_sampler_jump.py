"""Sampling calls of 2^18 stream words and more run on segments of the stream generated side by side
from jump-ahead windows (kernels_sample.cu, mt_jump.cu). Their values, and the stream position they
leave behind, must be OMPL's sampler stream bit for bit: calls of every size around the switch, AoS and
SoA output, sampleUniformNear (RealVector bounds and SO2 wrapping), and 153-segment calls, against the
oracle's sequential restatement of the stream."""
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


def same_bits(a, b):
    a, b = np.ascontiguousarray(a, dtype=np.float64), np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def rv(dim, lo=-1.5, hi=2.5):
    d = SpaceDesc(capi.SPACE_REAL_VECTOR, dim, np.linspace(lo, lo - 1.0, dim), np.linspace(hi, hi + 3.0, dim))
    return d, B.RealVectorStateSpace(dim, d.low, d.high)


@pytest.mark.parametrize("dim", [1, 3, 7, 10])
def test_calls_around_the_switch_continue_one_stream(port, dim):
    d, space = rv(dim)
    smp = B.StateSampler(space, 1000 + dim)
    words = [2 ** 18 - 2, 2 ** 18, 2 ** 18 + 2, 2 ** 20 + 10, 5 * 2 ** 17 + 6]
    sizes = [7]
    for w in words:
        sizes += [max(1, w // (2 * dim)), 3]
    got = []
    for i, n in enumerate(sizes):
        soa = i % 4 == 2
        a = smp.sampleUniform(n, soa=soa)
        got.append(a.T if soa else a)
    ref = port.sample_uniform(d, 1000 + dim, sum(sizes))
    off = 0
    for n, g in zip(sizes, got):
        assert same_bits(g, ref[off:off + n]), (dim, n, off)
        off += n


def test_many_segment_call(port):
    """1M 10-D states: 20M words of the stream in 153 segments of 2^17 words."""
    d, space = rv(10)
    smp = B.StateSampler(space, 5)
    a = smp.sampleUniform(311)
    b = smp.sampleUniform(1_000_000, soa=True, host=False)
    c = smp.sampleUniform(9)
    ref = port.sample_uniform(d, 5, 311 + 1_000_000 + 9)
    assert same_bits(a, ref[:311]) and same_bits(c, ref[-9:])
    assert same_bits(b.cpu().numpy().T, ref[311:-9])


def test_near_on_segments_real_vector(port):
    d, space = rv(7)
    rng = np.random.default_rng(3)
    near = rng.uniform(d.low, d.high, size=(300_000, 7))
    got = B.StateSampler(space, 77).sampleUniformNear(near, 0.3)
    assert same_bits(got, port.sample_uniform_near(d, 77, near, 0.3))


def test_near_on_segments_so2(port):
    d = SpaceDesc(capi.SPACE_SO2, 1, np.array([-math.pi]), np.array([math.pi]))
    rng = np.random.default_rng(4)
    near = rng.uniform(-math.pi, math.pi, size=(2 ** 18, 1))
    got = B.StateSampler(B.SO2StateSpace(), 21).sampleUniformNear(near, 2.5)
    assert same_bits(got, port.sample_uniform_near(d, 21, near, 2.5))


def test_gaussian_calls_on_segments_continue_one_stream(port):
    """sampleGaussian draws a large call's polar candidates on jump-ahead segments and commits exactly the
    words used: calls below and above the switch, interleaved with uniform calls and with the cached
    second value crossing calls, against the oracle's polar method (log rounded to nearest)."""
    d = SpaceDesc(capi.SPACE_REAL_VECTOR, 7, np.full(7, -2.0), np.full(7, 2.0))
    space = B.RealVectorStateSpace(7, d.low, d.high)
    rng = np.random.default_rng(8)
    ops = [("uniform", 300), ("gaussian", 20_001), ("gaussian", 40_000), ("uniform", 5), ("gaussian", 3),
           ("gaussian", 150_001), ("uniform", 7)]
    n_mean = sum(c for k, c in ops if k == "gaussian")
    mean = rng.uniform(-1.5, 1.5, size=(n_mean, 7))
    smp = B.StateSampler(space, 123)
    got, mi = [], 0
    for kind, c in ops:
        if kind == "uniform":
            got.append(smp.sampleUniform(c))
        else:
            got.append(smp.sampleGaussian(mean[mi:mi + c], 0.4))
            mi += c
    want = port.sample_script(d, 123, ops, mean, 0.4, log_mode=1)
    assert same_bits(np.vstack(got), want)
