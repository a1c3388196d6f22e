"""Jump-ahead on the sampler's mt19937 (ompl_gb300/csrc/mt_jump.cu, host form gbo_mt19937_discard):
after discard(J) the generator gives the outputs that J draws later give, for every block position and
for jumps below, at and far above the 1,248-word switch to the jump polynomial. The reference stream is
CPython's own MT19937 (random.Random with its state set to the same 624 words). Host code only."""
import ctypes as C
import os
import random

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if not os.path.exists(os.path.join(ROOT, "ompl_gb300", "libgbompl.so")):
    pytest.skip("libgbompl.so not built", allow_module_level=True)

from ompl_gb300 import capi  # noqa: E402


def seeded(seed):
    """std::mt19937(seed)'s block (its index is then 624)."""
    mt = [seed & 0xFFFFFFFF]
    for i in range(1, 624):
        mt.append((1812433253 * (mt[-1] ^ (mt[-1] >> 30)) + i) & 0xFFFFFFFF)
    return mt


def outputs(mt, pos, n):
    r = random.Random()
    r.setstate((3, tuple(mt) + (pos,), None))
    return [r.getrandbits(32) for _ in range(n)]


@pytest.mark.parametrize("seed,pre", [(5489, 0), (1, 1), (77, 300), (2024, 623), (9, 624), (3, 625)])
@pytest.mark.parametrize("J", [0, 1, 623, 1247, 1248, 1249, 20_000, 262_144, 1_000_003])
def test_discard_matches_stepping(seed, pre, J):
    r = random.Random()
    r.setstate((3, tuple(seeded(seed)) + (624,), None))
    for _ in range(pre):
        r.getrandbits(32)
    state = r.getstate()[1]
    mt, pos = list(state[:624]), state[624]
    want = outputs(mt, pos, J + 700)[J:]
    a = (C.c_uint32 * 624)(*mt)
    p = C.c_uint32(pos)
    assert capi.lib().gbo_mt19937_discard(a, C.byref(p), J) == capi.OK
    assert 1 <= p.value <= 624
    assert outputs(list(a), p.value, 700) == want


def test_discard_rejects_a_bad_position():
    a = (C.c_uint32 * 624)(*seeded(1))
    p = C.c_uint32(0)
    assert capi.lib().gbo_mt19937_discard(a, C.byref(p), 5) == capi.ERR_INVALID_ARGUMENT
