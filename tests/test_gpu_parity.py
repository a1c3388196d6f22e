"""GPU parity: libgbompl.so through its C ABI against OMPL's own outputs (golden fixtures) and the
oracle on seeded inputs. Booleans, first-invalid indices, segment counts, samples, and kNN index
sets must match exactly; FP64 values are compared bitwise except where the kinematic-chain space
evaluates sin/cos (CUDA's FP64 sin/cos vs glibc's may differ in the last bit; relative tolerance
1e-12 on those distances, see ulp_close)."""
import math

import numpy as np
import pytest

from helpers import checker_of, same_bits, space_of

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import capi  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402
from oracle.oracle import CheckerDesc, SpaceDesc  # noqa: E402

SCHEDULES = [capi.SCHEDULE_PLAIN, capi.SCHEDULE_TILE, capi.SCHEDULE_WARP]


def gpu_space(g_or_desc):
    d = g_or_desc if isinstance(g_or_desc, SpaceDesc) else space_of(g_or_desc)
    if d.kind == capi.SPACE_REAL_VECTOR:
        s = B.RealVectorStateSpace(d.dim, d.low, d.high)
    elif d.kind == capi.SPACE_SO2:
        s = B.SO2StateSpace()
    elif d.kind == capi.SPACE_KINEMATIC_CHAIN:
        s = B.KinematicChainSpace(d.dim, d.link_length)
    else:
        s = B.WrapL2StateSpace(d.dim)
    s.setLongestValidSegmentFraction(d.lvs_fraction)
    s.setValidSegmentCountFactor(d.factor)
    return s


def gpu_checker(space, ck: CheckerDesc):
    if ck.kind == capi.CHECK_CIRCLES:
        return B.CirclesValidityChecker(space, ck.obstacles)
    if ck.kind == capi.CHECK_CHAIN_SEGMENTS:
        return B.KinematicChainValidityChecker(space, ck.obstacles)
    if ck.kind == capi.CHECK_DH_SPHERES:
        return B.DHSphereArmValidityChecker(space, ck.dh, ck.obstacles, ck.spheres_per_link, ck.sphere_radius)
    return B.AllValidStateValidityChecker(space)


def ulp_close(a, b, rel=1e-12):
    """The kinematic-chain metric sums differences of sin/cos values; CUDA's FP64 sin/cos and glibc's
    differ in the last bit, and the cancellation in cos(t1) - cos(t2) magnifies that to a relative
    difference of up to ~1e-13 in the distance. Tolerance: relative 1e-12."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    diff = np.abs(a - b)
    tol = rel * np.maximum(np.abs(a), np.abs(b))
    return bool(np.all(both_nan | (diff <= tol) | (a == b)))


# ------------------------------------------------------------------ FP32 arithmetic error bounds
def test_fp32_sincos_error_bound():
    """The guard band of the FP32 chain path assumes |cos/sin error| <= 1.3e-7 per component."""
    rng = np.random.default_rng(8)
    th = np.concatenate([rng.uniform(-35, 35, 2_000_000), np.linspace(-35, 35, 200_001),
                         np.arange(-22, 23) * (math.pi / 4), np.array([0.0, 1e-30, -1e-20, 5e-9])])
    t = torch.as_tensor(th, device="cuda")
    c = torch.empty(len(th), dtype=torch.float32, device="cuda")
    s = torch.empty_like(c)
    capi.check(capi.lib().gbo_sincos32(B._ptr(t), len(th), B._ptr(c), B._ptr(s), B._stream(None)))
    ec = np.abs(c.cpu().numpy().astype(np.float64) - np.cos(th)).max()
    es = np.abs(s.cpu().numpy().astype(np.float64) - np.sin(th)).max()
    assert ec <= 1.3e-7 and es <= 1.3e-7, (ec, es)


# ------------------------------------------------------------------ spaces and samplers
@pytest.mark.parametrize("name", ["rv2", "rv7", "so2", "chain10", "wrap7"])
def test_space_distance_interpolate_vs_ompl(golden, name):
    g = golden(f"space_{name}")
    s = gpu_space(g)
    assert s.getMaximumExtent() == g["extent"] and s.getLongestValidSegmentLength() == g["lvs"]
    d = s.distance(g["a"], g["b"])
    it = s.interpolate(g["a"], g["b"], g["t"])
    if name == "chain10":
        assert ulp_close(d, g["distance"])
    else:
        assert same_bits(d, g["distance"])
    assert same_bits(it, g["interpolate"])


@pytest.mark.parametrize("name", ["rv2", "rv7", "so2", "chain10", "wrap7"])
def test_sampler_stream_vs_ompl(golden, name):
    g = golden(f"space_{name}")
    s = gpu_space(g)
    smp = B.StateSampler(s, int(g["sample_seed"]))
    # the stream continues across calls of odd sizes (word pairs straddle 624-word blocks)
    parts = [smp.sampleUniform(n) for n in (1, 155, 313, 231)]
    assert same_bits(np.vstack(parts), g["sample"])
    near = B.StateSampler(s, 11).sampleUniformNear(g["near"], float(g["near_distance"]))
    assert same_bits(near, g["sample_near"])


def _gpu_script(smp, ops, mean, stddev):
    rows, m = [], 0
    for kind, c in ops:
        if kind == "gaussian":
            rows.append(smp.sampleGaussian(mean[m:m + c], stddev))
            m += c
        else:
            rows.append(smp.sampleUniform(c))
    return np.vstack(rows)


def _gauss_rows(ops):
    return np.concatenate([np.full(c, k == "gaussian") for k, c in ops])


@pytest.mark.parametrize("name", ["rv2", "rv7", "so2", "chain10", "wrap7"])
def test_sampler_gaussian_vs_ompl(golden, port, name):
    """sampleGaussian interleaved with sampleUniform on one sampler, odd call sizes (the cached normal
    value crosses calls). Bitwise against the polar method with a log rounded to nearest (the oracle's
    log_mode 1); against OMPL's own output every uniform row is bitwise (same stream position) and a
    Gaussian value differs only where glibc's log rounds the other way: by at most 4 ulps of the
    value's magnitude or of the mean's, in under 1% of the values."""
    g = golden(f"space_{name}")
    sp = space_of(g)
    ops = [(("uniform", "gaussian")[int(k)], int(c)) for k, c in zip(g["gauss_kinds"], g["gauss_counts"])]
    mean, sd = g["gauss_mean"], float(g["gauss_stddev"])
    got = _gpu_script(B.StateSampler(gpu_space(g), int(g["gauss_seed"])), ops, mean, sd)
    assert same_bits(got, port.sample_script(sp, int(g["gauss_seed"]), ops, mean, sd, log_mode=1))
    ref = g["gauss_out"]
    gr = _gauss_rows(ops)
    assert same_bits(got[~gr], ref[~gr])
    a, b = got[gr], ref[gr]
    scale = np.maximum(np.maximum(np.abs(a), np.abs(b)), 1.0)
    assert np.all(np.abs(a - b) <= 4 * np.finfo(np.float64).eps * scale)
    assert np.count_nonzero(a != b) <= 0.01 * a.size


def test_sampler_gaussian_across_chunks_vs_oracle(port):
    """One sampleGaussian call of 14M values (more polar candidates than one chunk of the word scratch,
    2^25 words, holds, so two host rounds), then a uniform call: bitwise against the oracle's polar
    method with the log rounded to nearest, and the stream position after the call is OMPL's."""
    d = SpaceDesc(capi.SPACE_REAL_VECTOR, 7, np.full(7, -2.0), np.full(7, 2.0))
    s = gpu_space(d)
    n = 2_000_001
    rng = np.random.default_rng(5)
    mean = rng.uniform(-1.5, 1.5, size=(n + 3, 7))
    ops = [("gaussian", 2), ("gaussian", n), ("gaussian", 1), ("uniform", 9)]
    smp = B.StateSampler(s, 77)
    got = _gpu_script(smp, ops, mean, 0.5)
    want = port.sample_script(d, 77, ops, mean, 0.5, log_mode=1)
    assert same_bits(got[:1000], want[:1000]) and same_bits(got[-20:], want[-20:])
    assert same_bits(got, want)
    # the same values on the device through the torch wrapper (device mean rows)
    smp2 = B.StateSampler(s, 77)
    dm = torch.from_numpy(mean[:5]).cuda()
    assert same_bits(smp2.sampleGaussian(dm, 0.5).cpu().numpy(), want[:5])


def test_sampler_gaussian_so2_wraps_and_rv_clamps(port):
    """Large standard deviations: SO2 values wrap into [-pi, pi) and RealVector values clamp to the
    bounds, as OMPL's samplers do (bitwise against the oracle with the rounded-to-nearest log)."""
    for d, sd in ((SpaceDesc(capi.SPACE_SO2, 1), 9.0),
                  (SpaceDesc(capi.SPACE_REAL_VECTOR, 3, np.array([0.0, -1.0, 5.0]), np.array([1.0, 1.0, 5.5])), 3.0)):
        mean = np.random.default_rng(2).uniform(-3, 3, size=(5001, d.dim))
        got = B.StateSampler(gpu_space(d), 3).sampleGaussian(mean, sd)
        want = port.sample_script(d, 3, [("gaussian", 5001)], mean, sd, log_mode=1)
        assert same_bits(got, want)
        if d.kind == capi.SPACE_SO2:
            assert np.all((got >= -math.pi) & (got < math.pi))
        else:
            assert np.all((got >= d.low) & (got <= d.high)) and np.any(got == d.low) and np.any(got == d.high)


def test_sampler_large_stream_vs_oracle(port):
    d = SpaceDesc(capi.SPACE_REAL_VECTOR, 7, np.full(7, -math.pi), np.full(7, math.pi))
    s = gpu_space(d)
    smp = B.StateSampler(s, 4)
    a = smp.sampleUniform(100_000, soa=True)      # SoA output
    b = smp.sampleUniform(77_777)
    ref = port.sample_uniform(d, 4, 177_777)
    assert same_bits(a.T, ref[:100_000]) and same_bits(b, ref[100_000:])


def test_sampler_stream_across_word_chunks_vs_oracle(port):
    """A call of 9M values (18M words of the stream, more than one chunk of the word scratch) and the
    calls around it continue one stream exactly as OMPL's sampler draws it, odd-length calls included."""
    d = SpaceDesc(capi.SPACE_REAL_VECTOR, 2, np.array([-1.0, 0.0]), np.array([1.0, 3.0]))
    s = gpu_space(d)
    smp = B.StateSampler(s, 29)
    a = smp.sampleUniform(311)
    b = smp.sampleUniform(4_500_000, host=False)
    c = smp.sampleUniform(5)
    ref = port.sample_uniform(d, 29, 311 + 4_500_000 + 5)
    assert same_bits(a, ref[:311]) and same_bits(c, ref[-5:])
    bb = b.cpu().numpy()
    assert same_bits(bb[:1000], ref[311:1311]) and same_bits(bb[-1000:], ref[-1005:-5])
    assert same_bits(bb, ref[311:-5])


# ------------------------------------------------------------------ validity / motion vs OMPL fixtures
CASES = ["circles_seeded", "circles_ompl_tests", "chain_seeded", "chain_horn", "dh_arm"]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "fp32_guarded"])
def test_validity_vs_ompl(golden, name, precision):
    g = golden(name)
    s = gpu_space(g)
    ck = gpu_checker(s, checker_of(g))
    ck.setPrecision(precision)
    assert np.array_equal(ck.isValid(g["states"]), g["valid"].astype(bool))
    assert np.array_equal(ck.isValidHost(g["states"]), g["valid"].astype(bool))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "fp32_guarded"])
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_discrete_motion_vs_ompl(golden, name, precision, schedule):
    g = golden(name)
    s = gpu_space(g)
    ck = gpu_checker(s, checker_of(g))
    ck.setPrecision(precision)
    mv = B.DiscreteMotionValidator(ck)
    r = mv.checkMotions(g["s1"], g["s2"], schedule=schedule, last_valid=True)
    assert np.array_equal(r["ok"], g["ok"])
    assert np.array_equal(r["ok"], g["ok_bisect"])
    assert np.array_equal(r["nd"], g["nd"])
    assert np.array_equal(r["first_j"], g["first_j"])
    assert same_bits(r["last_t"], g["last_t"])
    assert same_bits(r["last_state"], g["last_state"])


@pytest.mark.parametrize("name", CASES)
def test_motion_host_dropin_vs_ompl(golden, name):
    g = golden(name)
    s = gpu_space(g)
    ck = gpu_checker(s, checker_of(g))
    mv = B.DiscreteMotionValidator(ck)
    ok, lt, ls = mv.checkMotionHost(g["s1"], g["s2"])
    assert np.array_equal(ok, g["ok"].astype(bool))
    assert same_bits(lt, g["last_t"]) and same_bits(ls, g["last_state"])
    # single-edge OMPL-style call
    lv = [None, 0.0]
    i = int(np.argmin(g["ok"]))
    assert mv.checkMotion(g["s1"][i], g["s2"][i], lv) == bool(g["ok"][i])
    if not g["ok"][i]:
        assert lv[1] == g["last_t"][i]


def test_motion_states_vs_ompl(golden):
    g = golden("motion_states")
    s = gpu_space(g)
    mv = B.DiscreteMotionValidator(gpu_checker(s, checker_of(g)))
    off = 0
    for i in range(len(g["count"])):
        n = int(g["lengths"][i])
        st = g["states"][off:off + n]
        off += n
        if n == 0:
            continue
        ok, fi = mv.checkMotionStates(st)
        assert ok == bool(g["ok"][i])
        if not ok:
            assert fi == g["first_invalid"][i]


def test_get_motion_states_vs_ompl(golden):
    """SpaceInformation::getMotionStates (alloc = true) per fixture edge, bitwise against OMPL; and the
    same edges batched per (count, endpoints)."""
    g = golden("motion_states")
    s = gpu_space(g)
    off = 0
    groups = {}
    for i in range(len(g["count"])):
        n = int(g["lengths"][i])
        want = g["states"][off:off + n]
        off += n
        cnt, ep = int(g["count"][i]), bool(g["endpoints"][i])
        got = s.getMotionStates(g["a"][i:i + 1], g["b"][i:i + 1], cnt, endpoints=ep)[0]
        assert same_bits(got, want), i
        groups.setdefault((cnt, ep), []).append((i, want))
    for (cnt, ep), items in groups.items():
        rows = [i for i, _ in items]
        got = s.getMotionStates(g["a"][rows], g["b"][rows], cnt, endpoints=ep)
        for j, (_, want) in enumerate(items):
            assert same_bits(got[j], want)


def _valid_sampler_walk(flags, n, attempts):
    """UniformValidStateSampler::sample n times over a stream with validity flags: (index, ok) per call
    and the number of draws consumed."""
    A = max(attempts, 1)
    out, q = [], 0
    for _ in range(n):
        for a in range(A):
            if flags[q] or a == A - 1:
                out.append((q, bool(flags[q])))
                q += 1
                break
            q += 1
    return out, q


@pytest.mark.parametrize("name,attempts", [("circles_seeded", 100), ("chain_seeded", 100), ("chain_seeded", 3)])
def test_sample_valid_vs_oracle(golden, port, name, attempts):
    g = golden(name)
    sd, ckd = space_of(g), checker_of(g)
    s = gpu_space(g)
    ck = gpu_checker(s, ckd)
    seed, n = 1234, 3000
    stream = port.sample_uniform(sd, seed, n * max(attempts, 1) + 64)
    flags = port.is_valid(sd, ckd, stream).astype(bool)
    calls, used = _valid_sampler_walk(flags, n, attempts)
    sampler = B.StateSampler(s, seed)
    for prec in ("fp32_guarded",):
        ck.setPrecision(prec)
        st, ok = sampler.sampleValid(ck, n, attempts=attempts)
        idx = np.array([i for i, _ in calls])
        assert np.array_equal(ok, np.array([v for _, v in calls]))
        assert same_bits(st, stream[idx])
        # the stream continues exactly where OMPL's would
        nxt = sampler.sampleUniform(5)
        assert same_bits(nxt, stream[used:used + 5])
    # host-memory form on a fresh sampler with the same seed
    import ctypes as C
    h = B.StateSampler(s, seed)
    out, okh = np.empty((n, sd.dim)), np.empty(n, dtype=np.uint8)
    capi.check(capi.lib().gbo_sample_valid_host(h._h, ck._h, n, attempts, out.ctypes.data_as(C.c_void_p),
                                                okh.ctypes.data_as(C.c_void_p)))
    assert np.array_equal(okh.astype(bool), ok) and same_bits(out, st)


# ------------------------------------------------------------------ larger seeded cases vs the oracle
@pytest.fixture(scope="module")
def chain_case(port):
    w = W.config1(n_states=200_000, n_edges=10, n_queries=10)
    sp = SpaceDesc(w.space_kind, w.dim, link_length=w.link_length, lvs_fraction=w.lvs_fraction)
    ck = CheckerDesc(w.checker_kind, w.obstacles)
    port.set_threads(16)
    valid = port.is_valid(sp, ck, w.states)
    return w, sp, ck, valid


def test_chain_validity_200k_vs_oracle(chain_case):
    w, sp, ckd, valid = chain_case
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    for p in ("fp64", "fp32_guarded"):
        ck.setPrecision(p)
        got = ck.isValid(torch.as_tensor(w.states.T.copy(), device="cuda"), soa=True).cpu().numpy()
        assert np.array_equal(got, valid), p


def test_chain_motion_valid_endpoints_vs_oracle(chain_case, port):
    w, sp, ckd, valid = chain_case
    vs = w.states[valid == 1]
    rng = np.random.default_rng(3)
    i, j = rng.integers(0, len(vs), 3000), rng.integers(0, len(vs), 3000)
    s1, s2 = vs[i], vs[j]
    ref = port.check_motion(sp, ckd, s1, s2, want_state=False, want_bisect=False)
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    mv = B.DiscreteMotionValidator(ck)
    for p in ("fp64", "fp32_guarded"):
        ck.setPrecision(p)
        for sch in SCHEDULES:
            r = mv.checkMotions(s1, s2, schedule=sch)
            assert np.array_equal(r["ok"], ref["ok"]) and np.array_equal(r["first_j"], ref["first_j"])
            assert np.array_equal(r["nd"], ref["nd"])


@pytest.mark.parametrize("n_seg", [600, 1500])
def test_chain_large_world_vs_oracle(port, n_seg):
    """Worlds of 600 and 1,500 short segments: the warp kernels' per-warp test tables then need fewer
    warps per CTA (128 and 64 threads) to fit in shared memory. Validity and motion vs the oracle."""
    rng = np.random.default_rng(n_seg)
    c = rng.uniform(-1, 1, size=(n_seg, 2))
    ang = rng.uniform(-math.pi, math.pi, n_seg)
    half = 0.004 * np.stack([np.cos(ang), np.sin(ang)], axis=1)
    world = np.concatenate([c - half, c + half], axis=1)
    sp = SpaceDesc(capi.SPACE_KINEMATIC_CHAIN, 10, link_length=0.1, lvs_fraction=0.005)
    ckd = CheckerDesc(capi.CHECK_CHAIN_SEGMENTS, world)
    states = rng.uniform(-math.pi, math.pi, size=(6000, 10))
    port.set_threads(16)
    valid = port.is_valid(sp, ckd, states).astype(bool)
    vs = states[valid]
    assert len(vs) > 100
    i, j = rng.integers(0, len(vs), 400), rng.integers(0, len(vs), 400)
    ref = port.check_motion(sp, ckd, vs[i], vs[j], want_state=False, want_bisect=False)
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    ck.setPrecision("fp32_guarded")
    assert np.array_equal(ck.isValid(states), valid)
    r = B.DiscreteMotionValidator(ck).checkMotions(vs[i], vs[j], schedule=capi.SCHEDULE_WARP)
    assert np.array_equal(r["ok"], ref["ok"]) and np.array_equal(r["first_j"], ref["first_j"])


def _chain_points(q, L=0.1):
    """Joint positions in the reference's operation order (KinematicChain.h:214-228)."""
    th, x, y, pts = 0.0, 0.0, 0.0, [(0.0, 0.0)]
    for a in q:
        th += a
        x += math.cos(th) * L
        y += math.sin(th) * L
        pts.append((x, y))
    return pts, th


def _boundary_world(q):
    """World segments on the reference test's boundaries for the chain at q: collinear with links 2-4,
    through joint 7 (2e-6 long), ending on joint 5, parallel to the chain 1e-9 away (plus 1e-12 tilt)."""
    pts, th = _chain_points(q)
    (x2, y2), (x5, y5), (x7, y7) = pts[2], pts[5], pts[7]
    c, s_ = math.cos(th), math.sin(th)
    return np.array([[x2, y2, x5, y5],
                     [x7 - 1e-6 * s_, y7 + 1e-6 * c, x7 + 1e-6 * s_, y7 - 1e-6 * c],
                     [x5, y5, x5 + 0.3 * s_, y5 - 0.3 * c],
                     [x2 + 1e-12, y2 + 1e-9, x7, y7 + 1e-9 + 1e-12],
                     [-1.5, 1.4, 1.5, 1.4], [1.4, -1.5, 1.4, 1.5]])  # axis-aligned, clear of the chain


def test_chain_boundary_configurations_vs_oracle(port):
    """States and worlds on the reference test's own boundaries (demos/KinematicChain.h:251-276):
    world segments collinear with links, through a joint point, ending on a joint, parallel within
    1e-9, axis-aligned (exact zero cross products); straight and folded chains perturbed by 0 to 1e-5.
    The FP32 path must send every undecided comparison to FP64 and agree with the oracle exactly."""
    rng = np.random.default_rng(12)
    n = 10
    bases = [np.r_[0.3, np.zeros(n - 1)], np.r_[0.0, np.zeros(n - 1)], np.r_[math.pi / 2, np.zeros(n - 1)],
             np.r_[-2.0, np.full(n - 1, 0.25)]]
    sd = SpaceDesc(capi.SPACE_KINEMATIC_CHAIN, n, link_length=0.1, lvs_fraction=0.005)
    s = gpu_space(sd)
    n_valid = n_invalid = 0
    for q in bases:
        ckd = CheckerDesc(capi.CHECK_CHAIN_SEGMENTS, _boundary_world(q))
        states = np.concatenate([q + rng.standard_normal((40, n)) * scale
                                 for scale in (0.0, 1e-15, 1e-12, 1e-9, 1e-7, 1e-5, 1e-3)])
        ref = port.is_valid(sd, ckd, states).astype(bool)
        n_valid += int(ref.sum())
        n_invalid += int((~ref).sum())
        ck = gpu_checker(s, ckd)
        for p in ("fp64", "fp32_guarded"):
            ck.setPrecision(p)
            assert np.array_equal(ck.isValid(states), ref), p
        # motions between the boundary states
        i, j = rng.integers(0, len(states), 300), rng.integers(0, len(states), 300)
        mref = port.check_motion(sd, ckd, states[i], states[j], want_state=False, want_bisect=False)
        mv = B.DiscreteMotionValidator(ck)
        for p in ("fp64", "fp32_guarded"):
            ck.setPrecision(p)
            for sch in SCHEDULES:
                r = mv.checkMotions(states[i], states[j], schedule=sch)
                assert np.array_equal(r["ok"], mref["ok"]), (p, sch)
                assert np.array_equal(r["first_j"], mref["first_j"]), (p, sch)
    assert n_valid > 0 and n_invalid > 0


def test_chain_motion_deferred_edges_vs_oracle(chain_case, port):
    """Edges the FP32 warp kernel hands to its FP64 follow-up kernel: a joint difference within 1e-9
    of pi (the interpolation's shortest-arc branch), and zero or tiny length (segment count not
    decided by the FP32 distance bound); mixed with ordinary edges in one batch."""
    w, sp, ckd, valid = chain_case
    vs = w.states[valid == 1]
    rng = np.random.default_rng(5)
    n = 600
    s1 = vs[rng.integers(0, len(vs), n)].copy()
    s2 = vs[rng.integers(0, len(vs), n)].copy()
    rows = np.arange(200)
    k = rng.integers(0, w.dim, 200)
    off = np.array([0.0, 5e-10, -5e-10, 2e-9])[rng.integers(0, 4, 200)]
    base = s1[rows, k]
    s2[rows, k] = np.clip(np.where(base > 0, base - math.pi, base + math.pi) + off, -math.pi, math.pi)
    s2[200:300] = s1[200:300]                       # zero length
    s2[300:350] = s1[300:350] + 1e-12               # below the FP32 distance bound
    ref = port.check_motion(sp, ckd, s1, s2, want_state=False, want_bisect=False)
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    mv = B.DiscreteMotionValidator(ck)
    for p in ("fp64", "fp32_guarded"):
        ck.setPrecision(p)
        for sch in SCHEDULES:
            r = mv.checkMotions(s1, s2, schedule=sch)
            assert np.array_equal(r["ok"], ref["ok"]), (p, sch)
            assert np.array_equal(r["first_j"], ref["first_j"]), (p, sch)
            assert np.array_equal(r["nd"], ref["nd"]), (p, sch)
    ck.setPrecision("fp32_guarded")
    mv.checkMotions(s1, s2, schedule=capi.SCHEDULE_WARP)
    assert ck.stats()["rechecked"] >= 200   # the last call's FP64 work: at least the deferred edges


def test_motion_host_pinned_and_pageable_vs_oracle(chain_case, port):
    """The host entry point reads and writes page-locked arrays in place (mapped over the host link)
    and copies pageable ones; both must equal the oracle for every edge, with and without lastValid,
    and with mixed pinned / pageable arguments."""
    import ctypes as C
    w, sp, ckd, valid = chain_case
    vs = w.states[valid == 1]
    rng = np.random.default_rng(17)
    n = 70_001
    s1, s2 = vs[rng.integers(0, len(vs), n)], vs[rng.integers(0, len(vs), n)]
    ref = port.check_motion(sp, ckd, s1, s2, want_state=True, want_bisect=False)
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    ck.setPrecision("fp32_guarded")
    mv = B.DiscreteMotionValidator(ck)
    ok, lt, ls = mv.checkMotionHost(s1, s2)                      # pageable
    assert np.array_equal(ok, ref["ok"].astype(bool))
    assert same_bits(lt, ref["last_t"]) and same_bits(ls, ref["last_state"])
    ok2, _, _ = mv.checkMotionHost(s1, s2, last_valid=False)
    assert np.array_equal(ok2, ok)
    p1, p2 = torch.as_tensor(s1).pin_memory(), torch.as_tensor(s2).pin_memory()
    for pinned_out in (True, False):
        okp = torch.zeros(n, dtype=torch.uint8)
        ltp = torch.zeros(n, dtype=torch.float64)
        lsp = torch.zeros((n, w.dim), dtype=torch.float64)
        if pinned_out:
            okp, ltp, lsp = okp.pin_memory(), ltp.pin_memory(), lsp.pin_memory()
        vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        capi.check(capi.lib().gbo_check_motion_host(ck._h, vp(p1), vp(p2), n, vp(okp), vp(ltp), vp(lsp)))
        assert np.array_equal(okp.numpy().astype(bool), ref["ok"].astype(bool)), pinned_out
        assert same_bits(ltp.numpy(), ref["last_t"]) and same_bits(lsp.numpy(), ref["last_state"]), pinned_out
    # validity through the host entry point, pinned in place and pageable
    st = w.states[:50_000]
    ref_v = valid[:50_000].astype(bool)
    assert np.array_equal(ck.isValidHost(st), ref_v)
    pst, pout = torch.as_tensor(st).pin_memory(), torch.zeros(len(st), dtype=torch.uint8).pin_memory()
    capi.check(capi.lib().gbo_is_valid_host(ck._h, C.c_void_p(pst.data_ptr()), len(st), C.c_void_p(pout.data_ptr())))
    assert np.array_equal(pout.numpy().astype(bool), ref_v)


def test_dh_arm_motion_vs_oracle(port):
    w = W.config2(n_edges=400, n_world=1024)
    sp = SpaceDesc(w.space_kind, 7, w.low, w.high, lvs_fraction=w.lvs_fraction)
    ckd = CheckerDesc(w.checker_kind, w.obstacles, dh=w.dh, spheres_per_link=8, sphere_radius=0.05)
    port.set_threads(16)
    ref = port.check_motion(sp, ckd, w.s1, w.s2, want_state=False, want_bisect=False)
    st = np.random.default_rng(9).uniform(-math.pi, math.pi, size=(3000, 7))
    vref = port.is_valid(sp, ckd, st)
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    mv = B.DiscreteMotionValidator(ck)
    for p in ("fp64", "fp32_guarded"):
        ck.setPrecision(p)
        assert np.array_equal(ck.isValid(st), vref.astype(bool)), p
        for sch in SCHEDULES:
            r = mv.checkMotions(w.s1, w.s2, schedule=sch)
            assert np.array_equal(r["ok"], ref["ok"]) and np.array_equal(r["first_j"], ref["first_j"]), (p, sch)
            assert np.array_equal(r["nd"], ref["nd"])


# ------------------------------------------------------------------ nearest neighbours
@pytest.mark.parametrize("name", ["rv2", "chain10", "wrap7"])
@pytest.mark.parametrize("precision", ["fp64", "fp32_guarded"])
def test_knn_vs_ompl(golden, name, precision):
    g = golden(f"knn_{name}")
    s = gpu_space(g)
    nn = B.NearestNeighborsGPU(s, capacity=len(g["pts"]) + 10, precision=precision)
    nn.add(g["pts"])
    assert nn.size() == len(g["pts"])
    k = int(g["k"])
    idx, dist = nn.nearestK(g["q"], k)
    assert np.array_equal(idx, g["linear_idx"])
    if name == "chain10":
        assert ulp_close(dist, g["linear_dist"])
    else:
        assert same_bits(dist, g["linear_dist"])
    pi_, pd_ = nn.nearestK(g["q"], k, prefix=g["prefix_limit"])
    assert np.array_equal(pi_, g["prefix_idx"])
    counts, ri, rd = nn.nearestR(g["q"], float(g["r"]))
    assert np.array_equal(counts, g["radius_counts"]) and np.array_equal(ri, g["radius_idx"])


def test_knn_add_remove_pattern_vs_oracle(port):
    # interleaved add / query / remove like nearestneighbors.cpp:205-280 (randomAccessPatternTest)
    rng = np.random.default_rng(21)
    d = SpaceDesc(capi.SPACE_WRAP_L2, 7, lvs_fraction=0.01)
    s = gpu_space(d)
    nn = B.NearestNeighborsGPU(s, capacity=5000)
    pts = rng.uniform(-math.pi, math.pi, size=(4000, 7))
    alive = np.zeros(4000, dtype=bool)
    added = 0
    for step in range(8):
        n = 500
        nn.add(pts[added:added + n])
        alive[added:added + n] = True
        added += n
        kill = rng.choice(np.flatnonzero(alive), size=120, replace=False)
        nn.remove(kill)
        alive[kill] = False
        assert nn.size() == alive.sum()
        q = rng.uniform(-math.pi, math.pi, size=(64, 7))
        k = int(rng.integers(1, 20))
        idx, dist = nn.nearestK(q, k)
        keys = np.flatnonzero(alive)
        ri, rd = port.knn(d, pts[keys], q, k)
        assert np.array_equal(idx, keys[ri]) and same_bits(dist, rd)


def test_knn_chain_large_vs_oracle(chain_case, port):
    w, sp, _, _ = chain_case
    s = gpu_space(sp)
    nn = B.NearestNeighborsGPU(s, capacity=len(w.states))
    nn.add(torch.as_tensor(w.states, device="cuda"))
    q = w.states[np.random.default_rng(2).integers(0, len(w.states), 40)]
    idx, dist = nn.nearestK(q, 16)
    ri, rd = port.knn(sp, w.states, q, 16)
    assert np.array_equal(idx, ri) and ulp_close(dist, rd)
    assert idx[:, 0].tolist() == [int(np.flatnonzero((w.states == qq).all(1))[0]) for qq in q]


@pytest.mark.parametrize("kind", ["chain10", "wrap7", "rv7"])
def test_knn_large_batch_vs_exact_scan(kind):
    """Large batches (4,500 queries over 70,000 elements; RealVector and wrapped spaces go through the
    cell index) with FP32 distances and FP64 re-check: index sets and FP64 distances must equal the
    exact FP64 scan's, with and without PRM prefix limits, for fresh and self queries, and after
    removals (which invalidate the cell index)."""
    rng = np.random.default_rng(21)
    n, dim = 70_000, (10 if kind == "chain10" else 7)
    if kind == "chain10":
        space = B.KinematicChainSpace(10, 0.1)
    elif kind == "wrap7":
        space = B.WrapL2StateSpace(7)
    else:
        space = B.RealVectorStateSpace(7, np.full(7, -math.pi), np.full(7, math.pi))
    pts = rng.uniform(-math.pi, math.pi, size=(n, dim))
    queries = np.concatenate([pts[:3000], rng.uniform(-math.pi, math.pi, size=(1500, dim))])
    nn = B.NearestNeighborsGPU(space, capacity=n)
    nn.add(pts)

    def both(k, prefix=None):
        nn.setPrecision("fp32_guarded")
        i32, d32 = nn.nearestK(queries, k, prefix=prefix)
        st = nn.stats()  # the measured FP32 metric error stays inside the bound the guard band assumes
        assert 0.0 < st["max_fp32_error"] <= st["fp32_error_bound"], (kind, st)
        nn.setPrecision("fp64")
        i64, d64 = nn.nearestK(queries, k, prefix=prefix)
        assert np.array_equal(i32, i64), (kind, k)
        assert same_bits(d32, d64), (kind, k)

    for k in (10, 16):
        both(k)
    both(10, prefix=np.minimum(np.arange(len(queries)) * 13, n))
    if kind != "chain10":  # kept lists of 48 and 72 entries (k up to 64, PRM*'s connection counts)
        both(33)
        both(64, prefix=np.minimum(np.arange(len(queries)) * 13, n))
    nn.remove(np.arange(0, n, 7))
    both(16)
    assert nn.stats()["queries"] > 0


def test_dh_arm_large_world_read_from_global_memory(port):
    """A 16,384-sphere world does not fit the shared-memory staging limit: the FP32 path reads the
    spheres from global memory. Validity and motion must still equal the oracle's."""
    w = W.config4(n_world=16_384)
    sp = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
    ckd = CheckerDesc(w.checker_kind, w.obstacles, dh=w.dh, spheres_per_link=8, sphere_radius=0.05)
    rng = np.random.default_rng(13)
    st = rng.uniform(-math.pi, math.pi, size=(400, 7))
    port.set_threads(16)
    vref = port.is_valid(sp, ckd, st).astype(bool)
    e1, e2 = st[:60], st[60:120] * 0.25
    mref = port.check_motion(sp, ckd, e1, e2, want_state=False, want_bisect=False)
    s = gpu_space(sp)
    ck = gpu_checker(s, ckd)
    mv = B.DiscreteMotionValidator(ck)
    for p in ("fp32_guarded", "fp64"):
        ck.setPrecision(p)
        assert np.array_equal(ck.isValid(st), vref), p
        assert ck.stats() is not None
        r = mv.checkMotions(e1, e2, schedule=capi.SCHEDULE_TILE if p == "fp32_guarded" else capi.SCHEDULE_PLAIN)
        assert np.array_equal(r["ok"], mref["ok"]) and np.array_equal(r["first_j"], mref["first_j"]), p
