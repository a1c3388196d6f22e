// Jump-ahead on the sampler's mt19937 stream, so that one sampling call's stretch of the stream can be
// generated by many CTAs at once, each from the generator state at the start of its segment.
//
// Method: Haramoto, Matsumoto, Nishimura, Panneton and L'Ecuyer, "Efficient jump ahead for F2-linear
// random number generators", INFORMS Journal on Computing 20(3), 2008. The generator state is a vector of
// 19937 bits over F2: the top bit of one raw word and the 623 raw words after it (a "window" of the raw
// output sequence x_t, before tempering). One step moves the window by one word; it is a linear map A
// whose characteristic polynomial phi has degree 19937. With p = x^J mod phi, A^J = p(A), so the window
// J steps ahead is sum_i p_i A^i s, and word w of it is the XOR, over the set coefficients p_i, of raw
// word i + w of the sequence that starts at window s.
// phi is recovered from 2 x 19937 bits of one output bit sequence with the Berlekamp-Massey algorithm
// (Massey, "Shift-register synthesis and BCH decoding", IEEE Trans. Inf. Theory 15(1), 1969); the
// polynomial arithmetic mod phi works on 64-bit words with 8-bit windows (products through a table of
// the 256 multiples of one factor, reduction through the 256 multiples of phi).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "kernels_nn.cuh"

namespace gbo
{
namespace mtj
{
constexpr int kDeg = 19937;          // degree of phi = bits of the state
constexpr int kW = 312;              // 64-bit words of a reduced polynomial (degree < 19937)
constexpr int kWP = 2 * kW;          // words of an unreduced product
constexpr int kWT = kW + 2;          // words of a table entry (degree < 19937 + 8, shifted by < 64)

using Poly = std::vector<uint64_t>;

static inline int bit(const uint64_t *a, int64_t i)
{
    return (int)((a[i >> 6] >> (i & 63)) & 1u);
}

static inline uint32_t twist_host(uint32_t cur, uint32_t next, uint32_t far)
{
    const uint32_t y = (cur & 0x80000000u) | (next & 0x7fffffffu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

struct Field
{
    Poly phi;                       // kW words, bit 19937 included (word 311, bit 33)
    uint8_t inv_top[256];           // byte t -> m with bits 19937..19944 of m * phi equal to t
    std::vector<uint64_t> red;      // [8 shift classes][256][kWT]: (m * phi) << 8c
    uint16_t spread[256];           // byte -> its bits at even positions
    bool ok = false;
};

// Berlekamp-Massey over F2 on bits s[0..n): the connection polynomial C (c_0 = 1) of the shortest
// LFSR generating s, and its length L.
static bool berlekamp_massey(const std::vector<uint8_t> &s, Poly &C, int &L)
{
    const int64_t n = (int64_t)s.size();
    const int64_t words = n / 64 + 3;
    std::vector<uint64_t> rs(words + 2, 0);  // s reversed: rs bit j = s[n-1-j]
    for (int64_t j = 0; j < n; ++j)
        if (s[n - 1 - j])
            rs[j >> 6] |= 1ull << (j & 63);
    C.assign(words, 0);
    Poly B(words, 0), T;
    C[0] = B[0] = 1;
    L = 0;
    int64_t m = 1, LB = 0;  // LB: degree bound of B
    for (int64_t i = 0; i < n; ++i)
    {
        // discrepancy: sum_{j=0..L} c_j s_{i-j}; s_{i-j} = rs bit (n-1-i+j)
        const int64_t off = n - 1 - i;
        const int64_t q = off >> 6, sh = off & 63;
        uint64_t acc = 0;
        for (int64_t k = 0; k <= L / 64; ++k)
        {
            uint64_t v = rs[q + k] >> sh;
            if (sh)
                v |= rs[q + k + 1] << (64 - sh);
            acc ^= v & C[k];
        }
        // bits of C above L are zero, so the words past L contribute nothing
        const int d = __builtin_parityll(acc);
        if (!d)
        {
            ++m;
            continue;
        }
        const bool grow = 2 * L <= i;
        if (grow)
            T.assign(C.begin(), C.begin() + (L / 64 + 2));
        // C += x^m B
        const int64_t ws = m >> 6, bs = m & 63;
        for (int64_t k = 0; k <= LB / 64 + 1 && k + ws + 1 < words; ++k)
        {
            C[k + ws] ^= B[k] << bs;
            if (bs)
                C[k + ws + 1] ^= B[k] >> (64 - bs);
        }
        if (grow)
        {
            const int64_t oldL = L;
            L = (int)(i + 1 - L);
            std::fill(B.begin(), B.end(), 0);
            std::copy(T.begin(), T.end(), B.begin());
            LB = oldL;
            m = 1;
        }
        else
            ++m;
    }
    return true;
}

static void build_field(Field &f)
{
    // one output bit sequence of the generator: bit 0 of raw word t + 1 (a coordinate of window t)
    const int64_t n = 2 * kDeg + 64;
    std::vector<uint32_t> x(n + 700);
    x[0] = 5489u;
    for (uint32_t i = 1; i < 624; ++i)
        x[i] = 1812433253u * (x[i - 1] ^ (x[i - 1] >> 30)) + i;
    for (size_t t = 624; t < x.size(); ++t)
        x[t] = twist_host(x[t - 624], x[t - 623], x[t - 227]);
    std::vector<uint8_t> s(n);
    for (int64_t t = 0; t < n; ++t)
        s[t] = (uint8_t)(x[t + 1] & 1u);
    Poly C;
    int L = 0;
    berlekamp_massey(s, C, L);
    if (L != kDeg)
        return;
    // phi(x) = x^L C(1/x): phi_j = c_{L-j}
    f.phi.assign(kW, 0);
    for (int j = 0; j <= kDeg; ++j)
        if (bit(C.data(), kDeg - j))
            f.phi[j >> 6] |= 1ull << (j & 63);
    if (!bit(f.phi.data(), kDeg) || !bit(f.phi.data(), 0))
        return;
    // multiples m * phi (m of degree < 8) and the inverse of their top byte
    std::vector<uint64_t> mul(256 * kWT, 0);
    for (int m = 1; m < 256; ++m)
        for (int u = 0; u < 8; ++u)
            if ((m >> u) & 1)
            {
                uint64_t *d = &mul[(size_t)m * kWT];
                for (int k = 0; k < kW; ++k)
                {
                    d[k] ^= f.phi[k] << u;
                    if (u)
                        d[k + 1] ^= f.phi[k] >> (64 - u);
                }
            }
    bool seen[256] = {};
    for (int m = 0; m < 256; ++m)
    {
        int t = 0;
        for (int u = 0; u < 8; ++u)
            t |= bit(&mul[(size_t)m * kWT], kDeg + u) << u;
        if (seen[t])
            return;
        seen[t] = true;
        f.inv_top[t] = (uint8_t)m;
    }
    f.red.assign((size_t)8 * 256 * kWT, 0);
    for (int c = 0; c < 8; ++c)
        for (int m = 0; m < 256; ++m)
        {
            const uint64_t *src = &mul[(size_t)m * kWT];
            uint64_t *d = &f.red[((size_t)c * 256 + m) * kWT];
            const int sh = 8 * c;
            for (int k = 0; k < kWT - 1; ++k)
            {
                d[k] ^= src[k] << sh;
                if (sh)
                    d[k + 1] ^= src[k] >> (64 - sh);
            }
        }
    for (int b = 0; b < 256; ++b)
    {
        uint16_t v = 0;
        for (int u = 0; u < 8; ++u)
            v |= (uint16_t)(((b >> u) & 1) << (2 * u));
        f.spread[b] = v;
    }
    f.ok = true;
}

static const Field &field()
{
    static Field f;
    static std::once_flag once;
    std::call_once(once, [] { build_field(f); });
    return f;
}

// p (kWP words, degree < 2 * 19937) reduced mod phi in place; returns the low kW words.
static Poly reduce(const Field &f, Poly &p)
{
    // clear bits 19937 + 8k .. 19937 + 8k + 7 from the top down
    const int K = (kWP * 64 - kDeg + 7) / 8;
    for (int k = K - 1; k >= 0; --k)
    {
        const int64_t pos = kDeg + 8 * (int64_t)k;
        const int64_t q = pos >> 6, sh = pos & 63;
        if (q >= kWP)
            continue;
        uint64_t v = p[q] >> sh;
        if (sh > 56 && q + 1 < kWP)
            v |= p[q + 1] << (64 - sh);
        const int t = (int)(v & 0xff);
        if (!t)
            continue;
        const uint64_t *r = &f.red[((size_t)(k & 7) * 256 + f.inv_top[t]) * kWT];
        const int ws = k >> 3;
        for (int j = 0; j < kWT && ws + j < kWP; ++j)
            p[ws + j] ^= r[j];
    }
    return Poly(p.begin(), p.begin() + kW);
}

static Poly mulmod(const Field &f, const Poly &a, const Poly &b)
{
    // table of t * b for bytes t; 8 accumulators by byte position mod 8, word-aligned
    std::vector<uint64_t> tb((size_t)256 * (kW + 1), 0);
    for (int k = 0; k < kW; ++k)
        tb[(size_t)1 * (kW + 1) + k] = b[k];
    for (int t = 2; t < 256; ++t)
    {
        uint64_t *d = &tb[(size_t)t * (kW + 1)];
        if (t & 1)
        {
            const uint64_t *e = &tb[(size_t)(t - 1) * (kW + 1)];
            for (int k = 0; k <= kW; ++k)
                d[k] = e[k] ^ (k < kW ? b[k] : 0);
        }
        else
        {
            const uint64_t *h = &tb[(size_t)(t / 2) * (kW + 1)];
            d[0] = h[0] << 1;
            for (int k = 1; k <= kW; ++k)
                d[k] = (h[k] << 1) | (h[k - 1] >> 63);
        }
    }
    std::vector<uint64_t> acc((size_t)8 * (kWP + 2), 0);
    for (int j = 0; j < kW * 8; ++j)
    {
        const int t = (int)((a[j >> 3] >> (8 * (j & 7))) & 0xff);
        if (!t)
            continue;
        uint64_t *d = &acc[(size_t)(j & 7) * (kWP + 2) + (j >> 3)];
        const uint64_t *e = &tb[(size_t)t * (kW + 1)];
        for (int k = 0; k <= kW; ++k)
            d[k] ^= e[k];
    }
    Poly p(kWP, 0);
    for (int c = 0; c < 8; ++c)
    {
        const uint64_t *s = &acc[(size_t)c * (kWP + 2)];
        const int sh = 8 * c;
        for (int k = 0; k < kWP; ++k)
        {
            p[k] ^= s[k] << sh;
            if (sh && k)
                p[k] ^= s[k - 1] >> (64 - sh);
        }
    }
    return reduce(f, p);
}

static Poly sqrmod(const Field &f, const Poly &a)
{
    Poly p(kWP, 0);
    for (int k = 0; k < kW; ++k)
    {
        uint64_t lo = 0, hi = 0;
        for (int u = 0; u < 4; ++u)
        {
            lo |= (uint64_t)f.spread[(a[k] >> (8 * u)) & 0xff] << (16 * u);
            hi |= (uint64_t)f.spread[(a[k] >> (8 * u + 32)) & 0xff] << (16 * u);
        }
        p[2 * k] = lo;
        p[2 * k + 1] = hi;
    }
    return reduce(f, p);
}

static Poly mulx(const Field &f, const Poly &a)
{
    Poly r(kW, 0);
    r[0] = a[0] << 1;
    for (int k = 1; k < kW; ++k)
        r[k] = (a[k] << 1) | (a[k - 1] >> 63);
    if (bit(r.data(), kDeg))
        for (int k = 0; k < kW; ++k)
            r[k] ^= f.phi[k];
    return r;
}

// x^J mod phi
static Poly xpow(const Field &f, uint64_t J)
{
    Poly r(kW, 0);
    r[0] = 1;
    int top = 63;
    while (top > 0 && !((J >> top) & 1))
        --top;
    for (int b = top; b >= 0; --b)
    {
        r = sqrmod(f, r);
        if ((J >> b) & 1)
            r = mulx(f, r);
    }
    return r;
}

// The coefficients of x^(k * L) mod phi for k = k0 .. k1 - 1, as 624 32-bit words each (bit i of the
// polynomial at word i / 32, bit i % 32), computed on up to 16 host threads.
static void jump_polys(uint64_t L, int k0, int k1, std::vector<uint32_t> &out)
{
    const Field &f = field();
    const int n = k1 - k0;
    out.assign((size_t)n * 624, 0);
    if (n <= 0)
        return;
    const Poly step = xpow(f, L);
    const int nt = std::max(1, std::min<int>(16, std::min<int>(n, (int)std::thread::hardware_concurrency())));
    auto work = [&](int t) {
        const int a = k0 + (int)((int64_t)n * t / nt), b = k0 + (int)((int64_t)n * (t + 1) / nt);
        if (a >= b)
            return;
        Poly p = xpow(f, L * (uint64_t)a);
        for (int k = a; k < b; ++k)
        {
            if (k > a)
                p = mulmod(f, p, step);
            uint32_t *d = &out[(size_t)(k - k0) * 624];
            for (int w = 0; w < kW; ++w)
            {
                d[2 * w] = (uint32_t)p[w];
                d[2 * w + 1] = (uint32_t)(p[w] >> 32);
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t)
        th.emplace_back(work, t);
    work(0);
    for (auto &x : th)
        x.join();
}

// Device tables of jump polynomials per segment length (x^(k L) mod phi for k = 1 .. K), grown on
// demand and kept until the process exits.
struct JumpTable
{
    uint32_t *dev = nullptr;
    int k_have = 0, k_cap = 0;
};
static std::mutex g_mu;
static std::map<std::pair<int, uint64_t>, JumpTable> g_tables;

}  // namespace mtj

bool mt_field_ready()
{
    return mtj::field().ok;
}

// Device pointer to the jump polynomials x^(k L) mod phi, k = 1 .. K (624 words each, row k - 1).
gbo_status mt_jump_table(uint64_t L, int K, const uint32_t **out)
{
    using namespace mtj;
    if (!field().ok)
        return GBO_ERR_UNSUPPORTED;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mu);
    JumpTable &t = g_tables[{dev, L}];
    if (t.k_have < K)
    {
        std::vector<uint32_t> host;
        jump_polys(L, t.k_have + 1, K + 1, host);
        if (t.k_cap < K)
        {
            const int cap = std::max(K, 2 * t.k_cap);
            uint32_t *nd = nullptr;
            if (cudaMalloc(&nd, (size_t)cap * 624 * sizeof(uint32_t)) != cudaSuccess)
                return GBO_ERR_OUT_OF_MEMORY;
            if (t.dev)
            {
                cudaMemcpy(nd, t.dev, (size_t)t.k_have * 624 * sizeof(uint32_t), cudaMemcpyDeviceToDevice);
                cudaFree(t.dev);
            }
            t.dev = nd;
            t.k_cap = cap;
        }
        if (cudaMemcpy(t.dev + (size_t)t.k_have * 624, host.data(), host.size() * sizeof(uint32_t),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return GBO_ERR_CUDA;
        t.k_have = K;
    }
    *out = t.dev;
    return GBO_OK;
}

}  // namespace gbo

// Host-side discard(J) of an mt19937 state (no device work): the state J outputs later. `pos` is the
// index of the next word of `mt` (1..624; 624: the block is used up), as std::mt19937 keeps it.
extern "C" gbo_status gbo_mt19937_discard(uint32_t *mt, uint32_t *pos, uint64_t J)
{
    using namespace gbo::mtj;
    if (!mt || !pos || *pos < 1 || *pos > 624)
        return GBO_ERR_INVALID_ARGUMENT;
    const uint32_t p0 = *pos;
    if (J < 2 * 624)
    {
        // step directly
        std::vector<uint32_t> x(mt, mt + 624);
        uint32_t p = p0;
        for (uint64_t j = 0; j < J; ++j)
        {
            if (p == 624)
            {
                for (int t = 0; t < 624; ++t)
                    x[t] = twist_host(x[t], x[(t + 1) % 624], x[(t + 397) % 624]);
                p = 0;
            }
            ++p;
        }
        std::copy(x.begin(), x.end(), mt);
        *pos = p;
        return GBO_OK;
    }
    const Field &f = field();
    if (!f.ok)
        return GBO_ERR_UNSUPPORTED;
    // raw sequence u_t = x_{T0 - 1 + t} (T0: the next output), from the block
    const int NU = kDeg + 624;
    std::vector<uint32_t> u(NU + 624);
    std::vector<uint32_t> blk(mt, mt + 624);
    int64_t n = 0;
    for (uint32_t t = p0 - 1; t < 624 && n < (int64_t)u.size(); ++t)
        u[n++] = blk[t];
    while (n < (int64_t)u.size())
    {
        std::vector<uint32_t> nx(624);
        for (int t = 0; t < 624; ++t)
            nx[t] = twist_host(blk[t], t + 1 < 624 ? blk[t + 1] : nx[0], t + 397 < 624 ? blk[t + 397] : nx[t - 227]);
        blk = nx;
        for (int t = 0; t < 624 && n < (int64_t)u.size(); ++t)
            u[n++] = blk[t];
    }
    const Poly p = xpow(f, J);
    std::vector<uint32_t> s(624, 0);
    for (int i = 0; i < kDeg; ++i)
        if (bit(p.data(), i))
            for (int w = 0; w < 624; ++w)
                s[w] ^= u[i + w];
    // the window at T0 - 1 + J: its word 0 is only meaningful in its top bit; the next output is word 1
    std::copy(s.begin(), s.end(), mt);
    *pos = 1;
    return GBO_OK;
}
