// gen.cu -- seeded synthetic workloads generated on the device, and the
// order-independent fingerprint of a join output.
//
// Every value is a pure function of (seed, stream, row), so the host-side
// generator used by the tests produces the same integers.  The shared key
// stream K(i) = splitmix64_mix(key_seed + (i + 1) * golden_gamma) is a
// bijection of i (Steele, Lea, Flood 2014), so K(0..n-1) are unique keys and
// K(n + j) never collides with them -- that is how non-matching probe keys
// are made.  Zipf ranks use rejection-inversion (Hoermann & Derflinger
// 1996).  Seeded permutations use cycle-walking over an invertible mix on
// the next power of two.
#include "internal.h"

#include <cmath>

namespace phjg
{
namespace
{
constexpr uint64_t kGamma = 0x9e3779b97f4a7c15ull;
constexpr uint64_t kStreamMul = 0xd1b54a32d192ed03ull;

__host__ __device__ __forceinline__ uint64_t mix_splitmix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint64_t mix_murmur(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__host__ __device__ __forceinline__ uint64_t rand64(uint64_t seed, uint64_t stream, uint64_t i)
{
    return mix_splitmix((seed ^ (stream * kStreamMul)) + (i + 1) * kGamma);
}

__host__ __device__ __forceinline__ uint64_t key_of(uint64_t key_seed, uint64_t i)
{
    return rand64(key_seed, 0, i);
}

// uniform integer in [0, n), n <= 2^32
__host__ __device__ __forceinline__ uint64_t uniform_below(uint64_t r, uint64_t n)
{
    return ((r >> 32) * n) >> 32;
}

struct Perm
{
    uint64_t n, mask, a1, c1, a2, c2;
    uint32_t s;
};

Perm make_perm(uint64_t n, uint64_t seed)
{
    uint32_t k = 1;
    while (k < 63 && (1ull << k) < n)
        ++k;
    Perm p;
    p.n = n;
    p.mask = (1ull << k) - 1;
    p.a1 = rand64(seed, 48, 0) | 1ull;
    p.c1 = rand64(seed, 49, 0);
    p.a2 = rand64(seed, 50, 0) | 1ull;
    p.c2 = rand64(seed, 51, 0);
    p.s = (k + 1) / 2;
    return p;
}

__host__ __device__ __forceinline__ uint64_t perm_step(const Perm & p, uint64_t x)
{
    x = (x * p.a1 + p.c1) & p.mask;
    x ^= x >> p.s;
    x = (x * p.a2 + p.c2) & p.mask;
    x ^= x >> p.s;
    x = (x * p.a1 + p.c2) & p.mask;
    return x;
}

// Cycle-walking: the cycle through i < n always returns below n.
__host__ __device__ __forceinline__ uint64_t perm_apply(const Perm & p, uint64_t i)
{
    uint64_t y = perm_step(p, i);
    while (y >= p.n)
        y = perm_step(p, y);
    return y;
}

struct Payloads
{
    void * col[kMaxCols];
    uint8_t width[kMaxCols];
    uint32_t n;
};

__device__ __forceinline__ void write_payloads(const Payloads & p, uint64_t seed, uint64_t i)
{
    for (uint32_t c = 0; c < p.n; ++c)
    {
        const uint64_t lo = rand64(seed, 16 + c, i);
        switch (p.width[c])
        {
            case 1: static_cast<uint8_t *>(p.col[c])[i] = (uint8_t)lo; break;
            case 2: static_cast<uint16_t *>(p.col[c])[i] = (uint16_t)lo; break;
            case 4: static_cast<uint32_t *>(p.col[c])[i] = (uint32_t)lo; break;
            case 8: static_cast<uint64_t *>(p.col[c])[i] = lo; break;
            default:
            {
                const uint64_t hi = rand64(seed, 32 + c, i);
                static_cast<ulonglong2 *>(p.col[c])[i] = make_ulonglong2(lo, hi);
                break;
            }
        }
    }
}

struct Zipf
{
    double s, h_x1, h_n, s_const;
    uint64_t n;
};

__host__ __device__ __forceinline__ double zhelper1(double x)
{
    return fabs(x) > 1e-8 ? log1p(x) / x : 1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x));
}
__host__ __device__ __forceinline__ double zhelper2(double x)
{
    return fabs(x) > 1e-8 ? expm1(x) / x : 1.0 + x * 0.5 * (1.0 + x * (1.0 / 3.0) * (1.0 + 0.25 * x));
}
__host__ __device__ __forceinline__ double zh_integral(double s, double x)
{
    const double lx = log(x);
    return zhelper2((1.0 - s) * lx) * lx;
}
__host__ __device__ __forceinline__ double zh(double s, double x)
{
    return exp(-s * log(x));
}
__host__ __device__ __forceinline__ double zh_integral_inv(double s, double x)
{
    double t = x * (1.0 - s);
    if (t < -1.0)
        t = -1.0;
    return exp(zhelper1(t) * x);
}

Zipf make_zipf(uint64_t n, double s)
{
    Zipf z;
    z.s = s;
    z.n = n;
    z.h_x1 = zh_integral(s, 1.5) - 1.0;
    z.h_n = zh_integral(s, (double)n + 0.5);
    z.s_const = 2.0 - zh_integral_inv(s, zh_integral(s, 2.5) - zh(s, 2.0));
    return z;
}

__device__ __forceinline__ uint64_t zipf_rank(const Zipf & z, uint64_t seed, uint64_t i)
{
    uint64_t k = 1;
    for (uint32_t attempt = 0; attempt < 64; ++attempt)
    {
        const double u01 = (double)(rand64(seed, 4, i * 64 + attempt) >> 11) * (1.0 / 9007199254740992.0);
        const double u = z.h_n + u01 * (z.h_x1 - z.h_n);
        const double x = zh_integral_inv(z.s, u);
        double kd = floor(x + 0.5);
        if (kd < 1.0)
            kd = 1.0;
        else if (kd > (double)z.n)
            kd = (double)z.n;
        k = (uint64_t)kd;
        if (kd - x <= z.s_const || u >= zh_integral(z.s, kd + 0.5) - zh(z.s, kd))
            return k;
    }
    return k;
}

__global__ void k_gen_rows(uint32_t kind, uint64_t rows, uint64_t seed, uint64_t key_seed, uint64_t domain, uint32_t match_permille, const __grid_constant__ Perm perm,
                           const __grid_constant__ Zipf zipf, uint64_t * __restrict__ keys, const __grid_constant__ Payloads pay)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (uint64_t)gridDim.x * blockDim.x)
    {
        uint64_t k = 0;
        switch (kind)
        {
            case 0: k = key_of(key_seed, i); break;
            case 1: k = perm_apply(perm, i) + 1; break;
            case 3: k = uniform_below(rand64(seed, 1, i), domain) + 1; break;
            case 4:
                k = uniform_below(rand64(seed, 2, i), 1000) < match_permille ? key_of(key_seed, uniform_below(rand64(seed, 3, i), domain))
                                                                             : key_of(key_seed, domain + i);
                break;
            case 5: k = key_of(key_seed, perm_apply(perm, zipf_rank(zipf, seed, i) - 1)); break;
            default: break;
        }
        keys[i] = k;
        write_payloads(pay, seed, i);
    }
}

// Multi-match build (kind 2): multiplicity of distinct key d is 1 plus the
// number of consecutive successes of p = 3/4, capped at 16 (mean ~3.96).
__global__ void k_gen_mult(uint64_t n_distinct, uint64_t seed, uint32_t * __restrict__ mult)
{
    for (uint64_t d = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_distinct; d += (uint64_t)gridDim.x * blockDim.x)
    {
        uint32_t m = 1;
        for (uint32_t j = 0; j < 15; ++j)
        {
            if (uniform_below(rand64(seed, 52, d * 16 + j), 4) == 0)
                break;
            ++m;
        }
        mult[d] = m;
    }
}

__global__ void k_gen_distinct_count(const uint32_t * __restrict__ cum, uint64_t n_distinct, uint64_t rows, unsigned long long * __restrict__ used)
{
    for (uint64_t d = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_distinct; d += (uint64_t)gridDim.x * blockDim.x)
        if (cum[d] < rows && cum[d + 1] >= rows)
            *used = d + 1;
}

__global__ void k_gen_multi_rows(uint64_t rows, uint64_t seed, uint64_t key_seed, const uint32_t * __restrict__ cum, uint64_t used, Perm perm,
                                 uint64_t * __restrict__ keys, Payloads pay)
{
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < rows; j += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint64_t e = perm_apply(perm, j);
        uint64_t lo = 0, hi = used; // cum[lo] <= e < cum[hi]
        while (hi - lo > 1)
        {
            const uint64_t mid = (lo + hi) >> 1;
            if (cum[mid] <= e)
                lo = mid;
            else
                hi = mid;
        }
        keys[j] = key_of(key_seed, lo);
        write_payloads(pay, seed, j);
    }
}

// ---- fingerprint -----------------------------------------------------------------

constexpr uint64_t kFpSeedA = 0x243f6a8885a308d3ull;
constexpr uint64_t kFpSeedB = 0x13198a2e03707344ull;

struct FpCols
{
    const uint64_t * keys;
    const void * left[kMaxCols];
    uint8_t lw[kMaxCols];
    uint32_t nl;
    const void * right[kMaxCols];
    uint8_t rw[kMaxCols];
    uint32_t nr;
};

__device__ __forceinline__ void fp_word(uint64_t & a, uint64_t & b, uint64_t w)
{
    a = mix_splitmix(a ^ w);
    b = mix_murmur(b + w * kGamma);
}

__device__ __forceinline__ void fp_value(uint64_t & a, uint64_t & b, const void * col, uint32_t w, uint64_t i)
{
    switch (w)
    {
        case 1: fp_word(a, b, static_cast<const uint8_t *>(col)[i]); break;
        case 2: fp_word(a, b, static_cast<const uint16_t *>(col)[i]); break;
        case 4: fp_word(a, b, static_cast<const uint32_t *>(col)[i]); break;
        case 8: fp_word(a, b, static_cast<const uint64_t *>(col)[i]); break;
        default:
        {
            const ulonglong2 v = static_cast<const ulonglong2 *>(col)[i];
            fp_word(a, b, v.x);
            fp_word(a, b, v.y);
            break;
        }
    }
}

__global__ void k_fingerprint(const __grid_constant__ FpCols f, uint64_t rows, unsigned long long * __restrict__ sums)
{
    uint64_t sa = 0, sb = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (uint64_t)gridDim.x * blockDim.x)
    {
        uint64_t a = kFpSeedA, b = kFpSeedB;
        fp_word(a, b, f.keys[i]);
        for (uint32_t c = 0; c < f.nl; ++c)
            fp_value(a, b, f.left[c], f.lw[c], i);
        for (uint32_t c = 0; c < f.nr; ++c)
            fp_value(a, b, f.right[c], f.rw[c], i);
        sa += a;
        sb += b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        sa += __shfl_xor_sync(0xffffffffu, sa, o);
        sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicAdd(&sums[0], (unsigned long long)sa);
        atomicAdd(&sums[1], (unsigned long long)sb);
    }
}

Payloads payloads_of(const phj_table & t)
{
    Payloads p{};
    p.n = t.schema.n_payloads;
    for (uint32_t c = 0; c < p.n; ++c)
    {
        p.col[c] = t.cols[c];
        p.width[c] = (uint8_t)payload_width(t.schema.types[c]);
    }
    return p;
}
} // namespace

uint64_t generate_rows(phj_ctx * ctx, const phj_gen_spec & spec, phj_table & t)
{
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(spec.rows, 256), (uint64_t)ctx->num_sms * 16));
    const Payloads pay = payloads_of(t);
    if (spec.kind == 2)
    {
        Scratch s(ctx);
        const uint64_t cap = spec.domain ? std::min<uint64_t>(spec.domain, spec.rows) : spec.rows;
        uint32_t * mult = s.get<uint32_t>(cap + 1);
        uint32_t * cum = s.get<uint32_t>(cap + 1);
        unsigned long long * used = s.get<unsigned long long>(1);
        PHJ_CUDA(cudaMemsetAsync(used, 0, sizeof(unsigned long long), ctx->stream));
        k_gen_mult<<<grid, 256, 0, ctx->stream>>>(cap, spec.seed, mult);
        PHJ_LAUNCHED(ctx, "gen_mult");
        scan_u32(ctx, s, mult, cum, cap);
        k_gen_distinct_count<<<grid, 256, 0, ctx->stream>>>(cum, cap, spec.rows, used);
        PHJ_LAUNCHED(ctx, "gen_distinct");
        unsigned long long n_used = 0;
        PHJ_CUDA(cudaMemcpyAsync(&n_used, used, sizeof(n_used), cudaMemcpyDeviceToHost, ctx->stream));
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
        if (n_used == 0) // the capped distinct keys cannot fill `rows`: use them all, rows shrink
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "multi-match generator: domain too small for the requested rows");
        const Perm perm = make_perm(spec.rows, spec.seed ^ 0x5bd1e9955bd1e995ull);
        k_gen_multi_rows<<<grid, 256, 0, ctx->stream>>>(spec.rows, spec.seed, spec.key_seed, cum, n_used, perm, t.keys, pay);
        PHJ_LAUNCHED(ctx, "gen_multi_rows");
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
        return n_used;
    }
    Perm perm{};
    Zipf zipf{};
    if (spec.kind == 1)
        perm = make_perm(spec.rows, spec.seed);
    if (spec.kind == 5)
    {
        perm = make_perm(spec.domain, spec.seed ^ 0x2545f4914f6cdd1dull);
        zipf = make_zipf(spec.domain, spec.theta);
    }
    k_gen_rows<<<grid, 256, 0, ctx->stream>>>(spec.kind, spec.rows, spec.seed, spec.key_seed, spec.domain, spec.match_permille, perm, zipf, t.keys,
                                             pay);
    PHJ_LAUNCHED(ctx, "gen_rows");
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    return spec.kind == 0 ? spec.rows : 0;
}

void fingerprint(phj_ctx * ctx, const phj_output & out, uint64_t fp[3])
{
    Scratch s(ctx);
    unsigned long long * sums = s.get<unsigned long long>(2);
    PHJ_CUDA(cudaMemsetAsync(sums, 0, 2 * sizeof(unsigned long long), ctx->stream));
    FpCols f{};
    f.keys = out.keys;
    f.nl = out.left.n_payloads;
    f.nr = out.right.n_payloads;
    for (uint32_t c = 0; c < f.nl; ++c)
    {
        f.left[c] = out.lcol[c];
        f.lw[c] = (uint8_t)payload_width(out.left.types[c]);
    }
    for (uint32_t c = 0; c < f.nr; ++c)
    {
        f.right[c] = out.rcol[c];
        f.rw[c] = (uint8_t)payload_width(out.right.types[c]);
    }
    if (out.rows)
    {
        const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(out.rows, 256), (uint64_t)ctx->num_sms * 8));
        k_fingerprint<<<grid, 256, 0, ctx->stream>>>(f, out.rows, sums);
        PHJ_LAUNCHED(ctx, "fingerprint");
    }
    unsigned long long h[2] = {0, 0};
    PHJ_CUDA(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    fp[0] = out.rows;
    fp[1] = h[0];
    fp[2] = h[1];
}

} // namespace phjg
