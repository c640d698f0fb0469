// scan.cu -- exclusive prefix sum over u32 arrays (histogram matrices, leaf
// sizes, table capacities).  Reduce-then-scan: each 512-thread block owns
// 4096 consecutive values; block sums are scanned recursively.  512 threads
// (14K registers) fit on an SM beside a first-pass scatter CTA, so the build
// side's scans do not wait for the probe side's pass to retire.
#include "internal.h"

namespace phjg
{
namespace
{
constexpr int kScanNT = 512;
constexpr int kScanPerThread = 8;
constexpr uint64_t kScanTile = (uint64_t)kScanNT * kScanPerThread;

__global__ void __launch_bounds__(kScanNT) k_scan_reduce(const uint32_t * __restrict__ in, uint64_t m, uint32_t * __restrict__ sums)
{
    __shared__ uint32_t ws[kScanNT / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k)
    {
        const uint64_t i = base + (uint64_t)k * kScanNT + threadIdx.x;
        if (i < m)
            acc += in[i];
    }
    uint32_t total;
    (void)block_excl_scan<kScanNT>(acc, ws, &total);
    if (threadIdx.x == 0)
        sums[blockIdx.x] = total;
}

// Scans one tile of 4096 values; thread t owns 8 consecutive values.  Adds
// `carry[blockIdx.x]` (when given) and writes total to out[m] from the last
// tile.  In-place (in == out) is allowed.
__global__ void __launch_bounds__(kScanNT) k_scan_tile(const uint32_t * in, uint64_t m, const uint32_t * __restrict__ carry, uint32_t * out)
{
    __shared__ uint32_t ws[kScanNT / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanPerThread;
    uint32_t v[kScanPerThread];
    uint32_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k)
    {
        const uint64_t i = base + k;
        v[k] = i < m ? in[i] : 0u;
        acc += v[k];
    }
    uint32_t total;
    uint32_t run = block_excl_scan<kScanNT>(acc, ws, &total);
    const uint32_t c = carry ? carry[blockIdx.x] : 0u;
    run += c;
#pragma unroll
    for (int k = 0; k < kScanPerThread; ++k)
    {
        const uint64_t i = base + k;
        if (i < m)
            out[i] = run;
        run += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        out[m] = c + total;
}
} // namespace

uint64_t scan_u32_carry(uint64_t m)
{
    const uint64_t tiles = ceil_div(m, kScanTile);
    return tiles <= 1 ? 0 : tiles + 1 + scan_u32_carry(tiles);
}

void scan_u32_into(phj_ctx * ctx, const uint32_t * in, uint32_t * out, uint64_t m, uint32_t * carry)
{
    if (m == 0)
    {
        PHJ_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), ctx->stream));
        return;
    }
    const uint64_t tiles = ceil_div(m, kScanTile);
    if (tiles == 1)
    {
        k_scan_tile<<<1, kScanNT, 0, ctx->stream>>>(in, m, nullptr, out);
        PHJ_LAUNCHED(ctx, "scan_tile");
        return;
    }
    uint32_t * sums = carry;
    k_scan_reduce<<<(unsigned)tiles, kScanNT, 0, ctx->stream>>>(in, m, sums);
    PHJ_LAUNCHED(ctx, "scan_reduce");
    scan_u32_into(ctx, sums, sums, tiles, carry + tiles + 1);
    k_scan_tile<<<(unsigned)tiles, kScanNT, 0, ctx->stream>>>(in, m, sums, out);
    PHJ_LAUNCHED(ctx, "scan_tile");
}

void scan_u32(phj_ctx * ctx, Scratch & s, const uint32_t * in, uint32_t * out, uint64_t m)
{
    const uint64_t c = scan_u32_carry(m);
    scan_u32_into(ctx, in, out, m, c ? s.get<uint32_t>(c) : nullptr);
}
} // namespace phjg
