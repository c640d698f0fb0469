// partition.cu -- radix partitioning on the top bits of intHash64
// (src/RadixPartition.cpp: scatterBatch :316-393, radixShuffle :546-577,
// refineToLeaves :417-539).
//
// One physical pass splits every segment of the previous pass (rows that
// share their top c_prev hash bits, stored contiguously) into 2^b
// sub-buckets on the next b bits.  Three kernels per pass:
//   k_part_hist    per 4096-row tile: shared-memory histogram of the b-bit
//                  digit, one count per (segment, digit, tile) written
//                  digit-major;
//   scan_u32       device-wide exclusive scan over those counts, which yields
//                  every tile's first output row for every digit;
//   k_part_scatter re-reads the tile, ranks its rows by digit in shared
//                  memory, and for each column (key first, then payloads of
//                  1/2/4/8/16 bytes) stages the tile in digit order and writes
//                  each digit's run contiguously -- the column-first scatter
//                  of the reference, with the staging done in shared memory so
//                  stores coalesce.
// No atomics touch global memory; the output is deterministic.
#include "internal.h"

namespace phjg
{
namespace
{
constexpr int kNT = 512;
constexpr int kRPT = 8;
constexpr uint32_t kTile = kNT * kRPT; // rows per tile
constexpr uint32_t kMaxPassBits = 11;  // shared-memory digit histogram <= 2048 bins

struct PassGeom
{
    const uint32_t * seg_off;  // n_segs + 1: first row of each input segment
    const uint32_t * tile_pre; // n_segs + 1: first tile of each input segment
    uint32_t n_segs;
    uint32_t shift;            // digit = (hash >> shift) & mask
    uint32_t b;
};

struct TileRef
{
    uint32_t seg, k, nt, row0, row1, tile0;
};

__device__ __forceinline__ bool locate_tile(const PassGeom & g, uint32_t t, TileRef & r)
{
    const uint32_t total = g.tile_pre[g.n_segs];
    if (t >= total)
        return false;
    // Largest s with tile_pre[s] <= t; segments without tiles are skipped
    // because then tile_pre[s] == tile_pre[s+1].
    uint32_t lo = 0, hi = g.n_segs; // invariant: tile_pre[lo] <= t < tile_pre[hi]
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (g.tile_pre[mid] <= t)
            lo = mid;
        else
            hi = mid;
    }
    r.seg = lo;
    r.tile0 = g.tile_pre[lo];
    r.k = t - r.tile0;
    r.nt = g.tile_pre[lo + 1] - r.tile0;
    const uint32_t s0 = g.seg_off[lo], s1 = g.seg_off[lo + 1];
    r.row0 = s0 + r.k * kTile;
    r.row1 = min(r.row0 + kTile, s1);
    return true;
}


__global__ void __launch_bounds__(kNT) k_part_hist(const uint64_t * __restrict__ keys, PassGeom g, uint32_t * __restrict__ counts)
{
    extern __shared__ uint32_t bins[];
    TileRef tr;
    if (!locate_tile(g, blockIdx.x, tr))
        return;
    const uint32_t nb = 1u << g.b, mask = nb - 1;
    for (uint32_t i = threadIdx.x; i < nb; i += kNT)
        bins[i] = 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRPT; ++j)
    {
        const uint32_t row = tr.row0 + j * kNT + threadIdx.x;
        if (row < tr.row1)
            atomicAdd(&bins[(uint32_t)(int_hash64(__ldcs(keys + row)) >> g.shift) & mask], 1u);
    }
    __syncthreads();
    const uint64_t base = (uint64_t)tr.tile0 * nb;
    for (uint32_t d = threadIdx.x; d < nb; d += kNT)
        counts[base + (uint64_t)d * tr.nt + tr.k] = bins[d];
}

// Exclusive scan of nb bins in shared memory by kNT threads.
// Exclusive scan of the tile's digit counts by the first warp alone (the
// caller's next barrier publishes excl).
__device__ __forceinline__ void smem_bins_scan(const uint32_t * bins, uint32_t * excl, uint32_t nb)
{
    if (threadIdx.x >= 32)
        return;
    const uint32_t lane = threadIdx.x;
    const uint32_t per = (nb + 31) / 32;
    const uint32_t b0 = lane * per;
    uint32_t local = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < nb)
            local += bins[b0 + i];
    uint32_t x = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= (uint32_t)d)
            x += y;
    }
    uint32_t run = x - local;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < nb)
        {
            excl[b0 + i] = run;
            run += bins[b0 + i];
        }
}

// One column of the tile: stage it in digit order in shared memory, then
// each thread stores its kRPT staged elements to their precomputed rows.
template <class T>
__device__ __forceinline__ void scatter_column(const T * __restrict__ src, T * __restrict__ dst, T * stage, const uint32_t (&lp)[kRPT],
                                               const uint32_t (&dest)[kRPT], const TileRef & tr)
{
#pragma unroll
    for (int j = 0; j < kRPT; ++j)
    {
        const uint32_t row = tr.row0 + j * kNT + threadIdx.x;
        if (row < tr.row1)
            stage[lp[j]] = __ldcs(src + row);
    }
    __syncthreads();
    const uint32_t cnt = tr.row1 - tr.row0;
#pragma unroll
    for (int j = 0; j < kRPT; ++j)
    {
        const uint32_t pos = j * kNT + threadIdx.x;
        if (pos < cnt)
            dst[dest[j]] = stage[pos];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kNT, 2) k_part_scatter(const __grid_constant__ Cols in, const __grid_constant__ Cols out,
                                                         const __grid_constant__ PassGeom g, const uint32_t * __restrict__ offs, uint32_t maxw)
{
    extern __shared__ __align__(16) uint8_t smem[];
    TileRef tr;
    if (!locate_tile(g, blockIdx.x, tr))
        return;
    const uint32_t nb = 1u << g.b, mask = nb - 1;
    uint8_t * stage = smem;
    uint16_t * sorted_d = reinterpret_cast<uint16_t *>(smem + (size_t)kTile * maxw);
    uint32_t * bins = reinterpret_cast<uint32_t *>(sorted_d + kTile);
    uint32_t * excl = bins + nb;
    uint32_t * gbase = excl + nb;

    for (uint32_t i = threadIdx.x; i < nb; i += kNT)
        bins[i] = 0;
    __syncthreads();

    // digit and rank within the digit (shared atomics return the rank)
    uint64_t key[kRPT];
    uint32_t lp[kRPT]; // digit, then position in the tile's digit order
    uint32_t rank[kRPT];
#pragma unroll
    for (int j = 0; j < kRPT; ++j)
    {
        const uint32_t row = tr.row0 + j * kNT + threadIdx.x;
        lp[j] = 0xFFFFFFFFu;
        key[j] = 0;
        rank[j] = 0;
        if (row < tr.row1)
        {
            key[j] = __ldcs(in.keys + row);
            lp[j] = (uint32_t)(int_hash64(key[j]) >> g.shift) & mask;
            rank[j] = atomicAdd(&bins[lp[j]], 1u);
        }
    }
    __syncthreads();
    smem_bins_scan(bins, excl, nb);
    const uint64_t ebase = (uint64_t)tr.tile0 * nb;
    for (uint32_t d = threadIdx.x; d < nb; d += kNT)
        gbase[d] = offs[ebase + (uint64_t)d * tr.nt + tr.k];
    __syncthreads();

    uint64_t * stage64 = reinterpret_cast<uint64_t *>(stage);
#pragma unroll
    for (int j = 0; j < kRPT; ++j)
        if (lp[j] != 0xFFFFFFFFu)
        {
            const uint32_t d = lp[j];
            lp[j] = excl[d] + rank[j];
            stage64[lp[j]] = key[j];
            sorted_d[lp[j]] = (uint16_t)d;
        }
        else
            lp[j] = 0;
    __syncthreads();
    // Each thread owns tile positions j*kNT + tid: their output rows.
    const uint32_t cnt = tr.row1 - tr.row0;
    uint32_t dest[kRPT];
#pragma unroll
    for (int j = 0; j < kRPT; ++j)
    {
        const uint32_t pos = j * kNT + threadIdx.x;
        dest[j] = 0;
        if (pos < cnt)
        {
            const uint32_t d = sorted_d[pos];
            dest[j] = gbase[d] + (pos - excl[d]);
            out.keys[dest[j]] = stage64[pos];
        }
    }
    __syncthreads();

    for (uint32_t c = 0; c < in.n; ++c)
    {
        switch (in.width[c])
        {
            case 1: scatter_column<uint8_t>((const uint8_t *)in.col[c], (uint8_t *)out.col[c], stage, lp, dest, tr); break;
            case 2: scatter_column<uint16_t>((const uint16_t *)in.col[c], (uint16_t *)out.col[c], (uint16_t *)stage, lp, dest, tr); break;
            case 4: scatter_column<uint32_t>((const uint32_t *)in.col[c], (uint32_t *)out.col[c], (uint32_t *)stage, lp, dest, tr); break;
            case 8: scatter_column<uint64_t>((const uint64_t *)in.col[c], (uint64_t *)out.col[c], (uint64_t *)stage, lp, dest, tr); break;
            default: scatter_column<uint4>((const uint4 *)in.col[c], (uint4 *)out.col[c], (uint4 *)stage, lp, dest, tr); break;
        }
    }
}

// ---------------------------------------------------------------------------
// First pass (one input segment): each CTA owns a contiguous range of whole
// tiles, so the histogram is per CTA (digit-major, 2^b x G counts) and the
// scatter keeps one running output cursor per digit in shared memory.  Tiles
// arrive by bulk asynchronous copies (cp.async.bulk through the TMA engine)
// into two shared-memory buffers: tile t+1 streams in while tile t is ranked
// and written out, with no registers spent on prefetching.
// ---------------------------------------------------------------------------
constexpr int kP1NT = 512;

struct P1Geom
{
    uint64_t n;
    uint32_t tiles_per_cta;
    uint32_t tile_rows;
    uint32_t shift, b;
};

// H CTAs share one scatter CTA's row range (counts are zeroed first and
// summed with global atomics), so the histogram keeps more loads in flight
// than the scatter's one-CTA-per-SM grid would.
// With `mark` set (PHJ/BEP probe batches) the same pass also flags the
// leaves the rows hash to: a shared-memory bitmap per CTA (a bit is read
// before it is set), ORed into the global bitmap at the end.
__global__ void __launch_bounds__(kP1NT) k_p1_hist(const uint64_t * __restrict__ keys, P1Geom g, uint32_t H, uint32_t G,
                                                   uint32_t * __restrict__ counts, LeafMark mark)
{
    extern __shared__ uint32_t bins[];
    const uint32_t nb = 1u << g.b, mask = nb - 1;
    uint32_t * bm = bins + nb;
    for (uint32_t i = threadIdx.x; i < nb; i += kP1NT)
        bins[i] = 0;
    if (mark.bits)
        for (uint32_t i = threadIdx.x; i < mark.words; i += kP1NT)
            bm[i] = 0;
    __syncthreads();
    const uint32_t gi = blockIdx.x / H, q = blockIdx.x % H;
    const uint64_t span = (uint64_t)g.tiles_per_cta * g.tile_rows;
    const uint64_t g0 = (uint64_t)gi * span;
    const uint64_t g1 = min(g.n, g0 + span);
    const uint64_t part = ceil_div(span, (uint64_t)H * 8 * kP1NT) * 8 * kP1NT;
    const uint64_t r0 = g0 + q * part;
    const uint64_t r1 = min(g1, r0 + part);
    for (uint64_t base = r0; base < r1; base += 8 * kP1NT)
    {
        uint64_t k[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
        {
            const uint64_t row = base + j * kP1NT + threadIdx.x;
            k[j] = row < r1 ? __ldcs(keys + row) : 0;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (base + j * kP1NT + threadIdx.x < r1)
            {
                const uint64_t h = int_hash64(k[j]);
                atomicAdd(&bins[(uint32_t)(h >> g.shift) & mask], 1u);
                if (mark.bits)
                {
                    const uint32_t L = (uint32_t)(h >> mark.shift);
                    if (!(bm[L >> 5] & (1u << (L & 31))))
                        atomicOr(&bm[L >> 5], 1u << (L & 31));
                }
            }
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d < nb; d += kP1NT)
        if (bins[d])
            atomicAdd(&counts[(uint64_t)d * G + gi], bins[d]);
    if (mark.bits)
        for (uint32_t w = threadIdx.x; w < mark.words; w += kP1NT)
        {
            const uint32_t v = bm[w];
            if (v && (__ldcg(mark.bits + w) & v) != v)
                atomicOr(mark.bits + w, v);
        }
}

struct P1Smem
{
    uint32_t buf_bytes;              // one tile of every column
    uint32_t col_off[kMaxCols + 1];  // byte offset of each payload column in a buffer (keys at 0)
};

template <class T, int RPT>
__device__ __forceinline__ void p1_write_column(const uint8_t * buf, T * __restrict__ dst, const uint32_t (&src)[RPT], const uint32_t (&dest)[RPT],
                                                uint32_t cnt)
{
    const T * b = reinterpret_cast<const T *>(buf);
#pragma unroll
    for (int j = 0; j < RPT; ++j)
        if (j * kP1NT + threadIdx.x < cnt)
            dst[dest[j]] = b[src[j]];
}

// kMinB 2 holds the kernel to 64 registers a thread (a launch bound of two
// CTAs, though shared memory admits one): half of the register file stays
// free, so the build side's later pass (scan, histogram, scatter) runs
// beside the probe side's first pass instead of waiting for it to retire.
// A pass that runs alone takes kMinB 1 (72 registers).
template <int RPT, int kMinB>
__global__ void __launch_bounds__(kP1NT, kMinB) k_p1_scatter(const __grid_constant__ Cols in, const __grid_constant__ Cols out, P1Geom g,
                                                         const __grid_constant__ P1Smem sm, uint32_t stages, const uint32_t * __restrict__ offs,
                                                         int use_tma, int * __restrict__ err)
{
    constexpr uint32_t kT = kP1NT * RPT;
    constexpr uint32_t kMaxStages = 4;
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ __align__(8) uint64_t bar[kMaxStages];
    uint16_t * inv = reinterpret_cast<uint16_t *>(smem + (size_t)stages * sm.buf_bytes);
    uint16_t * dsort = inv + kT;
    const uint32_t nb = 1u << g.b, mask = nb - 1;
    uint32_t * bins = reinterpret_cast<uint32_t *>(dsort + kT);
    uint32_t * excl = bins + nb;
    // running output cursors per digit, two arrays in turn: the scan of tile
    // t writes tile t+1's cursors while tile t's are still being read, so no
    // barrier is needed to advance them
    uint32_t * cur = excl + nb;
    uint32_t * nxt = cur + nb;

    const uint64_t n_tiles = ceil_div(g.n, kT);
    const uint64_t t_begin = (uint64_t)blockIdx.x * g.tiles_per_cta;
    const uint64_t t_end = min(n_tiles, t_begin + g.tiles_per_cta);
    if (t_begin >= t_end)
        return;
    for (uint32_t d = threadIdx.x; d < nb; d += kP1NT)
    {
        cur[d] = offs[(uint64_t)d * gridDim.x + blockIdx.x];
        bins[d] = 0;
    }
    if (threadIdx.x == 0)
    {
        for (uint32_t i = 0; i < stages; ++i)
            mbar_init(&bar[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    // A tile is fetched by bulk copy when every column slice is a whole
    // number of 16-byte units (always, except a short last tile).
    auto tile_rows = [&](uint64_t t) -> uint32_t { const uint64_t r = g.n - t * kT; return r < kT ? (uint32_t)r : kT; };
    auto tma_ok = [&](uint64_t t) -> bool {
        if (!use_tma)
            return false;
        const uint32_t r = tile_rows(t);
        if ((r * 8u) & 15u)
            return false;
        for (uint32_t c = 0; c < in.n; ++c)
            if ((r * in.width[c]) & 15u)
                return false;
        return true;
    };
    auto buffer = [&](uint32_t i) -> uint8_t * { return smem + (size_t)i * sm.buf_bytes; };
    auto issue = [&](uint64_t t, uint32_t bi) {
        const uint32_t r = tile_rows(t);
        uint32_t bytes = r * 8u;
        for (uint32_t c = 0; c < in.n; ++c)
            bytes += r * in.width[c];
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[bi], bytes);
        bulk_copy_g2s(buffer(bi), in.keys + t * kT, r * 8u, &bar[bi]);
        for (uint32_t c = 0; c < in.n; ++c)
            bulk_copy_g2s(buffer(bi) + sm.col_off[c], static_cast<const uint8_t *>(in.col[c]) + t * kT * in.width[c], r * in.width[c], &bar[bi]);
    };
    uint32_t parity = 0; // bit i: phase of bar[i] to wait for
    if (threadIdx.x == 0)
        for (uint32_t i = 0; i + 1 < stages && t_begin + i < t_end; ++i)
            if (tma_ok(t_begin + i))
                issue(t_begin + i, i);

    uint32_t bi = 0;
    for (uint64_t t = t_begin; t < t_end; ++t, bi = (bi + 1 == stages) ? 0 : bi + 1)
    {
        const uint32_t cnt = tile_rows(t);
        uint8_t * buf = buffer(bi);
        if (tma_ok(t))
        {
            const bool ok = mbar_wait(&bar[bi], (parity >> bi) & 1u, err, 1);
            if (!__syncthreads_and(ok))
                break;
            parity ^= 1u << bi;
        }
        else
        {
            uint64_t * bk = reinterpret_cast<uint64_t *>(buf);
            for (uint32_t i = threadIdx.x; i < cnt; i += kP1NT)
                bk[i] = in.keys[t * kT + i];
            for (uint32_t c = 0; c < in.n; ++c)
                for (uint32_t i = threadIdx.x; i < cnt; i += kP1NT)
                    copy_elem(buf + sm.col_off[c], i, in.col[c], t * kT + i, in.width[c]);
            __syncthreads();
        }
        // keep stages-1 tiles in flight: refill the buffer the previous tile
        // used (its readers finished at the barrier ending that iteration)
        const uint32_t nbi = (bi + stages - 1) % stages;
        if (threadIdx.x == 0 && t + stages - 1 < t_end && tma_ok(t + stages - 1))
            issue(t + stages - 1, nbi);
        // (bins were zeroed by the last tile's scan)

        const uint64_t * bk = reinterpret_cast<const uint64_t *>(buf);
        uint32_t dg[RPT], rk[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j)
        {
            const uint32_t i = j * kP1NT + threadIdx.x;
            dg[j] = 0xFFFFu;
            rk[j] = 0;
            if (i < cnt)
            {
                dg[j] = (uint32_t)(int_hash64(bk[i]) >> g.shift) & mask;
                rk[j] = atomicAdd(&bins[dg[j]], 1u);
            }
        }
        __syncthreads();
        // exclusive scan of the digit counts by the first warp alone (one
        // barrier instead of the block scan's three), which also advances
        // the cursors for the next tile and zeroes the counts
        if (threadIdx.x < 32)
        {
            const uint32_t lane = threadIdx.x;
            const uint32_t per = (nb + 31) / 32;
            const uint32_t b0 = lane * per;
            uint32_t local = 0;
            for (uint32_t i = 0; i < per; ++i)
                if (b0 + i < nb)
                    local += bins[b0 + i];
            uint32_t x = local;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= (uint32_t)d)
                    x += y;
            }
            uint32_t run = x - local;
            for (uint32_t i = 0; i < per; ++i)
                if (b0 + i < nb)
                {
                    const uint32_t c = bins[b0 + i];
                    excl[b0 + i] = run;
                    run += c;
                    nxt[b0 + i] = cur[b0 + i] + c;
                    bins[b0 + i] = 0;
                }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < RPT; ++j)
            if (dg[j] != 0xFFFFu)
            {
                const uint32_t pos = excl[dg[j]] + rk[j];
                inv[pos] = (uint16_t)(j * kP1NT + threadIdx.x);
                dsort[pos] = (uint16_t)dg[j];
            }
        __syncthreads();
        uint32_t src[RPT], dest[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j)
        {
            const uint32_t pos = j * kP1NT + threadIdx.x;
            src[j] = 0;
            dest[j] = 0;
            if (pos < cnt)
            {
                const uint32_t d = dsort[pos];
                src[j] = inv[pos];
                dest[j] = cur[d] + (pos - excl[d]);
            }
        }
        p1_write_column<uint64_t, RPT>(buf, out.keys, src, dest, cnt);
        for (uint32_t c = 0; c < in.n; ++c)
        {
            const uint8_t * cb = buf + sm.col_off[c];
            switch (in.width[c])
            {
                case 1: p1_write_column<uint8_t, RPT>(cb, (uint8_t *)out.col[c], src, dest, cnt); break;
                case 2: p1_write_column<uint16_t, RPT>(cb, (uint16_t *)out.col[c], src, dest, cnt); break;
                case 4: p1_write_column<uint32_t, RPT>(cb, (uint32_t *)out.col[c], src, dest, cnt); break;
                case 8: p1_write_column<uint64_t, RPT>(cb, (uint64_t *)out.col[c], src, dest, cnt); break;
                default: p1_write_column<uint4, RPT>(cb, (uint4 *)out.col[c], src, dest, cnt); break;
            }
        }
        // No barrier here: the next tile's first barrier (after its wait)
        // comes before this buffer is refilled, before the counts are
        // ranked into again and before `cur` is overwritten as the next
        // tile's `nxt`.
        uint32_t * t_swap = cur;
        cur = nxt;
        nxt = t_swap;
    }
    // Bulk copies still in flight (only after a timeout) must land before
    // the CTA's shared memory is released.
    if (threadIdx.x == 0 && *err)
        for (uint32_t i = 0; i < stages; ++i)
            (void)mbar_wait(&bar[i], (parity >> i) & 1u, err, 1);
}

__global__ void k_p1_bucket_offsets(const uint32_t * __restrict__ offs, uint32_t nb, uint32_t G, uint32_t n, uint32_t * __restrict__ out_off)
{
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < nb)
        out_off[d] = offs[(uint64_t)d * G];
    else if (d == nb)
        out_off[d] = n;
}

__global__ void k_tiles_per_seg(const uint32_t * __restrict__ seg_off, uint32_t n_segs, uint32_t * __restrict__ nt)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n_segs)
        nt[s] = (seg_off[s + 1] - seg_off[s] + kTile - 1) / kTile;
}

__global__ void k_init_single_seg(uint32_t * seg_off, uint32_t n)
{
    seg_off[0] = 0;
    seg_off[1] = n;
}

// Output bucket offsets of a pass: bucket (s, d) starts at the scanned
// offset of its first tile; a segment without tiles is empty and all its
// buckets start where it starts.
__global__ void k_bucket_offsets(PassGeom g, const uint32_t * __restrict__ offs, uint32_t n, uint32_t * __restrict__ out_off)
{
    const uint32_t nb = 1u << g.b;
    const uint64_t nbuckets = (uint64_t)g.n_segs * nb;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > nbuckets)
        return;
    if (i == nbuckets)
    {
        out_off[i] = n;
        return;
    }
    const uint32_t s = (uint32_t)(i >> g.b), d = (uint32_t)(i & (nb - 1));
    const uint32_t t0 = g.tile_pre[s], nt = g.tile_pre[s + 1] - t0;
    out_off[i] = nt ? offs[(uint64_t)t0 * nb + (uint64_t)d * nt] : g.seg_off[s];
}
} // namespace

// The first physical pass: histogram per CTA range, scan, bulk-copy fed
// scatter with running cursors, then the bucket offsets.
static void first_pass(phj_ctx * ctx, Scratch & s, const Cols & src, const Cols & dst, uint64_t n, uint32_t b, uint32_t * bucket_off,
                       const char * phase)
{
    const uint32_t nb = 1u << b;
    uint64_t row_bytes = 8;
    P1Smem sm{};
    for (uint32_t c = 0; c < src.n; ++c)
        row_bytes += src.width[c];
    // Tile rows (4096/2048/1024) and ring depth (2-4): the pair that keeps
    // the most bytes in flight ((stages - 1) tiles) within shared memory.
    // (Measured: two resident CTAs of half the tile, same bytes in flight,
    // run the 16M x 256M first passes 40% slower: the fixed per-tile work
    // doubles per row, and the build side's pass no longer fits beside the
    // probe side's on the SMs.)
    int rpt = 0;
    uint32_t stages = 0;
    uint64_t best = 0;
    for (int r = 8; r >= 2; r /= 2)
        for (uint32_t st = 2; st <= 4; ++st)
        {
            // context options (an autotuner's choice) pin the tile or the depth
            if ((ctx->p1_tile_rows && (uint32_t)(kP1NT * r) != ctx->p1_tile_rows) || (ctx->p1_stages && st != ctx->p1_stages))
                continue;
            const uint64_t kT = (uint64_t)kP1NT * r;
            uint64_t buf = kT * 8;
            for (uint32_t c = 0; c < src.n; ++c)
                buf += kT * src.width[c];
            buf = (buf + 127) & ~127ull;
            const uint64_t need_rs = st * buf + 4 * kT + 4ull * nb * 4;
            if (need_rs + 2048 > ctx->smem_optin)
                continue;
            const uint64_t inflight = (st - 1) * buf;
            if (inflight > best)
            {
                best = inflight;
                rpt = r;
                stages = st;
            }
        }
    if (rpt == 0)
        throw Error(PHJ_ERR_UNSUPPORTED, "row too wide for the shared-memory tile of the partition pass");
    const uint32_t kT = kP1NT * (uint32_t)rpt;
    uint32_t off = kT * 8;
    for (uint32_t c = 0; c < src.n; ++c)
    {
        sm.col_off[c] = off;
        off += kT * src.width[c];
    }
    sm.buf_bytes = (off + 127) & ~127u;
    const size_t need = (size_t)stages * sm.buf_bytes + 4ull * kT + 4ull * nb * 4;
    int per_sm = 1;
    auto kern = ctx->p1_beside ? (rpt == 8 ? k_p1_scatter<8, 2> : rpt == 4 ? k_p1_scatter<4, 2> : k_p1_scatter<2, 2>)
                               : (rpt == 8 ? k_p1_scatter<8, 1> : rpt == 4 ? k_p1_scatter<4, 1> : k_p1_scatter<2, 1>);
    PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kP1NT, need));
    const uint64_t n_tiles = ceil_div(n, kT);
    const uint32_t G = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(n_tiles, (uint64_t)ctx->num_sms * std::max(per_sm, 1)));
    P1Geom g{n, (uint32_t)ceil_div(n_tiles, G), kT, 64u - b, b};
    bool aligned = (reinterpret_cast<uintptr_t>(src.keys) & 15u) == 0;
    for (uint32_t c = 0; c < src.n; ++c)
        aligned = aligned && (reinterpret_cast<uintptr_t>(src.col[c]) & 15u) == 0;
    uint32_t * counts = s.get<uint32_t>((uint64_t)nb * G + 1);
    PHJ_CUDA(cudaMemsetAsync(counts, 0, ((uint64_t)nb * G + 1) * sizeof(uint32_t), ctx->stream));
    {
        const uint32_t H = 4;
        KTimer kt(ctx, "part_hist", n, n * 8);
        // a pending leaf mark (PHJ/BEP) rides on this pass, once
        const LeafMark mark = ctx->leaf_mark;
        ctx->leaf_mark = LeafMark{};
        k_p1_hist<<<G * H, kP1NT, (size_t)(nb + (mark.bits ? mark.words : 0)) * sizeof(uint32_t), ctx->stream>>>(src.keys, g, H, G, counts, mark);
        PHJ_LAUNCHED(ctx, "p1_hist");
    }
    scan_u32(ctx, s, counts, counts, (uint64_t)nb * G);
    {
        KTimer kt(ctx, phase, n, 2 * n * row_bytes);
        kern<<<G, kP1NT, need, ctx->stream>>>(src, dst, g, sm, stages, counts, aligned ? 1 : 0, ctx->d_err);
        PHJ_LAUNCHED(ctx, "p1_scatter");
    }
    k_p1_bucket_offsets<<<(unsigned)ceil_div(nb + 1, 256), 256, 0, ctx->stream>>>(counts, nb, G, (uint32_t)n, bucket_off);
    PHJ_LAUNCHED(ctx, "p1_offsets");
}

void radix_partition(phj_ctx * ctx, Scratch & s, const Cols & in, uint64_t n, const std::vector<uint32_t> & pass_bits, const Cols & out,
                     const Cols & tmp, uint32_t * leaf_off, const char * phase)
{
    uint32_t total_bits = 0;
    std::vector<uint32_t> phys; // physical passes
    for (uint32_t b : pass_bits)
    {
        total_bits += b;
    }
    // Physical passes: the leaf ranges depend only on the total bits, so the
    // logical passes are re-split into the fewest passes of at most
    // kMaxPassBits bits (3 x 6 bits run as 9 + 9); an odd bit goes to the
    // later pass (17 bits: 8 + 9), whose tiles each serve one first-pass
    // bucket, so the first pass keeps more rows per bucket and tile
    // (32M x 128M multi-match: 8.6 -> 8.3 ms).
    {
        const uint32_t pieces = (total_bits + kMaxPassBits - 1) / kMaxPassBits;
        for (uint32_t p = 0; p < pieces; ++p)
            phys.push_back(total_bits / pieces + (pieces - 1 - p < total_bits % pieces ? 1u : 0u));
    }
    if (total_bits == 0 || total_bits > 24)
        throw Error(PHJ_ERR_UNSUPPORTED, "device radix partitioning supports 1..24 total bits");
    if (n >= (1ull << 32))
        throw Error(PHJ_ERR_UNSUPPORTED, "device radix partitioning supports < 2^32 rows per side");
    const uint64_t n_leaves = 1ull << total_bits;
    if (n == 0)
    {
        PHJ_CUDA(cudaMemsetAsync(leaf_off, 0, (n_leaves + 1) * sizeof(uint32_t), ctx->stream));
        return;
    }
    const uint32_t maxw = max_width(in) < 8 ? 8 : max_width(in);

    // Segments of the first pass: the whole input.
    uint32_t * seg_off = s.get<uint32_t>(2);
    k_init_single_seg<<<1, 1, 0, ctx->stream>>>(seg_off, (uint32_t)n);
    PHJ_LAUNCHED(ctx, "part_init");
    uint32_t n_segs = 1, consumed = 0;
    const size_t np = phys.size();
    Cols src = in;
    for (size_t p = 0; p < np; ++p)
    {
        const uint32_t b = phys[p];
        const uint32_t nb = 1u << b;
        const Cols & dst = ((np - 1 - p) % 2 == 0) ? out : tmp;
        if (n_segs == 1)
        {
            // first pass: contiguous tile ranges per CTA, bulk-copy fed
            uint32_t * next_off = (p + 1 == np) ? leaf_off : s.get<uint32_t>((uint64_t)nb + 1);
            first_pass(ctx, s, src, dst, n, b, next_off, phase);
            seg_off = next_off;
            n_segs = nb;
            consumed += b;
            src = dst;
            continue;
        }
        // Tiles of each segment, then their prefix.
        uint32_t * nt = s.get<uint32_t>(n_segs + 1);
        k_tiles_per_seg<<<(unsigned)ceil_div(n_segs, 256), 256, 0, ctx->stream>>>(seg_off, n_segs, nt);
        PHJ_LAUNCHED(ctx, "part_tiles");
        uint32_t * tile_pre = s.get<uint32_t>(n_segs + 1);
        scan_u32(ctx, s, nt, tile_pre, n_segs);
        const uint64_t tiles_ub = ceil_div(n, kTile) + n_segs;
        const uint64_t entries_ub = tiles_ub * nb;
        // Entries past the real tile count stay unwritten; they only follow
        // the real ones in the scan, so they cannot disturb real offsets.
        uint32_t * counts = s.get<uint32_t>(entries_ub + 1);
        const PassGeom g{seg_off, tile_pre, n_segs, 64u - consumed - b, b};
        {
            KTimer kt(ctx, "part_hist", n, n * 8);
            k_part_hist<<<(unsigned)tiles_ub, kNT, nb * sizeof(uint32_t), ctx->stream>>>(src.keys, g, counts);
            PHJ_LAUNCHED(ctx, "part_hist");
        }
        scan_u32(ctx, s, counts, counts, entries_ub);
        {
            const size_t smem = (size_t)kTile * maxw + (size_t)kTile * sizeof(uint16_t) + 3ull * nb * sizeof(uint32_t) + 32 * sizeof(uint32_t);
            uint64_t row_bytes = 8;
            for (uint32_t c = 0; c < in.n; ++c)
                row_bytes += in.width[c];
            KTimer kt(ctx, phase, n, 2 * n * row_bytes);
            k_part_scatter<<<(unsigned)tiles_ub, kNT, smem, ctx->stream>>>(src, dst, g, counts, maxw);
            PHJ_LAUNCHED(ctx, "part_scatter");
        }
        const uint64_t nbuckets = (uint64_t)n_segs * nb;
        uint32_t * next_off = (p + 1 == np) ? leaf_off : s.get<uint32_t>(nbuckets + 1);
        k_bucket_offsets<<<(unsigned)ceil_div(nbuckets + 1, 256), 256, 0, ctx->stream>>>(g, counts, (uint32_t)n, next_off);
        PHJ_LAUNCHED(ctx, "part_offsets");
        seg_off = next_off;
        n_segs = (uint32_t)nbuckets;
        consumed += b;
        src = dst;
    }
}

void set_partition_smem_limits(int smem_optin)
{
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_scatter<8, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 1024));
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_scatter<4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 1024));
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_scatter<2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 1024));
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_scatter<8, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 1024));
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_scatter<4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 1024));
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_scatter<2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_optin - 1024));
    PHJ_CUDA(cudaFuncSetAttribute(k_p1_hist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::min<size_t>(((1u << kMaxPassBits) + (1u << 20) / 32) * sizeof(uint32_t), (size_t)smem_optin - 1024)));
    // The scatter kernel stages a 4096-row tile of the widest column (<= 16
    // bytes) plus digit bins: up to ~96 KiB.
    const size_t need = (size_t)kTile * 16 + (size_t)kTile * sizeof(uint16_t) + 3ull * (1u << kMaxPassBits) * sizeof(uint32_t) + 128;
    PHJ_CUDA(cudaFuncSetAttribute(k_part_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(need, (size_t)smem_optin)));
}

} // namespace phjg
