// probe.cu -- probe with output projection (probeOneBlock, src/JoinOps.h:236-272;
// probeOneBlockCHJ, src/JoinOps.h:381-429; ProbeMaterialiser::gatherFromProbeBlock,
// src/JoinOps.h:77-125).
//
// A persistent kernel walks the probe rows in chunks of 2048 (8 rounds of
// 256 rows per CTA).  Per row: hash the key, locate the leaf table (or CHJ
// sub-table) from the top hash bits, look the key up, and count the matches
// (1, or the next-chain length when some build key repeats).  Each warp
// scans its counts with shuffles; one shared-memory combine and one global
// atomic per chunk place the chunk's output rows, warp-major and
// round-major, so consecutive lanes write consecutive output rows.  The
// projection then runs column by column -- key column (the probe key, as
// the reference emits it), build payloads gathered through the RowRefCell,
// probe payloads -- with each column's eight loads issued before its eight
// stores.  This is the reference's "expand chains into flat
// (probe_idx, build_ref) arrays, then gather column-major", with the flat
// arrays held in registers.
#include "internal.h"

namespace phjg
{
namespace
{
constexpr int kPNT = 256;
constexpr int kPRPT = 8;
constexpr int kPWarps = kPNT / 32;
constexpr uint32_t kChunk = kPNT * kPRPT;

enum ProbeMode
{
    kLeafUniform = 0, // PHJ: every leaf table has 2^uniform_log2cap cells at leaf << log2cap
    kLeafMeta = 1,    // PHJ: leaf tables located through the LeafMeta directory
    kChj = 2          // CHJ: 256 sub-tables through LeafMeta; refs are (input block, row)
};

struct OutCols
{
    uint64_t * keys;
    void * left[kMaxCols];
    void * right[kMaxCols];
};

// Build row (index into the build payload columns) of a RowRefCell.
template <int kMode>
__device__ __forceinline__ uint32_t build_row_of(uint64_t ref, const ProbeArgs & a)
{
    if (kMode == kChj)
    {
        const uint32_t b = ref_block(ref);
        const uint64_t base = a.uniform_block_rows ? (uint64_t)b * a.uniform_block_rows : __ldg(a.block_off + b);
        return (uint32_t)(base + ref_row(ref));
    }
    return ref_row(ref); // PHJ: {block 0 = the partitioned build rows, row}
}

__device__ __noinline__ uint32_t chain_length(uint32_t brow, const ProbeArgs & a, int chj)
{
    uint32_t c = 1;
    uint64_t r = __ldg(a.next + brow);
    while (ref_valid(r))
    {
        ++c;
        r = __ldg(a.next + (chj ? build_row_of<kChj>(r, a) : build_row_of<kLeafMeta>(r, a)));
    }
    return c;
}

template <class T>
__device__ __forceinline__ void put(void * dst, uint64_t i, T v)
{
    __stcs(static_cast<T *>(dst) + i, v);
}

// One full output row (slow path for rows of duplicate-key chains).
__device__ __forceinline__ void emit_row(const ProbeArgs & a, const OutCols & o, uint32_t brow, uint64_t key, uint64_t prow, uint64_t pos)
{
    __stcs(o.keys + pos, key);
    for (uint32_t c = 0; c < a.build.n; ++c)
        switch (a.build.width[c])
        {
            case 1: put<uint8_t>(o.left[c], pos, __ldg(static_cast<const uint8_t *>(a.build.col[c]) + brow)); break;
            case 2: put<uint16_t>(o.left[c], pos, __ldg(static_cast<const uint16_t *>(a.build.col[c]) + brow)); break;
            case 4: put<uint32_t>(o.left[c], pos, __ldg(static_cast<const uint32_t *>(a.build.col[c]) + brow)); break;
            case 8: put<uint64_t>(o.left[c], pos, __ldg(static_cast<const uint64_t *>(a.build.col[c]) + brow)); break;
            default: put<uint4>(o.left[c], pos, __ldg(static_cast<const uint4 *>(a.build.col[c]) + brow)); break;
        }
    for (uint32_t c = 0; c < a.probe.n; ++c)
        switch (a.probe.width[c])
        {
            case 1: put<uint8_t>(o.right[c], pos, static_cast<const uint8_t *>(a.probe.col[c])[prow]); break;
            case 2: put<uint16_t>(o.right[c], pos, static_cast<const uint16_t *>(a.probe.col[c])[prow]); break;
            case 4: put<uint32_t>(o.right[c], pos, static_cast<const uint32_t *>(a.probe.col[c])[prow]); break;
            case 8: put<uint64_t>(o.right[c], pos, static_cast<const uint64_t *>(a.probe.col[c])[prow]); break;
            default: put<uint4>(o.right[c], pos, static_cast<const uint4 *>(a.probe.col[c])[prow]); break;
        }
}

// Column pass over the chunk's match list: thread i writes output row
// base + i, so every store of a column is coalesced; the loads are gathers
// through the list (build rows) or nearly sequential (probe rows).
template <class T, bool kBuild>
__device__ __forceinline__ void column_pass(const void * src_v, void * dst_v, const uint32_t * idx, uint32_t n, uint64_t base)
{
    const T * src = static_cast<const T *>(src_v);
    T * dst = static_cast<T *>(dst_v) + base;
    uint32_t i = threadIdx.x;
    for (; i + 3 * kPNT < n; i += 4 * kPNT)
    {
        T v0, v1, v2, v3;
        if (kBuild)
        {
            v0 = __ldg(src + idx[i]);
            v1 = __ldg(src + idx[i + kPNT]);
            v2 = __ldg(src + idx[i + 2 * kPNT]);
            v3 = __ldg(src + idx[i + 3 * kPNT]);
        }
        else
        {
            v0 = __ldcs(src + idx[i]);
            v1 = __ldcs(src + idx[i + kPNT]);
            v2 = __ldcs(src + idx[i + 2 * kPNT]);
            v3 = __ldcs(src + idx[i + 3 * kPNT]);
        }
        __stcs(dst + i, v0);
        __stcs(dst + i + kPNT, v1);
        __stcs(dst + i + 2 * kPNT, v2);
        __stcs(dst + i + 3 * kPNT, v3);
    }
    for (; i < n; i += kPNT)
        __stcs(dst + i, kBuild ? __ldg(src + idx[i]) : __ldcs(src + idx[i]));
}

template <bool kBuild>
__device__ __forceinline__ void columns_pass(const Cols & src, void * const * dst, const uint32_t * idx, uint32_t n, uint64_t base)
{
#pragma unroll 1
    for (uint32_t c = 0; c < src.n; ++c)
        switch (src.width[c])
        {
            case 1: column_pass<uint8_t, kBuild>(src.col[c], dst[c], idx, n, base); break;
            case 2: column_pass<uint16_t, kBuild>(src.col[c], dst[c], idx, n, base); break;
            case 4: column_pass<uint32_t, kBuild>(src.col[c], dst[c], idx, n, base); break;
            case 8: column_pass<uint64_t, kBuild>(src.col[c], dst[c], idx, n, base); break;
            default: column_pass<uint4, kBuild>(src.col[c], dst[c], idx, n, base); break;
        }
}

// Matches of one chunk, compacted in shared memory (the flat
// (probe_idx, build_ref) arrays of probeOneBlock, plus the key).
template <bool kDup>
struct MatchList
{
    static constexpr uint32_t kCap = kDup ? 2 * kChunk : kChunk;
    uint64_t key[kCap];
    uint32_t brow[kCap];
    uint32_t prow[kCap];
};

// kDup: some build key repeats, so rows may have several matches (chain
// walks); without it every matched row yields exactly one output row and the
// kernel carries no chain code at all.
// Chunk status words for the decoupled look-back that places each chunk's
// output rows: flag in the top two bits, row count below.
constexpr unsigned long long kFlagAgg = 1ull << 62;  // the chunk's own total
constexpr unsigned long long kFlagIncl = 2ull << 62; // total of chunks 0..c
constexpr unsigned long long kValMask = (1ull << 62) - 1;

// Publishes chunk c's total and finds the rows of all earlier chunks.  Only
// thread 0 of the CTA calls it.  Chunks are taken in increasing order by
// co-resident CTAs (cooperative launch), so the lowest unfinished chunk
// never waits; every wait is still bounded.
__device__ __forceinline__ unsigned long long chunk_base(unsigned long long * status, uint64_t c, uint32_t total, int * err)
{
    if (c == 0)
    {
        atomicExch(status, kFlagIncl | total);
        return 0;
    }
    atomicExch(status + c, kFlagAgg | total);
    unsigned long long acc = 0;
    uint64_t j = c - 1;
    for (uint32_t spins = 0;;)
    {
        const unsigned long long st = *reinterpret_cast<volatile unsigned long long *>(status + j);
        if (st & kFlagIncl)
        {
            acc += st & kValMask;
            break;
        }
        if (st & kFlagAgg)
        {
            acc += st & kValMask;
            --j; // chunk 0 always holds an inclusive value
            continue;
        }
        if (++spins >= kWaitLimit)
        {
            atomicExch(err, 2);
            return ~0ull;
        }
    }
    atomicExch(status + c, kFlagIncl | (acc + total));
    return acc;
}

template <int kMode, bool kDup>
__global__ void __launch_bounds__(kPNT) k_probe(const __grid_constant__ ProbeArgs a, const __grid_constant__ OutCols o,
                                                unsigned long long * __restrict__ status, uint64_t out_cap, int count_only,
                                                int * __restrict__ err)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    MatchList<kDup> & ml = *reinterpret_cast<MatchList<kDup> *>(smem_raw);
    __shared__ uint32_t warp_tot[kPWarps];
    __shared__ uint32_t chunk_total;
    __shared__ unsigned long long sh_base;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t n_chunks = ceil_div(a.probe_rows, kChunk);
    const uint32_t shift = 64u - a.leaf_bits;
    const uint32_t ulog = kMode == kLeafUniform ? (uint32_t)a.uniform_log2cap : 0u;
    const uint64_t ucap = 1ull << ulog;
    for (uint64_t chunk = blockIdx.x; chunk < n_chunks; chunk += gridDim.x)
    {
        const uint64_t row0 = chunk * kChunk + warp * 32 + lane; // + k * kPNT
        uint64_t key[kPRPT];
        uint32_t brow[kPRPT];
        uint32_t valid = 0, dup = 0;
        // ---- lookups: eight independent key -> table chains per thread
#pragma unroll
        for (int k = 0; k < kPRPT; ++k)
        {
            const uint64_t row = row0 + (uint64_t)k * kPNT;
            key[k] = 0;
            brow[k] = 0;
            if (row < a.probe_rows)
            {
                key[k] = __ldcs(a.probe.keys + row);
                const uint64_t h = int_hash64(key[k]);
                const uint32_t leaf = (uint32_t)(h >> shift);
                uint64_t head;
                if (kMode == kLeafUniform)
                {
                    head = table_find(a.cells + ((uint64_t)leaf << ulog), ucap, h, key[k]);
                    dup |= (kDup ? 1u : 0u) << k;
                }
                else
                {
                    const ulonglong2 mv = __ldg(reinterpret_cast<const ulonglong2 *>(a.meta + leaf));
                    const uint32_t log2cap = (uint32_t)(mv.y >> 32) & 0xffu;
                    const uint32_t has = (uint32_t)(mv.y >> 40) & 0xffu;
                    if (kDup)
                        dup |= (uint32_t)((mv.y >> 48) & 1u) << k;
                    head = has ? table_find(a.cells + mv.x, 1ull << log2cap, h, key[k]) : INVALID_REF;
                }
                if (ref_valid(head))
                {
                    valid |= 1u << k;
                    brow[k] = build_row_of<kMode>(head, a);
                }
            }
        }
        dup &= valid;
        // ---- counts and placement: warp scans, one combine per chunk
        uint32_t excl[kPRPT];
        uint32_t running = 0;
#pragma unroll
        for (int k = 0; k < kPRPT; ++k)
        {
            uint32_t c = valid >> k & 1u;
            if (kDup && (dup >> k & 1u))
                c = chain_length(brow[k], a, kMode == kChj);
            uint32_t x = c;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= (uint32_t)d)
                    x += y;
            }
            excl[k] = running + x - c;
            running += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0)
            warp_tot[warp] = running;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            uint32_t acc = 0;
            for (int w = 0; w < kPWarps; ++w)
            {
                const uint32_t t = warp_tot[w];
                warp_tot[w] = acc;
                acc += t;
            }
            chunk_total = acc;
            sh_base = chunk_base(status, chunk, acc, err);
        }
        __syncthreads();
        if (count_only || sh_base == ~0ull)
            continue;
        const uint64_t base = sh_base;
        const uint32_t total = chunk_total;
        const uint32_t wbase = warp_tot[warp];
        // ---- compact the matches into the chunk's list
#pragma unroll
        for (int k = 0; k < kPRPT; ++k)
        {
            if (!(valid >> k & 1u))
                continue;
            uint32_t i = wbase + excl[k];
            const uint32_t prow = (uint32_t)(row0 + (uint64_t)k * kPNT);
            uint32_t b = brow[k];
            for (;;)
            {
                if (i < MatchList<kDup>::kCap)
                {
                    ml.key[i] = key[k];
                    ml.brow[i] = b;
                    ml.prow[i] = prow;
                }
                else if (base + i < out_cap) // past the list: written directly
                    emit_row(a, o, b, key[k], prow, base + i);
                if (!kDup || !(dup >> k & 1u))
                    break;
                const uint64_t r = __ldg(a.next + b);
                if (!ref_valid(r))
                    break;
                b = build_row_of<kMode>(r, a);
                ++i;
            }
        }
        __syncthreads();
        // ---- column passes: key, build payloads, probe payloads
        uint32_t n = min(total, MatchList<kDup>::kCap);
        if (base + n > out_cap)
            n = base >= out_cap ? 0u : (uint32_t)(out_cap - base);
        for (uint32_t i = threadIdx.x; i < n; i += kPNT)
            __stcs(o.keys + base + i, ml.key[i]);
        columns_pass<true>(a.build, o.left, ml.brow, n, base);
        columns_pass<false>(a.probe, o.right, ml.prow, n, base);
        __syncthreads(); // the list is rewritten by the next chunk
    }
}
} // namespace

uint64_t probe_join(phj_ctx * ctx, Scratch & s, const ProbeArgs & a, phj_output * out, bool count_only, const char * name)
{
    const uint64_t n_chunks = ceil_div(a.probe_rows, kChunk);
    unsigned long long * status = s.get<unsigned long long>(n_chunks + 1);
    PHJ_CUDA(cudaMemsetAsync(status, 0, (n_chunks + 1) * sizeof(unsigned long long), ctx->stream));
    OutCols o{};
    uint64_t cap = 0;
    if (out)
    {
        o.keys = out->keys;
        for (uint32_t c = 0; c < out->left.n_payloads; ++c)
            o.left[c] = out->lcol[c];
        for (uint32_t c = 0; c < out->right.n_payloads; ++c)
            o.right[c] = out->rcol[c];
        cap = out->cap;
    }
    const int mode = a.chj ? kChj : (a.uniform_log2cap >= 0 ? kLeafUniform : kLeafMeta);
    auto kern = a.any_dup ? (mode == kChj ? k_probe<kChj, true> : mode == kLeafUniform ? k_probe<kLeafUniform, true> : k_probe<kLeafMeta, true>)
                          : (mode == kChj ? k_probe<kChj, false> : mode == kLeafUniform ? k_probe<kLeafUniform, false> : k_probe<kLeafMeta, false>);
    const size_t smem = a.any_dup ? sizeof(MatchList<true>) : sizeof(MatchList<false>);
    PHJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPNT, smem));
    // Every CTA must be resident (the look-back waits on other CTAs'
    // chunks): a cooperative launch of at most one wave.
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(std::max<uint64_t>(n_chunks, 1), (uint64_t)ctx->num_sms * (uint64_t)std::max(per_sm, 1)));
    uint64_t probe_row_bytes = 8, build_row_bytes = 0;
    for (uint32_t c = 0; c < a.probe.n; ++c)
        probe_row_bytes += a.probe.width[c];
    for (uint32_t c = 0; c < a.build.n; ++c)
        build_row_bytes += a.build.width[c];
    {
        KTimer kt(ctx, name, a.probe_rows, count_only ? a.probe_rows * 8 : a.probe_rows * probe_row_bytes);
        int co = count_only ? 1 : 0;
        ProbeArgs aa = a;
        void * args[] = {&aa, &o, &status, &cap, &co, &ctx->d_err};
        PHJ_CUDA(cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kPNT), args, smem, ctx->stream));
        PHJ_LAUNCHED(ctx, name);
    }
    unsigned long long last = 0;
    if (n_chunks)
        PHJ_CUDA(cudaMemcpyAsync(&last, status + n_chunks - 1, sizeof(last), cudaMemcpyDeviceToHost, ctx->stream));
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint64_t rows = last & kValMask;
    // Algorithmic bytes of the timed launch, now that the output size is
    // known: probe rows read + output rows (key + build + probe payloads).
    if (!count_only && !ctx->records.empty())
        ctx->records.back().bytes += rows * (8 + build_row_bytes + (probe_row_bytes - 8));
    return rows;
}

} // namespace phjg
