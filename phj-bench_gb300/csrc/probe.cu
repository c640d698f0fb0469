// probe.cu -- probe with output projection (probeOneBlock, src/JoinOps.h:236-272;
// probeOneBlockCHJ, src/JoinOps.h:381-429; ProbeMaterialiser::gatherFromProbeBlock,
// src/JoinOps.h:77-125).
//
// A persistent kernel streams the probe rows in chunks of 2048 taken from
// a device work counter.  For each row it hashes the key, finds the leaf
// (or CHJ sub-table) from the top hash bits, looks the key up (head
// RowRefCell), and counts the matches by walking the next-chain when the
// table holds duplicate keys.  A block-wide scan per 256-row round places
// every match, one atomic per chunk reserves the chunk's output range, and
// the rows are written column-major: key column (the probe key, as the
// reference emits it), build payloads gathered through the RowRefCell, then
// probe payloads.  This is the reference's "expand chains into flat
// (probe_idx, build_ref) arrays, then gather" with the flat arrays kept in
// registers instead of memory.
#include "internal.h"

namespace phjg
{
namespace
{
constexpr int kPNT = 256;
constexpr int kPRPT = 8;
constexpr uint32_t kChunk = kPNT * kPRPT;

struct OutCols
{
    uint64_t * keys;
    void * left[kMaxCols];
    void * right[kMaxCols];
};

template <class T>
__device__ __forceinline__ void put_stream(void * dst, uint64_t i, T v)
{
    __stcs(static_cast<T *>(dst) + i, v);
}

__device__ __forceinline__ void copy_gather(void * dst, uint64_t di, const void * src, uint64_t si, uint32_t w)
{
    switch (w)
    {
        case 1: put_stream<uint8_t>(dst, di, __ldg(static_cast<const uint8_t *>(src) + si)); break;
        case 2: put_stream<uint16_t>(dst, di, __ldg(static_cast<const uint16_t *>(src) + si)); break;
        case 4: put_stream<uint32_t>(dst, di, __ldg(static_cast<const uint32_t *>(src) + si)); break;
        case 8: put_stream<uint64_t>(dst, di, __ldg(static_cast<const uint64_t *>(src) + si)); break;
        default: put_stream<uint4>(dst, di, __ldg(static_cast<const uint4 *>(src) + si)); break;
    }
}

__device__ __forceinline__ void copy_stream(void * dst, uint64_t di, const void * src, uint64_t si, uint32_t w)
{
    switch (w)
    {
        case 1: put_stream<uint8_t>(dst, di, __ldcs(static_cast<const uint8_t *>(src) + si)); break;
        case 2: put_stream<uint16_t>(dst, di, __ldcs(static_cast<const uint16_t *>(src) + si)); break;
        case 4: put_stream<uint32_t>(dst, di, __ldcs(static_cast<const uint32_t *>(src) + si)); break;
        case 8: put_stream<uint64_t>(dst, di, __ldcs(static_cast<const uint64_t *>(src) + si)); break;
        default: put_stream<uint4>(dst, di, __ldcs(static_cast<const uint4 *>(src) + si)); break;
    }
}

template <bool kCHJ>
__device__ __forceinline__ uint64_t build_row_of(uint64_t ref, uint32_t leaf_row_off, const ProbeArgs & a)
{
    if (kCHJ)
    {
        const uint32_t b = ref_block(ref);
        const uint64_t base = a.uniform_block_rows ? (uint64_t)b * a.uniform_block_rows : __ldg(a.block_off + b);
        return base + ref_row(ref);
    }
    return (uint64_t)leaf_row_off + ref_row(ref);
}

template <bool kCHJ>
__device__ __noinline__ uint32_t chain_length(uint64_t head, uint32_t roff, const ProbeArgs & a)
{
    uint32_t c = 1;
    uint64_t r = __ldg(a.next + build_row_of<kCHJ>(head, roff, a));
    while (ref_valid(r))
    {
        ++c;
        r = __ldg(a.next + build_row_of<kCHJ>(r, roff, a));
    }
    return c;
}

// One output row: key column (probe key), build payloads via the
// RowRefCell's row, probe payloads via the probe row.
__device__ __forceinline__ void emit_row(const ProbeArgs & a, const OutCols & o, uint64_t brow, uint64_t key, uint64_t prow, uint64_t pos)
{
    __stcs(o.keys + pos, key);
    for (uint32_t c = 0; c < a.build.n; ++c)
        copy_gather(o.left[c], pos, a.build.col[c], brow, a.build.width[c]);
    for (uint32_t c = 0; c < a.probe.n; ++c)
        copy_stream(o.right[c], pos, a.probe.col[c], prow, a.probe.width[c]);
}

template <bool kCHJ>
__device__ __noinline__ void emit_chain(const ProbeArgs & a, const OutCols & o, uint64_t head, uint32_t roff, uint64_t key, uint64_t prow,
                                        uint64_t pos, uint64_t out_cap)
{
    for (uint64_t r = head; ref_valid(r) && pos < out_cap; ++pos)
    {
        const uint64_t brow = build_row_of<kCHJ>(r, roff, a);
        emit_row(a, o, brow, key, prow, pos);
        r = __ldg(a.next + brow);
    }
}

template <bool kCHJ>
__global__ void __launch_bounds__(kPNT) k_probe(const __grid_constant__ ProbeArgs a, const __grid_constant__ OutCols o, unsigned long long * __restrict__ ctrs, uint64_t out_cap, int count_only)
{
    // ctrs[0]: next chunk, ctrs[1]: output rows reserved
    __shared__ uint32_t ws[kPNT / 32];
    __shared__ uint32_t round_tot[kPRPT];
    __shared__ unsigned long long sh_chunk, sh_base;
    const uint64_t n_chunks = ceil_div(a.probe_rows, kChunk);
    const uint32_t shift = 64u - a.leaf_bits;
    for (;;)
    {
        if (threadIdx.x == 0)
            sh_chunk = atomicAdd(&ctrs[0], 1ull);
        __syncthreads();
        const uint64_t chunk = sh_chunk;
        if (chunk >= n_chunks)
            break;
        const uint64_t row0 = chunk * kChunk;

        uint64_t key[kPRPT], head[kPRPT];
        uint32_t cnt[kPRPT], roff[kPRPT], excl[kPRPT];
        uint8_t dupf[kPRPT];
#pragma unroll
        for (int k = 0; k < kPRPT; ++k)
        {
            const uint64_t row = row0 + (uint64_t)k * kPNT + threadIdx.x;
            head[k] = INVALID_REF;
            key[k] = 0;
            roff[k] = 0;
            dupf[k] = 0;
            if (row < a.probe_rows)
            {
                key[k] = __ldcs(a.probe.keys + row);
                const uint64_t h = int_hash64(key[k]);
                const uint32_t leaf = (uint32_t)(h >> shift);
                const ulonglong2 mv = __ldg(reinterpret_cast<const ulonglong2 *>(a.meta + leaf));
                const uint64_t table_off = mv.x;
                const uint32_t row_off = (uint32_t)mv.y;
                const uint32_t log2cap = (uint32_t)(mv.y >> 32) & 0xffu;
                const uint32_t has = (uint32_t)(mv.y >> 40) & 0xffu;
                dupf[k] = (uint8_t)((mv.y >> 48) & 0xffu);
                roff[k] = row_off;
                if (has)
                    head[k] = table_find(a.cells + table_off, 1ull << log2cap, h, key[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < kPRPT; ++k)
            cnt[k] = !ref_valid(head[k]) ? 0u : (dupf[k] ? chain_length<kCHJ>(head[k], roff[k], a) : 1u);
#pragma unroll
        for (int k = 0; k < kPRPT; ++k)
        {
            uint32_t tot;
            excl[k] = block_excl_scan<kPNT>(cnt[k], ws, &tot);
            if (threadIdx.x == 0)
                round_tot[k] = tot;
        }
        if (threadIdx.x == 0)
        {
            uint64_t all = 0;
            for (int k = 0; k < kPRPT; ++k)
                all += round_tot[k];
            sh_base = atomicAdd(&ctrs[1], (unsigned long long)all);
        }
        __syncthreads();
        const uint64_t base = sh_base;
        uint64_t round_base = base;
        if (!count_only)
        {
#pragma unroll
            for (int k = 0; k < kPRPT; ++k)
            {
                const uint64_t row = row0 + (uint64_t)k * kPNT + threadIdx.x;
                if (ref_valid(head[k]))
                {
                    const uint64_t pos = round_base + excl[k];
                    if (dupf[k])
                        emit_chain<kCHJ>(a, o, head[k], roff[k], key[k], row, pos, out_cap);
                    else if (pos < out_cap)
                        emit_row(a, o, build_row_of<kCHJ>(head[k], roff[k], a), key[k], row, pos);
                }
                round_base += round_tot[k];
            }
        }
        __syncthreads(); // round_tot / sh_chunk reuse
    }
}
} // namespace

uint64_t probe_join(phj_ctx * ctx, Scratch & s, const ProbeArgs & a, phj_output * out, bool count_only, const char * name)
{
    unsigned long long * ctrs = s.get<unsigned long long>(2);
    PHJ_CUDA(cudaMemsetAsync(ctrs, 0, 2 * sizeof(unsigned long long), ctx->stream));
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
    int per_sm = 0;
    if (a.chj)
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe<true>, kPNT, 0));
    else
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe<false>, kPNT, 0));
    const uint64_t n_chunks = ceil_div(a.probe_rows, kChunk);
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(n_chunks, (uint64_t)ctx->num_sms * (uint64_t)std::max(per_sm, 1)));
    uint64_t probe_row_bytes = 8, build_row_bytes = 0;
    for (uint32_t c = 0; c < a.probe.n; ++c)
        probe_row_bytes += a.probe.width[c];
    for (uint32_t c = 0; c < a.build.n; ++c)
        build_row_bytes += a.build.width[c];
    {
        KTimer kt(ctx, name, a.probe_rows, count_only ? a.probe_rows * 8 : a.probe_rows * probe_row_bytes);
        if (a.chj)
            k_probe<true><<<grid, kPNT, 0, ctx->stream>>>(a, o, ctrs, cap, count_only ? 1 : 0);
        else
            k_probe<false><<<grid, kPNT, 0, ctx->stream>>>(a, o, ctrs, cap, count_only ? 1 : 0);
        PHJ_LAUNCHED(ctx, name);
    }
    unsigned long long rows = 0;
    PHJ_CUDA(cudaMemcpyAsync(&rows, ctrs + 1, sizeof(rows), cudaMemcpyDeviceToHost, ctx->stream));
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    // Fix the algorithmic byte count of the timed launch now that the
    // output size is known: output rows x (key + build + probe payloads).
    if (!count_only && !ctx->records.empty())
        ctx->records.back().bytes += rows * (8 + build_row_bytes + (probe_row_bytes - 8));
    return rows;
}

} // namespace phjg
