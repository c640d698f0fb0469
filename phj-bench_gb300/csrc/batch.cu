// batch.cu -- many independent joins in one set of launches.
//
// A serving stream is dominated in count by small joins (a few thousand to a
// few hundred thousand build rows).  Run one at a time, each pays a dozen
// launches, two host round trips and grids too small to fill 152 SMs.  Here
// n joins share every launch: a device descriptor per join, prefix sums of
// their build tiles and probe warp chunks, and kernels whose work items are
// (join, tile) or (join, chunk) pairs found by binary search in the prefix.
//
// Per join the algorithm is the global-table join: one open-addressing table
// of bit_ceil(2 * build rows) 16-byte cells (the JoinHashTable layout,
// src/HashTable.h:27-166) with the BlockStore next-chain per build row
// (src/BlockStore.h:34-95), then lookups, an exact output size from a scan of
// per-chunk match counts, and the projection (key, build payloads, probe
// payloads: src/JoinOps.h:52-196).  Output multisets equal those of the
// single-join entry points.
#include "internal.h"

#include <numeric>

namespace phjg
{
namespace
{
constexpr int kBNT = 256;       // threads per CTA
constexpr int kBTile = 256;     // build rows per tile (one per thread)
constexpr int kBChunk = 256;    // probe rows per warp chunk
constexpr int kBRPT = kBChunk / 32;
constexpr uint32_t kBNoMatch = 0xFFFFFFFFu;

struct BatchJoin
{
    Cols build;        // keys + build payloads
    Cols probe;        // keys + probe payloads
    Cols out_b;        // keys = output key column, col[] = build payload outputs
    Cols out_p;        // col[] = probe payload outputs
    uint64_t build_rows, probe_rows;
    uint64_t cell_off;   // first cell of the join's table
    uint64_t build_base; // first slot of the join in the next-chain arena
    uint64_t probe_base; // first slot of the join in the head arena
    uint32_t log2cap;
};

// Index j with pre[j] <= t < pre[j+1] (pre non-decreasing, pre[0] = 0).
__device__ __forceinline__ uint32_t find_join(const uint64_t * __restrict__ pre, uint32_t n, uint64_t t)
{
    uint32_t lo = 0, hi = n; // pre[lo] <= t < pre[hi]
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(pre + mid) <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_batch_clear(Cell * __restrict__ cells, uint64_t n)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        reinterpret_cast<ulonglong2 *>(cells)[i] = make_ulonglong2(0ull, INVALID_REF);
}

__global__ void __launch_bounds__(kBNT) k_batch_build(const BatchJoin * __restrict__ d, uint32_t n, const uint64_t * __restrict__ tiles,
                                                      Cell * __restrict__ cells, uint64_t * __restrict__ next)
{
    const uint64_t n_tiles = tiles[n];
    for (uint64_t t = blockIdx.x; t < n_tiles; t += gridDim.x)
    {
        const uint32_t j = find_join(tiles, n, t);
        const BatchJoin & J = d[j];
        const uint64_t r = (t - tiles[j]) * kBTile + threadIdx.x;
        if (r < J.build_rows)
        {
            const uint64_t k = J.build.keys[r];
            next[J.build_base + r] = table_insert<false>(cells + J.cell_off, 1ull << J.log2cap, int_hash64(k), k, make_ref(0, (uint32_t)r));
        }
    }
}

__device__ __forceinline__ uint32_t chain_len(const uint64_t * __restrict__ next, uint64_t base, uint32_t head)
{
    uint32_t c = 1;
    for (uint64_t r = __ldg(next + base + head); ref_valid(r); r = __ldg(next + base + ref_row(r)))
        ++c;
    return c;
}

// A warp per chunk of 256 probe rows: heads, and the chunk's output rows.
// The batch's output rows are also summed in 64 bits (one atomic per warp),
// so the host can refuse a batch whose 32-bit chunk offsets would wrap.
__global__ void __launch_bounds__(kBNT) k_batch_lookup(const BatchJoin * __restrict__ d, uint32_t n, const uint64_t * __restrict__ chunks,
                                                       const Cell * __restrict__ cells, const uint64_t * __restrict__ next,
                                                       uint32_t * __restrict__ heads, uint32_t * __restrict__ counts,
                                                       unsigned long long * __restrict__ out_rows64)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_chunks = chunks[n];
    const uint64_t warps = ((uint64_t)gridDim.x * kBNT) >> 5;
    unsigned long long warp_rows = 0;
    for (uint64_t c = ((uint64_t)blockIdx.x * kBNT + threadIdx.x) >> 5; c < n_chunks; c += warps)
    {
        const uint32_t j = find_join(chunks, n, c);
        const BatchJoin & J = d[j];
        const uint64_t cap = 1ull << J.log2cap;
        const Cell * tab = cells + J.cell_off;
        const uint64_t row0 = (c - chunks[j]) * kBChunk + lane;
        unsigned long long total = 0;
#pragma unroll 4
        for (int k = 0; k < kBRPT; ++k)
        {
            const uint64_t r = row0 + (uint64_t)k * 32;
            if (r >= J.probe_rows)
                break;
            const uint64_t key = __ldcs(J.probe.keys + r);
            const uint64_t h = table_find(tab, cap, int_hash64(key), key);
            uint32_t head = kBNoMatch;
            if (ref_valid(h))
            {
                head = ref_row(h);
                total += chain_len(next, J.build_base, head);
            }
            heads[J.probe_base + r] = head;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            total += __shfl_xor_sync(0xffffffffu, total, o);
        if (lane == 0)
            counts[c] = (uint32_t)min(total, 0xFFFFFFFFull); // the host refuses the batch above 2^32 - 1 rows
        warp_rows += total;
    }
    if (lane == 0 && warp_rows)
        atomicAdd(out_rows64, warp_rows);
}

__global__ void k_batch_totals(const uint64_t * __restrict__ chunks, const uint32_t * __restrict__ offs, uint32_t n, uint64_t * __restrict__ totals)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n)
        totals[j] = (uint64_t)offs[chunks[j + 1]] - offs[chunks[j]];
}

// Output row o of join J: the probe key, the build payloads of build row b,
// the probe payloads of probe row p.
__device__ __forceinline__ void emit(const BatchJoin & J, uint64_t o, uint64_t key, uint32_t b, uint64_t p)
{
    J.out_b.keys[o] = key;
    for (uint32_t c = 0; c < J.build.n; ++c)
        copy_elem(J.out_b.col[c], o, J.build.col[c], b, J.build.width[c]);
    for (uint32_t c = 0; c < J.probe.n; ++c)
        copy_elem(J.out_p.col[c], o, J.probe.col[c], p, J.probe.width[c]);
}

__global__ void __launch_bounds__(kBNT) k_batch_project(const BatchJoin * __restrict__ d, uint32_t n, const uint64_t * __restrict__ chunks,
                                                        const uint64_t * __restrict__ next, const uint32_t * __restrict__ heads,
                                                        const uint32_t * __restrict__ offs)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_chunks = chunks[n];
    const uint64_t warps = ((uint64_t)gridDim.x * kBNT) >> 5;
    for (uint64_t c = ((uint64_t)blockIdx.x * kBNT + threadIdx.x) >> 5; c < n_chunks; c += warps)
    {
        const uint32_t j = find_join(chunks, n, c);
        const BatchJoin & J = d[j];
        uint64_t base = (uint64_t)offs[c] - offs[chunks[j]];
        const uint64_t row0 = (c - chunks[j]) * kBChunk + lane;
        for (int k = 0; k < kBRPT; ++k)
        {
            const uint64_t r = row0 + (uint64_t)k * 32;
            if (__all_sync(0xffffffffu, r >= J.probe_rows))
                break;
            uint32_t head = kBNoMatch, cnt = 0;
            if (r < J.probe_rows)
            {
                head = heads[J.probe_base + r];
                if (head != kBNoMatch)
                    cnt = chain_len(next, J.build_base, head);
            }
            uint32_t x = cnt;
#pragma unroll
            for (int s = 1; s < 32; s <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, s);
                if (lane >= (uint32_t)s)
                    x += y;
            }
            const uint64_t o0 = base + x - cnt;
            base += __shfl_sync(0xffffffffu, x, 31);
            if (cnt)
            {
                const uint64_t key = J.probe.keys[r];
                uint32_t b = head;
                for (uint32_t i = 0; i < cnt; ++i)
                {
                    emit(J, o0 + i, key, b, r);
                    const uint64_t nx = __ldg(next + J.build_base + b);
                    b = ref_row(nx);
                }
            }
        }
    }
}

unsigned grid_for(phj_ctx * ctx, uint64_t items_per_cta_units)
{
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(items_per_cta_units, (uint64_t)ctx->num_sms * 8));
}

void run_batch(phj_ctx * ctx, uint32_t n, const phj_table * const * builds, const phj_table * const * probes, phj_output ** outs,
               phj_batch_result * res)
{
    for (uint32_t j = 0; j < n; ++j)
    {
        if (!builds[j] || !probes[j])
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "batch: null build or probe table");
        if (builds[j]->rows >= (1ull << 31) || probes[j]->rows >= (1ull << 32))
            throw Error(PHJ_ERR_UNSUPPORTED, "batch: < 2^31 build rows and < 2^32 probe rows per join");
    }
    begin_run(ctx);
    Scratch s(ctx);
    cudaEvent_t e0 = take_event(ctx), e1 = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(e0, ctx->stream));

    std::vector<BatchJoin> h(n);
    std::vector<uint64_t> tiles(n + 1, 0), chunks(n + 1, 0);
    uint64_t cells = 0, brows = 0, prows = 0;
    for (uint32_t j = 0; j < n; ++j)
    {
        const phj_table & B = *builds[j];
        const phj_table & P = *probes[j];
        BatchJoin & J = h[j];
        J = BatchJoin{};
        J.build = cols_of(B);
        J.probe = cols_of(P);
        J.build_rows = B.rows;
        J.probe_rows = P.rows;
        const uint64_t cap = B.rows ? bit_ceil64(2 * B.rows) : 1;
        J.log2cap = (uint32_t)__builtin_ctzll(cap);
        J.cell_off = cells;
        J.build_base = brows;
        J.probe_base = prows;
        cells += cap;
        brows += B.rows;
        prows += P.rows;
        tiles[j + 1] = tiles[j] + ceil_div(B.rows, kBTile);
        chunks[j + 1] = chunks[j] + ceil_div(P.rows, kBChunk);
    }
    Cell * d_cells = s.get<Cell>(std::max<uint64_t>(cells, 1));
    uint64_t * d_next = s.get<uint64_t>(std::max<uint64_t>(brows, 1));
    uint32_t * d_heads = s.get<uint32_t>(std::max<uint64_t>(prows, 1));
    uint32_t * d_counts = s.get<uint32_t>(chunks[n] + 1);
    uint64_t * d_tiles = s.get<uint64_t>(n + 1);
    uint64_t * d_chunks = s.get<uint64_t>(n + 1);
    uint64_t * d_totals = s.get<uint64_t>(std::max<uint32_t>(n, 1));
    unsigned long long * d_rows64 = s.get<unsigned long long>(1);
    PHJ_CUDA(cudaMemsetAsync(d_rows64, 0, sizeof(unsigned long long), ctx->stream));
    BatchJoin * d_desc = s.get<BatchJoin>(std::max<uint32_t>(n, 1));
    PHJ_CUDA(cudaMemcpyAsync(d_tiles, tiles.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
    PHJ_CUDA(cudaMemcpyAsync(d_chunks, chunks.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
    PHJ_CUDA(cudaMemcpyAsync(d_desc, h.data(), n * sizeof(BatchJoin), cudaMemcpyHostToDevice, ctx->stream));

    {
        KTimer kt(ctx, "batch_clear", cells, cells * sizeof(Cell));
        k_batch_clear<<<grid_for(ctx, ceil_div(cells, kBNT)), kBNT, 0, ctx->stream>>>(d_cells, cells);
        PHJ_LAUNCHED(ctx, "batch_clear");
    }
    if (tiles[n])
    {
        KTimer kt(ctx, "batch_build", brows, brows * (8 + 16 + 8));
        k_batch_build<<<grid_for(ctx, tiles[n]), kBNT, 0, ctx->stream>>>(d_desc, n, d_tiles, d_cells, d_next);
        PHJ_LAUNCHED(ctx, "batch_build");
    }
    std::vector<uint64_t> totals(n, 0);
    if (chunks[n])
    {
        {
            KTimer kt(ctx, "batch_lookup", prows, prows * (8 + 4));
            k_batch_lookup<<<grid_for(ctx, ceil_div(chunks[n], kBNT / 32)), kBNT, 0, ctx->stream>>>(d_desc, n, d_chunks, d_cells, d_next, d_heads,
                                                                                                     d_counts, d_rows64);
            PHJ_LAUNCHED(ctx, "batch_lookup");
        }
        scan_u32(ctx, s, d_counts, d_counts, chunks[n]);
        k_batch_totals<<<(unsigned)ceil_div(n, 256), 256, 0, ctx->stream>>>(d_chunks, d_counts, n, d_totals);
        PHJ_LAUNCHED(ctx, "batch_totals");
        unsigned long long rows64 = 0;
        PHJ_CUDA(cudaMemcpyAsync(totals.data(), d_totals, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
        PHJ_CUDA(cudaMemcpyAsync(&rows64, d_rows64, sizeof(rows64), cudaMemcpyDeviceToHost, ctx->stream));
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
        if (rows64 >= (1ull << 32))
            throw Error(PHJ_ERR_CAPACITY, "the batch has " + std::to_string(rows64) +
                                              " output rows; batched joins place at most 2^32 - 1 in all (run large joins on their own)");
    }
    std::vector<phj_output *> made(n, nullptr);
    try
    {
        uint64_t out_rows = 0, out_bytes = 0;
        for (uint32_t j = 0; j < n; ++j)
        {
            made[j] = new_output(ctx, builds[j]->schema, probes[j]->schema, totals[j]);
            made[j]->rows = totals[j];
            BatchJoin & J = h[j];
            J.out_b = J.build;
            J.out_b.keys = made[j]->keys;
            for (uint32_t c = 0; c < J.build.n; ++c)
                J.out_b.col[c] = made[j]->lcol[c];
            J.out_p = J.probe;
            J.out_p.keys = nullptr;
            for (uint32_t c = 0; c < J.probe.n; ++c)
                J.out_p.col[c] = made[j]->rcol[c];
            out_rows += totals[j];
            out_bytes += made[j]->bytes;
        }
        if (chunks[n])
        {
            PHJ_CUDA(cudaMemcpyAsync(d_desc, h.data(), n * sizeof(BatchJoin), cudaMemcpyHostToDevice, ctx->stream));
            uint64_t in_bytes = 0;
            for (uint32_t j = 0; j < n; ++j)
                in_bytes += totals[j] * (8 + schema_bytes(probes[j]->schema));
            KTimer kt(ctx, "batch_project", prows, prows * 4 + in_bytes + out_bytes);
            k_batch_project<<<grid_for(ctx, ceil_div(chunks[n], kBNT / 32)), kBNT, 0, ctx->stream>>>(d_desc, n, d_chunks, d_next, d_heads, d_counts);
            PHJ_LAUNCHED(ctx, "batch_project");
        }
        PHJ_CUDA(cudaEventRecord(e1, ctx->stream));
        PHJ_CUDA(cudaEventSynchronize(e1));
        if (res)
        {
            res->e2e_wall_ms = event_ms(e0, e1);
            res->n_joins = n;
            res->build_rows = brows;
            res->probe_rows = prows;
            res->output_rows = out_rows;
            res->peak_mem_bytes = ctx->peak_bytes;
        }
    }
    catch (...)
    {
        for (phj_output * o : made)
            free_output(ctx, o);
        throw;
    }
    for (uint32_t j = 0; j < n; ++j)
        outs[j] = made[j];
}
} // namespace
} // namespace phjg

extern "C" phj_status phj_batch_run(phj_ctx * ctx, uint32_t n, const phj_table * const * builds, const phj_table * const * probes,
                                    phj_output ** outs, phj_batch_result * result)
{
    if (!ctx || (n && (!builds || !probes || !outs)))
        return PHJ_ERR_INVALID_ARGUMENT;
    for (uint32_t j = 0; j < n; ++j)
        outs[j] = nullptr;
    return phjg::guard(ctx, [&] { phjg::run_batch(ctx, n, builds, probes, outs, result); });
}
