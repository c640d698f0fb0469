// batch.cu -- many independent joins in one persistent launch.
//
// A serving stream is dominated in count by small and medium joins (a few
// thousand to a few million build rows).  Run one at a time, each pays a
// dozen launches, host round trips and grids too small to fill 152 SMs.
// Here n joins share every launch:
//   1. k_bt_hist     tiles of 4096 rows of every join's build and probe
//                    side, found by binary search in their prefix: each
//                    join's rows are counted per radix partition (the top
//                    bits of intHash64, src/Hash.h:18-25; enough bits for
//                    about 1024 build rows a partition, at most 11);
//   2. scan_u32      the counts of all joins' partitions -> offsets;
//   3. k_bt_scatter  the same tiles: each tile reserves its rows' places in
//                    each partition with one atomic per partition and
//                    writes them (src/RadixPartition.cpp:316-393);
//   4. k_bt_join     ONE persistent launch whose CTAs pop (join, partition)
//                    work items from a device queue (one atomic counter):
//                    the partition's build rows go into a shared-memory
//                    JoinHashTable with its next-chain (src/HashTable.h,
//                    src/BlockStore.h), its probe rows are looked up there,
//                    and the matches are projected (key, build payloads,
//                    probe payloads: src/JoinOps.h:52-196) after one
//                    reservation of output rows per step in the join's
//                    output.  A partition with more build rows than the
//                    shared table holds is built and probed in pieces.
// The chain (counter clears, the three kernels, the scans and cursor
// copies) reads no size back to the host: the join count and the joins'
// prefix arrays and descriptors are uploaded in one copy into a workspace
// the context keeps, the kernels read the count from there, and the chain
// is captured once into a CUDA graph at the workspace's capacity and
// replayed for every later batch that fits (option "batch_graph"; 0
// launches the same chain at the batch's own sizes, with each kernel timed).
// Each join's output is sized for one row per probe row; a join with more
// (repeated build keys) is counted exactly, flagged, and run again alone.
// Output multisets equal those of the single-join entry points; the order
// of the rows is not fixed.
#include "internal.h"

#include <cstring>
#include <numeric>

namespace phjg
{
namespace
{
constexpr int kTNT = 256;              // threads of the partition kernels
constexpr uint32_t kTile = 4096;       // rows per partition tile
constexpr int kJNT = 512;              // threads of the join kernel
constexpr uint32_t kPieceRows = 2048;  // build rows a shared table holds
constexpr uint32_t kPieceCells = 4096; // its cells (load <= 1/2)
constexpr uint32_t kNil = 0xFFFFFFFFu;

struct BatchJoin
{
    Cols build, probe; // inputs
    Cols bpart, ppart; // partitioned copies
    uint64_t * out_keys;
    void * out_l[kMaxCols];
    void * out_r[kMaxCols];
    uint64_t build_rows, probe_rows, out_cap;
    uint32_t bits;      // radix bits
    uint32_t part_base; // index of its first partition among all joins'
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

__device__ __forceinline__ uint32_t part_of(uint64_t key, uint32_t bits)
{
    return bits ? (uint32_t)(int_hash64(key) >> (64u - bits)) : 0u;
}

// Tile t of the build sides (t < tiles_b[n]) or of the probe sides.
struct TileRef
{
    const BatchJoin * J;
    bool build;
    uint64_t r0, r1;
};
__device__ __forceinline__ TileRef tile_ref(const BatchJoin * d, uint32_t n, const uint64_t * tb, const uint64_t * tp, uint64_t t)
{
    TileRef x;
    const uint64_t nb = tb[n];
    x.build = t < nb;
    const uint64_t u = x.build ? t : t - nb;
    const uint32_t j = find_join(x.build ? tb : tp, n, u);
    x.J = d + j;
    x.r0 = (u - (x.build ? tb : tp)[j]) * kTile;
    const uint64_t rows = x.build ? x.J->build_rows : x.J->probe_rows;
    x.r1 = x.r0 + kTile < rows ? x.r0 + kTile : rows;
    return x;
}

__global__ void __launch_bounds__(kTNT) k_bt_hist(const BatchJoin * __restrict__ d, const uint32_t * __restrict__ d_n,
                                                  const uint64_t * __restrict__ tb, const uint64_t * __restrict__ tp,
                                                  uint32_t * __restrict__ cnt_b, uint32_t * __restrict__ cnt_p)
{
    __shared__ uint32_t h[1u << 11];
    const uint32_t n = *d_n;
    const uint64_t n_tiles = tb[n] + tp[n];
    for (uint64_t t = blockIdx.x; t < n_tiles; t += gridDim.x)
    {
        const TileRef x = tile_ref(d, n, tb, tp, t);
        const uint32_t Q = 1u << x.J->bits;
        for (uint32_t q = threadIdx.x; q < Q; q += kTNT)
            h[q] = 0;
        __syncthreads();
        const uint64_t * keys = x.build ? x.J->build.keys : x.J->probe.keys;
        for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += kTNT)
            atomicAdd(&h[part_of(keys[r], x.J->bits)], 1u);
        __syncthreads();
        uint32_t * cnt = (x.build ? cnt_b : cnt_p) + x.J->part_base;
        for (uint32_t q = threadIdx.x; q < Q; q += kTNT)
            if (h[q])
                atomicAdd(cnt + q, h[q]);
        __syncthreads();
    }
}

// Rows of the tile to their partitions: one reservation per partition and
// tile on the running cursors (offsets over all joins' partitions), the
// row's rank inside the tile's share from a shared counter.
__global__ void __launch_bounds__(kTNT) k_bt_scatter(const BatchJoin * __restrict__ d, const uint32_t * __restrict__ d_n,
                                                     const uint64_t * __restrict__ tb, const uint64_t * __restrict__ tp,
                                                     const uint32_t * __restrict__ off_b, const uint32_t * __restrict__ off_p,
                                                     uint32_t * __restrict__ cur_b, uint32_t * __restrict__ cur_p)
{
    __shared__ uint32_t h[1u << 11];
    __shared__ uint32_t base[1u << 11];
    const uint32_t n = *d_n;
    const uint64_t n_tiles = tb[n] + tp[n];
    for (uint64_t t = blockIdx.x; t < n_tiles; t += gridDim.x)
    {
        const TileRef x = tile_ref(d, n, tb, tp, t);
        const uint32_t Q = 1u << x.J->bits;
        for (uint32_t q = threadIdx.x; q < Q; q += kTNT)
            h[q] = 0;
        __syncthreads();
        const Cols & src = x.build ? x.J->build : x.J->probe;
        const Cols & dst = x.build ? x.J->bpart : x.J->ppart;
        for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += kTNT)
            atomicAdd(&h[part_of(src.keys[r], x.J->bits)], 1u);
        __syncthreads();
        // this tile's places in each partition, as rows of the join's
        // partitioned columns
        const uint32_t * off = (x.build ? off_b : off_p) + x.J->part_base;
        uint32_t * cur = (x.build ? cur_b : cur_p) + x.J->part_base;
        const uint32_t first = off[0];
        for (uint32_t q = threadIdx.x; q < Q; q += kTNT)
        {
            base[q] = h[q] ? atomicAdd(cur + q, h[q]) - first : 0u;
            h[q] = 0;
        }
        __syncthreads();
        for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += kTNT)
        {
            const uint64_t k = src.keys[r];
            const uint32_t q = part_of(k, x.J->bits);
            const uint32_t pos = base[q] + atomicAdd(&h[q], 1u);
            dst.keys[pos] = k;
            for (uint32_t c = 0; c < src.n; ++c)
                copy_elem(dst.col[c], pos, src.col[c], r, src.width[c]);
        }
        __syncthreads();
    }
}

// The persistent join: CTAs pop (join, partition) items until the queue is
// empty.  out_cur[j] counts join j's output rows (also past its capacity,
// where nothing is written and over[j] is set).
__global__ void __launch_bounds__(kJNT) k_bt_join(const BatchJoin * __restrict__ d, const uint32_t * __restrict__ d_n,
                                                  const uint64_t * __restrict__ parts,
                                                  const uint32_t * __restrict__ off_b, const uint32_t * __restrict__ off_p,
                                                  unsigned int * __restrict__ next_item, unsigned long long * __restrict__ out_cur,
                                                  int * __restrict__ over)
{
    __shared__ Cell cells[kPieceCells];
    __shared__ uint32_t nxt[kPieceRows];
    __shared__ uint32_t ws[kJNT / 32];
    __shared__ uint32_t s_item;
    __shared__ unsigned long long s_out;
    const uint32_t n = *d_n;
    const uint64_t n_items = parts[n];
    for (;;)
    {
        if (threadIdx.x == 0)
            s_item = atomicAdd(next_item, 1u);
        __syncthreads();
        const uint64_t item = s_item;
        __syncthreads();
        if (item >= n_items)
            return;
        const uint32_t j = find_join(parts, n, item);
        const BatchJoin & J = d[j];
        const uint32_t g = J.part_base + (uint32_t)(item - parts[j]);
        const uint32_t b0 = off_b[g] - off_b[J.part_base], b1 = off_b[g + 1] - off_b[J.part_base];
        const uint32_t p0 = off_p[g] - off_p[J.part_base], p1 = off_p[g + 1] - off_p[J.part_base];
        if (b1 == b0 || p1 == p0)
            continue;
        // the partition's build rows, a piece at a time
        for (uint32_t c0 = b0; c0 < b1; c0 += kPieceRows)
        {
            const uint32_t c1 = c0 + kPieceRows < b1 ? c0 + kPieceRows : b1;
            const uint32_t cap = (uint32_t)bit_ceil64(2ull * (c1 - c0));
            for (uint32_t i = threadIdx.x; i < cap; i += kJNT)
                reinterpret_cast<ulonglong2 *>(cells)[i] = make_ulonglong2(0ull, INVALID_REF);
            __syncthreads();
            for (uint32_t r = c0 + threadIdx.x; r < c1; r += kJNT)
            {
                const uint64_t k = J.bpart.keys[r];
                const uint64_t prev = table_insert<true>(cells, cap, int_hash64(k), k, make_ref(0, r));
                nxt[r - c0] = ref_valid(prev) ? ref_row(prev) : kNil;
            }
            __syncthreads();
            // its probe rows: count, reserve, project
            for (uint32_t base = p0; base < p1; base += kJNT)
            {
                const uint32_t r = base + threadIdx.x;
                uint64_t key = 0;
                uint32_t head = kNil, cnt = 0;
                if (r < p1)
                {
                    key = J.ppart.keys[r];
                    const uint64_t h = int_hash64(key);
                    const uint64_t mask = cap - 1;
                    uint64_t pos = probe_start(h, cap);
                    for (uint32_t step = 0; step < cap; ++step)
                    {
                        const Cell c = cells[pos];
                        if (!ref_valid(c.ref))
                            break;
                        if (c.key == key)
                        {
                            head = ref_row(c.ref);
                            break;
                        }
                        pos = (pos + 1) & mask;
                    }
                    for (uint32_t b = head; b != kNil; b = nxt[b - c0])
                        ++cnt;
                }
                uint32_t total;
                const uint32_t ex = block_excl_scan<kJNT>(cnt, ws, &total);
                if (total == 0)
                    continue;
                if (threadIdx.x == 0)
                    s_out = atomicAdd(out_cur + j, (unsigned long long)total);
                __syncthreads();
                const uint64_t o0 = s_out + ex;
                if (threadIdx.x == 0 && s_out + total > J.out_cap)
                    over[j] = 1;
                uint64_t o = o0;
                for (uint32_t b = head; b != kNil; b = nxt[b - c0], ++o)
                    if (o < J.out_cap)
                    {
                        J.out_keys[o] = key;
                        for (uint32_t c = 0; c < J.bpart.n; ++c)
                            copy_elem(J.out_l[c], o, J.bpart.col[c], b, J.bpart.width[c]);
                        for (uint32_t c = 0; c < J.ppart.n; ++c)
                            copy_elem(J.out_r[c], o, J.ppart.col[c], r, J.ppart.width[c]);
                    }
                __syncthreads(); // s_out is reused by the next step
            }
        }
    }
}

uint32_t partition_bits(uint64_t build_rows)
{
    uint32_t b = 0;
    while (b < 11 && (build_rows >> b) > 1024)
        ++b;
    return b;
}

size_t round_up(size_t x, size_t a)
{
    return (x + a - 1) / a * a;
}
} // namespace

// The chain's workspace, kept by the context across batches at fixed
// addresses, so that one captured graph of the chain replays for every
// batch of at most n_cap joins and q_cap partitions in all.  Device block:
// the upload region (join count, the three prefix arrays, the join
// descriptors), then the per-join output counters and overflow flags
// (adjacent: one download), then the partitions' counts, offsets and
// cursors and the scan's carry space.  Pinned host block: the upload
// staging at the same offsets, then the download staging.
struct BatchGraph
{
    uint32_t n_cap = 0;
    uint64_t q_cap = 0;
    uint8_t * dev = nullptr;
    uint8_t * host = nullptr;
    size_t o_tb = 0, o_tp = 0, o_parts = 0, o_desc = 0, o_out = 0, o_cnt = 0, o_carry = 0, o_next = 0, bytes = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0; // kernel launches in one replay
};

void free_batch_graph(phj_ctx * ctx)
{
    BatchGraph * W = ctx->batch_ws;
    if (!W)
        return;
    if (W->exec)
        cudaGraphExecDestroy(W->exec);
    if (W->dev)
        cudaFree(W->dev);
    if (W->host)
        cudaFreeHost(W->host);
    delete W;
    ctx->batch_ws = nullptr;
}

namespace
{
struct Chain
{
    const uint8_t * base;
    const BatchGraph * W;
    uint32_t * n() const { return (uint32_t *)base; }
    uint64_t * tb() const { return (uint64_t *)(base + W->o_tb); }
    uint64_t * tp() const { return (uint64_t *)(base + W->o_tp); }
    uint64_t * parts() const { return (uint64_t *)(base + W->o_parts); }
    BatchJoin * desc() const { return (BatchJoin *)(base + W->o_desc); }
    unsigned long long * out_cur() const { return (unsigned long long *)(base + W->o_out); }
    int * over() const { return (int *)(base + W->o_out + 8ull * W->n_cap); }
    uint32_t * cnt(int k) const { return (uint32_t *)(base + W->o_cnt) + (uint64_t)k * (W->q_cap + 1); } // cnt_b, cnt_p, off_b, off_p, cur_b, cur_p
    uint32_t * carry() const { return (uint32_t *)(base + W->o_carry); }
    unsigned int * next() const { return (unsigned int *)(base + W->o_next); }
};

BatchGraph & batch_workspace(phj_ctx * ctx, uint32_t n, uint64_t nq)
{
    BatchGraph * W = ctx->batch_ws;
    if (W && n <= W->n_cap && nq <= W->q_cap)
        return *W;
    uint32_t n_cap = W ? W->n_cap : 16;
    uint64_t q_cap = W ? W->q_cap : 4096;
    while (n_cap < n)
        n_cap *= 2;
    while (q_cap < nq)
        q_cap *= 2;
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    free_batch_graph(ctx);
    W = new BatchGraph;
    ctx->batch_ws = W;
    W->n_cap = n_cap;
    W->q_cap = q_cap;
    size_t at = 0;
    auto take = [&](size_t bytes) {
        const size_t o = at;
        at = round_up(at + bytes, 256);
        return o;
    };
    take(sizeof(uint32_t));
    W->o_tb = take(8ull * (n_cap + 1));
    W->o_tp = take(8ull * (n_cap + 1));
    W->o_parts = take(8ull * (n_cap + 1));
    W->o_desc = take(sizeof(BatchJoin) * n_cap);
    W->o_out = take(12ull * n_cap);
    W->o_cnt = take(6 * 4ull * (q_cap + 1));
    W->o_carry = take(4ull * std::max<uint64_t>(scan_u32_carry(q_cap), 1));
    W->o_next = take(sizeof(unsigned int));
    W->bytes = at;
    try
    {
        PHJ_CUDA(cudaMalloc(&W->dev, W->bytes));
        PHJ_CUDA(cudaMallocHost(&W->host, W->o_cnt));
    }
    catch (...)
    {
        free_batch_graph(ctx); // no half-made workspace for the next call
        throw;
    }
    return *W;
}

// The chain on the context's stream: counts, offsets and cursors of q_len
// partitions (zero past the batch's own), then the three kernels.  With
// `bytes` (rows, input bytes) each kernel is timed; without, nothing but
// stream work is issued, so the chain can be captured.
void enqueue_chain(phj_ctx * ctx, const Chain & c, uint64_t q_len, unsigned tgrid, unsigned jgrid, const uint64_t * bytes)
{
    cudaStream_t st = ctx->stream;
    const uint64_t q_bytes = (q_len + 1) * sizeof(uint32_t);
    uint32_t *cnt_b = c.cnt(0), *cnt_p = c.cnt(1), *off_b = c.cnt(2), *off_p = c.cnt(3), *cur_b = c.cnt(4), *cur_p = c.cnt(5);
    PHJ_CUDA(cudaMemsetAsync(cnt_b, 0, q_bytes, st));
    PHJ_CUDA(cudaMemsetAsync(cnt_p, 0, q_bytes, st));
    PHJ_CUDA(cudaMemsetAsync(c.next(), 0, sizeof(unsigned int), st));
    PHJ_CUDA(cudaMemsetAsync(c.out_cur(), 0, 12ull * c.W->n_cap, st));
    {
        KTimer kt(ctx, bytes ? "batch_hist" : nullptr, bytes ? bytes[0] : 0, bytes ? bytes[0] * 8 : 0);
        k_bt_hist<<<tgrid, kTNT, 0, st>>>(c.desc(), c.n(), c.tb(), c.tp(), cnt_b, cnt_p);
        PHJ_LAUNCHED(ctx, "batch_hist");
    }
    scan_u32_into(ctx, cnt_b, off_b, q_len, c.carry());
    scan_u32_into(ctx, cnt_p, off_p, q_len, c.carry());
    PHJ_CUDA(cudaMemcpyAsync(cur_b, off_b, q_bytes, cudaMemcpyDeviceToDevice, st));
    PHJ_CUDA(cudaMemcpyAsync(cur_p, off_p, q_bytes, cudaMemcpyDeviceToDevice, st));
    {
        KTimer kt(ctx, bytes ? "batch_scatter" : nullptr, bytes ? bytes[0] : 0, bytes ? 2 * bytes[1] : 0);
        k_bt_scatter<<<tgrid, kTNT, 0, st>>>(c.desc(), c.n(), c.tb(), c.tp(), off_b, off_p, cur_b, cur_p);
        PHJ_LAUNCHED(ctx, "batch_scatter");
    }
    {
        KTimer kt(ctx, bytes ? "batch_join" : nullptr, bytes ? bytes[2] : 0, bytes ? bytes[1] : 0);
        k_bt_join<<<jgrid, kJNT, 0, st>>>(c.desc(), c.n(), c.parts(), off_b, off_p, c.next(), c.out_cur(), c.over());
        PHJ_LAUNCHED(ctx, "batch_join");
    }
}

unsigned join_grid(phj_ctx * ctx)
{
    int per_sm = 0;
    PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bt_join, kJNT, 0));
    return (unsigned)ctx->num_sms * (unsigned)std::max(per_sm, 1);
}

// Captures the chain at the workspace's capacity (every grid at its
// largest: CTAs past the batch's tiles and partitions find no work) and
// instantiates it.
void capture_chain(phj_ctx * ctx, BatchGraph & W)
{
    const unsigned jgrid = join_grid(ctx);
    const uint64_t before = ctx->launches;
    cudaGraph_t g = nullptr;
    PHJ_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try
    {
        enqueue_chain(ctx, Chain{W.dev, &W}, W.q_cap, (unsigned)ctx->num_sms * 8, jgrid, nullptr);
    }
    catch (...)
    {
        cudaStreamEndCapture(ctx->stream, &g);
        if (g)
            cudaGraphDestroy(g);
        cudaGetLastError();
        ctx->launches = before;
        throw;
    }
    PHJ_CUDA(cudaStreamEndCapture(ctx->stream, &g));
    W.kernels = ctx->launches - before;
    ctx->launches = before;
    const cudaError_t e = cudaGraphInstantiate(&W.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
        W.exec = nullptr;
    PHJ_CUDA(e);
}

void run_batch(phj_ctx * ctx, uint32_t n, const phj_table * const * builds, const phj_table * const * probes, phj_output ** outs,
               phj_batch_result * res)
{
    for (uint32_t j = 0; j < n; ++j)
    {
        if (!builds[j] || !probes[j])
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "batch: null build or probe table");
        if (builds[j]->rows >= (1ull << 31) || probes[j]->rows >= (1ull << 31))
            throw Error(PHJ_ERR_UNSUPPORTED, "batch: fewer than 2^31 build rows and 2^31 probe rows per join");
    }
    begin_run(ctx);
    Scratch s(ctx);
    cudaEvent_t e0 = take_event(ctx), e1 = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(e0, ctx->stream));

    std::vector<BatchJoin> h(n);
    std::vector<uint64_t> tb(n + 1, 0), tp(n + 1, 0), parts(n + 1, 0);
    uint64_t brows = 0, prows = 0, in_bytes = 0;
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
        J.bits = partition_bits(B.rows);
        J.part_base = (uint32_t)parts[j];
        J.bpart = alloc_cols_like(s, B.schema, std::max<uint64_t>(B.rows, 1));
        J.ppart = alloc_cols_like(s, P.schema, std::max<uint64_t>(P.rows, 1));
        parts[j + 1] = parts[j] + (1ull << J.bits);
        tb[j + 1] = tb[j] + ceil_div(B.rows, kTile);
        tp[j + 1] = tp[j] + ceil_div(P.rows, kTile);
        brows += B.rows;
        prows += P.rows;
        in_bytes += B.rows * (8 + schema_bytes(B.schema)) + P.rows * (8 + schema_bytes(P.schema));
    }
    if (brows >= (1ull << 32) || prows >= (1ull << 32))
        throw Error(PHJ_ERR_UNSUPPORTED, "batch: fewer than 2^32 build rows and 2^32 probe rows in all");
    const uint64_t NQ = parts[n];

    // outputs at one row per probe row (exact for unique build keys)
    std::vector<phj_output *> made(n, nullptr);
    try
    {
        for (uint32_t j = 0; j < n; ++j)
        {
            made[j] = new_output(ctx, builds[j]->schema, probes[j]->schema, probes[j]->rows);
            BatchJoin & J = h[j];
            J.out_keys = made[j]->keys;
            for (uint32_t c = 0; c < J.build.n; ++c)
                J.out_l[c] = made[j]->lcol[c];
            for (uint32_t c = 0; c < J.probe.n; ++c)
                J.out_r[c] = made[j]->rcol[c];
            J.out_cap = probes[j]->rows;
        }
        std::vector<unsigned long long> rows(n, 0);
        std::vector<int> ov(n, 0);
        if (n)
        {
            BatchGraph & W = batch_workspace(ctx, n, NQ);
            // one upload: join count, prefix arrays, descriptors
            uint8_t * H = W.host;
            std::memcpy(H, &n, sizeof(uint32_t));
            std::memcpy(H + W.o_tb, tb.data(), (n + 1) * sizeof(uint64_t));
            std::memcpy(H + W.o_tp, tp.data(), (n + 1) * sizeof(uint64_t));
            std::memcpy(H + W.o_parts, parts.data(), (n + 1) * sizeof(uint64_t));
            std::memcpy(H + W.o_desc, h.data(), n * sizeof(BatchJoin));
            PHJ_CUDA(cudaMemcpyAsync(W.dev, H, W.o_desc + n * sizeof(BatchJoin), cudaMemcpyHostToDevice, ctx->stream));
            const Chain c{W.dev, &W};
            if (ctx->batch_graph)
            {
                if (!W.exec)
                    capture_chain(ctx, W);
                KTimer kt(ctx, "batch_graph", brows + prows, (brows + prows) * 8 + 3 * in_bytes);
                PHJ_CUDA(cudaGraphLaunch(W.exec, ctx->stream));
                ctx->launches += W.kernels;
            }
            else
            {
                const uint64_t n_tiles = tb[n] + tp[n];
                const unsigned tgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(n_tiles, (uint64_t)ctx->num_sms * 8));
                const unsigned jgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(NQ, join_grid(ctx)));
                const uint64_t bytes[3] = {brows + prows, in_bytes, prows};
                enqueue_chain(ctx, c, NQ, tgrid, jgrid, bytes);
            }
            uint8_t * D = H + W.o_out;
            PHJ_CUDA(cudaMemcpyAsync(D, c.out_cur(), 12ull * W.n_cap, cudaMemcpyDeviceToHost, ctx->stream));
            PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
            std::memcpy(rows.data(), D, n * sizeof(unsigned long long));
            std::memcpy(ov.data(), D + 8ull * W.n_cap, n * sizeof(int));
        }
        uint64_t out_rows = 0;
        for (uint32_t j = 0; j < n; ++j)
        {
            if (ov[j])
            {
                // more output rows than probe rows (repeated build keys):
                // this join again, alone
                free_output(ctx, made[j]);
                made[j] = nullptr;
                made[j] = join_alone(ctx, *builds[j], *probes[j]);
            }
            else
                made[j]->rows = rows[j];
            out_rows += made[j]->rows;
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
            if (o)
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
