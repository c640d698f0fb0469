// build.cu -- hashtable build on the device.
//
// PHJ-PURE / PHJ: one JoinHashTable per leaf (src/PHJ.cpp:260-282,
// src/PHJBep.cpp:192-232).  Capacity follows JoinHashTable::reserve
// (src/HashTable.h:72-79): bit_ceil(2 * rows), i.e. load <= 1/2.  One CTA
// owns a leaf: it builds the table in shared memory with 128-bit CAS
// inserts, threads each row's previous head into the next-chain
// (BlockStore::setPrev, src/BlockStore.h:83-84; buildOneBlock,
// src/JoinOps.h:205-228), then streams the finished table to global memory.
// Leaves too large for shared memory are built in place in global memory.
//
// CHJ: one global table of 256 sub-tables selected by the top 8 hash bits
// (the mutex-free form of ChjSlottedTable, src/TwoLevelHashTable.h:57-91),
// filled by every thread of the grid with 128-bit CAS inserts.
#include "internal.h"

namespace phjg
{
namespace
{
constexpr int kBuildNT = 256;
constexpr uint32_t kSmemCellsMax = 8192; // 128 KiB of cells per CTA

// Cells of a table for r rows: the power of two at or above r * pct / 100
// (pct 200: load <= 1/2, the reference's JoinHashTable::reserve), and above r.
__host__ __device__ __forceinline__ uint64_t table_cells(uint64_t r, uint32_t pct)
{
    if (!r)
        return 0;
    const uint64_t want = (r * pct + 99) / 100;
    return bit_ceil64(want > r ? want : r + 1);
}

__global__ void k_leaf_caps(const uint32_t * __restrict__ leaf_off, uint32_t n_leaves, uint32_t pct, uint32_t * __restrict__ caps,
                            uint32_t * __restrict__ max_rows)
{
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n_leaves)
        return;
    const uint32_t r = leaf_off[l + 1] - leaf_off[l];
    caps[l] = (uint32_t)table_cells(r, pct);
    if (r)
        atomicMax(max_rows, r);
}

__device__ __forceinline__ uint32_t log2u(uint64_t x)
{
    return 63u - (uint32_t)__clzll((long long)x);
}

// One CTA per leaf.  Tables are either uniform (every leaf 2^ulog cells at
// leaf << ulog, ulog >= 0) or sized per leaf through table_off (ulog < 0).
// The RowRefCell of a build row is {0, row}: block 0 is the whole
// leaf-partitioned build side, row its index there.
template <int NT>
__global__ void __launch_bounds__(NT) k_build_leaf(const uint64_t * __restrict__ keys, const uint32_t * __restrict__ leaf_off,
                                                         const uint32_t * __restrict__ table_off, int ulog, uint32_t smem_cells,
                                                         Cell * __restrict__ cells, uint64_t * __restrict__ next, LeafMeta * __restrict__ meta,
                                                         int * __restrict__ any_dup)
{
    extern __shared__ __align__(16) Cell sh_cells[];
    __shared__ int dup;
    const uint32_t l = blockIdx.x;
    const uint32_t r0 = leaf_off[l], r = leaf_off[l + 1] - r0;
    const uint64_t t0 = ulog >= 0 ? ((uint64_t)l << ulog) : table_off[l];
    const uint64_t cap = ulog >= 0 ? (1ull << ulog) : table_off[l + 1] - t0;
    if (threadIdx.x == 0)
        dup = 0;
    const Cell empty{0ull, INVALID_REF};
    if (r == 0)
    {
        for (uint64_t i = threadIdx.x; i < cap; i += NT) // uniform layout: an empty table
            reinterpret_cast<ulonglong2 *>(cells + t0)[i] = make_ulonglong2(0ull, INVALID_REF);
        if (threadIdx.x == 0)
            meta[l] = LeafMeta{t0, r0, cap ? (uint8_t)log2u(cap) : (uint8_t)0, 0, 0, 0};
        return;
    }
    const bool in_smem = cap <= smem_cells;
    Cell * tab = in_smem ? sh_cells : cells + t0;
    for (uint64_t i = threadIdx.x; i < cap; i += NT)
        tab[i] = empty;
    __syncthreads();
    bool my_dup = false;
    for (uint32_t i = threadIdx.x; i < r; i += NT)
    {
        const uint64_t k = keys[r0 + i];
        const uint64_t h = int_hash64(k);
        const uint64_t ref = make_ref(0, r0 + i);
        const uint64_t prev = in_smem ? table_insert<true>(tab, cap, h, k, ref) : table_insert<false>(tab, cap, h, k, ref);
        next[r0 + i] = prev;
        my_dup |= ref_valid(prev);
    }
    if (__any_sync(0xffffffffu, my_dup) && (threadIdx.x & 31) == 0)
        dup = 1;
    __syncthreads();
    if (in_smem)
    {
        ulonglong2 * dst = reinterpret_cast<ulonglong2 *>(cells + t0);
        const ulonglong2 * src = reinterpret_cast<const ulonglong2 *>(sh_cells);
        for (uint64_t i = threadIdx.x; i < cap; i += NT)
            dst[i] = src[i];
    }
    if (threadIdx.x == 0)
    {
        meta[l] = LeafMeta{t0, r0, (uint8_t)log2u(cap), 1, (uint8_t)dup, 0};
        if (dup)
            atomicOr(any_dup, 1);
    }
}

// ---- grouped duplicates (PHJ-PURE with repeated build keys) ----------------
// Position of `key` in a finished table (the key is present).
__device__ __forceinline__ uint32_t cell_of(const Cell * tab, uint64_t cap, uint64_t h, uint64_t key)
{
    uint64_t pos = probe_start(h, cap);
    for (uint64_t step = 0; step < cap; ++step)
    {
        if (tab[pos].key == key && ref_valid(tab[pos].ref))
            return (uint32_t)pos;
        pos = (pos + 1) & (cap - 1);
    }
    return 0; // unreachable: every row's key was inserted
}

__device__ __forceinline__ void copy_row(const Cols & src, uint64_t si, const Cols & dst, uint64_t di)
{
    dst.keys[di] = src.keys[si];
    for (uint32_t c = 0; c < src.n; ++c)
        copy_elem(dst.col[c], di, src.col[c], si, src.width[c]);
}

// One CTA per leaf.  Rows of one key become contiguous in `dst`; the key's
// cell then holds {row count, first row} (block_no, which is always 0 for
// the single partitioned build block, carries the count), and the
// next-chain runs last -> ... -> first.  Leaves without repeated keys are
// copied unchanged.
__global__ void __launch_bounds__(kBuildNT) k_group_leaf(const __grid_constant__ Cols src, const __grid_constant__ Cols dst,
                                                         const uint32_t * __restrict__ leaf_off, const LeafMeta * __restrict__ meta,
                                                         Cell * __restrict__ cells, uint64_t * __restrict__ next)
{
    extern __shared__ uint32_t gsh[]; // cnt[cap] | start[cap] | fill[cap] | cell of each row[cap]
    __shared__ uint32_t warp_sums[kBuildNT / 32];
    const uint32_t l = blockIdx.x;
    const uint32_t r0 = leaf_off[l], r = leaf_off[l + 1] - r0;
    if (r == 0)
        return;
    const LeafMeta m = meta[l];
    if (!m.dup)
    {
        for (uint32_t i = threadIdx.x; i < r; i += kBuildNT)
            copy_row(src, r0 + i, dst, r0 + i);
        return;
    }
    const uint32_t cap = 1u << m.log2cap;
    Cell * tab = cells + m.table_off;
    uint32_t * cnt = gsh;
    uint32_t * start = gsh + cap;
    uint32_t * fill = gsh + 2 * cap;
    uint32_t * rowcell = gsh + 3 * cap; // a leaf has at most cap rows
    for (uint32_t i = threadIdx.x; i < cap; i += kBuildNT)
        cnt[i] = 0;
    __syncthreads();
    // each row's cell, found once and kept for the placement below
    for (uint32_t i = threadIdx.x; i < r; i += kBuildNT)
    {
        const uint64_t k = src.keys[r0 + i];
        const uint32_t c = cell_of(tab, cap, int_hash64(k), k);
        rowcell[i] = c;
        atomicAdd(&cnt[c], 1u);
    }
    __syncthreads();
    // one block scan: thread t owns cells [t * per, (t + 1) * per)
    const uint32_t per = (cap + kBuildNT - 1) / kBuildNT;
    const uint32_t c0 = threadIdx.x * per;
    uint32_t local = 0;
    for (uint32_t j = 0; j < per; ++j)
        if (c0 + j < cap)
            local += cnt[c0 + j];
    uint32_t tot;
    uint32_t run = block_excl_scan<kBuildNT>(local, warp_sums, &tot);
    for (uint32_t j = 0; j < per; ++j)
        if (c0 + j < cap)
        {
            const uint32_t c = c0 + j, v = cnt[c];
            start[c] = run;
            fill[c] = run;
            if (v)
                tab[c].ref = make_ref(v, r0 + run);
            run += v;
        }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < r; i += kBuildNT)
    {
        const uint32_t c = rowcell[i];
        const uint32_t slot = atomicAdd(&fill[c], 1u);
        const uint64_t pos = (uint64_t)r0 + slot;
        copy_row(src, r0 + i, dst, pos);
        next[pos] = slot > start[c] ? make_ref(0, (uint32_t)(pos - 1)) : INVALID_REF;
    }
}

// ---- CHJ --------------------------------------------------------------------

__global__ void k_slot_hist(const uint64_t * __restrict__ keys, uint64_t n, uint32_t slot_bits, uint32_t * __restrict__ counts)
{
    extern __shared__ uint32_t bins[];
    const uint32_t nb = 1u << slot_bits;
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x)
        bins[i] = 0;
    __syncthreads();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&bins[int_hash64(keys[i]) >> (64 - slot_bits)], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x)
        if (bins[i])
            atomicAdd(&counts[i], bins[i]);
}

__global__ void k_slot_meta(const uint32_t * __restrict__ counts, const uint32_t * __restrict__ table_off, uint32_t n_slots, LeafMeta * __restrict__ meta)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_slots)
        return;
    const uint64_t cap = table_off[s + 1] - table_off[s];
    meta[s] = LeafMeta{table_off[s], 0u, cap ? (uint8_t)log2u(cap) : (uint8_t)0, (uint8_t)(counts[s] != 0), 0, 0};
}

__global__ void k_fill_empty(Cell * __restrict__ cells, uint64_t n)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        reinterpret_cast<ulonglong2 *>(cells)[i] = make_ulonglong2(0ull, INVALID_REF);
}

__device__ __forceinline__ uint32_t block_of_row(uint64_t g, const uint64_t * __restrict__ block_off, uint32_t n_blocks, uint32_t uniform)
{
    if (uniform)
        return (uint32_t)(g / uniform);
    uint32_t lo = 0, hi = n_blocks; // block_off[lo] <= g < block_off[hi]
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (block_off[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_chj_insert(const uint64_t * __restrict__ keys, uint64_t n, uint32_t slot_bits, const uint64_t * __restrict__ block_off,
                             uint32_t n_blocks, uint32_t uniform, Cell * __restrict__ cells, LeafMeta * __restrict__ meta, uint64_t * __restrict__ next,
                             int * __restrict__ any_dup)
{
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint64_t k = keys[g];
        const uint64_t h = int_hash64(k);
        const uint32_t s = (uint32_t)(h >> (64 - slot_bits));
        const uint32_t b = block_of_row(g, block_off, n_blocks, uniform);
        const uint32_t row = (uint32_t)(g - block_off[b]);
        const LeafMeta m = meta[s];
        const uint64_t prev = table_insert<false>(cells + m.table_off, 1ull << m.log2cap, h, k, make_ref(b, row));
        next[g] = prev;
        // flags read before they are written: a repeated key must not make
        // every thread store to the same two addresses
        if (ref_valid(prev))
        {
            if (!*reinterpret_cast<volatile uint8_t *>(&meta[s].dup))
                meta[s].dup = 1;
            if (!*reinterpret_cast<volatile int *>(any_dup))
                *any_dup = 1;
        }
    }
}
} // namespace

void set_build_smem_limits(int smem_optin)
{
    const size_t need = (size_t)kSmemCellsMax * sizeof(Cell);
    PHJ_CUDA(cudaFuncSetAttribute(k_build_leaf<kBuildNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(need, (size_t)smem_optin - 1024)));
    PHJ_CUDA(cudaFuncSetAttribute(k_build_leaf<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::min<size_t>(need, (size_t)smem_optin - 1024)));
    PHJ_CUDA(cudaFuncSetAttribute(k_group_leaf, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::min<size_t>((size_t)kSmemCellsMax * 16, (size_t)smem_optin - 1024)));
}

bool group_leaf_duplicates(phj_ctx * ctx, const Cols & src, const Cols & dst, const uint32_t * leaf_off, uint32_t n_leaves, const LeafTables & lt)
{
    const uint64_t max_cap = lt.max_rows ? table_cells(lt.max_rows, ctx->table_cap_pct) : 1;
    if (!lt.any_dup || max_cap > kSmemCellsMax || lt.state)
        return false;
    uint64_t row_bytes = 8;
    for (uint32_t c = 0; c < src.n; ++c)
        row_bytes += src.width[c];
    KTimer kt(ctx, "group_leaf", 0, 0);
    k_group_leaf<<<n_leaves, kBuildNT, (size_t)max_cap * 16, ctx->stream>>>(src, dst, leaf_off, lt.meta, lt.cells, lt.next);
    PHJ_LAUNCHED(ctx, "group_leaf");
    (void)row_bytes;
    return true;
}

// Lazy layout (PHJ/BEP): the directory says where each leaf's table lives;
// the cells are built on first use by the probe (state NOT_BUILT).
__global__ void k_leaf_plan(const uint32_t * __restrict__ leaf_off, const uint32_t * __restrict__ table_off, int ulog, uint32_t n_leaves,
                            LeafMeta * __restrict__ meta)
{
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n_leaves)
        return;
    const uint32_t r0 = leaf_off[l], r = leaf_off[l + 1] - r0;
    const uint64_t t0 = ulog >= 0 ? ((uint64_t)l << ulog) : table_off[l];
    const uint64_t cap = ulog >= 0 ? (1ull << ulog) : table_off[l + 1] - t0;
    (void)r;
    meta[l] = LeafMeta{t0, r0, cap ? (uint8_t)log2u(cap) : (uint8_t)0, (uint8_t)(cap != 0), 1, 0};
}

void build_leaf_tables(phj_ctx * ctx, Scratch & s, const Cols & build_part, const uint32_t * leaf_off, uint32_t n_leaves, LeafTables & lt,
                       bool lazy)
{
    uint32_t * caps = s.get<uint32_t>(n_leaves + 1);
    uint32_t * table_off = s.get<uint32_t>(n_leaves + 1);
    uint32_t * small = s.get<uint32_t>(4); // [0] max rows, [1] any dup
    PHJ_CUDA(cudaMemsetAsync(small, 0, 4 * sizeof(uint32_t), ctx->stream));
    k_leaf_caps<<<(unsigned)ceil_div(n_leaves, 256), 256, 0, ctx->stream>>>(leaf_off, n_leaves, ctx->table_cap_pct, caps, small);
    PHJ_LAUNCHED(ctx, "leaf_caps");
    scan_u32(ctx, s, caps, table_off, n_leaves);
    uint32_t host[2] = {0, 0};
    read_small(ctx, {{&host[0], small, sizeof(uint32_t)}, {&host[1], table_off + n_leaves, sizeof(uint32_t)}});
    lt.max_rows = host[0];
    // at least one aligned cell pair: the probe's first load reads two cells
    const uint64_t max_cap = lt.max_rows ? table_cells(lt.max_rows, ctx->table_cap_pct) : 2;
    // Uniform capacity (the largest leaf's) lets the probe compute a table's
    // address from the leaf id alone; it is used unless it costs more than
    // 1.5x the cells of per-leaf sizing.
    const uint64_t uniform_cells = (uint64_t)n_leaves * max_cap;
    const bool uniform = uniform_cells <= (3 * (uint64_t)host[1]) / 2 + n_leaves;
    lt.uniform_log2cap = uniform ? (int)(63 - __builtin_clzll(max_cap)) : -1;
    lt.total_cells = uniform ? uniform_cells : host[1];
    lt.meta = s.get<LeafMeta>(n_leaves);
    lt.cells = s.get<Cell>(lt.total_cells);
    if (lazy)
    {
        lt.state = s.get<uint32_t>(n_leaves);
        PHJ_CUDA(cudaMemsetAsync(lt.state, 0, (size_t)n_leaves * sizeof(uint32_t), ctx->stream));
        k_leaf_plan<<<(unsigned)ceil_div(n_leaves, 256), 256, 0, ctx->stream>>>(leaf_off, table_off, lt.uniform_log2cap, n_leaves, lt.meta);
        PHJ_LAUNCHED(ctx, "leaf_plan");
        lt.any_dup = 1; // unknown until the tables are built: chains are followed
        return;
    }
    // Tables are built in shared memory and copied out when two CTAs fit
    // on an SM; larger ones (one resident CTA per SM would leave the SMs
    // idling through each leaf's copy-out) are built in place, in global
    // memory that stays in L2 (1M x 8M, 256 leaves of 8192 cells: 0.310 ->
    // 0.304 ms a join).
    const uint32_t smem_cells =
        max_cap * sizeof(Cell) * 2 <= ctx->smem_optin ? (uint32_t)std::min<uint64_t>(max_cap, kSmemCellsMax) : 0u;
    int * any_dup = reinterpret_cast<int *>(small + 1);
    {
        KTimer kt(ctx, "build_leaf_tables", 0, 0);
        // leaves of more than 1024 rows get 1024 threads
        auto kb = lt.max_rows > 1024 ? k_build_leaf<1024> : k_build_leaf<kBuildNT>;
        kb<<<n_leaves, lt.max_rows > 1024 ? 1024 : kBuildNT, (size_t)smem_cells * sizeof(Cell), ctx->stream>>>(build_part.keys, leaf_off, table_off, lt.uniform_log2cap,
                                                                                            smem_cells, lt.cells, lt.next, lt.meta, any_dup);
        PHJ_LAUNCHED(ctx, "build_leaf");
    }
    read_small(ctx, {{&lt.any_dup, any_dup, sizeof(int)}});
}

void build_global_table(phj_ctx * ctx, Scratch & s, const phj_table & build, uint32_t slot_bits, LeafTables & lt)
{
    const uint32_t n_slots = 1u << slot_bits;
    uint32_t * counts = s.get<uint32_t>(n_slots + 1);
    uint32_t * caps = s.get<uint32_t>(n_slots + 1);
    uint32_t * table_off = s.get<uint32_t>(n_slots + 1);
    int * any_dup = s.get<int>(1);
    PHJ_CUDA(cudaMemsetAsync(counts, 0, (n_slots + 1) * sizeof(uint32_t), ctx->stream));
    PHJ_CUDA(cudaMemsetAsync(any_dup, 0, sizeof(int), ctx->stream));
    const uint64_t n = build.rows;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(n, 256), (uint64_t)ctx->num_sms * 8));
    {
        KTimer kt(ctx, "chj_slot_hist", n, n * 8);
        k_slot_hist<<<grid, 256, n_slots * sizeof(uint32_t), ctx->stream>>>(build.keys, n, slot_bits, counts);
        PHJ_LAUNCHED(ctx, "chj_slot_hist");
    }
    uint32_t * max_rows = s.get<uint32_t>(1);
    PHJ_CUDA(cudaMemsetAsync(max_rows, 0, sizeof(uint32_t), ctx->stream));
    // counts -> capacities -> offsets: the offsets of leaf_off-style caps
    // reuse k_leaf_caps on a prefix of the counts.
    uint32_t * cnt_off = s.get<uint32_t>(n_slots + 1);
    scan_u32(ctx, s, counts, cnt_off, n_slots);
    k_leaf_caps<<<(unsigned)ceil_div(n_slots, 256), 256, 0, ctx->stream>>>(cnt_off, n_slots, 200u, caps, max_rows);
    PHJ_LAUNCHED(ctx, "chj_caps");
    scan_u32(ctx, s, caps, table_off, n_slots);
    uint32_t total = 0;
    read_small(ctx, {{&total, table_off + n_slots, sizeof(uint32_t)}});
    lt.total_cells = total;
    lt.meta = s.get<LeafMeta>(n_slots);
    lt.cells = s.get<Cell>(total);
    k_slot_meta<<<(unsigned)ceil_div(n_slots, 256), 256, 0, ctx->stream>>>(counts, table_off, n_slots, lt.meta);
    PHJ_LAUNCHED(ctx, "chj_meta");
    {
        KTimer kt(ctx, "chj_fill", 0, total * 16ull);
        k_fill_empty<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(total, 256), (uint64_t)ctx->num_sms * 16)), 256, 0, ctx->stream>>>(
            lt.cells, total);
        PHJ_LAUNCHED(ctx, "chj_fill");
    }
    {
        KTimer kt(ctx, "chj_insert", n, n * 16);
        k_chj_insert<<<grid, 256, 0, ctx->stream>>>(build.keys, n, slot_bits, build.block_off, build.n_blocks, build.uniform_block_rows, lt.cells,
                                                   lt.meta, lt.next, any_dup);
        PHJ_LAUNCHED(ctx, "chj_insert");
    }
    read_small(ctx, {{&lt.any_dup, any_dup, sizeof(int)}});
}

} // namespace phjg
