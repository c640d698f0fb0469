// bep_engine.cu -- PHJ (best-effort partitioning, src/PHJBep.cpp:113-790)
// with the probe side's byte budget kept on the device.
//
// One persistent grid, one CTA per SM; each CTA is one of the reference's
// workers (a "CTA group") with its own contiguous slice of the probe input
// and its own share of the budget (bep_budget_mib / groups).  Probe rows
// live in fixed-size blocks of `page` rows (column-major inside a block)
// taken from one device pool through a free-block stack.
//
// The grid runs in waves separated by grid-wide barriers:
//   S  each group scatters the next tile of its slice by the first radix
//      pass into its private pass-1 bucket chains (the reference's
//      per-worker `unrefined` chains) and adds the tile's bytes to its
//      unrefined count.  At the per-group high water (half the group's
//      budget) it refines its largest bucket, again and again until the
//      count is below the low water (a quarter): refining a bucket sorts
//      each of its blocks by leaf (passes 2..N) in shared memory and
//      publishes the block as a refined block of that bucket; the rows go
//      to the per-leaf counts (leaf_rows) and to the global leaf count.
//      (src/PHJBep.cpp:397-450 refinePartition, :508-528 evictAsNeeded
//      phase 1, :582-605 the main loop.)
//   E  when the global leaf bytes reach the leaf high water (5/8 of the
//      budget), the round-robin eviction cursor (next_evict_leaf) advances
//      over the leaves until the leaves it passed hold enough rows to take
//      the global count below the low water (5/8 of the high water); each
//      leaf passed is claimed with a CAS on its lock word and counted as an
//      eviction when it held rows; the claimed leaves whose table is
//      NOT_BUILT are built (NOT_BUILT -> BUILDING by CAS, BUILT when done; a
//      leaf found BUILDING is waited for, bounded); then every refined
//      block's rows of the claimed leaves are probed and projected, the
//      blocks in bucket order so one bucket's leaf tables stay in L2; a
//      block whose rows are all probed goes back to the pool.
//      (src/PHJBep.cpp:453-505 tryEvictOneLeaf, :530-571 phase 2.)
// After the last input wave every group refines what it still holds
// (:662-676), and a final E over all leaves drains the rest (the post-probe
// drain, :689-727).  The reference's cooperative end-of-slice drain
// (:619-655) has no separate form: the slices are equal and every group
// takes part in every E, so no group idles while another scatters.
//
// Counters as the reference defines them (src/PHJBep.h:13-39): evictions
// (leaves that held rows when claimed), refinements (bucket refines), peak
// (the largest global leaf bytes, seen after each wave's refines), skip
// retries (claims that found the leaf locked, and waits on a BUILDING leaf).
//
// Every wait is bounded: the grid barrier and the BUILDING wait give up
// after the context's wait limit, set an error code and end the grid.  A
// group that finds too few free blocks for its tile refines what it holds
// and the wave ends in a drain of every leaf (which frees every refined
// block); a second shortage right after such a drain ends the grid with a
// capacity error.  Each group takes its free blocks from a cache of its own,
// refilled from the pool's stack a batch at a time.
//
// Pool blocks, control words, per-leaf and per-block state and the lazily
// built tables are written by one group and read by others during the
// launch, so they are read through L2 (ld.global.cg): an SM's L1 may hold
// an older copy of the line.
#include "internal.h"

#include <cstdio>
#include <cstdlib>

namespace phjg
{
namespace
{
constexpr int kENT = 1024; // threads of a group's CTA
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kNotBuilt = 0, kBuilding = 1, kBuilt = 2, kBuiltDup = 3;

// error codes written to the context's error word
constexpr int kErrWait = 4;    // a BUILDING leaf was not published in time
constexpr int kErrBarrier = 5; // a grid barrier was not reached in time
constexpr int kErrPool = 6;    // the block pool ran out
constexpr int kErrChain = 7;   // a bucket chain outgrew its directory

struct EngineCtl
{
    unsigned int bar_count;
    unsigned int bar_gen;
    int abort;
    int evict_now;
    unsigned long long global_leaf_rows;
    unsigned long long peak_leaf_rows;
    unsigned long long cursor;   // next_evict_leaf, counted in leaves (mod n_leaves)
    unsigned long long ev_lo;    // the current E's range of cursor positions [ev_lo, ev_lo + ev_len)
    unsigned long long ev_len;
    unsigned long long out_rows; // output rows placed (the exact total, also past capacity)
    long long free_top;          // blocks on the free stack
    unsigned int work_n;
    unsigned int build_n, build_next;
    unsigned long long work_next;
    unsigned long long evictions, refinements, skip_retries, tables_built, evict_phases;
    unsigned long long ns_shuffle, ns_evict, ns_probe; // group 0's time in S, E bookkeeping, E probing
    unsigned long long rows_scattered, rows_refined, rows_probed, rows_claimed; // row totals per step (checks)
    unsigned int groups_done; // groups whose slice is scattered
    int more_input;           // some group still has input (decided at each wave's barrier)
    int pool_low;             // a group found too few free blocks for its tile this wave
    int forced_last;          // the previous E was a drain forced by a low pool
    int any_dup;              // some leaf built so far has a repeated key
    unsigned long long forced_drains;
    unsigned long long wave_s_max, ns_s_crit; // the slowest group's S time this wave; summed over waves
    unsigned long long ns_refine0, tiles0, blocks0; // group 0: time refining, tiles scattered, blocks refined
};

static_assert(sizeof(EngineCtl) + 8 <= kSmallReadBytes, "the control block and the error word are read back in one small read");

struct EngineArgs
{
    Cols pin; // probe side in input order
    uint64_t probe_rows;
    Cols bpart; // leaf-partitioned build side (keys and payloads)
    uint32_t * state;
    LeafMeta * meta;
    Cell * cells;
    uint64_t * next;
    const uint32_t * leaf_off;
    int ulog;            // >= 0: uniform tables of 2^ulog cells at leaf << ulog
    uint32_t smem_cells; // tables up to this many cells are built in shared memory
    uint32_t b1;         // first-pass bits
    uint32_t total_bits; // leaf bits
    uint32_t lb_log2;    // leaf-in-bucket bits (total_bits - b1)
    uint32_t n_leaves, n_buckets;
    // blocks of `page` rows: keys at 0, payload column c at col_off[c]
    uint8_t * pool;
    uint32_t page_log2;
    uint64_t block_bytes;
    uint32_t col_off[kMaxCols];
    uint32_t n_blocks;
    uint32_t * free_stack;
    uint32_t * blk_state; // refined and holding unprobed rows: its bucket; otherwise kNone
    uint32_t * blk_rows;
    uint32_t * blk_rem;
    uint32_t * blk_bucket; // the bucket of a refined block (kept after the block is freed)
    uint32_t * blk_lfirst; // leaf-in-bucket of a refined block's first and last row
    uint32_t * blk_llast;
    // the eviction cursor when the block was refined: the block's rows of
    // leaf L are probed when the cursor first passes L after that point
    unsigned long long * blk_c0;
    uint32_t * chain; // [group][bucket][maxb] block ids of the unrefined chains
    uint32_t maxb;
    uint32_t * leaf_rows; // unprobed refined rows per leaf
    uint32_t * leaf_lock;
    uint32_t * bucket_cnt;  // E: refined blocks per bucket, then their first work slot
    uint32_t * bucket_fill; // E: work slots taken per bucket
    uint32_t * work;        // E: refined blocks to probe, bucket by bucket
    uint32_t * build_queue; // E: claimed leaves to build
    // budget, bytes (src/PHJBep.cpp:186-190)
    uint64_t unref_high, unref_low, leaf_high, leaf_low;
    uint32_t rb;        // bytes of a probe row
    uint64_t tile_rows; // input rows a group scatters per wave
    uint32_t waves;
    // output
    uint64_t * out_keys;
    void * out_l[kMaxCols];
    void * out_r[kMaxCols];
    uint64_t out_cap;
    uint64_t wait_limit_ns;
    uint32_t test_stall_wave; // test hook: group 0 holds back from this wave's barrier (kNone: off)
    EngineCtl * ctl;
    int * err;
};

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const unsigned int * p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void fail(const EngineArgs & a, int code)
{
    atomicExch(&a.ctl->abort, code);
    atomicExch(a.err, code);
}

__device__ __forceinline__ bool aborted(const EngineArgs & a)
{
    return *reinterpret_cast<volatile int *>(&a.ctl->abort) != 0;
}

template <class T>
__device__ __forceinline__ T vload(const T * p)
{
    return *reinterpret_cast<const volatile T *>(p);
}

__device__ __forceinline__ uint64_t umin64(uint64_t x, uint64_t y) { return x < y ? x : y; }

// Element src_i of a pool column (read through L2) to element dst_i of an
// output column of the same width (a streaming store: output rows are not
// read again, so they should not push pool pages and tables out of L2).
__device__ __forceinline__ void copy_elem_cg(void * dst, uint64_t dst_i, const void * src, uint64_t src_i, uint32_t w)
{
    switch (w)
    {
        case 1: __stcs(static_cast<unsigned char *>(dst) + dst_i, (unsigned char)__ldcg(static_cast<const signed char *>(src) + src_i)); break;
        case 2: __stcs(static_cast<unsigned short *>(dst) + dst_i, __ldcg(static_cast<const unsigned short *>(src) + src_i)); break;
        case 4: __stcs(static_cast<unsigned int *>(dst) + dst_i, __ldcg(static_cast<const unsigned int *>(src) + src_i)); break;
        case 8: __stcs(static_cast<unsigned long long *>(dst) + dst_i, __ldcg(static_cast<const unsigned long long *>(src) + src_i)); break;
        default: __stcs(static_cast<uint4 *>(dst) + dst_i, __ldcg(static_cast<const uint4 *>(src) + src_i)); break;
    }
}

// Element src_i of a build payload column (written before the launch) to
// element dst_i of an output column, with a streaming store.
__device__ __forceinline__ void copy_elem_out(void * dst, uint64_t dst_i, const void * src, uint64_t src_i, uint32_t w)
{
    switch (w)
    {
        case 1: __stcs(static_cast<unsigned char *>(dst) + dst_i, __ldg(static_cast<const unsigned char *>(src) + src_i)); break;
        case 2: __stcs(static_cast<unsigned short *>(dst) + dst_i, __ldg(static_cast<const unsigned short *>(src) + src_i)); break;
        case 4: __stcs(static_cast<unsigned int *>(dst) + dst_i, __ldg(static_cast<const unsigned int *>(src) + src_i)); break;
        case 8: __stcs(static_cast<unsigned long long *>(dst) + dst_i, __ldg(static_cast<const unsigned long long *>(src) + src_i)); break;
        default: __stcs(static_cast<uint4 *>(dst) + dst_i, __ldg(static_cast<const uint4 *>(src) + src_i)); break;
    }
}

// Grid-wide barrier (every group is resident: cooperative launch).  The
// last group to arrive runs `last` before it releases the others.  A wait
// longer than the context's limit ends the grid with kErrBarrier.  Returns
// false when the grid is ending.
template <class F>
__device__ bool grid_sync(const EngineArgs & a, uint32_t & gen, F last)
{
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const uint32_t target = gen + 1;
        __threadfence();
        const uint32_t arrived = atomicAdd(&a.ctl->bar_count, 1u);
        if (arrived == gridDim.x - 1)
        {
            a.ctl->bar_count = 0;
            last();
            __threadfence();
            atomicExch(&a.ctl->bar_gen, target);
        }
        else
        {
            const uint64_t t0 = now_ns();
            uint32_t spins = 0;
            while (ld_acquire_u32(&a.ctl->bar_gen) != target)
            {
                if (aborted(a))
                    break;
                if ((++spins & 255u) == 0 && now_ns() - t0 > a.wait_limit_ns)
                {
                    fail(a, kErrBarrier);
                    break;
                }
                __nanosleep(64);
            }
        }
        gen = target;
        __threadfence();
    }
    __syncthreads();
    return !aborted(a);
}

struct NoOp
{
    __device__ void operator()() const {}
};

// Block-wide exclusive scan over `n` u32 bins in shared memory (in place);
// returns the total.  `ws` holds kENT/32 words.
__device__ uint32_t scan_bins(uint32_t * bins, uint32_t n, uint32_t * ws)
{
    const uint32_t per = (n + kENT - 1) / kENT;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < n)
            sum += bins[b0 + i];
    uint32_t total;
    const uint32_t excl = block_excl_scan<kENT>(sum, ws, &total);
    uint32_t run = excl;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < n)
        {
            const uint32_t v = bins[b0 + i];
            bins[b0 + i] = run;
            run += v;
        }
    __syncthreads();
    return total;
}

__device__ __forceinline__ uint8_t * block_ptr(const EngineArgs & a, uint32_t blk)
{
    return a.pool + (uint64_t)blk * a.block_bytes;
}

// Copies row `src_i` of a column-major tile in shared memory (keys at 0,
// payload c at col_off[c]) to row `dst_i` of a block of the same layout.
__device__ __forceinline__ void copy_row(const EngineArgs & a, uint8_t * dst, uint32_t dst_i, const uint8_t * src, uint32_t src_i)
{
    reinterpret_cast<uint64_t *>(dst)[dst_i] = reinterpret_cast<const uint64_t *>(src)[src_i];
    for (uint32_t c = 0; c < a.pin.n; ++c)
        copy_elem(dst + a.col_off[c], dst_i, src + a.col_off[c], src_i, a.pin.width[c]);
}

// Column c of rows i0 + u * kENT + threadIdx.x (u < 4, below n) from `src`
// (row r0 + i) into the stage column `dst`: the four loads are issued
// before any store.  kL2: the source was written during this launch (read
// through L2).
template <class T, bool kL2>
__device__ __forceinline__ void stage4(T * dst, const T * src, uint64_t r0, uint32_t i0, uint32_t n)
{
    T v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
    {
        const uint32_t i = i0 + u * kENT + threadIdx.x;
        if (i < n)
            v[u] = kL2 ? __ldcg(src + r0 + i) : __ldcs(src + r0 + i); // the input is read once
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
    {
        const uint32_t i = i0 + u * kENT + threadIdx.x;
        if (i < n)
            dst[i] = v[u];
    }
}

template <bool kL2>
__device__ __forceinline__ void stage4_column(void * dst, const void * src, uint64_t r0, uint32_t i0, uint32_t n, uint32_t w)
{
    switch (w)
    {
        case 1: stage4<unsigned char, kL2>(static_cast<unsigned char *>(dst), static_cast<const unsigned char *>(src), r0, i0, n); break;
        case 2: stage4<unsigned short, kL2>(static_cast<unsigned short *>(dst), static_cast<const unsigned short *>(src), r0, i0, n); break;
        case 4: stage4<unsigned int, kL2>(static_cast<unsigned int *>(dst), static_cast<const unsigned int *>(src), r0, i0, n); break;
        case 8: stage4<unsigned long long, kL2>(static_cast<unsigned long long *>(dst), static_cast<const unsigned long long *>(src), r0, i0, n); break;
        default: stage4<uint4, kL2>(static_cast<uint4 *>(dst), static_cast<const uint4 *>(src), r0, i0, n); break;
    }
}

struct Smem
{
    uint8_t * stage;  // page rows in the block layout; the leaf builds' cells
    uint16_t * perm;  // page entries
    uint16_t * src;   // page entries: the stage row of each sorted position
    uint32_t * bins;  // max(buckets, leaves per bucket, page) entries
    uint32_t * boff;  // buckets: scatter offsets
    uint32_t * nbpre; // buckets: new blocks per bucket, then their prefix
    uint32_t * fill;  // buckets: rows in each chain's last block (page: no block)
    uint32_t * clen;  // buckets: blocks in each chain
    uint32_t * urows; // buckets: unrefined rows per bucket
    uint32_t * acc;   // leaves per bucket: rows a refine adds to each leaf
    uint32_t * bcache; // the group's free blocks: 2 x buckets + 2 x kRefill entries
    uint32_t * ws;    // scan scratch (kENT / 32 words)
    uint32_t * scal;  // scalars (32 words, 8-byte aligned)
};

// ---------------------------------------------------------------------------
// S: scatter `n` (<= page) input rows from `r0` into the group's chains.
// ---------------------------------------------------------------------------
constexpr int kTileDone = 0, kTileNoRoom = 1, kTileFailed = 2;
constexpr uint32_t kRefill = 64; // free blocks a group takes beyond its need

// Returns kTileDone, kTileNoRoom (too few free blocks: nothing done) or
// kTileFailed (the grid is ending).  sm.bins[0, buckets) is zero on entry
// and on a kTileDone return.
__device__ int scatter_tile(const EngineArgs & a, const Smem & sm, uint32_t g, uint64_t r0, uint32_t n)
{
    const uint32_t page = 1u << a.page_log2;
    const uint32_t P1 = a.n_buckets;
    // the tile into the stage in input order (one read of the input), and
    // the first-pass bucket of every row
    for (uint32_t i0 = 0; i0 < n; i0 += 4 * kENT)
    {
        uint64_t k[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const uint32_t i = i0 + u * kENT + threadIdx.x;
            k[u] = i < n ? __ldcs(a.pin.keys + r0 + i) : 0ull;
        }
        for (uint32_t c = 0; c < a.pin.n; ++c)
            stage4_column<false>(sm.stage + a.col_off[c], a.pin.col[c], r0, i0, n, a.pin.width[c]);
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const uint32_t i = i0 + u * kENT + threadIdx.x;
            if (i < n)
            {
                reinterpret_cast<uint64_t *>(sm.stage)[i] = k[u];
                const uint32_t p = (uint32_t)(int_hash64(k[u]) >> (64u - a.b1));
                sm.perm[i] = (uint16_t)p;
                atomicAdd(&sm.bins[p], 1u);
            }
        }
    }
    __syncthreads();
    // per bucket its rows (high half) and the blocks its chain needs (low
    // half; an empty chain counts as a full last block), scanned at once
    for (uint32_t p = threadIdx.x; p < P1; p += kENT)
    {
        const uint32_t c = sm.bins[p];
        const uint32_t nb = c == 0 ? 0u : (sm.fill[p] + c + page - 1) / page - 1u;
        sm.boff[p] = (c << 16) | nb;
    }
    __syncthreads();
    const uint32_t tot = scan_bins(sm.boff, P1, sm.ws);
    const uint32_t nb_total = tot & 0xFFFFu;
    // blocks come from the group's cache of free blocks (sm.bcache, its
    // length in scal[16]), refilled from the pool's stack kRefill blocks
    // beyond the need at a time, so the groups rarely meet on the stack
    if (threadIdx.x == 0)
    {
        sm.scal[0] = 0;
        sm.scal[1] = 0;
        sm.scal[2] = 0;
        const uint32_t have = sm.scal[16];
        if (nb_total > have)
        {
            const uint32_t need = nb_total - have, want = need + kRefill;
            unsigned long long * top = reinterpret_cast<unsigned long long *>(&a.ctl->free_top);
            long long cur = (long long)vload(top);
            for (;;)
            {
                const long long take = cur >= (long long)want ? (long long)want : (cur >= (long long)need ? cur : 0);
                if (take == 0)
                {
                    sm.scal[0] = 2; // too few free blocks
                    break;
                }
                const long long seen = (long long)atomicCAS(top, (unsigned long long)cur, (unsigned long long)(cur - take));
                if (seen == cur)
                {
                    sm.scal[1] = (uint32_t)(cur - take);
                    sm.scal[2] = (uint32_t)take;
                    break;
                }
                cur = seen;
            }
        }
    }
    __syncthreads();
    if (sm.scal[0])
    {
        for (uint32_t p = threadIdx.x; p < P1; p += kENT)
            sm.bins[p] = 0;
        __syncthreads();
        return kTileNoRoom;
    }
    if (sm.scal[2])
    {
        const uint32_t have = sm.scal[16];
        for (uint32_t i = threadIdx.x; i < sm.scal[2]; i += kENT)
            sm.bcache[have + i] = __ldcg(a.free_stack + sm.scal[1] + i);
        __syncthreads();
        if (threadIdx.x == 0)
            sm.scal[16] = have + sm.scal[2];
        __syncthreads();
    }
    const uint32_t cache_base = sm.scal[16] - nb_total; // this tile's blocks: bcache[cache_base, +nb_total)
    // new blocks onto the chains; the cursors of the sorted tile
    for (uint32_t p = threadIdx.x; p < P1; p += kENT)
    {
        const uint32_t off = sm.boff[p] >> 16, nb0 = sm.boff[p] & 0xFFFFu;
        const uint32_t nb = ((p + 1 < P1 ? sm.boff[p + 1] : tot) & 0xFFFFu) - nb0;
        sm.bins[p] = off;
        if (nb == 0)
            continue;
        const uint32_t len = sm.clen[p];
        if (len + nb > a.maxb)
        {
            fail(a, kErrChain);
            sm.scal[0] = 1;
            continue;
        }
        uint32_t * ch = a.chain + ((uint64_t)g * P1 + p) * a.maxb;
        for (uint32_t j = 0; j < nb; ++j)
            ch[len + j] = sm.bcache[cache_base + nb0 + j];
    }
    __syncthreads();
    if (sm.scal[0])
        return kTileFailed;
    if (threadIdx.x == 0)
        sm.scal[16] = cache_base; // read by no thread before the next tile's syncs
    // the stage row of every sorted position
    for (uint32_t i = threadIdx.x; i < n; i += kENT)
        sm.src[atomicAdd(&sm.bins[sm.perm[i]], 1u)] = (uint16_t)i;
    __syncthreads();
    // the rows out to the chains' blocks in sorted order: consecutive rows
    // of a bucket go to consecutive rows of its blocks
    for (uint32_t s = threadIdx.x; s < n; s += kENT)
    {
        const uint32_t r = sm.src[s];
        const uint64_t key = reinterpret_cast<const uint64_t *>(sm.stage)[r];
        const uint32_t p = (uint32_t)(int_hash64(key) >> (64u - a.b1));
        const uint32_t q = sm.fill[p] + (s - (sm.boff[p] >> 16)); // slot counted from the chain's last block
        const uint32_t idx = sm.clen[p] + (q >> a.page_log2) - 1u;
        const uint32_t blk = a.chain[((uint64_t)g * P1 + p) * a.maxb + idx];
        copy_row(a, block_ptr(a, blk), q & (page - 1), sm.stage, r);
    }
    __syncthreads();
    for (uint32_t p = threadIdx.x; p < P1; p += kENT)
    {
        sm.bins[p] = 0;
        const uint32_t c = (sm.boff[p + 1 < P1 ? p + 1 : p] >> 16) - (sm.boff[p] >> 16);
        const uint32_t cnt = p + 1 < P1 ? c : n - (sm.boff[p] >> 16);
        if (cnt == 0)
            continue;
        const uint32_t nb = ((p + 1 < P1 ? sm.boff[p + 1] : tot) & 0xFFFFu) - (sm.boff[p] & 0xFFFFu);
        sm.fill[p] = ((sm.fill[p] + cnt - 1) & (page - 1)) + 1;
        sm.clen[p] += nb;
        sm.urows[p] += cnt;
    }
    __syncthreads();
    return kTileDone;
}

// ---------------------------------------------------------------------------
// S: refine bucket p of group g -- each block of its chain sorted by leaf
// in place and published as a refined block.  Returns the rows refined.
// ---------------------------------------------------------------------------
__device__ uint32_t refine_bucket(const EngineArgs & a, const Smem & sm, uint32_t g, uint32_t p)
{
    const uint32_t page = 1u << a.page_log2;
    const uint32_t LB = 1u << a.lb_log2;
    const uint32_t len = sm.clen[p], rows = sm.urows[p];
    const uint32_t * ch = a.chain + ((uint64_t)g * a.n_buckets + p) * a.maxb;
    const uint32_t shift = 64u - a.total_bits;
    // the rows each leaf gains, summed over the bucket's blocks
    for (uint32_t l = threadIdx.x; l < LB; l += kENT)
        sm.acc[l] = 0;
    for (uint32_t j = 0; j < len; ++j)
    {
        const uint32_t blk = ch[j];
        const uint32_t n = j + 1 == len ? sm.fill[p] : page;
        uint8_t * B = block_ptr(a, blk);
        for (uint32_t l = threadIdx.x; l < LB; l += kENT)
            sm.bins[l] = 0;
        __syncthreads();
        for (uint32_t i0 = 0; i0 < n; i0 += 4 * kENT)
        {
            uint64_t k[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                const uint32_t i = i0 + u * kENT + threadIdx.x;
                k[u] = i < n ? __ldcg(reinterpret_cast<const unsigned long long *>(B) + i) : 0ull;
            }
            for (uint32_t c = 0; c < a.pin.n; ++c)
                stage4_column<true>(sm.stage + a.col_off[c], B + a.col_off[c], 0, i0, n, a.pin.width[c]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                const uint32_t i = i0 + u * kENT + threadIdx.x;
                if (i < n)
                {
                    reinterpret_cast<uint64_t *>(sm.stage)[i] = k[u];
                    const uint32_t l = (uint32_t)(int_hash64(k[u]) >> shift) & (LB - 1u);
                    sm.perm[i] = (uint16_t)l;
                    atomicAdd(&sm.bins[l], 1u);
                }
            }
        }
        __syncthreads();
        for (uint32_t l = threadIdx.x; l < LB; l += kENT)
            sm.acc[l] += sm.bins[l];
        scan_bins(sm.bins, LB, sm.ws);
        // every row's sorted position (a row's order within its leaf does
        // not matter), inverted into the source row of every position
        // (bins reused: page entries), then the block written back in
        // sorted order with consecutive stores
        for (uint32_t i = threadIdx.x; i < n; i += kENT)
            sm.perm[i] = (uint16_t)atomicAdd(&sm.bins[sm.perm[i]], 1u);
        __syncthreads();
        uint32_t * src = sm.bins;
        for (uint32_t i = threadIdx.x; i < n; i += kENT)
            src[sm.perm[i]] = i;
        __syncthreads();
        for (uint32_t s = threadIdx.x; s < n; s += kENT)
            copy_row(a, B, s, sm.stage, src[s]);
        if (threadIdx.x == 0)
        {
            // the leaves of its first and last rows: E probes a block that
            // lies wholly inside its range without searching it
            a.blk_lfirst[blk] = (uint32_t)(int_hash64(reinterpret_cast<const uint64_t *>(sm.stage)[src[0]]) >> shift) & (LB - 1u);
            a.blk_llast[blk] = (uint32_t)(int_hash64(reinterpret_cast<const uint64_t *>(sm.stage)[src[n - 1]]) >> shift) & (LB - 1u);
            a.blk_rows[blk] = n;
            a.blk_rem[blk] = n;
            a.blk_bucket[blk] = p;
            a.blk_c0[blk] = vload(&a.ctl->cursor); // the cursor stands still outside E
            if (g == 0)
                a.ctl->blocks0 += 1;
            a.blk_state[blk] = p;
        }
        __syncthreads();
    }
    for (uint32_t l = threadIdx.x; l < LB; l += kENT)
        if (sm.acc[l])
            atomicAdd(a.leaf_rows + ((uint64_t)p << a.lb_log2) + l, sm.acc[l]);
    if (threadIdx.x == 0)
    {
        atomicAdd(&a.ctl->global_leaf_rows, (unsigned long long)rows);
        atomicAdd(&a.ctl->rows_refined, (unsigned long long)rows);
        atomicAdd(&a.ctl->refinements, 1ull);
        sm.clen[p] = 0;
        sm.fill[p] = page;
        sm.urows[p] = 0;
    }
    __syncthreads();
    return rows;
}

// Refines the group's largest bucket (src/PHJBep.cpp:376-395) until its
// unrefined bytes are below `low` (every bucket that holds rows when low
// is 0).
__device__ void refine_down_to(const EngineArgs & a, const Smem & sm, uint32_t g, uint64_t & unref_bytes, uint64_t low)
{
    unsigned long long * best_slot = reinterpret_cast<unsigned long long *>(sm.scal + 4);
    for (;;)
    {
        if (unref_bytes == 0 || (low && unref_bytes < low))
            return;
        if (threadIdx.x == 0)
            *best_slot = 0ull;
        __syncthreads();
        unsigned long long best = 0;
        for (uint32_t p = threadIdx.x; p < a.n_buckets; p += kENT)
        {
            // ties go to the lowest bucket
            const unsigned long long v = ((unsigned long long)sm.urows[p] << 32) | (0xFFFFFFFFu - p);
            if (sm.urows[p] && v > best)
                best = v;
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, best, o);
            best = y > best ? y : best;
        }
        if ((threadIdx.x & 31) == 0 && best)
            atomicMax(best_slot, best);
        __syncthreads();
        const unsigned long long top = *reinterpret_cast<volatile unsigned long long *>(best_slot);
        __syncthreads();
        if (top == 0)
            return;
        const uint32_t p = 0xFFFFFFFFu - (uint32_t)(top & 0xFFFFFFFFull);
        const uint32_t rows = refine_bucket(a, sm, g, p);
        const uint64_t b = (uint64_t)rows * a.rb;
        unref_bytes = unref_bytes > b ? unref_bytes - b : 0;
    }
}

// ---------------------------------------------------------------------------
// E0 (group 0 alone): the eviction range.  From the cursor on, leaves are
// taken until the rows they hold take the global leaf bytes below the low
// water (every leaf in the final drain).
// ---------------------------------------------------------------------------
__device__ void evict_range(const EngineArgs & a, const Smem & sm, bool final_drain)
{
    const uint64_t n = a.n_leaves;
    const uint64_t lo_abs = vload(&a.ctl->cursor), lo = lo_abs % n;
    const uint64_t g_rows = vload(&a.ctl->global_leaf_rows);
    uint64_t len = n;
    if (!final_drain)
    {
        // rows that may stay: (global - taken) * rb < leaf_low
        const uint64_t keep_max = a.leaf_low ? (a.leaf_low - 1) / a.rb : 0;
        const uint64_t need = g_rows > keep_max ? g_rows - keep_max : 0;
        uint64_t taken = 0;
        len = 0;
        constexpr uint32_t kPer = 8; // leaves a thread sums per step
        for (uint64_t base = 0; base < n && taken < need; base += (uint64_t)kENT * kPer)
        {
            const uint64_t i0 = base + (uint64_t)threadIdx.x * kPer;
            uint32_t v[kPer], mine = 0;
#pragma unroll
            for (uint32_t u = 0; u < kPer; ++u)
            {
                v[u] = i0 + u < n ? __ldcg(a.leaf_rows + (lo + i0 + u) % n) : 0u;
                mine += v[u];
            }
            uint32_t tot;
            const uint32_t ex = block_excl_scan<kENT>(mine, sm.ws, &tot);
            if (threadIdx.x == 0)
                sm.scal[6] = kNone;
            __syncthreads();
            // the leaf whose inclusive prefix first reaches `need`
            if (taken + ex < need && taken + ex + mine >= need)
            {
                uint64_t run = taken + ex;
                uint32_t u = 0;
                for (; u < kPer; ++u)
                {
                    run += v[u];
                    if (run >= need)
                        break;
                }
                sm.scal[6] = threadIdx.x * kPer + u;
            }
            __syncthreads();
            const uint32_t hit = sm.scal[6];
            __syncthreads();
            if (hit != kNone)
            {
                len = base + hit + 1;
                taken = need;
            }
            else
            {
                taken += tot;
                len = umin64(base + (uint64_t)kENT * kPer, n);
            }
        }
    }
    if (threadIdx.x == 0)
    {
        a.ctl->ev_lo = lo_abs;
        a.ctl->ev_len = len;
        a.ctl->cursor = lo_abs + len;
        a.ctl->work_next = 0;
        a.ctl->build_n = 0;
        a.ctl->build_next = 0;
        a.ctl->evict_phases += 1;
    }
    for (uint32_t p = threadIdx.x; p <= a.n_buckets; p += kENT)
    {
        a.bucket_cnt[p] = 0;
        a.bucket_fill[p] = 0;
    }
}

// Leaf-in-bucket intervals of bucket p inside the eviction range [lo,
// lo + len) (mod n_leaves): up to two, [x0, x1) and [y0, y1).
__device__ __forceinline__ void bucket_intervals(const EngineArgs & a, uint32_t p, uint64_t lo, uint64_t len, uint32_t & x0, uint32_t & x1,
                                                 uint32_t & y0, uint32_t & y1)
{
    const uint64_t n = a.n_leaves, LB = 1ull << a.lb_log2;
    const uint64_t start = (uint64_t)p << a.lb_log2;
    const uint64_t s = (start + n - lo) % n; // the bucket's first leaf, counted from the range's start
    x0 = x1 = y0 = y1 = 0;
    if (s + LB <= n)
    {
        if (len > s)
            x1 = (uint32_t)umin64(LB, len - s);
    }
    else
    {
        // the range starts inside this bucket: leaves [0, w) come last in
        // the range's order, leaves [w, LB) first
        const uint64_t w = n - s;
        if (len > s)
            x1 = (uint32_t)umin64(w, len - s);
        y0 = (uint32_t)w;
        y1 = (uint32_t)umin64(LB, w + len);
    }
}

__device__ __forceinline__ bool bucket_in_range(const EngineArgs & a, uint32_t p, uint64_t lo, uint64_t len)
{
    uint32_t x0, x1, y0, y1;
    bucket_intervals(a, p, lo, len, x0, x1, y0, y1);
    return x1 > x0 || y1 > y0;
}

// The part of this E's range [lo_abs, lo_abs + len) a block refined at
// cursor c0 still has unprobed rows in: a leaf's rows in the block are
// probed the first time the cursor reaches the leaf at or after c0, i.e.
// at positions [c0, c0 + n_leaves); rows of leaves passed since are probed.
__device__ __forceinline__ uint64_t block_len(const EngineArgs & a, unsigned long long c0, uint64_t lo_abs, uint64_t len)
{
    const uint64_t end = c0 + a.n_leaves;
    return end <= lo_abs ? 0 : umin64(len, end - lo_abs);
}

// Builds the table of leaf L in place (this warp won NOT_BUILT ->
// BUILDING) and threads the next-chain.  Returns whether a key repeats.
__device__ bool build_leaf_warp(const EngineArgs & a, uint32_t L, uint32_t lane)
{
    const LeafMeta m = a.meta[L]; // its place and size are planned before the launch
    bool dup = false;
    if (m.has_table)
    {
        const uint64_t cap = 1ull << m.log2cap;
        Cell * tab = a.cells + m.table_off;
        for (uint64_t j = lane; j < cap; j += 32)
            reinterpret_cast<ulonglong2 *>(tab)[j] = make_ulonglong2(0ull, INVALID_REF);
        __syncwarp();
        const uint32_t r0 = m.row_off, r1 = a.leaf_off[L + 1];
        for (uint32_t r = r0 + lane; r < r1; r += 32)
        {
            const uint64_t k = a.bpart.keys[r];
            const uint64_t prev = table_insert<false>(tab, cap, int_hash64(k), k, make_ref(0, r));
            a.next[r] = prev;
            dup |= ref_valid(prev);
        }
    }
    return __any_sync(0xffffffffu, dup);
}

// E1b: every warp takes claimed leaves from the queue and builds those it
// wins NOT_BUILT -> BUILDING for; a leaf another warp is building is waited
// for, bounded (the grid then ends with kErrWait).
__device__ void build_claimed(const EngineArgs & a)
{
    const uint32_t lane = threadIdx.x & 31;
    for (;;)
    {
        uint32_t L = kNone, won = 0;
        if (lane == 0)
        {
            const uint32_t i = atomicAdd(&a.ctl->build_next, 1u);
            L = i < vload(&a.ctl->build_n) ? __ldcg(a.build_queue + i) : kNone;
            if (L != kNone)
            {
                if (atomicCAS(a.state + L, kNotBuilt, kBuilding) == kNotBuilt)
                    won = 1;
                else if (ld_acquire_u32(a.state + L) < kBuilt)
                {
                    atomicAdd(&a.ctl->skip_retries, 1ull);
                    const uint64_t t0 = now_ns();
                    uint32_t spins = 0;
                    while (ld_acquire_u32(a.state + L) < kBuilt)
                    {
                        if (aborted(a))
                            break;
                        if ((++spins & 255u) == 0 && now_ns() - t0 > a.wait_limit_ns)
                        {
                            fail(a, kErrWait);
                            break;
                        }
                        __nanosleep(64);
                    }
                }
            }
        }
        L = __shfl_sync(0xffffffffu, L, 0);
        won = __shfl_sync(0xffffffffu, won, 0);
        if (L == kNone || aborted(a))
            return;
        if (won)
        {
            const bool dup = build_leaf_warp(a, L, lane);
            if (lane == 0)
            {
                a.meta[L].dup = dup ? 1 : 0;
                if (dup)
                    atomicExch(&a.ctl->any_dup, 1);
                __threadfence();
                atomicExch(a.state + L, dup ? kBuiltDup : kBuilt);
                atomicAdd(&a.ctl->tables_built, 1ull);
            }
        }
    }
}

// First row of the leaf-sorted block B (rows [lo, hi)) whose leaf-in-bucket
// is >= l: a 32-way search by one warp.
__device__ uint32_t lower_bound_warp(const EngineArgs & a, const uint8_t * B, uint32_t lo, uint32_t hi, uint32_t l, uint32_t lane)
{
    const uint32_t mask = (1u << a.lb_log2) - 1u, shift = 64u - a.total_bits;
    const unsigned long long * keys = reinterpret_cast<const unsigned long long *>(B);
    while (hi - lo > 32)
    {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t x = lo + lane * step;
        const bool below = x < hi && ((uint32_t)(int_hash64(__ldcg(keys + x)) >> shift) & mask) < l;
        const uint32_t c = __popc(__ballot_sync(0xffffffffu, below));
        // rows before lo are below l, rows from hi on are not
        const uint32_t nlo = c ? lo + (c - 1) * step + 1 : lo;
        const uint32_t nhi = c < 32 && lo + c * step < hi ? lo + c * step : hi;
        lo = nlo;
        hi = nhi;
    }
    const uint32_t x = lo + lane;
    const bool below = x < hi && ((uint32_t)(int_hash64(__ldcg(keys + x)) >> shift) & mask) < l;
    return lo + __popc(__ballot_sync(0xffffffffu, below));
}

// A lookup in two halves, so that several rows' first loads are in flight
// at once: probe_issue loads the aligned pair of cells the key's probe
// starts at (through L2: the leaf's table was built during this launch);
// probe_finish compares, follows the table past the pair when needed, and
// returns the match count (the next-chain's length when some leaf table has
// a repeated key) and the head build row.
__device__ __forceinline__ const Cell * leaf_table(const EngineArgs & a, uint64_t h, uint64_t & cap)
{
    const uint32_t L = (uint32_t)(h >> (64u - a.total_bits));
    if (a.ulog >= 0)
    {
        cap = 1ull << a.ulog;
        return a.cells + ((uint64_t)L << a.ulog);
    }
    const ulonglong2 m = __ldcg(reinterpret_cast<const ulonglong2 *>(a.meta + L));
    cap = ((m.y >> 40) & 0xffu) ? 1ull << ((uint32_t)(m.y >> 32) & 0xffu) : 0ull;
    return a.cells + m.x;
}

__device__ __forceinline__ CellPair probe_issue(const EngineArgs & a, uint64_t h)
{
    uint64_t cap;
    const Cell * tab = leaf_table(a, h, cap);
    if (cap == 0)
    {
        CellPair none;
        none.a = make_ulonglong2(0ull, INVALID_REF);
        none.b = none.a;
        return none;
    }
    return load_pair<true>(tab + probe_start(h, cap));
}

__device__ __forceinline__ uint32_t probe_finish(const EngineArgs & a, uint64_t key, uint64_t h, const CellPair & pr, bool chains, uint32_t & head)
{
    uint64_t r = INVALID_REF;
    if (ref_valid(pr.a.y))
    {
        if (pr.a.x == key)
            r = pr.a.y;
        else if (ref_valid(pr.b.y))
        {
            if (pr.b.x == key)
                r = pr.b.y;
            else
            {
                // past the pair: follow the table
                uint64_t cap;
                const Cell * tab = leaf_table(a, h, cap);
                const uint64_t mask = cap - 1;
                uint64_t pos = (probe_start(h, cap) + 2) & mask;
                for (uint64_t step = 2; step < cap; ++step)
                {
                    const ulonglong2 c = __ldcg(reinterpret_cast<const ulonglong2 *>(tab + pos));
                    if (!ref_valid(c.y))
                        break;
                    if (c.x == key)
                    {
                        r = c.y;
                        break;
                    }
                    pos = (pos + 1) & mask;
                }
            }
        }
    }
    if (!ref_valid(r))
        return 0;
    head = ref_row(r);
    if (!chains)
        return 1;
    uint32_t c = 1;
    for (unsigned long long x = __ldcg(reinterpret_cast<const unsigned long long *>(a.next) + head); ref_valid(x);
         x = __ldcg(reinterpret_cast<const unsigned long long *>(a.next) + ref_row(x)))
        ++c;
    return c;
}

// E2: one warp probes rows [r0, r1) of refined block B and projects the
// matches, 256 rows a step with one reservation of output rows; a step's
// output rows are placed round by round so each store instruction writes
// consecutive rows.
constexpr uint32_t kWarpRows = 4; // rows per lane per step
__device__ void probe_rows_warp(const EngineArgs & a, const uint8_t * B, uint32_t r0, uint32_t r1, uint32_t lane, bool chains)
{
    const unsigned long long * keys = reinterpret_cast<const unsigned long long *>(B);
    for (uint32_t base = r0; base < r1; base += 32 * kWarpRows)
    {
        uint64_t key[kWarpRows];
        uint32_t head[kWarpRows], cnt[kWarpRows];
#pragma unroll
        for (uint32_t k = 0; k < kWarpRows; ++k)
        {
            const uint32_t i = base + k * 32 + lane;
            key[k] = i < r1 ? __ldcg(keys + i) : 0ull;
        }
        // four first loads in flight, then their comparisons
#pragma unroll
        for (uint32_t g = 0; g < kWarpRows; g += 4)
        {
            CellPair pr[4];
#pragma unroll
            for (uint32_t u = 0; u < 4; ++u)
            {
                const uint32_t i = base + (g + u) * 32 + lane;
                if (i < r1)
                    pr[u] = probe_issue(a, int_hash64(key[g + u]));
            }
#pragma unroll
            for (uint32_t u = 0; u < 4; ++u)
            {
                const uint32_t i = base + (g + u) * 32 + lane;
                head[g + u] = 0;
                cnt[g + u] = i < r1 ? probe_finish(a, key[g + u], int_hash64(key[g + u]), pr[u], chains, head[g + u]) : 0u;
            }
        }
        // placement: a warp scan per round, rounds one after another
        uint32_t rel[kWarpRows], total = 0;
#pragma unroll
        for (uint32_t k = 0; k < kWarpRows; ++k)
        {
            uint32_t x = cnt[k];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= (uint32_t)d)
                    x += y;
            }
            rel[k] = total + x - cnt[k];
            total += __shfl_sync(0xffffffffu, x, 31);
        }
        if (total == 0)
            continue;
        unsigned long long out0 = 0;
        if (lane == 0)
            out0 = atomicAdd(&a.ctl->out_rows, (unsigned long long)total);
        out0 = __shfl_sync(0xffffffffu, out0, 0);
#pragma unroll 1
        for (uint32_t k = 0; k < kWarpRows; ++k)
        {
            if (cnt[k] == 0)
                continue;
            const uint32_t i = base + k * 32 + lane;
            uint64_t o = out0 + rel[k];
            uint32_t b = head[k];
            for (uint32_t m = 0; m < cnt[k]; ++m, ++o)
            {
                if (o < a.out_cap)
                {
                    __stcs(a.out_keys + o, (unsigned long long)key[k]);
                    for (uint32_t c = 0; c < a.bpart.n; ++c)
                        copy_elem_out(a.out_l[c], o, a.bpart.col[c], b, a.bpart.width[c]);
                    for (uint32_t c = 0; c < a.pin.n; ++c)
                        copy_elem_cg(a.out_r[c], o, B + a.col_off[c], i, a.pin.width[c]);
                }
                if (m + 1 < cnt[k])
                    b = ref_row(__ldcg(reinterpret_cast<const unsigned long long *>(a.next) + b));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// One E: range, claims, builds, probes.  False when the grid is ending.
// ---------------------------------------------------------------------------
__device__ bool evict_phase(const EngineArgs & a, const Smem & sm, uint32_t & gen, bool final_drain)
{
    const uint64_t t0 = now_ns();
    if (blockIdx.x == 0)
        evict_range(a, sm, final_drain);
    if (!grid_sync(a, gen, NoOp{}))
        return false;
    const uint64_t lo_abs = vload(&a.ctl->ev_lo), len = vload(&a.ctl->ev_len);
    const uint64_t n = a.n_leaves, lo = lo_abs % n;
    const uint64_t stride = (uint64_t)gridDim.x * kENT;
    // E1: claim every leaf of the range; count the refined blocks to probe
    // per bucket
    {
        unsigned long long rows = 0, ev = 0, skips = 0;
        for (uint64_t i = (uint64_t)blockIdx.x * kENT + threadIdx.x; i < len; i += stride)
        {
            const uint32_t L = (uint32_t)((lo + i) % n);
            if (atomicCAS(a.leaf_lock + L, 0u, 1u) != 0u)
            {
                ++skips; // held elsewhere
                continue;
            }
            const uint32_t r = __ldcg(a.leaf_rows + L);
            if (r)
            {
                a.leaf_rows[L] = 0;
                rows += r;
                ++ev;
                const uint32_t st = ld_acquire_u32(a.state + L);
                if (st < kBuilt)
                    a.build_queue[atomicAdd(&a.ctl->build_n, 1u)] = L;
                else if (st == kBuiltDup)
                    atomicExch(&a.ctl->any_dup, 1); // built by an earlier run over these tables
            }
            atomicExch(a.leaf_lock + L, 0u);
        }
        for (uint64_t b = (uint64_t)blockIdx.x * kENT + threadIdx.x; b < a.n_blocks; b += stride)
        {
            const uint32_t p = __ldcg(a.blk_state + b);
            if (p != kNone && bucket_in_range(a, p, lo, block_len(a, __ldcg(a.blk_c0 + b), lo_abs, len)))
                atomicAdd(a.bucket_cnt + p, 1u);
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            rows += __shfl_xor_sync(0xffffffffu, rows, o);
            ev += __shfl_xor_sync(0xffffffffu, ev, o);
            skips += __shfl_xor_sync(0xffffffffu, skips, o);
        }
        if ((threadIdx.x & 31) == 0)
        {
            if (rows)
            {
                atomicAdd(&a.ctl->global_leaf_rows, (unsigned long long)(-(long long)rows));
                atomicAdd(&a.ctl->rows_claimed, rows);
            }
            if (ev)
                atomicAdd(&a.ctl->evictions, ev);
            if (skips)
                atomicAdd(&a.ctl->skip_retries, skips);
        }
    }
    if (!grid_sync(a, gen, NoOp{}))
        return false;
    // E1b: group 0 turns the counts into work offsets, the buckets in the
    // range's order; every group builds claimed leaves
    if (blockIdx.x == 0)
    {
        const uint32_t P1 = a.n_buckets, first = (uint32_t)(lo >> a.lb_log2);
        for (uint32_t q = threadIdx.x; q < P1; q += kENT)
            sm.bins[q] = __ldcg(a.bucket_cnt + (first + q) % P1);
        __syncthreads();
        const uint32_t total = scan_bins(sm.bins, P1, sm.ws);
        for (uint32_t q = threadIdx.x; q < P1; q += kENT)
            a.bucket_cnt[(first + q) % P1] = sm.bins[q];
        if (threadIdx.x == 0)
            a.ctl->work_n = total;
        __syncthreads();
    }
    build_claimed(a);
    if (!grid_sync(a, gen, NoOp{}))
        return false;
    // E1c: the refined blocks of the range's buckets into the work list
    for (uint64_t b = (uint64_t)blockIdx.x * kENT + threadIdx.x; b < a.n_blocks; b += stride)
    {
        const uint32_t p = __ldcg(a.blk_state + b);
        if (p != kNone && bucket_in_range(a, p, lo, block_len(a, __ldcg(a.blk_c0 + b), lo_abs, len)))
            a.work[__ldcg(a.bucket_cnt + p) + atomicAdd(a.bucket_fill + p, 1u)] = (uint32_t)b;
    }
    if (!grid_sync(a, gen, NoOp{}))
        return false;
    const uint64_t t1 = now_ns();
    // E2: every warp takes a 1024-row part of a listed block at a time and
    // probes the range's rows in it.  Parts are handed out in list order
    // (bucket by bucket), so the warps in flight cover little more than one
    // bucket and its leaf tables and build rows stay in L2.
    {
        constexpr uint32_t kPart = 1024;
        const uint32_t lane = threadIdx.x & 31;
        const bool chains = vload(&a.ctl->any_dup) != 0; // some leaf table has a repeated key
        const uint32_t parts = (1u << a.page_log2) > kPart ? (1u << a.page_log2) / kPart : 1u;
        const uint32_t part_rows = (1u << a.page_log2) / parts;
        const uint64_t n_items = (uint64_t)vload(&a.ctl->work_n) * parts;
        for (;;)
        {
            unsigned long long w = 0;
            if (lane == 0)
                w = atomicAdd(&a.ctl->work_next, 1ull);
            w = __shfl_sync(0xffffffffu, w, 0);
            if (w >= n_items)
                break;
            const uint32_t blk = __ldcg(a.work + w / parts);
            const uint32_t c0r = (uint32_t)(w % parts) * part_rows; // the part's first row
            // (blk_state may already be cleared by the warp that probed the
            // block's last rows; the bucket stays)
            const uint32_t p = __ldcg(a.blk_bucket + blk);
            const uint32_t nrows = __ldcg(a.blk_rows + blk);
            if (c0r >= nrows)
                continue;
            const uint32_t c1r = c0r + part_rows < nrows ? c0r + part_rows : nrows;
            const uint32_t lf = __ldcg(a.blk_lfirst + blk), ll = __ldcg(a.blk_llast + blk);
            const uint8_t * B = block_ptr(a, blk);
            uint32_t x0, x1, y0, y1;
            bucket_intervals(a, p, lo, block_len(a, __ldcg(a.blk_c0 + blk), lo_abs, len), x0, x1, y0, y1);
            uint32_t done = 0;
            for (int part = 0; part < 2; ++part)
            {
                const uint32_t l0 = part ? y0 : x0, l1 = part ? y1 : x1;
                if (l1 <= l0 || l1 <= lf || l0 > ll)
                    continue; // no row of the block in these leaves
                uint32_t ra = l0 > lf ? lower_bound_warp(a, B, 0, nrows, l0, lane) : 0u;
                uint32_t rb = l1 <= ll ? lower_bound_warp(a, B, ra, nrows, l1, lane) : nrows;
                ra = ra > c0r ? ra : c0r;
                rb = rb < c1r ? rb : c1r;
                if (rb <= ra)
                    continue;
                probe_rows_warp(a, B, ra, rb, lane, chains);
                done += rb - ra;
            }
            if (lane == 0 && done)
            {
                atomicAdd(&a.ctl->rows_probed, (unsigned long long)done);
                const uint32_t left = atomicSub(a.blk_rem + blk, done) - done;
                if (left == 0)
                {
                    // every row probed: the block goes back to the pool
                    a.blk_state[blk] = kNone;
                    const long long slot = (long long)atomicAdd(reinterpret_cast<unsigned long long *>(&a.ctl->free_top), 1ull);
                    a.free_stack[slot] = blk;
                }
            }
        }
    }
    const uint64_t t2 = now_ns();
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        a.ctl->ns_evict += t1 - t0;
        a.ctl->ns_probe += t2 - t1;
    }
    return grid_sync(a, gen, NoOp{});
}

// The last group to arrive after a wave's S: records the peak, decides
// whether an E follows (the leaf high water, or a drain of every leaf when
// a group found too few free blocks) and whether input is left.  A low pool
// right after a forced drain cannot be helped: the grid ends.
struct WaveEnd
{
    const EngineArgs * a;
    __device__ void operator()() const
    {
        EngineCtl * c = a->ctl;
        const unsigned long long r = vload(&c->global_leaf_rows);
        if (r > c->peak_leaf_rows)
            c->peak_leaf_rows = r;
        const bool low = vload(&c->pool_low) != 0;
        if (low && c->forced_last)
        {
            atomicExch(&c->abort, kErrPool);
            atomicExch(a->err, kErrPool);
        }
        c->forced_last = low;
        if (low)
            c->forced_drains += 1;
        c->pool_low = 0;
        c->evict_now = low ? 2 : (r > 0 && r * a->rb >= a->leaf_high ? 1 : 0);
        c->ns_s_crit += c->wave_s_max;
        c->wave_s_max = 0;
        c->more_input = vload(&c->groups_done) < gridDim.x;
    }
};

__global__ void __launch_bounds__(kENT, 1) k_bep_engine(const __grid_constant__ EngineArgs a)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    const uint32_t page = 1u << a.page_log2;
    const uint32_t P1 = a.n_buckets, LB = 1u << a.lb_log2;
    Smem sm;
    {
        uint8_t * p = smem_raw;
        const uint64_t cells_bytes = (uint64_t)a.smem_cells * sizeof(Cell), rows_bytes = (uint64_t)page * a.rb;
        const uint64_t stage = rows_bytes > cells_bytes ? rows_bytes : cells_bytes;
        sm.stage = p;
        p += (stage + 15) & ~15ull;
        sm.perm = reinterpret_cast<uint16_t *>(p);
        p += ((uint64_t)page * 2 + 15) & ~15ull;
        sm.src = reinterpret_cast<uint16_t *>(p);
        p += ((uint64_t)page * 2 + 15) & ~15ull;
        const uint32_t nbins = P1 > LB ? (P1 > page ? P1 : page) : (LB > page ? LB : page);
        sm.bins = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)nbins * 4 + 15) & ~15ull;
        sm.boff = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)P1 * 4 + 15) & ~15ull;
        sm.nbpre = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)P1 * 4 + 15) & ~15ull;
        sm.fill = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)P1 * 4 + 15) & ~15ull;
        sm.clen = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)P1 * 4 + 15) & ~15ull;
        sm.urows = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)P1 * 4 + 15) & ~15ull;
        sm.acc = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)LB * 4 + 15) & ~15ull;
        sm.bcache = reinterpret_cast<uint32_t *>(p);
        p += ((uint64_t)(2 * P1 + 2 * kRefill) * 4 + 15) & ~15ull;
        sm.ws = reinterpret_cast<uint32_t *>(p);
        p += (kENT / 32) * 4;
        sm.scal = reinterpret_cast<uint32_t *>(p);
    }
    const uint32_t g = blockIdx.x, G = gridDim.x;
    for (uint32_t p = threadIdx.x; p < P1; p += kENT)
    {
        sm.fill[p] = page; // no block yet
        sm.clen[p] = 0;
        sm.urows[p] = 0;
    }
    for (uint32_t p = threadIdx.x; p < P1; p += kENT)
        sm.bins[p] = 0;
    if (threadIdx.x < 32)
        sm.scal[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t lo = a.probe_rows * g / G, hi = a.probe_rows * (g + 1) / G;
    uint64_t pos = lo, unref_bytes = 0;
    uint32_t gen = 0;
    bool counted = false; // this group is counted in groups_done
    for (uint32_t wave = 0;; ++wave)
    {
        // -------- S: this wave's tile of the slice, then the refine trigger --------
        const uint64_t t0 = now_ns();
        for (uint32_t p = threadIdx.x; p < P1; p += kENT)
            sm.bins[p] = 0; // refines and E use the bins too
        __syncthreads();
        const uint64_t end = umin64(hi, pos + a.tile_rows);
        while (pos < end)
        {
            const uint32_t n = (uint32_t)umin64(page, end - pos);
            const int st = scatter_tile(a, sm, g, pos, n);
            if (st == kTileFailed)
                return;
            if (st == kTileNoRoom)
            {
                // too few free blocks: the rest of the tile waits for the
                // drain this forces after the wave
                if (threadIdx.x == 0)
                    atomicExch(&a.ctl->pool_low, 1);
                break;
            }
            pos += n;
            unref_bytes += (uint64_t)n * a.rb;
            if (threadIdx.x == 0)
            {
                atomicAdd(&a.ctl->rows_scattered, (unsigned long long)n);
                if (g == 0)
                    a.ctl->tiles0 += 1;
            }
        }
        if (pos >= hi && !counted)
        {
            counted = true;
            if (threadIdx.x == 0)
                atomicAdd(&a.ctl->groups_done, 1u);
        }
        const uint64_t t_ref = now_ns();
        if (pos < end)
            refine_down_to(a, sm, g, unref_bytes, 0); // stalled: everything it holds goes to the drain
        else if (unref_bytes >= a.unref_high)
            refine_down_to(a, sm, g, unref_bytes, a.unref_low);
        if (g == 0 && threadIdx.x == 0)
            a.ctl->ns_refine0 += now_ns() - t_ref;
        if (threadIdx.x == 0)
        {
            const unsigned long long dt = now_ns() - t0;
            if (g == 0)
                a.ctl->ns_shuffle += dt;
            atomicMax(&a.ctl->wave_s_max, dt);
        }
        if (wave == a.test_stall_wave && g == 0 && threadIdx.x == 0)
        {
            // test hook: this group holds back from the barrier until the
            // others' bounded wait runs out and ends the grid (bounded too)
            const uint64_t ts = now_ns();
            while (!aborted(a) && now_ns() - ts < 4 * a.wait_limit_ns)
                __nanosleep(1000);
        }
        // the last group to arrive records the peak and decides the E
        if (!grid_sync(a, gen, WaveEnd{&a}))
            return;
        const int ev = vload(&a.ctl->evict_now);
        const bool more = vload(&a.ctl->more_input) != 0;
        if (ev)
            if (!evict_phase(a, sm, gen, ev == 2))
                return;
        if (!more)
            break;
    }
    // -------- end of the slice: refine every bucket that holds rows --------
    {
        const uint64_t t0 = now_ns();
        refine_down_to(a, sm, g, unref_bytes, 0);
        if (g == 0 && threadIdx.x == 0)
            a.ctl->ns_shuffle += now_ns() - t0;
    }
    if (!grid_sync(a, gen, WaveEnd{&a}))
        return;
    // -------- the post-probe drain: every leaf that holds rows --------
    evict_phase(a, sm, gen, true);
}

__global__ void k_engine_init(uint32_t * __restrict__ free_stack, uint32_t * __restrict__ blk_state, uint32_t n_blocks, EngineCtl * ctl)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
        ctl->free_top = (long long)n_blocks; // the stack starts full
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_blocks; i += gridDim.x * blockDim.x)
    {
        free_stack[i] = n_blocks - 1 - i;
        blk_state[i] = kNone;
    }
}
} // namespace

bool bep_engine_supported(uint32_t b1, uint32_t total_bits)
{
    return b1 >= 1 && b1 <= 11 && total_bits >= b1 && total_bits - b1 <= 13;
}

BepEngineResult bep_engine_run(phj_ctx * ctx, Scratch & s, const BepEngineInput & in, phj_output * out)
{
    BepEngineResult res{};
    const uint32_t G = (uint32_t)ctx->num_sms; // one group per SM
    EngineArgs a{};
    a.pin = in.probe;
    a.probe_rows = in.probe_rows;
    a.bpart = in.build;
    a.state = in.lt->state;
    a.meta = in.lt->meta;
    a.cells = in.lt->cells;
    a.next = in.lt->next;
    a.leaf_off = in.leaf_off;
    a.ulog = in.lt->uniform_log2cap;
    a.b1 = in.b1;
    a.total_bits = in.total_bits;
    a.lb_log2 = in.total_bits - in.b1;
    a.n_leaves = 1u << in.total_bits;
    a.n_buckets = 1u << in.b1;
    uint32_t rb = 8;
    for (uint32_t c = 0; c < in.probe.n; ++c)
        rb += in.probe.width[c];
    a.rb = rb;
    // the budget per group and the water marks (src/PHJBep.cpp:180-190)
    const uint64_t budget = in.budget_bytes;
    const uint64_t per_group = budget / G;
    a.unref_high = per_group / 2;
    a.unref_low = a.unref_high / 2;
    a.leaf_high = budget * 5 / 8;
    a.leaf_low = a.leaf_high * 5 / 8;
    const uint64_t P1 = a.n_buckets, LB = 1ull << a.lb_log2;
    const uint64_t high_rows = a.unref_high / rb;
    // block rows: a power of two, 64..8192, about what one bucket of a group
    // gathers before its group refines (so a refined block is mostly
    // full), and whose rows fit 96 KiB of shared memory (the refine sorts a
    // whole block there)
    uint32_t page_log2 = 6;
    while (page_log2 < 13 && (2ull << page_log2) <= std::max<uint64_t>(high_rows / P1, 1))
        ++page_log2;
    while (page_log2 > 6 && ((uint64_t)rb << page_log2) > (96u << 10))
        --page_log2;
    a.page_log2 = page_log2;
    const uint64_t page = 1ull << page_log2;
    uint64_t off = page * 8;
    for (uint32_t c = 0; c < in.probe.n; ++c)
    {
        a.col_off[c] = (uint32_t)off;
        off += page * in.probe.width[c];
    }
    a.block_bytes = (off + 255) & ~255ull;
    a.smem_cells = (uint32_t)std::min<uint64_t>(4096, std::max<uint64_t>((page * rb) / sizeof(Cell), 2048));
    // input rows a group scatters between two looks at the global leaf
    // count: half its unrefined high water, within [256, 64K], so one wave
    // overshoots the marks by little
    a.tile_rows = std::min<uint64_t>(std::min<uint64_t>(page * 16, 65536), std::max<uint64_t>(256, (high_rows / 2) & ~255ull));
    const uint64_t slice = ceil_div(std::max<uint64_t>(in.probe_rows, 1), G);
    a.waves = (uint32_t)std::max<uint64_t>(1, ceil_div(slice, a.tile_rows));
    // pool, in blocks: a group's unrefined chains hold at most its high
    // water plus a tile in full blocks and one part block per bucket; the
    // refined blocks hold the leaf rows (up to the leaf high water plus one
    // wave of refines) and one part block per refine still unprobed.  Past
    // the whole probe side (a quarter more for blocks partly probed) no
    // more is needed.  Should the pool still run low, the engine drains
    // every leaf and goes on.
    const uint64_t unref_blocks = G * (ceil_div(high_rows + a.tile_rows, page) + P1 + 1);
    const uint64_t leaf_rows_max = a.leaf_high / rb + G * (high_rows + a.tile_rows);
    const uint64_t by_budget = unref_blocks + ceil_div(leaf_rows_max, page) + 2 * G * P1;
    const uint64_t by_input = ceil_div(in.probe_rows + in.probe_rows / 4, page) + 2 * G * (P1 + 2) + G * ceil_div(a.tile_rows, page);
    const uint64_t n_blocks = std::max<uint64_t>(std::min(by_budget, by_input), 2 * unref_blocks) + (uint64_t)G * (kRefill + 8);
    if (n_blocks >= (1ull << 31))
        throw Error(PHJ_ERR_UNSUPPORTED, "PHJ (BEP): the probe side needs more blocks than the device budget engine indexes");
    a.n_blocks = (uint32_t)n_blocks;
    a.maxb = (uint32_t)(ceil_div(std::min<uint64_t>(high_rows + a.tile_rows + page, slice + page), page) + 2);
    a.pool = s.get<uint8_t>((uint64_t)a.n_blocks * a.block_bytes);
    a.free_stack = s.get<uint32_t>(a.n_blocks);
    a.blk_state = s.get<uint32_t>(a.n_blocks);
    a.blk_rows = s.get<uint32_t>(a.n_blocks);
    a.blk_rem = s.get<uint32_t>(a.n_blocks);
    a.blk_lfirst = s.get<uint32_t>(a.n_blocks);
    a.blk_llast = s.get<uint32_t>(a.n_blocks);
    a.blk_bucket = s.get<uint32_t>(a.n_blocks);
    a.blk_c0 = s.get<unsigned long long>(a.n_blocks);
    a.chain = s.get<uint32_t>((uint64_t)G * P1 * a.maxb);
    a.leaf_rows = s.get<uint32_t>(a.n_leaves);
    a.leaf_lock = s.get<uint32_t>(a.n_leaves);
    a.bucket_cnt = s.get<uint32_t>(P1 + 1);
    a.bucket_fill = s.get<uint32_t>(P1 + 1);
    a.work = s.get<uint32_t>(a.n_blocks);
    a.build_queue = s.get<uint32_t>(a.n_leaves);
    a.out_keys = out->keys;
    for (uint32_t c = 0; c < out->left.n_payloads; ++c)
        a.out_l[c] = out->lcol[c];
    for (uint32_t c = 0; c < out->right.n_payloads; ++c)
        a.out_r[c] = out->rcol[c];
    a.out_cap = out->cap;
    a.wait_limit_ns = (uint64_t)ctx->wait_limit_ms * 1000000ull;
    a.test_stall_wave = ctx->test_engine_stall_wave >= 0 ? (uint32_t)ctx->test_engine_stall_wave : kNone;
    a.ctl = s.get<EngineCtl>(1);
    a.err = ctx->d_err;
    PHJ_CUDA(cudaMemsetAsync(a.ctl, 0, sizeof(EngineCtl), ctx->stream));
    PHJ_CUDA(cudaMemsetAsync(a.leaf_rows, 0, (size_t)a.n_leaves * 4, ctx->stream));
    PHJ_CUDA(cudaMemsetAsync(a.leaf_lock, 0, (size_t)a.n_leaves * 4, ctx->stream));
    k_engine_init<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(a.n_blocks, 256), (uint64_t)ctx->num_sms * 8)), 256, 0,
                    ctx->stream>>>(a.free_stack, a.blk_state, a.n_blocks, a.ctl);
    PHJ_LAUNCHED(ctx, "bep_engine_init");
    // shared memory: stage, permutation, bins, the per-bucket state
    const uint64_t stage = std::max<uint64_t>(page * rb, (uint64_t)a.smem_cells * sizeof(Cell));
    const uint64_t nbins = std::max(std::max(P1, LB), page);
    const size_t smem = ((stage + 15) & ~15ull) + 2 * ((page * 2 + 15) & ~15ull) + ((nbins * 4 + 15) & ~15ull) + 5 * ((P1 * 4 + 15) & ~15ull) +
                        ((LB * 4 + 15) & ~15ull) + (((2 * P1 + 2 * kRefill) * 4 + 15) & ~15ull) + (kENT / 32) * 4 + 32 * 4;
    if (smem + 1024 > (size_t)ctx->smem_optin)
        throw Error(PHJ_ERR_UNSUPPORTED, "PHJ (BEP): the device budget engine's shared memory does not fit this configuration");
    PHJ_CUDA(cudaFuncSetAttribute(k_bep_engine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bep_engine, kENT, smem));
    if (per_sm < 1)
        throw Error(PHJ_ERR_UNSUPPORTED, "PHJ (BEP): the device budget engine does not fit on an SM");
    if (std::getenv("PHJ_DEBUG"))
        std::fprintf(stderr, "[phj] bep_engine: %u groups, page %llu rows (%llu B), %u blocks (%.2f GB), maxb %u, waves %u, tile %llu, smem %zu\n", G,
                     (unsigned long long)page, (unsigned long long)a.block_bytes, a.n_blocks, a.n_blocks * (double)a.block_bytes / 1e9, a.maxb,
                     a.waves, (unsigned long long)a.tile_rows, smem);
    {
        KTimer kt(ctx, "bep_engine", in.probe_rows, 0);
        void * args[] = {&a};
        PHJ_CUDA(cudaLaunchCooperativeKernel((const void *)k_bep_engine, dim3(G), dim3(kENT), args, smem, ctx->stream));
        PHJ_LAUNCHED(ctx, "bep_engine");
    }
    EngineCtl c{};
    int e = 0;
    read_small(ctx, {{&c, a.ctl, sizeof(c)}, {&e, ctx->d_err, sizeof(e)}});
    // the launch's algorithmic bytes, as the join's: every probe row read
    // once, every output row written once
    {
        uint64_t orow = 8;
        for (uint32_t c2 = 0; c2 < in.build.n; ++c2)
            orow += in.build.width[c2];
        for (uint32_t c2 = 0; c2 < in.probe.n; ++c2)
            orow += in.probe.width[c2];
        for (size_t i = ctx->records.size(); i-- > 0;)
            if (ctx->records[i].name == "bep_engine")
            {
                ctx->records[i].bytes = in.probe_rows * rb + std::min<uint64_t>(c.out_rows, a.out_cap) * orow;
                break;
            }
    }
    res.err = e;
    res.out_rows = c.out_rows;
    res.evictions = c.evictions;
    res.refinements = c.refinements;
    res.skip_retries = c.skip_retries;
    res.tables_built = c.tables_built;
    res.evict_phases = c.evict_phases;
    res.peak_bytes = c.peak_leaf_rows * rb;
    res.ms_shuffle = c.ns_shuffle * 1e-6;
    res.ms_evict = c.ns_evict * 1e-6;
    res.ms_probe = c.ns_probe * 1e-6;
    res.pool_bytes = (uint64_t)a.n_blocks * a.block_bytes;
    if (std::getenv("PHJ_DEBUG"))
        std::fprintf(stderr,
                     "[phj] bep_engine rows: scattered %llu refined %llu claimed %llu probed %llu out %llu; E phases %llu (forced %llu), "
                     "S critical path %.3f ms (group 0: %llu tiles, %llu blocks refined in %.3f ms), err %d\n",
                     c.rows_scattered, c.rows_refined, c.rows_claimed, c.rows_probed, c.out_rows, c.evict_phases, c.forced_drains, c.ns_s_crit * 1e-6,
                     c.tiles0, c.blocks0, c.ns_refine0 * 1e-6, e);
    res.groups = G;
    return res;
}
} // namespace phjg
