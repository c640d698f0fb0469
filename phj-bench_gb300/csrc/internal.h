// internal.h -- host-side internals shared by the library's translation
// units: the context, device tables and outputs, the stream-ordered
// allocator, kernel timing, and the entry points of each kernel module.
#pragma once

#include <algorithm>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/phj_gpu.h"
#include "common.cuh"

// ---------------------------------------------------------------------------
// Errors inside the library are C++ exceptions; the C ABI turns them into a
// status code plus phj_last_error().
// ---------------------------------------------------------------------------
namespace phjg
{
struct Error : std::runtime_error
{
    phj_status status;
    Error(phj_status s, const std::string & m)
        : std::runtime_error(m)
        , status(s)
    {
    }
};

void cuda_check(cudaError_t e, const char * what, const char * file, int line);
#define PHJ_CUDA(call) ::phjg::cuda_check((call), #call, __FILE__, __LINE__)
#define PHJ_LAUNCHED(ctx, name) ::phjg::after_launch((ctx), (name), __FILE__, __LINE__)

struct KernelRecord
{
    std::string name;
    cudaEvent_t start = nullptr, stop = nullptr;
    uint64_t rows = 0, bytes = 0;
};

inline uint32_t payload_width(uint8_t t)
{
    switch (t)
    {
        case PHJ_U8: return 1;
        case PHJ_U16: return 2;
        case PHJ_U32: return 4;
        case PHJ_U64: return 8;
        case PHJ_U128: return 16;
        default: return 0;
    }
}

inline uint64_t schema_bytes(const phj_schema & s)
{
    uint64_t b = 0;
    for (uint32_t c = 0; c < s.n_payloads; ++c)
        b += payload_width(s.types[c]);
    return b;
}
} // namespace phjg

// A request to flag leaves during the next first radix pass (PHJ/BEP
// batches): bit (hash >> shift) of `bits` (`words` 32-bit words).
struct LeafMark
{
    uint32_t * bits = nullptr;
    uint32_t shift = 0;
    uint32_t words = 0;
};

namespace phjg
{
struct BatchGraph; // batch.cu: phj_batch_run's workspace and captured chain
void free_batch_graph(phj_ctx * ctx);
} // namespace phjg

struct phj_ctx
{
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    size_t l2_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t h2d = nullptr, d2h = nullptr; // copy streams of the host-buffer entry points (made on first use)
    cudaStream_t side = nullptr;               // second compute stream: probe-side first pass beside the build
    cudaStream_t aux = nullptr;                // third compute stream: build payload packing beside the leaf tables
    cudaMemPool_t pool = nullptr;
    std::string last_error;
    uint64_t launches = 0;
    // Allocation accounting of the current run (peak_mem_bytes).
    uint64_t cur_bytes = 0, peak_bytes = 0;
    std::vector<std::pair<void *, uint64_t>> live; // small: a run holds tens of buffers
    // Per-kernel timing of the last run.
    bool time_kernels = true;
    std::vector<phjg::KernelRecord> records;
    std::vector<cudaEvent_t> event_pool;
    size_t event_next = 0;
    void * l2_flush = nullptr;
    size_t l2_flush_bytes = 0;
    int * d_err = nullptr; // device error word: bounded waits that gave up
    uint8_t * host_small = nullptr;     // mapped pinned buffer of read_small
    uint8_t * host_small_dev = nullptr; // its device address
    // Options (phj_ctx_set_int).
    int probe_materialize = -1; // -1 auto, 0 never, 1 always
    int64_t wait_limit_ms = 1000; // bound of a device wait on another warp's work
    int64_t host_chunk_rows = 16ll << 20; // probe rows per chunk of the host-buffer entry points
    uint32_t table_cap_pct = 200; // leaf table cells >= rows * pct / 100 (power of two)
    uint32_t p1_tile_rows = 0;    // first radix pass: rows per staged tile (0: chosen per row width)
    uint32_t p1_stages = 0;       // first radix pass: depth of the bulk-copy ring (0: chosen per row width)
    int pack_build = 1;           // pack unique-key build payloads row-major for the projection (0: columns)
    uint32_t chj_windows = 0;     // CHJ: probe in this many windows of sub-tables (0 or 1: one sweep)
    int bep_engine = 0;           // PHJ/BEP: 0 the device budget engine, 1 budget-sized probe batches
    int batch_graph = 1;          // phj_batch_run: 1 replays its chain as a CUDA graph, 0 launches it
    int probe_fused = 1;          // unique build keys, packed payloads: 1 looks up and projects in one kernel
    phjg::BatchGraph * batch_ws = nullptr;
    uint32_t probe_pass_bits = 0; // PHJ-PURE probe side's written pass (0: the first logical pass's bits)
    bool p1_beside = false;       // first radix passes run beside other kernels (register-capped scatter)
    int64_t test_stuck_leaf = -1; // test hook: PHJ/BEP leaf left BUILDING before the probe
    int64_t test_engine_stall_wave = -1; // test hook: a BEP engine group holds back from this wave's barrier
    int test_fail_build = 0;      // test hook: host-buffer joins fail on the host after the build shuffle
    LeafMark leaf_mark;           // consumed by the next first radix pass
};

struct phj_table
{
    phj_schema schema{};
    uint64_t rows = 0;
    uint32_t n_blocks = 0;
    uint64_t * keys = nullptr;
    void * cols[PHJ_MAX_PAYLOADS] = {};
    uint64_t * block_off = nullptr; // device, n_blocks + 1 (row offset of each block)
    uint32_t uniform_block_rows = 0; // all blocks but the last have this many rows (0: irregular)
    bool owned = false;
    uint64_t gen_distinct = 0; // distinct build keys of a generated multi-match side
};

struct phj_output
{
    uint64_t rows = 0, cap = 0;
    phj_schema left{}, right{};
    uint64_t * keys = nullptr;
    void * lcol[PHJ_MAX_PAYLOADS] = {};
    void * rcol[PHJ_MAX_PAYLOADS] = {};
    uint64_t bytes = 0;
};

namespace phjg
{
// ----- allocation (stream-ordered pool of the context) ---------------------
void * dalloc(phj_ctx * ctx, size_t bytes);
void dfree(phj_ctx * ctx, void * p);

// Small device-to-host reads (row counts, flags, the error word).  A kernel
// stores the values into the context's mapped pinned buffer and the host
// waits for the context's stream.  A copy-engine read would queue behind a
// large download in flight on another stream (the host-buffer join
// downloads one chunk's output while it probes the next); the kernel does
// not.  At most kMaxSmallReads values of at most kSmallReadBytes in all.
struct SmallRead
{
    void * dst;
    const void * src;
    uint32_t bytes;
};
constexpr uint32_t kMaxSmallReads = 8;
constexpr uint32_t kSmallReadBytes = 512;
void read_small(phj_ctx * ctx, std::initializer_list<SmallRead> reads);
void reset_accounting(phj_ctx * ctx);

template <class T>
T * dalloc_n(phj_ctx * ctx, uint64_t n)
{
    return static_cast<T *>(dalloc(ctx, (size_t)(n ? n : 1) * sizeof(T)));
}

// RAII holder for run-scoped scratch.
struct Scratch
{
    phj_ctx * ctx;
    std::vector<void *> ptrs;
    explicit Scratch(phj_ctx * c)
        : ctx(c)
    {
    }
    ~Scratch()
    {
        for (void * p : ptrs)
            dfree(ctx, p);
    }
    template <class T>
    T * get(uint64_t n)
    {
        T * p = dalloc_n<T>(ctx, n);
        ptrs.push_back(p);
        return p;
    }
    Scratch(const Scratch &) = delete;
    Scratch & operator=(const Scratch &) = delete;
};

// ----- timing ----------------------------------------------------------------
cudaEvent_t take_event(phj_ctx * ctx);
void begin_run(phj_ctx * ctx);
// Records an event pair around the next launch(es) when kernel timing is on
// (and `name` is not null).
struct KTimer
{
    phj_ctx * ctx;
    int idx = -1;
    KTimer(phj_ctx * c, const char * name, uint64_t rows, uint64_t bytes);
    ~KTimer();
};
void after_launch(phj_ctx * ctx, const char * name, const char * file, int line);
float event_ms(cudaEvent_t a, cudaEvent_t b);

// ----- columns ----------------------------------------------------------------
Cols cols_of(const phj_table & t);
Cols alloc_cols_like(Scratch & s, const phj_schema & schema, uint64_t rows);
uint32_t max_width(const Cols & c);

// ----- scan.cu -----------------------------------------------------------------
// Exclusive scan of m u32 values into out[0..m); out[m] = total.
void scan_u32(phj_ctx * ctx, Scratch & s, const uint32_t * in, uint32_t * out, uint64_t m);
// The same with caller-owned carry space of scan_u32_carry(m) values (none
// is allocated, so the launches can be captured into a CUDA graph).
uint64_t scan_u32_carry(uint64_t m);
void scan_u32_into(phj_ctx * ctx, const uint32_t * in, uint32_t * out, uint64_t m, uint32_t * carry);

// ----- partition.cu ---------------------------------------------------------------
// Radix-partitions n rows by the top sum(pass_bits) bits of intHash64(key)
// (src/RadixPartition.cpp:546-577).  Rows land in `out` in leaf order;
// leaf_off[0..2^bits] receives each leaf's first row (leaf_off[2^bits] = n).
// Passes wider than kMaxPassBits are run as several physical passes.
void radix_partition(phj_ctx * ctx, Scratch & s, const Cols & in, uint64_t n, const std::vector<uint32_t> & pass_bits,
                     const Cols & out, const Cols & tmp, uint32_t * leaf_off, const char * phase);

// ----- build.cu -----------------------------------------------------------------------
// Leaf (or sub-table) directory entry: where a table lives and how big it is.
struct __align__(16) LeafMeta
{
    uint64_t table_off; // first cell
    uint32_t row_off;   // first build row of the leaf (PHJ) / unused (CHJ)
    uint8_t log2cap;    // capacity = 1 << log2cap, 0 cells when has_table == 0
    uint8_t has_table;
    uint8_t dup;        // some key of this table has more than one build row
    uint8_t pad;
};

struct LeafTables
{
    LeafMeta * meta = nullptr; // n_leaves
    Cell * cells = nullptr;
    uint64_t * next = nullptr; // next-chain, one RowRefCell per build row (BlockStore next_chain_)
    uint64_t total_cells = 0;
    uint32_t max_rows = 0;
    int any_dup = 0;
    int uniform_log2cap = -1; // >= 0: every leaf table has 2^this cells at leaf << this
    uint32_t * state = nullptr; // lazy build (PHJ/BEP): per leaf NOT_BUILT / BUILDING / BUILT
};

// Per-leaf tables over leaf-partitioned build rows (PHJ-PURE / PHJ).  With
// `lazy` only the layout is planned; the probe builds each table on first
// use (PHJ/BEP).
void build_leaf_tables(phj_ctx * ctx, Scratch & s, const Cols & build_part, const uint32_t * leaf_off, uint32_t n_leaves,
                       LeafTables & lt, bool lazy = false);
// Makes the rows of each repeated key contiguous (src -> dst, one CTA per
// leaf) so the probe expands a match as a row range instead of a chain
// walk.  Returns false (nothing done) when no key repeats or a leaf table is
// too large for the shared-memory counters.
bool group_leaf_duplicates(phj_ctx * ctx, const Cols & src, const Cols & dst, const uint32_t * leaf_off, uint32_t n_leaves, const LeafTables & lt);
// One global table of 2^slot_bits sub-tables namespaced by the top hash bits (CHJ).
void build_global_table(phj_ctx * ctx, Scratch & s, const phj_table & build, uint32_t slot_bits, LeafTables & lt);

// ----- probe.cu -------------------------------------------------------------------------
struct ProbeArgs
{
    Cols probe;             // probe rows in the order they are streamed
    uint64_t probe_rows;
    Cols build;             // build payloads addressed by RowRefCell
    const LeafMeta * meta;
    const Cell * cells;
    const uint64_t * next;
    uint32_t leaf_bits;     // leaf = hash >> (64 - leaf_bits)
    int chj;                // 1: refs are (input block, row); 0: refs are (leaf, row in leaf)
    const uint64_t * block_off;
    uint32_t uniform_block_rows;
    int any_dup;
    int uniform_log2cap;    // >= 0: PHJ leaf tables of uniform capacity (no directory lookup)
    // Grouped leaves (PHJ-PURE with repeated keys): a cell holds {count,
    // first row}; the lookup records each probe row's match count here.
    int grouped;
    uint32_t * row_cnt;  // per probe row: its match count (when keys repeat)
    uint32_t * flat;     // chained duplicates: build row of every output row
    unsigned long long * out_rows64; // the lookup's 64-bit count of output rows
    // Build payloads also packed row-major (no repeated key; two or more
    // columns of 1-8 bytes, 16 bytes in all): build row r's payloads in the
    // 16 bytes at packed[r], column c at byte packed_off[c].  The projection
    // then gathers one 16-byte value per output row instead of one per
    // column.  nullptr: columns only.
    const uint4 * packed;
    uint8_t packed_off[kMaxCols];
    // CHJ windowed probe: only rows whose sub-table (top leaf_bits hash
    // bits) lies in [win_lo, win_hi) are looked up; the others record no
    // match.  win_hi == 0: no window.
    uint32_t win_lo, win_hi;
};
// PHJ/BEP lazy leaf tables.  Per probe batch: the leaves the batch touches
// are flagged (one eviction per leaf and batch), the touched leaves still
// NOT_BUILT are queued, and persistent CTAs take leaves from that queue and
// build them (NOT_BUILT -> BUILDING -> BUILT; a leaf found BUILDING is
// waited for, bounded by wait_limit_ns).  Counters: [0] tables built, [1]
// waits on a BUILDING leaf, [2] evictions.
struct BepLeaves
{
    uint32_t * state;             // per leaf: 0 NOT_BUILT, 1 BUILDING, 2 BUILT, 3 BUILT (keys repeat)
    uint32_t * touched;           // bitmap over the leaves: touched by the current batch
    const uint32_t * leaf_off;    // first build row of each leaf (n_leaves + 1)
    const uint64_t * build_keys;  // leaf-partitioned build keys
    LeafMeta * meta;
    Cell * cells;
    uint64_t * next;
    uint32_t leaf_bits;
    uint32_t n_leaves;
    uint32_t smem_cells;          // tables up to this many cells are built in shared memory
    uint64_t wait_limit_ns;
    unsigned long long * ctr;
    uint32_t * queue;             // n_leaves entries
    uint32_t * queue_len;         // [0] queued leaves, [1] leaves taken
    int * any_dup;                // set when a built leaf has a repeated key
};
// Builds the leaves the batch's probe keys touch.  Returns whether any leaf
// built so far has a repeated key (the lookup then follows chains).
// The batch's leaves are flagged in b.touched by its first radix pass
// (ctx->leaf_mark) before this runs.
bool bep_build_touched(phj_ctx * ctx, const BepLeaves & b);
void set_bep_smem_limits(int smem_optin);

// ----- bep_engine.cu ------------------------------------------------------------------
// PHJ/BEP with the probe-side byte budget kept on the device: one
// persistent grid of CTA groups with per-group unrefined chains, water
// marks, refinement, round-robin eviction and lazy leaf builds.
struct BepEngineInput
{
    Cols probe; // probe side in input order
    uint64_t probe_rows;
    Cols build; // leaf-partitioned build side (keys and payloads)
    const LeafTables * lt; // lazily built tables (lt->state set)
    const uint32_t * leaf_off;
    uint32_t b1, total_bits;
    uint64_t budget_bytes; // the whole run's budget (bep_budget_mib)
};
struct BepEngineResult
{
    int err;           // device error code (0: none)
    uint64_t out_rows; // output rows of the join (may exceed the output's capacity)
    uint64_t evictions, refinements, skip_retries, tables_built, evict_phases, peak_bytes, pool_bytes;
    double ms_shuffle, ms_evict, ms_probe; // one group's time in scatter/refine, eviction bookkeeping and probing
    uint32_t groups;
};
// Whether the engine takes this radix configuration (first pass 1..11 bits,
// at most 13 bits below it).
bool bep_engine_supported(uint32_t b1, uint32_t total_bits);
// One engine run into `out` (rows past out->cap are counted, not written).
BepEngineResult bep_engine_run(phj_ctx * ctx, Scratch & s, const BepEngineInput & in, phj_output * out);

// One join on its own (the CHJ scheme), for a batched join that needs more
// output rows than the batch gave it.
phj_output * join_alone(phj_ctx * ctx, const phj_table & B, const phj_table & P);

// Lookups, then an exactly sized output, then the projection.
phj_output * probe_join(phj_ctx * ctx, Scratch & s, const ProbeArgs & a, const phj_schema & left, const phj_schema & right);
// Sets a.packed (and packed_off) when the plain projection can use packed
// build payloads (a.any_dup known, build_rows rows in a.build).
void pack_build_payloads(phj_ctx * ctx, Scratch & s, ProbeArgs & a, uint64_t build_rows);
// The two halves: lookups + chunk-offset scan (returns the output rows), and
// the projection into `out` from row `out_base` on.
uint64_t probe_chunks(uint64_t probe_rows);
uint64_t probe_lookup(phj_ctx * ctx, Scratch & s, const ProbeArgs & a, uint32_t * heads, uint32_t * counts);
void probe_project(phj_ctx * ctx, const ProbeArgs & a, phj_output * out, uint64_t out_base, const uint32_t * heads, const uint32_t * offs,
                   uint64_t rows);
phj_output * new_output(phj_ctx * ctx, const phj_schema & left, const phj_schema & right, uint64_t cap);
void free_output(phj_ctx * ctx, phj_output * o);

// ----- gen.cu -----------------------------------------------------------------------------
// Fills t's columns; returns the number of distinct build keys for kinds 0/2.
uint64_t generate_rows(phj_ctx * ctx, const phj_gen_spec & spec, phj_table & t);
void fingerprint(phj_ctx * ctx, const phj_output & out, uint64_t fp[3]);

// ----- per-module kernel attributes (dynamic shared memory opt-in) -------------
void set_partition_smem_limits(int smem_optin);
void set_build_smem_limits(int smem_optin);

// Makes the context's device current for one call and gives the caller's
// device back afterwards: a context may be used from any host thread (the
// request loop's workers are threads of their own) whatever device that
// thread has current.
// A device that cannot be made current is recorded in `err` (the calls
// then fail with PHJ_ERR_CUDA before any launch); an error the caller had
// pending is left as it was unless one of these calls failed.
struct DeviceScope
{
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(const phj_ctx * ctx)
    {
        if (!ctx)
            return;
        int cur = -1;
        err = cudaGetDevice(&cur);
        if (err == cudaSuccess && cur != ctx->device)
        {
            err = cudaSetDevice(ctx->device);
            if (err == cudaSuccess)
                prev = cur;
        }
        if (err != cudaSuccess)
            cudaGetLastError(); // the error just recorded, not the caller's
    }
    bool ok() const { return err == cudaSuccess; }
    std::string message(const phj_ctx * ctx) const
    {
        return "cannot make device " + std::to_string(ctx ? ctx->device : -1) + " current: " + cudaGetErrorString(err);
    }
    ~DeviceScope()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope & operator=(const DeviceScope &) = delete;
};

// Runs f on the context's device, turning exceptions into a status and the
// context's last error.
template <class F>
inline phj_status guard(phj_ctx * ctx, F && f)
{
    DeviceScope dev(ctx);
    if (!dev.ok())
    {
        if (ctx)
            ctx->last_error = dev.message(ctx);
        return PHJ_ERR_CUDA;
    }
    try
    {
        f();
        if (ctx)
            ctx->last_error.clear();
        return PHJ_OK;
    }
    catch (const Error & e)
    {
        if (ctx)
            ctx->last_error = e.what();
        return e.status;
    }
    catch (const std::bad_alloc &)
    {
        if (ctx)
            ctx->last_error = "host allocation failed";
        return PHJ_ERR_OUT_OF_MEMORY;
    }
    catch (const std::exception & e)
    {
        if (ctx)
            ctx->last_error = e.what();
        return PHJ_ERR_CUDA;
    }
}

} // namespace phjg
