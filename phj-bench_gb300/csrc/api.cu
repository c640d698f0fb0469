// api.cu -- the C ABI (include/phj_gpu.h): context, streams of rows on the
// device, the three join schemes, outputs, and measurement hooks.
#include "internal.h"

#include <cstdio>
#include <functional>
#include <memory>
#include <cstring>
#include <new>

namespace phjg
{
// ---------------------------------------------------------------------------
// errors, launches, timing
// ---------------------------------------------------------------------------
void cuda_check(cudaError_t e, const char * what, const char * file, int line)
{
    if (e == cudaSuccess)
        return;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    throw Error(e == cudaErrorMemoryAllocation ? PHJ_ERR_OUT_OF_MEMORY : PHJ_ERR_CUDA, buf);
}

void after_launch(phj_ctx * ctx, const char * name, const char * file, int line)
{
    ++ctx->launches;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
    {
        char buf[512];
        std::snprintf(buf, sizeof(buf), "launch of %s failed: %s (%s:%d)", name, cudaGetErrorString(e), file, line);
        throw Error(PHJ_ERR_CUDA, buf);
    }
}

cudaEvent_t take_event(phj_ctx * ctx)
{
    if (ctx->event_next == ctx->event_pool.size())
    {
        cudaEvent_t e;
        PHJ_CUDA(cudaEventCreate(&e));
        ctx->event_pool.push_back(e);
    }
    return ctx->event_pool[ctx->event_next++];
}

void begin_run(phj_ctx * ctx)
{
    ctx->records.clear();
    ctx->event_next = 0;
    reset_accounting(ctx);
}

KTimer::KTimer(phj_ctx * c, const char * name, uint64_t rows, uint64_t bytes)
    : ctx(c)
{
    if (!ctx->time_kernels || !name)
        return;
    KernelRecord r;
    r.name = name;
    r.rows = rows;
    r.bytes = bytes;
    r.start = take_event(ctx);
    r.stop = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(r.start, ctx->stream));
    ctx->records.push_back(r);
    idx = (int)ctx->records.size() - 1;
}

KTimer::~KTimer()
{
    if (idx >= 0)
        cudaEventRecord(ctx->records[idx].stop, ctx->stream);
}

float event_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    PHJ_CUDA(cudaEventElapsedTime(&ms, a, b));
    return ms;
}

// ---------------------------------------------------------------------------
// allocation: the context's stream-ordered pool, with per-run accounting
// ---------------------------------------------------------------------------
void * dalloc(phj_ctx * ctx, size_t bytes)
{
    void * p = nullptr;
    const size_t rounded = (bytes + 255) & ~size_t(255);
    const cudaError_t e = cudaMallocFromPoolAsync(&p, rounded, ctx->pool, ctx->stream);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        char buf[160];
        std::snprintf(buf, sizeof(buf), "device allocation of %zu bytes failed: %s", rounded, cudaGetErrorString(e));
        throw Error(PHJ_ERR_OUT_OF_MEMORY, buf);
    }
    ctx->live.emplace_back(p, rounded);
    ctx->cur_bytes += rounded;
    ctx->peak_bytes = std::max(ctx->peak_bytes, ctx->cur_bytes);
    return p;
}

namespace
{
struct SmallReadArgs
{
    const uint8_t * src[kMaxSmallReads];
    uint32_t bytes[kMaxSmallReads];
    uint32_t off[kMaxSmallReads];
    uint32_t n;
};

__global__ void k_read_small(const __grid_constant__ SmallReadArgs r, uint8_t * dst)
{
    for (uint32_t i = 0; i < r.n; ++i)
        for (uint32_t b = threadIdx.x; b < r.bytes[i]; b += blockDim.x)
            dst[r.off[i] + b] = r.src[i][b];
    __threadfence_system();
}
} // namespace

void read_small(phj_ctx * ctx, std::initializer_list<SmallRead> reads)
{
    if (!ctx->host_small)
    {
        PHJ_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&ctx->host_small), kSmallReadBytes, cudaHostAllocMapped));
        PHJ_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&ctx->host_small_dev), ctx->host_small, 0));
    }
    SmallReadArgs r{};
    uint32_t off = 0;
    for (const SmallRead & x : reads)
    {
        if (r.n == kMaxSmallReads || off + x.bytes > kSmallReadBytes)
            throw Error(PHJ_ERR_CUDA, "internal: read_small over its buffer");
        r.src[r.n] = static_cast<const uint8_t *>(x.src);
        r.bytes[r.n] = x.bytes;
        r.off[r.n++] = off;
        off += (x.bytes + 7) & ~7u;
    }
    k_read_small<<<1, 32, 0, ctx->stream>>>(r, ctx->host_small_dev);
    PHJ_LAUNCHED(ctx, "read_small");
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    off = 0;
    for (const SmallRead & x : reads)
    {
        std::memcpy(x.dst, ctx->host_small + off, x.bytes);
        off += (x.bytes + 7) & ~7u;
    }
}

void dfree(phj_ctx * ctx, void * p)
{
    if (!p)
        return;
    for (size_t i = ctx->live.size(); i-- > 0;)
        if (ctx->live[i].first == p)
        {
            ctx->cur_bytes -= ctx->live[i].second;
            ctx->live[i] = ctx->live.back();
            ctx->live.pop_back();
            break;
        }
    cudaFreeAsync(p, ctx->stream);
}

void reset_accounting(phj_ctx * ctx)
{
    ctx->peak_bytes = ctx->cur_bytes;
}

// ---------------------------------------------------------------------------
// columns
// ---------------------------------------------------------------------------
Cols cols_of(const phj_table & t)
{
    Cols c{};
    c.keys = t.keys;
    c.n = t.schema.n_payloads;
    for (uint32_t i = 0; i < c.n; ++i)
    {
        c.col[i] = t.cols[i];
        c.width[i] = (uint8_t)payload_width(t.schema.types[i]);
    }
    return c;
}

Cols alloc_cols_like(Scratch & s, const phj_schema & schema, uint64_t rows)
{
    Cols c{};
    c.keys = s.get<uint64_t>(rows);
    c.n = schema.n_payloads;
    for (uint32_t i = 0; i < c.n; ++i)
    {
        c.width[i] = (uint8_t)payload_width(schema.types[i]);
        c.col[i] = s.get<uint8_t>(rows * c.width[i]);
    }
    return c;
}

uint32_t max_width(const Cols & c)
{
    uint32_t w = 0;
    for (uint32_t i = 0; i < c.n; ++i)
        w = std::max<uint32_t>(w, c.width[i]);
    return w;
}

// Moves an output to a larger capacity, keeping its first `keep` rows.
void grow_output(phj_ctx * ctx, phj_output * o, uint64_t cap, uint64_t keep)
{
    phj_output * n = new_output(ctx, o->left, o->right, cap);
    PHJ_CUDA(cudaMemcpyAsync(n->keys, o->keys, keep * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    for (uint32_t c = 0; c < o->left.n_payloads; ++c)
        PHJ_CUDA(cudaMemcpyAsync(n->lcol[c], o->lcol[c], keep * payload_width(o->left.types[c]), cudaMemcpyDeviceToDevice, ctx->stream));
    for (uint32_t c = 0; c < o->right.n_payloads; ++c)
        PHJ_CUDA(cudaMemcpyAsync(n->rcol[c], o->rcol[c], keep * payload_width(o->right.types[c]), cudaMemcpyDeviceToDevice, ctx->stream));
    std::swap(*o, *n);
    free_output(ctx, n);
}

namespace
{
// Non-empty first-pass buckets of a probe batch: each is one refinement
// (its rows go on to leaf depth).
__global__ void k_count_nonempty(const uint32_t * __restrict__ off, uint32_t n, unsigned long long * __restrict__ ctr)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ne = i < n && off[i + 1] > off[i];
    const uint32_t m = __ballot_sync(0xffffffffu, ne);
    if ((threadIdx.x & 31) == 0 && m)
        atomicAdd(ctr, (unsigned long long)__popc(m));
}

// Columns of a table advanced by `r0` rows.
Cols cols_from(const Cols & c, uint64_t r0)
{
    Cols o = c;
    if (o.keys)
        o.keys += r0;
    for (uint32_t i = 0; i < c.n; ++i)
        o.col[i] = static_cast<uint8_t *>(c.col[i]) + r0 * c.width[i];
    return o;
}
void check_schema(const phj_schema & s, const char * side)
{
    if (s.n_payloads > PHJ_MAX_PAYLOADS)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, std::string(side) + ": more than 8 payload columns");
    for (uint32_t c = 0; c < s.n_payloads; ++c)
        if (s.types[c] > PHJ_U128)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, std::string(side) + ": unknown payload type");
}

std::vector<uint32_t> check_bits(const uint8_t * bits, uint32_t n)
{
    if (n == 0 || bits == nullptr)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, "radixShuffle: at least one pass required");
    std::vector<uint32_t> v;
    uint32_t total = 0;
    for (uint32_t i = 0; i < n; ++i)
    {
        if (bits[i] == 0 || bits[i] > 16)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "partition bits per pass must be in [1, 16]");
        v.push_back(bits[i]);
        total += bits[i];
    }
    if (total == 0 || total > 32)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, "radixShuffle: total partition bits must be in [1, 32]");
    if (total > 24)
        throw Error(PHJ_ERR_UNSUPPORTED, "device schemes support at most 24 total partition bits (16M leaves)");
    return v;
}

void check_sides(const phj_table * b, const phj_table * p)
{
    if (!b || !p)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, "null build or probe table");
    if (b->rows >= (1ull << 31) || p->rows >= (1ull << 32))
        throw Error(PHJ_ERR_UNSUPPORTED, "device schemes support < 2^31 build rows and < 2^32 probe rows");
}

} // namespace

phj_output * new_output(phj_ctx * ctx, const phj_schema & left, const phj_schema & right, uint64_t cap)
{
    phj_output * o = new phj_output();
    o->left = left;
    o->right = right;
    o->cap = cap;
    try
    {
        o->keys = dalloc_n<uint64_t>(ctx, cap);
        o->bytes += cap * 8;
        for (uint32_t c = 0; c < left.n_payloads; ++c)
        {
            o->lcol[c] = dalloc(ctx, std::max<uint64_t>(1, cap * payload_width(left.types[c])));
            o->bytes += cap * payload_width(left.types[c]);
        }
        for (uint32_t c = 0; c < right.n_payloads; ++c)
        {
            o->rcol[c] = dalloc(ctx, std::max<uint64_t>(1, cap * payload_width(right.types[c])));
            o->bytes += cap * payload_width(right.types[c]);
        }
    }
    catch (...)
    {
        dfree(ctx, o->keys);
        for (uint32_t c = 0; c < PHJ_MAX_PAYLOADS; ++c)
        {
            dfree(ctx, o->lcol[c]);
            dfree(ctx, o->rcol[c]);
        }
        delete o;
        throw;
    }
    return o;
}

void free_output(phj_ctx * ctx, phj_output * o)
{
    if (!o)
        return;
    dfree(ctx, o->keys);
    for (uint32_t c = 0; c < PHJ_MAX_PAYLOADS; ++c)
    {
        dfree(ctx, o->lcol[c]);
        dfree(ctx, o->rcol[c]);
    }
    delete o;
}

namespace
{

void set_block_structure(phj_ctx * ctx, phj_table * t, uint32_t n_blocks, const uint32_t * block_rows)
{
    std::vector<uint64_t> off;
    if (!block_rows || n_blocks == 0)
    {
        off = {0, t->rows};
        t->n_blocks = 1;
        t->uniform_block_rows = 0;
    }
    else
    {
        off.resize(n_blocks + 1);
        off[0] = 0;
        for (uint32_t b = 0; b < n_blocks; ++b)
            off[b + 1] = off[b] + block_rows[b];
        if (off[n_blocks] != t->rows)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "block_rows do not add up to total_rows");
        t->n_blocks = n_blocks;
        uint32_t u = block_rows[0];
        for (uint32_t b = 0; b + 1 < n_blocks; ++b)
            if (block_rows[b] != u)
                u = 0;
        if (u && block_rows[n_blocks - 1] > u)
            u = 0;
        t->uniform_block_rows = u;
    }
    t->block_off = dalloc_n<uint64_t>(ctx, off.size());
    PHJ_CUDA(cudaMemcpyAsync(t->block_off, off.data(), off.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
}

void free_table(phj_ctx * ctx, phj_table * t)
{
    if (!t)
        return;
    if (t->owned)
    {
        dfree(ctx, t->keys);
        for (uint32_t c = 0; c < PHJ_MAX_PAYLOADS; ++c)
            dfree(ctx, t->cols[c]);
    }
    dfree(ctx, t->block_off);
    delete t;
}

phj_table * alloc_table(phj_ctx * ctx, const phj_schema & schema, uint64_t rows)
{
    phj_table * t = new phj_table();
    t->schema = schema;
    t->rows = rows;
    t->owned = true;
    try
    {
        t->keys = dalloc_n<uint64_t>(ctx, rows);
        for (uint32_t c = 0; c < schema.n_payloads; ++c)
            t->cols[c] = dalloc(ctx, std::max<uint64_t>(1, rows * payload_width(schema.types[c])));
    }
    catch (...)
    {
        free_table(ctx, t);
        throw;
    }
    return t;
}

void fill_phase(phj_phase_timing & p, float ms, uint64_t rows)
{
    p.wall_ms = ms;
    p.ns_per_row = rows ? (double)ms * 1e6 / (double)rows : 0.0;
}

// Whether the probe side's first radix pass is written out before probing.
// Materialising orders the probe rows by leaf group so that the tables a
// window of probe rows touches stay in L2; when every table plus the build
// payloads fit in a fraction of L2 anyway, the pass only costs bandwidth.
bool materialize_probe(phj_ctx * ctx, const LeafTables & lt, const phj_table & build, uint32_t n_leaves)
{
    if (ctx->probe_materialize >= 0)
        return ctx->probe_materialize != 0;
    const uint64_t table_bytes = lt.total_cells * sizeof(Cell) + (uint64_t)n_leaves * sizeof(LeafMeta);
    const uint64_t build_bytes = build.rows * (8 + schema_bytes(build.schema)) + (lt.any_dup ? build.rows * 8 : 0);
    return table_bytes + build_bytes > ctx->l2_bytes / 2;
}

// The same decision before the build: cells at load 1/2 (32 B per build
// row) plus the build rows against half of L2.
bool materialize_probe_estimate(phj_ctx * ctx, const phj_table & build)
{
    if (ctx->probe_materialize >= 0)
        return ctx->probe_materialize != 0;
    return build.rows * (32 + 8 + schema_bytes(build.schema)) > ctx->l2_bytes / 2;
}

Cols payload_cols(const Cols & c)
{
    Cols p = c;
    p.keys = nullptr;
    return p;
}

phj_output * probe_into_output(phj_ctx * ctx, Scratch & s, const ProbeArgs & a, const phj_schema & left, const phj_schema & right)
{
    return probe_join(ctx, s, a, left, right);
}

// CHJ probe in windows of sub-tables (the "chj_windows" option): the 256
// top-8-bit sub-tables are taken `windows` at a time in consecutive groups
// (one contiguous region of cells each); a sweep over the whole probe side
// looks up only the rows whose sub-table lies in the current group, so the
// tables that sweep touches are that group's alone and can stay in L2 while
// the probe keys stream past, then projects that sweep's matches after the
// previous sweeps' rows.  Every sweep reads all the probe keys again, and
// the build payloads are gathered in input order.  The output rows are
// those of the one-sweep probe, in another order.
phj_output * probe_chj_windows(phj_ctx * ctx, Scratch & s, const ProbeArgs & a_in, const phj_schema & left, const phj_schema & right,
                               uint32_t windows)
{
    ProbeArgs a = a_in;
    if (a.any_dup && !a.row_cnt)
        a.row_cnt = s.get<uint32_t>(std::max<uint64_t>(a.probe_rows, 1));
    uint32_t * heads = s.get<uint32_t>(std::max<uint64_t>(a.probe_rows, 1));
    uint32_t * counts = s.get<uint32_t>(probe_chunks(a.probe_rows) + 1);
    const uint32_t n_sub = 1u << a.leaf_bits, step = std::max<uint32_t>(n_sub / windows, 1);
    phj_output * o = nullptr;
    uint64_t total = 0;
    try
    {
        for (uint32_t lo = 0; lo < n_sub; lo += step)
        {
            a.win_lo = lo;
            a.win_hi = lo + step;
            Scratch sw(ctx);
            const uint64_t rows = probe_lookup(ctx, sw, a, heads, counts);
            if (!o)
            {
                // first window: the output sized for every window at its rate
                const uint64_t est = (uint64_t)((double)rows * (double)(n_sub / step) * 1.0625) + 4096;
                o = new_output(ctx, left, right, std::max(est, rows));
            }
            else if (total + rows > o->cap)
                grow_output(ctx, o, std::max(o->cap * 2, total + rows), total);
            probe_project(ctx, a, o, total, heads, counts, rows);
            total += rows;
        }
        if (!o)
            o = new_output(ctx, left, right, 0);
        o->rows = total;
    }
    catch (...)
    {
        if (o)
            free_output(ctx, o);
        throw;
    }
    return o;
}
} // namespace

// A bounded device wait that gave up leaves a code in the error word; the
// run fails with PHJ_ERR_DEVICE_TIMEOUT and the word is cleared.
static void check_device_error(phj_ctx * ctx)
{
    int e = 0;
    read_small(ctx, {{&e, ctx->d_err, sizeof(int)}});
    if (e != 0)
    {
        PHJ_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
        char buf[96];
        std::snprintf(buf, sizeof(buf), "a bounded device wait gave up (code %d)", e);
        throw Error(PHJ_ERR_DEVICE_TIMEOUT, buf);
    }
}

// With PHJ_DEBUG set: each timed kernel of the run with its start and end,
// ms from `t0` (kernels on both streams of a scheme).
static void debug_timeline(phj_ctx * ctx, cudaEvent_t t0)
{
    if (!std::getenv("PHJ_DEBUG") || !ctx->time_kernels)
        return;
    for (const auto & r : ctx->records)
    {
        float a = 0.f, b = 0.f;
        if (cudaEventElapsedTime(&a, t0, r.start) != cudaSuccess || cudaEventElapsedTime(&b, t0, r.stop) != cudaSuccess)
        {
            cudaGetLastError();
            continue;
        }
        std::fprintf(stderr, "[phj] timeline %-22s %8.3f %8.3f %7.3f\n", r.name.c_str(), a, b, b - a);
    }
}

// ---------------------------------------------------------------------------
// schemes
// ---------------------------------------------------------------------------
static void run_chj(phj_ctx * ctx, const phj_table & B, const phj_table & P, phj_output ** out, phj_chj_result * res)
{
    begin_run(ctx);
    Scratch s(ctx);
    cudaEvent_t e0 = take_event(ctx), e1 = take_event(ctx), e2 = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(e0, ctx->stream));
    LeafTables lt;
    lt.next = s.get<uint64_t>(B.rows);
    build_global_table(ctx, s, B, 8, lt);
    PHJ_CUDA(cudaEventRecord(e1, ctx->stream));
    ProbeArgs a{};
    a.probe = cols_of(P);
    a.probe_rows = P.rows;
    a.build = payload_cols(cols_of(B));
    a.meta = lt.meta;
    a.cells = lt.cells;
    a.next = lt.next;
    a.leaf_bits = 8;
    a.chj = 1;
    a.block_off = B.block_off;
    a.uniform_block_rows = B.uniform_block_rows;
    a.any_dup = lt.any_dup;
    a.uniform_log2cap = -1;
    pack_build_payloads(ctx, s, a, B.rows);
    phj_output * o =
        ctx->chj_windows > 1 ? probe_chj_windows(ctx, s, a, B.schema, P.schema, ctx->chj_windows) : probe_into_output(ctx, s, a, B.schema, P.schema);
    PHJ_CUDA(cudaEventRecord(e2, ctx->stream));
    PHJ_CUDA(cudaEventSynchronize(e2));
    check_device_error(ctx);
    debug_timeline(ctx, e0);
    if (res)
    {
        fill_phase(res->build, event_ms(e0, e1), B.rows);
        fill_phase(res->probe, event_ms(e1, e2), P.rows);
        res->e2e_wall_ms = event_ms(e0, e2);
        res->peak_mem_bytes = ctx->peak_bytes;
    }
    *out = o;
}

phj_output * join_alone(phj_ctx * ctx, const phj_table & B, const phj_table & P)
{
    phj_output * o = nullptr;
    run_chj(ctx, B, P, &o, nullptr);
    return o;
}

// Bits of the probe side's first (and only written) radix pass in PHJ-PURE.
// The lookup takes every row's leaf from the whole hash, so this width is a
// performance choice, not the configuration's: buckets narrow enough that
// one bucket's leaf tables and build payloads stay in L2 while its rows are
// probed, and otherwise as wide as possible (fewer buckets: longer runs per
// bucket in the scatter's tiles).  The working set is estimated before the
// tables exist (the pass runs beside the build side): cells at the load
// factor with up to 2x for power-of-two and uniform sizing, the next-chain
// and the payloads; the widest buckets whose share stays within a fifth of
// L2 are taken (16M x 256M: 6 bits, 6.83 ms against 7.12 ms at the
// configuration's 8 and 7.35 ms at 5).  "probe_pass_bits" overrides it.
static uint32_t probe_pass_bits(const phj_ctx * ctx, const std::vector<uint32_t> & bits, const phj_table & build)
{
    uint32_t total = 0;
    for (uint32_t b : bits)
        total += b;
    const uint32_t most = std::min<uint32_t>(total, 11);
    if (ctx->probe_pass_bits)
        return std::min<uint32_t>(ctx->probe_pass_bits, most);
    const uint64_t ws = build.rows * (16ull * ctx->table_cap_pct / 100 * 2 + 8 + schema_bytes(build.schema));
    const uint64_t target = std::max<uint64_t>(ctx->l2_bytes / 5, 1);
    uint32_t b = 1;
    while (b < most && (ws >> b) > target)
        ++b;
    return b;
}

static void run_phj_pure(phj_ctx * ctx, const phj_table & B, const phj_table & P, const std::vector<uint32_t> & bits, phj_output ** out,
                         phj_phj_result * res)
{
    begin_run(ctx);
    Scratch s(ctx);
    uint32_t total_bits = 0;
    for (uint32_t b : bits)
        total_bits += b;
    const uint32_t n_leaves = 1u << total_bits;
    cudaEvent_t ev[9];
    for (auto & e : ev)
        e = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(ev[0], ctx->stream));

    // -------- PROBE SHUFFLE (src/PHJ.cpp:225-228): first pass only, on the
    // side stream, beside the build side's work --------
    ProbeArgs a{};
    a.probe = cols_of(P);
    const bool mat = materialize_probe_estimate(ctx, B) && P.rows > 0;
    cudaStream_t main_stream = ctx->stream;
    // the two sides' partition passes share the GPU: register-capped scatter
    struct BesideGuard
    {
        phj_ctx * c;
        ~BesideGuard() { c->p1_beside = false; }
    } beside_guard{ctx};
    ctx->p1_beside = mat;
    if (mat)
    {
        if (!ctx->side)
            PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        PHJ_CUDA(cudaStreamWaitEvent(ctx->side, ev[0], 0));
        ctx->stream = ctx->side;
        try
        {
            PHJ_CUDA(cudaEventRecord(ev[5], ctx->stream));
            const uint32_t pb = probe_pass_bits(ctx, bits, B);
            const Cols ppart = alloc_cols_like(s, P.schema, P.rows);
            const bool split = pb > 11;
            const Cols ptmp = split ? alloc_cols_like(s, P.schema, P.rows) : ppart;
            uint32_t * poff = s.get<uint32_t>((1ull << pb) + 1);
            // a two-stage ring leaves shared memory on each SM for the build
            // side's kernels running beside this pass (unless pinned)
            const uint32_t pinned_stages = ctx->p1_stages;
            if (!pinned_stages)
                ctx->p1_stages = 2;
            try
            {
                radix_partition(ctx, s, a.probe, P.rows, {pb}, ppart, ptmp, poff, "probe_scatter");
            }
            catch (...)
            {
                ctx->p1_stages = pinned_stages;
                throw;
            }
            ctx->p1_stages = pinned_stages;
            a.probe = ppart;
            PHJ_CUDA(cudaEventRecord(ev[6], ctx->stream));
        }
        catch (...)
        {
            ctx->stream = main_stream;
            cudaStreamSynchronize(ctx->side);
            throw;
        }
        ctx->stream = main_stream;
    }

    // -------- BUILD SHUFFLE (src/PHJ.cpp:220-223) --------
    const Cols bin = cols_of(B);
    const Cols bpart = alloc_cols_like(s, B.schema, B.rows);
    const Cols btmp = alloc_cols_like(s, B.schema, B.rows);
    uint32_t * leaf_off = s.get<uint32_t>((uint64_t)n_leaves + 1);
    LeafTables lt;
    bool grouped = false;
    try
    {
        radix_partition(ctx, s, bin, B.rows, bits, bpart, btmp, leaf_off, "build_scatter");
        PHJ_CUDA(cudaEventRecord(ev[1], ctx->stream));

        // build payloads packed for the projection on a third stream,
        // beside the leaf tables (both only read the partitioned rows);
        // dropped if a key repeats
        a.build = payload_cols(bpart);
        a.any_dup = 0;
        if (!ctx->aux)
            PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
        PHJ_CUDA(cudaEventRecord(ev[7], ctx->stream));
        PHJ_CUDA(cudaStreamWaitEvent(ctx->aux, ev[7], 0));
        ctx->stream = ctx->aux;
        try
        {
            pack_build_payloads(ctx, s, a, B.rows);
        }
        catch (...)
        {
            ctx->stream = main_stream;
            throw;
        }
        PHJ_CUDA(cudaEventRecord(ev[8], ctx->stream));
        ctx->stream = main_stream;

        // -------- BUILD: per-leaf tables (src/PHJ.cpp:260-282) --------
        lt.next = s.get<uint64_t>(B.rows);
        build_leaf_tables(ctx, s, bpart, leaf_off, n_leaves, lt);
        // repeated keys: each key's rows made contiguous, so the probe
        // expands a match as a row range
        grouped = group_leaf_duplicates(ctx, bpart, btmp, leaf_off, n_leaves, lt);
        if (lt.any_dup)
            a.packed = nullptr;
        PHJ_CUDA(cudaEventRecord(ev[2], ctx->stream));
    }
    catch (...)
    {
        // the side and aux streams' buffers are freed with the scratch
        if (mat)
            cudaStreamSynchronize(ctx->side);
        if (ctx->aux)
            cudaStreamSynchronize(ctx->aux);
        throw;
    }
    if (mat)
        PHJ_CUDA(cudaStreamWaitEvent(ctx->stream, ev[6], 0));
    PHJ_CUDA(cudaStreamWaitEvent(ctx->stream, ev[8], 0));
    PHJ_CUDA(cudaEventRecord(ev[3], ctx->stream));

    // -------- PROBE with projection (src/PHJ.cpp:284-299) --------
    a.probe_rows = P.rows;
    a.build = payload_cols(grouped ? btmp : bpart);
    a.grouped = grouped ? 1 : 0;
    a.meta = lt.meta;
    a.cells = lt.cells;
    a.next = lt.next;
    a.leaf_bits = total_bits;
    a.chj = 0;
    a.any_dup = lt.any_dup;
    a.uniform_log2cap = lt.uniform_log2cap;
    phj_output * o = probe_into_output(ctx, s, a, B.schema, P.schema);
    PHJ_CUDA(cudaEventRecord(ev[4], ctx->stream));
    PHJ_CUDA(cudaEventSynchronize(ev[4]));
    check_device_error(ctx);
    debug_timeline(ctx, ev[0]);
    if (res)
    {
        fill_phase(res->build_shuffle, event_ms(ev[0], ev[1]), B.rows);
        fill_phase(res->build, event_ms(ev[1], ev[2]), B.rows);
        // the probe side's first pass runs beside the build: its own span
        fill_phase(res->probe_shuffle, mat ? event_ms(ev[5], ev[6]) : 0.f, P.rows);
        fill_phase(res->probe, event_ms(ev[3], ev[4]), P.rows);
        res->e2e_wall_ms = event_ms(ev[0], ev[4]);
        res->peak_mem_bytes = ctx->peak_bytes;
    }
    *out = o;
}

// PHJ (BEP).  The build side is shuffled to full leaf depth and its leaf
// tables are planned but left NOT_BUILT; the probe side streams through in
// batches of at most the byte budget.  Each batch is scattered by the first
// radix pass (probe shuffle), the leaves it touches and that are still
// NOT_BUILT are built from a device work queue, then the batch is probed.
// A batch's probe drains every leaf it touched, which is the device form of
// the reference's eviction (src/PHJBep.cpp:113-790).
static void run_phj_bep(phj_ctx * ctx, const phj_table & B, const phj_table & P, const std::vector<uint32_t> & bits, uint64_t budget_mib,
                        phj_output ** out, phj_bep_result * res)
{
    begin_run(ctx);
    Scratch s(ctx);
    uint32_t total_bits = 0;
    for (uint32_t b : bits)
        total_bits += b;
    const uint32_t n_leaves = 1u << total_bits;
    cudaEvent_t ev[3], eb[5];
    for (auto & e : ev)
        e = take_event(ctx);
    for (auto & e : eb)
        e = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(ev[0], ctx->stream));

    // probe batches: buffers, and the touched-leaf bitmap their first passes fill
    const uint64_t row_bytes = 8 + schema_bytes(P.schema);
    const uint64_t budget_rows = (budget_mib << 20) / row_bytes;
    const uint64_t batch_rows = std::min<uint64_t>(std::max<uint64_t>(P.rows, 1), std::max<uint64_t>(4096, budget_rows & ~uint64_t(255)));
    // the probe batches' written pass: the configuration's first pass, or
    // the "probe_pass_bits" option
    const uint32_t pb = ctx->probe_pass_bits ? std::min<uint32_t>(ctx->probe_pass_bits, std::min<uint32_t>(total_bits, 11)) : bits[0];
    const uint32_t p1 = 1u << pb;
    const Cols pin = cols_of(P);
    const Cols ppart = alloc_cols_like(s, P.schema, batch_rows);
    const Cols ptmp = pb > 11 ? alloc_cols_like(s, P.schema, batch_rows) : ppart;
    uint32_t * poff = s.get<uint32_t>((uint64_t)p1 + 1);
    uint32_t * touched = s.get<uint32_t>((n_leaves + 31) / 32);
    PHJ_CUDA(cudaMemsetAsync(touched, 0, (size_t)((n_leaves + 31) / 32) * 4, ctx->stream));
    const Cols bin = cols_of(B);
    const Cols bpart = alloc_cols_like(s, B.schema, B.rows);
    const Cols btmp = alloc_cols_like(s, B.schema, B.rows);
    uint32_t * leaf_off = s.get<uint32_t>((uint64_t)n_leaves + 1);

    // -------- PROBE SHUFFLE of the first batch, on the side stream beside
    // the build shuffle (it needs nothing of the build side) --------
    cudaStream_t main_stream = ctx->stream;
    const bool early = P.rows > 0;
    cudaEvent_t es[2] = {take_event(ctx), take_event(ctx)}; // the side pass's span
    struct BesideGuard
    {
        phj_ctx * c;
        ~BesideGuard() { c->p1_beside = false; }
    } beside_guard{ctx};
    ctx->p1_beside = early;
    if (early)
    {
        if (!ctx->side)
            PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        cudaEvent_t ready = take_event(ctx);
        PHJ_CUDA(cudaEventRecord(ready, ctx->stream));
        PHJ_CUDA(cudaStreamWaitEvent(ctx->side, ready, 0));
        ctx->stream = ctx->side;
        const uint32_t pinned_stages = ctx->p1_stages;
        try
        {
            PHJ_CUDA(cudaEventRecord(es[0], ctx->stream));
            // the batch's first radix pass also flags the leaves its rows
            // touch (its histogram reads every key once anyway); a two-stage
            // ring leaves shared memory for the build side's kernels
            ctx->leaf_mark = LeafMark{touched, 64u - total_bits, (n_leaves + 31) / 32};
            if (!pinned_stages)
                ctx->p1_stages = 2;
            radix_partition(ctx, s, pin, std::min(batch_rows, P.rows), {pb}, ppart, ptmp, poff, "probe_scatter");
            ctx->p1_stages = pinned_stages;
            ctx->leaf_mark = LeafMark{};
            PHJ_CUDA(cudaEventRecord(es[1], ctx->stream));
        }
        catch (...)
        {
            ctx->p1_stages = pinned_stages;
            ctx->leaf_mark = LeafMark{};
            ctx->stream = main_stream;
            cudaStreamSynchronize(ctx->side);
            throw;
        }
        ctx->stream = main_stream;
    }

    // -------- BUILD SHUFFLE, full leaf depth (src/PHJBep.cpp:128-141) --------
    try
    {
        radix_partition(ctx, s, bin, B.rows, bits, bpart, btmp, leaf_off, "build_scatter");
    }
    catch (...)
    {
        if (early)
            cudaStreamSynchronize(ctx->side); // its buffers are freed with the scratch
        throw;
    }
    PHJ_CUDA(cudaEventRecord(ev[1], ctx->stream));
    ctx->p1_beside = false;

    // -------- BUILD: table layout only; cells are built on first use --------
    LeafTables lt;
    lt.next = s.get<uint64_t>(B.rows);
    build_leaf_tables(ctx, s, bpart, leaf_off, n_leaves, lt, true);
    if (ctx->test_stuck_leaf >= 0 && (uint64_t)ctx->test_stuck_leaf < n_leaves)
    {
        const uint32_t building = 1;
        PHJ_CUDA(cudaMemcpyAsync(lt.state + ctx->test_stuck_leaf, &building, sizeof(building), cudaMemcpyHostToDevice, ctx->stream));
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    PHJ_CUDA(cudaEventRecord(ev[2], ctx->stream));

    unsigned long long * ctr = s.get<unsigned long long>(4);
    PHJ_CUDA(cudaMemsetAsync(ctr, 0, 4 * sizeof(unsigned long long), ctx->stream));

    ProbeArgs a{};
    a.build = payload_cols(bpart);
    a.meta = lt.meta;
    a.cells = lt.cells;
    a.next = lt.next;
    a.leaf_bits = total_bits;
    a.chj = 0;
    a.any_dup = 0;
    a.uniform_log2cap = lt.uniform_log2cap;
    BepLeaves bl{};
    bl.state = lt.state;
    bl.touched = touched;
    bl.leaf_off = leaf_off;
    bl.build_keys = bpart.keys;
    bl.meta = lt.meta;
    bl.cells = lt.cells;
    bl.next = lt.next;
    bl.leaf_bits = total_bits;
    bl.n_leaves = n_leaves;
    bl.smem_cells = (uint32_t)std::min<uint64_t>(lt.uniform_log2cap >= 0 ? (1ull << lt.uniform_log2cap) : bit_ceil64(2ull * std::max<uint32_t>(lt.max_rows, 1)),
                                                 8192);
    bl.wait_limit_ns = (uint64_t)ctx->wait_limit_ms * 1000000ull;
    bl.ctr = ctr;
    bl.queue = s.get<uint32_t>(n_leaves);
    bl.queue_len = s.get<uint32_t>(2);
    bl.any_dup = s.get<int>(1);
    PHJ_CUDA(cudaMemsetAsync(bl.any_dup, 0, sizeof(int), ctx->stream));

    // -------- PROBE: budget-sized batches --------
    uint32_t * heads = s.get<uint32_t>(batch_rows);
    uint32_t * counts = s.get<uint32_t>(probe_chunks(batch_rows) + 1);
    a.row_cnt = s.get<uint32_t>(batch_rows); // match counts when keys repeat
    phj_output * o = nullptr;
    uint64_t total = 0, peak_rows = 0;
    float t_shuffle = 0.f, t_probe = 0.f, t_lazy = 0.f;
    try
    {
        uint32_t e = 1;
        for (uint64_t r0 = 0; r0 < P.rows; r0 += batch_rows, ++e)
        {
            const uint64_t n_b = std::min(batch_rows, P.rows - r0);
            peak_rows = std::max(peak_rows, n_b);
            Scratch sb(ctx);
            PHJ_CUDA(cudaEventRecord(eb[0], ctx->stream));
            if (r0 == 0)
                PHJ_CUDA(cudaStreamWaitEvent(ctx->stream, es[1], 0)); // the first batch's pass ran on the side stream
            else
            {
                // the batch's first radix pass also flags the leaves its
                // rows touch (its histogram reads every key once anyway)
                ctx->leaf_mark = LeafMark{touched, 64u - total_bits, (n_leaves + 31) / 32};
                radix_partition(ctx, sb, cols_from(pin, r0), n_b, {pb}, ppart, ptmp, poff, "probe_scatter");
                ctx->leaf_mark = LeafMark{};
            }
            k_count_nonempty<<<(unsigned)ceil_div(p1, 256), 256, 0, ctx->stream>>>(poff, p1, ctr + 3);
            PHJ_LAUNCHED(ctx, "count_refinements");
            PHJ_CUDA(cudaEventRecord(eb[1], ctx->stream));
            a.probe = ppart;
            a.probe_rows = n_b;
            // lazy build of the leaves this batch touches
            PHJ_CUDA(cudaEventRecord(eb[3], ctx->stream));
            a.any_dup = bep_build_touched(ctx, bl) ? 1 : 0;
            check_device_error(ctx);
            PHJ_CUDA(cudaEventRecord(eb[4], ctx->stream));
            const uint64_t rows = probe_lookup(ctx, sb, a, heads, counts);
            if (!o)
            {
                // first batch: extrapolate the output size over the stream
                const uint64_t est = (uint64_t)((double)rows * (double)P.rows / (double)n_b * 1.0625) + 4096;
                o = new_output(ctx, B.schema, P.schema, std::max(est, rows));
            }
            else if (total + rows > o->cap)
                grow_output(ctx, o, std::max(o->cap * 2, total + rows), total);
            probe_project(ctx, a, o, total, heads, counts, rows);
            total += rows;
            PHJ_CUDA(cudaEventRecord(eb[2], ctx->stream));
            PHJ_CUDA(cudaEventSynchronize(eb[2]));
            t_shuffle += r0 == 0 ? event_ms(es[0], es[1]) : event_ms(eb[0], eb[1]);
            t_lazy += event_ms(eb[3], eb[4]);
            t_probe += event_ms(eb[4], eb[2]);
        }
        if (!o)
            o = new_output(ctx, B.schema, P.schema, 0);
        o->rows = total;
        PHJ_CUDA(cudaEventRecord(eb[0], ctx->stream));
        PHJ_CUDA(cudaEventSynchronize(eb[0]));
        check_device_error(ctx);
        debug_timeline(ctx, ev[0]);
    }
    catch (...)
    {
        free_output(ctx, o);
        throw;
    }
    if (res)
    {
        unsigned long long c[4] = {};
        PHJ_CUDA(cudaMemcpy(c, ctr, sizeof(c), cudaMemcpyDeviceToHost));
        const float bs = event_ms(ev[0], ev[1]), bd = event_ms(ev[1], ev[2]) + t_lazy, e2e = event_ms(ev[0], eb[0]);
        fill_phase(res->build_shuffle, bs, B.rows);
        fill_phase(res->build, bd, B.rows);
        fill_phase(res->probe_shuffle, t_shuffle, P.rows);
        fill_phase(res->probe, t_probe, P.rows);
        fill_phase(res->eviction_overhead, std::max(0.f, e2e - bs - bd - t_shuffle - t_probe), P.rows);
        res->e2e_wall_ms = e2e;
        res->peak_mem_bytes = ctx->peak_bytes;
        res->bep_budget_mib = budget_mib;
        res->bep_evictions = c[2];
        res->bep_refinements = c[3];
        res->bep_peak_bytes = peak_rows * row_bytes;
        res->bep_build_skip_retries = c[1];
    }
    *out = o;
}

// PHJ (BEP) with the byte budget on the device (bep_engine.cu): the build
// side is partitioned to full leaf depth (src/PHJBep.cpp:128-141) and its
// tables only planned; one persistent grid then streams the probe side
// through per-group unrefined chains, refines, evicts and builds leaves
// lazily, and projects into the output.  The output is sized for one row
// per probe row; a join with more output rows (repeated build keys) runs
// the grid again into an output of the exact size the first run counted.
static void run_phj_bep_engine(phj_ctx * ctx, const phj_table & B, const phj_table & P, const std::vector<uint32_t> & bits, uint64_t budget_mib,
                               phj_output ** out, phj_bep_result * res)
{
    begin_run(ctx);
    Scratch s(ctx);
    uint32_t total_bits = 0;
    for (uint32_t b : bits)
        total_bits += b;
    const uint32_t n_leaves = 1u << total_bits;
    cudaEvent_t ev[4];
    for (auto & e : ev)
        e = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(ev[0], ctx->stream));
    // -------- BUILD SHUFFLE, full leaf depth --------
    const Cols bin = cols_of(B);
    const Cols bpart = alloc_cols_like(s, B.schema, B.rows);
    const Cols btmp = alloc_cols_like(s, B.schema, B.rows);
    uint32_t * leaf_off = s.get<uint32_t>((uint64_t)n_leaves + 1);
    radix_partition(ctx, s, bin, B.rows, bits, bpart, btmp, leaf_off, "build_scatter");
    PHJ_CUDA(cudaEventRecord(ev[1], ctx->stream));
    // -------- BUILD: table layout only; each table is built on first use --------
    LeafTables lt;
    lt.next = s.get<uint64_t>(std::max<uint64_t>(B.rows, 1));
    build_leaf_tables(ctx, s, bpart, leaf_off, n_leaves, lt, true);
    if (ctx->test_stuck_leaf >= 0 && (uint64_t)ctx->test_stuck_leaf < n_leaves)
    {
        const uint32_t building = 1;
        PHJ_CUDA(cudaMemcpyAsync(lt.state + ctx->test_stuck_leaf, &building, sizeof(building), cudaMemcpyHostToDevice, ctx->stream));
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    PHJ_CUDA(cudaEventRecord(ev[2], ctx->stream));
    // -------- PROBE: the device budget engine --------
    BepEngineInput in{};
    in.probe = cols_of(P);
    in.probe_rows = P.rows;
    in.build = bpart;
    in.lt = &lt;
    in.leaf_off = leaf_off;
    in.b1 = bits[0];
    in.total_bits = total_bits;
    in.budget_bytes = budget_mib << 20;
    phj_output * o = new_output(ctx, B.schema, P.schema, P.rows);
    BepEngineResult r{};
    try
    {
        if (P.rows > 0)
        {
            r = bep_engine_run(ctx, s, in, o);
            if (r.err == 0 && r.out_rows > o->cap)
            {
                // repeated build keys: more output rows than probe rows
                free_output(ctx, o);
                o = nullptr;
                o = new_output(ctx, B.schema, P.schema, r.out_rows);
                Scratch s2(ctx);
                const uint64_t built = r.tables_built;
                r = bep_engine_run(ctx, s2, in, o);
                r.tables_built += built;
            }
            if (r.err != 0)
            {
                PHJ_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
                PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
                char buf[128];
                if (r.err == 6 || r.err == 7)
                {
                    std::snprintf(buf, sizeof(buf), "PHJ (BEP): the device budget engine ran out of probe blocks (code %d)", r.err);
                    throw Error(PHJ_ERR_CAPACITY, buf);
                }
                std::snprintf(buf, sizeof(buf), "a bounded device wait gave up (code %d)", r.err);
                throw Error(PHJ_ERR_DEVICE_TIMEOUT, buf);
            }
        }
        o->rows = r.out_rows;
        PHJ_CUDA(cudaEventRecord(ev[3], ctx->stream));
        PHJ_CUDA(cudaEventSynchronize(ev[3]));
        debug_timeline(ctx, ev[0]);
    }
    catch (...)
    {
        if (o)
            free_output(ctx, o);
        throw;
    }
    if (std::getenv("PHJ_DEBUG"))
        std::fprintf(stderr,
                     "[phj] bep_engine: %u groups, %llu evict phases, %llu evictions, %llu refinements, peak %.3f GB of %.3f GB budget, pool %.2f GB, "
                     "S %.3f ms E %.3f ms probe %.3f ms\n",
                     r.groups, (unsigned long long)r.evict_phases, (unsigned long long)r.evictions, (unsigned long long)r.refinements,
                     r.peak_bytes / 1e9, (double)(budget_mib << 20) / 1e9, r.pool_bytes / 1e9, r.ms_shuffle, r.ms_evict, r.ms_probe);
    if (res)
    {
        const float bs = event_ms(ev[0], ev[1]), plan = event_ms(ev[1], ev[2]), e2e = event_ms(ev[0], ev[3]);
        fill_phase(res->build_shuffle, bs, B.rows);
        fill_phase(res->build, plan, B.rows); // the lazy builds count as eviction overhead
        fill_phase(res->probe_shuffle, (float)r.ms_shuffle, P.rows);
        fill_phase(res->probe, (float)r.ms_probe, P.rows);
        fill_phase(res->eviction_overhead, std::max(0.f, e2e - bs - plan - (float)r.ms_shuffle - (float)r.ms_probe), P.rows);
        res->e2e_wall_ms = e2e;
        res->peak_mem_bytes = ctx->peak_bytes;
        res->bep_budget_mib = budget_mib;
        res->bep_evictions = r.evictions;
        res->bep_refinements = r.refinements;
        res->bep_peak_bytes = r.peak_bytes;
        res->bep_build_skip_retries = r.skip_retries;
    }
    *out = o;
}

// On every exit from a host-buffer join, errors included, waits for the
// copies still queued on the h2d and d2h streams, so that no buffer the
// table guard or the scratch hands back to the pool (both free in the
// compute stream's order only) is still read or written by a copy.
struct CopyDrain
{
    phj_ctx * c;
    ~CopyDrain()
    {
        if (c->h2d)
            cudaStreamSynchronize(c->h2d);
        if (c->d2h)
            cudaStreamSynchronize(c->d2h);
    }
};

// PHJ-PURE with the inputs and the output in host memory.  The build side
// is uploaded whole; the probe side streams through in chunks on three
// streams: chunk c+1 uploads (h2d) while chunk c is partitioned by the first
// radix pass, looked up and projected (compute) and the output of chunk c-1
// downloads (d2h).  Two device input buffers and per-chunk outputs, each
// reused or freed only after the copy that reads it has finished.  Output
// rows land in the host columns chunk after chunk.
static void run_phj_pure_host(phj_ctx * ctx, const phj_block_stream & hb, const phj_block_stream & hp, const std::vector<uint32_t> & bits,
                              uint64_t out_cap, uint64_t * out_keys, void * const * out_left, void * const * out_right, uint64_t * out_rows,
                              phj_phj_result * res, uint64_t chunk_rows)
{
    if (!ctx->h2d)
        PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking));
    if (!ctx->d2h)
        PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking));
    begin_run(ctx);
    Scratch s(ctx);
    cudaStream_t S = ctx->stream;
    uint32_t total_bits = 0;
    for (uint32_t b : bits)
        total_bits += b;
    const uint32_t n_leaves = 1u << total_bits;
    const uint64_t B_rows = hb.total_rows, P_rows = hp.total_rows;
    const uint64_t C = std::max<uint64_t>(1, std::min<uint64_t>(chunk_rows, std::max<uint64_t>(P_rows, 1)));
    // chunk c covers rows [start(c), start(c + 1)): the first chunk is a
    // quarter of the others, so the first output download starts sooner
    const uint64_t C0 = std::max<uint64_t>(1, std::min<uint64_t>(C, std::max<uint64_t>(C / 4, 4096)));
    auto start = [&](uint64_t c) -> uint64_t { return c == 0 ? 0 : std::min(P_rows, C0 + (c - 1) * C); };
    const uint64_t n_chunks = P_rows == 0 ? 0 : (P_rows <= C0 ? 1 : 1 + ceil_div(P_rows - C0, C));
    cudaEvent_t ev[4];
    for (auto & e : ev)
        e = take_event(ctx);

    // device buffers, all allocated on the compute stream before any copy
    phj_table * B = alloc_table(ctx, hb.schema, B_rows);
    std::unique_ptr<phj_table, std::function<void(phj_table *)>> B_guard(B, [ctx](phj_table * t) { free_table(ctx, t); });
    const CopyDrain drain{ctx}; // destroyed before B_guard and the scratch
    Cols in[2];
    for (auto & c : in)
        c = alloc_cols_like(s, hp.schema, C);
    const Cols bpart = alloc_cols_like(s, hb.schema, B_rows);
    const Cols btmp = alloc_cols_like(s, hb.schema, B_rows);
    uint32_t * leaf_off = s.get<uint32_t>((uint64_t)n_leaves + 1);
    PHJ_CUDA(cudaEventRecord(ev[0], S));
    PHJ_CUDA(cudaStreamWaitEvent(ctx->h2d, ev[0], 0));

    auto upload = [&](const Cols & dst, const phj_block_stream & src, uint64_t r0, uint64_t n) {
        PHJ_CUDA(cudaMemcpyAsync(dst.keys, src.keys + r0, n * 8, cudaMemcpyHostToDevice, ctx->h2d));
        for (uint32_t c = 0; c < src.schema.n_payloads; ++c)
        {
            const uint32_t w = payload_width(src.schema.types[c]);
            PHJ_CUDA(cudaMemcpyAsync(dst.col[c], static_cast<const uint8_t *>(src.payloads[c]) + r0 * w, n * w, cudaMemcpyHostToDevice, ctx->h2d));
        }
    };
    std::vector<cudaEvent_t> up(n_chunks), used(n_chunks), proj(n_chunks), down(n_chunks);
    for (uint64_t c = 0; c < n_chunks; ++c)
    {
        up[c] = take_event(ctx);
        used[c] = take_event(ctx);
        proj[c] = take_event(ctx);
        down[c] = take_event(ctx);
    }
    // build side, then the first two probe chunks
    const Cols bin = cols_of(*B);
    if (B_rows)
        upload(bin, hb, 0, B_rows);
    cudaEvent_t build_up = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(build_up, ctx->h2d));
    auto enqueue_chunk = [&](uint64_t c) {
        if (c >= 2)
            PHJ_CUDA(cudaStreamWaitEvent(ctx->h2d, used[c - 2], 0));
        upload(in[c & 1], hp, start(c), start(c + 1) - start(c));
        PHJ_CUDA(cudaEventRecord(up[c], ctx->h2d));
    };
    for (uint64_t c = 0; c < std::min<uint64_t>(2, n_chunks); ++c)
        enqueue_chunk(c);

    // -------- BUILD SHUFFLE + BUILD (src/PHJ.cpp:220-282) --------
    PHJ_CUDA(cudaStreamWaitEvent(S, build_up, 0));
    radix_partition(ctx, s, bin, B_rows, bits, bpart, btmp, leaf_off, "build_scatter");
    if (ctx->test_fail_build)
        throw Error(PHJ_ERR_CUDA, "test_fail_build: failure injected after the build shuffle");
    PHJ_CUDA(cudaEventRecord(ev[1], S));
    LeafTables lt;
    lt.next = s.get<uint64_t>(B_rows);
    build_leaf_tables(ctx, s, bpart, leaf_off, n_leaves, lt);
    const bool grouped = group_leaf_duplicates(ctx, bpart, btmp, leaf_off, n_leaves, lt);
    PHJ_CUDA(cudaEventRecord(ev[2], S));

    ProbeArgs a{};
    a.build = payload_cols(grouped ? btmp : bpart);
    a.grouped = grouped ? 1 : 0;
    a.meta = lt.meta;
    a.cells = lt.cells;
    a.next = lt.next;
    a.leaf_bits = total_bits;
    a.chj = 0;
    a.any_dup = lt.any_dup;
    a.uniform_log2cap = lt.uniform_log2cap;
    // (build payloads stay in columns: the host link bounds this path, and
    // packing them would only add to the time before the first download)
    const bool mat = materialize_probe(ctx, lt, *B, n_leaves) && P_rows > 0;
    const Cols ppart = mat ? alloc_cols_like(s, hp.schema, C) : Cols{};
    const uint32_t pb = probe_pass_bits(ctx, bits, *B);
    const Cols ptmp = mat && pb > 11 ? alloc_cols_like(s, hp.schema, C) : ppart;
    uint32_t * poff = s.get<uint32_t>((1ull << pb) + 1);
    uint32_t * heads = s.get<uint32_t>(C);
    uint32_t * counts = s.get<uint32_t>(probe_chunks(C) + 1);
    if (grouped || lt.any_dup)
        a.row_cnt = s.get<uint32_t>(C);

    // -------- PROBE, chunk by chunk --------
    std::vector<phj_output *> outs(n_chunks, nullptr);
    uint64_t total = 0, copied = 0;
    float t_shuffle = 0.f, t_probe = 0.f;
    cudaEvent_t c0 = take_event(ctx), c1 = take_event(ctx), c2 = take_event(ctx);
    try
    {
        for (uint64_t c = 0; c < n_chunks; ++c)
        {
            const uint64_t n = start(c + 1) - start(c);
            Scratch sc(ctx);
            PHJ_CUDA(cudaStreamWaitEvent(S, up[c], 0));
            PHJ_CUDA(cudaEventRecord(c0, S));
            a.probe = in[c & 1];
            if (mat)
            {
                radix_partition(ctx, sc, in[c & 1], n, {pb}, ppart, ptmp, poff, "probe_scatter");
                a.probe = ppart;
                PHJ_CUDA(cudaEventRecord(used[c], S)); // the input buffer is free again
            }
            PHJ_CUDA(cudaEventRecord(c1, S));
            a.probe_rows = n;
            const uint64_t rows = probe_lookup(ctx, sc, a, heads, counts);
            check_device_error(ctx);
            phj_output * o = new_output(ctx, hb.schema, hp.schema, rows);
            outs[c] = o;
            o->rows = rows;
            probe_project(ctx, a, o, 0, heads, counts, rows);
            if (!mat)
                PHJ_CUDA(cudaEventRecord(used[c], S));
            PHJ_CUDA(cudaEventRecord(proj[c], S));
            if (c + 2 < n_chunks)
                enqueue_chunk(c + 2);
            // download into the host columns at the running offset
            PHJ_CUDA(cudaStreamWaitEvent(ctx->d2h, proj[c], 0));
            const uint64_t keep = copied < out_cap ? std::min<uint64_t>(rows, out_cap - copied) : 0;
            if (keep)
            {
                PHJ_CUDA(cudaMemcpyAsync(out_keys + copied, o->keys, keep * 8, cudaMemcpyDeviceToHost, ctx->d2h));
                for (uint32_t k = 0; k < hb.schema.n_payloads; ++k)
                {
                    const uint32_t w = payload_width(hb.schema.types[k]);
                    PHJ_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(out_left[k]) + copied * w, o->lcol[k], keep * w, cudaMemcpyDeviceToHost, ctx->d2h));
                }
                for (uint32_t k = 0; k < hp.schema.n_payloads; ++k)
                {
                    const uint32_t w = payload_width(hp.schema.types[k]);
                    PHJ_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(out_right[k]) + copied * w, o->rcol[k], keep * w, cudaMemcpyDeviceToHost, ctx->d2h));
                }
            }
            copied += keep;
            PHJ_CUDA(cudaEventRecord(down[c], ctx->d2h));
            total += rows;
            // free the output two chunks back once its download is done
            if (c >= 2 && outs[c - 2])
            {
                PHJ_CUDA(cudaStreamWaitEvent(S, down[c - 2], 0));
                free_output(ctx, outs[c - 2]);
                outs[c - 2] = nullptr;
            }
            PHJ_CUDA(cudaEventRecord(c2, S));
            PHJ_CUDA(cudaEventSynchronize(c2));
            t_shuffle += event_ms(c0, c1);
            t_probe += event_ms(c1, c2);
        }
        if (n_chunks)
            PHJ_CUDA(cudaStreamWaitEvent(S, down[n_chunks - 1], 0));
        for (auto & o : outs)
            if (o)
            {
                free_output(ctx, o);
                o = nullptr;
            }
        PHJ_CUDA(cudaEventRecord(ev[3], S));
        PHJ_CUDA(cudaEventSynchronize(ev[3]));
    }
    catch (...)
    {
        cudaStreamSynchronize(ctx->h2d);
        cudaStreamSynchronize(ctx->d2h);
        for (auto & o : outs)
            free_output(ctx, o);
        throw;
    }
    if (out_rows)
        *out_rows = total;
    if (res)
    {
        fill_phase(res->build_shuffle, event_ms(ev[0], ev[1]), B_rows);
        fill_phase(res->build, event_ms(ev[1], ev[2]), B_rows);
        fill_phase(res->probe_shuffle, t_shuffle, P_rows);
        fill_phase(res->probe, t_probe, P_rows);
        res->e2e_wall_ms = event_ms(ev[0], ev[3]);
        res->peak_mem_bytes = ctx->peak_bytes;
    }
    if (std::getenv("PHJ_DEBUG"))
    {
        // when each stage of each chunk finished, ms from the start
        std::fprintf(stderr, "[phj] host join: build uploaded %.3f, built %.3f\n", event_ms(ev[0], build_up), event_ms(ev[0], ev[2]));
        for (uint64_t c = 0; c < n_chunks; ++c)
            std::fprintf(stderr, "[phj] chunk %llu (%llu rows): uploaded %.3f, input free %.3f, projected %.3f, downloaded %.3f\n",
                         (unsigned long long)c, (unsigned long long)(start(c + 1) - start(c)), event_ms(ev[0], up[c]), event_ms(ev[0], used[c]),
                         event_ms(ev[0], proj[c]), event_ms(ev[0], down[c]));
    }
    if (total > out_cap)
        throw Error(PHJ_ERR_CAPACITY, "host output holds " + std::to_string(out_cap) + " rows; the join has " + std::to_string(total) +
                                          " (the first rows up to the capacity were written)");
}


// PHJ (BEP) with the inputs and the output in host memory.  The build side
// is uploaded whole, shuffled to full leaf depth and its leaf tables laid
// out (built on first use, as in run_phj_bep).  The probe side streams
// through in batches of at most the budget's rows and at most
// `chunk_rows` (the first a quarter of that, so the first download starts
// sooner): batch c + 2 uploads on the h2d stream while batch c is
// scattered, its untouched leaves built, looked up and projected, and the
// output of batch c - 1 downloads on the d2h stream.  Two device input
// buffers and per-batch outputs, each reused or freed only after the copy
// that reads it has finished.
static void run_phj_bep_host(phj_ctx * ctx, const phj_block_stream & hb, const phj_block_stream & hp, const std::vector<uint32_t> & bits,
                             uint64_t budget_mib, uint64_t out_cap, uint64_t * out_keys, void * const * out_left, void * const * out_right,
                             uint64_t * out_rows, phj_bep_result * res, uint64_t chunk_rows)
{
    if (!ctx->h2d)
        PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking));
    if (!ctx->d2h)
        PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking));
    begin_run(ctx);
    Scratch s(ctx);
    cudaStream_t S = ctx->stream;
    uint32_t total_bits = 0;
    for (uint32_t b : bits)
        total_bits += b;
    const uint32_t n_leaves = 1u << total_bits;
    const uint64_t B_rows = hb.total_rows, P_rows = hp.total_rows;
    const uint64_t row_bytes = 8 + schema_bytes(hp.schema);
    const uint64_t budget_rows = std::max<uint64_t>(4096, ((budget_mib << 20) / row_bytes) & ~uint64_t(255));
    const uint64_t C = std::max<uint64_t>(1, std::min<uint64_t>({budget_rows, chunk_rows, std::max<uint64_t>(P_rows, 1)}));
    const uint64_t C0 = std::max<uint64_t>(1, std::min<uint64_t>(C, std::max<uint64_t>(C / 4, 4096)));
    auto start = [&](uint64_t c) -> uint64_t { return c == 0 ? 0 : std::min(P_rows, C0 + (c - 1) * C); };
    const uint64_t n_chunks = P_rows == 0 ? 0 : (P_rows <= C0 ? 1 : 1 + ceil_div(P_rows - C0, C));
    cudaEvent_t ev[4];
    for (auto & e : ev)
        e = take_event(ctx);

    // device buffers, all allocated on the compute stream before any copy
    phj_table * B = alloc_table(ctx, hb.schema, B_rows);
    std::unique_ptr<phj_table, std::function<void(phj_table *)>> B_guard(B, [ctx](phj_table * t) { free_table(ctx, t); });
    const CopyDrain drain{ctx}; // destroyed before B_guard and the scratch
    Cols in[2];
    for (auto & c : in)
        c = alloc_cols_like(s, hp.schema, C);
    const Cols bpart = alloc_cols_like(s, hb.schema, B_rows);
    const Cols btmp = alloc_cols_like(s, hb.schema, B_rows);
    uint32_t * leaf_off = s.get<uint32_t>((uint64_t)n_leaves + 1);
    const uint32_t p1 = 1u << bits[0];
    const Cols ppart = alloc_cols_like(s, hp.schema, C);
    const Cols ptmp = bits[0] > 11 ? alloc_cols_like(s, hp.schema, C) : ppart;
    uint32_t * poff = s.get<uint32_t>((uint64_t)p1 + 1);
    uint32_t * touched = s.get<uint32_t>((n_leaves + 31) / 32);
    unsigned long long * ctr = s.get<unsigned long long>(4);
    uint32_t * heads = s.get<uint32_t>(C);
    uint32_t * counts = s.get<uint32_t>(probe_chunks(C) + 1);
    uint32_t * rcnt = s.get<uint32_t>(C);
    PHJ_CUDA(cudaMemsetAsync(touched, 0, (size_t)((n_leaves + 31) / 32) * 4, S));
    PHJ_CUDA(cudaMemsetAsync(ctr, 0, 4 * sizeof(unsigned long long), S));
    PHJ_CUDA(cudaEventRecord(ev[0], S));
    PHJ_CUDA(cudaStreamWaitEvent(ctx->h2d, ev[0], 0));

    auto upload = [&](const Cols & dst, const phj_block_stream & src, uint64_t r0, uint64_t n) {
        PHJ_CUDA(cudaMemcpyAsync(dst.keys, src.keys + r0, n * 8, cudaMemcpyHostToDevice, ctx->h2d));
        for (uint32_t c = 0; c < src.schema.n_payloads; ++c)
        {
            const uint32_t w = payload_width(src.schema.types[c]);
            PHJ_CUDA(cudaMemcpyAsync(dst.col[c], static_cast<const uint8_t *>(src.payloads[c]) + r0 * w, n * w, cudaMemcpyHostToDevice, ctx->h2d));
        }
    };
    std::vector<cudaEvent_t> up(n_chunks), used(n_chunks), proj(n_chunks), down(n_chunks);
    for (uint64_t c = 0; c < n_chunks; ++c)
    {
        up[c] = take_event(ctx);
        used[c] = take_event(ctx);
        proj[c] = take_event(ctx);
        down[c] = take_event(ctx);
    }
    const Cols bin = cols_of(*B);
    if (B_rows)
        upload(bin, hb, 0, B_rows);
    cudaEvent_t build_up = take_event(ctx);
    PHJ_CUDA(cudaEventRecord(build_up, ctx->h2d));
    auto enqueue_chunk = [&](uint64_t c) {
        if (c >= 2)
            PHJ_CUDA(cudaStreamWaitEvent(ctx->h2d, used[c - 2], 0));
        upload(in[c & 1], hp, start(c), start(c + 1) - start(c));
        PHJ_CUDA(cudaEventRecord(up[c], ctx->h2d));
    };
    for (uint64_t c = 0; c < std::min<uint64_t>(2, n_chunks); ++c)
        enqueue_chunk(c);

    // -------- BUILD SHUFFLE, full leaf depth; tables laid out, built on
    // first use (src/PHJBep.cpp:128-141) --------
    PHJ_CUDA(cudaStreamWaitEvent(S, build_up, 0));
    radix_partition(ctx, s, bin, B_rows, bits, bpart, btmp, leaf_off, "build_scatter");
    if (ctx->test_fail_build)
        throw Error(PHJ_ERR_CUDA, "test_fail_build: failure injected after the build shuffle");
    PHJ_CUDA(cudaEventRecord(ev[1], S));
    LeafTables lt;
    lt.next = s.get<uint64_t>(B_rows);
    build_leaf_tables(ctx, s, bpart, leaf_off, n_leaves, lt, true);
    if (ctx->test_stuck_leaf >= 0 && (uint64_t)ctx->test_stuck_leaf < n_leaves)
    {
        const uint32_t building = 1;
        PHJ_CUDA(cudaMemcpyAsync(lt.state + ctx->test_stuck_leaf, &building, sizeof(building), cudaMemcpyHostToDevice, S));
        PHJ_CUDA(cudaStreamSynchronize(S));
    }
    PHJ_CUDA(cudaEventRecord(ev[2], S));

    ProbeArgs a{};
    a.build = payload_cols(bpart);
    a.meta = lt.meta;
    a.cells = lt.cells;
    a.next = lt.next;
    a.leaf_bits = total_bits;
    a.chj = 0;
    a.any_dup = 0;
    a.uniform_log2cap = lt.uniform_log2cap;
    a.row_cnt = rcnt;
    BepLeaves bl{};
    bl.state = lt.state;
    bl.touched = touched;
    bl.leaf_off = leaf_off;
    bl.build_keys = bpart.keys;
    bl.meta = lt.meta;
    bl.cells = lt.cells;
    bl.next = lt.next;
    bl.leaf_bits = total_bits;
    bl.n_leaves = n_leaves;
    bl.smem_cells = (uint32_t)std::min<uint64_t>(lt.uniform_log2cap >= 0 ? (1ull << lt.uniform_log2cap) : bit_ceil64(2ull * std::max<uint32_t>(lt.max_rows, 1)),
                                                 8192);
    bl.wait_limit_ns = (uint64_t)ctx->wait_limit_ms * 1000000ull;
    bl.ctr = ctr;
    bl.queue = s.get<uint32_t>(n_leaves);
    bl.queue_len = s.get<uint32_t>(2);
    bl.any_dup = s.get<int>(1);
    PHJ_CUDA(cudaMemsetAsync(bl.any_dup, 0, sizeof(int), S));

    // -------- PROBE, batch by batch --------
    std::vector<phj_output *> outs(n_chunks, nullptr);
    uint64_t total = 0, copied = 0, peak_rows = 0;
    float t_shuffle = 0.f, t_lazy = 0.f, t_probe = 0.f;
    cudaEvent_t c0 = take_event(ctx), c1 = take_event(ctx), c2 = take_event(ctx), c3 = take_event(ctx);
    try
    {
        for (uint64_t c = 0; c < n_chunks; ++c)
        {
            const uint64_t n = start(c + 1) - start(c);
            peak_rows = std::max(peak_rows, n);
            Scratch sc(ctx);
            PHJ_CUDA(cudaStreamWaitEvent(S, up[c], 0));
            PHJ_CUDA(cudaEventRecord(c0, S));
            // the batch's first radix pass also flags the leaves its rows
            // touch (its histogram reads every key once anyway)
            ctx->leaf_mark = LeafMark{touched, 64u - total_bits, (n_leaves + 31) / 32};
            try
            {
                radix_partition(ctx, sc, in[c & 1], n, {bits[0]}, ppart, ptmp, poff, "probe_scatter");
            }
            catch (...)
            {
                ctx->leaf_mark = LeafMark{};
                throw;
            }
            ctx->leaf_mark = LeafMark{};
            PHJ_CUDA(cudaEventRecord(used[c], S)); // the input buffer is free again
            k_count_nonempty<<<(unsigned)ceil_div(p1, 256), 256, 0, S>>>(poff, p1, ctr + 3);
            PHJ_LAUNCHED(ctx, "count_refinements");
            PHJ_CUDA(cudaEventRecord(c1, S));
            a.probe = ppart;
            a.probe_rows = n;
            // lazy build of the leaves this batch touches
            a.any_dup = bep_build_touched(ctx, bl) ? 1 : 0;
            check_device_error(ctx);
            PHJ_CUDA(cudaEventRecord(c2, S));
            const uint64_t rows = probe_lookup(ctx, sc, a, heads, counts);
            phj_output * o = new_output(ctx, hb.schema, hp.schema, rows);
            outs[c] = o;
            o->rows = rows;
            probe_project(ctx, a, o, 0, heads, counts, rows);
            PHJ_CUDA(cudaEventRecord(proj[c], S));
            if (c + 2 < n_chunks)
                enqueue_chunk(c + 2);
            // download into the host columns at the running offset
            PHJ_CUDA(cudaStreamWaitEvent(ctx->d2h, proj[c], 0));
            const uint64_t keep = copied < out_cap ? std::min<uint64_t>(rows, out_cap - copied) : 0;
            if (keep)
            {
                PHJ_CUDA(cudaMemcpyAsync(out_keys + copied, o->keys, keep * 8, cudaMemcpyDeviceToHost, ctx->d2h));
                for (uint32_t k = 0; k < hb.schema.n_payloads; ++k)
                {
                    const uint32_t w = payload_width(hb.schema.types[k]);
                    PHJ_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(out_left[k]) + copied * w, o->lcol[k], keep * w, cudaMemcpyDeviceToHost, ctx->d2h));
                }
                for (uint32_t k = 0; k < hp.schema.n_payloads; ++k)
                {
                    const uint32_t w = payload_width(hp.schema.types[k]);
                    PHJ_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(out_right[k]) + copied * w, o->rcol[k], keep * w, cudaMemcpyDeviceToHost, ctx->d2h));
                }
            }
            copied += keep;
            PHJ_CUDA(cudaEventRecord(down[c], ctx->d2h));
            total += rows;
            // free the output two batches back once its download is done
            if (c >= 2 && outs[c - 2])
            {
                PHJ_CUDA(cudaStreamWaitEvent(S, down[c - 2], 0));
                free_output(ctx, outs[c - 2]);
                outs[c - 2] = nullptr;
            }
            PHJ_CUDA(cudaEventRecord(c3, S));
            PHJ_CUDA(cudaEventSynchronize(c3));
            t_shuffle += event_ms(c0, c1);
            t_lazy += event_ms(c1, c2);
            t_probe += event_ms(c2, c3);
        }
        if (n_chunks)
            PHJ_CUDA(cudaStreamWaitEvent(S, down[n_chunks - 1], 0));
        for (auto & o : outs)
            if (o)
            {
                free_output(ctx, o);
                o = nullptr;
            }
        PHJ_CUDA(cudaEventRecord(ev[3], S));
        PHJ_CUDA(cudaEventSynchronize(ev[3]));
        check_device_error(ctx);
    }
    catch (...)
    {
        cudaStreamSynchronize(ctx->h2d);
        cudaStreamSynchronize(ctx->d2h);
        for (auto & o : outs)
            free_output(ctx, o);
        throw;
    }
    if (out_rows)
        *out_rows = total;
    if (res)
    {
        unsigned long long cv[4] = {};
        read_small(ctx, {{cv, ctr, sizeof(cv)}});
        const float bs = event_ms(ev[0], ev[1]), bd = event_ms(ev[1], ev[2]) + t_lazy, e2e = event_ms(ev[0], ev[3]);
        fill_phase(res->build_shuffle, bs, B_rows);
        fill_phase(res->build, bd, B_rows);
        fill_phase(res->probe_shuffle, t_shuffle, P_rows);
        fill_phase(res->probe, t_probe, P_rows);
        fill_phase(res->eviction_overhead, std::max(0.f, e2e - bs - bd - t_shuffle - t_probe), P_rows);
        res->e2e_wall_ms = e2e;
        res->peak_mem_bytes = ctx->peak_bytes;
        res->bep_budget_mib = budget_mib;
        res->bep_evictions = cv[2];
        res->bep_refinements = cv[3];
        res->bep_peak_bytes = peak_rows * row_bytes;
        res->bep_build_skip_retries = cv[1];
    }
    if (total > out_cap)
        throw Error(PHJ_ERR_CAPACITY, "host output holds " + std::to_string(out_cap) + " rows; the join has " + std::to_string(total) +
                                          " (the first rows up to the capacity were written)");
}

} // namespace phjg

using namespace phjg;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

uint32_t phj_abi_version(void)
{
    return PHJ_GPU_ABI_VERSION;
}

phj_status phj_ctx_create(int device, phj_ctx ** out)
{
    if (!out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    {
        cudaGetLastError();
        return PHJ_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n)
        return PHJ_ERR_INVALID_ARGUMENT;
    phj_ctx * ctx = new (std::nothrow) phj_ctx();
    if (!ctx)
        return PHJ_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    const phj_status st = guard(ctx, [&] {
        PHJ_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop;
        PHJ_CUDA(cudaGetDeviceProperties(&prop, device));
        if (prop.major < 10)
            throw Error(PHJ_ERR_UNSUPPORTED, "this library is built for sm_103a (Blackwell) only");
        ctx->num_sms = prop.multiProcessorCount;
        ctx->smem_optin = prop.sharedMemPerBlockOptin;
        ctx->l2_bytes = prop.l2CacheSize;
        PHJ_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        cudaMemPoolProps pp{};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = device;
        PHJ_CUDA(cudaMemPoolCreate(&ctx->pool, &pp));
        uint64_t keep = ~0ull; // keep freed memory in the pool across runs
        PHJ_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        PHJ_CUDA(cudaMalloc(&ctx->d_err, sizeof(int)));
        PHJ_CUDA(cudaMemset(ctx->d_err, 0, sizeof(int)));
        set_partition_smem_limits((int)ctx->smem_optin);
        set_build_smem_limits((int)ctx->smem_optin);
        set_bep_smem_limits((int)ctx->smem_optin);
    });
    if (st != PHJ_OK)
    {
        std::fprintf(stderr, "phj_ctx_create: %s\n", ctx->last_error.c_str());
        phj_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return PHJ_OK;
}

void phj_ctx_destroy(phj_ctx * ctx)
{
    if (!ctx)
        return;
    {
        DeviceScope dev(ctx);
        if (ctx->stream)
            cudaStreamSynchronize(ctx->stream);
        free_batch_graph(ctx);
        if (ctx->l2_flush)
            cudaFree(ctx->l2_flush);
        if (ctx->d_err)
            cudaFree(ctx->d_err);
        if (ctx->host_small)
            cudaFreeHost(ctx->host_small);
        for (cudaEvent_t e : ctx->event_pool)
            cudaEventDestroy(e);
        for (auto & lv : ctx->live)
            cudaFreeAsync(lv.first, ctx->stream);
        if (ctx->stream)
            cudaStreamSynchronize(ctx->stream);
        if (ctx->pool)
            cudaMemPoolDestroy(ctx->pool);
        if (ctx->stream)
            cudaStreamDestroy(ctx->stream);
        if (ctx->h2d)
            cudaStreamDestroy(ctx->h2d);
        if (ctx->d2h)
            cudaStreamDestroy(ctx->d2h);
        if (ctx->side)
            cudaStreamDestroy(ctx->side);
        if (ctx->aux)
            cudaStreamDestroy(ctx->aux);
    }
    delete ctx;
}

const char * phj_last_error(const phj_ctx * ctx)
{
    return ctx ? ctx->last_error.c_str() : "null context";
}

void * phj_ctx_stream(phj_ctx * ctx)
{
    return ctx ? (void *)ctx->stream : nullptr;
}

phj_status phj_ctx_set_int(phj_ctx * ctx, const char * name, int64_t value)
{
    if (!ctx || !name)
        return PHJ_ERR_INVALID_ARGUMENT;
    if (std::strcmp(name, "probe_materialize") == 0 && value >= -1 && value <= 1)
        ctx->probe_materialize = (int)value;
    else if (std::strcmp(name, "time_kernels") == 0)
        ctx->time_kernels = value != 0;
    else if (std::strcmp(name, "wait_limit_ms") == 0 && value >= 1 && value <= 60000)
        ctx->wait_limit_ms = value;
    else if (std::strcmp(name, "host_chunk_rows") == 0 && value >= 4096)
        ctx->host_chunk_rows = value;
    else if (std::strcmp(name, "table_cap_pct") == 0 && value >= 110 && value <= 800)
        ctx->table_cap_pct = (uint32_t)value;
    else if (std::strcmp(name, "p1_tile_rows") == 0 && (value == 0 || value == 1024 || value == 2048 || value == 4096))
        ctx->p1_tile_rows = (uint32_t)value;
    else if (std::strcmp(name, "p1_stages") == 0 && (value == 0 || (value >= 2 && value <= 4)))
        ctx->p1_stages = (uint32_t)value;
    else if (std::strcmp(name, "pack_build") == 0 && (value == 0 || value == 1))
        ctx->pack_build = (int)value;
    else if (std::strcmp(name, "chj_windows") == 0 && value >= 0 && value <= 256 && (value & (value - 1)) == 0)
        ctx->chj_windows = (uint32_t)value;
    else if (std::strcmp(name, "bep_engine") == 0 && (value == 0 || value == 1))
        ctx->bep_engine = (int)value;
    else if (std::strcmp(name, "batch_graph") == 0 && (value == 0 || value == 1))
        ctx->batch_graph = (int)value;
    else if (std::strcmp(name, "probe_fused") == 0 && (value == 0 || value == 1))
        ctx->probe_fused = (int)value;
    else if (std::strcmp(name, "probe_pass_bits") == 0 && value >= 0 && value <= 11)
        ctx->probe_pass_bits = (uint32_t)value;
    else if (std::strcmp(name, "test_stuck_leaf") == 0 && value >= -1)
        ctx->test_stuck_leaf = value;
    else if (std::strcmp(name, "test_engine_stall_wave") == 0 && value >= -1 && value < (1ll << 31))
        ctx->test_engine_stall_wave = value;
    else if (std::strcmp(name, "test_fail_build") == 0 && (value == 0 || value == 1))
        ctx->test_fail_build = (int)value;
    else
        return PHJ_ERR_INVALID_ARGUMENT;
    return PHJ_OK;
}

phj_status phj_ctx_get_int(const phj_ctx * ctx, const char * name, int64_t * value)
{
    if (!ctx || !name || !value)
        return PHJ_ERR_INVALID_ARGUMENT;
    if (std::strcmp(name, "probe_materialize") == 0)
        *value = ctx->probe_materialize;
    else if (std::strcmp(name, "time_kernels") == 0)
        *value = ctx->time_kernels ? 1 : 0;
    else if (std::strcmp(name, "wait_limit_ms") == 0)
        *value = ctx->wait_limit_ms;
    else if (std::strcmp(name, "host_chunk_rows") == 0)
        *value = ctx->host_chunk_rows;
    else if (std::strcmp(name, "table_cap_pct") == 0)
        *value = ctx->table_cap_pct;
    else if (std::strcmp(name, "p1_tile_rows") == 0)
        *value = ctx->p1_tile_rows;
    else if (std::strcmp(name, "p1_stages") == 0)
        *value = ctx->p1_stages;
    else if (std::strcmp(name, "pack_build") == 0)
        *value = ctx->pack_build;
    else if (std::strcmp(name, "chj_windows") == 0)
        *value = ctx->chj_windows;
    else if (std::strcmp(name, "bep_engine") == 0)
        *value = ctx->bep_engine;
    else if (std::strcmp(name, "batch_graph") == 0)
        *value = ctx->batch_graph;
    else if (std::strcmp(name, "probe_fused") == 0)
        *value = ctx->probe_fused;
    else if (std::strcmp(name, "probe_pass_bits") == 0)
        *value = ctx->probe_pass_bits;
    else if (std::strcmp(name, "test_stuck_leaf") == 0)
        *value = ctx->test_stuck_leaf;
    else if (std::strcmp(name, "test_engine_stall_wave") == 0)
        *value = ctx->test_engine_stall_wave;
    else if (std::strcmp(name, "test_fail_build") == 0)
        *value = ctx->test_fail_build;
    else if (std::strcmp(name, "device") == 0)
        *value = ctx->device;
    else if (std::strcmp(name, "num_sms") == 0)
        *value = ctx->num_sms;
    else if (std::strcmp(name, "l2_bytes") == 0)
        *value = (int64_t)ctx->l2_bytes;
    else
        return PHJ_ERR_INVALID_ARGUMENT;
    return PHJ_OK;
}

phj_status phj_autotune_radix(uint64_t build_rows, uint64_t probe_rows, uint8_t * out_bits, uint32_t * out_n_passes)
{
    if (!out_bits || !out_n_passes)
        return PHJ_ERR_INVALID_ARGUMENT;
    (void)probe_rows;
    // leaves of ~256 build rows: a leaf table of 512 cells (8 KiB) stays in
    // L2 next to the probe rows that hit it; first passes of <= 11 bits keep
    // the scatter's per-CTA digit counters in shared memory
    uint32_t bits = 1;
    while (bits < 24 && (build_rows >> (bits + 9)) > 0)
        ++bits;
    const uint32_t passes = bits <= 11 ? 1 : bits <= 22 ? 2 : 3;
    for (uint32_t i = 0; i < passes; ++i)
        out_bits[i] = (uint8_t)(bits / passes + (i < bits % passes ? 1 : 0));
    *out_n_passes = passes;
    return PHJ_OK;
}

phj_status phj_resolve_radix(uint64_t partitions, uint32_t passes, const uint8_t * bits_override, uint32_t n_bits_override, uint8_t * out_bits,
                             uint32_t * out_n_passes)
{
    if (!out_bits || !out_n_passes)
        return PHJ_ERR_INVALID_ARGUMENT;
    uint32_t total = 0;
    if (n_bits_override > 0)
    {
        if (!bits_override || n_bits_override > 32)
            return PHJ_ERR_INVALID_ARGUMENT;
        for (uint32_t i = 0; i < n_bits_override; ++i)
        {
            if (bits_override[i] == 0 || bits_override[i] > 16) // CLI.cpp parseBitsList
                return PHJ_ERR_INVALID_ARGUMENT;
            out_bits[i] = bits_override[i];
            total += bits_override[i];
        }
        *out_n_passes = n_bits_override;
    }
    else
    {
        const uint64_t parts = partitions == 0 ? 256 : partitions;
        if ((parts & (parts - 1)) != 0)
            return PHJ_ERR_INVALID_ARGUMENT; // --partitions must be a positive power of 2
        uint32_t tb = 0;
        while ((1ull << tb) < parts)
            ++tb;
        const uint32_t np = passes == 0 ? 1 : passes;
        if (np > tb)
            return PHJ_ERR_INVALID_ARGUMENT; // passes cannot exceed log2(partitions)
        for (uint32_t p = 0; p < np; ++p)
            out_bits[p] = (uint8_t)(tb / np + (p < tb % np ? 1u : 0u));
        *out_n_passes = np;
        total = tb;
    }
    if (total == 0 || total > 32)
        return PHJ_ERR_INVALID_ARGUMENT;
    return PHJ_OK;
}

static phj_status make_table(phj_ctx * ctx, const phj_block_stream * src, phj_table ** out, bool upload)
{
    if (!ctx || !src || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        check_schema(src->schema, "stream");
        if (src->total_rows && !src->keys)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "null key column");
        for (uint32_t c = 0; c < src->schema.n_payloads; ++c)
            if (src->total_rows && !src->payloads[c])
                throw Error(PHJ_ERR_INVALID_ARGUMENT, "null payload column");
        phj_table * t = nullptr;
        if (upload)
        {
            t = alloc_table(ctx, src->schema, src->total_rows);
            const cudaMemcpyKind kind = src->location == PHJ_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
            try
            {
                if (src->total_rows)
                {
                    PHJ_CUDA(cudaMemcpyAsync(t->keys, src->keys, src->total_rows * 8, kind, ctx->stream));
                    for (uint32_t c = 0; c < src->schema.n_payloads; ++c)
                        PHJ_CUDA(cudaMemcpyAsync(t->cols[c], src->payloads[c], src->total_rows * payload_width(src->schema.types[c]), kind,
                                                 ctx->stream));
                }
                set_block_structure(ctx, t, src->n_blocks, src->block_rows);
            }
            catch (...)
            {
                free_table(ctx, t);
                throw;
            }
        }
        else
        {
            if (src->location != PHJ_DEVICE)
                throw Error(PHJ_ERR_INVALID_ARGUMENT, "phj_table_wrap_device needs device columns");
            t = new phj_table();
            t->schema = src->schema;
            t->rows = src->total_rows;
            t->keys = const_cast<uint64_t *>(src->keys);
            for (uint32_t c = 0; c < src->schema.n_payloads; ++c)
                t->cols[c] = const_cast<void *>(src->payloads[c]);
            t->owned = false;
            try
            {
                set_block_structure(ctx, t, src->n_blocks, src->block_rows);
            }
            catch (...)
            {
                free_table(ctx, t);
                throw;
            }
        }
        *out = t;
    });
}

phj_status phj_table_upload(phj_ctx * ctx, const phj_block_stream * host_stream, phj_table ** out)
{
    return make_table(ctx, host_stream, out, true);
}

phj_status phj_table_wrap_device(phj_ctx * ctx, const phj_block_stream * device_stream, phj_table ** out)
{
    return make_table(ctx, device_stream, out, false);
}

phj_status phj_table_generate(phj_ctx * ctx, const phj_gen_spec * spec, phj_table ** out)
{
    if (!ctx || !spec || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        check_schema(spec->schema, "generated stream");
        if (spec->kind > 5)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "unknown generator kind");
        if (spec->rows >= (1ull << 32))
            throw Error(PHJ_ERR_UNSUPPORTED, "generated streams hold < 2^32 rows");
        if ((spec->kind == 3 || spec->kind == 4 || spec->kind == 5) && (spec->domain == 0 || spec->domain > (1ull << 32)))
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "generator domain must be in [1, 2^32]");
        phj_table * t = alloc_table(ctx, spec->schema, spec->rows);
        try
        {
            if (spec->rows)
                t->gen_distinct = generate_rows(ctx, *spec, *t);
            std::vector<uint32_t> br;
            const uint32_t bs = spec->block_rows ? spec->block_rows : 10000;
            for (uint64_t r = 0; r < spec->rows; r += bs)
                br.push_back((uint32_t)std::min<uint64_t>(bs, spec->rows - r));
            set_block_structure(ctx, t, (uint32_t)br.size(), br.empty() ? nullptr : br.data());
        }
        catch (...)
        {
            free_table(ctx, t);
            throw;
        }
        *out = t;
    });
}

phj_status phj_table_download(phj_ctx * ctx, const phj_table * t, uint64_t * keys, void * const * payloads)
{
    if (!ctx || !t)
        return PHJ_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] {
        if (t->rows == 0)
            return;
        if (keys)
            PHJ_CUDA(cudaMemcpyAsync(keys, t->keys, t->rows * 8, cudaMemcpyDeviceToHost, ctx->stream));
        if (payloads)
            for (uint32_t c = 0; c < t->schema.n_payloads; ++c)
                if (payloads[c])
                    PHJ_CUDA(cudaMemcpyAsync(payloads[c], t->cols[c], t->rows * payload_width(t->schema.types[c]), cudaMemcpyDeviceToHost,
                                             ctx->stream));
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

uint64_t phj_table_rows(const phj_table * t)
{
    return t ? t->rows : 0;
}

uint64_t phj_table_gen_distinct(const phj_table * t)
{
    return t ? t->gen_distinct : 0;
}

void phj_table_free(phj_ctx * ctx, phj_table * t)
{
    DeviceScope dev(ctx);
    if (ctx)
        free_table(ctx, t);
}

phj_status phj_run_chj(phj_ctx * ctx, const phj_table * build, const phj_table * probe, phj_output ** out, phj_chj_result * result)
{
    if (!ctx || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        check_sides(build, probe);
        run_chj(ctx, *build, *probe, out, result);
    });
}

phj_status phj_run_phj_pure(phj_ctx * ctx, const phj_table * build, const phj_table * probe, const uint8_t * pass_bits, uint32_t n_passes,
                            phj_output ** out, phj_phj_result * result)
{
    if (!ctx || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        const std::vector<uint32_t> bits = check_bits(pass_bits, n_passes);
        check_sides(build, probe);
        run_phj_pure(ctx, *build, *probe, bits, out, result);
    });
}

phj_status phj_radix_shuffle(phj_ctx * ctx, const phj_table * input, const uint8_t * pass_bits, uint32_t n_passes, phj_table ** out,
                             uint64_t * partition_rows)
{
    if (!ctx || !input || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    return guard(ctx, [&] {
        const std::vector<uint32_t> bits = check_bits(pass_bits, n_passes);
        if (input->rows >= (1ull << 32))
            throw Error(PHJ_ERR_UNSUPPORTED, "the device radix shuffle takes < 2^32 rows");
        uint32_t total_bits = 0;
        for (uint32_t b : bits)
            total_bits += b;
        const uint64_t n_parts = 1ull << total_bits;
        begin_run(ctx);
        Scratch s(ctx);
        phj_table * t = alloc_table(ctx, input->schema, input->rows);
        try
        {
            const Cols tmp = alloc_cols_like(s, input->schema, input->rows);
            uint32_t * leaf_off = s.get<uint32_t>(n_parts + 1);
            radix_partition(ctx, s, cols_of(*input), input->rows, bits, cols_of(*t), tmp, leaf_off, "radix_shuffle");
            // one block per partition (PartitionedShuffleOutput::chains[p])
            std::vector<uint32_t> off(n_parts + 1);
            PHJ_CUDA(cudaMemcpyAsync(off.data(), leaf_off, (n_parts + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
            PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
            std::vector<uint32_t> rows(n_parts);
            for (uint64_t p = 0; p < n_parts; ++p)
            {
                rows[p] = off[p + 1] - off[p];
                if (partition_rows)
                    partition_rows[p] = rows[p];
            }
            set_block_structure(ctx, t, (uint32_t)n_parts, rows.data()); // at most 2^24 partitions
        }
        catch (...)
        {
            free_table(ctx, t);
            throw;
        }
        *out = t;
    });
}

phj_status phj_run_phj_bep(phj_ctx * ctx, const phj_table * build, const phj_table * probe, const uint8_t * pass_bits, uint32_t n_passes,
                           uint64_t bep_budget_mib, uint32_t workers, phj_output ** out, phj_bep_result * result)
{
    if (!ctx || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    (void)workers; // the reference's threads; one device-wide batch replaces the per-worker split
    return guard(ctx, [&] {
        const std::vector<uint32_t> bits = check_bits(pass_bits, n_passes);
        check_sides(build, probe);
        if (bep_budget_mib == 0 || bep_budget_mib > (1ull << 30))
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "bep_budget_mib must be in [1, 2^30]");
        uint32_t total = 0;
        for (uint32_t b : bits)
            total += b;
        if (total > 20)
            throw Error(PHJ_ERR_UNSUPPORTED, "PHJ (BEP) on the device takes at most 20 radix bits (2^20 leaves)");
        // the engine counts a leaf's and a block's rows in 32 bits
        if (ctx->bep_engine == 0 && bep_engine_supported(bits[0], total) && probe->rows < (1ull << 32))
            run_phj_bep_engine(ctx, *build, *probe, bits, bep_budget_mib, out, result);
        else
            run_phj_bep(ctx, *build, *probe, bits, bep_budget_mib, out, result);
    });
}

phj_status phj_run_phj_pure_host(phj_ctx * ctx, const phj_block_stream * build, const phj_block_stream * probe, const uint8_t * pass_bits,
                                 uint32_t n_passes, uint64_t out_capacity, uint64_t * out_keys, void * const * out_left, void * const * out_right,
                                 uint64_t * out_rows, phj_phj_result * result)
{
    if (!ctx || !build || !probe)
        return PHJ_ERR_INVALID_ARGUMENT;
    if (out_rows)
        *out_rows = 0;
    return guard(ctx, [&] {
        const std::vector<uint32_t> bits = check_bits(pass_bits, n_passes);
        check_schema(build->schema, "build stream");
        check_schema(probe->schema, "probe stream");
        if (build->location != PHJ_HOST || probe->location != PHJ_HOST)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "phj_run_phj_pure_host takes host streams");
        if (build->total_rows >= (1ull << 31) || probe->total_rows >= (1ull << 32))
            throw Error(PHJ_ERR_UNSUPPORTED, "device schemes support < 2^31 build rows and < 2^32 probe rows");
        if ((build->total_rows && !build->keys) || (probe->total_rows && !probe->keys))
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "null key column");
        if (out_capacity && !out_keys)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "null output key column");
        for (uint32_t c = 0; c < build->schema.n_payloads; ++c)
            if ((build->total_rows && !build->payloads[c]) || (out_capacity && (!out_left || !out_left[c])))
                throw Error(PHJ_ERR_INVALID_ARGUMENT, "null build payload column");
        for (uint32_t c = 0; c < probe->schema.n_payloads; ++c)
            if ((probe->total_rows && !probe->payloads[c]) || (out_capacity && (!out_right || !out_right[c])))
                throw Error(PHJ_ERR_INVALID_ARGUMENT, "null probe payload column");
        run_phj_pure_host(ctx, *build, *probe, bits, out_capacity, out_keys, out_left, out_right, out_rows, result, (uint64_t)ctx->host_chunk_rows);
    });
}

phj_status phj_run_phj_bep_host(phj_ctx * ctx, const phj_block_stream * build, const phj_block_stream * probe, const uint8_t * pass_bits,
                                uint32_t n_passes, uint64_t bep_budget_mib, uint64_t out_capacity, uint64_t * out_keys, void * const * out_left,
                                void * const * out_right, uint64_t * out_rows, phj_bep_result * result)
{
    if (!ctx || !build || !probe)
        return PHJ_ERR_INVALID_ARGUMENT;
    if (out_rows)
        *out_rows = 0;
    return guard(ctx, [&] {
        const std::vector<uint32_t> bits = check_bits(pass_bits, n_passes);
        check_schema(build->schema, "build stream");
        check_schema(probe->schema, "probe stream");
        if (build->location != PHJ_HOST || probe->location != PHJ_HOST)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "phj_run_phj_bep_host takes host streams");
        if (build->total_rows >= (1ull << 31) || probe->total_rows >= (1ull << 32))
            throw Error(PHJ_ERR_UNSUPPORTED, "device schemes support < 2^31 build rows and < 2^32 probe rows");
        uint32_t total_bits = 0;
        for (uint32_t b : bits)
            total_bits += b;
        if (total_bits > 20)
            throw Error(PHJ_ERR_UNSUPPORTED, "PHJ (BEP) on the device takes at most 20 radix bits (2^20 leaves)");
        if ((build->total_rows && !build->keys) || (probe->total_rows && !probe->keys))
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "null key column");
        if (out_capacity && !out_keys)
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "null output key column");
        for (uint32_t c = 0; c < build->schema.n_payloads; ++c)
            if ((build->total_rows && !build->payloads[c]) || (out_capacity && (!out_left || !out_left[c])))
                throw Error(PHJ_ERR_INVALID_ARGUMENT, "null build payload column");
        for (uint32_t c = 0; c < probe->schema.n_payloads; ++c)
            if ((probe->total_rows && !probe->payloads[c]) || (out_capacity && (!out_right || !out_right[c])))
                throw Error(PHJ_ERR_INVALID_ARGUMENT, "null probe payload column");
        run_phj_bep_host(ctx, *build, *probe, bits, bep_budget_mib, out_capacity, out_keys, out_left, out_right, out_rows, result,
                         (uint64_t)ctx->host_chunk_rows);
    });
}

uint64_t phj_output_rows(const phj_output * out)
{
    return out ? out->rows : 0;
}

phj_status phj_output_device_columns(const phj_output * out, const uint64_t ** keys, const void ** left, const void ** right)
{
    if (!out)
        return PHJ_ERR_INVALID_ARGUMENT;
    if (keys)
        *keys = out->keys;
    if (left)
        for (uint32_t c = 0; c < out->left.n_payloads; ++c)
            left[c] = out->lcol[c];
    if (right)
        for (uint32_t c = 0; c < out->right.n_payloads; ++c)
            right[c] = out->rcol[c];
    return PHJ_OK;
}

phj_status phj_output_download(phj_ctx * ctx, const phj_output * out, uint64_t * keys, void * const * left, void * const * right)
{
    if (!ctx || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] {
        const uint64_t n = out->rows;
        if (n == 0)
            return;
        if (keys)
            PHJ_CUDA(cudaMemcpyAsync(keys, out->keys, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
        if (left)
            for (uint32_t c = 0; c < out->left.n_payloads; ++c)
                if (left[c])
                    PHJ_CUDA(cudaMemcpyAsync(left[c], out->lcol[c], n * payload_width(out->left.types[c]), cudaMemcpyDeviceToHost, ctx->stream));
        if (right)
            for (uint32_t c = 0; c < out->right.n_payloads; ++c)
                if (right[c])
                    PHJ_CUDA(
                        cudaMemcpyAsync(right[c], out->rcol[c], n * payload_width(out->right.types[c]), cudaMemcpyDeviceToHost, ctx->stream));
        PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

phj_status phj_output_fingerprint(phj_ctx * ctx, const phj_output * out, uint64_t fp[3])
{
    if (!ctx || !out || !fp)
        return PHJ_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] { fingerprint(ctx, *out, fp); });
}

void phj_output_free(phj_ctx * ctx, phj_output * out)
{
    DeviceScope dev(ctx);
    if (ctx)
        free_output(ctx, out);
}

uint32_t phj_last_kernel_times(const phj_ctx * ctx, phj_kernel_time * out, uint32_t cap)
{
    if (!ctx || !out)
        return 0;
    DeviceScope dev(ctx);
    uint32_t n = 0;
    // start offsets from the first record, then shifted so the earliest
    // launch (possibly on another stream) is at 0
    double first = 0.0;
    for (const auto & r : ctx->records)
    {
        if (n >= cap)
            break;
        phj_kernel_time & k = out[n++];
        std::memset(&k, 0, sizeof(k));
        std::strncpy(k.name, r.name.c_str(), sizeof(k.name) - 1);
        float ms = 0.f, at = 0.f;
        if (cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess)
        {
            cudaGetLastError();
            ms = -1.f;
        }
        if (cudaEventElapsedTime(&at, ctx->records.front().start, r.start) != cudaSuccess)
        {
            cudaGetLastError();
            at = 0.f;
        }
        k.ms = ms;
        k.rows = r.rows;
        k.bytes = r.bytes;
        k.start_ms = at;
        first = std::min(first, (double)at);
    }
    for (uint32_t i = 0; i < n; ++i)
        out[i].start_ms -= first;
    return n;
}

uint64_t phj_launch_count(const phj_ctx * ctx)
{
    return ctx ? ctx->launches : 0;
}

phj_status phj_host_alloc(phj_ctx * ctx, size_t bytes, void ** out)
{
    if (!ctx || !out)
        return PHJ_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] { PHJ_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault)); });
}

void phj_host_free(phj_ctx * ctx, void * p)
{
    (void)ctx;
    if (p)
        cudaFreeHost(p);
}

phj_status phj_flush_l2(phj_ctx * ctx)
{
    if (!ctx)
        return PHJ_ERR_INVALID_ARGUMENT;
    return guard(ctx, [&] {
        if (!ctx->l2_flush)
        {
            ctx->l2_flush_bytes = std::max<size_t>(ctx->l2_bytes * 2, 256u << 20);
            PHJ_CUDA(cudaMalloc(&ctx->l2_flush, ctx->l2_flush_bytes));
        }
        PHJ_CUDA(cudaMemsetAsync(ctx->l2_flush, ctx->launches & 0xff, ctx->l2_flush_bytes, ctx->stream));
    });
}

} // extern "C"
