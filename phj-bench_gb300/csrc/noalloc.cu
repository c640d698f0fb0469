// noalloc.cu -- a CHJ-style join that allocates no device memory.
//
// Some callers cannot allocate while they join: an operator running inside
// an engine whose memory manager owns all of HBM through its own arena (a
// cudaMalloc behind its back would break its accounting or fail outright), or
// a serving loop that reserved the device for resident tables and must not
// touch the allocator on the request path.  For them this file holds a
// variant of the global-table join (build into one open-addressing table,
// probe, project) whose only scratch is a file-scope device array of fixed
// size: the table's cells, the build side's next-chain, and a small header
// (the output-row cursor).  The caller passes the output columns.
//
// Limits: at most kNaMaxBuildRows build rows (the table holds 2x that many
// cells); any number of probe rows; output rows beyond the caller's capacity
// are counted and not written.  The scratch is one array per device and per
// process, so two calls in flight at the same time on one device (from two
// threads, streams or contexts) race on it and corrupt each other: callers
// serialise their calls.
#include "internal.h"

#include <mutex>

namespace phjg
{
namespace
{
constexpr uint64_t kNaMaxBuildRows = 1ull << 16;     // 65,536 build rows
constexpr uint64_t kNaCells = 2 * kNaMaxBuildRows;   // 2 MiB of 16-byte cells
constexpr uint64_t kNaHeaderBytes = 256;             // output cursor
constexpr uint64_t kNaScratchBytes = kNaHeaderBytes + kNaCells * sizeof(Cell) + kNaMaxBuildRows * sizeof(uint64_t);
constexpr int kNaNT = 256;

// header | cells[kNaCells] | next[kNaMaxBuildRows]  (2,621,696 bytes)
static __device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

struct NaScratch
{
    unsigned long long * rows; // output rows of the join (header)
    Cell * cells;
    uint64_t * next;
};

NaScratch carve(void * base)
{
    unsigned char * p = static_cast<unsigned char *>(base);
    NaScratch s;
    s.rows = reinterpret_cast<unsigned long long *>(p);
    s.cells = reinterpret_cast<Cell *>(p + kNaHeaderBytes);
    s.next = reinterpret_cast<uint64_t *>(p + kNaHeaderBytes + kNaCells * sizeof(Cell));
    return s;
}

// Set-up, once per device: the device address of the scratch array, taken
// with that device current.
constexpr int kNaMaxDevices = 64;
std::mutex g_na_mu;
void * g_na_addr[kNaMaxDevices] = {};

void * scratch_address(int device)
{
    if (device < 0 || device >= kNaMaxDevices)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, "device ordinal out of range for the no-allocation join");
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_addr[device])
    {
        int cur = -1;
        PHJ_CUDA(cudaGetDevice(&cur));
        if (cur != device)
            PHJ_CUDA(cudaSetDevice(device));
        void * p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (cur != device && cur >= 0)
            cudaSetDevice(cur);
        if (e != cudaSuccess || !p)
            throw Error(PHJ_ERR_CUDA, std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") + cudaGetErrorString(e));
        g_na_addr[device] = p;
    }
    return g_na_addr[device];
}

// Empty cells ({0, INVALID_REF}) and a zero output cursor.
__global__ void k_na_clear(NaScratch s, uint64_t cap)
{
    const uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 == 0)
        *s.rows = 0ull;
    for (uint64_t i = i0; i < cap; i += (uint64_t)gridDim.x * blockDim.x)
        reinterpret_cast<ulonglong2 *>(s.cells)[i] = make_ulonglong2(0ull, INVALID_REF);
}

// One table over all build rows; RowRefCell {0, row}.
__global__ void k_na_build(const uint64_t * __restrict__ keys, uint64_t n, NaScratch s, uint64_t cap)
{
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint64_t k = keys[r];
        s.next[r] = table_insert<false>(s.cells, cap, int_hash64(k), k, make_ref(0, (uint32_t)r));
    }
}

// A thread per probe row: find the head, count the chain, take the warp's
// output rows with one atomic on the cursor, then write its rows (probe
// key, build payloads, probe payloads).  Rows at or beyond `out_cap` are
// counted only.
__global__ void __launch_bounds__(kNaNT) k_na_probe(const __grid_constant__ Cols probe, uint64_t probe_rows, const __grid_constant__ Cols build, NaScratch s, uint64_t cap, const __grid_constant__ Cols out_left,
                                                    const __grid_constant__ Cols out_right, uint64_t out_cap)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < probe_rows; base += stride)
    {
        const uint64_t r = base + threadIdx.x;
        uint64_t key = 0, head = INVALID_REF;
        uint32_t cnt = 0;
        if (r < probe_rows)
        {
            key = probe.keys[r];
            head = table_find(s.cells, cap, int_hash64(key), key);
            for (uint64_t h = head; ref_valid(h); h = s.next[ref_row(h)])
                ++cnt;
        }
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d)
                incl += y;
        }
        const uint32_t warp_total = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long w0 = 0;
        if (lane == 31 && warp_total)
            w0 = atomicAdd(s.rows, (unsigned long long)warp_total);
        w0 = __shfl_sync(0xffffffffu, w0, 31);
        uint64_t o = w0 + incl - cnt;
        for (uint64_t h = head; ref_valid(h) && o < out_cap; h = s.next[ref_row(h)], ++o)
        {
            const uint32_t b = ref_row(h);
            out_left.keys[o] = key;
            for (uint32_t c = 0; c < build.n; ++c)
                copy_elem(out_left.col[c], o, build.col[c], b, build.width[c]);
            for (uint32_t c = 0; c < probe.n; ++c)
                copy_elem(out_right.col[c], o, probe.col[c], r, probe.width[c]);
        }
    }
}

void run_chj_noalloc(phj_ctx * ctx, const phj_table & B, const phj_table & P, uint64_t out_cap, uint64_t * out_keys, void * const * out_left,
                     void * const * out_right, uint64_t * out_rows)
{
    if (B.rows > kNaMaxBuildRows)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, "no-allocation join: the build side has " + std::to_string(B.rows) +
                                                  " rows; at most 65536 fit its fixed scratch");
    if (out_cap > 0 && !out_keys)
        throw Error(PHJ_ERR_INVALID_ARGUMENT, "no-allocation join: output key column missing");
    for (uint32_t c = 0; c < B.schema.n_payloads; ++c)
        if (out_cap > 0 && (!out_left || !out_left[c]))
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "no-allocation join: build payload output column missing");
    for (uint32_t c = 0; c < P.schema.n_payloads; ++c)
        if (out_cap > 0 && (!out_right || !out_right[c]))
            throw Error(PHJ_ERR_INVALID_ARGUMENT, "no-allocation join: probe payload output column missing");

    begin_run(ctx); // this call's kernel times replace the previous run's
    const NaScratch s = carve(scratch_address(ctx->device));
    const uint64_t cap = B.rows ? bit_ceil64(2 * B.rows) : 1;
    const Cols bc = cols_of(B), pc = cols_of(P);
    Cols ol = bc, orr = pc;
    ol.keys = out_keys;
    orr.keys = nullptr;
    // a caller asking only for the row count (capacity 0) may pass no
    // column arrays at all
    for (uint32_t c = 0; c < B.schema.n_payloads; ++c)
        ol.col[c] = out_left ? out_left[c] : nullptr;
    for (uint32_t c = 0; c < P.schema.n_payloads; ++c)
        orr.col[c] = out_right ? out_right[c] : nullptr;

    const unsigned fill_grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(cap, kNaNT), (uint64_t)ctx->num_sms * 4));
    {
        KTimer kt(ctx, "noalloc_clear", cap, cap * sizeof(Cell));
        k_na_clear<<<fill_grid, kNaNT, 0, ctx->stream>>>(s, cap);
        PHJ_LAUNCHED(ctx, "noalloc_clear");
    }
    if (B.rows)
    {
        KTimer kt(ctx, "noalloc_build", B.rows, B.rows * 8);
        k_na_build<<<(unsigned)std::min<uint64_t>(ceil_div(B.rows, kNaNT), (uint64_t)ctx->num_sms * 4), kNaNT, 0, ctx->stream>>>(bc.keys, B.rows,
                                                                                                                                 s, cap);
        PHJ_LAUNCHED(ctx, "noalloc_build");
    }
    if (P.rows)
    {
        KTimer kt(ctx, "noalloc_probe", P.rows, P.rows * 8);
        const unsigned grid = (unsigned)std::min<uint64_t>(ceil_div(P.rows, kNaNT), (uint64_t)ctx->num_sms * 8);
        k_na_probe<<<grid, kNaNT, 0, ctx->stream>>>(pc, P.rows, bc, s, cap, ol, orr, out_cap);
        PHJ_LAUNCHED(ctx, "noalloc_probe");
    }
    unsigned long long rows = 0;
    PHJ_CUDA(cudaMemcpyAsync(&rows, s.rows, sizeof(rows), cudaMemcpyDeviceToHost, ctx->stream));
    PHJ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (out_rows)
        *out_rows = rows;
    if (rows > out_cap)
        throw Error(PHJ_ERR_CAPACITY, "no-allocation join: " + std::to_string(rows) + " output rows, capacity " + std::to_string(out_cap) +
                                          " (the first rows up to the capacity are written)");
}
} // namespace
} // namespace phjg

extern "C" phj_status phj_run_chj_noalloc(phj_ctx * ctx, const phj_table * build, const phj_table * probe, uint64_t out_capacity,
                                          uint64_t * out_keys, void * const * out_left, void * const * out_right, uint64_t * out_rows)
{
    if (!ctx || !build || !probe)
        return PHJ_ERR_INVALID_ARGUMENT;
    if (out_rows)
        *out_rows = 0;
    phjg::DeviceScope dev(ctx);
    if (!dev.ok())
    {
        ctx->last_error = dev.message(ctx);
        return PHJ_ERR_CUDA;
    }
    try
    {
        phjg::run_chj_noalloc(ctx, *build, *probe, out_capacity, out_keys, out_left, out_right, out_rows);
        ctx->last_error.clear();
        return PHJ_OK;
    }
    catch (const phjg::Error & e)
    {
        ctx->last_error = e.what();
        return e.status;
    }
    catch (const std::exception & e)
    {
        ctx->last_error = e.what();
        return PHJ_ERR_CUDA;
    }
}
