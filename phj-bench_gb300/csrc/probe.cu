// probe.cu -- probe with output projection (probeOneBlock, src/JoinOps.h:236-272;
// probeOneBlockCHJ, src/JoinOps.h:381-429; ProbeMaterialiser::gatherFromProbeBlock,
// src/JoinOps.h:77-125).
//
// Two barrier-free kernels whose warps are independent workers over chunks
// of 256 probe rows, taken in increasing order across the grid so the whole
// grid sweeps the probe side front to back and the leaf tables of the rows
// in flight stay in L2:
//   k_probe_lookup   hash each key, locate its leaf table (or CHJ sub-table)
//                    from the top hash bits, look it up, and record the head
//                    build row (or none) per probe row plus the chunk's
//                    match count (1 per hit, or the next-chain length when
//                    some build key repeats);
//   scan_u32         chunk counts -> each chunk's first output row;
//   k_probe_project  re-walk the chunk, place each match with a warp scan,
//                    and write the output column-major: key column (the
//                    probe key, as the reference emits it), build payloads
//                    gathered through the RowRefCell, probe payloads.
// This is the reference's "batchFind heads, expand chains into flat
// (probe_idx, build_ref) arrays, then gather column-major" with the head
// array in memory and the expansion folded into the projection.
//
// When no build key repeats (a probe row then has at most one output row)
// and the build payloads are gathered in one piece, one kernel does both:
//   k_probe_fused    per warp chunk (taken by ticket): the lookups, one
//                    reservation of the chunk's output rows on the join's
//                    row counter, then the projection from shared memory;
//                    the output is sized by the probe rows beforehand.
#include "internal.h"

#include <cstdio>
#include <cstdlib>
#include <type_traits>

namespace phjg
{
namespace
{
constexpr int kPNT = 256;
constexpr int kPRPT = 8;
constexpr int kPWarps = kPNT / 32;
constexpr uint32_t kWChunk = 32 * kPRPT; // probe rows per warp chunk
constexpr uint32_t kNoMatch = 0xFFFFFFFFu;

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

// Every output column as one list for the projection loop: the key column
// (from the probe keys), the build payloads (gathered by build row), the
// probe payloads (by probe row).
constexpr int kMaxOutCols = 1 + 2 * kMaxCols;
struct ProjCols
{
    const void * src[kMaxOutCols];
    void * dst[kMaxOutCols];
    uint8_t width[kMaxOutCols];
    uint8_t by_build[kMaxOutCols];
    uint32_t n;
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

// Linear probing from cell `pos` on (the first cell collided).
__device__ __noinline__ uint64_t table_find_from(const Cell * cells, uint64_t cap, uint64_t pos, uint64_t key)
{
    const uint64_t mask = cap - 1;
    pos &= mask;
    for (uint64_t step = 1; step < cap; ++step)
    {
        const ulonglong2 c = __ldg(reinterpret_cast<const ulonglong2 *>(cells + pos));
        if (!ref_valid(c.y))
            return INVALID_REF;
        if (c.x == key)
            return c.y;
        pos = (pos + 1) & mask;
    }
    return INVALID_REF;
}

__device__ __noinline__ uint32_t chain_length(uint32_t brow, const ProbeArgs & a, int chj)
{
    uint32_t c = 1;
    uint64_t r = __ldg(a.next + brow);
    while (ref_valid(r))
    {
        ++c;
        const uint32_t b = chj ? build_row_of<kChj>(r, a) : build_row_of<kLeafMeta>(r, a);
        r = __ldg(a.next + b);
    }
    return c;
}


// Column pass of one warp over its match list: lane l writes output rows
// base + l, base + l + 32, ... (coalesced); eight loads are in flight per
// lane before its stores.
template <class T, bool kBuild>
__device__ __forceinline__ void column_pass(const void * src_v, void * dst_v, const uint32_t * idx, uint32_t n, uint64_t base, uint32_t lane)
{
    const T * src = static_cast<const T *>(src_v);
    T * dst = static_cast<T *>(dst_v) + base;
    uint32_t i = lane;
    for (; i + 7 * 32 < n; i += 8 * 32)
    {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
            v[u] = kBuild ? __ldg(src + idx[i + u * 32]) : __ldcs(src + idx[i + u * 32]);
#pragma unroll
        for (int u = 0; u < 8; ++u)
            __stcs(dst + i + u * 32, v[u]);
    }
    for (; i < n; i += 32)
        __stcs(dst + i, kBuild ? __ldg(src + idx[i]) : __ldcs(src + idx[i]));
}

template <bool kBuild>
__device__ __forceinline__ void columns_pass(const Cols & src, void * const * dst, const uint32_t * idx, uint32_t n, uint64_t base, uint32_t lane)
{
#pragma unroll 1
    for (uint32_t c = 0; c < src.n; ++c)
        switch (src.width[c])
        {
            case 1: column_pass<uint8_t, kBuild>(src.col[c], dst[c], idx, n, base, lane); break;
            case 2: column_pass<uint16_t, kBuild>(src.col[c], dst[c], idx, n, base, lane); break;
            case 4: column_pass<uint32_t, kBuild>(src.col[c], dst[c], idx, n, base, lane); break;
            case 8: column_pass<uint64_t, kBuild>(src.col[c], dst[c], idx, n, base, lane); break;
            default: column_pass<uint4, kBuild>(src.col[c], dst[c], idx, n, base, lane); break;
        }
}

// Lookup of one warp chunk (kWChunk probe rows from chunk * kWChunk): per
// row, its head build row (kNoMatch when the key is absent) and match count
// go to the sink (sink(i, brow, count) for row i of the chunk; sink.key(i,
// key) as each key is read); rows whose key lies past the first cell pair
// wait in the warp's queue (qkey, qrow) and are probed after the chunk.
// Returns this lane's share of the chunk's output rows.  kWin (CHJ only):
// rows outside the sub-table window [a.win_lo, a.win_hi) touch no table and
// record no match.
template <int kMode, bool kDup, bool kWin, class Sink>
__device__ __forceinline__ uint32_t lookup_chunk(const ProbeArgs & a, uint64_t chunk, uint32_t lane, uint64_t * qkey, uint16_t * qrow,
                                                 const Sink & sink)
{
    const uint32_t shift = 64u - a.leaf_bits;
    const uint32_t ulog = kMode == kLeafUniform ? (uint32_t)a.uniform_log2cap : 0u;
    const uint64_t ucap = 1ull << ulog;
    const uint64_t row0 = chunk * kWChunk + lane; // + k * 32
    uint64_t key[kPRPT];
    uint32_t live = 0;
#pragma unroll
    for (int k = 0; k < kPRPT; ++k)
    {
        const uint64_t row = row0 + (uint64_t)k * 32;
        key[k] = 0;
        if (row < a.probe_rows)
        {
            key[k] = __ldcs(a.probe.keys + row);
            live |= 1u << k;
            sink.key(k * 32 + lane, key[k]);
        }
    }
    uint32_t total = 0;
    uint32_t qn = 0; // rows in the warp's queue
    // four directory loads (per-leaf tables), four first-cell loads,
    // then the comparisons: four table requests in flight per lane
#pragma unroll
    for (int g = 0; g < kPRPT; g += 4)
    {
        ulonglong2 mv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            mv[u] = make_ulonglong2(0ull, 0ull);
            if (kWin && (live >> (g + u) & 1u) && (uint32_t)(int_hash64(key[g + u]) >> shift) - a.win_lo >= a.win_hi - a.win_lo)
                continue; // outside the window: the directory entry stays empty (no table)
            if (kMode != kLeafUniform && (live >> (g + u) & 1u))
                mv[u] = __ldg(reinterpret_cast<const ulonglong2 *>(a.meta + (uint32_t)(int_hash64(key[g + u]) >> shift)));
        }
        CellPair cell[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const int k = g + u;
            cell[u].a = make_ulonglong2(0ull, INVALID_REF);
            cell[u].b = cell[u].a;
            if (!(live >> k & 1u))
                continue;
            const uint64_t h = int_hash64(key[k]);
            if (kMode == kLeafUniform)
                cell[u] = load_pair<false>(a.cells + ((uint64_t)(uint32_t)(h >> shift) << ulog) + probe_start(h, ucap));
            else if ((mv[u].y >> 40) & 0xffu)
                cell[u] = load_pair<false>(a.cells + mv[u].x + probe_start(h, 1ull << ((uint32_t)(mv[u].y >> 32) & 0xffu)));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const int k = g + u;
            uint32_t brow = kNoMatch, mcnt = 0;
            // the pair's two cells are the first two probe positions
            uint64_t head = INVALID_REF;
            bool more = false;
            if (ref_valid(cell[u].a.y))
            {
                if (cell[u].a.x == key[k])
                    head = cell[u].a.y;
                else if (ref_valid(cell[u].b.y))
                {
                    if (cell[u].b.x == key[k])
                        head = cell[u].b.y;
                    else
                        more = true;
                }
            }
            {
                // rows whose key lies past the cell pair wait in the
                // warp's queue and are probed together after the chunk
                const uint32_t m = __ballot_sync(0xffffffffu, more);
                if (more)
                {
                    const uint32_t slot = qn + __popc(m & ((1u << lane) - 1u));
                    qkey[slot] = key[k];
                    qrow[slot] = (uint16_t)(k * 32 + lane);
                }
                qn += __popc(m);
            }
            if (!more)
            {
                if (ref_valid(head))
                {
                    brow = build_row_of<kMode>(head, a);
                    const bool leaf_dup = kMode == kLeafUniform ? true : ((mv[u].y >> 48) & 1u) != 0;
                    if (kDup && kMode != kChj && a.grouped)
                        mcnt = ref_block(head) ? ref_block(head) : 1u; // grouped: {count, first row}
                    else
                        mcnt = (kDup && leaf_dup) ? chain_length(brow, a, kMode == kChj) : 1u;
                    total += mcnt;
                }
            }
            if ((live >> k & 1u) && !more)
                sink(k * 32 + lane, brow, mcnt);
        }
    }
    {
        __syncwarp();
        for (uint32_t j = lane; j < qn; j += 32)
        {
            const uint64_t qk = qkey[j];
            const uint64_t h = int_hash64(qk);
            uint64_t head;
            bool leaf_dup = true;
            if (kMode == kLeafUniform)
                head = table_find_from(a.cells + ((uint64_t)(uint32_t)(h >> shift) << ulog), ucap, probe_start(h, ucap) + 2, qk);
            else
            {
                const ulonglong2 m = __ldg(reinterpret_cast<const ulonglong2 *>(a.meta + (uint32_t)(h >> shift)));
                const uint64_t c = 1ull << ((uint32_t)(m.y >> 32) & 0xffu);
                head = table_find_from(a.cells + m.x, c, probe_start(h, c) + 2, qk);
                leaf_dup = ((m.y >> 48) & 1u) != 0;
            }
            uint32_t brow = kNoMatch, mcnt = 0;
            if (ref_valid(head))
            {
                brow = build_row_of<kMode>(head, a);
                if (kDup && kMode != kChj && a.grouped)
                    mcnt = ref_block(head) ? ref_block(head) : 1u;
                else
                    mcnt = (kDup && leaf_dup) ? chain_length(brow, a, kMode == kChj) : 1u;
                total += mcnt;
            }
            sink(qrow[j], brow, mcnt);
        }
        __syncwarp();
    }
    return total;
}

// Lookup results to global memory: the head array and (keys repeat) the
// per-row match counts.
template <bool kDup>
struct HeadSink
{
    uint32_t * heads;
    uint32_t * row_cnt;
    uint64_t row0; // first row of the chunk
    __device__ __forceinline__ void key(uint32_t, uint64_t) const {}
    __device__ __forceinline__ void operator()(uint32_t i, uint32_t brow, uint32_t mcnt) const
    {
        heads[row0 + i] = brow;
        if (kDup && row_cnt)
            row_cnt[row0 + i] = mcnt;
    }
};

// Lookups: per probe row its head build row (kNoMatch when the key is
// absent), per warp chunk its number of output rows.
template <int kMode, bool kDup, bool kWin = false>
__global__ void __launch_bounds__(kPNT, 4) k_probe_lookup(const __grid_constant__ ProbeArgs a, uint32_t * __restrict__ heads,
                                                       uint32_t * __restrict__ counts)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
    const uint64_t n_workers = ((uint64_t)gridDim.x * kPNT) >> 5;
    __shared__ uint64_t q_key[kPWarps * kWChunk];
    __shared__ uint16_t q_row[kPWarps * kWChunk];
    uint64_t * qkey = q_key + (threadIdx.x >> 5) * kWChunk;
    uint16_t * qrow = q_row + (threadIdx.x >> 5) * kWChunk;
    unsigned long long grand = 0;
    for (uint64_t chunk = ((uint64_t)blockIdx.x * kPNT + threadIdx.x) >> 5; chunk < n_chunks; chunk += n_workers)
    {
        const HeadSink<kDup> sink{heads, a.row_cnt, chunk * kWChunk};
        uint32_t total = lookup_chunk<kMode, kDup, kWin>(a, chunk, lane, qkey, qrow, sink);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            total += __shfl_xor_sync(0xffffffffu, total, o);
        if (lane == 0)
            counts[chunk] = total;
        grand += total;
    }
    // the join's row count in 64 bits (the chunk offsets are 32-bit)
    if (lane == 0 && grand)
        atomicAdd(a.out_rows64, grand);
}

// The projection walks a warp chunk in halves of kPH rounds (to bound
// registers); the output offset carries over from one half to the next.
constexpr int kPH = 4;
// window projection: four CTAs of 256 threads per SM (at most 64 registers
// a thread) keep more gathers in flight than three CTAs with more registers
// each (measured)
constexpr int kProjMinBlocks = 4;

// One column over a lane's single-match rows of a half: four loads, then
// four stores.  Output row of round k is base + rel[k].
template <class T, int kN = kPH>
__device__ __forceinline__ void project_column(const void * src_v, void * dst_v, const uint32_t (&sidx)[kN], uint64_t base,
                                               const uint32_t (&rel)[kN], uint32_t one, bool gather)
{
    const T * src = static_cast<const T *>(src_v);
    T * dst = static_cast<T *>(dst_v) + base;
    T v[kN];
#pragma unroll
    for (int u = 0; u < kN; ++u)
        if (one >> u & 1u)
            v[u] = gather ? __ldg(src + sidx[u]) : __ldcs(src + sidx[u]);
#pragma unroll
    for (int u = 0; u < kN; ++u)
        if (one >> u & 1u)
            __stcs(dst + rel[u], v[u]);
}

// All output columns, one switch instance for the loop.  Without 16-byte
// columns (kWide false) the widest staged value is 8 bytes, which keeps the
// plain projection at four CTAs per SM.
template <bool kWide = true, int kN = kPH>
__device__ __forceinline__ void project_all(const ProjCols & pc, const uint32_t (&brow)[kN], const uint32_t (&prow)[kN], uint64_t base,
                                            const uint32_t (&rel)[kN], uint32_t one)
{
#pragma unroll 1
    for (uint32_t c = 0; c < pc.n; ++c)
    {
        const bool g = pc.by_build[c] != 0;
        uint32_t idx[kN];
#pragma unroll
        for (int u = 0; u < kN; ++u)
            idx[u] = g ? brow[u] : prow[u];
        switch (pc.width[c])
        {
            case 1: project_column<uint8_t, kN>(pc.src[c], pc.dst[c], idx, base, rel, one, g); break;
            case 2: project_column<uint16_t, kN>(pc.src[c], pc.dst[c], idx, base, rel, one, g); break;
            case 4: project_column<uint32_t, kN>(pc.src[c], pc.dst[c], idx, base, rel, one, g); break;
            case 8: project_column<uint64_t, kN>(pc.src[c], pc.dst[c], idx, base, rel, one, g); break;
            default:
                if constexpr (kWide)
                    project_column<uint4, kN>(pc.src[c], pc.dst[c], idx, base, rel, one, g);
                break;
        }
    }
}

// Projection when no key repeats: warp chunk c writes its output rows from
// offs[c] on, column by column.
template <int kMode, bool kWide>
__global__ void __launch_bounds__(kPNT, kWide ? 1 : 4) k_probe_project(const __grid_constant__ ProbeArgs a, const __grid_constant__ ProjCols pc,
                                                        const uint32_t * __restrict__ heads, const uint32_t * __restrict__ offs, uint64_t out_cap)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
    const uint64_t n_workers = ((uint64_t)gridDim.x * kPNT) >> 5;
    for (uint64_t chunk = ((uint64_t)blockIdx.x * kPNT + threadIdx.x) >> 5; chunk < n_chunks; chunk += n_workers)
    {
        uint64_t base = offs[chunk];
#pragma unroll 1
        for (int half = 0; half < kPRPT / kPH; ++half)
        {
            const uint64_t row0 = chunk * kWChunk + (uint64_t)half * kPH * 32 + lane;
            uint32_t brow[kPH], prow[kPH], cnt[kPH];
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                const uint64_t row = row0 + (uint64_t)k * 32;
                prow[k] = (uint32_t)row;
                brow[k] = row < a.probe_rows ? __ldcs(heads + row) : kNoMatch;
            }
            uint32_t one = 0;
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                cnt[k] = brow[k] != kNoMatch ? 1u : 0u;
                one |= cnt[k] << k;
            }
            // placement: warp scan per round, round-major
            uint32_t rel[kPH];
            uint32_t running = 0;
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                uint32_t x = cnt[k];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1)
                {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                    if (lane >= (uint32_t)d)
                        x += y;
                }
                rel[k] = running + x - cnt[k];
                running += __shfl_sync(0xffffffffu, x, 31);
                if (base + rel[k] >= out_cap)
                    one &= ~(1u << k);
            }
            // key column (the probe key), build payloads, probe payloads
            project_all<kWide>(pc, brow, prow, base, rel, one);
            base += running;
        }
    }
}

// Build payload columns of the packed projection: output column, width and
// byte offset in the packed 16-byte row.
struct PackedCols
{
    void * dst[kMaxCols];
    uint8_t width[kMaxCols];
    uint8_t off[kMaxCols];
    uint32_t n;
};

// One build payload column of a half from the gathered packed rows.  The
// offset is a multiple of the width, so a value lies in one 8-byte half.
template <class T, int kN = kPH>
__device__ __forceinline__ void packed_column(const uint4 (&row)[kN], uint32_t off, void * dst_v, uint64_t base, const uint32_t (&rel)[kN],
                                              uint32_t one)
{
    T * dst = static_cast<T *>(dst_v) + base;
#pragma unroll
    for (int u = 0; u < kN; ++u)
        if (one >> u & 1u)
        {
            if constexpr (sizeof(T) == 8)
                __stcs(dst + rel[u], off ? ((uint64_t)row[u].w << 32 | row[u].z) : ((uint64_t)row[u].y << 32 | row[u].x));
            else
            {
                // the 32-bit word holding the value, then its bytes
                const uint32_t wd = (off & 8u) ? ((off & 4u) ? row[u].w : row[u].z) : ((off & 4u) ? row[u].y : row[u].x);
                __stcs(dst + rel[u], (T)(wd >> ((off & 3u) * 8u)));
            }
        }
}

// Projection when no key repeats and the build payloads are packed: as
// k_probe_project, with one 16-byte gather per output row for all build
// payload columns (fewer random requests through L1, the kernel's busiest
// path); pc holds the key column and the probe payload columns only.
template <bool kWide>
__global__ void __launch_bounds__(kPNT, kWide ? 1 : 4) k_probe_project_packed(const __grid_constant__ ProbeArgs a, const __grid_constant__ ProjCols pc,
                                                                           const __grid_constant__ PackedCols bc, const uint32_t * __restrict__ heads,
                                                                           const uint32_t * __restrict__ offs, uint64_t out_cap)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
    const uint64_t n_workers = ((uint64_t)gridDim.x * kPNT) >> 5;
    for (uint64_t chunk = ((uint64_t)blockIdx.x * kPNT + threadIdx.x) >> 5; chunk < n_chunks; chunk += n_workers)
    {
        uint64_t base = offs[chunk];
#pragma unroll 1
        for (int half = 0; half < kPRPT / kPH; ++half)
        {
            const uint64_t row0 = chunk * kWChunk + (uint64_t)half * kPH * 32 + lane;
            uint32_t brow[kPH], prow[kPH], one = 0;
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                const uint64_t row = row0 + (uint64_t)k * 32;
                prow[k] = (uint32_t)row;
                brow[k] = row < a.probe_rows ? __ldcs(heads + row) : kNoMatch;
                if (brow[k] != kNoMatch)
                    one |= 1u << k;
            }
            uint32_t rel[kPH], running = 0;
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                const uint32_t m = __ballot_sync(0xffffffffu, one >> k & 1u);
                rel[k] = running + __popc(m & ((1u << lane) - 1u));
                running += __popc(m);
                if (base + rel[k] >= out_cap)
                    one &= ~(1u << k);
            }
            // key and probe payload columns first (prow is then dead)
            project_all<kWide>(pc, brow, prow, base, rel, one);
            {
                uint4 row[kPH];
#pragma unroll
                for (int u = 0; u < kPH; ++u)
                    if (one >> u & 1u)
                        row[u] = __ldg(a.packed + brow[u]);
#pragma unroll 1
                for (uint32_t c = 0; c < bc.n; ++c)
                    switch (bc.width[c])
                    {
                        case 1: packed_column<uint8_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                        case 2: packed_column<uint16_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                        case 4: packed_column<uint32_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                        default: packed_column<uint64_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                    }
            }
            base += running;
        }
    }
}

// The fused kernel's lookup of one warp chunk (no repeated build key): the
// chunk's keys arrive in the warp's part of shared memory by asynchronous
// copies (no register waits on them) and are read back four at a time for
// the table loads; each row's head build row (kNoMatch when absent) goes to
// brow_s; rows whose key lies past the first cell pair wait in the warp's
// queue (their chunk rows in qrow) and are probed after the chunk.  Returns
// this lane's number of matches.
template <int kMode>
__device__ __forceinline__ uint32_t fused_lookup(const ProbeArgs & a, uint64_t chunk, uint32_t lane, uint64_t * key_s, uint32_t * brow_s,
                                                 uint16_t * qrow)
{
    const uint32_t shift = 64u - a.leaf_bits;
    const uint32_t ulog = kMode == kLeafUniform ? (uint32_t)a.uniform_log2cap : 0u;
    const uint64_t ucap = 1ull << ulog;
    const uint64_t row0 = chunk * kWChunk + lane; // + k * 32
    uint32_t live = 0;
    const uint64_t stream = l2_evict_first(); // keys are read once
#pragma unroll
    for (int k = 0; k < kPRPT; ++k)
    {
        const uint64_t row = row0 + (uint64_t)k * 32;
        if (row < a.probe_rows)
        {
            cp_async8(key_s + k * 32 + lane, a.probe.keys + row, stream);
            live |= 1u << k;
        }
    }
    cp_async_wait_all();
    uint32_t total = 0;
    uint32_t qn = 0;
#pragma unroll
    for (int g = 0; g < kPRPT; g += 4)
    {
        uint64_t key[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            key[u] = (live >> (g + u) & 1u) ? ld_shared_u64(key_s + (g + u) * 32 + lane) : 0ull;
        ulonglong2 mv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            mv[u] = make_ulonglong2(0ull, 0ull);
            if (kMode != kLeafUniform && (live >> (g + u) & 1u))
                mv[u] = __ldg(reinterpret_cast<const ulonglong2 *>(a.meta + (uint32_t)(int_hash64(key[u]) >> shift)));
        }
        CellPair cell[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            cell[u].a = make_ulonglong2(0ull, INVALID_REF);
            cell[u].b = cell[u].a;
            if (!(live >> (g + u) & 1u))
                continue;
            const uint64_t h = int_hash64(key[u]);
            if (kMode == kLeafUniform)
                cell[u] = load_pair<false>(a.cells + ((uint64_t)(uint32_t)(h >> shift) << ulog) + probe_start(h, ucap));
            else if ((mv[u].y >> 40) & 0xffu)
                cell[u] = load_pair<false>(a.cells + mv[u].x + probe_start(h, 1ull << ((uint32_t)(mv[u].y >> 32) & 0xffu)));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const uint32_t i = (uint32_t)(g + u) * 32 + lane;
            uint64_t head = INVALID_REF;
            bool more = false;
            if (ref_valid(cell[u].a.y))
            {
                if (cell[u].a.x == key[u])
                    head = cell[u].a.y;
                else if (ref_valid(cell[u].b.y))
                {
                    if (cell[u].b.x == key[u])
                        head = cell[u].b.y;
                    else
                        more = true;
                }
            }
            const uint32_t m = __ballot_sync(0xffffffffu, more);
            if (more)
                qrow[qn + __popc(m & ((1u << lane) - 1u))] = (uint16_t)i;
            qn += __popc(m);
            if ((live >> (g + u) & 1u) && !more)
            {
                const uint32_t brow = ref_valid(head) ? build_row_of<kMode>(head, a) : kNoMatch;
                total += brow != kNoMatch;
                brow_s[i] = brow;
            }
        }
    }
    __syncwarp();
    for (uint32_t j = lane; j < qn; j += 32)
    {
        const uint32_t i = qrow[j];
        const uint64_t qk = key_s[i];
        const uint64_t h = int_hash64(qk);
        uint64_t head;
        if (kMode == kLeafUniform)
            head = table_find_from(a.cells + ((uint64_t)(uint32_t)(h >> shift) << ulog), ucap, probe_start(h, ucap) + 2, qk);
        else
        {
            const ulonglong2 m = __ldg(reinterpret_cast<const ulonglong2 *>(a.meta + (uint32_t)(h >> shift)));
            const uint64_t c = 1ull << ((uint32_t)(m.y >> 32) & 0xffu);
            head = table_find_from(a.cells + m.x, c, probe_start(h, c) + 2, qk);
        }
        const uint32_t brow = ref_valid(head) ? build_row_of<kMode>(head, a) : kNoMatch;
        total += brow != kNoMatch;
        brow_s[i] = brow;
    }
    __syncwarp();
    return total;
}

// Shared memory of one warp of the fused kernel: the build rows' gather
// stage (half a chunk of 16-byte rows), the chunk's keys, head build rows
// and queue; 44 KB a CTA, static, so three CTAs a SM leave L1 about 120 KB
// (16 KB more a CTA ran the 16M x 256M probe 5% slower).
constexpr uint32_t kFStage = 0, kFKeys = 2048, kFBrow = 4096, kFQueue = 5120, kFWarpBytes = 5632;

// Lookup and projection in one pass, when no build key repeats and the
// build payloads are packed (kGather 16: one 16-byte row of a.packed), or
// are one column of 4 or 8 bytes (kGather 4 or 8: a.build.col[0]), or are
// none (kGather 0).  A probe row then has at most one output row,
// so the output is sized by the probe rows before the probe, and a warp
// needs no offsets from other chunks: it looks its chunk up, reserves the
// chunk's output rows with one atomic on the join's row counter, and
// writes them -- no head array written and read back, no second read of
// the probe keys.  Per half chunk, the build rows' gathers go to the
// warp's stage by asynchronous copies while the key column (from
// shared memory) and the probe payload columns are written, then the build
// payloads are written from the stage.  Warps take chunks by ticket (one
// atomic a chunk).  A chunk's output rows are contiguous; chunks land in
// reservation order.  pc holds the probe payload columns only.
template <int kMode, int kGather>
__global__ void __launch_bounds__(kPNT, 3) k_probe_fused(const __grid_constant__ ProbeArgs a, const __grid_constant__ ProjCols pc,
                                                      const __grid_constant__ PackedCols bc, uint64_t * __restrict__ out_keys,
                                                      unsigned long long * __restrict__ out_rows, unsigned long long * __restrict__ tickets,
                                                      uint64_t out_cap)
{
    __shared__ __align__(16) uint8_t fsm[kPWarps * kFWarpBytes];
    const uint32_t lane = threadIdx.x & 31;
    uint8_t * wsm = fsm + (threadIdx.x >> 5) * kFWarpBytes;
    uint4 * stage = reinterpret_cast<uint4 *>(wsm + kFStage);
    uint64_t * key_s = reinterpret_cast<uint64_t *>(wsm + kFKeys);
    uint32_t * brow_s = reinterpret_cast<uint32_t *>(wsm + kFBrow);
    uint16_t * qrow = reinterpret_cast<uint16_t *>(wsm + kFQueue);
    const uint32_t n_chunks = (uint32_t)ceil_div(a.probe_rows, kWChunk); // probe rows < 2^32
    // chunks in ticket order: the warps in flight stay within a few hundred
    // chunks of each other, so the leaf tables and packed build rows of the
    // buckets being probed stay in L2 (with a fixed stride per warp, warps
    // drifted across buckets and the kernel read twice its bytes from DRAM)
    unsigned long long t0 = 0;
    if (lane == 0)
        t0 = atomicAdd(tickets, 1ull);
    uint32_t chunk = (uint32_t)__shfl_sync(0xffffffffu, t0, 0);
    while (chunk < n_chunks)
    {
        unsigned long long tn = 0; // the next chunk's ticket, taken early
        if (lane == 0)
            tn = atomicAdd(tickets, 1ull);
        uint32_t total = fused_lookup<kMode>(a, chunk, lane, key_s, brow_s, qrow);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            total += __shfl_xor_sync(0xffffffffu, total, o);
        if (total == 0)
        {
            chunk = (uint32_t)__shfl_sync(0xffffffffu, tn, 0);
            continue;
        }
        unsigned long long b0 = 0;
        if (lane == 0)
            b0 = atomicAdd(out_rows, (unsigned long long)total);
        uint64_t base = __shfl_sync(0xffffffffu, b0, 0);
#pragma unroll 1
        for (int half = 0; half < 2; ++half)
        {
            const uint32_t i0 = (uint32_t)half * (kWChunk / 2) + lane;
            uint32_t brow[kPH], prow[kPH], one = 0;
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                const uint32_t i = i0 + (uint32_t)k * 32;
                const uint64_t row = (uint64_t)chunk * kWChunk + i;
                prow[k] = (uint32_t)row;
                brow[k] = row < a.probe_rows ? brow_s[i] : kNoMatch;
                if (brow[k] != kNoMatch)
                {
                    one |= 1u << k;
                    if constexpr (kGather == 16)
                        cp_async16(stage + k * 32 + lane, a.packed + brow[k]);
                    else if constexpr (kGather != 0)
                        cp_async_small<kGather>(stage + k * 32 + lane, static_cast<const uint8_t *>(a.build.col[0]) + (uint64_t)brow[k] * kGather);
                }
            }
            uint32_t rel[kPH], running = 0;
#pragma unroll
            for (int k = 0; k < kPH; ++k)
            {
                const uint32_t m = __ballot_sync(0xffffffffu, one >> k & 1u);
                rel[k] = running + __popc(m & ((1u << lane) - 1u));
                running += __popc(m);
                if (base + rel[k] >= out_cap)
                    one &= ~(1u << k);
            }
#pragma unroll
            for (int u = 0; u < kPH; ++u)
                if (one >> u & 1u)
                    __stcs(out_keys + base + rel[u], key_s[i0 + (uint32_t)u * 32]);
            project_all<false>(pc, brow, prow, base, rel, one);
            if constexpr (kGather != 0)
            {
                cp_async_wait_all();
                uint4 row[kPH];
#pragma unroll
                for (int u = 0; u < kPH; ++u)
                    row[u] = stage[u * 32 + lane];
#pragma unroll 1
                for (uint32_t c = 0; c < bc.n; ++c)
                    switch (bc.width[c])
                    {
                        case 1: packed_column<uint8_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                        case 2: packed_column<uint16_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                        case 4: packed_column<uint32_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                        default: packed_column<uint64_t>(row, bc.off[c], bc.dst[c], base, rel, one); break;
                    }
            }
            base += running;
            __syncwarp(); // the stage is refilled by the next half
        }
        chunk = (uint32_t)__shfl_sync(0xffffffffu, tn, 0);
    }
}

// Projection over grouped leaves (a probe row's matches are the build rows
// [first, first + count)) or over a flat chain expansion (kFlat: the build
// row of every output row), expanded over a whole warp chunk: the 256 rows'
// first output offsets and first build rows are staged in the warp's part
// of shared memory, and each step places 4 x 32 consecutive output rows of
// the chunk, a lane finding the probe row that owns output j by an 8-step
// binary search of the offsets.  Every output row costs the same whatever
// the match counts, the stores of a step are consecutive, and every step is
// full (expanding 32 probe rows at a time left most slots of a step empty
// at two matches a row: 4.9 ms against 3.6 ms for 32M x 128M).
template <bool kFlat>
__global__ void __launch_bounds__(kPNT, kProjMinBlocks) k_probe_project_window(const __grid_constant__ ProbeArgs a,
                                                                         const __grid_constant__ ProjCols pc, const uint32_t * __restrict__ heads,
                                                                         const uint32_t * __restrict__ offs, uint64_t out_cap)
{
    __shared__ uint32_t s_start[kPWarps][kWChunk];
    __shared__ uint32_t s_first[kPWarps][kWChunk];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t * st = s_start[warp];
    uint32_t * sf = s_first[warp];
    const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
    const uint64_t n_workers = ((uint64_t)gridDim.x * kPNT) >> 5;
    for (uint64_t chunk = ((uint64_t)blockIdx.x * kPNT + threadIdx.x) >> 5; chunk < n_chunks; chunk += n_workers)
    {
        const uint64_t base = offs[chunk];
        // each row's first output (exclusive prefix over the chunk, rows in
        // order) and first build row; rows without a match share the start
        // of the next row, so the search lands on the matching one
        uint32_t running = 0;
#pragma unroll 1
        for (int k = 0; k < kPRPT; ++k)
        {
            const uint64_t row = chunk * kWChunk + (uint64_t)k * 32 + lane;
            uint32_t first = 0, cnt = 0;
            if (row < a.probe_rows)
            {
                first = __ldcs(heads + row);
                if (first != kNoMatch)
                    cnt = __ldcs(a.row_cnt + row);
            }
            uint32_t incl = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= (uint32_t)d)
                    incl += y;
            }
            st[k * 32 + lane] = running + incl - cnt;
            sf[k * 32 + lane] = first;
            running += __shfl_sync(0xffffffffu, incl, 31);
        }
        __syncwarp();
        const uint32_t T = running;
#pragma unroll 1
        for (uint32_t t = 0; t < T; t += kPH * 32)
        {
            uint32_t brow[kPH], prow[kPH], rel[kPH], one = 0;
#pragma unroll
            for (int u = 0; u < kPH; ++u)
            {
                const uint32_t j = t + (uint32_t)u * 32 + lane;
                // largest L with start[L] <= j
                uint32_t L = 0;
#pragma unroll
                for (uint32_t b = kWChunk / 2; b >= 1; b >>= 1)
                    if (st[L + b] <= j)
                        L += b;
                if (kFlat)
                    brow[u] = j < T ? __ldcs(a.flat + base + j) : 0u; // expanded chain
                else
                    brow[u] = sf[L] + (j - st[L]);
                prow[u] = (uint32_t)(chunk * kWChunk + L);
                rel[u] = j;
                if (j < T && base + j < out_cap)
                    one |= 1u << u;
            }
            project_all(pc, brow, prow, base, rel, one);
        }
        __syncwarp();
    }
}

// Packs build payload columns row-major (pack_row) into out[r].
__global__ void k_pack_rows(const __grid_constant__ Cols in, uint64_t n, const __grid_constant__ PackSpec pk, uint4 * __restrict__ out)
{
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x)
        out[r] = pack_row(in, r, pk);
}

// Chained duplicates (CHJ, leaves too large to group, lazily built BEP
// tables): each probe row's chain is walked once and its build rows are
// written to a flat array at the row's output offsets, which the range
// projection then reads in output order.
template <int kMode>
__global__ void __launch_bounds__(kPNT) k_probe_expand(const __grid_constant__ ProbeArgs a, const uint32_t * __restrict__ heads,
                                                       const uint32_t * __restrict__ offs, uint64_t out_cap)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
    const uint64_t n_workers = ((uint64_t)gridDim.x * kPNT) >> 5;
    for (uint64_t chunk = ((uint64_t)blockIdx.x * kPNT + threadIdx.x) >> 5; chunk < n_chunks; chunk += n_workers)
    {
        uint64_t base = offs[chunk];
#pragma unroll 1
        for (int k = 0; k < kPRPT; ++k)
        {
            const uint64_t row = chunk * kWChunk + (uint64_t)k * 32 + lane;
            uint32_t b = kNoMatch, cnt = 0;
            if (row < a.probe_rows)
            {
                b = __ldcs(heads + row);
                if (b != kNoMatch)
                    cnt = __ldcs(a.row_cnt + row);
            }
            uint32_t incl = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= (uint32_t)d)
                    incl += y;
            }
            uint64_t o = base + incl - cnt;
            for (uint32_t i = 0; i < cnt && o < out_cap; ++i, ++o)
            {
                a.flat[o] = b;
                if (i + 1 < cnt)
                    b = build_row_of<kMode>(__ldg(a.next + b), a);
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

} // namespace

static ProjCols proj_cols(const ProbeArgs & a, const OutCols & o)
{
    ProjCols pc{};
    uint32_t n = 0;
    pc.src[n] = a.probe.keys;
    pc.dst[n] = o.keys;
    pc.width[n] = 8;
    pc.by_build[n++] = 0;
    for (uint32_t c = 0; c < a.build.n; ++c)
    {
        pc.src[n] = a.build.col[c];
        pc.dst[n] = o.left[c];
        pc.width[n] = a.build.width[c];
        pc.by_build[n++] = 1;
    }
    for (uint32_t c = 0; c < a.probe.n; ++c)
    {
        pc.src[n] = a.probe.col[c];
        pc.dst[n] = o.right[c];
        pc.width[n] = a.probe.width[c];
        pc.by_build[n++] = 0;
    }
    pc.n = n;
    return pc;
}

template <int kMode, bool kDup>
static void launch_probe(phj_ctx * ctx, const ProbeArgs & a, const OutCols * o, uint32_t * heads, uint32_t * counts, uint64_t cap, bool lookup,
                         const char * name, uint64_t bytes)
{
    auto lk = k_probe_lookup<kMode, kDup>;
    if constexpr (kMode == kChj)
        if (a.win_hi != 0)
            lk = k_probe_lookup<kMode, kDup, true>;
    if (kMode != kChj && a.win_hi != 0)
        throw Error(PHJ_ERR_CUDA, "internal: sub-table windows are a CHJ probe form");
    // projection: plain (no repeated keys), range (grouped leaves) or flat
    // (chains expanded first)
    const int proj = !kDup ? 0 : (kMode != kChj && a.grouped) ? 1 : 2;
    bool wide = false; // a 16-byte payload column
    for (uint32_t c = 0; c < a.build.n; ++c)
        wide = wide || a.build.width[c] > 8;
    for (uint32_t c = 0; c < a.probe.n; ++c)
        wide = wide || a.probe.width[c] > 8;
    // packed build payloads: one gather per output row for all of them
    const bool packed = !lookup && proj == 0 && a.packed;
    bool wide_probe = false;
    for (uint32_t c = 0; c < a.probe.n; ++c)
        wide_probe = wide_probe || a.probe.width[c] > 8;
    int per_sm = 0;
    if (lookup)
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lk, kPNT, 0));
    else if (packed)
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wide_probe ? k_probe_project_packed<true> : k_probe_project_packed<false>,
                                                               kPNT, 0));
    else if (proj == 0)
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wide ? k_probe_project<kMode, true> : k_probe_project<kMode, false>, kPNT, 0));
    else
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_project_window<false>, kPNT, 0));
    const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>(ceil_div(std::max<uint64_t>(n_chunks, 1), kPWarps), (uint64_t)ctx->num_sms * (uint64_t)std::max(per_sm, 1)));
    if (std::getenv("PHJ_DEBUG"))
        std::fprintf(stderr, "[phj] %s: mode %d dup %d proj %d grid %u x %d threads, %d CTAs/SM, chunks %llu\n", name, kMode, (int)kDup, proj, grid,
                     kPNT, per_sm, (unsigned long long)n_chunks);
    // the first probe load reads an aligned pair of cells
    if ((kMode == kLeafUniform && a.uniform_log2cap < 1) || (reinterpret_cast<uintptr_t>(a.cells) & 31) != 0)
        throw Error(PHJ_ERR_CUDA, "internal: leaf tables need aligned pairs of cells");
    if (!lookup && proj == 2)
    {
        KTimer kt(ctx, "probe_expand", a.probe_rows, a.probe_rows * 8 + cap * 12);
        k_probe_expand<kMode><<<grid, kPNT, 0, ctx->stream>>>(a, heads, counts, cap);
        PHJ_LAUNCHED(ctx, "probe_expand");
    }
    KTimer kt(ctx, name, a.probe_rows, bytes);
    if (lookup)
        lk<<<grid, kPNT, 0, ctx->stream>>>(a, heads, counts);
    else if (packed)
    {
        // key column and probe payloads by column, build payloads packed
        ProjCols pc{};
        PackedCols bc{};
        const ProjCols all = proj_cols(a, *o);
        for (uint32_t j = 0; j < all.n; ++j)
            if (!all.by_build[j])
            {
                pc.src[pc.n] = all.src[j];
                pc.dst[pc.n] = all.dst[j];
                pc.width[pc.n] = all.width[j];
                pc.by_build[pc.n++] = 0;
            }
        for (uint32_t c = 0; c < a.build.n; ++c)
        {
            bc.dst[c] = o->left[c];
            bc.width[c] = (uint8_t)a.build.width[c];
            bc.off[c] = a.packed_off[c];
        }
        bc.n = a.build.n;
        if (wide_probe)
            k_probe_project_packed<true><<<grid, kPNT, 0, ctx->stream>>>(a, pc, bc, heads, counts, cap);
        else
            k_probe_project_packed<false><<<grid, kPNT, 0, ctx->stream>>>(a, pc, bc, heads, counts, cap);
    }
    else if (proj == 0 && wide)
        k_probe_project<kMode, true><<<grid, kPNT, 0, ctx->stream>>>(a, proj_cols(a, *o), heads, counts, cap);
    else if (proj == 0)
        k_probe_project<kMode, false><<<grid, kPNT, 0, ctx->stream>>>(a, proj_cols(a, *o), heads, counts, cap);
    else if (proj == 1)
        k_probe_project_window<false><<<grid, kPNT, 0, ctx->stream>>>(a, proj_cols(a, *o), heads, counts, cap);
    else
        k_probe_project_window<true><<<grid, kPNT, 0, ctx->stream>>>(a, proj_cols(a, *o), heads, counts, cap);
    PHJ_LAUNCHED(ctx, name);
}

template <int kMode>
static void launch_probe_mode(phj_ctx * ctx, const ProbeArgs & a, const OutCols * o, uint32_t * heads, uint32_t * counts, uint64_t cap, bool lookup,
                              const char * name, uint64_t bytes)
{
    if (a.any_dup)
        launch_probe<kMode, true>(ctx, a, o, heads, counts, cap, lookup, name, bytes);
    else
        launch_probe<kMode, false>(ctx, a, o, heads, counts, cap, lookup, name, bytes);
}

static void launch_any(phj_ctx * ctx, const ProbeArgs & a, const OutCols * o, uint32_t * heads, uint32_t * counts, uint64_t cap, bool lookup,
                       const char * name, uint64_t bytes)
{
    if (a.chj)
        launch_probe_mode<kChj>(ctx, a, o, heads, counts, cap, lookup, name, bytes);
    else if (a.uniform_log2cap >= 0)
        launch_probe_mode<kLeafUniform>(ctx, a, o, heads, counts, cap, lookup, name, bytes);
    else
        launch_probe_mode<kLeafMeta>(ctx, a, o, heads, counts, cap, lookup, name, bytes);
}

static uint64_t row_bytes_of(const Cols & c, bool with_key)
{
    uint64_t b = with_key ? 8 : 0;
    for (uint32_t i = 0; i < c.n; ++i)
        b += c.width[i];
    return b;
}

uint64_t probe_lookup(phj_ctx * ctx, Scratch & s, const ProbeArgs & a_in, uint32_t * heads, uint32_t * counts)
{
    const uint64_t n_chunks = ceil_div(a_in.probe_rows, kWChunk);
    ProbeArgs a = a_in;
    a.out_rows64 = s.get<unsigned long long>(1);
    PHJ_CUDA(cudaMemsetAsync(a.out_rows64, 0, sizeof(unsigned long long), ctx->stream));
    // algorithmic bytes: probe keys read, head array written
    launch_any(ctx, a, nullptr, heads, counts, 0, true, "probe_lookup", a.probe_rows * (8 + 4));
    scan_u32(ctx, s, counts, counts, n_chunks);
    unsigned long long total = 0;
    read_small(ctx, {{&total, a.out_rows64, sizeof(total)}});
    if (total >= (1ull << 32))
        throw Error(PHJ_ERR_CAPACITY, "the join has " + std::to_string(total) + " output rows; the device schemes place at most 2^32 - 1");
    return total;
}

// The packed layout of payload columns, when they pack: 2+ columns of 1-8
// bytes, 16 bytes in all.
static bool pack_spec_of(const Cols & payloads, PackSpec & pk)
{
    pk = PackSpec{};
    if (payloads.n < 2)
        return false;
    // widest column first, so every offset is a multiple of its width
    uint32_t order[kMaxCols];
    for (uint32_t c = 0; c < payloads.n; ++c)
        order[c] = c;
    std::stable_sort(order, order + payloads.n, [&](uint32_t x, uint32_t y) { return payloads.width[x] > payloads.width[y]; });
    uint32_t off = 0;
    for (uint32_t i = 0; i < payloads.n; ++i)
    {
        const uint32_t c = order[i];
        if (payloads.width[c] > 8)
            return false;
        pk.off[c] = (uint8_t)off;
        off += payloads.width[c];
    }
    if (off > 16)
        return false;
    pk.n = payloads.n;
    return true;
}

void pack_build_payloads(phj_ctx * ctx, Scratch & s, ProbeArgs & a, uint64_t build_rows)
{
    a.packed = nullptr;
    PackSpec pk;
    if (!ctx->pack_build || a.any_dup || build_rows == 0 || !pack_spec_of(a.build, pk))
        return;
    uint32_t bytes = 0;
    for (uint32_t c = 0; c < a.build.n; ++c)
        bytes += a.build.width[c];
    uint4 * p = s.get<uint4>(build_rows);
    {
        KTimer kt(ctx, "pack_build", build_rows, build_rows * (bytes + 16));
        // two CTAs per SM: the leaf-table build runs beside it
        k_pack_rows<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(build_rows, 256), (uint64_t)ctx->num_sms * 2)), 256, 0, ctx->stream>>>(
            a.build, build_rows, pk, p);
        PHJ_LAUNCHED(ctx, "pack_build");
    }
    for (uint32_t c = 0; c < a.build.n; ++c)
        a.packed_off[c] = pk.off[c];
    a.packed = p;
}

uint64_t probe_chunks(uint64_t probe_rows)
{
    return ceil_div(probe_rows, kWChunk);
}

void probe_project(phj_ctx * ctx, const ProbeArgs & a, phj_output * out, uint64_t out_base, const uint32_t * heads, const uint32_t * offs,
                   uint64_t rows)
{
    OutCols o{};
    o.keys = out->keys + out_base;
    for (uint32_t c = 0; c < out->left.n_payloads; ++c)
        o.left[c] = static_cast<uint8_t *>(out->lcol[c]) + out_base * payload_width(out->left.types[c]);
    for (uint32_t c = 0; c < out->right.n_payloads; ++c)
        o.right[c] = static_cast<uint8_t *>(out->rcol[c]) + out_base * payload_width(out->right.types[c]);
    // algorithmic bytes: the head array, the probe key and payloads of every
    // output row (read), the output rows (written)
    const uint64_t pr = row_bytes_of(a.probe, true), br = row_bytes_of(a.build, false);
    ProbeArgs b = a;
    const bool flat = a.any_dup && !(a.grouped && !a.chj);
    if (flat)
        b.flat = dalloc_n<uint32_t>(ctx, std::max<uint64_t>(rows, 1));
    try
    {
        launch_any(ctx, b, &o, const_cast<uint32_t *>(heads), const_cast<uint32_t *>(offs), rows, false, "probe_project",
                   a.probe_rows * 4 + rows * pr + rows * (8 + br + (pr - 8)));
    }
    catch (...)
    {
        dfree(ctx, b.flat);
        throw;
    }
    dfree(ctx, b.flat);
}

// Bytes the one-pass probe gathers a build row: 16 (packed payloads), 4 or
// 8 (one payload column of that width), 0 (no payload); -1: it does not
// apply.
static int fused_gather_bytes(const ProbeArgs & a)
{
    if (a.packed)
        return 16;
    if (a.build.n == 0)
        return 0;
    if (a.build.n == 1 && (a.build.width[0] == 4 || a.build.width[0] == 8))
        return (int)a.build.width[0];
    return -1;
}

// The fused probe: unique build keys whose payloads it gathers in one
// piece, no 16-byte probe payload column (its staged values would not fit
// the kernel's registers).
static bool probe_fused_eligible(const phj_ctx * ctx, const ProbeArgs & a)
{
    bool narrow = true;
    for (uint32_t c = 0; c < a.probe.n; ++c)
        narrow = narrow && a.probe.width[c] <= 8;
    return ctx->probe_fused && narrow && !a.any_dup && fused_gather_bytes(a) >= 0 && a.win_hi == 0 && a.probe_rows > 0 &&
           a.probe_rows < (1ull << 32);
}

// Unique build keys, packed build payloads: one pass that looks up and
// projects (k_probe_fused) into an output of one row per probe row.
static phj_output * probe_fused(phj_ctx * ctx, Scratch & s, const ProbeArgs & a, const phj_schema & left, const phj_schema & right)
{
    unsigned long long * counter = s.get<unsigned long long>(2); // output rows, chunk tickets
    PHJ_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned long long), ctx->stream));
    phj_output * out = new_output(ctx, left, right, a.probe_rows);
    try
    {
        OutCols o{};
        o.keys = out->keys;
        for (uint32_t c = 0; c < out->left.n_payloads; ++c)
            o.left[c] = out->lcol[c];
        for (uint32_t c = 0; c < out->right.n_payloads; ++c)
            o.right[c] = out->rcol[c];
        ProjCols pc{};
        for (uint32_t c = 0; c < a.probe.n; ++c)
        {
            pc.src[pc.n] = a.probe.col[c];
            pc.dst[pc.n] = o.right[c];
            pc.width[pc.n] = a.probe.width[c];
            pc.by_build[pc.n++] = 0;
        }
        const int gather = fused_gather_bytes(a);
        PackedCols bc{};
        for (uint32_t c = 0; c < a.build.n; ++c)
        {
            bc.dst[c] = o.left[c];
            bc.width[c] = (uint8_t)a.build.width[c];
            bc.off[c] = gather == 16 ? a.packed_off[c] : 0; // one unpacked column sits at byte 0 of its stage slot
        }
        bc.n = a.build.n;
        auto launch = [&](auto kernel) {
            int per_sm = 0;
            PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPNT, 0));
            const uint64_t n_chunks = ceil_div(a.probe_rows, kWChunk);
            const unsigned grid = (unsigned)std::max<uint64_t>(
                1, std::min<uint64_t>(ceil_div(n_chunks, kPWarps), (uint64_t)ctx->num_sms * (uint64_t)std::max(per_sm, 1)));
            if (std::getenv("PHJ_DEBUG"))
                std::fprintf(stderr, "[phj] probe_fused: grid %u x %d threads, %d CTAs/SM, chunks %llu\n", grid, kPNT, per_sm,
                             (unsigned long long)n_chunks);
            kernel<<<grid, kPNT, 0, ctx->stream>>>(a, pc, bc, o.keys, counter, counter + 1, a.probe_rows);
        };
        if ((a.uniform_log2cap >= 0 && a.uniform_log2cap < 1) || (reinterpret_cast<uintptr_t>(a.cells) & 31) != 0)
            throw Error(PHJ_ERR_CUDA, "internal: leaf tables need aligned pairs of cells");
        int rec = -1;
        {
            KTimer kt(ctx, "probe_fused", a.probe_rows, 0);
            rec = kt.idx;
            auto by_mode = [&](auto g) {
                constexpr int kG = decltype(g)::value;
                if (a.chj)
                    launch(k_probe_fused<kChj, kG>);
                else if (a.uniform_log2cap >= 0)
                    launch(k_probe_fused<kLeafUniform, kG>);
                else
                    launch(k_probe_fused<kLeafMeta, kG>);
            };
            switch (gather)
            {
                case 16: by_mode(std::integral_constant<int, 16>{}); break;
                case 8: by_mode(std::integral_constant<int, 8>{}); break;
                case 4: by_mode(std::integral_constant<int, 4>{}); break;
                default: by_mode(std::integral_constant<int, 0>{}); break;
            }
            PHJ_LAUNCHED(ctx, "probe_fused");
        }
        unsigned long long total = 0;
        read_small(ctx, {{&total, counter, sizeof(total)}});
        if (total > out->cap)
            throw Error(PHJ_ERR_CUDA, "internal: the one-pass probe counted more output rows than probe rows");
        out->rows = total;
        // algorithmic bytes: every probe row read, every output row written
        if (rec >= 0)
            ctx->records[rec].bytes = a.probe_rows * row_bytes_of(a.probe, true) + total * (8 + row_bytes_of(a.build, false) + row_bytes_of(a.probe, false));
    }
    catch (...)
    {
        free_output(ctx, out);
        throw;
    }
    return out;
}

phj_output * probe_join(phj_ctx * ctx, Scratch & s, const ProbeArgs & a_in, const phj_schema & left, const phj_schema & right)
{
    if (probe_fused_eligible(ctx, a_in))
        return probe_fused(ctx, s, a_in, left, right);
    ProbeArgs a = a_in;
    if ((a.grouped || a.any_dup) && !a.row_cnt)
        a.row_cnt = s.get<uint32_t>(std::max<uint64_t>(a.probe_rows, 1));
    uint32_t * heads = s.get<uint32_t>(a.probe_rows);
    uint32_t * counts = s.get<uint32_t>(probe_chunks(a.probe_rows) + 1);
    const uint64_t total = probe_lookup(ctx, s, a, heads, counts);
    phj_output * out = new_output(ctx, left, right, total);
    out->rows = total;
    try
    {
        probe_project(ctx, a, out, 0, heads, counts, total);
    }
    catch (...)
    {
        free_output(ctx, out);
        throw;
    }
    return out;
}

} // namespace phjg
