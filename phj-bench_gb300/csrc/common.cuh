// common.cuh -- device primitives shared by every kernel of the GB300 join
// path: the join hash, the 16-byte (key, RowRefCell) cell with 128-bit CAS,
// column descriptors, and small block-wide helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace phjg
{

// ---------------------------------------------------------------------------
// intHash64 (src/Hash.h:18-25): salt xor, then the Murmur3 fmix64 finaliser.
// The constants define the function, so they are necessarily the same.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t int_hash64(uint64_t x)
{
    x ^= 0x4cf5ad432745937fULL;
    x = (x ^ (x >> 33)) * 0xff51afd7ed558ccdULL;
    x = (x ^ (x >> 33)) * 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

// RowRefCell (src/Types.h:95-104) packed in one u64: block_no in the low
// word, row_no in the high word, i.e. the little-endian image of the struct.
constexpr uint32_t INVALID_BLOCK = 0xFFFFFFFFu;
constexpr uint64_t INVALID_REF = 0x00000000FFFFFFFFull; // {INVALID_BLOCK, 0}

__host__ __device__ __forceinline__ uint64_t make_ref(uint32_t block_no, uint32_t row_no)
{
    return (uint64_t)block_no | ((uint64_t)row_no << 32);
}
__host__ __device__ __forceinline__ uint32_t ref_block(uint64_t r) { return (uint32_t)r; }
__host__ __device__ __forceinline__ uint32_t ref_row(uint64_t r) { return (uint32_t)(r >> 32); }
__host__ __device__ __forceinline__ bool ref_valid(uint64_t r) { return (uint32_t)r != INVALID_BLOCK; }

// JoinHashTable::Cell (src/HashTable.h:33-38): {u64 key; RowRefCell ref}.
// Empty cell = {0, INVALID_REF} (src/HashTable.h:150), so key 0 stays legal.
struct __align__(16) Cell
{
    uint64_t key;
    uint64_t ref;
};

// 128-bit compare-and-swap on a cell (PTX atom.cas.b128, sm_90+).  Returns
// the cell's previous contents as one atomic snapshot.
__device__ __forceinline__ Cell cas_cell_global(Cell *p, Cell cmp, Cell val)
{
    Cell old;
    asm volatile(
        "{\n\t.reg .b128 c, v, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 v, {%4, %5};\n\t"
        "atom.global.cas.b128 o, [%6], c, v;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(old.key), "=l"(old.ref)
        : "l"(cmp.key), "l"(cmp.ref), "l"(val.key), "l"(val.ref), "l"(p)
        : "memory");
    return old;
}

__device__ __forceinline__ Cell cas_cell_shared(Cell *p, Cell cmp, Cell val)
{
    Cell old;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile(
        "{\n\t.reg .b128 c, v, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 v, {%4, %5};\n\t"
        "atom.shared.cas.b128 o, [%6], c, v;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(old.key), "=l"(old.ref)
        : "l"(cmp.key), "l"(cmp.ref), "l"(val.key), "l"(val.ref), "r"(a)
        : "memory");
    return old;
}

// Linear probing starts at the even cell of the hash's pair, so that the
// first two probe positions share one aligned 32-byte sector and arrive
// with one load.
__host__ __device__ __forceinline__ uint64_t probe_start(uint64_t hash, uint64_t cap)
{
    return hash & (cap - 1) & ~1ull;
}

// Insert (key, ref) into an open-addressing table of `cap` (power of two)
// cells with linear probing from probe_start(hash) (src/HashTable.h:84-109
// probes from hash & (cap-1); starting at the pair's even cell changes no
// lookup result).
// Returns the previous head ref for `key` (INVALID_REF when new), which the
// caller threads into the next-chain.  Concurrent inserters are safe: an
// empty cell is claimed with one 128-bit CAS; a cell that already holds the
// key gets its ref half swapped with a 64-bit exchange.  A claimed cell's
// key never changes, so the CAS snapshot decides every step.  The loop is
// bounded by `cap` steps (a table is never full: load <= 1/2).
template <bool kShared>
__device__ __forceinline__ uint64_t table_insert(Cell *cells, uint64_t cap, uint64_t hash, uint64_t key, uint64_t ref)
{
    const uint64_t mask = cap - 1;
    uint64_t pos = probe_start(hash, cap);
    const Cell empty{0ull, INVALID_REF};
    const Cell mine{key, ref};
    for (uint64_t step = 0; step < cap; ++step)
    {
        Cell *c = cells + pos;
        const Cell old = kShared ? cas_cell_shared(c, empty, mine) : cas_cell_global(c, empty, mine);
        if (old.key == 0ull && old.ref == INVALID_REF)
            return INVALID_REF;
        if (old.key == key)
            return (uint64_t)atomicExch((unsigned long long *)&c->ref, (unsigned long long)ref);
        pos = (pos + 1) & mask;
    }
    return INVALID_REF; // unreachable for tables at <= 50% load
}

// Lookup after the build barrier (src/HashTable.h:112-127): plain loads.
__device__ __forceinline__ uint64_t table_find(const Cell *cells, uint64_t cap, uint64_t hash, uint64_t key)
{
    if (cap == 0)
        return INVALID_REF;
    const uint64_t mask = cap - 1;
    uint64_t pos = probe_start(hash, cap);
    for (uint64_t step = 0; step < cap; ++step)
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

// The two cells of an aligned pair with one 256-bit load (cap >= 2): through
// the read-only path, or through L2 when the table may still be written
// (coherent).
struct CellPair
{
    ulonglong2 a, b;
};
template <bool kCoherent>
__device__ __forceinline__ CellPair load_pair(const Cell *p)
{
    CellPair r;
    if (kCoherent)
        asm volatile("ld.global.cg.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(r.a.x), "=l"(r.a.y), "=l"(r.b.x), "=l"(r.b.y) : "l"(p) : "memory");
    else
        asm("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(r.a.x), "=l"(r.a.y), "=l"(r.b.x), "=l"(r.b.y) : "l"(p));
    return r;
}

// ---------------------------------------------------------------------------
// Column descriptors.  A side (build or probe) is a key column plus up to
// kMaxCols payload columns of width 1/2/4/8/16 bytes, all column-major.
// ---------------------------------------------------------------------------
constexpr int kMaxCols = 8;

struct Cols
{
    uint64_t *keys;
    void *col[kMaxCols];
    uint8_t width[kMaxCols];
    uint32_t n;
};

// Build payload columns packed row-major into 16 bytes: column c at byte
// off[c] (widest first, so each offset is a multiple of its width; unused
// bytes zero).
struct PackSpec
{
    uint8_t off[kMaxCols];
    uint32_t n;
};

// Row r of the payload columns `in`, packed.
__device__ __forceinline__ uint4 pack_row(const Cols &in, uint64_t r, const PackSpec &pk)
{
    uint64_t h[2] = {0, 0};
    for (uint32_t c = 0; c < in.n; ++c)
    {
        uint64_t v;
        switch (in.width[c])
        {
            case 1: v = static_cast<const uint8_t *>(in.col[c])[r]; break;
            case 2: v = static_cast<const uint16_t *>(in.col[c])[r]; break;
            case 4: v = static_cast<const uint32_t *>(in.col[c])[r]; break;
            default: v = static_cast<const uint64_t *>(in.col[c])[r]; break;
        }
        h[pk.off[c] >> 3] |= v << ((pk.off[c] & 7u) * 8u);
    }
    return make_uint4((uint32_t)h[0], (uint32_t)(h[0] >> 32), (uint32_t)h[1], (uint32_t)(h[1] >> 32));
}

// Copy element `src_i` of a column to element `dst_i` of another column of
// the same width.
__device__ __forceinline__ void copy_elem(void *dst, uint64_t dst_i, const void *src, uint64_t src_i, uint32_t w)
{
    switch (w)
    {
        case 1: static_cast<uint8_t *>(dst)[dst_i] = static_cast<const uint8_t *>(src)[src_i]; break;
        case 2: static_cast<uint16_t *>(dst)[dst_i] = static_cast<const uint16_t *>(src)[src_i]; break;
        case 4: static_cast<uint32_t *>(dst)[dst_i] = static_cast<const uint32_t *>(src)[src_i]; break;
        case 8: static_cast<uint64_t *>(dst)[dst_i] = static_cast<const uint64_t *>(src)[src_i]; break;
        default: static_cast<uint4 *>(dst)[dst_i] = static_cast<const uint4 *>(src)[src_i]; break;
    }
}

// ---------------------------------------------------------------------------
// Block-wide exclusive scan of one u32 per thread (NT threads, NT % 32 == 0).
// `warp_sums` must hold NT/32 entries of shared memory.  Returns the
// exclusive prefix; *total gets the block sum.
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *warp_sums, uint32_t *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t s = lane < NT / 32 ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o)
                s += y;
        }
        if (lane < NT / 32)
            warp_sums[lane] = s; // inclusive warp prefix
    }
    __syncthreads();
    const uint32_t warp_base = warp == 0 ? 0u : warp_sums[warp - 1];
    *total = warp_sums[NT / 32 - 1];
    const uint32_t excl = warp_base + x - v;
    __syncthreads(); // warp_sums may be reused by the caller
    return excl;
}

__host__ __device__ __forceinline__ uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

__host__ __device__ __forceinline__ uint64_t bit_ceil64(uint64_t x)
{
    if (x <= 1)
        return 1;
    uint64_t p = 1;
    while (p < x)
        p <<= 1;
    return p;
}

} // namespace phjg

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (cp.async.bulk, the TMA engine's 1-D form) into
// shared memory, completed through an mbarrier.  Every wait is bounded: after
// kWaitLimit polls it records `code` in the kernel's error word and gives up,
// so a stuck copy surfaces as PHJ_ERR_DEVICE_TIMEOUT on the host instead of
// a hung GPU.
// ---------------------------------------------------------------------------
namespace phjg
{
constexpr uint32_t kWaitLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void * p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t * bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation visible to the async (bulk copy) proxy.
__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy ones (a bulk copy refilling a buffer threads just read).
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t * bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Global -> shared bulk copy; dst, src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_copy_g2s(void * dst, const void * src, uint32_t bytes, uint64_t * bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// An L2 cache policy that evicts the lines it touches first: for data read
// once (streamed probe rows), so it does not push out tables still in use.
__device__ __forceinline__ uint64_t l2_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// 8-byte asynchronous copy from global to shared memory (cp.async: no
// register waits for the value) under the L2 cache policy `pol`; dst and
// src 8-byte aligned.  A thread's copies are complete after its
// cp_async_wait_all.
__device__ __forceinline__ void cp_async8(void * dst, const void * src, uint64_t pol)
{
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src), "l"(pol) : "memory");
}

// 4- or 8-byte asynchronous copy from global to shared memory; dst and src
// aligned to the size.
template <int kBytes>
__device__ __forceinline__ void cp_async_small(void * dst, const void * src)
{
    static_assert(kBytes == 4 || kBytes == 8, "cp.async.ca copies 4, 8 or 16 bytes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"(kBytes) : "memory");
}

// 16-byte asynchronous copy from global to shared memory through L2 only;
// dst and src 16-byte aligned.
__device__ __forceinline__ void cp_async16(void * dst, const void * src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// A shared-memory read the compiler may not fold into an earlier value held
// in a register.
__device__ __forceinline__ uint64_t ld_shared_u64(const uint64_t * p)
{
    uint64_t v;
    asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}

// Bulk prefetch of [src, src + bytes) into L2 by the TMA engine (no
// registers, no shared memory); src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_prefetch_l2(const void * src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test_parity(uint64_t * bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of `bar` to complete; false (and *err = code) on
// timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t * bar, uint32_t parity, int * err, int code)
{
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_test_parity(bar, parity))
            return true;
    atomicExch(err, code);
    return false;
}
} // namespace phjg
