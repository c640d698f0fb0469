// bep.cu -- lazy leaf tables of the PHJ (BEP) scheme: each leaf table is
// built the first time a probe batch needs it.
//
// Per batch, before its lookups: the batch's first radix pass (its
// histogram kernel) flags the leaves the probe keys touch in a bitmap;
// k_bep_collect counts each touched leaf as one eviction (its buffered rows are probed in this batch) and queues
// the touched leaves that are not yet built.  k_bep_build is a persistent
// grid whose CTAs take leaves from that queue: a CTA wins NOT_BUILT ->
// BUILDING with a CAS, builds the table in shared memory with 128-bit CAS
// inserts, threads the next-chain and publishes BUILT; a CTA that finds a
// leaf BUILDING waits for it, bounded by a wall-clock limit, then gives up
// with an error code.  The lookups that follow read only BUILT tables, from
// a later kernel.
#include "internal.h"

namespace phjg
{
namespace
{
constexpr uint32_t kNotBuilt = 0, kBuilding = 1, kBuilt = 2, kBuiltDup = 3;
constexpr int kBepNT = 256;
constexpr uint32_t kBepSmemCellsMax = 8192; // 128 KiB of cells per CTA

__device__ __forceinline__ uint32_t load_acquire(const uint32_t * p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One pass over the leaves, a warp per bitmap word: each touched leaf is one
// eviction (its buffered rows are probed in this batch); touched leaves not
// yet built are queued.  The word is cleared for the next batch.
__global__ void k_bep_collect(BepLeaves b)
{
    const uint32_t L = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t word = 0;
    if (lane == 0 && L < b.n_leaves)
    {
        word = b.touched[L >> 5];
        b.touched[L >> 5] = 0;
    }
    word = __shfl_sync(0xffffffffu, word, 0);
    const bool t = L < b.n_leaves && (word >> lane & 1u);
    const bool q = t && b.state[L] < kBuilt;
    const uint32_t tm = __ballot_sync(0xffffffffu, t), qm = __ballot_sync(0xffffffffu, q);
    uint32_t base = 0;
    if (lane == 0)
    {
        if (tm)
            atomicAdd(b.ctr + 2, (unsigned long long)__popc(tm));
        if (qm)
            base = atomicAdd(b.queue_len, (uint32_t)__popc(qm));
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    if (q)
        b.queue[base + __popc(qm & ((1u << lane) - 1u))] = L;
}

// A CTA per queued leaf: it wins NOT_BUILT -> BUILDING, builds the table in
// shared memory (or in place when it is larger than `smem_cells`), copies it
// out, threads the next-chain and publishes BUILT; or it finds the leaf
// BUILDING and waits for it (bounded).
// Leaves a CTA claims from the queue at once: their NOT_BUILT -> BUILDING
// CASes and, after the builds, their BUILT stores run in parallel, so the
// per-leaf cost is the build itself rather than a chain of global round
// trips.
constexpr uint32_t kClaim = 8;

__global__ void __launch_bounds__(kBepNT) k_bep_build(BepLeaves b, int * __restrict__ err)
{
    extern __shared__ __align__(16) Cell sh_cells[];
    __shared__ uint32_t s_leaf[kClaim], s_won[kClaim], s_dup[kClaim];
    __shared__ uint32_t s_n, s_stop;
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            const uint32_t base = atomicAdd(b.queue_len + 1, kClaim);
            const uint32_t qlen = *reinterpret_cast<volatile uint32_t *>(b.queue_len);
            s_n = base < qlen ? min(kClaim, qlen - base) : 0u;
            s_stop = 0;
            s_leaf[0] = base; // read below by the claiming threads
        }
        __syncthreads();
        const uint32_t n = s_n;
        if (n == 0)
            return;
        const uint32_t base = s_leaf[0];
        __syncthreads();
        if (threadIdx.x < n)
        {
            const uint32_t L = b.queue[base + threadIdx.x];
            s_leaf[threadIdx.x] = L;
            s_won[threadIdx.x] = atomicCAS(b.state + L, kNotBuilt, kBuilding) == kNotBuilt;
            s_dup[threadIdx.x] = 0;
        }
        __syncthreads();
        for (uint32_t i = 0; i < n; ++i)
        {
            const uint32_t L = s_leaf[i];
            if (s_won[i])
            {
                const LeafMeta m = b.meta[L];
                bool dup = false;
                if (m.has_table)
                {
                    const uint64_t cap = 1ull << m.log2cap;
                    const bool in_smem = cap <= b.smem_cells;
                    Cell * tab = in_smem ? sh_cells : b.cells + m.table_off;
                    for (uint64_t j = threadIdx.x; j < cap; j += kBepNT)
                        reinterpret_cast<ulonglong2 *>(tab)[j] = make_ulonglong2(0ull, INVALID_REF);
                    __syncthreads();
                    const uint32_t r0 = m.row_off, r1 = b.leaf_off[L + 1];
                    for (uint32_t r = r0 + threadIdx.x; r < r1; r += kBepNT)
                    {
                        const uint64_t k = b.build_keys[r];
                        const uint64_t h = int_hash64(k);
                        const uint64_t prev =
                            in_smem ? table_insert<true>(tab, cap, h, k, make_ref(0, r)) : table_insert<false>(tab, cap, h, k, make_ref(0, r));
                        b.next[r] = prev;
                        dup |= ref_valid(prev);
                    }
                    dup = __syncthreads_or(dup);
                    if (in_smem)
                        for (uint64_t j = threadIdx.x; j < cap; j += kBepNT)
                            reinterpret_cast<ulonglong2 *>(b.cells + m.table_off)[j] = reinterpret_cast<const ulonglong2 *>(sh_cells)[j];
                }
                if (threadIdx.x == 0)
                    s_dup[i] = dup;
                __syncthreads(); // the shared table is reused by the next leaf
            }
            else if (threadIdx.x == 0 && load_acquire(b.state + L) < kBuilt)
            {
                atomicAdd(b.ctr + 1, 1ull);
                const uint64_t t0 = global_ns();
                uint32_t spins = 0;
                while (load_acquire(b.state + L) < kBuilt)
                    if (++spins >= kWaitLimit || global_ns() - t0 > b.wait_limit_ns)
                    {
                        atomicExch(err, 4);
                        s_stop = 1;
                        break;
                    }
            }
        }
        __syncthreads();
        // the tables are read by the lookups of a later kernel, so BUILT
        // needs no fence for them; it only releases waiters
        if (threadIdx.x < n && s_won[threadIdx.x])
        {
            const uint32_t L = s_leaf[threadIdx.x];
            const bool dup = s_dup[threadIdx.x] != 0;
            b.meta[L].dup = dup ? 1 : 0;
            atomicExch(b.state + L, dup ? kBuiltDup : kBuilt);
            atomicAdd(b.ctr + 0, 1ull);
            if (dup)
                atomicExch(b.any_dup, 1);
        }
        __syncthreads();
        if (s_stop)
            return;
    }
}
} // namespace

void set_bep_smem_limits(int smem_optin)
{
    PHJ_CUDA(cudaFuncSetAttribute(k_bep_build, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::min<size_t>((size_t)kBepSmemCellsMax * sizeof(Cell), (size_t)smem_optin - 1024)));
}

bool bep_build_touched(phj_ctx * ctx, const BepLeaves & b)
{
    PHJ_CUDA(cudaMemsetAsync(b.queue_len, 0, 2 * sizeof(uint32_t), ctx->stream));
    k_bep_collect<<<(unsigned)ceil_div(b.n_leaves, kBepNT), kBepNT, 0, ctx->stream>>>(b);
    PHJ_LAUNCHED(ctx, "bep_collect");
    {
        KTimer kt(ctx, "bep_build", 0, 0);
        int per_sm = 0;
        PHJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bep_build, kBepNT, (size_t)b.smem_cells * sizeof(Cell)));
        k_bep_build<<<(unsigned)(ctx->num_sms * std::max(per_sm, 1)), kBepNT, (size_t)b.smem_cells * sizeof(Cell), ctx->stream>>>(b, ctx->d_err);
        PHJ_LAUNCHED(ctx, "bep_build");
    }
    int dup = 0;
    read_small(ctx, {{&dup, b.any_dup, sizeof(int)}});
    return dup != 0;
}
} // namespace phjg
