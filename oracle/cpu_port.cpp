// cpu_port.cpp -- C++ restatement of the reference's CPU CHJ, PHJ-PURE and
// PHJ (BEP) schemes, timed as the CPU baseline where the reference cannot be
// compiled.  Test and measurement infrastructure only, never on the device
// path.  See cpu_port.h for the reference file:line map.
#include "cpu_port.h"
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <bit>
#include <chrono>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace
{
using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// intHash64, src/Hash.h:18-25
inline uint64_t int_hash64(uint64_t x)
{
    x ^= 0x4cf5ad432745937fULL;
    x = (x ^ (x >> 33)) * 0xff51afd7ed558ccdULL;
    x = (x ^ (x >> 33)) * 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

uint32_t width_of(uint8_t t)
{
    static const uint32_t w[5] = {1, 2, 4, 8, 16};
    return t < 5 ? w[t] : 0;
}

template <class F>
void run_threads(uint32_t threads, F && fn)
{
    if (threads <= 1)
    {
        fn(0u);
        return;
    }
    std::vector<std::thread> tv;
    for (uint32_t t = 0; t < threads; ++t)
        tv.emplace_back([t, &fn] { fn(t); });
    for (auto & th : tv)
        th.join();
}

struct Schema
{
    std::vector<uint32_t> w;
    size_t initial_rows() const // initialOutBlockRows: ~4 KiB of the widest column
    {
        size_t m = 8;
        for (uint32_t x : w)
            m = std::max<size_t>(m, x);
        return std::max<size_t>(1, 4096 / m);
    }
};

// A batch of rows: key column plus payload columns (BlockView).
struct View
{
    size_t rows = 0;
    const uint64_t * keys = nullptr;
    const uint8_t * cols[8] = {};
};

// OutBlock, src/RadixPartition.h:44-109
struct OutBlk
{
    size_t rows = 0, cap = 0;
    std::vector<uint64_t> keys;
    std::vector<std::vector<uint8_t>> cols;
    View view() const
    {
        View v;
        v.rows = rows;
        v.keys = keys.data();
        for (size_t c = 0; c < cols.size(); ++c)
            v.cols[c] = cols[c].data();
        return v;
    }
};

// PartitionOut, src/RadixPartition.h:229-317: growable chain, doubling
// capacity from ~4 KiB up to 65,536 rows.
struct Chain
{
    std::vector<OutBlk> blocks;
    size_t next_cap = 0;
    bool has_cur = false;
    void grow(const Schema & s, size_t min_required)
    {
        const size_t cap = std::max(next_cap, min_required);
        OutBlk b;
        b.cap = cap;
        b.keys.assign(cap, 0);
        b.cols.resize(s.w.size());
        for (size_t c = 0; c < s.w.size(); ++c)
            b.cols[c].assign(cap * s.w[c], 0);
        blocks.push_back(std::move(b));
        has_cur = true;
        next_cap = std::min<size_t>(cap * 2, 65536);
    }
};

struct Scratch
{
    std::vector<uint64_t> hashes;
    std::vector<uint32_t> pids, hist;
    std::vector<uint64_t *> key_ptrs;
    std::vector<uint8_t *> ptrs; // [col * parts + p]
};

// scatterBatch, src/RadixPartition.cpp:316-393: hash -> pid, histogram,
// pre-grow, column-first branch-free scatter.
void scatter_batch(const View & in, const Schema & s, uint32_t shift, size_t parts, Chain * out, Scratch & sc)
{
    const size_t n = in.rows;
    if (n == 0)
        return;
    const size_t K = s.w.size();
    const uint64_t mask = parts - 1;
    if (sc.hashes.size() < n)
        sc.hashes.resize(n), sc.pids.resize(n);
    sc.hist.assign(parts, 0);
    if (sc.key_ptrs.size() < parts)
        sc.key_ptrs.resize(parts);
    if (sc.ptrs.size() < K * parts)
        sc.ptrs.resize(K * parts);
    for (size_t j = 0; j < n; ++j)
        sc.hashes[j] = int_hash64(in.keys[j]);
    for (size_t j = 0; j < n; ++j)
        sc.pids[j] = (uint32_t)((sc.hashes[j] >> shift) & mask);
    for (size_t j = 0; j < n; ++j)
        ++sc.hist[sc.pids[j]];
    for (size_t p = 0; p < parts; ++p)
    {
        if (!sc.hist[p])
            continue;
        Chain & ch = out[p];
        if (!ch.has_cur || ch.blocks.back().rows + sc.hist[p] > ch.blocks.back().cap)
            ch.grow(s, sc.hist[p]);
        OutBlk & ob = ch.blocks.back();
        const size_t base = ob.rows;
        ob.rows += sc.hist[p];
        sc.key_ptrs[p] = ob.keys.data() + base;
        for (size_t c = 0; c < K; ++c)
            sc.ptrs[c * parts + p] = ob.cols[c].data() + base * s.w[c];
    }
    for (size_t j = 0; j < n; ++j)
        *sc.key_ptrs[sc.pids[j]]++ = in.keys[j];
    for (size_t c = 0; c < K; ++c)
    {
        const uint32_t w = s.w[c];
        uint8_t ** cp = sc.ptrs.data() + c * parts;
        const uint8_t * src = in.cols[c];
        for (size_t j = 0; j < n; ++j)
        {
            uint8_t *& d = cp[sc.pids[j]];
            std::memcpy(d, src + j * w, w);
            d += w;
        }
    }
}

using Partitions = std::vector<std::vector<OutBlk>>;

Partitions collect(std::vector<std::vector<Chain>> & shards, size_t parts)
{
    Partitions out(parts);
    for (size_t p = 0; p < parts; ++p)
        for (auto & sh : shards)
            for (auto & b : sh[p].blocks)
                if (b.rows)
                    out[p].push_back(std::move(b));
    return out;
}

// radixShuffle, src/RadixPartition.cpp:546-577
Partitions radix_shuffle(const port_stream & st, const Schema & s, const std::vector<uint32_t> & bits, uint32_t threads)
{
    const size_t block_rows = st.block_rows ? st.block_rows : 10000;
    const size_t n_blocks = (st.rows + block_rows - 1) / block_rows;
    uint32_t consumed = bits[0];
    size_t parts = size_t{1} << bits[0];
    std::vector<std::vector<Chain>> shards(threads, std::vector<Chain>(parts));
    for (auto & sh : shards)
        for (auto & c : sh)
            c.next_cap = s.initial_rows();
    run_threads(threads, [&](uint32_t tid) {
        Scratch sc;
        const size_t b0 = n_blocks * tid / threads, b1 = n_blocks * (tid + 1) / threads;
        for (size_t b = b0; b < b1; ++b)
        {
            View v;
            const size_t r0 = b * block_rows;
            v.rows = std::min(block_rows, st.rows - r0);
            v.keys = st.keys + r0;
            for (size_t c = 0; c < s.w.size(); ++c)
                v.cols[c] = static_cast<const uint8_t *>(st.cols[c]) + r0 * s.w[c];
            scatter_batch(v, s, 64u - bits[0], parts, shards[tid].data(), sc);
        }
    });
    Partitions cur = collect(shards, parts);
    for (size_t pass = 1; pass < bits.size(); ++pass)
    {
        const size_t sub = size_t{1} << bits[pass];
        const uint32_t shift = 64u - consumed - bits[pass];
        const size_t out_parts = parts * sub;
        std::vector<std::vector<Chain>> sh2(threads, std::vector<Chain>(out_parts));
        for (auto & sh : sh2)
            for (auto & c : sh)
                c.next_cap = s.initial_rows();
        run_threads(threads, [&](uint32_t tid) {
            Scratch sc;
            for (size_t ip = tid; ip < parts; ip += threads)
                for (const OutBlk & ob : cur[ip])
                    scatter_batch(ob.view(), s, shift, sub, sh2[tid].data() + ip * sub, sc);
        });
        cur = collect(sh2, out_parts);
        parts = out_parts;
        consumed += bits[pass];
    }
    return cur;
}

// JoinHashTable, src/HashTable.h:27-166
struct Ref
{
    uint32_t block = 0xFFFFFFFFu, row = 0;
    bool valid() const { return block != 0xFFFFFFFFu; }
};
struct Cell
{
    uint64_t key;
    Ref ref;
};
struct Table
{
    std::vector<Cell> cells;
    size_t n = 0;
    void ensure(size_t cap)
    {
        if (cap <= cells.size())
            return;
        std::vector<Cell> old = std::move(cells);
        cells.assign(cap, Cell{0, Ref{}});
        n = 0;
        for (const Cell & c : old)
            if (c.ref.valid())
            {
                size_t pos = int_hash64(c.key) & (cap - 1);
                while (cells[pos].ref.valid())
                    pos = (pos + 1) & (cap - 1);
                cells[pos] = c;
                ++n;
            }
    }
    void reserve(size_t rows) { ensure(std::bit_ceil(rows * 2)); }
    Ref insert(uint64_t h, uint64_t k, Ref r)
    {
        if (n * 2 >= cells.size())
            ensure(cells.empty() ? 128 * 1024 : cells.size() * 2);
        const size_t mask = cells.size() - 1;
        for (size_t pos = h & mask;; pos = (pos + 1) & mask)
        {
            Cell & c = cells[pos];
            if (!c.ref.valid())
            {
                c.key = k;
                c.ref = r;
                ++n;
                return Ref{};
            }
            if (c.key == k)
            {
                const Ref prev = c.ref;
                c.ref = r;
                return prev;
            }
        }
    }
    Ref find(uint64_t h, uint64_t k) const
    {
        if (cells.empty())
            return Ref{};
        const size_t mask = cells.size() - 1;
        for (size_t pos = h & mask;; pos = (pos + 1) & mask)
        {
            const Cell & c = cells[pos];
            if (!c.ref.valid())
                return Ref{};
            if (c.key == k)
                return c.ref;
        }
    }
};

// BlockStore, src/BlockStore.h:34-95
struct Store
{
    std::vector<View> blocks;
    std::vector<std::vector<Ref>> next;
    uint32_t append(const View & v)
    {
        blocks.push_back(v);
        next.emplace_back(v.rows, Ref{});
        return (uint32_t)(blocks.size() - 1);
    }
};

// OutputBlock + ProbeMaterialiser, src/JoinOutput.h:18-42, src/JoinOps.h:52-196
struct OutputBlock
{
    size_t rows = 0;
    std::vector<uint64_t> keys;
    std::vector<std::vector<uint8_t>> left, right;
};

struct Materialiser
{
    const Schema *ls, *rs;
    std::vector<OutputBlock> done;
    OutputBlock cur;
    bool have = false;
    uint64_t total = 0;
    void ensure()
    {
        if (have)
            return;
        cur = OutputBlock{};
        cur.keys.assign(10000, 0);
        cur.left.resize(ls->w.size());
        for (size_t c = 0; c < ls->w.size(); ++c)
            cur.left[c].assign(10000 * ls->w[c], 0);
        cur.right.resize(rs->w.size());
        for (size_t c = 0; c < rs->w.size(); ++c)
            cur.right[c].assign(10000 * rs->w[c], 0);
        have = true;
    }
    void gather(const View & probe, const Store & st, const size_t * pidx, const Ref * bref, size_t m)
    {
        size_t done_rows = 0;
        while (done_rows < m)
        {
            ensure();
            const size_t take = std::min(m - done_rows, 10000 - cur.rows);
            for (size_t k = 0; k < take; ++k)
                cur.keys[cur.rows + k] = probe.keys[pidx[done_rows + k]];
            for (size_t c = 0; c < ls->w.size(); ++c)
            {
                const uint32_t w = ls->w[c];
                uint8_t * dst = cur.left[c].data() + cur.rows * w;
                for (size_t k = 0; k < take; ++k)
                {
                    const Ref r = bref[done_rows + k];
                    std::memcpy(dst + k * w, st.blocks[r.block].cols[c] + (size_t)r.row * w, w);
                }
            }
            for (size_t c = 0; c < rs->w.size(); ++c)
            {
                const uint32_t w = rs->w[c];
                uint8_t * dst = cur.right[c].data() + cur.rows * w;
                for (size_t k = 0; k < take; ++k)
                    std::memcpy(dst + k * w, probe.cols[c] + pidx[done_rows + k] * w, w);
            }
            cur.rows += take;
            done_rows += take;
            total += take;
            if (cur.rows == 10000)
            {
                done.push_back(std::move(cur));
                have = false;
            }
        }
    }
    void finish()
    {
        if (have && cur.rows)
            done.push_back(std::move(cur));
        have = false;
    }
};

struct ProbeScratch
{
    std::vector<uint64_t> hashes;
    std::vector<Ref> heads;
    std::vector<size_t> pidx;
    std::vector<Ref> bref;
};

// probeOneBlock, src/JoinOps.h:236-272
void probe_block(const View & v, const Store & st, const Table & ht, Materialiser & mat, ProbeScratch & ps)
{
    if (!v.rows)
        return;
    ps.hashes.resize(v.rows);
    ps.heads.resize(v.rows);
    for (size_t i = 0; i < v.rows; ++i)
        ps.hashes[i] = int_hash64(v.keys[i]);
    for (size_t i = 0; i < v.rows; ++i)
        ps.heads[i] = ht.find(ps.hashes[i], v.keys[i]);
    ps.pidx.clear();
    ps.bref.clear();
    for (size_t i = 0; i < v.rows; ++i)
        for (Ref r = ps.heads[i]; r.valid(); r = st.next[r.block][r.row])
        {
            ps.pidx.push_back(i);
            ps.bref.push_back(r);
        }
    mat.gather(v, st, ps.pidx.data(), ps.bref.data(), ps.pidx.size());
}

// buildOneBlock, src/JoinOps.h:205-228
void build_block(const View & v, Store & st, Table & ht, std::vector<uint64_t> & hashes)
{
    if (!v.rows)
        return;
    hashes.resize(v.rows);
    for (size_t i = 0; i < v.rows; ++i)
        hashes[i] = int_hash64(v.keys[i]);
    const uint32_t b = st.append(v);
    for (size_t i = 0; i < v.rows; ++i)
        st.next[b][i] = ht.insert(hashes[i], v.keys[i], Ref{b, (uint32_t)i});
}

Schema schema_of(const port_stream & s)
{
    Schema sc;
    for (uint32_t c = 0; c < s.n_payloads; ++c)
        sc.w.push_back(width_of(s.types[c]));
    return sc;
}

// The order-independent fingerprint of every materialised output row (the
// oracle's, oracle_columns_fingerprint: row count and two sums of per-row
// hashes), taken after the timed region so the check costs the timing
// nothing.
void fingerprint_outputs(const std::vector<Materialiser> & mats, const port_stream & b, const port_stream & p, uint64_t * fp)
{
    if (!fp)
        return;
    fp[0] = fp[1] = fp[2] = 0;
    for (const Materialiser & m : mats)
        for (const OutputBlock & blk : m.done)
        {
            const void * l[8] = {};
            const void * r[8] = {};
            for (size_t c = 0; c < blk.left.size(); ++c)
                l[c] = blk.left[c].data();
            for (size_t c = 0; c < blk.right.size(); ++c)
                r[c] = blk.right[c].data();
            uint64_t f[3];
            oracle_columns_fingerprint(blk.rows, blk.keys.data(), b.n_payloads, b.types, l, p.n_payloads, p.types, r, f);
            fp[0] += f[0];
            fp[1] += f[1];
            fp[2] += f[2];
        }
}
} // namespace

extern "C" int64_t port_run_phj_pure(const port_stream * build, const port_stream * probe, const uint8_t * pass_bits, uint32_t n_passes,
                                     uint32_t threads, double * phase_ms, uint64_t * fp)
{
    if (!build || !probe || !pass_bits || n_passes == 0)
        return -1;
    threads = std::max(1u, threads);
    std::vector<uint32_t> bits(pass_bits, pass_bits + n_passes);
    const Schema bs = schema_of(*build), ps = schema_of(*probe);
    const auto t0 = Clock::now();
    Partitions bpart = radix_shuffle(*build, bs, bits, threads);
    const double t_bs = ms_since(t0);
    const auto t1 = Clock::now();
    Partitions ppart = radix_shuffle(*probe, ps, bits, threads);
    const double t_ps = ms_since(t1);
    const size_t parts = bpart.size();
    std::atomic<size_t> next{0};
    std::vector<double> build_ms(threads, 0), probe_ms(threads, 0);
    std::vector<Materialiser> mats(threads);
    run_threads(threads, [&](uint32_t tid) {
        Materialiser & mat = mats[tid];
        mat.ls = &bs;
        mat.rs = &ps;
        std::vector<uint64_t> hashes;
        ProbeScratch scr;
        for (;;)
        {
            const size_t p = next.fetch_add(1, std::memory_order_relaxed);
            if (p >= parts)
                break;
            const auto tb = Clock::now();
            Store st;
            Table ht;
            size_t rows = 0;
            for (const auto & b : bpart[p])
                rows += b.rows;
            if (rows)
                ht.reserve(rows);
            for (const auto & b : bpart[p])
                build_block(b.view(), st, ht, hashes);
            build_ms[tid] += ms_since(tb);
            const auto tp = Clock::now();
            if (!st.blocks.empty())
                for (const auto & b : ppart[p])
                    probe_block(b.view(), st, ht, mat, scr);
            probe_ms[tid] += ms_since(tp);
        }
        mat.finish();
    });
    const double e2e = ms_since(t0);
    int64_t total = 0;
    for (auto & m : mats)
        total += (int64_t)m.total;
    if (phase_ms)
    {
        phase_ms[0] = t_bs;
        phase_ms[1] = *std::max_element(build_ms.begin(), build_ms.end());
        phase_ms[2] = t_ps;
        phase_ms[3] = *std::max_element(probe_ms.begin(), probe_ms.end());
        phase_ms[4] = e2e;
    }
    fingerprint_outputs(mats, *build, *probe, fp);
    return total;
}

namespace
{
struct Slot
{
    std::mutex mu;
    Store store;
    Table ht;
    std::vector<OutBlk> owned; // sub-block storage (the store holds views into it)
};
} // namespace

extern "C" int64_t port_run_chj(const port_stream * build, const port_stream * probe, uint32_t threads, double * phase_ms, uint64_t * fp)
{
    if (!build || !probe)
        return -1;
    threads = std::max(1u, threads);
    const Schema bs = schema_of(*build), ps = schema_of(*probe);
    const size_t n_slots = std::min<size_t>(std::bit_ceil<size_t>(std::min<size_t>(threads, 256)), 256);
    std::vector<Slot> slots(n_slots);
    const size_t bbr = build->block_rows ? build->block_rows : 10000, pbr = probe->block_rows ? probe->block_rows : 10000;
    const size_t nbb = (build->rows + bbr - 1) / bbr, npb = (probe->rows + pbr - 1) / pbr;
    for (auto & s : slots)
        s.owned.reserve(nbb), s.store.blocks.reserve(nbb);
    const auto t0 = Clock::now();
    // build: bin rows of each block by slot, copy sub-blocks, try-lock insert
    run_threads(threads, [&](uint32_t tid) {
        std::vector<uint64_t> hashes;
        std::vector<std::vector<size_t>> rows_of(n_slots);
        for (size_t b = nbb * tid / threads; b < nbb * (tid + 1) / threads; ++b)
        {
            const size_t r0 = b * bbr, n = std::min(bbr, build->rows - r0);
            const uint64_t * keys = build->keys + r0;
            hashes.resize(n);
            for (size_t i = 0; i < n; ++i)
                hashes[i] = int_hash64(keys[i]);
            for (auto & v : rows_of)
                v.clear();
            for (size_t i = 0; i < n; ++i)
                rows_of[hashes[i] & (n_slots - 1)].push_back(i);
            std::vector<OutBlk> subs(n_slots);
            size_t left = 0;
            for (size_t s = 0; s < n_slots; ++s)
            {
                const auto & ri = rows_of[s];
                if (ri.empty())
                    continue;
                OutBlk & sb = subs[s];
                sb.rows = sb.cap = ri.size();
                sb.keys.resize(ri.size());
                for (size_t k = 0; k < ri.size(); ++k)
                    sb.keys[k] = keys[ri[k]];
                sb.cols.resize(bs.w.size());
                for (size_t c = 0; c < bs.w.size(); ++c)
                {
                    const uint32_t w = bs.w[c];
                    sb.cols[c].resize(ri.size() * w);
                    const uint8_t * src = static_cast<const uint8_t *>(build->cols[c]) + r0 * w;
                    for (size_t k = 0; k < ri.size(); ++k)
                        std::memcpy(sb.cols[c].data() + k * w, src + ri[k] * w, w);
                }
                ++left;
            }
            while (left)
            {
                bool progress = false;
                for (size_t s = 0; s < n_slots; ++s)
                {
                    if (!subs[s].rows)
                        continue;
                    std::unique_lock lk(slots[s].mu, std::try_to_lock);
                    if (!lk.owns_lock())
                        continue;
                    progress = true;
                    slots[s].owned.push_back(std::move(subs[s]));
                    build_block(slots[s].owned.back().view(), slots[s].store, slots[s].ht, hashes);
                    subs[s].rows = 0;
                    --left;
                }
                if (!progress)
                    std::this_thread::yield();
            }
        }
    });
    const double t_build = ms_since(t0);
    const auto t1 = Clock::now();
    std::vector<Materialiser> mats(threads);
    run_threads(threads, [&](uint32_t tid) {
        Materialiser & mat = mats[tid];
        mat.ls = &bs;
        mat.rs = &ps;
        std::vector<uint64_t> hashes;
        std::vector<std::vector<size_t>> rows_of(n_slots);
        std::vector<size_t> pidx;
        std::vector<Ref> bref;
        for (size_t b = npb * tid / threads; b < npb * (tid + 1) / threads; ++b)
        {
            View v;
            const size_t r0 = b * pbr;
            v.rows = std::min(pbr, probe->rows - r0);
            v.keys = probe->keys + r0;
            for (size_t c = 0; c < ps.w.size(); ++c)
                v.cols[c] = static_cast<const uint8_t *>(probe->cols[c]) + r0 * ps.w[c];
            hashes.resize(v.rows);
            for (size_t i = 0; i < v.rows; ++i)
                hashes[i] = int_hash64(v.keys[i]);
            for (auto & r : rows_of)
                r.clear();
            for (size_t i = 0; i < v.rows; ++i)
                rows_of[hashes[i] & (n_slots - 1)].push_back(i);
            for (size_t s = 0; s < n_slots; ++s)
            {
                if (rows_of[s].empty())
                    continue;
                pidx.clear();
                bref.clear();
                for (size_t i : rows_of[s])
                    for (Ref r = slots[s].ht.find(hashes[i], v.keys[i]); r.valid(); r = slots[s].store.next[r.block][r.row])
                    {
                        pidx.push_back(i);
                        bref.push_back(r);
                    }
                if (!pidx.empty())
                    mat.gather(v, slots[s].store, pidx.data(), bref.data(), pidx.size());
            }
        }
        mat.finish();
    });
    const double t_probe = ms_since(t1);
    int64_t total = 0;
    for (auto & m : mats)
        total += (int64_t)m.total;
    if (phase_ms)
    {
        phase_ms[0] = t_build;
        phase_ms[1] = t_probe;
        phase_ms[2] = ms_since(t0);
    }
    fingerprint_outputs(mats, *build, *probe, fp);
    return total;
}

// ---------------------------------------------------------------------------
// runPhjBep, src/PHJBep.cpp:113-790: full-depth build shuffle, eager leaf
// tables; per worker, its slice of probe blocks is scattered by pass 1 into
// private chains; a chain is refined to leaf depth (passes 2..N) into shared
// per-leaf chains when the worker's private bytes pass half its share of the
// budget (down to a quarter); shared leaves are evicted (probed and dropped)
// round-robin with try-lock once they hold 5/8 of the budget (down to 5/8 of
// that); finished workers help evict while others still scatter; residual
// private chains are refined and every leaf is drained at the end.
// ---------------------------------------------------------------------------
namespace
{
struct BepLeaf
{
    std::mutex mu;
    std::vector<OutBlk> blocks;
    std::atomic<size_t> rows{0};
};

// refineToLeaves: passes 2..N of one pass-1 chain (src/RadixPartition.cpp:417-539)
void refine_chain(std::vector<OutBlk> && in, const Schema & s, const std::vector<uint32_t> & bits, std::vector<Chain> & out_leaves, Scratch & sc)
{
    std::vector<std::vector<OutBlk>> cur(1);
    cur[0] = std::move(in);
    uint32_t consumed = bits[0];
    size_t parts = 1;
    for (size_t pass = 1; pass < bits.size(); ++pass)
    {
        const size_t sub = size_t{1} << bits[pass];
        const uint32_t shift = 64u - consumed - bits[pass];
        std::vector<Chain> next(parts * sub);
        for (auto & c : next)
            c.next_cap = s.initial_rows();
        for (size_t ip = 0; ip < parts; ++ip)
            for (const OutBlk & ob : cur[ip])
                scatter_batch(ob.view(), s, shift, sub, next.data() + ip * sub, sc);
        cur.assign(parts * sub, {});
        for (size_t p = 0; p < parts * sub; ++p)
            for (auto & b : next[p].blocks)
                if (b.rows)
                    cur[p].push_back(std::move(b));
        parts *= sub;
        consumed += bits[pass];
    }
    out_leaves.assign(parts, Chain{});
    for (size_t p = 0; p < parts; ++p)
        out_leaves[p].blocks = std::move(cur[p]);
}
} // namespace

extern "C" int64_t port_run_phj_bep(const port_stream * build, const port_stream * probe, const uint8_t * pass_bits, uint32_t n_passes,
                                    uint32_t threads, uint64_t budget_mib, double * phase_ms, uint64_t * counters, uint64_t * fp)
{
    if (!build || !probe || !pass_bits || n_passes == 0 || budget_mib == 0)
        return -1;
    threads = std::max(1u, threads);
    const std::vector<uint32_t> bits(pass_bits, pass_bits + n_passes);
    const Schema bs = schema_of(*build), ps = schema_of(*probe);
    const auto t0 = Clock::now();
    Partitions bpart = radix_shuffle(*build, bs, bits, threads);
    const double t_bs = ms_since(t0);
    const size_t total_leaves = bpart.size();
    const size_t P = size_t{1} << bits[0];
    const size_t leaves_per_p1 = total_leaves / P;
    size_t bpr = 8;
    for (uint32_t w : ps.w)
        bpr += w;
    const size_t budget = (size_t)budget_mib << 20;
    const size_t per_worker = budget / threads;
    const size_t unref_high = per_worker / 2, unref_low = unref_high / 2;
    const size_t leaf_high = budget * 5 / 8, leaf_low = leaf_high * 5 / 8;

    // eager leaf tables, work-stealing over leaves
    const auto tb0 = Clock::now();
    std::vector<Store> stores(total_leaves);
    std::vector<Table> tables(total_leaves);
    {
        std::atomic<size_t> next{0};
        run_threads(threads, [&](uint32_t) {
            std::vector<uint64_t> hashes;
            for (;;)
            {
                const size_t L = next.fetch_add(1, std::memory_order_relaxed);
                if (L >= total_leaves)
                    break;
                size_t rows = 0;
                for (const auto & b : bpart[L])
                    rows += b.rows;
                if (!rows)
                    continue;
                tables[L].reserve(rows);
                for (const auto & b : bpart[L])
                    build_block(b.view(), stores[L], tables[L], hashes);
            }
        });
    }
    const double t_build = ms_since(tb0);

    std::vector<BepLeaf> leaves(total_leaves);
    std::atomic<size_t> global_rows{0}, cursor{0}, peak{0}, active{threads};
    std::atomic<uint64_t> evictions{0}, refinements{0}, skips{0};
    std::vector<Materialiser> mats(threads);
    std::vector<double> shuffle_ms(threads, 0), probe_ms(threads, 0), evict_ms(threads, 0);
    const size_t block_rows = probe->block_rows ? probe->block_rows : 10000;
    const size_t n_blocks = (probe->rows + block_rows - 1) / block_rows;
    auto probe_leaf = [&](std::vector<OutBlk> & blocks, size_t L, Materialiser & mat, ProbeScratch & scr) {
        if (!stores[L].blocks.empty())
            for (const auto & b : blocks)
                probe_block(b.view(), stores[L], tables[L], mat, scr);
        blocks.clear();
    };
    // one round-robin eviction attempt; returns the rows evicted
    auto try_evict = [&](uint32_t tid, Materialiser & mat, ProbeScratch & scr) -> size_t {
        const auto te = Clock::now();
        const size_t L = cursor.fetch_add(1, std::memory_order_relaxed) % total_leaves;
        BepLeaf & lf = leaves[L];
        if (lf.rows.load(std::memory_order_relaxed) == 0)
        {
            evict_ms[tid] += ms_since(te);
            return 0;
        }
        std::unique_lock<std::mutex> lock(lf.mu, std::try_to_lock);
        if (!lock.owns_lock())
        {
            skips.fetch_add(1, std::memory_order_relaxed);
            evict_ms[tid] += ms_since(te);
            return 0;
        }
        const size_t rows = lf.rows.load(std::memory_order_relaxed);
        if (!rows)
            return 0;
        std::vector<OutBlk> stolen = std::move(lf.blocks);
        lf.blocks.clear();
        lf.rows.store(0, std::memory_order_relaxed);
        lock.unlock();
        global_rows.fetch_sub(rows, std::memory_order_relaxed);
        evict_ms[tid] += ms_since(te);
        const auto tp = Clock::now();
        probe_leaf(stolen, L, mat, scr);
        probe_ms[tid] += ms_since(tp);
        evictions.fetch_add(1, std::memory_order_relaxed);
        return rows;
    };

    run_threads(threads, [&](uint32_t tid) {
        Materialiser & mat = mats[tid];
        mat.ls = &bs;
        mat.rs = &ps;
        ProbeScratch scr;
        Scratch sc, rsc;
        std::vector<Chain> unref(P);
        for (auto & c : unref)
            c.next_cap = ps.initial_rows();
        std::vector<size_t> unref_rows(P, 0);
        size_t unref_bytes = 0;
        std::vector<Chain> inter;
        auto refine = [&](size_t p1) {
            std::vector<OutBlk> blocks;
            for (auto & b : unref[p1].blocks)
                if (b.rows)
                    blocks.push_back(std::move(b));
            unref[p1] = Chain{};
            unref[p1].next_cap = ps.initial_rows();
            unref_bytes -= unref_rows[p1] * bpr;
            unref_rows[p1] = 0;
            refine_chain(std::move(blocks), ps, bits, inter, rsc);
            size_t added_total = 0;
            for (size_t i = 0; i < inter.size(); ++i)
            {
                size_t added = 0;
                for (const auto & b : inter[i].blocks)
                    added += b.rows;
                if (!added)
                    continue;
                BepLeaf & lf = leaves[p1 * leaves_per_p1 + i];
                std::lock_guard<std::mutex> lock(lf.mu);
                for (auto & b : inter[i].blocks)
                    if (b.rows)
                        lf.blocks.push_back(std::move(b));
                lf.rows.fetch_add(added, std::memory_order_relaxed);
                added_total += added;
            }
            global_rows.fetch_add(added_total, std::memory_order_relaxed);
            refinements.fetch_add(1, std::memory_order_relaxed);
        };
        const size_t b0 = n_blocks * tid / threads, b1 = n_blocks * (tid + 1) / threads;
        for (size_t blk = b0; blk < b1; ++blk)
        {
            const auto ts = Clock::now();
            View v;
            const size_t r0 = blk * block_rows;
            v.rows = std::min(block_rows, probe->rows - r0);
            v.keys = probe->keys + r0;
            for (size_t c = 0; c < ps.w.size(); ++c)
                v.cols[c] = static_cast<const uint8_t *>(probe->cols[c]) + r0 * ps.w[c];
            scatter_batch(v, ps, 64u - bits[0], P, unref.data(), sc);
            for (size_t p = 0; p < P; ++p)
                unref_rows[p] += sc.hist[p];
            unref_bytes += v.rows * bpr;
            const size_t cur = global_rows.load(std::memory_order_relaxed) * bpr;
            size_t old = peak.load(std::memory_order_relaxed);
            while (cur > old && !peak.compare_exchange_weak(old, cur, std::memory_order_relaxed))
            {
            }
            // private chains above the high-water mark: refine the largest
            if (unref_bytes >= unref_high)
                while (unref_bytes >= unref_low)
                {
                    size_t best = SIZE_MAX, best_rows = 0;
                    for (size_t p = 0; p < P; ++p)
                        if (unref_rows[p] > best_rows)
                            best_rows = unref_rows[p], best = p;
                    if (best == SIZE_MAX)
                        break;
                    refine(best);
                }
            shuffle_ms[tid] += ms_since(ts);
            // shared leaves above the high-water mark: evict
            size_t cached = global_rows.load(std::memory_order_relaxed) * bpr;
            if (cached >= leaf_high)
            {
                size_t misses = 0, since = 0;
                while (cached >= leaf_low)
                {
                    const size_t rows = try_evict(tid, mat, scr);
                    if (!rows)
                    {
                        if (++misses >= 64)
                        {
                            cached = global_rows.load(std::memory_order_relaxed) * bpr;
                            misses = 0;
                        }
                        continue;
                    }
                    misses = 0;
                    cached = cached > rows * bpr ? cached - rows * bpr : 0;
                    if (++since >= 4)
                    {
                        cached = global_rows.load(std::memory_order_relaxed) * bpr;
                        since = 0;
                    }
                }
            }
        }
        // help evict while other workers still scatter
        active.fetch_sub(1, std::memory_order_acq_rel);
        while (active.load(std::memory_order_acquire) > 0)
        {
            if (global_rows.load(std::memory_order_relaxed) * bpr >= leaf_low && try_evict(tid, mat, scr))
                continue;
            std::this_thread::yield();
        }
        const auto tf = Clock::now();
        for (size_t p = 0; p < P; ++p)
            if (unref_rows[p])
                refine(p);
        shuffle_ms[tid] += ms_since(tf);
    });
    // drain every leaf, work-stealing
    {
        std::atomic<size_t> next{0};
        run_threads(threads, [&](uint32_t tid) {
            Materialiser & mat = mats[tid];
            ProbeScratch scr;
            for (;;)
            {
                const size_t L = next.fetch_add(1, std::memory_order_relaxed);
                if (L >= total_leaves)
                    break;
                if (leaves[L].rows.load(std::memory_order_relaxed) == 0)
                    continue;
                const auto tp = Clock::now();
                probe_leaf(leaves[L].blocks, L, mat, scr);
                leaves[L].rows.store(0, std::memory_order_relaxed);
                probe_ms[tid] += ms_since(tp);
                evictions.fetch_add(1, std::memory_order_relaxed);
            }
            mat.finish();
        });
    }
    const double e2e = ms_since(t0);
    int64_t total = 0;
    for (auto & m : mats)
        total += (int64_t)m.total;
    if (phase_ms)
    {
        phase_ms[0] = t_bs;
        phase_ms[1] = t_build;
        phase_ms[2] = *std::max_element(shuffle_ms.begin(), shuffle_ms.end());
        phase_ms[3] = *std::max_element(probe_ms.begin(), probe_ms.end());
        phase_ms[4] = *std::max_element(evict_ms.begin(), evict_ms.end());
        phase_ms[5] = e2e;
    }
    if (counters)
    {
        counters[0] = evictions.load();
        counters[1] = refinements.load();
        counters[2] = peak.load();
        counters[3] = skips.load();
    }
    fingerprint_outputs(mats, *build, *probe, fp);
    return total;
}
