// phj_gpu.hpp -- the reference's C++ scheme interface on top of the C ABI.
//
// A phj-bench maintainer replaces
//     phj::runCHJ(build, probe, threads)                       (src/CHJ.h:31)
//     phj::runPHJ(build, probe, cfg, threads)                  (src/PHJ.h:31)
//     phj::runPhjBep(build, probe, cfg, threads, budget_mib)   (src/PHJBep.h:97-98)
// with the same calls in namespace phj::gpu.  Results carry the same fields
// (PhaseTiming phases, e2e_wall_ms, peak_mem_bytes, JoinOutput with
// per-worker OutputBlocks of <= 10,000 rows), so serializeOutput,
// compareOutputs and the report consume them unchanged.
//
// Two ways to use it:
//   * with the reference's own types: include the reference headers
//     (Block.h, JoinOutput.h, RadixPartition.h, CHJ.h, PHJ.h, PHJBep.h), define
//     PHJ_GPU_WITH_REFERENCE_TYPES, then include this header;
//   * stand-alone: this header defines mirror types with the same names and
//     fields in namespace phj::gpu.
// Errors throw std::invalid_argument (bad radix configuration, as
// radixShuffle does) or std::runtime_error (device errors).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/phj_gpu.h"

#ifndef PHJ_GPU_WITH_REFERENCE_TYPES
namespace phj::gpu
{
// Mirror of src/Types.h, src/Block.h, src/JoinOutput.h, src/RadixPartition.h
// (RadixConfig) and the result structs of src/CHJ.h, src/PHJ.h, src/PHJBep.h:
// the same names and fields, plain std::vector storage.
enum class PayloadType : uint8_t
{
    UInt8 = 0,
    UInt16 = 1,
    UInt32 = 2,
    UInt64 = 3,
    UInt128 = 4,
};
inline constexpr size_t payloadTypeSize(PayloadType t) noexcept
{
    return t == PayloadType::UInt8 ? 1 : t == PayloadType::UInt16 ? 2 : t == PayloadType::UInt32 ? 4 : t == PayloadType::UInt64 ? 8 : 16;
}
struct PayloadSchema
{
    std::vector<PayloadType> types;
};
struct Column
{
    PayloadType type = PayloadType::UInt8;
    std::vector<std::byte> data;
    std::byte * raw() noexcept { return data.data(); }
    const std::byte * raw() const noexcept { return data.data(); }
};
struct Block
{
    size_t rows = 0;
    std::vector<uint64_t> keys;
    std::vector<Column> payloads;
};
struct BlockStream
{
    PayloadSchema schema;
    std::vector<Block> blocks;
    size_t total_rows = 0;
};
struct RadixConfig
{
    std::vector<uint8_t> pass_bits;
};
struct OutputBlock
{
    size_t rows = 0;
    std::vector<uint64_t> keys;
    std::vector<Column> left;
    std::vector<Column> right;
};
struct OutputWorker
{
    std::vector<OutputBlock> blocks;
    size_t totalRows() const noexcept
    {
        size_t s = 0;
        for (const auto & b : blocks)
            s += b.rows;
        return s;
    }
};
struct JoinOutput
{
    PayloadSchema left_schema;
    PayloadSchema right_schema;
    std::vector<OutputWorker> workers;
    size_t totalRows() const noexcept
    {
        size_t s = 0;
        for (const auto & w : workers)
            s += w.totalRows();
        return s;
    }
};
struct PhaseTiming
{
    double wall_ms = 0.0;
    double ns_per_row = 0.0;
};
struct ChjResult
{
    PhaseTiming build, probe;
    double e2e_wall_ms = 0.0;
    size_t peak_mem_bytes = 0;
    JoinOutput output;
};
struct PhjResult
{
    PhaseTiming build_shuffle, build, probe_shuffle, probe;
    double e2e_wall_ms = 0.0;
    size_t peak_mem_bytes = 0;
    JoinOutput output;
};
struct PhjBepResult
{
    PhaseTiming build_shuffle, build, probe_shuffle, probe, eviction_overhead;
    double e2e_wall_ms = 0.0;
    size_t peak_mem_bytes = 0;
    JoinOutput output;
    size_t bep_budget_mib = 0, bep_evictions = 0, bep_refinements = 0, bep_peak_bytes = 0, bep_build_skip_retries = 0;
};
} // namespace phj::gpu
namespace phj::gpu::types
{
using phj::gpu::BlockStream;
using phj::gpu::ChjResult;
using phj::gpu::JoinOutput;
using phj::gpu::OutputBlock;
using phj::gpu::OutputWorker;
using phj::gpu::PayloadSchema;
using phj::gpu::PayloadType;
using phj::gpu::PhaseTiming;
using phj::gpu::PhjBepResult;
using phj::gpu::PhjResult;
using phj::gpu::RadixConfig;
inline size_t typeSize(PayloadType t) { return phj::gpu::payloadTypeSize(t); }
}
#else
namespace phj::gpu::types
{
using phj::BlockStream;
using phj::ChjResult;
using phj::JoinOutput;
using phj::OutputBlock;
using phj::OutputWorker;
using phj::PayloadSchema;
using phj::PayloadType;
using phj::PhaseTiming;
using phj::PhjBepResult;
using phj::PhjResult;
using phj::RadixConfig;
inline size_t typeSize(PayloadType t) { return phj::payloadTypeSize(t); }
}
#endif

namespace phj::gpu
{
namespace detail
{
using namespace phj::gpu::types;

inline void check(phj_status st, phj_ctx * ctx, const char * what)
{
    if (st == PHJ_OK)
        return;
    std::string msg = std::string(what) + ": " + (ctx ? phj_last_error(ctx) : "no context");
    if (st == PHJ_ERR_INVALID_ARGUMENT)
        throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

// One context per process (device 0); the reference's calls are blocking
// calls from one thread, and so are these.
inline phj_ctx * context()
{
    static std::unique_ptr<phj_ctx, void (*)(phj_ctx *)> ctx(
        [] {
            phj_ctx * c = nullptr;
            check(phj_ctx_create(0, &c), nullptr, "phj_ctx_create");
            return c;
        }(),
        phj_ctx_destroy);
    return ctx.get();
}

inline phj_schema schema_of(const PayloadSchema & s)
{
    if (s.types.size() > PHJ_MAX_PAYLOADS)
        throw std::invalid_argument("more than 8 payload columns");
    phj_schema out{};
    out.n_payloads = (uint32_t)s.types.size();
    for (size_t c = 0; c < s.types.size(); ++c)
        out.types[c] = (uint8_t)s.types[c];
    return out;
}

// Packs a BlockStream (blocks laid end to end) into pinned host columns and
// uploads it.  Block numbers are preserved (CHJ's RowRefCell uses them).
struct Uploaded
{
    phj_ctx * ctx;
    phj_table * table = nullptr;
    std::vector<void *> pinned;
    ~Uploaded()
    {
        if (table)
            phj_table_free(ctx, table);
        for (void * p : pinned)
            phj_host_free(ctx, p);
    }
};

inline void upload(phj_ctx * ctx, const BlockStream & s, Uploaded & u)
{
    u.ctx = ctx;
    const size_t n = s.total_rows, K = s.schema.types.size();
    void * keys = nullptr;
    check(phj_host_alloc(ctx, std::max<size_t>(n, 1) * 8, &keys), ctx, "phj_host_alloc");
    u.pinned.push_back(keys);
    std::vector<void *> cols(K);
    for (size_t c = 0; c < K; ++c)
    {
        check(phj_host_alloc(ctx, std::max<size_t>(n, 1) * typeSize(s.schema.types[c]), &cols[c]), ctx, "phj_host_alloc");
        u.pinned.push_back(cols[c]);
    }
    std::vector<uint32_t> block_rows;
    size_t at = 0;
    for (const auto & b : s.blocks)
    {
        std::memcpy(static_cast<uint8_t *>(keys) + at * 8, b.keys.data(), b.rows * 8);
        for (size_t c = 0; c < K; ++c)
        {
            const size_t w = typeSize(s.schema.types[c]);
            std::memcpy(static_cast<uint8_t *>(cols[c]) + at * w, b.payloads[c].raw(), b.rows * w);
        }
        at += b.rows;
        block_rows.push_back((uint32_t)b.rows);
    }
    phj_block_stream d{};
    d.schema = schema_of(s.schema);
    d.total_rows = at;
    d.n_blocks = (uint32_t)block_rows.size();
    d.block_rows = block_rows.empty() ? nullptr : block_rows.data();
    d.keys = static_cast<const uint64_t *>(keys);
    for (size_t c = 0; c < K; ++c)
        d.payloads[c] = cols[c];
    d.location = PHJ_HOST;
    check(phj_table_upload(ctx, &d, &u.table), ctx, "phj_table_upload");
}

// Downloads a device output into per-worker OutputBlocks of <= 10,000 rows
// (ProbeMaterialiser's block size, src/Types.h:107).
inline void download(phj_ctx * ctx, phj_output * out, const PayloadSchema & ls, const PayloadSchema & rs, JoinOutput & jo)
{
    jo.left_schema = ls;
    jo.right_schema = rs;
    jo.workers.assign(1, OutputWorker{});
    const uint64_t n = phj_output_rows(out);
    std::vector<uint64_t> keys(n);
    std::vector<std::vector<std::byte>> left(ls.types.size()), right(rs.types.size());
    std::vector<void *> lp(PHJ_MAX_PAYLOADS, nullptr), rp(PHJ_MAX_PAYLOADS, nullptr);
    for (size_t c = 0; c < ls.types.size(); ++c)
    {
        left[c].resize(n * typeSize(ls.types[c]));
        lp[c] = left[c].data();
    }
    for (size_t c = 0; c < rs.types.size(); ++c)
    {
        right[c].resize(n * typeSize(rs.types[c]));
        rp[c] = right[c].data();
    }
    check(phj_output_download(ctx, out, keys.data(), lp.data(), rp.data()), ctx, "phj_output_download");
    constexpr size_t kRows = 10000;
    for (size_t r0 = 0; r0 < n; r0 += kRows)
    {
        const size_t m = std::min<size_t>(kRows, n - r0);
        OutputBlock ob;
        ob.rows = m;
        ob.keys.assign(keys.begin() + (std::ptrdiff_t)r0, keys.begin() + (std::ptrdiff_t)(r0 + m));
        ob.left.resize(ls.types.size());
        for (size_t c = 0; c < ls.types.size(); ++c)
        {
            const size_t w = typeSize(ls.types[c]);
            ob.left[c].type = ls.types[c];
            ob.left[c].data.assign(left[c].begin() + (std::ptrdiff_t)(r0 * w), left[c].begin() + (std::ptrdiff_t)((r0 + m) * w));
        }
        ob.right.resize(rs.types.size());
        for (size_t c = 0; c < rs.types.size(); ++c)
        {
            const size_t w = typeSize(rs.types[c]);
            ob.right[c].type = rs.types[c];
            ob.right[c].data.assign(right[c].begin() + (std::ptrdiff_t)(r0 * w), right[c].begin() + (std::ptrdiff_t)((r0 + m) * w));
        }
        jo.workers[0].blocks.push_back(std::move(ob));
    }
}

inline void timing(PhaseTiming & d, const phj_phase_timing & s)
{
    d.wall_ms = s.wall_ms;
    d.ns_per_row = s.ns_per_row;
}

struct OutputHolder
{
    phj_ctx * ctx;
    phj_output * out = nullptr;
    ~OutputHolder()
    {
        if (out)
            phj_output_free(ctx, out);
    }
};
} // namespace detail

/// runCHJ (src/CHJ.h:31).  `threads` has no device meaning.
inline types::ChjResult runCHJ(const types::BlockStream & build, const types::BlockStream & probe, size_t /*threads*/)
{
    phj_ctx * ctx = detail::context();
    detail::Uploaded b, p;
    detail::upload(ctx, build, b);
    detail::upload(ctx, probe, p);
    detail::OutputHolder o{ctx};
    phj_chj_result r{};
    detail::check(phj_run_chj(ctx, b.table, p.table, &o.out, &r), ctx, "runCHJ");
    types::ChjResult res;
    detail::timing(res.build, r.build);
    detail::timing(res.probe, r.probe);
    res.e2e_wall_ms = r.e2e_wall_ms;
    res.peak_mem_bytes = r.peak_mem_bytes;
    detail::download(ctx, o.out, build.schema, probe.schema, res.output);
    return res;
}

/// runPHJ (src/PHJ.h:31): the PHJ-PURE scheme.
inline types::PhjResult runPHJ(const types::BlockStream & build, const types::BlockStream & probe, const types::RadixConfig & cfg, size_t /*threads*/)
{
    phj_ctx * ctx = detail::context();
    detail::Uploaded b, p;
    detail::upload(ctx, build, b);
    detail::upload(ctx, probe, p);
    detail::OutputHolder o{ctx};
    phj_phj_result r{};
    detail::check(phj_run_phj_pure(ctx, b.table, p.table, cfg.pass_bits.data(), (uint32_t)cfg.pass_bits.size(), &o.out, &r), ctx, "runPHJ");
    types::PhjResult res;
    detail::timing(res.build_shuffle, r.build_shuffle);
    detail::timing(res.build, r.build);
    detail::timing(res.probe_shuffle, r.probe_shuffle);
    detail::timing(res.probe, r.probe);
    res.e2e_wall_ms = r.e2e_wall_ms;
    res.peak_mem_bytes = r.peak_mem_bytes;
    detail::download(ctx, o.out, build.schema, probe.schema, res.output);
    return res;
}

/// runPhjBep (src/PHJBep.h:97-98): the PHJ (best-effort partitioning) scheme.
inline types::PhjBepResult runPhjBep(const types::BlockStream & build, const types::BlockStream & probe, const types::RadixConfig & cfg,
                                     size_t /*threads*/, size_t bep_budget_mib)
{
    phj_ctx * ctx = detail::context();
    detail::Uploaded b, p;
    detail::upload(ctx, build, b);
    detail::upload(ctx, probe, p);
    detail::OutputHolder o{ctx};
    phj_bep_result r{};
    detail::check(phj_run_phj_bep(ctx, b.table, p.table, cfg.pass_bits.data(), (uint32_t)cfg.pass_bits.size(), bep_budget_mib, 0, &o.out, &r), ctx,
                  "runPhjBep");
    types::PhjBepResult res;
    detail::timing(res.build_shuffle, r.build_shuffle);
    detail::timing(res.build, r.build);
    detail::timing(res.probe_shuffle, r.probe_shuffle);
    detail::timing(res.probe, r.probe);
    detail::timing(res.eviction_overhead, r.eviction_overhead);
    res.e2e_wall_ms = r.e2e_wall_ms;
    res.peak_mem_bytes = r.peak_mem_bytes;
    res.bep_budget_mib = r.bep_budget_mib;
    res.bep_evictions = r.bep_evictions;
    res.bep_refinements = r.bep_refinements;
    res.bep_peak_bytes = r.bep_peak_bytes;
    res.bep_build_skip_retries = r.bep_build_skip_retries;
    detail::download(ctx, o.out, build.schema, probe.schema, res.output);
    return res;
}
} // namespace phj::gpu
