// ref_shim.cpp -- a C-ABI shim over the UNMODIFIED reference functions of
// harikrishnan94/phj-bench, compiled together with the reference's own
// sources (src/{DataGen,RadixPartition,CHJ,PHJ,PHJBep,Reference}.cpp) by
// oracle/Makefile into oracle/_ref/libphjref.so.  TEST INFRASTRUCTURE ONLY:
// it is how the oracle restatement (oracle.c) and the golden fixtures are
// pinned to the reference itself.  It copies no reference code; it only
// calls the reference's public functions:
//   intHash64                 src/Hash.h:18
//   generateBuild/Probe       src/DataGen.h:20-34
//   referenceOutput et al.    src/Reference.h:15-25
//   runCHJ/runPHJ/runPhjBep   src/CHJ.h:31, src/PHJ.h:31, src/PHJBep.h:97
//   radixShuffle              src/RadixPartition.h:187-197
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "CHJ.h"
#include "DataGen.h"
#include "Hash.h"
#include "PHJ.h"
#include "PHJBep.h"
#include "RadixPartition.h"
#include "Reference.h"

namespace
{

struct ShimStream
{
    uint64_t rows;
    const uint64_t * keys;
    uint32_t n_payloads;
    uint8_t types[8];
    const void * cols[8];
};

phj::BlockStream toBlockStream(const ShimStream & s, size_t block_rows)
{
    phj::BlockStream out;
    for (uint32_t c = 0; c < s.n_payloads; ++c)
        out.schema.types.push_back(static_cast<phj::PayloadType>(s.types[c]));
    out.total_rows = s.rows;
    for (size_t start = 0; start < s.rows; start += block_rows)
    {
        const size_t n = std::min<size_t>(block_rows, s.rows - start);
        phj::Block blk;
        blk.init(out.schema, n);
        std::memcpy(blk.keys.data(), s.keys + start, n * sizeof(uint64_t));
        for (uint32_t c = 0; c < s.n_payloads; ++c)
        {
            const size_t w = phj::payloadTypeSize(out.schema.types[c]);
            std::memcpy(blk.payloads[c].raw(), static_cast<const uint8_t *>(s.cols[c]) + start * w, n * w);
        }
        out.blocks.push_back(std::move(blk));
    }
    return out;
}

// The reference's MemTracker caches its owner in a thread_local that
// outlives the tracker (src/MemTracker.h:85-135); on a thread that runs two
// schemes in a row the stale owner is written through.  Each reference call
// therefore runs on a fresh thread, as the reference's own worker threads do.
template <class F>
void onFreshThread(F && f)
{
    std::thread t(std::forward<F>(f));
    t.join();
}

int64_t emitRows(std::vector<std::string> rows, uint8_t * out, uint64_t cap, uint64_t width)
{
    std::sort(rows.begin(), rows.end());
    if (rows.size() > cap)
        return -1;
    for (size_t i = 0; i < rows.size(); ++i)
    {
        if (rows[i].size() != width)
            return -3;
        std::memcpy(out + i * width, rows[i].data(), width);
    }
    return static_cast<int64_t>(rows.size());
}

}

extern "C" {

uint64_t ref_int_hash64(uint64_t x)
{
    return phj::intHash64(x);
}

/// Keys of the reference's own DataGen (uniform build keys; probe keys drawn
/// from the build keys), for known-answer tests.
void ref_generate_keys(uint64_t build_rows, uint64_t probe_rows, uint64_t seed, uint64_t block_rows, uint64_t * build_keys, uint64_t * probe_keys)
{
    phj::PayloadSchema empty;
    phj::BlockStream b = phj::generateBuild(build_rows, empty, seed, 1, block_rows);
    phj::BlockStream p = phj::generateProbe(probe_rows, empty, seed, b, 1, block_rows);
    size_t i = 0;
    for (const auto & blk : b.blocks)
        for (size_t r = 0; r < blk.rows; ++r)
            build_keys[i++] = blk.keys[r];
    i = 0;
    for (const auto & blk : p.blocks)
        for (size_t r = 0; r < blk.rows; ++r)
            probe_keys[i++] = blk.keys[r];
}

/// referenceOutput, sorted, rows copied into `out`.  Returns the row count,
/// -1 if `cap` is too small.
int64_t ref_reference_rows(const ShimStream * build, const ShimStream * probe, uint64_t block_rows, uint8_t * out, uint64_t cap, uint64_t width)
{
    phj::BlockStream b = toBlockStream(*build, block_rows);
    phj::BlockStream p = toBlockStream(*probe, block_rows);
    return emitRows(phj::referenceOutput(b, p), out, cap, width);
}

/// Run one reference scheme (0 = CHJ, 1 = PHJ-PURE, 2 = PHJ/BEP), serialise
/// its output (serializeOutput), sort, and copy.  `stats` receives
/// e2e_wall_ms, then for BEP evictions, refinements, peak bytes, skip retries.
int64_t ref_run_scheme(
    int scheme,
    const ShimStream * build,
    const ShimStream * probe,
    uint64_t block_rows,
    const uint8_t * pass_bits,
    uint32_t n_passes,
    uint64_t threads,
    uint64_t budget_mib,
    uint8_t * out,
    uint64_t cap,
    uint64_t width,
    double * stats)
{
    phj::BlockStream b = toBlockStream(*build, block_rows);
    phj::BlockStream p = toBlockStream(*probe, block_rows);
    phj::RadixConfig cfg;
    cfg.pass_bits.assign(pass_bits, pass_bits + n_passes);
    std::vector<std::string> rows;
    onFreshThread([&] {
        if (scheme == 0)
        {
            phj::ChjResult r = phj::runCHJ(b, p, threads);
            stats[0] = r.e2e_wall_ms;
            rows = phj::serializeOutput(r.output);
        }
        else if (scheme == 1)
        {
            phj::PhjResult r = phj::runPHJ(b, p, cfg, threads);
            stats[0] = r.e2e_wall_ms;
            rows = phj::serializeOutput(r.output);
        }
        else
        {
            phj::PhjBepResult r = phj::runPhjBep(b, p, cfg, threads, budget_mib);
            stats[0] = r.e2e_wall_ms;
            stats[1] = static_cast<double>(r.bep_evictions);
            stats[2] = static_cast<double>(r.bep_refinements);
            stats[3] = static_cast<double>(r.bep_peak_bytes);
            stats[4] = static_cast<double>(r.bep_build_skip_retries);
            rows = phj::serializeOutput(r.output);
        }
    });
    return emitRows(std::move(rows), out, cap, width);
}

/// Timing-only run of one scheme; output is dropped.  Returns e2e_wall_ms.
double ref_time_scheme(
    int scheme,
    const ShimStream * build,
    const ShimStream * probe,
    uint64_t block_rows,
    const uint8_t * pass_bits,
    uint32_t n_passes,
    uint64_t threads,
    uint64_t budget_mib,
    uint64_t * out_rows)
{
    phj::BlockStream b = toBlockStream(*build, block_rows);
    phj::BlockStream p = toBlockStream(*probe, block_rows);
    phj::RadixConfig cfg;
    cfg.pass_bits.assign(pass_bits, pass_bits + n_passes);
    double ms = 0.0;
    onFreshThread([&] {
        if (scheme == 0)
        {
            phj::ChjResult r = phj::runCHJ(b, p, threads);
            *out_rows = r.output.totalRows();
            ms = r.e2e_wall_ms;
        }
        else if (scheme == 1)
        {
            phj::PhjResult r = phj::runPHJ(b, p, cfg, threads);
            *out_rows = r.output.totalRows();
            ms = r.e2e_wall_ms;
        }
        else
        {
            phj::PhjBepResult r = phj::runPhjBep(b, p, cfg, threads, budget_mib);
            *out_rows = r.output.totalRows();
            ms = r.e2e_wall_ms;
        }
    });
    return ms;
}

/// radixShuffle: per-partition row counts and the keys in partition order
/// (within-partition order is whatever the reference produced).
int64_t ref_radix_shuffle_keys(const ShimStream * s, uint64_t block_rows, const uint8_t * pass_bits, uint32_t n_passes, uint64_t threads, uint64_t * part_rows, uint64_t * keys_out)
{
    phj::BlockStream b = toBlockStream(*s, block_rows);
    phj::RadixConfig cfg;
    cfg.pass_bits.assign(pass_bits, pass_bits + n_passes);
    phj::PartitionedShuffleOutput out = phj::radixShuffle(b, cfg, threads);
    size_t k = 0;
    for (size_t p = 0; p < out.partitions; ++p)
    {
        part_rows[p] = out.partition_rows[p];
        for (const auto & ob : out.chains[p].blocks)
            for (size_t r = 0; r < ob.rows; ++r)
                keys_out[k++] = ob.keys[r];
    }
    return static_cast<int64_t>(k);
}

}
