// Drives phj::gpu::runPHJ / runCHJ (phj-bench_gb300/host/phj_gpu.hpp) the way
// phj-bench's Main.cpp drives the reference schemes: BlockStreams of
// 10,000-row blocks in, JoinOutput of OutputBlocks out.  Reads the two
// streams from raw column files and writes the output columns (blocks
// concatenated) for the test to compare with the oracle.
//   adapter_main <dir> <scheme: chj|phj-pure|phj> <bits,...> <budget_mib>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../phj-bench_gb300/host/phj_gpu.hpp"

using namespace phj::gpu;

static std::vector<std::byte> slurp(const std::string & path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f)
        return {};
    const std::streamsize n = f.tellg();
    f.seekg(0);
    std::vector<std::byte> b((size_t)n);
    f.read(reinterpret_cast<char *>(b.data()), n);
    return b;
}

static BlockStream load(const std::string & dir, const std::string & side)
{
    BlockStream s;
    std::ifstream meta(dir + "/" + side + ".schema");
    int t;
    while (meta >> t)
        s.schema.types.push_back((PayloadType)t);
    const auto keys = slurp(dir + "/" + side + ".keys");
    const size_t n = keys.size() / 8;
    std::vector<std::vector<std::byte>> cols;
    for (size_t c = 0; c < s.schema.types.size(); ++c)
        cols.push_back(slurp(dir + "/" + side + ".col" + std::to_string(c)));
    for (size_t r0 = 0; r0 < n; r0 += 10000)
    {
        const size_t m = std::min<size_t>(10000, n - r0);
        Block b;
        b.rows = m;
        b.keys.resize(m);
        std::memcpy(b.keys.data(), keys.data() + r0 * 8, m * 8);
        for (size_t c = 0; c < s.schema.types.size(); ++c)
        {
            const size_t w = payloadTypeSize(s.schema.types[c]);
            Column col;
            col.type = s.schema.types[c];
            col.data.assign(cols[c].begin() + (std::ptrdiff_t)(r0 * w), cols[c].begin() + (std::ptrdiff_t)((r0 + m) * w));
            b.payloads.push_back(std::move(col));
        }
        s.blocks.push_back(std::move(b));
    }
    s.total_rows = n;
    return s;
}

static void dump(const std::string & dir, const JoinOutput & out)
{
    std::ofstream k(dir + "/out.keys", std::ios::binary);
    std::vector<std::ofstream> l, r;
    for (size_t c = 0; c < out.left_schema.types.size(); ++c)
        l.emplace_back(dir + "/out.left" + std::to_string(c), std::ios::binary);
    for (size_t c = 0; c < out.right_schema.types.size(); ++c)
        r.emplace_back(dir + "/out.right" + std::to_string(c), std::ios::binary);
    for (const auto & w : out.workers)
        for (const auto & b : w.blocks)
        {
            k.write(reinterpret_cast<const char *>(b.keys.data()), (std::streamsize)(b.rows * 8));
            for (size_t c = 0; c < b.left.size(); ++c)
                l[c].write(reinterpret_cast<const char *>(b.left[c].raw()), (std::streamsize)b.left[c].data.size());
            for (size_t c = 0; c < b.right.size(); ++c)
                r[c].write(reinterpret_cast<const char *>(b.right[c].raw()), (std::streamsize)b.right[c].data.size());
        }
}

int main(int argc, char ** argv)
{
    if (argc < 5)
        return 2;
    const std::string dir = argv[1], scheme = argv[2];
    RadixConfig cfg;
    std::stringstream ss(argv[3]);
    for (std::string tok; std::getline(ss, tok, ',');)
        cfg.pass_bits.push_back((uint8_t)std::stoi(tok));
    const size_t budget = std::stoul(argv[4]);
    const BlockStream build = load(dir, "build"), probe = load(dir, "probe");
    try
    {
        if (scheme == "chj")
        {
            const ChjResult r = runCHJ(build, probe, 8);
            dump(dir, r.output);
            std::printf("rows %zu e2e_ms %.3f\n", r.output.totalRows(), r.e2e_wall_ms);
        }
        else if (scheme == "phj-pure")
        {
            const PhjResult r = runPHJ(build, probe, cfg, 8);
            dump(dir, r.output);
            std::printf("rows %zu e2e_ms %.3f\n", r.output.totalRows(), r.e2e_wall_ms);
        }
        else
        {
            const PhjBepResult r = runPhjBep(build, probe, cfg, 8, budget);
            dump(dir, r.output);
            std::printf("rows %zu e2e_ms %.3f evictions %zu\n", r.output.totalRows(), r.e2e_wall_ms, r.bep_evictions);
        }
    }
    catch (const std::invalid_argument & e)
    {
        std::printf("invalid_argument: %s\n", e.what());
        return 3;
    }
    return 0;
}
