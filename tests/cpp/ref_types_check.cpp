// Compiles phj_gpu.hpp against the reference's own types (Block.h,
// JoinOutput.h, RadixPartition.h and the scheme headers): the adapter is a
// drop-in for phj::runCHJ / runPHJ / runPhjBep.  Compile-only check.
#include "Block.h"
#include "CHJ.h"
#include "JoinOutput.h"
#include "PHJ.h"
#include "PHJBep.h"
#include "RadixPartition.h"
#define PHJ_GPU_WITH_REFERENCE_TYPES
#include "../../phj-bench_gb300/host/phj_gpu.hpp"

phj::ChjResult use_chj(const phj::BlockStream & b, const phj::BlockStream & p)
{
    return phj::gpu::runCHJ(b, p, 8);
}
phj::PhjResult use_phj(const phj::BlockStream & b, const phj::BlockStream & p, const phj::RadixConfig & cfg)
{
    return phj::gpu::runPHJ(b, p, cfg, 8);
}
phj::PhjBepResult use_bep(const phj::BlockStream & b, const phj::BlockStream & p, const phj::RadixConfig & cfg)
{
    return phj::gpu::runPhjBep(b, p, cfg, 8, 32);
}
