/*
 * cpu_port.h -- a C++ restatement of the reference's CPU join schemes, used
 * as the timed CPU baseline on machines where the reference itself cannot
 * be compiled (its sources are not there).  TEST/BASELINE INFRASTRUCTURE
 * ONLY: the product never calls it.
 *
 * It follows the reference's algorithms and data structures step for step:
 *   radixShuffle / scatterBatch / OutBlock chains  src/RadixPartition.cpp:30-586
 *   JoinHashTable (16-byte cells, linear probing)  src/HashTable.h:27-166
 *   BlockStore next-chain                          src/BlockStore.h:34-95
 *   buildOneBlock / probeOneBlock / materialiser   src/JoinOps.h:52-272
 *   runPHJ work-stealing over partitions           src/PHJ.cpp:19-150
 *   runCHJ slotted table, try-lock build           src/CHJ.cpp:16-119, src/JoinOps.h:290-429
 *   runPhjBep budgeted probe buffering, eviction   src/PHJBep.cpp:113-790
 */
#ifndef PHJ_CPU_PORT_H
#define PHJ_CPU_PORT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct port_stream {
    uint64_t rows;
    const uint64_t *keys;
    uint32_t n_payloads;
    uint8_t types[8];
    const void *cols[8];
    uint32_t block_rows; /* pipeline block size (10000 in the reference) */
} port_stream;

/* phase_ms: [0] build_shuffle, [1] build, [2] probe_shuffle, [3] probe, [4] e2e.
 * Returns output rows (materialised, then dropped), or -1 on bad arguments.
 * fp, when not NULL, receives the oracle's order-independent fingerprint of
 * the materialised rows (oracle_columns_fingerprint), taken after timing. */
int64_t port_run_phj_pure(const port_stream *build, const port_stream *probe, const uint8_t *pass_bits, uint32_t n_passes,
                          uint32_t threads, double *phase_ms, uint64_t *fp);

/* phase_ms: [0] build_shuffle, [1] build, [2] probe_shuffle, [3] probe,
 * [4] eviction_overhead, [5] e2e; counters: [0] evictions, [1] refinements,
 * [2] peak buffered leaf bytes, [3] skipped try-locks. */
int64_t port_run_phj_bep(const port_stream *build, const port_stream *probe, const uint8_t *pass_bits, uint32_t n_passes,
                         uint32_t threads, uint64_t budget_mib, double *phase_ms, uint64_t *counters, uint64_t *fp);

/* phase_ms: [0] build, [1] probe, [2] e2e. */
int64_t port_run_chj(const port_stream *build, const port_stream *probe, uint32_t threads, double *phase_ms, uint64_t *fp);

#ifdef __cplusplus
}
#endif

#endif
