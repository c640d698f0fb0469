/*
 * phj_gpu.h -- C ABI of the GB300 (sm_103a) hash-join hot path.
 *
 * The reference (harikrishnan94/phj-bench) has no FFI: its boundary is three
 * C++ entry points over host BlockStreams,
 *     runCHJ    (src/CHJ.h:31)
 *     runPHJ    (src/PHJ.h:31)      -- the "phj-pure" scheme
 *     runPhjBep (src/PHJBep.h:97-98) -- the "phj" (best-effort partitioning) scheme
 * and their result structs.  This header is the C form of that boundary:
 * plain pointers and sizes, status codes instead of exceptions, one device,
 * one CUDA stream per context.  Each declaration names the reference
 * interface it replaces.  phj-bench_gb300/host/phj_gpu.hpp layers the
 * reference's C++ signatures on top of it.
 *
 * Threading: a context is used by one host thread at a time (the reference's
 * run* functions are likewise blocking calls from one thread); which thread
 * does not matter, and contexts on different threads run concurrently.  Each
 * call makes the context's device current for its duration and gives the
 * caller's current device back on return.  Every run call is blocking: it
 * returns when the join is complete on the device.
 */
#ifndef PHJ_GPU_H
#define PHJ_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHJ_GPU_ABI_VERSION 3u
#define PHJ_MAX_PAYLOADS 8u /* payload columns per side */

/* Error codes.  The reference throws std::invalid_argument / std::bad_alloc
 * (src/RadixPartition.cpp:554-560); across a C ABI they become codes, with
 * the message available from phj_last_error(). */
typedef enum phj_status {
    PHJ_OK = 0,
    PHJ_ERR_INVALID_ARGUMENT = 1,
    PHJ_ERR_CUDA = 2,
    PHJ_ERR_OUT_OF_MEMORY = 3,
    PHJ_ERR_UNSUPPORTED = 4,
    PHJ_ERR_DEVICE_TIMEOUT = 5, /* a bounded device wait gave up */
    PHJ_ERR_NO_DEVICE = 6,
    PHJ_ERR_CAPACITY = 7        /* caller-provided capacity too small */
} phj_status;

/* PayloadType, src/Types.h:23-30 (same codes, same widths 1/2/4/8/16). */
typedef enum phj_payload_type {
    PHJ_U8 = 0,
    PHJ_U16 = 1,
    PHJ_U32 = 2,
    PHJ_U64 = 3,
    PHJ_U128 = 4
} phj_payload_type;

/* RowRefCell, src/Types.h:95-104: 8 bytes; empty <=> block_no == 0xFFFFFFFF. */
typedef struct phj_row_ref {
    uint32_t block_no;
    uint32_t row_no;
} phj_row_ref;

/* JoinHashTable::Cell, src/HashTable.h:33-38: 16 bytes (key, RowRefCell). */
typedef struct phj_ht_cell {
    uint64_t key;
    phj_row_ref ref;
} phj_ht_cell;

/* PayloadSchema, src/Types.h:69-80. */
typedef struct phj_schema {
    uint32_t n_payloads;
    uint8_t types[PHJ_MAX_PAYLOADS];
} phj_schema;

typedef enum phj_location { PHJ_HOST = 0, PHJ_DEVICE = 1 } phj_location;

/* BlockStream, src/Block.h:157-162, with its blocks laid end to end: one key
 * column and one column per payload, `total_rows` long, split into
 * `n_blocks` blocks of `block_rows[i]` rows (block_rows == NULL: one block).
 * Block numbers are the build side's RowRefCell.block_no for CHJ. */
typedef struct phj_block_stream {
    phj_schema schema;
    uint64_t total_rows;
    uint32_t n_blocks;
    const uint32_t *block_rows;               /* host array of n_blocks, or NULL */
    const uint64_t *keys;
    const void *payloads[PHJ_MAX_PAYLOADS];   /* column c: total_rows * width(c) bytes */
    int32_t location;                         /* phj_location of keys/payloads */
} phj_block_stream;

/* PhaseTiming, src/JoinOutput.h:79-83 (device time from CUDA events). */
typedef struct phj_phase_timing {
    double wall_ms;
    double ns_per_row;
} phj_phase_timing;

/* ChjResult minus the output, src/CHJ.h:12-19. */
typedef struct phj_chj_result {
    phj_phase_timing build;
    phj_phase_timing probe;
    double e2e_wall_ms;
    uint64_t peak_mem_bytes; /* peak device bytes held by the run */
} phj_chj_result;

/* PhjResult minus the output, src/PHJ.h:13-22. */
typedef struct phj_phj_result {
    phj_phase_timing build_shuffle;
    phj_phase_timing build;
    phj_phase_timing probe_shuffle;
    phj_phase_timing probe;
    double e2e_wall_ms;
    uint64_t peak_mem_bytes;
} phj_phj_result;

/* PhjBepResult minus the output, src/PHJBep.h:13-39. */
typedef struct phj_bep_result {
    phj_phase_timing build_shuffle;
    phj_phase_timing build;
    phj_phase_timing probe_shuffle;
    phj_phase_timing probe;
    phj_phase_timing eviction_overhead;
    double e2e_wall_ms;
    uint64_t peak_mem_bytes;
    uint64_t bep_budget_mib;
    uint64_t bep_evictions;
    uint64_t bep_refinements;
    uint64_t bep_peak_bytes;
    uint64_t bep_build_skip_retries;
} phj_bep_result;

typedef struct phj_batch_result {
    double e2e_wall_ms;
    uint32_t n_joins;
    uint64_t build_rows;  /* summed over the joins */
    uint64_t probe_rows;
    uint64_t output_rows;
    uint64_t peak_mem_bytes;
} phj_batch_result;

typedef struct phj_ctx phj_ctx;       /* device, stream, memory pool, timers */
typedef struct phj_table phj_table;   /* a device-resident BlockStream */
typedef struct phj_output phj_output; /* a device-resident JoinOutput (src/JoinOutput.h:64-84) */

/* ---- context ---------------------------------------------------------- */

/* Opens `device`, creates the context's stream and stream-ordered pool. */
phj_status phj_ctx_create(int device, phj_ctx **out);
void phj_ctx_destroy(phj_ctx *ctx);
/* Message of the last failing call on this context ("" if none). */
const char *phj_last_error(const phj_ctx *ctx);
uint32_t phj_abi_version(void);
/* The context's CUDA stream (a cudaStream_t). */
void *phj_ctx_stream(phj_ctx *ctx);
/* Integer options of a context:
 *   "probe_materialize": -1 auto (default), 0 never, 1 always -- whether the
 *        partitioned schemes write the probe side's first radix pass to
 *        memory or probe the input order directly against the leaf tables;
 *   "time_kernels": 1 (default) records CUDA events around each kernel;
 *   "wait_limit_ms": bound of a device wait on another warp's work
 *        (PHJ/BEP leaf builds), 1..60000, default 1000;
 *   "host_chunk_rows": probe rows per chunk of phj_run_phj_pure_host (>= 4096);
 *   "table_cap_pct": leaf table cells >= rows * pct / 100, rounded up to a
 *        power of two (110..800, default 200: the reference's bit_ceil(2 rows));
 *   "p1_tile_rows", "p1_stages": tile rows (1024/2048/4096) and bulk-copy
 *        ring depth (2..4) of the first radix pass, 0 (default) chosen per
 *        row width;
 *   "pack_build": 1 (default) packs the build payloads row-major (16 bytes a
 *        row) for CHJ and PHJ-PURE joins without repeated build keys whose
 *        2+ build payload columns fit 16 bytes, so the projection gathers one
 *        value per output row; 0 gathers column by column;
 *   "chj_windows": CHJ probes in this many sweeps over the probe side
 *        (a power of two up to 256), each looking up only the keys of one
 *        group of consecutive top-8-bit sub-tables, so the tables a sweep
 *        touches can stay in L2; 0 or 1 (default): one sweep.  Same output
 *        rows, in another order;
 *   "bep_engine": PHJ (BEP) form; 0 (default) the device budget engine: one
 *        persistent grid whose CTA groups (one per SM) each hold a share of
 *        bep_budget_mib, scatter their slice of the probe side into
 *        first-pass chains, refine at the reference's water marks and
 *        evict leaves round-robin (first pass 1..11 bits with at most 13
 *        bits below it, fewer than 2^32 probe rows; other joins take the
 *        batch form); 1 budget-sized probe batches;
 *   "probe_fused": joins whose build keys are unique and whose build
 *        payloads are packed (2+ columns of 1-8 bytes, 16 bytes in all), one
 *        column of 4 or 8 bytes, or none (and no 16-byte probe column): 1
 *        (default) looks up and projects in one
 *        kernel, the output sized by the probe rows and its rows placed in
 *        reservation order; 0 looks up, scans and projects in two kernels.
 *        Same output rows;
 *   "batch_graph": phj_batch_run's chain; 1 (default) replays it as a
 *        captured CUDA graph (one timing record, "batch_graph"), 0 launches
 *        it kernel by kernel at the batch's own sizes (a timing record per
 *        kernel).  Same output rows;
 *   "probe_pass_bits": bits of the radix pass written out for the probe
 *        side, 1..11; 0 (default): PHJ-PURE chooses them from the build
 *        side's size so one bucket's leaf tables stay in L2, PHJ/BEP's
 *        batches take the configuration's first pass;
 *   "test_stuck_leaf": test hook, -1 (default) off; >= 0 leaves that PHJ/BEP
 *        leaf BUILDING before the probe, so its waits run out;
 *   "test_engine_stall_wave": test hook, -1 (default) off; >= 0 makes one
 *        CTA group of the PHJ (BEP) budget engine hold back from that
 *        wave's grid barrier until the others' bounded wait runs out, so
 *        the run fails with PHJ_ERR_DEVICE_TIMEOUT;
 *   "test_fail_build": test hook, 0 (default) off; 1 makes the host-buffer
 *        joins return PHJ_ERR_CUDA right after the build shuffle, with
 *        their uploads still queued. */
phj_status phj_ctx_set_int(phj_ctx *ctx, const char *name, int64_t value);
/* Reads an option above, or a device property: "device", "num_sms",
 * "l2_bytes", "wait_limit_ms". */
phj_status phj_ctx_get_int(const phj_ctx *ctx, const char *name, int64_t *value);

/* ---- radix configuration: src/CLI.cpp:330-355 ---------------------------- */

/* Resolves --partitions/--passes (or an explicit --partition-bits-per-pass
 * list when n_bits_override > 0) into per-pass bits exactly as the
 * reference CLI does: bits split evenly, the extra bits to the earlier
 * passes; total bits in [1, 32].  `out_bits` must hold 32 entries. */
phj_status phj_resolve_radix(uint64_t partitions, uint32_t passes, const uint8_t *bits_override,
                             uint32_t n_bits_override, uint8_t *out_bits, uint32_t *out_n_passes);

/* No counterpart in the reference (its radix bits come from the CLI): radix
 * bits for a build side of `build_rows` rows, aiming at leaves of about 256
 * rows (1 pass up to 11 bits, then 2 or 3 passes split evenly). */
phj_status phj_autotune_radix(uint64_t build_rows, uint64_t probe_rows, uint8_t *out_bits, uint32_t *out_n_passes);

/* ---- input streams -------------------------------------------------------- */

/* Copies a host BlockStream into device memory (replaces nothing in the
 * reference, whose streams are host-resident; needed because the schemes
 * below read device memory). */
phj_status phj_table_upload(phj_ctx *ctx, const phj_block_stream *host_stream, phj_table **out);
/* Wraps device columns without copying; the caller keeps them alive. */
phj_status phj_table_wrap_device(phj_ctx *ctx, const phj_block_stream *device_stream, phj_table **out);
/* Fills device columns with a seeded synthetic workload (see phj_gen_spec). */
typedef struct phj_gen_spec {
    uint32_t kind;        /* 0 build, unique keys K(i)                      */
                          /* 1 build, keys = permutation of 1..rows           */
                          /* 2 build, multi-match: geometric multiplicities   */
                          /* 3 probe, uniform over [1, key_domain]            */
                          /* 4 probe, K(uniform(domain)) w.p. match_permille/1000, else non-matching */
                          /* 5 probe, Zipf(theta) ranks through a permutation of K(0..domain-1) */
    uint64_t rows;
    uint64_t seed;
    uint64_t key_seed;    /* seed of the K(i) key stream shared by both sides */
    uint64_t domain;      /* kind 3: max key; kind 4/5: number of build keys K(0..domain-1); kind 2: distinct-key cap */
    uint32_t match_permille;
    double theta;         /* kind 5 */
    phj_schema schema;
    uint32_t block_rows;  /* block size of the generated stream (10000 in the reference) */
} phj_gen_spec;
phj_status phj_table_generate(phj_ctx *ctx, const phj_gen_spec *spec, phj_table **out);
/* Copies a device table back to host columns (keys, then payload columns). */
phj_status phj_table_download(phj_ctx *ctx, const phj_table *t, uint64_t *keys, void *const *payloads);
uint64_t phj_table_rows(const phj_table *t);
/* Distinct keys of a table generated with kind 0 or 2 (0 otherwise). */
uint64_t phj_table_gen_distinct(const phj_table *t);
void phj_table_free(phj_ctx *ctx, phj_table *t);

/* ---- the radix partition operator ------------------------------------------ */

/* radixShuffle(input, cfg, threads) (src/RadixPartition.h:198-199,
 * src/RadixPartition.cpp:546-586): partitions `input` by the top
 * sum(pass_bits) bits of intHash64(key), pass by pass as the reference does,
 * into a new device table whose rows are in partition order, one block per
 * partition (PartitionedShuffleOutput::chains[p]).  partition_rows, when not
 * NULL, receives the 2^sum(pass_bits) row counts
 * (PartitionedShuffleOutput::partition_rows).  Rows keep their payloads; the
 * order of rows inside a partition is unspecified, as in the reference. */
phj_status phj_radix_shuffle(phj_ctx *ctx, const phj_table *input, const uint8_t *pass_bits, uint32_t n_passes,
                             phj_table **out, uint64_t *partition_rows);

/* ---- the three schemes ---------------------------------------------------- */

/* runCHJ (src/CHJ.h:31, src/CHJ.cpp:49-152): one global device table of
 * 16-byte cells namespaced by the top 8 hash bits, 128-bit CAS inserts, then
 * an unpartitioned probe.  `threads` of the reference has no device meaning. */
phj_status phj_run_chj(phj_ctx *ctx, const phj_table *build, const phj_table *probe, phj_output **out,
                       phj_chj_result *result);

/* runPHJ (src/PHJ.h:31, src/PHJ.cpp:19-150): radix shuffle of both sides
 * over `pass_bits` (n_passes passes, total bits in [1, 24] on the device),
 * per-leaf tables, probe with output projection. */
phj_status phj_run_phj_pure(phj_ctx *ctx, const phj_table *build, const phj_table *probe, const uint8_t *pass_bits,
                            uint32_t n_passes, phj_output **out, phj_phj_result *result);

/* runPHJ with the BlockStreams and the JoinOutput in host memory (pinned
 * for full speed), the form a host caller of runPHJ uses.  The build side is
 * uploaded whole; the probe side streams through in chunks of
 * "host_chunk_rows" rows (context option, default 16M) with the upload of
 * the next chunk, the join of this one and the download of the previous
 * output overlapped.  Output rows go to the host columns (`out_keys`,
 * `out_left[build payloads]`, `out_right[probe payloads]`, `out_capacity`
 * rows); *out_rows receives the join's row count, and above the capacity
 * the call returns PHJ_ERR_CAPACITY with the first rows written. */
phj_status phj_run_phj_pure_host(phj_ctx *ctx, const phj_block_stream *build, const phj_block_stream *probe,
                                 const uint8_t *pass_bits, uint32_t n_passes, uint64_t out_capacity, uint64_t *out_keys,
                                 void *const *out_left, void *const *out_right, uint64_t *out_rows,
                                 phj_phj_result *result);

/* runPhjBep (src/PHJBep.h:97-98, src/PHJBep.cpp:113-790): bounded probe-side
 * buffering with lazily built leaf tables.  The probe side streams through
 * in batches of at most `bep_budget_mib` MiB of probe rows (the reference's
 * whole-run budget, src/PHJBep.cpp:151; at least 4096 rows a batch); each
 * batch is scattered by the first radix pass, then probed, the first warp
 * to need a leaf table building it (NOT_BUILT -> BUILDING -> BUILT).
 * `workers` is the reference's `threads` and does not change the device
 * schedule. */
phj_status phj_run_phj_bep(phj_ctx *ctx, const phj_table *build, const phj_table *probe, const uint8_t *pass_bits,
                           uint32_t n_passes, uint64_t bep_budget_mib, uint32_t workers, phj_output **out,
                           phj_bep_result *result);

/* runPhjBep with the BlockStreams and the JoinOutput in host memory (pinned
 * for full speed).  The build side is uploaded whole; the probe side
 * streams through in batches of at most `bep_budget_mib` MiB and at most
 * "host_chunk_rows" rows, with the upload of the next batch, the join of
 * this one and the download of the previous output overlapped (the smaller
 * batches count more evictions than phj_run_phj_bep with the same budget).
 * Output and capacity as phj_run_phj_pure_host. */
phj_status phj_run_phj_bep_host(phj_ctx *ctx, const phj_block_stream *build, const phj_block_stream *probe,
                                const uint8_t *pass_bits, uint32_t n_passes, uint64_t bep_budget_mib, uint64_t out_capacity,
                                uint64_t *out_keys, void *const *out_left, void *const *out_right, uint64_t *out_rows,
                                phj_bep_result *result);

/* Batching (no counterpart in the reference: it runs one join per call).
 * Runs n independent joins together: every join's build and probe sides are
 * radix-partitioned by the same launches (histogram, scan, scatter over
 * (join, tile) items, about 1024 build rows a partition), then ONE
 * persistent launch whose CTAs take (join, partition) items from a device
 * queue builds each partition's table in shared memory, probes its rows and
 * projects the matches; outs[j] receives join j's output, the same multiset
 * of rows as a single-join entry point gives for that pair, in no fixed
 * order.  A join is given one output row per probe row; one that needs more
 * (repeated build keys) is counted, then run again on its own.  Meant for
 * small and medium joins, whose single launches would not fill the device;
 * fewer than 2^31 build rows and 2^31 probe rows a join, and fewer than
 * 2^32 on each side in all (PHJ_ERR_UNSUPPORTED otherwise).  The chain
 * between the one upload of the batch's descriptors and the one download
 * of its row counts reads nothing back to the host; it is captured into a
 * CUDA graph on the first call and replayed by later calls whose batch fits
 * the context's workspace (it grows, and the chain is captured again, for a
 * larger batch; option "batch_graph").  The workspace (a few MiB: the
 * joins' descriptors and the partitions' counts and offsets) lives until
 * phj_ctx_destroy and is not counted in peak_mem_bytes.  The call
 * synchronizes the context's stream. */
phj_status phj_batch_run(phj_ctx *ctx, uint32_t n, const phj_table *const *builds, const phj_table *const *probes,
                         phj_output **outs, phj_batch_result *result);

/* ---- serving (no counterpart in the reference) ------------------------------
 * A request loop: requests with arrival times, admission while the summed
 * estimated HBM footprint of the requests in flight stays within a budget,
 * `workers` execution slots (a context and stream each) whose work overlaps
 * on the device, and continuous batching: a free slot takes either the
 * oldest ready request alone (run through phj_run_phj_pure with `pass_bits`)
 * or, when that request is small, every small ready request that fits, up
 * to `batch_max_joins`, run through phj_batch_run.  Each request's inputs
 * are generated on the device when it starts (phj_gen_spec); its output is
 * fingerprinted on the device and freed.  workers = 1 with batching off is
 * the plain one-join-per-call form. */
typedef struct phj_serve_config {
    int device;
    uint32_t workers;              /* execution slots, 1..64 */
    uint64_t hbm_budget_bytes;     /* admission budget over requests in flight */
    uint64_t batch_max_build_rows; /* requests with at most this many build rows are batched (0: never) */
    uint32_t batch_max_joins;      /* joins per batch (<= 1: never batch) */
    uint8_t pass_bits[8];          /* radix configuration of the joins run alone */
    uint32_t n_passes;             /* 0: phj_autotune_radix per request */
} phj_serve_config;

typedef struct phj_serve_request {
    phj_gen_spec build;
    phj_gen_spec probe;
    double arrival_s;              /* seconds after phj_serve_start */
} phj_serve_request;

typedef struct phj_serve_record {
    uint64_t id;
    double arrival_s, admit_s, start_s, done_s; /* seconds after phj_serve_start */
    uint64_t build_rows, probe_rows, output_rows;
    uint64_t footprint_bytes;      /* the admission estimate */
    uint64_t fingerprint[3];       /* phj_output_fingerprint of the output */
    uint32_t batch_size;           /* joins in the launch set that ran it (1: alone) */
    uint32_t slot;
    int32_t status;                /* phj_status; -1 while not done */
    uint64_t job_peak_bytes;       /* measured peak device bytes of the launch set (inputs included) */
    double gen_s;                  /* host seconds generating the request's inputs on the device */
    double call_s;                 /* host seconds of the join call (its launch set's share when batched) */
    double device_ms;              /* the join's device time, first kernel to last (its share when batched) */
} phj_serve_record;

typedef struct phj_server phj_server;
phj_status phj_serve_create(const phj_serve_config *cfg, phj_server **out);
/* Adds a request to the trace; all requests are submitted before start. */
phj_status phj_serve_submit(phj_server *s, const phj_serve_request *r, uint64_t *id);
/* Starts the clock, the dispatcher and the slots. */
phj_status phj_serve_start(phj_server *s);
/* Waits until every request is done: PHJ_OK, PHJ_ERR_DEVICE_TIMEOUT when
 * `timeout_s` passed first, PHJ_ERR_CUDA when a request failed. */
phj_status phj_serve_wait(phj_server *s, double timeout_s);
/* Copies up to `cap` records (request order); returns the request count. */
uint32_t phj_serve_records(phj_server *s, phj_serve_record *out, uint32_t cap);
const char *phj_serve_error(const phj_server *s);
void phj_serve_destroy(phj_server *s);
/* The admission estimate of a request, run alone (batched = 0) or batched. */
uint64_t phj_serve_footprint(const phj_serve_request *r, int batched);

/* No counterpart in the reference.  A CHJ-style join (one global table,
 * probe, projection) that allocates no device memory, for callers that must
 * not allocate while they join.  Its scratch is a fixed 2.5 MiB array in the
 * library (build sides of at most 65,536 rows); the output goes into the
 * caller's device columns (`out_keys`, `out_left[build payloads]`,
 * `out_right[probe payloads]`) of `out_capacity` rows, in no particular
 * order.  `*out_rows` receives the join's row count; above the capacity the
 * call returns PHJ_ERR_CAPACITY with the first `out_capacity` rows written.
 * The first call on a device sets up (it resolves the scratch address):
 * make that first call before any stream capture.  Every call waits for its
 * context's stream before it returns (it reads the row count back), and its
 * kernels are recorded for phj_last_kernel_times.  With out_capacity 0 the
 * column arrays may be NULL: the call only counts.  Calls that overlap in
 * time on one device race on the shared scratch: serialise them. */
phj_status phj_run_chj_noalloc(phj_ctx *ctx, const phj_table *build, const phj_table *probe, uint64_t out_capacity,
                               uint64_t *out_keys, void *const *out_left, void *const *out_right, uint64_t *out_rows);

/* ---- output --------------------------------------------------------------- */

uint64_t phj_output_rows(const phj_output *out);
/* Device column pointers: key column, build (left) columns, probe (right)
 * columns; the schemas are the build and probe schemas (OutputBlock,
 * src/JoinOutput.h:18-42). */
phj_status phj_output_device_columns(const phj_output *out, const uint64_t **keys, const void **left,
                                     const void **right);
/* Copies the output to host columns sized phj_output_rows() rows. */
phj_status phj_output_download(phj_ctx *ctx, const phj_output *out, uint64_t *keys, void *const *left,
                               void *const *right);
/* Order-independent fingerprint of the output multiset computed on the
 * device: fp[0] rows, fp[1], fp[2] sums of two per-row hashes (the oracle
 * computes the same for the reference join). */
phj_status phj_output_fingerprint(phj_ctx *ctx, const phj_output *out, uint64_t fp[3]);
void phj_output_free(phj_ctx *ctx, phj_output *out);

/* ---- measurement hooks ------------------------------------------------------ */

/* Per-kernel device times of the last run (CUDA events on the stream each
 * kernel was launched on).  Fills up to `cap` entries; returns the number
 * recorded.  `start_ms` places each launch on the run's timeline (0 = the
 * earliest timed launch), so a caller can tell which launches overlapped
 * launches on another of the context's streams. */
typedef struct phj_kernel_time {
    char name[32];
    double ms;
    uint64_t rows;   /* rows the launch processed */
    uint64_t bytes;  /* algorithmic bytes the launch read+wrote */
    double start_ms; /* start of the launch after the run's earliest timed launch */
} phj_kernel_time;
uint32_t phj_last_kernel_times(const phj_ctx *ctx, phj_kernel_time *out, uint32_t cap);
/* Number of this library's kernel launches issued since the context was
 * created. */
uint64_t phj_launch_count(const phj_ctx *ctx);

/* Pinned host memory (for host buffers of the end-to-end path). */
phj_status phj_host_alloc(phj_ctx *ctx, size_t bytes, void **out);
void phj_host_free(phj_ctx *ctx, void *p);

/* Writes `bytes` bytes over a scratch buffer larger than L2 so the next
 * timed run starts with a cold cache. */
phj_status phj_flush_l2(phj_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif /* PHJ_GPU_H */
