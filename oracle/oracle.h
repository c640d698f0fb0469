/*
 * oracle.h -- CPU restatement of phj-bench's correctness reference.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only tests/, bench.py's CPU-baseline leg and
 * __graft_entry__.smoke() use it, and only as the checker.
 *
 * What it restates (file:line in harikrishnan94/phj-bench):
 *   - intHash64                     src/Hash.h:18-25
 *   - referenceOutput               src/Reference.cpp:48-76  (key -> every build
 *                                   row with that key, emitted per probe row)
 *   - serializeRow / serializeOutput src/Reference.cpp:22-43, 79-110  (row bytes
 *                                   = key(8 LE) || build payloads || probe payloads)
 *   - compareOutputs                src/Reference.cpp:113-133 (sort both, compare)
 *   - radix partition id            src/RadixPartition.cpp:358-361, 562-574
 *                                   (top bits of the hash, pass by pass)
 * plus an order-independent fingerprint of an output multiset (row count and
 * two 64-bit sums of per-row hashes) for sizes where sorted row vectors do
 * not fit in host memory.
 *
 * Parity pinning: tests/golden/ holds digests produced by the reference
 * itself (compiled from its own sources by oracle/Makefile into oracle/_ref/)
 * and tests/test_oracle.py checks this restatement against them.
 */
#ifndef PHJ_ORACLE_H
#define PHJ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_MAX_PAYLOADS 8

/* Payload type codes follow src/Types.h:23-30 (u8=0 .. u128=4). */
typedef struct oracle_stream {
    uint64_t rows;
    const uint64_t *keys;
    uint32_t n_payloads;
    uint8_t types[ORACLE_MAX_PAYLOADS];
    const void *cols[ORACLE_MAX_PAYLOADS]; /* column c: rows * size(types[c]) bytes */
} oracle_stream;

uint64_t oracle_int_hash64(uint64_t x);
void oracle_int_hash64_batch(const uint64_t *in, uint64_t n, uint64_t *out);
uint32_t oracle_payload_size(uint8_t type);
uint64_t oracle_row_width(const oracle_stream *build, const oracle_stream *probe);

/* Number of rows referenceOutput would produce. */
int64_t oracle_join_count(const oracle_stream *build, const oracle_stream *probe);

/* referenceOutput: serialised rows, unsorted, `cap` rows at most.
 * Returns rows written, or -1 if `cap` is too small. */
int64_t oracle_join_rows(const oracle_stream *build, const oracle_stream *probe, uint8_t *out, uint64_t cap);

/* serializeOutput for a columnar output (key column + left columns + right
 * columns, `rows` long each). */
void oracle_serialize_columns(uint64_t rows, const uint64_t *keys,
                              uint32_t n_left, const uint8_t *left_types, const void *const *left,
                              uint32_t n_right, const uint8_t *right_types, const void *const *right,
                              uint8_t *out);

/* Byte-lexicographic sort of fixed-width rows (std::string ordering). */
void oracle_sort_rows(uint8_t *rows, uint64_t n, uint64_t width);

/* compareOutputs: sorts both and compares.  Returns -1 when equal, -2 on a
 * row-count mismatch, else the first differing sorted position. */
int64_t oracle_compare_rows(uint8_t *expected, uint64_t n_expected, uint8_t *actual, uint64_t n_actual,
                            uint64_t width);

/* Fingerprint of the join result that referenceOutput would produce:
 * fp[0] = rows, fp[1] = sum of row_hash_a, fp[2] = sum of row_hash_b (mod 2^64).
 * Runs on `threads` host threads (0 = 1). */
void oracle_join_fingerprint(const oracle_stream *build, const oracle_stream *probe, uint32_t threads, uint64_t fp[3]);

/* Same fingerprint over a columnar output. */
void oracle_columns_fingerprint(uint64_t rows, const uint64_t *keys,
                                uint32_t n_left, const uint8_t *left_types, const void *const *left,
                                uint32_t n_right, const uint8_t *right_types, const void *const *right,
                                uint64_t fp[3]);

/* Same fingerprint over serialised rows with the given schemas. */
void oracle_rows_fingerprint(const uint8_t *rows, uint64_t n,
                             uint32_t n_left, const uint8_t *left_types,
                             uint32_t n_right, const uint8_t *right_types, uint64_t fp[3]);

/* Leaf (final radix partition) of each key under `total_bits` top hash bits. */
void oracle_leaf_ids(const uint64_t *keys, uint64_t n, uint32_t total_bits, uint32_t *out);

#ifdef __cplusplus
}
#endif

#endif
