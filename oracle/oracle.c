/*
 * oracle.c -- CPU restatement of phj-bench's correctness reference
 * (src/Reference.cpp) and of its hash (src/Hash.h).  TEST INFRASTRUCTURE
 * ONLY: the product never links or calls it.  See oracle.h for the map of
 * reference file:line to function.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* src/Hash.h:18-25: salt xor, then the Murmur3 fmix64 finaliser. */
uint64_t oracle_int_hash64(uint64_t x)
{
    x ^= 0x4cf5ad432745937fULL;
    x = (x ^ (x >> 33)) * 0xff51afd7ed558ccdULL;
    x = (x ^ (x >> 33)) * 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

void oracle_int_hash64_batch(const uint64_t *in, uint64_t n, uint64_t *out)
{
    for (uint64_t i = 0; i < n; ++i)
        out[i] = oracle_int_hash64(in[i]);
}

/* src/Types.h:32-48 */
uint32_t oracle_payload_size(uint8_t type)
{
    switch (type) {
    case 0: return 1;
    case 1: return 2;
    case 2: return 4;
    case 3: return 8;
    case 4: return 16;
    default: return 0;
    }
}

static uint64_t schema_bytes(uint32_t n, const uint8_t *types)
{
    uint64_t s = 0;
    for (uint32_t c = 0; c < n; ++c)
        s += oracle_payload_size(types[c]);
    return s;
}

uint64_t oracle_row_width(const oracle_stream *build, const oracle_stream *probe)
{
    return 8 + schema_bytes(build->n_payloads, build->types) + schema_bytes(probe->n_payloads, probe->types);
}

/* ---------------------------------------------------------------------- */
/* Key index: key -> build rows in input order (the std::unordered_map of
 * src/Reference.cpp:52-59).  Open addressing on a mixer unrelated to
 * intHash64, so the oracle shares no hashing with the code under test. */

static uint64_t mix_splitmix(uint64_t z) /* Steele, Lea, Flood 2014 finaliser */
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static uint64_t mix_murmur(uint64_t k) /* Appleby's MurmurHash3 fmix64 */
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

typedef struct key_index {
    uint64_t cap;      /* power of two */
    uint64_t *keys;
    int64_t *head;     /* first build row with this key, -1 = empty slot */
    int64_t *tail;
    int64_t *next;     /* per build row: next row with the same key, in input order */
} key_index;

static int index_build(key_index *ix, const oracle_stream *b)
{
    uint64_t cap = 16;
    while (cap < 2 * b->rows + 16)
        cap <<= 1;
    ix->cap = cap;
    ix->keys = (uint64_t *)malloc(cap * sizeof(uint64_t));
    ix->head = (int64_t *)malloc(cap * sizeof(int64_t));
    ix->tail = (int64_t *)malloc(cap * sizeof(int64_t));
    ix->next = (int64_t *)malloc((b->rows ? b->rows : 1) * sizeof(int64_t));
    if (!ix->keys || !ix->head || !ix->tail || !ix->next)
        return -1;
    for (uint64_t i = 0; i < cap; ++i)
        ix->head[i] = -1;
    for (uint64_t r = 0; r < b->rows; ++r) {
        const uint64_t k = b->keys[r];
        uint64_t pos = mix_splitmix(k) & (cap - 1);
        while (ix->head[pos] >= 0 && ix->keys[pos] != k)
            pos = (pos + 1) & (cap - 1);
        ix->next[r] = -1;
        if (ix->head[pos] < 0) {
            ix->keys[pos] = k;
            ix->head[pos] = (int64_t)r;
            ix->tail[pos] = (int64_t)r;
        } else {
            ix->next[ix->tail[pos]] = (int64_t)r;
            ix->tail[pos] = (int64_t)r;
        }
    }
    return 0;
}

static int64_t index_find(const key_index *ix, uint64_t k)
{
    uint64_t pos = mix_splitmix(k) & (ix->cap - 1);
    while (ix->head[pos] >= 0) {
        if (ix->keys[pos] == k)
            return ix->head[pos];
        pos = (pos + 1) & (ix->cap - 1);
    }
    return -1;
}

static void index_free(key_index *ix)
{
    free(ix->keys);
    free(ix->head);
    free(ix->tail);
    free(ix->next);
}

int64_t oracle_join_count(const oracle_stream *build, const oracle_stream *probe)
{
    key_index ix;
    if (index_build(&ix, build) != 0)
        return -1;
    int64_t n = 0;
    for (uint64_t p = 0; p < probe->rows; ++p)
        for (int64_t r = index_find(&ix, probe->keys[p]); r >= 0; r = ix.next[r])
            ++n;
    index_free(&ix);
    return n;
}

/* Append one stream row's payload bytes (src/Reference.cpp:30-40). */
static uint8_t *put_payloads(uint8_t *dst, const oracle_stream *s, uint64_t row)
{
    for (uint32_t c = 0; c < s->n_payloads; ++c) {
        const uint32_t w = oracle_payload_size(s->types[c]);
        memcpy(dst, (const uint8_t *)s->cols[c] + row * w, w);
        dst += w;
    }
    return dst;
}

int64_t oracle_join_rows(const oracle_stream *build, const oracle_stream *probe, uint8_t *out, uint64_t cap)
{
    key_index ix;
    if (index_build(&ix, build) != 0)
        return -1;
    const uint64_t width = oracle_row_width(build, probe);
    uint64_t n = 0;
    for (uint64_t p = 0; p < probe->rows; ++p) {
        const uint64_t k = probe->keys[p];
        for (int64_t r = index_find(&ix, k); r >= 0; r = ix.next[r]) {
            if (n >= cap) {
                index_free(&ix);
                return -1;
            }
            uint8_t *dst = out + n * width;
            memcpy(dst, &k, 8);
            dst = put_payloads(dst + 8, build, (uint64_t)r);
            put_payloads(dst, probe, p);
            ++n;
        }
    }
    index_free(&ix);
    return (int64_t)n;
}

void oracle_serialize_columns(uint64_t rows, const uint64_t *keys,
                              uint32_t n_left, const uint8_t *left_types, const void *const *left,
                              uint32_t n_right, const uint8_t *right_types, const void *const *right,
                              uint8_t *out)
{
    const uint64_t width = 8 + schema_bytes(n_left, left_types) + schema_bytes(n_right, right_types);
    for (uint64_t i = 0; i < rows; ++i) {
        uint8_t *dst = out + i * width;
        memcpy(dst, &keys[i], 8);
        dst += 8;
        for (uint32_t c = 0; c < n_left; ++c) {
            const uint32_t w = oracle_payload_size(left_types[c]);
            memcpy(dst, (const uint8_t *)left[c] + i * w, w);
            dst += w;
        }
        for (uint32_t c = 0; c < n_right; ++c) {
            const uint32_t w = oracle_payload_size(right_types[c]);
            memcpy(dst, (const uint8_t *)right[c] + i * w, w);
            dst += w;
        }
    }
}

/* ---------------------------------------------------------------------- */
/* Sorting fixed-width rows: LSD radix sort on bytes would be fastest, but a
 * comparison sort keeps the oracle obviously right. */

static uint64_t g_sort_width; /* qsort has no context argument in C99 */

static int cmp_rows(const void *a, const void *b)
{
    return memcmp(a, b, g_sort_width);
}

void oracle_sort_rows(uint8_t *rows, uint64_t n, uint64_t width)
{
    if (n < 2)
        return;
    g_sort_width = width;
    qsort(rows, n, width, cmp_rows);
}

int64_t oracle_compare_rows(uint8_t *expected, uint64_t n_expected, uint8_t *actual, uint64_t n_actual,
                            uint64_t width)
{
    if (n_expected != n_actual)
        return -2;
    oracle_sort_rows(expected, n_expected, width);
    oracle_sort_rows(actual, n_actual, width);
    for (uint64_t i = 0; i < n_expected; ++i)
        if (memcmp(expected + i * width, actual + i * width, width) != 0)
            return (int64_t)i;
    return -1;
}

/* ---------------------------------------------------------------------- */
/* Order-independent fingerprint.  A row is the word sequence: key, then each
 * build payload, then each probe payload; a payload narrower than 8 bytes is
 * one zero-extended word, a u128 is two words (low, high).  Two independent
 * chained mixes give row_hash_a and row_hash_b; the fingerprint is
 * (rows, sum a, sum b) mod 2^64.  The GPU library computes the same. */

#define FP_SEED_A 0x243f6a8885a308d3ULL
#define FP_SEED_B 0x13198a2e03707344ULL
#define FP_GAMMA  0x9e3779b97f4a7c15ULL

typedef struct fp_acc {
    uint64_t a, b;
} fp_acc;

static inline void fp_word(fp_acc *h, uint64_t w)
{
    h->a = mix_splitmix(h->a ^ w);
    h->b = mix_murmur(h->b + w * FP_GAMMA);
}

static inline void fp_payload(fp_acc *h, uint8_t type, const uint8_t *src)
{
    uint64_t lo = 0, hi = 0;
    switch (type) {
    case 0: lo = *src; break;
    case 1: { uint16_t v; memcpy(&v, src, 2); lo = v; break; }
    case 2: { uint32_t v; memcpy(&v, src, 4); lo = v; break; }
    case 3: memcpy(&lo, src, 8); break;
    case 4: memcpy(&lo, src, 8); memcpy(&hi, src + 8, 8); break;
    default: break;
    }
    fp_word(h, lo);
    if (type == 4)
        fp_word(h, hi);
}

typedef struct fp_job {
    const oracle_stream *build, *probe;
    const key_index *ix;
    uint64_t begin, end;
    uint64_t fp[3];
} fp_job;

static void *fp_worker(void *arg)
{
    fp_job *j = (fp_job *)arg;
    uint64_t n = 0, sa = 0, sb = 0;
    const oracle_stream *b = j->build, *p = j->probe;
    for (uint64_t pr = j->begin; pr < j->end; ++pr) {
        const uint64_t k = p->keys[pr];
        for (int64_t r = index_find(j->ix, k); r >= 0; r = j->ix->next[r]) {
            fp_acc h = {FP_SEED_A, FP_SEED_B};
            fp_word(&h, k);
            for (uint32_t c = 0; c < b->n_payloads; ++c) {
                const uint32_t w = oracle_payload_size(b->types[c]);
                fp_payload(&h, b->types[c], (const uint8_t *)b->cols[c] + (uint64_t)r * w);
            }
            for (uint32_t c = 0; c < p->n_payloads; ++c) {
                const uint32_t w = oracle_payload_size(p->types[c]);
                fp_payload(&h, p->types[c], (const uint8_t *)p->cols[c] + pr * w);
            }
            ++n;
            sa += h.a;
            sb += h.b;
        }
    }
    j->fp[0] = n;
    j->fp[1] = sa;
    j->fp[2] = sb;
    return NULL;
}

void oracle_join_fingerprint(const oracle_stream *build, const oracle_stream *probe, uint32_t threads, uint64_t fp[3])
{
    fp[0] = fp[1] = fp[2] = 0;
    key_index ix;
    if (index_build(&ix, build) != 0) {
        fp[0] = ~0ULL;
        return;
    }
    if (threads == 0)
        threads = 1;
    if (threads > 256)
        threads = 256;
    fp_job jobs[256];
    pthread_t tids[256];
    for (uint32_t t = 0; t < threads; ++t) {
        jobs[t].build = build;
        jobs[t].probe = probe;
        jobs[t].ix = &ix;
        jobs[t].begin = probe->rows * t / threads;
        jobs[t].end = probe->rows * (t + 1) / threads;
        if (t > 0)
            pthread_create(&tids[t], NULL, fp_worker, &jobs[t]);
    }
    fp_worker(&jobs[0]);
    for (uint32_t t = 1; t < threads; ++t)
        pthread_join(tids[t], NULL);
    for (uint32_t t = 0; t < threads; ++t) {
        fp[0] += jobs[t].fp[0];
        fp[1] += jobs[t].fp[1];
        fp[2] += jobs[t].fp[2];
    }
    index_free(&ix);
}

void oracle_columns_fingerprint(uint64_t rows, const uint64_t *keys,
                                uint32_t n_left, const uint8_t *left_types, const void *const *left,
                                uint32_t n_right, const uint8_t *right_types, const void *const *right,
                                uint64_t fp[3])
{
    uint64_t sa = 0, sb = 0;
    for (uint64_t i = 0; i < rows; ++i) {
        fp_acc h = {FP_SEED_A, FP_SEED_B};
        fp_word(&h, keys[i]);
        for (uint32_t c = 0; c < n_left; ++c) {
            const uint32_t w = oracle_payload_size(left_types[c]);
            fp_payload(&h, left_types[c], (const uint8_t *)left[c] + i * w);
        }
        for (uint32_t c = 0; c < n_right; ++c) {
            const uint32_t w = oracle_payload_size(right_types[c]);
            fp_payload(&h, right_types[c], (const uint8_t *)right[c] + i * w);
        }
        sa += h.a;
        sb += h.b;
    }
    fp[0] = rows;
    fp[1] = sa;
    fp[2] = sb;
}

void oracle_rows_fingerprint(const uint8_t *rows, uint64_t n,
                             uint32_t n_left, const uint8_t *left_types,
                             uint32_t n_right, const uint8_t *right_types, uint64_t fp[3])
{
    const uint64_t width = 8 + schema_bytes(n_left, left_types) + schema_bytes(n_right, right_types);
    uint64_t sa = 0, sb = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint8_t *src = rows + i * width;
        fp_acc h = {FP_SEED_A, FP_SEED_B};
        uint64_t k;
        memcpy(&k, src, 8);
        fp_word(&h, k);
        src += 8;
        for (uint32_t c = 0; c < n_left; ++c) {
            fp_payload(&h, left_types[c], src);
            src += oracle_payload_size(left_types[c]);
        }
        for (uint32_t c = 0; c < n_right; ++c) {
            fp_payload(&h, right_types[c], src);
            src += oracle_payload_size(right_types[c]);
        }
        sa += h.a;
        sb += h.b;
    }
    fp[0] = n;
    fp[1] = sa;
    fp[2] = sb;
}

/* src/RadixPartition.cpp:358-361 with shifts from :562-574: every pass takes
 * the next bits from the top of the hash, so the final partition of a row is
 * its top `total_bits` hash bits. */
void oracle_leaf_ids(const uint64_t *keys, uint64_t n, uint32_t total_bits, uint32_t *out)
{
    for (uint64_t i = 0; i < n; ++i)
        out[i] = total_bits == 0 ? 0u : (uint32_t)(oracle_int_hash64(keys[i]) >> (64u - total_bits));
}
