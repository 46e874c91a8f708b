/*
 * oracle.c -- CPU restatement of Fiuncho's exhaustive epistasis-search hot
 * path.  TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and
 * by bench.py's CPU-baseline leg as the checker; never part of the product
 * path (the product is the CUDA library under fiuncho_gb300/).
 *
 * Each function states the reference code it follows (paths are relative to
 * the UDC-GAC/fiuncho source tree).  Plain C11 + pthreads, no SIMD intrinsics,
 * so it builds unchanged on x86-64 and aarch64.
 *
 * Layout conventions (identical to the reference):
 *   - one SNP = GenotypeTable of order 1: [cases: 3 rows x cases_words]
 *     followed by [ctrls: 3 rows x ctrls_words] uint64 words, row g holds the
 *     bit "genotype == g" of every sample (GenotypeTable.h:63-103).
 *   - all SNPs contiguous, SNP-major (GenotypeTable::make_array,
 *     GenotypeTable.h:77-103).
 *   - a contingency table of order k holds 3^k uint32 cells per class; cell
 *     index = sum_i g_i * 3^(k-1-i) (first SNP most significant), as produced
 *     by chained combine (src/base/gt_combine.cpp:9-17) and
 *     combine_and_popcnt (src/base/gt_popcnt.cpp:37-46).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ref/tabledigest.h"

#define ORC_MAX_ORDER 8

static inline uint32_t popc64(uint64_t x) { return (uint32_t)__builtin_popcountll(x); }

/* ------------------------------------------------------------------------ */
/* Data set packing: TPEDFile::fill (include/fiuncho/dataset/TPEDFile.hpp:176-269)
 * and RawFile::fill (include/fiuncho/dataset/RAWFile.hpp:209-290).
 * geno[snp * samples + s] in {0,1,2} (minor-allele count), is_case[s] != 0
 * for cases.  Samples of a class are shifted in MSB-first: within a full word
 * the first sample of the word is bit 63; the last, partial word of a row is
 * right-aligned (its last sample is bit 0), TPEDFile.hpp:213-254.  Words past
 * the data are zero (TPEDFile.hpp:255-267). */
void orc_pack(const uint8_t *geno, const uint8_t *is_case, size_t snps, size_t samples,
              size_t cases_words, size_t ctrls_words, uint64_t *out)
{
    const size_t per_snp = 3 * (cases_words + ctrls_words);
    for (size_t i = 0; i < snps; ++i) {
        uint64_t *cs = out + i * per_snp, *ct = cs + 3 * cases_words;
        memset(cs, 0, per_snp * sizeof(uint64_t));
        uint64_t bc[3] = {0, 0, 0}, bt[3] = {0, 0, 0};
        size_t nc = 0, nt = 0;
        const uint8_t *g = geno + i * samples;
        for (size_t s = 0; s < samples; ++s) {
            const unsigned v = g[s];
            if (is_case[s]) {
                for (int k = 0; k < 3; ++k) bc[k] = (bc[k] << 1) | (uint64_t)(v == (unsigned)k);
                if (++nc % 64 == 0) {
                    for (int k = 0; k < 3; ++k) { cs[k * cases_words + nc / 64 - 1] = bc[k]; bc[k] = 0; }
                }
            } else {
                for (int k = 0; k < 3; ++k) bt[k] = (bt[k] << 1) | (uint64_t)(v == (unsigned)k);
                if (++nt % 64 == 0) {
                    for (int k = 0; k < 3; ++k) { ct[k * ctrls_words + nt / 64 - 1] = bt[k]; bt[k] = 0; }
                }
            }
        }
        if (nc % 64)
            for (int k = 0; k < 3; ++k) cs[k * cases_words + nc / 64] = bc[k];
        if (nt % 64)
            for (int k = 0; k < 3; ++k) ct[k * ctrls_words + nt / 64] = bt[k];
    }
}

/* ------------------------------------------------------------------------ */
/* GenotypeTable::combine, scalar form (src/base/gt_combine.cpp:3-27):
 * out[(i*3+j)*words + w] = t1[i*words + w] & t2[j*words + w]. One class. */
void orc_combine(const uint64_t *t1, size_t size1, const uint64_t *t2, size_t words, uint64_t *out)
{
    for (size_t i = 0; i < size1; ++i)
        for (size_t j = 0; j < 3; ++j)
            for (size_t w = 0; w < words; ++w)
                out[(i * 3 + j) * words + w] = t1[i * words + w] & t2[j * words + w];
}

/* GenotypeTable::combine_and_popcnt, scalar form (src/base/gt_popcnt.cpp:4-35):
 * ct[i*3+j] = sum_w popcount(t1[i*words+w] & t2[j*words+w]); cells past
 * 3*size1 up to ct_size are zeroed (gt_popcnt.cpp:20-22). One class. */
void orc_popcnt(const uint64_t *t1, size_t size1, const uint64_t *t2, size_t words, uint32_t *ct,
                size_t ct_size)
{
    for (size_t i = 0; i < size1; ++i)
        for (size_t j = 0; j < 3; ++j) {
            uint32_t c = 0;
            for (size_t w = 0; w < words; ++w) c += popc64(t1[i * words + w] & t2[j * words + w]);
            ct[i * 3 + j] = c;
        }
    for (size_t i = size1 * 3; i < ct_size; ++i) ct[i] = 0;
}

/* ------------------------------------------------------------------------ */
/* MutualInformation<float>: constructor (include/fiuncho/algorithms/
 * MutualInformation.h:58-65) and scalar compute (src/base/mi_compute.cpp:16-41).
 * FP32 throughout, natural log, 0*log0 = 0.  This is the reference's own
 * arithmetic; its error against the exact value is what orc_mi_f64 shows. */
float orc_mi_f32(const uint32_t *cases, const uint32_t *ctrls, size_t size, uint32_t n_cases,
                 uint32_t n_ctrls)
{
    const float inv = (float)(1.0 / (double)(n_cases + n_ctrls));
    float p = n_cases * inv;
    float h_y = (float)((-1.0) * p * logf(p));
    p = n_ctrls * inv;
    h_y -= p * logf(p);
    float h_x = 0.0f, h_all = 0.0f;
    for (size_t i = 0; i < size; ++i) {
        const float pc = cases[i] * inv, pt = ctrls[i] * inv, pa = pc + pt;
        if (pc != 0.0f) h_all -= pc * logf(pc);
        if (pt != 0.0f) h_all -= pt * logf(pt);
        if (pa != 0.0f) h_x -= pa * logf(pa);
    }
    return h_x + h_y - h_all;
}

/* The same quantity, MI = H(X) + H(Y) - H(X,Y), evaluated directly from its
 * definition in FP64 (the accuracy oracle). */
double orc_mi_f64(const uint32_t *cases, const uint32_t *ctrls, size_t size, uint32_t n_cases,
                  uint32_t n_ctrls)
{
    const double n = (double)n_cases + (double)n_ctrls;
    double h_y = 0.0, h_x = 0.0, h_xy = 0.0;
    if (n_cases) h_y -= (n_cases / n) * log(n_cases / n);
    if (n_ctrls) h_y -= (n_ctrls / n) * log(n_ctrls / n);
    for (size_t i = 0; i < size; ++i) {
        const double pc = cases[i] / n, pt = ctrls[i] / n, pa = pc + pt;
        if (cases[i]) h_xy -= pc * log(pc);
        if (ctrls[i]) h_xy -= pt * log(pt);
        if (cases[i] + ctrls[i]) h_x -= pa * log(pa);
    }
    return h_x + h_y - h_xy;
}

/* ------------------------------------------------------------------------ */
/* Distribution<int>::const_iterator (include/fiuncho/Distribution.h:54-130):
 * lexicographic enumeration of k-combinations of n, advancing `step`
 * combinations per ++ and `offset` combinations at begin(). */
typedef struct {
    int n, k;
    int c[ORC_MAX_ORDER];
} orc_iter;

static void orc_increment_left(orc_iter *it) /* Distribution.h:60-78 */
{
    int p = it->k - 2;
    while (p >= 0 && it->c[p] + 1 > it->n - (it->k - p)) --p;
    if (p < 0) {
        it->c[0] = it->n;
    } else {
        ++it->c[p];
        for (int i = p + 1; i < it->k - 1; ++i) it->c[i] = it->c[i - 1] + 1;
    }
}

static void orc_increment(orc_iter *it, int x) /* Distribution.h:80-87 */
{
    const int k = it->k;
    it->c[k - 1] += x;
    while (it->c[0] < it->n && it->c[k - 1] >= it->n) {
        orc_increment_left(it);
        it->c[k - 1] += (it->c[k - 2] + 1) - it->n;
    }
}

static void orc_iter_begin(orc_iter *it, int n, int k, int offset) /* Distribution.h:96-103 */
{
    it->n = n;
    it->k = k;
    for (int i = 0; i < k; ++i) it->c[i] = i;
    orc_increment(it, offset);
}

static int orc_iter_valid(const orc_iter *it) /* it < end(): end has c[0] = n (Distribution.h:194-199) */
{
    return it->c[0] < it->n;
}

/* Enumerate the prefixes a Distribution(n, k, step, offset) owns into
 * out[count*k]; returns the count (or the count needed if > cap). */
long orc_distribution_prefixes(int n, int k, int step, int offset, int32_t *out, long cap)
{
    orc_iter it;
    long cnt = 0;
    if (k < 1 || k > ORC_MAX_ORDER) return -1;
    for (orc_iter_begin(&it, n, k, offset); orc_iter_valid(&it); orc_increment(&it, step)) {
        if (cnt < cap)
            for (int i = 0; i < k; ++i) out[cnt * k + i] = it.c[i];
        ++cnt;
    }
    return cnt;
}

/* ------------------------------------------------------------------------ */
/* MaxArray<Result<int,float>>::add (include/fiuncho/utils/MaxArray.h:31-46):
 * fills up to capacity, then replaces the first minimum only when the new value
 * is strictly greater.  `val` is the ranking key (float for the reference
 * arithmetic, the double is carried along). */
typedef struct {
    int32_t c[ORC_MAX_ORDER];
    float val;
    double val64;
} orc_result;

typedef struct {
    orc_result *a;
    size_t cap, size, min_pos;
} orc_maxarray;

static void orc_max_add(orc_maxarray *m, const orc_result *r, int by64)
{
    if (m->size < m->cap) {
        m->a[m->size] = *r;
        const orc_result *mn = &m->a[m->min_pos];
        if (by64 ? (r->val64 < mn->val64) : (r->val < mn->val)) m->min_pos = m->size;
        m->size++;
    } else if (m->cap && (by64 ? (r->val64 > m->a[m->min_pos].val64) : (r->val > m->a[m->min_pos].val))) {
        m->a[m->min_pos] = *r;
        size_t mp = 0;
        for (size_t i = 1; i < m->cap; ++i)
            if (by64 ? (m->a[i].val64 < m->a[mp].val64) : (m->a[i].val < m->a[mp].val)) mp = i;
        m->min_pos = mp;
    }
}

/* ------------------------------------------------------------------------ */
/* The search: ThreadedSearch::nonsegmented_search + run
 * (include/fiuncho/ThreadedSearch.h:142-182, 207-246).  Each thread owns
 * distribution.layer(nthreads, t) (Distribution.h:172-176) of the
 * (order-1)-prefixes, builds the prefix table with chained combine
 * (ThreadedSearch.h:160-164) and runs the last-SNP loop (ThreadedSearch.h:169-180)
 * with combine_and_popcnt + MI + MaxArray::add.  mi_mode 0 ranks by the
 * reference FP32 MI, mi_mode 1 by the FP64 MI. */
typedef struct {
    const uint64_t *data;
    size_t snps, n_cases, n_ctrls, cw, tw;
    int order, n, step, offset, mi_mode;
    orc_maxarray max;
    uint64_t combos;
    int digest_mode; /* 1: add each table's digest term (ref/tabledigest.h) instead of ranking */
    uint64_t digest;
} orc_thread_args;

static void *orc_thread_main(void *p)
{
    orc_thread_args *a = (orc_thread_args *)p;
    const int order = a->order, k = order - 1;
    const size_t per_snp = 3 * (a->cw + a->tw);
    size_t rows = 1;
    for (int i = 0; i < order - 1; ++i) rows *= 3;
    /* prefix tables of order 2..order-1 for each class */
    uint64_t *gc[ORC_MAX_ORDER] = {0}, *gt[ORC_MAX_ORDER] = {0};
    size_t r = 3;
    for (int o = 2; o < order; ++o) {
        r *= 3;
        gc[o] = (uint64_t *)malloc(r * a->cw * sizeof(uint64_t) + 8);
        gt[o] = (uint64_t *)malloc(r * a->tw * sizeof(uint64_t) + 8);
    }
    const size_t cells = rows * 3;
    uint32_t *ctc = (uint32_t *)malloc(cells * sizeof(uint32_t)), *ctt = (uint32_t *)malloc(cells * sizeof(uint32_t));
    orc_iter it;
    for (orc_iter_begin(&it, a->n, k, a->offset); orc_iter_valid(&it); orc_increment(&it, a->step)) {
        const uint64_t *pc = a->data + (size_t)it.c[0] * per_snp, *pt = pc + 3 * a->cw;
        size_t sz = 3;
        for (int o = 2; o < order; ++o) { /* ThreadedSearch.h:160-164 */
            const uint64_t *sc = a->data + (size_t)it.c[o - 1] * per_snp, *st = sc + 3 * a->cw;
            orc_combine(pc, sz, sc, a->cw, gc[o]);
            orc_combine(pt, sz, st, a->tw, gt[o]);
            pc = gc[o];
            pt = gt[o];
            sz *= 3;
        }
        for (int l = it.c[k - 1] + 1; l < (int)a->snps; ++l) { /* ThreadedSearch.h:169-180 */
            const uint64_t *lc = a->data + (size_t)l * per_snp, *lt = lc + 3 * a->cw;
            orc_popcnt(pc, sz, lc, a->cw, ctc, cells);
            orc_popcnt(pt, sz, lt, a->tw, ctt, cells);
            if (a->digest_mode) {
                int cmb[ORC_MAX_ORDER];
                for (int i = 0; i < k; ++i) cmb[i] = it.c[i];
                cmb[k] = l;
                a->digest += td_term(cmb, order, a->snps, ctc, ctt, (int)cells);
                a->combos++;
                continue;
            }
            orc_result res;
            memset(&res, 0, sizeof(res));
            for (int i = 0; i < k; ++i) res.c[i] = it.c[i];
            res.c[k] = l;
            if (a->mi_mode == 0) {
                res.val = orc_mi_f32(ctc, ctt, cells, (uint32_t)a->n_cases, (uint32_t)a->n_ctrls);
                res.val64 = res.val;
            } else {
                res.val64 = orc_mi_f64(ctc, ctt, cells, (uint32_t)a->n_cases, (uint32_t)a->n_ctrls);
                res.val = (float)res.val64;
            }
            orc_max_add(&a->max, &res, a->mi_mode == 1);
            a->combos++;
        }
    }
    for (int o = 2; o < order; ++o) { free(gc[o]); free(gt[o]); }
    free(ctc);
    free(ctt);
    return NULL;
}

/* Final ordering: descending value (ThreadedSearch.h:241-245 sorts by value
 * only and leaves ties unordered); ties here are broken by ascending
 * lexicographic combination so that the oracle is deterministic. */
static int g_cmp_order;
static int g_cmp_by64;
static int orc_cmp_desc(const void *x, const void *y)
{
    const orc_result *a = (const orc_result *)x, *b = (const orc_result *)y;
    if (g_cmp_by64) {
        if (a->val64 > b->val64) return -1;
        if (a->val64 < b->val64) return 1;
    } else {
        if (a->val > b->val) return -1;
        if (a->val < b->val) return 1;
    }
    for (int i = 0; i < g_cmp_order; ++i) {
        if (a->c[i] < b->c[i]) return -1;
        if (a->c[i] > b->c[i]) return 1;
    }
    return 0;
}

static pthread_mutex_t g_sort_lock = PTHREAD_MUTEX_INITIALIZER;

/* Returns the number of results written (<= outputs) or a negative error.
 * out_combos[outputs*order], out_vals (float), out_vals64 (double, may be NULL).
 * combos_done (may be NULL) receives the number of combinations evaluated. */
long orc_search(const uint64_t *data, size_t snps, size_t n_cases, size_t n_ctrls, size_t cases_words,
                size_t ctrls_words, int order, int dist_n, int dist_step, int dist_offset, int nthreads,
                unsigned outputs, int mi_mode, int32_t *out_combos, float *out_vals, double *out_vals64,
                uint64_t *combos_done)
{
    if (order < 2 || order > ORC_MAX_ORDER || nthreads < 1 || dist_step < 1) return -1;
    orc_thread_args *args = (orc_thread_args *)calloc((size_t)nthreads, sizeof(orc_thread_args));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        orc_thread_args *a = &args[t];
        a->data = data;
        a->snps = snps;
        a->n_cases = n_cases;
        a->n_ctrls = n_ctrls;
        a->cw = cases_words;
        a->tw = ctrls_words;
        a->order = order;
        a->n = dist_n;
        a->step = dist_step * nthreads;              /* Distribution::layer (Distribution.h:172-176) */
        a->offset = dist_offset * nthreads + t;
        a->mi_mode = mi_mode;
        a->max.a = (orc_result *)calloc(outputs ? outputs : 1, sizeof(orc_result));
        a->max.cap = outputs;
        pthread_create(&th[t], NULL, orc_thread_main, a);
    }
    size_t total = 0;
    uint64_t combos = 0;
    for (int t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        total += args[t].max.size;
        combos += args[t].combos;
    }
    orc_result *all = (orc_result *)calloc(total ? total : 1, sizeof(orc_result));
    size_t pos = 0;
    for (int t = 0; t < nthreads; ++t) {
        memcpy(all + pos, args[t].max.a, args[t].max.size * sizeof(orc_result));
        pos += args[t].max.size;
        free(args[t].max.a);
    }
    pthread_mutex_lock(&g_sort_lock);
    g_cmp_order = order;
    g_cmp_by64 = mi_mode == 1;
    qsort(all, total, sizeof(orc_result), orc_cmp_desc);
    pthread_mutex_unlock(&g_sort_lock);
    const size_t nout = total < outputs ? total : outputs;
    for (size_t i = 0; i < nout; ++i) {
        for (int j = 0; j < order; ++j) out_combos[i * order + j] = all[i].c[j];
        out_vals[i] = all[i].val;
        if (out_vals64) out_vals64[i] = all[i].val64;
    }
    free(all);
    free(args);
    free(th);
    if (combos_done) *combos_done = combos;
    return (long)nout;
}

/* ------------------------------------------------------------------------ */
/* Contingency tables of arbitrary combinations (sampled parity checks): for
 * combination q (order ascending SNP indices in combos[q*order..]) write 3^order
 * cells per class into cases_out/ctrls_out[q*3^order ..], built with chained
 * combine + combine_and_popcnt exactly as the search does. */
int orc_tables(const uint64_t *data, size_t cases_words, size_t ctrls_words, int order, const int32_t *combos,
               size_t count, uint32_t *cases_out, uint32_t *ctrls_out)
{
    if (order < 2 || order > ORC_MAX_ORDER) return -1;
    const size_t per_snp = 3 * (cases_words + ctrls_words);
    size_t cells = 1;
    for (int i = 0; i < order; ++i) cells *= 3;
    uint64_t *bufc[2], *buft[2];
    for (int b = 0; b < 2; ++b) {
        bufc[b] = (uint64_t *)malloc(cells / 3 * cases_words * sizeof(uint64_t) + 8);
        buft[b] = (uint64_t *)malloc(cells / 3 * ctrls_words * sizeof(uint64_t) + 8);
    }
    for (size_t q = 0; q < count; ++q) {
        const int32_t *c = combos + q * (size_t)order;
        const uint64_t *pc = data + (size_t)c[0] * per_snp, *pt = pc + 3 * cases_words;
        size_t sz = 3;
        for (int o = 1; o < order - 1; ++o) {
            const uint64_t *sc = data + (size_t)c[o] * per_snp, *st = sc + 3 * cases_words;
            orc_combine(pc, sz, sc, cases_words, bufc[o & 1]);
            orc_combine(pt, sz, st, ctrls_words, buft[o & 1]);
            pc = bufc[o & 1];
            pt = buft[o & 1];
            sz *= 3;
        }
        const uint64_t *lc = data + (size_t)c[order - 1] * per_snp, *lt = lc + 3 * cases_words;
        orc_popcnt(pc, sz, lc, cases_words, cases_out + q * cells, cells);
        orc_popcnt(pt, sz, lt, ctrls_words, ctrls_out + q * cells, cells);
    }
    for (int b = 0; b < 2; ++b) { free(bufc[b]); free(buft[b]); }
    return 0;
}

/* MI of a batch of tables, both arithmetics (for MutualInformation::compute
 * parity): tables are `size` cells per class, count tables. */
void orc_mi_batch(const uint32_t *cases, const uint32_t *ctrls, size_t size, size_t count, uint32_t n_cases,
                  uint32_t n_ctrls, float *out32, double *out64)
{
    for (size_t q = 0; q < count; ++q) {
        if (out32) out32[q] = orc_mi_f32(cases + q * size, ctrls + q * size, size, n_cases, n_ctrls);
        if (out64) out64[q] = orc_mi_f64(cases + q * size, ctrls + q * size, size, n_cases, n_ctrls);
    }
}

/* ------------------------------------------------------------------------ */
/* Digest (ref/tabledigest.h) of the tables of every combination that
 * orc_search would visit for the same distribution and threads, built by the
 * same combine / popcnt chain (ThreadedSearch.h:157-180).  Returns the number
 * of combinations hashed, or a negative error. */
long orc_table_digest(const uint64_t *data, size_t snps, size_t cases_words, size_t ctrls_words, int order,
                      int dist_n, int dist_step, int dist_offset, int nthreads, uint64_t *digest)
{
    if (order < 2 || order > ORC_MAX_ORDER || nthreads < 1 || dist_step < 1) return -1;
    orc_thread_args *args = (orc_thread_args *)calloc((size_t)nthreads, sizeof(orc_thread_args));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        orc_thread_args *a = &args[t];
        a->data = data;
        a->snps = snps;
        a->cw = cases_words;
        a->tw = ctrls_words;
        a->order = order;
        a->n = dist_n;
        a->step = dist_step * nthreads;
        a->offset = dist_offset * nthreads + t;
        a->digest_mode = 1;
        pthread_create(&th[t], NULL, orc_thread_main, a);
    }
    uint64_t sum = 0, combos = 0;
    for (int t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        sum += args[t].digest;
        combos += args[t].combos;
    }
    free(args);
    free(th);
    *digest = sum;
    return (long)combos;
}

/* ------------------------------------------------------------------------ */
/* The depth-first traversal of the reference's sequential benchmark programs
 * (stack_search in benchmarks/nonsegmented_sequential_search.cpp:31-104 and
 * benchmarks/segmented_sequential_search.cpp:31-117): for each first SNP i
 * ascending, the pairs (i, j) go onto a stack with j ascending; a popped
 * combination shorter than the order gets its genotype table (combine of its
 * parent's table with its last SNP) and pushes its children (last SNP + 1 ..
 * n - 1, ascending); a popped combination of full order is counted
 * (combine_and_popcnt of its parent's table with its last SNP).  So the
 * combinations are visited first SNP ascending, the rest in descending
 * lexicographic order.  The segmented program collects `block` tables before
 * computing their MI and feeding the MaxArray in visiting order (block = 1 is
 * the non-segmented program; the benchmarks use 1 474 560 / 3^order).
 * mi_mode as in orc_search.  Returns the number of results written. */
typedef struct {
    int size;
    int32_t pos[ORC_MAX_ORDER];
} orc_node;

long orc_search_dfs(const uint64_t *data, size_t snps, size_t n_cases, size_t n_ctrls, size_t cw, size_t tw,
                    int order, size_t block, unsigned outputs, int mi_mode, int32_t *out_combos, float *out_vals,
                    double *out_vals64, uint64_t *combos_done)
{
    if (order < 2 || order > ORC_MAX_ORDER || block < 1 || snps < 2) return -1;
    const size_t per_snp = 3 * (cw + tw);
    size_t cells = 1;
    for (int i = 0; i < order; ++i) cells *= 3;
    /* genotype table of the combination of size s on the current path: rows 3^s */
    uint64_t *gc[ORC_MAX_ORDER + 1] = {0}, *gt[ORC_MAX_ORDER + 1] = {0};
    size_t rows = 3;
    for (int s = 2; s < order; ++s) {
        rows *= 3;
        gc[s] = (uint64_t *)malloc(rows * cw * sizeof(uint64_t) + 8);
        gt[s] = (uint64_t *)malloc(rows * tw * sizeof(uint64_t) + 8);
    }
    /* at most (order - 1) levels of at most snps children each are stacked at once */
    const size_t stack_cap = snps * (size_t)order;
    orc_node *stack = (orc_node *)malloc(stack_cap * sizeof(orc_node));
    uint32_t *bc = (uint32_t *)malloc(block * cells * sizeof(uint32_t));
    uint32_t *bt = (uint32_t *)malloc(block * cells * sizeof(uint32_t));
    orc_result *br = (orc_result *)calloc(block, sizeof(orc_result));
    orc_maxarray max = {(orc_result *)calloc(outputs ? outputs : 1, sizeof(orc_result)), outputs, 0, 0};
    size_t top = 0, filled = 0;
    uint64_t combos = 0;
    long rc = 0;
    for (int i = 0; i < (int)snps && rc == 0; ++i) {
        for (int j = i + 1; j < (int)snps; ++j) {
            orc_node nd;
            memset(&nd, 0, sizeof(nd));
            nd.size = 2;
            nd.pos[0] = i;
            nd.pos[1] = j;
            stack[top++] = nd;
        }
        while (top > 0) {
            const orc_node nd = stack[--top];
            const int s = nd.size, last = nd.pos[s - 1];
            /* the parent's table: SNP pos[0] itself for a pair, else the path's table of size s - 1 */
            const uint64_t *pc = s == 2 ? data + (size_t)nd.pos[0] * per_snp : gc[s - 1];
            const uint64_t *pt = s == 2 ? pc + 3 * cw : gt[s - 1];
            size_t prow = 1;
            for (int q = 1; q < s; ++q) prow *= 3;
            const uint64_t *lc = data + (size_t)last * per_snp, *lt = lc + 3 * cw;
            if (s == order) {
                orc_popcnt(pc, prow, lc, cw, bc + filled * cells, cells);
                orc_popcnt(pt, prow, lt, tw, bt + filled * cells, cells);
                memset(&br[filled], 0, sizeof(orc_result));
                for (int q = 0; q < order; ++q) br[filled].c[q] = nd.pos[q];
                if (++filled == block) {
                    for (size_t b = 0; b < filled; ++b) {
                        const uint32_t *tc = bc + b * cells, *tt = bt + b * cells;
                        if (mi_mode == 0) {
                            br[b].val = orc_mi_f32(tc, tt, cells, (uint32_t)n_cases, (uint32_t)n_ctrls);
                            br[b].val64 = br[b].val;
                        } else {
                            br[b].val64 = orc_mi_f64(tc, tt, cells, (uint32_t)n_cases, (uint32_t)n_ctrls);
                            br[b].val = (float)br[b].val64;
                        }
                        orc_max_add(&max, &br[b], mi_mode == 1);
                    }
                    combos += filled;
                    filled = 0;
                }
            } else {
                orc_combine(pc, prow, lc, cw, gc[s]);
                orc_combine(pt, prow, lt, tw, gt[s]);
                if (top + snps > stack_cap) {
                    rc = -2;
                    break;
                }
                for (int l = last + 1; l < (int)snps; ++l) {
                    orc_node ch = nd;
                    ch.size = s + 1;
                    ch.pos[s] = l;
                    stack[top++] = ch;
                }
            }
        }
    }
    for (size_t b = 0; b < filled; ++b) { /* the last, partial block */
        const uint32_t *tc = bc + b * cells, *tt = bt + b * cells;
        if (mi_mode == 0) {
            br[b].val = orc_mi_f32(tc, tt, cells, (uint32_t)n_cases, (uint32_t)n_ctrls);
            br[b].val64 = br[b].val;
        } else {
            br[b].val64 = orc_mi_f64(tc, tt, cells, (uint32_t)n_cases, (uint32_t)n_ctrls);
            br[b].val = (float)br[b].val64;
        }
        orc_max_add(&max, &br[b], mi_mode == 1);
    }
    combos += filled;
    for (int s = 2; s < order; ++s) { free(gc[s]); free(gt[s]); }
    free(stack);
    free(bc);
    free(bt);
    free(br);
    if (rc) {
        free(max.a);
        return rc;
    }
    pthread_mutex_lock(&g_sort_lock);
    g_cmp_order = order;
    g_cmp_by64 = mi_mode == 1;
    qsort(max.a, max.size, sizeof(orc_result), orc_cmp_desc);
    pthread_mutex_unlock(&g_sort_lock);
    const size_t nout = max.size < outputs ? max.size : outputs;
    for (size_t i = 0; i < nout; ++i) {
        for (int j = 0; j < order; ++j) out_combos[i * order + j] = max.a[i].c[j];
        out_vals[i] = max.a[i].val;
        if (out_vals64) out_vals64[i] = max.a[i].val64;
    }
    free(max.a);
    if (combos_done) *combos_done = combos;
    return (long)nout;
}
