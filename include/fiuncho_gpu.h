/*
 * fiuncho_gpu.h -- C ABI of the GB300 (sm_103a) exhaustive epistasis search.
 *
 * Plain pointers and sizes only.  A maintainer binds these from the reference
 * tree's C++ (include/fiuncho/GpuSearch.h in this repository shows the
 * Search-derived class), from Python (ctypes) or from any FFI.
 *
 * Data layout accepted everywhere (identical to the reference's
 * GenotypeTable<uint64_t>::make_array, include/fiuncho/GenotypeTable.h:77-103):
 * SNP-major; per SNP 3 case rows of `cases_words` uint64 followed by 3 control
 * rows of `ctrls_words` uint64; row g holds bit "minor-allele count == g".
 *
 * Results follow Search::run (include/fiuncho/Search.h:40-43): at most
 * `outputs` combinations of `order` ascending 0-based SNP indices, sorted by
 * mutual information (natural log) in descending order; equal values are
 * ordered by ascending combination so that the output is deterministic.
 *
 * Every function returns FIU_OK (0) or an FIU_ERR_* code; the message of the
 * last failure of a context is fiu_last_error(ctx).  A context is used from
 * one host thread at a time.
 */
#ifndef FIUNCHO_GPU_H
#define FIUNCHO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIU_OK 0
#define FIU_ERR_INVALID 1     /* invalid argument (sizes, order, distribution, pointers) */
#define FIU_ERR_NOMEM 2       /* device or host allocation failed / over the memory budget */
#define FIU_ERR_CUDA 3        /* CUDA runtime error (message in fiu_last_error) */
#define FIU_ERR_UNSUPPORTED 4 /* valid request outside this build's limits */
#define FIU_ERR_TIMEOUT 5     /* a device wait ran past its limit */
#define FIU_ERR_CANCELLED 6   /* request cancelled */

#define FIU_MAX_ORDER 8       /* highest interaction order supported */

/* Counting kernels (fiu_set_kernel, fiu_scan_tables). */
#define FIU_KERNEL_AUTO 0        /* pick per request (default) */
#define FIU_KERNEL_FULL 1        /* all 3^order cells, any data, orders 2..8 */
#define FIU_KERNEL_ELIDED_POPC 2 /* one-hot data, orders 2-4: 2^order cells + exact marginals, POPC
                                    (order 4 over the whole data set: pair-major schedule) */
#define FIU_KERNEL_ELIDED_HS 3   /* as 2, Harley-Seal carry-save counting on the ALU pipe */
#define FIU_KERNEL_TENSOR 4      /* one-hot data, order 2, 3 or 4, whole data set: core cells on tcgen05 (e4m3, FP32 accumulate) */
#define FIU_MAX_OUTPUTS 7000  /* largest top-N supported */

typedef struct fiu_ctx fiu_ctx;           /* one per device per host thread */
typedef struct fiu_resident fiu_resident; /* a data set held in device memory */

/* Host view of Dataset<uint64_t> (include/fiuncho/Dataset.h:26-152). */
typedef struct {
    const uint64_t *data;  /* snps * 3 * (cases_words + ctrls_words) words, reference layout */
    uint64_t snps;         /* Dataset::snps */
    uint64_t cases;        /* Dataset::cases */
    uint64_t ctrls;        /* Dataset::ctrls */
    uint64_t cases_words;  /* GenotypeTable::cases_words */
    uint64_t ctrls_words;  /* GenotypeTable::ctrls_words */
} fiu_dataset;

/* Distribution<int>(n, k, step, offset) (include/fiuncho/Distribution.h:147-152):
 * the (order-1)-SNP prefixes of lexicographic rank offset, offset+step, ...
 * For one process that is (snps, order-1, 1, 0) (include/fiuncho/MPIEngine.h:133-134). */
typedef struct {
    int32_t n;
    int32_t k;
    int32_t step;
    int32_t offset;
} fiu_distribution;

/* ---- context -------------------------------------------------------------- */
/* Creates a context on CUDA device `device` (its own stream and scratch). */
int fiu_create(int device, fiu_ctx **out);
void fiu_destroy(fiu_ctx *ctx);
/* ctx NULL: the message of this thread's last failed call made without a
 * context (fiu_read_genotypes). */
const char *fiu_last_error(const fiu_ctx *ctx);
/* Sum of the GPU-side launches made by this context since creation (kernels of
 * this library only); used to report how many launches a timed region made. */
uint64_t fiu_launch_count(const fiu_ctx *ctx);

/* The context's CUDA stream (a cudaStream_t), on which every kernel of the
 * context is launched; callers may record events on it. */
void *fiu_stream(const fiu_ctx *ctx);
/* Per-context timing of the search's counting kernels with CUDA events on the
 * context's stream (off by default).  fiu_kernel_timing returns the summed
 * duration, the number of counting launches and the number of combinations
 * they evaluated since timing was (re)enabled. */
int fiu_set_kernel_timing(fiu_ctx *ctx, int enable);
int fiu_kernel_timing(const fiu_ctx *ctx, double *count_ms, uint64_t *count_launches, uint64_t *combinations);
/* Measures this GPU's sustained 32-bit AND+POPC+ADD rate (word-ops per second)
 * with a short in-bounds kernel; the integer-pipe peak for roofline reports. */
int fiu_probe_popc_rate(fiu_ctx *ctx, double *word_ops_per_s);
/* Self-check of the tensor kernels' threshold prefilter: the largest absolute
 * error, against double precision, of the single-precision log2 it uses, over
 * every input it can see (x = c + 2^-20 rounded to float, integer counts c in
 * [0, max_c]).  The prefilter's error bound assumes it stays below 2^-18. */
int fiu_probe_lg2_error(fiu_ctx *ctx, unsigned max_c, double *max_abs_err);
/* Self-check of the bounded device waits (the failure detection of the
 * tensor kernels, which report FIU_ERR_TIMEOUT when a wait runs out): a
 * one-thread kernel waits, with a limit of limit_us (at most 1 s), on an
 * mbarrier phase that nothing completes -- or, with arrive != 0, that the
 * thread completes itself first.  *completed = 1 if the phase completed,
 * 0 if the wait gave up; *elapsed_ms = time spent waiting.  No GPU fault
 * and no hang either way: the wait always ends. */
int fiu_probe_wait_limit(fiu_ctx *ctx, unsigned limit_us, int arrive, int *completed, double *elapsed_ms);

/* Forces a counting kernel for this context's searches (FIU_KERNEL_*);
 * FIU_KERNEL_AUTO restores the automatic choice.  A kernel that cannot serve a
 * request (e.g. an elided kernel on data that is not one-hot) makes the search
 * fail with FIU_ERR_UNSUPPORTED. */
int fiu_set_kernel(fiu_ctx *ctx, int kernel);

/* Autotuning of the counting kernel's variant and l-tile width (threads per
 * prefix: 32, 64, 128 or 256) on a sample of each large request (default on;
 * results never depend on it).  fiu_last_tile reports the kernel and width the
 * last single-scan search used. */
int fiu_set_autotune(fiu_ctx *ctx, int enable);
int fiu_last_tile(const fiu_ctx *ctx, int *kernel, int *tp);

/* ---- data sets -------------------------------------------------------------- */
/* Copies a host data set to the device (Dataset<uint64_t>::read output ->
 * device buffers) and derives the device layouts the kernels read. */
int fiu_dataset_upload(fiu_ctx *ctx, const fiu_dataset *host, fiu_resident **out);
void fiu_dataset_free(fiu_ctx *ctx, fiu_resident *res);
/* ---- ingest: genotype files -> codes -> packed on the device -----------------
 * fiu_read_genotypes replaces Dataset<uint64_t>::read's parsing
 * (include/fiuncho/Dataset.h:48-94 with TPEDFile.hpp:72-296 / RAWFile.hpp:18-313):
 * one .raw file, or a .tped + .tfam pair in either order (f2 NULL for .raw),
 * parsed by `threads` host threads (<= 0: all cores) into minor-allele
 * counts (snps x samples, SNP-major) and per-sample case flags, with the
 * reference's input rules and error messages (the first failing line of the
 * file).  ctx may be NULL: the message is then fiu_last_error(NULL). */
typedef struct fiu_genotypes fiu_genotypes;
int fiu_read_genotypes(fiu_ctx *ctx, const char *f1, const char *f2, int threads, fiu_genotypes **out);
/* Sizes and host arrays of parsed genotypes (valid until fiu_genotypes_free). */
int fiu_genotypes_info(const fiu_genotypes *g, uint64_t *snps, uint64_t *samples, const uint8_t **codes,
                       const uint8_t **is_case);
void fiu_genotypes_free(fiu_genotypes *g);
/* A resident data set from genotype codes (snps x samples, values 0..2; other
 * values match no row) and case flags: the codes are copied to the device and
 * packed there into the reference layout (TPEDFile.hpp:176-269: per class,
 * samples in file order, most-significant bit first, the last word
 * right-aligned, unaligned rows), then prepared as by fiu_dataset_upload. */
int fiu_dataset_upload_genotypes(fiu_ctx *ctx, const uint8_t *codes, const uint8_t *is_case, uint64_t snps,
                                 uint64_t samples, fiu_resident **out);
/* Layout of a resident data set (desc, data pointer NULL) and, when data is
 * not NULL, a copy of its packed words (snps * 3 * (cases_words + ctrls_words)). */
int fiu_dataset_packed(fiu_ctx *ctx, const fiu_resident *res, fiu_dataset *desc, uint64_t *data);

/* 1 when every SNP's three rows are disjoint, cover each class exactly and
 * padding words are zero (the reference's own invariant, tests/dataset.cpp:25-44). */
int fiu_dataset_is_one_hot(const fiu_resident *res);

/* ---- the search (replaces Search::run, include/fiuncho/Search.h:40-43,
 *      as implemented by ThreadedSearch::run, include/fiuncho/ThreadedSearch.h:207-246) */
/* Host data set in, results out: upload + search + release, all inside. */
int fiu_search(fiu_ctx *ctx, const fiu_dataset *dataset, unsigned order, const fiu_distribution *distribution,
               unsigned outputs, int32_t *out_combinations /* outputs*order */, float *out_vals /* outputs */,
               unsigned *out_count);
/* Same on a resident data set. */
int fiu_search_resident(fiu_ctx *ctx, const fiu_resident *res, unsigned order,
                        const fiu_distribution *distribution, unsigned outputs, int32_t *out_combinations,
                        float *out_vals, unsigned *out_count);
/* As fiu_search_resident and also returns the FP64 MI of each result. */
int fiu_search_resident64(fiu_ctx *ctx, const fiu_resident *res, unsigned order,
                          const fiu_distribution *distribution, unsigned outputs, int32_t *out_combinations,
                          float *out_vals, double *out_vals64, unsigned *out_count);
/* One shard of the whole search (Distribution(snps, order-1, 1, 0)): shard
 * `shard` of `n_shards` contiguous, equal ranges of the work units of the
 * kernel that serves the whole data set (tensor-core work items, pair-major
 * items, or prefix ordinals).  The shards cover every combination exactly
 * once, so each GPU of a multi-GPU search keeps the whole-data-set kernels
 * (where MPIEngine.h:133-174 gives rank r the strided Distribution(snps,
 * order-1, N, r)); merging the shards' results by (MI descending,
 * combination ascending) and truncating gives the whole search's result. */
int fiu_search_shard(fiu_ctx *ctx, const fiu_dataset *dataset, unsigned order, unsigned shard, unsigned n_shards,
                     unsigned outputs, int32_t *out_combinations, float *out_vals, unsigned *out_count);
int fiu_search_shard_resident64(fiu_ctx *ctx, const fiu_resident *res, unsigned order, unsigned shard,
                                unsigned n_shards, unsigned outputs, int32_t *out_combinations, float *out_vals,
                                double *out_vals64, unsigned *out_count);

/* ---- many scans at once (batched form) ---------------------------------------
 * Each scan is a search of its own resident data set with its own order,
 * distribution and top-N; the scans progress together on the device in
 * rounds (one persistent launch over every scan's next chunk of prefixes, then
 * an on-device top-N selection per scan), optionally as one CUDA graph.
 * Results are identical to fiu_search_resident on each scan alone. */
typedef struct {
    const fiu_resident *res;         /* in: resident data set */
    unsigned order;                  /* in: interaction order */
    fiu_distribution distribution;   /* in: k must be order-1 */
    unsigned outputs;                /* in: top-N */
    int32_t *out_combinations;       /* out (host): outputs * order */
    float *out_vals;                 /* out (host): outputs */
    double *out_vals64;              /* out (host, optional): outputs */
    unsigned out_count;              /* out: results written */
    int status;                      /* out: FIU_OK or FIU_ERR_* of this scan */
    unsigned shard, n_shards;        /* in: search shard `shard` of `n_shards` of the scan's work
                                        units, as fiu_search_shard (n_shards 0 or 1: all of it;
                                        with n_shards > 1 the distribution must be the whole
                                        data set's) */
} fiu_scan;
/* use_graph: 1 = capture the rounds into a CUDA graph and launch it once.
 * Returns FIU_OK when every scan ran (see each scan's status). */
int fiu_search_batch(fiu_ctx *ctx, fiu_scan *scans, unsigned n_scans, int use_graph);

/* ---- served request stream (continuous batching) --------------------------------
 * A server owns one device context and one worker thread.  Submitted scans
 * (host data copied at submit) wait in a queue until their device footprint
 * fits the memory budget; admitted scans keep their data set, candidate
 * buffers and running top-N resident and progress in rounds shared with every
 * other admitted scan, so a scan that arrives while others run starts in the
 * next round.  Scans that run best alone (tensor-core and pair-major order-4
 * scans) take one of two solo lanes (a worker thread with its own stream
 * each), concurrent with each other and with the rounds.
 * Each scan's result is identical to fiu_search on it alone.
 * Thread-safe: submit/poll/stats may be called from any thread. */
typedef struct fiu_server fiu_server;
typedef struct {
    uint64_t submitted, completed, failed, queued, active;
    uint64_t rounds;              /* rounds executed */
    uint64_t bytes_in_use;        /* device bytes held by admitted scans */
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> result latency of completed scans */
    double combos_samples;        /* combinations x samples completed */
    uint64_t solo;                /* scans run alone on a solo lane (tensor-core and pair-major
                                     order-4 scans, full-table scans above order 4), on the
                                     lane's own stream beside the rounds */
    uint64_t overlapped;          /* completed scans whose device work overlapped another
                                     scan's (either lane) */
    uint64_t peak_bytes;          /* largest bytes_in_use so far (never above the budget, except
                                     for one scan larger than the budget left, run alone) */
} fiu_serve_stats;
/* budget_bytes: device memory the admitted scans may hold (0 = 120 GB): a scan
 * is admitted -- its data set uploaded -- when its footprint fits what the
 * admitted scans leave, whichever lane then runs it; scans larger than the
 * whole budget are rejected at submit. */
int fiu_server_create(int device, uint64_t budget_bytes, fiu_server **out);
/* Order in which queued scans are admitted and the solo lanes take them:
 * FIU_SERVE_FIFO (the default: submission order) or FIU_SERVE_SHORTEST_FIRST
 * (least combinations x samples first, submission order among equals).  Under
 * an offered load above the device's throughput shortest-first completes the
 * small scans with short latency while the largest wait; FIFO bounds every
 * scan's wait by the work submitted before it.  Applies to scans not yet
 * taken. */
#define FIU_SERVE_FIFO 0
#define FIU_SERVE_SHORTEST_FIRST 1
int fiu_server_set_policy(fiu_server *srv, int policy);
/* Queues a scan of the whole data set (Distribution(snps, order-1, 1, 0)). */
int fiu_server_submit(fiu_server *srv, const fiu_dataset *dataset, unsigned order, unsigned outputs,
                      uint64_t *ticket);
/* Queues shard `shard` of `n_shards` of such a scan (as fiu_search_shard). */
int fiu_server_submit_shard(fiu_server *srv, const fiu_dataset *dataset, unsigned order, unsigned outputs,
                            unsigned shard, unsigned n_shards, uint64_t *ticket);
/* Waits up to wait_ms (0 = do not wait, < 0 = forever) for a ticket; FIU_OK and
 * the results once done (the ticket is then released), FIU_ERR_TIMEOUT if not
 * yet done, the scan's error code if it failed, FIU_ERR_INVALID for an unknown
 * ticket.  latency_ms (optional) receives submit-to-result time. */
int fiu_server_poll(fiu_server *srv, uint64_t ticket, int wait_ms, int32_t *out_combinations, float *out_vals,
                    double *out_vals64, unsigned *out_count, double *latency_ms);
int fiu_server_stats(fiu_server *srv, fiu_serve_stats *out);
/* Stops the worker after the current round and cancels the scans running on
 * the solo lanes after their current chunk; pending scans are dropped. */
void fiu_server_destroy(fiu_server *srv);

/* ---- kernel-level entries ------------------------------------------------------- */
/* GenotypeTable<uint64_t>::combine (include/fiuncho/GenotypeTable.h:123-124,
 * src/base/gt_combine.cpp:3-27): t1 has size1 rows per class, t2 3 rows per class,
 * out receives 3*size1 rows per class; each table is [cases rows][ctrls rows]. */
int fiu_combine(fiu_ctx *ctx, const uint64_t *t1, unsigned size1, const uint64_t *t2, uint64_t cases_words,
                uint64_t ctrls_words, uint64_t *out);
/* GenotypeTable<uint64_t>::combine_and_popcnt<uint32_t> (GenotypeTable.h:137-140,
 * src/base/gt_popcnt.cpp:4-35): cases_out/ctrls_out receive ct_size cells each;
 * cells from 3*size1 on are zero. */
int fiu_combine_and_popcnt(fiu_ctx *ctx, const uint64_t *t1, unsigned size1, const uint64_t *t2,
                           uint64_t cases_words, uint64_t ctrls_words, uint32_t *cases_out, uint32_t *ctrls_out,
                           unsigned ct_size);
/* MutualInformation<float>(n_cases, n_ctrls).compute (include/fiuncho/algorithms/
 * MutualInformation.h:58-84) over `count` tables of `cells` cells per class.
 * mode 0: the search's fused fixed-point arithmetic; mode 1: FP64. */
int fiu_mi_compute(fiu_ctx *ctx, const uint32_t *cases, const uint32_t *ctrls, size_t cells, size_t count,
                   unsigned n_cases, unsigned n_ctrls, int mode, float *out, double *out64);
/* No counterpart in the reference.  MutualInformation::compute's fixed-point
 * arithmetic (mode 0 of fiu_mi_compute, bit-identical results) for callers
 * that cannot allocate device memory at run time (a host that has handed all
 * GPU memory to its own pool, a pipeline that cannot take cudaMalloc's
 * device-wide synchronisation, a plugin host owning the memory policy).
 * Allocates nothing: tables and outputs are the caller's device buffers
 * (d_cases/d_ctrls: count x cells uint32 each, d_out: count floats), and the
 * only scratch is a library-owned static device table of c ln c values sized
 * for n_cases + n_ctrls <= FIU_NOALLOC_MAX_SAMPLES (512 KiB per GPU that loads
 * the library, kept until exit); larger requests return FIU_ERR_UNSUPPORTED.
 * Work is enqueued on `stream` (a cudaStream_t, NULL = legacy default stream)
 * and not waited for.  Set-up: the first call on a device -- and the first
 * after the device's context changed, e.g. after cudaDeviceReset, which
 * discards the table -- looks up the table's device address with that device
 * current and fills it with a synchronous 512 KiB copy; make that call before
 * any stream capture.  Calls after the set-up only read the table, so calls
 * may overlap; a set-up that overlaps another call on the same device (in
 * another thread) races with it. */
#define FIU_NOALLOC_MAX_SAMPLES 65536
int fiu_mi_compute_noalloc(const uint32_t *d_cases, const uint32_t *d_ctrls, size_t cells, size_t count,
                           unsigned n_cases, unsigned n_ctrls, float *d_out, void *stream);
/* Contingency tables (3^order cells per class) of given combinations
 * (count x order ascending indices), computed on the device. */
int fiu_tables(fiu_ctx *ctx, const fiu_resident *res, unsigned order, const int32_t *combinations, size_t count,
               uint32_t *cases_out, uint32_t *ctrls_out);
/* The hot kernel's own tables for every combination of a (small) search
 * (kernel = FIU_KERNEL_* + 256 * l-tile width, width 0 = automatic):
 * out[((m * snps) + l) * 2 * 3^order + class * 3^order + cell] for owned
 * prefix ordinal m and last SNP l (entries with l <= prefix end stay as given). */
int fiu_scan_tables(fiu_ctx *ctx, const fiu_resident *res, unsigned order, const fiu_distribution *distribution,
                    int kernel, uint32_t *out, size_t out_words);
/* Digest of every table of a scan, for parity checks at full size.  No
 * counterpart in the reference's API; it checks what combine_and_popcnt
 * (src/base/gt_popcnt.cpp:4-35) gives for every combination ThreadedSearch
 * visits (include/fiuncho/ThreadedSearch.h:157-180) without storing the tables.
 * The kernel `kernel` (FIU_KERNEL_*, FIU_KERNEL_AUTO = the search's own
 * choice; orders <= 4 for FIU_KERNEL_FULL) evaluates every combination of
 * `distribution` (NULL = the whole data set) and
 *   *digest = sum over the combinations c (mod 2^64) of h(c), where
 *   v = c[0] snps^(order-1) + ... + c[order-1]   (uint64, wrapping),
 *   h = mix(v + 0x9E3779B97F4A7C15), then for each cell x in the reference's
 *   cell order (first SNP most significant) h = mix(h ^ (cases[x] << 32 | ctrls[x])),
 *   mix(z): z = (z ^ z >> 30) * 0xBF58476D1CE4E5B9; z = (z ^ z >> 27) * 0x94D049BB133111EB;
 *           z ^ z >> 31  (the SplitMix64 output function);
 * *combinations = the number of combinations hashed.  The same sum over the
 * reference's own tables must come out equal. */
int fiu_scan_digest(fiu_ctx *ctx, const fiu_resident *res, unsigned order, const fiu_distribution *distribution,
                    int kernel, uint64_t *digest, uint64_t *combinations);

#ifdef __cplusplus
}
#endif

#endif
