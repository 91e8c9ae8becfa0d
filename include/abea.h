/*
 * abea.h — C ABI of the GB300-native Adaptive Banded Event Alignment (ABEA).
 *
 * The library replaces f5c's CPU `align()` (prototype in the reference at
 * GPU/f5cmisc.h:48-50) and its batch GPU entry `align_cuda(core, db)`
 * (GPU/f5cmisc.h:99-102), whose OpenCL re-implementation in the reference is
 * `align_ocl(core, db)` (GPU/align_cuda.c:391-943).  All computation runs in
 * hand-written sm_103a CUDA kernels; there is no CPU fallback.  Every entry
 * point takes plain pointers and sizes and never exits the process: failures
 * are reported as negative `abea_status_t` codes plus a thread-local message
 * (`abea_last_error`).
 *
 * Data layouts are byte-identical to the reference's shared types
 * (GPU/f5c.h:113-181) on LP64 targets (x86-64 and aarch64):
 *   abea_event_t        == event_t        (24 B: u64 start, f32 length/mean/stdv, 4 B pad)
 *   abea_event_table_t  == event_table    (n, start, end, event*)
 *   abea_model_t        == model_t        (12 B, CACHED_LOG layout)
 *   abea_scalings_t     == scalings_t     (16 B, CACHED_LOG layout)
 *   abea_aligned_pair_t == AlignedPair    (8 B)
 *   abea_event_kmer_pair_t == EventKmerPair (8 B)
 *   abea_index_pair_t   == index_pair_t   (8 B)
 *   abea_event_alignment_t == event_alignment_t (32 B)
 */
#ifndef ABEA_H
#define ABEA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Algorithm constants: KMER_SIZE, NUM_KMER, ALN_BANDWIDTH (GPU/f5c.h:26-30). */
#define ABEA_KMER_SIZE 6
#define ABEA_NUM_KMER 4096
#define ABEA_BANDWIDTH 100

/* ---- shared types (GPU/f5c.h:113-207) ---------------------------------- */
typedef struct {
    uint64_t start;
    float length;
    float mean;
    float stdv;
} abea_event_t;

typedef struct {
    size_t n;
    size_t start;
    size_t end;
    abea_event_t *event;
} abea_event_table_t;

typedef struct {
    float level_mean;
    float level_stdv;
    float level_log_stdv;
} abea_model_t;

typedef struct {
    float scale;
    float shift;
    float var;
    float log_var;
} abea_scalings_t;

typedef struct {
    int32_t ref_pos;
    int32_t read_pos;
} abea_aligned_pair_t;

typedef struct {
    int32_t event_idx;
    int32_t kmer_idx;
} abea_event_kmer_pair_t;

/* Outputs of f5c's postalign (GPU/f5cmisc.h:51-52): index_pair_t and
 * event_alignment_t (GPU/f5c.h:184-207).  `rc` is the reference's `bool`
 * (one byte); the 32-byte layout is the same. */
typedef struct {
    int32_t start;
    int32_t stop; /* inclusive */
} abea_index_pair_t;

typedef struct {
    char ref_kmer[ABEA_KMER_SIZE + 1];
    int32_t ref_position;
    int32_t read_idx;
    int32_t event_idx;
    uint8_t rc;
    char model_kmer[ABEA_KMER_SIZE + 1];
    char hmm_state;
} abea_event_alignment_t;

/* ---- status codes ------------------------------------------------------ */
typedef enum {
    ABEA_OK = 0,
    ABEA_ERR_INVALID_ARG = -1,   /* null pointer, negative size, non-finite model */
    ABEA_ERR_CAPACITY = -2,      /* an alignment path longer than its output slot */
    ABEA_ERR_OUT_OF_MEMORY = -3, /* device or pinned-host allocation failed */
    ABEA_ERR_CUDA = -4,          /* a CUDA runtime call failed */
    ABEA_ERR_TIMEOUT = -5,       /* a bounded device-side wait gave up */
    ABEA_ERR_NO_DEVICE = -6,     /* no CUDA device, or the library's kernels do not run on it */
    ABEA_ERR_INTERNAL = -7,      /* a device-side consistency check failed */
    ABEA_ERR_UNDEFINED = -8      /* the reference's traceback would read outside the read's band
                                    arrays for this read; no defined answer exists */
} abea_status_t;

/* Execution forms.
 *  PLAIN   — the reference's structure: three kernels (pre, core, post) launched
 *            one after the other, one thread block per read, the backpointer
 *            (trace) matrix in HBM (GPU/align_cuda.c:680-850); every band's
 *            scores too only with ABEA_OPT_STORE_SCORES.
 *  BATCHED — one persistent kernel (pre, fill and traceback fused) of one
 *            512-thread block per SM: the longest reads on the wide shape
 *            (twelve warps: four run the band-to-band chain, eight compute the
 *            emissions ahead of it; the traceback is walked by the whole block),
 *            which the blocks pull longest first, one after another (every read,
 *            when the batch's longest read bounds it or it has few reads per SM);
 *            the rest one warp each, first spread round-robin over the other
 *            blocks, then pulled longest-first from a device queue; replayed as
 *            one CUDA graph. */
typedef enum { ABEA_MODE_PLAIN = 0, ABEA_MODE_BATCHED = 1 } abea_mode_t;

/* Context options (abea_ctx_set_option). */
typedef enum {
    ABEA_OPT_MODE = 0,          /* abea_mode_t */
    ABEA_OPT_STORE_SCORES = 1,  /* 1: keep every band's scores in HBM (reference layout, GPU/align_cuda.c:573-577) */
    ABEA_OPT_USE_GRAPH = 2,     /* BATCHED only: 1 = replay the step as one CUDA graph */
    ABEA_OPT_LONG_READ_BANDS = 3,  /* BATCHED: reads with at least this many bands use the wide shape; 0 = autotuned */
    ABEA_OPT_SPIN_LIMIT = 4,    /* upper bound on any device-side wait, in polling iterations */
    ABEA_OPT_VAR_AWARE = 5,     /* 1: emissions use level_stdv*var and level_log_stdv+log_var (the
                                   reference ignores var, GPU/align_cuda.cl:509); taken at batch creation */
    ABEA_OPT_TRACE_BUDGET = 6,  /* bytes of backpointers a read may keep in HBM (128 per band); a read
                                   needing more keeps band-score checkpoints every 256 bands (4 bytes per
                                   band) and its traceback recomputes the trace 256 bands at a time.
                                   0 (default) = keep every trace.  Taken at batch creation. */
    ABEA_OPT_WIDE_CLUSTER = 7,  /* BATCHED: 1 = the longest reads run on a cluster of two blocks (the
                                   second SM computes the emissions ahead into the first one's shared
                                   memory); 0 = one block per wide read */
    ABEA_OPT_MEDIUM_READ_BANDS = 8 /* BATCHED: reads with at least this many bands that do not take the
                                   wide shape run on the medium shape (eight warps per read, two reads
                                   per block); 0 = autotuned (none when not tuned) */
} abea_option_t;

typedef struct abea_ctx abea_ctx_t;
typedef struct abea_batch abea_batch_t;

/* Stage timings of the most recent run of a batch, milliseconds (CUDA events on
 * the context's stream). */
typedef struct {
    float pre_ms;
    float core_ms;
    float post_ms;
    float total_ms;
    float h2d_ms;
    float d2h_ms;
    int32_t kernel_launches;
} abea_timing_t;

/* ---- context ------------------------------------------------------------ */
/* Creates a context (one CUDA stream and its scratch buffers) on `device`. */
abea_status_t abea_ctx_create(abea_ctx_t **ctx, int device, abea_mode_t mode);
void abea_ctx_destroy(abea_ctx_t *ctx);
abea_status_t abea_ctx_set_option(abea_ctx_t *ctx, abea_option_t opt, int64_t value);
abea_status_t abea_ctx_get_option(abea_ctx_t *ctx, abea_option_t opt, int64_t *value);
/* Message of the last failure on the calling thread ("" if none). */
const char *abea_last_error(void);
const char *abea_status_string(abea_status_t status);
/* Library version string. */
const char *abea_version(void);

/* ---- drop-in single-read entry: f5c align() (GPU/f5cmisc.h:48-50) -------
 * Same arguments, same meaning: `out_2` is caller-allocated; f5c sizes it at
 * 2*events.n pairs (GPU/align_cuda.c:496).  Returns the number of AlignedPairs
 * written, 0 when the alignment failed the reference's quality checks
 * (GPU/align_cuda.cl:856-882), or a negative abea_status_t on error.
 * `sample_rate` is unused by the algorithm, as in the reference.
 * Thread-safe (f5c calls it from many worker threads, GPU/f5c.h:57-59): each
 * calling thread gets its own context (a stream and 24 CUDA events) on the
 * current device, created by its first call and destroyed when the thread
 * exits, and a device slab grown to that thread's largest read so far (about
 * 132 bytes per band + 48 per event + 17 per base, plus 136 KB, plus 512 KB of
 * traceback scratch for a read of 512 bands or more; a 20 kb read: about 9.5 MB).  Each read runs alone on the wide shape of the batched form. */
int32_t abea_align(abea_aligned_pair_t *out_2, char *sequence, int32_t sequence_len,
                   abea_event_table_t events, abea_model_t *models, abea_scalings_t scaling,
                   float sample_rate);

/* Same as abea_align with an explicit output capacity (in pairs). */
int32_t abea_align_cap(abea_aligned_pair_t *out_2, int32_t out_capacity, const char *sequence,
                       int32_t sequence_len, const abea_event_t *events, int32_t n_events,
                       const abea_model_t *models, abea_scalings_t scaling);

/* ---- batch entry: align_cuda(core, db) / align_ocl(core, db) ------------
 * Host arrays in the reference's flattened layout (GPU/align_cuda.c:432-497):
 *   read[read_ptr[i] .. read_ptr[i]+read_len[i])  bases of read i (NUL separators allowed)
 *   event_table[event_ptr[i] .. +n_events[i])     events of read i
 *   scalings[i], model[4096]
 * Outputs (host): event_align_pairs[2*event_ptr[i] ...] gets read i's pairs
 * (capacity 2*n_events[i], as in the reference), n_event_align_pairs[i] its
 * count (0 = failed QC; negative = per-read abea_status_t).  Host->device and
 * device->host copies happen inside the call. */
abea_status_t abea_align_batch(abea_ctx_t *ctx, int32_t n_reads, const char *read,
                               const int64_t *read_ptr, const int32_t *read_len,
                               const abea_event_t *event_table, const int64_t *event_ptr,
                               const int32_t *n_events, const abea_scalings_t *scalings,
                               const abea_model_t *model, abea_aligned_pair_t *event_align_pairs,
                               int32_t *n_event_align_pairs);

/* abea_align_batch in the batched form whatever the context's ABEA_OPT_MODE: the
 * persistent kernel over the device work queue, replayed as one CUDA graph. */
abea_status_t abea_align_batch_persistent(abea_ctx_t *ctx, int32_t n_reads, const char *read,
                                          const int64_t *read_ptr, const int32_t *read_len,
                                          const abea_event_t *event_table, const int64_t *event_ptr,
                                          const int32_t *n_events, const abea_scalings_t *scalings,
                                          const abea_model_t *model, abea_aligned_pair_t *event_align_pairs,
                                          int32_t *n_event_align_pairs);

/* f5c's per-read arrays (db_t's read[i], read_len[i], et[i], scalings[i],
 * event_align_pairs[i], n_event_align_pairs[i]; GPU/f5c.h) aligned as one batch:
 * the flattening of GPU/align_cuda.c:432-497 done inside the library, through
 * pinned staging kept by the context (copied on up to eight host threads for
 * batches of 8 MB or more, as are the results back to event_align_pairs[i]).
 * event_align_pairs[i] must hold 2*et[i].n pairs; n_event_align_pairs[i] as in
 * abea_align_batch. */
abea_status_t abea_align_db(abea_ctx_t *ctx, int32_t n_reads, char *const *read, const int32_t *read_len,
                            const abea_event_table_t *et, const abea_scalings_t *scalings,
                            const abea_model_t *model, abea_aligned_pair_t *const *event_align_pairs,
                            int32_t *n_event_align_pairs);

/* ---- device-resident batches --------------------------------------------
 * abea_batch_create copies a batch (same host layout as abea_align_batch) into
 * HBM once; abea_batch_run aligns it on the context's stream (asynchronous);
 * abea_batch_sync waits; abea_batch_results copies results to the host. */
abea_status_t abea_batch_create(abea_ctx_t *ctx, int32_t n_reads, const char *read,
                                const int64_t *read_ptr, const int32_t *read_len,
                                const abea_event_t *event_table, const int64_t *event_ptr,
                                const int32_t *n_events, const abea_scalings_t *scalings,
                                const abea_model_t *model, abea_batch_t **batch);
abea_status_t abea_batch_run(abea_ctx_t *ctx, abea_batch_t *batch);
abea_status_t abea_batch_sync(abea_ctx_t *ctx);
abea_status_t abea_batch_results(abea_ctx_t *ctx, abea_batch_t *batch,
                                 abea_aligned_pair_t *event_align_pairs, int32_t *n_event_align_pairs);
abea_status_t abea_batch_timing(abea_ctx_t *ctx, abea_batch_t *batch, abea_timing_t *timing);
void abea_batch_destroy(abea_batch_t *batch);

/* Autotuner: runs the batched form on `batch` with several thresholds for the
 * wide shape and keeps the fastest for this workload's signature
 * (log2 buckets of its longest read, read count and total bands); later
 * batched runs with ABEA_OPT_LONG_READ_BANDS = 0 and the same signature use it.
 * Returns the threshold (INT64_MAX = no wide reads) and its time. */
abea_status_t abea_autotune(abea_ctx_t *ctx, abea_batch_t *batch, int64_t *best_threshold, float *best_ms);

/* The autotuner's results as a text file: a header naming the device's SM count,
 * then one "signature threshold" line per tuned workload signature.  Loading
 * merges the file's entries into the context (a file written on a device with
 * another SM count is refused with ABEA_ERR_INVALID_ARG); *n_entries (may be
 * NULL) gets the number of entries written or read. */
abea_status_t abea_autotune_save(abea_ctx_t *ctx, const char *path, int32_t *n_entries);
abea_status_t abea_autotune_load(abea_ctx_t *ctx, const char *path, int32_t *n_entries);

/* Band matrices of one read after a run, converted to the reference layout
 * (GPU/align_cuda.c:573-583): bands[n_bands*100] scores (needs
 * ABEA_OPT_STORE_SCORES=1, else NULL must be passed), trace[n_bands*100]
 * backpointers (0=D, 1=U, 2=L), band_lower_left[n_bands].  n_bands =
 * n_events + n_kmers + 2.  For tests and debugging. */
abea_status_t abea_batch_read_bands(abea_ctx_t *ctx, abea_batch_t *batch, int32_t read_index,
                                    float *bands, uint8_t *trace,
                                    abea_event_kmer_pair_t *band_lower_left);

/* Per-read best end score (the maximum of the last k-mer column plus trim
 * penalties, GPU/align_cuda.cl:722-746) of the last run, host array [n_reads]. */
abea_status_t abea_batch_best_scores(abea_ctx_t *ctx, abea_batch_t *batch, float *best_scores);

/* Number of band cells whose exact double-rounded scores were taken from the
 * FP64 slow path during the last run (diagnostic). */
abea_status_t abea_batch_slow_cells(abea_ctx_t *ctx, abea_batch_t *batch, int64_t *count);

/* Pinned host memory for fast host<->device copies (cudaHostAlloc). */
void *abea_host_alloc(size_t bytes);
void abea_host_free(void *ptr);

/* Timing and copy volume of the last abea_align_batch / abea_align call on a
 * context: stage times, and the host->device / device->host bytes moved. */
abea_status_t abea_ctx_last_timing(abea_ctx_t *ctx, abea_timing_t *timing, int64_t *h2d_bytes,
                                   int64_t *d2h_bytes);

/* Copy volume of a batch and its band-cell count (sum of n_bands*100). */
abea_status_t abea_batch_io_bytes(abea_batch_t *batch, int64_t *h2d_bytes, int64_t *d2h_bytes,
                                  int64_t *band_cells);

/* Timing markers on the context's stream (CUDA events), for callers that time
 * several runs as one region: abea_ctx_mark(ctx, i) records marker i (0..15);
 * abea_ctx_elapsed(ctx, i, j, &ms) waits for marker j and returns j - i. */
abea_status_t abea_ctx_mark(abea_ctx_t *ctx, int marker);
abea_status_t abea_ctx_elapsed(abea_ctx_t *ctx, int from_marker, int to_marker, float *ms);

/* Evicts the GPU's L2 cache by writing a buffer larger than it on the
 * context's stream (benchmark hygiene between timed runs). */
abea_status_t abea_ctx_flush_l2(abea_ctx_t *ctx);

/* Self-test of the kernels' exact FP32 arithmetic on the current device:
 * `cases` pseudo-random and near-rounding-midpoint cases of the division and
 * of the double-rounded sums, checked against IEEE division and FP64 adds.
 * out[5]: division wrong, division declined, sum wrong, sum declined, cases.
 * "wrong" must be 0; "declined" cases take the FP64 path in the kernels. */
abea_status_t abea_selftest_arith(int64_t cases, uint64_t seed, int64_t *out);

/* ---- adjoint (no counterpart in the reference) ---------------------------
 * Gradients of each read's best-path log-likelihood, evaluated in FP64 along the
 * path that the last run of the batch stored (the moves and trims on a fixed path
 * do not depend on the parameters; only the emissions of the cells entered by a
 * step or a stay do).  The batch must have been run (abea_batch_run +
 * abea_batch_sync) or aligned.  Outputs (host arrays, each may be NULL):
 *   grad_scalings[n_reads*3]: d/d shift, d/d scale, d/d var (var only counts
 *       with ABEA_OPT_VAR_AWARE; 0 otherwise);
 *   grad_model[4096*2]: d/d level_mean, d/d level_stdv of every k-mer (rank
 *       order, summed over the reads that have a gradient);
 *   path_emission[n_reads]: the FP64 sum of the emissions on the path;
 *   read_status[n_reads]: 0, or the abea_status_t saying why the read has no
 *       gradient (no path, truncated path); those reads' entries are 0.
 * Reads whose alignment failed the quality checks still have a path and a
 * gradient. */
abea_status_t abea_batch_backward(abea_ctx_t *ctx, abea_batch_t *batch, double *grad_scalings,
                                  double *grad_model, double *path_emission, int32_t *read_status);
/* The same entry under the name of the batch-form plan (abea_backward_batch). */
abea_status_t abea_backward_batch(abea_ctx_t *ctx, abea_batch_t *batch, double *grad_scalings,
                                  double *grad_model, double *path_emission, int32_t *read_status);

/* Replaces the per-read scalings of a device-resident batch (host array
 * [n_reads]); the next abea_batch_run aligns with them. */
abea_status_t abea_batch_set_scalings(abea_ctx_t *ctx, abea_batch_t *batch, const abea_scalings_t *scalings);

/* Gauss-Newton recalibration of (shift, scale) per read: `iterations` rounds of
 * align -> fixed-path normal equations (residuals (x - scale*mu - shift)/stdv of the
 * emitting cells) -> step.  Round it of n aligns with every emission stdv
 * multiplied by first_temperature^((n-1-it)/(n-1)) (annealing: the last round,
 * and every round when first_temperature = 1, uses the model as it is); 5 suits
 * scalings that are off by several pA and several percent.  A read whose path is
 * missing or whose normal equations are singular keeps its scalings.  The batch
 * is left aligned with the final scalings, which are written to out[n_reads]
 * (may be NULL). */
abea_status_t abea_batch_recalibrate(abea_ctx_t *ctx, abea_batch_t *batch, int32_t iterations,
                                     double first_temperature, abea_scalings_t *out);

/* Method-of-moments scalings of every read of a batch (f5c's
 * estimate_scalings_using_mom, GPU/f5cmisc.h:47, prototype only in the
 * reference): scale = sqrt(var(event means) / var(k-mer levels along the read)),
 * shift = mean(event means) - scale * mean(k-mer levels), var = 1, log_var = 0,
 * sums in FP64.  Written to out[n_reads] (may be NULL); apply != 0 also makes
 * them the batch's scalings for the next run. */
abea_status_t abea_batch_estimate_scalings(abea_ctx_t *ctx, abea_batch_t *batch, abea_scalings_t *out,
                                           int32_t apply);

/* f5c's postalign (GPU/f5cmisc.h:51-52, prototype only in the reference) for
 * every read of a batch after abea_batch_run, on the AlignedPairs in HBM:
 *   base_to_event_map[read_ptr[i] + k], k < n_kmers: the first and last event
 *       aligned to k-mer k, counting a pair only when its event differs from
 *       the previous pair's; {-1, -1} for a k-mer with none.  Entries past
 *       n_kmers of each read are {-1, -1}.  Size: max(read_ptr[i] +
 *       read_len[i]) entries.
 *   alignment[event_ptr[i] + j], j < n_alignment[i]: for every k-mer k in
 *       order and every event of its range, {ref_kmer = model_kmer = the six
 *       bases at k, ref_position = k, read_idx = i, event_idx, rc = 0,
 *       hmm_state = 'M' when the k-mer's rank differs from the previous
 *       record's, else 'E'}.  Size: max event_ptr[i] + n_events[i] records.
 *   events_per_base[i] = (last event - first event on the path) / n_kmers.
 *   n_alignment[i]: the record count (at most n_events[i]); 0 with
 *       events_per_base 0 for a read without AlignedPairs (failed quality
 *       checks, nothing to align).
 * Any output pointer may be NULL. */
abea_status_t abea_batch_postalign(abea_ctx_t *ctx, abea_batch_t *batch, abea_event_alignment_t *alignment,
                                   abea_index_pair_t *base_to_event_map, double *events_per_base,
                                   int32_t *n_alignment);

/* ---- serving stream (no counterpart in the reference) --------------------
 * A stream of reads in the batch layout of abea_align_batch, admitted in input
 * order into device batches whose device footprint (sequence, events, k-mer
 * tables, trace or checkpoints, outputs) stays under `batch_bytes`.  Two
 * batches are in flight: batch i+1 is copied to the device on a second stream
 * while batch i runs on the context's stream, and batch i's results go back on
 * that second stream.  Per batch: the alignment and, with `recalibrate`, the
 * adjoint, one Gauss-Newton step of every read's (shift, scale) and the
 * re-alignment with the new scalings (whose AlignedPairs are the ones returned).
 * A read larger than `batch_bytes` forms a batch of its own. */
typedef struct {
    int64_t batch_bytes;  /* device footprint limit of one batch; 0 = the smaller of 16 GiB and
                             40% of the device's free memory */
    int32_t recalibrate;  /* 0 = align; 1 = align, adjoint, one Gauss-Newton step, re-align */
    int32_t reserved;     /* 0 */
} abea_stream_config_t;

typedef struct {
    int32_t n_batches;
    int32_t max_batch_reads;
    int64_t max_batch_bytes;  /* largest device footprint of one batch */
    int64_t band_cells;       /* sum of n_bands*100 over the reads (each read once) */
    double wall_ms;           /* from the call to the last batch's results in host memory */
    double compute_ms;        /* sum of the batches' device time on the context's stream */
} abea_stream_stats_t;

/* Inputs and outputs as abea_align_batch, with reads whose event ranges follow
 * one another (event_ptr[i] + n_events[i] <= event_ptr[i+1]).  Host buffers from
 * abea_host_alloc let the copies overlap the alignment; pageable buffers work but
 * their copies wait for the device.  Outputs (each may be NULL except the pairs
 * and counts): scalings_out[n_reads] the scalings each read was finally aligned
 * with; read_latency_ms[n_reads] the time from the admission of the read's batch
 * (the host queuing its copy to the device) to its results being in host memory;
 * stats.  Returns the first failing read's status after every batch has run,
 * like abea_align_batch. */
abea_status_t abea_align_stream(abea_ctx_t *ctx, const abea_stream_config_t *cfg, int32_t n_reads,
                                const char *read, const int64_t *read_ptr, const int32_t *read_len,
                                const abea_event_t *event_table, const int64_t *event_ptr,
                                const int32_t *n_events, const abea_scalings_t *scalings,
                                const abea_model_t *model, abea_aligned_pair_t *event_align_pairs,
                                int32_t *n_event_align_pairs, abea_scalings_t *scalings_out,
                                double *read_latency_ms, abea_stream_stats_t *stats);

/* ---- no-allocation entry point ------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory themselves or through this library: a framework whose own allocator
 * owns the whole device and hands out every buffer, or a service whose device
 * memory budget is fixed when it starts.  Aligns one read with
 * the plain pre/core/post kernels on `stream` (a cudaStream_t; NULL = default
 * stream) and returns without waiting.  Inputs (sequence, events, model) and
 * outputs (pairs, capacity out_capacity; *n_pairs = count, 0 = failed QC,
 * negative = abea_status_t of the read) are caller-owned device-accessible
 * memory.  All scratch comes from one fixed 32 MiB (33,554,432-byte) device
 * array inside this library, present on every GPU that loads it until the
 * process exits.  A read needs, each region rounded up to 256 bytes: the read's
 * descriptor (256), 2 regions of 4 * round16(n_events) bytes, 4 of
 * 4 * round16(n_kmers), one of 128 * round4(n_bands) and one of
 * 4 * round4(n_bands), plus 512 (n_kmers = sequence_len - 5, n_bands =
 * n_events + n_kmers + 2, roundM = rounded up to a multiple of M) — about
 * 143 bytes per band, so reads of up to about 230,000 bands fit; larger reads
 * are rejected with ABEA_ERR_INVALID_ARG before any device work.  No cudaMalloc
 * or other allocation happens.  The first call in each CUDA context (once per
 * device, and again after a device reset or in a context the caller created)
 * looks up the array's device address (cudaGetSymbolAddress), so make it
 * before any stream capture.  Every call uses the same array: calls whose work
 * overlaps on the GPU (other streams, other threads) race; order them on one
 * stream. */
abea_status_t abea_align_noalloc(abea_aligned_pair_t *pairs, int32_t *n_pairs, int32_t out_capacity,
                                 const char *sequence, int32_t sequence_len, const abea_event_t *events,
                                 int32_t n_events, const abea_model_t *model, abea_scalings_t scaling,
                                 void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ABEA_H */
