/*
 * abea_oracle.h — CPU oracle for ABEA.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU-side algorithm for f5c's
 * `align()`: the fill of the single-work-item kernel
 * (FPGA/code/device/align_swi.cl:184-503) and the best-end / traceback /
 * quality-check post stage (FPGA/code/host/src/align_swi.cpp:1093-1314, with
 * the double-precision emission sum of GPU/align_cuda.cl:713-714).  It is the
 * checker used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg; the product library never links or calls it.
 *
 * Pinned against the reference's golden dump (FPGA/code/bins/dump_small, 143
 * reads, bit-exact AlignedPairs) and against the reference's own SWI code
 * compiled by oracle/build_ref.sh.  Must be compiled with
 * -ffp-contract=off (no FMA contraction: the reference has none).
 */
#ifndef ABEA_ORACLE_H
#define ABEA_ORACLE_H

#include "../include/abea.h"

#ifdef __cplusplus
extern "C" {
#endif

/* flags */
#define ORACLE_LOG_UNCACHED 0x1 /* gp_log_stdv = (float)log(level_stdv) as align_swi.cl:106-107 */
#define ORACLE_QC_FLOAT 0x2     /* float sum_emission as align_swi.cpp:1164-1165 */
#define ORACLE_VAR_AWARE 0x4    /* stdv*var and log_stdv+log_var (not the reference's parity mode) */

/* optional outputs of one alignment; any pointer may be NULL */
typedef struct {
    float *bands;                          /* [n_bands*100] scores, reference layout */
    uint8_t *trace;                        /* [n_bands*100] backpointers */
    abea_event_kmer_pair_t *band_lower_left; /* [n_bands] */
    float best_score;                      /* best end score (-inf if none) */
    int32_t best_event;                    /* event index of the best end */
    double sum_emission;                   /* QC sum along the path */
    int32_t path_len;                      /* pairs on the path before QC */
    int32_t max_gap;
    int32_t last_from;                     /* move into the last walked cell (0=D, 1=U, 2=L) */
} oracle_debug_t;

/* One read.  Returns the number of pairs written to out (0 = QC failure), or
 * ABEA_ERR_CAPACITY / ABEA_ERR_UNDEFINED / ABEA_ERR_INVALID_ARG. */
int32_t oracle_align(abea_aligned_pair_t *out, int32_t out_cap, const char *seq, int32_t seq_len,
                     const abea_event_t *events, int32_t n_events, const abea_model_t *model,
                     abea_scalings_t scaling, uint32_t flags, oracle_debug_t *dbg);

/* Band count of a read: n_events + n_kmers + 2. */
int64_t oracle_n_bands(int32_t seq_len, int32_t n_events);

/* Batch in the reference's flattened layout (GPU/align_cuda.c:432-497); reads
 * are spread over n_threads host threads, longest first.  out_pairs has
 * capacity 2*n_events[i] at offset 2*event_ptr[i]. */
void oracle_align_batch(int32_t n_reads, const char *read, const int64_t *read_ptr,
                        const int32_t *read_len, const abea_event_t *event_table,
                        const int64_t *event_ptr, const int32_t *n_events,
                        const abea_scalings_t *scalings, const abea_model_t *model,
                        abea_aligned_pair_t *out_pairs, int32_t *out_n, float *best_scores,
                        uint32_t flags, int n_threads);

/* FP64 twin: the same recurrence with every score, emission and constant in
 * double.  Returns the path length after QC like oracle_align; *best_score
 * receives the double best end score. */
int32_t oracle_align_f64(abea_aligned_pair_t *out, int32_t out_cap, const char *seq,
                         int32_t seq_len, const abea_event_t *events, int32_t n_events,
                         const abea_model_t *model, abea_scalings_t scaling, uint32_t flags,
                         double *best_score);
/* The FP64 twin over a flattened batch on n_threads threads (longest read first);
 * best_scores[i] = the read's FP64 best-end score (-inf when none is finite). */
void oracle_align_f64_batch(int32_t n_reads, const char *read, const int64_t *read_ptr,
                            const int32_t *read_len, const abea_event_t *event_table,
                            const int64_t *event_ptr, const int32_t *n_events,
                            const abea_scalings_t *scalings, const abea_model_t *model,
                            abea_aligned_pair_t *out_pairs, int32_t *out_n, double *best_scores,
                            uint32_t flags, int n_threads);

/* The reference emission, float arithmetic in the reference's order
 * (GPU/align_cuda.cl:85-110, align_swi.cl:77-111). */
float oracle_emission(float event_mean, const abea_model_t *m, abea_scalings_t scaling,
                      uint32_t flags);

/* FP64 adjoint of one read's fixed path (no counterpart in the reference).
 * walk[0..n) in walk order (walk[0] = best end), last_from = the move into
 * walk[n-1].  Emissions in double: a = (x - (scale*mu + shift))/sd,
 * em = -log(sqrt(2 pi)) - log_stdv - a^2/2, sd = stdv (times var and log_stdv
 * plus log var with ORACLE_VAR_AWARE).  theta = (shift, scale, var) in double
 * (NULL: the scalings'); k-mer d_kmer (-1: none) has level_mean + d_mean and
 * level_stdv + d_stdv (log stdv moved by log1p(d_stdv/stdv)).  Returns the sum
 * of the emitting cells' emissions; grad3 = d/d(shift, scale, var), gn5 = Gauss-
 * Newton sums (J^T J 11, 12, 22; J^T r 1, 2) of the residuals a in (shift,
 * scale), grad_model[4096*2] += d/d(level_mean, level_stdv).  Any output may be
 * NULL. */
double oracle_path_adjoint(const abea_aligned_pair_t *walk, int32_t n, int32_t last_from,
                           const char *seq, const abea_event_t *events, const abea_model_t *model,
                           abea_scalings_t sc, const double *theta, int32_t d_kmer, double d_mean,
                           double d_stdv, uint32_t flags, double *grad3, double *gn5,
                           double *grad_model);

/* Method-of-moments scalings of one read (f5c's estimate_scalings_using_mom,
 * prototype only in the reference, GPU/f5cmisc.h:47): scale = sqrt(var(event
 * means) / var(k-mer levels along the read)), shift = mean(event means) -
 * scale * mean(k-mer levels); FP64; (1, 0) for a read with nothing to align. */
void oracle_mom(const char *seq, int32_t seq_len, const abea_event_t *events, int32_t n_events,
                const abea_model_t *model, double *scale, double *shift);

/* Rank of the 6-mer starting at s (GPU/align_cuda.cl:22-51). */
uint32_t oracle_kmer_rank(const char *s);

/* The double-rounded cell sum of the reference, (float)(((double)a + b) + (double)c). */
float oracle_add3(float a, double b, float c);

/* f5c's postalign restated (prototype only in the reference, GPU/f5cmisc.h:51-52):
 * map[n_kmers] and out[<= out_cap] from one read's AlignedPairs.  Returns the
 * record count, ABEA_ERR_CAPACITY or ABEA_ERR_INVALID_ARG. */
int32_t oracle_postalign(abea_event_alignment_t *out, int32_t out_cap, abea_index_pair_t *map,
                         double *events_per_base, const char *seq, int32_t n_kmers,
                         const abea_aligned_pair_t *pairs, int32_t n_pairs, int32_t read_idx);

#ifdef __cplusplus
}
#endif

#endif
