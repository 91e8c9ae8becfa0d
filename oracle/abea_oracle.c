/*
 * abea_oracle.c — CPU oracle for ABEA.  TEST INFRASTRUCTURE ONLY: the checker
 * for tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.  The
 * product library never links or calls it.
 *
 * Restates, in plain C, the reference's algorithm for f5c's align():
 *   fill  : FPGA/code/device/align_swi.cl:184-503 (single-work-item kernel)
 *   post  : FPGA/code/host/src/align_swi.cpp:1093-1314 (best end, traceback,
 *           reverse, QC), with the double-precision sum_emission of the
 *           GPU NDRange post kernel GPU/align_cuda.cl:713-714 (f5c's form).
 * Compile with -ffp-contract=off: the reference's arithmetic has no fused
 * multiply-add, and contraction changes AlignedPairs (142/143 on the dump).
 */
#include "abea_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define W ABEA_BANDWIDTH
#define HALF_W (ABEA_BANDWIDTH / 2)
#define FROM_D 0
#define FROM_U 1
#define FROM_L 2
#define MAX_GAP_THRESHOLD 50        /* GPU/align_cuda.cl:128 */
#define MIN_AVG_LOG_EMISSION (-5.0) /* GPU/align_cuda.cl:133 */
#define LOG_INV_SQRT_2PI (-0.918938f) /* GPU/align_cuda.cl:66 */

/* A/C/G/T -> 0..3, anything else 0 (GPU/align_cuda.cl:22-35). */
static inline uint32_t base_rank(char b) {
    switch (b) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return 0;
    }
}

/* First base most significant: rank = sum_j rank(s[j]) << 2*(5-j)
 * (GPU/align_cuda.cl:39-51). */
uint32_t oracle_kmer_rank(const char *s) {
    uint32_t r = 0;
    for (int j = 0; j < ABEA_KMER_SIZE; ++j) r = (r << 2) | base_rank(s[j]);
    return r;
}

/* log_probability_match_r9 + log_normal_pdf in float, reference order:
 *   gp_mean = scale*level_mean + shift; a = (x - gp_mean)/gp_stdv;
 *   lp = (log_inv_sqrt_2pi - gp_log_stdv) + ((-0.5f*a)*a)
 * gp_stdv ignores scaling.var in the reference (GPU/align_cuda.cl:95,509,
 * align_swi.cl:99); ORACLE_VAR_AWARE applies var like nanopolish does. */
float oracle_emission(float x, const abea_model_t *m, abea_scalings_t sc, uint32_t flags) {
    float gp_mean = sc.scale * m->level_mean;
    gp_mean = gp_mean + sc.shift;
    float gp_stdv = m->level_stdv;
    float gp_log_stdv;
    if (flags & ORACLE_LOG_UNCACHED)
        gp_log_stdv = (float)log((double)m->level_stdv);
    else
        gp_log_stdv = m->level_log_stdv;
    if (flags & ORACLE_VAR_AWARE) {
        gp_stdv = gp_stdv * sc.var;
        gp_log_stdv = gp_log_stdv + sc.log_var;
    }
    float a = (x - gp_mean) / gp_stdv;
    float t = -0.5f * a;
    t = t * a;
    float c = LOG_INV_SQRT_2PI - gp_log_stdv;
    return c + t;
}

float oracle_add3(float a, double b, float c) {
    double t = (double)a + b;
    t = t + (double)c;
    return (float)t;
}

int64_t oracle_n_bands(int32_t seq_len, int32_t n_events) {
    return (int64_t)n_events + (int64_t)(seq_len - ABEA_KMER_SIZE + 1) + 2;
}

typedef struct {
    double lp_skip, lp_stay, lp_step, lp_trim;
} penalties_t;

/* Transition log-probabilities, double (align_swi.cl:233-250). */
static penalties_t make_penalties(int32_t n_events, int32_t n_kmers) {
    penalties_t p;
    double events_per_kmer = (double)n_events / n_kmers;
    double p_stay = 1 - (1 / (events_per_kmer + 1));
    p.lp_skip = log(1e-10);
    p.lp_stay = log(p_stay);
    p.lp_step = log(1.0 - exp(p.lp_skip) - exp(p.lp_stay));
    p.lp_trim = log(0.01);
    return p;
}

#define BAND(b, o) bands[(size_t)(b) * W + (size_t)(o)]
#define TRACE(b, o) trace[(size_t)(b) * W + (size_t)(o)]
#define VALID(o) ((o) >= 0 && (o) < W)

int32_t oracle_align(abea_aligned_pair_t *out, int32_t out_cap, const char *seq, int32_t seq_len,
                     const abea_event_t *events, int32_t n_events, const abea_model_t *model,
                     abea_scalings_t sc, uint32_t flags, oracle_debug_t *dbg) {
    if (dbg) {
        dbg->best_score = -INFINITY;
        dbg->last_from = FROM_L;
        dbg->best_event = 0;
        dbg->sum_emission = 0.0;
        dbg->path_len = 0;
        dbg->max_gap = 0;
    }
    if (!out || !seq || !model || (n_events > 0 && !events) || n_events < 0 || seq_len < 0)
        return ABEA_ERR_INVALID_ARG;
    int32_t n_kmers = seq_len - ABEA_KMER_SIZE + 1;
    /* The reference has no defined result for these (division by zero /
     * reading events[0] of an empty table); the library returns 0 pairs. */
    if (n_kmers <= 0 || n_events <= 0) return 0;

    penalties_t pen = make_penalties(n_events, n_kmers);
    int64_t n_bands = (int64_t)n_events + n_kmers + 2;

    uint32_t *ranks = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n_kmers);
    float *bands = (float *)malloc(sizeof(float) * (size_t)n_bands * W);
    uint8_t *trace = (uint8_t *)calloc((size_t)n_bands * W, 1);
    abea_event_kmer_pair_t *bll =
        (abea_event_kmer_pair_t *)malloc(sizeof(abea_event_kmer_pair_t) * (size_t)n_bands);
    if (!ranks || !bands || !trace || !bll) {
        free(ranks); free(bands); free(trace); free(bll);
        return ABEA_ERR_OUT_OF_MEMORY;
    }
    for (int32_t k = 0; k < n_kmers; ++k) ranks[k] = oracle_kmer_rank(seq + k);
    for (int64_t i = 0; i < n_bands * W; ++i) bands[i] = -INFINITY;

    /* ---- fill (align_swi.cl:305-503) ---- */
    bll[0].event_idx = HALF_W - 1;
    bll[0].kmer_idx = -1 - HALF_W;
    bll[1].event_idx = bll[0].event_idx + 1;
    bll[1].kmer_idx = bll[0].kmer_idx;
    BAND(0, -1 - bll[0].kmer_idx) = 0.0f;            /* start cell (e=-1,k=-1) */
    BAND(1, bll[1].event_idx - 0) = (float)pen.lp_trim; /* first event trimmed */
    TRACE(1, bll[1].event_idx - 0) = FROM_U;

    for (int64_t b = 2; b < n_bands; ++b) {
        float ll = BAND(b - 1, 0);
        float ur = BAND(b - 1, W - 1);
        int right;
        if (ll == -INFINITY && ur == -INFINITY)
            right = (int)(b & 1); /* alternate when both ends are out of band */
        else
            right = ll < ur; /* Suzuki-Kasahara rule */
        abea_event_kmer_pair_t cur = bll[b - 1];
        if (right)
            cur.kmer_idx += 1;
        else
            cur.event_idx += 1;
        bll[b] = cur;

        int trim_offset = -1 - cur.kmer_idx;
        if (VALID(trim_offset)) {
            int32_t e = cur.event_idx - trim_offset;
            if (e >= 0 && e < n_events) {
                BAND(b, trim_offset) = (float)(pen.lp_trim * (e + 1));
                TRACE(b, trim_offset) = FROM_U;
            } else {
                BAND(b, trim_offset) = -INFINITY;
            }
        }

        int lo = -cur.kmer_idx;
        int t = cur.event_idx - (n_events - 1);
        if (t > lo) lo = t;
        if (lo < 0) lo = 0;
        int hi = n_kmers - cur.kmer_idx;
        t = cur.event_idx + 1;
        if (t < hi) hi = t;
        if (W < hi) hi = W;

        const abea_event_kmer_pair_t p1 = bll[b - 1], p2 = bll[b - 2];
        for (int o = lo; o < hi; ++o) {
            int e = cur.event_idx - o;
            int k = cur.kmer_idx + o;
            int o_up = p1.event_idx - (e - 1);
            int o_left = (k - 1) - p1.kmer_idx;
            int o_diag = (k - 1) - p2.kmer_idx;
            float up = VALID(o_up) ? BAND(b - 1, o_up) : -INFINITY;
            float left = VALID(o_left) ? BAND(b - 1, o_left) : -INFINITY;
            float diag = VALID(o_diag) ? BAND(b - 2, o_diag) : -INFINITY;
            float em = oracle_emission(events[e].mean, &model[ranks[k]], sc, flags);
            /* float + double + float evaluated in double, rounded once to float */
            float s_d = oracle_add3(diag, pen.lp_step, em);
            float s_u = oracle_add3(up, pen.lp_stay, em);
            float s_l = (float)((double)left + pen.lp_skip);
            float best = s_d;
            uint8_t from = FROM_D;
            best = s_u > best ? s_u : best;
            from = best == s_u ? FROM_U : from;
            best = s_l > best ? s_l : best;
            from = best == s_l ? FROM_L : from;
            BAND(b, o) = best;
            TRACE(b, o) = from;
        }
    }

    /* ---- best end on the last k-mer column (align_swi.cpp:1149-1171) ---- */
    float max_score = -INFINITY;
    int32_t cur_e = 0;
    int32_t cur_k = n_kmers - 1;
    for (int32_t e = 0; e < n_events; ++e) {
        int64_t b = (int64_t)e + cur_k + 2;
        int o = bll[b].event_idx - e;
        if (VALID(o)) {
            float s = (float)((double)BAND(b, o) + (n_events - e) * pen.lp_trim);
            if (s > max_score) {
                max_score = s;
                cur_e = e;
            }
        }
    }
    if (dbg) {
        dbg->best_score = max_score;
        dbg->best_event = cur_e;
    }

    /* ---- traceback (align_swi.cpp:1178-1236) ---- */
    /* A path longer than the output slot makes the reference write past it
     * (into the next read's slot in a batch); the walk continues without
     * writing so that the QC verdict is still the reference's, and such a read
     * is reported as ABEA_ERR_CAPACITY only when it passes QC. */
    int32_t n_out = 0, gap = 0, max_gap = 0, status = 0, last_k = cur_k, last_from = FROM_L;
    double sum_em = 0.0;
    float sum_em_f = 0.0f;
    double n_aligned = 0.0;
    while (cur_k >= 0 && cur_e >= 0) {
        if (n_out < out_cap) {
            out[n_out].ref_pos = cur_k;
            out[n_out].read_pos = cur_e;
        }
        last_k = cur_k;
        n_out++;
        float em = oracle_emission(events[cur_e].mean, &model[ranks[cur_k]], sc, flags);
        sum_em += (double)em;
        sum_em_f += em;
        n_aligned += 1;
        int64_t b = (int64_t)cur_e + cur_k + 2;
        /* The reference indexes the flat band array: an offset outside the
         * band reads a neighbouring band's row.  Within the read's own rows
         * that is reproduced; beyond them the reference has no defined answer. */
        int64_t idx = b * W + (int64_t)(bll[b].event_idx - cur_e);
        if (idx < 0 || idx >= n_bands * W) {
            status = ABEA_ERR_UNDEFINED;
            break;
        }
        uint8_t from = trace[idx];
        last_from = from;
        if (from == FROM_D) {
            cur_k -= 1;
            cur_e -= 1;
            gap = 0;
        } else if (from == FROM_U) {
            cur_e -= 1;
            gap = 0;
        } else {
            cur_k -= 1;
            gap += 1;
            if (gap > max_gap) max_gap = gap;
        }
    }

    if (dbg) {
        if (dbg->bands) memcpy(dbg->bands, bands, sizeof(float) * (size_t)n_bands * W);
        if (dbg->trace) memcpy(dbg->trace, trace, (size_t)n_bands * W);
        if (dbg->band_lower_left)
            memcpy(dbg->band_lower_left, bll, sizeof(abea_event_kmer_pair_t) * (size_t)n_bands);
        dbg->sum_emission = (flags & ORACLE_QC_FLOAT) ? (double)sum_em_f : sum_em;
        dbg->path_len = n_out;
        dbg->max_gap = max_gap;
        dbg->last_from = last_from;
    }
    free(ranks);
    free(bands);
    free(trace);
    free(bll);
    if (status) return status;
    if (n_out == 0) return 0; /* reference reads out[-1] here; defined as failure */

    /* QC (GPU/align_cuda.cl:856-882).  After the reversal out[0] is the last
     * cell walked and out[n-1] the first, (n_kmers-1, best end). */
    double avg = (flags & ORACLE_QC_FLOAT) ? (double)(sum_em_f / (float)n_aligned)
                                           : sum_em / n_aligned;
    int spanned = last_k == 0;
    if (avg < MIN_AVG_LOG_EMISSION || !spanned || max_gap > MAX_GAP_THRESHOLD) return 0;
    if (n_out > out_cap) return ABEA_ERR_CAPACITY;
    /* reverse in place (align_swi.cpp:1240-1252) */
    for (int32_t i = 0, j = n_out - 1; i < j; ++i, --j) {
        abea_aligned_pair_t tmp = out[i];
        out[i] = out[j];
        out[j] = tmp;
    }
    return n_out;
}

/* ---------------- FP64 twin ---------------- */
static double emission_f64(float x, const abea_model_t *m, abea_scalings_t sc, uint32_t flags) {
    double gp_mean = (double)sc.scale * m->level_mean + sc.shift;
    double gp_stdv = m->level_stdv;
    double gp_log_stdv = (flags & ORACLE_LOG_UNCACHED) ? log((double)m->level_stdv)
                                                       : (double)m->level_log_stdv;
    if (flags & ORACLE_VAR_AWARE) {
        gp_stdv *= sc.var;
        gp_log_stdv += sc.log_var;
    }
    double a = ((double)x - gp_mean) / gp_stdv;
    return (-0.91893853320467274 - gp_log_stdv) + (-0.5 * a * a);
}

int32_t oracle_align_f64(abea_aligned_pair_t *out, int32_t out_cap, const char *seq,
                         int32_t seq_len, const abea_event_t *events, int32_t n_events,
                         const abea_model_t *model, abea_scalings_t sc, uint32_t flags,
                         double *best_score) {
    if (best_score) *best_score = -INFINITY;
    int32_t n_kmers = seq_len - ABEA_KMER_SIZE + 1;
    if (n_kmers <= 0 || n_events <= 0) return 0;
    penalties_t pen = make_penalties(n_events, n_kmers);
    int64_t n_bands = (int64_t)n_events + n_kmers + 2;
    uint32_t *ranks = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n_kmers);
    double *bands = (double *)malloc(sizeof(double) * (size_t)n_bands * W);
    uint8_t *trace = (uint8_t *)calloc((size_t)n_bands * W, 1);
    abea_event_kmer_pair_t *bll =
        (abea_event_kmer_pair_t *)malloc(sizeof(abea_event_kmer_pair_t) * (size_t)n_bands);
    if (!ranks || !bands || !trace || !bll) {
        free(ranks); free(bands); free(trace); free(bll);
        return ABEA_ERR_OUT_OF_MEMORY;
    }
    for (int32_t k = 0; k < n_kmers; ++k) ranks[k] = oracle_kmer_rank(seq + k);
    for (int64_t i = 0; i < n_bands * W; ++i) bands[i] = -INFINITY;
    bll[0].event_idx = HALF_W - 1;
    bll[0].kmer_idx = -1 - HALF_W;
    bll[1].event_idx = bll[0].event_idx + 1;
    bll[1].kmer_idx = bll[0].kmer_idx;
    BAND(0, -1 - bll[0].kmer_idx) = 0.0;
    BAND(1, bll[1].event_idx) = pen.lp_trim;
    TRACE(1, bll[1].event_idx) = FROM_U;
    for (int64_t b = 2; b < n_bands; ++b) {
        double ll = BAND(b - 1, 0), ur = BAND(b - 1, W - 1);
        int right = (ll == -INFINITY && ur == -INFINITY) ? (int)(b & 1) : (ll < ur);
        abea_event_kmer_pair_t cur = bll[b - 1];
        if (right) cur.kmer_idx += 1; else cur.event_idx += 1;
        bll[b] = cur;
        int trim_offset = -1 - cur.kmer_idx;
        if (VALID(trim_offset)) {
            int32_t e = cur.event_idx - trim_offset;
            if (e >= 0 && e < n_events) {
                BAND(b, trim_offset) = pen.lp_trim * (e + 1);
                TRACE(b, trim_offset) = FROM_U;
            }
        }
        int lo = -cur.kmer_idx, t = cur.event_idx - (n_events - 1);
        if (t > lo) lo = t;
        if (lo < 0) lo = 0;
        int hi = n_kmers - cur.kmer_idx;
        t = cur.event_idx + 1;
        if (t < hi) hi = t;
        if (W < hi) hi = W;
        const abea_event_kmer_pair_t p1 = bll[b - 1], p2 = bll[b - 2];
        for (int o = lo; o < hi; ++o) {
            int e = cur.event_idx - o, k = cur.kmer_idx + o;
            int o_up = p1.event_idx - (e - 1), o_left = (k - 1) - p1.kmer_idx,
                o_diag = (k - 1) - p2.kmer_idx;
            double up = VALID(o_up) ? BAND(b - 1, o_up) : -INFINITY;
            double left = VALID(o_left) ? BAND(b - 1, o_left) : -INFINITY;
            double diag = VALID(o_diag) ? BAND(b - 2, o_diag) : -INFINITY;
            double em = emission_f64(events[e].mean, &model[ranks[k]], sc, flags);
            double s_d = diag + pen.lp_step + em, s_u = up + pen.lp_stay + em,
                   s_l = left + pen.lp_skip;
            double best = s_d;
            uint8_t from = FROM_D;
            best = s_u > best ? s_u : best;
            from = best == s_u ? FROM_U : from;
            best = s_l > best ? s_l : best;
            from = best == s_l ? FROM_L : from;
            BAND(b, o) = best;
            TRACE(b, o) = from;
        }
    }
    double max_score = -INFINITY;
    int32_t cur_e = 0, cur_k = n_kmers - 1;
    for (int32_t e = 0; e < n_events; ++e) {
        int64_t b = (int64_t)e + cur_k + 2;
        int o = bll[b].event_idx - e;
        if (VALID(o)) {
            double s = BAND(b, o) + (n_events - e) * pen.lp_trim;
            if (s > max_score) {
                max_score = s;
                cur_e = e;
            }
        }
    }
    if (best_score) *best_score = max_score;
    int32_t n_out = 0, gap = 0, max_gap = 0, status = 0, last_k = cur_k;
    double sum_em = 0.0;
    while (cur_k >= 0 && cur_e >= 0) {
        if (n_out < out_cap) {
            out[n_out].ref_pos = cur_k;
            out[n_out].read_pos = cur_e;
        }
        last_k = cur_k;
        n_out++;
        sum_em += emission_f64(events[cur_e].mean, &model[ranks[cur_k]], sc, flags);
        int64_t b = (int64_t)cur_e + cur_k + 2;
        int64_t idx = b * W + (int64_t)(bll[b].event_idx - cur_e);
        if (idx < 0 || idx >= n_bands * W) { status = ABEA_ERR_UNDEFINED; break; }
        uint8_t from = trace[idx];
        if (from == FROM_D) { cur_k--; cur_e--; gap = 0; }
        else if (from == FROM_U) { cur_e--; gap = 0; }
        else { cur_k--; gap++; if (gap > max_gap) max_gap = gap; }
    }
    free(ranks); free(bands); free(trace); free(bll);
    if (status) return status;
    if (n_out == 0) return 0;
    double avg = sum_em / n_out;
    if (avg < MIN_AVG_LOG_EMISSION || last_k != 0 || max_gap > MAX_GAP_THRESHOLD) return 0;
    if (n_out > out_cap) return ABEA_ERR_CAPACITY;
    for (int32_t i = 0, j = n_out - 1; i < j; ++i, --j) {
        abea_aligned_pair_t tmp = out[i]; out[i] = out[j]; out[j] = tmp;
    }
    return n_out;
}

/* ---------------- threaded batch (CPU baseline) ---------------- */
typedef struct {
    int32_t n_reads;
    const char *read;
    const int64_t *read_ptr;
    const int32_t *read_len;
    const abea_event_t *event_table;
    const int64_t *event_ptr;
    const int32_t *n_events;
    const abea_scalings_t *scalings;
    const abea_model_t *model;
    abea_aligned_pair_t *out_pairs;
    int32_t *out_n;
    float *best_scores;
    uint32_t flags;
    const int32_t *order;
    int next;
    pthread_mutex_t lock;
    double *best_f64;  /* non-NULL: the all-FP64 twin (oracle_align_f64) */
} batch_job_t;

static void *batch_worker(void *arg) {
    batch_job_t *job = (batch_job_t *)arg;
    for (;;) {
        pthread_mutex_lock(&job->lock);
        int slot = job->next++;
        pthread_mutex_unlock(&job->lock);
        if (slot >= job->n_reads) break;
        int32_t i = job->order[slot];
        oracle_debug_t dbg;
        memset(&dbg, 0, sizeof(dbg));
        int32_t ne = job->n_events[i];
        if (job->best_f64) {
            job->out_n[i] = oracle_align_f64(job->out_pairs + 2 * job->event_ptr[i], 2 * ne,
                                             job->read + job->read_ptr[i], job->read_len[i],
                                             job->event_table + job->event_ptr[i], ne, job->model,
                                             job->scalings[i], job->flags, &job->best_f64[i]);
            continue;
        }
        job->out_n[i] = oracle_align(job->out_pairs + 2 * job->event_ptr[i], 2 * ne,
                                     job->read + job->read_ptr[i], job->read_len[i],
                                     job->event_table + job->event_ptr[i], ne, job->model,
                                     job->scalings[i], job->flags, &dbg);
        if (job->best_scores) job->best_scores[i] = dbg.best_score;
    }
    return NULL;
}

static const int64_t *g_sort_key;
static int cmp_desc(const void *a, const void *b) {
    int64_t ka = g_sort_key[*(const int32_t *)a], kb = g_sort_key[*(const int32_t *)b];
    if (ka != kb) return ka > kb ? -1 : 1;
    return *(const int32_t *)a - *(const int32_t *)b;
}

static void run_batch(int32_t n_reads, const char *read, const int64_t *read_ptr,
                      const int32_t *read_len, const abea_event_t *event_table,
                      const int64_t *event_ptr, const int32_t *n_events,
                      const abea_scalings_t *scalings, const abea_model_t *model,
                      abea_aligned_pair_t *out_pairs, int32_t *out_n, float *best_scores,
                      double *best_f64, uint32_t flags, int n_threads);

void oracle_align_batch(int32_t n_reads, const char *read, const int64_t *read_ptr,
                        const int32_t *read_len, const abea_event_t *event_table,
                        const int64_t *event_ptr, const int32_t *n_events,
                        const abea_scalings_t *scalings, const abea_model_t *model,
                        abea_aligned_pair_t *out_pairs, int32_t *out_n, float *best_scores,
                        uint32_t flags, int n_threads) {
    run_batch(n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events, scalings, model,
              out_pairs, out_n, best_scores, NULL, flags, n_threads);
}

void oracle_align_f64_batch(int32_t n_reads, const char *read, const int64_t *read_ptr,
                            const int32_t *read_len, const abea_event_t *event_table,
                            const int64_t *event_ptr, const int32_t *n_events,
                            const abea_scalings_t *scalings, const abea_model_t *model,
                            abea_aligned_pair_t *out_pairs, int32_t *out_n, double *best_scores,
                            uint32_t flags, int n_threads) {
    run_batch(n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events, scalings, model,
              out_pairs, out_n, NULL, best_scores, flags, n_threads);
}

static void run_batch(int32_t n_reads, const char *read, const int64_t *read_ptr,
                      const int32_t *read_len, const abea_event_t *event_table,
                      const int64_t *event_ptr, const int32_t *n_events,
                      const abea_scalings_t *scalings, const abea_model_t *model,
                      abea_aligned_pair_t *out_pairs, int32_t *out_n, float *best_scores,
                      double *best_f64, uint32_t flags, int n_threads) {
    if (n_reads <= 0) return;
    if (n_threads < 1) n_threads = 1;
    int32_t *order = (int32_t *)malloc(sizeof(int32_t) * (size_t)n_reads);
    int64_t *key = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_reads);
    for (int32_t i = 0; i < n_reads; ++i) {
        order[i] = i;
        key[i] = oracle_n_bands(read_len[i], n_events[i]);
    }
    static pthread_mutex_t sort_lock = PTHREAD_MUTEX_INITIALIZER;
    pthread_mutex_lock(&sort_lock);
    g_sort_key = key;
    qsort(order, (size_t)n_reads, sizeof(int32_t), cmp_desc);
    pthread_mutex_unlock(&sort_lock);

    batch_job_t job = {n_reads, read, read_ptr, read_len, event_table, event_ptr, n_events,
                       scalings, model, out_pairs, out_n, best_scores, flags, order, 0,
                       PTHREAD_MUTEX_INITIALIZER, best_f64};
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
    int started = 0;
    for (int t = 0; t < n_threads; ++t)
        if (pthread_create(&th[t], NULL, batch_worker, &job) == 0) started++;
        else break;
    if (started == 0) batch_worker(&job);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
    free(order);
    free(key);
}

/* ---- FP64 path adjoint (no counterpart in the reference) ----
 * The best-path score is the sum of the transition and trim log-probabilities
 * along the path (independent of the scalings and the pore model) and of the
 * emissions of the cells entered by a step (D) or a stay (U).  walk[j+1] is the
 * predecessor of walk[j], so walk[j] emits iff walk[j+1].read_pos ==
 * walk[j].read_pos - 1; the last walked cell emits iff it was entered by D or U. */
double oracle_path_adjoint(const abea_aligned_pair_t *walk, int32_t n, int32_t last_from,
                           const char *seq, const abea_event_t *events, const abea_model_t *model,
                           abea_scalings_t sc, const double *theta, int32_t d_kmer, double d_mean,
                           double d_stdv, uint32_t flags, double *grad3, double *gn5,
                           double *grad_model) {
    const double shift = theta ? theta[0] : (double)sc.shift;
    const double scale = theta ? theta[1] : (double)sc.scale;
    const double var = theta ? theta[2] : (double)sc.var;
    const int var_aware = (flags & ORACLE_VAR_AWARE) != 0;
    double g[3] = {0, 0, 0}, h[5] = {0, 0, 0, 0, 0}, em_sum = 0.0;
    for (int32_t j = 0; j < n; ++j) {
        int emits = j + 1 < n ? walk[j + 1].read_pos == walk[j].read_pos - 1 : last_from != FROM_L;
        if (!emits) continue;
        uint32_t rank = oracle_kmer_rank(seq + walk[j].ref_pos);
        const abea_model_t *m = &model[rank];
        double mu = m->level_mean, sig = m->level_stdv, lsd = m->level_log_stdv;
        if ((int32_t)rank == d_kmer) {
            mu += d_mean;
            lsd += log1p(d_stdv / sig);
            sig += d_stdv;
        }
        double sd = sig;
        if (var_aware) {
            sd = sig * var;
            lsd += (double)sc.log_var + log(var / (double)sc.var);
        }
        double x = events[walk[j].read_pos].mean;
        double a = (x - (scale * mu + shift)) / sd;
        em_sum += -0.91893853320467274178 - lsd - 0.5 * a * a;
        g[0] += a / sd;
        g[1] += a * mu / sd;
        if (var_aware) g[2] += (a * a - 1.0) / var;
        h[0] += 1.0 / (sd * sd);
        h[1] += mu / (sd * sd);
        h[2] += mu * mu / (sd * sd);
        h[3] -= a / sd;
        h[4] -= a * mu / sd;
        if (grad_model) {
            grad_model[2 * rank] += a * scale / sd;
            grad_model[2 * rank + 1] += (a * a - 1.0) / sig;
        }
    }
    if (grad3)
        for (int i = 0; i < 3; ++i) grad3[i] = g[i];
    if (gn5)
        for (int i = 0; i < 5; ++i) gn5[i] = h[i];
    return em_sum;
}

/* ---- method-of-moments scalings (no counterpart in the reference) ----
 * f5c's estimate_scalings_using_mom is only a prototype in the reference
 * (GPU/f5cmisc.h:47); restated from the method of moments: the scale and shift
 * that map the k-mer levels along the read onto the mean and variance of the
 * event means.  FP64 serial sums. */
void oracle_mom(const char *seq, int32_t seq_len, const abea_event_t *events, int32_t n_events,
                const abea_model_t *model, double *scale, double *shift) {
    const int32_t n_kmers = seq_len - ABEA_KMER_SIZE + 1;
    if (n_kmers <= 0 || n_events <= 0) {
        *scale = 1.0;
        *shift = 0.0;
        return;
    }
    double es = 0, es2 = 0, ks = 0, ks2 = 0;
    for (int32_t e = 0; e < n_events; ++e) {
        const double x = events[e].mean;
        es += x;
        es2 += x * x;
    }
    for (int32_t k = 0; k < n_kmers; ++k) {
        const double l = model[oracle_kmer_rank(seq + k)].level_mean;
        ks += l;
        ks2 += l * l;
    }
    const double em = es / n_events, ev = es2 / n_events - em * em;
    const double km = ks / n_kmers, kv = ks2 / n_kmers - km * km;
    *scale = sqrt(ev / kv);
    *shift = em - *scale * km;
}

/* ---- postalign (no body in the reference) ----
 * f5c's postalign is only a prototype in the reference (GPU/f5cmisc.h:51-52;
 * its output types index_pair_t and event_alignment_t are GPU/f5c.h:184-207).
 * Restated as two serial loops, for any array of pairs: (1) over the pairs in
 * order, a pair whose event differs from the previous pair's sets its k-mer's
 * map start (when still -1) and stop; (2) over the k-mers in order, one record
 * for every event of each k-mer's range, 'M' when the k-mer's rank differs
 * from the previous record's, else 'E'.  events_per_base = (largest event -
 * smallest event) / n_kmers; 0 with no pairs.  Returns the record count,
 * ABEA_ERR_CAPACITY past out_cap, ABEA_ERR_INVALID_ARG for a pair outside the
 * read. */
int32_t oracle_postalign(abea_event_alignment_t *out, int32_t out_cap, abea_index_pair_t *map,
                         double *events_per_base, const char *seq, int32_t n_kmers,
                         const abea_aligned_pair_t *pairs, int32_t n_pairs, int32_t read_idx) {
    for (int32_t k = 0; k < n_kmers; ++k) {
        map[k].start = -1;
        map[k].stop = -1;
    }
    *events_per_base = 0.0;
    if (n_pairs <= 0) return 0;
    int32_t lo = INT32_MAX, hi = INT32_MIN, prev_event = -1;
    for (int32_t i = 0; i < n_pairs; ++i) {
        const int32_t k = pairs[i].ref_pos, e = pairs[i].read_pos;
        if (k < 0 || k >= n_kmers || e < 0) return ABEA_ERR_INVALID_ARG;
        if (e != prev_event) {
            if (map[k].start == -1) map[k].start = e;
            map[k].stop = e;
        }
        if (e < lo) lo = e;
        if (e > hi) hi = e;
        prev_event = e;
    }
    *events_per_base = (double)(hi - lo) / n_kmers;
    int32_t n = 0, prev_rank = -1;
    for (int32_t k = 0; k < n_kmers; ++k) {
        if (map[k].start == -1) continue;
        const int32_t rank = (int32_t)oracle_kmer_rank(seq + k);
        for (int32_t e = map[k].start; e <= map[k].stop; ++e) {
            if (n >= out_cap) return ABEA_ERR_CAPACITY;
            abea_event_alignment_t *a = &out[n++];
            memset(a, 0, sizeof(*a));
            memcpy(a->ref_kmer, seq + k, ABEA_KMER_SIZE);
            memcpy(a->model_kmer, seq + k, ABEA_KMER_SIZE);
            a->ref_position = k;
            a->read_idx = read_idx;
            a->event_idx = e;
            a->rc = 0;
            a->hmm_state = rank != prev_rank ? 'M' : 'E';
            prev_rank = rank;
        }
    }
    return n;
}
