/* f5c's GPU batch entry, align_cuda(core, db) (reference GPU/f5cmisc.h:99-102),
 * on this library: the shim a maintainer adds to f5c, compiled and run by
 * tests/test_f5c_shim.py.  f5c's own core_t and db_t (GPU/f5c.h:291-348, 386-)
 * hold many more members (htslib handles, C++ maps); the mirrors below keep
 * only the members the shim reads, with f5c's names and types, so that the
 * shim's body is the one f5c would compile against its own f5c.h.
 *
 * No long-read routing: f5c sends reads over `ultra_thresh` bases, or over
 * `cuda_max_readlen` times the batch's mean length, to the CPU
 * (GPU/f5c.h:98,105).  Here every read goes to the GPU: the device batch is
 * sized per call, and reads whose trace would not fit a memory budget keep
 * band-score checkpoints instead (ABEA_OPT_TRACE_BUDGET). */
#include <stdio.h>
#include <stdlib.h>

#include "abea.h"

/* ---- the members of f5c's structures that the shim uses ---------------- */
typedef abea_event_table_t event_table;     /* GPU/f5c.h:125-130 */
typedef abea_scalings_t scalings_t;         /* GPU/f5c.h:148-154 */
typedef abea_model_t model_t;               /* GPU/f5c.h:133-138 */
typedef abea_aligned_pair_t AlignedPair;    /* GPU/f5c.h:178-181 */

typedef struct {
    int32_t cuda_dev_id;                    /* opt_t: the GPU f5c was told to use */
} opt_t;

typedef struct {
    model_t *model;                         /* the pore model, 4096 entries */
    opt_t opt;
} core_t;

typedef struct {
    int32_t n_bam_rec;                      /* reads in the batch */
    char **read;                            /* read sequences (NUL terminated) */
    int32_t *read_len;
    event_table *et;                        /* event table per read */
    scalings_t *scalings;                   /* per-read scalings */
    AlignedPair **event_align_pairs;        /* per-read output, 2*et[i].n pairs each */
    int32_t *n_event_align_pairs;           /* per-read count (0: failed QC) */
} db_t;

/* ---- the shim ------------------------------------------------------------ */
void align_cuda(core_t *core, db_t *db) {
    static abea_ctx_t *ctx; /* one context per process: f5c calls align_cuda from one thread */
    if (!ctx && abea_ctx_create(&ctx, core->opt.cuda_dev_id, ABEA_MODE_BATCHED) != ABEA_OK) {
        fprintf(stderr, "abea: %s\n", abea_last_error());
        exit(EXIT_FAILURE);
    }
    abea_status_t st = abea_align_db(ctx, db->n_bam_rec, db->read, db->read_len, db->et, db->scalings,
                                     core->model, db->event_align_pairs, db->n_event_align_pairs);
    if (st != ABEA_OK && st != ABEA_ERR_CAPACITY) fprintf(stderr, "abea: %s\n", abea_last_error());
    for (int32_t i = 0; i < db->n_bam_rec; ++i) /* a per-read error counts as a failed alignment */
        if (db->n_event_align_pairs[i] < 0) db->n_event_align_pairs[i] = 0;
}

/* Test entry: fills the two structures from plain arrays and calls the shim. */
int shim_align_batch(int32_t dev, int32_t n, char **read, int32_t *read_len, event_table *et,
                     scalings_t *scalings, model_t *model, AlignedPair **out, int32_t *counts) {
    core_t core;
    core.model = model;
    core.opt.cuda_dev_id = dev;
    db_t db;
    db.n_bam_rec = n;
    db.read = read;
    db.read_len = read_len;
    db.et = et;
    db.scalings = scalings;
    db.event_align_pairs = out;
    db.n_event_align_pairs = counts;
    align_cuda(&core, &db);
    return 0;
}
