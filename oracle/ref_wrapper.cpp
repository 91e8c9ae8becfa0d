/* C entry around the reference's own ABEA code, compiled from its sources by
 * build_ref.sh into oracle/_ref/libref.so.  TEST INFRASTRUCTURE ONLY: used to
 * pin the oracle restatement on synthetic reads.
 *   fill: align_kernel_single (FPGA/code/device/align_swi.cl:157-663), compiled as C
 *   post: host_post_processing (FPGA/code/host/src/align_swi.cpp:1093-1314)
 * The types below restate the host-side layouts of FPGA/code/host/src/f5c.h
 * (CACHED_LOG on) and the device-side event1_t / scalings_t of
 * FPGA/code/device/f5c.h:108-164 (packed, 32-byte aligned). */
#include <assert.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

typedef int64_t ptr_t;
typedef struct { uint64_t start; float length; float mean; float stdv; } event_t;
typedef struct { float level_mean; float level_stdv; float level_log_stdv; } model_t;
typedef struct { float scale; float shift; float var; float log_var; } scalings_t;
typedef struct { int event_idx; int kmer_idx; } EventKmerPair;
typedef struct { int ref_pos; int read_pos; } AlignedPair;
#define KMER_SIZE 6
#define ALN_BANDWIDTH 100
#define CACHED_LOG 1
#define WARNING(arg, ...) ((void)0)
#define bandwidth ALN_BANDWIDTH
#define half_bandwidth ALN_BANDWIDTH / 2
#define max_gap_threshold 50
#define min_average_log_emission -5.0
#define epsilon 1e-10
#define FROM_D 0
#define FROM_U 1
#define FROM_L 2

#include "host_post.inc"

struct __attribute__((packed, aligned(32))) dev_event1_t { uint64_t start; float length; float mean; float stdv; };
struct __attribute__((packed, aligned(32))) dev_scalings_t { float scale; float shift; float var; float log_var; };

extern "C" void align_kernel_single(char *read, int32_t *read_len, ptr_t *read_ptr,
                                    dev_event1_t *event_table, int32_t *n_events1,
                                    ptr_t *event_ptr, dev_scalings_t *scalings, model_t *models,
                                    int32_t n_bam_rec, uint32_t *kmer_ranks1, float *bands1,
                                    uint8_t *trace1, EventKmerPair *band_lower_lefts);

/* One read through the reference's fill + host post.  Returns the pair count;
 * bands/trace/bll (reference layout, n_bands rows) are copied out when non-null. */
extern "C" int32_t ref_align(AlignedPair *out, int32_t cap, const char *seq, int32_t len,
                             const event_t *ev, int32_t n_ev, const model_t *model,
                             scalings_t sc, float *bands_out, uint8_t *trace_out,
                             EventKmerPair *bll_out) {
    int32_t n_kmers = len - KMER_SIZE + 1;
    if (n_kmers <= 0 || n_ev <= 0) return 0;
    int64_t rows = (int64_t)len + 1 + n_ev; /* (read_ptr + event_ptr) stride of the reference */
    std::vector<char> read(len + 1, 0);
    memcpy(read.data(), seq, len);
    int32_t read_len = len, n_events = n_ev;
    ptr_t zero = 0;
    std::vector<dev_event1_t> dev_ev(n_ev);
    for (int32_t i = 0; i < n_ev; ++i) {
        dev_ev[i].start = ev[i].start;
        dev_ev[i].length = ev[i].length;
        dev_ev[i].mean = ev[i].mean;
        dev_ev[i].stdv = ev[i].stdv;
    }
    dev_scalings_t dsc;
    dsc.scale = sc.scale; dsc.shift = sc.shift; dsc.var = sc.var; dsc.log_var = sc.log_var;
    std::vector<model_t> models(model, model + 4096);
    std::vector<uint32_t> ranks(len + 1);
    std::vector<float> bands(rows * ALN_BANDWIDTH);
    std::vector<uint8_t> trace(rows * ALN_BANDWIDTH);
    std::vector<EventKmerPair> bll(rows);
    align_kernel_single(read.data(), &read_len, &zero, dev_ev.data(), &n_events, &zero, &dsc,
                        models.data(), 1, ranks.data(), bands.data(), trace.data(), bll.data());
    std::vector<AlignedPair> pairs((size_t)2 * n_ev + (size_t)len + 8);
    std::vector<event_t> hev(ev, ev + n_ev);
    int32_t n_out = 0;
    host_post_processing(pairs.data(), &n_out, read.data(), &read_len, &zero, hev.data(),
                         &n_events, &zero, &sc, models.data(), 1, ranks.data(), bands.data(),
                         trace.data(), bll.data());
    int64_t n_bands = (int64_t)n_ev + n_kmers + 2;
    if (bands_out) memcpy(bands_out, bands.data(), sizeof(float) * n_bands * ALN_BANDWIDTH);
    if (trace_out) memcpy(trace_out, trace.data(), n_bands * ALN_BANDWIDTH);
    if (bll_out) memcpy(bll_out, bll.data(), sizeof(EventKmerPair) * n_bands);
    if (n_out > cap) return -2;
    memcpy(out, pairs.data(), sizeof(AlignedPair) * n_out);
    return n_out;
}
