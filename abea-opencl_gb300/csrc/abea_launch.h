// abea_launch.h — kernel arguments and launch entry points used by the host
// orchestration (abea_host.cu) and defined in abea_kernels.cu.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "abea_internal.h"

extern "C" const char* abea_internal_set_error(const char* msg);

namespace abea {

// Pinned host memory of abea_align_batch's caller that the pre stage reads each
// read's bases and events from (device-mapped; no copy to HBM first), or nulls.
struct InMirror {
    const char* seq;
    const abea_event_t* ev;
};

struct PreArgs {
    const ReadDesc* reads;
    int n_reads;
    GlobalConsts g;
    const char* seq;
    const abea_event_t* ev_in;
    const abea_model_t* model;
    float* ev_mean;
    float* km_gm;
    float* km_sd;
    float* km_rsd;
    float* km_k1;
    float* last_col;
    const InMirror* inm;  // nullptr, or a device copy of the input mirror
};

struct CoreArgs {
    const ReadDesc* reads;
    int n_reads;
    GlobalConsts g;
    const float* ev_mean;
    const float* km_gm;
    const float* km_sd;
    const float* km_rsd;
    const float* km_k1;
    float* last_col;
    uint8_t* trace;
    float* scores;                 // nullptr: scores not kept
    int32_t* band_k0;
    unsigned long long* counters;  // [0] cells on the FP64 tier, [1] cells on the exact-all tier
    const int32_t* order;          // read indices, longest first
    int32_t* queue;                // zeroed work counters of the batched form
    int32_t n_wide;                // leading reads of `order` that run on the wide shape
    float* ck;                     // checkpoint records of checkpointed reads
    uint8_t* ck_scratch;           // recompute scratch: kCkBands bands of trace per checkpointed read
    int32_t* spec;                 // traceback cell maps: kSpecRound * kSpecBands int32 per slot
    int32_t n_spec;                // slots (queue[2] hands them out)
    long long spin_limit;          // polls before a device-side wait gives up (counters[2] counts those)
    int32_t n_mid;                 // the reads after the wide ones that run on the medium shape (batched form)
};

// Host memory the kernels write each read's results into as the read finishes
// (device-mapped pinned buffers of abea_align_batch's caller), or nulls.
struct OutMirror {
    abea_aligned_pair_t* pairs;  // the caller's event_align_pairs
    int32_t* n_pairs;            // the caller's n_event_align_pairs
};

struct PostArgs {
    const ReadDesc* reads;
    int n_reads;
    GlobalConsts g;
    const float* ev_mean;
    const float* km_gm;
    const float* km_sd;
    const float* km_k1;
    const float* km_rsd;
    const float* last_col;
    const uint8_t* trace;
    const int32_t* band_k0;
    abea_aligned_pair_t* pairs;
    int32_t* n_pairs;
    float* best_scores;
    int32_t* status;  // per-read abea_status_t (0 = ok)
    int32_t* path_len;    // optional (nullptr): path length, for the adjoint
    int32_t* path_flags;  // kPath* bits | move into the last walked cell << 8
    int32_t* best_event;  // event of the best end
    const OutMirror* outm;  // nullptr, or a device copy of the mirror (batched form)
};

constexpr int32_t kPathReversed = 1, kPathTruncated = 2, kPathNoEnd = 4, kPathError = 8;

struct AdjArgs {
    const ReadDesc* reads;
    int n_reads;
    int var_aware;
    const char* seq;
    const abea_model_t* model;
    const float* ev_mean;
    const abea_aligned_pair_t* pairs;
    const int32_t* path_len;
    const int32_t* path_flags;
    double* grad_scalings;  // [n][3]: d/d shift, scale, var
    double* gn;             // [n][5]: J^T J (11, 12, 22), J^T r (1, 2) of the (shift, scale) residuals
    double* path_em;        // [n]: sum of the path's emissions (FP64)
    double* grad_model;     // [4096][2]: d/d level_mean, level_stdv, summed over reads
    int32_t* adj_status;    // [n]: 0, or why the read has no gradient
};

// Backward pass over the stored paths of a finished forward run.
cudaError_t launch_adjoint(const AdjArgs& a, cudaStream_t stream);

struct MomArgs {
    const ReadDesc* reads;
    int n_reads;
    const char* seq;
    const abea_event_t* ev;
    const abea_model_t* model;
    double* out;  // [n][2]: scale, shift
};

// Method-of-moments scalings, one warp per read.
cudaError_t launch_mom(const MomArgs& a, cudaStream_t stream);

struct PostalignArgs {
    const ReadDesc* reads;
    int n_reads;
    const char* seq;
    const abea_aligned_pair_t* pairs;  // the run's AlignedPairs (2*event_ptr per read)
    const int32_t* n_pairs;
    abea_index_pair_t* map;            // [seq bytes], preset to {-1, -1}; read i from seq_off
    abea_event_alignment_t* rec;       // [events], preset to 0; read i from ev_src (32-byte aligned)
    double* epb;                       // [n] events per base
    int32_t* count;                    // [n] records, or ABEA_ERR_INTERNAL for a malformed path
};

// f5c's postalign over a finished run's AlignedPairs, one warp per read.
cudaError_t launch_postalign(const PostalignArgs& a, cudaStream_t stream);

struct LaunchArgs {
    PreArgs pre;
    CoreArgs core;
    PostArgs post;
    int sm_count;
    cudaStream_t stream;
    cudaEvent_t ev_pre;   // recorded after pre
    cudaEvent_t ev_core;  // recorded after core (batched: after the fused core+post)
    bool capturing;       // the launches are being captured into a CUDA graph
    bool cluster;         // batched form on clusters of two blocks (the cluster-pair wide shape)
};

// Plain form: pre, core, post — one block per read each, as the reference.
cudaError_t launch_plain(const LaunchArgs& a, int* launches);
// Batched form: pre, then one persistent fused core+post kernel.
cudaError_t launch_batched(const LaunchArgs& a, int* launches);
// Resident blocks per SM of the batched kernel.
int batched_blocks_per_sm(bool scores);

// Per-read constants of one read laid out at offset 0 of every scratch region.
ReadDesc describe_single_read(int32_t sequence_len, int32_t n_events, abea_scalings_t sc, int32_t out_capacity);
GlobalConsts parity_consts();

}  // namespace abea
