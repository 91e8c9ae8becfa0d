// abea_launch.h — kernel launch entry points used by the host orchestration.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "abea_internal.h"

namespace abea {

struct LaunchArgs {
    const ReadDesc* reads;
    int n_reads;
    GlobalConsts g;
    const char* seq;
    const abea_event_t* ev_in;
    const abea_model_t* model;
    float* ev_mean;
    float* km_gm;
    float* km_sd;
    float* km_k1;
    float* last_col;
    uint8_t* trace;
    float* scores;  // nullptr: scores not kept
    int32_t* band_k0;
    abea_aligned_pair_t* pairs;
    int32_t* n_pairs;
    float* best;
    int32_t* status;
    unsigned long long* slow;
    const int32_t* order;  // read indices, longest first
    int32_t* queue;        // zeroed work counters
    int32_t n_wide;        // leading reads of `order` that run on the wide shape
    int sm_count;
    int32_t spin_limit;
    cudaStream_t stream;
    cudaEvent_t ev_pre;   // recorded after pre
    cudaEvent_t ev_core;  // recorded after core
};

// Plain form: pre, core, post — one block per read each, as the reference.
cudaError_t launch_plain(const LaunchArgs& a, int* launches);
// Batched form: pre, then one persistent fused core+post kernel.
cudaError_t launch_batched(const LaunchArgs& a, int* launches);
// Number of leading reads of `order` that the batched form runs on the wide shape.
int choose_wide_reads(const std::vector<ReadDesc>& reads, const std::vector<int32_t>& order, int sm_count,
                      int64_t long_read_bands);

}  // namespace abea
