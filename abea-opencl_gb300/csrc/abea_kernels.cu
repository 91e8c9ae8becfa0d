// abea_kernels.cu — the three ABEA stages as sm_103a kernels.
//
//   pre   (abea_pre_kernel)   k-mer ranks -> per-position scaled pore-model
//                             parameters; event means; last-column init.
//                             Replaces align_kernel_pre_2d (GPU/align_cuda.cl:162-276).
//   core  (abea_core_*)       the adaptive banded max-plus fill.
//                             Replaces align_kernel_core_2d_shm (GPU/align_cuda.cl:297-609).
//   post  (abea_post_kernel)  best end, traceback, reverse, quality checks.
//                             Replaces align_kernel_post (GPU/align_cuda.cl:618-899).
//
// Core kernel shapes:
//   warp  — one warp per read, lane l holds k-mer slots 4l..4l+3.  Neighbour
//           scores move by one shuffle per band; the band move is decided from
//           two shuffled end cells.  No block barrier anywhere.
//   wide  — four warps per read, one slot per thread; the four warps exchange
//           their edge cells through shared memory with one named barrier per
//           band.  Shorter band latency for long reads.
// Both are used by the plain form (one block per read) and the batched form
// (persistent blocks pulling reads longest-first from a device queue).
#include <cuda_runtime.h>
#include <stdint.h>

#include "abea_cell.cuh"
#include "abea_internal.h"
#include "abea_launch.h"

namespace abea {

constexpr unsigned kFull = 0xffffffffu;

__host__ __device__ __forceinline__ int round_up_dev(int x) { return (x + kChunk - 1) & ~(kChunk - 1); }

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

__device__ __forceinline__ float sel4(const float (&v)[4], int j) {
    float r = v[0];
    r = (j == 1) ? v[1] : r;
    r = (j == 2) ? v[2] : r;
    r = (j == 3) ? v[3] : r;
    return r;
}

// k-mer rank, first base most significant; non-ACGT -> 0 (GPU/align_cuda.cl:22-51).
__device__ __forceinline__ uint32_t base_rank(char c) {
    return c == 'C' ? 1u : c == 'G' ? 2u : c == 'T' ? 3u : 0u;
}

__device__ __forceinline__ CellConsts make_consts(const ReadDesc& r, const GlobalConsts& g) {
    CellConsts c;
    c.step_h = r.step_h;
    c.step_l = r.step_l;
    c.stay_h = r.stay_h;
    c.stay_l = r.stay_l;
    c.skip_h = g.skip_h;
    c.skip_l = g.skip_l;
    c.b_max = r.b_max;
    c.em_floor = r.em_floor;
    c.lp_step = r.lp_step;
    c.lp_stay = r.lp_stay;
    c.lp_skip = g.lp_skip;
    return c;
}

// ---------------------------------------------------------------- pre
// One block per read.  Thread t handles k-mer positions t, t+blockDim, ...
__global__ void __launch_bounds__(256) abea_pre_kernel(
    const ReadDesc* __restrict__ reads, int n_reads, GlobalConsts g, const char* __restrict__ seq,
    const abea_event_t* __restrict__ ev_in, const abea_model_t* __restrict__ model,
    float* __restrict__ ev_mean, float* __restrict__ km_gm, float* __restrict__ km_sd,
    float* __restrict__ km_k1, float* __restrict__ last_col) {
    int i = blockIdx.x;
    if (i >= n_reads) return;
    const ReadDesc r = reads[i];
    if (r.skip) return;
    const char* s = seq + r.seq_off;
    int nk = r.n_kmers;
    int nk_pad = (int)round_up_dev(nk);
    for (int k = threadIdx.x; k < nk_pad; k += blockDim.x) {
        float gm = 0.f, sd = 1.f, k1 = 0.f;
        if (k < nk) {
            uint32_t rank = 0;
#pragma unroll
            for (int j = 0; j < ABEA_KMER_SIZE; ++j) rank = (rank << 2) | base_rank(s[k + j]);
            abea_model_t m = model[rank];
            // gp_mean = scale*level_mean + shift; gp_stdv = level_stdv (scaling.var
            // ignored by the reference, GPU/align_cuda.cl:509); log stdv cached.
            gm = __fadd_rn(__fmul_rn(r.scale, m.level_mean), r.shift);
            sd = m.level_stdv;
            float lsd = m.level_log_stdv;
            if (g.var_aware) {
                sd = __fmul_rn(sd, r.var);
                lsd = __fadd_rn(lsd, r.log_var);
            }
            k1 = __fsub_rn(kLogInvSqrt2Pi, lsd);
        }
        km_gm[r.km_off + k] = gm;
        km_sd[r.km_off + k] = sd;
        km_k1[r.km_off + k] = k1;
    }
    int ne = r.n_events;
    int ne_pad = (int)round_up_dev(ne);
    for (int e = threadIdx.x; e < ne_pad; e += blockDim.x) {
        ev_mean[r.ev_off + e] = e < ne ? ev_in[r.ev_src + e].mean : 0.f;
        last_col[r.ev_off + e] = -INFINITY;
    }
}

// ---------------------------------------------------------------- core, warp shape
struct CoreArgs {
    const ReadDesc* reads;
    int n_reads;
    GlobalConsts g;
    const float* ev_mean;
    const float* km_gm;
    const float* km_sd;
    const float* km_k1;
    float* last_col;
    uint8_t* trace;
    float* scores;        // nullptr: scores not kept
    int32_t* band_k0;
    unsigned long long* slow_cells;
    const int32_t* order;  // read order (longest first) for the persistent forms
    int32_t* queue;        // work counter for the persistent forms
    int32_t n_warp_reads;  // reads [0, n_warp_reads) of `order` go to the warp shape
    int32_t spin_limit;
};

struct WarpSmem {
    float gm[kSlots];
    float sd[kSlots];
    float k1[kSlots];
    float ev[kEvRing];
};

// Copies k-mer chunk [c, c+16) of the three parameter arrays into the slot ring
// (lanes 0-11) and event chunk [ce, ce+16) into the event ring (lanes 12-15).
__device__ __forceinline__ void issue_chunks(WarpSmem& sm, const CoreArgs& a, const ReadDesc& r,
                                             int lane, bool do_k, int kc, bool do_e, int ec) {
    if (do_k && lane < 12) {
        int arr = lane >> 2, part = lane & 3;
        const float* src = (arr == 0 ? a.km_gm : arr == 1 ? a.km_sd : a.km_k1) + r.km_off + kc + 4 * part;
        float* dst = (arr == 0 ? sm.gm : arr == 1 ? sm.sd : sm.k1) + ((kc + 4 * part) & (kSlots - 1));
        cp_async16(dst, src);
    }
    if (do_e && lane >= 12 && lane < 16) {
        int part = lane & 3;
        cp_async16(&sm.ev[(ec + 4 * part) & (kEvRing - 1)], a.ev_mean + r.ev_off + ec + 4 * part);
    }
}

template <bool kScores>
__device__ void align_read_warp(const CoreArgs& a, const ReadDesc& r, WarpSmem& sm, int lane) {
    const CellConsts cc = make_consts(r, a.g);
    const int n_events = r.n_events, n_kmers = r.n_kmers, n_bands = r.n_bands;
    const int km_end = (int)round_up_dev(n_kmers), ev_end = (int)round_up_dev(n_events);
    uint8_t* trace = a.trace + r.band_off * kSlots;
    float* scores = kScores ? a.scores + r.band_off * kSlots : nullptr;
    int32_t* bk0 = a.band_k0 + r.band_off;
    float* lastc = a.last_col + r.ev_off;

    // band 1 window (band 0 lower-left is (49,-51), band 1 moved down)
    int k0 = -1 - kBand / 2, e0 = kBand / 2;
    // prefetch rings
    int k_iss = 0, e_iss = 0;
    while (k_iss < km_end && k_iss + 15 <= k0 + 127) {
        issue_chunks(sm, a, r, lane, true, k_iss, false, 0);
        k_iss += kChunk;
    }
    while (e_iss < ev_end && e_iss + 15 <= e0 + 156) {
        issue_chunks(sm, a, r, lane, false, 0, true, e_iss);
        e_iss += kChunk;
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();
    int k_rdy = k_iss, e_rdy = e_iss;

    // band 0: start cell (e=-1,k=-1) = 0 in slot 127; band 1: trim cell
    // (e=0,k=-1) = (float)lp_trim, FROM_U, slot 127 (GPU/align_cuda.cl:249-268).
    float S1[4], LP[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        S1[j] = -INFINITY;
        LP[j] = -INFINITY;
    }
    if (lane == 31) S1[3] = a.g.trim_f;
    if (lane == 0) LP[0] = 0.0f;  // band 0 shifted by one slot: diagonal source of band 2
    uint32_t tacc[4] = {0u, lane == 31 ? (ABEA_FROM_U << 24) : 0u, 0u, 0u};
    if (kScores) {
        float4 z = make_float4(-INFINITY, -INFINITY, -INFINITY, -INFINITY);
        float4 b0 = z, b1 = z;
        if (lane == 31) {
            b0.w = 0.0f;
            b1.w = a.g.trim_f;
        }
        reinterpret_cast<float4*>(scores)[lane] = b0;
        reinterpret_cast<float4*>(scores + kSlots)[lane] = b1;
    }
    int my_k0 = (lane == 0 || lane == 1) ? k0 : 0;
    unsigned long long slow = 0;

    for (int b = 2; b < n_bands; ++b) {
        // ---- band placement (Suzuki-Kasahara), GPU/align_cuda.cl:394-430
        int sl = k0 & 127, su = (k0 + kBand - 1) & 127;
        float ll = __shfl_sync(kFull, sel4(S1, sl & 3), sl >> 2);
        float ur = __shfl_sync(kFull, sel4(S1, su & 3), su >> 2);
        bool right = (ll == -INFINITY && ur == -INFINITY) ? (bool)(b & 1) : (ll < ur);
        if (right)
            ++k0;
        else
            ++e0;

        // ---- prefetch rings
        bool do_k = k_iss < km_end && k_iss + 15 <= k0 + 127;
        bool do_e = e_iss < ev_end && e_iss + 15 <= e0 + 156;
        if (do_k || do_e) {
            issue_chunks(sm, a, r, lane, do_k, k_iss, do_e, e_iss);
            cp_async_commit();
            if (do_k) k_iss += kChunk;
            if (do_e) e_iss += kChunk;
        }
        if ((k0 + kBand - 1 >= k_rdy && k_rdy < km_end) || (e0 >= e_rdy && e_rdy < ev_end)) {
            cp_async_wait_all();
            __syncwarp();
            k_rdy = k_iss;
            e_rdy = e_iss;
        }

        // ---- computed offsets [lo, hi) of this band (GPU/align_cuda.cl:457-470)
        int lo = max(max(-k0, e0 - (n_events - 1)), 0);
        int hi = min(min(n_kmers - k0, e0 + 1), kBand);

        float left[4];
        left[0] = __shfl_sync(kFull, S1[3], (lane + 31) & 31);
        left[1] = S1[0];
        left[2] = S1[1];
        left[3] = S1[2];

        const float4 gm4 = *reinterpret_cast<const float4*>(&sm.gm[4 * lane]);
        const float4 sd4 = *reinterpret_cast<const float4*>(&sm.sd[4 * lane]);
        const float4 k14 = *reinterpret_cast<const float4*>(&sm.k1[4 * lane]);
        const float gmv[4] = {gm4.x, gm4.y, gm4.z, gm4.w};
        const float sdv[4] = {sd4.x, sd4.y, sd4.z, sd4.w};
        const float k1v[4] = {k14.x, k14.y, k14.z, k14.w};

        float d[4], u[4], l[4], em[4];
        bool valid[4], bad[4];
        bool any_bad = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int o = (4 * lane + j - k0) & 127;
            int e = e0 - o;
            valid[j] = (o >= lo) && (o < hi);
            float x = sm.ev[e & (kEvRing - 1)];
            em[j] = emission(x, gmv[j], sdv[j], k1v[j]);
            bool ok;
            candidates_fast(LP[j], S1[j], left[j], em[j], cc, d[j], u[j], l[j], ok);
            bad[j] = valid[j] && !ok;
            any_bad |= bad[j];
        }
        if (__any_sync(kFull, any_bad)) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (bad[j]) {
                    candidates_slow(LP[j], S1[j], left[j], em[j], cc, d[j], u[j], l[j]);
                    ++slow;
                }
        }

        uint32_t word = 0;
        float best[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            uint32_t from;
            float v = pick(d[j], u[j], l[j], from);
            best[j] = valid[j] ? v : -INFINITY;
            word |= (valid[j] ? from : 0u) << (8 * j);
        }
        // trim cell (k = -1, slot 127), GPU/align_cuda.cl:431-443
        if (k0 <= -1 && k0 >= -kBand && lane == 31) {
            int et = e0 + 1 + k0;
            if (et >= 0 && et < n_events) {
                best[3] = __double2float_rn(__dmul_rn(a.g.lp_trim, (double)(et + 1)));
                word = (word & 0x00ffffffu) | (ABEA_FROM_U << 24);
            } else {
                best[3] = -INFINITY;
                word &= 0x00ffffffu;
            }
        }
        // last k-mer column, consumed by the post stage (GPU/align_cuda.cl:722-746)
        {
            int ol = n_kmers - 1 - k0;
            int sl_last = (n_kmers - 1) & 127;
            if (ol >= lo && ol < hi && lane == (sl_last >> 2)) lastc[e0 - ol] = sel4(best, sl_last & 3);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            LP[j] = left[j];
            S1[j] = best[j];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if ((b & 3) == j) tacc[j] = word;
        if ((b & 3) == 3 || b == n_bands - 1) {
            reinterpret_cast<uint4*>(trace + (int64_t)(b >> 2) * 512)[lane] =
                make_uint4(tacc[0], tacc[1], tacc[2], tacc[3]);
            tacc[0] = tacc[1] = tacc[2] = tacc[3] = 0u;
        }
        if (kScores)
            reinterpret_cast<float4*>(scores + (int64_t)b * kSlots)[lane] =
                make_float4(best[0], best[1], best[2], best[3]);
        if ((b & 31) == lane) my_k0 = k0;
        if ((b & 31) == 31 || b == n_bands - 1) {
            int base = b & ~31;
            if (lane <= (b & 31)) bk0[base + lane] = my_k0;
        }
    }
    // band_k0 of bands 0 and 1 is written by the first 32-band flush (lanes 0
    // and 1 start with k0 = -51); n_bands >= 4 whenever a read is aligned.
    cp_async_wait_all();  // no copy may land in shared memory after the read is done
    __syncwarp();
    if (slow) atomicAdd(a.slow_cells, slow);
}

// Plain form: one block (one warp) per read.
template <bool kScores>
__global__ void __launch_bounds__(32) abea_core_warp_kernel(CoreArgs a) {
    __shared__ __align__(16) WarpSmem sm;
    int i = blockIdx.x;
    if (i >= a.n_reads) return;
    const ReadDesc r = a.reads[i];
    if (r.skip) return;
    align_read_warp<kScores>(a, r, sm, threadIdx.x);
}

// ---------------------------------------------------------------- post
struct PostArgs {
    const ReadDesc* reads;
    int n_reads;
    GlobalConsts g;
    const float* ev_mean;
    const float* km_gm;
    const float* km_sd;
    const float* km_k1;
    const float* last_col;
    const uint8_t* trace;
    const int32_t* band_k0;
    abea_aligned_pair_t* pairs;
    int32_t* n_pairs;
    float* best_scores;
    int32_t* status;   // per-read abea_status_t (0 = ok)
    const int32_t* order;
    int32_t* queue;
};

constexpr int kPostChunkBands = 64;  // trace bands staged per shared-memory chunk

struct PostSmem {
    uint8_t tr[2][kPostChunkBands * kSlots];
};

// Emission of path cell (k, e), as in the fill.
__device__ __forceinline__ float path_emission(const PostArgs& a, const ReadDesc& r, int k, int e) {
    int64_t ko = r.km_off + k;
    return emission(a.ev_mean[r.ev_off + e], a.km_gm[ko], a.km_sd[ko], a.km_k1[ko]);
}

// One traceback step: backpointer -> next cell; returns false for L moves' gap.
__device__ __forceinline__ void step_back(uint32_t from, int& k, int& e, int& gap, int& max_gap) {
    if (from == ABEA_FROM_D) {
        --k;
        --e;
        gap = 0;
    } else if (from == ABEA_FROM_U) {
        --e;
        gap = 0;
    } else {
        --k;
        ++gap;
        max_gap = max(max_gap, gap);
    }
}

// Serial double sum of the path's emissions in the reference's order (from the
// walk's first cell backwards), re-walking the trace from global memory.  Used
// only when the path does not fit its output slot.  `flat` re-walks through the
// emulated flat band array (no finite end, see post_read_warp).
__device__ double serial_path_sum(const PostArgs& a, const ReadDesc& r, const uint8_t* trace,
                                  const int32_t* bk0, bool flat, int e, int k) {
    double sum = 0.0;
    int gap = 0, mg = 0;
    while (k >= 0 && e >= 0) {
        sum = __dadd_rn(sum, (double)path_emission(a, r, k, e));
        int64_t band = (int64_t)e + k + 2;
        if (flat) {
            int64_t f = band * kBand + ((band - 2 - bk0[band]) - e);
            if (f < 0 || f >= (int64_t)r.n_bands * kBand) break;
            int64_t b2 = f / kBand;
            int o2 = (int)(f - b2 * kBand);
            step_back(trace[trace_index(b2, (bk0[b2] + o2) & 127)], k, e, gap, mg);
        } else {
            step_back(trace[trace_index(band, k & 127)], k, e, gap, mg);
        }
    }
    return sum;
}

// One warp per read: best end, traceback, reverse, QC (GPU/align_cuda.cl:618-899).
__device__ void post_read_warp(const PostArgs& a, int ri, PostSmem& sm, int lane) {
    const ReadDesc r = a.reads[ri];
    if (r.skip) {
        if (lane == 0) {
            a.n_pairs[ri] = 0;
            a.best_scores[ri] = -INFINITY;
            a.status[ri] = 0;
        }
        return;
    }
    const int n_events = r.n_events, n_kmers = r.n_kmers, n_bands = r.n_bands;
    const double lp_trim = a.g.lp_trim;
    const float* lastc = a.last_col + r.ev_off;

    // ---- best end: first strict maximum of s(e) = (float)(band + (n_events-e)*lp_trim)
    float best = -INFINITY;
    int best_e = 0x7fffffff;
    for (int e = lane; e < n_events; e += 32) {
        float s = __double2float_rn(
            __dadd_rn((double)lastc[e], __dmul_rn((double)(n_events - e), lp_trim)));
        if (s > best) {
            best = s;
            best_e = e;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        float ob = __shfl_xor_sync(kFull, best, off);
        int oe = __shfl_xor_sync(kFull, best_e, off);
        if (ob > best || (ob == best && oe < best_e)) {
            best = ob;
            best_e = oe;
        }
    }
    if (!(best > -INFINITY)) best_e = 0;

    abea_aligned_pair_t* out = a.pairs + r.out_off;
    const uint8_t* trace = a.trace + r.band_off * kSlots;
    const int32_t* bk0 = a.band_k0 + r.band_off;
    const int cap = r.out_cap;
    int n_out = 0, max_gap = 0, status = 0, last_k = n_kmers - 1;

    if (best > -INFINITY) {
        // A finite end: the path only visits computed cells.  Walked by lane 0
        // over shared-memory chunks of 64 bands, the next chunk in flight.
        int cur_e = best_e, cur_k = n_kmers - 1, gap = 0;
        int chunk_lo = ((cur_e + cur_k + 2) / kPostChunkBands) * kPostChunkBands;
        const int bands_pad = (n_bands + 3) & ~3;
        int buf = 0;
        auto stage = [&](int lo_band, int which) {
            int bytes = min(kPostChunkBands, bands_pad - lo_band) * kSlots;
            const uint8_t* src = trace + (int64_t)lo_band * kSlots;
            for (int off = lane * 16; off < bytes; off += 32 * 16) cp_async16(&sm.tr[which][off], src + off);
            cp_async_commit();
        };
        stage(chunk_lo, buf);
        bool done = false;
        while (!done) {
            cp_async_wait_all();
            __syncwarp();
            int next_lo = chunk_lo - kPostChunkBands;
            if (next_lo >= 0) stage(next_lo, buf ^ 1);
            if (lane == 0) {
                while (true) {
                    if (cur_k < 0 || cur_e < 0) {
                        done = true;
                        break;
                    }
                    int band = cur_e + cur_k + 2;
                    if (band < chunk_lo) break;
                    if (n_out < cap) out[n_out] = abea_aligned_pair_t{cur_k, cur_e};
                    ++n_out;
                    last_k = cur_k;
                    int lb = band - chunk_lo, slot = cur_k & 127;
                    uint32_t from = sm.tr[buf][(lb >> 2) * 512 + (slot >> 2) * 16 + (lb & 3) * 4 + (slot & 3)];
                    step_back(from, cur_k, cur_e, gap, max_gap);
                }
            }
            done = __shfl_sync(kFull, (int)done, 0) != 0;
            chunk_lo = next_lo;
            buf ^= 1;
            if (chunk_lo < 0) done = true;
        }
        cp_async_wait_all();
        __syncwarp();
    } else if (lane == 0) {
        // No finite end: the reference walks from (0, n_kmers-1) through its flat
        // band array, where an offset outside the band reads a neighbouring row.
        // Emulated cell by cell from band_k0; reads outside the read's rows have
        // no defined answer.
        int cur_e = 0, cur_k = n_kmers - 1, gap = 0;
        while (cur_k >= 0 && cur_e >= 0) {
            if (n_out < cap) out[n_out] = abea_aligned_pair_t{cur_k, cur_e};
            ++n_out;
            last_k = cur_k;
            int64_t band = (int64_t)cur_e + cur_k + 2;
            int64_t flat = band * kBand + ((band - 2 - bk0[band]) - cur_e);
            if (flat < 0 || flat >= (int64_t)n_bands * kBand) {
                status = ABEA_ERR_UNDEFINED;
                break;
            }
            int64_t b2 = flat / kBand;
            int o2 = (int)(flat - b2 * kBand);
            step_back(trace[trace_index(b2, (bk0[b2] + o2) & 127)], cur_k, cur_e, gap, max_gap);
        }
    }
    n_out = __shfl_sync(kFull, n_out, 0);
    max_gap = __shfl_sync(kFull, max_gap, 0);
    status = __shfl_sync(kFull, status, 0);
    last_k = __shfl_sync(kFull, last_k, 0);
    __syncwarp();
    __threadfence_block();

    int result = 0;
    if (status == 0 && n_out > 0) {
        // QC (GPU/align_cuda.cl:856-882).  After the reversal out[0] is the last
        // cell walked and out[n-1] the first, so spanned <=> last_k == 0.
        double sum;
        if (n_out <= cap) {
            // Every emission with 0.5 <= |em| < 2^20 is a multiple of 2^-24; when
            // the magnitudes sum below 2^29 all of the reference's partial double
            // sums are exact and equal this integer sum, in any order.
            long long isum = 0, iabs = 0;
            bool exact = true;
            for (int i2 = lane; i2 < n_out; i2 += 32) {
                abea_aligned_pair_t p = out[i2];
                float em = path_emission(a, r, p.ref_pos, p.read_pos);
                float aem = fabsf(em);
                if (aem >= 0.5f && aem < 1048576.0f) {
                    long long q = __float2ll_rn(__fmul_rn(em, 16777216.0f));
                    isum += q;
                    iabs += q < 0 ? -q : q;
                } else {
                    exact = false;
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                isum += __shfl_xor_sync(kFull, isum, off);
                iabs += __shfl_xor_sync(kFull, iabs, off);
            }
            exact = __all_sync(kFull, exact) && iabs < (1ll << 53);
            if (exact) {
                sum = __dmul_rn((double)isum, 5.9604644775390625e-08);  // * 2^-24
            } else {
                sum = 0.0;  // serial, in walk order (out[0] is the first cell walked)
                if (lane == 0)
                    for (int i2 = 0; i2 < n_out; ++i2)
                        sum = __dadd_rn(sum, (double)path_emission(a, r, out[i2].ref_pos, out[i2].read_pos));
                sum = __shfl_sync(kFull, sum, 0);
            }
        } else {
            sum = 0.0;
            if (lane == 0) sum = serial_path_sum(a, r, trace, bk0, !(best > -INFINITY), best > -INFINITY ? best_e : 0, n_kmers - 1);
            sum = __shfl_sync(kFull, sum, 0);
        }
        double avg = __ddiv_rn(sum, (double)n_out);
        bool pass = !(avg < -5.0) && last_k == 0 && max_gap <= 50;
        if (pass && n_out > cap) {
            status = ABEA_ERR_CAPACITY;
            result = ABEA_ERR_CAPACITY;
        } else if (pass) {
            // reverse in place (GPU/align_cuda.cl:830-843)
            for (int i2 = lane; i2 < n_out / 2; i2 += 32) {
                abea_aligned_pair_t x = out[i2], y = out[n_out - 1 - i2];
                out[i2] = y;
                out[n_out - 1 - i2] = x;
            }
            result = n_out;
        }
    } else if (status != 0) {
        result = status;
    }
    if (lane == 0) {
        a.n_pairs[ri] = result;
        a.best_scores[ri] = best;
        a.status[ri] = status;
    }
}

__global__ void __launch_bounds__(32) abea_post_kernel(PostArgs a) {
    __shared__ __align__(16) PostSmem sm;
    int i = blockIdx.x;
    if (i >= a.n_reads) return;
    post_read_warp(a, i, sm, threadIdx.x);
}

}  // namespace abea

// ---------------------------------------------------------------- launches
namespace abea {

static CoreArgs core_args(const LaunchArgs& a) {
    CoreArgs c;
    c.reads = a.reads;
    c.n_reads = a.n_reads;
    c.g = a.g;
    c.ev_mean = a.ev_mean;
    c.km_gm = a.km_gm;
    c.km_sd = a.km_sd;
    c.km_k1 = a.km_k1;
    c.last_col = a.last_col;
    c.trace = a.trace;
    c.scores = a.scores;
    c.band_k0 = a.band_k0;
    c.slow_cells = a.slow;
    c.order = a.order;
    c.queue = a.queue;
    c.n_warp_reads = a.n_reads - a.n_wide;
    c.spin_limit = a.spin_limit;
    return c;
}

static PostArgs post_args(const LaunchArgs& a) {
    PostArgs p;
    p.reads = a.reads;
    p.n_reads = a.n_reads;
    p.g = a.g;
    p.ev_mean = a.ev_mean;
    p.km_gm = a.km_gm;
    p.km_sd = a.km_sd;
    p.km_k1 = a.km_k1;
    p.last_col = a.last_col;
    p.trace = a.trace;
    p.band_k0 = a.band_k0;
    p.pairs = a.pairs;
    p.n_pairs = a.n_pairs;
    p.best_scores = a.best;
    p.status = a.status;
    p.order = a.order;
    p.queue = a.queue;
    return p;
}

cudaError_t launch_plain(const LaunchArgs& a, int* launches) {
    int n = a.n_reads;
    abea_pre_kernel<<<n, 128, 0, a.stream>>>(a.reads, n, a.g, a.seq, a.ev_in, a.model, a.ev_mean, a.km_gm,
                                             a.km_sd, a.km_k1, a.last_col);
    cudaEventRecord(a.ev_pre, a.stream);
    CoreArgs c = core_args(a);
    if (a.scores)
        abea_core_warp_kernel<true><<<n, 32, 0, a.stream>>>(c);
    else
        abea_core_warp_kernel<false><<<n, 32, 0, a.stream>>>(c);
    cudaEventRecord(a.ev_core, a.stream);
    abea_post_kernel<<<n, 32, 0, a.stream>>>(post_args(a));
    *launches = 3;
    return cudaGetLastError();
}

cudaError_t launch_batched(const LaunchArgs& a, int* launches) { return launch_plain(a, launches); }

int choose_wide_reads(const std::vector<ReadDesc>&, const std::vector<int32_t>&, int, int64_t) { return 0; }

}  // namespace abea
