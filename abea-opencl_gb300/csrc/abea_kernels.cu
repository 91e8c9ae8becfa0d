// abea_kernels.cu — the three ABEA stages as sm_103a kernels.
//
//   pre   (abea_pre_kernel)    k-mer ranks -> per-position scaled pore-model
//                              parameters; event means; last-column init.
//                              Replaces align_kernel_pre_2d (GPU/align_cuda.cl:162-276).
//   core                       the adaptive banded max-plus fill.
//                              Replaces align_kernel_core_2d_shm (GPU/align_cuda.cl:297-609).
//   post  (post_read_warp)     best end, traceback, reverse, quality checks.
//                              Replaces align_kernel_post (GPU/align_cuda.cl:618-899).
//
// Fill shapes (all bit-exact, same trace layout):
//   warp   — one warp per read, lane l holds k-mer slots 4l..4l+3.  Neighbour
//            scores move by one shuffle per band, the band move is decided from two
//            shuffled end cells; no block barrier.  Most reads per SM.
//   wide   — twelve warps of a 512-thread block per read (fill_chain): four run
//            the band-to-band chain (one slot per thread, one barrier per band, cells
//            exchanged in shared memory), eight compute the emissions and their exact
//            splits up to 16 bands ahead into a ring.  Shortest band latency.
//   medium — the same chain and producer with four producer warps, two reads per
//            block (off unless tuned).
// Forms:
//   plain   — pre, core (warp shape, one block per read), post (one block per
//             read): the reference's three launches.
//   batched — one persistent kernel of one block per SM (each read's pre runs
//             in the block or warp that fills it): the blocks take the wide reads
//             from a queue, longest first, one after another, each walking its
//             read's traceback with the whole block (post_wide_block); then the
//             medium reads; the blocks without a wide read take the first wave of the
//             other reads round-robin, one per warp, and then every warp pulls the
//             rest longest-first from a device queue; a warp-shape read's post runs
//             in the warp that filled it, right after its fill (trace still in L2).
//   The wide shape on a cluster of two blocks (emissions on the second SM) is an
//   option, measured slower.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "abea_cell.cuh"
#include "abea_internal.h"
#include "abea_launch.h"

namespace abea {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kPostChunkBands = 16;  // trace bands per chunk of post's four-chunk shared-memory ring

__host__ __device__ __forceinline__ int round_up_dev(int x) { return (x + kChunk - 1) & ~(kChunk - 1); }

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_group1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ float sel4(const float (&v)[4], int j) {
    float r = v[0];
    r = (j == 1) ? v[1] : r;
    r = (j == 2) ? v[2] : r;
    r = (j == 3) ? v[3] : r;
    return r;
}

// k-mer rank, first base most significant; non-ACGT -> 0 (GPU/align_cuda.cl:22-51).
__device__ __forceinline__ uint32_t base_rank(char c) { return c == 'C' ? 1u : c == 'G' ? 2u : c == 'T' ? 3u : 0u; }

__device__ __forceinline__ CellConsts make_consts(const ReadDesc& r, const GlobalConsts& g) {
    CellConsts c;
    c.step_h = r.step_h;
    c.step_l = r.step_l;
    c.stay_h = r.stay_h;
    c.stay_l = r.stay_l;
    c.skip_h = g.skip_h;
    c.skip_l = g.skip_l;
    c.lp_step = r.lp_step;
    c.lp_stay = r.lp_stay;
    c.lp_skip = g.lp_skip;
    return c;
}

// ---------------------------------------------------------------- pre
// One block per read; thread t handles k-mer positions t, t+blockDim, ...
// Pre of read i by nt cooperating threads (thread index t): the read's k-mer
// parameters, event means and last-column initialisation.  The batched form runs
// it in the block or warp that fills the read, just before the fill.
//
// The bases and events come from HBM, or, when the caller's buffers are pinned
// (a.inm), straight from host memory over the CPU-GPU link: no copy of the
// inputs precedes the kernel, and every read's pre stage loads its own (but the
// first few reads the kernel starts, copied to HBM before it: in_hbm).  A thread
// takes kPreUnroll k-mer positions (kEvUnroll events) per pass with every load
// issued before any use (indexes clamped into the read), so that many round trips
// to host memory are in flight at once: a warp-shape read's pre stage is latency-
// bound on them (a k-mer's six bases share the cache lines of its neighbours').
constexpr int kPreUnroll = 4, kEvUnroll = 16;
__device__ __forceinline__ void pre_read(const PreArgs& a, int i, int t, int nt) {
    const ReadDesc r = a.reads[i];
    if (r.skip) return;
    const InMirror* m = r.in_hbm ? nullptr : a.inm;
    const char* seq = a.seq;
    const abea_event_t* ev_in = a.ev_in;
    if (m) {
        const InMirror mv = *m;
        if (mv.seq) seq = mv.seq;
        if (mv.ev) ev_in = mv.ev;
    }
    const char* s = seq + r.seq_off;
    const int nk = r.n_kmers, nk_pad = round_up_dev(nk);
    for (int k0 = t; k0 < nk_pad; k0 += kPreUnroll * nt) {
        char base[kPreUnroll][ABEA_KMER_SIZE];
#pragma unroll
        for (int u = 0; u < kPreUnroll; ++u) {
            const int kc = min(k0 + u * nt, nk - 1);  // nk >= 1: the read is not skipped
#pragma unroll
            for (int j = 0; j < ABEA_KMER_SIZE; ++j) base[u][j] = s[kc + j];
        }
#pragma unroll
        for (int u = 0; u < kPreUnroll; ++u) {
            const int k = k0 + u * nt;
            if (k >= nk_pad) break;
            float gm = 0.f, sd = 1.f, rsd = 1.f, k1 = 0.f;
            if (k < nk) {
                uint32_t rank = 0;
#pragma unroll
                for (int j = 0; j < ABEA_KMER_SIZE; ++j) rank = (rank << 2) | base_rank(base[u][j]);
                abea_model_t mm = a.model[rank];
                // gp_mean = scale*level_mean + shift; gp_stdv = level_stdv (scaling.var is
                // ignored by the reference, GPU/align_cuda.cl:509); cached log stdv.
                gm = __fadd_rn(__fmul_rn(r.scale, mm.level_mean), r.shift);
                sd = mm.level_stdv;
                float lsd = mm.level_log_stdv;
                if (a.g.var_aware) {
                    sd = __fmul_rn(sd, r.var);
                    lsd = __fadd_rn(lsd, r.log_var);
                }
                rsd = __frcp_rn(sd);
                k1 = __fsub_rn(kLogInvSqrt2Pi, lsd);
            }
            a.km_gm[r.km_off + k] = gm;
            a.km_sd[r.km_off + k] = sd;
            a.km_rsd[r.km_off + k] = rsd;
            a.km_k1[r.km_off + k] = k1;
        }
    }
    const int ne = r.n_events, ne_pad = round_up_dev(ne);
    const abea_event_t* ev = ev_in + r.ev_src;
    for (int e0 = t; e0 < ne_pad; e0 += kEvUnroll * nt) {
        float mean[kEvUnroll];
#pragma unroll
        for (int u = 0; u < kEvUnroll; ++u) mean[u] = ev[min(e0 + u * nt, ne - 1)].mean;  // ne >= 1
#pragma unroll
        for (int u = 0; u < kEvUnroll; ++u) {
            const int e = e0 + u * nt;
            if (e >= ne_pad) break;
            a.ev_mean[r.ev_off + e] = e < ne ? mean[u] : 0.f;
            a.last_col[r.ev_off + e] = -INFINITY;
        }
    }
}

__global__ void __launch_bounds__(128) abea_pre_kernel(PreArgs a) {
    const int i = blockIdx.x;
    if (i >= a.n_reads) return;
    pre_read(a, i, threadIdx.x, blockDim.x);
}

// ---------------------------------------------------------------- prefetch rings
// k-mer parameters live in a 128-entry ring indexed by k-mer & 127 (= the slot),
// event means in a 256-entry ring indexed by event & 255.  Chunks of 16 are
// copied with cp.async as soon as the entries they overwrite have left the band:
// a k-mer chunk [c, c+16) once c+15 <= k0+127, an event chunk once c+15 <= e0+156.
// 16-byte aligned: cp.async copies 16 bytes and the warp shape reads float4s.
struct alignas(16) Rings {
    float gm[kSlots];
    float sd[kSlots];
    float rsd[kSlots];
    float k1[kSlots];
    float ev[kEvRing];
};

struct RingState {
    int k_iss, e_iss, k_rdy, e_rdy, km_end, ev_end;
};

// `t` = index of the calling thread among the read's cooperating threads (>= 20).
__device__ __forceinline__ void issue_chunks(Rings& rg, const CoreArgs& a, const ReadDesc& r, int t, bool do_k,
                                             int kc, bool do_e, int ec) {
    if (do_k && t < 16) {
        const int arr = t >> 2, part = t & 3;
        const float* base = arr == 0 ? a.km_gm : arr == 1 ? a.km_sd : arr == 2 ? a.km_rsd : a.km_k1;
        float* dst = arr == 0 ? rg.gm : arr == 1 ? rg.sd : arr == 2 ? rg.rsd : rg.k1;
        cp_async16(dst + ((kc + 4 * part) & (kSlots - 1)), base + r.km_off + kc + 4 * part);
    }
    if (do_e && t >= 16 && t < 20) {
        const int part = t & 3;
        cp_async16(&rg.ev[(ec + 4 * part) & (kEvRing - 1)], a.ev_mean + r.ev_off + ec + 4 * part);
    }
}

// Initial fill for the band-1 window (k0 = -51, e0 = 50).  Caller syncs.
__device__ __forceinline__ void rings_init(Rings& rg, RingState& rs, const CoreArgs& a, const ReadDesc& r, int t,
                                           int k0, int e0) {
    rs.km_end = round_up_dev(r.n_kmers);
    rs.ev_end = round_up_dev(r.n_events);
    rs.k_iss = 0;
    rs.e_iss = 0;
    while (rs.k_iss < rs.km_end && rs.k_iss + 15 <= k0 + 127) {
        issue_chunks(rg, a, r, t, true, rs.k_iss, false, 0);
        rs.k_iss += kChunk;
    }
    while (rs.e_iss < rs.ev_end && rs.e_iss + 15 <= e0 + 156) {
        issue_chunks(rg, a, r, t, false, 0, true, rs.e_iss);
        rs.e_iss += kChunk;
    }
    cp_async_commit();
    cp_async_wait_all();
    rs.k_rdy = rs.k_iss;
    rs.e_rdy = rs.e_iss;
}

// Initial fill for a window (k0, e0) reached in the middle of a read (a resumed
// checkpoint): the chunks that hold the window's k-mers and events, from the
// 16-aligned chunk at or below k0 (events: e0 - 100), at most one ring's worth.
// Caller syncs.
__device__ __forceinline__ void rings_seek(Rings& rg, RingState& rs, const CoreArgs& a, const ReadDesc& r, int t,
                                           int k0, int e0) {
    rs.km_end = round_up_dev(r.n_kmers);
    rs.ev_end = round_up_dev(r.n_events);
    const int k_start = max(k0, 0) & ~(kChunk - 1), e_start = max(e0 - kBand, 0) & ~(kChunk - 1);
    rs.k_iss = k_start;
    rs.e_iss = e_start;
    while (rs.k_iss < rs.km_end && rs.k_iss + 15 <= k0 + 127 && rs.k_iss < k_start + kSlots) {
        issue_chunks(rg, a, r, t, true, rs.k_iss, false, 0);
        rs.k_iss += kChunk;
    }
    while (rs.e_iss < rs.ev_end && rs.e_iss + 15 <= e0 + 156 && rs.e_iss < e_start + kEvRing) {
        issue_chunks(rg, a, r, t, false, 0, true, rs.e_iss);
        rs.e_iss += kChunk;
    }
    cp_async_commit();
    cp_async_wait_all();
    rs.k_rdy = rs.k_iss;
    rs.e_rdy = rs.e_iss;
}

// Called once per group of bands with the current window: waits for the data the
// next `ahead` bands need and issues the chunks whose ring entries are free.
// Returns true when it waited (the caller then syncs the cooperating threads).
__device__ __forceinline__ bool rings_step(Rings& rg, RingState& rs, const CoreArgs& a, const ReadDesc& r, int t,
                                           int k0, int e0, int ahead) {
    bool waited = false;
    const int k_prev = rs.k_iss, e_prev = rs.e_iss;  // issued before this call
    const bool do_k = rs.k_iss < rs.km_end && rs.k_iss + 15 <= k0 + 127;
    const bool do_e = rs.e_iss < rs.ev_end && rs.e_iss + 15 <= e0 + 156;
    if (do_k || do_e) {
        issue_chunks(rg, a, r, t, do_k, rs.k_iss, do_e, rs.e_iss);
        cp_async_commit();
        if (do_k) rs.k_iss += kChunk;
        if (do_e) rs.e_iss += kChunk;
    }
    auto needs = [&](int k_have, int e_have) {
        return (k0 + kBand - 1 + ahead >= k_have && k_have < rs.km_end) || (e0 + ahead >= e_have && e_have < rs.ev_end);
    };
    if (needs(rs.k_rdy, rs.e_rdy)) {
        if ((do_k || do_e) && !needs(k_prev, e_prev)) {
            // the chunks just issued are not needed yet: wait for the older ones only
            cp_async_wait_group1();
            rs.k_rdy = k_prev;
            rs.e_rdy = e_prev;
        } else {
            cp_async_wait_all();
            rs.k_rdy = rs.k_iss;
            rs.e_rdy = rs.e_iss;
        }
        waited = true;
    }
    return waited;
}

// Computed offsets [lo, hi) of a band (GPU/align_cuda.cl:457-470).
__device__ __forceinline__ void band_range(int k0, int e0, int n_events, int n_kmers, int& lo, int& hi) {
    lo = max(max(-k0, e0 - (n_events - 1)), 0);
    hi = min(min(n_kmers - k0, e0 + 1), kBand);
}

// ---------------------------------------------------------------- warp shape
// Slot s of a band holds the cell of k-mer k(s) = k0 + ((s - k0) & 127) and event
// e = (band - 2) - k(s).  A slot inside band b+1 has kept its k-mer since band
// b-1, so its event is two more than under band b-1's placement: the emission of
// band b+1 and its exact diagonal candidate (diagonal = left neighbour of band b)
// are computed during band b, before band b's own placement is decided.  Band b
// itself then only needs its up candidate (from the slot's own previous score),
// the exchange of neighbour cells, the skip candidate and the comparison.

// 4x4 byte transpose: w[j] holds band j's backpointers of slots 0..3 (byte s);
// returns o[s] holding slot s's backpointers of bands 0..3 (byte j).
__device__ __forceinline__ uint4 transpose_bytes(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3) {
    const uint32_t a = __byte_perm(w0, w1, 0x5140), c = __byte_perm(w2, w3, 0x5140);
    const uint32_t b = __byte_perm(w0, w1, 0x7362), d = __byte_perm(w2, w3, 0x7362);
    return make_uint4(__byte_perm(a, c, 0x5410), __byte_perm(a, c, 0x7632), __byte_perm(b, d, 0x5410),
                      __byte_perm(b, d, 0x7632));
}

// The bands a fill_warp call computes and where its results go.
//   forward pass: bands [2, n_bands), band-side outputs (last column, band
//     origins, scores, slow-cell count) written, the trace into `trace` (kept
//     traces) or checkpoints into `ck_out` (checkpointed reads);
//   recompute: bands [b_begin, b_end) of a checkpointed read from the record
//     `ck_in` (nullptr: from the start), the trace into a scratch segment.
// Trace band b is stored at trace + trace_index(b - trace_band0, slot).
struct FillSpan {
    int b_begin, b_end;
    const float* ck_in;
    float* ck_out;
    uint8_t* trace;
    int trace_band0;
    int trace_tiles;  // 4-band tiles in the trace region (bounds checks)
    bool side;
};

// Debug builds (ABEA_BOUNDS_CHECK): the global stores of the fill and of the
// traceback check their index against their region; a store out of it is skipped
// and counted in counters[3] (the run then reports ABEA_ERR_INTERNAL).
#ifdef ABEA_BOUNDS_CHECK
__device__ __forceinline__ bool in_bounds(int64_t i, int64_t n, unsigned long long* counters) {
    const bool ok = i >= 0 && i < n;
    if (!ok) atomicAdd(&counters[3], 1ull);
    return ok;
}
#else
__device__ __forceinline__ bool in_bounds(int64_t, int64_t, unsigned long long*) { return true; }
#endif

__device__ __forceinline__ FillSpan forward_span(const CoreArgs& a, const ReadDesc& r) {
    FillSpan sp;
    sp.b_begin = 2;
    sp.b_end = r.n_bands;
    sp.ck_in = nullptr;
    sp.ck_out = r.ck ? a.ck + r.ck_off : nullptr;
    sp.trace = r.ck ? nullptr : a.trace + r.trace_off * kSlots;
    sp.trace_band0 = 0;
    sp.trace_tiles = r.ck ? 0 : (r.n_bands + 3) / 4;
    sp.side = true;
    return sp;
}

// kSpan = false: the forward pass of a read that keeps its trace, with none of
// the span's choices left to run time (the common case); kSpan = true: any span.
template <bool kScores, bool kSpan>
__device__ void fill_warp(const CoreArgs& a, const ReadDesc& r, Rings& rg, int lane, const FillSpan& spr) {
    FillSpan sp = spr;
    if (!kSpan) {
        sp.b_begin = 2;
        sp.b_end = r.n_bands;
        sp.ck_in = nullptr;
        sp.ck_out = nullptr;
        sp.trace = a.trace + r.trace_off * kSlots;
        sp.trace_band0 = 0;
        sp.trace_tiles = (r.n_bands + 3) / 4;
        sp.side = true;
    }
    const CellConsts cc = make_consts(r, a.g);
    const int n_events = r.n_events, n_kmers = r.n_kmers, n_bands = sp.b_end;
    uint8_t* trace = sp.trace;
    float* scores = kScores && sp.side ? a.scores + r.band_off * kSlots : nullptr;
    int32_t* bk0 = a.band_k0 + r.band_off;
    float* lastc = a.last_col + r.ev_off;

    // band 0: start cell (e=-1,k=-1) = 0 in slot 127; band 1: trim cell (e=0,k=-1)
    // = (float)lp_trim, FROM_U, slot 127 (GPU/align_cuda.cl:249-268).  A resumed
    // checkpoint gives band b_begin-1's scores and placement and band
    // b_begin-2's scores shifted by one slot.
    int k0 = -1 - kBand / 2, e0 = kBand / 2;  // band 1 (band 0 is (49,-51), band 1 moved down)
    float S1[4], LP[4];
    if (kSpan && sp.ck_in) {
        const float4 s4 = reinterpret_cast<const float4*>(sp.ck_in)[lane];
        const float4 l4 = reinterpret_cast<const float4*>(sp.ck_in + kSlots)[lane];
        S1[0] = s4.x; S1[1] = s4.y; S1[2] = s4.z; S1[3] = s4.w;
        LP[0] = l4.x; LP[1] = l4.y; LP[2] = l4.z; LP[3] = l4.w;
        k0 = __float_as_int(sp.ck_in[2 * kSlots]);
        e0 = __float_as_int(sp.ck_in[2 * kSlots + 1]);
    }
    RingState rs;
    if (kSpan && sp.ck_in)
        rings_seek(rg, rs, a, r, lane, k0, e0);
    else
        rings_init(rg, rs, a, r, lane, k0, e0);
    __syncwarp();

    int ep[4];  // event of each slot under the previous band's placement
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (!sp.ck_in) S1[j] = LP[j] = -INFINITY;
        ep[j] = e0 - ((4 * lane + j - k0) & 127);
    }
    if (!sp.ck_in) {
        if (lane == 31) S1[3] = a.g.trim_f;
        if (lane == 0) LP[0] = 0.0f;  // band 0 shifted by one slot = diagonal source of band 2
    }
    if (kScores && scores) {
        float4 b0 = make_float4(-INFINITY, -INFINITY, -INFINITY, lane == 31 ? 0.0f : -INFINITY);
        float4 b1 = make_float4(-INFINITY, -INFINITY, -INFINITY, lane == 31 ? a.g.trim_f : -INFINITY);
        reinterpret_cast<float4*>(scores)[lane] = b0;
        reinterpret_cast<float4*>(scores + kSlots)[lane] = b1;
    }
    NextCell nc[4];  // band b's emission side, prepared during band b-1
    {
        const float4 gm4 = *reinterpret_cast<const float4*>(&rg.gm[4 * lane]);
        const float4 sd4 = *reinterpret_cast<const float4*>(&rg.sd[4 * lane]);
        const float4 rs4 = *reinterpret_cast<const float4*>(&rg.rsd[4 * lane]);
        const float4 k14 = *reinterpret_cast<const float4*>(&rg.k1[4 * lane]);
        const float gmv[4] = {gm4.x, gm4.y, gm4.z, gm4.w}, sdv[4] = {sd4.x, sd4.y, sd4.z, sd4.w};
        const float rsv[4] = {rs4.x, rs4.y, rs4.z, rs4.w}, k1v[4] = {k14.x, k14.y, k14.z, k14.w};
#pragma unroll
        for (int j = 0; j < 4; ++j)
            nc[j] = next_cell(LP[j], rg.ev[(ep[j] + 1) & (kEvRing - 1)], gmv[j], sdv[j], rsv[j], k1v[j], cc);
    }
    int my_k0 = k0;  // bands 0 and 1 (lanes 0, 1) both have k0 = -51
    unsigned long long slow = 0;
    const int sl_last = (n_kmers - 1) & 127;
    uint32_t tw0 = 0u, tw1 = (lane == 31 && !sp.ck_in) ? (ABEA_FROM_U << 24) : 0u, tw2 = 0u, tw3 = 0u;

    // Band state kept across the exit to the slow path: a band in which a proof
    // failed in any lane leaves the inner loop (warp-uniform) and is finished
    // below with the reference's FP64 arithmetic, so that the inner loop holds
    // no division routine and no FP64 code.
    int b = sp.b_begin, lo = 0, hi = 0;
    float best[4], left[4];
    uint32_t from[4];
    bool valid[4], bad[4];
    NextCell nn[4];
    auto finish = [&]() {
        uint32_t word = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            best[j] = valid[j] ? best[j] : -INFINITY;
            word |= (valid[j] ? from[j] : 0u) << (8 * j);
        }
        // edges of the read: trim cell (k = -1, slot 127; GPU/align_cuda.cl:431-443)
        // and the last k-mer column read by the post stage (GPU/align_cuda.cl:722-746)
        const int ol = n_kmers - 1 - k0;
        if (k0 <= -1 || ol < kBand) {
            if (k0 <= -1) {  // uniform
                const int e_t = e0 + 1 + k0;
                const bool in = e_t >= 0 && e_t < n_events;
                const float tv = in ? __double2float_rn(__dmul_rn(a.g.lp_trim, (double)(e_t + 1))) : -INFINITY;
                const bool here = lane == 31 && k0 >= -kBand;
                best[3] = here ? tv : best[3];
                word = here ? ((word & 0x00ffffffu) | (in ? (ABEA_FROM_U << 24) : 0u)) : word;
            }
            if (sp.side && ol >= lo && ol < hi && lane == (sl_last >> 2) && in_bounds(e0 - ol, n_events, a.counters))
                lastc[e0 - ol] = sel4(best, sl_last & 3);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            LP[j] = left[j];
            S1[j] = best[j];
            nc[j] = nn[j];
        }
        const int jb = b & 3;
        tw0 = jb == 0 ? word : tw0;
        tw1 = jb == 1 ? word : tw1;
        tw2 = jb == 2 ? word : tw2;
        tw3 = jb == 3 ? word : tw3;
        if (jb == 3 || b == n_bands - 1) {
            if ((!kSpan || trace) && in_bounds((b - sp.trace_band0) >> 2, sp.trace_tiles, a.counters))
                reinterpret_cast<uint4*>(trace + (int64_t)((b - sp.trace_band0) >> 2) * 512)[lane] =
                    transpose_bytes(tw0, tw1, tw2, tw3);
            tw0 = tw1 = tw2 = tw3 = 0u;
        }
        if (kScores && scores && in_bounds(b, r.n_bands, a.counters))
            reinterpret_cast<float4*>(scores + (int64_t)b * kSlots)[lane] = make_float4(best[0], best[1], best[2], best[3]);
        my_k0 = ((b & 31) == lane) ? k0 : my_k0;
        if (sp.side && ((b & 31) == 31 || b == n_bands - 1)) {
            if (lane <= (b & 31) && in_bounds((b & ~31) + lane, r.n_bands, a.counters)) bk0[(b & ~31) + lane] = my_k0;
        }
    };
    while (true) {
        bool to_slow = false;
        for (; b < n_bands; ++b) {
            if (kSpan && sp.ck_out && (b & (kCkBands - 1)) == 0 &&
                in_bounds(b / kCkBands, r.n_bands / kCkBands + 1, a.counters)) {
                // checkpoint s = b / kCkBands: the state this loop resumes from at band b
                float* rec = sp.ck_out + (int64_t)(b / kCkBands) * kCkStride;
                reinterpret_cast<float4*>(rec)[lane] = make_float4(S1[0], S1[1], S1[2], S1[3]);
                reinterpret_cast<float4*>(rec + kSlots)[lane] = make_float4(LP[0], LP[1], LP[2], LP[3]);
                if (lane == 0) {
                    rec[2 * kSlots] = __int_as_float(k0);
                    rec[2 * kSlots + 1] = __int_as_float(e0);
                }
            }
            if ((b & 3) == 0) {
                if (rings_step(rg, rs, a, r, lane, k0, e0, 6)) __syncwarp();
            }
            // ---- exchange: end cells for the placement, left neighbour of slot 4*lane
            const int sl = k0 & 127, su = (k0 + kBand - 1) & 127;
            const float ll = __shfl_sync(kFull, sel4(S1, sl & 3), sl >> 2);
            const float ur = __shfl_sync(kFull, sel4(S1, su & 3), su >> 2);
            const float left0 = __shfl_sync(kFull, S1[3], (lane + 31) & 31);
            left[0] = left0;
            left[1] = S1[0];
            left[2] = S1[1];
            left[3] = S1[2];
            // ---- up candidates of band b
            float u[4];
            bool oku[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) u[j] = cell_u(S1[j], nc[j], cc, oku[j]);
            // ---- band b+1's emission side (placement-independent)
            const float4 gm4 = *reinterpret_cast<const float4*>(&rg.gm[4 * lane]);
            const float4 sd4 = *reinterpret_cast<const float4*>(&rg.sd[4 * lane]);
            const float4 rs4 = *reinterpret_cast<const float4*>(&rg.rsd[4 * lane]);
            const float4 k14 = *reinterpret_cast<const float4*>(&rg.k1[4 * lane]);
            const float gmv[4] = {gm4.x, gm4.y, gm4.z, gm4.w}, sdv[4] = {sd4.x, sd4.y, sd4.z, sd4.w};
            const float rsv[4] = {rs4.x, rs4.y, rs4.z, rs4.w}, k1v[4] = {k14.x, k14.y, k14.z, k14.w};
#pragma unroll
            for (int j = 0; j < 4; ++j)
                nn[j] = next_cell(left[j], rg.ev[(ep[j] + 2) & (kEvRing - 1)], gmv[j], sdv[j], rsv[j], k1v[j], cc);
            // ---- band placement (Suzuki-Kasahara), GPU/align_cuda.cl:394-430
            const bool right = (ll == -INFINITY && ur == -INFINITY) ? (bool)(b & 1) : (ll < ur);
            k0 += right ? 1 : 0;
            e0 += right ? 0 : 1;
            band_range(k0, e0, n_events, n_kmers, lo, hi);
            // ---- skip candidate (exact), comparison
            bool rare = false;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int o = (4 * lane + j - k0) & 127;
                ep[j] = e0 - o;
                valid[j] = (o >= lo) && (o < hi);
                uint32_t from_du;
                const float best_du = pick_du(nc[j].d, u[j], from_du);
                bool okl;
                const float l = exact_skip(left[j], cc.skip_h, cc.skip_l, okl);
                best[j] = pick_l(best_du, from_du, l, from[j]);
                bad[j] = valid[j] && !(nc[j].ok && oku[j] && okl);
                rare |= bad[j];
            }
            if (__any_sync(kFull, rare)) {
                to_slow = true;
                break;
            }
            finish();
        }
        if (!to_slow) break;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (bad[j]) {  // a proof failed: the reference's FP64 arithmetic
                const int sj = 4 * lane + j;
                best[j] = cell_slow(LP[j], S1[j], left[j], rg.ev[ep[j] & (kEvRing - 1)], rg.gm[sj], rg.sd[sj],
                                    rg.k1[sj], cc, from[j]);
                ++slow;
            }
        }
        finish();
        ++b;
    }
    cp_async_wait_all();  // no copy may land in shared memory after the read is done
    __syncwarp();
    if (slow && sp.side) atomicAdd(&a.counters[0], slow);
}

// ---------------------------------------------------------------- wide shape
// Twelve warps per read (the block's other warps wait at its next barrier):
//   B (warps 0-3)   the band-to-band chain, one k-mer slot per thread.  Per band:
//                   the end cells and the left neighbour of band b-1 from shared
//                   memory, the placement, the in-band test, the exact up and
//                   diagonal candidates (both from registers), the exact skip
//                   candidate, the comparison, and the
//                   bookkeeping (backpointers packed four bands to a word and
//                   stored once per tile, band origins packed one per lane,
//                   last k-mer column).  One 128-thread named barrier per band.
//   E (warps 4-11)  the emissions and their exact splits, kWideChunk bands at a
//                   time for the thread's slot (a slot keeps its k-mer while its
//                   event advances by one per band: one load of its pore-model
//                   parameters per chunk), up to kWideRing chunks ahead of B, into a
//                   ring in shared memory; warps 4-7 take the even chunks, warps
//                   8-11 the odd ones.
// A band's cells lie on one anti-diagonal, so the placement of any band p with
// bn - p <= 28 gives a window [k0(p), k0(p) + 128) that holds band bn's k-mers
// (each band moves k0 by at most one): E computes a chunk from the placement B
// published when it released the ring slot, kWideChunk * kWideRing + 1 = 17
// bands before the chunk's last band.  B and E hand the ring slots over with
// named barriers, FULL[s] (E arrives, B waits) and EMPTY[s] (B arrives, E waits);
// every use of a barrier completes before its next, so arrivals never pile up.
//
// The medium shape is the same chain and producer with one E group (warps 4-7)
// and a ring of kMidRing chunks: eight warps per read, two reads per block (warps
// 0-7 and 8-15), each half on its own named barriers.
constexpr int kWideThreads = 512;   // block size of the batched kernel
constexpr int kWideChunk = 4;       // bands per emission chunk
constexpr int kWideRing = 4;        // chunks in the wide shape's ring (kWideChunk * ring + 1 <= 28)
constexpr int kMidRing = 2;         // chunks in the medium shape's ring
constexpr int kMidThreads = 256;    // threads per medium read
// Named barriers of one read (IDs from a base): base = B's per-band barrier,
// base + 1 + s = FULL[s], base + 1 + ring + s = EMPTY[s]; the medium shape adds
// base + 1 + 2 * ring, the half-block barrier between its reads.
constexpr int kMidBars = 2 + 2 * kMidRing;
static_assert(kWideChunk * kWideRing + 1 <= 28, "E's k-mer window must hold the chunk's bands");
static_assert(kWideRing % 2 == 0, "each ring slot, and its two barriers, belongs to one of the two E groups");
static_assert(1 + 1 + 2 * kWideRing <= 16 && 1 + 2 * kMidBars <= 16, "named barriers 0-15");

template <int kRing>
struct alignas(16) ChainSmem {
    // band kWideChunk*j + 2 + q of chunk j in slot j % kRing, entry [q]:
    // {p_step, p_stay, w_step, w_stay} and {|em| + |step_h|, |em| + |stay_h|} (NaN
    // when the emission's division was not proven)
    float4 ems[kRing][kWideChunk][kSlots];
    float2 emm[kRing][kWideChunk][kSlots];
    float sc[2][kSlots];                  // band scores, buffer b & 1
    float trim[kRing][kWideChunk];        // the trim cell's value of each band (-inf: past the read's events)
    int32_t k0h[64];                      // placement of band b at [b & 63] (b a multiple of 4), for E
};
using WideSmem = ChainSmem<kWideRing>;
using MidSmem = ChainSmem<kMidRing>;

__device__ __forceinline__ void named_bar_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void named_bar_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;\n" ::"r"(id), "r"(n) : "memory");
}
// bar.sync that also returns whether p held in any of the n threads
__device__ __forceinline__ bool named_bar_any(int id, int n, bool p) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.or.pred po, %2, %3, pi;\n selp.u32 %0, 1, 0, po;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)p), "r"(id), "r"(n)
        : "memory");
    return r != 0u;
}

__device__ __forceinline__ bool band_moves_right(float ll, float ur, int b) {
    // Suzuki-Kasahara (GPU/align_cuda.cl:394-430); both ends -inf: alternate
    return (ll == -INFINITY && ur == -INFINITY) ? (bool)(b & 1) : (ll < ur);
}

// E: chunk j's emissions for slot t, from the placement kp of an earlier band.
template <int kRing>
__device__ __forceinline__ void wide_chunk(ChainSmem<kRing>& ws, const CoreArgs& a, const ReadDesc& r,
                                           const CellConsts& cc, int t, int j, int kp) {
    const int s = j % kRing, bb = 2 + kWideChunk * j;
    const int kk = kp + ((t - kp) & (kSlots - 1));  // slot t's k-mer in the window
    const bool kin = kk >= 0 && kk < r.n_kmers;
    const int64_t ko = r.km_off + (kin ? kk : 0);
    const float gm = a.km_gm[ko], sd = a.km_sd[ko], rsd = a.km_rsd[ko], k1 = a.km_k1[ko];
    const float* ev = a.ev_mean + r.ev_off;
    const int e_first = bb - 2 - kk;
    float x[kWideChunk];
#pragma unroll
    for (int q = 0; q < kWideChunk; ++q) {
        // cells outside the read get a finite stand-in; B's in-band test keeps them out
        const int e = e_first + q;
        x[q] = (kin && e >= 0 && e < r.n_events) ? ev[e] : gm;
    }
#pragma unroll
    for (int q = 0; q < kWideChunk; ++q) {
        bool ok;
        const float em = emission_fast(x[q], gm, sd, rsd, k1, ok);
        const EmSplit s1 = em_split(em, cc.step_h, cc.step_l);
        const EmSplit s2 = em_split(em, cc.stay_h, cc.stay_l);
        const float nan = __int_as_float(0x7fc00000);
        ws.ems[s][q][t] = make_float4(s1.p, s2.p, s1.w, s2.w);
        ws.emm[s][q][t] = ok ? make_float2(__fadd_rn(fabsf(em), fabsf(cc.step_h)), __fadd_rn(fabsf(em), fabsf(cc.stay_h)))
                             : make_float2(nan, nan);
    }
    if (t < kWideChunk) {
        // the trim cell (k = -1) of band bb + t: event bb + t - 1, (float)(lp_trim * (e + 1))
        // (GPU/align_cuda.cl:431-443); B uses it while the band reaches below k-mer 0
        const int e_t = bb + t - 1;
        ws.trim[s][t] = e_t < r.n_events ? __double2float_rn(__dmul_rn(a.g.lp_trim, (double)(e_t + 1))) : -INFINITY;
    }
}

// The reference's arithmetic for one cell whose exactness proof failed, as a
// call: its division routine and FP64 code stay out of the band loop's body.
struct SlowCell {
    float best;
    uint32_t from;
};
__device__ __noinline__ SlowCell slow_cell_call(float diag, float up, float left, float x, float gm, float sd, float k1,
                                                double lp_step, double lp_stay, double lp_skip) {
    CellConsts c{};
    c.lp_step = lp_step;
    c.lp_stay = lp_stay;
    c.lp_skip = lp_skip;
    SlowCell o;
    o.best = cell_slow(diag, up, left, x, gm, sd, k1, c, o.from);
    return o;
}

// One read's fill by warps 0 .. 4 + 4 * kGroups - 1 of the calling threads
// (tid = index among them; others return at once): B = warps 0-3, E = the
// kGroups groups of four warps after them, group g taking chunks g, g + kGroups,
// ...  bar0 = the read's first named barrier.  The wide shape is kGroups = 2 with
// kWideRing chunks, the medium shape kGroups = 1 with kMidRing.
template <bool kScores, int kGroups, int kRing>
__device__ void fill_chain(const CoreArgs& a, const ReadDesc& r, ChainSmem<kRing>& ws, int tid, int bar0) {
    static_assert(kGroups == 1 || kRing % kGroups == 0, "each ring slot belongs to one E group");
    const int warp = tid >> 5;
    if (warp >= 4 + 4 * kGroups) return;
    const CellConsts cc = make_consts(r, a.g);
    const int n_events = r.n_events, n_kmers = r.n_kmers, n_bands = r.n_bands;
    const int n_chunks = (n_bands - 2 + kWideChunk - 1) / kWideChunk;
    const int t = tid & (kSlots - 1);
    constexpr int kPair = 2 * kSlots;  // B and E threads on FULL / EMPTY
    const int kBarChain = bar0, kBarFull = bar0 + 1, kBarEmpty = bar0 + 1 + kRing;

    if (warp >= 4) {
        // ------------------------------------------------ E: the emission chunks; with
        // two groups each has two chunks of B's time for the loads and arithmetic of one
        for (int j = (warp >> 2) - 1; j < n_chunks; j += kGroups) {
            const int s = j % kRing;
            int kp = -1 - kBand / 2;  // band 1's placement, for the first kRing chunks
            if (j >= kRing) {
                named_bar_sync(kBarEmpty + s, kPair);  // B released chunk j - kRing
                kp = ws.k0h[(kWideChunk * (j - kRing) + kWideChunk) & 63];  // band bb(j - R) + C - 2
            }
            wide_chunk(ws, a, r, cc, t, j, kp);
            named_bar_arrive(kBarFull + s, kPair);
        }
        return;
    }

    // ------------------------------------------------ B: the chain
    // One iteration per chunk, its kWideChunk bands unrolled: the chunk's barriers
    // and the backpointer tile stores fall on fixed bands.  Band b-1's bookkeeping
    // (backpointers, band origin, last k-mer column, scores) runs just after band
    // b's barrier, beside the loads, so that nothing but the chain stands between
    // a band's comparison and the next barrier.
    const int lane = tid & 31;
    uint8_t* trace = a.trace + r.trace_off * kSlots;
    int32_t* bk0 = a.band_k0 + r.band_off;
    float* lastc = a.last_col + r.ev_off;
    float* scores = kScores ? a.scores + r.band_off * kSlots : nullptr;
    const int sl_last = (n_kmers - 1) & (kSlots - 1);

    // band b's placement: lower-left k-mer k0, event e0 = b - 2 - k0 (a band's cells
    // lie on one anti-diagonal), so only k0 is carried
    int k0 = -1 - kBand / 2;                         // band 1 (band 0 is (49,-51), band 1 moved down)
    float s1 = (t == 127) ? a.g.trim_f : -INFINITY;  // band b-1's score of this slot
    float lp = (t == 0) ? 0.0f : -INFINITY;          // band b-2's score of slot t-1: band b's diagonal
    ws.sc[1][t] = s1;
    if (kScores) {
        scores[t] = (t == 127) ? 0.0f : -INFINITY;
        scores[kSlots + t] = s1;
    }
    int my_k0 = k0;                                      // band origins: band b in lane b & 31 (bands 0, 1: -51)
    uint32_t tw = 0u;                                    // backpointers of bands 4m..4m+3, byte b & 3
    uint32_t from_p = (t == 127) ? ABEA_FROM_U : 0u;     // band b-1's backpointer (band 1: the trim cell)
    unsigned long long slow = 0;
    // Band bk's bookkeeping; q1 = bk & 3 when known at compile time, else -1.  No
    // branches: a branch in the unrolled band body splits the code the compiler
    // schedules as one block (measured: a band-uniform branch around the
    // last-column store cost 27 cycles per band).  The placement of every fourth
    // band (the one E reads) goes to the ring k0h; band origins are kept one per
    // lane of warp 0 and stored 32 bands at a time.
    auto book = [&](int bk, int q1, bool last_col, bool mine) {
        if (q1 >= 0) {  // the byte's place known when compiled: one byte insert
            constexpr unsigned kSel[4] = {0x3214u, 0x3240u, 0x3410u, 0x4210u};
            tw = __byte_perm(tw, from_p, kSel[q1 & 3]);
        } else {
            tw |= from_p << (8 * (bk & 3));
        }
        // band bk's placement is still k0: the band after it moves k0 after this
        my_k0 = mine ? k0 : my_k0;
        if (t == 0 && (bk & 3) == 0) ws.k0h[bk & 63] = k0;
        if (last_col) {
            const int ol = n_kmers - 1 - k0, e0p = bk - 2 - k0;
            int lop, hip;  // band bk's computed offsets
            band_range(k0, e0p, n_events, n_kmers, lop, hip);
            if (t == sl_last && ol >= lop && ol < hip && in_bounds(e0p - ol, n_events, a.counters))
                lastc[e0p - ol] = s1;
        }
        if (kScores && in_bounds(bk, n_bands, a.counters)) scores[(int64_t)bk * kSlots + t] = s1;
    };
    auto store_tile = [&](int bk) {
        if (in_bounds(bk >> 2, (n_bands + 3) / 4, a.counters))
            reinterpret_cast<uint32_t*>(trace + (int64_t)(bk >> 2) * 512)[t] = tw;
        tw = 0u;
    };
    auto store_origins = [&](int bk, bool now) {  // bands (bk & ~31) .. bk, when `now`
        const int band = (bk & ~31) + lane;
        if (now && warp == 0 && lane <= (bk & 31) && in_bounds(band, n_bands, a.counters)) bk0[band] = my_k0;
    };
    // One chunk of kWideChunk bands; kLast: the read may end inside it (the only
    // chunk that tests for the end: a test per band is a branch in the band body).
    // kMid: a chunk inside the read, where every band's computed cells are all 100
    // (offsets [0, 100)), none is the trim cell and none lies on the last k-mer
    // column (and neither does band bb-1, whose bookkeeping the chunk finishes): k0
    // and e0 each move by at most one per band, so the placement of band bb-1
    // decides it for the whole chunk.
    // kOpt: optimistic (middle chunks only): no per-band check of the exactness
    // proofs; each thread ORs its failed proofs into `dirty`, the barrier that ends
    // the chunk reduces them (open_chunk), and a chunk with any is done again with
    // the checks (kRedo: its emissions are still in the ring, whose slot is
    // released only after that barrier).  The chunk's first chain barrier is the
    // caller's (open_chunk), except in a redo.
    bool dirty = false;
    auto chunk = [&](int j, auto last, auto mid, auto opt, auto redo) {
        constexpr bool kLast = decltype(last)::value, kMid = decltype(mid)::value;
        constexpr bool kOpt = decltype(opt)::value, kRedo = decltype(redo)::value;
        static_assert(!kOpt || kMid, "only middle chunks run optimistic");
        const int s = j % kRing, bb = 2 + kWideChunk * j;
        const int dl = (lane - 1 - kWideChunk * j) & 31;  // band bb-1+q's origin goes to lane (bb-1+q) & 31: dl == q
#pragma unroll
        for (int q = 0; q < kWideChunk; ++q) {
            const int b = bb + q;
            if (kLast && b >= n_bands) break;
            if (q > 0 || kRedo) named_bar_sync(kBarChain, kSlots);  // band b-1's scores are in shared memory
            if (q == 0 && !kRedo) named_bar_sync(kBarFull + s, kPair);  // chunk j's emissions are in the ring
            const int pb = (b - 1) & 1;
            const float ll = ws.sc[pb][k0 & 127];
            const float ur = ws.sc[pb][(k0 + kBand - 1) & 127];
            const float left = ws.sc[pb][(t + 127) & 127];
            const float4 ep = ws.ems[s][q][t];
            const float2 mm = ws.emm[s][q][t];
            const float tv = ws.trim[s][q];
            // band b-1's bookkeeping (bands 2 + 4j + q - 1: b-1 & 3 == (q + 1) & 3)
            book(b - 1, (q + 1) & 3, !kMid, dl == q);
            if (q == 2) {  // band b-1 closes a tile of four bands, every eighth one 32 bands
                store_tile(b - 1);
                store_origins(b - 1, ((b - 1) & 31) == 31);
            }
            // the exact diagonal and up candidates of band b
            bool okd, oku;
            const float d = exact_from_split(lp, EmSplit{ep.x, ep.z}, mm.x, okd);
            const float u = exact_from_split(s1, EmSplit{ep.y, ep.w}, mm.y, oku);
            const bool right = band_moves_right(ll, ur, b);
            k0 += right ? 1 : 0;
            const int e0 = b - 2 - k0;
            int lo = 0, hi = kBand;
            if (!kMid) band_range(k0, e0, n_events, n_kmers, lo, hi);
            const int o = (t - k0) & 127;
            const bool valid = kMid ? o < kBand : (o >= lo && o < hi);
            // d vs u (U wins ties), then the skip candidate (L wins ties)
            uint32_t from_du, from;
            const float best_du = pick_du(d, u, from_du);
            bool okl;
            const float l = exact_skip(left, cc.skip_h, cc.skip_l, okl);
            float best = pick_l(best_du, from_du, l, from);
            const bool proven = okd && oku && okl;
            const bool bad = valid && !proven;
            best = valid ? best : -INFINITY;
            if (!kMid) from = valid ? from : 0u;  // a middle chunk's invalid slots are outside the band
            const bool here = !kMid && (t == 127) && (k0 <= -1) && (k0 >= -kBand);
            best = here ? tv : best;
            from = here ? (tv == -INFINITY ? 0u : ABEA_FROM_U) : from;
            ws.sc[b & 1][t] = best;  // stored before the check: only the rare path stores again
            if (kOpt) {
                // out-of-band cells count too: one test fewer per band, a redo
                // seldom more (measured 1.6% faster)
                dirty = dirty || !proven;
            } else if (__any_sync(kFull, bad)) {
                // Rare: a proof failed in some lane, whose cell takes the reference's
                // FP64 arithmetic and stores its score again.  The whole warp calls (a
                // divergent branch around the call cost 20 cycles per band); the other
                // lanes pass k-mer 0 and event 0 of the read, which exist because the
                // bad lane's cell does, and drop the result.
                const int64_t ko = r.km_off + (bad ? k0 + o : 0);
                const SlowCell c = slow_cell_call(lp, s1, left, a.ev_mean[r.ev_off + (bad ? e0 - o : 0)], a.km_gm[ko],
                                                  a.km_sd[ko], a.km_k1[ko], cc.lp_step, cc.lp_stay, cc.lp_skip);
                const bool use = bad && !here;
                best = use ? c.best : best;
                from = use ? c.from : from;
                slow += use ? 1 : 0;
                ws.sc[b & 1][t] = best;
            }
            if (!kOpt && !kRedo && q == kWideChunk - 1 && j + kRing < n_chunks)
                named_bar_arrive(kBarEmpty + s, kPair);  // chunk j read: E may refill its slot
            lp = left;
            s1 = best;
            from_p = from;
        }
    };
    // The state an optimistic chunk starts from (band bb-1's placement, score,
    // backpointer and the diagonal of band bb, the backpointer word, the band
    // origins: its last band may have started the next 32), for its redo.
    int sv_k0 = 0, sv_myk0 = 0, pj = -1;
    float sv_s1 = 0.f, sv_lp = 0.f;
    uint32_t sv_from = 0u, sv_tw = 0u;
    using F = std::false_type;
    using T = std::true_type;
    // The barrier that ends band bb-1 before chunk j (bb = 2 + 4j), or before the
    // last band's bookkeeping (j = n_chunks).  After an optimistic chunk it also
    // reduces that chunk's failed proofs; with any, the chunk is done again from
    // its saved state, with the checks.  Then the chunk's ring slot is released.
    auto open_chunk = [&](int j) {
        if (pj < 0) {
            named_bar_sync(kBarChain, kSlots);
            return;
        }
        if (named_bar_any(kBarChain, kSlots, dirty)) {
            k0 = sv_k0;
            s1 = sv_s1;
            lp = sv_lp;
            from_p = sv_from;
            tw = sv_tw;
            my_k0 = sv_myk0;
            ws.sc[(1 + kWideChunk * pj) & 1][t] = s1;  // band bb-1's scores, which the chunk overwrote
            chunk(pj, F{}, T{}, F{}, T{});              // its first barrier publishes them
            named_bar_sync(kBarChain, kSlots);
        }
        if (pj + kRing < n_chunks) named_bar_arrive(kBarEmpty + pj % kRing, kPair);  // E may refill the slot
        pj = -1;
        dirty = false;
        (void)j;
    };
    const int n_full = (n_bands - 2) / kWideChunk;
    for (int j = 0; j < n_full; ++j) {
        open_chunk(j);
        const int e0 = kWideChunk * j - 1 - k0;  // band bb-1's event (bb = 2 + 4j)
        if (k0 >= 0 && k0 + kWideChunk <= n_kmers - 1 - kBand && e0 >= kBand - 1 && e0 + kWideChunk <= n_events - 1) {
            sv_k0 = k0;
            sv_s1 = s1;
            sv_lp = lp;
            sv_from = from_p;
            sv_tw = tw;
            sv_myk0 = my_k0;
            pj = j;
            chunk(j, F{}, T{}, T{}, F{});
        } else {
            chunk(j, F{}, F{}, F{}, F{});
        }
    }
    if (n_full < n_chunks) {
        open_chunk(n_full);
        chunk(n_full, T{}, F{}, F{}, F{});
    } else if (n_bands > 2) {
        open_chunk(n_chunks);  // the last chunk may have been optimistic
    }
    if (n_bands > 2) {  // the last band's bookkeeping and the stores it closes
        const int bl = n_bands - 1;
        book(bl, -1, true, (bl & 31) == lane);
        store_tile(bl);
        store_origins(bl, true);
    }
    if (slow) atomicAdd(&a.counters[0], slow);
}

// ---------------------------------------------------------------- wide shape on a cluster pair
// The wide fill with its emission work on a second SM: blocks run in clusters
// of two.  The cluster's first block holds the read's band state and runs three
// groups of 128 threads (B: the band-to-band chain, D: diagonal candidates and
// inside flags, K: bookkeeping and the prefetch rings of the FP64 slow path).
// The second block's four groups compute the emissions and their exact splits,
// group g the bands 2+g, 6+g, ..., stage them in their own shared memory and
// bulk-copy them into the first block's (distributed shared memory) up to
// kClRing bands ahead of the chain; one mbarrier per ring slot counts a band's
// bytes.  D waits on it before it prepares the band's diagonal candidates, and
// the block barrier that follows hands the band to B.
// A band's cells lie on one anti-diagonal (event + k-mer = band - 2), so the
// emissions of band bn only need a k-mer window that holds the band: the
// placement k0 of any earlier band p with bn - p <= 28 gives one, [k0, k0+128),
// because each band moves k0 by at most one.  The first block publishes its
// progress, with the placement of the band it names, into the second block's
// shared memory every kClPublish bands (each release is a cluster-scope fence:
// once per band they cost ~400 cycles per band).  E reads its inputs straight
// from the pre stage's arrays (L2), one band ahead.  Every wait is bounded by
// spin_limit polls; a wait that runs out counts in counters[2] and goes on (the
// batch then reports a timeout).  Measured: 1,030 cycles per band against 600
// for the single-block wide shape, so the option is off by default.
constexpr int kClRing = 16;    // bands of emissions in flight (<= 28: the k-mer window above)
constexpr int kClPublish = 8;  // block 0 publishes its progress every kClPublish bands (< kClRing)

struct alignas(16) ClSmem {
    Rings rg;                                   // block 0: rings of the FP64 slow path
    float sc[2][kSlots];
    // written by block 1, per band slot and k-mer slot: {pstay, wstay, magu, em} and {pstep, wstep}
    float4 emu[kClRing][kSlots];
    float2 emd[kClRing][kSlots];
    float dc[2][kSlots];
    int32_t flags[2][kSlots];
    float trim[2];
    uint32_t fr[8][kSlots];
    int32_t k0h[8];
};

// Cluster state that outlives the fill (the fill's shared memory is reused
// afterwards; the mbarriers and the partner's stores must not land there).
struct ClShared {
    uint64_t full[kClRing];  // block 0: band b's emissions in slot (b-2) % kClRing have landed
                             // (phase (b-2) / kClRing of that slot's mbarrier)
    int32_t k0ring[64];      // block 1: placement of band b at [b & 63], from block 0
    int32_t progress;        // block 1: block 0 is done with the emissions of bands <= progress
    int32_t pick;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Waits for the phase of parity `parity` of a local mbarrier, at most limit/64
// polls (each poll may itself suspend the thread for a while); false when they
// ran out.  CTA-scope acquire: the data that completes the phase (bulk copies
// counted by complete_tx) is visible to the waiting thread once it observes the
// completion, whichever block issued the copies.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, long long limit) {
    const unsigned a = smem_u32(bar);
    const long long polls = limit > 0 ? (limit >> 6) + 1 : 0;
    for (long long i = 0; i < polls; ++i) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Remote shared-memory address of `p`'s counterpart in block `rank`.
__device__ __forceinline__ unsigned mapa_u32(const void* p, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from
// this block's shared memory to another block's (remote address `rdst`),
// counted on that block's mbarrier `rbar` (complete_tx).
__device__ __forceinline__ void bulk_to_remote(unsigned rdst, const void* src, unsigned bytes, unsigned rbar) {
    asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     rdst),
                 "r"(smem_u32(src)), "r"(bytes), "r"(rbar)
                 : "memory");
}

// One arrival on block `rank`'s mbarrier that also expects `bytes` of
// complete_tx stores in the current phase.
__device__ __forceinline__ void mbar_arrive_expect_remote(unsigned rbar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cluster.shared::cluster.b64 _, [%0], %1;\n" ::"r"(rbar),
                 "r"(bytes)
                 : "memory");
}

// Release store of v to the int at the same place in block `rank`.
__device__ __forceinline__ void st_release_remote(int32_t* p, unsigned rank, int32_t v) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    asm volatile("st.release.cluster.shared::cluster.u32 [%0], %1;\n" ::"r"(r), "r"(v) : "memory");
}

__device__ __forceinline__ int32_t ld_acquire_local(const int32_t* p) {
    int32_t v;
    asm volatile("ld.acquire.cluster.shared::cta.u32 %0, [%1];\n" : "=r"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}

__device__ __forceinline__ void cl_barrier() { asm volatile("bar.sync 1, 384;\n" ::: "memory"); }
__device__ __forceinline__ void e_barrier(int group) { asm volatile("bar.sync %0, 128;\n" ::"r"(2 + group) : "memory"); }
// Called by every thread of both blocks of the cluster (rank = block rank).
template <bool kScores>
__device__ void fill_wide_cl(const CoreArgs& a, const ReadDesc& r, ClSmem& ws, ClShared& cs, int tid,
                             unsigned rank) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const CellConsts cc = make_consts(r, a.g);
    const int n_events = r.n_events, n_kmers = r.n_kmers, n_bands = r.n_bands;
    const int group = tid >> 7;  // block 0: 0 = B, 1 = D, 2 = K, 3 = idle; block 1: E groups 0-3
    const int t = tid & (kSlots - 1);
    const long long lim = a.spin_limit;
    unsigned long long timeouts = 0;
    bool dead = false;  // a wait ran out: later waits do not wait (the batch reports a timeout)

    int k0 = -1 - kBand / 2, e0 = kBand / 2;  // band 1 (band 0 is (49,-51), band 1 moved down)
    RingState rs;
    if (rank == 0 && group == 2) rings_init(ws.rg, rs, a, r, t, k0, e0);
    if (rank == 0 && tid == 0) {
        for (int i = 0; i < kClRing; ++i) mbar_init(&cs.full[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (rank == 1 && tid == 0) {
        cs.k0ring[1] = k0;
        cs.progress = 1;
    }
    cluster.sync();  // barriers initialised, progress 1 published, rings filled

    if (rank == 1) {
        // ------------------------------------------------ E (block 1): group g, bands 2+g, 6+g, ...
        const float* gm_p = a.km_gm + r.km_off;
        const float* sd_p = a.km_sd + r.km_off;
        const float* rsd_p = a.km_rsd + r.km_off;
        const float* k1_p = a.km_k1 + r.km_off;
        const float* ev_p = a.ev_mean + r.ev_off;
        struct In {
            float x, gm, sd, rsd, k1;
        };
        // band bn's inputs in slot t, k-mer window from the latest published placement;
        // waits until that placement is at most kClRing bands back (its ring slot is free)
        auto fetch = [&](int bn) {
            int prog = ld_acquire_local(&cs.progress);
            for (long long i = 0; prog < bn - kClRing && i < (dead ? 0 : lim); ++i)
                prog = ld_acquire_local(&cs.progress);
            if (prog < bn - kClRing) {
                ++timeouts;
                dead = true;
            }
            const int kp = cs.k0ring[prog & 63];
            const int kk = kp + ((t - kp) & 127);
            const int e = bn - 2 - kk;
            // cells outside the read get finite stand-ins; their flags keep them out of the band
            const bool in = kk >= 0 && kk < n_kmers && e >= 0 && e < n_events;
            const int kc = in ? kk : 0, ec = in ? e : 0;
            return In{__ldg(ev_p + ec), __ldg(gm_p + kc), __ldg(sd_p + kc), __ldg(rsd_p + kc), __ldg(k1_p + kc)};
        };
        int bn = 2 + group;
        In cur = bn < n_bands ? fetch(bn) : In{0.0f, 0.0f, 1.0f, 1.0f, 0.0f};
        for (; bn < n_bands; bn += 4) {
            bool ok;
            const float em = emission_fast(cur.x, cur.gm, cur.sd, cur.rsd, cur.k1, ok);
            const EmSplit s1 = em_split(em, cc.step_h, cc.step_l);
            const EmSplit s2 = em_split(em, cc.stay_h, cc.stay_l);
            if (bn + 4 < n_bands) cur = fetch(bn + 4);  // loads in flight across the stores
            // staged in this block's own copy of the slot (free: the band kClRing back
            // was consumed, so its copy has been read), then one bulk copy per array
            const int s = (bn - 2) % kClRing;
            ws.emu[s][t] = make_float4(s2.p, s2.w,
                                       ok ? __fadd_rn(fabsf(em), fabsf(cc.stay_h)) : __int_as_float(0x7fc00000), em);
            ws.emd[s][t] = make_float2(s1.p, s1.w);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // visible to the bulk copy
            e_barrier(group);
            if (t == 0) {
                const unsigned rbar = mapa_u32(&cs.full[s], 0);
                // one arrival and the band's 128 x 24 bytes complete the slot's phase
                mbar_arrive_expect_remote(rbar, kSlots * 24);
                bulk_to_remote(mapa_u32(&ws.emu[s][0], 0), &ws.emu[s][0], kSlots * 16, rbar);
                bulk_to_remote(mapa_u32(&ws.emd[s][0], 0), &ws.emd[s][0], kSlots * 8, rbar);
            }
        }
    } else if (group == 0) {
        // ------------------------------------------------ B (block 0): the chain
        ws.sc[1][t] = (t == 127) ? a.g.trim_f : -INFINITY;
        ws.fr[0][t] = 0u;
        ws.fr[1][t] = (t == 127) ? ABEA_FROM_U : 0u;
        if (t == 0) {
            ws.k0h[0] = k0;
            ws.k0h[1] = k0;
            a.band_k0[r.band_off] = k0;
        }
    }
    if (rank == 0 && group < 3) {
        cl_barrier();  // band 1 in shared memory
        if (group == 0) {
            float* scores = kScores ? a.scores + r.band_off * kSlots : nullptr;
            float s_prev = (t == 127) ? a.g.trim_f : -INFINITY;  // band 1
            float lp = (t == 0) ? 0.0f : -INFINITY;              // band 0 shifted by one slot
            if (kScores) {
                scores[t] = (t == 127) ? 0.0f : -INFINITY;
                scores[kSlots + t] = s_prev;
            }
            unsigned long long slow = 0;
            int b = 2, cb = 0;
            float best = 0.0f, left = 0.0f;
            uint32_t from = 0u;
            bool valid = false, bad = false;
            auto finish = [&]() {
                best = valid ? best : -INFINITY;
                from = valid ? from : 0u;
                if (k0 <= -1) {  // trim cell (k = -1, slot 127) while the band reaches below k-mer 0
                    const bool here = (t == 127) && (k0 >= -kBand);
                    const float tv = ws.trim[cb];
                    best = here ? tv : best;
                    from = here ? (tv == -INFINITY ? 0u : ABEA_FROM_U) : from;
                }
                ws.sc[cb][t] = best;
                ws.fr[b & 7][t] = from;
                if (kScores && in_bounds(b, n_bands, a.counters)) scores[(int64_t)b * kSlots + t] = best;
                lp = left;
                s_prev = best;
            };
            while (true) {
                bool to_slow = false;
                for (; b < n_bands; ++b) {
                    cl_barrier();  // B_{b-1}
                    const int pb = (b - 1) & 1, es = (b - 2) % kClRing;
                    cb = b & 1;
                    // band b's emissions: D saw their mbarrier phase complete before the
                    // barrier above (it prepared band b's diagonal candidates from them)
                    const float ll = ws.sc[pb][k0 & 127];
                    const float ur = ws.sc[pb][(k0 + kBand - 1) & 127];
                    left = ws.sc[pb][(t + 127) & 127];
                    const float d = ws.dc[cb][t];
                    const int f = ws.flags[cb][t];
                    const float4 eu = ws.emu[es][t];
                    const EmSplit su{eu.x, eu.y};
                    const float mu = eu.z;
                    bool oku;
                    const float u = exact_from_split(s_prev, su, mu, oku);
                    const bool right = band_moves_right(ll, ur, b);
                    k0 += right ? 1 : 0;
                    e0 += right ? 0 : 1;
                    valid = (f & (right ? 2 : 1)) != 0;
                    uint32_t from_du;
                    const float best_du = pick_du(d, u, from_du);
                    bool okl;
                    const float l = exact_skip(left, cc.skip_h, cc.skip_l, okl);
                    best = pick_l(best_du, from_du, l, from);
                    bad = valid && !(oku && okl && (f & 4));
                    if (__any_sync(kFull, bad)) {
                        to_slow = true;
                        break;
                    }
                    finish();
                }
                if (!to_slow) break;
                if (bad) {  // a proof failed: the reference's FP64 arithmetic
                    const int ep = e0 - ((t - k0) & 127);
                    best = cell_slow(lp, s_prev, left, ws.rg.ev[ep & (kEvRing - 1)], ws.rg.gm[t], ws.rg.sd[t],
                                     ws.rg.k1[t], cc, from);
                    ++slow;
                }
                finish();
                ++b;
            }
            cl_barrier();  // B_{n_bands-1}
            if (slow) atomicAdd(&a.counters[0], slow);
        } else if (group == 1) {
            // ------------------------------------------------ D (block 0)
            // band bn's diagonal candidates, inside flags and trim value, with the
            // band before it placed at k0
            auto prep = [&](int bn, float diag) {
                const int es = (bn - 2) % kClRing;
                if (!mbar_wait(&cs.full[es], (unsigned)((bn - 2) / kClRing) & 1u, dead ? 0 : lim)) {
                    ++timeouts;
                    dead = true;
                }
                const float em = ws.emu[es][t].w;
                const float2 ed = ws.emd[es][t];
                const EmSplit s1{ed.x, ed.y};
                bool okd;
                const float d = exact_from_split(diag, s1, __fadd_rn(fabsf(em), fabsf(cc.step_h)), okd);
                const int o = (t - k0) & 127;
                const int kk = k0 + o;
                const int e = bn - 2 - kk;
                const bool inb = (kk >= 0) && (kk < n_kmers) && (e >= 0) && (e < n_events);
                ws.dc[bn & 1][t] = d;
                ws.flags[bn & 1][t] =
                    ((inb && o < kBand) ? 1 : 0) | ((inb && o >= 1 && o <= kBand) ? 2 : 0) | (okd ? 4 : 0);
                if (k0 <= 0 && t == 0) {  // trim cell of band bn (GPU/align_cuda.cl:431-443)
                    const int e_t = bn - 1;
                    ws.trim[bn & 1] =
                        (e_t < n_events) ? __double2float_rn(__dmul_rn(a.g.lp_trim, (double)(e_t + 1))) : -INFINITY;
                }
            };
            prep(2, (t == 0) ? 0.0f : -INFINITY);  // band 0 shifted by one slot
            for (int b = 2; b < n_bands; ++b) {
                cl_barrier();  // B_{b-1}
                // B is done with the emissions of bands <= b-1, D with those of band b:
                // E may reuse their ring slots; band b-1's placement was published with them
                // (every kClPublish bands: each release is a cluster-scope fence)
                if (t == 0 && (b & (kClPublish - 1)) == 0) st_release_remote(&cs.progress, 1, b - 1);
                const int pb = (b - 1) & 1;
                const float ll = ws.sc[pb][k0 & 127];
                const float ur = ws.sc[pb][(k0 + kBand - 1) & 127];
                const bool right = band_moves_right(ll, ur, b);
                k0 += right ? 1 : 0;
                if (t == 0) {
                    ws.k0h[b & 7] = k0;
                    // E reads the placement of the published band only (b - 1 at b a multiple of
                    // kClPublish): written with the next progress store's release
                    if (((b + 1) & (kClPublish - 1)) == 0) *cluster.map_shared_rank(&cs.k0ring[b & 63], 1) = k0;
                }
                if (b + 1 < n_bands) prep(b + 1, ws.sc[pb][(t + 127) & 127]);
            }
            cl_barrier();  // B_{n_bands-1}
        } else if (group == 2) {
            // ------------------------------------------------ K (block 0): bookkeeping, rings
            uint8_t* trace = a.trace + r.trace_off * kSlots;
            int32_t* bk0 = a.band_k0 + r.band_off;
            float* lastc = a.last_col + r.ev_off;
            const int sl_last = (n_kmers - 1) & 127;
            for (int b = 2; b <= n_bands; ++b) {
                cl_barrier();  // B_{b-1}
                const int bp = b - 1;
                const int kp = ws.k0h[bp & 7];
                if ((b & 3) == 2) rings_step(ws.rg, rs, a, r, t, kp, bp - 2 - kp, 9);
                const int ep0 = bp - 2 - kp;
                const int ol = n_kmers - 1 - kp;
                if (ol < kBand && t == sl_last && bp >= 2) {  // last k-mer column (GPU/align_cuda.cl:722-746)
                    int lo, hi;
                    band_range(kp, ep0, n_events, n_kmers, lo, hi);
                    if (ol >= lo && ol < hi && in_bounds(ep0 - ol, n_events, a.counters))
                        lastc[ep0 - ol] = ws.sc[bp & 1][t];
                }
                if (t == 0 && in_bounds(bp, n_bands, a.counters)) bk0[bp] = kp;
                if ((bp & 3) == 3 || bp == n_bands - 1) {
                    const int q0 = bp & ~3, nj = bp - q0;
                    uint32_t word = 0u;
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (j <= nj) word |= (ws.fr[(q0 + j) & 7][t] & 0xffu) << (8 * j);
                    if (in_bounds(bp >> 2, (n_bands + 3) / 4, a.counters))
                        reinterpret_cast<uint32_t*>(trace + (int64_t)(bp >> 2) * 512)[t] = word;
                }
            }
            cp_async_wait_all();
        }
    }
    if (timeouts) atomicAdd(&a.counters[2], timeouts);
}

// ---------------------------------------------------------------- post
struct alignas(16) PostSmem {
    uint8_t tr[4 * kPostChunkBands * kSlots];  // ring of 64 bands of trace, tile layout
};

__device__ __forceinline__ float path_emission(const PostArgs& a, const ReadDesc& r, int k, int e) {
    const int64_t ko = r.km_off + k;
    return emission_ieee(a.ev_mean[r.ev_off + e], a.km_gm[ko], a.km_sd[ko], a.km_k1[ko]);
}

// One pair's emission for the QC sum as an integer multiple of 2^-24 (exact when
// 0.5 <= |em| < 2^20; `exact` turns false otherwise).  The division is Markstein's
// (div_rn): no routine call, so that the loads of several cells are in flight at once.
__device__ __forceinline__ void qc_term(const PostArgs& a, const ReadDesc& r, abea_aligned_pair_t p, long long& isum,
                                        long long& iabs, bool& exact) {
    const int64_t ko = r.km_off + p.ref_pos;
    bool ok;
    const float em =
        emission_rn(a.ev_mean[r.ev_off + p.read_pos], a.km_gm[ko], a.km_sd[ko], a.km_rsd[ko], a.km_k1[ko], ok);
    const float aem = fabsf(em);
    const long long q = __float2ll_rn(__fmul_rn(em, 16777216.0f));
    const bool in = ok && aem >= 0.5f && aem < 1048576.0f;
    isum += in ? q : 0ll;
    iabs += in ? (q < 0 ? -q : q) : 0ll;
    exact = exact && in;
}

__device__ __forceinline__ void post_write(const PostArgs& a, int ri, int result, float best, int best_e, int status,
                                           int n_out, int cap, bool reversed, int last_from);

// One traceback step: D -> (k-1, e-1), U -> (k, e-1), L -> (k-1, e); gap counting.
__device__ __forceinline__ void step_back(uint32_t from, int& k, int& e, int& gap, int& max_gap) {
    k -= (from != ABEA_FROM_U) ? 1 : 0;
    e -= (from != ABEA_FROM_L) ? 1 : 0;
    gap = (from == ABEA_FROM_L) ? gap + 1 : 0;
    max_gap = max(max_gap, gap);
}

// Serial double sum of the path's emissions in the reference's order (from the
// walk's first cell), re-walking the trace from global memory.  Used only when
// the path is longer than its output slot.  `flat` re-walks through the emulated
// flat band array (no finite end, see post_read_warp).
__device__ double serial_path_sum(const PostArgs& a, const ReadDesc& r, const uint8_t* trace, const int32_t* bk0,
                                  bool flat, int e, int k) {
    double sum = 0.0;
    int gap = 0, mg = 0;
    while (k >= 0 && e >= 0) {
        sum = __dadd_rn(sum, (double)path_emission(a, r, k, e));
        const int64_t band = (int64_t)e + k + 2;
        if (flat) {
            const int64_t f = band * kBand + ((band - 2 - bk0[band]) - e);
            if (f < 0 || f >= (int64_t)r.n_bands * kBand) break;
            const int64_t b2 = f / kBand;
            step_back(trace[trace_index(b2, (bk0[b2] + (int)(f - b2 * kBand)) & 127)], k, e, gap, mg);
        } else {
            step_back(trace[trace_index(band, k & 127)], k, e, gap, mg);
        }
    }
    return sum;
}

// Lane 0's state of a traceback walk.
struct Walk {
    int k, e, n_out, gap, max_gap, last_k, last_from;
    double sum;  // emissions of the walked cells in walk order (kSum)
};

// What a walk does with each cell: store the pair, sum its emission (walk
// order), or record it in a speculative segment map (spec[band - band_lo] =
// k | index << 22 for the cells below band spec_hi).
enum WalkMode { kWalkPairs = 0, kWalkSum = 1, kWalkSpec = 2 };

// Walks the path from (w.k, w.e) while its band is >= band_lo.  The trace tiles
// come from `trace` (band trace_band0 at its start; bands below bands_end exist)
// through a shared-memory ring of kRing 16-band chunks: the chunk being walked
// and the one below it resident, the others in flight.  Each round of loads
// takes the backpointers of the nine cells two moves can reach and takes up to
// three steps from them; the moves are decoded arithmetically (D = 0, U = 1,
// L = 2: the k-mer steps back unless U, the event unless L).  Every lane walks
// the same path; lane 0 stores.  Returns true once the path has ended (k or e
// below 0); false when it left the segment.

template <int kMode, int kRing>
__device__ bool walk_segment(const uint8_t* trace, int trace_band0, int bands_end, int band_lo, uint8_t* ring,
                             int lane, Walk& w, abea_aligned_pair_t* out, int cap, const PostArgs& a,
                             const ReadDesc& r, int32_t* spec = nullptr, int spec_hi = 0) {
    constexpr bool kSum = kMode == kWalkSum;
    static_assert(kRing >= 4 && (kRing & (kRing - 1)) == 0, "ring of a power of two chunks, at least four");
    const int bands_pad = (bands_end + 3) & ~3;
    const int c_lo = band_lo / kPostChunkBands;
    auto stage = [&](int c) {  // chunk c = bands [16c, 16c + 16)
        if (c >= c_lo) {
            const int lo_band = c * kPostChunkBands;
            const int bytes = min(kPostChunkBands, bands_pad - lo_band) * kSlots;
            const uint8_t* src = trace + (int64_t)(lo_band - trace_band0) * kSlots;
            uint8_t* dst = ring + (c & (kRing - 1)) * (kPostChunkBands * kSlots);
            for (int off = lane * 16; off < bytes; off += 32 * 16) cp_async16(dst + off, src + off);
        }
        cp_async_commit();  // an empty group keeps the group count in step
    };
    const uint8_t* tb = ring;
    auto T = [&](int band, int k) -> uint32_t {  // 0, 1 or 2; the clamp keeps every step a move
        const int rb = band & (kRing * kPostChunkBands - 1);
        return min((uint32_t)tb[((rb >> 2) << 9) | ((k & 127) << 2) | (rb & 3)], 2u);
    };
    int k = __shfl_sync(kFull, w.k, 0), e = __shfl_sync(kFull, w.e, 0);
    int c = (e + k + 2) / kPostChunkBands;
    // chunks c and c-1 resident while chunk c is walked, kRing - 2 more in flight
#pragma unroll
    for (int j = 0; j < kRing - 1; ++j) stage(c - j);
    bool ended = false, left_seg = false;
    for (; c >= c_lo && !ended && !left_seg; --c) {
        cp_async_wait_group<kRing - 3>();  // chunks c and c-1 have landed
        __syncwarp();
        stage(c - (kRing - 1));  // into the ring slot of chunk c+1, already walked
        // Every lane walks the same path (warp-uniform branches: the walk in one
        // divergent lane ran slower); lane 0 stores the pairs.
        {
            const int lo = c * kPostChunkBands;
            auto emit = [&](int kk, int ee, uint32_t f) {
                if (kMode == kWalkSpec) {
                    const int band = ee + kk + 2;
                    if (band < spec_hi) {
                        if (lane == 0) spec[band - band_lo] = kk | (w.n_out << 22);
                        ++w.n_out;
                    }
                    return;
                }
                if (kSum)
                    w.sum = __dadd_rn(w.sum, (double)path_emission(a, r, kk, ee));
                else if (w.n_out < cap && lane == 0)
                    out[w.n_out] = abea_aligned_pair_t{kk, ee};
                ++w.n_out;
                w.last_k = kk;
                w.last_from = (int)f;
                w.gap = (f == ABEA_FROM_L) ? w.gap + 1 : 0;
                w.max_gap = max(w.max_gap, w.gap);
            };
            k = w.k;
            e = w.e;
            while (true) {
                const int band = e + k + 2;
                if ((k | e) < 0) {
                    ended = true;
                    break;
                }
                if (band < lo) {
                    left_seg = band < band_lo;
                    break;
                }
                // Up to three steps from one round of loads: the backpointers of every
                // cell two moves can reach (band offset db <= 4, k-mer offset dk <= 2;
                // bands >= lo - 4, resident) packed 2 bits each at position 3*db + dk.
                // A move adds 7 (D: db+2, dk+1), 3 (U: db+1) or 4 (L: db+1, dk+1).
                const uint32_t W = T(band, k) | (T(band - 1, k) << 6) | (T(band - 1, k - 1) << 8) |
                                   (T(band - 2, k) << 12) | (T(band - 2, k - 1) << 14) |
                                   (T(band - 2, k - 2) << 16) | (T(band - 3, k - 1) << 20) |
                                   (T(band - 3, k - 2) << 22) | (T(band - 4, k - 2) << 28);
                uint32_t pos2 = 0;  // 2 * position
#pragma unroll
                for (int st = 0; st < 3; ++st) {
                    const uint32_t f = (W >> pos2) & 3u;
                    emit(k, e, f);
                    k -= (int)((f & 1u) ^ 1u);
                    e -= (int)((f >> 1) ^ 1u);
                    pos2 += (0x86eu >> (4 * f)) & 0xfu;
                    // a step that ends the path or leaves the resident segment stops the round
                    if ((k | e) < 0 || e + k + 2 < band_lo) break;
                }
            }
            w.k = k;
            w.e = e;
        }
    }
    cp_async_wait_all();
    __syncwarp();
    return ended;
}

// Recomputes the trace of segment seg (bands [seg*kCkBands, (seg+1)*kCkBands)) of
// a checkpointed read into its scratch slot.  The whole warp calls it.
__device__ __forceinline__ void recompute_segment(const CoreArgs& ca, const ReadDesc& r, Rings& rg, int lane, int seg) {
    FillSpan sp;
    sp.b_begin = max(2, seg * kCkBands);
    sp.b_end = min((seg + 1) * kCkBands, r.n_bands);
    sp.ck_in = seg > 0 ? ca.ck + r.ck_off + (int64_t)seg * kCkStride : nullptr;
    sp.ck_out = nullptr;
    sp.trace = ca.ck_scratch + (int64_t)r.ck_slot * (kCkBands * kSlots);
    sp.trace_band0 = seg * kCkBands;
    sp.trace_tiles = kCkBands / 4;
    sp.side = false;
    fill_warp<false, true>(ca, r, rg, lane, sp);
    __syncwarp();
    __threadfence_block();
}

// One warp per read: best end, traceback, QC, reverse (GPU/align_cuda.cl:618-899).
// Best end (GPU/align_cuda.cl:722-746): the first strict maximum of
// s(e) = (float)(band + (n_events-e)*lp_trim) on the last k-mer column; the
// whole warp calls it and every lane gets the result (best_e = 0 when no end is finite).
__device__ void best_end_warp(const PostArgs& a, const ReadDesc& r, int lane, float& best_out, int& best_e_out) {
    const int n_events = r.n_events;
    const double lp_trim = a.g.lp_trim;
    const float* lastc = a.last_col + r.ev_off;
    float best = -INFINITY;
    int best_e = 0x7fffffff;
    for (int e = lane; e < n_events; e += 32) {
        const float v = lastc[e];
        if (v == -INFINITY) continue;  // -inf + finite is -inf: never a strict maximum
        const float s = __double2float_rn(__dadd_rn((double)v, __dmul_rn((double)(n_events - e), lp_trim)));
        if (s > best) {
            best = s;
            best_e = e;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float ob = __shfl_xor_sync(kFull, best, off);
        const int oe = __shfl_xor_sync(kFull, best_e, off);
        if (ob > best || (ob == best && oe < best_e)) {
            best = ob;
            best_e = oe;
        }
    }
    if (!(best > -INFINITY)) best_e = 0;
    best_out = best;
    best_e_out = best_e;
}


// QC, reverse and the per-read results of a walked path (GPU/align_cuda.cl:830-897).
template <int kRing>
__device__ void post_tail(const CoreArgs& ca, const PostArgs& a, int ri, const ReadDesc& r, uint8_t* ring, Rings& rg,
                          int lane, float best, int best_e, int n_out, int max_gap, int status, int last_k,
                          int last_from);

// `ring`: kRing * 2 KB of shared memory (16-byte aligned) for the traceback's trace chunks.
// A finished read's pairs out[0, n) into the caller's host buffer, when the batch
// mirrors its results there (threads t of nt; the pairs are final and visible to them).
__device__ __forceinline__ void mirror_pairs(const PostArgs& a, const ReadDesc& r, const abea_aligned_pair_t* out,
                                             int n, int t, int nt) {
    abea_aligned_pair_t* h = a.outm ? a.outm->pairs : nullptr;
    if (!h || n <= 0) return;
    h += r.out_off;
    for (int i = t; i < n; i += nt) h[i] = out[i];
}

template <int kRing>
__device__ void post_read_warp(const CoreArgs& ca, const PostArgs& a, int ri, uint8_t* ring, Rings& rg, int lane) {
    const ReadDesc r = a.reads[ri];
    if (r.skip) {
        if (lane == 0) {
            a.n_pairs[ri] = 0;
            if (a.outm && a.outm->n_pairs) a.outm->n_pairs[ri] = 0;
            a.best_scores[ri] = -INFINITY;
            a.status[ri] = 0;
        }
        return;
    }
    const int n_kmers = r.n_kmers, n_bands = r.n_bands;
    float best;
    int best_e;
    best_end_warp(a, r, lane, best, best_e);

    abea_aligned_pair_t* out = a.pairs + r.out_off;
    const uint8_t* trace = a.trace + r.trace_off * kSlots;
    const uint8_t* ck_seg = ca.ck_scratch + (int64_t)r.ck_slot * (kCkBands * kSlots);
    const int32_t* bk0 = a.band_k0 + r.band_off;
    const int cap = r.out_cap;
    int n_out = 0, max_gap = 0, status = 0, last_k = n_kmers - 1, last_from = 0;

    if (best > -INFINITY) {
        // A finite end: the path only visits computed cells.
        Walk w{n_kmers - 1, best_e, 0, 0, 0, n_kmers - 1, 0, 0.0};
        if (!r.ck) {
            walk_segment<kWalkPairs, kRing>(trace, 0, n_bands, 0, ring, lane, w, out, cap, a, r);
        } else {
            // the trace was not kept: recompute it kCkBands bands at a time from
            // the checkpoints, top segment first, and walk each
            for (int seg = (w.k + w.e + 2) / kCkBands; seg >= 0; --seg) {
                recompute_segment(ca, r, rg, lane, seg);
                if (walk_segment<kWalkPairs, kRing>(ck_seg, seg * kCkBands, min((seg + 1) * kCkBands, n_bands),
                                               seg * kCkBands, ring, lane, w, out, cap, a, r))
                    break;
            }
        }
        n_out = w.n_out;
        max_gap = w.max_gap;
        last_k = w.last_k;
        last_from = w.last_from;
    } else if (lane == 0 && r.ck) {
        // No finite end on a read whose trace was not kept: the flat-array walk
        // below needs the whole trace.  Reported as undefined.
        status = ABEA_ERR_UNDEFINED;
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
            const int64_t band = (int64_t)cur_e + cur_k + 2;
            const int64_t flat = band * kBand + ((band - 2 - bk0[band]) - cur_e);
            if (flat < 0 || flat >= (int64_t)n_bands * kBand) {
                status = ABEA_ERR_UNDEFINED;
                break;
            }
            const int64_t b2 = flat / kBand;
            const uint32_t from = trace[trace_index(b2, (bk0[b2] + (int)(flat - b2 * kBand)) & 127)];
            last_from = (int)from;
            step_back(from, cur_k, cur_e, gap, max_gap);
        }
    }
    n_out = __shfl_sync(kFull, n_out, 0);
    max_gap = __shfl_sync(kFull, max_gap, 0);
    status = __shfl_sync(kFull, status, 0);
    last_k = __shfl_sync(kFull, last_k, 0);
    last_from = __shfl_sync(kFull, last_from, 0);
    __syncwarp();
    __threadfence_block();
    post_tail<kRing>(ca, a, ri, r, ring, rg, lane, best, best_e, n_out, max_gap, status, last_k, last_from);
}

template <int kRing>
__device__ void post_tail(const CoreArgs& ca, const PostArgs& a, int ri, const ReadDesc& r, uint8_t* ring, Rings& rg,
                          int lane, float best, int best_e, int n_out, int max_gap, int status, int last_k,
                          int last_from) {
    const int n_kmers = r.n_kmers, n_bands = r.n_bands;
    abea_aligned_pair_t* out = a.pairs + r.out_off;
    const uint8_t* trace = a.trace + r.trace_off * kSlots;
    const uint8_t* ck_seg = ca.ck_scratch + (int64_t)r.ck_slot * (kCkBands * kSlots);
    const int32_t* bk0 = a.band_k0 + r.band_off;
    const int cap = r.out_cap;
    int result = 0;
    bool reversed = false;
    if (status == 0 && n_out > 0) {
        // QC (GPU/align_cuda.cl:856-882).  After the reversal out[0] is the last
        // cell walked and out[n-1] the first, so spanned <=> last_k == 0.
        double sum;
        if (n_out <= cap) {
            // Every emission with 0.5 <= |em| < 2^20 is a multiple of 2^-24; when the
            // magnitudes sum below 2^53 * 2^-24 all of the reference's partial double
            // sums are exact and equal this integer sum, whatever the order.
            long long isum = 0, iabs = 0;
            bool exact = true;
#pragma unroll 4
            for (int i2 = lane; i2 < n_out; i2 += 32) qc_term(a, r, out[i2], isum, iabs, exact);
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
        } else if (!r.ck) {
            sum = 0.0;
            if (lane == 0)
                sum = serial_path_sum(a, r, trace, bk0, !(best > -INFINITY), best > -INFINITY ? best_e : 0,
                                      n_kmers - 1);
            sum = __shfl_sync(kFull, sum, 0);
        } else {
            // the path outgrew its output slot on a read whose trace was not kept:
            // recompute and walk again, summing the emissions in walk order
            Walk w{n_kmers - 1, best_e, 0, 0, 0, n_kmers - 1, 0, 0.0};
            for (int seg = (w.k + w.e + 2) / kCkBands; seg >= 0; --seg) {
                recompute_segment(ca, r, rg, lane, seg);
                if (walk_segment<kWalkSum, kRing>(ck_seg, seg * kCkBands, min((seg + 1) * kCkBands, n_bands),
                                              seg * kCkBands, ring, lane, w, out, cap, a, r))
                    break;
            }
            sum = __shfl_sync(kFull, w.sum, 0);
        }
        const double avg = __ddiv_rn(sum, (double)n_out);
        const bool pass = !(avg < -5.0) && last_k == 0 && max_gap <= 50;
        if (pass && n_out > cap) {
            status = ABEA_ERR_CAPACITY;
            result = ABEA_ERR_CAPACITY;
        } else if (pass) {
            // reverse in place (GPU/align_cuda.cl:830-843)
            for (int i2 = lane; i2 < n_out / 2; i2 += 32) {
                const abea_aligned_pair_t x = out[i2], y = out[n_out - 1 - i2];
                out[i2] = y;
                out[n_out - 1 - i2] = x;
            }
            result = n_out;
            reversed = true;
            __syncwarp();
            mirror_pairs(a, r, out, n_out, lane, 32);
        }
    } else if (status != 0) {
        result = status;
    }
    if (lane == 0) post_write(a, ri, result, best, best_e, status, n_out, cap, reversed, last_from);
}

// The per-read results, and the path the adjoint reads: its length, whether the
// output holds it in walk order or reversed, and the move into its last walked cell.
__device__ __forceinline__ void post_write(const PostArgs& a, int ri, int result, float best, int best_e, int status,
                                           int n_out, int cap, bool reversed, int last_from) {
    {
        a.n_pairs[ri] = result;
        if (a.outm && a.outm->n_pairs) a.outm->n_pairs[ri] = result;
        a.best_scores[ri] = best;
        a.status[ri] = status;
        if (a.path_len) {
            // the path for the adjoint: its length, whether the output holds it in
            // walk order or reversed, and the move into its last walked cell
            a.path_len[ri] = n_out;
            a.path_flags[ri] = (reversed ? kPathReversed : 0) | (n_out > cap ? kPathTruncated : 0) |
                               (best > -INFINITY ? 0 : kPathNoEnd) | (status != 0 ? kPathError : 0) |
                               (last_from << 8);
            a.best_event[ri] = best_e;
        }
    }
}

// ---------------------------------------------------------------- wide read's traceback, block-parallel
// The wide read's traceback is on the batch's critical path while the rest of its
// block waits, so the whole block walks it.  The path is cut into segments of
// kSpecBands bands.  Every thread walks one segment speculatively (up to
// kSpecRound segments at once), from the middle of the band kSpecMargin bands
// above it (paths from different cells of a band merge within a few dozen bands),
// recording its cells in a map in global scratch (L2); warp 0 then walks the true
// path through the round and, at the first cell it shares with a segment's
// speculative path, takes the rest of that segment from the map (the
// backpointers after a shared cell are the same); the block copies those cells
// into the output.  A segment whose speculative path the true one never meets is
// walked cell by cell, so the result never depends on the speculation.  Gaps, the
// last cell and the QC follow from the written pairs.
constexpr int kSpecMargin = 64;
constexpr int kSpecWarps = kWideThreads / 32;
constexpr int kPostRingDeep = 8;  // trace chunks of a traceback with shared memory to spare (16 KB)

struct WidePostSmem {  // overlays the wide fill's shared memory once the fill is done
    float best;
    int32_t best_e, k, e, n_out, done, max_gap, last_from, last_k, pass, qc_exact, slot;
    float wbest[kSpecWarps];
    int32_t wbest_e[kSpecWarps], qexact[kSpecWarps];
    long long qsum[kSpecWarps], qabs[kSpecWarps];
    union {
        struct {  // per segment of the round: where its speculative walk left, and the splice
            int32_t exit_k[kSpecRound], exit_e[kSpecRound], count[kSpecRound], ended[kSpecRound];
            int32_t task_idx[kSpecRound], task_off[kSpecRound];
        } seg;
        int32_t run[kWideThreads][4];  // per thread: leading L run, trailing L run, longest run, all L
    };
};

// All kWideThreads threads of the block call it.
__device__ void post_wide_block(const CoreArgs& ca, const PostArgs& a, int ri, uint8_t* wide_mem, Rings& rg0, int t,
                                int slot_of_block) {
    const int warp = t >> 5, lane = t & 31;
    WidePostSmem& ps = *reinterpret_cast<WidePostSmem*>(wide_mem);
    const ReadDesc r = a.reads[ri];
    // a path of several segments whose trace was kept and whose k-mers fit the map's 22 bits
    if (r.skip || r.ck || r.n_kmers >= (1 << 22) || r.n_bands < kSpecMinBands) {
        if (warp == 0) post_read_warp<kPostRingDeep>(ca, a, ri, wide_mem, rg0, lane);
        return;
    }
    {
        // best end by the block: the first strict maximum is the largest value at the
        // smallest event among equals, per thread, per warp, then over the warps
        const double lp_trim = a.g.lp_trim;
        const float* lastc = a.last_col + r.ev_off;
        float b = -INFINITY;
        int be = 0x7fffffff;
        for (int e = t; e < r.n_events; e += kWideThreads) {
            const float v = lastc[e];
            if (v == -INFINITY) continue;
            const float sv = __double2float_rn(__dadd_rn((double)v, __dmul_rn((double)(r.n_events - e), lp_trim)));
            if (sv > b) {
                b = sv;
                be = e;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float ob = __shfl_xor_sync(kFull, b, off);
            const int oe = __shfl_xor_sync(kFull, be, off);
            if (ob > b || (ob == b && oe < be)) {
                b = ob;
                be = oe;
            }
        }
        if (lane == 0) {
            ps.wbest[warp] = b;
            ps.wbest_e[warp] = be;
        }
        __syncthreads();
        if (t == 0) {
            for (int w = 1; w < kSpecWarps; ++w)
                if (ps.wbest[w] > b || (ps.wbest[w] == b && ps.wbest_e[w] < be)) {
                    b = ps.wbest[w];
                    be = ps.wbest_e[w];
                }
            ps.best = b;
            ps.best_e = b > -INFINITY ? be : 0;
            ps.slot = slot_of_block;  // the block's scratch slot for the maps (one wide read at a time)
        }
    }
    __syncthreads();
    const float best = ps.best;
    const int best_e = ps.best_e, slot = ps.slot;
    __syncthreads();  // read before warp 0 may reuse the memory below
    if (!(best > -INFINITY) || slot >= ca.n_spec) {
        if (warp == 0) post_read_warp<kPostRingDeep>(ca, a, ri, wide_mem, rg0, lane);
        return;
    }
    const int n_kmers = r.n_kmers, n_events = r.n_events, n_bands = r.n_bands, cap = r.out_cap;
    const uint8_t* trace = a.trace + r.trace_off * kSlots;
    const int32_t* bk0 = a.band_k0 + r.band_off;
    abea_aligned_pair_t* out = a.pairs + r.out_off;
    int32_t* map = ca.spec + (int64_t)slot * (kSpecRound * kSpecBands);
    const int b0 = best_e + n_kmers - 1 + 2;  // band of the path's first cell
    const int jtop = b0 / kSpecBands;
    if (t == 0) {
        ps.k = n_kmers - 1;
        ps.e = best_e;
        ps.n_out = 0;
        ps.done = 0;
    }
    for (int jr = jtop; jr >= 0; jr -= kSpecRound) {
        const int nseg = min(kSpecRound, jr + 1);  // segments jr, jr-1, ..., jr-nseg+1
        for (int i = t; i < nseg * kSpecBands; i += kWideThreads) map[i] = -1;
        __syncthreads();
        // ---- speculative walks: thread t takes segment jr - t, its trace bytes from L2
        if (t < nseg) {
            const int j = jr - t;
            const int seg_lo = j * kSpecBands, seg_hi = min(seg_lo + kSpecBands, n_bands);
            int k = n_kmers - 1, e = best_e;  // the top segment starts at the true start
            if (j != jtop) {
                const int sb = min(seg_hi - 1 + kSpecMargin, b0);
                int kk = bk0[sb] + kBand / 2;  // the middle of band sb, moved inside the read
                kk = max(kk, max(0, sb - 2 - (n_events - 1)));
                kk = min(kk, min(n_kmers - 1, sb - 2));
                k = kk;
                e = sb - 2 - kk;
            }
            int32_t* row = map + t * kSpecBands;
            int cnt = 0, ended = 0;
            while (true) {
                if ((k | e) < 0) {
                    ended = 1;
                    break;
                }
                const int band = e + k + 2;
                if (band < seg_lo) break;
                const uint32_t f = min((uint32_t)trace[trace_index(band, k & 127)], 2u);
                if (band < seg_hi && in_bounds(band - seg_lo, kSpecBands, ca.counters)) row[band - seg_lo] = k | (cnt++ << 22);
                k -= (int)((f & 1u) ^ 1u);
                e -= (int)((f >> 1) ^ 1u);
            }
            ps.seg.exit_k[t] = k;
            ps.seg.exit_e[t] = e;
            ps.seg.count[t] = cnt;
            ps.seg.ended[t] = ended;
            ps.seg.task_idx[t] = -1;
        }
        __syncthreads();
        // ---- the true path through the round (warp 0, every lane alike)
        if (warp == 0) {
            int k = ps.k, e = ps.e, n_out = ps.n_out;
            bool done = ps.done != 0;
            for (int wi = 0; wi < nseg && !done; ++wi) {
                const int seg_lo = (jr - wi) * kSpecBands;
                const int32_t* row = map + wi * kSpecBands;
                while (true) {
                    if ((k | e) < 0) {
                        done = true;
                        break;
                    }
                    const int band = e + k + 2;
                    if (band < seg_lo) break;
                    const int sp = row[band - seg_lo];
                    if (sp >= 0 && (sp & 0x3fffff) == k) {
                        // shared cell: the rest of the segment is the recorded path
                        const int idx = sp >> 22;
                        if (lane == 0) {
                            ps.seg.task_idx[wi] = idx;
                            ps.seg.task_off[wi] = n_out;
                        }
                        n_out += ps.seg.count[wi] - idx;
                        k = ps.seg.exit_k[wi];
                        e = ps.seg.exit_e[wi];
                        done = ps.seg.ended[wi] != 0;
                        break;
                    }
                    const uint32_t f = min((uint32_t)trace[trace_index(band, k & 127)], 2u);
                    if (lane == 0 && n_out < cap) out[n_out] = abea_aligned_pair_t{k, e};
                    ++n_out;
                    k -= (int)((f & 1u) ^ 1u);
                    e -= (int)((f >> 1) ^ 1u);
                }
            }
            if (lane == 0) {
                ps.k = k;
                ps.e = e;
                ps.n_out = n_out;
                ps.done = done ? 1 : 0;
            }
        }
        __syncthreads();
        // ---- the recorded parts, copied by the block
        for (int i = t; i < nseg * kSpecBands; i += kWideThreads) {
            const int wi = i / kSpecBands, idx0 = ps.seg.task_idx[wi];
            if (idx0 < 0) continue;
            const int sp = map[i];
            if (sp < 0 || (sp >> 22) < idx0) continue;
            const int pos = ps.seg.task_off[wi] + (sp >> 22) - idx0, kk = sp & 0x3fffff;
            if (pos < cap) out[pos] = abea_aligned_pair_t{kk, (jr - wi) * kSpecBands + (i % kSpecBands) - 2 - kk};
        }
        __syncthreads();
        if (ps.done) break;
    }
    const int n_out = ps.n_out;
    __syncthreads();  // read before warp 0 may reuse the memory below
    if (n_out > cap) {
        // the path outgrew its output slot: the serial walk handles what the reference does
        if (warp == 0) post_read_warp<kPostRingDeep>(ca, a, ri, wide_mem, rg0, lane);
        return;
    }
    // ---- gaps: the move out of pair i is L iff pair i+1 is the k-mer before at the same event;
    // out of the last pair, its backpointer
    if (t == 0) {
        const abea_aligned_pair_t lp = out[n_out - 1];
        ps.last_from = (int)min((uint32_t)trace[trace_index(lp.read_pos + lp.ref_pos + 2, lp.ref_pos & 127)], 2u);
    }
    __syncthreads();
    {
        const int per = (n_out + kWideThreads - 1) / kWideThreads;
        const int i0 = min(t * per, n_out), i1 = min(i0 + per, n_out);
        int pre = 0, cur = 0, mx = 0;
        bool all = true;
        abea_aligned_pair_t p = i0 < i1 ? out[i0] : abea_aligned_pair_t{0, 0};
        for (int i = i0; i < i1; ++i) {
            bool is_l;
            if (i + 1 < n_out) {
                const abea_aligned_pair_t q = out[i + 1];
                is_l = q.read_pos == p.read_pos && q.ref_pos == p.ref_pos - 1;
                p = q;
            } else {
                is_l = ps.last_from == ABEA_FROM_L;
            }
            cur = is_l ? cur + 1 : 0;
            mx = max(mx, cur);
            if (all && is_l) ++pre;
            all = all && is_l;
        }
        ps.run[t][0] = pre;
        ps.run[t][1] = cur;
        ps.run[t][2] = mx;
        ps.run[t][3] = all ? 1 : 0;
    }
    // ---- QC (GPU/align_cuda.cl:856-882): the exact integer emission sum by the block
    {
        long long isum = 0, iabs = 0;
        bool exact = true;
#pragma unroll 4
        for (int i = t; i < n_out; i += kWideThreads) qc_term(a, r, out[i], isum, iabs, exact);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            isum += __shfl_xor_sync(kFull, isum, off);
            iabs += __shfl_xor_sync(kFull, iabs, off);
        }
        exact = __all_sync(kFull, exact);
        if (lane == 0) {
            ps.qsum[warp] = isum;
            ps.qabs[warp] = iabs;
            ps.qexact[warp] = exact ? 1 : 0;
        }
    }
    __syncthreads();
    if (t == 0) {
        int carry = 0, best_run = 0;
        for (int i = 0; i < kWideThreads; ++i) {
            if (ps.run[i][3]) {
                carry += ps.run[i][0];
            } else {
                best_run = max(best_run, carry + ps.run[i][0]);
                carry = ps.run[i][1];
            }
            best_run = max(best_run, max(carry, ps.run[i][2]));
        }
        long long isum = 0, iabs = 0;
        bool exact = true;
        for (int w = 0; w < kSpecWarps; ++w) {
            isum += ps.qsum[w];
            iabs += ps.qabs[w];
            exact = exact && ps.qexact[w];
        }
        exact = exact && iabs < (1ll << 53);
        const int last_k = out[n_out - 1].ref_pos;  // the last cell walked (before the reversal)
        const double sum = __dmul_rn((double)isum, 5.9604644775390625e-08);  // * 2^-24
        const double avg = __ddiv_rn(sum, (double)n_out);
        ps.max_gap = best_run;
        ps.last_k = last_k;
        ps.qc_exact = exact ? 1 : 0;
        ps.pass = (!(avg < -5.0) && last_k == 0 && best_run <= 50) ? 1 : 0;
    }
    __syncthreads();
    const int max_gap = ps.max_gap, last_from = ps.last_from, last_k = ps.last_k;
    if (!ps.qc_exact) {
        // emissions outside the exact integer form: warp 0 sums serially in walk order
        if (warp == 0)
            post_tail<kPostRingDeep>(ca, a, ri, r, wide_mem, rg0, lane, best, best_e, n_out, max_gap, 0, last_k,
                                     last_from);
        return;
    }
    const bool pass = ps.pass != 0;
    if (pass)  // reverse in place (GPU/align_cuda.cl:830-843)
        for (int i = t; i < n_out / 2; i += kWideThreads) {
            const abea_aligned_pair_t x = out[i], y = out[n_out - 1 - i];
            out[i] = y;
            out[n_out - 1 - i] = x;
        }
    if (pass && a.outm) {
        __syncthreads();  // the reversal is done
        mirror_pairs(a, r, out, n_out, t, kWideThreads);
    }
    if (t == 0) post_write(a, ri, pass ? n_out : 0, best, best_e, 0, n_out, cap, pass, last_from);
}

// ---------------------------------------------------------------- plain form kernels
template <bool kScores>
__global__ void __launch_bounds__(32) abea_core_warp_kernel(CoreArgs a) {
    __shared__ __align__(16) Rings rg;
    const int i = blockIdx.x;
    if (i >= a.n_reads) return;
    const ReadDesc& r = a.reads[i];
    if (r.skip) return;
    if (r.ck)
        fill_warp<kScores, true>(a, r, rg, threadIdx.x, forward_span(a, r));
    else
        fill_warp<kScores, false>(a, r, rg, threadIdx.x, forward_span(a, r));
}

__global__ void __launch_bounds__(32) abea_post_kernel(CoreArgs ca, PostArgs a) {
    __shared__ __align__(16) uint8_t ring[kPostRingDeep * kPostChunkBands * kSlots];
    __shared__ __align__(16) Rings rg;  // recompute of checkpointed reads
    const int i = blockIdx.x;
    if (i >= a.n_reads) return;
    post_read_warp<kPostRingDeep>(ca, a, i, ring, rg, threadIdx.x);
}

// ---------------------------------------------------------------- batched form
constexpr int kBatchedWarps = kWideThreads / 32;

struct BatchedSmem {
    WideSmem wide;                     // phase 1: the block's wide read
    Rings warp_rings[kBatchedWarps];   // phase 2: one per warp
    // every warp's post staging; in phase 1b each half's medium read uses its eight
    // warps' entries (post[8 * half] on), which no other warp touches meanwhile
    PostSmem post[kBatchedWarps];
    int32_t pick;                      // the block's wide read, or -1
    int32_t wide_slot;                 // the block's first pick: its traceback scratch slot
    int32_t free_rank;                 // rank among the blocks with neither a wide nor medium reads, or -1
    int32_t mid_block;                 // 1: a block of the medium reads
    int32_t mid_pick[2];               // each half's medium read
};
static_assert(offsetof(BatchedSmem, warp_rings) % 16 == 0 && offsetof(BatchedSmem, post) % 16 == 0 &&
                  sizeof(Rings) % 16 == 0 && sizeof(PostSmem) % 16 == 0,
              "cp.async destinations must be 16-byte aligned");
static_assert(sizeof(BatchedSmem) <= 227 * 1024, "batched kernel shared memory exceeds the per-block limit");
static_assert(offsetof(WideSmem, ems) % 16 == 0 && offsetof(WideSmem, emm) % 8 == 0,
              "vector accesses to the emission ring must be aligned");
static_assert(sizeof(WideSmem) >= kPostRingDeep * kPostChunkBands * kSlots && alignof(WideSmem) >= 16,
              "the wide read's traceback ring lives in the wide fill's shared memory");
static_assert(sizeof(WidePostSmem) <= sizeof(WideSmem), "the wide read's traceback state fits the fill's memory");
static_assert(sizeof(MidSmem) <= (kBatchedWarps / 2) * sizeof(PostSmem) &&
                  sizeof(MidSmem) >= kPostRingDeep * kPostChunkBands * kSlots,
              "a medium read's fill, and then its traceback ring, fit its half's post staging");



template <bool kScores>
__global__ void __launch_bounds__(kWideThreads, 1) abea_batched_kernel(CoreArgs a, PostArgs p, PreArgs pa) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BatchedSmem& sm = *reinterpret_cast<BatchedSmem*>(smem_raw);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    // phase 1: the wide reads, longest first
    // Each block's first pick decides its role: the first blocks to arrive take a
    // wide read each (and then pull the wide reads past the first wave, one after
    // another); the next ones the medium reads (two at a time per block, enough
    // blocks for each half to start one); the others the first wave of the
    // warp-shape reads.
    const int n_midb = min((a.n_mid + 1) / 2, max((int)gridDim.x - a.n_wide, 0));
    if (t == 0) {
        const int q = atomicAdd(&a.queue[0], 1);
        sm.pick = q < a.n_wide ? a.order[q] : -1;
        sm.wide_slot = q;  // the block's traceback scratch slot: wide reads go longest first, so only
                           // the first blocks' reads (and the reads they pull later) need one
        sm.mid_block = (q >= a.n_wide && q < a.n_wide + n_midb) ? 1 : 0;
        sm.free_rank = q < a.n_wide + n_midb ? -1 : q - a.n_wide - n_midb;
    }
    __syncthreads();
    int wide_read = sm.pick;
    const int free_rank = sm.free_rank, wide_slot = sm.wide_slot;
    while (wide_read >= 0) {
        const ReadDesc& r = a.reads[wide_read];
        pre_read(pa, wide_read, t, kWideThreads);
        __syncthreads();  // the read's parameters are in memory for the whole block
        if (!r.skip) fill_chain<kScores, 2, kWideRing>(a, r, sm.wide, t, 1);
        __syncthreads();
        __threadfence_block();
        // the whole block walks the wide read's traceback (the fill's shared memory is free)
        post_wide_block(a, p, wide_read, reinterpret_cast<uint8_t*>(&sm.wide), sm.warp_rings[0], t, wide_slot);
        // then the next wide read past the first wave (one per block), longest first
        __syncthreads();  // the traceback is done with the block's shared memory and the pick
        if (t == 0) {
            const int q = (int)gridDim.x + atomicAdd(&a.queue[4], 1);
            sm.pick = q < a.n_wide ? a.order[q] : -1;
        }
        __syncthreads();
        wide_read = sm.pick;
    }
    // phase 1b: the medium reads, each half of a medium block (eight warps) pulling
    // one at a time: pre, fill, and the traceback by the half's first warp; the
    // blocks done with their wide reads join in
    if (a.n_mid > 0 && free_rank < 0) {
        const int half = warp >> 3, ht = t & (kMidThreads - 1), hw = ht >> 5;
        MidSmem& ms = *reinterpret_cast<MidSmem*>(&sm.post[half * (kBatchedWarps / 2)]);
        const int bar0 = 1 + half * kMidBars, bar_half = bar0 + kMidBars - 1;
        while (true) {
            if (ht == 0) sm.mid_pick[half] = atomicAdd(&a.queue[3], 1);
            named_bar_sync(bar_half, kMidThreads);  // the pick is visible; the last read's traceback is done
            const int q = sm.mid_pick[half];
            if (q >= a.n_mid) break;  // the whole half leaves together
            const int ri = a.order[a.n_wide + q];
            const ReadDesc& r = a.reads[ri];
            pre_read(pa, ri, ht, kMidThreads);
            named_bar_sync(bar_half, kMidThreads);  // the read's parameters are in memory; the pick was read
            if (!r.skip) fill_chain<kScores, 1, kMidRing>(a, r, ms, ht, bar0);
            named_bar_sync(bar_half, kMidThreads);  // the fill is done: its memory becomes the traceback ring
            __threadfence_block();
            if (hw == 0) post_read_warp<kPostRingDeep>(a, p, ri, reinterpret_cast<uint8_t*>(&ms), sm.warp_rings[warp], lane);
        }
    }
    // phase 2: the first wave is static, the blocks with neither a wide nor medium
    // reads taking the longest remaining reads round-robin (warp w of free block f:
    // read f + F*w), so that the long ones spread over the SMs; then every warp
    // pulls the rest longest-first.
    const int n_pre = a.n_wide + a.n_mid;
    const int n_rest = a.n_reads - n_pre;
    const int n_free = max((int)gridDim.x - a.n_wide - n_midb, 0);
    const int wave = min(n_rest, n_free * kBatchedWarps);
    for (int pass = 0;; ++pass) {
        int q;
        if (pass == 0) {
            if (free_rank < 0) continue;
            q = free_rank + n_free * warp;
            if (q >= wave) continue;
        } else {
            q = 0;
            if (lane == 0) q = wave + atomicAdd(&a.queue[1], 1);
            q = __shfl_sync(kFull, q, 0);
            if (q >= n_rest) break;
        }
        const int ri = a.order[n_pre + q];
        const ReadDesc& r = a.reads[ri];
        pre_read(pa, ri, lane, 32);
        __syncwarp();  // the read's parameters are in memory for the warp
        if (!r.skip) {
            if (r.ck)
                fill_warp<kScores, true>(a, r, sm.warp_rings[warp], lane, forward_span(a, r));
            else
                fill_warp<kScores, false>(a, r, sm.warp_rings[warp], lane, forward_span(a, r));
        }
        __syncwarp();
        __threadfence_block();
        post_read_warp<4>(a, p, ri, sm.post[warp].tr, sm.warp_rings[warp], lane);
    }
}

struct BatchedClSmem {
    union {
        ClSmem wide;                       // phase 1: the cluster's wide read
        Rings warp_rings[kBatchedWarps];   // then: one per warp
    };
    PostSmem post[kBatchedWarps];          // every warp's post staging
    ClShared cs;
};
static_assert(offsetof(BatchedClSmem, warp_rings) % 16 == 0 && offsetof(BatchedClSmem, post) % 16 == 0,
              "cp.async destinations must be 16-byte aligned");
static_assert(sizeof(BatchedClSmem) <= 227 * 1024, "cluster kernel shared memory exceeds the per-block limit");

// The batched form on clusters of two blocks: phase 1 fills one of the longest
// reads per cluster with the cluster-pair wide shape, phase 2 as the
// single-block kernel.
template <bool kScores>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kWideThreads, 1)
    abea_batched_cl_kernel(CoreArgs a, PostArgs p) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BatchedClSmem& sm = *reinterpret_cast<BatchedClSmem*>(smem_raw);
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank();
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    if (rank == 0 && t == 0) {
        const int q = atomicAdd(&a.queue[0], 1);
        const int pick = q < a.n_wide ? a.order[q] : -1;
        sm.cs.pick = pick;
        *cluster.map_shared_rank(&sm.cs.pick, 1) = pick;
    }
    cluster.sync();
    const int wide_read = sm.cs.pick;
    if (wide_read >= 0) {
        const ReadDesc& r = a.reads[wide_read];
        if (!r.skip) fill_wide_cl<kScores>(a, r, sm.wide, sm.cs, t, rank);
        // every emission copy has landed (block 0 consumed them all) before either
        // block reuses the fill's shared memory
        cluster.sync();
        __threadfence_block();
        if (rank == 0 && warp == 0) post_read_warp<4>(a, p, wide_read, sm.post[0].tr, sm.warp_rings[0], lane);
    }
    // phase 2: every warp pulls reads longest-first
    const int n_rest = a.n_reads - a.n_wide;
    while (true) {
        int q = 0;
        if (lane == 0) q = atomicAdd(&a.queue[1], 1);
        q = __shfl_sync(kFull, q, 0);
        if (q >= n_rest) break;
        const int ri = a.order[a.n_wide + q];
        const ReadDesc& r = a.reads[ri];
        if (!r.skip) {
            if (r.ck)
                fill_warp<kScores, true>(a, r, sm.warp_rings[warp], lane, forward_span(a, r));
            else
                fill_warp<kScores, false>(a, r, sm.warp_rings[warp], lane, forward_span(a, r));
        }
        __syncwarp();
        __threadfence_block();
        post_read_warp<4>(a, p, ri, sm.post[warp].tr, sm.warp_rings[warp], lane);
    }
    cluster.sync();  // neither block leaves while the other may still write its shared memory
}

// ---------------------------------------------------------------- launches
cudaError_t launch_plain(const LaunchArgs& la, int* launches) {
    const int n = la.core.n_reads;
    abea_pre_kernel<<<n, 128, 0, la.stream>>>(la.pre);
    cudaEventRecordWithFlags(la.ev_pre, la.stream, la.capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    if (la.core.scores)
        abea_core_warp_kernel<true><<<n, 32, 0, la.stream>>>(la.core);
    else
        abea_core_warp_kernel<false><<<n, 32, 0, la.stream>>>(la.core);
    cudaEventRecordWithFlags(la.ev_core, la.stream, la.capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    abea_post_kernel<<<n, 32, 0, la.stream>>>(la.core, la.post);
    *launches = 3;
    return cudaGetLastError();
}

int batched_blocks_per_sm(bool scores) {
    static int cached[2] = {0, 0};
    int& c = cached[scores ? 1 : 0];
    if (c == 0) {
        const size_t smem = sizeof(BatchedSmem);
        if (scores) {
            cudaFuncSetAttribute(abea_batched_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, abea_batched_kernel<true>, kWideThreads, smem);
        } else {
            cudaFuncSetAttribute(abea_batched_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, abea_batched_kernel<false>, kWideThreads, smem);
        }
        if (c <= 0) c = 1;
    }
    return c;
}

static int cl_max_dyn_smem_set() {
    static int done = 0;
    if (!done) {
        cudaFuncSetAttribute(abea_batched_cl_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(BatchedClSmem));
        cudaFuncSetAttribute(abea_batched_cl_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(BatchedClSmem));
        done = 1;
    }
    return done;
}

cudaError_t launch_batched(const LaunchArgs& la, int* launches) {
    const int n = la.core.n_reads;
    if (la.cluster) abea_pre_kernel<<<n, 128, 0, la.stream>>>(la.pre);  // otherwise pre runs inside the kernel
    cudaEventRecordWithFlags(la.ev_pre, la.stream, la.capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    const bool scores = la.core.scores != nullptr;
    if (la.cluster) {
        // one wide read per cluster of two blocks; an even grid of one block per SM
        cl_max_dyn_smem_set();
        const int want = 2 * la.core.n_wide + (n - la.core.n_wide + kBatchedWarps - 1) / kBatchedWarps;
        const int grid = 2 * std::max(1, std::min(la.sm_count / 2, (want + 1) / 2));
        const size_t smem = sizeof(BatchedClSmem);
        if (scores)
            abea_batched_cl_kernel<true><<<grid, kWideThreads, smem, la.stream>>>(la.core, la.post);
        else
            abea_batched_cl_kernel<false><<<grid, kWideThreads, smem, la.stream>>>(la.core, la.post);
        cudaEventRecordWithFlags(la.ev_core, la.stream,
                                 la.capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
        *launches = 2;
        return cudaGetLastError();
    }
    // every resident block: the blocks without a wide read share the first wave
    const int max_blocks = batched_blocks_per_sm(scores) * la.sm_count;
    const int grid = std::max(1, std::min(max_blocks, n));
    const size_t smem = sizeof(BatchedSmem);
    if (scores)
        abea_batched_kernel<true><<<grid, kWideThreads, smem, la.stream>>>(la.core, la.post, la.pre);
    else
        abea_batched_kernel<false><<<grid, kWideThreads, smem, la.stream>>>(la.core, la.post, la.pre);
    cudaEventRecordWithFlags(la.ev_core, la.stream, la.capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
    *launches = 1;
    return cudaGetLastError();
}

}  // namespace abea

// ---------------------------------------------------------------- no-allocation entry point
// For callers that cannot allocate device memory: a framework whose own
// allocator owns the whole device and hands out every buffer, or a service whose
// device memory budget is fixed when it starts.  One read goes through the plain
// pre/core/post kernels with every scratch buffer carved out of one file-scope
// device array, which exists on every GPU that loads this library for the life
// of the process.  Calls whose work overlaps on the GPU race on that array.
namespace abea {

constexpr size_t kNoAllocScratchBytes = 32ull << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

__global__ void noalloc_write_desc(ReadDesc* dst, ReadDesc d) { *dst = d; }

// The array's device address differs per CUDA context: one per device for the
// runtime's primary contexts, a new one after cudaDeviceReset, and one in each
// context a caller creates itself.  The addresses are kept per context, keyed by
// the context's process-unique id (cuCtxGetId; a context's handle may be reused
// after a reset, its id is not).  The two driver calls are found through the
// runtime (cudaGetDriverEntryPointByVersion), so the library needs no link
// against the driver library.
static std::mutex g_noalloc_mutex;
struct NoAllocSlot {
    unsigned long long ctx_id;
    void* ptr;
};
static NoAllocSlot g_noalloc_slots[64];  // most recently looked up first
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

// Id of the current context, 0 when none is current or the driver calls are missing.
static unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = (CtxGetCurrentFn)f1;
            get_id = (CtxGetIdFn)f2;
        }
        looked_up = true;
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of g_noalloc_scratch in the current context: looked up with
// cudaGetSymbolAddress the first time a context asks, then kept.  nullptr on failure.
static void* noalloc_scratch_address(cudaError_t* err) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = current_ctx_id();
    if (id != 0) {
        for (int i = 0; i < 64 && g_noalloc_slots[i].ptr; ++i)
            if (g_noalloc_slots[i].ctx_id == id) return g_noalloc_slots[i].ptr;
    }
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // makes the device's primary context current if none is
    if (*err != cudaSuccess || !p) return nullptr;
    if (id == 0) id = current_ctx_id();
    if (id != 0) {  // keep it, most recent first (the oldest of a full table is dropped)
        for (int i = 63; i > 0; --i) g_noalloc_slots[i] = g_noalloc_slots[i - 1];
        g_noalloc_slots[0] = NoAllocSlot{id, p};
    }
    return p;
}

static size_t noalloc_align(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of scratch one read needs.
static size_t noalloc_bytes(int32_t sequence_len, int32_t n_events) {
    const int64_t nk = std::max<int64_t>(sequence_len - ABEA_KMER_SIZE + 1, 0);
    const int64_t ne = std::max<int64_t>(n_events, 0);
    const int64_t nb = (nk > 0 && ne > 0) ? ne + nk + 2 : 0;
    const size_t ne_pad = (size_t)round_up(std::max<int64_t>(ne, 1), kChunk);
    const size_t nk_pad = (size_t)round_up(std::max<int64_t>(nk, 1), kChunk);
    const size_t nb_pad = (size_t)round_up(std::max<int64_t>(nb, 4), 4);
    return noalloc_align(sizeof(ReadDesc)) + 2 * noalloc_align(4 * ne_pad) + 4 * noalloc_align(4 * nk_pad) +
           noalloc_align(nb_pad * kSlots) + noalloc_align(4 * nb_pad) + noalloc_align(16) + noalloc_align(32);
}

}  // namespace abea

extern "C" abea_status_t abea_align_noalloc(abea_aligned_pair_t* pairs, int32_t* n_pairs, int32_t out_capacity,
                                            const char* sequence, int32_t sequence_len, const abea_event_t* events,
                                            int32_t n_events, const abea_model_t* model, abea_scalings_t scaling,
                                            void* stream) {
    using namespace abea;
    if (!pairs || !n_pairs || !sequence || !model || out_capacity < 0 || sequence_len < 0 || n_events < 0 ||
        (n_events > 0 && !events)) {
        abea_internal_set_error("abea_align_noalloc: invalid argument");
        return ABEA_ERR_INVALID_ARG;
    }
    const size_t need = noalloc_bytes(sequence_len, n_events);
    if (need > kNoAllocScratchBytes) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "abea_align_noalloc: the read needs %zu bytes of scratch but the fixed scratch holds %zu "
                 "bytes (reads of up to about 230,000 bands, n_events + n_kmers + 2)",
                 need, kNoAllocScratchBytes);
        abea_internal_set_error(msg);
        return ABEA_ERR_INVALID_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        abea_internal_set_error("abea_align_noalloc: no current CUDA device");
        return ABEA_ERR_NO_DEVICE;
    }
    // the first call in each context (per device, and again after a device
    // reset) looks up the array's address; later calls reuse it
    cudaError_t serr = cudaSuccess;
    unsigned char* base = (unsigned char*)noalloc_scratch_address(&serr);
    if (!base) {
        char msg[256];
        snprintf(msg, sizeof(msg), "abea_align_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(serr));
        abea_internal_set_error(msg);
        return ABEA_ERR_CUDA;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int32_t nk = sequence_len - ABEA_KMER_SIZE + 1;
    const int64_t nb = (nk > 0 && n_events > 0) ? (int64_t)n_events + nk + 2 : 0;
    const size_t ne_pad = (size_t)round_up(std::max<int64_t>(n_events, 1), kChunk);
    const size_t nk_pad = (size_t)round_up(std::max<int64_t>(nk, 1), kChunk);
    const size_t nb_pad = (size_t)round_up(std::max<int64_t>(nb, 4), 4);
    unsigned char* p = base;
    auto carve = [&](size_t bytes) {
        unsigned char* q = p;
        p += noalloc_align(bytes);
        return q;
    };
    ReadDesc* d_desc = (ReadDesc*)carve(sizeof(ReadDesc));
    float* ev_mean = (float*)carve(4 * ne_pad);
    float* last_col = (float*)carve(4 * ne_pad);
    float* km_gm = (float*)carve(4 * nk_pad);
    float* km_sd = (float*)carve(4 * nk_pad);
    float* km_rsd = (float*)carve(4 * nk_pad);
    float* km_k1 = (float*)carve(4 * nk_pad);
    uint8_t* trace = (uint8_t*)carve(nb_pad * kSlots);
    int32_t* band_k0 = (int32_t*)carve(4 * nb_pad);
    float* best = (float*)carve(4);
    int32_t* status = (int32_t*)(best + 1);
    unsigned long long* counters = (unsigned long long*)carve(32);

    const ReadDesc desc = describe_single_read(sequence_len, n_events, scaling, out_capacity);
    const GlobalConsts g = parity_consts();
    // every call shares the array: clear what must start at zero
    if (cudaMemsetAsync(counters, 0, 32, st) != cudaSuccess) {
        abea_internal_set_error("abea_align_noalloc: cudaMemsetAsync failed");
        return ABEA_ERR_CUDA;
    }
    noalloc_write_desc<<<1, 1, 0, st>>>(d_desc, desc);
    PreArgs pre{d_desc, 1, g, sequence, events, model, ev_mean, km_gm, km_sd, km_rsd, km_k1, last_col};
    CoreArgs core{d_desc, 1, g, ev_mean, km_gm, km_sd, km_rsd, km_k1, last_col, trace, nullptr, band_k0,
                  counters, nullptr, nullptr, 0, nullptr, nullptr, nullptr, 0, 1ll << 22};
    PostArgs post{d_desc,   1,      g,     ev_mean, km_gm,  km_sd,   km_k1,   km_rsd,  last_col,
                  trace,    band_k0, pairs, n_pairs, best,   status,  nullptr, nullptr, nullptr};
    abea_pre_kernel<<<1, 128, 0, st>>>(pre);
    abea_core_warp_kernel<false><<<1, 32, 0, st>>>(core);
    abea_post_kernel<<<1, 32, 0, st>>>(core, post);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof(msg), "abea_align_noalloc: launch failed: %s", cudaGetErrorString(e));
        abea_internal_set_error(msg);
        return ABEA_ERR_CUDA;
    }
    return ABEA_OK;
}

// ---------------------------------------------------------------- adjoint
// Gradient of the best path's log-likelihood along the fixed path of a finished
// forward run: the transitions and trims do not depend on the scalings or the
// pore model, so d(score)/d(theta) is the sum, over the path cells entered by a
// D or U move (the cells whose emission the score contains), of
//   d em/d shift = a/sd, d em/d scale = a*mu/sd, d em/d mu_k = a*scale/sd,
//   d em/d stdv_k = (a^2 - 1)/stdv_k, d em/d var = (a^2 - 1)/var (var-aware only),
// with em = log_inv_sqrt_2pi - log(sd) - a^2/2, a = (x - (scale*mu + shift))/sd,
// sd = stdv (times var when var-aware).  Everything is evaluated and accumulated
// in FP64.  Also accumulated: the Gauss-Newton normal equations of the residuals
// a in (shift, scale) — J^T J and J^T a with J = (-1/sd, -mu/sd) — and the FP64
// emission sum of the path.
namespace abea {

__global__ void __launch_bounds__(32) abea_adjoint_kernel(AdjArgs a) {
    const int ri = blockIdx.x, lane = threadIdx.x;
    if (ri >= a.n_reads) return;
    const ReadDesc r = a.reads[ri];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // shift, scale, var, j11, j12, j22, t1, t2, em
    int st = 0;
    const int len = r.skip ? 0 : a.path_len[ri];
    const int flags = r.skip ? 0 : a.path_flags[ri];
    if (len > 0 && (flags & (kPathTruncated | kPathNoEnd | kPathError))) {
        st = (flags & kPathTruncated) ? ABEA_ERR_CAPACITY : ABEA_ERR_UNDEFINED;
    } else if (len > 0) {
        const abea_aligned_pair_t* out = a.pairs + r.out_off;
        const bool rev = (flags & kPathReversed) != 0;
        const int last_from = flags >> 8;
        const char* s = a.seq + r.seq_off;
        const double scale = r.scale, shift = r.shift, var = r.var, log_var = r.log_var;
        for (int j = lane; j < len; j += 32) {
            const int w = rev ? len - 1 - j : j;  // walk position, 0 = best end
            const abea_aligned_pair_t c = out[j];
            bool counted;
            if (w < len - 1) {
                const abea_aligned_pair_t nx = rev ? out[j - 1] : out[j + 1];
                counted = nx.read_pos == c.read_pos - 1;  // D or U: the next walked cell is one event back
            } else {
                counted = last_from != (int)ABEA_FROM_L;
            }
            if (!counted) continue;
            uint32_t rank = 0;
#pragma unroll
            for (int q = 0; q < ABEA_KMER_SIZE; ++q) rank = (rank << 2) | base_rank(s[c.ref_pos + q]);
            const abea_model_t m = a.model[rank];
            const double mu = m.level_mean, sig = m.level_stdv;
            const double sd = a.var_aware ? sig * var : sig;
            const double lsd = a.var_aware ? (double)m.level_log_stdv + log_var : (double)m.level_log_stdv;
            const double x = a.ev_mean[r.ev_off + c.read_pos];
            const double isd = 1.0 / sd;
            const double av = (x - (scale * mu + shift)) * isd;
            acc[0] += av * isd;
            acc[1] += av * mu * isd;
            if (a.var_aware) acc[2] += (av * av - 1.0) / var;
            acc[3] += isd * isd;
            acc[4] += mu * isd * isd;
            acc[5] += mu * mu * isd * isd;
            acc[6] -= av * isd;
            acc[7] -= av * mu * isd;
            acc[8] += -0.91893853320467274 - lsd - 0.5 * av * av;
            if (a.grad_model) {
                atomicAdd(&a.grad_model[2 * rank], av * scale * isd);
                atomicAdd(&a.grad_model[2 * rank + 1], (av * av - 1.0) / sig);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_xor_sync(kFull, acc[i], off);
    if (lane == 0) {
        for (int i = 0; i < 3; ++i) a.grad_scalings[3 * ri + i] = acc[i];
        for (int i = 0; i < 5; ++i) a.gn[5 * ri + i] = acc[3 + i];
        a.path_em[ri] = acc[8];
        a.adj_status[ri] = st;
    }
}

cudaError_t launch_adjoint(const AdjArgs& a, cudaStream_t stream) {
    if (a.n_reads > 0) abea_adjoint_kernel<<<a.n_reads, 32, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace abea

// ---------------------------------------------------------------- method of moments
// f5c's estimate_scalings_using_mom (GPU/f5cmisc.h:47; its body is not part of the
// reference): the scale and shift that map the k-mer levels along the read onto
// the event means' mean and variance.  FP64 sums, one warp per read.
namespace abea {

__global__ void __launch_bounds__(32) abea_mom_kernel(MomArgs a) {
    const int ri = blockIdx.x, lane = threadIdx.x;
    if (ri >= a.n_reads) return;
    const ReadDesc r = a.reads[ri];
    double es = 0.0, es2 = 0.0, ks = 0.0, ks2 = 0.0;
    if (!r.skip) {
        for (int e = lane; e < r.n_events; e += 32) {
            const double x = a.ev[r.ev_src + e].mean;
            es += x;
            es2 += x * x;
        }
        const char* s = a.seq + r.seq_off;
        for (int k = lane; k < r.n_kmers; k += 32) {
            uint32_t rank = 0;
#pragma unroll
            for (int q = 0; q < ABEA_KMER_SIZE; ++q) rank = (rank << 2) | base_rank(s[k + q]);
            const double l = a.model[rank].level_mean;
            ks += l;
            ks2 += l * l;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        es += __shfl_xor_sync(kFull, es, off);
        es2 += __shfl_xor_sync(kFull, es2, off);
        ks += __shfl_xor_sync(kFull, ks, off);
        ks2 += __shfl_xor_sync(kFull, ks2, off);
    }
    if (lane == 0) {
        double scale = 1.0, shift = 0.0;
        if (!r.skip) {
            const double em = es / r.n_events, ev = es2 / r.n_events - em * em;
            const double km = ks / r.n_kmers, kv = ks2 / r.n_kmers - km * km;
            scale = sqrt(ev / kv);
            shift = em - scale * km;
        }
        a.out[2 * ri] = scale;
        a.out[2 * ri + 1] = shift;
    }
}

cudaError_t launch_mom(const MomArgs& a, cudaStream_t stream) {
    if (a.n_reads > 0) abea_mom_kernel<<<a.n_reads, 32, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace abea

// ---------------------------------------------------------------- postalign
// f5c's postalign (GPU/f5cmisc.h:51-52, prototype only; the output types are
// GPU/f5c.h:184-207): the AlignedPairs of a read turned into its base-to-event
// map and its event alignment records.  One warp per read over the pairs in
// order, 32 at a time.
//
// A pair counts for its k-mer when its event differs from the previous pair's;
// such a pair is the first one of its event on the path.  The traceback's path
// moves by one k-mer, one event or both at every step, so the counting pairs
// are exactly one per event from the first event on the path to the last, in
// order: the record of event e sits at e - first event, and a k-mer's map
// entry runs from its first counting pair's event to its last one's.  The first
// pass checks that shape (and the bounds every store below relies on).
namespace abea {

constexpr int kPaUnroll = 8;  // chunks of 32 pairs whose loads are in flight together

__global__ void __launch_bounds__(128) abea_postalign_kernel(PostalignArgs a) {
    const int lane = threadIdx.x & 31;
    const int ri = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (ri >= a.n_reads) return;  // whole warps
    const ReadDesc r = a.reads[ri];
    int n = r.skip ? 0 : a.n_pairs[ri];
    if (n < 0) n = 0;  // a read that ended with an error status has no pairs
    const abea_aligned_pair_t* P = a.pairs + r.out_off;
    bool ok = n <= r.out_cap;
    // pass 1: bounds and unit steps; pair i-1 of lane 0 is lane 31 of the previous chunk
    if (__all_sync(kFull, ok)) {
        int k31 = -1, e31 = -1;
        for (int base = 0; base < n; base += 32 * kPaUnroll) {
            int kk[kPaUnroll], ee[kPaUnroll];
#pragma unroll
            for (int u = 0; u < kPaUnroll; ++u) {
                const int i = base + 32 * u + lane;
                kk[u] = -1;
                ee[u] = -1;
                if (i < n) {
                    const abea_aligned_pair_t p = P[i];
                    kk[u] = p.ref_pos;
                    ee[u] = p.read_pos;
                }
            }
#pragma unroll
            for (int u = 0; u < kPaUnroll; ++u) {
                const int i = base + 32 * u + lane;
                int qk = __shfl_up_sync(kFull, kk[u], 1), qe = __shfl_up_sync(kFull, ee[u], 1);
                if (lane == 0) {
                    qk = k31;
                    qe = e31;
                }
                if (i < n) {
                    if (kk[u] < 0 || kk[u] >= r.n_kmers || ee[u] < 0 || ee[u] >= r.n_events) {
                        ok = false;
                    } else if (i > 0) {
                        const int dk = kk[u] - qk, de = ee[u] - qe;
                        ok = ok && dk >= 0 && dk <= 1 && de >= 0 && de <= 1 && (dk | de) != 0;
                    }
                }
                k31 = __shfl_sync(kFull, kk[u], 31);
                e31 = __shfl_sync(kFull, ee[u], 31);
            }
        }
    }
    ok = __all_sync(kFull, ok);
    if (!ok || n == 0) {
        if (lane == 0) {
            a.count[ri] = ok ? 0 : ABEA_ERR_INTERNAL;
            a.epb[ri] = 0.0;
        }
        return;
    }
    // Pass 1 above accepted only paths whose every step moves the k-mer and the
    // event forward by 0 or 1 (not both 0): the events are non-decreasing along
    // the path, so its first and last pairs hold the smallest and largest event
    // (the oracle takes the minimum and maximum; a path that is not monotone
    // never gets here, it is ABEA_ERR_INTERNAL).
    const int e_first = P[0].read_pos, e_last = P[n - 1].read_pos;
    const char* s = a.seq + r.seq_off;
    abea_index_pair_t* map = a.map + r.seq_off;
    uint4* rec = reinterpret_cast<uint4*>(a.rec + r.ev_src);
    int carry_e = -1, carry_k = -1, carry_rank = -1;  // the previous pair's event; the previous counting pair
    for (int base = 0; base < n; base += 32 * kPaUnroll) {
        int kk[kPaUnroll], ee[kPaUnroll];
#pragma unroll
        for (int u = 0; u < kPaUnroll; ++u) {
            const int i = base + 32 * u + lane;
            kk[u] = -1;
            ee[u] = -1;
            if (i < n) {
                const abea_aligned_pair_t p = P[i];
                kk[u] = p.ref_pos;
                ee[u] = p.read_pos;
            }
        }
        // counting pairs (event differs from the previous pair's) and their k-mers' bases
        bool qq[kPaUnroll];
        uint32_t w0[kPaUnroll], w1[kPaUnroll];  // bases 0-3 and 4-5 of the k-mer, little-endian
#pragma unroll
        for (int u = 0; u < kPaUnroll; ++u) {
            int e_prev = __shfl_up_sync(kFull, ee[u], 1);
            if (lane == 0) e_prev = carry_e;
            qq[u] = base + 32 * u + lane < n && ee[u] != e_prev;
            carry_e = __shfl_sync(kFull, ee[u], 31);
            w0[u] = 0;
            w1[u] = 0;
            if (qq[u]) {
                const uint8_t* sb = reinterpret_cast<const uint8_t*>(s + kk[u]);
                w0[u] = (uint32_t)sb[0] | (uint32_t)sb[1] << 8 | (uint32_t)sb[2] << 16 | (uint32_t)sb[3] << 24;
                w1[u] = (uint32_t)sb[4] | (uint32_t)sb[5] << 8;
            }
        }
#pragma unroll
        for (int u = 0; u < kPaUnroll; ++u) {
            const int k = kk[u], e = ee[u];
            const bool q = qq[u];
            int rank = 0;
            if (q) {
#pragma unroll
                for (int j = 0; j < ABEA_KMER_SIZE; ++j)
                    rank = (rank << 2) | (int)base_rank((char)((j < 4 ? w0[u] >> (8 * j) : w1[u] >> (8 * (j - 4))) & 0xff));
            }
            const unsigned qm = __ballot_sync(kFull, q);
            const unsigned below = qm & ((1u << lane) - 1u);
            const unsigned above = qm & ~((2u << lane) - 1u);  // lane 31: 2u << 31 wraps to 0, so none above
            const int src = below ? 31 - __clz(below) : lane;
            const int dst = above ? __ffs(above) - 1 : lane;
            const int k_below = __shfl_sync(kFull, k, src);
            const int rank_below = __shfl_sync(kFull, rank, src);
            const int k_above = __shfl_sync(kFull, k, dst);
            if (q) {
                const int pk = below ? k_below : carry_k;
                const int pr = below ? rank_below : carry_rank;
                if (pk != k) map[k].start = e;                // first counting pair of this k-mer
                if (!above || k_above != k) map[k].stop = e;  // last one in this chunk; later chunks overwrite
                const uint32_t hmm = rank != pr ? 'M' : 'E';
                // the 32-byte event_alignment_t: ref_kmer[7] + pad, ref_position, read_idx,
                // event_idx, rc, model_kmer[7], hmm_state, pad (little-endian bytes)
                const uint4 lo = make_uint4(w0[u], w1[u], (uint32_t)k, (uint32_t)ri);
                const uint4 hi = make_uint4((uint32_t)e, w0[u] << 8, w0[u] >> 24 | w1[u] << 8, hmm);
                rec[2 * (e - e_first)] = lo;
                rec[2 * (e - e_first) + 1] = hi;
            }
            if (qm) {
                const int lq = 31 - __clz(qm);
                carry_k = __shfl_sync(kFull, k, lq);
                carry_rank = __shfl_sync(kFull, rank, lq);
            }
            __syncwarp();  // orders this chunk's map stores before the next chunk's
        }
    }
    if (lane == 0) {
        a.count[ri] = e_last - e_first + 1;
        a.epb[ri] = (double)(e_last - e_first) / r.n_kmers;
    }
}

cudaError_t launch_postalign(const PostalignArgs& a, cudaStream_t stream) {
    if (a.n_reads > 0) abea_postalign_kernel<<<(a.n_reads + 3) / 4, 128, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace abea
