// abea_internal.h — layouts shared by the host orchestration and the kernels.
//
// Device data layout of one batch (all in HBM, 16-byte aligned regions):
//   reads[i]            ReadDesc: offsets and per-read constants (below)
//   seq                 bases, copied as given (reference layout, NUL separated)
//   ev_in               abea_event_t[sum n_events] as given (24 B/event)
//   model               abea_model_t[4096]
//   ev_mean             f32 [per read: round_up(n_events,16)]   event means (pre)
//   km_gm/km_sd/km_rsd/km_k1  f32 [per read: round_up(n_kmers,16)]  scaled level mean,
//                       level stdv, RN(1/stdv), (log_inv_sqrt_2pi - log stdv) per
//                       k-mer position (pre)
//   last_col            f32 [per read: round_up(n_events,16)]   scores of the last
//                       k-mer column, -inf where the cell was not computed (core)
//   trace               u8  [per read: round_up(n_bands,4) * 128]  backpointers in
//                       tiles of 4 bands x 128 k-mer slots, slot-major: one 32-bit
//                       word per slot holds its 4 bands (see trace_index)
//   scores              f32 [per read: round_up(n_bands,4) * 128]  optional, band-major, slot order
//   band_k0             i32 [per read: round_up(n_bands,4)]        kmer_idx of each band's
//                       lower-left cell (EventKmerPair.kmer_idx; event_idx = band-2-kmer_idx)
//   pairs / n_pairs     outputs in the reference layout (capacity 2*n_events at 2*event_ptr)
//
// A band's 100 cells live in 128 "k-mer slots": cell (e,k) of band b sits in slot
// k & 127, so a cell's up neighbour (e-1,k) is the same slot of band b-1 and its
// left/diagonal neighbours (k-1) are slot-1 of bands b-1 / b-2, whichever way the
// band moved.  The 28 slots outside the band hold -inf.
#pragma once
#include <stdint.h>

#include "../../include/abea.h"

namespace abea {

constexpr int kBand = ABEA_BANDWIDTH;  // 100 cells per band
constexpr int kSlots = 128;            // k-mer slots per band
constexpr int kEvRing = 256;           // event-mean ring (shared memory), entries
constexpr int kChunk = 16;             // prefetch granularity (k-mers / events)

struct ReadDesc {
    int64_t seq_off;    // first base in seq
    int64_t ev_src;     // first event in ev_in (reference event_ptr)
    int64_t ev_off;     // first entry in ev_mean / last_col (16-aligned)
    int64_t km_off;     // first entry in km_* (16-aligned)
    int64_t band_off;   // first band (multiple of 4) in scores/band_k0
    int64_t trace_off;  // first band (multiple of 4) of the read's trace (kept traces only)
    int64_t ck_off;     // first float of the read's band-score checkpoints (checkpointed reads)
    int32_t ck;         // 1: the trace is not kept; checkpoints every kCkBands bands instead
    int32_t ck_slot;    // recompute scratch slot of a checkpointed read
    int64_t out_off;    // first pair in the output (2*event_ptr)
    int32_t n_events;
    int32_t n_kmers;    // read_len - 5
    int32_t n_bands;    // n_events + n_kmers + 2
    int32_t out_cap;    // 2*n_events
    double lp_step;     // log(1 - exp(lp_skip) - exp(lp_stay)), computed on the host
    double lp_stay;     // log(p_stay)
    float step_h, step_l;  // lp_step = step_h + step_l + O(2^-48 lp_step)
    float stay_h, stay_l;
    float scale, shift, var, log_var;
    int32_t skip;       // 1: nothing to align (n_kmers <= 0 or n_events <= 0)
    int32_t in_hbm;     // 1: the pre stage reads this read's bases and events from HBM even
                        // when the batch's inputs are read from host memory
};

// Band-score checkpoints of reads whose trace exceeds the memory budget: at
// every band b = s*kCkBands (s >= 1) the fill stores the state it resumes from
// (band b-1's scores, band b-2's scores shifted by one slot, band b-1's
// placement) as one record of kCkStride floats; the traceback recomputes the
// trace of one kCkBands-band segment at a time into a scratch slot.
constexpr int kCkBands = 256;
constexpr int kCkStride = 264;  // 128 + 128 scores, k0, e0, padding to 16 bytes

// Block-parallel traceback of a wide read: segments of kSpecBands bands, walked
// speculatively kSpecRound at a time (one thread each), their cell maps in a
// scratch slot of kSpecRound * kSpecBands int32 per wide read in flight.  Reads of
// at least kSpecMinBands bands qualify; at most kSpecMaxSlots slots per batch.
constexpr int kSpecBands = 256;
constexpr int kSpecRound = 512;
constexpr int kSpecMinBands = 2 * kSpecBands;
constexpr int kSpecMaxSlots = 256;

struct GlobalConsts {
    double lp_skip;  // log(1e-10)
    double lp_trim;  // log(0.01)
    float skip_h, skip_l;
    float trim_f;    // (float)lp_trim
    int32_t var_aware;
};

// Per-read status written by the post stage (0 = ok).
enum ReadStatus : int32_t {
    kReadOk = 0,
};

// Byte index of cell (band, slot) inside a read's trace region.
__host__ __device__ inline int64_t trace_index(int64_t band, int slot) {
    return (band >> 2) * 512 + (int64_t)slot * 4 + (band & 3);
}

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

}  // namespace abea
