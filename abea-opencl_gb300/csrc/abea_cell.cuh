// abea_cell.cuh — per-cell arithmetic of the banded recurrence.
//
// The reference scores a cell as (GPU/align_cuda.cl:530-542, align_swi.cl:478-488)
//     d = (float)(((double)diag + lp_step) + (double)em)
//     u = (float)(((double)up   + lp_stay) + (double)em)
//     l = (float)( (double)left + lp_skip)
// i.e. float scores plus double constants, rounded twice in double and once to
// float.  GB300 runs FP64 adds and f32<->f64 conversions at ~1/70 of the FP32
// rate, so the kernels evaluate these sums in FP32 with error-free
// transformations:
//   * the double constant B is split as B = Bh + Bl + r (Bh = RN32(B),
//     Bl = RN32(B - Bh), |r| <= 2^-48 |B|);
//   * Fast2Sum (Dekker 1971) gives p + q = em + Bh and s + e = a + p exactly;
//   * the remaining tail t = e + (q + Bl) is tiny, and the exact sum
//     S = a + B + em lies within eb of s + t, where eb = 2^-42 (|a| + |em| + |Bh|)
//     also covers the reference's own two double roundings (<= 2^-52 of the
//     same magnitudes);
//   * RN32(s + (t + eb)) == RN32(s + (t - eb)) proves, by monotonicity of
//     rounding, that every value in [S - eb, S + eb] — in particular the
//     reference's double result — rounds to that float.
// When the proof does not go through (operands too close to a rounding
// boundary, Fast2Sum preconditions not met, non-finite inputs) the cell is
// recomputed with native FP64 exactly as the reference does.  The fallback is
// rare (about one candidate in 10^5 on nanopore-like data, plus the first
// bands of each read where scores are still small).
//
// All float operations go through __f*_rn intrinsics so that nvcc never
// contracts them into FMAs; the library is also built with -fmad=false.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace abea {

#define ABEA_FROM_D 0u
#define ABEA_FROM_U 1u
#define ABEA_FROM_L 2u

constexpr float kLogInvSqrt2Pi = -0.918938f;  // GPU/align_cuda.cl:66
constexpr float kErrScale = 2.2737367544323206e-13f;  // 2^-42

struct CellConsts {
    float step_h, step_l, stay_h, stay_l, skip_h, skip_l;
    float b_max;     // max(|step_h|, |stay_h|)
    float em_floor;  // power of two <= both |step_h| and |stay_h| magnitudes' floors
    double lp_step, lp_stay, lp_skip;
};

// log_normal_pdf of the reference in its operation order
// (GPU/align_cuda.cl:68-75, 511-528): a = (x - mean)/stdv;
// lp = (log_inv_sqrt_2pi - log_stdv) + ((-0.5f*a)*a).  k1 is the first
// bracket, precomputed per k-mer with the same rounding.
__device__ __forceinline__ float emission(float x, float gm, float sd, float k1) {
    float a = __fdiv_rn(__fsub_rn(x, gm), sd);
    float t = __fmul_rn(__fmul_rn(-0.5f, a), a);
    return __fadd_rn(k1, t);
}

// Exact (float)(((double)a + (Bh+Bl)) + (double)em) or ok=false.
// p, q: Fast2Sum(em, Bh) computed by the caller; mc = |em| + b_max.
__device__ __forceinline__ float add_fast(float a, float p, float w, float mc, bool em_ok,
                                          bool& ok) {
    float s = __fadd_rn(a, p);
    float e = __fsub_rn(p, __fsub_rn(s, a));
    float t = __fadd_rn(e, w);
    float eb = __fmul_rn(__fadd_rn(fabsf(a), mc), kErrScale);
    float hp = __fadd_rn(s, __fadd_rn(t, eb));
    float hm = __fadd_rn(s, __fsub_rn(t, eb));
    bool a_inf = (a == -INFINITY);
    ok = ((hp == hm) && (fabsf(a) >= fabsf(p)) && em_ok) || (a_inf && em_ok);
    return a_inf ? -INFINITY : hp;
}

// Exact (float)((double)a + (Bh+Bl)) (single double rounding) or ok=false.
__device__ __forceinline__ float add2_fast(float a, float bh, float bl, bool& ok) {
    float s = __fadd_rn(a, bh);
    float e = __fsub_rn(bh, __fsub_rn(s, a));
    float t = __fadd_rn(e, bl);
    float eb = __fmul_rn(__fadd_rn(fabsf(a), fabsf(bh)), kErrScale);
    float hp = __fadd_rn(s, __fadd_rn(t, eb));
    float hm = __fadd_rn(s, __fsub_rn(t, eb));
    bool a_inf = (a == -INFINITY);
    ok = ((hp == hm) && (fabsf(a) >= fabsf(bh))) || a_inf;
    return a_inf ? -INFINITY : hp;
}

// The three candidates of one cell on the fast path.
__device__ __forceinline__ void candidates_fast(float diag, float up, float left, float em,
                                                const CellConsts& c, float& d, float& u,
                                                float& l, bool& ok) {
    // Fast2Sum(em, Bh) is exact when exponent(em) >= exponent(Bh).
    bool em_ok = fabsf(em) >= c.em_floor && fabsf(em) < INFINITY;
    float mc = __fadd_rn(fabsf(em), c.b_max);
    float pd = __fadd_rn(em, c.step_h);
    float wd = __fadd_rn(__fsub_rn(c.step_h, __fsub_rn(pd, em)), c.step_l);
    float pu = __fadd_rn(em, c.stay_h);
    float wu = __fadd_rn(__fsub_rn(c.stay_h, __fsub_rn(pu, em)), c.stay_l);
    bool okd, oku, okl;
    d = add_fast(diag, pd, wd, mc, em_ok, okd);
    u = add_fast(up, pu, wu, mc, em_ok, oku);
    l = add2_fast(left, c.skip_h, c.skip_l, okl);
    ok = okd && oku && okl;
}

// The reference's arithmetic verbatim, in FP64 (slow path).
__device__ __forceinline__ void candidates_slow(float diag, float up, float left, float em,
                                             const CellConsts& c, float& d, float& u,
                                             float& l) {
    d = __double2float_rn(__dadd_rn(__dadd_rn((double)diag, c.lp_step), (double)em));
    u = __double2float_rn(__dadd_rn(__dadd_rn((double)up, c.lp_stay), (double)em));
    l = __double2float_rn(__dadd_rn((double)left, c.lp_skip));
}

// max with the reference's tie rules (GPU/align_cuda.cl:536-542):
// U wins ties with D, L wins ties with both; NaN candidates never win.
__device__ __forceinline__ float pick(float d, float u, float l, uint32_t& from) {
    float best = d;
    from = ABEA_FROM_D;
    best = u > best ? u : best;
    from = (best == u) ? ABEA_FROM_U : from;
    best = l > best ? l : best;
    from = (best == l) ? ABEA_FROM_L : from;
    return best;
}

}  // namespace abea
