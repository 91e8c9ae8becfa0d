// abea_cell.cuh — per-cell arithmetic of the banded recurrence.
//
// The reference scores a cell as (GPU/align_cuda.cl:530-542, align_swi.cl:478-488)
//     d = (float)(((double)diag + lp_step) + (double)em)
//     u = (float)(((double)up   + lp_stay) + (double)em)
//     l = (float)( (double)left + lp_skip)
// then keeps the largest with U winning ties over D and L over both.  GB300 runs
// FP64 adds and f32<->f64 conversions at ~1/70 of the FP32 rate, so a cell is
// evaluated in FP32, bit-exactly:
//
//  * d and u are evaluated exactly with exact_sum (below) and compared exactly;
//    they depend only on the previous bands, so the kernels compute them before
//    the band's exchange of neighbour cells (off the band-to-band critical path);
//  * l is evaluated exactly too (exact_skip), without a branch: the skip move
//    wins in most cells away from the path (about 70% of the computed cells of
//    the synthetic reads), so it is no rare case;
//  * the emission's division uses a reciprocal and a proven correction step;
//  * if any exactness proof does not go through, the cell is recomputed with
//    native FP64 and IEEE division, literally as the reference does (cell_slow),
//    outside the kernels' band loops.
//
// exact_sum(a, B, c) returns RN32(RN64(RN64(a + B) + c)) for floats a, c and a
// double B = bh + bl + r (bh = RN32(B), bl = RN32(B - bh), |r| <= 2^-48|B|).
// Write M = |a| + |c| + |bh| and u = 2^-24 (float unit roundoff).
//  1. TwoSum (Knuth) gives p + q = c + bh exactly (|q| <= u|p|); Fast2Sum
//     (Dekker 1971) gives s + e = a + p exactly when |a| >= |p| (checked;
//     |e| <= u|s|).  So the exact sum T = a + B + c = s + e + q + bl + r.
//  2. w = RN32(q + bl) and t = RN32(e + w) round once each:
//     |w - (q + bl)| <= u|w| <= 2u^2 M and |t - (e + w)| <= u|t| <= 4u^2 M,
//     with |r| <= 2^-48 M, so |T - (s + t)| <= 7u^2 M < 2^-45 M.
//  3. The reference rounds twice in double: X1 = RN64(a + B), X = RN64(X1 + c),
//     |X - T| <= 2^-53 (|a + B| + |X1 + c|) <= 2^-51 M.  Hence
//     |X - (s + t)| <= D with D = 2^-45 M + 2^-51 M < 2^-44 M.
//  4. eb = RN32(RN32(|a| + |c| + ...) * 2^-42) >= 2^-42 M (1 - 2u) (the scaling
//     by a power of two is exact).  RN32(t + eb) rounds t + eb once:
//     RN32(t + eb) >= t + eb - u(|t| + eb) >= t + D, because |t| <= 4uM and
//     eb (1 - u) - u|t| >= 2^-42 M (1 - 3u) - 4u^2 M > 2^-44 M >= D.
//     Likewise RN32(t - eb) <= t - D.
//  5. So s + RN32(t - eb) <= X <= s + RN32(t + eb) as real numbers, and by
//     monotonicity of RN32, hm = RN32(s + RN32(t - eb)) <= RN32(X) <=
//     hp = RN32(s + RN32(t + eb)).  hp == hm proves RN32(X) == hp: the
//     reference's double result rounds to that float.  The margin is a factor
//     4 or more (eb >= 4D), so the check declines only within a few 2^-42 M of
//     a float rounding boundary.
//
// All float arithmetic goes through __f*_rn intrinsics so nvcc never contracts
// it into FMAs (the library is also built with -fmad=false); the only FMAs are
// the explicit ones of the division.
#pragma once
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

namespace abea {

#define ABEA_FROM_D 0u
#define ABEA_FROM_U 1u
#define ABEA_FROM_L 2u

constexpr float kLogInvSqrt2Pi = -0.918938f;           // GPU/align_cuda.cl:66
constexpr float kErrScale = 2.2737367544323206e-13f;   // 2^-42
constexpr float kDivHi = 1.0000009536743164f;          // 1 + 2^-20
constexpr float kDivLo = 0.99999904632568359f;         // 1 - 2^-20
constexpr float kTiny = 7.8886090522101181e-31f;       // 2^-100

struct CellConsts {
    float step_h, step_l, stay_h, stay_l, skip_h, skip_l;
    double lp_step, lp_stay, lp_skip;
};

// Division n/sd rounded to nearest, from the precomputed rsd = RN(1/sd): one
// correction step in the style of Markstein (IBM J. Res. Dev. 34, 1990) gives
// q0 + delta with |delta - (n/sd - q0)| < 2^-21 |delta|; the two roundings of
// q0 + delta*(1 +- 2^-20) bracket RN(n/sd), so equal results prove it.
__device__ __forceinline__ float div_fast(float n, float sd, float rsd, bool& ok) {
    float q0 = __fmul_rn(n, rsd);
    float r = __fmaf_rn(-q0, sd, n);
    float d = __fmul_rn(r, rsd);
    float hp = __fmaf_rn(d, kDivHi, q0);
    float hm = __fmaf_rn(d, kDivLo, q0);
    ok = (hp == hm) && (fabsf(q0) >= kTiny || n == 0.0f);
    return hp;
}

// Division n/sd rounded to nearest from rsd = RN(1/sd): q0 = RN(n*rsd), the
// exact remainder r = n - sd*q0 by FMA, and q = RN(q0 + r*rsd), which is RN(n/sd)
// by Markstein's theorem (IBM J. Res. Dev. 34, 1990; Cornea-Hasegan, Golliver
// and Markstein, ARITH-14, 1999) when rsd is the correctly rounded reciprocal
// and nothing under- or overflows.  ok = false outside 2^-100 <= |q0| <= 2^100
// (n = 0 excepted) or when rsd is not a finite positive number.
constexpr float kHuge = 1.2676506002282294e30f;  // 2^100
__device__ __forceinline__ float div_rn(float n, float sd, float rsd, bool& ok) {
    const float q0 = __fmul_rn(n, rsd);
    const float r = __fmaf_rn(-q0, sd, n);
    const float q = __fmaf_rn(r, rsd, q0);
    const float aq = fabsf(q0);
    ok = ((aq >= kTiny && aq <= kHuge) || n == 0.0f) && rsd > 0.0f && rsd < INFINITY;
    return q;
}

// log_normal_pdf of the reference in its operation order
// (GPU/align_cuda.cl:68-75, 511-528): a = (x - mean)/stdv;
// lp = (log_inv_sqrt_2pi - log_stdv) + ((-0.5f*a)*a); k1 is the first bracket,
// precomputed per k-mer with the same rounding.
__device__ __forceinline__ float emission_fast(float x, float gm, float sd, float rsd, float k1, bool& ok) {
    float a = div_fast(__fsub_rn(x, gm), sd, rsd, ok);
    float t = __fmul_rn(__fmul_rn(-0.5f, a), a);
    return __fadd_rn(k1, t);
}

// emission_fast with div_rn: no bracket, one FMA fewer.
__device__ __forceinline__ float emission_rn(float x, float gm, float sd, float rsd, float k1, bool& ok) {
    float a = div_rn(__fsub_rn(x, gm), sd, rsd, ok);
    float t = __fmul_rn(__fmul_rn(-0.5f, a), a);
    return __fadd_rn(k1, t);
}

__device__ __forceinline__ float emission_ieee(float x, float gm, float sd, float k1) {
    float a = __fdiv_rn(__fsub_rn(x, gm), sd);
    float t = __fmul_rn(__fmul_rn(-0.5f, a), a);
    return __fadd_rn(k1, t);
}

// RN32(RN64(RN64(a + (bh+bl)) + c)) for finite a and c, or ok = false.
// p + q = c + bh by TwoSum (Knuth; no precondition), s + e = a + p by Fast2Sum,
// exact when |a| >= |p| (checked: fails only in a read's first bands).
__device__ __forceinline__ float exact_sum(float a, float bh, float bl, float c, bool& ok) {
    const float p = __fadd_rn(c, bh);
    const float bv = __fsub_rn(p, c);
    const float q = __fadd_rn(__fsub_rn(c, __fsub_rn(p, bv)), __fsub_rn(bh, bv));
    const float w = __fadd_rn(q, bl);
    const float s = __fadd_rn(a, p);
    const float e = __fsub_rn(p, __fsub_rn(s, a));
    const float t = __fadd_rn(e, w);
    const float eb = __fmul_rn(__fadd_rn(__fadd_rn(fabsf(a), fabsf(c)), fabsf(bh)), kErrScale);
    const float hp = __fadd_rn(s, __fadd_rn(t, eb));
    const float hm = __fadd_rn(s, __fsub_rn(t, eb));
    ok = (hp == hm) && (fabsf(a) >= fabsf(p));
    return hp;
}

// The skip candidate RN32(RN64(a + B)) for float a and double B = bh + bl + r:
// Fast2Sum gives s + e = a + bh exactly when |a| >= |bh|, the exact sum lies
// within 2^-47 (|a| + |bh|) of s + (e + bl) (RN64's own rounding included), and
// equal roundings of the bracket +-eb, eb = 2^-42 (|a| + |bh|), prove the result
// as in exact_sum.  a = -inf gives -inf (proven); otherwise ok = false when not
// proven, which happens only while |a| < |bh| (a read's first bands).
//
// a = -inf (a cell outside the band, or not reached): the error terms are taken
// from ac = max(a, -FLT_MAX), which equals a for every finite a; s = a + bh is
// -inf, so hp = hm = -inf and the proof holds without a test of a.
__device__ __forceinline__ float exact_skip(float a, float bh, float bl, bool& ok) {
    const float ac = fmaxf(a, -FLT_MAX);
    const float s = __fadd_rn(a, bh);
    const float sc = __fadd_rn(ac, bh);
    const float e = __fsub_rn(bh, __fsub_rn(sc, ac));
    const float t = __fadd_rn(e, bl);
    const float eb = __fmul_rn(__fadd_rn(fabsf(ac), fabsf(bh)), kErrScale);
    const float hp = __fadd_rn(s, __fadd_rn(t, eb));
    const float hm = __fadd_rn(s, __fsub_rn(t, eb));
    ok = (hp == hm) && (fabsf(a) >= fabsf(bh));
    return hp;
}

// max(best_du, l) with L winning ties (GPU/align_cuda.cl:536-542); all three
// candidates -inf resolve to -inf, FROM_L.
__device__ __forceinline__ float pick_l(float best_du, uint32_t from_du, float l, uint32_t& from) {
    const float best = l > best_du ? l : best_du;
    from = (best == l) ? ABEA_FROM_L : from_du;
    return best;
}

// exact_sum that also accepts a = -inf (result -inf, exact for finite c).
__device__ __forceinline__ float exact_sum_inf(float a, float bh, float bl, float c, bool& ok) {
    bool ok1;
    float v = exact_sum(a, bh, bl, c, ok1);
    bool a_inf = a == -INFINITY;
    ok = ok1 || (a_inf && fabsf(c) < INFINITY);
    return a_inf ? -INFINITY : v;
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

// Emission-side half of exact_sum: p + q = em + bh by TwoSum, w = q + bl.
struct EmSplit {
    float p, w;
};
__device__ __forceinline__ EmSplit em_split(float em, float bh, float bl) {
    EmSplit r;
    r.p = __fadd_rn(em, bh);
    const float bv = __fsub_rn(r.p, em);
    const float q = __fadd_rn(__fsub_rn(em, __fsub_rn(r.p, bv)), __fsub_rn(bh, bv));
    r.w = __fadd_rn(q, bl);
    return r;
}

// Score-side half: RN32(RN64(RN64(a + B) + em)) from a and the emission split;
// a = -inf gives -inf.  `mag` = |em| + |bh|: NaN or +inf (a division that was not
// proven, or an infinite emission) make the candidate unproven whatever a is.
// ok = false when not proven.  As in exact_skip, the error terms come from
// ac = max(a, -FLT_MAX): for a = -inf, s = -inf gives hp = hm = -inf when mag
// is finite, and NaN (not proven) when it is not.
__device__ __forceinline__ float exact_from_split(float a, EmSplit sp, float mag, bool& ok) {
    const float ac = fmaxf(a, -FLT_MAX);
    const float s = __fadd_rn(a, sp.p);
    const float sc = __fadd_rn(ac, sp.p);
    const float e = __fsub_rn(sp.p, __fsub_rn(sc, ac));
    const float t = __fadd_rn(e, sp.w);
    const float eb = __fmul_rn(__fadd_rn(fabsf(ac), mag), kErrScale);
    const float hp = __fadd_rn(s, __fadd_rn(t, eb));
    const float hm = __fadd_rn(s, __fsub_rn(t, eb));
    ok = (hp == hm) && (fabsf(a) >= fabsf(sp.p));
    return hp;
}

// The next band's emission of a slot and the split for its up candidate; the
// exact diagonal candidate once its diagonal score is known.
struct NextCell {
    float em;         // emission
    EmSplit su;       // em + stay, for u
    float d;          // exact diagonal candidate
    bool ok;          // division and d proven
};
__device__ __forceinline__ NextCell next_cell(float diag, float x, float gm, float sd, float rsd, float k1,
                                              const CellConsts& c) {
    NextCell n;
    bool div_ok, okd;
    n.em = emission_fast(x, gm, sd, rsd, k1, div_ok);
    const EmSplit sd_ = em_split(n.em, c.step_h, c.step_l);
    n.d = exact_from_split(diag, sd_, __fadd_rn(fabsf(n.em), fabsf(c.step_h)), okd);
    n.su = em_split(n.em, c.stay_h, c.stay_l);
    n.ok = div_ok && okd;
    return n;
}

// The up candidate from the previous band's score of the same slot.
__device__ __forceinline__ float cell_u(float up, const NextCell& n, const CellConsts& c, bool& ok) {
    return exact_from_split(up, n.su, __fadd_rn(fabsf(n.em), fabsf(c.stay_h)), ok);
}

// max(d, u) with U winning ties (no L candidate).
__device__ __forceinline__ float pick_du(float d, float u, uint32_t& from) {
    float best = u > d ? u : d;
    from = (best == u) ? ABEA_FROM_U : ABEA_FROM_D;
    return best;
}

// The reference's arithmetic verbatim (IEEE division, FP64 adds): the fallback
// when an exactness proof does not go through.
static __device__ __forceinline__ float cell_slow(float diag, float up, float left, float x, float gm, float sd, float k1,
                                        const CellConsts c, uint32_t& from) {
    float em = emission_ieee(x, gm, sd, k1);
    float d = __double2float_rn(__dadd_rn(__dadd_rn((double)diag, c.lp_step), (double)em));
    float u = __double2float_rn(__dadd_rn(__dadd_rn((double)up, c.lp_stay), (double)em));
    float l = __double2float_rn(__dadd_rn((double)left, c.lp_skip));
    return pick(d, u, l, from);
}

}  // namespace abea
