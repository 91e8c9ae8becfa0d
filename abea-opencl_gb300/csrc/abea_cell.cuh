// abea_cell.cuh — per-cell arithmetic of the banded recurrence.
//
// The reference scores a cell as (GPU/align_cuda.cl:530-542, align_swi.cl:478-488)
//     d = (float)(((double)diag + lp_step) + (double)em)
//     u = (float)(((double)up   + lp_stay) + (double)em)
//     l = (float)( (double)left + lp_skip)
// then keeps the largest with U winning ties over D and L over both.  GB300 runs
// FP64 adds and f32<->f64 conversions at ~1/70 of the FP32 rate, so a cell is
// evaluated in FP32 in three tiers, every tier bit-exact:
//
//  1. fast: the three candidates are approximated in plain FP32 (error < 2^-22
//     relative when no term is positive, which holds for every pore model whose
//     log_inv_sqrt_2pi - log(stdv) is <= 0).  When one candidate beats both others
//     by more than 2^-19 of their magnitude, the reference's comparison outcome
//     is certain and only the winner is evaluated exactly (exact_sum).
//  2. medium: otherwise all three are evaluated with exact_sum and compared.
//  3. slow: if any exact_sum cannot prove its result (or the emission's
//     division cannot), the cell is recomputed with native FP64 and IEEE
//     division, literally as the reference does.
//
// exact_sum(a, B, c) returns RN32(RN64(RN64(a + B) + c)) for floats a, c and a
// double B = bh + bl + r (bh = RN32(B), bl = RN32(B - bh), |r| <= 2^-48|B|):
// Fast2Sum (Dekker 1971) gives p + q = c + bh and s + e = a + p exactly, the
// exact sum a + B + c lies within eb = 2^-42 (|a| + |c| + |bh|) of s + t with
// t = e + (q + bl) (eb also covers the reference's own two double roundings,
// each <= 2^-53 of the same magnitudes), and RN32(s + (t + eb)) ==
// RN32(s + (t - eb)) proves by monotonicity of rounding that the reference's
// double result rounds to that float.
//
// All float arithmetic goes through __f*_rn intrinsics so nvcc never contracts
// it into FMAs (the library is also built with -fmad=false); the only FMAs are
// the explicit ones of the division.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace abea {

#define ABEA_FROM_D 0u
#define ABEA_FROM_U 1u
#define ABEA_FROM_L 2u

constexpr float kLogInvSqrt2Pi = -0.918938f;           // GPU/align_cuda.cl:66
constexpr float kErrScale = 2.2737367544323206e-13f;   // 2^-42
constexpr float kClear = 0.99999809265136719f;         // 1 - 2^-19
constexpr float kDivHi = 1.0000009536743164f;          // 1 + 2^-20
constexpr float kDivLo = 0.99999904632568359f;         // 1 - 2^-20
constexpr float kTiny = 7.8886090522101181e-31f;       // 2^-100

struct CellConsts {
    float step_h, step_l, stay_h, stay_l, skip_h, skip_l;
    float em_floor;  // power of two <= max(|step_h|, |stay_h|): Fast2Sum(em, Bh) precondition
    int nonpos;      // every emission of this read is <= 0 (tier 1 allowed)
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

// log_normal_pdf of the reference in its operation order
// (GPU/align_cuda.cl:68-75, 511-528): a = (x - mean)/stdv;
// lp = (log_inv_sqrt_2pi - log_stdv) + ((-0.5f*a)*a); k1 is the first bracket,
// precomputed per k-mer with the same rounding.
__device__ __forceinline__ float emission_fast(float x, float gm, float sd, float rsd, float k1, bool& ok) {
    float a = div_fast(__fsub_rn(x, gm), sd, rsd, ok);
    float t = __fmul_rn(__fmul_rn(-0.5f, a), a);
    return __fadd_rn(k1, t);
}

__device__ __forceinline__ float emission_ieee(float x, float gm, float sd, float k1) {
    float a = __fdiv_rn(__fsub_rn(x, gm), sd);
    float t = __fmul_rn(__fmul_rn(-0.5f, a), a);
    return __fadd_rn(k1, t);
}

// RN32(RN64(RN64(a + (bh+bl)) + c)) for finite a and c, or ok = false.
// c_ok: Fast2Sum(c, bh) is exact (c == 0 or exponent(c) >= exponent(bh)).
__device__ __forceinline__ float exact_sum(float a, float bh, float bl, float c, bool c_ok, bool& ok) {
    float p = __fadd_rn(c, bh);
    float q = __fsub_rn(bh, __fsub_rn(p, c));
    float w = __fadd_rn(q, bl);
    float s = __fadd_rn(a, p);
    float e = __fsub_rn(p, __fsub_rn(s, a));
    float t = __fadd_rn(e, w);
    float eb = __fmul_rn(__fadd_rn(__fadd_rn(fabsf(a), fabsf(c)), fabsf(bh)), kErrScale);
    float hp = __fadd_rn(s, __fadd_rn(t, eb));
    float hm = __fadd_rn(s, __fsub_rn(t, eb));
    ok = (hp == hm) && (fabsf(a) >= fabsf(p)) && c_ok;
    return hp;
}

// exact_sum that also accepts a = -inf (result -inf, exact for finite c).
__device__ __forceinline__ float exact_sum_inf(float a, float bh, float bl, float c, bool c_ok, bool& ok) {
    bool ok1;
    float v = exact_sum(a, bh, bl, c, c_ok, ok1);
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

// Tier 1.  Returns the cell score; tier = 0 when done, 1 when the medium tier
// must decide, 2 when the slow tier must recompute.
__device__ __forceinline__ float cell_fast(float diag, float up, float left, float x, float gm, float sd,
                                           float rsd, float k1, const CellConsts& c, uint32_t& from,
                                           int& tier, float& em) {
    bool div_ok;
    em = emission_fast(x, gm, sd, rsd, k1, div_ok);
    // approximations, error < 2^-22 of their magnitude when no term is positive
    float dA = __fadd_rn(__fadd_rn(diag, c.step_h), em);
    float uA = __fadd_rn(__fadd_rn(up, c.stay_h), em);
    float lA = __fadd_rn(left, c.skip_h);
    float tD = __fmul_rn(dA, kClear), tU = __fmul_rn(uA, kClear), tL = __fmul_rn(lA, kClear);
    bool winD = (dA > tU) && (dA > tL);
    bool winU = (uA > tD) && (uA > tL);
    bool winL = (lA > tD) && (lA > tU);
    bool all_inf = (diag == -INFINITY) && (up == -INFINITY) && (left == -INFINITY);
    float a = winD ? diag : (winU ? up : left);
    float bh = winD ? c.step_h : (winU ? c.stay_h : c.skip_h);
    float bl = winD ? c.step_l : (winU ? c.stay_l : c.skip_l);
    float cc = winL ? 0.0f : em;
    bool c_ok = winL || (fabsf(em) >= c.em_floor);
    from = winD ? ABEA_FROM_D : (winU ? ABEA_FROM_U : ABEA_FROM_L);
    bool ok;
    float v = exact_sum(a, bh, bl, cc, c_ok, ok);
    bool decided = c.nonpos && (winD || winU || winL);
    tier = all_inf ? 0 : (!div_ok ? 2 : (!decided ? 1 : (ok ? 0 : 2)));
    return all_inf ? -INFINITY : v;
}

// Tier 2: all three candidates exactly, then the reference's comparison.
__device__ __forceinline__ float cell_medium(float diag, float up, float left, float em, const CellConsts& c,
                                             uint32_t& from, bool& ok) {
    bool c_ok = fabsf(em) >= c.em_floor;
    bool okd, oku, okl;
    float d = exact_sum_inf(diag, c.step_h, c.step_l, em, c_ok, okd);
    float u = exact_sum_inf(up, c.stay_h, c.stay_l, em, c_ok, oku);
    float l = exact_sum_inf(left, c.skip_h, c.skip_l, 0.0f, true, okl);
    ok = okd && oku && okl;
    return pick(d, u, l, from);
}

// Tier 3: the reference's arithmetic verbatim (IEEE division, FP64 adds).
__device__ __forceinline__ float cell_slow(float diag, float up, float left, float x, float gm, float sd,
                                           float k1, const CellConsts& c, uint32_t& from) {
    float em = emission_ieee(x, gm, sd, k1);
    float d = __double2float_rn(__dadd_rn(__dadd_rn((double)diag, c.lp_step), (double)em));
    float u = __double2float_rn(__dadd_rn(__dadd_rn((double)up, c.lp_stay), (double)em));
    float l = __double2float_rn(__dadd_rn((double)left, c.lp_skip));
    return pick(d, u, l, from);
}

}  // namespace abea
