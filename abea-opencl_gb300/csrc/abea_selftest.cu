// abea_selftest.cu — on-device self-test of the exact FP32 arithmetic that the
// fill kernels use in place of the reference's FP64 adds and IEEE division.
//
// For pseudo-random and adversarial inputs it compares
//   div_fast(n, sd, RN(1/sd))          with __fdiv_rn(n, sd)
//   div_rn(n, sd, RN(1/sd))            with __fdiv_rn(n, sd)
//   exact_sum(a, bh, bl, c)            with RN32(RN64(RN64(a + B) + c))
//   exact_skip(a, bh, bl)              with RN32(RN64(a + B))
// and counts the cases where the fast routine claims success but differs
// (must be zero) and the cases where it declines (the kernels then fall back).
// Adversarial sums are built around float rounding midpoints, where double
// rounding can differ from a single rounding.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/abea.h"
#include "abea_cell.cuh"

namespace abea {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__device__ __forceinline__ float unit(uint64_t& s) {  // [0, 1)
    s = mix64(s + 0x9e3779b97f4a7c15ull);
    return (float)(s >> 40) * (1.0f / 16777216.0f);
}

// counters: [0] div claimed-but-wrong, [1] div declined, [2] sum claimed-but-wrong,
// [3] sum declined, [4] cases
__global__ void selftest_kernel(uint64_t seed, int iters, unsigned long long* counters) {
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t s = mix64(seed ^ (tid * 0x632be59bd9b4e019ull));
    unsigned long long c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    for (int it = 0; it < iters; ++it) {
        // ---- division: nanopore-like and wide-range operands
        float sd = (it & 1) ? 0.3f + 4.0f * unit(s) : __int_as_float(0x3f800000 | (int)(unit(s) * 8388607.0f));
        float n = (unit(s) - 0.5f) * ((it & 2) ? 200.0f : 1e-3f + 40.0f * unit(s));
        if (it % 7 == 0) n = __int_as_float((__float_as_int(n) & 0x807fffff) | ((100 + (int)(unit(s) * 50.0f)) << 23));
        bool ok;
        float q = div_fast(n, sd, __frcp_rn(sd), ok);
        float ref = __fdiv_rn(n, sd);
        if (ok && __float_as_int(q) != __float_as_int(ref)) ++c0;
        if (!ok) ++c1;
        // Markstein's form (div_rn): counted with the division
        float q2 = div_rn(n, sd, __frcp_rn(sd), ok);
        if (ok && __float_as_int(q2) != __float_as_int(ref)) ++c0;
        if (!ok) ++c1;
        // ---- sums: a + B + c with B a double constant
        double B;
        float a, c;
        if (it & 1) {
            B = -(0.1 + 30.0 * (double)unit(s)) - (double)unit(s) * 1e-9;
            a = -(float)(10000.0 * (double)unit(s));
            c = -(0.5f + 20.0f * unit(s));
        } else {
            // Aim the exact sum at a float rounding midpoint: B has no bits below
            // 2^-30, c is chosen so that a + B + c lands next to the midpoint m
            // of RN32(a + B + c0) and its neighbour.
            B = -(double)(33554432ull + (uint64_t)(unit(s) * 3.2e10f)) * 9.313225746154785e-10;  // k * 2^-30
            a = -(float)(20000.0 * (double)unit(s)) - 1.0f;
            float c0 = -(0.5f + 20.0f * unit(s));
            float s1 = __double2float_rn((double)a + B + (double)c0);
            float nb = nextafterf(s1, (unit(s) < 0.5f) ? 0.0f : -INFINITY);
            double m = 0.5 * ((double)s1 + (double)nb);
            c = __double2float_rn(m - (double)a - B);
        }
        float bh = (float)B, bl = (float)(B - (double)bh);
        float v = exact_sum(a, bh, bl, c, ok);
        float r = __double2float_rn(__dadd_rn(__dadd_rn((double)a, B), (double)c));
        if (ok && __float_as_int(v) != __float_as_int(r)) ++c2;
        if (!ok) ++c3;
        // ---- the skip candidate a + B: f5c's lp_skip or the random B; random a,
        // or a aimed so that a + B lands next to a float rounding midpoint
        {
            const double bs = (it & 4) ? -23.025850929940457 : B;
            float as;
            if (it & 8) {
                as = -(float)(50000.0 * (double)unit(s)) - 31.0f;
            } else {
                const float a0 = -(float)(20000.0 * (double)unit(s)) - 31.0f;
                const float s1 = __double2float_rn((double)a0 + bs);
                const float nb = nextafterf(s1, (unit(s) < 0.5f) ? 0.0f : -INFINITY);
                const double m = 0.5 * ((double)s1 + (double)nb);
                as = __double2float_rn(m - bs);
            }
            const float bhs = (float)bs, bls = (float)(bs - (double)bhs);
            const float vs = exact_skip(as, bhs, bls, ok);
            const float rs = __double2float_rn(__dadd_rn((double)as, bs));
            if (ok && __float_as_int(vs) != __float_as_int(rs)) ++c2;
            if (!ok) ++c3;
        }
        // ---- a = -inf (a cell outside the band): -inf and proven for a finite
        // emission; not proven when the emission's division was not (mag = NaN)
        {
            bool o1, o2, o3;
            const float v1 = exact_skip(-INFINITY, bh, bl, o1);
            const EmSplit sp = em_split(c, bh, bl);
            const float v2 = exact_from_split(-INFINITY, sp, __fadd_rn(fabsf(c), fabsf(bh)), o2);
            exact_from_split(-INFINITY, sp, __int_as_float(0x7fc00000), o3);
            if (!o1 || v1 != -INFINITY || !o2 || v2 != -INFINITY || o3) ++c2;
        }
    }
    atomicAdd(&counters[0], c0);
    atomicAdd(&counters[1], c1);
    atomicAdd(&counters[2], c2);
    atomicAdd(&counters[3], c3);
    atomicAdd(&counters[4], (unsigned long long)iters);  // per kind (the sums count two per case)
}

}  // namespace abea

// Runs the self-test on the current device: `cases` random cases of each kind.
// out[0..4]: division wrong, division declined, sum wrong, sum declined, cases.
extern "C" abea_status_t abea_selftest_arith(int64_t cases, uint64_t seed, int64_t* out) {
    if (!out || cases <= 0) return ABEA_ERR_INVALID_ARG;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long) * 5) != cudaSuccess) return ABEA_ERR_OUT_OF_MEMORY;
    cudaMemset(d, 0, sizeof(unsigned long long) * 5);
    const int threads = 256, blocks = 1216;
    int iters = (int)std::max<int64_t>(1, cases / (threads * (int64_t)blocks));
    abea::selftest_kernel<<<blocks, threads>>>(seed, iters, d);
    unsigned long long h[5] = {0, 0, 0, 0, 0};
    cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return ABEA_ERR_CUDA;
    for (int i = 0; i < 5; ++i) out[i] = (int64_t)h[i];
    return ABEA_OK;
}
