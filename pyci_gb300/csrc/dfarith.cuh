// Double-float arithmetic shared by the implicit-form products (fcix.cu,
// docx.cu): FP64-accurate sums of FP32 high/low products in FP32
// instructions (GB300's FP64 rate is a small fraction of its FP32 rate).
#pragma once

#include <cuda_runtime.h>

namespace pyci_gpu {

// (s, c) += p with TwoSum: s the running sum, c the accumulated errors.
__device__ __forceinline__ void df_two_sum(float &s, float &c, float p) {
    const float u = __fadd_rn(s, p);
    const float z = __fadd_rn(u, -s);
    const float d = __fadd_rn(__fadd_rn(s, -__fadd_rn(u, -z)), __fadd_rn(p, -z));
    s = u;
    c = __fadd_rn(c, d);
}

// Term (vh + vl)(xh + xl) added to (s, c): p = fl(vh xh), its exact error
// fma(vh, xh, -p), the small products vh xl + vl xh in FP32, p added with
// TwoSum.
template<int K>
__device__ __forceinline__ void df_term(float vh, float vl, const float xh[K], const float xl[K], float s[K],
                                        float c[K]) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float p = __fmul_rn(vh, xh[k]);
        const float err = fmaf(vh, xh[k], -p);
        const float t = fmaf(vh, xl[k], fmaf(vl, xh[k], err));
        df_two_sum(s[k], c[k], p);
        c[k] = __fadd_rn(c[k], t);
    }
}

// One entry with value (vh, vl) times the x row at xr: FP32 (MODE 0, x
// rows of K floats, accumulation in acc) or double-float (MODE 2, x rows of
// K high parts then K low parts, accumulation in (acc, cc)).
template<int MODE, int K>
__device__ __forceinline__ void df_acc(const float *xr, float vh, float vl, float acc[K], float cc[K]) {
    if constexpr (MODE == 0) {
        float xv[K];
        if constexpr (K % 4 == 0) {
#pragma unroll
            for (int v = 0; v < K / 4; ++v) {
                const float4 q = reinterpret_cast<const float4 *>(xr)[v];
                xv[4 * v] = q.x, xv[4 * v + 1] = q.y, xv[4 * v + 2] = q.z, xv[4 * v + 3] = q.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k)
                xv[k] = xr[k];
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
            acc[k] = fmaf(vh, xv[k], acc[k]);
    } else {
        float xh[K], xl[K];
        if constexpr (K == 4) {
            const float4 a = reinterpret_cast<const float4 *>(xr)[0];
            const float4 b = reinterpret_cast<const float4 *>(xr)[1];
            xh[0] = a.x, xh[1] = a.y, xh[2] = a.z, xh[3] = a.w;
            xl[0] = b.x, xl[1] = b.y, xl[2] = b.z, xl[3] = b.w;
        } else if constexpr (K == 2) {
            const float4 a = reinterpret_cast<const float4 *>(xr)[0];
            xh[0] = a.x, xh[1] = a.y, xl[0] = a.z, xl[1] = a.w;
        } else {
            const float2 a = reinterpret_cast<const float2 *>(xr)[0];
            xh[0] = a.x, xl[0] = a.y;
        }
        df_term<K>(vh, vl, xh, xl, acc, cc);
    }
}

} // namespace pyci_gpu
