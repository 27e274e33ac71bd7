// NEP descriptor math shared by the fused evaluation (nep_eval.cu) and the training
// operators (nep_train.cu): the Chebyshev radial basis f_k(r) with its derivative
// (cal_fk, src/model/nep_net.py:691-715), the 24 real harmonic polynomials b_lm of the unit
// vector with their gradients (cal_blm_ij, nep_net.py:816-838) and the 3-/4-/5-body constants
// (nep_net.py:230-242).
#pragma once
#include "common.cuh"

namespace matpl {
namespace {

// descriptor constants of nep_net.py:230-242 (C3B with the factor 2 of m > 0 folded in)
__constant__ double kC3B[24] = {
    0.238732414637843, 0.238732414637843, 0.238732414637843,
    0.099471839432435, 1.1936620731892151, 1.1936620731892151, 0.2984155182973038,
    0.2984155182973038,
    0.139260575205408, 0.20889086280811264, 0.20889086280811264, 2.088908628081126,
    2.088908628081126, 0.34815143801352105, 0.34815143801352105,
    0.01119058193614889, 0.44762327744595565, 0.44762327744595565, 0.22381163872297782,
    0.22381163872297782, 3.1333629421216895, 3.1333629421216895, 0.3916703677652112,
    0.3916703677652112};
__constant__ double kC4B[5] = {-0.007499480826664, -0.134990654879954, 0.067495327439977,
                               0.404971964639861, -0.809943929279723};
__constant__ double kC5B[3] = {0.026596810706114, 0.053193621412227, 0.026596810706114};

// l of each lm (l = 1..4 -> 0..3) and the first lm of each l
__host__ __device__ constexpr int l_of(int lm) { return lm < 3 ? 0 : (lm < 8 ? 1 : (lm < 15 ? 2 : 3)); }

// descriptor constants in FP32 for the FP32 kernel (the same values as kC3B / kC4B / kC5B)
__constant__ float kC3Bf[24] = {
    0.238732414637843f, 0.238732414637843f, 0.238732414637843f,
    0.099471839432435f, 1.1936620731892151f, 1.1936620731892151f, 0.2984155182973038f,
    0.2984155182973038f,
    0.139260575205408f, 0.20889086280811264f, 0.20889086280811264f, 2.088908628081126f,
    2.088908628081126f, 0.34815143801352105f, 0.34815143801352105f,
    0.01119058193614889f, 0.44762327744595565f, 0.44762327744595565f, 0.22381163872297782f,
    0.22381163872297782f, 3.1333629421216895f, 3.1333629421216895f, 0.3916703677652112f,
    0.3916703677652112f};
__constant__ float kC4Bf[5] = {-0.007499480826664f, -0.134990654879954f, 0.067495327439977f,
                               0.404971964639861f, -0.809943929279723f};
__constant__ float kC5Bf[3] = {0.026596810706114f, 0.053193621412227f, 0.026596810706114f};

template <typename T> __device__ __forceinline__ T C3(int i);
template <> __device__ __forceinline__ float C3<float>(int i) { return kC3Bf[i]; }
template <> __device__ __forceinline__ double C3<double>(int i) { return kC3B[i]; }
template <typename T> __device__ __forceinline__ T C4(int i);
template <> __device__ __forceinline__ float C4<float>(int i) { return kC4Bf[i]; }
template <> __device__ __forceinline__ double C4<double>(int i) { return kC4B[i]; }
template <typename T> __device__ __forceinline__ T C5(int i);
template <> __device__ __forceinline__ float C5<float>(int i) { return kC5Bf[i]; }
template <> __device__ __forceinline__ double C5<double>(int i) { return kC5B[i]; }

template <typename T> __device__ __forceinline__ void sincospi_t(T x, T *s, T *c);
template <> __device__ __forceinline__ void sincospi_t<float>(float x, float *s, float *c) {
    __sincosf(x * 3.14159265358979323846f, s, c);   // x in [0, 1): fast intrinsic suffices
}
template <> __device__ __forceinline__ void sincospi_t<double>(double x, double *s, double *c) {
    sincospi(x, s, c);
}

// f_k(r) and df_k/dr, k < K (zero at and beyond rc)
template <typename T, int KM>
__device__ __forceinline__ void basis(T r, T rc, T rcinv, int K, T *f, T *df) {
    if (!(r < rc)) {
#pragma unroll
        for (int k = 0; k < KM; ++k) f[k] = df[k] = T(0);
        return;
    }
    T sn, cs;
    sincospi_t<T>(r * rcinv, &sn, &cs);
    const T fc = T(0.5) * cs + T(0.5);
    const T dfc = T(-0.5) * T(3.14159265358979323846) * rcinv * sn;
    const T u = r * rcinv - T(1);
    const T x = T(2) * u * u - T(1);
    const T dx = T(4) * u * rcinv;
    T t0 = T(1), t1 = x, d0 = T(0), d1 = T(1);
    f[0] = fc;
    df[0] = dfc;
    if (KM > 1) {
        f[1] = T(0.5) * (x + T(1)) * fc;
        df[1] = T(0.5) * (dx * fc + (x + T(1)) * dfc);
    }
#pragma unroll
    for (int k = 2; k < KM; ++k) {
        const T t2 = T(2) * x * t1 - t0;
        const T d2 = T(2) * t1 + T(2) * x * d1 - d0;
        f[k] = k < K ? T(0.5) * (t2 + T(1)) * fc : T(0);
        df[k] = k < K ? T(0.5) * (d2 * dx * fc + (t2 + T(1)) * dfc) : T(0);
        t0 = t1; t1 = t2; d0 = d1; d1 = d2;
    }
}

// b_lm of the unit vector (x, y, z) and its gradient in (x, y, z) taken as independent
template <typename T>
__device__ __forceinline__ void harmonic(int lm, T x, T y, T z, T &b, T &gx, T &gy, T &gz) {
    const T x2 = x * x, y2 = y * y, z2 = z * z, d = x2 - y2;
    switch (lm) {
    case 0: b = z; gx = 0; gy = 0; gz = 1; break;
    case 1: b = x; gx = 1; gy = 0; gz = 0; break;
    case 2: b = y; gx = 0; gy = 1; gz = 0; break;
    case 3: b = T(3) * z2 - T(1); gx = 0; gy = 0; gz = T(6) * z; break;
    case 4: b = x * z; gx = z; gy = 0; gz = x; break;
    case 5: b = y * z; gx = 0; gy = z; gz = y; break;
    case 6: b = d; gx = T(2) * x; gy = T(-2) * y; gz = 0; break;
    case 7: b = T(2) * x * y; gx = T(2) * y; gy = T(2) * x; gz = 0; break;
    case 8: b = (T(5) * z2 - T(3)) * z; gx = 0; gy = 0; gz = T(15) * z2 - T(3); break;
    case 9: b = (T(5) * z2 - T(1)) * x; gx = T(5) * z2 - T(1); gy = 0; gz = T(10) * x * z; break;
    case 10: b = (T(5) * z2 - T(1)) * y; gx = 0; gy = T(5) * z2 - T(1); gz = T(10) * y * z; break;
    case 11: b = d * z; gx = T(2) * x * z; gy = T(-2) * y * z; gz = d; break;
    case 12: b = T(2) * x * y * z; gx = T(2) * y * z; gy = T(2) * x * z; gz = T(2) * x * y; break;
    case 13: b = (x2 - T(3) * y2) * x; gx = T(3) * x2 - T(3) * y2; gy = T(-6) * x * y; gz = 0; break;
    case 14: b = (T(3) * x2 - y2) * y; gx = T(6) * x * y; gy = T(3) * x2 - T(3) * y2; gz = 0; break;
    case 15: b = (T(35) * z2 - T(30)) * z2 + T(3); gx = 0; gy = 0;
             gz = (T(140) * z2 - T(60)) * z; break;
    case 16: b = (T(7) * z2 - T(3)) * x * z; gx = (T(7) * z2 - T(3)) * z; gy = 0;
             gz = (T(21) * z2 - T(3)) * x; break;
    case 17: b = (T(7) * z2 - T(3)) * y * z; gx = 0; gy = (T(7) * z2 - T(3)) * z;
             gz = (T(21) * z2 - T(3)) * y; break;
    case 18: b = (T(7) * z2 - T(1)) * d; gx = T(2) * x * (T(7) * z2 - T(1));
             gy = T(-2) * y * (T(7) * z2 - T(1)); gz = T(14) * z * d; break;
    case 19: b = (T(7) * z2 - T(1)) * x * y * T(2); gx = T(2) * y * (T(7) * z2 - T(1));
             gy = T(2) * x * (T(7) * z2 - T(1)); gz = T(28) * x * y * z; break;
    case 20: b = (x2 - T(3) * y2) * x * z; gx = (T(3) * x2 - T(3) * y2) * z;
             gy = T(-6) * x * y * z; gz = (x2 - T(3) * y2) * x; break;
    case 21: b = (T(3) * x2 - y2) * y * z; gx = T(6) * x * y * z;
             gy = (T(3) * x2 - T(3) * y2) * z; gz = (T(3) * x2 - y2) * y; break;
    case 22: b = d * d - T(4) * x2 * y2; gx = T(4) * x * d - T(8) * x * y2;
             gy = T(-4) * y * d - T(8) * x2 * y; gz = 0; break;
    default: b = T(4) * x * y * d; gx = T(12) * x2 * y - T(4) * y2 * y;
             gy = T(4) * x2 * x - T(12) * x * y2; gz = 0; break;
    }
}

}  // namespace
}  // namespace matpl
