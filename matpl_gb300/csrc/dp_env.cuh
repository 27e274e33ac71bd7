// Environment-matrix row of one neighbor slot and its derivative, shared by the DP kernels
// (src/model/dp_dp.py:217-302: switching function s(r), Ri = (s, s x/r, s y/r, s z/r),
// normalised (Ri - davg) / dstd, Ri_d = -dfeat / dstd).
#pragma once
#include <cuda_runtime.h>

namespace matpl {
namespace dp {

template <typename T>
__device__ __forceinline__ void switch_fn(T R, T rmin, T rmax, T &s, T &ds) {
    s = T(0);
    ds = T(0);
    if (R > T(0) && R < rmin) {
        s = T(1) / R;
        ds = -T(1) / (R * R);
    } else if (R > rmin && R < rmax) {
        const T u = (R - rmin) / (rmax - rmin);
        const T q = T(-6) * u * u + T(15) * u - T(10);
        const T poly = u * u * u * q + T(1);
        const T dpoly = (T(3) * u * u * q + u * u * u * (T(-12) * u + T(15))) / (rmax - rmin);
        s = poly / R;
        ds = dpoly / R - poly / (R * R);
    }
}

// Normalised Ri row (4 values) of one slot (dp_dp.py:241-297).
template <typename T>
__device__ __forceinline__ void env_row(T R, T x, T y, T z, T rmin, T rmax, const T *avg,
                                        const T *sd, T rh[4]) {
    T s, ds;
    switch_fn(R, rmin, rmax, s, ds);
    const bool mask = fabs((double)R) > 1e-5;
    const T inv = mask ? T(1) / R : T(0);
    rh[0] = (s - avg[0]) / sd[0];
    rh[1] = ((mask ? s * x * inv : T(0)) - avg[1]) / sd[1];
    rh[2] = ((mask ? s * y * inv : T(0)) - avg[2]) / sd[2];
    rh[3] = ((mask ? s * z * inv : T(0)) - avg[3]) / sd[3];
}

// f_a = sum_c g[c] * Ri_d[c][a] with Ri_d = -dfeat / dstd (dp_dp.py:266-299).
template <typename T>
__device__ __forceinline__ void contract_rid(T R, T x, T y, T z, T rmin, T rmax, const T *sd,
                                             const T g[4], T f[3]) {
    T s, ds;
    switch_fn(R, rmin, rmax, s, ds);
    const bool mask = fabs((double)R) > 1e-5;
    f[0] = f[1] = f[2] = T(0);
    if (!mask) return;
    const T inv = T(1) / R;
    const T common = (ds - s * inv) * inv * inv;
    const T xyz[3] = {x, y, z};
    const T g0 = g[0] / sd[0], g1 = g[1] / sd[1], g2 = g[2] / sd[2], g3 = g[3] / sd[3];
    // sum_{c>=1} g_c * common * xyz[c-1]
    const T cg = common * (g1 * x + g2 * y + g3 * z);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T gd = (a == 0 ? g1 : (a == 1 ? g2 : g3)) * s * inv;
        f[a] = -(g0 * ds * xyz[a] * inv + cg * xyz[a] + gd);
    }
}

// Directional derivative of the normalised row along a pair-vector displacement u:
// rd[c] = sum_a Ri_d[c][a] u[a], with the same Ri_d as contract_rid (so that
// sum_c g[c] rd[c] = f . u for the f that contract_rid returns).
template <typename T>
__device__ __forceinline__ void rid_dir(T R, T x, T y, T z, T rmin, T rmax, const T *sd,
                                        const T u[3], T rd[4]) {
    T s, ds;
    switch_fn(R, rmin, rmax, s, ds);
    rd[0] = rd[1] = rd[2] = rd[3] = T(0);
    if (!(fabs((double)R) > 1e-5)) return;
    const T inv = T(1) / R;
    const T common = (ds - s * inv) * inv * inv;
    const T xu = x * u[0] + y * u[1] + z * u[2];
    rd[0] = -(ds * inv * xu) / sd[0];
    rd[1] = -(common * x * xu + s * inv * u[0]) / sd[1];
    rd[2] = -(common * y * xu + s * inv * u[1]) / sd[2];
    rd[3] = -(common * z * xu + s * inv * u[2]) / sd[3];
}

}  // namespace dp
}  // namespace matpl
