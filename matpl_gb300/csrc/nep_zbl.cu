// NEP ZBL term: the universal screened-Coulomb pair energy NEP adds below an outer cutoff
// zbl (src/model/nep_net.py:399-408 gate, calculate_zbl :916-955, cal_zbl :957-991).
//
// For every angular-list slot of atom i with neighbor j (NL >= 0) and 0 < r <= zbl:
//   x   = r * s_ij * 2.134563,         s_ij = Z_i^0.23 + Z_j^0.23
//   phi = sum_k a_k exp(-b_k x)          (the four-term universal screening function)
//   fc  = 1 (r < zbl/2), 0.5 + 0.5 cos(pi/(zbl/2) (r - zbl/2)) (zbl/2 <= r <= zbl)
//   e   = c_ij * phi * fc / r,          c_ij = K Z_i Z_j
// and E_i += e / 2.  The element factors s_ij and c_ij come from the host in the precision the
// reference forms them in (torch's default dtype on the int64 element numbers); the rest is
// computed in the kernel's dtype in the reference's operation order.  Forces and virial:
// f = (1/2) de/dr (x, y, z) / r is dE/d(r_ij) of the slot (the reference's autograd on the r
// column contracted with d r / d(x, y, z)); F_i += f, F_j -= f, virial[image(i)] -= f (x) r.
// One warp per atom, lanes over slots; E and virial sums in FP64.  Pairs are rare (r below
// ~2 A), so every update is an atomic add.
#include <algorithm>

#include "common.cuh"

namespace matpl {
namespace {

__constant__ double kZblA[4] = {0.18175, 0.50986, 0.28022, 0.02817};
__constant__ double kZblB[4] = {3.1998, 0.94229, 0.4029, 0.20162};

template <typename T> __device__ __forceinline__ T zexp(T v);
template <> __device__ __forceinline__ double zexp<double>(double v) { return exp(v); }
template <> __device__ __forceinline__ float zexp<float>(float v) { return expf(v); }
template <typename T> __device__ __forceinline__ void zsincos(T v, T *s, T *c);
template <> __device__ __forceinline__ void zsincos<double>(double v, double *s, double *c) {
    sincos(v, s, c);
}
template <> __device__ __forceinline__ void zsincos<float>(float v, float *s, float *c) {
    sincosf(v, s, c);
}

template <typename T, typename TI>
__global__ void __launch_bounds__(256)
nep_zbl_kernel(long long natoms, int nn, int nimages, const long long *__restrict__ NL,
               const TI *__restrict__ Ri, const long long *__restrict__ type_map,
               const long long *__restrict__ image_of, int ntypes,
               const double *__restrict__ pair_s, const double *__restrict__ pair_c, double zbl,
               T *__restrict__ Ei, double *__restrict__ Etot, T *__restrict__ force,
               double *__restrict__ virial, int *__restrict__ err) {
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    const T rcut = (T)(zbl * 0.5);
    const T kpi = (T)(3.14159265358979323846 / (zbl * 0.5));
    const T zb = (T)zbl;
    for (long long i = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < natoms;
         i += nw) {
        const long long ti = type_map[i];
        if (ti < 0 || ti >= ntypes) {
            if (lane == 0) atomicOr(err, MATPL_KERR_BAD_TYPE);
            continue;
        }
        double e_sum = 0.0, v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        T fi[3] = {T(0), T(0), T(0)};
        bool any = false;
        for (int s = lane; s < nn; s += 32) {
            const long long q = i * nn + s;
            const long long j = NL[q];
            if (j < 0) continue;
            const T r = (T)Ri[4 * q];
            if (!(r > T(0) && r <= zb)) continue;
            if (j >= natoms) {
                atomicOr(err, MATPL_KERR_BAD_COUNT);
                continue;
            }
            const long long tj = type_map[j];
            if (tj < 0 || tj >= ntypes) {
                atomicOr(err, MATPL_KERR_BAD_TYPE);
                continue;
            }
            any = true;
            const T sij = (T)pair_s[ti * ntypes + tj], cij = (T)pair_c[ti * ntypes + tj];
            const T dxdr = sij * T(2.134563);
            const T x = r * sij * T(2.134563);
            T phi = T(0), dphi = T(0);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const T a = (T)kZblA[k], b = (T)kZblB[k];
                const T ex = zexp<T>(-b * x);
                phi += a * ex;
                dphi -= a * b * ex;
            }
            T fc = T(1), dfc = T(0);
            if (r >= rcut) {
                T sn, cs;
                zsincos<T>(kpi * (r - rcut), &sn, &cs);
                fc = T(0.5) + T(0.5) * cs;
                dfc = -T(0.5) * sn * kpi;
            }
            const T e = cij * phi * fc / r;
            const T dedr = cij * (dphi * dxdr * fc / r + phi * dfc / r - phi * fc / (r * r));
            e_sum += 0.5 * (double)e;
            const T xyz[3] = {(T)Ri[4 * q + 1], (T)Ri[4 * q + 2], (T)Ri[4 * q + 3]};
            const T g = T(0.5) * dedr / r;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const T f = g * xyz[a];
                fi[a] += f;
                atomicAdd(force + 3 * j + a, -f);
#pragma unroll
                for (int b = 0; b < 3; ++b) v[3 * a + b] -= (double)f * (double)xyz[b];
            }
        }
        if (!__any_sync(0xffffffffu, any)) continue;
        e_sum = warp_sum(e_sum);
#pragma unroll
        for (int a = 0; a < 3; ++a) fi[a] = warp_sum(fi[a]);
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = warp_sum(v[k]);
        if (lane == 0) {
            Ei[i] += (T)e_sum;
#pragma unroll
            for (int a = 0; a < 3; ++a) atomicAdd(force + 3 * i + a, fi[a]);
            const long long b = image_of[i];
            if (b < 0 || b >= nimages) {
                atomicOr(err, MATPL_KERR_BAD_COUNT);
            } else {
                if (Etot) atomicAdd(Etot + b, e_sum);
#pragma unroll
                for (int k = 0; k < 9; ++k) atomicAdd(virial + 9 * b + k, v[k]);
            }
        }
    }
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" int matpl_nep_zbl(int dtype, int ri_dtype, long long natoms, int max_nn, int nimages,
                             const long long *NL, const void *Ri, const long long *type_map,
                             const long long *image_of, int ntypes, const double *pair_s,
                             const double *pair_c, double zbl, void *Ei, double *Etot,
                             void *force, double *virial, int *err_dev, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_nep_zbl: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(ri_dtype == MATPL_F64 || (ri_dtype == MATPL_F32 && dtype == MATPL_F32),
                  MATPL_ERR_DTYPE, "matpl_nep_zbl: Ri is f64, or f32 with an f32 computation");
    MATPL_REQUIRE(natoms >= 0 && max_nn >= 0 && nimages >= 1 && ntypes >= 1 && zbl > 0,
                  MATPL_ERR_INVALID, "bad sizes or zbl <= 0");
    MATPL_REQUIRE(err_dev && (natoms * (long long)max_nn == 0 ||
                              (NL && Ri && type_map && image_of && pair_s && pair_c && Ei &&
                               force && virial)),
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(force, "matpl_nep_zbl");
    if (natoms == 0 || max_nn == 0) return MATPL_OK;
    cudaStream_t s = as_stream(stream);
    ProfScope ps("nep_zbl", s);
    const int grid = (int)std::min<long long>((natoms + 7) / 8, (long long)device_sms() * 16);
    if (dtype == MATPL_F64)
        nep_zbl_kernel<double, double><<<grid, 256, 0, s>>>(
            natoms, max_nn, nimages, NL, (const double *)Ri, type_map, image_of, ntypes, pair_s,
            pair_c, zbl, (double *)Ei, Etot, (double *)force, virial, err_dev);
    else if (ri_dtype == MATPL_F64)
        nep_zbl_kernel<float, double><<<grid, 256, 0, s>>>(
            natoms, max_nn, nimages, NL, (const double *)Ri, type_map, image_of, ntypes, pair_s,
            pair_c, zbl, (float *)Ei, Etot, (float *)force, virial, err_dev);
    else
        nep_zbl_kernel<float, float><<<grid, 256, 0, s>>>(
            natoms, max_nn, nimages, NL, (const float *)Ri, type_map, image_of, ntypes, pair_s,
            pair_c, zbl, (float *)Ei, Etot, (float *)force, virial, err_dev);
    return check_launch("matpl_nep_zbl");
}
