// Force / virial custom ops and their backward, the drop-in for MatPL's CalcOps_cuda
// calculateForce / calculateVirial (src/op/src/CalcOps.cpp:6-72, 170-236).
//
// One thread per neighbor slot, grid sized in multiples of the SM count.  Each slot reads its
// 4 dE values and 12 Ri_d values (contiguous, so a warp reads a contiguous 1.5 KB (f32) /
// 3 KB (f64) span), forms f = dE . Ri_d (3 values) and scatters it with red.global.add.
// The virial op also reduces the per-slot outer product f (x) Rij in FP64 per block before a
// single global add per component, instead of a second reduction kernel.
#include "common.cuh"

namespace matpl {
namespace {

constexpr int kThreads = 256;

inline int grid_for(long long work) {
    long long g = (work + kThreads - 1) / kThreads;
    const long long cap = (long long)device_sms() * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

template <typename T>
__global__ void copy_center_force(const T *__restrict__ Fc, T *__restrict__ out, int batch,
                                  int natoms, int nghost) {
    const long long total = (long long)batch * (natoms + nghost) * 3;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long per = (long long)(natoms + nghost) * 3;
        const long long b = t / per, r = t % per;
        out[t] = (r < (long long)natoms * 3) ? Fc[b * natoms * 3 + r] : T(0);
    }
}

template <typename T>
__device__ __forceinline__ void slot_f(const T *__restrict__ dE, const T *__restrict__ Rd,
                                       long long slot, T f[3]) {
    const T *e = dE + slot * 4;
    const T *d = Rd + slot * 12;
    T e0 = e[0], e1 = e[1], e2 = e[2], e3 = e[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) f[a] = e0 * d[a] + e1 * d[3 + a] + e2 * d[6 + a] + e3 * d[9 + a];
}

template <typename T>
__global__ void force_scatter(const int32_t *__restrict__ nl, const T *__restrict__ dE,
                              const T *__restrict__ Rd, T *__restrict__ force, int batch,
                              int natoms, int nslots, int nghost) {
    const long long total = (long long)batch * natoms * nslots;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < total;
         s += (long long)gridDim.x * blockDim.x) {
        const int j = nl[s];
        if (j < 0) continue;
        const long long b = s / ((long long)natoms * nslots);
        T f[3];
        slot_f(dE, Rd, s, f);
        T *dst = force + (b * (natoms + nghost) + j) * 3;
        atomicAdd(dst + 0, f[0]);
        atomicAdd(dst + 1, f[1]);
        atomicAdd(dst + 2, f[2]);
    }
}

template <typename T>
__global__ void virial_scatter(const int32_t *__restrict__ nl, const T *__restrict__ dE,
                               const T *__restrict__ Rij, const T *__restrict__ Rd,
                               T *__restrict__ virial, T *__restrict__ atom_virial, int batch,
                               int natoms, int nslots, int nghost) {
    // Each block covers slots of one configuration at a time; per-block FP64 partials.
    __shared__ double part[kThreads / 32][9];
    const long long per_b = (long long)natoms * nslots;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = 0; b < batch; ++b) {
        double acc[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = 0.0;
        for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < per_b;
             t += (long long)gridDim.x * blockDim.x) {
            const long long s = b * per_b + t;
            const int j = nl[s];
            if (j < 0) continue;
            T f[3];
            slot_f(dE, Rd, s, f);
            const T r[3] = {Rij[s * 3], Rij[s * 3 + 1], Rij[s * 3 + 2]};
            T *dst = atom_virial + ((long long)b * (natoms + nghost) + j) * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const T v = f[a] * r[c];   // calculateVirial.cu:80 order: (Ri_d comp, Rij comp)
                    atomicAdd(dst + 3 * a + c, v);
                    acc[3 * a + c] += (double)v;
                }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = warp_sum(acc[q]);
        if (lane == 0)
            for (int q = 0; q < 9; ++q) part[warp][q] = acc[q];
        __syncthreads();
        if (threadIdx.x < 9) {
            double v = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) v += part[w][threadIdx.x];
            atomicAdd(virial + b * 9 + threadIdx.x, (T)v);
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void force_grad_kernel(const int32_t *__restrict__ nl, const T *__restrict__ Rd,
                                  const T *__restrict__ gF, T *__restrict__ grad, int batch,
                                  int natoms, int nslots, int nghost) {
    // grad[b,i,4k+w] = -gF[b,i] . Rd[w]  +  (j>=0 ? gF[b, j % N] . Rd[w] : 0)
    // (calculateForceGrad.cu:10-60, including its j % nloc folding of ghost indices)
    const long long total = (long long)batch * natoms * nslots;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < total;
         s += (long long)gridDim.x * blockDim.x) {
        const long long bi = s / nslots;
        const long long b = bi / natoms;
        const int i = (int)(bi % natoms);
        const T *gi = gF + (b * (natoms + nghost) + i) * 3;
        T gc[3] = {gi[0], gi[1], gi[2]};
        const int j = nl[s];
        T gj[3] = {T(0), T(0), T(0)};
        if (j >= 0) {
            const T *p = gF + (b * (natoms + nghost) + (j % natoms)) * 3;
            gj[0] = p[0]; gj[1] = p[1]; gj[2] = p[2];
        }
        const T *d = Rd + s * 12;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const T dw0 = d[3 * w], dw1 = d[3 * w + 1], dw2 = d[3 * w + 2];
            grad[s * 4 + w] = -(gc[0] * dw0 + gc[1] * dw1 + gc[2] * dw2)
                              + (gj[0] * dw0 + gj[1] * dw1 + gj[2] * dw2);
        }
    }
}

template <typename T>
__global__ void virial_grad_kernel(const int32_t *__restrict__ nl, const T *__restrict__ Rij,
                                   const T *__restrict__ Rd, const T *__restrict__ gV,
                                   T *__restrict__ grad, int batch, int natoms, int nslots) {
    // grad[b,i,4k+w] = sum_{a,c} gV[b, 3a+c] * Rij[c] * Rd[w][a]   (calculateVirialGrad.cu:16-66)
    const long long total = (long long)batch * natoms * nslots;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < total;
         s += (long long)gridDim.x * blockDim.x) {
        const long long b = s / ((long long)natoms * nslots);
        const int j = nl[s];
        if (j < 0) {
#pragma unroll
            for (int w = 0; w < 4; ++w) grad[s * 4 + w] = T(0);
            continue;
        }
        const T *g = gV + b * 9;
        const T r0 = Rij[s * 3], r1 = Rij[s * 3 + 1], r2 = Rij[s * 3 + 2];
        T ga[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) ga[a] = g[3 * a] * r0 + g[3 * a + 1] * r1 + g[3 * a + 2] * r2;
        const T *d = Rd + s * 12;
#pragma unroll
        for (int w = 0; w < 4; ++w)
            grad[s * 4 + w] = ga[0] * d[3 * w] + ga[1] * d[3 * w + 1] + ga[2] * d[3 * w + 2];
    }
}

int check_common(int dtype, int batch, int natoms, int nslots, int nghost) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "force/virial ops support f32 and f64");
    MATPL_REQUIRE(batch >= 0 && natoms >= 0 && nslots >= 0 && nghost >= 0, MATPL_ERR_INVALID,
                  "negative size");
    return MATPL_OK;
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" int matpl_calc_force(int dtype, const int32_t *list_neigh, const void *dE,
                                const void *Ri_d, const void *F_center, int batch, int natoms,
                                int nslots, int nghost, void *force_out, void *stream) {
    int st = check_common(dtype, batch, natoms, nslots, nghost);
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    const long long nout = (long long)batch * (natoms + nghost) * 3;
    const long long nsl = (long long)batch * natoms * nslots;
    MATPL_REQUIRE((nout == 0 || force_out) && ((long long)batch * natoms == 0 || F_center) &&
                      (nsl == 0 || (list_neigh && dE && Ri_d)),
                  MATPL_ERR_INVALID, "matpl_calc_force: null pointer argument");
    if (nout == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(force_out, "matpl_calc_force");
    if (dtype == MATPL_F64) {
        copy_center_force<double><<<grid_for(nout), kThreads, 0, s>>>(
            (const double *)F_center, (double *)force_out, batch, natoms, nghost);
        if (nsl)
            force_scatter<double><<<grid_for(nsl), kThreads, 0, s>>>(
                list_neigh, (const double *)dE, (const double *)Ri_d, (double *)force_out, batch,
                natoms, nslots, nghost);
    } else {
        copy_center_force<float><<<grid_for(nout), kThreads, 0, s>>>(
            (const float *)F_center, (float *)force_out, batch, natoms, nghost);
        if (nsl)
            force_scatter<float><<<grid_for(nsl), kThreads, 0, s>>>(
                list_neigh, (const float *)dE, (const float *)Ri_d, (float *)force_out, batch,
                natoms, nslots, nghost);
    }
    return check_launch("matpl_calc_force");
}

extern "C" int matpl_calc_virial(int dtype, const int32_t *list_neigh, const void *dE,
                                 const void *Rij, const void *Ri_d, int batch, int natoms,
                                 int nslots, int nghost, void *virial_out, void *atom_virial_out,
                                 void *stream) {
    int st = check_common(dtype, batch, natoms, nslots, nghost);
    if (st) return st;
    MATPL_REQUIRE((batch == 0 || (virial_out && (natoms + nghost == 0 || atom_virial_out))) &&
                      ((long long)batch * natoms * nslots == 0 || (list_neigh && dE && Rij && Ri_d)),
                  MATPL_ERR_INVALID, "matpl_calc_virial: null pointer argument");
    if (batch == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(virial_out, "matpl_calc_virial");
    cudaStream_t s = as_stream(stream);
    const size_t es = dtype == MATPL_F64 ? 8 : 4;
    if (cudaMemsetAsync(virial_out, 0, es * 9 * (size_t)batch, s) != cudaSuccess ||
        cudaMemsetAsync(atom_virial_out, 0, es * 9 * (size_t)batch * (natoms + nghost), s) !=
            cudaSuccess) {
        set_error("matpl_calc_virial: memset failed");
        return MATPL_ERR_CUDA;
    }
    const long long per_b = (long long)natoms * nslots;
    if (batch == 0 || per_b == 0) return MATPL_OK;
    if (dtype == MATPL_F64)
        virial_scatter<double><<<grid_for(per_b), kThreads, 0, s>>>(
            list_neigh, (const double *)dE, (const double *)Rij, (const double *)Ri_d,
            (double *)virial_out, (double *)atom_virial_out, batch, natoms, nslots, nghost);
    else
        virial_scatter<float><<<grid_for(per_b), kThreads, 0, s>>>(
            list_neigh, (const float *)dE, (const float *)Rij, (const float *)Ri_d,
            (float *)virial_out, (float *)atom_virial_out, batch, natoms, nslots, nghost);
    return check_launch("matpl_calc_virial");
}

extern "C" int matpl_calc_force_grad(int dtype, const int32_t *list_neigh, const void *Ri_d,
                                     const void *grad_force, int batch, int natoms, int nslots,
                                     int nghost, void *grad_dE, void *stream) {
    int st = check_common(dtype, batch, natoms, nslots, nghost);
    if (st) return st;
    const long long nsl = (long long)batch * natoms * nslots;
    if (nsl == 0) return MATPL_OK;
    MATPL_REQUIRE(list_neigh && Ri_d && grad_force && grad_dE, MATPL_ERR_INVALID,
                  "matpl_calc_force_grad: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(grad_dE, "matpl_calc_force_grad");
    cudaStream_t s = as_stream(stream);
    if (dtype == MATPL_F64)
        force_grad_kernel<double><<<grid_for(nsl), kThreads, 0, s>>>(
            list_neigh, (const double *)Ri_d, (const double *)grad_force, (double *)grad_dE,
            batch, natoms, nslots, nghost);
    else
        force_grad_kernel<float><<<grid_for(nsl), kThreads, 0, s>>>(
            list_neigh, (const float *)Ri_d, (const float *)grad_force, (float *)grad_dE, batch,
            natoms, nslots, nghost);
    return check_launch("matpl_calc_force_grad");
}

extern "C" int matpl_calc_virial_grad(int dtype, const int32_t *list_neigh, const void *Rij,
                                      const void *Ri_d, const void *grad_virial, int batch,
                                      int natoms, int nslots, void *grad_dE, void *stream) {
    int st = check_common(dtype, batch, natoms, nslots, 0);
    if (st) return st;
    const long long nsl = (long long)batch * natoms * nslots;
    if (nsl == 0) return MATPL_OK;
    MATPL_REQUIRE(list_neigh && Rij && Ri_d && grad_virial && grad_dE, MATPL_ERR_INVALID,
                  "matpl_calc_virial_grad: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(grad_dE, "matpl_calc_virial_grad");
    cudaStream_t s = as_stream(stream);
    if (dtype == MATPL_F64)
        virial_grad_kernel<double><<<grid_for(nsl), kThreads, 0, s>>>(
            list_neigh, (const double *)Rij, (const double *)Ri_d, (const double *)grad_virial,
            (double *)grad_dE, batch, natoms, nslots);
    else
        virial_grad_kernel<float><<<grid_for(nsl), kThreads, 0, s>>>(
            list_neigh, (const float *)Rij, (const float *)Ri_d, (const float *)grad_virial,
            (float *)grad_dE, batch, natoms, nslots);
    return check_launch("matpl_calc_virial_grad");
}
