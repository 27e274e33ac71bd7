// Data-path statistics: the sums behind davg / dstd, replacing the per-image calc_stat +
// smooth of src/pre_data/dpuni_data_loader.py:422-563 (called from calculate_davg_dstd,
// :377-420, for the images set_davg_dstd picks, :180-215).
//
// For every configuration b and centre type t it accumulates over all slots of the atoms of
// type t the smoothed environment rows Ri = vv(r) * (1/r, x/r^2, y/r^2, z/r^2), r and r^2
// from the pair vector (x, y, z) of image_dr as calc_stat forms them (vv the
// switching function of smooth with the model's Rmin / Rmax): sums of Ri_0, Ri_0^2 and of the
// three angular channels and their squares, in FP64.  The caller turns them into davg / dstd
// (the slot count per type is known on the host).  One warp per atom, lanes over slots, warp
// reduction, one FP64 atomic per (b, t, channel) and warp.
#include <algorithm>

#include "common.cuh"

namespace matpl {
namespace {

__global__ void __launch_bounds__(128)
env_stats_kernel(int batch, int natoms, int nslots, int ntypes, const int32_t *__restrict__ type_map,
                 const int32_t *__restrict__ list_neigh, const double *__restrict__ image_dr,
                 double rmin, double rmax, double *__restrict__ sums, int32_t *__restrict__ err) {
    const int lane = threadIdx.x & 31;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    const long long total = (long long)batch * natoms;
    for (long long ba = gw; ba < total; ba += nw) {
        const int b = (int)(ba / natoms), a = (int)(ba - (long long)b * natoms);
        const int t = type_map[a];
        if (t < 0 || t >= ntypes) {
            if (lane == 0) atomicOr(err, MATPL_KERR_BAD_TYPE);
            continue;
        }
        double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int s = lane; s < nslots; s += 32) {
            const long long q = ba * nslots + s;
            if (list_neigh[q] <= 0) continue;
            // the reference's order: dR2 from the pair vector, Rij = sqrt(dR2), r = dR2 / Rij
            const double x = image_dr[4 * q + 1], y = image_dr[4 * q + 2], z = image_dr[4 * q + 3];
            const double r2 = x * x + y * y + z * z;
            const double r = r2 / sqrt(r2);
            double vv;
            if (r < rmin) vv = 1.0;
            else if (r < rmax) {
                const double u = (r - rmin) / (rmax - rmin);
                vv = u * u * u * (-6.0 * u * u + 15.0 * u - 10.0) + 1.0;
            } else vv = 0.0;
            const double c[4] = {vv / r, vv * x / r2, vv * y / r2, vv * z / r2};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                acc[2 * k] += c[k];
                acc[2 * k + 1] += c[k] * c[k];
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = warp_sum(acc[k]);
        if (lane < 8) {
            double v = acc[0];
#pragma unroll
            for (int k = 1; k < 8; ++k) v = lane == k ? acc[k] : v;
            atomicAdd(&sums[((long long)b * ntypes + t) * 8 + lane], v);
        }
    }
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" int matpl_env_stats(int batch, int natoms, int nslots, int ntypes,
                               const int32_t *type_map, const int32_t *list_neigh,
                               const double *image_dr, double rmin, double rmax, double *sums,
                               int32_t *err_dev, void *stream) {
    MATPL_REQUIRE(batch >= 0 && natoms >= 0 && nslots >= 0 && ntypes >= 1, MATPL_ERR_INVALID,
                  "bad sizes");
    MATPL_REQUIRE(rmax > rmin && rmin >= 0, MATPL_ERR_INVALID, "need 0 <= rmin < rmax");
    MATPL_REQUIRE(sums && err_dev && (batch * (long long)natoms == 0 ||
                                      (type_map && list_neigh && image_dr)),
                  MATPL_ERR_INVALID, "null pointer argument");
    cudaStream_t s = as_stream(stream);
    MATPL_REQUIRE_ON_DEVICE(sums, "matpl_env_stats");
    if (cudaMemsetAsync(sums, 0, sizeof(double) * 8 * (size_t)batch * ntypes, s) != cudaSuccess) {
        set_error("matpl_env_stats: memset failed");
        return MATPL_ERR_CUDA;
    }
    const long long total = (long long)batch * natoms;
    if (total == 0 || nslots == 0) return MATPL_OK;
    ProfScope ps("env_stats", s);
    const long long grid = std::min<long long>((total + 3) / 4, (long long)device_sms() * 16);
    env_stats_kernel<<<(int)grid, 128, 0, s>>>(batch, natoms, nslots, ntypes, type_map,
                                               list_neigh, image_dr, rmin, rmax, sums, err_dev);
    return check_launch("matpl_env_stats");
}
