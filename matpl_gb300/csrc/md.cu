// Batched molecular dynamics of many replicas of uneven size with one DP model: the kernels
// around the evaluation.  All replicas live in one ragged atom array (replica r owns atoms
// [rep_start[r], rep_start[r+1])), so one launch of each kernel covers every replica:
//
//   md_drift         x += v dt + a dt^2 / 2; flags a list rebuild when an atom has moved more
//                    than half the skin since the last build (the displacement rule LAMMPS
//                    applies to the pair style's list, pair_matpl.cpp:1096-1110);
//   md_skin_build    the Verlet list at Rc + skin of every replica (all periodic images), run
//                    only when the rebuild flag is set: a device-side gate, so a captured step
//                    needs no host decision;
//   md_skin_filter   every step, the pairs of the skin list inside Rc at the current positions
//                    as the occupied-slot list the evaluation reads (1-based global neighbor
//                    index, (r, x_j - x_i) rows, per-type block lengths);
//   md_kick          a = F / m, v += (a_old + a) dt / 2, and per replica the kinetic and
//                    potential energy summed in FP64 (one block per replica, fixed order).
//
// A pair between Rc and Rc + skin is left out of the filtered list, so the evaluation counts it
// among the empty slots of its type block (m - count), which is what a pair outside Rc is in
// the reference's list: the forces equal those of an exact search at the same positions.
#include "common.cuh"

namespace matpl {
namespace {

constexpr int kBuildThreads = 128;
constexpr int kMaxImg = 127;   // image indices are stored as signed bytes

__device__ __forceinline__ int pack_img(int a, int b, int c) {
    return (a & 0xff) | ((b & 0xff) << 8) | ((c & 0xff) << 16);
}
__device__ __forceinline__ void unpack_img(int p, int &a, int &b, int &c) {
    a = (int)(signed char)(p & 0xff);
    b = (int)(signed char)((p >> 8) & 0xff);
    c = (int)(signed char)((p >> 16) & 0xff);
}

__global__ void md_drift_kernel(int ntot, double dt, double half_skin2, double *__restrict__ x,
                                const double *__restrict__ v, const double *__restrict__ a,
                                const double *__restrict__ x_ref, int32_t *gate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool far = false;
    if (i < ntot) {
        double d2 = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double xn = x[3 * i + c] + v[3 * i + c] * dt + 0.5 * dt * dt * a[3 * i + c];
            x[3 * i + c] = xn;
            const double d = xn - x_ref[3 * i + c];
            d2 += d * d;
        }
        far = d2 > half_skin2;
    }
    if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicOr(gate, 1);
}

// One block = up to 128 atoms i of one replica against every atom j of that replica and every
// periodic image within reach.  Coordinates are fractional (x L^-1) wrapped into [0, 1), tested
// in FP32 against (Rc + skin + margin)^2; the filter recomputes every kept pair exactly.  The
// stored image (n_a, n_b, n_c) refers to the unwrapped positions: d = x_j - x_i + n L.
__global__ void __launch_bounds__(kBuildThreads)
md_skin_build_kernel(int ntypes, int cap, float rs2, const int32_t *__restrict__ rep_start,
                     const int2 *__restrict__ work, const double *__restrict__ lattice,
                     const double *__restrict__ inv_lattice, const int32_t *__restrict__ type_map,
                     const double *__restrict__ x, int32_t *__restrict__ nbr,
                     int32_t *__restrict__ img, int32_t *__restrict__ cnt,
                     double *__restrict__ x_ref, const int32_t *gate, int32_t *err) {
    if (*gate == 0) return;
    __shared__ float4 sf[kBuildThreads];        // wrapped fractional coordinates + type
    __shared__ int sfl[kBuildThreads];          // packed floor of the unwrapped coordinates
    __shared__ float sL[9];
    __shared__ int sK[3];
    const int2 w = work[blockIdx.x];
    const int r = w.x;
    const int a0 = rep_start[r], a1 = rep_start[r + 1];
    const double *L = lattice + 9 * r, *Li = inv_lattice + 9 * r;
    if (threadIdx.x < 9) sL[threadIdx.x] = (float)L[threadIdx.x];
    if (threadIdx.x < 3) {
        // images needed along cell vector d: ceil((Rc + skin) / width_d), width_d = vol / |b x c|
        const int d = threadIdx.x, e = (d + 1) % 3, f = (d + 2) % 3;
        const double cx = L[3 * e + 1] * L[3 * f + 2] - L[3 * e + 2] * L[3 * f + 1];
        const double cy = L[3 * e + 2] * L[3 * f + 0] - L[3 * e + 0] * L[3 * f + 2];
        const double cz = L[3 * e + 0] * L[3 * f + 1] - L[3 * e + 1] * L[3 * f + 0];
        const double vol = fabs(L[3 * d] * cx + L[3 * d + 1] * cy + L[3 * d + 2] * cz);
        const double width = vol / sqrt(cx * cx + cy * cy + cz * cz);
        int k = (int)ceil(sqrt((double)rs2) / width);
        if (k > kMaxImg / 2) {
            atomicMax(err, MATPL_KERR_BAD_BOX);
            k = 0;
        }
        sK[d] = k;
    }
    const int i = a0 + w.y + threadIdx.x;
    const bool live = i < a1;
    float fi[3] = {0.f, 0.f, 0.f};
    int fli[3] = {0, 0, 0};
    if (live) {
        for (int c = 0; c < 3; ++c) {
            const double f = x[3 * i] * Li[c] + x[3 * i + 1] * Li[3 + c] + x[3 * i + 2] * Li[6 + c];
            const double fl = floor(f);
            fli[c] = (int)fl;
            fi[c] = (float)(f - fl);
        }
        for (int c = 0; c < 3; ++c) x_ref[3 * i + c] = x[3 * i + c];
    }
    int count[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) count[t] = 0;
    bool over = false, bad = false;
    const size_t row = (size_t)(live ? i : 0) * ntypes * cap;
    __syncthreads();
    const int K0 = sK[0], K1 = sK[1], K2 = sK[2];
    for (int j0 = a0; j0 < a1; j0 += kBuildThreads) {
        __syncthreads();
        const int jl = j0 + threadIdx.x;
        if (jl < a1) {
            float f3[3];
            int fl3[3];
            for (int c = 0; c < 3; ++c) {
                const double f = x[3 * jl] * Li[c] + x[3 * jl + 1] * Li[3 + c] +
                                 x[3 * jl + 2] * Li[6 + c];
                const double fl = floor(f);
                fl3[c] = (int)fl;
                f3[c] = (float)(f - fl);
            }
            int tj = type_map[jl];
            if (tj < 0 || tj >= ntypes) {
                atomicMax(err, MATPL_KERR_BAD_TYPE);
                tj = -1;
            }
            sf[threadIdx.x] = make_float4(f3[0], f3[1], f3[2], __int_as_float(tj));
            bad |= abs(fl3[0]) > kMaxImg / 2 || abs(fl3[1]) > kMaxImg / 2 ||
                   abs(fl3[2]) > kMaxImg / 2;
            sfl[threadIdx.x] = pack_img(fl3[0], fl3[1], fl3[2]);
        }
        __syncthreads();
        if (!live) continue;
        const int nj = min(kBuildThreads, a1 - j0);
        for (int q = 0; q < nj; ++q) {
            const float4 fj = sf[q];
            const int tj = __float_as_int(fj.w);
            if (tj < 0) continue;
            const float e0 = fj.x - fi[0], e1 = fj.y - fi[1], e2 = fj.z - fi[2];
            for (int n0 = -K0; n0 <= K0; ++n0) {
                const float g0 = e0 + (float)n0;
                for (int n1 = -K1; n1 <= K1; ++n1) {
                    const float g1 = e1 + (float)n1;
                    const float p0 = g0 * sL[0] + g1 * sL[3], p1 = g0 * sL[1] + g1 * sL[4],
                                p2 = g0 * sL[2] + g1 * sL[5];
                    for (int n2 = -K2; n2 <= K2; ++n2) {
                        const float g2 = e2 + (float)n2;
                        const float dx = p0 + g2 * sL[6], dy = p1 + g2 * sL[7],
                                    dz = p2 + g2 * sL[8];
                        const float rr = dx * dx + dy * dy + dz * dz;
                        if (rr >= rs2) continue;
                        if (j0 + q == i && n0 == 0 && n1 == 0 && n2 == 0) continue;
                        int fa, fb, fc;
                        unpack_img(sfl[q], fa, fb, fc);
                        const int ia = n0 - fa + fli[0], ib = n1 - fb + fli[1],
                                  ic = n2 - fc + fli[2];
                        bad |= abs(ia) > kMaxImg || abs(ib) > kMaxImg || abs(ic) > kMaxImg;
                        const int c = count[tj];
                        if (c < cap) {
                            nbr[row + (size_t)tj * cap + c] = j0 + q;
                            img[row + (size_t)tj * cap + c] = pack_img(ia, ib, ic);
                        } else {
                            over = true;
                        }
                        count[tj] = c + 1;
                    }
                }
            }
        }
    }
    if (live) {
        for (int t = 0; t < ntypes; ++t) cnt[(size_t)i * ntypes + t] = min(count[t], cap);
        bad |= abs(fli[0]) > kMaxImg / 2 || abs(fli[1]) > kMaxImg / 2 ||
               abs(fli[2]) > kMaxImg / 2;
    }
    if (over) atomicMax(err, MATPL_KERR_NEIGHBOR_OVERFLOW);
    if (bad) atomicMax(err, MATPL_KERR_BAD_BOX);
}

__global__ void md_gate_clear_kernel(int32_t *gate, int32_t *nbuild) {
    if (*gate != 0) {
        if (nbuild) *nbuild += 1;
        *gate = 0;
    }
}

// One warp per atom: the skin entries of each type block inside Rc at the current positions,
// compacted in list order.
template <typename TO>
__global__ void md_skin_filter_kernel(int ntot, int ntypes, int cap, int m, double rc2,
                                      const int32_t *__restrict__ atom_rep,
                                      const double *__restrict__ lattice,
                                      const int32_t *__restrict__ nbr,
                                      const int32_t *__restrict__ img,
                                      const int32_t *__restrict__ cnt,
                                      const double *__restrict__ x,
                                      int32_t *__restrict__ list_neigh, TO *__restrict__ image_dr,
                                      int32_t *__restrict__ num_neigh, int32_t *err) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= ntot) return;
    const double *L = lattice + 9 * atom_rep[i];
    double Lr[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) Lr[q] = L[q];
    const double xi0 = x[3 * i], xi1 = x[3 * i + 1], xi2 = x[3 * i + 2];
    const int S = ntypes * m;
    bool over = false;
    for (int t = 0; t < ntypes; ++t) {
        const size_t src = ((size_t)i * ntypes + t) * cap;
        const size_t dst = (size_t)i * S + (size_t)t * m;
        const int n = cnt[(size_t)i * ntypes + t];
        int c = 0;
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            bool keep = false;
            int j = 0;
            double dx = 0.0, dy = 0.0, dz = 0.0, rr = 0.0;
            if (k < n) {
                j = nbr[src + k];
                int na, nb, nc;
                unpack_img(img[src + k], na, nb, nc);
                dx = x[3 * j] - xi0 + (na * Lr[0] + nb * Lr[3] + nc * Lr[6]);
                dy = x[3 * j + 1] - xi1 + (na * Lr[1] + nb * Lr[4] + nc * Lr[7]);
                dz = x[3 * j + 2] - xi2 + (na * Lr[2] + nb * Lr[5] + nc * Lr[8]);
                rr = dx * dx + dy * dy + dz * dz;
                keep = rr < rc2 && rr > 1.0e-8;
            }
            const unsigned mk = __ballot_sync(0xffffffffu, keep);
            const int at = c + __popc(mk & ((1u << lane) - 1u));
            if (keep && at < m) {
                list_neigh[dst + at] = j + 1;
                TO *o = image_dr + 4 * (dst + at);
                o[0] = pair_r<TO>(rr);
                o[1] = conv<TO>(dx);
                o[2] = conv<TO>(dy);
                o[3] = conv<TO>(dz);
            }
            c += __popc(mk);
        }
        over |= c > m;
        if (lane == 0) num_neigh[(size_t)i * ntypes + t] = min(c, m);
    }
    if (over && lane == 0) atomicMax(err, MATPL_KERR_NEIGHBOR_OVERFLOW);
}

// One block per replica.  mode 0: a = F / m only (the first force evaluation); mode 1: the
// closing half kick of velocity Verlet.  ke / pe: per replica, FP64, block-order sums.
template <typename TI>
__global__ void md_kick_kernel(int mode, double dt, double conv_ke,
                               const int32_t *__restrict__ rep_start,
                               const double *__restrict__ inv_mass, const double *__restrict__ mass,
                               const TI *__restrict__ force, const TI *__restrict__ ei,
                               double *__restrict__ v, double *__restrict__ a,
                               double *__restrict__ ke, double *__restrict__ pe) {
    const int r = blockIdx.x;
    const int a0 = rep_start[r], a1 = rep_start[r + 1];
    double sk = 0.0, sp = 0.0;
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        double vv = 0.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double an = (double)force[3 * i + c] * inv_mass[i];
            double vc = v[3 * i + c];
            if (mode == 1) vc += 0.5 * dt * (a[3 * i + c] + an);
            v[3 * i + c] = vc;
            a[3 * i + c] = an;
            vv += vc * vc;
        }
        sk += 0.5 * conv_ke * mass[i] * vv;
        sp += (double)ei[i];
    }
    __shared__ double rk[32], rp[32];
    sk = warp_sum(sk);
    sp = warp_sum(sp);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        rk[wid] = sk;
        rp[wid] = sp;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tk = 0.0, tp = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
            tk += rk[q];
            tp += rp[q];
        }
        ke[r] = tk;
        pe[r] = tp;
    }
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" int matpl_md_drift(int ntot, double dt, double skin, double *x, const double *v,
                              const double *a, const double *x_ref, int32_t *gate,
                              void *stream) {
    MATPL_REQUIRE(ntot >= 0 && dt > 0.0 && skin >= 0.0, MATPL_ERR_INVALID,
                  "matpl_md_drift: bad sizes");
    if (ntot == 0) return MATPL_OK;
    MATPL_REQUIRE(x && v && a && x_ref && gate, MATPL_ERR_INVALID,
                  "matpl_md_drift: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(x, "matpl_md_drift");
    const double h = 0.5 * skin;
    md_drift_kernel<<<(ntot + 255) / 256, 256, 0, as_stream(stream)>>>(ntot, dt, h * h, x, v, a,
                                                                        x_ref, gate);
    return check_launch("matpl_md_drift");
}

extern "C" int matpl_md_skin_build(int nrep, int ntot, int ntypes, int cap, double r_list,
                                   const int32_t *rep_start, const int32_t *work, int nwork,
                                   const double *lattice, const double *inv_lattice,
                                   const int32_t *type_map, const double *x, int32_t *nbr,
                                   int32_t *img, int32_t *cnt, double *x_ref, int32_t *gate,
                                   int32_t *nbuild, int32_t *err, void *stream) {
    MATPL_REQUIRE(nrep >= 0 && ntot >= 0 && nwork >= 0 && ntypes >= 1 && ntypes <= 8 &&
                      cap >= 1 && r_list > 0.0,
                  MATPL_ERR_INVALID, "matpl_md_skin_build: bad sizes (ntypes 1..8)");
    if (ntot == 0 || nwork == 0) return MATPL_OK;
    MATPL_REQUIRE(rep_start && work && lattice && inv_lattice && type_map && x && nbr && img &&
                      cnt && x_ref && gate && err,
                  MATPL_ERR_INVALID, "matpl_md_skin_build: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(x, "matpl_md_skin_build");
    cudaStream_t s = as_stream(stream);
    const float rs = (float)r_list * (1.0f + 1e-5f) + 1e-3f;   // margin for the FP32 test
    md_skin_build_kernel<<<nwork, kBuildThreads, 0, s>>>(
        ntypes, cap, rs * rs, rep_start, reinterpret_cast<const int2 *>(work), lattice,
        inv_lattice, type_map, x, nbr, img, cnt, x_ref, gate, err);
    md_gate_clear_kernel<<<1, 1, 0, s>>>(gate, nbuild);
    return check_launch("matpl_md_skin_build");
}

extern "C" int matpl_md_skin_filter(int dtype, int ntot, int ntypes, int cap, int m, double rc,
                                    const int32_t *atom_rep, const double *lattice,
                                    const int32_t *nbr, const int32_t *img, const int32_t *cnt,
                                    const double *x, int32_t *list_neigh, void *image_dr,
                                    int32_t *num_neigh, int32_t *err, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F64 || dtype == MATPL_F32, MATPL_ERR_DTYPE,
                  "matpl_md_skin_filter: dtype must be MATPL_F64 or MATPL_F32");
    MATPL_REQUIRE(ntot >= 0 && ntypes >= 1 && cap >= 1 && m >= 1 && rc > 0.0,
                  MATPL_ERR_INVALID, "matpl_md_skin_filter: bad sizes");
    if (ntot == 0) return MATPL_OK;
    MATPL_REQUIRE(atom_rep && lattice && nbr && img && cnt && x && list_neigh && image_dr &&
                      num_neigh && err,
                  MATPL_ERR_INVALID, "matpl_md_skin_filter: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(x, "matpl_md_skin_filter");
    cudaStream_t s = as_stream(stream);
    const int threads = 256;
    const long long blocks = ((long long)ntot * 32 + threads - 1) / threads;
    if (dtype == MATPL_F64)
        md_skin_filter_kernel<double><<<(unsigned)blocks, threads, 0, s>>>(
            ntot, ntypes, cap, m, rc * rc, atom_rep, lattice, nbr, img, cnt, x, list_neigh,
            (double *)image_dr, num_neigh, err);
    else
        md_skin_filter_kernel<float><<<(unsigned)blocks, threads, 0, s>>>(
            ntot, ntypes, cap, m, rc * rc, atom_rep, lattice, nbr, img, cnt, x, list_neigh,
            (float *)image_dr, num_neigh, err);
    return check_launch("matpl_md_skin_filter");
}

extern "C" int matpl_md_kick(int dtype, int mode, int nrep, double dt, double conv_ke,
                             const int32_t *rep_start, const double *inv_mass,
                             const double *mass, const void *force, const void *ei, double *v,
                             double *a, double *ke, double *pe, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F64 || dtype == MATPL_F32, MATPL_ERR_DTYPE,
                  "matpl_md_kick: dtype must be MATPL_F64 or MATPL_F32");
    MATPL_REQUIRE(nrep >= 0 && (mode == 0 || mode == 1), MATPL_ERR_INVALID,
                  "matpl_md_kick: bad sizes or mode");
    if (nrep == 0) return MATPL_OK;
    MATPL_REQUIRE(rep_start && inv_mass && mass && force && ei && v && a && ke && pe,
                  MATPL_ERR_INVALID, "matpl_md_kick: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(v, "matpl_md_kick");
    cudaStream_t s = as_stream(stream);
    if (dtype == MATPL_F64)
        md_kick_kernel<double><<<nrep, 256, 0, s>>>(mode, dt, conv_ke, rep_start, inv_mass, mass,
                                                    (const double *)force, (const double *)ei, v,
                                                    a, ke, pe);
    else
        md_kick_kernel<float><<<nrep, 256, 0, s>>>(mode, dt, conv_ke, rep_start, inv_mass, mass,
                                                   (const float *)force, (const float *)ei, v, a,
                                                   ke, pe);
    return check_launch("matpl_md_kick");
}
