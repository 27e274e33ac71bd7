// Fused NEP energy + force + virial: the drop-in for NEP.forward + calculate_force_virial
// (src/model/nep_net.py:293-438, 486-648) on the lists of calculate_neighbor, replacing the
// CalcOps chain calculateNepFeat / calculateNepMbFeat (descriptor, src/op/src/CalcOps.cpp:669-1023),
// the per-element FittingNet (src/model/nep_fitting.py:136-160), autograd for dE/dRi, and
// calculateNepForce / calculateNepVirial (src/op/kernel/calculateNepForce.cu,
// calculateNepVirial.cu).
//
// One warp owns one centre atom at a time (a contiguous run of atoms per warp):
//   radial    lanes over radial slots: Chebyshev basis f_k(r) (cal_fk, nep_net.py:691-715),
//             q_n = sum_j sum_k c2[ti,tj,n,k] f_k, warp-reduced;
//   angular   lanes over angular slots in chunks of 32: g_n(r) and the 24 real harmonics
//             b_lm(r_hat) (cal_blm_ij, nep_net.py:816-838) are staged in shared memory, then
//             lanes over lm form s_nlm = sum_j g_n b_lm;  q_nl = sum_m C3B s^2 and the 4-/5-body
//             invariants (cal_feat_multi_body, nep_net.py:745-814);
//   network   feats * q_scaler -> tanh layer (lanes over hidden units) -> Ei; the adjoint
//             dE/dq (lanes over features) and dE/ds_nlm (lanes over lm) stay in shared memory;
//   forces    lanes over slots again: f_ij = dE/dr_ij from g_n', b_lm and grad b_lm in closed
//             form, F_i += f_ij, F_j -= f_ij (float4 reductions into a padded accumulator),
//             virial[a*3+c] -= f_a r_c kept per lane and reduced once per frame.
// Nothing per pair or per feature goes to HBM.  Energies and the virial are summed in FP64.
#include "common.cuh"
#include "nep_math.cuh"

namespace matpl {
namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kMaxHidden = 128;

struct NepLayout {
    int ntypes, nr, kr, na, ka, nfeat, hidden;
    int two;                 // radial features (nr when train_2b, else 0)
    int l3, four, five;      // 3-body l_max (0 or 4), 4-body / 5-body present
    double rc_r_d, rc_a_d;
    int off_c2, off_c3, off_qs, off_net, net_stride;   // element offsets in params
    int nparams;
    // shared-memory copy: hidden width padded to hp (a multiple of 4 with hp / 4 odd, so that
    // 16-byte row loads of consecutive lanes fall in different banks), features padded to fmp
    int hp, fmp, off_net_s, net_stride_s, nparams_s;
    int kpr, kpa, off_c2_s, off_c3_s, off_qs_s;        // coefficient rows padded to 4
};

struct EvalArgs {
    NepLayout L;
    const void *params;
    long long natoms;
    int nframes;
    const long long *frame_start;   // [nframes + 1]
    const long long *type_map;
    int max_r, max_a;
    const long long *NN_r, *NL_r, *NN_a, *NL_a;
    const double *Ri_r, *Ri_a;
    // compact lists (MD skin form): int32 NN / NL, float4 (r, x, y, z); used when CL
    const int *cNN_r, *cNL_r, *cNN_a, *cNL_a;
    const float4 *cRi_r, *cRi_a;
    void *Ei;
    double *Etot, *virial;
    void *facc;                     // float4 [N] (f32) or double [N, 3] (f64)
    void *feats;                    // descriptor only: q [N, F] before q_scaler, else NULL
    int *err;
    // shared-memory layout (bytes): parameters, then one scratch area per warp
    int smem_params, warp_bytes;
    int o_stash_g, o_stash_b, o_s, o_dEds, o_fin, o_dq, o_dpre;
    int o_rj, o_rv, o_rgp, o_aj, o_av, o_ag, o_agp;
};

// f64 -> f32, round to nearest even, with integer instructions: the FP64 pipe of this part
// issues two lanes per clock, so the FP32 kernel keeps conversions off it.  Magnitudes below
// 2^-126 become signed zero (inputs are pair vectors in Angstrom).
__device__ __forceinline__ float f64_to_f32(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const unsigned ex = (hi >> 20) & 0x7ffu;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    if (ex == 0x7ffu) return __uint_as_float(sign | 0x7f800000u | (m | (lo & 0x1fffffffu) ? 0x400000u : 0u));
    const int e = (int)ex - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned r = ((unsigned)e << 23) | m;
    r += (rest > 0x10000000u) || (rest == 0x10000000u && (m & 1u));
    return __uint_as_float(sign | r);
}
template <typename T> __device__ __forceinline__ T ld_conv(const double *p);
template <> __device__ __forceinline__ float ld_conv<float>(const double *p) {
    return f64_to_f32(__ldg(p));
}
template <> __device__ __forceinline__ double ld_conv<double>(const double *p) { return __ldg(p); }

// four consecutive elements from 16-byte aligned shared memory
__device__ __forceinline__ void lds4(const float *p, float *o) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void lds4(const double *p, double *o) {
    const double2 a = reinterpret_cast<const double2 *>(p)[0];
    const double2 b = reinterpret_cast<const double2 *>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}

__device__ __forceinline__ void sts4(float *p, float a, float b, float c, float d) {
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void sts4(double *p, double a, double b, double c, double d) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2 *>(p)[1] = make_double2(c, d);
}

template <typename T>
__device__ __forceinline__ void add_force(void *facc, long long j, T fx, T fy, T fz);
template <>
__device__ __forceinline__ void add_force<float>(void *facc, long long j, float fx, float fy,
                                                 float fz) {
    atomicAdd(reinterpret_cast<float4 *>(facc) + j, make_float4(fx, fy, fz, 0.f));
}
template <>
__device__ __forceinline__ void add_force<double>(void *facc, long long j, double fx, double fy,
                                                  double fz) {
    double *p = reinterpret_cast<double *>(facc) + 3 * j;
    atomicAdd(p, fx);
    atomicAdd(p + 1, fy);
    atomicAdd(p + 2, fz);
}

// List access for the reference layout (int64 NN / NL, f64 (r, x, y, z)) and the compact one.
template <bool CL>
__device__ __forceinline__ long long list_count(const EvalArgs &A, bool radial, long long i) {
    if (CL) return radial ? A.cNN_r[i] : A.cNN_a[i];
    return radial ? A.NN_r[i] : A.NN_a[i];
}
template <bool CL>
__device__ __forceinline__ long long list_index(const EvalArgs &A, bool radial, long long e) {
    if (CL) return radial ? A.cNL_r[e] : A.cNL_a[e];
    return radial ? A.NL_r[e] : A.NL_a[e];
}
// (r, x, y, z) of list entry e, or r = 0 when !valid
template <typename T, bool CL>
__device__ __forceinline__ void list_pair(const EvalArgs &A, bool radial, long long e, bool valid,
                                          T &r, T &x, T &y, T &z) {
    r = x = y = z = T(0);
    if (!valid) return;
    if (CL) {
        const float4 v = __ldg((radial ? A.cRi_r : A.cRi_a) + e);
        r = (T)v.x; x = (T)v.y; y = (T)v.z; z = (T)v.w;
    } else {
        const double *rr = (radial ? A.Ri_r : A.Ri_a) + e * 4;
        r = ld_conv<T>(rr);
        x = ld_conv<T>(rr + 1);
        y = ld_conv<T>(rr + 2);
        z = ld_conv<T>(rr + 3);
    }
}

template <typename T>
__device__ __forceinline__ void flush_frame(const EvalArgs &A, int frame, double e, T *vir,
                                            int lane) {
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double v = warp_sum((double)vir[q]);
        if (lane == 0 && v != 0.0) atomicAdd(A.virial + 9 * frame + q, v);
        vir[q] = T(0);
    }
    if (lane == 0 && e != 0.0) atomicAdd(A.Etot + frame, e);
}

// NRM / KRM / NAM / KAM: compiled maxima of n_max + 1 and basis_size + 1; EX: the model has
// exactly these sizes (the size guards inside the unrolled loops then fold away).
template <typename T, int NRM, int KRM, int NAM, int KAM, bool CL, bool EX>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
nep_eval_kernel(EvalArgs A, long long atoms_per_warp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const NepLayout &L = A.L;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    T *P = reinterpret_cast<T *>(smem_raw);
    // the 3-body constants in shared memory: lanes index them by their own lm, and lane-varying
    // indices into __constant__ memory are served one address at a time
    __shared__ T c3s[24];
    if (threadIdx.x < 24) c3s[threadIdx.x] = C3<T>(threadIdx.x);
    // parameters: c2, c3, q_scaler as packed; per element W0 rows padded to Hp, b0, W1, b1
    {
        const T *gp = reinterpret_cast<const T *>(A.params);
        const int T2 = L.ntypes * L.ntypes;
        for (int q = threadIdx.x; q < T2 * L.nr * L.kpr; q += blockDim.x) {
            const int row = q / L.kpr, k = q - row * L.kpr;
            P[L.off_c2_s + q] = k < L.kr ? gp[L.off_c2 + row * L.kr + k] : T(0);
        }
        if (L.l3)
            for (int q = threadIdx.x; q < T2 * L.na * L.kpa; q += blockDim.x) {
                const int row = q / L.kpa, k = q - row * L.kpa;
                P[L.off_c3_s + q] = k < L.ka ? gp[L.off_c3 + row * L.ka + k] : T(0);
            }
        for (int q = threadIdx.x; q < L.nfeat; q += blockDim.x) P[L.off_qs_s + q] = gp[L.off_qs + q];
        const int Hp = L.hp;
        for (int t = 0; t < L.ntypes; ++t) {
            const T *src = gp + L.off_net + t * L.net_stride;
            T *dst = P + L.off_net_s + t * L.net_stride_s;
            for (int q = threadIdx.x; q < L.nfeat * Hp; q += blockDim.x) {
                const int f = q / Hp, k = q - f * Hp;
                dst[q] = k < L.hidden ? src[f * L.hidden + k] : T(0);
            }
            for (int q = threadIdx.x; q < Hp; q += blockDim.x) {
                dst[L.nfeat * Hp + q] = q < L.hidden ? src[L.nfeat * L.hidden + q] : T(0);
                dst[L.nfeat * Hp + Hp + q] = q < L.hidden ? src[L.nfeat * L.hidden + L.hidden + q] : T(0);
            }
            if (threadIdx.x == 0) dst[L.nfeat * Hp + 2 * Hp] = src[L.nfeat * L.hidden + 2 * L.hidden];
        }
    }
    unsigned char *Wb = smem_raw + A.smem_params + (size_t)A.warp_bytes * wib;
    constexpr int NAMP = (NAM + 3) / 4 * 4;                   // rows padded for 16-byte loads
    const int nr_ = EX ? NRM : L.nr, kr_ = EX ? KRM : L.kr, na_ = EX ? NAM : L.na,
              ka_ = EX ? KAM : L.ka;
    const int kpr_ = EX ? (KRM + 3) / 4 * 4 : L.kpr, kpa_ = EX ? (KAM + 3) / 4 * 4 : L.kpa;
    T *stash_g = reinterpret_cast<T *>(Wb + A.o_stash_g);    // [32][NAMP]
    T *stash_b = reinterpret_cast<T *>(Wb + A.o_stash_b);    // [32][25]
    T *s_sm = reinterpret_cast<T *>(Wb + A.o_s);             // [NAM][24]
    T *dEds = reinterpret_cast<T *>(Wb + A.o_dEds);          // [24][NAMP]
    T *fin = reinterpret_cast<T *>(Wb + A.o_fin);            // [FMp] scaled features
    T *dq = reinterpret_cast<T *>(Wb + A.o_dq);              // [FMp] dE/dq
    T *dpre = reinterpret_cast<T *>(Wb + A.o_dpre);          // [Hp]
    int *rj = reinterpret_cast<int *>(Wb + A.o_rj);          // radial pairs: neighbor
    T *rv = reinterpret_cast<T *>(Wb + A.o_rv);              //   (x, y, z, 1/r)
    T *rgp = reinterpret_cast<T *>(Wb + A.o_rgp);            //   g_n'(r)   [max_r][NRM]
    int *aj = reinterpret_cast<int *>(Wb + A.o_aj);          // angular pairs: neighbor
    T *av = reinterpret_cast<T *>(Wb + A.o_av);              //   (x, y, z, 1/r)
    T *ag = reinterpret_cast<T *>(Wb + A.o_ag);              //   g_n(r)    [max_a][NAM]
    T *agp = reinterpret_cast<T *>(Wb + A.o_agp);            //   g_n'(r)   [max_a][NAM]
    for (int q = lane; q < L.fmp; q += 32) fin[q] = T(0);
    for (int q = lane; q < L.hp; q += 32) dpre[q] = T(0);
    __syncthreads();

    const T *c2 = P + L.off_c2_s, *c3 = P + L.off_c3_s, *qs = P + L.off_qs_s;
    constexpr int KRP = (KRM + 3) / 4 * 4, KAP = (KAM + 3) / 4 * 4;
    const T rc_r = (T)L.rc_r_d, rc_a = (T)L.rc_a_d;
    const T rcinv_r = T(1) / rc_r, rcinv_a = T(1) / rc_a;

    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    const long long a_begin = gw * atoms_per_warp;
    long long a_end = a_begin + atoms_per_warp;
    if (a_end > A.natoms) a_end = A.natoms;
    if (a_begin >= a_end) return;
    int frame = 0;
    {
        int lo = 0, hi = A.nframes - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.frame_start[mid] <= a_begin) lo = mid; else hi = mid - 1;
        }
        frame = lo;
    }
    long long frame_end = A.frame_start[frame + 1];
    double e_frame = 0.0;
    T vir[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) vir[q] = T(0);

    // the next atom's element and list lengths are loaded while the current atom is processed
    long long ti_next = A.type_map[a_begin];
    long long nr_next = L.two ? list_count<CL>(A, true, a_begin) : 0;
    long long na_next = L.l3 ? list_count<CL>(A, false, a_begin) : 0;
    for (long long i = a_begin; i < a_end; ++i) {
        const int ti = (int)ti_next;
        const long long nr_i = nr_next, na_i = na_next;
        if (i + 1 < a_end) {
            ti_next = A.type_map[i + 1];
            if (L.two) nr_next = list_count<CL>(A, true, i + 1);
            if (L.l3) na_next = list_count<CL>(A, false, i + 1);
        }
        while (i >= frame_end && frame + 1 < A.nframes) {
            if (!A.feats) flush_frame<T>(A, frame, e_frame, vir, lane);
            e_frame = 0.0;
            ++frame;
            frame_end = A.frame_start[frame + 1];
        }
        if (ti < 0 || ti >= L.ntypes) {
            if (lane == 0) {
                atomicOr(A.err, MATPL_KERR_BAD_TYPE);
                if (!A.feats) reinterpret_cast<T *>(A.Ei)[i] = T(0);
            }
            continue;
        }
        const int nnr = L.two ? (int)min(nr_i, (long long)A.max_r) : 0;
        const int nna = L.l3 ? (int)min(na_i, (long long)A.max_a) : 0;
        const long long row_r = i * A.max_r, row_a = i * A.max_a;

        // ---------------- radial descriptor; pair vector and g_n' kept for the force pass
        T qr[NRM];
#pragma unroll
        for (int n = 0; n < NRM; ++n) qr[n] = T(0);
        // element of neighbor j, -1 (and the error recorded) when j or its type is out of range
        auto type_of = [&](long long j) -> int {
            int tj = -1;
            if (j >= 0 && j < A.natoms) {
                tj = (int)A.type_map[j];
                if (tj < 0 || tj >= L.ntypes) { atomicOr(A.err, MATPL_KERR_BAD_TYPE); tj = -1; }
            } else if (j >= A.natoms) {
                atomicOr(A.err, MATPL_KERR_BAD_COUNT);
            }
            return tj;
        };
        auto radial_one = [&](int sl, long long j, int tj, T r, T px, T py, T pz) {
            if (tj < 0 || !(r > T(0))) { rj[sl] = -1; return; }
            const T rinv = T(1) / r;
            sts4(rv + 4 * sl, px, py, pz, rinv);
            rj[sl] = (int)j;
            T f[KRP], df[KRP];
            basis<T, KRM>(r, rc_r, rcinv_r, kr_, f, df);
#pragma unroll
            for (int k = KRM; k < KRP; ++k) f[k] = df[k] = T(0);
            const T *c = c2 + (ti * L.ntypes + tj) * nr_ * kpr_;
#pragma unroll
            for (int n = 0; n < NRM; ++n) {
                T g = T(0), gp = T(0);
                if (n < nr_) {
#pragma unroll
                    for (int k4 = 0; k4 < KRP; k4 += 4) {
                        T c4[4];
                        lds4(c + n * kpr_ + k4, c4);
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            g += c4[u] * f[k4 + u];
                            gp += c4[u] * df[k4 + u];
                        }
                    }
                }
                qr[n] += g;
                rgp[sl * NRM + n] = gp;
            }
        };
        // two slots per lane and pass: both slots' list loads are in flight before either's
        // neighbor-type gather, and both gathers before the arithmetic
        for (int sl0 = lane; sl0 < nnr; sl0 += 64) {
            const int sl1 = sl0 + 32;
            const bool two = sl1 < nnr;
            const long long j0 = list_index<CL>(A, true, row_r + sl0);
            const long long j1 = two ? list_index<CL>(A, true, row_r + sl1) : -1;
            T r0, x0, y0, z0, r1, x1, y1, z1;
            list_pair<T, CL>(A, true, row_r + sl0, true, r0, x0, y0, z0);
            list_pair<T, CL>(A, true, row_r + sl1, two, r1, x1, y1, z1);
            const int tj0 = type_of(j0);
            const int tj1 = two ? type_of(j1) : -1;
            radial_one(sl0, j0, tj0, r0, x0, y0, z0);
            if (two) radial_one(sl1, j1, tj1, r1, x1, y1, z1);
        }
#pragma unroll
        for (int n = 0; n < NRM; ++n) qr[n] = warp_sum(qr[n]);

        // ---------------- angular descriptor: s_nlm = sum_j g_n(r) b_lm(r_hat)
        T sacc[NAM];
#pragma unroll
        for (int n = 0; n < NAM; ++n) sacc[n] = T(0);
        for (int base = 0; base < nna; base += 32) {
            const int sl = base + lane;
            if (sl < nna) {
                const long long j = list_index<CL>(A, false, row_a + sl);
                T r, px, py, pz;
                list_pair<T, CL>(A, false, row_a + sl, true, r, px, py, pz);
                const int tj = type_of(j);
                const bool ok = tj >= 0 && r > T(0);
                T f[KAP], df[KAP];
                basis<T, KAM>(ok ? r : rc_a, rc_a, rcinv_a, ka_, f, df);
#pragma unroll
                for (int k = KAM; k < KAP; ++k) f[k] = df[k] = T(0);
                const T *c = c3 + (ok ? (ti * L.ntypes + tj) : 0) * na_ * kpa_;
#pragma unroll
                for (int n = 0; n < NAM; ++n) {
                    T g = T(0), gp = T(0);
                    if (n < na_ && ok) {
#pragma unroll
                        for (int k4 = 0; k4 < KAP; k4 += 4) {
                            T c4[4];
                            lds4(c + n * kpa_ + k4, c4);
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                g += c4[u] * f[k4 + u];
                                gp += c4[u] * df[k4 + u];
                            }
                        }
                    }
                    stash_g[lane * NAMP + n] = g;
                    ag[sl * NAM + n] = g;
                    agp[sl * NAM + n] = gp;
                }
                const T rinv = ok ? T(1) / r : T(0);
                const T x = ok ? px : T(0), y = ok ? py : T(0), z = ok ? pz : T(0);
                aj[sl] = ok ? (int)j : -1;
                sts4(av + 4 * sl, x, y, z, rinv);
                const T ux = x * rinv, uy = y * rinv, uz = z * rinv;
#pragma unroll
                for (int lm = 0; lm < 24; ++lm) {
                    T b, gx, gy, gz;
                    harmonic<T>(lm, ux, uy, uz, b, gx, gy, gz);
                    stash_b[lane * 25 + lm] = b;
                }
            }
            __syncwarp();
            const int cnt = min(32, nna - base);
            if (lane < 24) {
                for (int jj = 0; jj < cnt; ++jj) {
                    const T b = stash_b[jj * 25 + lane];
#pragma unroll
                    T gv[NAMP];
#pragma unroll
                    for (int q = 0; q < NAMP; q += 4) lds4(stash_g + jj * NAMP + q, gv + q);
#pragma unroll
                    for (int n = 0; n < NAM; ++n) sacc[n] += gv[n] * b;
                }
            }
            __syncwarp();
        }
        if (lane < 24) {
#pragma unroll
            for (int n = 0; n < NAM; ++n) s_sm[n * 24 + lane] = sacc[n];
        }
        if (lane == 0) {
#pragma unroll
            for (int n = 0; n < NRM; ++n)
                if (n < L.two) {
                    fin[n] = qr[n] * qs[n];
                    if (A.feats) reinterpret_cast<T *>(A.feats)[i * L.nfeat + n] = qr[n];
                }
        }
        __syncwarp();

        // ---------------- angular features, scaled
        for (int fa = lane; fa < L.nfeat - L.two; fa += 32) {
            T q;
            const int n3 = L.l3 * na_;
            if (fa < n3) {
                const int l = fa / na_, n = fa - l * na_;
                const int lo = l == 0 ? 0 : (l == 1 ? 3 : (l == 2 ? 8 : 15));
                const int hi = l == 0 ? 3 : (l == 1 ? 8 : (l == 2 ? 15 : 24));
                q = T(0);
                for (int lm = lo; lm < hi; ++lm) {
                    const T sv = s_sm[n * 24 + lm];
                    q += c3s[lm] * sv * sv;
                }
            } else if (L.four && fa < n3 + na_) {
                const T *s = s_sm + (fa - n3) * 24;
                q = C4<T>(0) * s[3] * s[3] * s[3] + C4<T>(1) * s[3] * (s[4] * s[4] + s[5] * s[5]) +
                    C4<T>(2) * s[3] * (s[6] * s[6] + s[7] * s[7]) +
                    C4<T>(3) * s[6] * (s[5] * s[5] - s[4] * s[4]) + C4<T>(4) * s[4] * s[5] * s[7];
            } else {
                const T *s = s_sm + (fa - n3 - (L.four ? na_ : 0)) * 24;
                const T a0 = s[0] * s[0], a12 = s[1] * s[1] + s[2] * s[2];
                q = C5<T>(0) * a0 * a0 + C5<T>(1) * a0 * a12 + C5<T>(2) * a12 * a12;
            }
            fin[L.two + fa] = q * qs[L.two + fa];
            if (A.feats) reinterpret_cast<T *>(A.feats)[i * L.nfeat + L.two + fa] = q;
        }
        __syncwarp();
        if (A.feats) continue;            // descriptor only

        // ---------------- fitting net of element ti and its adjoint
        const int Hp = L.hp;
        const T *net = P + L.off_net_s + ti * L.net_stride_s;
        const T *W0 = net, *b0 = net + L.nfeat * Hp, *W1 = b0 + Hp;
        const T b1 = W1[Hp];
        T e = T(0);
        for (int k = lane; k < L.hidden; k += 32) {
            T pre = b0[k];
            for (int f4 = 0; f4 < L.nfeat; f4 += 4) {
                T x4[4];
                lds4(fin + f4, x4);
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (f4 + u < L.nfeat) pre += x4[u] * W0[(f4 + u) * Hp + k];
            }
            const T h = dev_tanh(pre);
            e += W1[k] * h;
            dpre[k] = W1[k] * (T(1) - h * h);
        }
        const T Ei = warp_sum(e) + b1;
        __syncwarp();
        for (int f = lane; f < L.nfeat; f += 32) {
            T d = T(0);
            const T *w = W0 + f * Hp;
            for (int k4 = 0; k4 < Hp; k4 += 4) {
                T a4[4], b4[4];
                lds4(w + k4, a4);
                lds4(dpre + k4, b4);
                d += a4[0] * b4[0] + a4[1] * b4[1] + a4[2] * b4[2] + a4[3] * b4[3];
            }
            dq[f] = d * qs[f];
        }
        __syncwarp();

        // ---------------- dE/ds_nlm (lanes over lm)
        if (lane < 24 && L.l3) {
            const int lm = lane, l = l_of(lm);
            const int n3 = L.l3 * na_;
#pragma unroll
            for (int n = 0; n < NAM; ++n) {
                if (n >= na_) {              // rows past n_max are read (times zero) below
                    dEds[lm * NAMP + n] = T(0);
                    continue;
                }
                const T *s = s_sm + n * 24;
                T d = dq[L.two + l * na_ + n] * T(2) * c3s[lm] * s[lm];
                if (L.four && lm >= 3 && lm <= 7) {
                    const T g4 = dq[L.two + n3 + n];
                    T dd;
                    if (lm == 3)
                        dd = T(3) * C4<T>(0) * s[3] * s[3] + C4<T>(1) * (s[4] * s[4] + s[5] * s[5]) +
                             C4<T>(2) * (s[6] * s[6] + s[7] * s[7]);
                    else if (lm == 4)
                        dd = T(2) * C4<T>(1) * s[3] * s[4] - T(2) * C4<T>(3) * s[6] * s[4] +
                             C4<T>(4) * s[5] * s[7];
                    else if (lm == 5)
                        dd = T(2) * C4<T>(1) * s[3] * s[5] + T(2) * C4<T>(3) * s[6] * s[5] +
                             C4<T>(4) * s[4] * s[7];
                    else if (lm == 6)
                        dd = T(2) * C4<T>(2) * s[3] * s[6] + C4<T>(3) * (s[5] * s[5] - s[4] * s[4]);
                    else
                        dd = T(2) * C4<T>(2) * s[3] * s[7] + C4<T>(4) * s[4] * s[5];
                    d += g4 * dd;
                }
                if (L.five && lm <= 2) {
                    const T g5 = dq[L.two + n3 + (L.four ? na_ : 0) + n];
                    const T a0 = s[0] * s[0], a12 = s[1] * s[1] + s[2] * s[2];
                    const T dd = lm == 0
                                     ? T(4) * C5<T>(0) * a0 * s[0] + T(2) * C5<T>(1) * s[0] * a12
                                     : T(2) * C5<T>(1) * a0 * s[lm] + T(4) * C5<T>(2) * a12 * s[lm];
                    d += g5 * dd;
                }
                dEds[lm * NAMP + n] = d;
            }
        }
        __syncwarp();

        // ---------------- forces: radial pairs
        T fi0 = T(0), fi1 = T(0), fi2 = T(0);
        T dqr[NRM];
#pragma unroll
        for (int n = 0; n < NRM; ++n) dqr[n] = n < L.two ? dq[n] : T(0);
        for (int sl = lane; sl < nnr; sl += 32) {
            const int j = rj[sl];
            if (j < 0) continue;
            T dEdr = T(0);
#pragma unroll
            for (int n = 0; n < NRM; ++n) dEdr += dqr[n] * rgp[sl * NRM + n];
            T v4[4];
            lds4(rv + 4 * sl, v4);
            const T x = v4[0], y = v4[1], z = v4[2];
            const T s = dEdr * v4[3];
            const T fx = s * x, fy = s * y, fz = s * z;
            fi0 += fx; fi1 += fy; fi2 += fz;
            add_force<T>(A.facc, j, -fx, -fy, -fz);
            vir[0] -= fx * x; vir[1] -= fx * y; vir[2] -= fx * z;
            vir[3] -= fy * x; vir[4] -= fy * y; vir[5] -= fy * z;
            vir[6] -= fz * x; vir[7] -= fz * y; vir[8] -= fz * z;
        }

        // ---------------- forces: angular pairs
        for (int sl = lane; sl < nna; sl += 32) {
            const int j = aj[sl];
            if (j < 0) continue;
            T v4[4];
            lds4(av + 4 * sl, v4);
            const T x = v4[0], y = v4[1], z = v4[2], rinv = v4[3];
            T g[NAM], An[NAM];
#pragma unroll
            for (int n = 0; n < NAM; ++n) {
                g[n] = ag[sl * NAM + n];
                An[n] = T(0);
            }
            const T ux = x * rinv, uy = y * rinv, uz = z * rinv;
            T G0 = T(0), G1 = T(0), G2 = T(0);
#pragma unroll
            for (int lm = 0; lm < 24; ++lm) {
                T b, gx, gy, gz;
                harmonic<T>(lm, ux, uy, uz, b, gx, gy, gz);
                T Bl = T(0), dv[NAMP];
#pragma unroll
                for (int q = 0; q < NAMP; q += 4) lds4(dEds + lm * NAMP + q, dv + q);
#pragma unroll
                for (int n = 0; n < NAM; ++n) {
                    const T d = dv[n];
                    Bl += d * g[n];
                    An[n] += d * b;
                }
                G0 += Bl * gx; G1 += Bl * gy; G2 += Bl * gz;
            }
            T dEdr = T(0);
#pragma unroll
            for (int n = 0; n < NAM; ++n) dEdr += agp[sl * NAM + n] * An[n];
            const T ug = ux * G0 + uy * G1 + uz * G2;
            const T fx = dEdr * ux + (G0 - ug * ux) * rinv;
            const T fy = dEdr * uy + (G1 - ug * uy) * rinv;
            const T fz = dEdr * uz + (G2 - ug * uz) * rinv;
            fi0 += fx; fi1 += fy; fi2 += fz;
            add_force<T>(A.facc, j, -fx, -fy, -fz);
            vir[0] -= fx * x; vir[1] -= fx * y; vir[2] -= fx * z;
            vir[3] -= fy * x; vir[4] -= fy * y; vir[5] -= fy * z;
            vir[6] -= fz * x; vir[7] -= fz * y; vir[8] -= fz * z;
        }
        fi0 = warp_sum(fi0);
        fi1 = warp_sum(fi1);
        fi2 = warp_sum(fi2);
        if (lane == 0) {
            add_force<T>(A.facc, i, fi0, fi1, fi2);
            reinterpret_cast<T *>(A.Ei)[i] = Ei;
            e_frame += (double)Ei;
        }
        __syncwarp();
    }
    if (!A.feats) flush_frame<T>(A, frame, e_frame, vir, lane);
}

__global__ void nep_frame_start(const long long *__restrict__ num_atom, int nframes,
                                long long natoms, long long *__restrict__ start,
                                int *__restrict__ err) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        long long a = 0;
        for (int f = 0; f < nframes; ++f) {
            start[f] = a;
            a += num_atom[f] > 0 ? num_atom[f] : 0;
        }
        start[nframes] = a;
        if (a != natoms) atomicOr(err, MATPL_KERR_BAD_COUNT);
    }
}

__global__ void nep_force_out(const float4 *__restrict__ acc, float *__restrict__ force,
                              long long natoms) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < natoms;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 v = acc[i];
        force[3 * i] = v.x;
        force[3 * i + 1] = v.y;
        force[3 * i + 2] = v.z;
    }
}

int make_layout(const matpl_nep_model *m, NepLayout *L) {
    MATPL_REQUIRE(m != nullptr, MATPL_ERR_INVALID, "null model");
    MATPL_REQUIRE(m->ntypes >= 1 && m->ntypes <= 64, MATPL_ERR_INVALID, "ntypes must be 1..64");
    MATPL_REQUIRE(m->n_max_radial >= 0 && m->n_max_angular >= 0 && m->basis_radial >= 0 &&
                      m->basis_angular >= 0,
                  MATPL_ERR_INVALID, "negative n_max / basis_size");
    MATPL_REQUIRE(m->l_max_3b == 0 || m->l_max_3b == 4, MATPL_ERR_UNSUPPORTED,
                  "l_max (3-body) must be 0 or 4");
    MATPL_REQUIRE(m->l_max_4b == 0 || m->l_max_4b == 2, MATPL_ERR_UNSUPPORTED,
                  "l_max (4-body) must be 0 or 2");
    MATPL_REQUIRE(m->l_max_5b == 0 || m->l_max_5b == 1, MATPL_ERR_UNSUPPORTED,
                  "l_max (5-body) must be 0 or 1");
    MATPL_REQUIRE(m->neuron >= 1 && m->neuron <= kMaxHidden, MATPL_ERR_UNSUPPORTED,
                  "hidden layer must have 1..128 neurons");
    MATPL_REQUIRE(m->cutoff_radial > 0 && m->cutoff_angular > 0, MATPL_ERR_INVALID,
                  "cutoffs must be positive");
    NepLayout l{};
    l.ntypes = m->ntypes;
    l.nr = m->n_max_radial + 1;
    l.kr = m->basis_radial + 1;
    l.na = m->n_max_angular + 1;
    l.ka = m->basis_angular + 1;
    l.two = m->train_2b ? l.nr : 0;
    l.l3 = m->l_max_3b;
    l.four = l.l3 && m->l_max_4b > 0;
    l.five = l.l3 && m->l_max_5b > 0;
    l.nfeat = l.two + (l.l3 ? l.na * (4 + l.four + l.five) : 0);
    MATPL_REQUIRE(l.nfeat > 0, MATPL_ERR_INVALID, "no descriptor components");
    l.hidden = m->neuron;
    l.rc_r_d = m->cutoff_radial;
    l.rc_a_d = m->cutoff_angular;
    const int T2 = l.ntypes * l.ntypes;
    l.off_c2 = 0;
    l.off_c3 = T2 * l.nr * l.kr;
    l.off_qs = l.off_c3 + (l.l3 ? T2 * l.na * l.ka : 0);
    l.off_net = l.off_qs + l.nfeat;
    l.net_stride = l.nfeat * l.hidden + 2 * l.hidden + 1;
    l.nparams = l.off_net + l.ntypes * l.net_stride;
    l.hp = (l.hidden + 3) / 4 * 4;
    if ((l.hp / 4) % 2 == 0) l.hp += 4;
    l.fmp = (l.nfeat + 3) / 4 * 4;
    l.kpr = (l.kr + 3) / 4 * 4;
    l.kpa = (l.ka + 3) / 4 * 4;
    l.off_c2_s = 0;
    l.off_c3_s = T2 * l.nr * l.kpr;
    l.off_qs_s = l.off_c3_s + (l.l3 ? T2 * l.na * l.kpa : 0);
    l.off_net_s = (l.off_qs_s + l.nfeat + 3) / 4 * 4;
    l.net_stride_s = (l.nfeat * l.hp + 2 * l.hp + 1 + 3) / 4 * 4;
    l.nparams_s = l.off_net_s + l.ntypes * l.net_stride_s;
    *L = l;
    return MATPL_OK;
}

size_t ws_layout(int dtype, int nframes, long long natoms, unsigned char *base,
                 long long **frame_start, void **facc) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes, 256);
        return base ? base + o : nullptr;
    };
    unsigned char *fs = take(sizeof(long long) * ((size_t)nframes + 1));
    unsigned char *fa = dtype == MATPL_F32 ? take(sizeof(float4) * (size_t)natoms) : nullptr;
    if (frame_start) *frame_start = (long long *)fs;
    if (facc) *facc = fa;
    return off;
}

template <typename T, int NRM, int KRM, int NAM, int KAM, bool CL, bool EX>
int launch_eval(const EvalArgs &A0, cudaStream_t s) {
    EvalArgs A = A0;
    const NepLayout &L = A.L;
    auto kern = nep_eval_kernel<T, NRM, KRM, NAM, KAM, CL, EX>;
    // per-warp scratch, 16-byte aligned pieces
    int off = 0;
    auto take = [&](size_t bytes) {
        const int o = off;
        off += (int)((bytes + 15) / 16 * 16);
        return o;
    };
    const size_t t = sizeof(T);
    const int mr = A.max_r > 0 ? A.max_r : 1, ma = A.max_a > 0 ? A.max_a : 1;
    constexpr int NAMP = (NAM + 3) / 4 * 4;
    A.o_stash_g = take(32 * NAMP * t);
    A.o_stash_b = take(32 * 25 * t);
    A.o_s = take(NAM * 24 * t);
    A.o_dEds = take(NAMP * 24 * t);
    A.o_fin = take(L.fmp * t);
    A.o_dq = take(L.fmp * t);
    A.o_dpre = take(L.hp * t);
    A.o_rj = take(mr * 4);
    A.o_rv = take((size_t)mr * 4 * t);
    A.o_rgp = take((size_t)mr * NRM * t);
    A.o_aj = take(ma * 4);
    A.o_av = take((size_t)ma * 4 * t);
    A.o_ag = take((size_t)ma * NAM * t);
    A.o_agp = take((size_t)ma * NAM * t);
    A.warp_bytes = off;
    A.smem_params = (int)((L.nparams_s * t + 15) / 16 * 16);
    int wpb = kWarpsPerBlock;
    while (wpb > 1 && (size_t)A.smem_params + (size_t)wpb * A.warp_bytes > 220 * 1024) --wpb;
    const size_t smem = (size_t)A.smem_params + (size_t)wpb * A.warp_bytes;
    MATPL_REQUIRE(smem <= 220 * 1024, MATPL_ERR_UNSUPPORTED,
                  "NEP parameters and per-warp lists do not fit in shared memory "
                  "(max_nn_radial / max_nn_angular too large)");
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return check_launch("cudaFuncSetAttribute(nep_eval)");
    int dev = 0, sms = device_sms(), per_sm = 1;
    cudaGetDevice(&dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * wpb, smem);
    if (per_sm < 1) per_sm = 1;
    const long long warps = (long long)sms * per_sm * wpb;
    const long long apw = (A.natoms + warps - 1) / warps;
    const long long nwarps = (A.natoms + apw - 1) / apw;
    const int grid = (int)((nwarps + wpb - 1) / wpb);
    {
        ProfScope ps(A.feats ? "nep_descriptor" : "nep_eval", s);
        kern<<<grid, 32 * wpb, smem, s>>>(A, apw);
    }
    return check_launch("matpl_nep_eval");
}

template <typename T, bool CL>
int dispatch(const EvalArgs &A, cudaStream_t s) {
    const NepLayout &L = A.L;
    if (L.nr == 5 && L.kr == 9 && L.na == 5 && L.ka == 9)      // n_max 4, basis_size 8
        return launch_eval<T, 5, 9, 5, 9, CL, true>(A, s);
    if (L.nr <= 5 && L.kr <= 9 && L.na <= 5 && L.ka <= 9)
        return launch_eval<T, 5, 9, 5, 9, CL, false>(A, s);
    MATPL_REQUIRE(L.nr <= 8 && L.kr <= 16 && L.na <= 8 && L.ka <= 16, MATPL_ERR_UNSUPPORTED,
                  "n_max <= 7 and basis_size <= 15 are compiled");
    return launch_eval<T, 8, 16, 8, 16, CL, false>(A, s);
}

// the compact list form: float4 entries only in FP32
struct CompactLists {
    const int *NN_r, *NL_r, *NN_a, *NL_a;
    const float *Ri_r, *Ri_a;
};

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" size_t matpl_nep_param_count(const matpl_nep_model *model) {
    NepLayout L;
    if (make_layout(model, &L) != MATPL_OK) return 0;
    return (size_t)L.nparams;
}

extern "C" size_t matpl_nep_workspace_bytes(int dtype, int nframes, long long natoms) {
    if (nframes <= 0 || natoms < 0) return 0;
    return ws_layout(dtype, nframes, natoms, nullptr, nullptr, nullptr);
}

namespace matpl {
namespace {

int nep_run(int dtype, const matpl_nep_model *model, int nframes, long long natoms,
            const long long *num_atom, const long long *type_map, int max_nn_radial,
            const long long *NN_radial, const long long *NL_radial, const double *Ri_radial,
            int max_nn_angular, const long long *NN_angular, const long long *NL_angular,
            const double *Ri_angular, void *Ei, double *Etot, void *force, double *virial,
            void *feats, void *workspace, size_t workspace_bytes, void *stream,
            const CompactLists *cl = nullptr) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "NEP entry points support MATPL_F32 and MATPL_F64");
    MATPL_REQUIRE(!cl || dtype == MATPL_F32, MATPL_ERR_DTYPE,
                  "the compact (float4) list form is evaluated in MATPL_F32 only");
    NepLayout L;
    int st = make_layout(model, &L);
    if (st) return st;
    MATPL_REQUIRE(nframes > 0 && natoms >= 0, MATPL_ERR_INVALID, "bad frame / atom count");
    MATPL_REQUIRE(model->params && model->err_dev && num_atom && type_map, MATPL_ERR_INVALID,
                  "null pointer argument");
    MATPL_REQUIRE(feats || (Ei && Etot && force && virial), MATPL_ERR_INVALID,
                  "null output pointer");
    if (cl) {
        MATPL_REQUIRE(!L.two || (max_nn_radial >= 0 && cl->NN_r && cl->NL_r && cl->Ri_r),
                      MATPL_ERR_INVALID, "radial list required");
        MATPL_REQUIRE(!L.l3 || (max_nn_angular >= 0 && cl->NN_a && cl->NL_a && cl->Ri_a),
                      MATPL_ERR_INVALID, "angular list required");
        MATPL_REQUIRE(((uintptr_t)cl->Ri_r & 15u) == 0 && ((uintptr_t)cl->Ri_a & 15u) == 0,
                      MATPL_ERR_INVALID, "Ri_radial / Ri_angular must be 16-byte aligned");
    } else {
        MATPL_REQUIRE(!L.two || (max_nn_radial >= 0 && NN_radial && NL_radial && Ri_radial),
                      MATPL_ERR_INVALID, "radial list required");
        MATPL_REQUIRE(!L.l3 || (max_nn_angular >= 0 && NN_angular && NL_angular && Ri_angular),
                      MATPL_ERR_INVALID, "angular list required");
    }
    const size_t need = ws_layout(dtype, nframes, natoms, nullptr, nullptr, nullptr);
    MATPL_REQUIRE(workspace && workspace_bytes >= need, MATPL_ERR_WORKSPACE,
                  "workspace smaller than matpl_nep_workspace_bytes()");
    cudaStream_t s = as_stream(stream);
    EvalArgs A;
    A.L = L;
    A.params = model->params;
    A.natoms = natoms;
    A.nframes = nframes;
    long long *fs = nullptr;
    void *facc = nullptr;
    ws_layout(dtype, nframes, natoms, (unsigned char *)workspace, &fs, &facc);
    A.frame_start = fs;
    A.type_map = type_map;
    A.max_r = max_nn_radial;
    A.max_a = max_nn_angular;
    A.NN_r = NN_radial; A.NL_r = NL_radial; A.Ri_r = Ri_radial;
    A.NN_a = NN_angular; A.NL_a = NL_angular; A.Ri_a = Ri_angular;
    A.cNN_r = cl ? cl->NN_r : nullptr; A.cNL_r = cl ? cl->NL_r : nullptr;
    A.cNN_a = cl ? cl->NN_a : nullptr; A.cNL_a = cl ? cl->NL_a : nullptr;
    A.cRi_r = cl ? (const float4 *)cl->Ri_r : nullptr;
    A.cRi_a = cl ? (const float4 *)cl->Ri_a : nullptr;
    A.Ei = Ei;
    A.Etot = Etot;
    A.virial = virial;
    A.err = model->err_dev;
    A.facc = dtype == MATPL_F32 ? facc : force;
    A.feats = feats;
    if (!feats) {
        cudaMemsetAsync(Etot, 0, sizeof(double) * nframes, s);
        cudaMemsetAsync(virial, 0, sizeof(double) * 9 * nframes, s);
        if (dtype == MATPL_F32)
            cudaMemsetAsync(facc, 0, sizeof(float4) * (size_t)natoms, s);
        else
            cudaMemsetAsync(force, 0, sizeof(double) * 3 * (size_t)natoms, s);
    }
    nep_frame_start<<<1, 32, 0, s>>>(num_atom, nframes, natoms, fs, model->err_dev);
    if (natoms == 0) return check_launch("matpl_nep_eval");
    st = cl ? dispatch<float, true>(A, s)
            : (dtype == MATPL_F32 ? dispatch<float, false>(A, s) : dispatch<double, false>(A, s));
    if (st) return st;
    if (dtype == MATPL_F32 && !feats) {
        const long long g = (natoms + 255) / 256;
        nep_force_out<<<(int)(g > device_sms() * 8 ? device_sms() * 8 : g), 256, 0, s>>>(
            (const float4 *)facc, (float *)force, natoms);
    }
    return check_launch("matpl_nep_eval");
}

}  // namespace
}  // namespace matpl

extern "C" int matpl_nep_eval(int dtype, const matpl_nep_model *model, int nframes,
                              long long natoms, const long long *num_atom,
                              const long long *type_map, int max_nn_radial,
                              const long long *NN_radial, const long long *NL_radial,
                              const double *Ri_radial, int max_nn_angular,
                              const long long *NN_angular, const long long *NL_angular,
                              const double *Ri_angular, void *Ei, double *Etot, void *force,
                              double *virial, void *workspace, size_t workspace_bytes,
                              void *stream) {
    MATPL_REQUIRE(Ei && Etot && force && virial, MATPL_ERR_INVALID, "null output pointer");
    MATPL_REQUIRE_ON_DEVICE(force, "matpl_nep_eval");
    return nep_run(dtype, model, nframes, natoms, num_atom, type_map, max_nn_radial, NN_radial,
                   NL_radial, Ri_radial, max_nn_angular, NN_angular, NL_angular, Ri_angular, Ei,
                   Etot, force, virial, nullptr, workspace, workspace_bytes, stream);
}

extern "C" int matpl_nep_descriptor(int dtype, const matpl_nep_model *model, int nframes,
                                    long long natoms, const long long *num_atom,
                                    const long long *type_map, int max_nn_radial,
                                    const long long *NN_radial, const long long *NL_radial,
                                    const double *Ri_radial, int max_nn_angular,
                                    const long long *NN_angular, const long long *NL_angular,
                                    const double *Ri_angular, void *feats, void *workspace,
                                    size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE(feats, MATPL_ERR_INVALID, "null feats");
    MATPL_REQUIRE_ON_DEVICE(feats, "matpl_nep_descriptor");
    return nep_run(dtype, model, nframes, natoms, num_atom, type_map, max_nn_radial, NN_radial,
                   NL_radial, Ri_radial, max_nn_angular, NN_angular, NL_angular, Ri_angular,
                   nullptr, nullptr, nullptr, nullptr, feats, workspace, workspace_bytes, stream);
}

extern "C" int matpl_nep_eval_compact(int dtype, const matpl_nep_model *model, int nframes,
                                      long long natoms, const long long *num_atom,
                                      const long long *type_map, int max_nn_radial,
                                      const int *NN_radial, const int *NL_radial,
                                      const float *Ri_radial, int max_nn_angular,
                                      const int *NN_angular, const int *NL_angular,
                                      const float *Ri_angular, void *Ei, double *Etot,
                                      void *force, double *virial, void *workspace,
                                      size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE(Ei && Etot && force && virial, MATPL_ERR_INVALID, "null output pointer");
    MATPL_REQUIRE_ON_DEVICE(force, "matpl_nep_eval_compact");
    CompactLists cl{NN_radial, NL_radial, NN_angular, NL_angular, Ri_radial, Ri_angular};
    return nep_run(dtype, model, nframes, natoms, num_atom, type_map, max_nn_radial, nullptr,
                   nullptr, nullptr, max_nn_angular, nullptr, nullptr, nullptr, Ei, Etot, force,
                   virial, nullptr, workspace, workspace_bytes, stream, &cl);
}
