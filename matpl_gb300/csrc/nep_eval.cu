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

namespace matpl {
namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kMaxHidden = 128;

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

struct NepLayout {
    int ntypes, nr, kr, na, ka, nfeat, hidden;
    int two;                 // radial features (nr when train_2b, else 0)
    int l3, four, five;      // 3-body l_max (0 or 4), 4-body / 5-body present
    double rc_r_d, rc_a_d;
    int off_c2, off_c3, off_qs, off_net, net_stride;   // element offsets in params
    int nparams;
};

template <typename T> __device__ __forceinline__ void sincospi_t(T x, T *s, T *c);
template <> __device__ __forceinline__ void sincospi_t<float>(float x, float *s, float *c) {
    sincospif(x, s, c);
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
    void *Ei;
    double *Etot, *virial;
    void *facc;                     // float4 [N] (f32) or double [N, 3] (f64)
    void *feats;                    // descriptor only: q [N, F] before q_scaler, else NULL
    int *err;
};

// per-warp shared scratch (element counts, T elements)
template <int NAM> struct WarpScratch {
    static constexpr int FM = 8 + 6 * NAM;          // radial (<= 8) + angular features
    static constexpr int stash_g = 0;               // [32][NAM]
    static constexpr int stash_b = 32 * NAM;        // [32][24]
    static constexpr int s = stash_b + 32 * 24;     // [NAM][24]
    static constexpr int dEds = s + NAM * 24;       // [NAM][24]
    static constexpr int fin = dEds + NAM * 24;     // [FM] scaled features
    static constexpr int dq = fin + FM;             // [FM] dE/dq
    static constexpr int dpre = dq + FM;            // [kMaxHidden]
    static constexpr int size = dpre + kMaxHidden;
};

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

template <typename T, int NRM, int KRM, int NAM, int KAM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
nep_eval_kernel(EvalArgs A, long long atoms_per_warp) {
    using WS = WarpScratch<NAM>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *P = reinterpret_cast<T *>(smem_raw);
    const NepLayout &L = A.L;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const T *gp = reinterpret_cast<const T *>(A.params);
    for (int q = threadIdx.x; q < L.nparams; q += blockDim.x) P[q] = gp[q];
    T *W = P + ((L.nparams + 3) & ~3) + WS::size * wib;
    __syncthreads();

    const T *c2 = P + L.off_c2, *c3 = P + L.off_c3, *qs = P + L.off_qs;
    const T rc_r = (T)L.rc_r_d, rc_a = (T)L.rc_a_d;
    const T rcinv_r = T(1) / rc_r, rcinv_a = T(1) / rc_a;
    T *stash_g = W + WS::stash_g, *stash_b = W + WS::stash_b, *s_sm = W + WS::s,
      *dEds = W + WS::dEds, *fin = W + WS::fin, *dq = W + WS::dq, *dpre = W + WS::dpre;

    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    const long long a_begin = gw * atoms_per_warp;
    long long a_end = a_begin + atoms_per_warp;
    if (a_end > A.natoms) a_end = A.natoms;
    if (a_begin >= a_end) return;
    // frame of the first atom
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

    for (long long i = a_begin; i < a_end; ++i) {
        while (i >= frame_end && frame + 1 < A.nframes) {
            flush_frame<T>(A, frame, e_frame, vir, lane);
            e_frame = 0.0;
            ++frame;
            frame_end = A.frame_start[frame + 1];
        }
        const int ti = (int)A.type_map[i];
        if (ti < 0 || ti >= L.ntypes) {
            if (lane == 0) {
                atomicOr(A.err, MATPL_KERR_BAD_TYPE);
                reinterpret_cast<T *>(A.Ei)[i] = T(0);
            }
            continue;
        }
        const long long nnr = L.two ? min(A.NN_r[i], (long long)A.max_r) : 0;
        const long long nna = L.l3 ? min(A.NN_a[i], (long long)A.max_a) : 0;
        const long long row_r = i * A.max_r, row_a = i * A.max_a;

        // ---------------- radial descriptor
        T qr[NRM];
#pragma unroll
        for (int n = 0; n < NRM; ++n) qr[n] = T(0);
        for (long long sl = lane; sl < nnr; sl += 32) {
            const long long j = A.NL_r[row_r + sl];
            if (j < 0) continue;
            if (j >= A.natoms) { atomicOr(A.err, MATPL_KERR_BAD_COUNT); continue; }
            const int tj = (int)A.type_map[j];
            if (tj < 0 || tj >= L.ntypes) { atomicOr(A.err, MATPL_KERR_BAD_TYPE); continue; }
            const T r = (T)A.Ri_r[(row_r + sl) * 4];
            T f[KRM], df[KRM];
            basis<T, KRM>(r, rc_r, rcinv_r, L.kr, f, df);
            const T *c = c2 + (ti * L.ntypes + tj) * L.nr * L.kr;
#pragma unroll
            for (int n = 0; n < NRM; ++n) {
                if (n < L.nr) {
                    T g = T(0);
#pragma unroll
                    for (int k = 0; k < KRM; ++k)
                        if (k < L.kr) g += c[n * L.kr + k] * f[k];
                    qr[n] += g;
                }
            }
        }
#pragma unroll
        for (int n = 0; n < NRM; ++n) qr[n] = warp_sum(qr[n]);

        // ---------------- angular descriptor: s_nlm = sum_j g_n(r) b_lm(r_hat)
        T sacc[NAM];
#pragma unroll
        for (int n = 0; n < NAM; ++n) sacc[n] = T(0);
        for (long long base = 0; base < nna; base += 32) {
            const long long sl = base + lane;
            if (sl < nna) {
                long long j = A.NL_a[row_a + sl];
                if (j >= A.natoms) {
                    atomicOr(A.err, MATPL_KERR_BAD_COUNT);
                    j = -1;
                }
                const int tj = j >= 0 ? (int)A.type_map[j] : -1;
                const bool ok = tj >= 0 && tj < L.ntypes;
                if (j >= 0 && !ok) atomicOr(A.err, MATPL_KERR_BAD_TYPE);
                const double *rr = A.Ri_a + (row_a + sl) * 4;
                const T r = ok ? (T)rr[0] : T(0);
                T f[KAM], df[KAM];
                basis<T, KAM>(r, rc_a, rcinv_a, L.ka, f, df);
                const T *c = c3 + (ok ? (ti * L.ntypes + tj) : 0) * L.na * L.ka;
#pragma unroll
                for (int n = 0; n < NAM; ++n) {
                    T g = T(0);
                    if (n < L.na && ok) {
#pragma unroll
                        for (int k = 0; k < KAM; ++k)
                            if (k < L.ka) g += c[n * L.ka + k] * f[k];
                    }
                    stash_g[lane * NAM + n] = g;
                }
                const T rinv = ok && r > T(0) ? T(1) / r : T(0);
                const T x = (T)rr[1] * rinv, y = (T)rr[2] * rinv, z = (T)rr[3] * rinv;
#pragma unroll
                for (int lm = 0; lm < 24; ++lm) {
                    T b, gx, gy, gz;
                    harmonic<T>(lm, x, y, z, b, gx, gy, gz);
                    stash_b[lane * 24 + lm] = b;
                }
            }
            __syncwarp();
            const int cnt = (int)min(32LL, nna - base);
            if (lane < 24) {
                for (int jj = 0; jj < cnt; ++jj) {
                    const T b = stash_b[jj * 24 + lane];
#pragma unroll
                    for (int n = 0; n < NAM; ++n) sacc[n] += stash_g[jj * NAM + n] * b;
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
            const int n3 = L.l3 * L.na;
            if (fa < n3) {
                const int l = fa / L.na, n = fa - l * L.na;
                const int lo = l == 0 ? 0 : (l == 1 ? 3 : (l == 2 ? 8 : 15));
                const int hi = l == 0 ? 3 : (l == 1 ? 8 : (l == 2 ? 15 : 24));
                q = T(0);
                for (int lm = lo; lm < hi; ++lm) {
                    const T sv = s_sm[n * 24 + lm];
                    q += (T)kC3B[lm] * sv * sv;
                }
            } else if (L.four && fa < n3 + L.na) {
                const T *s = s_sm + (fa - n3) * 24;
                q = (T)kC4B[0] * s[3] * s[3] * s[3] +
                    (T)kC4B[1] * s[3] * (s[4] * s[4] + s[5] * s[5]) +
                    (T)kC4B[2] * s[3] * (s[6] * s[6] + s[7] * s[7]) +
                    (T)kC4B[3] * s[6] * (s[5] * s[5] - s[4] * s[4]) +
                    (T)kC4B[4] * s[4] * s[5] * s[7];
            } else {
                const T *s = s_sm + (fa - n3 - (L.four ? L.na : 0)) * 24;
                const T a0 = s[0] * s[0], a12 = s[1] * s[1] + s[2] * s[2];
                q = (T)kC5B[0] * a0 * a0 + (T)kC5B[1] * a0 * a12 + (T)kC5B[2] * a12 * a12;
            }
            fin[L.two + fa] = q * qs[L.two + fa];
            if (A.feats) reinterpret_cast<T *>(A.feats)[i * L.nfeat + L.two + fa] = q;
        }
        __syncwarp();
        if (A.feats) continue;            // descriptor only

        // ---------------- fitting net of element ti and its adjoint
        const T *net = P + L.off_net + ti * L.net_stride;
        const T *W0 = net, *b0 = net + L.nfeat * L.hidden, *W1 = b0 + L.hidden;
        const T b1 = W1[L.hidden];
        T e = T(0);
        for (int k = lane; k < L.hidden; k += 32) {
            T pre = b0[k];
            for (int f = 0; f < L.nfeat; ++f) pre += fin[f] * W0[f * L.hidden + k];
            const T h = dev_tanh(pre);
            e += W1[k] * h;
            dpre[k] = W1[k] * (T(1) - h * h);
        }
        const T Ei = warp_sum(e) + b1;
        __syncwarp();
        for (int f = lane; f < L.nfeat; f += 32) {
            T d = T(0);
            const T *w = W0 + f * L.hidden;
            for (int k = 0; k < L.hidden; ++k) d += w[k] * dpre[k];
            dq[f] = d * qs[f];
        }
        __syncwarp();

        // ---------------- dE/ds_nlm (lanes over lm)
        if (lane < 24 && L.l3) {
            const int lm = lane, l = l_of(lm);
            const int n3 = L.l3 * L.na;
#pragma unroll
            for (int n = 0; n < NAM; ++n) {
                if (n >= L.na) {              // rows past n_max are read (times zero) below
                    dEds[n * 24 + lm] = T(0);
                    continue;
                }
                const T *s = s_sm + n * 24;
                T d = dq[L.two + l * L.na + n] * T(2) * (T)kC3B[lm] * s[lm];
                if (L.four && lm >= 3 && lm <= 7) {
                    const T g4 = dq[L.two + n3 + n];
                    T dd;
                    if (lm == 3)
                        dd = T(3) * (T)kC4B[0] * s[3] * s[3] +
                             (T)kC4B[1] * (s[4] * s[4] + s[5] * s[5]) +
                             (T)kC4B[2] * (s[6] * s[6] + s[7] * s[7]);
                    else if (lm == 4)
                        dd = T(2) * (T)kC4B[1] * s[3] * s[4] - T(2) * (T)kC4B[3] * s[6] * s[4] +
                             (T)kC4B[4] * s[5] * s[7];
                    else if (lm == 5)
                        dd = T(2) * (T)kC4B[1] * s[3] * s[5] + T(2) * (T)kC4B[3] * s[6] * s[5] +
                             (T)kC4B[4] * s[4] * s[7];
                    else if (lm == 6)
                        dd = T(2) * (T)kC4B[2] * s[3] * s[6] +
                             (T)kC4B[3] * (s[5] * s[5] - s[4] * s[4]);
                    else
                        dd = T(2) * (T)kC4B[2] * s[3] * s[7] + (T)kC4B[4] * s[4] * s[5];
                    d += g4 * dd;
                }
                if (L.five && lm <= 2) {
                    const T g5 = dq[L.two + n3 + (L.four ? L.na : 0) + n];
                    const T a0 = s[0] * s[0], a12 = s[1] * s[1] + s[2] * s[2];
                    const T dd = lm == 0
                                     ? T(4) * (T)kC5B[0] * a0 * s[0] + T(2) * (T)kC5B[1] * s[0] * a12
                                     : T(2) * (T)kC5B[1] * a0 * s[lm] +
                                           T(4) * (T)kC5B[2] * a12 * s[lm];
                    d += g5 * dd;
                }
                dEds[n * 24 + lm] = d;
            }
        }
        __syncwarp();

        // ---------------- forces: radial pairs
        T fi0 = T(0), fi1 = T(0), fi2 = T(0);
        for (long long sl = lane; sl < nnr; sl += 32) {
            const long long j = A.NL_r[row_r + sl];
            if (j < 0 || j >= A.natoms) continue;
            const int tj = (int)A.type_map[j];
            if (tj < 0 || tj >= L.ntypes) continue;
            const double *rr = A.Ri_r + (row_r + sl) * 4;
            const T r = (T)rr[0], x = (T)rr[1], y = (T)rr[2], z = (T)rr[3];
            if (!(r > T(0))) continue;
            T f[KRM], df[KRM];
            basis<T, KRM>(r, rc_r, rcinv_r, L.kr, f, df);
            const T *c = c2 + (ti * L.ntypes + tj) * L.nr * L.kr;
            T dEdr = T(0);
#pragma unroll
            for (int n = 0; n < NRM; ++n) {
                if (n < L.nr) {
                    T gp = T(0);
#pragma unroll
                    for (int k = 0; k < KRM; ++k)
                        if (k < L.kr) gp += c[n * L.kr + k] * df[k];
                    dEdr += dq[n] * gp;
                }
            }
            const T s = dEdr / r;
            const T fx = s * x, fy = s * y, fz = s * z;
            fi0 += fx; fi1 += fy; fi2 += fz;
            add_force<T>(A.facc, j, -fx, -fy, -fz);
            vir[0] -= fx * x; vir[1] -= fx * y; vir[2] -= fx * z;
            vir[3] -= fy * x; vir[4] -= fy * y; vir[5] -= fy * z;
            vir[6] -= fz * x; vir[7] -= fz * y; vir[8] -= fz * z;
        }

        // ---------------- forces: angular pairs
        for (long long sl = lane; sl < nna; sl += 32) {
            const long long j = A.NL_a[row_a + sl];
            if (j < 0 || j >= A.natoms) continue;
            const int tj = (int)A.type_map[j];
            if (tj < 0 || tj >= L.ntypes) continue;
            const double *rr = A.Ri_a + (row_a + sl) * 4;
            const T r = (T)rr[0], x = (T)rr[1], y = (T)rr[2], z = (T)rr[3];
            if (!(r > T(0))) continue;
            T f[KAM], df[KAM];
            basis<T, KAM>(r, rc_a, rcinv_a, L.ka, f, df);
            const T *c = c3 + (ti * L.ntypes + tj) * L.na * L.ka;
            T g[NAM], gp[NAM], An[NAM];
#pragma unroll
            for (int n = 0; n < NAM; ++n) {
                T a = T(0), b = T(0);
                if (n < L.na) {
#pragma unroll
                    for (int k = 0; k < KAM; ++k)
                        if (k < L.ka) {
                            a += c[n * L.ka + k] * f[k];
                            b += c[n * L.ka + k] * df[k];
                        }
                }
                g[n] = a; gp[n] = b; An[n] = T(0);
            }
            const T rinv = T(1) / r;
            const T ux = x * rinv, uy = y * rinv, uz = z * rinv;
            T G0 = T(0), G1 = T(0), G2 = T(0);
#pragma unroll
            for (int lm = 0; lm < 24; ++lm) {
                T b, gx, gy, gz;
                harmonic<T>(lm, ux, uy, uz, b, gx, gy, gz);
                T Bl = T(0);
#pragma unroll
                for (int n = 0; n < NAM; ++n) {
                    const T d = dEds[n * 24 + lm];
                    Bl += d * g[n];
                    An[n] += d * b;
                }
                G0 += Bl * gx; G1 += Bl * gy; G2 += Bl * gz;
            }
            T dEdr = T(0);
#pragma unroll
            for (int n = 0; n < NAM; ++n) dEdr += gp[n] * An[n];
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
    flush_frame<T>(A, frame, e_frame, vir, lane);
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

template <typename T, int NRM, int KRM, int NAM, int KAM>
int launch_eval(const EvalArgs &A0, cudaStream_t s) {
    EvalArgs A = A0;
    auto kern = nep_eval_kernel<T, NRM, KRM, NAM, KAM>;
    const size_t pbytes = (size_t)((A.L.nparams + 3) & ~3) * sizeof(T);
    const size_t wbytes = (size_t)WarpScratch<NAM>::size * sizeof(T);
    int wpb = kWarpsPerBlock;
    while (wpb > 1 && pbytes + wpb * wbytes > 220 * 1024) --wpb;
    const size_t smem = pbytes + wpb * wbytes;
    MATPL_REQUIRE(smem <= 220 * 1024, MATPL_ERR_UNSUPPORTED,
                  "NEP parameters do not fit in shared memory");
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return check_launch("cudaFuncSetAttribute(nep_eval)");
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * wpb, smem);
    if (per_sm < 1) per_sm = 1;
    const long long warps = (long long)sms * per_sm * wpb;
    const long long apw = (A.natoms + warps - 1) / warps;
    const long long nwarps = (A.natoms + apw - 1) / apw;
    const int grid = (int)((nwarps + wpb - 1) / wpb);
    {
        ProfScope ps("nep_eval", s);
        kern<<<grid, 32 * wpb, smem, s>>>(A, apw);
    }
    return check_launch("matpl_nep_eval");
}

template <typename T>
int dispatch(const EvalArgs &A, cudaStream_t s) {
    const NepLayout &L = A.L;
    if (L.nr <= 5 && L.kr <= 9 && L.na <= 5 && L.ka <= 9)
        return launch_eval<T, 5, 9, 5, 9>(A, s);
    MATPL_REQUIRE(L.nr <= 8 && L.kr <= 16 && L.na <= 8 && L.ka <= 16, MATPL_ERR_UNSUPPORTED,
                  "n_max <= 7 and basis_size <= 15 are compiled");
    return launch_eval<T, 8, 16, 8, 16>(A, s);
}

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
            void *feats, void *workspace, size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "NEP entry points support MATPL_F32 and MATPL_F64");
    NepLayout L;
    int st = make_layout(model, &L);
    if (st) return st;
    MATPL_REQUIRE(nframes > 0 && natoms >= 0, MATPL_ERR_INVALID, "bad frame / atom count");
    MATPL_REQUIRE(model->params && model->err_dev && num_atom && type_map, MATPL_ERR_INVALID,
                  "null pointer argument");
    MATPL_REQUIRE(feats || (Ei && Etot && force && virial), MATPL_ERR_INVALID,
                  "null output pointer");
    MATPL_REQUIRE(!L.two || (max_nn_radial >= 0 && NN_radial && NL_radial && Ri_radial),
                  MATPL_ERR_INVALID, "radial list required");
    MATPL_REQUIRE(!L.l3 || (max_nn_angular >= 0 && NN_angular && NL_angular && Ri_angular),
                  MATPL_ERR_INVALID, "angular list required");
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
    st = dtype == MATPL_F32 ? dispatch<float>(A, s) : dispatch<double>(A, s);
    if (st) return st;
    if (dtype == MATPL_F32 && !feats) {
        const long long g = (natoms + 255) / 256;
        nep_force_out<<<(int)(g > 152 * 8 ? 152 * 8 : g), 256, 0, s>>>(
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
    return nep_run(dtype, model, nframes, natoms, num_atom, type_map, max_nn_radial, NN_radial,
                   NL_radial, Ri_radial, max_nn_angular, NN_angular, NL_angular, Ri_angular,
                   nullptr, nullptr, nullptr, nullptr, feats, workspace, workspace_bytes, stream);
}
