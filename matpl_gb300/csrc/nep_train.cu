// NEP training operators: the descriptor of one neighbor list with its first and second
// derivatives, the drop-in for CalcOps calculateNepFeat (radial, src/op/src/CalcOps.cpp:385-680)
// and calculateNepMbFeat (3-/4-/5-body, CalcOps.cpp:680-1023) with their Grad functions.
//
// For a descriptor q(c, d12) of one list (d12 [N, NN, 4] = (r, x, y, z) of every slot, c the
// coefficients [T, T, n, K]) and the features' gradient G = dL/dq [N, F]:
//   FWD   q [N, F]
//   BWD   grad_d12 = G . dq/dd12 [N, NN, 4] and W (either may be skipped), from which dL/dc
//         follows by a sum over the atoms of each centre type (matpl_nep_cgrad):
//           radial   W [N, T, K] = sum over neighbors j of type t of f_k(r_ij),
//                    dL/dc[ti, t, n, k] = sum_i G[i, n] W[i, t, k];
//           angular  W [N, T, n, K] = sum_j of type t of f_k(r_ij) sum_m Sbar_nm b_m(r_ij),
//                    Sbar = G . dq/ds (s_nm = sum_j g_n b_m), dL/dc[ti] = sum_i W[i].
//   BWD2  for H = dL/d(grad_d12) [N, NN, 4] (the second backward of the Grad function):
//         gso = dq/dd12 . H [N, F] (the gradient of L with respect to G) and W2 [N, T, n, K]
//         with dL/dc[ti] = sum_i W2[i] (radial: W2 [N, T, K] = sum_j H_r f_k'(r), times G).
// The derivatives are those of the reference's CPU descriptor (nep_net.py:651-870) under
// autograd, i.e. partial derivatives in the four columns of d12 taken as independent inputs:
// f_k depends on r, b_lm on (x, y, z) / r.
// One warp per centre atom, lanes over its slots 32 at a time; per-pair values are staged in
// shared memory and lanes switch to (n, lm) or (t, n, k) entries for the sums over pairs.
#include <algorithm>

#include "common.cuh"
#include "nep_math.cuh"

namespace matpl {
namespace {

constexpr int kFeatWarps = 4;
enum { kFwd = 0, kBwd = 1, kBwd2 = 2 };

struct FeatArgs {
    int natoms, nn, ntypes, nmax, nbase;
    double rc;
    const void *coeff;          // [T, T, nmax, nbase]
    const void *d12;            // [N, nn, 4]
    const long long *NL;        // [N, nn], -1 = empty
    const long long *type;      // [N]
    const void *G;              // [N, ldG] dL/dq (BWD, BWD2)
    long long ldG;
    const void *H;              // [N, nn, 4] (BWD2)
    void *q;                    // [N, ldQ] (FWD) or gso (BWD2)
    long long ldQ;
    void *grad_d12;             // [N, nn, 4] (BWD), zero-filled by the caller
    void *W;                    // partial c-gradient per atom, zero-filled by the caller
    int l3, four, five;         // angular: l_max of the 3-body part, 4-/5-body present
    int *err;
};

template <typename T>
__device__ __forceinline__ T ld(const void *p, long long k) { return static_cast<const T *>(p)[k]; }

// ---------------------------------------------------------------- radial (calculateNepFeat)
template <typename T, int MODE, int NM, int KM>
__global__ void __launch_bounds__(32 * kFeatWarps) nep2b_op(FeatArgs A) {
    __shared__ T s_st[kFeatWarps][32][KM + 1];
    __shared__ int s_tj[kFeatWarps][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int T_ = A.ntypes, n_ = A.nmax, K = A.nbase;
    const T rc = (T)A.rc, rcinv = T(1) / rc;
    const T *c = static_cast<const T *>(A.coeff);
    const long long gw = (long long)blockIdx.x * kFeatWarps + wib;
    const long long nw = (long long)gridDim.x * kFeatWarps;
    for (long long i = gw; i < A.natoms; i += nw) {
        const int ti = (int)A.type[i];
        if (ti < 0 || ti >= T_) {
            if (lane == 0) atomicOr(A.err, MATPL_KERR_BAD_TYPE);
            continue;
        }
        T G[NM], acc[NM];
#pragma unroll
        for (int n = 0; n < NM; ++n) {
            acc[n] = T(0);
            G[n] = (MODE != kFwd && n < n_) ? ld<T>(A.G, i * A.ldG + n) : T(0);
        }
        for (int base = 0; base < A.nn; base += 32) {
            const int slot = base + lane;
            const long long ps = i * A.nn + slot;
            const long long j = slot < A.nn ? A.NL[ps] : -1;
            const bool ok = j >= 0 && j < A.natoms;
            if (j >= A.natoms) atomicOr(A.err, MATPL_KERR_BAD_COUNT);
            if (!__any_sync(0xffffffffu, ok)) break;
            T f[KM], df[KM];
            int tj = -1;
            if (ok) {
                tj = (int)A.type[j];
                if (tj < 0 || tj >= T_) {
                    atomicOr(A.err, MATPL_KERR_BAD_TYPE);
                    tj = -1;
                }
            }
            const bool use = ok && tj >= 0;
            const T r = use ? ld<T>(A.d12, ps * 4) : T(0);
            basis<T, KM>(r, rc, rcinv, K, f, df);
            const T *cr = c + ((long long)(ti * T_ + (tj < 0 ? 0 : tj)) * n_) * K;
            if (MODE == kFwd) {
                if (use)
#pragma unroll
                    for (int n = 0; n < NM; ++n) {
                        if (n >= n_) break;
                        T g = T(0);
#pragma unroll
                        for (int k = 0; k < KM; ++k)
                            if (k < K) g += cr[n * K + k] * f[k];
                        acc[n] += g;
                    }
            } else if (MODE == kBwd) {
                if (use && A.grad_d12) {
                    T gp = T(0);
#pragma unroll
                    for (int n = 0; n < NM; ++n) {
                        if (n >= n_) break;
                        T d = T(0);
#pragma unroll
                        for (int k = 0; k < KM; ++k)
                            if (k < K) d += cr[n * K + k] * df[k];
                        gp += G[n] * d;
                    }
                    static_cast<T *>(A.grad_d12)[ps * 4] = gp;
                }
#pragma unroll
                for (int k = 0; k < KM; ++k) s_st[wib][lane][k] = use ? f[k] : T(0);
                s_tj[wib][lane] = use ? tj : -1;
            } else {
                const T h0 = use ? ld<T>(A.H, ps * 4) : T(0);
                if (use)
#pragma unroll
                    for (int n = 0; n < NM; ++n) {
                        if (n >= n_) break;
                        T d = T(0);
#pragma unroll
                        for (int k = 0; k < KM; ++k)
                            if (k < K) d += cr[n * K + k] * df[k];
                        acc[n] += h0 * d;
                    }
#pragma unroll
                for (int k = 0; k < KM; ++k) s_st[wib][lane][k] = use ? h0 * df[k] : T(0);
                s_tj[wib][lane] = use ? tj : -1;
            }
            if (MODE == kBwd2 || (MODE == kBwd && A.W)) {
                __syncwarp();
                T *W = static_cast<T *>(A.W) + i * (long long)T_ * K;
                for (int e = lane; e < T_ * K; e += 32) {
                    const int t = e / K, k = e - t * K;
                    T sum = T(0);
                    for (int p = 0; p < 32; ++p)
                        if (s_tj[wib][p] == t) sum += s_st[wib][p][k];
                    W[e] += sum;
                }
                __syncwarp();
            }
        }
        if (MODE != kBwd) {
#pragma unroll
            for (int n = 0; n < NM; ++n) {
                const T v = warp_sum(acc[n]);
                if (lane == 0 && n < n_) static_cast<T *>(A.q)[i * A.ldQ + n] = v;
            }
        }
    }
}

// ---------------------------------------------------------------- angular (calculateNepMbFeat)
// feature index of the 3-body (l, n), the 4-body n and the 5-body n (l-major, then n)
__device__ __forceinline__ int f3(int l, int n, int nmax) { return l * nmax + n; }

// dq_f / ds_m for the features of one n (3-body of l(m), 4-body, 5-body) contracted with G:
// returns sum_f G_f dq_f/ds_m.  sv = s_n[0..23] of this atom; c3 = the 3-body constants in
// shared memory (lanes index them by their own m).
template <typename T>
__device__ __forceinline__ T sbar_of(const T *c3, int m, const T *sv, T g3, T g4, T g5, bool four,
                                     bool five) {
    T v = g3 * T(2) * c3[m] * sv[m];
    if (four && m >= 3 && m <= 7) {
        const T s3 = sv[3], s4 = sv[4], s5 = sv[5], s6 = sv[6], s7 = sv[7];
        T d;
        if (m == 3) d = T(3) * C4<T>(0) * s3 * s3 + C4<T>(1) * (s4 * s4 + s5 * s5) +
                        C4<T>(2) * (s6 * s6 + s7 * s7);
        else if (m == 4) d = T(2) * C4<T>(1) * s3 * s4 - T(2) * C4<T>(3) * s6 * s4 + C4<T>(4) * s5 * s7;
        else if (m == 5) d = T(2) * C4<T>(1) * s3 * s5 + T(2) * C4<T>(3) * s6 * s5 + C4<T>(4) * s4 * s7;
        else if (m == 6) d = T(2) * C4<T>(2) * s3 * s6 + C4<T>(3) * (s5 * s5 - s4 * s4);
        else d = T(2) * C4<T>(2) * s3 * s7 + C4<T>(4) * s4 * s5;
        v += g4 * d;
    }
    if (five && m <= 2) {
        const T a0 = sv[0] * sv[0], a12 = sv[1] * sv[1] + sv[2] * sv[2];
        const T da = m == 0 ? T(2) * C5<T>(0) * a0 + C5<T>(1) * a12 : C5<T>(1) * a0 + T(2) * C5<T>(2) * a12;
        v += g5 * da * T(2) * sv[m];
    }
    return v;
}

// the derivative of sbar_of along sd (Hessian of q in s times sd, contracted with G)
template <typename T>
__device__ __forceinline__ T sbar_dot(const T *c3, int m, const T *sv, const T *sd, T g3, T g4,
                                      T g5, bool four, bool five) {
    T v = g3 * T(2) * c3[m] * sd[m];
    if (four && m >= 3 && m <= 7) {
        const T s3 = sv[3], s4 = sv[4], s5 = sv[5], s6 = sv[6], s7 = sv[7];
        const T d3 = sd[3], d4 = sd[4], d5 = sd[5], d6 = sd[6], d7 = sd[7];
        T d;
        if (m == 3) d = T(6) * C4<T>(0) * s3 * d3 + T(2) * C4<T>(1) * (s4 * d4 + s5 * d5) +
                        T(2) * C4<T>(2) * (s6 * d6 + s7 * d7);
        else if (m == 4) d = T(2) * C4<T>(1) * (d3 * s4 + s3 * d4) - T(2) * C4<T>(3) * (d6 * s4 + s6 * d4) +
                             C4<T>(4) * (d5 * s7 + s5 * d7);
        else if (m == 5) d = T(2) * C4<T>(1) * (d3 * s5 + s3 * d5) + T(2) * C4<T>(3) * (d6 * s5 + s6 * d5) +
                             C4<T>(4) * (d4 * s7 + s4 * d7);
        else if (m == 6) d = T(2) * C4<T>(2) * (d3 * s6 + s3 * d6) + T(2) * C4<T>(3) * (s5 * d5 - s4 * d4);
        else d = T(2) * C4<T>(2) * (d3 * s7 + s3 * d7) + C4<T>(4) * (d4 * s5 + s4 * d5);
        v += g4 * d;
    }
    if (five && m <= 2) {
        const T a0 = sv[0] * sv[0], a12 = sv[1] * sv[1] + sv[2] * sv[2];
        const T a0d = T(2) * sv[0] * sd[0], a12d = T(2) * (sv[1] * sd[1] + sv[2] * sd[2]);
        T da, dad;
        if (m == 0) {
            da = T(2) * C5<T>(0) * a0 + C5<T>(1) * a12;
            dad = T(2) * C5<T>(0) * a0d + C5<T>(1) * a12d;
        } else {
            da = C5<T>(1) * a0 + T(2) * C5<T>(2) * a12;
            dad = C5<T>(1) * a0d + T(2) * C5<T>(2) * a12d;
        }
        v += g5 * (dad * T(2) * sv[m] + da * T(2) * sd[m]);
    }
    return v;
}

// per warp shared memory of the angular operator
template <typename T, int NM, int KM>
struct MbSmem {
    T s[NM][24], sd[NM][24], sb[NM][24], sbd[NM][24];
    T ga[32][NM], gb[32][NM];        // pass 1: g_n, g_n dot; pass 2: B_n / P_n, Q_n
    T ba[32][25], bb[32][25];        // pass 1: b_m, b_m dot
    T fa[32][KM + 1], fb[32][KM + 1];// pass 2: f_k, f_k'
    int tj[32];
};

// pair quantities of slot ps: f, f' (K), g_n, g_n' (n), the unit vector and 1/r (0 outside
// (1e-5, rc), where b_lm is zero)
template <typename T, int NM, int KM>
__device__ __forceinline__ void mb_pair(const FeatArgs &A, const T *cr, long long ps, T *f, T *df, T *g,
                                        T *gp, T &ux, T &uy, T &uz, T &ri) {
    const T rc = (T)A.rc, rcinv = T(1) / rc;
    const T r = ld<T>(A.d12, ps * 4);
    basis<T, KM>(r, rc, rcinv, A.nbase, f, df);
#pragma unroll
    for (int n = 0; n < NM; ++n) {
        T a = T(0), d = T(0);
        if (n < A.nmax)
#pragma unroll
            for (int k = 0; k < KM; ++k)
                if (k < A.nbase) {
                    a += cr[n * A.nbase + k] * f[k];
                    d += cr[n * A.nbase + k] * df[k];
                }
        g[n] = a;
        gp[n] = d;
    }
    const bool in = r < rc && r > T(1e-5);
    ri = in ? T(1) / r : T(0);
    ux = ld<T>(A.d12, ps * 4 + 1) * ri;
    uy = ld<T>(A.d12, ps * 4 + 2) * ri;
    uz = ld<T>(A.d12, ps * 4 + 3) * ri;
}

// b_m and its partials in r and in (x, y, z) (= grad_u b / r; d/dr = -(u . grad_u b) / r)
template <typename T>
__device__ __forceinline__ void harm_d(int m, T ux, T uy, T uz, T ri, T &b, T &br, T &bx, T &by,
                                       T &bz) {
    T v, gx, gy, gz;
    harmonic<T>(m, ux, uy, uz, v, gx, gy, gz);
    b = ri != T(0) ? v : T(0);
    bx = gx * ri;
    by = gy * ri;
    bz = gz * ri;
    br = -(gx * ux + gy * uy + gz * uz) * ri;
}

template <typename T, int MODE, int NM, int KM>
__global__ void __launch_bounds__(32 * kFeatWarps) nepmb_op(FeatArgs A) {
    extern __shared__ __align__(16) unsigned char mb_raw[];
    using Sm = MbSmem<T, NM, KM>;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Sm &S = reinterpret_cast<Sm *>(mb_raw)[wib];
    const int T_ = A.ntypes, n_ = A.nmax, K = A.nbase;
    const bool four = A.four, five = A.five;
    const T *c = static_cast<const T *>(A.coeff);
    const long long gw = (long long)blockIdx.x * kFeatWarps + wib;
    const long long nw = (long long)gridDim.x * kFeatWarps;
    const int nlm = n_ * 24;
    // the 3-body constants in shared memory: lane-varying indices into __constant__ memory are
    // served one address at a time
    __shared__ T c3s[24];
    if (threadIdx.x < 24) c3s[threadIdx.x] = C3<T>(threadIdx.x);
    __syncthreads();
    for (long long i = gw; i < A.natoms; i += nw) {
        const int ti = (int)A.type[i];
        if (ti < 0 || ti >= T_) {
            if (lane == 0) atomicOr(A.err, MATPL_KERR_BAD_TYPE);
            continue;
        }
        // ---- pass 1: s_nm (and its tangent along H)
        T sacc[6], sdacc[6];     // entries e = lane + 32 q of the n x 24 table (n <= 8)
#pragma unroll
        for (int q = 0; q < 6; ++q) sacc[q] = sdacc[q] = T(0);
        int nvalid = 0;
        for (int base = 0; base < A.nn; base += 32) {
            const int slot = base + lane;
            const long long ps = i * A.nn + slot;
            const long long j = slot < A.nn ? A.NL[ps] : -1;
            bool ok = j >= 0 && j < A.natoms;
            if (j >= A.natoms) atomicOr(A.err, MATPL_KERR_BAD_COUNT);
            if (!__any_sync(0xffffffffu, ok)) break;
            nvalid = base + 32;
            int tj = ok ? (int)A.type[j] : -1;
            if (ok && (tj < 0 || tj >= T_)) {
                atomicOr(A.err, MATPL_KERR_BAD_TYPE);
                ok = false;
            }
            T f[KM], df[KM], g[NM], gp[NM], ux, uy, uz, ri;
            const T *cr = c + ((long long)(ti * T_ + (ok ? tj : 0)) * n_) * K;
            mb_pair<T, NM, KM>(A, cr, ok ? ps : 0, f, df, g, gp, ux, uy, uz, ri);
            T h0 = T(0), h1 = T(0), h2 = T(0), h3 = T(0);
            if (MODE == kBwd2 && ok) {
                h0 = ld<T>(A.H, ps * 4);
                h1 = ld<T>(A.H, ps * 4 + 1);
                h2 = ld<T>(A.H, ps * 4 + 2);
                h3 = ld<T>(A.H, ps * 4 + 3);
            }
#pragma unroll
            for (int n = 0; n < NM; ++n) {
                S.ga[lane][n] = ok ? g[n] : T(0);
                if (MODE == kBwd2) S.gb[lane][n] = ok ? gp[n] * h0 : T(0);
            }
#pragma unroll
            for (int m = 0; m < 24; ++m) {
                T b, br, bx, by, bz;
                harm_d<T>(m, ux, uy, uz, ri, b, br, bx, by, bz);
                S.ba[lane][m] = ok ? b : T(0);
                if (MODE == kBwd2)
                    S.bb[lane][m] = ok ? br * h0 + bx * h1 + by * h2 + bz * h3 : T(0);
            }
            __syncwarp();
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const int e = lane + 32 * q;
                if (e < nlm) {
                    const int n = e / 24, m = e - n * 24;
                    T a = T(0), d = T(0);
                    for (int p = 0; p < 32; ++p) {
                        a += S.ga[p][n] * S.ba[p][m];
                        if (MODE == kBwd2) d += S.gb[p][n] * S.ba[p][m] + S.ga[p][n] * S.bb[p][m];
                    }
                    sacc[q] += a;
                    sdacc[q] += d;
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int e = lane + 32 * q;
            if (e < nlm) {
                S.s[e / 24][e % 24] = sacc[q];
                S.sd[e / 24][e % 24] = sdacc[q];
            }
        }
        __syncwarp();
        // ---- features (FWD) / their tangent (BWD2); Sbar, Sbar dot (BWD, BWD2)
        if (MODE == kFwd || MODE == kBwd2) {
            T *out = static_cast<T *>(A.q) + i * A.ldQ;
            for (int e = lane; e < n_ * (A.l3 + four + five); e += 32) {
                const int blk = e / n_, n = e - blk * n_;
                const T *sv = S.s[n];
                const T *sd = S.sd[n];
                T v = T(0);
                if (blk < A.l3) {
                    const int m0 = blk == 0 ? 0 : blk == 1 ? 3 : blk == 2 ? 8 : 15;
                    const int m1 = blk == 0 ? 3 : blk == 1 ? 8 : blk == 2 ? 15 : 24;
                    for (int m = m0; m < m1; ++m)
                        v += MODE == kFwd ? c3s[m] * sv[m] * sv[m] : T(2) * c3s[m] * sv[m] * sd[m];
                } else if (four && blk == A.l3) {
                    if (MODE == kFwd) {
                        const T s3 = sv[3], s4 = sv[4], s5 = sv[5], s6 = sv[6], s7 = sv[7];
                        v = C4<T>(0) * s3 * s3 * s3 + C4<T>(1) * s3 * (s4 * s4 + s5 * s5) +
                            C4<T>(2) * s3 * (s6 * s6 + s7 * s7) + C4<T>(3) * s6 * (s5 * s5 - s4 * s4) +
                            C4<T>(4) * s4 * s5 * s7;
                    } else {
                        for (int m = 3; m <= 7; ++m)
                            v += sbar_of<T>(c3s, m, sv, T(0), T(1), T(0), true, false) * sd[m];
                    }
                } else {
                    if (MODE == kFwd) {
                        const T a0 = sv[0] * sv[0], a12 = sv[1] * sv[1] + sv[2] * sv[2];
                        v = C5<T>(0) * a0 * a0 + C5<T>(1) * a0 * a12 + C5<T>(2) * a12 * a12;
                    } else {
                        for (int m = 0; m <= 2; ++m)
                            v += sbar_of<T>(c3s, m, sv, T(0), T(0), T(1), false, true) * sd[m];
                    }
                }
                out[blk * n_ + n] = v;
            }
        }
        if (MODE == kFwd) continue;
        const T *Gr = static_cast<const T *>(A.G) + i * A.ldG;
        for (int e = lane; e < nlm; e += 32) {
            const int n = e / 24, m = e - n * 24;
            const int l = l_of(m);
            const T g3 = l < A.l3 ? Gr[f3(l, n, n_)] : T(0);
            const T g4 = four ? Gr[A.l3 * n_ + n] : T(0);
            const T g5 = five ? Gr[(A.l3 + four) * n_ + n] : T(0);
            S.sb[n][m] = sbar_of<T>(c3s, m, S.s[n], g3, g4, g5, four, five);
            if (MODE == kBwd2)
                S.sbd[n][m] = sbar_dot<T>(c3s, m, S.s[n], S.sd[n], g3, g4, g5, four, five);
        }
        __syncwarp();
        // ---- pass 2: grad_d12 (BWD) and the per-atom c-gradient table W (either may be
        // skipped in BWD: null pointer)
        T *W = A.W ? static_cast<T *>(A.W) + i * (long long)T_ * n_ * K : nullptr;
        for (int base = 0; base < nvalid; base += 32) {
            const int slot = base + lane;
            const long long ps = i * A.nn + slot;
            const long long j = slot < A.nn ? A.NL[ps] : -1;
            int tj = (j >= 0 && j < A.natoms) ? (int)A.type[j] : -1;
            const bool ok = tj >= 0 && tj < T_;
            T f[KM], df[KM], g[NM], gp[NM], ux, uy, uz, ri;
            const T *cr = c + ((long long)(ti * T_ + (ok ? tj : 0)) * n_) * K;
            mb_pair<T, NM, KM>(A, cr, ok ? ps : 0, f, df, g, gp, ux, uy, uz, ri);
            if (MODE == kBwd && !A.grad_d12) {
                // c-gradient only: B_n = sum_m Sbar_nm b_m
                T Bn[NM];
#pragma unroll
                for (int n = 0; n < NM; ++n) Bn[n] = T(0);
#pragma unroll
                for (int m = 0; m < 24; ++m) {
                    T b, br, bx, by, bz;
                    harm_d<T>(m, ux, uy, uz, ri, b, br, bx, by, bz);
#pragma unroll
                    for (int n = 0; n < NM; ++n) Bn[n] += (n < n_ ? S.sb[n][m] : T(0)) * b;
                }
#pragma unroll
                for (int n = 0; n < NM; ++n) S.ga[lane][n] = ok ? Bn[n] : T(0);
            } else if (MODE == kBwd) {
                T Bn[NM], Br[NM], Bx[NM], By[NM], Bz[NM];
#pragma unroll
                for (int n = 0; n < NM; ++n) Bn[n] = Br[n] = Bx[n] = By[n] = Bz[n] = T(0);
#pragma unroll
                for (int m = 0; m < 24; ++m) {
                    T b, br, bx, by, bz;
                    harm_d<T>(m, ux, uy, uz, ri, b, br, bx, by, bz);
#pragma unroll
                    for (int n = 0; n < NM; ++n) {
                        const T w = n < n_ ? S.sb[n][m] : T(0);
                        Bn[n] += w * b;
                        Br[n] += w * br;
                        Bx[n] += w * bx;
                        By[n] += w * by;
                        Bz[n] += w * bz;
                    }
                }
                T c0 = T(0), cx = T(0), cy = T(0), cz = T(0);
#pragma unroll
                for (int n = 0; n < NM; ++n) {
                    c0 += gp[n] * Bn[n] + g[n] * Br[n];
                    cx += g[n] * Bx[n];
                    cy += g[n] * By[n];
                    cz += g[n] * Bz[n];
                    S.ga[lane][n] = ok ? Bn[n] : T(0);
                }
                if (ok) {
                    T *o = static_cast<T *>(A.grad_d12) + ps * 4;
                    o[0] = c0;
                    o[1] = cx;
                    o[2] = cy;
                    o[3] = cz;
                }
            } else {
                T h0 = T(0), h1 = T(0), h2 = T(0), h3 = T(0);
                if (ok) {
                    h0 = ld<T>(A.H, ps * 4);
                    h1 = ld<T>(A.H, ps * 4 + 1);
                    h2 = ld<T>(A.H, ps * 4 + 2);
                    h3 = ld<T>(A.H, ps * 4 + 3);
                }
                T P[NM], Q[NM];
#pragma unroll
                for (int n = 0; n < NM; ++n) P[n] = Q[n] = T(0);
#pragma unroll
                for (int m = 0; m < 24; ++m) {
                    T b, br, bx, by, bz;
                    harm_d<T>(m, ux, uy, uz, ri, b, br, bx, by, bz);
                    const T bd = br * h0 + bx * h1 + by * h2 + bz * h3;
#pragma unroll
                    for (int n = 0; n < NM; ++n) {
                        const T w = n < n_ ? S.sb[n][m] : T(0);
                        const T wd = n < n_ ? S.sbd[n][m] : T(0);
                        P[n] += w * b;
                        Q[n] += w * bd + wd * b;
                    }
                }
#pragma unroll
                for (int n = 0; n < NM; ++n) {
                    S.ga[lane][n] = ok ? P[n] * h0 : T(0);
                    S.gb[lane][n] = ok ? Q[n] : T(0);
                }
            }
            if (MODE == kBwd && !A.W) continue;     // grad_d12 only
#pragma unroll
            for (int k = 0; k < KM; ++k) {
                S.fa[lane][k] = ok ? f[k] : T(0);
                S.fb[lane][k] = ok ? df[k] : T(0);
            }
            S.tj[lane] = ok ? tj : -1;
            __syncwarp();
            for (int e = lane; e < T_ * n_ * K; e += 32) {
                const int t = e / (n_ * K), rem = e - t * n_ * K, n = rem / K, k = rem - n * K;
                T sum = T(0);
                for (int p = 0; p < 32; ++p) {
                    if (S.tj[p] != t) continue;
                    if (MODE == kBwd) sum += S.ga[p][n] * S.fa[p][k];
                    else sum += S.ga[p][n] * S.fb[p][k] + S.gb[p][n] * S.fa[p][k];
                }
                W[e] += sum;
            }
            __syncwarp();
        }
    }
}

template <typename T, int MODE, int NM, int KM>
int launch_mb(const FeatArgs &A, cudaStream_t s) {
    const size_t smem = sizeof(MbSmem<T, NM, KM>) * kFeatWarps;
    auto k = nepmb_op<T, MODE, NM, KM>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) {
        set_error("matpl_nep_feat: shared-memory attribute rejected");
        return MATPL_ERR_CUDA;
    }
    const long long blocks = std::min<long long>((A.natoms + kFeatWarps - 1) / kFeatWarps, (long long)device_sms() * 32);
    k<<<(int)std::max<long long>(blocks, 1), 32 * kFeatWarps, smem, s>>>(A);
    return check_launch("matpl_nep_feat");
}

template <typename T, int MODE, int NM, int KM>
int launch_2b(const FeatArgs &A, cudaStream_t s) {
    const long long blocks = std::min<long long>((A.natoms + kFeatWarps - 1) / kFeatWarps, (long long)device_sms() * 32);
    nep2b_op<T, MODE, NM, KM><<<(int)std::max<long long>(blocks, 1), 32 * kFeatWarps, 0, s>>>(A);
    return check_launch("matpl_nep_feat");
}

template <typename T, int MODE>
int dispatch(bool angular, const FeatArgs &A, cudaStream_t s) {
    if (angular) {
        if (A.nmax <= 5 && A.nbase <= 9) return launch_mb<T, MODE, 5, 9>(A, s);
        return launch_mb<T, MODE, 8, 16>(A, s);
    }
    if (A.nmax <= 5 && A.nbase <= 9) return launch_2b<T, MODE, 5, 9>(A, s);
    return launch_2b<T, MODE, 8, 16>(A, s);
}

}  // namespace
}  // namespace matpl

using namespace matpl;

namespace matpl {
namespace {

// dL/dc [T, T, n, K] from the per-atom tables of the backward modes.  A block takes kCgAtoms
// consecutive atoms; for each centre type t present among them it compacts their indices
// (warp ballots, list order kept), its 8 warps split those atoms, and each lane sums kCols
// columns (a 256-column pass: lane + 32 c) of their rows - radial G[i, nn] * W[i, tt, k],
// angular W[i, tt, nn, k] - with the loads of all its columns in flight together.  The warps'
// partial sums meet in shared memory and each column leaves with one atomic into dc[t] per
// block.  The work of a block does not depend on how the types are mixed (sorted or
// interleaved atoms cost the same).
constexpr int kCgWarps = 8;
constexpr int kCgAtoms = 64;
constexpr int kCols = 8;
constexpr int kPass = 32 * kCols;

template <typename T>
__global__ void __launch_bounds__(32 * kCgWarps)
nep_cgrad_kernel(int part, int natoms, int ntypes, int nmax, int K,
                 const long long *__restrict__ type_map, const T *__restrict__ G, long long ldG,
                 const T *__restrict__ W, T *__restrict__ dc, int *__restrict__ err) {
    __shared__ int tsh[kCgAtoms];
    __shared__ int idx[kCgAtoms];
    __shared__ int wbase[kCgAtoms / 32];
    __shared__ int cnt;
    __shared__ T part_sum[kCgWarps][kPass];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long base = (long long)blockIdx.x * kCgAtoms;
    if (threadIdx.x < kCgAtoms) {
        const long long a = base + threadIdx.x;
        int ta = -1;
        if (a < natoms) {
            const long long v = type_map[a];
            if (v < 0 || v >= ntypes) atomicOr(err, MATPL_KERR_BAD_TYPE);
            else ta = (int)v;
        }
        tsh[threadIdx.x] = ta;
    }
    __syncthreads();
    const int E = ntypes * nmax * K;
    for (int t = 0; t < ntypes; ++t) {
        if (threadIdx.x < kCgAtoms) {
            const bool mine = tsh[threadIdx.x] == t;
            const unsigned bal = __ballot_sync(0xffffffffu, mine);
            if (lane == 0) wbase[warp] = __popc(bal);
            __syncwarp();
            if (mine) idx[32 * warp + __popc(bal & ((1u << lane) - 1u))] = threadIdx.x;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // close the gap between the warps' runs (list order kept)
            int n0 = wbase[0];
            for (int w = 1; w < kCgAtoms / 32; ++w) {
                for (int k = 0; k < wbase[w]; ++k) idx[n0 + k] = idx[32 * w + k];
                n0 += wbase[w];
            }
            cnt = n0;
        }
        __syncthreads();
        const int n = cnt;
        if (n == 0) continue;
        for (int e0 = 0; e0 < E; e0 += kPass) {
            T acc[kCols];
            long long goff[kCols], woff[kCols];
#pragma unroll
            for (int c = 0; c < kCols; ++c) {
                acc[c] = 0;
                const int e = e0 + lane + 32 * c;
                const int tt = e / (nmax * K), nn = (e / K) % nmax, k = e % K;
                goff[c] = nn;
                woff[c] = part == 0 ? (long long)tt * K + k : e;
            }
            for (int j = warp; j < n; j += kCgWarps) {
                const long long i = base + idx[j];
                if (part == 0) {
                    const T *g = G + i * ldG;
                    const T *w = W + i * ntypes * K;
#pragma unroll
                    for (int c = 0; c < kCols; ++c)
                        if (e0 + lane + 32 * c < E) acc[c] += g[goff[c]] * w[woff[c]];
                } else {
                    const T *w = W + i * E;
#pragma unroll
                    for (int c = 0; c < kCols; ++c)
                        if (e0 + lane + 32 * c < E) acc[c] += w[woff[c]];
                }
            }
#pragma unroll
            for (int c = 0; c < kCols; ++c) part_sum[warp][lane + 32 * c] = acc[c];
            __syncthreads();
            const int e = e0 + threadIdx.x;
            if (threadIdx.x < kPass && e < E) {
                T v = 0;
#pragma unroll
                for (int w = 0; w < kCgWarps; ++w) v += part_sum[w][threadIdx.x];
                atomicAdd(dc + (long long)t * E + e, v);
            }
            __syncthreads();
        }
    }
}

// Forces and per-image virial of one NEP list from dE = dE/d(r, x, y, z) [N, NN, 4] and the
// rows Ri = (r, x, y, z) themselves (the expanded d(r, x, y, z)/d(x, y, z) of nep_net.py:440-468
// has x_a / r in row 0 and the identity below, so it is formed in registers): per slot
// f_a = dE_0 x_a / r + dE_(1+a) (empty slots, |r| <= 1e-5, give 0), the centre gets -f, the
// neighbor NL +f, and the slot adds f_a r_b to the virial of the centre's image.  A block takes
// kFvAtoms consecutive atoms, each warp kFvAtoms / 8 of them (lanes over slots, warp sums of the
// centre force); the virial is summed per warp and then per block in shared memory, runs of one
// image (frames are contiguous) leaving with 9 atomics, so the atomics on the few virial
// addresses stay at one set per block.
constexpr int kFvWarps = 8;
constexpr int kFvAtoms = 32;

template <typename T>
__global__ void __launch_bounds__(32 * kFvWarps)
nep_force_virial_kernel(int natoms, int nn, int nimages, const long long *__restrict__ NL,
                        const long long *__restrict__ image_of, const T *__restrict__ dE,
                        const T *__restrict__ Ri, T *__restrict__ force, T *__restrict__ virial,
                        int *__restrict__ err) {
    __shared__ T vsh[kFvWarps][9];
    __shared__ long long bsh[kFvWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int per_warp = kFvAtoms / kFvWarps;
    const long long a0 = (long long)blockIdx.x * kFvAtoms + (long long)warp * per_warp;
    T v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long cur = -1;
    for (int k = 0; k < per_warp; ++k) {
        const long long i = a0 + k;
        if (i >= natoms) break;
        const long long b = image_of[i];
        if (b < 0 || b >= nimages) {
            if (lane == 0) atomicOr(err, MATPL_KERR_BAD_COUNT);
            continue;
        }
        if (b != cur) {                 // a frame boundary inside the warp's atoms
            if (cur >= 0 && lane < 9) atomicAdd(virial + 9 * cur + lane, v[0]);
#pragma unroll
            for (int c = 0; c < 9; ++c) v[c] = 0;
            cur = b;
        }
        T fc[3] = {0, 0, 0}, vi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int s = lane; s < nn; s += 32) {
            const long long q = i * nn + s;
            const T r = Ri[4 * q];
            if (!(fabs(r) > T(1e-5))) continue;
            const T x[3] = {Ri[4 * q + 1], Ri[4 * q + 2], Ri[4 * q + 3]};
            const T e0 = dE[4 * q];
            T f[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) f[c] = e0 * (x[c] / r) + dE[4 * q + 1 + c];
            const long long j = NL[q];
            if (j >= natoms) {
                atomicOr(err, MATPL_KERR_BAD_COUNT);
            } else if (j >= 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) atomicAdd(force + 3 * j + c, f[c]);
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                fc[c] -= f[c];
#pragma unroll
                for (int d = 0; d < 3; ++d) vi[3 * c + d] += f[c] * x[d];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) fc[c] = warp_sum(fc[c]);
        if (lane < 3) atomicAdd(force + 3 * i + lane, lane == 0 ? fc[0] : lane == 1 ? fc[1] : fc[2]);
        // the warp's 9 virial sums, lane c < 9 keeping term c in v[0]
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            const T t = warp_sum(vi[c]);
            if (lane == c) v[0] += t;
        }
    }
    if (lane < 9) vsh[warp][lane] = v[0];
    if (lane == 0) bsh[warp] = cur;
    __syncthreads();
    if (threadIdx.x < 9) {
        long long run = -1;
        T acc = 0;
        for (int w = 0; w < kFvWarps; ++w) {
            const long long b = bsh[w];
            if (b < 0) continue;
            if (b != run) {
                if (run >= 0) atomicAdd(virial + 9 * run + threadIdx.x, acc);
                run = b;
                acc = 0;
            }
            acc += vsh[w][threadIdx.x];
        }
        if (run >= 0) atomicAdd(virial + 9 * run + threadIdx.x, acc);
    }
}

// The gradient of the kernel above (linear in dE): per slot u_a = gF[NL]_a - gF[i]_a +
// sum_b gV[image(i)][a][b] r_b, then gdE = (sum_a u_a x_a / r, u_0, u_1, u_2); empty slots 0.
// One thread per slot; gF or gV may be absent (zero).
template <typename T>
__global__ void __launch_bounds__(256)
nep_force_virial_grad_kernel(int natoms, int nn, int nimages, const long long *__restrict__ NL,
                             const long long *__restrict__ image_of, const T *__restrict__ Ri,
                             const T *__restrict__ gF, const T *__restrict__ gV,
                             T *__restrict__ gdE, int *__restrict__ err) {
    const long long total = (long long)natoms * nn;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long i = q / nn;
        const T r = Ri[4 * q];
        T g[4] = {0, 0, 0, 0};
        if (fabs(r) > T(1e-5)) {
            const T x[3] = {Ri[4 * q + 1], Ri[4 * q + 2], Ri[4 * q + 3]};
            T u[3] = {0, 0, 0};
            if (gF) {
                const long long j = NL[q];
#pragma unroll
                for (int a = 0; a < 3; ++a) u[a] = -gF[3 * i + a];
                if (j >= natoms) {
                    atomicOr(err, MATPL_KERR_BAD_COUNT);
                } else if (j >= 0) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) u[a] += gF[3 * j + a];
                }
            }
            if (gV) {
                const long long b = image_of[i];
                if (b < 0 || b >= nimages) {
                    atomicOr(err, MATPL_KERR_BAD_COUNT);
                } else {
#pragma unroll
                    for (int a = 0; a < 3; ++a)
#pragma unroll
                        for (int c = 0; c < 3; ++c) u[a] += gV[9 * b + 3 * a + c] * x[c];
                }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                g[0] += u[a] * (x[a] / r);
                g[1 + a] = u[a];
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) gdE[4 * q + c] = g[c];
    }
}

}  // namespace
}  // namespace matpl

extern "C" int matpl_nep_cgrad(int dtype, int part, int natoms, int ntypes, int n_max, int n_base,
                               const long long *type_map, const void *G, long long ldG,
                               const void *W, void *dc, int *err_dev, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_nep_cgrad: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(part == 0 || part == 1, MATPL_ERR_INVALID, "part: 0 radial, 1 angular");
    MATPL_REQUIRE(natoms >= 0 && ntypes >= 1 && n_max >= 1 && n_base >= 1, MATPL_ERR_INVALID,
                  "bad sizes");
    MATPL_REQUIRE(part == 1 || ldG >= n_max, MATPL_ERR_INVALID, "radial: ldG >= n_max");
    MATPL_REQUIRE(dc && err_dev && (natoms == 0 || (type_map && W && (part == 1 || G))),
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(dc, "matpl_nep_cgrad");
    cudaStream_t s = as_stream(stream);
    const size_t esz = dtype == MATPL_F64 ? sizeof(double) : sizeof(float);
    const size_t nout = (size_t)ntypes * ntypes * n_max * n_base;
    if (cudaMemsetAsync(dc, 0, esz * nout, s) != cudaSuccess) {
        set_error("matpl_nep_cgrad: memset failed");
        return MATPL_ERR_CUDA;
    }
    if (natoms == 0) return MATPL_OK;
    ProfScope ps("nep_cgrad", s);
    const int grid = (int)((natoms + kCgAtoms - 1) / kCgAtoms);
    if (dtype == MATPL_F64)
        nep_cgrad_kernel<double><<<grid, 32 * kCgWarps, 0, s>>>(
            part, natoms, ntypes, n_max, n_base, type_map, (const double *)G, ldG,
            (const double *)W, (double *)dc, err_dev);
    else
        nep_cgrad_kernel<float><<<grid, 32 * kCgWarps, 0, s>>>(
            part, natoms, ntypes, n_max, n_base, type_map, (const float *)G, ldG,
            (const float *)W, (float *)dc, err_dev);
    return check_launch("matpl_nep_cgrad");
}

extern "C" int matpl_nep_force_virial(int dtype, int natoms, int max_nn, int nimages,
                                      const long long *NL, const long long *image_of,
                                      const void *dE, const void *Ri, void *force, void *virial,
                                      int *err_dev, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_nep_force_virial: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(natoms >= 0 && max_nn >= 0 && nimages >= 1, MATPL_ERR_INVALID, "bad sizes");
    MATPL_REQUIRE(force && virial && err_dev &&
                      (natoms * (long long)max_nn == 0 || (NL && image_of && dE && Ri)),
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(force, "matpl_nep_force_virial");
    cudaStream_t s = as_stream(stream);
    const size_t esz = dtype == MATPL_F64 ? sizeof(double) : sizeof(float);
    if (cudaMemsetAsync(force, 0, esz * 3 * (size_t)natoms, s) != cudaSuccess ||
        cudaMemsetAsync(virial, 0, esz * 9 * (size_t)nimages, s) != cudaSuccess) {
        set_error("matpl_nep_force_virial: memset failed");
        return MATPL_ERR_CUDA;
    }
    if (natoms == 0 || max_nn == 0) return MATPL_OK;
    ProfScope ps("nep_force_virial", s);
    const int grid = (int)((natoms + kFvAtoms - 1) / kFvAtoms);
    if (dtype == MATPL_F64)
        nep_force_virial_kernel<double><<<grid, 32 * kFvWarps, 0, s>>>(
            natoms, max_nn, nimages, NL, image_of, (const double *)dE, (const double *)Ri,
            (double *)force, (double *)virial, err_dev);
    else
        nep_force_virial_kernel<float><<<grid, 32 * kFvWarps, 0, s>>>(
            natoms, max_nn, nimages, NL, image_of, (const float *)dE, (const float *)Ri,
            (float *)force, (float *)virial, err_dev);
    return check_launch("matpl_nep_force_virial");
}

extern "C" int matpl_nep_force_virial_grad(int dtype, int natoms, int max_nn, int nimages,
                                           const long long *NL, const long long *image_of,
                                           const void *Ri, const void *g_force,
                                           const void *g_virial, void *g_dE, int *err_dev,
                                           void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_nep_force_virial_grad: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(natoms >= 0 && max_nn >= 0 && nimages >= 1, MATPL_ERR_INVALID, "bad sizes");
    MATPL_REQUIRE(err_dev && (natoms * (long long)max_nn == 0 || (NL && image_of && Ri && g_dE)),
                  MATPL_ERR_INVALID, "null pointer argument");
    const long long total = (long long)natoms * max_nn;
    if (total == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(g_dE, "matpl_nep_force_virial_grad");
    cudaStream_t s = as_stream(stream);
    ProfScope ps("nep_force_virial_grad", s);
    const int grid = (int)std::min<long long>((total + 255) / 256, (long long)device_sms() * 16);
    if (dtype == MATPL_F64)
        nep_force_virial_grad_kernel<double><<<grid, 256, 0, s>>>(
            natoms, max_nn, nimages, NL, image_of, (const double *)Ri, (const double *)g_force,
            (const double *)g_virial, (double *)g_dE, err_dev);
    else
        nep_force_virial_grad_kernel<float><<<grid, 256, 0, s>>>(
            natoms, max_nn, nimages, NL, image_of, (const float *)Ri, (const float *)g_force,
            (const float *)g_virial, (float *)g_dE, err_dev);
    return check_launch("matpl_nep_force_virial_grad");
}

extern "C" int matpl_nep_feat_op(int dtype, int part, int mode, int natoms, int max_nn,
                                 int ntypes, int n_max, int n_base, int l_max_3b, int l_max_4b,
                                 int l_max_5b, double cutoff, const void *coeff, const void *d12,
                                 const long long *NL, const long long *type_map, const void *G,
                                 long long ldG, const void *H, void *q, long long ldQ,
                                 void *grad_d12, void *W, int *err_dev, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_nep_feat_op: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(part == 0 || part == 1, MATPL_ERR_INVALID, "part: 0 radial, 1 angular");
    MATPL_REQUIRE(mode >= 0 && mode <= 2, MATPL_ERR_INVALID, "mode: 0 fwd, 1 bwd, 2 bwd2");
    MATPL_REQUIRE(natoms >= 0 && max_nn >= 0 && ntypes >= 1 && cutoff > 0, MATPL_ERR_INVALID,
                  "bad sizes");
    MATPL_REQUIRE(n_max >= 1 && n_max <= 8 && n_base >= 1 && n_base <= 16, MATPL_ERR_UNSUPPORTED,
                  "compiled for n_max <= 8 and basis size <= 16 (coefficient dims 2, 3)");
    MATPL_REQUIRE(part == 0 || (l_max_3b >= 0 && l_max_3b <= 4 && (l_max_4b == 0 || l_max_4b == 2) &&
                                (l_max_5b == 0 || l_max_5b == 1)),
                  MATPL_ERR_UNSUPPORTED, "angular l_max (<= 4, 2 or 0, 1 or 0)");
    MATPL_REQUIRE(err_dev && coeff && type_map && (natoms == 0 || (d12 && NL)), MATPL_ERR_INVALID,
                  "null pointer argument");
    MATPL_REQUIRE(mode != 0 || q, MATPL_ERR_INVALID, "fwd needs q");
    MATPL_REQUIRE(mode != 1 || (G && (W || grad_d12)), MATPL_ERR_INVALID,
                  "bwd needs G and grad_d12 or W");
    MATPL_REQUIRE(mode != 2 || (G && H && q && W), MATPL_ERR_INVALID, "bwd2 needs G, H, gso, W");
    if (natoms == 0 || max_nn == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(d12, "matpl_nep_feat_op");
    FeatArgs A{};
    A.natoms = natoms;
    A.nn = max_nn;
    A.ntypes = ntypes;
    A.nmax = n_max;
    A.nbase = n_base;
    A.rc = cutoff;
    A.coeff = coeff;
    A.d12 = d12;
    A.NL = NL;
    A.type = type_map;
    A.G = G;
    A.ldG = ldG;
    A.H = H;
    A.q = q;
    A.ldQ = ldQ;
    A.grad_d12 = grad_d12;
    A.W = W;
    A.l3 = l_max_3b;
    A.four = l_max_4b > 0;
    A.five = l_max_5b > 0;
    A.err = err_dev;
    cudaStream_t s = as_stream(stream);
    ProfScope ps(part ? "nep_mb_op" : "nep_2b_op", s);
    const bool ang = part == 1;
    if (dtype == MATPL_F64) {
        if (mode == 0) return dispatch<double, kFwd>(ang, A, s);
        if (mode == 1) return dispatch<double, kBwd>(ang, A, s);
        return dispatch<double, kBwd2>(ang, A, s);
    }
    if (mode == 0) return dispatch<float, kFwd>(ang, A, s);
    if (mode == 1) return dispatch<float, kBwd>(ang, A, s);
    return dispatch<float, kBwd2>(ang, A, s);
}
