// NEP training operators: the descriptor of one neighbor list with its first and second
// derivatives, the drop-in for CalcOps calculateNepFeat (radial, src/op/src/CalcOps.cpp:385-680)
// and calculateNepMbFeat (3-/4-/5-body, CalcOps.cpp:680-1023) with their Grad functions.
//
// For a descriptor q(c, d12) of one list (d12 [N, NN, 4] = (r, x, y, z) of every slot, c the
// coefficients [T, T, n, K]) and the features' gradient G = dL/dq [N, F]:
//   FWD   q [N, F]
//   BWD   grad_d12 = G . dq/dd12 [N, NN, 4] and W, from which dL/dc follows by a sum over the
//         atoms of each centre type (the caller's index_add):
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
                if (use) {
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
            if (MODE != kFwd) {
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
// returns sum_f G_f dq_f/ds_m.  sv = s_n[0..23] of this atom.
template <typename T>
__device__ __forceinline__ T sbar_of(int m, const T *sv, T g3, T g4, T g5, bool four, bool five) {
    T v = g3 * T(2) * C3<T>(m) * sv[m];
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
__device__ __forceinline__ T sbar_dot(int m, const T *sv, const T *sd, T g3, T g4, T g5, bool four,
                                      bool five) {
    T v = g3 * T(2) * C3<T>(m) * sd[m];
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
                        v += MODE == kFwd ? C3<T>(m) * sv[m] * sv[m] : T(2) * C3<T>(m) * sv[m] * sd[m];
                } else if (four && blk == A.l3) {
                    if (MODE == kFwd) {
                        const T s3 = sv[3], s4 = sv[4], s5 = sv[5], s6 = sv[6], s7 = sv[7];
                        v = C4<T>(0) * s3 * s3 * s3 + C4<T>(1) * s3 * (s4 * s4 + s5 * s5) +
                            C4<T>(2) * s3 * (s6 * s6 + s7 * s7) + C4<T>(3) * s6 * (s5 * s5 - s4 * s4) +
                            C4<T>(4) * s4 * s5 * s7;
                    } else {
                        for (int m = 3; m <= 7; ++m)
                            v += sbar_of<T>(m, sv, T(0), T(1), T(0), true, false) * sd[m];
                    }
                } else {
                    if (MODE == kFwd) {
                        const T a0 = sv[0] * sv[0], a12 = sv[1] * sv[1] + sv[2] * sv[2];
                        v = C5<T>(0) * a0 * a0 + C5<T>(1) * a0 * a12 + C5<T>(2) * a12 * a12;
                    } else {
                        for (int m = 0; m <= 2; ++m)
                            v += sbar_of<T>(m, sv, T(0), T(0), T(1), false, true) * sd[m];
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
            S.sb[n][m] = sbar_of<T>(m, S.s[n], g3, g4, g5, four, five);
            if (MODE == kBwd2) S.sbd[n][m] = sbar_dot<T>(m, S.s[n], S.sd[n], g3, g4, g5, four, five);
        }
        __syncwarp();
        // ---- pass 2: grad_d12 (BWD) and the per-atom c-gradient table W
        T *W = static_cast<T *>(A.W) + i * (long long)T_ * n_ * K;
        for (int base = 0; base < nvalid; base += 32) {
            const int slot = base + lane;
            const long long ps = i * A.nn + slot;
            const long long j = slot < A.nn ? A.NL[ps] : -1;
            int tj = (j >= 0 && j < A.natoms) ? (int)A.type[j] : -1;
            const bool ok = tj >= 0 && tj < T_;
            T f[KM], df[KM], g[NM], gp[NM], ux, uy, uz, ri;
            const T *cr = c + ((long long)(ti * T_ + (ok ? tj : 0)) * n_) * K;
            mb_pair<T, NM, KM>(A, cr, ok ? ps : 0, f, df, g, gp, ux, uy, uz, ri);
            if (MODE == kBwd) {
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
    const long long blocks = std::min<long long>((A.natoms + kFeatWarps - 1) / kFeatWarps, 152LL * 32);
    k<<<(int)std::max<long long>(blocks, 1), 32 * kFeatWarps, smem, s>>>(A);
    return check_launch("matpl_nep_feat");
}

template <typename T, int MODE, int NM, int KM>
int launch_2b(const FeatArgs &A, cudaStream_t s) {
    const long long blocks = std::min<long long>((A.natoms + kFeatWarps - 1) / kFeatWarps, 152LL * 32);
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
    MATPL_REQUIRE(mode != 1 || (G && W && (grad_d12 || natoms == 0)), MATPL_ERR_INVALID,
                  "bwd needs G, grad_d12, W");
    MATPL_REQUIRE(mode != 2 || (G && H && q && W), MATPL_ERR_INVALID, "bwd2 needs G, H, gso, W");
    if (natoms == 0 || max_nn == 0) return MATPL_OK;
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
