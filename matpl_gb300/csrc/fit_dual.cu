// The fitting part of the fused DP force-loss training step (dp_trainer.py:162-275 through
// dp_embedding.py:140-163): for the rows of one element, D [rows, 400] and its tangent
// D_dot along the force seed, the fitting net DIN -> F -> F -> F -> 1 is run on both streams
// (primal E, tangent E_dot = dE/dD . D_dot) and
//
//   phi = sum_r (a_r E_r + E_dot_r)
//
// is differentiated once in every input: grad_D, grad_D_dot per row and the gradient of every
// fitting parameter.  phi is the scalar whose first-order gradient is the force-loss gradient of
// the fitting part (a_r = dL/dE of the row's configuration; the force term enters through
// D_dot), so the training step needs no second-order autograd through the fitting net.
//
//   fit_dual_rows   CTA per tile of 32 rows; every product is CTA-wide and register-blocked
//                   (both streams of two rows x four columns per thread, operands staged in
//                   shared memory): forward of both streams through the three tanh layers, the closed-form
//                   reverse pass (for h = tanh(z), h_dot = (1 - h^2) z_dot:
//                     dz     = (g_h - 2 g_hd h z_dot)(1 - h^2),   dz_dot = g_hd (1 - h^2)),
//                   grad_D / grad_D_dot = (dz0, dz0_dot) W0^T, and per row the factors of the
//                   weight gradients (layer inputs and dz of every layer);
//   fit_dual_wgrad  the weight gradients as sums over rows (dW = X^T dz + X_dot^T dz_dot, the
//                   bias, resnet_dt and output-layer sums): CTA per (row chunk, output tile),
//                   register-blocked 4 x 4 outputs per thread, atomically added.
#include "common.cuh"
#include "dp_layout.cuh"

namespace matpl {
namespace {

using dp::DIN;
using dp::F;
using dp::FitOff;

constexpr int kTile = 32;                 // rows per CTA in fit_dual_rows
constexpr int kNF = 13;                   // per-row factor arrays written for the reductions

// factor arrays [kNF][F][nrp] in the workspace (column-major: a thread's two rows are adjacent,
// nrp = rows rounded up to 32)
enum Factor { fG0 = 0, fGD0, fX1, fXD1, fG1, fGD1, fX2, fXD2, fG2, fGD2, fC1, fC2, fC3 };

template <typename T>
struct RowsArgs {
    long long nrows;
    const T *fw;          // FitOff block of this element
    const T *D, *Dd;      // [nrows][DIN]
    const T *a;           // [nrows] dphi/dE of each row
    T *gD, *gDd;          // [nrows][DIN]
    T *fac;               // [kNF][F][nrp]
    long long nrp;
    double *phi;          // += sum_r (a_r E_r + E_dot_r)
};

__device__ __forceinline__ void store2(float *p, float a, float b) {
    *reinterpret_cast<float2 *>(p) = make_float2(a, b);
}
__device__ __forceinline__ void store2(double *p, double a, double b) {
    *reinterpret_cast<double2 *>(p) = make_double2(a, b);
}
__device__ __forceinline__ void store4(float *p, const float *v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void store4(double *p, const double *v) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
}

// CTA-wide products on a tile of kTile rows and both streams.  Activations are kept transposed,
// A[k][m] with m < kTile the primal rows and m >= kTile the same rows' tangent (row stride kLdA,
// even and = 2 mod 32 words so that the staging stores do not collide in one bank).  Thread
// (mg, ng), mg < 16, ng < 13, owns rows {2 mg, 2 mg + 1} of both streams and columns
// 4 ng .. 4 ng + 3 of the output: 16 accumulators, 2 + 2 + 4 shared loads per 16 FMAs.
constexpr int kLdA = 2 * kTile + 2;       // 66
constexpr int kLdW = 52;                  // F padded to 4-wide column groups
constexpr int kGroups = 16 * 13;          // threads that own outputs
constexpr int kKC = 16;                   // k rows of D / W0 staged per step

template <typename T>
__device__ __forceinline__ void cta_gemm(const T *At, const T *W, int K, int mg, int ng,
                                         T acc[2][4], T accd[2][4]) {
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
        const T *a = At + k * kLdA;
        const T x0 = a[2 * mg], x1 = a[2 * mg + 1];
        const T d0 = a[kTile + 2 * mg], d1 = a[kTile + 2 * mg + 1];
        T w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) w[j] = W[k * kLdW + 4 * ng + j];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            acc[0][j] += x0 * w[j];
            acc[1][j] += x1 * w[j];
            accd[0][j] += d0 * w[j];
            accd[1][j] += d1 * w[j];
        }
    }
}

// asynchronous element copies global -> shared (zero fill when !ok), one group per stage
__device__ __forceinline__ uint32_t sptr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
template <typename T>
__device__ __forceinline__ void cp_elem(T *dst, const T *src, bool ok) {
    const int n = ok ? (int)sizeof(T) : 0;
    if (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sptr(dst)), "l"(src),
                     "r"(n));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sptr(dst)), "l"(src),
                     "r"(n));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// stage a [rows][F] block of the packed parameters (row stride ld) as [rows][kLdW], zero padded
template <typename T>
__device__ __forceinline__ void stage_w(T *dst, const T *__restrict__ src, int rows, int ld,
                                        int col0, int ncols) {
    for (int q = threadIdx.x; q < rows * kLdW; q += blockDim.x) {
        const int r = q / kLdW, c = q - r * kLdW;
        dst[q] = c < ncols ? __ldg(src + (long long)r * ld + col0 + c) : T(0);
    }
}

// shared arrays (elements): X1 = [h0; hd0], X2, X3 (layer inputs / output layer input; X3 later
// holds the reverse pass's [dz; dz_dot]), H1 = [h1; hd1], H2, transposed [kLdW][kLdA]; z_dot of
// the three hidden layers [kLdW][kTile]; one staging area for weights and D chunks
constexpr int kArr = kLdW * kLdA;
constexpr int kChunkS = kKC * kLdA + kKC * kLdW;     // one D / W0 chunk (two are in flight)
constexpr int kWT = kLdW * 50;                       // one W0^T column chunk (two in flight)
constexpr int kStage = 2 * kWT > 2 * kChunkS ? 2 * kWT : 2 * kChunkS;
constexpr int kRowsSmem = 5 * kArr + 3 * kLdW * kTile + kStage;

template <typename T>
__global__ void __launch_bounds__(256) fit_dual_rows(RowsArgs<T> A) {
    extern __shared__ __align__(16) unsigned char fd_raw[];
    T *X1 = reinterpret_cast<T *>(fd_raw);
    T *X2 = X1 + kArr, *X3 = X2 + kArr, *H1 = X3 + kArr, *H2 = H1 + kArr;
    T *ZD = H2 + kArr;                                   // [3][kLdW][kTile]
    T *S = ZD + 3 * kLdW * kTile;                        // staging
    T *DZ = X3;                                          // reverse pass: [dz; dz_dot]
    const T *fw = A.fw;
    const int t = threadIdx.x;
    const bool own = t < kGroups;
    const int mg = t & 15, ng = own ? t >> 4 : 0;
    const long long ntiles = (A.nrows + kTile - 1) / kTile;
    const long long nr = A.nrows;
    double phi_acc = 0.0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long row0 = tile * kTile;
        const int nrow = (int)(nr - row0 < kTile ? nr - row0 : kTile);
        T acc[2][4], accd[2][4];
        auto zero = [&]() {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = accd[i][j] = T(0);
        };
        // ---------------- layer 0: [z0; z0_dot] = [D; D_dot] W0, K = DIN in chunks; the next
        // chunk's copies are in flight while the current one is used
        zero();
        auto issue = [&](int k0, T *buf) {
            T *St = buf, *Sw = buf + kKC * kLdA;
            for (int q = t; q < 2 * kTile * kKC; q += blockDim.x) {
                const int m = q / kKC, kk = q - m * kKC;          // m < 2 kTile
                const int r = m < kTile ? m : m - kTile;
                const T *src = m < kTile ? A.D : A.Dd;
                const bool ok = r < nrow;
                cp_elem(St + kk * kLdA + m, src + (row0 + (ok ? r : 0)) * DIN + k0 + kk, ok);
            }
            for (int q = t; q < kKC * kLdW; q += blockDim.x) {
                const int r = q / kLdW, c = q - r * kLdW;
                const bool ok = c < F;
                cp_elem(Sw + q, fw + FitOff::W0 + (long long)(k0 + r) * F + (ok ? c : 0), ok);
            }
            cp_commit();
        };
        __syncthreads();                         // the staging area is free
        issue(0, S);
        for (int k0 = 0, b = 0; k0 < DIN; k0 += kKC, b ^= 1) {
            if (k0 + kKC < DIN) {
                issue(k0 + kKC, S + (b ^ 1) * kChunkS);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();
            T *cur = S + b * kChunkS;
            if (own) cta_gemm(cur, cur + kKC * kLdA, kKC, mg, ng, acc, accd);
            __syncthreads();                     // before the next issue overwrites this buffer
        }
        // epilogue: h0 = tanh(z0 + b0), hd0 = (1 - h0^2) zd0
        if (own) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * ng + j;
                const T b = c < F ? fw[FitOff::B0 + c] : T(0);
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const int m = 2 * mg + i;
                    const T h = c < F ? dev_tanh(acc[i][j] + b) : T(0), zd = accd[i][j];
                    X1[c * kLdA + m] = h;
                    X1[c * kLdA + kTile + m] = (T(1) - h * h) * zd;
                    ZD[c * kTile + m] = zd;
                }
            }
        }
        // ---------------- layers 1, 2: x_out = tanh(x_in W + b) dt + x_in
#pragma unroll
        for (int l = 1; l <= 2; ++l) {
            const T *Xin = l == 1 ? X1 : X2;
            T *Xout = l == 1 ? X2 : X3;
            T *Hl = l == 1 ? H1 : H2;
            T *ZDl = ZD + l * kLdW * kTile;
            const int OB = l == 1 ? FitOff::B1 : FitOff::B2;
            const int OD = l == 1 ? FitOff::DT1 : FitOff::DT2;
            __syncthreads();
            stage_w(S, fw + (l == 1 ? FitOff::W1 : FitOff::W2), F, F, 0, F);
            __syncthreads();
            zero();
            if (own) {
                cta_gemm(Xin, S, F, mg, ng, acc, accd);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = 4 * ng + j;
                    const bool v = c < F;
                    const T b = v ? fw[OB + c] : T(0), dt = v ? fw[OD + c] : T(0);
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        const int m = 2 * mg + i;
                        const T h = v ? dev_tanh(acc[i][j] + b) : T(0), zd = accd[i][j];
                        const T hd = (T(1) - h * h) * zd;
                        Hl[c * kLdA + m] = h;
                        Hl[c * kLdA + kTile + m] = hd;
                        ZDl[c * kTile + m] = zd;
                        Xout[c * kLdA + m] = h * dt + Xin[c * kLdA + m];
                        Xout[c * kLdA + kTile + m] = hd * dt + Xin[c * kLdA + kTile + m];
                    }
                }
            }
        }
        __syncthreads();
        // ---------------- output layer E = x3 . W3 + b3, E_dot = x3_dot . W3; phi
        if (t < nrow) {
            T e = T(0), ed = T(0);
            for (int c = 0; c < F; ++c) {
                const T w3 = fw[FitOff::W3 + c];
                e += X3[c * kLdA + t] * w3;
                ed += X3[c * kLdA + kTile + t] * w3;
            }
            phi_acc += (double)A.a[row0 + t] * (double)(e + fw[FitOff::B3]) + (double)ed;
        }
        // ---------------- reverse pass; g / gd = dphi/dx, dphi/dx_dot at each layer's output
        T g[2][4], gd[2][4], arow[2];
        bool live[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            live[i] = own && 2 * mg + i < nrow;
            arow[i] = live[i] ? A.a[row0 + 2 * mg + i] : T(0);
        }
        // factor values of this thread's two rows at column c
        auto put = [&](int which, int c, T v0, T v1) {
            T *p = A.fac + ((long long)which * F + c) * A.nrp + row0 + 2 * mg;
            if (live[1]) store2(p, v0, v1);
            else if (live[0]) p[0] = v0;
        };
        if (own) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * ng + j;
                const T w3 = c < F ? fw[FitOff::W3 + c] : T(0);
                T v[2];
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    g[i][j] = arow[i] * w3;
                    gd[i][j] = w3;
                    v[i] = arow[i] * X3[c * kLdA + 2 * mg + i] + X3[c * kLdA + kTile + 2 * mg + i];
                }
                if (c < F) put(fC3, c, v[0], v[1]);
            }
        }
#pragma unroll
        for (int l = 2; l >= 1; --l) {
            const T *Hl = l == 1 ? H1 : H2;
            const T *ZDl = ZD + l * kLdW * kTile;
            const T *Xin = l == 1 ? X1 : X2;
            const int OD = l == 1 ? FitOff::DT1 : FitOff::DT2;
            const int wG = l == 1 ? fG1 : fG2, wGD = l == 1 ? fGD1 : fGD2;
            const int wX = l == 1 ? fX1 : fX2, wXD = l == 1 ? fXD1 : fXD2, wC = l == 1 ? fC1 : fC2;
            __syncthreads();                 // X3 (l = 2) / DZ (l = 1) is read no more
            if (own) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = 4 * ng + j;
                    const bool v = c < F;
                    const T dt = v ? fw[OD + c] : T(0);
                    T vc[2], vg[2], vgd[2];
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        const int m = 2 * mg + i;
                        const T h = Hl[c * kLdA + m], hd = Hl[c * kLdA + kTile + m];
                        const T zd = ZDl[c * kTile + m];
                        const T gh = g[i][j] * dt, ghd = gd[i][j] * dt, s = T(1) - h * h;
                        const T dz = v ? (gh - T(2) * ghd * h * zd) * s : T(0);
                        const T dzd = v ? ghd * s : T(0);
                        vc[i] = g[i][j] * h + gd[i][j] * hd;
                        vg[i] = dz;
                        vgd[i] = dzd;
                        DZ[c * kLdA + m] = dz;
                        DZ[c * kLdA + kTile + m] = dzd;
                    }
                    if (v) {
                        const int m = 2 * mg;
                        put(wC, c, vc[0], vc[1]);
                        put(wG, c, vg[0], vg[1]);
                        put(wGD, c, vgd[0], vgd[1]);
                        put(wX, c, Xin[c * kLdA + m], Xin[c * kLdA + m + 1]);
                        put(wXD, c, Xin[c * kLdA + kTile + m], Xin[c * kLdA + kTile + m + 1]);
                    }
                }
            }
            stage_w(S, fw + (l == 1 ? FitOff::W1T : FitOff::W2T), F, F, 0, F);
            __syncthreads();
            if (own) {
                zero();
                cta_gemm(DZ, S, F, mg, ng, acc, accd);
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        g[i][j] += acc[i][j];
                        gd[i][j] += accd[i][j];
                    }
            }
        }
        // layer 0: x1 = tanh(D W0 + b0), no residual
        __syncthreads();
        if (own) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * ng + j;
                const bool v = c < F;
                T vg[2], vgd[2];
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const int m = 2 * mg + i;
                    const T h = X1[c * kLdA + m], zd = ZD[c * kTile + m];
                    const T s = T(1) - h * h;
                    const T dz = v ? (g[i][j] - T(2) * gd[i][j] * h * zd) * s : T(0);
                    const T dzd = v ? gd[i][j] * s : T(0);
                    vg[i] = dz;
                    vgd[i] = dzd;
                    DZ[c * kLdA + m] = dz;
                    DZ[c * kLdA + kTile + m] = dzd;
                }
                if (v) {
                    put(fG0, c, vg[0], vg[1]);
                    put(fGD0, c, vgd[0], vgd[1]);
                }
            }
        }
        // grad_D / grad_D_dot = [dz0; dz0_dot] W0^T, output columns in chunks of kLdW, the next
        // chunk of W0^T in flight while the current one is used
        auto issue_wt = [&](int c0, T *buf) {
            const int ncols = DIN - c0 < kLdW ? DIN - c0 : kLdW;
            for (int q = t; q < F * kLdW; q += blockDim.x) {
                const int r = q / kLdW, c = q - r * kLdW;
                const bool ok = c < ncols;
                cp_elem(buf + q, fw + FitOff::W0T + (long long)r * DIN + c0 + (ok ? c : 0), ok);
            }
            cp_commit();
        };
        __syncthreads();                         // the staging area is free
        issue_wt(0, S);
        for (int c0 = 0, b = 0; c0 < DIN; c0 += kLdW, b ^= 1) {
            const int ncols = DIN - c0 < kLdW ? DIN - c0 : kLdW;
            if (c0 + kLdW < DIN) {
                issue_wt(c0 + kLdW, S + (b ^ 1) * kWT);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();
            if (own) {
            zero();
            cta_gemm(DZ, S + b * kWT, F, mg, ng, acc, accd);
            // ncols is a multiple of 4: whole 16-byte groups per row
            if (4 * ng < ncols) {
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    if (!live[i]) continue;
                    const long long o = (row0 + 2 * mg + i) * DIN + c0 + 4 * ng;
                    store4(A.gD + o, acc[i]);
                    store4(A.gDd + o, accd[i]);
                }
            }
            }
            __syncthreads();                     // before the next issue overwrites this buffer
        }
    }
    phi_acc = warp_sum(phi_acc);
    if ((threadIdx.x & 31) == 0 && phi_acc != 0.0) atomicAdd(A.phi, phi_acc);
}

// ---------------------------------------------------------------- weight-gradient reductions
constexpr int kChunk = 256;     // rows per CTA
template <typename T> constexpr int kSub = 128 / sizeof(T);   // rows staged at a time (32 f32)
constexpr int kKT = 64;         // output rows (k) per CTA tile
constexpr int kUT = 52;         // output columns (u) per tile: F = 50 padded to 4-wide groups

template <typename T>
struct WgradArgs {
    long long nrows;
    const T *D, *Dd;      // [nrows][DIN]
    const T *a;           // [nrows]
    const T *fac;         // [kNF][F][nrp]
    long long nrp;
    T *grad;              // FitOff layout W0 .. B3 (+=)
};

// blockIdx.y: 0..6 the 64-row k tiles of W0 (DIN = 400), 7: W1, 8: W2, 9: the vector sums.
// Thread (tk, tu) of a 16 x 13 grid owns outputs k = k0 + 4 tk + i, u = 4 tu + j (i, j < 4).
template <typename T>
__global__ void __launch_bounds__(256) fit_dual_wgrad(WgradArgs<T> A) {
    constexpr int SUB = kSub<T>;
    // two staging buffers (dynamic shared memory), each X, X_dot [SUB][kKT + 1] then G, G_dot
    // [SUB][kUT + 1] (+1: column-order staging stores fall in distinct banks)
    extern __shared__ __align__(16) unsigned char wg_raw[];
    using RowA = T[SUB][kKT + 1];
    using RowB = T[SUB][kUT + 1];
    struct Buf { RowA a[2]; RowB b[2]; };
    Buf *bufs = reinterpret_cast<Buf *>(wg_raw);
    const long long rbeg = (long long)blockIdx.x * kChunk;
    if (rbeg >= A.nrows) return;
    const long long rend = rbeg + kChunk < A.nrows ? rbeg + kChunk : A.nrows;
    const int which = blockIdx.y;
    if (which == 9) {
        // bias / resnet_dt / output-layer sums: one warp per column of the factor arrays, lanes
        // over rows
        const int sums[6][2] = {{fG0, FitOff::B0}, {fG1, FitOff::B1}, {fG2, FitOff::B2},
                                {fC1, FitOff::DT1}, {fC2, FitOff::DT2}, {fC3, FitOff::W3}};
        const int lane = threadIdx.x & 31;
        for (int job = threadIdx.x >> 5; job < 6 * F + 1; job += blockDim.x >> 5) {
            const T *src = A.a;
            int dst = FitOff::B3;
            if (job < 6 * F) {
                const int v = job / F, u = job - v * F;
                src = A.fac + ((long long)sums[v][0] * F + u) * A.nrp;
                dst = sums[v][1] + u;
            }
            T s = T(0);
            for (long long r = rbeg + lane; r < rend; r += 32) s += src[r];
            s = warp_sum(s);
            if (lane == 0) atomicAdd(A.grad + dst, s);
        }
        return;
    }
    // the product: X^T G + X_dot^T G_dot over the rows of this chunk; X = D / D_dot row-major
    // [rows][DIN] for W0, else column-major factors [F][nrp] like G
    const T *X, *XD, *G, *GD;
    int K, k0, gbase;
    const long long nrp = A.nrp;
    const bool rowmajor = which < 7;
    if (rowmajor) {
        X = A.D; XD = A.Dd; K = DIN; k0 = which * kKT; gbase = FitOff::W0;
        G = A.fac + (long long)fG0 * F * nrp; GD = A.fac + (long long)fGD0 * F * nrp;
    } else {
        const bool one = which == 7;
        X = A.fac + (long long)(one ? fX1 : fX2) * F * nrp;
        XD = A.fac + (long long)(one ? fXD1 : fXD2) * F * nrp;
        G = A.fac + (long long)(one ? fG1 : fG2) * F * nrp;
        GD = A.fac + (long long)(one ? fGD1 : fGD2) * F * nrp;
        K = F; k0 = 0; gbase = one ? FitOff::W1 : FitOff::W2;
    }
    const int tk = threadIdx.x / 13, tu = threadIdx.x - tk * 13;    // 19 x 13 (tk < 16 used)
    const bool active = threadIdx.x < 16 * 13;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    // stage X / X_dot and G / G_dot of rows s0 .. s0 + SUB - 1 (zero past the ends)
    auto issue = [&](long long s0, Buf &B) {
        for (int q = threadIdx.x; q < SUB * kKT; q += blockDim.x) {
            int r, k;
            if (rowmajor) { r = q / kKT; k = q - r * kKT; }     // reads along a row
            else { k = q / SUB; r = q - k * SUB; }              // reads along a column
            const long long row = s0 + r;
            const bool ok = row < rend && k0 + k < K;
            const long long at =
                ok ? (rowmajor ? row * DIN + k0 + k : (long long)(k0 + k) * nrp + row) : 0;
            cp_elem(&B.a[0][r][k], X + at, ok);
            cp_elem(&B.a[1][r][k], XD + at, ok);
        }
        for (int q = threadIdx.x; q < SUB * kUT; q += blockDim.x) {
            const int u = q / SUB, r = q - u * SUB;
            const long long row = s0 + r;
            const bool ok = row < rend && u < F;
            const long long at = ok ? (long long)u * nrp + row : 0;
            cp_elem(&B.b[0][r][u], G + at, ok);
            cp_elem(&B.b[1][r][u], GD + at, ok);
        }
        cp_commit();
    };
    issue(rbeg, bufs[0]);
    for (long long s0 = rbeg, b = 0; s0 < rend; s0 += SUB, b ^= 1) {
        if (s0 + SUB < rend) {
            issue(s0 + SUB, bufs[b ^ 1]);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        __syncthreads();
        if (active) {
            const Buf &B = bufs[b];
#pragma unroll 4
            for (int r = 0; r < SUB; ++r) {
#pragma unroll
                for (int st = 0; st < 2; ++st) {
                    T xv[4], gv[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) xv[i] = B.a[st][r][4 * tk + i];
#pragma unroll
                    for (int j = 0; j < 4; ++j) gv[j] = B.b[st][r][4 * tu + j];
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] += xv[i] * gv[j];
                }
            }
        }
        __syncthreads();                         // before the next issue overwrites it
    }
    if (!active) return;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int k = k0 + 4 * tk + i;
        if (k >= K) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int u = 4 * tu + j;
            if (u < F) atomicAdd(A.grad + gbase + k * F + u, acc[i][j]);
        }
    }
}

inline long long padded_rows(long long nrows) { return (nrows + 31) / 32 * 32; }

size_t ws_bytes_for(int dtype, long long nrows) {
    const size_t t = dtype == MATPL_F64 ? 8 : 4;
    return align_up((size_t)kNF * (size_t)padded_rows(nrows) * F * t, 256);
}

template <typename T>
int run(long long nrows, const void *fit_params, const void *D, const void *Dd, const void *a,
        void *gD, void *gDd, void *grad, double *phi, void *ws, cudaStream_t s) {
    RowsArgs<T> R;
    R.nrows = nrows; R.fw = (const T *)fit_params; R.D = (const T *)D; R.Dd = (const T *)Dd;
    R.a = (const T *)a; R.gD = (T *)gD; R.gDd = (T *)gDd; R.fac = (T *)ws; R.phi = phi;
    R.nrp = padded_rows(nrows);
    const long long ntiles = (nrows + kTile - 1) / kTile;
    long long g1 = ntiles;
    const long long cap = (long long)device_sms() * 2;
    if (g1 > cap) g1 = cap;
    const size_t smem = sizeof(T) * (size_t)kRowsSmem;
    if (cudaFuncSetAttribute(fit_dual_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(fit_dual_rows)");
    {
        ProfScope ps("dp_fit_dual", s);
        fit_dual_rows<T><<<(int)g1, 256, smem, s>>>(R);
    }
    WgradArgs<T> W;
    W.nrows = nrows; W.D = (const T *)D; W.Dd = (const T *)Dd; W.a = (const T *)a;
    W.fac = (const T *)ws; W.nrp = padded_rows(nrows); W.grad = (T *)grad;
    const long long chunks = (nrows + kChunk - 1) / kChunk;
    MATPL_REQUIRE(chunks < (1LL << 31), MATPL_ERR_INVALID, "too many rows");
    constexpr int SUB = kSub<T>;
    const size_t smem_w = 2 * sizeof(T) * (size_t)(2 * SUB * (kKT + 1) + 2 * SUB * (kUT + 1));
    if (cudaFuncSetAttribute(fit_dual_wgrad<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_w) != cudaSuccess)
        return check_launch("cudaFuncSetAttribute(fit_dual_wgrad)");
    {
        ProfScope ps("dp_fit_dual_wgrad", s);
        fit_dual_wgrad<T><<<dim3((unsigned)chunks, 10), 256, smem_w, s>>>(W);
    }
    return check_launch("matpl_dp_fit_dual");
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" size_t matpl_dp_fit_dual_workspace_bytes(int dtype, long long nrows) {
    if (nrows < 0 || (dtype != MATPL_F32 && dtype != MATPL_F64)) return 0;
    return ws_bytes_for(dtype, nrows);
}

extern "C" int matpl_dp_fit_dual(int dtype, long long nrows, const void *fit_params,
                                 const void *D, const void *D_dot, const void *a, void *grad_D,
                                 void *grad_D_dot, void *grad_params, double *phi,
                                 void *workspace, size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_dp_fit_dual: dtype must be MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(nrows >= 0, MATPL_ERR_INVALID, "matpl_dp_fit_dual: negative row count");
    if (nrows == 0) return MATPL_OK;
    MATPL_REQUIRE(fit_params && D && D_dot && a && grad_D && grad_D_dot && grad_params && phi,
                  MATPL_ERR_INVALID, "matpl_dp_fit_dual: null pointer argument");
    MATPL_REQUIRE(workspace && workspace_bytes >= ws_bytes_for(dtype, nrows), MATPL_ERR_WORKSPACE,
                  "matpl_dp_fit_dual: workspace smaller than matpl_dp_fit_dual_workspace_bytes()");
    MATPL_REQUIRE_ON_DEVICE(D, "matpl_dp_fit_dual");
    cudaStream_t s = as_stream(stream);
    return dtype == MATPL_F32
               ? run<float>(nrows, fit_params, D, D_dot, a, grad_D, grad_D_dot, grad_params, phi,
                            workspace, s)
               : run<double>(nrows, fit_params, D, D_dot, a, grad_D, grad_D_dot, grad_params, phi,
                             workspace, s);
}
