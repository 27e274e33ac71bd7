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
//   fit_dual_rows   CTA per tile of 32 rows, warp per 4 rows, lanes over the F = 50 columns:
//                   forward of both streams through the three tanh layers, the closed-form
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
constexpr int kRW = kTile / 8;            // rows per warp
constexpr int kNC = 2;                    // column slots per lane (lane, lane + 32) for F = 50
constexpr int kNF = 13;                   // per-row factor arrays written for the reductions

// factor arrays [kNF][rows][F] in the workspace
enum Factor { G0 = 0, GD0, X1, XD1, G1, GD1, X2, XD2, G2, GD2, C1, C2, C3 };

// out[r][col] += sum_k X[r][k] W[k][col] and outd[r][col] += sum_k Xd[r][k] W[k][col] for this
// warp's RW rows of X and Xd (row stride ldx), lanes over columns col = lane + 32 q < ncols.
template <typename T, int RW, int NC>
__device__ __forceinline__ void warp_gemm2(const T *X, const T *Xd, int ldx, int K,
                                           const T *__restrict__ W, int ldw, int ncols, int lane,
                                           T acc[RW][NC], T accd[RW][NC]) {
#pragma unroll 2
    for (int k = 0; k < K; ++k) {
        T w[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            const int col = lane + 32 * q;
            w[q] = col < ncols ? __ldg(W + (long long)k * ldw + col) : T(0);
        }
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const T xv = X[r * ldx + k], xd = Xd[r * ldx + k];
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                acc[r][q] += xv * w[q];
                accd[r][q] += xd * w[q];
            }
        }
    }
}

template <typename T>
struct RowsArgs {
    long long nrows;
    const T *fw;          // FitOff block of this element
    const T *D, *Dd;      // [nrows][DIN]
    const T *a;           // [nrows] dphi/dE of each row
    T *gD, *gDd;          // [nrows][DIN]
    T *fac;               // [kNF][nrows][F]
    double *phi;          // += sum_r (a_r E_r + E_dot_r)
};

// per row activations of the tile (dynamic shared memory): h, h_dot, z_dot of the three hidden
// layers, then the inputs of layers 2 and 3 and their tangents
constexpr int kRowsSmem = (3 * 3 + 4) * kTile * F;      // elements

template <typename T>
__global__ void __launch_bounds__(256) fit_dual_rows(RowsArgs<T> A) {
    extern __shared__ __align__(16) unsigned char fd_raw[];
    using Arr = T[kTile][F];
    Arr *sm = reinterpret_cast<Arr *>(fd_raw);
    Arr *sH = sm, *sHD = sm + 3, *sZD = sm + 6;
    Arr &sX2 = sm[9], &sXD2 = sm[10], &sX3 = sm[11], &sXD3 = sm[12];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T *fw = A.fw;
    const long long ntiles = (A.nrows + kTile - 1) / kTile;
    double phi_acc = 0.0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int rl0 = warp * kRW;                        // first local row of this warp
        const long long r0 = tile * kTile + rl0;           // its global row
        // rows past the end are computed on row 0 of the tile's range (values unused)
        long long rr[kRW];
        bool live[kRW];
#pragma unroll
        for (int r = 0; r < kRW; ++r) {
            live[r] = r0 + r < A.nrows;
            rr[r] = live[r] ? r0 + r : 0;
        }
        // ---------------- forward
        {
            T acc[kRW][kNC], accd[kRW][kNC];
#pragma unroll
            for (int r = 0; r < kRW; ++r)
#pragma unroll
                for (int q = 0; q < kNC; ++q) acc[r][q] = accd[r][q] = T(0);
            // rows r0 .. r0 + kRW - 1 are consecutive in D unless the tile runs past the end
            if (live[kRW - 1]) {
                warp_gemm2<T, kRW, kNC>(A.D + r0 * DIN, A.Dd + r0 * DIN, DIN, DIN,
                                        fw + FitOff::W0, F, F, lane, acc, accd);
            } else {
#pragma unroll
                for (int r = 0; r < kRW; ++r) {
                    T a1[1][kNC] = {}, d1[1][kNC] = {};
                    warp_gemm2<T, 1, kNC>(A.D + rr[r] * DIN, A.Dd + rr[r] * DIN, DIN, DIN,
                                          fw + FitOff::W0, F, F, lane, a1, d1);
#pragma unroll
                    for (int q = 0; q < kNC; ++q) { acc[r][q] = a1[0][q]; accd[r][q] = d1[0][q]; }
                }
            }
#pragma unroll
            for (int q = 0; q < kNC; ++q) {
                const int o = lane + 32 * q;
                if (o >= F) continue;
                const T b = fw[FitOff::B0 + o];
#pragma unroll
                for (int r = 0; r < kRW; ++r) {
                    const T h = dev_tanh(acc[r][q] + b), zd = accd[r][q];
                    sH[0][rl0 + r][o] = h;
                    sHD[0][rl0 + r][o] = (T(1) - h * h) * zd;
                    sZD[0][rl0 + r][o] = zd;
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int l = 1; l <= 2; ++l) {
            const int OW = l == 1 ? FitOff::W1 : FitOff::W2;
            const int OB = l == 1 ? FitOff::B1 : FitOff::B2;
            const int OD = l == 1 ? FitOff::DT1 : FitOff::DT2;
            const T *Xin = l == 1 ? &sH[0][rl0][0] : &sX2[rl0][0];
            const T *XDin = l == 1 ? &sHD[0][rl0][0] : &sXD2[rl0][0];
            T acc[kRW][kNC], accd[kRW][kNC];
#pragma unroll
            for (int r = 0; r < kRW; ++r)
#pragma unroll
                for (int q = 0; q < kNC; ++q) acc[r][q] = accd[r][q] = T(0);
            warp_gemm2<T, kRW, kNC>(Xin, XDin, F, F, fw + OW, F, F, lane, acc, accd);
            __syncwarp();
#pragma unroll
            for (int q = 0; q < kNC; ++q) {
                const int o = lane + 32 * q;
                if (o >= F) continue;
                const T b = fw[OB + o], dt = fw[OD + o];
#pragma unroll
                for (int r = 0; r < kRW; ++r) {
                    const int rl = rl0 + r;
                    const T h = dev_tanh(acc[r][q] + b), zd = accd[r][q];
                    const T hd = (T(1) - h * h) * zd;
                    sH[l][rl][o] = h;
                    sHD[l][rl][o] = hd;
                    sZD[l][rl][o] = zd;
                    const T xin = l == 1 ? sH[0][rl][o] : sX2[rl][o];
                    const T xdin = l == 1 ? sHD[0][rl][o] : sXD2[rl][o];
                    if (l == 1) {
                        sX2[rl][o] = h * dt + xin;
                        sXD2[rl][o] = hd * dt + xdin;
                    } else {
                        sX3[rl][o] = h * dt + xin;
                        sXD3[rl][o] = hd * dt + xdin;
                    }
                }
            }
            __syncwarp();
        }
        // output layer: E = x3 . W3 + b3, E_dot = x_dot3 . W3
        T arow[kRW];
#pragma unroll
        for (int r = 0; r < kRW; ++r) {
            T e = T(0), ed = T(0);
#pragma unroll
            for (int q = 0; q < kNC; ++q) {
                const int o = lane + 32 * q;
                if (o < F) {
                    e += sX3[rl0 + r][o] * fw[FitOff::W3 + o];
                    ed += sXD3[rl0 + r][o] * fw[FitOff::W3 + o];
                }
            }
            e = warp_sum(e);
            ed = warp_sum(ed);
            arow[r] = live[r] ? A.a[rr[r]] : T(0);
            if (lane == 0 && live[r])
                phi_acc += (double)arow[r] * (double)(e + fw[FitOff::B3]) + (double)ed;
        }
        // ---------------- reverse pass; g / gd: dphi/dx, dphi/dx_dot of the current layer's
        // output, per owned column
        T g[kRW][kNC], gd[kRW][kNC];
        const long long nr = A.nrows;
        auto fac = [&](int which, long long row, int o) -> T * {
            return A.fac + ((long long)which * nr + row) * F + o;
        };
#pragma unroll
        for (int q = 0; q < kNC; ++q) {
            const int o = lane + 32 * q;
            const T w3 = o < F ? fw[FitOff::W3 + o] : T(0);
#pragma unroll
            for (int r = 0; r < kRW; ++r) {
                g[r][q] = arow[r] * w3;
                gd[r][q] = w3;
                if (o < F && live[r])
                    *fac(C3, rr[r], o) = arow[r] * sX3[rl0 + r][o] + sXD3[rl0 + r][o];
            }
        }
        // layers 2, 1 (residual): x_out = h dt + x_in
#pragma unroll
        for (int l = 2; l >= 1; --l) {
            const int OD = l == 1 ? FitOff::DT1 : FitOff::DT2;
            const int OWT = l == 1 ? FitOff::W1T : FitOff::W2T;
            const int fG = l == 1 ? G1 : G2, fGD = l == 1 ? GD1 : GD2;
            const int fX = l == 1 ? X1 : X2, fXD = l == 1 ? XD1 : XD2;
            const int fC = l == 1 ? C1 : C2;
#pragma unroll
            for (int q = 0; q < kNC; ++q) {
                const int o = lane + 32 * q;
                if (o >= F) continue;
                const T dt = fw[OD + o];
#pragma unroll
                for (int r = 0; r < kRW; ++r) {
                    const int rl = rl0 + r;
                    const T h = sH[l][rl][o], hd = sHD[l][rl][o], zd = sZD[l][rl][o];
                    const T gh = g[r][q] * dt, ghd = gd[r][q] * dt;
                    const T s = T(1) - h * h;
                    const T dz = (gh - T(2) * ghd * h * zd) * s, dzd = ghd * s;
                    if (live[r]) {
                        *fac(fC, rr[r], o) = g[r][q] * h + gd[r][q] * hd;
                        *fac(fG, rr[r], o) = dz;
                        *fac(fGD, rr[r], o) = dzd;
                        *fac(fX, rr[r], o) = l == 1 ? sH[0][rl][o] : sX2[rl][o];
                        *fac(fXD, rr[r], o) = l == 1 ? sHD[0][rl][o] : sXD2[rl][o];
                    }
                    // the tanh values are no longer needed: dz goes in their place
                    sH[l][rl][o] = dz;
                    sHD[l][rl][o] = dzd;
                }
            }
            __syncwarp();
            T acc[kRW][kNC], accd[kRW][kNC];
#pragma unroll
            for (int r = 0; r < kRW; ++r)
#pragma unroll
                for (int q = 0; q < kNC; ++q) acc[r][q] = accd[r][q] = T(0);
            warp_gemm2<T, kRW, kNC>(&sH[l][rl0][0], &sHD[l][rl0][0], F, F, fw + OWT, F, F, lane,
                                    acc, accd);
#pragma unroll
            for (int r = 0; r < kRW; ++r)
#pragma unroll
                for (int q = 0; q < kNC; ++q) {
                    g[r][q] += acc[r][q];
                    gd[r][q] += accd[r][q];
                }
            __syncwarp();
        }
        // layer 0: x1 = tanh(D W0 + b0)
#pragma unroll
        for (int q = 0; q < kNC; ++q) {
            const int o = lane + 32 * q;
            if (o >= F) continue;
#pragma unroll
            for (int r = 0; r < kRW; ++r) {
                const int rl = rl0 + r;
                const T h = sH[0][rl][o], zd = sZD[0][rl][o];
                const T s = T(1) - h * h;
                const T dz = (g[r][q] - T(2) * gd[r][q] * h * zd) * s, dzd = gd[r][q] * s;
                if (live[r]) {
                    *fac(G0, rr[r], o) = dz;
                    *fac(GD0, rr[r], o) = dzd;
                }
                sH[0][rl][o] = dz;
                sHD[0][rl][o] = dzd;
            }
        }
        __syncwarp();
        // grad_D = dz0 W0^T, grad_D_dot = dz0_dot W0^T, two rows at a time
        constexpr int NCD = (DIN + 31) / 32;   // 13
#pragma unroll
        for (int rp = 0; rp < kRW; rp += 2) {
            T acc[2][NCD], accd[2][NCD];
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int q = 0; q < NCD; ++q) acc[r][q] = accd[r][q] = T(0);
            warp_gemm2<T, 2, NCD>(&sH[0][rl0 + rp][0], &sHD[0][rl0 + rp][0], F, F,
                                  fw + FitOff::W0T, DIN, DIN, lane, acc, accd);
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                if (!live[rp + r]) continue;
                const long long row = rr[rp + r];
#pragma unroll
                for (int q = 0; q < NCD; ++q) {
                    const int col = lane + 32 * q;
                    if (col < DIN) {
                        A.gD[row * DIN + col] = acc[r][q];
                        A.gDd[row * DIN + col] = accd[r][q];
                    }
                }
            }
        }
        __syncwarp();
    }
    if (lane == 0 && phi_acc != 0.0) atomicAdd(A.phi, phi_acc);
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
    const T *fac;         // [kNF][nrows][F]
    T *grad;              // FitOff layout W0 .. B3 (+=)
};

// blockIdx.y: 0..6 the 64-row k tiles of W0 (DIN = 400), 7: W1, 8: W2, 9: the vector sums.
// Thread (tk, tu) of a 16 x 13 grid owns outputs k = k0 + 4 tk + i, u = 4 tu + j (i, j < 4).
template <typename T>
__global__ void __launch_bounds__(256) fit_dual_wgrad(WgradArgs<T> A) {
    constexpr int SUB = kSub<T>;
    __shared__ __align__(16) T sA[2][SUB][kKT];
    __shared__ __align__(16) T sB[2][SUB][kUT];
    const long long rbeg = (long long)blockIdx.x * kChunk;
    if (rbeg >= A.nrows) return;
    const long long rend = rbeg + kChunk < A.nrows ? rbeg + kChunk : A.nrows;
    const int which = blockIdx.y;
    const long long nr = A.nrows;
    if (which == 9) {
        // bias / resnet_dt / output-layer sums: column u of the factor arrays
        const int sums[6][2] = {{G0, FitOff::B0}, {G1, FitOff::B1}, {G2, FitOff::B2},
                                {C1, FitOff::DT1}, {C2, FitOff::DT2}, {C3, FitOff::W3}};
        for (int job = threadIdx.x; job < 6 * F + 1; job += blockDim.x) {
            T s = T(0);
            if (job < 6 * F) {
                const int v = job / F, u = job - v * F;
                const T *src = A.fac + (long long)sums[v][0] * nr * F + u;
                for (long long r = rbeg; r < rend; ++r) s += src[r * F];
                atomicAdd(A.grad + sums[v][1] + u, s);
            } else {
                for (long long r = rbeg; r < rend; ++r) s += A.a[r];
                atomicAdd(A.grad + FitOff::B3, s);
            }
        }
        return;
    }
    // the product: X^T G + X_dot^T G_dot over the rows of this chunk
    const T *X, *XD, *G, *GD;
    int K, k0, gbase;
    if (which < 7) {
        X = A.D; XD = A.Dd; K = DIN; k0 = which * kKT; gbase = FitOff::W0;
        G = A.fac + (long long)G0 * nr * F; GD = A.fac + (long long)GD0 * nr * F;
    } else {
        const bool one = which == 7;
        X = A.fac + (long long)(one ? X1 : X2) * nr * F;
        XD = A.fac + (long long)(one ? XD1 : XD2) * nr * F;
        G = A.fac + (long long)(one ? G1 : G2) * nr * F;
        GD = A.fac + (long long)(one ? GD1 : GD2) * nr * F;
        K = F; k0 = 0; gbase = one ? FitOff::W1 : FitOff::W2;
    }
    const int ldx = K;
    const int tk = threadIdx.x / 13, tu = threadIdx.x - tk * 13;    // 19 x 13 (tk < 16 used)
    const bool active = threadIdx.x < 16 * 13;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    for (long long s0 = rbeg; s0 < rend; s0 += SUB) {
        __syncthreads();
        // stage X / X_dot [kSub][kKT] and G / G_dot [kSub][kUT] (zero past the ends)
        for (int q = threadIdx.x; q < SUB * kKT; q += blockDim.x) {
            const int r = q / kKT, k = q - r * kKT;
            const long long row = s0 + r;
            const bool ok = row < rend && k0 + k < K;
            sA[0][r][k] = ok ? X[row * ldx + k0 + k] : T(0);
            sA[1][r][k] = ok ? XD[row * ldx + k0 + k] : T(0);
        }
        for (int q = threadIdx.x; q < SUB * kUT; q += blockDim.x) {
            const int r = q / kUT, u = q - r * kUT;
            const long long row = s0 + r;
            const bool ok = row < rend && u < F;
            sB[0][r][u] = ok ? G[row * F + u] : T(0);
            sB[1][r][u] = ok ? GD[row * F + u] : T(0);
        }
        __syncthreads();
        if (!active) continue;
#pragma unroll 4
        for (int r = 0; r < SUB; ++r) {
#pragma unroll
            for (int st = 0; st < 2; ++st) {
                T xv[4], gv[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) xv[i] = sA[st][r][4 * tk + i];
#pragma unroll
                for (int j = 0; j < 4; ++j) gv[j] = sB[st][r][4 * tu + j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] += xv[i] * gv[j];
            }
        }
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

size_t ws_bytes_for(int dtype, long long nrows) {
    const size_t t = dtype == MATPL_F64 ? 8 : 4;
    return align_up((size_t)kNF * (size_t)nrows * F * t, 256);
}

template <typename T>
int run(long long nrows, const void *fit_params, const void *D, const void *Dd, const void *a,
        void *gD, void *gDd, void *grad, double *phi, void *ws, cudaStream_t s) {
    RowsArgs<T> R;
    R.nrows = nrows; R.fw = (const T *)fit_params; R.D = (const T *)D; R.Dd = (const T *)Dd;
    R.a = (const T *)a; R.gD = (T *)gD; R.gDd = (T *)gDd; R.fac = (T *)ws; R.phi = phi;
    const long long ntiles = (nrows + kTile - 1) / kTile;
    long long g1 = ntiles;
    const long long cap = (long long)device_sms() * 4;
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
    W.fac = (const T *)ws; W.grad = (T *)grad;
    const long long chunks = (nrows + kChunk - 1) / kChunk;
    MATPL_REQUIRE(chunks < (1LL << 31), MATPL_ERR_INVALID, "too many rows");
    {
        ProfScope ps("dp_fit_dual_wgrad", s);
        fit_dual_wgrad<T><<<dim3((unsigned)chunks, 10), 256, 0, s>>>(W);
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
