// Fused DP se_e2_a energy + force + virial (plain FP32 / FP64 SIMT form).
//
// Replaces DP.forward on the GPU (src/model/dp_dp.py:167-530): calculate_Ri, the per type-pair
// embedding nets, calculate_xyz_scater, the fitting nets, autograd dE/dRi and the
// CalcOps calculateForce / calculateVirial scatter.  Nothing per pair ever reaches HBM:
//
//   dp_pad       G(s_pad) (x) R_pad for each (t_i, t_j): empty slots enter the descriptor as
//                the constant (0 - davg)/dstd (dp_dp.py:293-297); their contribution is
//                n_empty * R_pad^T G(s_pad), evaluated once per type pair.
//   dp_embed_fwd warp per centre atom, lane per occupied slot: environment row -> embedding
//                MLP -> A[4][25] += R^T G (smem-staged, lanes own A entries) -> A / (m T).
//   dp_fit       CTA per tile of atoms: D = A^T A[:, :16], fitting net forward (Ei) and its
//                adjoint down to dE/dA, with tanh outputs kept in shared memory.
//   dp_embed_bwd warp per centre atom: recomputes the environment row and the embedding
//                activations (never stored), back-propagates dE/dA to dE/dR_k, contracts with
//                dR_k/dr (Ri_d, dp_dp.py:266-299), scatters F_j += f, F_i -= f, and keeps
//                the per-atom virial sum_k f_a Rij_c in FP64.
//   dp_reduce    per configuration: Etot = sum Ei and virial = sum of per-atom virials, FP64,
//                fixed order (deterministic).
#include "common.cuh"
#include "dp_layout.cuh"
#include "dp_env.cuh"
#include <algorithm>

namespace matpl {
int mixed_ga(int S);
size_t mixed_smem(int ntypes, int S);
size_t mixed_tile_bytes(int ntypes);
int prep_mixed_tiles(const float *params, unsigned char *out, int ntypes, cudaStream_t s);
size_t fit_tile_bytes(int ntypes, int natoms);
int launch_fit_tc(bool fast, const float *A, const int32_t *type_map, const float *params,
                  unsigned char *tiles, float *Ei, float *dA, int32_t *err, int batch, int natoms,
                  int ntypes, int present_mask, cudaStream_t s);
template <int SPLIT, bool FAST>
int launch_mixed_embed(bool backward, const int32_t *list_neigh, const int32_t *num_neigh,
                       const float *idr, const int32_t *type_map, const float *params,
                       const unsigned char *wtiles, const float *davg, const float *dstd,
                       const float *pad_or_dA, float *A_or_force, double *atom_vir, int32_t *err,
                       int batch, int natoms, int nslots, int nghost, int ntypes, int m,
                       int present_mask, double rmin, double rmax, double inv_mT,
                       cudaStream_t s);

namespace {

using namespace dp;
constexpr int kWarps = 4;
constexpr int kMaxPresent = 8;

struct EvalParams {
    int batch, natoms, nslots, nghost, ntypes, m, npresent;
    int present_mask;     // bit t set when model type t is an image type
    double rmin, rmax;
    double inv_mT;        // 1 / (m * npresent)   (dp_dp.py:413)
    // compressed model (tabulated embedding), ctab == NULL: embedding nets
    const void *ctab;     // [ntypes^2 * crows][E][cnc]
    int crows, cnc;
    double cdx, cdx10, csmin, csmax;
    int *err;
    const int32_t *num_neigh;   // [B*N][ntypes] block lengths (occupied-slot lists), or NULL
};

// --------------------------------------------------------------------------- compressed model
// G(s) and dG/ds of one type pair from the tables of calc_compress_polynomial (dp_dp.py:572-601):
// fine grid below smax (interval dx from smin), coarse grid of 10 dx above it; the interval
// index truncates; the grid point xk is formed in float32 (the reference multiplies the int64
// index by the Python float step under torch's float32 default dtype) and f2 = s - xk in the
// compute dtype; the row is idx + k * rows in both grids (the reference adds no offset for the
// coarse grid either); polynomial coefficients highest power first (calculateCompress).
template <typename T>
__device__ __forceinline__ void cmp_forward(const T *__restrict__ tab, int k, T s,
                                            const EvalParams &P, T G[E], T dG[E]) {
    const bool fine = s < (T)P.csmax;
    const T xr = fine ? (s - (T)P.csmin) / (T)P.cdx : (s - (T)P.csmax) / (T)P.cdx10;
    long long idx = (long long)xr;
    const float fi = (float)idx;
    const float xk = fine ? __fadd_rn(__fmul_rn(fi, (float)P.cdx), (float)P.csmin)
                          : __fadd_rn((float)P.csmax, __fmul_rn(__fmul_rn(fi, (float)P.cdx), 10.f));
    const T f2 = s - (T)xk;
    if (idx < 0 || idx >= P.crows) {
        if (P.err) atomicOr(P.err, MATPL_KERR_TABLE_RANGE);
        idx = idx < 0 ? 0 : P.crows - 1;
    }
    const T *c = tab + ((long long)k * P.crows + idx) * E * P.cnc;
#pragma unroll
    for (int o = 0; o < E; ++o) {
        const T *co = c + o * P.cnc;
        T g = co[0], dg = T(0);
        for (int q = 1; q < P.cnc; ++q) {
            dg = dg * f2 + g;
            g = g * f2 + co[q];
        }
        G[o] = g;
        if (dG) dG[o] = dg;
    }
}

// --------------------------------------------------------------------------- embedding MLP
// x[E] <- emb(s); optionally saves layer-1/2 tanh outputs (strided by `st`) and returns the
// layer-3 tanh output in t3.
template <typename T, bool SAVE>
__device__ __forceinline__ void emb_forward(const T *__restrict__ w, T s, T x[E], T t3[E],
                                            T *t1s, T *t2s, int st) {
#pragma unroll
    for (int o = 0; o < E; ++o) {
        x[o] = dev_tanh(s * w[EmbOff::W0 + o] + w[EmbOff::B0 + o]);
        if (SAVE) t1s[o * st] = x[o];
    }
    // Warp barriers between layers keep the scheduler from hoisting the next layer's weight
    // loads over the current one (that blows the register file of the backward kernel).
    if (SAVE) __syncwarp();
    T h[E];
#pragma unroll
    for (int o = 0; o < E; ++o) h[o] = w[EmbOff::B1 + o];
#pragma unroll
    for (int i = 0; i < E; ++i)
#pragma unroll
        for (int o = 0; o < E; ++o) h[o] += x[i] * w[EmbOff::W1 + i * E + o];
#pragma unroll
    for (int o = 0; o < E; ++o) {
        const T t = dev_tanh(h[o]);
        if (SAVE) t2s[o * st] = t;
        x[o] = t * w[EmbOff::DT1 + o] + x[o];
    }
    if (SAVE) __syncwarp();
#pragma unroll
    for (int o = 0; o < E; ++o) h[o] = w[EmbOff::B2 + o];
#pragma unroll
    for (int i = 0; i < E; ++i)
#pragma unroll
        for (int o = 0; o < E; ++o) h[o] += x[i] * w[EmbOff::W2 + i * E + o];
#pragma unroll
    for (int o = 0; o < E; ++o) {
        const T t = dev_tanh(h[o]);
        t3[o] = t;
        x[o] = t * w[EmbOff::DT2 + o] + x[o];
    }
}

// --------------------------------------------------------------------------- dp_pad
// One warp per (t_i, t_j) net, lane o holding output o of every layer (the layer inputs are
// broadcast by shuffles): the same arithmetic, term order and tanh as emb_forward.
template <typename T>
__global__ void dp_pad(const T *__restrict__ params, const T *__restrict__ davg,
                       const T *__restrict__ dstd, T *__restrict__ pad, int ntypes,
                       EvalParams P) {
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= ntypes * ntypes) return;
    const int ti = k / ntypes;
    T rp[4];
    for (int c = 0; c < 4; ++c) rp[c] = (T(0) - davg[4 * ti + c]) / dstd[4 * ti + c];
    T xo = T(0);
    if (P.ctab) {
        T x[E];
        if (lane == 0) cmp_forward<T>((const T *)P.ctab, k, rp[0], P, x, nullptr);
#pragma unroll
        for (int p = 0; p < E; ++p) {
            const T v = __shfl_sync(0xffffffffu, x[p], 0);
            if (lane == p) xo = v;
        }
    } else {
        const T *w = params + (long long)k * EmbOff::SIZE;
        const int o = lane < E ? lane : 0;
        xo = dev_tanh(rp[0] * w[EmbOff::W0 + o] + w[EmbOff::B0 + o]);
        for (int l = 0; l < 2; ++l) {
            const T *W = w + (l == 0 ? EmbOff::W1 : EmbOff::W2);
            T h = w[(l == 0 ? EmbOff::B1 : EmbOff::B2) + o];
#pragma unroll
            for (int i = 0; i < E; ++i) h += __shfl_sync(0xffffffffu, xo, i) * W[i * E + o];
            xo = dev_tanh(h) * w[(l == 0 ? EmbOff::DT1 : EmbOff::DT2) + o] + xo;
        }
    }
    if (lane < E)
        for (int c = 0; c < 4; ++c) pad[(long long)k * NA + c * E + lane] = rp[c] * xo;
}

// Build the warp's list of occupied slots of one centre atom (ascending slot order) and
// return its length.  Slots of image types that are absent are skipped.
__device__ __forceinline__ int scan_slots(const int32_t *__restrict__ ln,
                                          const int32_t *__restrict__ counts, int nt, int S,
                                          int m, int present_mask, int *list, int lane) {
    int cnt = 0;
    if (counts) {            // block lengths given: the occupied slots are each block's prefix
        for (int tj = 0; tj < nt; ++tj) {
            if (!((present_mask >> tj) & 1)) continue;
            int c = counts[tj];
            c = c < 0 ? 0 : (c > m ? m : c);
            for (int k = lane; k < c; k += 32) list[cnt + k] = tj * m + k;
            cnt += c;
        }
        __syncwarp();
        return cnt;
    }
    for (int s0 = 0; s0 < S; s0 += 32) {
        const int s = s0 + lane;
        const int v = s < S ? ln[s] : 0;
        const int blk = s / m;
        const bool active = v != 0 && blk < 16 && ((present_mask >> blk) & 1);
        const unsigned msk = __ballot_sync(0xffffffffu, active);
        if (active) list[cnt + __popc(msk & ((1u << lane) - 1u))] = s;
        cnt += __popc(msk);
    }
    __syncwarp();
    return cnt;
}

// Occupied slots of type block tj in the (ascending) list.
__device__ __forceinline__ int count_block(const int *list, int cnt, int m, int tj, int lane) {
    int c = 0;
    for (int k = lane; k < cnt; k += 32) c += (list[k] / m) == tj;
    return warp_sum(c);
}

template <typename T>
__device__ __forceinline__ void stage_weights(const T *__restrict__ src, T *dst, long long n) {
    for (long long q = threadIdx.x; q < n; q += blockDim.x) dst[q] = src[q];
    __syncthreads();
}

// --------------------------------------------------------------------------- dp_embed_fwd
template <typename T, bool WS, bool CMP>
__global__ void __launch_bounds__(kWarps * 32)
dp_embed_fwd(const int32_t *__restrict__ list_neigh, const T *__restrict__ idr,
             const int32_t *__restrict__ type_map, const T *__restrict__ params,
             const T *__restrict__ davg, const T *__restrict__ dstd, const T *__restrict__ pad,
             T *__restrict__ Aout, EvalParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nnet = P.ntypes * P.ntypes;
    T *wsm = reinterpret_cast<T *>(smem_raw);
    const int wcount = WS ? nnet * EmbOff::SIZE : 0;
    T *Gs_all = wsm + wcount;                                  // [kWarps][32][E+1]
    T *Rs_all = Gs_all + kWarps * 32 * (E + 1);                // [kWarps][32][4]
    int *list_all = reinterpret_cast<int *>(Rs_all + kWarps * 32 * 4);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *Gs = Gs_all + warp * 32 * (E + 1);
    T *Rs = Rs_all + warp * 32 * 4;
    int *list = list_all + warp * P.nslots;
    if (WS) stage_weights(params, wsm, wcount);
    const int S = P.nslots;
    const long long total = (long long)P.batch * P.natoms;
    for (long long t = (long long)blockIdx.x * kWarps + warp; t < total;
         t += (long long)gridDim.x * kWarps) {
        const int i = (int)(t % P.natoms);
        const int ti = type_map[i];
        T *Arow = Aout + t * NA;
        if (ti < 0 || ti >= P.ntypes || !((P.present_mask >> ti) & 1)) {
            for (int e = lane; e < NA; e += 32) Arow[e] = T(0);
            continue;
        }
        const int cnt = scan_slots(list_neigh + t * S, P.num_neigh ? P.num_neigh + t * P.ntypes : nullptr,
                                       P.ntypes, S, P.m, P.present_mask, list, lane);
        T acc[4] = {T(0), T(0), T(0), T(0)};
        const T *avg = davg + 4 * ti;
        const T *sd = dstd + 4 * ti;
        for (int c0 = 0; c0 < cnt; c0 += 32) {
            const int k = c0 + lane;
            T x[E], t3[E], rh[4] = {T(0), T(0), T(0), T(0)};
            int tj = 0;
            T R = T(0), px = T(0), py = T(0), pz = T(0);
            if (k < cnt) {
                const int slot = list[k];
                tj = slot / P.m;
                const T *row = idr + (t * S + slot) * 4;
                R = row[0]; px = row[1]; py = row[2]; pz = row[3];
            }
            env_row(R, px, py, pz, (T)P.rmin, (T)P.rmax, avg, sd, rh);
            const T *w = WS ? wsm + (ti * P.ntypes + tj) * EmbOff::SIZE
                            : params + (long long)(ti * P.ntypes + tj) * EmbOff::SIZE;
            if (CMP) cmp_forward<T>((const T *)P.ctab, ti * P.ntypes + tj, rh[0], P, x, nullptr);
            else emb_forward<T, false>(w, rh[0], x, t3, nullptr, nullptr, 0);
            if (k >= cnt) {
#pragma unroll
                for (int c = 0; c < 4; ++c) rh[c] = T(0);
            }
            __syncwarp();
#pragma unroll
            for (int p = 0; p < E; ++p) Gs[lane * (E + 1) + p] = x[p];
#pragma unroll
            for (int c = 0; c < 4; ++c) Rs[lane * 4 + c] = rh[c];
            __syncwarp();
            const int nv = min(32, cnt - c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = lane + 32 * q;
                if (e < NA) {
                    const int c = e / E, p = e - (e / E) * E;
                    T a = acc[q];
                    for (int l = 0; l < nv; ++l) a += Rs[l * 4 + c] * Gs[l * (E + 1) + p];
                    acc[q] = a;
                }
            }
        }
        // empty slots: n_empty(t_j) * R_pad (x) G(s_pad)
        for (int tj = 0; tj < P.ntypes; ++tj) {
            if (!((P.present_mask >> tj) & 1)) continue;
            const T nemp = (T)(P.m - count_block(list, cnt, P.m, tj, lane));
            const T *pp = pad + (long long)(ti * P.ntypes + tj) * NA;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = lane + 32 * q;
                if (e < NA) acc[q] += nemp * pp[e];
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = lane + 32 * q;
            if (e < NA) Arow[e] = acc[q] * (T)P.inv_mT;
        }
        __syncwarp();
    }
}

// --------------------------------------------------------------------------- dp_fit
// Row-tiled GEMM helper: out[r][col] (+)= sum_k X[r][k] * W[k][col] for this warp's rows.
template <typename T, int RW, int NC>
__device__ __forceinline__ void warp_gemm(const T *X, int ldx, int K, const T *__restrict__ W,
                                          int ldw, int ncols, int lane, T acc[RW][NC]) {
    for (int k = 0; k < K; ++k) {
        T w[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            const int col = lane + 32 * q;
            w[q] = col < ncols ? W[(long long)k * ldw + col] : T(0);
        }
#pragma unroll
        for (int r = 0; r < RW; ++r) {
            const T xv = X[r * ldx + k];
#pragma unroll
            for (int q = 0; q < NC; ++q) acc[r][q] += xv * w[q];
        }
    }
}

template <typename T, int TILE>
__global__ void __launch_bounds__(256)
dp_fit(const T *__restrict__ Ain, const int32_t *__restrict__ type_map,
       const T *__restrict__ params, T *__restrict__ Ei, T *__restrict__ dAout, EvalParams P) {
    constexpr int RW = TILE / 8;                 // rows per warp
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *As = reinterpret_cast<T *>(smem_raw);     // [TILE][NA]
    T *Ds = As + TILE * NA;                      // [TILE][DIN]  (D, later dE/dD)
    T *T1 = Ds + TILE * DIN;                     // [TILE][F]
    T *T2 = T1 + TILE * F;
    T *T3 = T2 + TILE * F;
    T *X = T3 + TILE * F;                        // [TILE][F] running activation / adjoint
    __shared__ int rtype[TILE];
    __shared__ int tflag[16];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long total = (long long)P.batch * P.natoms;
    const long long ntiles = (total + TILE - 1) / TILE;
    const long long woff = (long long)P.ntypes * P.ntypes * EmbOff::SIZE;

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long t0 = tile * TILE;
        __syncthreads();
        for (int q = threadIdx.x; q < 16; q += blockDim.x) tflag[q] = 0;
        __syncthreads();
        for (int r = threadIdx.x; r < TILE; r += blockDim.x) {
            const long long t = t0 + r;
            int ty = -1;
            if (t < total) {
                ty = type_map[(int)(t % P.natoms)];
                if (ty < 0 || ty >= P.ntypes || !((P.present_mask >> ty) & 1)) ty = -1;
            }
            rtype[r] = ty;
            if (ty >= 0) tflag[ty] = 1;
        }
        for (int q = threadIdx.x; q < TILE * NA; q += blockDim.x) {
            const long long t = t0 + q / NA;
            As[q] = t < total ? Ain[t0 * NA + q] : T(0);
        }
        __syncthreads();
        for (int tt = 0; tt < P.ntypes; ++tt) {
            if (!tflag[tt]) continue;
            const T *fw = params + woff + (long long)tt * FitOff::SIZE;
            // D[r][p*M2+q] = sum_c A[r][c][p] A[r][c][q]
            for (int q = threadIdx.x; q < TILE * DIN; q += blockDim.x) {
                const int r = q / DIN, e = q - r * DIN;
                const int p = e / M2, qq = e - p * M2;
                const T *a = As + r * NA;
                Ds[q] = a[p] * a[qq] + a[E + p] * a[E + qq] + a[2 * E + p] * a[2 * E + qq] +
                        a[3 * E + p] * a[3 * E + qq];
            }
            __syncthreads();
            const int r0 = warp * RW;
            {   // layer 0: T1 = tanh(D W0 + b0), X = T1
                T acc[RW][2];
#pragma unroll
                for (int r = 0; r < RW; ++r) { acc[r][0] = T(0); acc[r][1] = T(0); }
                warp_gemm<T, RW, 2>(Ds + r0 * DIN, DIN, DIN, fw + FitOff::W0, F, F, lane, acc);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int o = lane + 32 * q;
                    if (o < F) {
                        const T b = fw[FitOff::B0 + o];
#pragma unroll
                        for (int r = 0; r < RW; ++r) {
                            const T tv = dev_tanh(acc[r][q] + b);
                            T1[(r0 + r) * F + o] = tv;
                            X[(r0 + r) * F + o] = tv;
                        }
                    }
                }
            }
            __syncwarp();
            // layers 1, 2: X = tanh(X W + b) * dt + X
#pragma unroll
            for (int l = 1; l <= 2; ++l) {
                const int OW = l == 1 ? FitOff::W1 : FitOff::W2;
                const int OB = l == 1 ? FitOff::B1 : FitOff::B2;
                const int OD = l == 1 ? FitOff::DT1 : FitOff::DT2;
                T *Tl = l == 1 ? T2 : T3;
                T acc[RW][2];
#pragma unroll
                for (int r = 0; r < RW; ++r) { acc[r][0] = T(0); acc[r][1] = T(0); }
                warp_gemm<T, RW, 2>(X + r0 * F, F, F, fw + OW, F, F, lane, acc);
                __syncwarp();
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int o = lane + 32 * q;
                    if (o < F) {
                        const T b = fw[OB + o], dt = fw[OD + o];
#pragma unroll
                        for (int r = 0; r < RW; ++r) {
                            const T tv = dev_tanh(acc[r][q] + b);
                            Tl[(r0 + r) * F + o] = tv;
                            X[(r0 + r) * F + o] = tv * dt + X[(r0 + r) * F + o];
                        }
                    }
                }
                __syncwarp();
            }
            // Ei = X W3 + b3 ; backward seed dX = W3
#pragma unroll
            for (int r = 0; r < RW; ++r) {
                T part = T(0);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int o = lane + 32 * q;
                    if (o < F) part += X[(r0 + r) * F + o] * fw[FitOff::W3 + o];
                }
                part = warp_sum(part);
                const long long t = t0 + r0 + r;
                if (lane == 0 && t < total && rtype[r0 + r] == tt) Ei[t] = part + fw[FitOff::B3];
            }
            __syncwarp();
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int o = lane + 32 * q;
                if (o < F)
#pragma unroll
                    for (int r = 0; r < RW; ++r) X[(r0 + r) * F + o] = fw[FitOff::W3 + o];
            }
            __syncwarp();
            // back through layers 2, 1: g = dX * dt * (1 - t^2);  dX += g W^T
#pragma unroll
            for (int l = 2; l >= 1; --l) {
                const int OWT = l == 1 ? FitOff::W1T : FitOff::W2T;
                const int OD = l == 1 ? FitOff::DT1 : FitOff::DT2;
                T *Tl = l == 1 ? T2 : T3;
                // g into Tl (tanh values no longer needed afterwards)
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int o = lane + 32 * q;
                    if (o < F) {
                        const T dt = fw[OD + o];
#pragma unroll
                        for (int r = 0; r < RW; ++r) {
                            const T tv = Tl[(r0 + r) * F + o];
                            Tl[(r0 + r) * F + o] = X[(r0 + r) * F + o] * dt * (T(1) - tv * tv);
                        }
                    }
                }
                __syncwarp();
                T acc[RW][2];
#pragma unroll
                for (int r = 0; r < RW; ++r) { acc[r][0] = T(0); acc[r][1] = T(0); }
                warp_gemm<T, RW, 2>(Tl + r0 * F, F, F, fw + OWT, F, F, lane, acc);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int o = lane + 32 * q;
                    if (o < F)
#pragma unroll
                        for (int r = 0; r < RW; ++r) X[(r0 + r) * F + o] += acc[r][q];
                }
                __syncwarp();
            }
            // layer 0: g1 = dX * (1 - T1^2);  dD = g1 W0^T  (into Ds)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int o = lane + 32 * q;
                if (o < F)
#pragma unroll
                    for (int r = 0; r < RW; ++r) {
                        const T tv = T1[(r0 + r) * F + o];
                        T1[(r0 + r) * F + o] = X[(r0 + r) * F + o] * (T(1) - tv * tv);
                    }
            }
            __syncwarp();
            {
                constexpr int NC = (DIN + 31) / 32;   // 13
                T acc[RW][NC];
#pragma unroll
                for (int r = 0; r < RW; ++r)
#pragma unroll
                    for (int q = 0; q < NC; ++q) acc[r][q] = T(0);
                warp_gemm<T, RW, NC>(T1 + r0 * F, F, F, fw + FitOff::W0T, DIN, DIN, lane, acc);
#pragma unroll
                for (int q = 0; q < NC; ++q) {
                    const int col = lane + 32 * q;
                    if (col < DIN)
#pragma unroll
                        for (int r = 0; r < RW; ++r) Ds[(r0 + r) * DIN + col] = acc[r][q];
                }
            }
            __syncthreads();
            // dA[r][c][p] = sum_q dD[p][q] A[c][q] + (p < M2 ? sum_p' dD[p'][p] A[c][p'] : 0)
            for (int q = threadIdx.x; q < TILE * NA; q += blockDim.x) {
                const int r = q / NA, e = q - r * NA;
                const long long t = t0 + r;
                if (t >= total || rtype[r] != tt) continue;
                const int c = e / E, p = e - c * E;
                const T *dd = Ds + r * DIN;
                const T *a = As + r * NA + c * E;
                T v = T(0);
#pragma unroll
                for (int qq = 0; qq < M2; ++qq) v += dd[p * M2 + qq] * a[qq];
                if (p < M2) {
#pragma unroll
                    for (int pp = 0; pp < E; ++pp) v += dd[pp * M2 + p] * a[pp];
                }
                dAout[t * NA + e] = v;
            }
            __syncthreads();
        }
        // rows without a present type
        for (int q = threadIdx.x; q < TILE * NA; q += blockDim.x) {
            const int r = q / NA;
            const long long t = t0 + r;
            if (t < total && rtype[r] < 0) dAout[t * NA + (q - r * NA)] = T(0);
        }
        for (int r = threadIdx.x; r < TILE; r += blockDim.x) {
            const long long t = t0 + r;
            if (t < total && rtype[r] < 0) Ei[t] = T(0);
        }
    }
}

// --------------------------------------------------------------------------- dp_embed_bwd
template <typename T, bool WS, bool CMP>
__global__ void __launch_bounds__(kWarps * 32)
dp_embed_bwd(const int32_t *__restrict__ list_neigh, const T *__restrict__ idr,
             const int32_t *__restrict__ type_map, const T *__restrict__ params,
             const T *__restrict__ davg, const T *__restrict__ dstd, const T *__restrict__ dAin,
             T *__restrict__ force, double *__restrict__ atom_vir, EvalParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nnet = P.ntypes * P.ntypes;
    T *wsm = reinterpret_cast<T *>(smem_raw);
    const int wcount = WS ? nnet * EmbOff::SIZE : 0;
    T *act_all = wsm + wcount;                                 // [kWarps][2][E][32]
    T *dA_all = act_all + kWarps * 2 * E * 32;                 // [kWarps][NA]
    int *list_all = reinterpret_cast<int *>(dA_all + kWarps * NA);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *t1s = act_all + warp * 2 * E * 32 + lane;
    T *t2s = t1s + E * 32;
    T *dAs = dA_all + warp * NA;
    int *list = list_all + warp * P.nslots;
    if (WS) stage_weights(params, wsm, wcount);
    const int S = P.nslots;
    const int nall = P.natoms + P.nghost;
    const long long total = (long long)P.batch * P.natoms;
    for (long long t = (long long)blockIdx.x * kWarps + warp; t < total;
         t += (long long)gridDim.x * kWarps) {
        const int b = (int)(t / P.natoms);
        const int i = (int)(t - (long long)b * P.natoms);
        const int ti = type_map[i];
        double vir[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) vir[q] = 0.0;
        if (ti >= 0 && ti < P.ntypes && ((P.present_mask >> ti) & 1)) {
            const int cnt = scan_slots(list_neigh + t * S, P.num_neigh ? P.num_neigh + t * P.ntypes : nullptr,
                                       P.ntypes, S, P.m, P.present_mask, list, lane);
            for (int e = lane; e < NA; e += 32) dAs[e] = dAin[t * NA + e] * (T)P.inv_mT;
            __syncwarp();
            const T *avg = davg + 4 * ti;
            const T *sd = dstd + 4 * ti;
            T fi[3] = {T(0), T(0), T(0)};
            for (int c0 = 0; c0 < cnt; c0 += 32) {
                const int k = c0 + lane;
                int tj = 0, j = -1;
                T R = T(0), px = T(0), py = T(0), pz = T(0);
                if (k < cnt) {
                    const int slot = list[k];
                    tj = slot / P.m;
                    j = list_neigh[t * S + slot] - 1;
                    const T *row = idr + (t * S + slot) * 4;
                    R = row[0]; px = row[1]; py = row[2]; pz = row[3];
                }
                T rh[4];
                env_row(R, px, py, pz, (T)P.rmin, (T)P.rmax, avg, sd, rh);
                const T *w = WS ? wsm + (ti * P.ntypes + tj) * EmbOff::SIZE
                                : params + (long long)(ti * P.ntypes + tj) * EmbOff::SIZE;
                T x[E], h[E];
                if (CMP) cmp_forward<T>((const T *)P.ctab, ti * P.ntypes + tj, rh[0], P, x, h);
                else emb_forward<T, true>(w, rh[0], x, h, t1s, t2s, 32);
                // dE/dR_k[c] = sum_p dA[c][p] G[p];  dE/dG[p] = sum_c dA[c][p] R_k[c]
                T g[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int p = 0; p < E; ++p) {
                    const T gp = x[p];
                    g[0] += dAs[p] * gp;
                    g[1] += dAs[E + p] * gp;
                    g[2] += dAs[2 * E + p] * gp;
                    g[3] += dAs[3 * E + p] * gp;
                    x[p] = dAs[p] * rh[0] + dAs[E + p] * rh[1] + dAs[2 * E + p] * rh[2] +
                           dAs[3 * E + p] * rh[3];
                }
                __syncwarp();
                T dsv = T(0);
                if (CMP) {
                    // tabulated embedding: dE/ds = sum_p dE/dG[p] dG[p]/ds (dG in h)
#pragma unroll
                    for (int p = 0; p < E; ++p) dsv += x[p] * h[p];
                } else {
                // layer 2 adjoint: G = t3*dt2 + x2
#pragma unroll
                for (int o = 0; o < E; ++o) h[o] = x[o] * w[EmbOff::DT2 + o] * (T(1) - h[o] * h[o]);
#pragma unroll
                for (int ii = 0; ii < E; ++ii) {
                    T a = x[ii];
#pragma unroll
                    for (int o = 0; o < E; ++o) a += w[EmbOff::W2 + ii * E + o] * h[o];
                    x[ii] = a;
                }
                __syncwarp();
                // layer 1 adjoint: x2 = t2*dt1 + x1
#pragma unroll
                for (int o = 0; o < E; ++o) {
                    const T tv = t2s[o * 32];
                    h[o] = x[o] * w[EmbOff::DT1 + o] * (T(1) - tv * tv);
                }
#pragma unroll
                for (int ii = 0; ii < E; ++ii) {
                    T a = x[ii];
#pragma unroll
                    for (int o = 0; o < E; ++o) a += w[EmbOff::W1 + ii * E + o] * h[o];
                    x[ii] = a;
                }
                __syncwarp();
                // layer 0 adjoint: x1 = tanh(s W0 + b0)
#pragma unroll
                for (int o = 0; o < E; ++o) {
                    const T tv = t1s[o * 32];
                    dsv += w[EmbOff::W0 + o] * x[o] * (T(1) - tv * tv);
                }
                }
                g[0] += dsv;
                T f[3];
                contract_rid(R, px, py, pz, (T)P.rmin, (T)P.rmax, sd, g, f);
                if (k < cnt) {
                    fi[0] -= f[0]; fi[1] -= f[1]; fi[2] -= f[2];
                    if (j >= 0 && j < nall) {
                        T *dst = force + ((long long)b * nall + j) * 3;
                        atomicAdd(dst + 0, f[0]);
                        atomicAdd(dst + 1, f[1]);
                        atomicAdd(dst + 2, f[2]);
                    }
                    const double rr[3] = {(double)px, (double)py, (double)pz};
#pragma unroll
                    for (int a = 0; a < 3; ++a)
#pragma unroll
                        for (int c = 0; c < 3; ++c) vir[3 * a + c] += (double)f[a] * rr[c];
                }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) fi[a] = warp_sum(fi[a]);
            if (lane == 0) {
                T *dst = force + ((long long)b * nall + i) * 3;
                atomicAdd(dst + 0, fi[0]);
                atomicAdd(dst + 1, fi[1]);
                atomicAdd(dst + 2, fi[2]);
            }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) vir[q] = warp_sum(vir[q]);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < 9; ++q) atom_vir[t * 9 + q] = vir[q];
        __syncwarp();
    }
}

// --------------------------------------------------------------------------- dp_reduce
// Two fixed-order passes (deterministic): kReduceBlocks partial sums per configuration, then
// one warp per configuration adds the partials in index order.
constexpr int kReduceBlocks = 64;

template <typename T>
__global__ void dp_reduce_partial(const T *__restrict__ Ei, const double *__restrict__ atom_vir,
                                  double *__restrict__ part_out, int natoms) {
    const int b = blockIdx.y;
    __shared__ double part[10][8];
    double acc[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) acc[q] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < natoms; i += gridDim.x * blockDim.x) {
        const long long t = (long long)b * natoms + i;
        acc[0] += (double)Ei[t];
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q + 1] += atom_vir[t * 9 + q];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 10; ++q) {
        const double v = warp_sum(acc[q]);
        if (lane == 0) part[q][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 10) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += part[threadIdx.x][w];
        part_out[((long long)b * gridDim.x + blockIdx.x) * 10 + threadIdx.x] = v;
    }
}

// One warp per output (E, then the nine virial components): lanes over the partial sums, then
// a fixed shuffle tree, so the order of the additions never changes.
__global__ void dp_reduce_final(const double *__restrict__ part, double *__restrict__ Etot,
                                double *__restrict__ virial, int nblk) {
    const int b = blockIdx.x;
    const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (q >= 10) return;
    double v = 0.0;
    for (int k = lane; k < nblk; k += 32) v += part[((long long)b * nblk + k) * 10 + q];
    v = warp_sum(v);
    if (lane == 0) {
        if (q == 0) Etot[b] = v;
        else virial[b * 9 + q - 1] = v;
    }
}

struct DpLayout {
    size_t A, dA, pad, vir, red, tiles, ftiles, total;
};

DpLayout dp_layout(size_t es, int batch, int natoms, int ntypes) {
    DpLayout l;
    size_t o = 0;
    const size_t na = (size_t)batch * natoms;
    l.A = o;   o = align_up(o + es * na * NA, 256);
    l.dA = o;  o = align_up(o + es * na * NA, 256);
    l.pad = o; o = align_up(o + es * (size_t)ntypes * ntypes * NA, 256);
    l.vir = o; o = align_up(o + 8 * na * 9, 256);
    l.red = o; o = align_up(o + 8 * (size_t)batch * kReduceBlocks * 10, 256);
    l.tiles = o; o = align_up(o + mixed_tile_bytes(ntypes), 256);
    l.ftiles = o; o = align_up(o + fit_tile_bytes(ntypes, natoms), 256);
    l.total = o;
    return l;
}

template <typename T>
int run_mixed(int mode, bool backward, const EvalParams &P, const int32_t *ln, const T *idr,
              const int32_t *tm, const T *params, const unsigned char *wt, const T *davg,
              const T *dstd, const T *in, T *out, double *avir, int32_t *err, cudaStream_t s) {
    if (sizeof(T) != 4) return MATPL_ERR_DTYPE;
    const float *fi = (const float *)idr;
    const float *fp = (const float *)params, *fa = (const float *)davg, *fs = (const float *)dstd;
    const float *fin = (const float *)in;
    float *fo = (float *)out;
    switch (mode) {
        case MATPL_MIXED:
            return launch_mixed_embed<3, true>(backward, ln, P.num_neigh, fi, tm, fp, wt, fa, fs, fin, fo, avir, err,
                                               P.batch, P.natoms, P.nslots, P.nghost, P.ntypes,
                                               P.m, P.present_mask, P.rmin, P.rmax, P.inv_mT, s);
        case MATPL_MIXED_FAST:
            return launch_mixed_embed<1, true>(backward, ln, P.num_neigh, fi, tm, fp, wt, fa, fs, fin, fo, avir, err,
                                               P.batch, P.natoms, P.nslots, P.nghost, P.ntypes,
                                               P.m, P.present_mask, P.rmin, P.rmax, P.inv_mT, s);
        default:
            return launch_mixed_embed<3, false>(backward, ln, P.num_neigh, fi, tm, fp, wt, fa, fs, fin, fo, avir,
                                                err, P.batch, P.natoms, P.nslots, P.nghost,
                                                P.ntypes, P.m, P.present_mask, P.rmin, P.rmax,
                                                P.inv_mT, s);
    }
}

template <typename T>
int launch_eval(int mode, const matpl_dp_model *M, const EvalParams &P,
                const int32_t *list_neigh, const T *idr, const int32_t *type_map, T *Ei,
                double *Etot, T *force, double *virial, char *ws, const DpLayout &lay,
                cudaStream_t s) {
    const T *params = (const T *)M->params;
    const T *davg = (const T *)M->davg, *dstd = (const T *)M->dstd;
    T *A = (T *)(ws + lay.A), *dA = (T *)(ws + lay.dA), *pad = (T *)(ws + lay.pad);
    double *avir = (double *)(ws + lay.vir);
    unsigned char *wt = (unsigned char *)(ws + lay.tiles);
    const long long total = (long long)P.batch * P.natoms;
    const size_t nall3 = (size_t)P.batch * (P.natoms + P.nghost) * 3;
    if (cudaMemsetAsync(force, 0, sizeof(T) * nall3, s) != cudaSuccess) {
        set_error("matpl_dp_eval: memset failed");
        return MATPL_ERR_CUDA;
    }
    const int nnet = P.ntypes * P.ntypes;
    {
        ProfScope ps("dp_pad", s);
        dp_pad<T><<<(nnet + 3) / 4, 128, 0, s>>>(params, davg, dstd, pad, P.ntypes, P);
    }

    const long long nwarp_blocks = (total + kWarps - 1) / kWarps;
    const int gridw = (int)(nwarp_blocks < (long long)device_sms() * 8 ? (nwarp_blocks < 1 ? 1 : nwarp_blocks) : (long long)device_sms() * 8);
    const size_t wbytes = sizeof(T) * (size_t)nnet * EmbOff::SIZE;
    const bool ws_ok = wbytes <= 128 * 1024 && P.ctab == nullptr;   // tables: no net weights
    const size_t wpart = ws_ok ? wbytes : 0;
    const size_t smem_f = wpart + sizeof(T) * kWarps * 32 * (E + 1 + 4) +
                          sizeof(int) * kWarps * P.nslots;
    const size_t smem_b = wpart + sizeof(T) * kWarps * (2 * E * 32 + NA) +
                          sizeof(int) * kWarps * P.nslots;
    auto kf = P.ctab ? dp_embed_fwd<T, false, true>
                     : (ws_ok ? dp_embed_fwd<T, true, false> : dp_embed_fwd<T, false, false>);
    auto kb = P.ctab ? dp_embed_bwd<T, false, true>
                     : (ws_ok ? dp_embed_bwd<T, true, false> : dp_embed_bwd<T, false, false>);
    int st = MATPL_OK;
    // compressed models take the SIMT embedding kernels in every form (the table polynomial is
    // no GEMM); the mixed forms still run the fitting nets on the tensor cores
    const bool simt_embed = mode == MATPL_F32 || mode == MATPL_F64 || P.ctab != nullptr;
    if (simt_embed) {
        cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f);
        cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
        ProfScope ps("dp_embed_fwd", s);
        kf<<<gridw, kWarps * 32, smem_f, s>>>(list_neigh, idr, type_map, params, davg, dstd, pad, A, P);
    } else {
        st = prep_mixed_tiles((const float *)params, wt, P.ntypes, s);
        if (st) return st;
        st = run_mixed(mode, false, P, list_neigh, idr, type_map, params, wt, davg, dstd, pad, A,
                       nullptr, M->err_dev, s);
        if (st) return st;
    }
    constexpr int TILE = sizeof(T) == 8 ? 32 : 64;
    const size_t smem_fit = sizeof(T) * (size_t)TILE * (NA + DIN + 4 * F);
    cudaFuncSetAttribute(dp_fit<T, TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_fit);
    const long long ntiles = (total + TILE - 1) / TILE;
    const int gridf = (int)(ntiles < (long long)device_sms() * 4 ? ntiles : (long long)device_sms() * 4);
    if (mode == MATPL_F32 || mode == MATPL_F64) {
        ProfScope ps("dp_fit", s);
        dp_fit<T, TILE><<<gridf, 256, smem_fit, s>>>(A, type_map, params, Ei, dA, P);
    } else {
        st = launch_fit_tc(mode != MATPL_MIXED_TANHF, (const float *)A, type_map, (const float *)params,
                           (unsigned char *)(ws + lay.ftiles), (float *)Ei, (float *)dA,
                           M->err_dev, P.batch, P.natoms, P.ntypes, P.present_mask, s);
        if (st) return st;
    }
    if (simt_embed) {
        ProfScope ps("dp_embed_bwd", s);
        kb<<<gridw, kWarps * 32, smem_b, s>>>(list_neigh, idr, type_map, params, davg, dstd, dA,
                                              force, avir, P);
    } else {
        st = run_mixed(mode, true, P, list_neigh, idr, type_map, params, wt, davg, dstd, dA,
                       force, avir, M->err_dev, s);
        if (st) return st;
    }
    {
        ProfScope ps("dp_reduce", s);
        const int nblk = (int)std::min<long long>(kReduceBlocks, (P.natoms + 255) / 256);
        double *red = (double *)(ws + lay.red);
        dp_reduce_partial<T><<<dim3(nblk, P.batch), 256, 0, s>>>(Ei, avir, red, P.natoms);
        dp_reduce_final<<<P.batch, 320, 0, s>>>(red, Etot, virial, nblk);
    }
    return check_launch("matpl_dp_eval");
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" size_t matpl_dp_param_count(int ntypes) {
    return ntypes < 1 ? 0 : (size_t)dp::param_count(ntypes);
}

extern "C" size_t matpl_dp_workspace_bytes(int dtype, int batch, int natoms) {
    const size_t es = dtype == MATPL_F64 ? 8 : 4;
    return dp_layout(es, batch < 0 ? 0 : batch, natoms < 0 ? 0 : natoms, 16).total;
}

static int dp_eval(int dtype, const matpl_dp_model *model, int batch, int natoms, int nslots,
                   int nghost, const int32_t *list_neigh, const int32_t *num_neigh,
                   const void *image_dr, const int32_t *type_map, void *Ei, double *Etot,
                   void *force, double *virial, void *workspace, size_t workspace_bytes,
                   void *stream) {
    MATPL_REQUIRE(model != nullptr, MATPL_ERR_INVALID, "model is NULL");
    MATPL_REQUIRE(dtype >= MATPL_F32 && dtype <= MATPL_MIXED_TANHF, MATPL_ERR_DTYPE,
                  "matpl_dp_eval: unknown dtype / compute form");
    MATPL_REQUIRE(model->ntypes >= 1 && model->ntypes <= 16, MATPL_ERR_UNSUPPORTED,
                  "ntypes must be in [1, 16]");
    MATPL_REQUIRE(model->npresent >= 1 && model->npresent <= kMaxPresent, MATPL_ERR_INVALID,
                  "npresent must be in [1, 8]");
    MATPL_REQUIRE(model->m >= 1 && nslots >= 1, MATPL_ERR_INVALID, "bad m / nslots");
    MATPL_REQUIRE(batch >= 0 && natoms >= 0 && nghost >= 0, MATPL_ERR_INVALID, "negative size");
    MATPL_REQUIRE(nslots <= 4096, MATPL_ERR_UNSUPPORTED, "nslots must be <= 4096");
    int mask = 0;
    for (int q = 0; q < model->npresent; ++q) {
        const int t = model->present[q];
        MATPL_REQUIRE(t >= 0 && t < model->ntypes, MATPL_ERR_INVALID, "present[] out of range");
        MATPL_REQUIRE((long long)(t + 1) * model->m <= nslots, MATPL_ERR_INVALID,
                      "list has fewer slots than present type blocks need");
        mask |= 1 << t;
    }
    const size_t es = dtype == MATPL_F64 ? 8 : 4;
    const DpLayout lay = dp_layout(es, batch, natoms, model->ntypes);
    MATPL_REQUIRE(workspace != nullptr && workspace_bytes >= lay.total, MATPL_ERR_WORKSPACE,
                  "dp workspace too small");
    if (batch == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(workspace, "matpl_dp_eval");
    EvalParams P;
    P.batch = batch; P.natoms = natoms; P.nslots = nslots; P.nghost = nghost;
    P.ntypes = model->ntypes; P.m = model->m; P.npresent = model->npresent;
    P.present_mask = mask;
    P.rmin = model->rmin; P.rmax = model->rmax;
    P.inv_mT = 1.0 / ((double)model->m * model->npresent);
    P.ctab = model->ctable;
    P.crows = model->ctab_rows;
    P.cnc = model->ctab_order + 1;
    P.cdx = model->ctab_dx;
    P.cdx10 = 10.0 * model->ctab_dx;
    P.csmin = model->ctab_smin;
    P.csmax = model->ctab_smax;
    P.err = model->err_dev;
    P.num_neigh = num_neigh;
    if (model->ctable) {
        MATPL_REQUIRE((model->ctab_order == 3 || model->ctab_order == 5) &&
                          model->ctab_rows >= 1 && model->ctab_dx > 0,
                      MATPL_ERR_INVALID, "compressed model: order 3 or 5, rows >= 1, dx > 0");
    }
    MATPL_REQUIRE(Etot && virial && (nghost == 0 || force) &&
                      (natoms == 0 || (model->params && model->davg && model->dstd && list_neigh &&
                                       image_dr && type_map && Ei && force)),
                  MATPL_ERR_INVALID, "matpl_dp_eval: null pointer argument");
    cudaStream_t s = as_stream(stream);
    if (natoms == 0) {
        cudaMemsetAsync(Etot, 0, 8 * (size_t)batch, s);
        cudaMemsetAsync(virial, 0, 72 * (size_t)batch, s);
        if (nghost) cudaMemsetAsync(force, 0, es * 3 * (size_t)batch * nghost, s);
        return check_launch("matpl_dp_eval");
    }
    if (dtype >= MATPL_MIXED) {
        MATPL_REQUIRE(model->ntypes <= 15, MATPL_ERR_UNSUPPORTED,
                      "mixed-precision forms support up to 15 types");
        MATPL_REQUIRE(model->ctable || mixed_smem(model->ntypes, nslots) <= 220 * 1024,
                      MATPL_ERR_UNSUPPORTED,
                      "mixed-precision form: too many slots for the shared-memory pair list");
    }
    if (dtype == MATPL_F64)
        return launch_eval<double>(dtype, model, P, list_neigh, (const double *)image_dr,
                                   type_map, (double *)Ei, Etot, (double *)force, virial,
                                   (char *)workspace, lay, s);
    return launch_eval<float>(dtype, model, P, list_neigh, (const float *)image_dr, type_map,
                              (float *)Ei, Etot, (float *)force, virial, (char *)workspace, lay,
                              s);
}

extern "C" int matpl_dp_eval(int dtype, const matpl_dp_model *model, int batch, int natoms,
                             int nslots, int nghost, const int32_t *list_neigh,
                             const void *image_dr, const int32_t *type_map, void *Ei,
                             double *Etot, void *force, double *virial, void *workspace,
                             size_t workspace_bytes, void *stream) {
    return dp_eval(dtype, model, batch, natoms, nslots, nghost, list_neigh, nullptr, image_dr,
                   type_map, Ei, Etot, force, virial, workspace, workspace_bytes, stream);
}

extern "C" int matpl_dp_eval_occupied(int dtype, const matpl_dp_model *model, int batch,
                                      int natoms, int nslots, int nghost,
                                      const int32_t *list_neigh, const int32_t *num_neigh,
                                      const void *image_dr, const int32_t *type_map, void *Ei,
                                      double *Etot, void *force, double *virial,
                                      void *workspace, size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE(num_neigh != nullptr || (long long)batch * natoms == 0, MATPL_ERR_INVALID,
                  "matpl_dp_eval_occupied: num_neigh is required (it gives the block lengths)");
    return dp_eval(dtype, model, batch, natoms, nslots, nghost, list_neigh, num_neigh, image_dr,
                   type_map, Ei, Etot, force, virial, workspace, workspace_bytes, stream);
}
