// Force-loss training of DP se_e2_a: the embedding-net part of the second-order gradient,
// written by hand (the reference gets it from torch autograd with create_graph=True,
// src/PWMLFF/dp_mods/dp_trainer.py:172-275 through src/model/dp_dp.py:417-530).
//
// For a loss L(E, F, V) the trainer needs dL/dtheta = gE . dE/dtheta + gF . dF/dtheta (+ gV .
// dV/dtheta) with gE = dL/dE, gF = dL/dF, gV = dL/dV.  Forces and virial are built from the
// per-slot vectors f_s = sum_c dE/dRi_s[c] Ri_d_s[c][:] (F_i -= f_s, F_j += f_s, V += f_s r_s^T),
// so
//     gF . F + gV . V = sum_s f_s . u_s,   u_s = gF_j - gF_i + gV r_s,
//                     = sum_s sum_c dE/dRi_s[c] Rdot_s[c],   Rdot_s = Ri_d_s u_s,
// the derivative of E along the input tangent Rdot (Ri_d does not depend on the parameters).
// Its parameter gradient is a forward-over-reverse product:
//   dp_dual_fwd   tangent (forward-mode) pass through every embedding net: per occupied slot
//                 G = emb(s), Gdot = emb'(s) sdot, and per atom
//                 A = k sum_s R_s^T G_s,  Adot = k sum_s (Rdot_s^T G_s + R_s^T Gdot_s)
//                 (k = 1 / (m T); empty slots contribute to A only, their tangent is zero);
//   (host)        the per-atom part - descriptor D = A^T A<, fitting nets, E and its tangent
//                 Edot = dE/dA . Adot - and its reverse give Abar = dPhi/dA, Adotbar = dPhi/dAdot
//                 for Phi = sum gE E + sum Edot;
//   dp_dual_bwd   reverse through the tangent pass, recomputing the embedding activations slot
//                 by slot instead of storing them, and reducing the embedding-weight gradients
//                 (outer products of layer inputs and pre-activation adjoints, both for the
//                 primal and the tangent stream) per CTA in shared memory.
#include "common.cuh"
#include "dp_layout.cuh"
#include "dp_env.cuh"

namespace matpl {
namespace {

using namespace dp;
constexpr int kStg = E + 1;   // staging row stride (odd: conflict-free column access)

// Shared-memory copy of one embedding net: the vectors, then the two E x E matrices with rows
// padded to kRp (16-byte aligned rows: a row is 7 vector loads instead of 25 scalar ones) and,
// for the backward kernel, their transposes (columns as rows).
constexpr int kRp = 28;
struct NetS {
    static constexpr int W0 = 0, B0 = E, B1 = 2 * E, DT1 = 3 * E, B2 = 4 * E, DT2 = 5 * E;
    static constexpr int M1 = 152, M2 = M1 + E * kRp;          // W1, W2 [in][out]
    static constexpr int M1T = M2 + E * kRp, M2T = M1T + E * kRp;   // W1^T, W2^T [out][in]
    static constexpr int FWD = M1T;                            // per-net size without transposes
    static constexpr int BWD = M2T + E * kRp;
};
static_assert(NetS::M1 % 4 == 0 && NetS::M1 >= 6 * E, "aligned matrix block after the vectors");

// params (EmbOff layout, nnet nets) -> shared NetS layout (stride = NetS::FWD or NetS::BWD)
template <typename T>
__device__ __forceinline__ void load_nets(T *dst, const T *__restrict__ params, int nnet,
                                          int stride) {
    const bool tr = stride == NetS::BWD;
    for (int q = threadIdx.x; q < nnet * stride; q += blockDim.x) {
        const int n = q / stride, e = q - n * stride;
        const T *src = params + (long long)n * EmbOff::SIZE;
        T v = T(0);
        if (e < 6 * E) {
            const int which = e / E, o = e - which * E;
            const int off[6] = {EmbOff::W0, EmbOff::B0, EmbOff::B1, EmbOff::DT1, EmbOff::B2,
                                EmbOff::DT2};
            v = src[off[which] + o];
        } else if (e >= NetS::M1 && (e < NetS::M1T || tr)) {
            const int blk = (e - NetS::M1) / (E * kRp), r = (e - NetS::M1) % (E * kRp);
            const int row = r / kRp, col = r - row * kRp;
            if (col < E) {
                const int W = (blk & 1) ? EmbOff::W2 : EmbOff::W1;
                v = blk < 2 ? src[W + row * E + col] : src[W + col * E + row];
            }
        }
        dst[q] = v;
    }
}

// 28 consecutive values of a 16-byte aligned shared row
__device__ __forceinline__ void ld_row(const float *p, float v[kRp]) {
#pragma unroll
    for (int q = 0; q < kRp / 4; ++q) {
        const float4 f = reinterpret_cast<const float4 *>(p)[q];
        v[4 * q] = f.x; v[4 * q + 1] = f.y; v[4 * q + 2] = f.z; v[4 * q + 3] = f.w;
    }
}
__device__ __forceinline__ void ld_row(const double *p, double v[kRp]) {
#pragma unroll
    for (int q = 0; q < kRp / 2; ++q) {
        const double2 f = reinterpret_cast<const double2 *>(p)[q];
        v[2 * q] = f.x; v[2 * q + 1] = f.y;
    }
}

struct TrainParams {
    int batch, natoms, nslots, ntypes, m, present_mask, has_gv;
    double rmin, rmax, inv_mT;
};

// Occupied slots of one centre atom (ascending), image types absent from the model skipped.
__device__ __forceinline__ int occupied_slots(const int32_t *__restrict__ ln, int S, int m,
                                              int present_mask, int *list, int lane) {
    int cnt = 0;
    for (int s0 = 0; s0 < S; s0 += 32) {
        const int s = s0 + lane;
        const bool occ = s < S && ln[s] > 0 && ((present_mask >> (s / m)) & 1);
        const unsigned b = __ballot_sync(0xffffffffu, occ);
        if (occ) list[cnt + __popc(b & ((1u << lane) - 1u))] = s;
        cnt += __popc(b);
    }
    __syncwarp();
    return cnt;
}

// One slot's normalised row, its tangent and the embedding input (s, sdot).
template <typename T>
__device__ __forceinline__ void slot_rows(const T *__restrict__ idr, const T *__restrict__ gF,
                                          const T *__restrict__ gV, const int32_t *__restrict__ ln,
                                          long long t, long long cfg0, int slot, int S,
                                          const T *avg, const T *sd, const TrainParams &P,
                                          T rh[4], T rd[4]) {
    const T *row = idr + (t * S + slot) * 4;
    const T R = row[0], x = row[1], y = row[2], z = row[3];
    env_row(R, x, y, z, (T)P.rmin, (T)P.rmax, avg, sd, rh);
    const long long j = cfg0 + ln[t * S + slot] - 1;
    T u[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) u[a] = gF[3 * j + a] - gF[3 * t + a];
    if (P.has_gv) {
        const T *g = gV + 9 * (t / P.natoms);
#pragma unroll
        for (int a = 0; a < 3; ++a) u[a] += g[3 * a] * x + g[3 * a + 1] * y + g[3 * a + 2] * z;
    }
    rid_dir(R, x, y, z, (T)P.rmin, (T)P.rmax, sd, u, rd);
}

// Embedding layer 0 (1 -> E) and its tangent.
template <typename T>
__device__ __forceinline__ void layer0(const T *w, T s, T sdot, T x[E], T xd[E]) {
#pragma unroll
    for (int o = 0; o < E; ++o) {
        const T t = dev_tanh(s * w[NetS::W0 + o] + w[NetS::B0 + o]);
        x[o] = t;
        xd[o] = (T(1) - t * t) * sdot * w[NetS::W0 + o];
    }
}

// Pre-activations of an E -> E layer for a lane's input row x (and its tangent xd) kept in
// shared memory: h = x W + b, hd = xd W (OW: the padded matrix W[in][out] in the NetS copy).
// The input index loop stays rolled (small code, few registers); the output index is unrolled
// into registers.
template <typename T>
__device__ __forceinline__ void pre_act(const T *w, int OW, int OB, const T *x, const T *xd,
                                        T h[E], T hd[E]) {
#pragma unroll
    for (int o = 0; o < E; ++o) { h[o] = w[OB + o]; hd[o] = T(0); }
#pragma unroll 1
    for (int i = 0; i < E; ++i) {
        const T xi = x[i], xdi = xd[i];
        T wr[kRp];
        ld_row(w + OW + i * kRp, wr);
#pragma unroll
        for (int o = 0; o < E; ++o) {
            h[o] += xi * wr[o];
            hd[o] += xdi * wr[o];
        }
    }
}

// acc[i] += sum_o W[i][o] z[o] and accd[i] += sum_o W[i][o] zd[o] (z, zd in shared memory;
// WT: the padded transpose W^T[out][in] in the NetS copy).
template <typename T>
__device__ __forceinline__ void back_act(const T *WT, const T *z, const T *zd, T acc[E],
                                         T accd[E]) {
#pragma unroll 1
    for (int o = 0; o < E; ++o) {
        const T zo = z[o], zdo = zd[o];
        T wc[kRp];
        ld_row(WT + o * kRp, wc);
#pragma unroll
        for (int i = 0; i < E; ++i) {
            acc[i] += wc[i] * zo;
            accd[i] += wc[i] * zdo;
        }
    }
}

// Residual layer applied in place to a lane's shared-memory rows x, xd:
// x <- tanh(x W + b) dt + x with its tangent.
template <typename T>
__device__ __forceinline__ void layer_res(const T *w, int OW, int OB, int OD, T *x, T *xd) {
    T h[E], hd[E];
    pre_act(w, OW, OB, x, xd, h, hd);
#pragma unroll
    for (int o = 0; o < E; ++o) {
        const T t = dev_tanh(h[o]);
        const T dt = w[OD + o];
        x[o] = t * dt + x[o];
        xd[o] = (T(1) - t * t) * hd[o] * dt + xd[o];
    }
}

// ------------------------------------------------------------------------------ dual forward
// Per-lane shared row: G (the running activation), Gdot, then rh and rd.
constexpr int kFwdRow = 2 * kStg + 8;

template <typename T>
__global__ void __launch_bounds__(256)
dp_dual_fwd(const int32_t *__restrict__ list_neigh, const T *__restrict__ idr,
            const int32_t *__restrict__ type_map, const T *__restrict__ params,
            const T *__restrict__ davg, const T *__restrict__ dstd, const T *__restrict__ gF,
            const T *__restrict__ gV, T *__restrict__ Aout, T *__restrict__ Adout,
            TrainParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nnet = P.ntypes * P.ntypes, S = P.nslots;
    const int warps = blockDim.x >> 5;
    T *wsm = reinterpret_cast<T *>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *stg = wsm + nnet * NetS::FWD + warp * 32 * kFwdRow;
    int *list = reinterpret_cast<int *>(wsm + nnet * NetS::FWD + warps * 32 * kFwdRow) +
                warp * S;
    load_nets(wsm, params, nnet, NetS::FWD);
    __syncthreads();
    const long long total = (long long)P.batch * P.natoms;
    T *my = stg + lane * kFwdRow;
    for (long long t = (long long)blockIdx.x * warps + warp; t < total;
         t += (long long)gridDim.x * warps) {
        const int ti = type_map[t % P.natoms];
        T *Arow = Aout + t * NA, *Adrow = Adout + t * NA;
        if (ti < 0 || ti >= P.ntypes || !((P.present_mask >> ti) & 1)) {
            for (int e = lane; e < NA; e += 32) Arow[e] = Adrow[e] = T(0);
            continue;
        }
        const long long cfg0 = (t / P.natoms) * P.natoms;
        const int cnt = occupied_slots(list_neigh + t * S, S, P.m, P.present_mask, list, lane);
        const T *avg = davg + 4 * ti, *sd = dstd + 4 * ti;
        T a[4], ad[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = ad[q] = T(0);
        for (int c0 = 0; c0 < cnt; c0 += 32) {
            const int k = c0 + lane;
            T rh[4] = {T(0), T(0), T(0), T(0)}, rd[4] = {T(0), T(0), T(0), T(0)};
            int tj = 0;
            if (k < cnt) {
                const int slot = list[k];
                tj = slot / P.m;
                slot_rows(idr, gF, gV, list_neigh, t, cfg0, slot, S, avg, sd, P, rh, rd);
            }
            const T *w = wsm + (ti * P.ntypes + tj) * NetS::FWD;
            __syncwarp();
            {
                T x[E], xd[E];
                layer0(w, rh[0], rd[0], x, xd);
#pragma unroll
                for (int p = 0; p < E; ++p) { my[p] = x[p]; my[kStg + p] = xd[p]; }
            }
            layer_res(w, NetS::M1, NetS::B1, NetS::DT1, my, my + kStg);
            layer_res(w, NetS::M2, NetS::B2, NetS::DT2, my, my + kStg);
            const bool valid = k < cnt;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                my[2 * kStg + c] = valid ? rh[c] : T(0);
                my[2 * kStg + 4 + c] = valid ? rd[c] : T(0);
            }
            __syncwarp();
            const int nv = min(32, cnt - c0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = lane + 32 * q;
                if (e < NA) {
                    const int c = e / E, p = e - c * E;
                    T s0 = a[q], s1 = ad[q];
                    for (int l = 0; l < nv; ++l) {
                        const T *r = stg + l * kFwdRow;
                        const T g = r[p];
                        s0 += r[2 * kStg + c] * g;
                        s1 += r[2 * kStg + 4 + c] * g + r[2 * kStg + c] * r[kStg + p];
                    }
                    a[q] = s0;
                    ad[q] = s1;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = lane + 32 * q;
            if (e < NA) {
                Arow[e] = a[q] * (T)P.inv_mT;
                Adrow[e] = ad[q] * (T)P.inv_mT;
            }
        }
        __syncwarp();
    }
}

// ----------------------------------------------------------------------------- dual backward
// Per-warp staging of one layer for the weight-gradient reduction: layer input x and its
// tangent xd, pre-activation adjoints zb / zdb, and the dt-gradient term q.
struct Stage {
    static constexpr int X = 0, XD = kStg, ZB = 2 * kStg, ZDB = 3 * kStg, Q = 4 * kStg;
    static constexpr int ROW = 5 * kStg + 3;          // + (s, sdot, pad)
};

// Adds, for every net present among the chunk's lanes, sum over its lanes of the layer's
// gradient terms into the CTA accumulator gacc (shared).  lay = 1 or 2 (W/b/dt of that layer),
// lay = 0: W0 / b0 from (s, sdot).
template <typename T>
__device__ __forceinline__ void reduce_layer(const T *stg, int nv, int ti, int ntypes,
                                             unsigned tmask[], int lay, T *gacc, int lane) {
    for (int tj = 0; tj < ntypes; ++tj) {
        const unsigned mk = tmask[tj];
        if (!mk) continue;
        const int lo = __ffs(mk) - 1, hi = 32 - __clz(mk);
        T *g = gacc + (ti * ntypes + tj) * EmbOff::SIZE;
        if (lay == 0) {
            for (int e = lane; e < 2 * E; e += 32) {
                const int o = e < E ? e : e - E;
                T acc = T(0);
                for (int l = lo; l < hi; ++l) {
                    const T *r = stg + l * Stage::ROW;
                    acc += e < E ? r[5 * kStg] * r[Stage::ZB + o] + r[5 * kStg + 1] * r[Stage::ZDB + o]
                                 : r[Stage::ZB + o];
                }
                atomicAdd(g + (e < E ? EmbOff::W0 : EmbOff::B0) + o, acc);
            }
            continue;
        }
        const int OW = lay == 1 ? EmbOff::W1 : EmbOff::W2;
        const int OB = lay == 1 ? EmbOff::B1 : EmbOff::B2;
        const int OD = lay == 1 ? EmbOff::DT1 : EmbOff::DT2;
        // weight gradient sum_l x_i zb_o + xd_i zdb_o: lane < 25 owns a 5 x 5 block (i, o), so
        // a row costs 20 shared loads for 50 FMAs
        static_assert(E == 25, "5 x 5 register blocks of the 25 x 25 weight gradient");
        if (lane < 25) {
            const int i0 = 5 * (lane / 5), o0 = 5 * (lane % 5);
            T acc[5][5];
#pragma unroll
            for (int a = 0; a < 5; ++a)
#pragma unroll
                for (int b = 0; b < 5; ++b) acc[a][b] = T(0);
            for (int l = lo; l < hi; ++l) {
                const T *r = stg + l * Stage::ROW;
                T xi[5], xdi[5], zo[5], zdo[5];
#pragma unroll
                for (int a = 0; a < 5; ++a) {
                    xi[a] = r[Stage::X + i0 + a];
                    xdi[a] = r[Stage::XD + i0 + a];
                    zo[a] = r[Stage::ZB + o0 + a];
                    zdo[a] = r[Stage::ZDB + o0 + a];
                }
#pragma unroll
                for (int a = 0; a < 5; ++a)
#pragma unroll
                    for (int b = 0; b < 5; ++b) acc[a][b] += xi[a] * zo[b] + xdi[a] * zdo[b];
            }
#pragma unroll
            for (int a = 0; a < 5; ++a)
#pragma unroll
                for (int b = 0; b < 5; ++b) atomicAdd(g + OW + (i0 + a) * E + o0 + b, acc[a][b]);
        }
        for (int o = lane; o < 2 * E; o += 32) {
            T acc = T(0);
            const int col = o < E ? Stage::ZB + o : Stage::Q + (o - E);
            for (int l = lo; l < hi; ++l) acc += stg[l * Stage::ROW + col];
            atomicAdd(g + (o < E ? OB + o : OD + (o - E)), acc);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
dp_dual_bwd(const int32_t *__restrict__ list_neigh, const T *__restrict__ idr,
            const int32_t *__restrict__ type_map, const T *__restrict__ params,
            const T *__restrict__ davg, const T *__restrict__ dstd, const T *__restrict__ gF,
            const T *__restrict__ gV, const T *__restrict__ Abar, const T *__restrict__ Adbar,
            T *__restrict__ grad, TrainParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nnet = P.ntypes * P.ntypes, S = P.nslots;
    const int warps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *wsm = reinterpret_cast<T *>(smem_raw);                   // weights (NetS layout)
    T *gacc = wsm + nnet * NetS::BWD;                           // gradient accumulator
    T *stg_all = gacc + nnet * EmbOff::SIZE;                    // [warps][32][Stage::ROW]
    T *ab_all = stg_all + warps * 32 * Stage::ROW;              // [warps][2][NA]
    int *list_all = reinterpret_cast<int *>(ab_all + warps * 2 * NA);
    T *stg = stg_all + warp * 32 * Stage::ROW;
    T *ab = ab_all + warp * 2 * NA;
    int *list = list_all + warp * S;
    T *my = stg + lane * Stage::ROW;
    load_nets(wsm, params, nnet, NetS::BWD);
    for (int q = threadIdx.x; q < nnet * EmbOff::SIZE; q += blockDim.x) gacc[q] = T(0);
    __syncthreads();
    const T k = (T)P.inv_mT;
    const long long total = (long long)P.batch * P.natoms;
    for (long long t = (long long)blockIdx.x * warps + warp; t < total;
         t += (long long)gridDim.x * warps) {
        const int ti = type_map[t % P.natoms];
        if (ti < 0 || ti >= P.ntypes || !((P.present_mask >> ti) & 1)) continue;
        const long long cfg0 = (t / P.natoms) * P.natoms;
        const int cnt = occupied_slots(list_neigh + t * S, S, P.m, P.present_mask, list, lane);
        for (int e = lane; e < NA; e += 32) {
            ab[e] = Abar[t * NA + e] * k;
            ab[NA + e] = Adbar[t * NA + e] * k;
        }
        __syncwarp();
        const T *avg = davg + 4 * ti, *sd = dstd + 4 * ti;
        for (int c0 = 0; c0 < cnt; c0 += 32) {
            const int kk = c0 + lane;
            const bool valid = kk < cnt;
            T rh[4] = {T(0), T(0), T(0), T(0)}, rd[4] = {T(0), T(0), T(0), T(0)};
            int tj = 0;
            if (valid) {
                const int slot = list[kk];
                tj = slot / P.m;
                slot_rows(idr, gF, gV, list_neigh, t, cfg0, slot, S, avg, sd, P, rh, rd);
            }
            unsigned tmask[16];
#pragma unroll
            for (int q = 0; q < 16; ++q)
                tmask[q] = q < P.ntypes ? __ballot_sync(0xffffffffu, valid && tj == q) : 0u;
            const int nv = min(32, cnt - c0);
            const T *w = wsm + (ti * P.ntypes + tj) * NetS::BWD;
            // seeds: Gbar = k (R Abar + Rdot Adbar), Gdotbar = k R Adbar (k folded into ab)
            T gb[E], gdb[E];
#pragma unroll
            for (int p = 0; p < E; ++p) {
                T s0 = T(0), s1 = T(0);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    s0 += rh[c] * ab[c * E + p] + rd[c] * ab[NA + c * E + p];
                    s1 += rh[c] * ab[NA + c * E + p];
                }
                gb[p] = valid ? s0 : T(0);
                gdb[p] = valid ? s1 : T(0);
            }
            __syncwarp();
            // ---- layer 2: recompute its input x1 (staged in X / XD), reverse through it
            {
                T x[E], xd[E];
                layer0(w, rh[0], rd[0], x, xd);
#pragma unroll
                for (int p = 0; p < E; ++p) { my[Stage::X + p] = x[p]; my[Stage::XD + p] = xd[p]; }
            }
            layer_res(w, NetS::M1, NetS::B1, NetS::DT1, my + Stage::X, my + Stage::XD);
            {
                T h[E], hd[E];
                pre_act(w, NetS::M2, NetS::B2, my + Stage::X, my + Stage::XD, h, hd);
#pragma unroll
                for (int o = 0; o < E; ++o) {
                    const T t2 = dev_tanh(h[o]);
                    const T dt = w[NetS::DT2 + o], g = T(1) - t2 * t2;
                    const T tb = gb[o] * dt, tdb = gdb[o] * dt;
                    my[Stage::Q + o] = gb[o] * t2 + gdb[o] * g * hd[o];
                    my[Stage::ZB + o] = g * (tb - T(2) * t2 * hd[o] * tdb);
                    my[Stage::ZDB + o] = g * tdb;
                }
            }
            // x1bar = Gbar + W2 zb2, x1dotbar = Gdotbar + W2 zdb2
            back_act(w + NetS::M2T, my + Stage::ZB, my + Stage::ZDB, gb, gdb);
            __syncwarp();
            reduce_layer(stg, nv, ti, P.ntypes, tmask, 2, gacc, lane);
            __syncwarp();
            // ---- layer 1: recompute its input x0 (staged), reverse through it
            {
                T x[E], xd[E];
                layer0(w, rh[0], rd[0], x, xd);
#pragma unroll
                for (int p = 0; p < E; ++p) { my[Stage::X + p] = x[p]; my[Stage::XD + p] = xd[p]; }
            }
            {
                T h[E], hd[E];
                pre_act(w, NetS::M1, NetS::B1, my + Stage::X, my + Stage::XD, h, hd);
#pragma unroll
                for (int o = 0; o < E; ++o) {
                    const T t1 = dev_tanh(h[o]);
                    const T dt = w[NetS::DT1 + o], g = T(1) - t1 * t1;
                    const T tb = gb[o] * dt, tdb = gdb[o] * dt;
                    my[Stage::Q + o] = gb[o] * t1 + gdb[o] * g * hd[o];
                    my[Stage::ZB + o] = g * (tb - T(2) * t1 * hd[o] * tdb);
                    my[Stage::ZDB + o] = g * tdb;
                }
            }
            back_act(w + NetS::M1T, my + Stage::ZB, my + Stage::ZDB, gb, gdb);
            __syncwarp();
            reduce_layer(stg, nv, ti, P.ntypes, tmask, 1, gacc, lane);
            __syncwarp();
            // ---- layer 0: x0 = tanh(s W0 + b0), x0dot = (1 - x0^2) sdot W0 (x0 still staged)
#pragma unroll
            for (int o = 0; o < E; ++o) {
                const T x0 = my[Stage::X + o];
                const T g = T(1) - x0 * x0;
                const T zd0 = rd[0] * w[NetS::W0 + o];
                my[Stage::ZB + o] = g * (gb[o] - T(2) * x0 * zd0 * gdb[o]);
                my[Stage::ZDB + o] = g * gdb[o];
            }
            my[5 * kStg] = rh[0];
            my[5 * kStg + 1] = rd[0];
            __syncwarp();
            reduce_layer(stg, nv, ti, P.ntypes, tmask, 0, gacc, lane);
            __syncwarp();
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nnet * EmbOff::SIZE; q += blockDim.x)
        if (gacc[q] != T(0)) atomicAdd(grad + q, gacc[q]);
}

// ---------------------------------------------------------------- descriptor and its tangent
// Per atom D = A^T A< and Ddot = Adot^T A< + A^T Adot< (A, Adot [4][E], A< its first m2
// columns; D [E][m2]): the products of dp_dp.py:304-330 (xyz_scater_a^T xyz_scater_b) for the
// training step's primal and tangent streams.  One thread per (output row, p, q); output row r
// holds atom rows[r] (rows: a permutation, e.g. atoms grouped by element; NULL = identity).
template <typename T>
__global__ void __launch_bounds__(256)
desc_dual_kernel(long long natoms, int m2, const long long *__restrict__ rows,
                 const T *__restrict__ A, const T *__restrict__ Ad, T *__restrict__ D,
                 T *__restrict__ Dd) {
    const long long per = (long long)E * m2, total = natoms * per;
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < total;
         o += (long long)gridDim.x * blockDim.x) {
        const long long r = o / per;
        const int pq = (int)(o - r * per), p = pq / m2, q = pq - p * m2;
        const long long a = rows ? rows[r] : r;
        const T *ar = A + a * NA, *dr = Ad + a * NA;
        T d = T(0), dd = T(0);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const T ap = __ldg(ar + c * E + p), aq = __ldg(ar + c * E + q);
            d += ap * aq;
            dd += __ldg(dr + c * E + p) * aq + ap * __ldg(dr + c * E + q);
        }
        D[o] = d;
        Dd[o] = dd;
    }
}

// The transpose map: for gD = dPhi/dD, gDd = dPhi/dDdot (either may be absent)
//   gA[c][x]  = sum_q gD[x][q] A[c][q] + [x < m2] sum_p gD[p][x] A[c][p]
//             + sum_q gDd[x][q] Ad[c][q] + [x < m2] sum_p gDd[p][x] Ad[c][p],
//   gAd[c][x] = sum_q gDd[x][q] A[c][q] + [x < m2] sum_p gDd[p][x] A[c][p].
// One thread per (row, x) writes the 4 + 4 entries of atom rows[r] (a permutation: no two rows
// write the same atom).
template <typename T>
__global__ void __launch_bounds__(256)
desc_dual_grad_kernel(long long natoms, int m2, const long long *__restrict__ rows,
                      const T *__restrict__ A, const T *__restrict__ Ad, const T *__restrict__ gD,
                      const T *__restrict__ gDd, T *__restrict__ gA, T *__restrict__ gAd) {
    const long long total = natoms * E;
    const long long per = (long long)E * m2;
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < total;
         o += (long long)gridDim.x * blockDim.x) {
        const long long r = o / E;
        const int x = (int)(o - r * E);
        const long long a = rows ? rows[r] : r;
        const T *ar = A + a * NA, *dr = Ad + a * NA;
        const T *g = gD ? gD + r * per : nullptr, *gd = gDd ? gDd + r * per : nullptr;
        T ga[4] = {T(0), T(0), T(0), T(0)}, gad[4] = {T(0), T(0), T(0), T(0)};
        for (int q = 0; q < m2; ++q) {
            const T u = g ? __ldg(g + x * m2 + q) : T(0);
            const T v = gd ? __ldg(gd + x * m2 + q) : T(0);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const T aq = __ldg(ar + c * E + q), dq = __ldg(dr + c * E + q);
                ga[c] += u * aq + v * dq;
                gad[c] += v * aq;
            }
        }
        if (x < m2) {
            for (int p = 0; p < E; ++p) {
                const T u = g ? __ldg(g + p * m2 + x) : T(0);
                const T v = gd ? __ldg(gd + p * m2 + x) : T(0);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const T ap = __ldg(ar + c * E + p), dp = __ldg(dr + c * E + p);
                    ga[c] += u * ap + v * dp;
                    gad[c] += v * ap;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            gA[a * NA + c * E + x] = ga[c];
            gAd[a * NA + c * E + x] = gad[c];
        }
    }
}

template <typename T>
int launch_desc(bool grad, long long natoms, int m2, const long long *rows, const void *A,
                const void *Ad, const void *gD, const void *gDd, void *o0, void *o1,
                cudaStream_t s) {
    const long long work = grad ? natoms * E : natoms * E * m2;
    long long grid = (work + 255) / 256;
    if (grid > (long long)device_sms() * 32) grid = (long long)device_sms() * 32;
    if (grid < 1) grid = 1;
    if (!grad) {
        ProfScope ps("dp_desc_dual", s);
        desc_dual_kernel<T><<<(int)grid, 256, 0, s>>>(natoms, m2, rows, (const T *)A,
                                                       (const T *)Ad, (T *)o0, (T *)o1);
        return check_launch("matpl_dp_desc_dual");
    }
    ProfScope ps("dp_desc_dual_grad", s);
    desc_dual_grad_kernel<T><<<(int)grid, 256, 0, s>>>(natoms, m2, rows, (const T *)A,
                                                        (const T *)Ad, (const T *)gD,
                                                        (const T *)gDd, (T *)o0, (T *)o1);
    return check_launch("matpl_dp_desc_dual_grad");
}

// ---- empty-slot term of A ------------------------------------------------------------------
// Every empty slot of type block t_j holds the row R_pad(t_i) = (0 - davg[t_i]) / dstd[t_i]
// (dp_dp.py's normalised zero row), so the slots the dual kernels skip add
//     A_pad = k sum_{t_j present} n_empty(t_j) R_pad(t_i)^T G_{t_i t_j}(s_pad(t_i)),
// one row per (t_i, t_j) pair, k = 1 / (m T).  prow[pair] = k R_pad (x) G is computed once per
// pair (dp_pad_rows), then added per atom with the atom's empty counts (dp_pad_add).  The
// reverse reduces dPhi/dprow over the atoms (dp_pad_reduce, FP64 sums) and runs each pair's
// three-layer net backward (dp_pad_net_bwd).
constexpr int kMaxPresent = 8;

struct PadParams {
    int rows, natoms, nslots, ntypes, m, npresent;
    int present[kMaxPresent];
    double inv_mT;
};

// The pair's net at s_pad with its activations: x0 = tanh(s W0 + b0), h_l = tanh(x W_l + b_l),
// x_l = h_l dt_l + x_{l-1}.  One warp, lane e < E owns column e; sx holds the layer input.
template <typename T>
__device__ __forceinline__ void pad_net_fwd(const T *__restrict__ w, T s, T *sx, int lane,
                                            T &x0, T &h1, T &x1, T &h2, T &x2) {
    x0 = h1 = x1 = h2 = x2 = T(0);
    if (lane < E) x0 = dev_tanh(s * w[EmbOff::W0 + lane] + w[EmbOff::B0 + lane]);
    if (lane < E) sx[lane] = x0;
    __syncwarp();
    if (lane < E) {
        T z = w[EmbOff::B1 + lane];
        for (int i = 0; i < E; ++i) z += sx[i] * w[EmbOff::W1 + i * E + lane];
        h1 = dev_tanh(z);
        x1 = h1 * w[EmbOff::DT1 + lane] + x0;
    }
    __syncwarp();
    if (lane < E) sx[lane] = x1;
    __syncwarp();
    if (lane < E) {
        T z = w[EmbOff::B2 + lane];
        for (int i = 0; i < E; ++i) z += sx[i] * w[EmbOff::W2 + i * E + lane];
        h2 = dev_tanh(z);
        x2 = h2 * w[EmbOff::DT2 + lane] + x1;
    }
    __syncwarp();
}

template <typename T>
__device__ __forceinline__ T pad_row_value(const T *davg, const T *dstd, int ti, int c) {
    return (T(0) - davg[ti * 4 + c]) / dstd[ti * 4 + c];
}

// One warp per present (t_i, t_j) pair: prow[qi * np + qj][c * E + e] = k R_pad[c] G[e].
template <typename T>
__global__ void __launch_bounds__(32) dp_pad_rows(const T *__restrict__ params,
                                                  const T *__restrict__ davg,
                                                  const T *__restrict__ dstd, PadParams P,
                                                  T *__restrict__ prow) {
    __shared__ T sx[32];
    const int pair = blockIdx.x, lane = threadIdx.x;
    const int ti = P.present[pair / P.npresent], tj = P.present[pair % P.npresent];
    const T *w = params + (long long)(ti * P.ntypes + tj) * EmbOff::SIZE;
    T x0, h1, x1, h2, x2;
    pad_net_fwd(w, pad_row_value(davg, dstd, ti, 0), sx, lane, x0, h1, x1, h2, x2);
    if (lane < E) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
            prow[(long long)pair * NA + c * E + lane] =
                T(P.inv_mT) * pad_row_value(davg, dstd, ti, c) * x2;
    }
}

// One warp per atom row (b, i): empty counts of the present types (written to n_empty for the
// reverse) and A = A_occ + sum_j n_empty(t_j) prow[(t_i, t_j)] (A_occ copied through for atoms
// whose type is absent from present[]).  A may alias A_occ.
template <typename T>
__global__ void __launch_bounds__(256) dp_pad_add(const int32_t *__restrict__ ln,
                                                  const int32_t *__restrict__ tm,
                                                  const T *__restrict__ prow, PadParams P,
                                                  const T *A_occ, T *A,
                                                  int32_t *__restrict__ n_empty) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         row < P.rows; row += warps) {
        const int32_t *l = ln + row * P.nslots;
        const int ti = tm[row % P.natoms];
        // per-lane counts of occupied slots by present type (independent loads, then one
        // warp reduction per type)
        int ne[kMaxPresent];
#pragma unroll
        for (int q = 0; q < kMaxPresent; ++q) ne[q] = 0;
#pragma unroll 4
        for (int s = lane; s < P.nslots; s += 32) {
            if (l[s] > 0) {
                const int t = s / P.m;
#pragma unroll
                for (int q = 0; q < kMaxPresent; ++q) ne[q] += q < P.npresent && P.present[q] == t;
            }
        }
        int qi = -1;
#pragma unroll
        for (int q = 0; q < kMaxPresent; ++q) {
            if (q < P.npresent) {
                ne[q] = P.m - (int)__reduce_add_sync(0xffffffffu, (unsigned)ne[q]);
                if (P.present[q] == ti) qi = q;
                if (lane == 0) n_empty[row * P.npresent + q] = ne[q];
            }
        }
#pragma unroll
        for (int k = 0; k < (NA + 31) / 32; ++k) {
            const int idx = lane + 32 * k;
            if (idx >= NA) break;
            T acc = A_occ[row * NA + idx];
            if (qi >= 0) {
#pragma unroll
                for (int q = 0; q < kMaxPresent; ++q)
                    if (q < P.npresent)
                        acc += T(ne[q]) * prow[(long long)(qi * P.npresent + q) * NA + idx];
            }
            A[row * NA + idx] = acc;
        }
    }
}

// gsum[rep][qi * np + qj][idx] += sum over rows of type t_i of n_empty(t_j) Abar[row][idx].
// A CTA of G groups of 128 threads: thread idx < NA of a group owns one column and keeps the
// group's sums in shared memory (np^2 x NA values of the compute type: a group sums a few
// dozen rows); the groups are then added together in FP64 and the CTA adds its sums into
// replica rep = blockIdx.x % kPadReps (only for the centre types it met), so that the atomics
// of different CTAs spread over kPadReps copies.
constexpr int kPadReps = 16;

template <typename T>
__global__ void __launch_bounds__(512, 2) dp_pad_reduce(const int32_t *__restrict__ tm,
                                                        const int32_t *__restrict__ n_empty,
                                                        const T *__restrict__ A_bar,
                                                        PadParams P, int chunk,
                                                        double *__restrict__ gsum) {
    extern __shared__ __align__(16) unsigned char pad_smem[];
    T *sacc = reinterpret_cast<T *>(pad_smem);
    __shared__ int seen[kMaxPresent];
    __shared__ int qof[16];
    const int np = P.npresent, G = blockDim.x >> 7, grp = threadIdx.x >> 7;
    const int idx = threadIdx.x & 127;
    const int per = np * np * NA;
    for (int q = threadIdx.x; q < G * per; q += blockDim.x) sacc[q] = T(0);
    if (threadIdx.x < kMaxPresent) seen[threadIdx.x] = 0;
    if (threadIdx.x < 16) {
        int v = -1;
        for (int q = 0; q < np; ++q)
            if (P.present[q] == (int)threadIdx.x) v = q;
        qof[threadIdx.x] = v;
    }
    __syncthreads();
    const int r0 = blockIdx.x * chunk;
    const int r1 = r0 + chunk < P.rows ? r0 + chunk : P.rows;
    T *acc = sacc + grp * per;
    constexpr int U = 8;       // rows in flight per thread: their loads issue together
    for (int row0 = r0 + grp; row0 < r1; row0 += U * G) {
        int qv[U];
        T gv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int row = row0 + u * G;
            int t = -1;
            if (row < r1) t = tm[row < P.natoms ? row : row % P.natoms];
            qv[u] = t >= 0 && t < 16 ? qof[t] : -1;
            gv[u] = qv[u] >= 0 && idx < NA ? A_bar[(long long)row * NA + idx] : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (qv[u] >= 0 && idx == 0) seen[qv[u]] = 1;
        if (idx < NA) {
            for (int q = 0; q < np; ++q) {       // the U rows' counts of t_j load together
                T nv[U];
#pragma unroll
                for (int u = 0; u < U; ++u)
                    nv[u] = qv[u] >= 0 ? T(n_empty[(row0 + u * G) * np + q]) : T(0);
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (qv[u] >= 0) acc[(qv[u] * np + q) * NA + idx] += nv[u] * gv[u];
            }
        }
    }
    __syncthreads();
    double *out = gsum + (long long)(blockIdx.x % kPadReps) * per;
    for (int q = threadIdx.x; q < per; q += blockDim.x) {
        if (!seen[q / (np * NA)]) continue;
        double v = 0.0;
        for (int g = 0; g < G; ++g) v += (double)sacc[g * per + q];
        atomicAdd(out + q, v);
    }
}

// One warp per present pair: the net's reverse from dPhi/dG = k sum_c R_pad[c] gsum[c][:],
// writing the pair's gradient block of grad (EmbOff layout; other nets stay as zeroed).
template <typename T>
__global__ void __launch_bounds__(32) dp_pad_net_bwd(const T *__restrict__ params,
                                                     const T *__restrict__ davg,
                                                     const T *__restrict__ dstd, PadParams P,
                                                     const double *__restrict__ gsum,
                                                     T *__restrict__ grad) {
    __shared__ T sx[32], sg[32];
    const int pair = blockIdx.x, lane = threadIdx.x;
    const int ti = P.present[pair / P.npresent], tj = P.present[pair % P.npresent];
    const long long net = (long long)(ti * P.ntypes + tj) * EmbOff::SIZE;
    const T *w = params + net;
    T *g = grad + net;
    const T s = pad_row_value(davg, dstd, ti, 0);
    T x0, h1, x1, h2, x2;
    pad_net_fwd(w, s, sx, lane, x0, h1, x1, h2, x2);
    T gx = T(0);
    if (lane < E) {
        double a = 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double v = 0.0;
            for (int r = 0; r < kPadReps; ++r)
                v += gsum[((long long)r * P.npresent * P.npresent + pair) * NA + c * E + lane];
            a += (double)pad_row_value(davg, dstd, ti, c) * v;
        }
        gx = T(P.inv_mT * a);
    }
    // layers 2 and 1: x_l = tanh(z_l) dt_l + x_{l-1}, z_l = x_{l-1} W_l + b_l
    const int offW[2] = {EmbOff::W2, EmbOff::W1}, offB[2] = {EmbOff::B2, EmbOff::B1},
              offD[2] = {EmbOff::DT2, EmbOff::DT1};
    for (int L = 0; L < 2; ++L) {
        const T h = L == 0 ? h2 : h1, xin = L == 0 ? x1 : x0;
        T gz = T(0);
        if (lane < E) {
            g[offD[L] + lane] = gx * h;
            gz = gx * w[offD[L] + lane] * (T(1) - h * h);
            g[offB[L] + lane] = gz;
            sg[lane] = gz;
            sx[lane] = xin;
        }
        __syncwarp();
        if (lane < E) {
            T back = T(0);
            for (int e = 0; e < E; ++e) {
                g[offW[L] + e * E + lane] = sx[e] * gz;        // dW[e][lane] = xin[e] gz[lane]
                back += w[offW[L] + lane * E + e] * sg[e];      // (W gz)[lane]
            }
            gx += back;
        }
        __syncwarp();
    }
    if (lane < E) {
        const T gz0 = gx * (T(1) - x0 * x0);
        g[EmbOff::B0 + lane] = gz0;
        g[EmbOff::W0 + lane] = s * gz0;
    }
}

int pad_params(const matpl_dp_model *md, int batch, int natoms, int nslots, PadParams &P) {
    P.rows = batch * natoms; P.natoms = natoms; P.nslots = nslots;
    P.ntypes = md->ntypes; P.m = md->m; P.npresent = md->npresent;
    for (int q = 0; q < kMaxPresent; ++q) P.present[q] = q < md->npresent ? md->present[q] : 0;
    P.inv_mT = 1.0 / ((double)md->m * (double)md->npresent);
    return MATPL_OK;
}

template <typename T>
int launch_pad(bool backward, const matpl_dp_model *md, int batch, int natoms, int nslots,
               const int32_t *ln, const int32_t *tm, const void *in, void *out,
               int32_t *n_empty, void *ws, cudaStream_t s) {
    PadParams P;
    pad_params(md, batch, natoms, nslots, P);
    const int np = P.npresent, sms = device_sms();
    if (!backward) {
        T *prow = static_cast<T *>(ws);
        {
            ProfScope ps("dp_pad_rows", s);
            dp_pad_rows<T><<<np * np, 32, 0, s>>>((const T *)md->params, (const T *)md->davg,
                                                   (const T *)md->dstd, P, prow);
        }
        int st = check_launch("matpl_dp_pad_forward");
        if (st) return st;
        long long grid = ((long long)P.rows + 7) / 8;
        if (grid > (long long)sms * 16) grid = (long long)sms * 16;
        ProfScope ps("dp_pad_add", s);
        dp_pad_add<T><<<(int)grid, 256, 0, s>>>(ln, tm, prow, P, (const T *)in, (T *)out,
                                                n_empty);
        return check_launch("matpl_dp_pad_forward");
    }
    double *gsum = static_cast<double *>(ws);
    const size_t per = (size_t)np * np * NA * sizeof(double);
    cudaMemsetAsync(gsum, 0, per * kPadReps, s);
    cudaMemsetAsync(out, 0, (size_t)md->ntypes * md->ntypes * EmbOff::SIZE * sizeof(T), s);
    const size_t sper = (size_t)np * np * NA * sizeof(T);   // one group's shared sums
    int G = 4;                                       // row groups per CTA, as shared memory allows
    while (G > 1 && sper * G > 100 * 1024) --G;
    const long long nblk = (long long)sms * (16 / G);
    const int chunk = (int)(((long long)P.rows + nblk - 1) / nblk);
    const int grid = (P.rows + chunk - 1) / chunk;
    cudaFuncSetAttribute(dp_pad_reduce<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sper * G));
    {
        ProfScope ps("dp_pad_reduce", s);
        dp_pad_reduce<T><<<grid, 128 * G, sper * G, s>>>(tm, n_empty, (const T *)in, P, chunk,
                                                         gsum);
    }
    int st = check_launch("matpl_dp_pad_backward");
    if (st) return st;
    ProfScope ps("dp_pad_net_bwd", s);
    dp_pad_net_bwd<T><<<np * np, 32, 0, s>>>((const T *)md->params, (const T *)md->davg,
                                              (const T *)md->dstd, P, gsum, (T *)out);
    return check_launch("matpl_dp_pad_backward");
}

int check_args(int dtype, int batch, int natoms, int nslots, int ntypes, int m) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "the training kernels support MATPL_F32 and MATPL_F64");
    MATPL_REQUIRE(batch > 0 && natoms > 0 && ntypes >= 1 && ntypes <= 16 && m > 0 &&
                      nslots == ntypes * m && nslots <= 4096,
                  MATPL_ERR_INVALID, "bad batch / natoms / ntypes / m / nslots");
    return MATPL_OK;
}

template <typename T>
int launch(bool backward, const matpl_dp_model *md, int batch, int natoms, int nslots,
           const int32_t *ln, const void *idr, const int32_t *tm, const void *gF, const void *gV,
           const void *a_in, const void *ad_in, void *out0, void *out1, cudaStream_t s) {
    TrainParams P;
    P.batch = batch; P.natoms = natoms; P.nslots = nslots; P.ntypes = md->ntypes; P.m = md->m;
    P.present_mask = 0;
    for (int q = 0; q < md->npresent; ++q) P.present_mask |= 1 << md->present[q];
    P.has_gv = gV != nullptr;
    P.rmin = md->rmin; P.rmax = md->rmax;
    P.inv_mT = 1.0 / ((double)md->m * (double)md->npresent);
    const int nnet = md->ntypes * md->ntypes;
    const size_t wbytes = (size_t)nnet * EmbOff::SIZE * sizeof(T);          // gradient block
    const size_t wf = (size_t)nnet * NetS::FWD * sizeof(T), wb = (size_t)nnet * NetS::BWD * sizeof(T);
    int dev = 0, sms = device_sms();
    cudaGetDevice(&dev);
    const long long total = (long long)batch * natoms;
    if (!backward) {
        int warps = 8;
        auto needf = [&](int w) {
            return wf + (size_t)w * 32 * kFwdRow * sizeof(T) + (size_t)w * nslots * sizeof(int);
        };
        while (warps > 1 && needf(warps) > 110 * 1024) --warps;
        const size_t smem = needf(warps);
        MATPL_REQUIRE(smem <= 220 * 1024, MATPL_ERR_UNSUPPORTED, "too many types for shared memory");
        cudaFuncSetAttribute(dp_dual_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        long long grid = (total + warps - 1) / warps;
        if (grid > (long long)sms * 8) grid = (long long)sms * 8;
        ProfScope ps("dp_dual_fwd", s);
        dp_dual_fwd<T><<<(int)grid, 32 * warps, smem, s>>>(
            ln, (const T *)idr, tm, (const T *)md->params, (const T *)md->davg,
            (const T *)md->dstd, (const T *)gF, (const T *)gV, (T *)out0, (T *)out1, P);
        return check_launch("matpl_dp_dual_forward");
    }
    int warps = 8;
    auto need = [&](int w) {
        return wb + wbytes + (size_t)w * 32 * Stage::ROW * sizeof(T) +
               (size_t)w * 2 * NA * sizeof(T) + (size_t)w * nslots * sizeof(int);
    };
    while (warps > 1 && need(warps) > 220 * 1024) --warps;
    const size_t smem = need(warps);
    MATPL_REQUIRE(smem <= 220 * 1024, MATPL_ERR_UNSUPPORTED, "too many types for shared memory");
    cudaFuncSetAttribute(dp_dual_bwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    long long grid = (total + warps - 1) / warps;
    if (grid > (long long)sms * 4) grid = (long long)sms * 4;
    cudaMemsetAsync(out0, 0, wbytes, s);
    ProfScope ps("dp_dual_bwd", s);
    dp_dual_bwd<T><<<(int)grid, 32 * warps, smem, s>>>(
        ln, (const T *)idr, tm, (const T *)md->params, (const T *)md->davg, (const T *)md->dstd,
        (const T *)gF, (const T *)gV, (const T *)a_in, (const T *)ad_in, (T *)out0, P);
    return check_launch("matpl_dp_dual_backward");
}

int validate(int dtype, const matpl_dp_model *model, int batch, int natoms, int nslots,
             const int32_t *ln, const void *idr, const int32_t *tm, const void *gF) {
    MATPL_REQUIRE(model != nullptr, MATPL_ERR_INVALID, "null model");
    int st = check_args(dtype, batch, natoms, nslots, model->ntypes, model->m);
    if (st) return st;
    MATPL_REQUIRE(model->npresent >= 1 && model->npresent <= 8, MATPL_ERR_INVALID,
                  "npresent must be 1..8");
    for (int q = 0; q < model->npresent; ++q)
        MATPL_REQUIRE(model->present[q] >= 0 && model->present[q] < model->ntypes,
                      MATPL_ERR_INVALID, "present[] entry outside [0, ntypes)");
    MATPL_REQUIRE(model->params && model->davg && model->dstd && ln && idr && tm && gF,
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE(model->ctable == nullptr, MATPL_ERR_UNSUPPORTED,
                  "the training kernels take the embedding nets, not a compressed table");
    return MATPL_OK;
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" int matpl_dp_dual_forward(int dtype, const matpl_dp_model *model, int batch,
                                     int natoms, int nslots, const int32_t *list_neigh,
                                     const void *image_dr, const int32_t *type_map,
                                     const void *grad_force, const void *grad_virial, void *A,
                                     void *A_dot, void *stream) {
    int st = validate(dtype, model, batch, natoms, nslots, list_neigh, image_dr, type_map,
                      grad_force);
    if (st) return st;
    MATPL_REQUIRE(A && A_dot, MATPL_ERR_INVALID, "null output");
    MATPL_REQUIRE_ON_DEVICE(A, "matpl_dp_dual_forward");
    return dtype == MATPL_F64
               ? launch<double>(false, model, batch, natoms, nslots, list_neigh, image_dr,
                                type_map, grad_force, grad_virial, nullptr, nullptr, A, A_dot,
                                as_stream(stream))
               : launch<float>(false, model, batch, natoms, nslots, list_neigh, image_dr,
                               type_map, grad_force, grad_virial, nullptr, nullptr, A, A_dot,
                               as_stream(stream));
}

extern "C" int matpl_dp_dual_backward(int dtype, const matpl_dp_model *model, int batch,
                                      int natoms, int nslots, const int32_t *list_neigh,
                                      const void *image_dr, const int32_t *type_map,
                                      const void *grad_force, const void *grad_virial,
                                      const void *A_bar, const void *A_dot_bar,
                                      void *grad_embedding, void *stream) {
    int st = validate(dtype, model, batch, natoms, nslots, list_neigh, image_dr, type_map,
                      grad_force);
    if (st) return st;
    MATPL_REQUIRE(A_bar && A_dot_bar && grad_embedding, MATPL_ERR_INVALID, "null pointer");
    MATPL_REQUIRE_ON_DEVICE(grad_embedding, "matpl_dp_dual_backward");
    return dtype == MATPL_F64
               ? launch<double>(true, model, batch, natoms, nslots, list_neigh, image_dr,
                                type_map, grad_force, grad_virial, A_bar, A_dot_bar,
                                grad_embedding, nullptr, as_stream(stream))
               : launch<float>(true, model, batch, natoms, nslots, list_neigh, image_dr,
                               type_map, grad_force, grad_virial, A_bar, A_dot_bar,
                               grad_embedding, nullptr, as_stream(stream));
}

extern "C" size_t matpl_dp_pad_workspace_bytes(int npresent) {
    if (npresent < 1 || npresent > kMaxPresent) return 0;
    return (size_t)kPadReps * npresent * npresent * NA * sizeof(double);
}

extern "C" int matpl_dp_pad_forward(int dtype, const matpl_dp_model *model, int batch,
                                    int natoms, int nslots, const int32_t *list_neigh,
                                    const int32_t *type_map, const void *A_occ, void *A,
                                    int32_t *n_empty, void *workspace, size_t workspace_bytes,
                                    void *stream) {
    MATPL_REQUIRE(model != nullptr, MATPL_ERR_INVALID, "null model");
    int st = check_args(dtype, batch, natoms, nslots, model->ntypes, model->m);
    if (st) return st;
    MATPL_REQUIRE(model->npresent >= 1 && model->npresent <= kMaxPresent, MATPL_ERR_INVALID,
                  "npresent must be 1..8");
    MATPL_REQUIRE((long long)batch * natoms < (1LL << 28), MATPL_ERR_INVALID,
                  "batch * natoms must stay below 2^28");
    for (int q = 0; q < model->npresent; ++q)
        MATPL_REQUIRE(model->present[q] >= 0 && model->present[q] < model->ntypes,
                      MATPL_ERR_INVALID, "present[] entry outside [0, ntypes)");
    MATPL_REQUIRE(model->params && model->davg && model->dstd && list_neigh && type_map &&
                      A_occ && A && n_empty,
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE(workspace && workspace_bytes >= matpl_dp_pad_workspace_bytes(model->npresent),
                  MATPL_ERR_WORKSPACE, "workspace smaller than matpl_dp_pad_workspace_bytes");
    MATPL_REQUIRE_ON_DEVICE(A, "matpl_dp_pad_forward");
    return dtype == MATPL_F64
               ? launch_pad<double>(false, model, batch, natoms, nslots, list_neigh, type_map,
                                    A_occ, A, n_empty, workspace, as_stream(stream))
               : launch_pad<float>(false, model, batch, natoms, nslots, list_neigh, type_map,
                                   A_occ, A, n_empty, workspace, as_stream(stream));
}

extern "C" int matpl_dp_pad_backward(int dtype, const matpl_dp_model *model, int batch,
                                     int natoms, int nslots, const int32_t *type_map,
                                     const int32_t *n_empty, const void *A_bar,
                                     void *grad_embedding, void *workspace,
                                     size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE(model != nullptr, MATPL_ERR_INVALID, "null model");
    int st = check_args(dtype, batch, natoms, nslots, model->ntypes, model->m);
    if (st) return st;
    MATPL_REQUIRE(model->npresent >= 1 && model->npresent <= kMaxPresent, MATPL_ERR_INVALID,
                  "npresent must be 1..8");
    MATPL_REQUIRE((long long)batch * natoms < (1LL << 28), MATPL_ERR_INVALID,
                  "batch * natoms must stay below 2^28");
    for (int q = 0; q < model->npresent; ++q)
        MATPL_REQUIRE(model->present[q] >= 0 && model->present[q] < model->ntypes,
                      MATPL_ERR_INVALID, "present[] entry outside [0, ntypes)");
    MATPL_REQUIRE(model->params && model->davg && model->dstd && type_map && n_empty && A_bar &&
                      grad_embedding,
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE(workspace && workspace_bytes >= matpl_dp_pad_workspace_bytes(model->npresent),
                  MATPL_ERR_WORKSPACE, "workspace smaller than matpl_dp_pad_workspace_bytes");
    MATPL_REQUIRE_ON_DEVICE(grad_embedding, "matpl_dp_pad_backward");
    return dtype == MATPL_F64
               ? launch_pad<double>(true, model, batch, natoms, nslots, nullptr, type_map, A_bar,
                                    grad_embedding, const_cast<int32_t *>(n_empty), workspace,
                                    as_stream(stream))
               : launch_pad<float>(true, model, batch, natoms, nslots, nullptr, type_map, A_bar,
                                   grad_embedding, const_cast<int32_t *>(n_empty), workspace,
                                   as_stream(stream));
}

extern "C" int matpl_dp_desc_dual(int dtype, long long natoms, int m2, const long long *rows,
                                  const void *A, const void *A_dot, void *D, void *D_dot,
                                  void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_dp_desc_dual: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(natoms >= 0 && m2 >= 1 && m2 <= dp::E, MATPL_ERR_INVALID,
                  "natoms >= 0 and 1 <= m2 <= 25");
    MATPL_REQUIRE(natoms == 0 || (A && A_dot && D && D_dot), MATPL_ERR_INVALID,
                  "null pointer argument");
    if (natoms == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(D, "matpl_dp_desc_dual");
    return dtype == MATPL_F64
               ? launch_desc<double>(false, natoms, m2, rows, A, A_dot, nullptr, nullptr, D,
                                     D_dot, as_stream(stream))
               : launch_desc<float>(false, natoms, m2, rows, A, A_dot, nullptr, nullptr, D,
                                    D_dot, as_stream(stream));
}

extern "C" int matpl_dp_desc_dual_grad(int dtype, long long natoms, int m2,
                                       const long long *rows, const void *A, const void *A_dot,
                                       const void *grad_D, const void *grad_D_dot, void *grad_A,
                                       void *grad_A_dot, void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "matpl_dp_desc_dual_grad: dtype is MATPL_F32 or MATPL_F64");
    MATPL_REQUIRE(natoms >= 0 && m2 >= 1 && m2 <= dp::E, MATPL_ERR_INVALID,
                  "natoms >= 0 and 1 <= m2 <= 25");
    MATPL_REQUIRE(natoms == 0 || (A && A_dot && grad_A && grad_A_dot), MATPL_ERR_INVALID,
                  "null pointer argument");
    if (natoms == 0) return MATPL_OK;
    MATPL_REQUIRE_ON_DEVICE(grad_A, "matpl_dp_desc_dual_grad");
    return dtype == MATPL_F64
               ? launch_desc<double>(true, natoms, m2, rows, A, A_dot, grad_D, grad_D_dot,
                                     grad_A, grad_A_dot, as_stream(stream))
               : launch_desc<float>(true, natoms, m2, rows, A, A_dot, grad_D, grad_D_dot,
                                    grad_A, grad_A_dot, as_stream(stream));
}
