// Mixed-precision DP se_e2_a embedding stage on the 5th-generation tensor cores.
//
// Same math as dp_fused.cu's dp_embed_fwd / dp_embed_bwd (src/model/dp_dp.py:217-415 and the
// autograd adjoint of it), reorganised for tcgen05:
//
//   * A CTA (128 threads) takes a group of up to 16 centre atoms, builds their occupied-slot
//     list in shared memory ordered by embedding net (t_i, t_j), then walks it in tiles of
//     128 pair rows: thread r owns row r.
//   * Layer 1 (1 -> 25, rank one) and every tanh / residual stay on the SIMT cores in FP32.
//   * Layers 2 and 3 (25 x 25, padded to 32 x 32) run as tcgen05.mma kind::f16 with BF16
//     operands staged in shared memory (K-major, no swizzle) and FP32 accumulators in TMEM
//     (32 columns); thread r reads row r back with tcgen05.ld.32x32b.  SPLIT = 3 keeps FP32-
//     level accuracy with hi/lo BF16 halves (x_h W_h + x_h W_l + x_l W_h).
//   * Forward: A[4][25] per atom = sum over its rows of R^T G (rows of one atom are
//     contiguous in a tile; one task per (atom segment, A entry)), + empty-slot term, / (m T).
//   * Backward: recomputes layers 1-3, back-propagates dE/dA through the two transposed
//     GEMMs (again tcgen05), contracts with Ri_d, scatters F_j, and reduces F_i and the
//     per-atom virial (FP64) per atom.
// Every mbarrier wait is bounded; a timeout sets MATPL_KERR_TIMEOUT in err_dev.
#include <algorithm>
#include <atomic>
#include "common.cuh"
#include "dp_layout.cuh"
#include "tc.cuh"

namespace matpl {
namespace {

using namespace dp;
constexpr int TM = 128;                 // pair rows per tile = threads per CTA
constexpr int GAMAX = 16;               // centre atoms per group
constexpr int KP = 32;                  // padded embedding width
constexpr int XKS = TM / 8 * 128;       // K-chunk stride of an activation tile (2048 B)
constexpr int WKS = KP / 8 * 128;       // K-chunk stride of a weight tile (512 B)
constexpr int XT = TM * KP * 2;         // activation tile bytes (8 KB)
constexpr int WT = KP * KP * 2;         // weight tile bytes (2 KB)
constexpr int STG = 29;                 // staging row stride (floats, odd: conflict-free)
constexpr int kWaitLimit = 1 << 24;
constexpr int kMaxTypes = 16;
constexpr int VEC = 6 * E;              // per-net FP32 vectors: W0 b0 b1 dt1 b2 dt2

struct MixParams {
    int batch, natoms, nslots, nghost, ntypes, m, present_mask, ga;
    float rmin, rmax, inv_mT;
};

struct MixSmem {
    unsigned char *wt;     // 8 weight tiles of the current net: fw1 h/l, fw2 h/l, bw2 h/l, bw1 h/l
    unsigned char *xh, *xl;
    float *stage;          // [TM][STG], aliases xh/xl (free once a tile's last MMA completed)
    int *seg;              // [GAMAX + 1] segment starts of the current tile, seg_atom follows
    int *seg_atom;         // [GAMAX]
    float *vec;            // [nnet][VEC]
    int *list;             // [ga * S]
    int *cnt;              // [GAMAX][kMaxTypes]
    int *off;              // [GAMAX][kMaxTypes]
    int *net_start;        // [kMaxTypes*kMaxTypes + 1]
    int *tia;              // [GAMAX] model type of each group atom (-1: skipped)
    float *acc;            // fwd: A [GAMAX][NA]; bwd: dA [GAMAX][NA]
    float *fi;             // bwd: [GAMAX][3]
    double *vir;           // bwd: [GAMAX][9]
};

__host__ __device__ inline size_t mix_smem_bytes(int nnet, int S, int ga) {
    size_t o = 0;
    o += 8 * WT;                                  // weight tiles
    o += 2 * XT;                                  // activation tiles (stage aliases them)
    o += sizeof(int) * (2 * GAMAX + 1);
    o = (o + 15) / 16 * 16;
    o += sizeof(float) * nnet * VEC;
    o += sizeof(int) * (size_t)ga * S;
    o += sizeof(int) * 2 * GAMAX * kMaxTypes + sizeof(int) * (kMaxTypes * kMaxTypes + 1);
    o += sizeof(int) * GAMAX;
    o = (o + 15) / 16 * 16;
    o += sizeof(float) * GAMAX * NA + sizeof(float) * GAMAX * 4;
    o = (o + 15) / 16 * 16;
    o += sizeof(double) * GAMAX * 9;
    return o + 64;
}

__device__ MixSmem carve(unsigned char *base, int nnet, int S, int ga) {
    MixSmem m;
    size_t o = 0;
    m.wt = base + o; o += 8 * WT;
    m.xh = base + o; o += XT;
    m.xl = base + o; o += XT;
    m.stage = reinterpret_cast<float *>(m.xh);
    m.seg = reinterpret_cast<int *>(base + o); o += sizeof(int) * (GAMAX + 1);
    m.seg_atom = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX;
    o = (o + 15) / 16 * 16;
    m.vec = reinterpret_cast<float *>(base + o); o += sizeof(float) * nnet * VEC;
    m.list = reinterpret_cast<int *>(base + o); o += sizeof(int) * (size_t)ga * S;
    m.cnt = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX * kMaxTypes;
    m.off = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX * kMaxTypes;
    m.net_start = reinterpret_cast<int *>(base + o); o += sizeof(int) * (kMaxTypes * kMaxTypes + 1);
    m.tia = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX;
    o = (o + 15) / 16 * 16;
    m.acc = reinterpret_cast<float *>(base + o); o += sizeof(float) * GAMAX * NA;
    m.fi = reinterpret_cast<float *>(base + o); o += sizeof(float) * GAMAX * 4;
    o = (o + 15) / 16 * 16;
    m.vir = reinterpret_cast<double *>(base + o);
    return m;
}

template <bool FAST>
__device__ __forceinline__ float act(float x) {
    if (FAST) return tc::tanh_fast(x);
    return tanhf(x);
}

// FP32 environment row (dp_dp.py:241-297) and the Ri_d contraction, single precision.
__device__ __forceinline__ void switch_f(float R, float rmin, float rmax, float &s, float &ds) {
    s = 0.f;
    ds = 0.f;
    if (R > 0.f && R < rmin) {
        s = 1.f / R;
        ds = -1.f / (R * R);
    } else if (R > rmin && R < rmax) {
        const float u = (R - rmin) / (rmax - rmin);
        const float q = -6.f * u * u + 15.f * u - 10.f;
        const float poly = u * u * u * q + 1.f;
        const float dpoly = (3.f * u * u * q + u * u * u * (-12.f * u + 15.f)) / (rmax - rmin);
        s = poly / R;
        ds = dpoly / R - poly / (R * R);
    }
}

__device__ __forceinline__ void rid_contract_f(float R, float x, float y, float z, float rmin,
                                               float rmax, const float *sd, const float g[4],
                                               float f[3]) {
    float s, ds;
    switch_f(R, rmin, rmax, s, ds);
    f[0] = f[1] = f[2] = 0.f;
    if (!(fabsf(R) > 1e-5f)) return;
    const float inv = 1.f / R;
    const float common = (ds - s * inv) * inv * inv;
    const float xyz[3] = {x, y, z};
    const float g0 = g[0] / sd[0], g1 = g[1] / sd[1], g2 = g[2] / sd[2], g3 = g[3] / sd[3];
    const float cg = common * (g1 * x + g2 * y + g3 * z);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float gd = (a == 0 ? g1 : (a == 1 ? g2 : g3)) * s * inv;
        f[a] = -(g0 * ds * xyz[a] * inv + cg * xyz[a] + gd);
    }
}

// Stage the per-net FP32 vectors of every net (W0, b0, b1, dt1, b2, dt2).  Entries of dt are
// used as multipliers, so nothing is divided in the per-row code.
__device__ void stage_vectors(const float *__restrict__ params, float *vec, int nnet) {
    for (int q = threadIdx.x; q < nnet * VEC; q += blockDim.x) {
        const int k = q / VEC, r = q - k * VEC;
        const int part = r / E, o = r - part * E;
        const float *w = params + (long long)k * EmbOff::SIZE;
        const int src[6] = {EmbOff::W0, EmbOff::B0, EmbOff::B1, EmbOff::DT1, EmbOff::B2, EmbOff::DT2};
        vec[q] = w[src[part] + o];
    }
}

// The 8 BF16 weight tiles (hi / lo) of every net, prepared once per call in global memory:
// fw1[n=o][k=i] = W1[i][o], fw2 likewise, bw2[n=i][k=o] = W2[i][o], bw1[n=i][k=o] = W1[i][o];
// zero outside 25 x 25.  Layout [net][8][WT bytes].
__global__ void prep_weight_tiles(const float *__restrict__ params, unsigned char *__restrict__ out,
                                  int nnet) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nnet * 4 * KP * KP;
         q += gridDim.x * blockDim.x) {
        const int k = q / (4 * KP * KP), rr = q - k * 4 * KP * KP;
        const int mat = rr / (KP * KP), rem = rr - mat * KP * KP;
        const int n = rem / KP, kk = rem - (rem / KP) * KP;
        const float *w = params + (long long)k * EmbOff::SIZE;
        float v = 0.f;
        if (n < E && kk < E) {
            switch (mat) {
                case 0: v = w[EmbOff::W1 + kk * E + n]; break;   // fw1: W1[i=kk][o=n]
                case 1: v = w[EmbOff::W2 + kk * E + n]; break;   // fw2
                case 2: v = w[EmbOff::W2 + n * E + kk]; break;   // bw2: W2[i=n][o=kk]
                default: v = w[EmbOff::W1 + n * E + kk]; break;  // bw1
            }
        }
        const __nv_bfloat16 hi = __float2bfloat16_rn(v);
        const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
        unsigned char *base = out + (size_t)k * 8 * WT;
        *reinterpret_cast<__nv_bfloat16 *>(base + (2 * mat) * WT + tc::tile_off(n, kk, WKS)) = hi;
        *reinterpret_cast<__nv_bfloat16 *>(base + (2 * mat + 1) * WT + tc::tile_off(n, kk, WKS)) = lo;
    }
}

__device__ __forceinline__ void load_weight_tiles(const unsigned char *__restrict__ src, int k,
                                                  unsigned char *wt) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src + (size_t)k * 8 * WT);
    uint4 *d4 = reinterpret_cast<uint4 *>(wt);
    for (int q = threadIdx.x; q < 8 * WT / 16; q += blockDim.x) d4[q] = __ldg(s4 + q);
}

// Segments of the current tile: maximal runs of one atom (rows are sorted by atom).  Every
// thread flags whether its row starts a segment; a ballot per warp and a prefix over the four
// warps place the segment starts.  Returns the segment count (includes __syncthreads).
__device__ __forceinline__ int tile_segments(const MixSmem &sm, int r0, int nrows) {
    __shared__ unsigned ballots[TM / 32];
    const int r = threadIdx.x, lane = r & 31, warp = r >> 5;
    int at = -1;
    bool start = false;
    if (r < nrows) {
        at = sm.list[r0 + r] >> 16;
        start = r == 0 || (sm.list[r0 + r - 1] >> 16) != at;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, start);
    if (lane == 0) ballots[warp] = bal;
    __syncthreads();
    int before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < TM / 32; ++w) {
        const int c = __popc(ballots[w]);
        before += w < warp ? c : 0;
        total += c;
    }
    if (start) {
        const int idx = before + __popc(bal & ((1u << lane) - 1u));
        sm.seg[idx] = r;
        sm.seg_atom[idx] = at;
    }
    if (r == 0) sm.seg[total] = nrows;
    __syncthreads();
    return total;
}

// Write this thread's 32-wide row (hi and, for SPLIT 3, lo halves) into the activation tiles.
template <int SPLIT>
__device__ __forceinline__ void store_act_row(const MixSmem &sm, int r, const float v[KP]) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float h[8], l[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            h[q] = v[8 * c + q];
            if (SPLIT == 3) l[q] = v[8 * c + q] - __bfloat162float(__float2bfloat16_rn(v[8 * c + q]));
        }
        tc::store_row8(sm.xh, r, c, XKS, h);
        if (SPLIT == 3) tc::store_row8(sm.xl, r, c, XKS, l);
    }
}

// D[128 x 32] = X W (weight tile pair `mat`), FP32 in TMEM; one thread issues.
template <int SPLIT>
__device__ __forceinline__ void issue_layer(const MixSmem &sm, uint32_t tmem, int mat,
                                            uint64_t *mbar) {
    const uint32_t id = tc::idesc_bf16(TM, KP);
    const uint32_t xh = tc::smem_u32(sm.xh), xl = tc::smem_u32(sm.xl);
    const uint32_t wh = tc::smem_u32(sm.wt + (2 * mat) * WT);
    const uint32_t wl = tc::smem_u32(sm.wt + (2 * mat + 1) * WT);
    uint32_t acc = 0;
#pragma unroll
    for (int p = 0; p < SPLIT; ++p) {
        const uint32_t xa = p == 2 ? xl : xh;
        const uint32_t wb = p == 1 ? wl : wh;
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
            tc::mma_bf16(tmem, tc::desc_kmajor(xa + kk * 2 * XKS, XKS, 128),
                         tc::desc_kmajor(wb + kk * 2 * WKS, WKS, 128), id, acc);
            acc = 1;
        }
    }
    tc::commit(mbar);
}

// Run one MMA layer: all rows staged -> issue -> wait -> every thread loads its row.
template <int SPLIT>
__device__ __forceinline__ void run_layer(const MixSmem &sm, uint32_t tmem, int mat,
                                          uint64_t *mbar, uint32_t &phase, bool &ok,
                                          float out[KP]) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) issue_layer<SPLIT>(sm, tmem, mat, mbar);
    ok &= tc::mbar_wait(mbar, phase, kWaitLimit);
    phase ^= 1u;
    tc::fence_after_sync();
    const int warp = threadIdx.x >> 5;
    tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), out);
}

// Build the group's occupied-slot list ordered by (net, atom, slot); fills cnt / off /
// net_start / tia.  A 32-slot chunk spans at most a few type blocks (usually one): one ballot
// per spanned block counts / places its occupied slots.  All threads participate.
__device__ void build_group_list(const MixSmem &sm, const int32_t *__restrict__ list_neigh,
                                 const int32_t *__restrict__ type_map, long long g0, int ga,
                                 const MixParams &P) {
    const int S = P.nslots, nt = P.ntypes, nnet = nt * nt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long total = (long long)P.batch * P.natoms;
    const unsigned lt = (1u << lane) - 1u;
    for (int a = warp; a < ga; a += TM / 32) {
        const long long t = g0 + a;
        int ti = -1;
        if (t < total) {
            ti = type_map[(int)(t % P.natoms)];
            if (ti < 0 || ti >= nt || !((P.present_mask >> ti) & 1)) ti = -1;
        }
        if (lane < kMaxTypes) sm.cnt[a * kMaxTypes + lane] = 0;
        if (lane == 0) sm.tia[a] = ti;
        __syncwarp();
        if (ti < 0) continue;
        const int32_t *ln = list_neigh + t * S;
        for (int s0 = 0; s0 < S; s0 += 32) {
            const int s = s0 + lane;
            const int blk = s / P.m;
            const bool active = s < S && ln[s] != 0 && blk < nt && ((P.present_mask >> blk) & 1);
            const int blo = s0 / P.m;
            const int bhi = min(min(S - 1, s0 + 31) / P.m, nt - 1);
            for (int q = blo; q <= bhi; ++q) {
                const unsigned mq = __ballot_sync(0xffffffffu, active && blk == q);
                if (lane == 0 && mq) sm.cnt[a * kMaxTypes + q] += __popc(mq);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int pos = 0;
        for (int k = 0; k < nnet; ++k) {
            sm.net_start[k] = pos;
            const int ti = k / nt, tj = k - ti * nt;
            for (int a = 0; a < ga; ++a) {
                if (sm.tia[a] != ti) continue;
                sm.off[a * kMaxTypes + tj] = pos;
                pos += sm.cnt[a * kMaxTypes + tj];
            }
        }
        sm.net_start[nnet] = pos;
    }
    __syncthreads();
    for (int a = warp; a < ga; a += TM / 32) {
        const long long t = g0 + a;
        if (sm.tia[a] < 0) continue;
        const int32_t *ln = list_neigh + t * S;
        for (int s0 = 0; s0 < S; s0 += 32) {
            const int s = s0 + lane;
            const int blk = s / P.m;
            const bool active = s < S && ln[s] != 0 && blk < nt && ((P.present_mask >> blk) & 1);
            const int blo = s0 / P.m;
            const int bhi = min(min(S - 1, s0 + 31) / P.m, nt - 1);
            for (int q = blo; q <= bhi; ++q) {
                const unsigned mq = __ballot_sync(0xffffffffu, active && blk == q);
                if (!mq) continue;
                const int base = sm.off[a * kMaxTypes + q];
                if (active && blk == q) sm.list[base + __popc(mq & lt)] = (a << 16) | s;
                __syncwarp();
                if (lane == 0) sm.off[a * kMaxTypes + q] = base + __popc(mq);
                __syncwarp();
            }
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------------ forward (A descriptor)
template <int SPLIT, bool FAST>
__global__ void __launch_bounds__(TM, 4)
dp_embed_fwd_tc(const int32_t *__restrict__ list_neigh, const float *__restrict__ idr,
                const int32_t *__restrict__ type_map, const float *__restrict__ params,
                const unsigned char *__restrict__ wtiles, const float *__restrict__ davg,
                const float *__restrict__ dstd, const float *__restrict__ pad,
                float *__restrict__ Aout, int32_t *__restrict__ err, MixParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int nt = P.ntypes, nnet = nt * nt, S = P.nslots;
    const MixSmem sm = carve(smem_raw, nnet, S, P.ga);
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_vectors(params, sm.vec, nnet);
    for (int q = tid; q < 2 * XT / 16; q += TM)
        reinterpret_cast<uint4 *>(sm.xh)[q] = make_uint4(0, 0, 0, 0);   // xh, xl contiguous
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 32);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    uint32_t phase = 0;
    bool ok = true;
    int cur_net = -1;
    const long long total = (long long)P.batch * P.natoms;
    const long long ngroups = (total + P.ga - 1) / P.ga;
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long long g0 = grp * P.ga;
        const int ga = (int)(total - g0 < P.ga ? total - g0 : P.ga);
        build_group_list(sm, list_neigh, type_map, g0, ga, P);
        for (int q = tid; q < GAMAX * NA; q += TM) sm.acc[q] = 0.f;
        __syncthreads();
        for (int k = 0; k < nnet; ++k) {
            const int ns = sm.net_start[k], ne = sm.net_start[k + 1];
            if (ns == ne) continue;
            if (k != cur_net) {
                __syncthreads();
                load_weight_tiles(wtiles, k, sm.wt);
                cur_net = k;
                __syncthreads();
            }
            const int ti = k / nt;
            const float *v = sm.vec + k * VEC;
            const float av0 = davg[4 * ti], av1 = davg[4 * ti + 1], av2 = davg[4 * ti + 2],
                        av3 = davg[4 * ti + 3];
            const float is0 = 1.f / dstd[4 * ti], is1 = 1.f / dstd[4 * ti + 1],
                        is2 = 1.f / dstd[4 * ti + 2], is3 = 1.f / dstd[4 * ti + 3];
            for (int r0 = ns; r0 < ne; r0 += TM) {
                const int nrows = ne - r0 < TM ? ne - r0 : TM;
                const bool valid = tid < nrows;
                float R = 0.f, px = 0.f, py = 0.f, pz = 0.f;
                if (valid) {
                    const int e = sm.list[r0 + tid];
                    const long long t = g0 + (e >> 16);
                    const float4 q4 = __ldg(reinterpret_cast<const float4 *>(idr) + t * S + (e & 0xFFFF));
                    R = q4.x; px = q4.y; py = q4.z; pz = q4.w;
                }
                float s, dsw;
                switch_f(R, P.rmin, P.rmax, s, dsw);
                const float inv = fabsf(R) > 1e-5f ? __frcp_rn(R) : 0.f;
                float rh[4];
                rh[0] = (s - av0) * is0;
                rh[1] = (s * px * inv - av1) * is1;
                rh[2] = (s * py * inv - av2) * is2;
                rh[3] = (s * pz * inv - av3) * is3;
                float x[KP], h[KP];
#pragma unroll
                for (int o = 0; o < KP; ++o) x[o] = o < E ? act<FAST>(rh[0] * v[o] + v[E + o]) : 0.f;
                store_act_row<SPLIT>(sm, tid, x);
                run_layer<SPLIT>(sm, tmem, 0, &mbar, phase, ok, h);
#pragma unroll
                for (int o = 0; o < E; ++o) x[o] += act<FAST>(h[o] + v[2 * E + o]) * v[3 * E + o];
                store_act_row<SPLIT>(sm, tid, x);
                run_layer<SPLIT>(sm, tmem, 1, &mbar, phase, ok, h);
                // the layer-3 MMA has completed: the activation tiles are free for staging
                float *st = sm.stage + tid * STG;
#pragma unroll
                for (int o = 0; o < E; ++o)
                    st[o] = valid ? act<FAST>(h[o] + v[4 * E + o]) * v[5 * E + o] + x[o] : 0.f;
#pragma unroll
                for (int c = 0; c < 4; ++c) st[E + c] = valid ? rh[c] : 0.f;
                const int nseg = tile_segments(sm, r0, nrows);   // includes __syncthreads
                // A[atom][c][p] += sum over the atom's rows of R[c] G[p]: (segment, entry) tasks
                for (int task = tid; task < nseg * NA; task += TM) {
                    const int sg = task / NA, e = task - sg * NA;
                    const int c = e / E, p = e - (e / E) * E;
                    const int ra = sm.seg[sg], rb = sm.seg[sg + 1];
                    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
                    int r = ra;
                    for (; r + 4 <= rb; r += 4) {
                        a0 += sm.stage[r * STG + E + c] * sm.stage[r * STG + p];
                        a1 += sm.stage[(r + 1) * STG + E + c] * sm.stage[(r + 1) * STG + p];
                        a2 += sm.stage[(r + 2) * STG + E + c] * sm.stage[(r + 2) * STG + p];
                        a3 += sm.stage[(r + 3) * STG + E + c] * sm.stage[(r + 3) * STG + p];
                    }
                    for (; r < rb; ++r) a0 += sm.stage[r * STG + E + c] * sm.stage[r * STG + p];
                    sm.acc[sm.seg_atom[sg] * NA + e] += (a0 + a1) + (a2 + a3);
                }
                __syncthreads();
            }
        }
        // empty-slot term, scale, write A
        for (int q = tid; q < ga * NA; q += TM) {
            const int a = q / NA, e = q - a * NA;
            const int ti = sm.tia[a];
            float val = 0.f;
            if (ti >= 0) {
                val = sm.acc[q];
                for (int tj = 0; tj < nt; ++tj) {
                    if (!((P.present_mask >> tj) & 1)) continue;
                    const float nemp = (float)(P.m - sm.cnt[a * kMaxTypes + tj]);
                    val += nemp * pad[(ti * nt + tj) * NA + e];
                }
                val *= P.inv_mT;
            }
            Aout[(g0 + a) * NA + e] = val;
        }
        __syncthreads();
    }
    if (!ok) atomicMax(err, MATPL_KERR_TIMEOUT);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

// ------------------------------------------------------------------ backward (forces)
template <int SPLIT, bool FAST>
__global__ void __launch_bounds__(TM, 3)
dp_embed_bwd_tc(const int32_t *__restrict__ list_neigh, const float *__restrict__ idr,
                const int32_t *__restrict__ type_map, const float *__restrict__ params,
                const unsigned char *__restrict__ wtiles, const float *__restrict__ davg,
                const float *__restrict__ dstd, const float *__restrict__ dAin,
                float *__restrict__ force, double *__restrict__ atom_vir,
                int32_t *__restrict__ err, MixParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int nt = P.ntypes, nnet = nt * nt, S = P.nslots;
    const MixSmem sm = carve(smem_raw, nnet, S, P.ga);
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_vectors(params, sm.vec, nnet);
    for (int q = tid; q < 2 * XT / 16; q += TM)
        reinterpret_cast<uint4 *>(sm.xh)[q] = make_uint4(0, 0, 0, 0);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 32);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    uint32_t phase = 0;
    bool ok = true;
    int cur_net = -1;
    const int nall = P.natoms + P.nghost;
    const long long total = (long long)P.batch * P.natoms;
    const long long ngroups = (total + P.ga - 1) / P.ga;
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long long g0 = grp * P.ga;
        const int ga = (int)(total - g0 < P.ga ? total - g0 : P.ga);
        build_group_list(sm, list_neigh, type_map, g0, ga, P);
        for (int q = tid; q < GAMAX * NA; q += TM) {
            const int a = q / NA;
            sm.acc[q] = a < ga ? dAin[g0 * NA + q] * P.inv_mT : 0.f;
        }
        for (int q = tid; q < GAMAX * 4; q += TM) sm.fi[q] = 0.f;
        for (int q = tid; q < GAMAX * 9; q += TM) sm.vir[q] = 0.0;
        __syncthreads();
        for (int k = 0; k < nnet; ++k) {
            const int ns = sm.net_start[k], ne = sm.net_start[k + 1];
            if (ns == ne) continue;
            if (k != cur_net) {
                __syncthreads();
                load_weight_tiles(wtiles, k, sm.wt);
                cur_net = k;
                __syncthreads();
            }
            const int ti = k / nt;
            const float *v = sm.vec + k * VEC;
            const float av0 = davg[4 * ti], av1 = davg[4 * ti + 1], av2 = davg[4 * ti + 2],
                        av3 = davg[4 * ti + 3];
            const float isd[4] = {1.f / dstd[4 * ti], 1.f / dstd[4 * ti + 1],
                                  1.f / dstd[4 * ti + 2], 1.f / dstd[4 * ti + 3]};
            for (int r0 = ns; r0 < ne; r0 += TM) {
                const int nrows = ne - r0 < TM ? ne - r0 : TM;
                const bool valid = tid < nrows;
                float R = 0.f, px = 0.f, py = 0.f, pz = 0.f;
                int a_loc = 0, j = -1;
                long long t = g0;
                if (valid) {
                    const int e = sm.list[r0 + tid];
                    a_loc = e >> 16;
                    t = g0 + a_loc;
                    const int slot = e & 0xFFFF;
                    const float4 q4 = __ldg(reinterpret_cast<const float4 *>(idr) + t * S + slot);
                    R = q4.x; px = q4.y; py = q4.z; pz = q4.w;
                    j = __ldg(list_neigh + t * S + slot) - 1;
                }
                float s, dsw;
                switch_f(R, P.rmin, P.rmax, s, dsw);
                const bool mask = fabsf(R) > 1e-5f;
                const float inv = mask ? __frcp_rn(R) : 0.f;
                float rh[4];
                rh[0] = (s - av0) * isd[0];
                rh[1] = (s * px * inv - av1) * isd[1];
                rh[2] = (s * py * inv - av2) * isd[2];
                rh[3] = (s * pz * inv - av3) * isd[3];
                // recompute forward, keeping t1 (= x1), t2, t3
                float x[KP], h[KP], t1[E], t2[E];
#pragma unroll
                for (int o = 0; o < KP; ++o) {
                    x[o] = o < E ? act<FAST>(rh[0] * v[o] + v[E + o]) : 0.f;
                    if (o < E) t1[o] = x[o];
                }
                store_act_row<SPLIT>(sm, tid, x);
                run_layer<SPLIT>(sm, tmem, 0, &mbar, phase, ok, h);
#pragma unroll
                for (int o = 0; o < E; ++o) {
                    t2[o] = act<FAST>(h[o] + v[2 * E + o]);
                    x[o] += t2[o] * v[3 * E + o];
                }
                store_act_row<SPLIT>(sm, tid, x);
                run_layer<SPLIT>(sm, tmem, 1, &mbar, phase, ok, h);
#pragma unroll
                for (int o = 0; o < E; ++o) {
                    h[o] = act<FAST>(h[o] + v[4 * E + o]);       // t3
                    x[o] += h[o] * v[5 * E + o];                 // G
                }
                // dE/dR[c] = sum_p dA[c][p] G[p];  dG[p] = sum_c dA[c][p] R[c]
                const float *dA = sm.acc + a_loc * NA;
                float g[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int p = 0; p < E; ++p) {
                    const float d0 = dA[p], d1 = dA[E + p], d2 = dA[2 * E + p], d3 = dA[3 * E + p];
                    g[0] += d0 * x[p];
                    g[1] += d1 * x[p];
                    g[2] += d2 * x[p];
                    g[3] += d3 * x[p];
                    x[p] = d0 * rh[0] + d1 * rh[1] + d2 * rh[2] + d3 * rh[3];
                }
                float y[KP];
#pragma unroll
                for (int o = 0; o < KP; ++o) y[o] = o < E ? x[o] * v[5 * E + o] * (1.f - h[o] * h[o]) : 0.f;
                store_act_row<SPLIT>(sm, tid, y);
                run_layer<SPLIT>(sm, tmem, 2, &mbar, phase, ok, h);
#pragma unroll
                for (int o = 0; o < E; ++o) x[o] += h[o];
#pragma unroll
                for (int o = 0; o < KP; ++o) y[o] = o < E ? x[o] * v[3 * E + o] * (1.f - t2[o] * t2[o]) : 0.f;
                store_act_row<SPLIT>(sm, tid, y);
                run_layer<SPLIT>(sm, tmem, 3, &mbar, phase, ok, h);
                float dsv = 0.f;
#pragma unroll
                for (int o = 0; o < E; ++o) dsv += v[o] * (x[o] + h[o]) * (1.f - t1[o] * t1[o]);
                g[0] += dsv;
                float f[3] = {0.f, 0.f, 0.f};
                if (mask) {   // f_a = sum_c g[c] Ri_d[c][a], Ri_d = -dfeat / dstd
                    const float common = (dsw - s * inv) * inv * inv;
                    const float g0 = g[0] * isd[0], g1 = g[1] * isd[1], g2 = g[2] * isd[2],
                                g3 = g[3] * isd[3];
                    const float cg = common * (g1 * px + g2 * py + g3 * pz);
                    const float sv = s * inv;
                    f[0] = -(g0 * dsw * px * inv + cg * px + g1 * sv);
                    f[1] = -(g0 * dsw * py * inv + cg * py + g2 * sv);
                    f[2] = -(g0 * dsw * pz * inv + cg * pz + g3 * sv);
                }
                float *st = sm.stage + tid * STG;     // activation tiles are free again
                if (valid) {
                    const long long b = t / P.natoms;
                    if (j >= 0 && j < nall) {
                        float *dst = force + (b * nall + j) * 3;
                        atomicAdd(dst + 0, f[0]);
                        atomicAdd(dst + 1, f[1]);
                        atomicAdd(dst + 2, f[2]);
                    }
                    st[0] = f[0]; st[1] = f[1]; st[2] = f[2];
                    st[3] = px; st[4] = py; st[5] = pz;
                } else {
#pragma unroll
                    for (int q = 0; q < 6; ++q) st[q] = 0.f;
                }
                const int nseg = tile_segments(sm, r0, nrows);   // includes __syncthreads
                // per-atom F_i (3) and virial (9): (segment, quantity) tasks
                for (int task = tid; task < nseg * 12; task += TM) {
                    const int sg = task / 12, q = task - sg * 12;
                    const int ra = sm.seg[sg], rb = sm.seg[sg + 1];
                    const int qa = q < 3 ? q : (q - 3) / 3, qc = q < 3 ? 0 : (q - 3) % 3;
                    double a0 = 0.0, a1 = 0.0;
                    int r = ra;
                    for (; r + 2 <= rb; r += 2) {
                        const float *s0 = sm.stage + r * STG, *s1 = s0 + STG;
                        a0 += q < 3 ? (double)s0[qa] : (double)s0[qa] * (double)s0[3 + qc];
                        a1 += q < 3 ? (double)s1[qa] : (double)s1[qa] * (double)s1[3 + qc];
                    }
                    if (r < rb) {
                        const float *s0 = sm.stage + r * STG;
                        a0 += q < 3 ? (double)s0[qa] : (double)s0[qa] * (double)s0[3 + qc];
                    }
                    const int at = sm.seg_atom[sg];
                    if (q < 3) sm.fi[at * 4 + q] -= (float)(a0 + a1);
                    else sm.vir[at * 9 + q - 3] += a0 + a1;
                }
                __syncthreads();
            }
        }
        for (int q = tid; q < ga * 9; q += TM) atom_vir[(g0 + q / 9) * 9 + q % 9] = sm.vir[q];
        for (int q = tid; q < ga * 3; q += TM) {
            const int a = q / 3, c = q - a * 3;
            const long long t = g0 + a;
            const long long b = t / P.natoms;
            const int i = (int)(t - b * P.natoms);
            atomicAdd(force + (b * nall + i) * 3 + c, sm.fi[a * 4 + c]);
        }
        __syncthreads();
    }
    if (!ok) atomicMax(err, MATPL_KERR_TIMEOUT);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

}  // namespace

// Tuning of the mixed embedding kernels (matpl_dp_set_tuning): centre atoms per CTA group
// (how many pair rows feed each 128-row MMA tile) and resident CTAs per SM; 0 = automatic.
static std::atomic<int> g_ga_override{0}, g_ctas_override{0};

// Launch helpers used by dp_fused.cu's matpl_dp_eval for the MATPL_MIXED forms.
int mixed_ga(int S) {
    const int lim = std::max(1, std::min(GAMAX, 9600 / std::max(1, S)));
    const int o = g_ga_override.load();
    return o > 0 ? std::min(o, lim) : lim;
}

size_t mixed_smem(int ntypes, int S) { return mix_smem_bytes(ntypes * ntypes, S, mixed_ga(S)); }

size_t mixed_tile_bytes(int ntypes) { return (size_t)ntypes * ntypes * 8 * WT; }

int prep_mixed_tiles(const float *params, unsigned char *out, int ntypes, cudaStream_t s) {
    const int n = ntypes * ntypes * 4 * KP * KP;
    ProfScope ps("prep_weight_tiles", s);
    prep_weight_tiles<<<(n + 255) / 256, 256, 0, s>>>(params, out, ntypes * ntypes);
    return check_launch("prep_weight_tiles");
}

template <int SPLIT, bool FAST>
int launch_mixed_embed(bool backward, const int32_t *list_neigh, const float *idr,
                       const int32_t *type_map, const float *params, const unsigned char *wtiles,
                       const float *davg, const float *dstd, const float *pad_or_dA,
                       float *A_or_force, double *atom_vir, int32_t *err, int batch, int natoms,
                       int nslots, int nghost, int ntypes, int m, int present_mask, double rmin,
                       double rmax, double inv_mT, cudaStream_t s) {
    MixParams P;
    P.batch = batch; P.natoms = natoms; P.nslots = nslots; P.nghost = nghost;
    P.ntypes = ntypes; P.m = m; P.present_mask = present_mask; P.ga = mixed_ga(nslots);
    P.rmin = (float)rmin; P.rmax = (float)rmax; P.inv_mT = (float)inv_mT;
    const size_t smem = mix_smem_bytes(ntypes * ntypes, nslots, P.ga);
    const long long total = (long long)batch * natoms;
    const long long ngroups = (total + P.ga - 1) / P.ga;
    // resident CTAs per SM: what shared memory allows (the automatic choice stays at 3, the
    // tuning hook may ask for up to 6; the backward's registers cap it at 3 anyway)
    const int fit = (int)std::max<size_t>(1, (220 * 1024) / (smem + 2048));
    int per_sm = std::min(fit, 3);
    if (g_ctas_override.load() > 0) per_sm = std::min(fit, g_ctas_override.load());
    const int grid = (int)std::min<long long>(ngroups, (long long)device_sms() * per_sm);
    if (!backward) {
        auto k = dp_embed_fwd_tc<SPLIT, FAST>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        ProfScope ps("dp_embed_fwd_tc", s);
        k<<<grid, TM, smem, s>>>(list_neigh, idr, type_map, params, wtiles, davg, dstd,
                                 pad_or_dA, A_or_force, err, P);
    } else {
        auto k = dp_embed_bwd_tc<SPLIT, FAST>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        ProfScope ps("dp_embed_bwd_tc", s);
        k<<<grid, TM, smem, s>>>(list_neigh, idr, type_map, params, wtiles, davg, dstd,
                                 pad_or_dA, A_or_force, atom_vir, err, P);
    }
    return check_launch(backward ? "dp_embed_bwd_tc" : "dp_embed_fwd_tc");
}

template int launch_mixed_embed<1, true>(
    bool, const int32_t *, const float *, const int32_t *, const float *, const unsigned char *,
    const float *, const float *, const float *, float *, double *, int32_t *, int, int, int,
    int, int, int, int, double, double, double, cudaStream_t);
template int launch_mixed_embed<3, false>(
    bool, const int32_t *, const float *, const int32_t *, const float *, const unsigned char *,
    const float *, const float *, const float *, float *, double *, int32_t *, int, int, int,
    int, int, int, int, double, double, double, cudaStream_t);
template int launch_mixed_embed<3, true>(
    bool, const int32_t *, const float *, const int32_t *, const float *, const unsigned char *,
    const float *, const float *, const float *, float *, double *, int32_t *, int, int, int,
    int, int, int, int, double, double, double, cudaStream_t);

}  // namespace matpl

extern "C" int matpl_dp_set_tuning(int mixed_group_atoms, int mixed_ctas_per_sm) {
    using namespace matpl;
    MATPL_REQUIRE(mixed_group_atoms >= 0 && mixed_group_atoms <= GAMAX, MATPL_ERR_INVALID,
                  "mixed_group_atoms must be 0 (automatic) .. 16");
    MATPL_REQUIRE(mixed_ctas_per_sm >= 0 && mixed_ctas_per_sm <= 6, MATPL_ERR_INVALID,
                  "mixed_ctas_per_sm must be 0 (automatic) .. 6");
    g_ga_override.store(mixed_group_atoms);
    g_ctas_override.store(mixed_ctas_per_sm);
    return MATPL_OK;
}

extern "C" int matpl_dp_get_tuning(int *mixed_group_atoms, int *mixed_ctas_per_sm) {
    using namespace matpl;
    MATPL_REQUIRE(mixed_group_atoms && mixed_ctas_per_sm, MATPL_ERR_INVALID, "null pointer");
    *mixed_group_atoms = g_ga_override.load();
    *mixed_ctas_per_sm = g_ctas_override.load();
    return MATPL_OK;
}
