// Mixed-precision DP se_e2_a embedding stage on the 5th-generation tensor cores.
//
// Same math as dp_fused.cu's dp_embed_fwd / dp_embed_bwd (src/model/dp_dp.py:217-415 and the
// autograd adjoint of it), organised around tcgen05 MMAs:
//
//   * A CTA (128 threads) takes a group of up to 16 centre atoms, builds their occupied-slot
//     list in shared memory ordered by embedding net (t_i, t_j), then walks it in tiles of
//     128 pair rows: thread r owns row r (the M row of every MMA of the tile).
//   * Layer 1 (1 -> 25, rank one) and every tanh / residual stay on the SIMT cores in FP32.
//   * Layers 2 and 3 (25 x 25, padded to 32 x 32) run as tcgen05.mma kind::f16 with BF16
//     operands in shared memory (K-major, no swizzle) and FP32 accumulators in TMEM; the layer
//     biases ride in the MMA (activation column 25 holds 1, weight row 25 holds the bias).
//     SPLIT = 3 keeps FP32-level accuracy with hi / lo BF16 halves (x_h W_h + x_h W_l + x_l W_h).
//   * Forward descriptor contraction A[a][c][p] = sum over the atom's rows of R[c] G[p]
//     (dp_dp.py:344-415) runs on the tensor cores too: the G tile the threads write row by row
//     is read as an MN-major B operand whose K index is the pair row, against an A operand
//     that holds, in column r, row r's environment row at M = 8 a + 2 c + h (h = BF16 hi / lo
//     half), so one accumulator D[128 x 32] in TMEM collects every atom of the group over all
//     its tiles and nets.
//   * Backward: recomputes layers 1-3, forms dE/dR and dE/dG from dE/dA on the SIMT cores,
//     back-propagates through the two transposed layer GEMMs (tcgen05), contracts with Ri_d,
//     scatters F_j, and reduces each atom's F_i and virial with one more MMA: a one-hot A
//     operand (column r = atom of row r) against the per-row (f, f x r) values, accumulated in
//     TMEM over the group.
// Every mbarrier wait is bounded.  A wait that gives up sets MATPL_KERR_TIMEOUT; the CTA then
// issues no further MMA and no further TMEM load, drains what it already issued (bounded
// again), frees its TMEM and returns.
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
constexpr int ONE = E;                  // activation column that carries the bias (value 1)
constexpr int XKS = TM / 8 * 128;       // K-chunk stride of an activation tile (2048 B)
constexpr int WKS = KP / 8 * 128;       // K-chunk stride of a weight tile (512 B)
constexpr int XT = TM * KP * 2;         // activation tile bytes (8 KB)
constexpr int WT = KP * KP * 2;         // weight tile bytes (2 KB)
constexpr int RT = 128 * TM * 2;        // contraction A operand: 128 (M) x 128 (K) bf16 (32 KB)
constexpr int ET = 64 * TM * 2;         // one-hot A operand of the backward: 64 (M) x 128 (K)
constexpr int OLBO = 128;               // MN-major operands: K-group stride
constexpr int OSBO = TM / 8 * 128;      //                    MN-group stride (2048 B)
constexpr int QN = 16;                  // per-row reduction values (f: 3, f x r: 9, 4 zero)
constexpr int QT = QN * TM * 2;         // reduction B operand bytes (4 KB)
constexpr int VW = 28;                  // per-net vector stride in floats (25 padded to 7 float4)
constexpr int kMaxTypes = 16;
constexpr int kDrainPolls = 1 << 24;    // bound of the waits that drain MMAs before exit

// TMEM columns: [0, 32) layer accumulator; forward: [64, 128) descriptor accumulator (the G hi
// and lo halves side by side); backward: [32, 64) layer-2 tanh stash, [64, 112) F_i / virial
// accumulator (the three BF16 parts side by side).  Each small MMA costs the tensor core about
// as much as its issue, so the split parts of an operand are laid side by side along N (one
// MMA per K step) rather than issued as separate products.
constexpr uint32_t TCOL_A = 64, TCOL_STASH = 32, TCOL_RED = 64;

struct MixParams {
    int batch, natoms, nslots, nghost, ntypes, m, present_mask, ga;
    float rmin, rmax, inv_mT;
    int wait_polls;                      // bound of every completion wait
    const int32_t *num_neigh;            // [B*N][ntypes] block lengths, or NULL (scan the list)
};

struct MixSmem {
    unsigned char *wt;     // weight tiles of the current net: fw1 h/l, fw2 h/l
    unsigned char *xh, *xl;
    unsigned char *rop;    // fwd: contraction A operand (M = 128); bwd: one-hot A operand (M = 64)
    unsigned char *qh, *qm, *ql;   // bwd: per-row reduction values, three BF16 parts (MN-major B)
    float *vec;            // [4][VW] of the current net: W0, b0, dt1, dt2
    float *dA;             // bwd: [GAMAX][E] float4 (c fastest) of dE/dA * k
    uint16_t *list;        // [ga * S] rows: atom << 12 | slot
    int *cnt;              // [GAMAX][kMaxTypes]
    int *off;              // [GAMAX][kMaxTypes]
    int *net_start;        // [kMaxTypes*kMaxTypes + 1]
    int *tia;              // [GAMAX] model type of each group atom (-1: skipped)
    int *tiles;            // [tile_cap] the group's tiles in order: net << 16 | first row
    int *ntiles;           // [1]
};

// Upper bound of a group's tiles (each net's rows rounded up to whole tiles).
__host__ __device__ inline int tile_cap(int S, int ga) { return ga * S / TM + kMaxTypes * kMaxTypes + 1; }

__host__ __device__ inline size_t mix_smem_bytes(bool bwd, int S, int ga) {
    size_t o = 0;
    o += 4 * WT;
    o += 2 * XT + (bwd ? ET : RT);
    if (bwd) o += 3 * QT;
    o += sizeof(float) * 4 * VW;
    if (bwd) o += sizeof(float) * GAMAX * E * 4;
    o += align_up(sizeof(uint16_t) * (size_t)ga * S, 16);
    o += sizeof(int) * (2 * GAMAX * kMaxTypes + kMaxTypes * kMaxTypes + 1 + GAMAX);
    o += sizeof(int) * (tile_cap(S, ga) + 1);
    return o + 128;
}

__device__ MixSmem carve(unsigned char *base, bool bwd, int S, int ga) {
    MixSmem m;
    size_t o = 0;
    m.wt = base + o; o += 4 * WT;
    m.xh = base + o; o += XT;
    m.xl = base + o; o += XT;
    m.rop = base + o; o += bwd ? ET : RT;
    m.qh = m.qm = m.ql = nullptr;
    if (bwd) { m.qh = base + o; o += QT; m.qm = base + o; o += QT; m.ql = base + o; o += QT; }
    m.vec = reinterpret_cast<float *>(base + o); o += sizeof(float) * 4 * VW;
    m.dA = nullptr;
    if (bwd) { m.dA = reinterpret_cast<float *>(base + o); o += sizeof(float) * GAMAX * E * 4; }
    m.list = reinterpret_cast<uint16_t *>(base + o); o += align_up(sizeof(uint16_t) * (size_t)ga * S, 16);
    m.cnt = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX * kMaxTypes;
    m.off = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX * kMaxTypes;
    m.net_start = reinterpret_cast<int *>(base + o); o += sizeof(int) * (kMaxTypes * kMaxTypes + 1);
    m.tia = reinterpret_cast<int *>(base + o); o += sizeof(int) * GAMAX;
    m.tiles = reinterpret_cast<int *>(base + o); o += sizeof(int) * tile_cap(S, ga);
    m.ntiles = reinterpret_cast<int *>(base + o);
    return m;
}

template <bool FAST>
__device__ __forceinline__ float act(float x) {
    if (FAST) return tc::tanh_fast(x);
    return tanhf(x);
}

// FP32 switching function of dp_dp.py:241-266 and its r-derivative.
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

// The 4 BF16 weight tiles (hi / lo) of every net, prepared once per call in global memory:
// fw1[n=o][k=i] = W1[i][o] with row k = 25 the bias b1[o], fw2 likewise with W2 and b2; zero
// elsewhere.  Layout [net][4][WT bytes]: fw1 h, fw1 l, fw2 h, fw2 l.  The backward's
// transposed products read the same tiles as MN-major B operands (n = i, k = o): the bias
// row then lands in output column 25, which nothing reads.
__global__ void prep_weight_tiles(const float *__restrict__ params, unsigned char *__restrict__ out,
                                  int nnet) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nnet * 2 * KP * KP;
         q += gridDim.x * blockDim.x) {
        const int k = q / (2 * KP * KP), rr = q - k * 2 * KP * KP;
        const int mat = rr / (KP * KP), rem = rr - mat * KP * KP;
        const int n = rem / KP, kk = rem - (rem / KP) * KP;
        const float *w = params + (long long)k * EmbOff::SIZE;
        float v = 0.f;
        if (n < E && kk < E)
            v = w[(mat == 0 ? EmbOff::W1 : EmbOff::W2) + kk * E + n];   // W[i=kk][o=n]
        else if (n < E && kk == ONE)
            v = w[(mat == 0 ? EmbOff::B1 : EmbOff::B2) + n];
        const __nv_bfloat16 hi = __float2bfloat16_rn(v);
        const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
        unsigned char *base = out + (size_t)k * 4 * WT;
        *reinterpret_cast<__nv_bfloat16 *>(base + (2 * mat) * WT + tc::tile_off(n, kk, WKS)) = hi;
        *reinterpret_cast<__nv_bfloat16 *>(base + (2 * mat + 1) * WT + tc::tile_off(n, kk, WKS)) = lo;
    }
}

// The 4 weight tiles and the per-net vectors of net k.
__device__ __forceinline__ void load_net(const unsigned char *__restrict__ wsrc,
                                         const float *__restrict__ params, int k,
                                         const MixSmem &sm) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(wsrc + (size_t)k * 4 * WT);
    uint4 *d4 = reinterpret_cast<uint4 *>(sm.wt);
    for (int q = threadIdx.x; q < 4 * WT / 16; q += blockDim.x) d4[q] = __ldg(s4 + q);
    const float *w = params + (long long)k * EmbOff::SIZE;
    for (int q = threadIdx.x; q < 4 * VW; q += blockDim.x) {
        const int part = q / VW, o = q - part * VW;
        const int src[4] = {EmbOff::W0, EmbOff::B0, EmbOff::DT1, EmbOff::DT2};
        sm.vec[q] = o < E ? __ldg(w + src[part] + o) : 0.f;
    }
}

// Write this thread's 32-wide row into the activation tiles (hi, and lo for SPLIT 3).
// Column ONE gets `one` (1 for forward layers: the bias; 0 for the backward ones).
template <int SPLIT>
__device__ __forceinline__ void store_row(const MixSmem &sm, int r, const float v[E], float one) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float w[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int o = 8 * c + q;
            w[q] = o < E ? v[o] : (o == ONE ? one : 0.f);
        }
        uint4 h, l;
        tc::split8(w, h, SPLIT == 3 ? &l : nullptr);
        const uint32_t off = tc::tile_off(r, 8 * c, XKS);
        *reinterpret_cast<uint4 *>(sm.xh + off) = h;
        if (SPLIT == 3) *reinterpret_cast<uint4 *>(sm.xl + off) = l;
    }
}

// Column-r chunk of an MN-major operand with K = pair row r: byte offset of the 16-byte chunk
// holding M / N elements 8 g .. 8 g + 7.
__device__ __forceinline__ uint32_t mn_chunk(int r, int g) {
    return (uint32_t)((r & 7) * 16 + (r >> 3) * OLBO + g * OSBO);
}

// D[128 x 32] (+)= X W for weight tile pair `mat` (0: layer 2, 1: layer 3), or X W^T with
// `transposed` (the same tiles read MN-major); one thread issues, then commits.
template <int SPLIT>
__device__ __forceinline__ void issue_layer(const MixSmem &sm, uint32_t tmem, int mat,
                                            bool transposed, uint64_t *mbar) {
    const uint32_t id = tc::idesc_bf16_mn(TM, KP, false, transposed);
    const uint32_t xh = tc::smem_u32(sm.xh), xl = tc::smem_u32(sm.xl);
    const uint32_t wh = tc::smem_u32(sm.wt + (2 * mat) * WT);
    const uint32_t wl = tc::smem_u32(sm.wt + (2 * mat + 1) * WT);
    // K-major: K-chunk stride WKS, row-group stride 128; transposed (n = i, k = o): K-group
    // stride 128, N-group stride WKS
    const uint32_t lbo = transposed ? 128u : (uint32_t)WKS, sbo = transposed ? (uint32_t)WKS : 128u;
    uint32_t acc = 0;
#pragma unroll
    for (int p = 0; p < SPLIT; ++p) {
        const uint32_t xa = p == 2 ? xl : xh;
        const uint32_t wb = p == 1 ? wl : wh;
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
            tc::mma_bf16(tmem, tc::desc_kmajor(xa + kk * 2 * XKS, XKS, 128),
                         tc::desc_kmajor(wb + kk * 2 * lbo, lbo, sbo), id, acc);
            acc = 1;
        }
    }
    tc::commit(mbar);
}

// D[M x N] (+)= Aop B over K = 128 pair rows, both operands MN-major; B is given as NB tiles
// whose sum it is (BF16 hi / lo parts).  `first`: the first product of the group starts the
// accumulator.
// (With M = 64, rows 0..15 of D sit in TMEM lanes 0..15.)
template <int NB, int M, int N>
__device__ __forceinline__ void issue_rows(uint32_t tmem, const unsigned char *aop,
                                           const unsigned char *b0, const unsigned char *b1,
                                           const unsigned char *b2, bool first, uint64_t *mbar) {
    const uint32_t id = tc::idesc_bf16_mn(M, N, true, true);
    const uint32_t a0 = tc::smem_u32(aop);
    const uint32_t bb[3] = {tc::smem_u32(b0), NB > 1 ? tc::smem_u32(b1) : 0u,
                            NB > 2 ? tc::smem_u32(b2) : 0u};
#pragma unroll
    for (int s = 0; s < TM / 16; ++s) {
        const uint64_t ad = tc::desc_kmajor(a0 + s * 2 * OLBO, OLBO, OSBO);
#pragma unroll
        for (int q = 0; q < NB; ++q)
            tc::mma_bf16(tmem, ad, tc::desc_kmajor(bb[q] + s * 2 * OLBO, OLBO, OSBO), id,
                         (first && s == 0 && q == 0) ? 0u : 1u);
    }
    tc::commit(mbar);
}

// Completion wait shared by all threads; `polls` below 64 selects plain polling (a test hook
// that makes waits give up), otherwise the suspending try_wait.
__device__ __forceinline__ bool wait_done(uint64_t *mbar, uint32_t parity, int polls) {
    return polls < 64 ? tc::mbar_poll(mbar, parity, polls) : tc::mbar_wait(mbar, parity, polls);
}

// Barrier before an MMA issue: makes the generic-proxy shared stores visible to the tensor
// cores and returns true (on every thread) when some thread has seen a wait give up.
__device__ __forceinline__ bool pre_issue(bool ok) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    const int bad = __syncthreads_or(!ok);
    tc::fence_after_sync();
    return bad != 0;
}

// Wait for one commit of `mbar`; on success flips the phase.  The result is made uniform
// across the warp (tcgen05.ld that may follow is a warp-wide instruction).
__device__ __forceinline__ bool wait_commit(uint64_t *mbar, uint32_t &phase, bool &pending,
                                            int polls) {
    const bool got = __all_sync(0xffffffffu, wait_done(mbar, phase, polls));
    if (got) {
        phase ^= 1u;
        pending = false;
    }
    tc::fence_after_sync();
    return got;
}

// TMEM row load that is skipped (zeros) once this warp has seen a wait give up: the CTA then
// leaves at its next barrier without touching the tensor cores again.
__device__ __forceinline__ void ld32_if(bool ok, uint32_t taddr, float v[32]) {
    if (ok) {
        tc::tmem_ld32(taddr, v);
    } else {
#pragma unroll
        for (int q = 0; q < 32; ++q) v[q] = 0.f;
    }
}

// Build the group's occupied-slot list ordered by (net, atom, slot); fills cnt / off /
// net_start / tia.  With block lengths (num_neigh) the occupied slots of each type block are
// its first num_neigh slots; otherwise every slot of the list is tested (ballot per 32 slots).
__device__ void build_group_list(const MixSmem &sm, const int32_t *__restrict__ list_neigh,
                                 const int32_t *__restrict__ type_map, long long g0, int ga,
                                 const MixParams &P) {
    const int S = P.nslots, nt = P.ntypes, nnet = nt * nt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long total = (long long)P.batch * P.natoms;
    const unsigned lt = (1u << lane) - 1u;
    for (int a = warp; a < GAMAX; a += TM / 32) {
        const long long t = g0 + a;
        int ti = -1;
        if (a < ga && t < total) {
            ti = type_map[(int)(t % P.natoms)];
            if (ti < 0 || ti >= nt || !((P.present_mask >> ti) & 1)) ti = -1;
        }
        if (lane < kMaxTypes) sm.cnt[a * kMaxTypes + lane] = 0;
        if (lane == 0) sm.tia[a] = ti;
        __syncwarp();
        if (ti < 0) continue;
        if (P.num_neigh) {
            if (lane < nt && ((P.present_mask >> lane) & 1)) {
                const int c = P.num_neigh[t * nt + lane];
                sm.cnt[a * kMaxTypes + lane] = c < 0 ? 0 : (c > P.m ? P.m : c);
            }
            continue;
        }
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
        int nt_ = 0;                       // tile schedule: tiles never span two nets
        for (int k = 0; k < nnet; ++k)
            for (int r0 = sm.net_start[k]; r0 < sm.net_start[k + 1]; r0 += TM)
                sm.tiles[nt_++] = (k << 16) | r0;
        *sm.ntiles = nt_;
    }
    __syncthreads();
    for (int a = warp; a < ga; a += TM / 32) {
        const long long t = g0 + a;
        if (sm.tia[a] < 0) continue;
        if (P.num_neigh) {
            for (int tj = 0; tj < nt; ++tj) {
                const int c = sm.cnt[a * kMaxTypes + tj], base = sm.off[a * kMaxTypes + tj];
                for (int k = lane; k < c; k += 32)
                    sm.list[base + k] = (uint16_t)((a << 12) | (tj * P.m + k));
            }
            continue;
        }
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
                if (active && blk == q) sm.list[base + __popc(mq & lt)] = (uint16_t)((a << 12) | s);
                __syncwarp();
                if (lane == 0) sm.off[a * kMaxTypes + q] = base + __popc(mq);
                __syncwarp();
            }
        }
    }
    __syncthreads();
}

// Environment row of one pair (dp_dp.py:241-297) for centre type ti.
struct EnvRow {
    float R, x, y, z, s, ds, inv, rh[4];
};

__device__ __forceinline__ void env_of(EnvRow &e, const float4 q4, float rmin, float rmax,
                                       const float *av, const float *isd) {
    e.R = q4.x; e.x = q4.y; e.y = q4.z; e.z = q4.w;
    switch_f(e.R, rmin, rmax, e.s, e.ds);
    e.inv = fabsf(e.R) > 1e-5f ? __frcp_rn(e.R) : 0.f;
    e.rh[0] = (e.s - av[0]) * isd[0];
    e.rh[1] = (e.s * e.x * e.inv - av[1]) * isd[1];
    e.rh[2] = (e.s * e.y * e.inv - av[2]) * isd[2];
    e.rh[3] = (e.s * e.z * e.inv - av[3]) * isd[3];
}

// ------------------------------------------------------------------ forward (A descriptor)
template <int SPLIT, bool FAST>
__global__ void __launch_bounds__(TM, 3)
dp_embed_fwd_tc(const int32_t *__restrict__ list_neigh, const float *__restrict__ idr,
                const int32_t *__restrict__ type_map, const float *__restrict__ params,
                const unsigned char *__restrict__ wtiles, const float *__restrict__ davg,
                const float *__restrict__ dstd, const float *__restrict__ pad,
                float *__restrict__ Aout, int32_t *__restrict__ err, MixParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t mbar_l, mbar_c;
    __shared__ uint32_t tmem_base;
    const int nt = P.ntypes, nnet = nt * nt, S = P.nslots;
    const MixSmem sm = carve(smem_raw, false, S, P.ga);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int q = tid; q < (2 * XT + RT) / 16; q += TM)       // xh, xl, rop are contiguous
        reinterpret_cast<uint4 *>(sm.xh)[q] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        tc::mbar_init(&mbar_l, 1);
        tc::mbar_init(&mbar_c, 1);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t lane_q = (uint32_t)(warp * 32) << 16;
    uint32_t ph_l = 0, ph_c = 0;
    bool pend_l = false, pend_c = false, ok = true;
    int cur_net = -1;
    int my_chunk = -1;                  // this thread's nonzero chunk of the contraction operand
    const long long total = (long long)P.batch * P.natoms;
    const long long ngroups = (total + P.ga - 1) / P.ga;
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long long g0 = grp * P.ga;
        const int ga = (int)(total - g0 < P.ga ? total - g0 : P.ga);
        build_group_list(sm, list_neigh, type_map, g0, ga, P);
        bool first = true;
        const int ntl = *sm.ntiles;
        // this thread's pair row of tile `it`, fetched one tile ahead of its use
        int a_n = 0;
        float4 q4_n = make_float4(0.f, 0.f, 0.f, 0.f);
        auto fetch = [&](int it) {
            const int tw = sm.tiles[it], k2 = tw >> 16, r = (tw & 0xFFFF) + tid;
            a_n = 0;
            q4_n = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < sm.net_start[k2 + 1]) {
                const int e = sm.list[r];
                a_n = e >> 12;
                q4_n = __ldg(reinterpret_cast<const float4 *>(idr) + (g0 + a_n) * S + (e & 0xFFF));
            }
        };
        if (ntl > 0) fetch(0);
        for (int it = 0; it < ntl; ++it) {
            const int k = sm.tiles[it] >> 16, r0 = sm.tiles[it] & 0xFFFF;
            const int ne = sm.net_start[k + 1];
            if (k != cur_net) {            // no MMA in flight reads the weight tiles here
                __syncthreads();
                load_net(wtiles, params, k, sm);
                cur_net = k;
                __syncthreads();
            }
            const int ti = k / nt;
            const float av[4] = {davg[4 * ti], davg[4 * ti + 1], davg[4 * ti + 2], davg[4 * ti + 3]};
            const float isd[4] = {1.f / dstd[4 * ti], 1.f / dstd[4 * ti + 1],
                                  1.f / dstd[4 * ti + 2], 1.f / dstd[4 * ti + 3]};
            const float4 *v4 = reinterpret_cast<const float4 *>(sm.vec);
            {
                const int nrows = ne - r0 < TM ? ne - r0 : TM;
                const bool valid = tid < nrows;
                const int a = a_n;
                const float4 q4 = q4_n;
                if (it + 1 < ntl) fetch(it + 1);
                EnvRow en;
                env_of(en, q4, P.rmin, P.rmax, av, isd);
                float x[E];
#pragma unroll
                for (int o4 = 0; o4 < 7; ++o4) {
                    const float4 w = v4[o4], b = v4[VW / 4 + o4];
                    const float wv[4] = {w.x, w.y, w.z, w.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (4 * o4 + q < E) x[4 * o4 + q] = act<FAST>(en.rh[0] * wv[q] + bv[q]);
                }
                // the previous tile's contraction still reads the tiles written below
                if (pend_c && !wait_commit(&mbar_c, ph_c, pend_c, P.wait_polls)) ok = false;
                store_row<SPLIT>(sm, tid, x, 1.f);
                {   // contraction operand: column tid holds this row's (R_h, R_l) at M = 8 a + 2 c + h
                    if (my_chunk >= 0)
                        *reinterpret_cast<uint4 *>(sm.rop + my_chunk) = make_uint4(0, 0, 0, 0);
                    my_chunk = -1;
                    if (valid) {
                        float rv[8];
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const float h = __bfloat162float(__float2bfloat16_rn(en.rh[c]));
                            rv[2 * c] = h;
                            rv[2 * c + 1] = SPLIT == 3 ? en.rh[c] - h : 0.f;
                        }
                        uint4 pk;
                        tc::split8(rv, pk, nullptr);
                        my_chunk = (int)mn_chunk(tid, a);
                        *reinterpret_cast<uint4 *>(sm.rop + my_chunk) = pk;
                    }
                }
                if (pre_issue(ok)) goto done;
                if (tid == 0) issue_layer<SPLIT>(sm, tmem, 0, false, &mbar_l);
                pend_l = true;
                if (!wait_commit(&mbar_l, ph_l, pend_l, P.wait_polls)) ok = false;
                {
                    float h[KP];
                    ld32_if(ok, tmem + lane_q, h);
#pragma unroll
                    for (int o4 = 0; o4 < 7; ++o4) {
                        const float4 d = v4[2 * VW / 4 + o4];
                        const float dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (4 * o4 + q < E) x[4 * o4 + q] += act<FAST>(h[4 * o4 + q]) * dv[q];
                    }
                }
                store_row<SPLIT>(sm, tid, x, 1.f);
                if (pre_issue(ok)) goto done;
                if (tid == 0) issue_layer<SPLIT>(sm, tmem, 1, false, &mbar_l);
                pend_l = true;
                if (!wait_commit(&mbar_l, ph_l, pend_l, P.wait_polls)) ok = false;
                {
                    float h[KP];
                    ld32_if(ok, tmem + lane_q, h);
#pragma unroll
                    for (int o4 = 0; o4 < 7; ++o4) {
                        const float4 d = v4[3 * VW / 4 + o4];
                        const float dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (4 * o4 + q < E) x[4 * o4 + q] += act<FAST>(h[4 * o4 + q]) * dv[q];
                    }
                }
                store_row<SPLIT>(sm, tid, x, 0.f);       // G, the B operand of the contraction
                if (pre_issue(ok)) goto done;
                if (tid == 0)
                    // N = 64: columns [0, 32) against the G hi tile, [32, 64) against the lo
                    // tile that follows it in shared memory
                    issue_rows<1, 128, SPLIT == 3 ? 2 * KP : KP>(tmem + TCOL_A, sm.rop, sm.xh,
                                                                nullptr, nullptr, first, &mbar_c);
                pend_c = true;
                first = false;
            }
        }
        // A of the group: D[8 a + 2 c + h][p] summed over h, + empty-slot term, / (m T)
        if (pend_c && !wait_commit(&mbar_c, ph_c, pend_c, P.wait_polls)) ok = false;
        if (__syncthreads_or(!ok)) goto done;
        {
            float d[KP];
            if (!first) {
                tc::tmem_ld32(tmem + TCOL_A + lane_q, d);
                if (SPLIT == 3) {
                    float dl[KP];
                    tc::tmem_ld32(tmem + TCOL_A + KP + lane_q, dl);
#pragma unroll
                    for (int p = 0; p < KP; ++p) d[p] += dl[p];
                }
            } else {
#pragma unroll
                for (int p = 0; p < KP; ++p) d[p] = 0.f;
            }
#pragma unroll
            for (int p = 0; p < E; ++p) d[p] += __shfl_xor_sync(0xffffffffu, d[p], 1);
            const int a = tid >> 3, c = (tid >> 1) & 3;
            if ((tid & 1) == 0 && a < ga) {
                const int ti = sm.tia[a];
                float *dst = Aout + (g0 + a) * NA + c * E;
                if (ti < 0) {
#pragma unroll
                    for (int p = 0; p < E; ++p) dst[p] = 0.f;
                } else {
                    for (int tj = 0; tj < nt; ++tj) {
                        if (!((P.present_mask >> tj) & 1)) continue;
                        const float nemp = (float)(P.m - sm.cnt[a * kMaxTypes + tj]);
                        const float *pp = pad + (ti * nt + tj) * NA + c * E;
#pragma unroll
                        for (int p = 0; p < E; ++p) d[p] += nemp * pp[p];
                    }
#pragma unroll
                    for (int p = 0; p < E; ++p) dst[p] = d[p] * P.inv_mT;
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
done:
    // drain: nothing this CTA issued may still run when its TMEM is freed
    if (pend_l) tc::mbar_wait(&mbar_l, ph_l, kDrainPolls);
    if (pend_c) tc::mbar_wait(&mbar_c, ph_c, kDrainPolls);
    if (!ok && (tid & 31) == 0) atomicMax(err, MATPL_KERR_TIMEOUT);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
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
    __shared__ __align__(8) uint64_t mbar_l, mbar_c;
    __shared__ uint32_t tmem_base;
    const int nt = P.ntypes, nnet = nt * nt, S = P.nslots;
    const MixSmem sm = carve(smem_raw, true, S, P.ga);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int q = tid; q < (2 * XT + ET + 3 * QT) / 16; q += TM)   // xh, xl, rop, qh, qm, ql
        reinterpret_cast<uint4 *>(sm.xh)[q] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        tc::mbar_init(&mbar_l, 1);
        tc::mbar_init(&mbar_c, 1);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t lane_q = (uint32_t)(warp * 32) << 16;
    uint32_t ph_l = 0, ph_c = 0;
    bool pend_l = false, pend_c = false, ok = true;
    int cur_net = -1;
    int my_chunk = -1;                  // this thread's nonzero chunk of the one-hot operand
    const int nall = P.natoms + P.nghost;
    const long long total = (long long)P.batch * P.natoms;
    const long long ngroups = (total + P.ga - 1) / P.ga;
    const float4 *dA4 = reinterpret_cast<const float4 *>(sm.dA);
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long long g0 = grp * P.ga;
        const int ga = (int)(total - g0 < P.ga ? total - g0 : P.ga);
        build_group_list(sm, list_neigh, type_map, g0, ga, P);
        for (int q = tid; q < GAMAX * E; q += TM) {          // dA[a][p][c] = dE/dA[c][p] k
            const int a = q / E, p = q - a * E;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (a < ga) {
                const float *s = dAin + (g0 + a) * NA + p;
                v = make_float4(s[0] * P.inv_mT, s[E] * P.inv_mT, s[2 * E] * P.inv_mT,
                                s[3 * E] * P.inv_mT);
            }
            reinterpret_cast<float4 *>(sm.dA)[q] = v;
        }
        __syncthreads();
        bool first = true;
        const int ntl = *sm.ntiles;
        // this thread's pair row of tile `it` (and its neighbor index), fetched one tile ahead
        int a_n = 0, j_n = -1;
        float4 q4_n = make_float4(0.f, 0.f, 0.f, 0.f);
        auto fetch = [&](int it) {
            const int tw = sm.tiles[it], k2 = tw >> 16, r = (tw & 0xFFFF) + tid;
            a_n = 0;
            j_n = -1;
            q4_n = make_float4(0.f, 0.f, 0.f, 0.f);
            if (r < sm.net_start[k2 + 1]) {
                const int e = sm.list[r];
                a_n = e >> 12;
                const long long row = (g0 + a_n) * S + (e & 0xFFF);
                q4_n = __ldg(reinterpret_cast<const float4 *>(idr) + row);
                j_n = __ldg(list_neigh + row) - 1;
            }
        };
        if (ntl > 0) fetch(0);
        for (int it = 0; it < ntl; ++it) {
            const int k = sm.tiles[it] >> 16, r0 = sm.tiles[it] & 0xFFFF;
            const int ne = sm.net_start[k + 1];
            if (k != cur_net) {
                __syncthreads();
                load_net(wtiles, params, k, sm);
                cur_net = k;
                __syncthreads();
            }
            const int ti = k / nt;
            const float av[4] = {davg[4 * ti], davg[4 * ti + 1], davg[4 * ti + 2], davg[4 * ti + 3]};
            const float isd[4] = {1.f / dstd[4 * ti], 1.f / dstd[4 * ti + 1],
                                  1.f / dstd[4 * ti + 2], 1.f / dstd[4 * ti + 3]};
            const float4 *v4 = reinterpret_cast<const float4 *>(sm.vec);
            {
                const int nrows = ne - r0 < TM ? ne - r0 : TM;
                const bool valid = tid < nrows;
                const int a = a_n, j = j_n;
                const long long t = g0 + a;
                const float4 q4 = q4_n;
                if (it + 1 < ntl) fetch(it + 1);
                EnvRow en;
                env_of(en, q4, P.rmin, P.rmax, av, isd);
                float x[E];
#pragma unroll
                for (int o4 = 0; o4 < 7; ++o4) {
                    const float4 w = v4[o4], b = v4[VW / 4 + o4];
                    const float wv[4] = {w.x, w.y, w.z, w.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (4 * o4 + q < E) x[4 * o4 + q] = act<FAST>(en.rh[0] * wv[q] + bv[q]);
                }
                store_row<SPLIT>(sm, tid, x, 1.f);
                if (pre_issue(ok)) goto done;
                if (tid == 0) issue_layer<SPLIT>(sm, tmem, 0, false, &mbar_l);
                pend_l = true;
                if (!wait_commit(&mbar_l, ph_l, pend_l, P.wait_polls)) ok = false;
                {
                    float h[KP];
                    ld32_if(ok, tmem + lane_q, h);
#pragma unroll
                    for (int o4 = 0; o4 < 7; ++o4) {
                        const float4 d = v4[2 * VW / 4 + o4];
                        const float dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int o = 4 * o4 + q;
                            if (o < E) {
                                h[o] = act<FAST>(h[o]);           // t2, stashed in TMEM
                                x[o] += h[o] * dv[q];
                            }
                        }
                    }
                    if (ok) tc::tmem_st32(tmem + TCOL_STASH + lane_q, h);
                }
                store_row<SPLIT>(sm, tid, x, 1.f);
                if (pre_issue(ok)) goto done;
                if (tid == 0) issue_layer<SPLIT>(sm, tmem, 1, false, &mbar_l);
                pend_l = true;
                if (!wait_commit(&mbar_l, ph_l, pend_l, P.wait_polls)) ok = false;
                float g[4] = {0.f, 0.f, 0.f, 0.f};
                {
                    // G = x + dt2 t3;  dE/dR[c] = sum_p dA[c][p] G[p];  dG[p] = sum_c dA[c][p] R[c];
                    // y = dG dt2 (1 - t3^2) feeds the transposed layer-3 GEMM
                    float h[KP];
                    ld32_if(ok, tmem + lane_q, h);
                    const float4 *da = dA4 + a * E;
#pragma unroll
                    for (int o4 = 0; o4 < 7; ++o4) {
                        const float4 d = v4[3 * VW / 4 + o4];
                        const float dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int o = 4 * o4 + q;
                            if (o < E) {
                                const float t3 = act<FAST>(h[o]);
                                const float G = x[o] + dv[q] * t3;
                                const float4 w = da[o];
                                g[0] += w.x * G; g[1] += w.y * G; g[2] += w.z * G; g[3] += w.w * G;
                                const float dG = w.x * en.rh[0] + w.y * en.rh[1] + w.z * en.rh[2] +
                                                 w.w * en.rh[3];
                                x[o] = dG;                               // x now holds dG
                                h[o] = dG * dv[q] * (1.f - t3 * t3);     // h now holds y
                            }
                        }
                    }
                    store_row<SPLIT>(sm, tid, h, 0.f);
                }
                if (pre_issue(ok)) goto done;
                if (tid == 0) issue_layer<SPLIT>(sm, tmem, 1, true, &mbar_l);
                pend_l = true;
                if (!wait_commit(&mbar_l, ph_l, pend_l, P.wait_polls)) ok = false;
                {
                    float h[KP], t2[KP];
                    ld32_if(ok, tmem + lane_q, h);
                    ld32_if(ok, tmem + TCOL_STASH + lane_q, t2);
#pragma unroll
                    for (int o4 = 0; o4 < 7; ++o4) {
                        const float4 d = v4[2 * VW / 4 + o4];
                        const float dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int o = 4 * o4 + q;
                            if (o < E) {
                                x[o] += h[o];                              // dx2
                                h[o] = x[o] * dv[q] * (1.f - t2[o] * t2[o]);
                            }
                        }
                    }
                    store_row<SPLIT>(sm, tid, h, 0.f);
                }
                if (pre_issue(ok)) goto done;
                if (tid == 0) issue_layer<SPLIT>(sm, tmem, 0, true, &mbar_l);
                pend_l = true;
                if (!wait_commit(&mbar_l, ph_l, pend_l, P.wait_polls)) ok = false;
                {
                    // dE/ds = sum_o W0[o] (dx2 + h)[o] (1 - t1^2), t1 recomputed
                    float h[KP];
                    ld32_if(ok, tmem + lane_q, h);
                    float dsv = 0.f;
#pragma unroll
                    for (int o4 = 0; o4 < 7; ++o4) {
                        const float4 w = v4[o4], b = v4[VW / 4 + o4];
                        const float wv[4] = {w.x, w.y, w.z, w.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int o = 4 * o4 + q;
                            if (o < E) {
                                const float t1 = act<FAST>(en.rh[0] * wv[q] + bv[q]);
                                dsv += wv[q] * (x[o] + h[o]) * (1.f - t1 * t1);
                            }
                        }
                    }
                    g[0] += dsv;
                }
                {
                    // f_a = sum_c g[c] Ri_d[c][a], Ri_d = -dfeat / dstd (dp_dp.py:266-299)
                    float f[3] = {0.f, 0.f, 0.f};
                    if (valid && fabsf(en.R) > 1e-5f) {
                        const float common = (en.ds - en.s * en.inv) * en.inv * en.inv;
                        const float g0 = g[0] * isd[0], g1 = g[1] * isd[1], g2 = g[2] * isd[2],
                                    g3 = g[3] * isd[3];
                        const float cg = common * (g1 * en.x + g2 * en.y + g3 * en.z);
                        const float sv = en.s * en.inv;
                        f[0] = -(g0 * en.ds * en.x * en.inv + cg * en.x + g1 * sv);
                        f[1] = -(g0 * en.ds * en.y * en.inv + cg * en.y + g2 * sv);
                        f[2] = -(g0 * en.ds * en.z * en.inv + cg * en.z + g3 * sv);
                    }
                    if (valid && j >= 0 && j < nall) {
                        const long long b = t / P.natoms;
                        float *dst = force + (b * nall + j) * 3;
                        atomicAdd(dst + 0, f[0]);
                        atomicAdd(dst + 1, f[1]);
                        atomicAdd(dst + 2, f[2]);
                    }
                    // the previous tile's reduction still reads the operands written below
                    if (pend_c && !wait_commit(&mbar_c, ph_c, pend_c, P.wait_polls)) ok = false;
                    const float qv[QN] = {f[0], f[1], f[2],
                                          f[0] * en.x, f[0] * en.y, f[0] * en.z,
                                          f[1] * en.x, f[1] * en.y, f[1] * en.z,
                                          f[2] * en.x, f[2] * en.y, f[2] * en.z, 0.f, 0.f, 0.f, 0.f};
                    // three BF16 parts (hi, mid, lo: 24 significant bits) so the per-atom sums
                    // keep FP32 accuracy
#pragma unroll
                    for (int gq = 0; gq < 2; ++gq) {
                        uint4 hq, mq;
                        float rem[8];
                        tc::split8(qv + 8 * gq, hq, SPLIT == 3 ? &mq : nullptr);
                        *reinterpret_cast<uint4 *>(sm.qh + mn_chunk(tid, gq)) = hq;
                        if (SPLIT == 3) {
                            const uint32_t hw[4] = {hq.x, hq.y, hq.z, hq.w};
                            const uint32_t mw[4] = {mq.x, mq.y, mq.z, mq.w};
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                const uint32_t hb = (hw[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
                                const uint32_t mb = (mw[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
                                rem[e] = qv[8 * gq + e] - __uint_as_float(hb << 16) -
                                         __uint_as_float(mb << 16);
                            }
                            uint4 lq;
                            tc::split8(rem, lq, nullptr);
                            *reinterpret_cast<uint4 *>(sm.qm + mn_chunk(tid, gq)) = mq;
                            *reinterpret_cast<uint4 *>(sm.ql + mn_chunk(tid, gq)) = lq;
                        }
                    }
                    // one-hot operand: column tid holds 1 at M = a
                    if (my_chunk >= 0)
                        *reinterpret_cast<uint4 *>(sm.rop + my_chunk) = make_uint4(0, 0, 0, 0);
                    my_chunk = -1;
                    if (valid) {
                        uint32_t w[4] = {0u, 0u, 0u, 0u};
                        w[(a & 7) >> 1] = 0x3F80u << (16 * (a & 1));   // bf16 1.0
                        my_chunk = (int)mn_chunk(tid, a >> 3);
                        *reinterpret_cast<uint4 *>(sm.rop + my_chunk) = make_uint4(w[0], w[1], w[2], w[3]);
                    }
                }
                if (pre_issue(ok)) goto done;
                if (tid == 0)
                    // N = 48: the hi, mid and lo tiles follow one another in shared memory
                    issue_rows<1, 64, SPLIT == 3 ? 3 * QN : QN>(tmem + TCOL_RED, sm.rop, sm.qh,
                                                               nullptr, nullptr, first, &mbar_c);
                pend_c = true;
                first = false;
            }
        }
        // F_i = -sum f and the per-atom virial of the group's atoms (TMEM rows 0..15)
        if (pend_c && !wait_commit(&mbar_c, ph_c, pend_c, P.wait_polls)) ok = false;
        if (__syncthreads_or(!ok)) goto done;
        if (warp == 0) {
            float d[QN];
            if (!first) {
                tc::tmem_ld16(tmem + TCOL_RED, d);
                if (SPLIT == 3) {
                    float dm[QN], dl[QN];
                    tc::tmem_ld16(tmem + TCOL_RED + QN, dm);
                    tc::tmem_ld16(tmem + TCOL_RED + 2 * QN, dl);
#pragma unroll
                    for (int q = 0; q < QN; ++q) d[q] += dm[q] + dl[q];
                }
            } else {
#pragma unroll
                for (int q = 0; q < QN; ++q) d[q] = 0.f;
            }
            const int a = tid;
            if (a < ga) {
                const long long t = g0 + a;
                double *av9 = atom_vir + t * 9;
#pragma unroll
                for (int q = 0; q < 9; ++q) av9[q] = (double)d[3 + q];
                if (sm.tia[a] >= 0) {
                    const long long b = t / P.natoms;
                    const int i = (int)(t - b * P.natoms);
                    float *dst = force + (b * nall + i) * 3;
                    atomicAdd(dst + 0, -d[0]);
                    atomicAdd(dst + 1, -d[1]);
                    atomicAdd(dst + 2, -d[2]);
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
done:
    if (pend_l) tc::mbar_wait(&mbar_l, ph_l, kDrainPolls);
    if (pend_c) tc::mbar_wait(&mbar_c, ph_c, kDrainPolls);
    if (!ok && (tid & 31) == 0) atomicMax(err, MATPL_KERR_TIMEOUT);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

}  // namespace

// Tuning of the mixed embedding kernels (matpl_dp_set_tuning): centre atoms per CTA group
// (how many pair rows feed each 128-row MMA tile) and resident CTAs per SM; 0 = automatic.
static std::atomic<int> g_ga_override{0}, g_ctas_override{0};
// Bound of every completion wait of the mixed embedding kernels (matpl_dp_set_wait_limit).
static std::atomic<int> g_wait_polls{1 << 24};

// Launch helpers used by dp_fused.cu's matpl_dp_eval for the MATPL_MIXED forms.
int mixed_ga(int S) {
    const int lim = std::max(1, std::min(GAMAX, 8192 / std::max(1, S)));
    const int o = g_ga_override.load();
    return o > 0 ? std::min(o, lim) : lim;
}

size_t mixed_smem(int ntypes, int S) {
    (void)ntypes;
    return std::max(mix_smem_bytes(false, S, mixed_ga(S)), mix_smem_bytes(true, S, mixed_ga(S)));
}

size_t mixed_tile_bytes(int ntypes) { return (size_t)ntypes * ntypes * 4 * WT; }

int prep_mixed_tiles(const float *params, unsigned char *out, int ntypes, cudaStream_t s) {
    const int n = ntypes * ntypes * 2 * KP * KP;
    ProfScope ps("prep_weight_tiles", s);
    prep_weight_tiles<<<(n + 255) / 256, 256, 0, s>>>(params, out, ntypes * ntypes);
    return check_launch("prep_weight_tiles");
}

template <int SPLIT, bool FAST>
int launch_mixed_embed(bool backward, const int32_t *list_neigh, const int32_t *num_neigh,
                       const float *idr, const int32_t *type_map, const float *params,
                       const unsigned char *wtiles, const float *davg, const float *dstd,
                       const float *pad_or_dA, float *A_or_force, double *atom_vir, int32_t *err,
                       int batch, int natoms, int nslots, int nghost, int ntypes, int m,
                       int present_mask, double rmin, double rmax, double inv_mT,
                       cudaStream_t s) {
    MixParams P;
    P.batch = batch; P.natoms = natoms; P.nslots = nslots; P.nghost = nghost;
    P.ntypes = ntypes; P.m = m; P.present_mask = present_mask; P.ga = mixed_ga(nslots);
    P.rmin = (float)rmin; P.rmax = (float)rmax; P.inv_mT = (float)inv_mT;
    P.wait_polls = g_wait_polls.load();
    P.num_neigh = num_neigh;
    const size_t smem = mix_smem_bytes(backward, nslots, P.ga);
    const long long total = (long long)batch * natoms;
    const long long ngroups = (total + P.ga - 1) / P.ga;
    // resident CTAs per SM: what shared memory and TMEM allow (128 columns per CTA, four);
    // the tuning hook may ask for fewer
    const int fit = (int)std::max<size_t>(1, (227 * 1024) / (smem + 1024));
    int per_sm = std::min(fit, backward ? 3 : 4);
    if (g_ctas_override.load() > 0) per_sm = std::min(per_sm, g_ctas_override.load());
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

#define MATPL_INSTANTIATE_MIXED(SPLIT, FAST)                                                   \
    template int launch_mixed_embed<SPLIT, FAST>(                                              \
        bool, const int32_t *, const int32_t *, const float *, const int32_t *, const float *, \
        const unsigned char *, const float *, const float *, const float *, float *, double *,  \
        int32_t *, int, int, int, int, int, int, int, double, double, double, cudaStream_t);
MATPL_INSTANTIATE_MIXED(1, true)
MATPL_INSTANTIATE_MIXED(3, false)
MATPL_INSTANTIATE_MIXED(3, true)
#undef MATPL_INSTANTIATE_MIXED

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

extern "C" int matpl_dp_set_wait_limit(int polls) {
    using namespace matpl;
    MATPL_REQUIRE(polls >= 0, MATPL_ERR_INVALID, "polls must be >= 0 (0: default)");
    g_wait_polls.store(polls == 0 ? (1 << 24) : polls);
    return MATPL_OK;
}
