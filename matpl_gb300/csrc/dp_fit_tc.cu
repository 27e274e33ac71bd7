// Mixed-precision DP fitting net (and its adjoint) on the tcgen05 tensor cores.
//
// Same math as dp_fused.cu's dp_fit (src/model/dp_embedding.py:140-163 and dp_dp.py:304-342 plus
// the autograd adjoint down to dE/dA): per atom D = A^T A[:, :16] (400), Ei = fit(D), dE/dA.
// Atoms are first sorted by element (fit_order, a stable counting sort), so that a CTA of 128
// threads owns a tile of 128 atoms of one element (thread r = atom r, MMA M = 128) and runs
// that element's net only:
//
//   layer 1  h1 = D W0: 13 K-chunks of 32; each chunk of D is built on the SIMT cores from the
//            atom's A (kept in shared memory) and double-buffered into the MMA (N = 64, the 50
//            outputs padded), FP32 accumulator in 64 TMEM columns.
//   layers 2, 3 (50 x 50 padded to 64 x 64) and the two transposed GEMMs of the adjoint run as
//            single MMAs (K = 64); tanh / residual / bias on SIMT; the three layers' tanh
//            outputs are stashed in TMEM (tcgen05.st) for the adjoint.
//   dE/dD = g1 W0^T (N = 400) in 7 chunks of 64 columns, each consumed straight from TMEM into
//            dE/dA = sum_q dD[p][q] A[c][q] + sum_p' dD[p'][p] A[c][p'].
// BF16x3 (hi/lo split) operands keep FP32-level accuracy; weight tiles are prepared once per
// call in global memory (prep_fit_tiles).  Every mbarrier wait is bounded (MATPL_KERR_TIMEOUT).
#include "common.cuh"
#include "dp_layout.cuh"
#include "tc.cuh"

namespace matpl {
namespace {

using namespace dp;
constexpr int FM = 128;                   // atoms per tile = threads
constexpr int FN = 64;                    // padded fitting width
constexpr int K1C = 13;                   // K chunks of layer 1 (32 each; 400 padded to 416)
constexpr int NDC = 7;                    // N chunks of dE/dD (64 each; 400 padded to 448)
constexpr int XKS = FM / 8 * 128;         // K-chunk stride of a 128-row activation tile (2048 B)
constexpr int BKS = FN / 8 * 128;         // K-chunk stride of a 64-row weight tile (1024 B)
constexpr int X32 = FM * 32 * 2;          // 128 x 32 bf16 tile (8 KB)
constexpr int X64 = FM * 64 * 2;          // 128 x 64 bf16 tile (16 KB)
constexpr int W32 = FN * 32 * 2;          // 64 x 32 bf16 weight tile (4 KB)
constexpr int W64 = FN * 64 * 2;          // 64 x 64 bf16 weight tile (8 KB)
constexpr int ASTR = NA + 1;              // A row stride in shared memory (floats)
constexpr int kWait = 1 << 24;

// Per-net tile offsets in the prepared buffer (each entry is a hi tile followed by a lo tile).
constexpr size_t OFF_F0 = 0;                                  // [13] 64 x 32: B[n=o][k] = W0[32c+k][o]
constexpr size_t OFF_F1 = OFF_F0 + (size_t)K1C * 2 * W32;     // 64 x 64: B[n=o][k=i] = W1[i][o]
constexpr size_t OFF_F2 = OFF_F1 + 2 * W64;                   // W2 likewise
constexpr size_t OFF_B2 = OFF_F2 + 2 * W64;                   // B[n=i][k=o] = W2[i][o]
constexpr size_t OFF_B1 = OFF_B2 + 2 * W64;                   // B[n=i][k=o] = W1[i][o]
constexpr size_t OFF_B0 = OFF_B1 + 2 * W64;                   // [7] 64 x 64: B[n=kD][k=o] = W0[64c+n][o]
constexpr size_t FIT_TILE_BYTES = OFF_B0 + (size_t)NDC * 2 * W64;

__device__ __forceinline__ void put_hilo(unsigned char *hi, unsigned char *lo, uint32_t off,
                                         float v) {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    *reinterpret_cast<__nv_bfloat16 *>(hi + off) = h;
    *reinterpret_cast<__nv_bfloat16 *>(lo + off) = __float2bfloat16_rn(v - __bfloat162float(h));
}

__global__ void prep_fit_tiles(const float *__restrict__ params, unsigned char *__restrict__ out,
                               int ntypes) {
    const long long woff = (long long)ntypes * ntypes * EmbOff::SIZE;
    // work items: per net, (13 + 7) chunks x 64 x 64 elements + 4 matrices x 64 x 64
    const int per_net = (K1C * 32 + NDC * 64 + 4 * 64) * FN;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
         q < (long long)ntypes * per_net; q += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(q / per_net);
        int r = (int)(q - (long long)t * per_net);
        const float *fw = params + woff + (long long)t * FitOff::SIZE;
        unsigned char *base = out + (size_t)t * FIT_TILE_BYTES;
        const int n = r % FN;                 // weight-tile row
        int k = r / FN;                       // running K index over all tiles of the net
        if (k < K1C * 32) {                   // layer-1 chunks (K = 32 each)
            const int c = k / 32, kk = k % 32, kD = 32 * c + kk;
            const float v = (kD < DIN && n < F) ? fw[FitOff::W0 + kD * F + n] : 0.f;
            unsigned char *hi = base + OFF_F0 + (size_t)c * 2 * W32;
            put_hilo(hi, hi + W32, tc::tile_off(n, kk, BKS), v);
            continue;
        }
        k -= K1C * 32;
        if (k < 4 * 64) {                     // the four 64 x 64 hidden-layer tiles
            const int mat = k / 64, kk = k % 64;
            float v = 0.f;
            if (n < F && kk < F) {
                switch (mat) {
                    case 0: v = fw[FitOff::W1 + kk * F + n]; break;   // F1: W1[i=kk][o=n]
                    case 1: v = fw[FitOff::W2 + kk * F + n]; break;   // F2
                    case 2: v = fw[FitOff::W2 + n * F + kk]; break;   // B2: W2[i=n][o=kk]
                    default: v = fw[FitOff::W1 + n * F + kk]; break;  // B1
                }
            }
            const size_t offs[4] = {OFF_F1, OFF_F2, OFF_B2, OFF_B1};
            unsigned char *hi = base + offs[mat];
            put_hilo(hi, hi + W64, tc::tile_off(n, kk, BKS), v);
            continue;
        }
        k -= 4 * 64;                          // dE/dD chunks: N = 64 rows of D index, K = o
        const int c = k / 64, kk = k % 64, kD = 64 * c + n;
        const float v = (kD < DIN && kk < F) ? fw[FitOff::W0 + kD * F + kk] : 0.f;
        unsigned char *hi = base + OFF_B0 + (size_t)c * 2 * W64;
        put_hilo(hi, hi + W64, tc::tile_off(n, kk, BKS), v);
    }
}

// Asynchronous 16-byte global -> shared copies (cp.async), waited for with cp_async_wait_all.
__device__ __forceinline__ void copy_tiles_async(const unsigned char *__restrict__ src,
                                                 unsigned char *dst, int bytes) {
    for (int q = threadIdx.x; q < bytes / 16; q += blockDim.x)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(dst + 16 * q)),
                     "l"(src + 16 * q)
                     : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void copy_tiles(const unsigned char *__restrict__ src, unsigned char *dst,
                                           int bytes) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int q = threadIdx.x; q < bytes / 16; q += blockDim.x) d4[q] = __ldg(s4 + q);
}

// Row r of a 128-row K-major tile: NK values as BF16 hi and lo halves.
template <int NK>
__device__ __forceinline__ void store_row_hilo(unsigned char *hi, unsigned char *lo, int r,
                                               const float *v) {
#pragma unroll
    for (int c = 0; c < NK / 8; ++c) {
        float h[8], l[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            h[q] = v[8 * c + q];
            l[q] = v[8 * c + q] - __bfloat162float(__float2bfloat16_rn(v[8 * c + q]));
        }
        tc::store_row8(hi, r, c, XKS, h);
        tc::store_row8(lo, r, c, XKS, l);
    }
}

// Shared memory written by the threads becomes visible to the tensor core, and prior TMEM
// reads are ordered before the next MMA.
__device__ __forceinline__ void mma_sync_point() {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// D[128 x 64] (+)= X W with BF16x3 operands; KCH K-steps of 16.
template <int KCH>
__device__ __forceinline__ void issue_split3(uint32_t tmem, const unsigned char *xh,
                                             const unsigned char *xl, const unsigned char *wh,
                                             const unsigned char *wl, bool accumulate) {
    const uint32_t id = tc::idesc_bf16(FM, FN);
    const uint32_t a[2] = {tc::smem_u32(xh), tc::smem_u32(xl)};
    const uint32_t b[2] = {tc::smem_u32(wh), tc::smem_u32(wl)};
    uint32_t acc = accumulate ? 1u : 0u;
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const uint32_t xa = a[p == 2 ? 1 : 0], wb = b[p == 1 ? 1 : 0];
#pragma unroll
        for (int kk = 0; kk < KCH; ++kk) {
            tc::mma_bf16(tmem, tc::desc_kmajor(xa + kk * 2 * XKS, XKS, 128),
                         tc::desc_kmajor(wb + kk * 2 * BKS, BKS, 128), id, acc);
            acc = 1u;
        }
    }
}

__device__ __forceinline__ void ld64(uint32_t tmem, float v[64]) {
    const uint32_t base = tmem + ((uint32_t)((threadIdx.x >> 5) * 32) << 16);
    tc::tmem_ld32(base, v);
    tc::tmem_ld32(base + 32, v + 32);
}

template <bool FAST>
__device__ __forceinline__ float fit_act(float x) {
    if (FAST) return tc::tanh_fast(x);
    return tanhf(x);
}

constexpr size_t FIT_SMEM = sizeof(float) * (FM * ASTR) + 2 * X64 + 2 * W64;
constexpr int FIT_TCOLS = 256;   // TMEM: [0, 64) accumulator, [64 + 64 l, 128 + 64 l) tanh of layer l

// Stable counting sort of the atoms of one image by model type into order[natoms], with
// type_start[0..ntypes+1] (bucket ntypes: atoms whose type is not evaluated), in two launches
// over 1024-atom blocks: per-block bucket counts, then per-block offsets (previous blocks'
// counts) and the ranks inside the block (warp match + a prefix over the block's warps).
constexpr int kOrderBlock = 1024;

__device__ __forceinline__ int fit_bucket(const int32_t *__restrict__ type_map, int i, int ntypes,
                                          int present_mask) {
    const int t = type_map[i];
    return (t >= 0 && t < ntypes && ((present_mask >> t) & 1)) ? t : ntypes;
}

__global__ void fit_order_count(const int32_t *__restrict__ type_map, int natoms, int ntypes,
                                int present_mask, int *__restrict__ blk_count) {
    __shared__ int cnt[17];
    if (threadIdx.x < 17) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * kOrderBlock + threadIdx.x;
    if (i < natoms) atomicAdd(&cnt[fit_bucket(type_map, i, ntypes, present_mask)], 1);
    __syncthreads();
    if (threadIdx.x <= ntypes) blk_count[blockIdx.x * 17 + threadIdx.x] = cnt[threadIdx.x];
}

__global__ void fit_order_scatter(const int32_t *__restrict__ type_map, int natoms, int ntypes,
                                  int present_mask, const int *__restrict__ blk_count,
                                  int *__restrict__ order, int *__restrict__ type_start) {
    __shared__ int base[17];                   // global start of this block's atoms per bucket
    __shared__ int wcnt[kOrderBlock / 32][17];
    __shared__ int before_s[17], total_s[17];  // per bucket: earlier blocks' atoms, all atoms
    const int T = ntypes + 1, nblk = gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // every block's bucket counts, summed by one warp per bucket (lanes over blocks, then a
    // shuffle tree), instead of one thread walking them serially
    for (int q = warp; q < T; q += kOrderBlock / 32) {
        int bef = 0, tot = 0;
        for (int b = lane; b < nblk; b += 32) {
            const int v = blk_count[b * 17 + q];
            tot += v;
            if (b < (int)blockIdx.x) bef += v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            bef += __shfl_xor_sync(0xffffffffu, bef, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if (lane == 0) {
            before_s[q] = bef;
            total_s[q] = tot;
        }
    }
    __syncthreads();
    if (threadIdx.x < T) {
        const int q = threadIdx.x;
        int total_lower = 0;
        for (int p = 0; p < q; ++p) total_lower += total_s[p];
        base[q] = total_lower + before_s[q];
        if (blockIdx.x == 0) type_start[q] = total_lower;
        if (blockIdx.x == 0 && q == T - 1) type_start[T] = natoms;
    }
    const int i = blockIdx.x * kOrderBlock + threadIdx.x;
    const int q = i < natoms ? fit_bucket(type_map, i, ntypes, present_mask) : 17;
    const unsigned peers = __match_any_sync(0xffffffffu, q);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (lane < 17) wcnt[warp][lane] = 0;
    __syncwarp();
    if (q < 17 && rank == 0) wcnt[warp][q] = __popc(peers);
    __syncthreads();
    if (q < 17) {
        int off = base[q] + rank;
        for (int w = 0; w < warp; ++w) off += wcnt[w][q];
        order[off] = i;
    }
}

__device__ __forceinline__ void st64(uint32_t taddr, const float v[64]) {
    tc::tmem_st32(taddr, v);
    tc::tmem_st32(taddr + 32, v + 32);
}

template <bool FAST>
__global__ void __launch_bounds__(FM, 2)
dp_fit_tc(const float *__restrict__ Ain, const int *__restrict__ order,
          const int *__restrict__ type_start, const float *__restrict__ params,
          const unsigned char *__restrict__ ftiles, float *__restrict__ Ei,
          float *__restrict__ dAout, int32_t *__restrict__ err, int batch, int natoms,
          int ntypes) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    __shared__ long long ratom[FM];
    __shared__ float vec[6 * FN + 4];
    float *As = reinterpret_cast<float *>(smem_raw);
    unsigned char *XB = reinterpret_cast<unsigned char *>(As + FM * ASTR);
    unsigned char *WB = XB + 2 * X64;
    const int r = threadIdx.x, warp = r >> 5;
    if (r == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, FIT_TCOLS);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t lane_q = (uint32_t)(warp * 32) << 16;
    uint32_t ph[2] = {0u, 0u};
    bool ok = true;
    const long long woff = (long long)ntypes * ntypes * EmbOff::SIZE;
    const int vsrc[6] = {FitOff::B0, FitOff::B1, FitOff::DT1, FitOff::B2, FitOff::DT2, FitOff::W3};
    // tiles: per image, ceil(n_t / 128) tiles of each element t (an upper bound of their number
    // per image is ceil(natoms / 128) + ntypes; the surplus indices have no work)
    const long long tiles_b = (natoms + FM - 1) / FM + ntypes;
    for (long long v = blockIdx.x; v < (long long)batch * tiles_b; v += gridDim.x) {
        const long long b = v / tiles_b;
        int rem = (int)(v - b * tiles_b), tt = -1, chunk = 0;
        for (int q = 0; q < ntypes; ++q) {
            const int nq = (type_start[q + 1] - type_start[q] + FM - 1) / FM;
            if (rem < nq) {
                tt = q;
                chunk = rem;
                break;
            }
            rem -= nq;
        }
        if (tt < 0) continue;                      // the same for every thread of the CTA
        const int idx = type_start[tt] + chunk * FM + r;
        const bool valid = idx < type_start[tt + 1];
        const long long t = valid ? b * natoms + order[idx] : -1;
        __syncthreads();
        ratom[r] = t;
        __syncthreads();
        for (int q = r; q < FM * NA; q += FM) {
            const int row = q / NA, e = q - row * NA;
            const long long tr = ratom[row];
            As[row * ASTR + e] = tr >= 0 ? Ain[tr * NA + e] : 0.f;
        }
        __syncthreads();
        const float *a = As + r * ASTR;
        {
            const float *fw = params + woff + (long long)tt * FitOff::SIZE;
            const unsigned char *tw = ftiles + (size_t)tt * FIT_TILE_BYTES;
            __syncthreads();
            for (int q = r; q < 6 * FN; q += FM) {
                const int part = q / FN, o = q - part * FN;
                vec[q] = o < F ? fw[vsrc[part] + o] : 0.f;
            }
            if (r == 0) vec[6 * FN] = fw[FitOff::B3];
            __syncthreads();
            const bool mine = valid;
            // ---- layer 1: 13 double-buffered K chunks of D W0.  The weights of chunk c + 1
            // are copied asynchronously while chunk c is formed and multiplied; buffer b of
            // chunk c is free once the MMA of chunk c - 2 is done (waited at the end of the
            // previous chunk, before that chunk's prefetch).
            float aq[4][M2];                      // A[c][q], q < M2: every chunk's right factor
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
                for (int q = 0; q < M2; ++q) aq[c4][q] = a[c4 * E + q];
            copy_tiles_async(tw + OFF_F0, WB, 2 * W32);
            for (int c = 0; c < K1C; ++c) {
                const int b = c & 1;
                float d[32];
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    const int p = 2 * c + h2;
                    const float ap0 = p < E ? a[p] : 0.f, ap1 = p < E ? a[E + p] : 0.f,
                                ap2 = p < E ? a[2 * E + p] : 0.f, ap3 = p < E ? a[3 * E + p] : 0.f;
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int k = 32 * c + 16 * h2 + q;
                        d[16 * h2 + q] = k < DIN ? ap0 * aq[0][q] + ap1 * aq[1][q] +
                                                       ap2 * aq[2][q] + ap3 * aq[3][q]
                                                 : 0.f;
                    }
                }
                unsigned char *xh = XB + b * 2 * X32;
                store_row_hilo<32>(xh, xh + X32, r, d);
                cp_async_wait_all();
                mma_sync_point();
                if (r == 0) {
                    issue_split3<2>(tmem, xh, xh + X32, WB + b * 2 * W32, WB + b * 2 * W32 + W32, c > 0);
                    tc::commit(&mbar[b]);
                }
                if (c + 1 < K1C) {
                    if (c >= 1) {                     // the MMA of chunk c - 1 read buffer b ^ 1
                        ok &= tc::mbar_wait(&mbar[b ^ 1], ph[b ^ 1], kWait);
                        ph[b ^ 1] ^= 1u;
                    }
                    copy_tiles_async(tw + OFF_F0 + (size_t)(c + 1) * 2 * W32,
                                     WB + (b ^ 1) * 2 * W32, 2 * W32);
                }
            }
            ok &= tc::mbar_wait(&mbar[1], ph[1], kWait);
            ph[1] ^= 1u;
            ok &= tc::mbar_wait(&mbar[0], ph[0], kWait);
            ph[0] ^= 1u;
            tc::fence_after_sync();
            float h[64], x[64];
            ld64(tmem, h);
#pragma unroll
            for (int o = 0; o < 64; ++o) x[o] = o < F ? fit_act<FAST>(h[o] + vec[o]) : 0.f;
            st64(tmem + 64 + lane_q, x);
            // ---- layers 2, 3
#pragma unroll 1
            for (int l = 1; l <= 2; ++l) {
                store_row_hilo<64>(XB, XB + X64, r, x);
                copy_tiles(tw + (l == 1 ? OFF_F1 : OFF_F2), WB, 2 * W64);
                mma_sync_point();
                if (r == 0) {
                    issue_split3<4>(tmem, XB, XB + X64, WB, WB + W64, false);
                    tc::commit(&mbar[0]);
                }
                ok &= tc::mbar_wait(&mbar[0], ph[0], kWait);
                ph[0] ^= 1u;
                tc::fence_after_sync();
                ld64(tmem, h);
                const float *bias = vec + (l == 1 ? FN : 3 * FN);
                const float *dt = vec + (l == 1 ? 2 * FN : 4 * FN);
#pragma unroll
                for (int o = 0; o < 64; ++o) {
                    h[o] = o < F ? fit_act<FAST>(h[o] + bias[o]) : 0.f;
                    if (o < F) x[o] = h[o] * dt[o] + x[o];
                }
                st64(tmem + 64 + 64 * l + lane_q, h);
            }
            float e = vec[6 * FN];
#pragma unroll
            for (int o = 0; o < F; ++o) e += x[o] * vec[5 * FN + o];
            if (mine) Ei[t] = e;
            // ---- adjoint: dx3 = W3; through layers 3 and 2
#pragma unroll
            for (int o = 0; o < F; ++o) x[o] = vec[5 * FN + o];
#pragma unroll 1
            for (int l = 2; l >= 1; --l) {
                const float *dt = vec + (l == 2 ? 4 * FN : 2 * FN);
                ld64(tmem + 64 + 64 * l, h);          // tanh outputs of layer l
#pragma unroll
                for (int o = 0; o < 64; ++o) h[o] = o < F ? x[o] * dt[o] * (1.f - h[o] * h[o]) : 0.f;
                store_row_hilo<64>(XB, XB + X64, r, h);
                copy_tiles(tw + (l == 2 ? OFF_B2 : OFF_B1), WB, 2 * W64);
                mma_sync_point();
                if (r == 0) {
                    issue_split3<4>(tmem, XB, XB + X64, WB, WB + W64, false);
                    tc::commit(&mbar[0]);
                }
                ok &= tc::mbar_wait(&mbar[0], ph[0], kWait);
                ph[0] ^= 1u;
                tc::fence_after_sync();
                ld64(tmem, h);
#pragma unroll
                for (int o = 0; o < F; ++o) x[o] += h[o];
            }
            ld64(tmem + 64, h);                       // tanh outputs of layer 1
#pragma unroll
            for (int o = 0; o < 64; ++o) h[o] = o < F ? x[o] * (1.f - h[o] * h[o]) : 0.f;
            store_row_hilo<64>(XB, XB + X64, r, h);
            // ---- dE/dD = g1 W0^T in 7 chunks of 64 D entries, folded into dE/dA
            float acc2[4][16];
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
                for (int q = 0; q < 16; ++q) acc2[c4][q] = 0.f;
#pragma unroll 1
            for (int c = 0; c < NDC; ++c) {
                copy_tiles(tw + OFF_B0 + (size_t)c * 2 * W64, WB, 2 * W64);
                mma_sync_point();
                if (r == 0) {
                    issue_split3<4>(tmem, XB, XB + X64, WB, WB + W64, false);
                    tc::commit(&mbar[0]);
                }
                ok &= tc::mbar_wait(&mbar[0], ph[0], kWait);
                ph[0] ^= 1u;
                tc::fence_after_sync();
                ld64(tmem, h);                        // h[n] = dE/dD[64c + n]
#pragma unroll
                for (int c4 = 0; c4 < 4; ++c4) {
                    float ap[4], sj[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int j = 0; j < 4; ++j) ap[j] = 4 * c + j < E ? a[c4 * E + 4 * c + j] : 0.f;
#pragma unroll
                    for (int q = 0; q < M2; ++q) {
                        const float aqv = a[c4 * E + q];
                        float acc = acc2[c4][q];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            if (4 * c + j >= E) break;
                            sj[j] += h[16 * j + q] * aqv;
                            acc += h[16 * j + q] * ap[j];
                        }
                        acc2[c4][q] = acc;
                    }
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (mine && 4 * c + j < E) dAout[t * NA + c4 * E + 4 * c + j] = sj[j];
                }
            }
            if (mine) {
#pragma unroll
                for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
                    for (int q = 0; q < M2; ++q) dAout[t * NA + c4 * E + q] += acc2[c4][q];
            }
        }
    }
    // atoms whose element is not evaluated: Ei = 0, dE/dA = 0
    const int nskip = type_start[ntypes + 1] - type_start[ntypes];
    for (long long q = (long long)blockIdx.x * FM + r; q < (long long)batch * nskip;
         q += (long long)gridDim.x * FM) {
        const long long b = q / nskip;
        const long long t = b * natoms + order[type_start[ntypes] + (int)(q - b * nskip)];
        Ei[t] = 0.f;
        for (int e = 0; e < NA; ++e) dAout[t * NA + e] = 0.f;
    }
    if (!ok) atomicMax(err, MATPL_KERR_TIMEOUT);
    // nothing issued may still run when the TMEM is freed: one more commit after all of this
    // thread's MMAs, waited for (bounded) by every thread
    __shared__ __align__(8) uint64_t mbar_drain;
    if (r == 0) {
        tc::mbar_init(&mbar_drain, 1);
        tc::commit(&mbar_drain);
    }
    __syncthreads();
    tc::mbar_wait(&mbar_drain, 0u, kWait);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, FIT_TCOLS);
}

}  // namespace

// Prepared tiles of every element, then the element order of the atoms (order [natoms],
// type_start [ntypes + 2], per-block bucket counts of the sort).
size_t fit_tile_bytes(int ntypes, int natoms) {
    const size_t nblk = ((size_t)natoms + kOrderBlock - 1) / kOrderBlock;
    return align_up((size_t)ntypes * FIT_TILE_BYTES, 256) + align_up(sizeof(int) * natoms, 256) +
           sizeof(int) * (32 + 17 * nblk);
}

// Prepares the BF16 fitting tiles of every type into `tiles`, then runs the fitting kernel.
int launch_fit_tc(bool fast, const float *A, const int32_t *type_map, const float *params,
                  unsigned char *tiles, float *Ei, float *dA, int32_t *err, int batch, int natoms,
                  int ntypes, int present_mask, cudaStream_t s) {
    {
        ProfScope ps("prep_fit_tiles", s);
        const long long n = (long long)ntypes * (K1C * 32 + NDC * 64 + 4 * 64) * FN;
        prep_fit_tiles<<<(int)((n + 255) / 256), 256, 0, s>>>(params, tiles, ntypes);
    }
    int *order = reinterpret_cast<int *>(tiles + align_up((size_t)ntypes * FIT_TILE_BYTES, 256));
    int *type_start = order + align_up(sizeof(int) * natoms, 256) / sizeof(int);
    int *blk_count = type_start + 32;
    const int nblk = (natoms + kOrderBlock - 1) / kOrderBlock;
    if (nblk > 0) {
        ProfScope ps("fit_order", s);
        fit_order_count<<<nblk, kOrderBlock, 0, s>>>(type_map, natoms, ntypes, present_mask,
                                                    blk_count);
        fit_order_scatter<<<nblk, kOrderBlock, 0, s>>>(type_map, natoms, ntypes, present_mask,
                                                      blk_count, order, type_start);
    }
    const long long tiles_b = (natoms + FM - 1) / FM + ntypes;
    const long long ntiles = (long long)batch * tiles_b;
    const long long cap = 2LL * device_sms();            // two resident CTAs per SM
    const int grid = (int)(ntiles < cap ? ntiles : cap);
    auto k = fast ? dp_fit_tc<true> : dp_fit_tc<false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FIT_SMEM);
    ProfScope ps("dp_fit_tc", s);
    k<<<grid, FM, FIT_SMEM, s>>>(A, order, type_start, params, tiles, Ei, dA, err, batch, natoms,
                                 ntypes);
    return check_launch("dp_fit_tc");
}

}  // namespace matpl
