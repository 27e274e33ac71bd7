// Tabulated ("compressed") embedding net: the drop-in for MatPL's CalcOps_cuda calculateCompress
// (src/op/src/CalcOps.cpp:331-383; kernels src/op/kernel/calculateCompress.cu:3-55 and
// calculateCompress_grad.cu:3-53).
//
//   G[s][i]   = polynomial of f2[s] with the coefficients coefficient[s][i][0..coe_num-1]
//               (highest power first; order 3 for coe_num = 4, order 5 for coe_num = 6)
//   grad_f2[s] = sum_i grad_G[s][i] * dG[s][i]/df2
//
// One warp per table row s, lanes over the output nodes i: a warp reads the row's contiguous
// layer_node * coe_num coefficients once (coalesced), and the backward reduces over i with warp
// shuffles instead of materialising dG/df2 [nsij, layer_node] the way the reference does.
#include "common.cuh"

namespace matpl {
namespace {

constexpr int kThreads = 256;

template <typename T, int NC>
__device__ __forceinline__ void poly(const T *c, T x, T &g, T &dg) {
    // Horner for the value and the derivative together
    g = c[0];
    dg = T(0);
#pragma unroll
    for (int k = 1; k < NC; ++k) {
        dg = dg * x + g;
        g = g * x + c[k];
    }
}

template <typename T, int NC>
__global__ void compress_fwd(const T *__restrict__ f2, const T *__restrict__ coef,
                             T *__restrict__ G, long long nsij, int nodes) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long s = w0; s < nsij; s += nw) {
        const T x = f2[s];
        for (int i = lane; i < nodes; i += 32) {
            const T *c = coef + (s * nodes + i) * NC;
            T cc[NC];
#pragma unroll
            for (int k = 0; k < NC; ++k) cc[k] = c[k];
            T g, dg;
            poly<T, NC>(cc, x, g, dg);
            G[s * nodes + i] = g;
        }
    }
}

template <typename T, int NC>
__global__ void compress_bwd(const T *__restrict__ f2, const T *__restrict__ coef,
                             const T *__restrict__ gG, T *__restrict__ gf2, long long nsij,
                             int nodes) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long s = w0; s < nsij; s += nw) {
        const T x = f2[s];
        T acc = T(0);
        for (int i = lane; i < nodes; i += 32) {
            const T *c = coef + (s * nodes + i) * NC;
            T cc[NC];
#pragma unroll
            for (int k = 0; k < NC; ++k) cc[k] = c[k];
            T g, dg;
            poly<T, NC>(cc, x, g, dg);
            acc += gG[s * nodes + i] * dg;
        }
        acc = warp_sum(acc);
        if (lane == 0) gf2[s] = acc;
    }
}

inline int grid_for_rows(long long nsij) {
    long long g = (nsij * 32 + kThreads - 1) / kThreads;
    if (g > (long long)device_sms() * 16) g = (long long)device_sms() * 16;
    return (int)(g < 1 ? 1 : g);
}

template <typename T>
int launch(bool backward, const void *f2, const void *coef, const void *gG, long long nsij,
           int nodes, int coe_num, void *out, cudaStream_t s) {
    const int grid = grid_for_rows(nsij);
    ProfScope ps(backward ? "compress_bwd" : "compress_fwd", s);
    if (coe_num == 4) {
        if (backward)
            compress_bwd<T, 4><<<grid, kThreads, 0, s>>>((const T *)f2, (const T *)coef,
                                                         (const T *)gG, (T *)out, nsij, nodes);
        else
            compress_fwd<T, 4><<<grid, kThreads, 0, s>>>((const T *)f2, (const T *)coef, (T *)out,
                                                         nsij, nodes);
    } else {
        if (backward)
            compress_bwd<T, 6><<<grid, kThreads, 0, s>>>((const T *)f2, (const T *)coef,
                                                         (const T *)gG, (T *)out, nsij, nodes);
        else
            compress_fwd<T, 6><<<grid, kThreads, 0, s>>>((const T *)f2, (const T *)coef, (T *)out,
                                                         nsij, nodes);
    }
    return check_launch(backward ? "matpl_calc_compress_grad" : "matpl_calc_compress");
}

int check_args(int dtype, long long nsij, int nodes, int coe_num) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "calculateCompress supports f32 and f64");
    MATPL_REQUIRE(nsij >= 0 && nodes >= 0, MATPL_ERR_INVALID, "negative size");
    MATPL_REQUIRE(coe_num == 4 || coe_num == 6, MATPL_ERR_UNSUPPORTED,
                  "coefficient last dimension must be 4 (order 3) or 6 (order 5)");
    return MATPL_OK;
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" int matpl_calc_compress(int dtype, const void *f2, const void *coefficient,
                                   long long nsij, int layer_node, int coe_num, void *G,
                                   void *stream) {
    int st = check_args(dtype, nsij, layer_node, coe_num);
    if (st) return st;
    if (nsij == 0 || layer_node == 0) return MATPL_OK;
    MATPL_REQUIRE(f2 && coefficient && G, MATPL_ERR_INVALID,
                  "matpl_calc_compress: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(G, "matpl_calc_compress");
    return dtype == MATPL_F64
               ? launch<double>(false, f2, coefficient, nullptr, nsij, layer_node, coe_num, G,
                                as_stream(stream))
               : launch<float>(false, f2, coefficient, nullptr, nsij, layer_node, coe_num, G,
                               as_stream(stream));
}

extern "C" int matpl_calc_compress_grad(int dtype, const void *f2, const void *coefficient,
                                        const void *grad_G, long long nsij, int layer_node,
                                        int coe_num, void *grad_f2, void *stream) {
    int st = check_args(dtype, nsij, layer_node, coe_num);
    if (st) return st;
    if (nsij == 0) return MATPL_OK;
    MATPL_REQUIRE(f2 && grad_f2 && (layer_node == 0 || (coefficient && grad_G)), MATPL_ERR_INVALID,
                  "matpl_calc_compress_grad: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(grad_f2, "matpl_calc_compress_grad");
    return dtype == MATPL_F64
               ? launch<double>(true, f2, coefficient, grad_G, nsij, layer_node, coe_num, grad_f2,
                                as_stream(stream))
               : launch<float>(true, f2, coefficient, grad_G, nsij, layer_node, coe_num, grad_f2,
                               as_stream(stream));
}
