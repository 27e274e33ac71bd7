// DP neighbor search and environment matrix.
//
// Semantics: src/pre_data/gen_feature/NeighConst.f90:14-149 (find_neighbore), applied to
// each image on its own (MatPL's loader always calls it with images = 1,
// dpuni_data_loader.py:619), then the r column of compute_Ri (dpuni_data_loader.py:669-673).
//
//  * Per-type slot blocks of m slots, filled in ascending neighbor index j and, for small
//    cells (any |a_v| < 2 Rc), in the Fortran image order (i1, i2, i3) inside each j.
//  * Cells with all |a_v| >= 2 Rc use the per-component nearest-image rule of
//    NeighConst.f90:98-108.  Candidates come from a cell list whose bins (in fractional
//    coordinates) are at least Rc/h_k wide (h_k = cell thickness along reciprocal direction
//    k), so every pair within Rc under that rule sits in one of the 27 (or fewer, distinct)
//    adjacent bins.  The candidate order does not matter: the warp rank-sorts the accepted
//    neighbors by (j, image) to reproduce the Fortran slot order exactly.
//  * All pair arithmetic is evaluated in the Fortran source order with explicit
//    round-to-nearest intrinsics (no FMA contraction), so dR and the accept / reject
//    decisions are bit-identical to the restatement in plain C.
#include <mutex>
#include <string>
#include "common.cuh"

namespace matpl {
namespace {

constexpr int kWarps = 4;
constexpr int kMaxTypes = 16;

struct NbImage {
    double L[9];
    int iflag;       // 1: enumerate periodic images (NeighConst.f90:55-92)
    int nper[3];     // nperiod (NeighConst.f90:42)
    int nb[3];       // cell bins per fractional axis (minimum-image branch)
    int ncells;
    int ortho;       // off-diagonal lattice entries all (signed) zero
};

struct NbParams {
    int batch, natoms, ntypes, m;
    double rc2;                    // Rc_M**2
    double rct2[kMaxTypes];        // Rc_type(t)**2
    int cell_cap;                  // cell capacity per image
    int occupied_only;             // 1: write the occupied slots only (counts in num_neigh)
};

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ void cart(const double *L, double d1, double d2, double d3, double &x,
                                     double &y, double &z, double &dd) {
    x = da(da(dm(L[0], d1), dm(L[3], d2)), dm(L[6], d3));
    y = da(da(dm(L[1], d1), dm(L[4], d2)), dm(L[7], d3));
    z = da(da(dm(L[2], d1), dm(L[5], d2)), dm(L[8], d3));
    dd = da(da(dm(x, x), dm(y, y)), dm(z, z));
}

// mic with integer tests on the bit pattern: for |d| < 2 (fractional differences of wrapped
// positions lie in (-1, 1)) d + 1 and d - 1 are exact (Sterbenz), so |d + 1| < |d| holds exactly
// when d < -0.5 and |d - 1| < |d| when d > 0.5.  Called by all lanes of the warp: the one FP64
// add is issued only when some lane needs it.
__device__ __forceinline__ void mic_bits(double &d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const bool need = (u & 0x7FFFFFFFFFFFFFFFull) > 0x3FE0000000000000ull;
    if (__any_sync(0xffffffffu, need)) {
        const double dn = da(d, (u >> 63) ? 1.0 : -1.0);
        if (need) d = dn;
    }
}

__device__ __forceinline__ bool is_zero_bits(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull) == 0ull;
}

// cart() for a lattice whose off-diagonal entries are (signed) zeros: a non-zero product plus
// signed zeros is that product exactly, so only a zero diagonal product needs the full sum (for
// its sign); bit-identical to cart().  Called by all lanes of the warp (the full sums are issued
// only when some lane has a zero product).
__device__ __forceinline__ void cart_ortho(const double *L, double d1, double d2, double d3,
                                           double &x, double &y, double &z, double &dd) {
    x = dm(L[0], d1);
    y = dm(L[4], d2);
    z = dm(L[8], d3);
    const bool zx = is_zero_bits(x), zy = is_zero_bits(y), zz = is_zero_bits(z);
    if (__any_sync(0xffffffffu, zx || zy || zz)) {
        const double fx = da(da(x, dm(L[3], d2)), dm(L[6], d3));
        const double fy = da(da(dm(L[1], d1), y), dm(L[7], d3));
        const double fz = da(da(dm(L[2], d1), dm(L[5], d2)), z);
        if (zx) x = fx;
        if (zy) y = fy;
        if (zz) z = fz;
    }
    dd = da(da(dm(x, x), dm(y, y)), dm(z, z));
}

// a < b for non-negative doubles (and +inf / NaN above every finite value) as integers
__device__ __forceinline__ bool lt_bits(double a, double b) {
    return __double_as_longlong(a) < __double_as_longlong(b);
}

__device__ __forceinline__ void store4(float *p, float a, float b, float c, float d) {
    *reinterpret_cast<float4 *>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void store4(double *p, double a, double b, double c, double d) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2 *>(p)[1] = make_double2(c, d);
}

__global__ void nb_setup(const double *__restrict__ lattice, NbImage *__restrict__ img,
                         int batch, double Rc, int cell_cap) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < batch; b += gridDim.x * blockDim.x) {
        NbImage im;
        const double *L = lattice + 9 * b;
        for (int q = 0; q < 9; ++q) im.L[q] = L[q];
        im.iflag = 0;
        for (int v = 0; v < 3; ++v) {
            double d = sqrt(da(da(dm(L[3 * v], L[3 * v]), dm(L[3 * v + 1], L[3 * v + 1])),
                               dm(L[3 * v + 2], L[3 * v + 2])));
            im.nper[v] = (int)(Rc / d) + 1;
            if (d < 2 * Rc) im.iflag = 1;
        }
        // thickness h_k = V / |a_i x a_j|
        const double *a = L, *bb = L + 3, *c = L + 6;
        double cr[3][3];
        const double *vv[3][2] = {{bb, c}, {c, a}, {a, bb}};
        for (int k = 0; k < 3; ++k) {
            const double *p = vv[k][0], *q = vv[k][1];
            cr[k][0] = p[1] * q[2] - p[2] * q[1];
            cr[k][1] = p[2] * q[0] - p[0] * q[2];
            cr[k][2] = p[0] * q[1] - p[1] * q[0];
        }
        const double V = fabs(a[0] * cr[0][0] + a[1] * cr[0][1] + a[2] * cr[0][2]);
        long long prod = 1;
        for (int k = 0; k < 3; ++k) {
            double area = sqrt(cr[k][0] * cr[k][0] + cr[k][1] * cr[k][1] + cr[k][2] * cr[k][2]);
            double h = V / area;
            int n = (int)floor(h / (Rc * 1.0000001));
            im.nb[k] = n < 1 ? 1 : (n > 1024 ? 1024 : n);
        }
        for (;;) {
            prod = (long long)im.nb[0] * im.nb[1] * im.nb[2];
            if (prod <= cell_cap) break;
            int kmax = 0;
            for (int k = 1; k < 3; ++k)
                if (im.nb[k] > im.nb[kmax]) kmax = k;
            im.nb[kmax] = (im.nb[kmax] + 1) / 2;
        }
        im.ncells = im.iflag ? 0 : (int)prod;
        im.ortho = L[1] == 0.0 && L[2] == 0.0 && L[3] == 0.0 && L[5] == 0.0 && L[6] == 0.0 &&
                   L[7] == 0.0;
        img[b] = im;
    }
}

__global__ void nb_bin(const double *__restrict__ frac, const NbImage *__restrict__ img,
                       double *__restrict__ wpos, float4 *__restrict__ wpos32,
                       int *__restrict__ cell_of, int *__restrict__ cell_count, NbParams P) {
    const long long total = (long long)P.batch * P.natoms;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(t / P.natoms);
        double f[3];
        for (int k = 0; k < 3; ++k) {
            f[k] = fmod(da(frac[3 * t + k], 10.0), 1.0);   // NeighConst.f90:46-50
            wpos[3 * t + k] = f[k];
        }
        wpos32[t] = make_float4((float)f[0], (float)f[1], (float)f[2], 0.f);
        const NbImage &im = img[b];
        if (im.iflag) {
            cell_of[t] = -1;
            continue;
        }
        int c[3];
        for (int k = 0; k < 3; ++k) {
            int q = (int)(f[k] * im.nb[k]);
            c[k] = q >= im.nb[k] ? im.nb[k] - 1 : (q < 0 ? 0 : q);
        }
        const int cell = (c[0] * im.nb[1] + c[1]) * im.nb[2] + c[2];
        cell_of[t] = cell;
        atomicAdd(cell_count + (long long)b * P.cell_cap + cell, 1);
    }
}

// Exclusive scan of cell counts, one block per image.
__global__ void nb_scan(const NbImage *__restrict__ img, const int *__restrict__ cell_count,
                        int *__restrict__ cell_start, NbParams P) {
    const int b = blockIdx.x;
    const int n = img[b].ncells;
    const int *cnt = cell_count + (long long)b * P.cell_cap;
    int *st = cell_start + (long long)b * (P.cell_cap + 1);
    __shared__ int wsum[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        int v = i < n ? cnt[i] : 0;
        int x = v;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            int s = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            wsum[lane] = s;
        }
        __syncthreads();
        const int excl = carry + x - v + (w > 0 ? wsum[w - 1] : 0);
        if (i < n) st[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) st[n] = carry;
}

__global__ void nb_fill(const int *__restrict__ cell_of, const int *__restrict__ cell_start,
                        int *__restrict__ cell_fill, int *__restrict__ cell_atoms, NbParams P) {
    const long long total = (long long)P.batch * P.natoms;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int cell = cell_of[t];
        if (cell < 0) continue;
        const int b = (int)(t / P.natoms);
        const int pos = atomicAdd(cell_fill + (long long)b * P.cell_cap + cell, 1);
        cell_atoms[(long long)b * P.natoms + cell_start[(long long)b * (P.cell_cap + 1) + cell] +
                   pos] = (int)(t - (long long)b * P.natoms);
    }
}

// FP32 pre-filter: a candidate whose single-precision distance is clearly beyond Rc (by a
// margin far larger than the FP32 rounding error of the pair vector) is dropped; everything
// else, including nearest-image ties, goes to the exact FP64 test below.
__device__ __forceinline__ bool maybe_within(const float *Lf, float d1, float d2, float d3,
                                             float thr2) {
    const float x = Lf[0] * d1 + Lf[3] * d2 + Lf[6] * d3;
    const float y = Lf[1] * d1 + Lf[4] * d2 + Lf[7] * d3;
    const float z = Lf[2] * d1 + Lf[5] * d2 + Lf[8] * d3;
    return x * x + y * y + z * z < thr2;
}

__device__ __forceinline__ float mic_f(float d, bool &tie) {
    if (fabsf(d + 1.f) < fabsf(d)) d += 1.f;
    if (fabsf(d - 1.f) < fabsf(d)) d -= 1.f;
    tie |= fabsf(fabsf(d) - 0.5f) < 1e-5f;
    return d;
}

template <typename TO>
__global__ void __launch_bounds__(kWarps * 32)
nb_search(const NbImage *__restrict__ img, const double *__restrict__ wpos,
          const float4 *__restrict__ wpos32, const int32_t *__restrict__ type_map,
          const int *__restrict__ cell_start, const int *__restrict__ cell_atoms,
          int32_t *__restrict__ list_neigh, TO *__restrict__ image_dr,
          int32_t *__restrict__ num_neigh, int32_t *__restrict__ err, NbParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int S = P.ntypes * P.m;
    const int CAP = 2 * S;                         // pre-filtered candidates per atom
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // accepted pairs: the output row (r, x, y, z) in the output dtype (the f64 values are the
    // exact ones; the f32 ones their rounding, formed here once)
    constexpr int KV = sizeof(TO) * 4;              // bytes per accepted pair
    TO *kvec = reinterpret_cast<TO *>(smem_raw) + 4 * warp * S;
    int *cand = reinterpret_cast<int *>(smem_raw + (size_t)KV * kWarps * S) + warp * (CAP + S);
    int *keys = cand + CAP;
    unsigned char *ktype = reinterpret_cast<unsigned char *>(
                               reinterpret_cast<int *>(smem_raw + (size_t)KV * kWarps * S) +
                               kWarps * (CAP + S)) + warp * S;
    const long long total = (long long)P.batch * P.natoms;
    for (long long t = (long long)blockIdx.x * kWarps + warp; t < total;
         t += (long long)gridDim.x * kWarps) {
        const int b = (int)(t / P.natoms);
        const int i = (int)(t - (long long)b * P.natoms);
        const NbImage &im = img[b];
        const double *pos = wpos + (long long)b * P.natoms * 3;
        const float4 *pos32 = wpos32 + (long long)b * P.natoms;
        const double pi0 = pos[3 * i], pi1 = pos[3 * i + 1], pi2 = pos[3 * i + 2];
        const float4 fi = pos32[i];
        const int ti = type_map[i];
        if (ti < 0 || ti >= P.ntypes) {
            if (lane == 0) atomicMax(err, MATPL_KERR_BAD_TYPE);
            continue;
        }
        float Lf[9], lsum = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            Lf[q] = (float)im.L[q];
            lsum += fabsf(Lf[q]);
        }
        const float rc2f = (float)P.rc2;
        const float thr2 = rc2f + 0.01f + 1e-5f * lsum * sqrtf(rc2f);
        const int nimg1 = 2 * im.nper[2] + 1, nimg2 = 2 * im.nper[1] + 1;
        const int nimg = im.iflag ? (2 * im.nper[0] + 1) * nimg2 * nimg1 : 1;

        // ---- phase A: enumerate candidates (flattened over cell ranges / images), FP32 filter
        int ncand = 0;
        bool cap_hit = false;
        if (im.iflag) {
            long long T = (long long)P.natoms * nimg;
            if (T > 0x7fffffffLL) {           // keys would overflow int32: no candidates
                if (lane == 0) atomicMax(err, MATPL_KERR_BAD_BOX);
                T = 0;
            }
            for (long long c0 = 0; c0 < T; c0 += 32) {
                const long long c = c0 + lane;
                bool keep = false;
                int key = 0;
                if (c < T) {
                    const int j = (int)(c / nimg), idx = (int)(c - (long long)j * nimg);
                    const int i3 = idx % nimg1 - im.nper[2];
                    const int i2 = (idx / nimg1) % nimg2 - im.nper[1];
                    const int i1 = idx / (nimg1 * nimg2) - im.nper[0];
                    const float4 fj = pos32[j];
                    keep = maybe_within(Lf, fj.x - fi.x + i1, fj.y - fi.y + i2, fj.z - fi.z + i3, thr2);
                    key = j * nimg + idx;
                }
                const unsigned mk = __ballot_sync(0xffffffffu, keep);
                const int at = ncand + __popc(mk & ((1u << lane) - 1u));
                if (keep && at < CAP) cand[at] = key;
                ncand += __popc(mk);
            }
        } else {
            // up to 9 (x, y) columns x 2 z-ranges; lane q < nr holds range q
            int ci[3];
            ci[0] = min((int)(fi.x * im.nb[0]), im.nb[0] - 1);
            ci[1] = min((int)(fi.y * im.nb[1]), im.nb[1] - 1);
            ci[2] = min((int)(fi.z * im.nb[2]), im.nb[2] - 1);
            // the FP32 bin may differ from the FP64 bin at a bin edge: use the FP64 one
            {
                const double f[3] = {pi0, pi1, pi2};
                for (int k = 0; k < 3; ++k) {
                    int q = (int)(f[k] * im.nb[k]);
                    ci[k] = q >= im.nb[k] ? im.nb[k] - 1 : (q < 0 ? 0 : q);
                }
            }
            const int *cs = cell_start + (long long)b * (P.cell_cap + 1);
            const int *ca = cell_atoms + (long long)b * P.natoms;
            const int nx = im.nb[0] >= 3 ? 3 : im.nb[0], ny = im.nb[1] >= 3 ? 3 : im.nb[1];
            const int nz = im.nb[2] >= 3 ? 3 : im.nb[2];
            const int ox0 = im.nb[0] >= 3 ? -1 : 0, oy0 = im.nb[1] >= 3 ? -1 : 0;
            const int oz0 = im.nb[2] >= 3 ? -1 : 0;
            // lane q (< 18) builds range q: column q/2, part q%2
            int rs = 0, rl = 0;
            if (lane < 18) {
                const int col = lane >> 1, part = lane & 1;
                if (col < nx * ny) {
                    const int cx = (ci[0] + ox0 + col / ny + im.nb[0]) % im.nb[0];
                    const int cy = (ci[1] + oy0 + col % ny + im.nb[1]) % im.nb[1];
                    const int base = (cx * im.nb[1] + cy) * im.nb[2];
                    const int zlo = ci[2] + oz0;                // may be -1
                    const int zhi = zlo + nz - 1;               // may be nb
                    int a0, a1;                                 // z-cell interval of this part
                    if (part == 0) {
                        a0 = zlo < 0 ? 0 : zlo;
                        a1 = zhi >= im.nb[2] ? im.nb[2] - 1 : zhi;
                    } else if (zlo < 0) {
                        a0 = im.nb[2] - 1; a1 = im.nb[2] - 1;
                    } else if (zhi >= im.nb[2]) {
                        a0 = 0; a1 = 0;
                    } else {
                        a0 = 1; a1 = 0;                          // empty
                    }
                    if (a0 <= a1) {
                        rs = cs[base + a0];
                        rl = cs[base + a1 + 1] - rs;
                    }
                }
            }
            int incl = rl;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int T = __shfl_sync(0xffffffffu, incl, 31);
            const int excl = incl - rl;
            for (int c0 = 0; c0 < T; c0 += 32) {
                const int c = c0 + lane;
                // find the range holding flat index c: the last q < 18 with excl_q <= c (an
                // empty range shares its start with the next one, so that q is not empty)
                int q = 0, qhi = 17;
#pragma unroll
                for (int it = 0; it < 5; ++it) {
                    const int mid = (q + qhi + 1) >> 1;
                    const int e_m = __shfl_sync(0xffffffffu, excl, mid);
                    if (e_m <= c) q = mid; else qhi = mid - 1;
                }
                const int s_q = __shfl_sync(0xffffffffu, rs, q);
                const int e_q = __shfl_sync(0xffffffffu, excl, q);
                bool keep = false;
                int j = 0;
                if (c < T) {
                    j = ca[s_q + c - e_q];
                    const float4 fj = pos32[j];
                    bool tie = false;
                    const float d1 = mic_f(fj.x - fi.x, tie), d2 = mic_f(fj.y - fi.y, tie),
                                d3 = mic_f(fj.z - fi.z, tie);
                    keep = tie || maybe_within(Lf, d1, d2, d3, thr2);
                }
                const unsigned mk = __ballot_sync(0xffffffffu, keep);
                const int at = ncand + __popc(mk & ((1u << lane) - 1u));
                if (keep && at < CAP) cand[at] = j;
                ncand += __popc(mk);
            }
        }
        if (ncand > CAP) { cap_hit = true; ncand = CAP; }
        __syncwarp();

        // ---- phase B: exact FP64 test (NeighConst.f90 arithmetic) on the survivors
        int cntM[kMaxTypes];
#pragma unroll
        for (int q = 0; q < kMaxTypes; ++q) cntM[q] = 0;
        int n_acc = 0;
        const double rct2 = P.rct2[ti];
        for (int c0 = 0; c0 < ncand; c0 += 32) {
            // every lane evaluates a candidate (lanes past the end repeat the last one and are
            // masked), so the warp-wide votes in mic_bits / cart_ortho see the whole warp
            const int c = c0 + lane;
            const bool valid = c < ncand;
            const int key = cand[valid ? c : ncand - 1];
            const int j = key / nimg, idx = key - (key / nimg) * nimg;
            double d1, d2, d3, px, py, pz, pdd;
            if (im.iflag) {
                const int i3 = idx % nimg1 - im.nper[2];
                const int i2 = (idx / nimg1) % nimg2 - im.nper[1];
                const int i1 = idx / (nimg1 * nimg2) - im.nper[0];
                d1 = da(da(pos[3 * j], -pi0), (double)i1);
                d2 = da(da(pos[3 * j + 1], -pi1), (double)i2);
                d3 = da(da(pos[3 * j + 2], -pi2), (double)i3);
            } else {
                d1 = da(pos[3 * j], -pi0); mic_bits(d1);
                d2 = da(pos[3 * j + 1], -pi1); mic_bits(d2);
                d3 = da(pos[3 * j + 2], -pi2); mic_bits(d3);
            }
            if (im.ortho) cart_ortho(im.L, d1, d2, d3, px, py, pz, pdd);
            else cart(im.L, d1, d2, d3, px, py, pz, pdd);
            // pdd >= +0: the comparisons as integer comparisons of the bit patterns
            bool inM = valid && lt_bits(pdd, P.rc2) && lt_bits(1.0e-8, pdd);
            bool inT = inM && lt_bits(pdd, rct2);
            int tj = type_map[j];
            if (tj < 0 || tj >= P.ntypes) {
                if (valid) atomicMax(err, MATPL_KERR_BAD_TYPE);
                inM = inT = false;
                tj = 0;
            }
#pragma unroll
            for (int q = 0; q < kMaxTypes; ++q)
                if (q < P.ntypes) cntM[q] += __popc(__ballot_sync(0xffffffffu, inM && tj == q));
            const unsigned ma = __ballot_sync(0xffffffffu, inT);
            const int at = n_acc + __popc(ma & ((1u << lane) - 1u));
            if (inT && at < S) {
                keys[at] = key;
                ktype[at] = (unsigned char)tj;
                store4(kvec + 4 * at, pair_r<TO>(pdd), conv<TO>(px), conv<TO>(py), conv<TO>(pz));
            }
            n_acc += __popc(ma);
        }
        bool overflow = cap_hit;
#pragma unroll
        for (int q = 0; q < kMaxTypes; ++q) overflow |= (q < P.ntypes) && cntM[q] > P.m;
        if (overflow && lane == 0) atomicMax(err, MATPL_KERR_NEIGHBOR_OVERFLOW);
        const int nst = n_acc < S ? n_acc : S;
        __syncwarp();
        int ncount[kMaxTypes];
#pragma unroll
        for (int q = 0; q < kMaxTypes; ++q) {
            int c = 0;
            if (q < P.ntypes) {
                for (int e = lane; e < nst; e += 32) c += ktype[e] == q;
                c = warp_sum(c);
            }
            ncount[q] = c < P.m ? c : P.m;
        }
        const long long row = t * (long long)S;
        // ---- phase C: rank sort by (j, image) inside each type block, write occupied slots
        for (int e = lane; e < nst; e += 32) {
            const int key = keys[e];
            const int ty = ktype[e];
            int rank = 0;
            for (int f = 0; f < nst; ++f) rank += (ktype[f] == ty) & (keys[f] < key);
            if (rank >= P.m) continue;
            const int j = key / nimg;
            const TO *kv = kvec + 4 * e;
            const long long slot = row + (long long)ty * P.m + rank;
            list_neigh[slot] = j + 1;
            store4(image_dr + 4 * slot, kv[0], kv[1], kv[2], kv[3]);
        }
        // ---- phase D: clear the empty slots (the occupied-slot form leaves them untouched:
        // its readers take the block lengths from num_neigh)
        for (int s = lane; s < S && !P.occupied_only; s += 32) {
            const int ty = s / P.m;
            int nt = 0;
#pragma unroll
            for (int q = 0; q < kMaxTypes; ++q)
                if (q == ty) nt = ncount[q];
            if (s - ty * P.m < nt) continue;
            list_neigh[row + s] = 0;
            store4(image_dr + 4 * (row + s), TO(0), TO(0), TO(0), TO(0));
        }
        if (num_neigh != nullptr && lane < P.ntypes) {
            int c = 0;
#pragma unroll
            for (int q = 0; q < kMaxTypes; ++q)
                if (q == lane) c = ncount[q];
            num_neigh[t * P.ntypes + lane] = c;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------
// Environment matrix (dp_dp.py:217-302).  One thread per slot.
template <typename T>
__global__ void env_mat_kernel(const int32_t *__restrict__ type_map, const T *__restrict__ idr,
                               const T *__restrict__ davg, const T *__restrict__ dstd, T rmin,
                               T rmax, T *__restrict__ Ri, T *__restrict__ Rid, int batch,
                               int natoms, int nslots) {
    const long long total = (long long)batch * natoms * nslots;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < total;
         s += (long long)gridDim.x * blockDim.x) {
        const long long bi = s / nslots;
        const int i = (int)(bi % natoms);
        const int k = (int)(s - bi * nslots);
        const int ti = type_map[i];
        const T R = idr[4 * s], x = idr[4 * s + 1], y = idr[4 * s + 2], z = idr[4 * s + 3];
        T sr = 0, ds = 0;
        if (R > 0 && R < rmin) {
            sr = T(1) / R;
            ds = -T(1) / (R * R);
        } else if (R > rmin && R < rmax) {
            const T u = (R - rmin) / (rmax - rmin);
            const T poly = u * u * u * (T(-6) * u * u + T(15) * u - T(10)) + T(1);
            const T dpoly = (T(3) * u * u * (T(-6) * u * u + T(15) * u - T(10)) +
                             u * u * u * (T(-12) * u + T(15))) / (rmax - rmin);
            sr = poly / R;
            ds = dpoly / R - poly / (R * R);
        }
        const bool mask = fabs((double)R) > 1e-5;
        const T *av = davg + ((long long)ti * nslots + k) * 4;
        const T *sd = dstd + ((long long)ti * nslots + k) * 4;
        const T raw[4] = {sr, mask ? sr * x / R : T(0), mask ? sr * y / R : T(0),
                          mask ? sr * z / R : T(0)};
        for (int c = 0; c < 4; ++c) Ri[4 * s + c] = (raw[c] - av[c]) / sd[c];
        T d[4][3];
        const T xyz[3] = {x, y, z};
        const T common = mask ? (ds - sr / R) / (R * R) : T(0);
        for (int bcol = 0; bcol < 3; ++bcol) {
            d[0][bcol] = mask ? ds * xyz[bcol] / R : T(0);
            for (int a = 0; a < 3; ++a) {
                T v = common * xyz[a] * xyz[bcol];
                if (a == bcol) v += mask ? sr / R : T(0);
                d[a + 1][bcol] = mask ? v : T(0);
            }
        }
        for (int c = 0; c < 4; ++c)
            for (int bcol = 0; bcol < 3; ++bcol) Rid[12 * s + 3 * c + bcol] = -d[c][bcol] / sd[c];
    }
}

struct NbLayout {
    size_t img, wpos, wpos32, cell_of, cell_count, cell_fill, cell_start, cell_atoms, total;
};

NbLayout nb_layout(int batch, int natoms) {
    NbLayout l;
    const size_t cap = (size_t)natoms + 27;
    size_t o = 0;
    l.img = o;        o = align_up(o + sizeof(NbImage) * batch, 256);
    l.wpos = o;       o = align_up(o + 8 * 3 * (size_t)batch * natoms, 256);
    l.wpos32 = o;     o = align_up(o + 16 * (size_t)batch * natoms, 256);
    l.cell_of = o;    o = align_up(o + 4 * (size_t)batch * natoms, 256);
    l.cell_count = o; o = align_up(o + 4 * cap * batch, 256);
    l.cell_fill = o;  o = align_up(o + 4 * cap * batch, 256);
    l.cell_start = o; o = align_up(o + 4 * (cap + 1) * batch, 256);
    l.cell_atoms = o; o = align_up(o + 4 * (size_t)batch * natoms, 256);
    l.total = o;
    return l;
}

inline int grid_for(long long work, int per_block) {
    long long g = (work + per_block - 1) / per_block;
    if (g > (long long)device_sms() * 32) g = (long long)device_sms() * 32;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" size_t matpl_neighbor_workspace_bytes(int batch, int natoms) {
    if (batch < 0 || natoms < 0) return 0;
    return nb_layout(batch, natoms).total;
}

static int neighbor_build(int batch, int natoms, int ntypes, int m_neigh, double Rc_M,
                          const double *Rc_type, const int32_t *type_map, const double *lattice,
                          const double *frac_pos, int out_dtype, int32_t *list_neigh,
                          void *image_dr, int32_t *num_neigh, int32_t *err_dev, void *workspace,
                          size_t workspace_bytes, void *stream, bool occupied_only) {
    MATPL_REQUIRE(batch >= 0 && natoms >= 0, MATPL_ERR_INVALID, "negative size");
    MATPL_REQUIRE(ntypes >= 1 && ntypes <= kMaxTypes, MATPL_ERR_UNSUPPORTED,
                  "ntypes must be in [1, 16]");
    MATPL_REQUIRE(m_neigh >= 1, MATPL_ERR_INVALID, "m_neigh must be >= 1");
    MATPL_REQUIRE((long long)ntypes * m_neigh <= 1024, MATPL_ERR_UNSUPPORTED,
                  "ntypes * m_neigh must be <= 1024");
    MATPL_REQUIRE(Rc_M > 0 && Rc_type != nullptr, MATPL_ERR_INVALID, "bad cutoff");
    MATPL_REQUIRE(out_dtype == MATPL_F32 || out_dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "image_dr dtype must be f32 or f64");
    MATPL_REQUIRE(err_dev != nullptr, MATPL_ERR_INVALID, "err_dev is required");
    const NbLayout lay = nb_layout(batch, natoms);
    MATPL_REQUIRE(workspace != nullptr && workspace_bytes >= lay.total, MATPL_ERR_WORKSPACE,
                  "neighbor workspace too small");
    if (batch == 0 || natoms == 0) return MATPL_OK;
    // candidate keys j * nimages + image are int32: nb_search refuses (MATPL_KERR_BAD_BOX,
    // empty lists) an image whose natoms * nimages would not fit
    MATPL_REQUIRE(type_map && lattice && frac_pos && list_neigh && image_dr, MATPL_ERR_INVALID,
                  "matpl_neighbor_build: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(list_neigh, "matpl_neighbor_build");
    cudaStream_t s = as_stream(stream);
    NbParams P;
    P.batch = batch; P.natoms = natoms; P.ntypes = ntypes; P.m = m_neigh;
    P.rc2 = Rc_M * Rc_M;
    for (int q = 0; q < kMaxTypes; ++q) P.rct2[q] = q < ntypes ? Rc_type[q] * Rc_type[q] : 0.0;
    P.cell_cap = natoms + 27;
    P.occupied_only = occupied_only ? 1 : 0;
    char *ws = static_cast<char *>(workspace);
    NbImage *img = reinterpret_cast<NbImage *>(ws + lay.img);
    double *wpos = reinterpret_cast<double *>(ws + lay.wpos);
    float4 *wpos32 = reinterpret_cast<float4 *>(ws + lay.wpos32);
    int *cell_of = reinterpret_cast<int *>(ws + lay.cell_of);
    int *cell_count = reinterpret_cast<int *>(ws + lay.cell_count);
    int *cell_fill = reinterpret_cast<int *>(ws + lay.cell_fill);
    int *cell_start = reinterpret_cast<int *>(ws + lay.cell_start);
    int *cell_atoms = reinterpret_cast<int *>(ws + lay.cell_atoms);
    if (cudaMemsetAsync(ws + lay.cell_count, 0, lay.cell_start - lay.cell_count, s) !=
        cudaSuccess) {
        set_error("matpl_neighbor_build: memset failed");
        return MATPL_ERR_CUDA;
    }
    const long long na = (long long)batch * natoms;
    {
        ProfScope ps("nb_cells", s);
        nb_setup<<<(batch + 127) / 128, 128, 0, s>>>(lattice, img, batch, Rc_M, P.cell_cap);
        nb_bin<<<grid_for(na, 256), 256, 0, s>>>(frac_pos, img, wpos, wpos32, cell_of, cell_count, P);
        nb_scan<<<batch, 1024, 0, s>>>(img, cell_count, cell_start, P);
        nb_fill<<<grid_for(na, 256), 256, 0, s>>>(cell_of, cell_start, cell_fill, cell_atoms, P);
    }
    ProfScope ps("nb_search", s);
    const int S = ntypes * m_neigh;
    const size_t smem = (size_t)kWarps * (S * 4 * (out_dtype == MATPL_F64 ? 8 : 4) + 3 * S * 4 + S);
    if (out_dtype == MATPL_F64) {
        cudaFuncSetAttribute(nb_search<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        nb_search<double><<<grid_for(na, kWarps), kWarps * 32, smem, s>>>(
            img, wpos, wpos32, type_map, cell_start, cell_atoms, list_neigh, (double *)image_dr,
            num_neigh, err_dev, P);
    } else {
        cudaFuncSetAttribute(nb_search<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        nb_search<float><<<grid_for(na, kWarps), kWarps * 32, smem, s>>>(
            img, wpos, wpos32, type_map, cell_start, cell_atoms, list_neigh, (float *)image_dr,
            num_neigh, err_dev, P);
    }
    return check_launch("matpl_neighbor_build");
}

extern "C" int matpl_neighbor_build(int batch, int natoms, int ntypes, int m_neigh, double Rc_M,
                                    const double *Rc_type, const int32_t *type_map,
                                    const double *lattice, const double *frac_pos, int out_dtype,
                                    int32_t *list_neigh, void *image_dr, int32_t *num_neigh,
                                    int32_t *err_dev, void *workspace, size_t workspace_bytes,
                                    void *stream) {
    return neighbor_build(batch, natoms, ntypes, m_neigh, Rc_M, Rc_type, type_map, lattice,
                          frac_pos, out_dtype, list_neigh, image_dr, num_neigh, err_dev,
                          workspace, workspace_bytes, stream, false);
}

extern "C" int matpl_neighbor_build_occupied(int batch, int natoms, int ntypes, int m_neigh,
                                             double Rc_M, const double *Rc_type,
                                             const int32_t *type_map, const double *lattice,
                                             const double *frac_pos, int out_dtype,
                                             int32_t *list_neigh, void *image_dr,
                                             int32_t *num_neigh, int32_t *err_dev,
                                             void *workspace, size_t workspace_bytes,
                                             void *stream) {
    MATPL_REQUIRE(num_neigh != nullptr, MATPL_ERR_INVALID,
                  "matpl_neighbor_build_occupied: num_neigh is required (it gives the block "
                  "lengths)");
    return neighbor_build(batch, natoms, ntypes, m_neigh, Rc_M, Rc_type, type_map, lattice,
                          frac_pos, out_dtype, list_neigh, image_dr, num_neigh, err_dev,
                          workspace, workspace_bytes, stream, true);
}

extern "C" int matpl_env_mat(int dtype, int batch, int natoms, int nslots,
                             const int32_t *type_map, const void *image_dr, const void *davg,
                             const void *dstd, double rmin, double rmax, void *Ri, void *Ri_d,
                             void *stream) {
    MATPL_REQUIRE(dtype == MATPL_F32 || dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "env_mat supports f32 and f64");
    MATPL_REQUIRE(batch >= 0 && natoms >= 0 && nslots >= 0, MATPL_ERR_INVALID, "negative size");
    const long long total = (long long)batch * natoms * nslots;
    if (total == 0) return MATPL_OK;
    MATPL_REQUIRE(type_map && image_dr && davg && dstd && Ri && Ri_d, MATPL_ERR_INVALID,
                  "matpl_env_mat: null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(Ri, "matpl_env_mat");
    cudaStream_t s = as_stream(stream);
    if (dtype == MATPL_F64)
        env_mat_kernel<double><<<grid_for(total, 256), 256, 0, s>>>(
            type_map, (const double *)image_dr, (const double *)davg, (const double *)dstd, rmin,
            rmax, (double *)Ri, (double *)Ri_d, batch, natoms, nslots);
    else
        env_mat_kernel<float><<<grid_for(total, 256), 256, 0, s>>>(
            type_map, (const float *)image_dr, (const float *)davg, (const float *)dstd,
            (float)rmin, (float)rmax, (float *)Ri, (float *)Ri_d, batch, natoms, nslots);
    return check_launch("matpl_env_mat");
}

// ---------------------------------------------------------------------------------------
// Allocation-free neighbor search.  Some hosts cannot hand this library device memory: an MD
// engine's per-step force callback that owns all device memory through its own pool (or a C /
// Fortran host with no device allocator at hand) must not call cudaMalloc, which also blocks
// the whole device while it runs.  matpl_neighbor_build_noalloc keeps its scratch in the
// fixed array below (one copy on every GPU that loads this library, kept until the process
// exits) and otherwise runs exactly matpl_neighbor_build.
namespace {
constexpr size_t kNoAllocScratchBytes = 4u << 20;          // 4 MiB: ~65,000 atoms per call
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_nb_scratch[kNoAllocScratchBytes];

extern "C" int matpl_neighbor_build_noalloc(int batch, int natoms, int ntypes, int m_neigh,
                                            double Rc_M, const double *Rc_type,
                                            const int32_t *type_map, const double *lattice,
                                            const double *frac_pos, int out_dtype,
                                            int32_t *list_neigh, void *image_dr,
                                            int32_t *num_neigh, int32_t *err_dev, void *stream) {
    MATPL_REQUIRE(batch >= 0 && natoms >= 0, MATPL_ERR_INVALID, "negative size");
    const size_t need = nb_layout(batch, natoms).total;
    MATPL_REQUIRE(need <= kNoAllocScratchBytes, MATPL_ERR_WORKSPACE,
                  "matpl_neighbor_build_noalloc: " + std::to_string(batch) + " x " +
                      std::to_string(natoms) + " atoms need " + std::to_string(need) +
                      " scratch bytes, above its fixed 4 MiB (about 65,000 atoms per call); use "
                      "matpl_neighbor_build with a caller workspace");
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("matpl_neighbor_build_noalloc: no usable current device");
        return MATPL_ERR_CUDA;
    }
    void *scratch = nullptr;
    {
        // Set-up on the first call on each device (with that device current): the array's
        // name is only a host-side handle, so look up its device address once.
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (g_noalloc_ptr[dev] == nullptr) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_nb_scratch);
            if (e != cudaSuccess || p == nullptr) {
                set_error(std::string("matpl_neighbor_build_noalloc: cudaGetSymbolAddress failed: ") +
                          cudaGetErrorString(e));
                return MATPL_ERR_CUDA;
            }
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    // matpl_neighbor_build clears the parts of the scratch that must start at zero (cell
    // counters) on the stream before its kernels run, so stale contents of the previous call
    // do not matter.
    return matpl_neighbor_build(batch, natoms, ntypes, m_neigh, Rc_M, Rc_type, type_map, lattice,
                                frac_pos, out_dtype, list_neigh, image_dr, num_neigh, err_dev,
                                scratch, kNoAllocScratchBytes, stream);
}
