// NEP neighbor lists: the drop-in for MatPL's CalcOps calculate_neighbor / calculate_maxneigh
// (src/op/src/CalcOps.cpp:1025-1172 -> src/op/kernel/calculateNepNeighbor.cu:8-380; CPU twin
// src/op/src/cpu_calculate_nepneighbor.cpp:6-203).
//
// Output contract (identical to the reference, bit for bit): for every atom n1 of a frame, the
// neighbors n2 of the same frame in ascending order and, for one n2, the replica offsets
// (ia, ib, ic) in [0, num_cell) with ic fastest; the pair vector is ((pos2 + delta) - pos1),
// delta = box_orig . (ia, ib, ic), folded by the minimum image of the replicated cell
// (box[9:18] = h^-1, box[0:9] = h), and the pair is kept when x^2 + y^2 + z^2 < rc^2.
// NL is int64 [N, max_NN] padded with -1, Ri f64 [N, max_NN, 4] = (r, x, y, z) (or 3 wide
// without r) padded with 0, NN the count.
//
// The reference runs one 256-thread block per frame over all N^2 * num_cell^3 candidates.  Here:
//  * frames whose cell is at least three cut-off widths thick in every direction (num_cell = 1)
//    go through a cell list: one warp per atom scans the 27 surrounding cells, drops candidates
//    with an FP32 distance test (margin far above the FP32 error), recomputes every survivor in
//    FP64 with the reference's operation order and no FMA (__dmul_rn / __dadd_rn), and sorts the
//    kept pairs by n2 in shared memory (each n2 occurs once: a single image can lie within rc);
//  * other frames (small or thin cells) enumerate (n2, image) in the reference's order with one
//    warp per atom, so warp ballots give the output positions without sorting.
// A list that would exceed max_NN is not written past its end: the kernel records
// MATPL_KERR_NEIGHBOR_OVERFLOW in err_dev and stores the full count in NN.
#include "common.cuh"

namespace matpl {
namespace {

constexpr int kSetupThreads = 256;

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }
constexpr float kPrefilterMargin = 0.02f;   // Angstrom, on top of a relative 1e-5

struct NepFrame {
    long long atom0;      // first atom of the frame
    long long cell0;      // first cell of the frame in the global cell arrays
    int n;                // atoms
    int mode;             // 0: cell list, 1: enumerate (n2, image)
    int nc[3];            // cell bins per fractional axis (mode 0)
    int ncells;
    int rep[3];           // num_cell replicas (mode 1)
    int ortho;            // h and h^-1 off-diagonals are all (signed) zeros
    double box[18];
    double bo[9];
    double zdelta[3];     // delta of replica (0, 0, 0), with the reference's signed zeros
    float H[9];           // box_orig as float (columns = lattice vectors)
    float Hinv[9];
};

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// ((p2 + delta) - p1), minimum image of the replicated cell, squared length: the operation
// order of cpu_calculate_nepneighbor.cpp:149-158 and nep_cpu.cpp:4-15.
__device__ __forceinline__ double exact_pair(const double *__restrict__ box, const double *p1,
                                             const double *p2, const double *delta, double &x,
                                             double &y, double &z) {
    x = ds(da(p2[0], delta[0]), p1[0]);
    y = ds(da(p2[1], delta[1]), p1[1]);
    z = ds(da(p2[2], delta[2]), p1[2]);
    double sx = da(da(dm(box[9], x), dm(box[10], y)), dm(box[11], z));
    double sy = da(da(dm(box[12], x), dm(box[13], y)), dm(box[14], z));
    double sz = da(da(dm(box[15], x), dm(box[16], y)), dm(box[17], z));
    sx = ds(sx, nearbyint(sx));
    sy = ds(sy, nearbyint(sy));
    sz = ds(sz, nearbyint(sz));
    x = da(da(dm(box[0], sx), dm(box[1], sy)), dm(box[2], sz));
    y = da(da(dm(box[3], sx), dm(box[4], sy)), dm(box[5], sz));
    z = da(da(dm(box[6], sx), dm(box[7], sy)), dm(box[8], sz));
    return da(da(dm(x, x), dm(y, y)), dm(z, z));
}

// Orthorhombic cells: every off-diagonal product in exact_pair is a signed zero, which leaves a
// nonzero sum unchanged.  A sum that is zero is +0 unless all of its terms are -0, so the
// result is the diagonal product when it is nonzero, else a zero whose sign is the AND of the
// terms' signs.  Same values, bit for bit, with 23 instead of 47 FP64 operations.
__device__ __forceinline__ unsigned sgn(double v) {
    return (unsigned)((unsigned long long)__double_as_longlong(v) >> 63);
}
__device__ __forceinline__ double zsum3(double diag, unsigned s1, unsigned s2) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(diag);
    if (b << 1) return diag;                                   // nonzero (or NaN)
    return __longlong_as_double((long long)((unsigned long long)(sgn(diag) & s1 & s2) << 63));
}
__device__ __forceinline__ double exact_pair_ortho(const double *__restrict__ box,
                                                   const double *p1, const double *p2,
                                                   const double *delta, double &x, double &y,
                                                   double &z) {
    x = ds(da(p2[0], delta[0]), p1[0]);
    y = ds(da(p2[1], delta[1]), p1[1]);
    z = ds(da(p2[2], delta[2]), p1[2]);
    const unsigned sx_ = sgn(x), sy_ = sgn(y), sz_ = sgn(z);
    double sx = zsum3(dm(box[9], x), sgn(box[10]) ^ sy_, sgn(box[11]) ^ sz_);
    double sy = zsum3(dm(box[13], y), sgn(box[12]) ^ sx_, sgn(box[14]) ^ sz_);
    double sz = zsum3(dm(box[17], z), sgn(box[15]) ^ sx_, sgn(box[16]) ^ sy_);
    sx = ds(sx, nearbyint(sx));
    sy = ds(sy, nearbyint(sy));
    sz = ds(sz, nearbyint(sz));
    const unsigned tx = sgn(sx), ty = sgn(sy), tz = sgn(sz);
    x = zsum3(dm(box[0], sx), sgn(box[1]) ^ ty, sgn(box[2]) ^ tz);
    y = zsum3(dm(box[4], sy), sgn(box[3]) ^ tx, sgn(box[5]) ^ tz);
    z = zsum3(dm(box[8], sz), sgn(box[6]) ^ tx, sgn(box[7]) ^ ty);
    return da(da(dm(x, x), dm(y, y)), dm(z, z));
}

__device__ __forceinline__ void replica_delta(const double *bo, int ia, int ib, int ic,
                                              double *d) {
    const double a = ia, b = ib, c = ic;
    d[0] = da(da(dm(bo[0], a), dm(bo[1], b)), dm(bo[2], c));
    d[1] = da(da(dm(bo[3], a), dm(bo[4], b)), dm(bo[5], c));
    d[2] = da(da(dm(bo[6], a), dm(bo[7], b)), dm(bo[8], c));
}

__device__ __forceinline__ int frame_of(const NepFrame *__restrict__ fr, int nframes,
                                        long long atom) {
    int lo = 0, hi = nframes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (fr[mid].atom0 <= atom) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void nepnb_setup(const long long *__restrict__ num_atom,
                            const double *__restrict__ box, const double *__restrict__ box_orig,
                            const long long *__restrict__ num_cell, NepFrame *__restrict__ fr,
                            int nframes, long long natoms, double rc_max, int *__restrict__ err,
                            const int *gate) {
    if (gate && *gate == 0) return;
    // frame offsets first; counts that overrun natoms are clipped and reported
    if (threadIdx.x == 0) {
        long long a0 = 0;
        for (int f = 0; f < nframes; ++f) {
            long long n = num_atom[f];
            if (n < 0 || a0 + n > natoms) {
                atomicOr(err, MATPL_KERR_BAD_COUNT);
                n = n < 0 ? 0 : natoms - a0;
            }
            fr[f].atom0 = a0;
            fr[f].n = (int)n;
            a0 += n;
        }
        if (a0 != natoms) atomicOr(err, MATPL_KERR_BAD_COUNT);
    }
    __syncthreads();
    for (int f = threadIdx.x; f < nframes; f += blockDim.x) {
        NepFrame F;
        F.atom0 = fr[f].atom0;
        F.n = fr[f].n;
        for (int q = 0; q < 18; ++q) F.box[q] = box[18 * f + q];
        for (int q = 0; q < 9; ++q) F.bo[q] = box_orig[9 * f + q];
        replica_delta(F.bo, 0, 0, 0, F.zdelta);
        {
            const int off[12] = {1, 2, 3, 5, 6, 7, 10, 11, 12, 14, 15, 16};
            bool o = true;
            for (int q = 0; q < 12; ++q) o &= F.box[off[q]] == 0.0;
            F.ortho = o;
        }
        bool single = true;
        for (int k = 0; k < 3; ++k) {
            F.rep[k] = (int)num_cell[3 * f + k];
            single &= F.rep[k] == 1;
            if (F.rep[k] < 1) atomicOr(err, MATPL_KERR_BAD_BOX);
        }
        // cell geometry of the original cell: columns of box_orig are the lattice vectors
        double a[3], b[3], c[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = F.bo[3 * k];
            b[k] = F.bo[3 * k + 1];
            c[k] = F.bo[3 * k + 2];
        }
        double cr[3][3];
        const double *uv[3][2] = {{b, c}, {c, a}, {a, b}};
        for (int k = 0; k < 3; ++k) {
            const double *p = uv[k][0], *q = uv[k][1];
            cr[k][0] = p[1] * q[2] - p[2] * q[1];
            cr[k][1] = p[2] * q[0] - p[0] * q[2];
            cr[k][2] = p[0] * q[1] - p[1] * q[0];
        }
        const double det = a[0] * cr[0][0] + a[1] * cr[0][1] + a[2] * cr[0][2];
        const double V = fabs(det);
        // Hinv rows = (b x c, c x a, a x b) / det
        for (int k = 0; k < 3; ++k)
            for (int q = 0; q < 3; ++q) {
                F.Hinv[3 * k + q] = (float)(cr[k][q] / det);
                F.H[3 * k + q] = (float)F.bo[3 * k + q];
            }
        const double width = rc_max * 1.00001 + kPrefilterMargin;
        long long prod = 1;
        bool thick = V > 0.0;
        for (int k = 0; k < 3; ++k) {
            const double area = sqrt(cr[k][0] * cr[k][0] + cr[k][1] * cr[k][1] +
                                     cr[k][2] * cr[k][2]);
            const double h = V / area;
            long long n = (long long)floor(h / width);
            if (n > 1024) n = 1024;
            F.nc[k] = (int)(n < 1 ? 1 : n);
        }
        // at most n + 27 cells per frame (the workspace bound)
        for (;;) {
            prod = (long long)F.nc[0] * F.nc[1] * F.nc[2];
            if (prod <= (long long)F.n + 27) break;
            int kmax = 0;
            for (int k = 1; k < 3; ++k)
                if (F.nc[k] > F.nc[kmax]) kmax = k;
            F.nc[kmax] = (F.nc[kmax] + 1) / 2;
        }
        for (int k = 0; k < 3; ++k) thick &= F.nc[k] >= 3;
        F.mode = (single && thick) ? 0 : 1;
        F.ncells = F.mode == 0 ? (int)prod : 0;
        fr[f] = F;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long c0 = 0;
        for (int f = 0; f < nframes; ++f) {
            fr[f].cell0 = c0;
            c0 += fr[f].ncells;
        }
    }
}

__global__ void nepnb_bin(const double *__restrict__ pos, const NepFrame *__restrict__ fr,
                          int nframes, long long natoms, float4 *__restrict__ spos,
                          int *__restrict__ cell_of, int *__restrict__ cell_count,
                          const int *gate, double *__restrict__ x_ref,
                          float4 *__restrict__ delta) {
    if (gate && *gate == 0) return;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < natoms;
         t += (long long)gridDim.x * blockDim.x) {
        if (x_ref)
            for (int k = 0; k < 3; ++k) x_ref[3 * t + k] = pos[3 * t + k];
        if (delta) delta[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        const NepFrame &F = fr[frame_of(fr, nframes, t)];
        if (F.mode != 0) {
            cell_of[t] = -1;
            continue;
        }
        const float p[3] = {(float)pos[3 * t], (float)pos[3 * t + 1], (float)pos[3 * t + 2]};
        float s[3];
        int c[3];
        for (int k = 0; k < 3; ++k) {
            float v = F.Hinv[3 * k] * p[0] + F.Hinv[3 * k + 1] * p[1] + F.Hinv[3 * k + 2] * p[2];
            v -= floorf(v);
            s[k] = v;
            int q = (int)(v * F.nc[k]);
            c[k] = q >= F.nc[k] ? F.nc[k] - 1 : (q < 0 ? 0 : q);
        }
        spos[t] = make_float4(s[0], s[1], s[2], 0.f);
        const int cell = (c[0] * F.nc[1] + c[1]) * F.nc[2] + c[2];
        cell_of[t] = cell;
        atomicAdd(cell_count + F.cell0 + cell, 1);
    }
}

// exclusive scan of one frame's cell counts, one block per frame
__global__ void nepnb_scan(const NepFrame *__restrict__ fr, const int *__restrict__ cell_count,
                           int *__restrict__ cell_start, const int *gate) {
    if (gate && *gate == 0) return;
    const NepFrame &F = fr[blockIdx.x];
    const int n = F.ncells;
    const int *cnt = cell_count + F.cell0;
    int *st = cell_start + F.cell0;
    __shared__ int wsum[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < n ? cnt[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            int s = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, s, o);
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
}

__global__ void nepnb_fill(const NepFrame *__restrict__ fr, int nframes, long long natoms,
                           const int *__restrict__ cell_of, const int *__restrict__ cell_start,
                           int *__restrict__ cell_fill, int *__restrict__ cell_atoms,
                           const int *gate) {
    if (gate && *gate == 0) return;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < natoms;
         t += (long long)gridDim.x * blockDim.x) {
        const int cell = cell_of[t];
        if (cell < 0) continue;
        const NepFrame &F = fr[frame_of(fr, nframes, t)];
        const int slot = atomicAdd(cell_fill + F.cell0 + cell, 1);
        cell_atoms[F.atom0 + cell_start[F.cell0 + cell] + slot] = (int)(t - F.atom0);
    }
}

// Per-warp shared scratch of the search: a queue of FP32-prefilter survivors, then (list mode)
// int keys and (x, y, z, r) doubles of the kept pairs, or (typed count mode) per-element counts.
constexpr int kQueue = 64;

__host__ __device__ inline size_t key_bytes(int max_r, int max_a) {
    return ((size_t)(max_r + max_a) * 4 + 15) / 16 * 16;
}
__host__ __device__ inline size_t warp_scratch(bool count, bool typed, int max_r, int max_a,
                                               int ntypes) {
    const size_t q = kQueue * 4;
    if (count) return q + (typed ? ((size_t)2 * ntypes * 4 + 15) / 16 * 16 : 0);
    return q + key_bytes(max_r, max_a) + (size_t)(max_r + max_a) * 32;
}

struct SearchArgs {
    const NepFrame *fr;
    int nframes;
    long long natoms;
    const double *pos;
    const float4 *spos;
    const int *cell_start;
    const int *cell_count;
    const int *cell_atoms;
    const long long *type_map;
    double rc2_r, rc2_a;
    float pre2;              // FP32 pre-filter radius squared
    int max_r, max_a, width, ntypes;
    long long *NN_r, *NN_a, *NL_r, *NL_a;
    double *Ri_r, *Ri_a;
    int *err;
    // skin-list build (Verlet reuse): the kept pairs within rc_r go to skin [natoms, max_r]
    // int32 (global n2, ascending) and their number to skin_cnt; no NL / Ri.  Runs only when
    // *gate != 0.
    int *skin, *skin_cnt;
    float4 *skin_vec;        // optional: the pair vector (x, y, z, 0) at the build, FP32
    const int *gate;
};

struct WarpLists {
    int *queue;
    int *key_r, *key_a;
    double *val_r, *val_a;   // (x, y, z, r) per kept pair
    int *tcount;             // typed counts [2 * ntypes]
};

__device__ __forceinline__ void write_entry(const SearchArgs &A, bool radial, long long n1,
                                            int slot, long long n2, double x, double y, double z,
                                            double r) {
    if (A.skin) {
        if (radial) {
            A.skin[n1 * A.max_r + slot] = (int)n2;
            if (A.skin_vec)
                A.skin_vec[n1 * A.max_r + slot] = make_float4((float)x, (float)y, (float)z, 0.f);
        }
        return;
    }
    const int mx = radial ? A.max_r : A.max_a;
    long long *NL = radial ? A.NL_r : A.NL_a;
    double *Ri = radial ? A.Ri_r : A.Ri_a;
    NL[n1 * mx + slot] = n2;
    double *o = Ri + (n1 * mx + slot) * A.width;
    if (A.width == 4) {
        reinterpret_cast<double2 *>(o)[0] = make_double2(r, x);
        reinterpret_cast<double2 *>(o)[1] = make_double2(y, z);
    } else {
        o[0] = x; o[1] = y; o[2] = z;
    }
}

__device__ __forceinline__ void pad_rows(const SearchArgs &A, long long n1, int cr, int ca,
                                         int lane) {
    for (int s = cr + lane; s < A.max_r; s += 32) {
        A.NL_r[n1 * A.max_r + s] = -1;
        for (int q = 0; q < A.width; ++q) A.Ri_r[(n1 * A.max_r + s) * A.width + q] = 0.0;
    }
    for (int s = ca + lane; s < A.max_a; s += 32) {
        A.NL_a[n1 * A.max_a + s] = -1;
        for (int q = 0; q < A.width; ++q) A.Ri_a[(n1 * A.max_a + s) * A.width + q] = 0.0;
    }
}

template <bool TYPED>
__device__ __forceinline__ void count_types(const SearchArgs &A, const WarpLists &W, long long n2,
                                            bool in_r, bool in_a) {
    if (TYPED && (in_r || in_a)) {
        const int t2 = (int)A.type_map[n2];
        if (t2 >= 0 && t2 < A.ntypes) {
            if (in_r) atomicAdd(&W.tcount[t2], 1);
            if (in_a) atomicAdd(&W.tcount[A.ntypes + t2], 1);
        } else {
            atomicOr(A.err, MATPL_KERR_BAD_TYPE);
        }
    }
}

// Exact FP64 test of the first k (<= 32) queued candidates of atom n1 (cell list: replica
// (0, 0, 0) only), one candidate per lane so that the FP64 pipe runs full warps.  Kept pairs
// are appended to the per-warp lists (list mode) or counted.
template <bool COUNT, bool TYPED>
__device__ __forceinline__ void drain(const SearchArgs &A, const NepFrame &F, const double *p1,
                                      int k, int lane, const WarpLists &W, int &cr, int &ca) {
    const unsigned lt = (1u << lane) - 1u;
    bool in_r = false, in_a = false;
    long long n2 = -1;
    double x = 0, y = 0, z = 0, d2 = 0;
    if (lane < k) {
        n2 = F.atom0 + W.queue[lane];
        const double p2[3] = {A.pos[3 * n2], A.pos[3 * n2 + 1], A.pos[3 * n2 + 2]};
        d2 = F.ortho ? exact_pair_ortho(F.box, p1, p2, F.zdelta, x, y, z)
                     : exact_pair(F.box, p1, p2, F.zdelta, x, y, z);
        in_r = d2 < A.rc2_r;
        in_a = d2 < A.rc2_a;
    }
    const unsigned br = __ballot_sync(0xffffffffu, in_r);
    const unsigned ba = __ballot_sync(0xffffffffu, in_a);
    if (COUNT) {
        count_types<TYPED>(A, W, n2, in_r, in_a);
    } else {
        const double r = (A.width == 4 && (in_r || in_a)) ? sqrt(d2) : 0.0;
        if (in_r) {
            const int slot = cr + __popc(br & lt);
            if (slot < A.max_r) {
                W.key_r[slot] = (int)(n2 - F.atom0);
                double *v = W.val_r + 4 * slot;
                v[0] = x; v[1] = y; v[2] = z; v[3] = r;
            }
        }
        if (in_a) {
            const int slot = ca + __popc(ba & lt);
            if (slot < A.max_a) {
                W.key_a[slot] = (int)(n2 - F.atom0);
                double *v = W.val_a + 4 * slot;
                v[0] = x; v[1] = y; v[2] = z; v[3] = r;
            }
        }
    }
    cr += __popc(br);
    ca += __popc(ba);
}

// COUNT: only count neighbors (calculate_maxneigh); TYPED: counts per neighbor element.
template <bool COUNT, bool TYPED>
__global__ void __launch_bounds__(128) nepnb_search(SearchArgs A, int warps_per_block) {
    if (A.gate && *A.gate == 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const size_t per_warp = warp_scratch(COUNT, TYPED, A.max_r, A.max_a, A.ntypes);
    unsigned char *mine = smem + per_warp * wib;
    WarpLists W;
    W.queue = reinterpret_cast<int *>(mine);
    unsigned char *rest = mine + kQueue * 4;
    W.tcount = reinterpret_cast<int *>(rest);
    W.key_r = reinterpret_cast<int *>(rest);
    W.key_a = W.key_r + A.max_r;
    W.val_r = reinterpret_cast<double *>(rest + key_bytes(A.max_r, A.max_a));
    W.val_a = W.val_r + 4 * (size_t)A.max_r;

    const long long gw = (long long)blockIdx.x * warps_per_block + wib;
    const long long nw = (long long)gridDim.x * warps_per_block;
    for (long long n1 = gw; n1 < A.natoms; n1 += nw) {
        const NepFrame &F = A.fr[frame_of(A.fr, A.nframes, n1)];
        const double p1[3] = {A.pos[3 * n1], A.pos[3 * n1 + 1], A.pos[3 * n1 + 2]};
        int cr = 0, ca = 0;
        if (TYPED) {
            for (int t = lane; t < 2 * A.ntypes; t += 32) W.tcount[t] = 0;
            __syncwarp();
        }
        if (A.skin && F.mode != 0) {   // the skin list is built for cell-list frames only
            if (lane == 0) {
                A.skin_cnt[n1] = 0;
                atomicOr(A.err, MATPL_KERR_BAD_BOX);
            }
            continue;
        }
        if (F.mode == 0) {
            const float4 s1 = A.spos[n1];
            const float sv[3] = {s1.x, s1.y, s1.z};
            int c1[3];
            for (int k = 0; k < 3; ++k) {
                const float v = sv[k] * F.nc[k];
                c1[k] = v >= 0.f ? min((int)v, F.nc[k] - 1) : 0;   // also maps NaN to 0
            }
            float H[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) H[q] = F.H[q];
            // the 27 neighbor cells, one per lane: start, count and periodic shift, read in
            // parallel; the candidates of all cells are then walked as one flat range, 32 at a
            // time (the kept pairs are rank-sorted by n2 afterwards, so the order of the walk
            // does not matter)
            int cbeg = 0, ccnt = 0, csh = 0;
            if (lane < 27) {
                const int d[3] = {lane / 9 - 1, (lane / 3) % 3 - 1, lane % 3 - 1};
                int c[3], sh[3];
                for (int k = 0; k < 3; ++k) {
                    c[k] = c1[k] + d[k];
                    sh[k] = 0;
                    if (c[k] < 0) { c[k] += F.nc[k]; sh[k] = -1; }
                    if (c[k] >= F.nc[k]) { c[k] -= F.nc[k]; sh[k] = 1; }
                }
                const long long cell = F.cell0 + (c[0] * F.nc[1] + c[1]) * F.nc[2] + c[2];
                cbeg = A.cell_start[cell];
                ccnt = A.cell_count[cell];
                csh = (sh[0] + 1) | ((sh[1] + 1) << 2) | ((sh[2] + 1) << 4);
            }
            int incl = ccnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int excl = incl - ccnt;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            int qn = 0;
            for (int base = 0; base < total; base += 32) {
                const int e = base + lane;
                // the last cell q with excl_q <= e (it holds e: cells with no atoms share
                // their start with the next one)
                int lo = 0, hi = 26;
#pragma unroll
                for (int it = 0; it < 5; ++it) {
                    const int mid = (lo + hi + 1) >> 1;
                    const int em = __shfl_sync(0xffffffffu, excl, mid);
                    if (em <= e) lo = mid; else hi = mid - 1;
                }
                const int q = lo;
                const int qbeg = __shfl_sync(0xffffffffu, cbeg, q);
                const int qex = __shfl_sync(0xffffffffu, excl, q);
                const int qsh = __shfl_sync(0xffffffffu, csh, q);
                bool pass = false;
                int loc = -1;
                if (e < total) {
                    loc = A.cell_atoms[F.atom0 + qbeg + (e - qex)];
                    if (F.atom0 + loc != n1) {
                        const float4 s2 = A.spos[F.atom0 + loc];
                        const float f0 = s2.x + (float)((qsh & 3) - 1) - s1.x,
                                    f1 = s2.y + (float)(((qsh >> 2) & 3) - 1) - s1.y,
                                    f2 = s2.z + (float)(((qsh >> 4) & 3) - 1) - s1.z;
                        const float xf = H[0] * f0 + H[1] * f1 + H[2] * f2;
                        const float yf = H[3] * f0 + H[4] * f1 + H[5] * f2;
                        const float zf = H[6] * f0 + H[7] * f1 + H[8] * f2;
                        pass = xf * xf + yf * yf + zf * zf < A.pre2;
                    }
                }
                const unsigned b = __ballot_sync(0xffffffffu, pass);
                if (pass) W.queue[qn + __popc(b & lt)] = loc;
                qn += __popc(b);
                if (qn >= 32) {
                    __syncwarp();
                    drain<COUNT, TYPED>(A, F, p1, 32, lane, W, cr, ca);
                    const int left = qn - 32;
                    const int v = lane < left ? W.queue[32 + lane] : 0;
                    __syncwarp();
                    if (lane < left) W.queue[lane] = v;
                    __syncwarp();
                    qn = left;
                }
            }
            if (qn > 0) {
                __syncwarp();
                drain<COUNT, TYPED>(A, F, p1, qn, lane, W, cr, ca);
            }
            if (!COUNT) {
                __syncwarp();
                // rank sort by n2 (keys are distinct) and store in order
                for (int pass = 0; pass < 2; ++pass) {
                    const bool radial = pass == 0;
                    const int n = min(radial ? cr : ca, radial ? A.max_r : A.max_a);
                    const int *key = radial ? W.key_r : W.key_a;
                    const double *val = radial ? W.val_r : W.val_a;
                    for (int e = lane; e < n; e += 32) {
                        const int k = key[e];
                        int rank = 0;
                        for (int o = 0; o < n; ++o) rank += key[o] < k;
                        const double *v = val + 4 * e;
                        write_entry(A, radial, n1, rank, F.atom0 + k, v[0], v[1], v[2], v[3]);
                    }
                }
                __syncwarp();
            }
        } else {
            // enumerate (n2, image) in the reference's order; ballots keep that order
            const int nimg = F.rep[0] * F.rep[1] * F.rep[2];
            const long long total = (long long)F.n * nimg;
            const long long self = n1 - F.atom0;
            for (long long base = 0; base < total; base += 32) {
                const long long qq = base + lane;
                bool in_r = false, in_a = false;
                long long n2 = -1;
                double x = 0, y = 0, z = 0, d2 = 0;
                if (qq < total) {
                    const long long j = qq / nimg;
                    const int im = (int)(qq - j * nimg);
                    const int ia = im / (F.rep[1] * F.rep[2]);
                    const int ib = (im / F.rep[2]) % F.rep[1];
                    const int ic = im % F.rep[2];
                    if (!(im == 0 && j == self)) {
                        n2 = F.atom0 + j;
                        double delta[3];
                        replica_delta(F.bo, ia, ib, ic, delta);
                        const double p2[3] = {A.pos[3 * n2], A.pos[3 * n2 + 1], A.pos[3 * n2 + 2]};
                        d2 = exact_pair(F.box, p1, p2, delta, x, y, z);
                        in_r = d2 < A.rc2_r;
                        in_a = d2 < A.rc2_a;
                    }
                }
                const unsigned br = __ballot_sync(0xffffffffu, in_r);
                const unsigned ba = __ballot_sync(0xffffffffu, in_a);
                if (COUNT) {
                    count_types<TYPED>(A, W, n2, in_r, in_a);
                } else {
                    const double r = (A.width == 4 && (in_r || in_a)) ? sqrt(d2) : 0.0;
                    if (in_r) {
                        const int slot = cr + __popc(br & lt);
                        if (slot < A.max_r) write_entry(A, true, n1, slot, n2, x, y, z, r);
                    }
                    if (in_a) {
                        const int slot = ca + __popc(ba & lt);
                        if (slot < A.max_a) write_entry(A, false, n1, slot, n2, x, y, z, r);
                    }
                }
                cr += __popc(br);
                ca += __popc(ba);
            }
        }
        if (COUNT) {
            if (TYPED) {
                __syncwarp();
                for (int t = lane; t < A.ntypes; t += 32) {
                    A.NN_r[n1 * A.ntypes + t] = W.tcount[t];
                    A.NN_a[n1 * A.ntypes + t] = W.tcount[A.ntypes + t];
                }
                __syncwarp();
            } else if (lane == 0) {
                A.NN_r[n1] = cr;
                A.NN_a[n1] = ca;
            }
            continue;
        }
        if (A.skin) {
            if (lane == 0) {
                A.skin_cnt[n1] = min(cr, A.max_r);
                if (cr > A.max_r) atomicOr(A.err, MATPL_KERR_NEIGHBOR_OVERFLOW);
            }
            continue;
        }
        pad_rows(A, n1, min(cr, A.max_r), min(ca, A.max_a), lane);
        if (lane == 0) {
            A.NN_r[n1] = cr;
            A.NN_a[n1] = ca;
            if (cr > A.max_r || ca > A.max_a) atomicOr(A.err, MATPL_KERR_NEIGHBOR_OVERFLOW);
        }
    }
}

// ---- Verlet-skin reuse (MD-style callers) ----------------------------------------------
// The skin list holds, per atom, every n2 within r_list = max(rc) + skin at the positions of
// the last build (ascending, from the cell search above).  While no atom has moved more than
// skin / 2 since that build, every pair inside max(rc) now is in the list, and the filter
// below recomputes each listed pair with the search's own FP64 arithmetic, so its NL / Ri /
// NN equal calculate_neighbor's at the same positions bit for bit (same pairs, same n2 order,
// same values).  The rebuild decision is a device flag that every build kernel reads (the
// displacement rule of pair_matpl.cpp:1096-1110), so a captured step needs no host decision.

__global__ void nepnb_skin_check(long long natoms, double half_skin2,
                                 const double *__restrict__ pos,
                                 const double *__restrict__ x_ref, int *gate,
                                 float4 *__restrict__ delta) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    bool far = false;
    if (t < natoms) {
        double d[3], d2 = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            d[k] = pos[3 * t + k] - x_ref[3 * t + k];
            d2 += d[k] * d[k];
        }
        far = !(d2 <= half_skin2);   // NaN positions rebuild too
        if (delta) delta[t] = make_float4((float)d[0], (float)d[1], (float)d[2], 0.f);
    }
    if (__any_sync(0xffffffffu, far) && (threadIdx.x & 31) == 0) atomicOr(gate, 1);
}

__global__ void nepnb_zero_gated(int *__restrict__ a, int *__restrict__ b, long long n,
                                 const int *gate) {
    if (*gate == 0) return;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        a[t] = 0;
        b[t] = 0;
    }
}

__global__ void nepnb_gate_clear(int *gate, int *nbuild) {
    if (*gate != 0) {
        if (nbuild) *nbuild += 1;
        *gate = 0;
    }
}

// Wrapped fractional coordinates (FP32) of every atom at the current positions, for the
// filter's pre-test; the frame table is the last build's.
__global__ void nepnb_skin_frac(const double *__restrict__ pos, const NepFrame *__restrict__ fr,
                                int nframes, long long natoms, float4 *__restrict__ spos) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < natoms;
         t += (long long)gridDim.x * blockDim.x) {
        const NepFrame &F = fr[frame_of(fr, nframes, t)];
        const float p[3] = {(float)pos[3 * t], (float)pos[3 * t + 1], (float)pos[3 * t + 2]};
        float s[3];
        for (int k = 0; k < 3; ++k) {
            const float v = F.Hinv[3 * k] * p[0] + F.Hinv[3 * k + 1] * p[1] + F.Hinv[3 * k + 2] * p[2];
            s[k] = v - floorf(v);
        }
        spos[t] = make_float4(s[0], s[1], s[2], 0.f);
    }
}

constexpr int kFilterWarps = 8;

// Exact FP64 test of the first k (<= 32) queued skin entries, written in queue order.
__device__ __forceinline__ void skin_drain(const NepFrame &F, const double *__restrict__ pos,
                                           const double *p1, const int *queue, int k, int lane,
                                           long long n1, double rc2_r, double rc2_a, int max_r,
                                           int max_a, int width, long long *__restrict__ NL_r,
                                           long long *__restrict__ NL_a,
                                           double *__restrict__ Ri_r, double *__restrict__ Ri_a,
                                           int &cr, int &ca) {
    const unsigned lt = (1u << lane) - 1u;
    bool in_r = false, in_a = false;
    long long n2 = -1;
    double x = 0, y = 0, z = 0, d2 = 0;
    if (lane < k) {
        n2 = queue[lane];
        const double p2[3] = {pos[3 * n2], pos[3 * n2 + 1], pos[3 * n2 + 2]};
        d2 = F.ortho ? exact_pair_ortho(F.box, p1, p2, F.zdelta, x, y, z)
                     : exact_pair(F.box, p1, p2, F.zdelta, x, y, z);
        in_r = d2 < rc2_r;
        in_a = d2 < rc2_a;
    }
    const unsigned br = __ballot_sync(0xffffffffu, in_r);
    const unsigned ba = __ballot_sync(0xffffffffu, in_a);
    const double r = (width == 4 && (in_r || in_a)) ? sqrt(d2) : 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        const bool radial = pass == 0;
        if (!(radial ? in_r : in_a)) continue;
        const int slot = (radial ? cr : ca) + __popc((radial ? br : ba) & lt);
        const int mx = radial ? max_r : max_a;
        if (slot >= mx) continue;
        (radial ? NL_r : NL_a)[n1 * mx + slot] = n2;
        double *o = (radial ? Ri_r : Ri_a) + (n1 * mx + slot) * width;
        if (width == 4) {
            reinterpret_cast<double2 *>(o)[0] = make_double2(r, x);
            reinterpret_cast<double2 *>(o)[1] = make_double2(y, z);
        } else {
            o[0] = x; o[1] = y; o[2] = z;
        }
    }
    cr += __popc(br);
    ca += __popc(ba);
}

// One warp per atom: the listed pairs inside the cutoffs at the current positions, in list
// order (ascending n2), in calculate_neighbor's layout.  An FP32 pre-test on the fractional
// coordinates (margin far above its error) drops the entries clearly outside the larger cutoff;
// the survivors are queued so that the exact FP64 recomputation runs on full warps.
__global__ void __launch_bounds__(kFilterWarps * 32)
nepnb_skin_filter(const NepFrame *__restrict__ fr, int nframes, long long natoms,
                  const double *__restrict__ pos, const float4 *__restrict__ spos,
                  const int *__restrict__ skin, const int *__restrict__ skin_cnt, int cap,
                  double rc2_r, double rc2_a, float pre2, int max_r, int max_a, int width,
                  long long *__restrict__ NN_r, long long *__restrict__ NN_a,
                  long long *__restrict__ NL_r, long long *__restrict__ NL_a,
                  double *__restrict__ Ri_r, double *__restrict__ Ri_a, int *err) {
    __shared__ int queue_s[kFilterWarps][64];
    const int lane = threadIdx.x & 31;
    int *queue = queue_s[threadIdx.x >> 5];
    const unsigned lt = (1u << lane) - 1u;
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long n1 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; n1 < natoms;
         n1 += nw) {
        const NepFrame &F = fr[frame_of(fr, nframes, n1)];
        const double p1[3] = {pos[3 * n1], pos[3 * n1 + 1], pos[3 * n1 + 2]};
        const float4 s1 = spos[n1];
        float H[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) H[q] = F.H[q];
        const int n = min(skin_cnt[n1], cap);
        int cr = 0, ca = 0, qn = 0;
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            bool pass = false;
            int n2 = -1;
            if (k < n) {
                n2 = skin[n1 * cap + k];
                if (n2 >= 0 && n2 < natoms) {
                    const float4 s2 = spos[n2];
                    float f0 = s2.x - s1.x, f1 = s2.y - s1.y, f2 = s2.z - s1.z;
                    f0 -= rintf(f0);
                    f1 -= rintf(f1);
                    f2 -= rintf(f2);
                    const float xf = H[0] * f0 + H[1] * f1 + H[2] * f2;
                    const float yf = H[3] * f0 + H[4] * f1 + H[5] * f2;
                    const float zf = H[6] * f0 + H[7] * f1 + H[8] * f2;
                    pass = xf * xf + yf * yf + zf * zf < pre2;
                } else {
                    atomicOr(err, MATPL_KERR_BAD_COUNT);
                }
            }
            const unsigned b = __ballot_sync(0xffffffffu, pass);
            if (pass) queue[qn + __popc(b & lt)] = n2;
            qn += __popc(b);
            if (qn >= 32) {
                __syncwarp();
                skin_drain(F, pos, p1, queue, 32, lane, n1, rc2_r, rc2_a, max_r, max_a, width,
                           NL_r, NL_a, Ri_r, Ri_a, cr, ca);
                const int left = qn - 32;
                const int v = lane < left ? queue[32 + lane] : 0;
                __syncwarp();
                if (lane < left) queue[lane] = v;
                __syncwarp();
                qn = left;
            }
        }
        if (qn > 0) {
            __syncwarp();
            skin_drain(F, pos, p1, queue, qn, lane, n1, rc2_r, rc2_a, max_r, max_a, width, NL_r,
                       NL_a, Ri_r, Ri_a, cr, ca);
        }
        __syncwarp();
        for (int s = min(cr, max_r) + lane; s < max_r; s += 32) {
            NL_r[n1 * max_r + s] = -1;
            for (int q = 0; q < width; ++q) Ri_r[(n1 * max_r + s) * width + q] = 0.0;
        }
        for (int s = min(ca, max_a) + lane; s < max_a; s += 32) {
            NL_a[n1 * max_a + s] = -1;
            for (int q = 0; q < width; ++q) Ri_a[(n1 * max_a + s) * width + q] = 0.0;
        }
        if (lane == 0) {
            NN_r[n1] = cr;
            NN_a[n1] = ca;
            if (cr > max_r || ca > max_a) atomicOr(err, MATPL_KERR_NEIGHBOR_OVERFLOW);
        }
    }
}

// The compact MD form: the pair vector now = its FP32 vector at the build plus the two atoms'
// displacements since then (all FP32; no minimum-image fold is needed while every atom stays
// within skin / 2 of its build position), kept when r^2 < rc^2 in FP32; written as int32 NL
// and float4 (r, x, y, z) in list order, count in NN (int32).  Slots past NN are not written.
__global__ void __launch_bounds__(256)
nepnb_skin_filter_compact(long long natoms, const int *__restrict__ skin,
                          const int *__restrict__ skin_cnt, const float4 *__restrict__ skin_vec,
                          const float4 *__restrict__ delta, int cap, float rc2_r, float rc2_a,
                          int max_r, int max_a, int *__restrict__ NN_r, int *__restrict__ NN_a,
                          int *__restrict__ NL_r, int *__restrict__ NL_a,
                          float4 *__restrict__ Ri_r, float4 *__restrict__ Ri_a, int *err) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long n1 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; n1 < natoms;
         n1 += nw) {
        const float4 d1 = delta[n1];
        const int n = min(skin_cnt[n1], cap);
        int cr = 0, ca = 0;
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            bool in_r = false, in_a = false;
            int n2 = -1;
            float x = 0.f, y = 0.f, z = 0.f, r2 = 0.f;
            if (k < n) {
                n2 = skin[n1 * cap + k];
                if (n2 >= 0 && n2 < natoms) {
                    const float4 v = skin_vec[n1 * cap + k];
                    const float4 d2 = delta[n2];
                    x = v.x + (d2.x - d1.x);
                    y = v.y + (d2.y - d1.y);
                    z = v.z + (d2.z - d1.z);
                    r2 = x * x + y * y + z * z;
                    in_r = r2 < rc2_r;
                    in_a = r2 < rc2_a;
                } else {
                    atomicOr(err, MATPL_KERR_BAD_COUNT);
                }
            }
            const unsigned br = __ballot_sync(0xffffffffu, in_r);
            const unsigned ba = __ballot_sync(0xffffffffu, in_a);
            if (in_r || in_a) {
                const float4 o = make_float4(sqrtf(r2), x, y, z);
                const int sr = cr + __popc(br & lt), sa = ca + __popc(ba & lt);
                if (in_r && sr < max_r) {
                    NL_r[n1 * max_r + sr] = n2;
                    Ri_r[n1 * max_r + sr] = o;
                }
                if (in_a && sa < max_a) {
                    NL_a[n1 * max_a + sa] = n2;
                    Ri_a[n1 * max_a + sa] = o;
                }
            }
            cr += __popc(br);
            ca += __popc(ba);
        }
        if (lane == 0) {
            NN_r[n1] = cr;
            NN_a[n1] = ca;
            if (cr > max_r || ca > max_a) atomicOr(err, MATPL_KERR_NEIGHBOR_OVERFLOW);
        }
    }
}

struct Workspace {
    NepFrame *fr;
    float4 *spos;
    int *cell_of, *cell_count, *cell_start, *cell_fill, *cell_atoms;
};

size_t workspace_layout(int nframes, long long natoms, unsigned char *base, Workspace *w) {
    const long long cells = natoms + 27LL * nframes;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes, 256);
        return base ? base + o : nullptr;
    };
    Workspace tmp;
    tmp.fr = (NepFrame *)take(sizeof(NepFrame) * (size_t)nframes);
    tmp.spos = (float4 *)take(sizeof(float4) * (size_t)natoms);
    tmp.cell_of = (int *)take(sizeof(int) * (size_t)natoms);
    tmp.cell_atoms = (int *)take(sizeof(int) * (size_t)natoms);
    tmp.cell_count = (int *)take(sizeof(int) * (size_t)cells);
    tmp.cell_fill = (int *)take(sizeof(int) * (size_t)cells);
    tmp.cell_start = (int *)take(sizeof(int) * (size_t)cells);
    if (w) *w = tmp;
    return off;
}

inline int blocks_for(long long work, int per_block, int cap) {
    long long g = (work + per_block - 1) / per_block;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

int run(int nframes, long long natoms, const long long *num_atom, const long long *type_map,
        int ntypes, const double *box, const double *box_orig, const long long *num_cell,
        const double *pos, double rc_r, double rc_a, int max_r, int max_a, int with_rij,
        bool count_only, bool typed, long long *NN_r, long long *NN_a, long long *NL_r,
        long long *NL_a, double *Ri_r, double *Ri_a, int *err, void *ws, size_t ws_bytes,
        cudaStream_t s) {
    MATPL_REQUIRE(nframes > 0 && natoms >= 0, MATPL_ERR_INVALID, "nframes must be > 0");
    MATPL_REQUIRE(natoms < (1LL << 31), MATPL_ERR_INVALID, "at most 2^31 - 1 atoms");
    MATPL_REQUIRE(rc_r > 0 && rc_a > 0, MATPL_ERR_INVALID, "cutoffs must be positive");
    MATPL_REQUIRE(num_atom && box && box_orig && num_cell && pos && NN_r && NN_a && err,
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE(!typed || (type_map && ntypes > 0 && ntypes <= 1024), MATPL_ERR_INVALID,
                  "typed counts need type_map and 0 < ntypes <= 1024");
    if (!count_only) {
        MATPL_REQUIRE(max_r >= 0 && max_a >= 0, MATPL_ERR_INVALID, "negative max_NN");
        MATPL_REQUIRE(NL_r && NL_a && Ri_r && Ri_a, MATPL_ERR_INVALID, "null output list");
        MATPL_REQUIRE((size_t)(max_r + max_a) * 36 <= 200 * 1024, MATPL_ERR_UNSUPPORTED,
                      "max_NN_radial + max_NN_angular must be <= 5688");
    }
    const size_t need = workspace_layout(nframes, natoms, nullptr, nullptr);
    MATPL_REQUIRE(ws && ws_bytes >= need, MATPL_ERR_INVALID, "workspace too small");
    Workspace w;
    workspace_layout(nframes, natoms, (unsigned char *)ws, &w);
    const long long cells = natoms + 27LL * nframes;
    ProfScope ps(count_only ? "nep_maxneigh" : "nep_neighbor", s);
    cudaMemsetAsync(w.cell_count, 0, sizeof(int) * (size_t)cells, s);
    cudaMemsetAsync(w.cell_fill, 0, sizeof(int) * (size_t)cells, s);
    const double rc_max = rc_r > rc_a ? rc_r : rc_a;
    nepnb_setup<<<1, kSetupThreads, 0, s>>>(num_atom, box, box_orig, num_cell, w.fr, nframes,
                                            natoms, rc_max, err, nullptr);
    if (natoms == 0) return check_launch("nep_neighbor");
    const int g1 = blocks_for(natoms, 256, device_sms() * 16);
    nepnb_bin<<<g1, 256, 0, s>>>(pos, w.fr, nframes, natoms, w.spos, w.cell_of, w.cell_count,
                                 nullptr, nullptr, nullptr);
    nepnb_scan<<<nframes, 1024, 0, s>>>(w.fr, w.cell_count, w.cell_start, nullptr);
    nepnb_fill<<<g1, 256, 0, s>>>(w.fr, nframes, natoms, w.cell_of, w.cell_start, w.cell_fill,
                                  w.cell_atoms, nullptr);
    SearchArgs A;
    A.fr = w.fr; A.nframes = nframes; A.natoms = natoms; A.pos = pos; A.spos = w.spos;
    A.cell_start = w.cell_start; A.cell_count = w.cell_count; A.cell_atoms = w.cell_atoms;
    A.type_map = type_map; A.rc2_r = rc_r * rc_r; A.rc2_a = rc_a * rc_a;
    const float pre = (float)(rc_max * 1.00001) + kPrefilterMargin;
    A.pre2 = pre * pre;
    A.max_r = max_r; A.max_a = max_a; A.width = with_rij ? 4 : 3; A.ntypes = typed ? ntypes : 1;
    A.NN_r = NN_r; A.NN_a = NN_a; A.NL_r = NL_r; A.NL_a = NL_a; A.Ri_r = Ri_r; A.Ri_a = Ri_a;
    A.err = err;
    A.skin = nullptr; A.skin_cnt = nullptr; A.skin_vec = nullptr; A.gate = nullptr;
    const size_t per_warp = warp_scratch(count_only, typed, max_r, max_a, ntypes);
    int wpb = 4;
    while (wpb > 1 && per_warp * wpb > 96 * 1024) wpb >>= 1;
    const size_t smem = align_up(per_warp * wpb, 16);
    const int grid = blocks_for(natoms, wpb, device_sms() * 64);
    if (count_only) {
        if (typed) {
            cudaFuncSetAttribute(nepnb_search<true, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            nepnb_search<true, true><<<grid, 32 * wpb, smem, s>>>(A, wpb);
        } else {
            nepnb_search<true, false><<<grid, 32 * wpb, smem, s>>>(A, wpb);
        }
    } else {
        cudaFuncSetAttribute(nepnb_search<false, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        nepnb_search<false, false><<<grid, 32 * wpb, smem, s>>>(A, wpb);
    }
    return check_launch(count_only ? "matpl_nep_maxneigh" : "matpl_nep_neighbor");
}

int run_skin_update(int nframes, long long natoms, const long long *num_atom, const double *box,
                    const double *box_orig, const long long *num_cell, const double *pos,
                    double r_list, double skin, int cap, int *skin_nbr, int *skin_cnt,
                    double *x_ref, float4 *skin_vec, float4 *delta, int *gate, int *nbuild,
                    int *err, void *ws, size_t ws_bytes, cudaStream_t s) {
    MATPL_REQUIRE(nframes > 0 && natoms >= 0, MATPL_ERR_INVALID, "nframes must be > 0");
    MATPL_REQUIRE(natoms < (1LL << 31), MATPL_ERR_INVALID, "at most 2^31 - 1 atoms");
    MATPL_REQUIRE(r_list > 0 && skin >= 0 && cap >= 1, MATPL_ERR_INVALID,
                  "r_list > 0, skin >= 0 and cap >= 1 required");
    MATPL_REQUIRE((size_t)cap * 36 <= 200 * 1024, MATPL_ERR_UNSUPPORTED,
                  "skin capacity must be <= 5688");
    MATPL_REQUIRE((skin_vec == nullptr) == (delta == nullptr), MATPL_ERR_INVALID,
                  "skin_vec and delta go together");
    MATPL_REQUIRE(aligned16(skin_vec) && aligned16(delta), MATPL_ERR_INVALID,
                  "skin_vec and delta must be 16-byte aligned");
    if (natoms == 0) return MATPL_OK;
    MATPL_REQUIRE(num_atom && box && box_orig && num_cell && pos && skin_nbr && skin_cnt &&
                      x_ref && gate && err,
                  MATPL_ERR_INVALID, "null pointer argument");
    const size_t need = workspace_layout(nframes, natoms, nullptr, nullptr);
    MATPL_REQUIRE(ws && ws_bytes >= need, MATPL_ERR_INVALID, "workspace too small");
    Workspace w;
    workspace_layout(nframes, natoms, (unsigned char *)ws, &w);
    const long long cells = natoms + 27LL * nframes;
    ProfScope ps("nep_skin_update", s);
    const double h = 0.5 * skin;
    nepnb_skin_check<<<(unsigned)((natoms + 255) / 256), 256, 0, s>>>(natoms, h * h, pos, x_ref,
                                                                      gate, delta);
    const int g1 = blocks_for(natoms, 256, device_sms() * 16);
    nepnb_zero_gated<<<blocks_for(cells, 256, device_sms() * 16), 256, 0, s>>>(
        w.cell_count, w.cell_fill, cells, gate);
    nepnb_setup<<<1, kSetupThreads, 0, s>>>(num_atom, box, box_orig, num_cell, w.fr, nframes,
                                            natoms, r_list, err, gate);
    nepnb_bin<<<g1, 256, 0, s>>>(pos, w.fr, nframes, natoms, w.spos, w.cell_of, w.cell_count,
                                 gate, x_ref, delta);
    nepnb_scan<<<nframes, 1024, 0, s>>>(w.fr, w.cell_count, w.cell_start, gate);
    nepnb_fill<<<g1, 256, 0, s>>>(w.fr, nframes, natoms, w.cell_of, w.cell_start, w.cell_fill,
                                  w.cell_atoms, gate);
    SearchArgs A;
    A.fr = w.fr; A.nframes = nframes; A.natoms = natoms; A.pos = pos; A.spos = w.spos;
    A.cell_start = w.cell_start; A.cell_count = w.cell_count; A.cell_atoms = w.cell_atoms;
    A.type_map = nullptr; A.rc2_r = r_list * r_list; A.rc2_a = 0.0;
    const float pre = (float)(r_list * 1.00001) + kPrefilterMargin;
    A.pre2 = pre * pre;
    // width 3: the skin list keeps n2 and the vector, so no pair needs its FP64 root
    A.max_r = cap; A.max_a = 0; A.width = 3; A.ntypes = 1;
    A.NN_r = nullptr; A.NN_a = nullptr; A.NL_r = nullptr; A.NL_a = nullptr;
    A.Ri_r = nullptr; A.Ri_a = nullptr; A.err = err;
    A.skin = skin_nbr; A.skin_cnt = skin_cnt; A.skin_vec = skin_vec; A.gate = gate;
    const size_t per_warp = warp_scratch(false, false, cap, 0, 1);
    int wpb = 4;
    while (wpb > 1 && per_warp * wpb > 96 * 1024) wpb >>= 1;
    const size_t smem = align_up(per_warp * wpb, 16);
    const int grid = blocks_for(natoms, wpb, device_sms() * 64);
    cudaFuncSetAttribute(nepnb_search<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    nepnb_search<false, false><<<grid, 32 * wpb, smem, s>>>(A, wpb);
    nepnb_gate_clear<<<1, 1, 0, s>>>(gate, nbuild);
    return check_launch("matpl_nep_skin_update");
}

int run_skin_filter(int nframes, long long natoms, const double *pos, double rc_r, double rc_a,
                    int max_r, int max_a, int with_rij, int cap, const int *skin_nbr,
                    const int *skin_cnt, long long *NN_r, long long *NN_a, long long *NL_r,
                    long long *NL_a, double *Ri_r, double *Ri_a, int *err, void *ws,
                    size_t ws_bytes, cudaStream_t s) {
    MATPL_REQUIRE(nframes > 0 && natoms >= 0, MATPL_ERR_INVALID, "nframes must be > 0");
    MATPL_REQUIRE(natoms < (1LL << 31), MATPL_ERR_INVALID, "at most 2^31 - 1 atoms");
    MATPL_REQUIRE(rc_r > 0 && rc_a > 0 && cap >= 1 && max_r >= 0 && max_a >= 0,
                  MATPL_ERR_INVALID, "positive cutoffs, cap >= 1 and max_nn >= 0 required");
    if (natoms == 0) return MATPL_OK;
    MATPL_REQUIRE(pos && skin_nbr && skin_cnt && NN_r && NN_a && NL_r && NL_a && Ri_r && Ri_a &&
                      err,
                  MATPL_ERR_INVALID, "null pointer argument");
    const size_t need = workspace_layout(nframes, natoms, nullptr, nullptr);
    MATPL_REQUIRE(ws && ws_bytes >= need, MATPL_ERR_INVALID, "workspace too small");
    Workspace w;
    workspace_layout(nframes, natoms, (unsigned char *)ws, &w);
    ProfScope ps("nep_skin_filter", s);
    nepnb_skin_frac<<<blocks_for(natoms, 256, device_sms() * 16), 256, 0, s>>>(pos, w.fr, nframes,
                                                                             natoms, w.spos);
    const double rc_max = rc_r > rc_a ? rc_r : rc_a;
    const float pre = (float)(rc_max * 1.00001) + kPrefilterMargin;
    const int grid = blocks_for(natoms, kFilterWarps, device_sms() * 32);
    nepnb_skin_filter<<<grid, kFilterWarps * 32, 0, s>>>(
        w.fr, nframes, natoms, pos, w.spos, skin_nbr, skin_cnt, cap, rc_r * rc_r, rc_a * rc_a,
        pre * pre, max_r, max_a, with_rij ? 4 : 3, NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a, err);
    return check_launch("matpl_nep_skin_filter");
}

int run_skin_filter_compact(long long natoms, double rc_r, double rc_a, int max_r, int max_a,
                            int cap, const int *skin_nbr, const int *skin_cnt,
                            const float4 *skin_vec, const float4 *delta, int *NN_r, int *NN_a,
                            int *NL_r, int *NL_a, float4 *Ri_r, float4 *Ri_a, int *err,
                            cudaStream_t s) {
    MATPL_REQUIRE(natoms >= 0 && natoms < (1LL << 31), MATPL_ERR_INVALID,
                  "natoms must be in [0, 2^31)");
    MATPL_REQUIRE(rc_r > 0 && rc_a > 0 && cap >= 1 && max_r >= 0 && max_a >= 0,
                  MATPL_ERR_INVALID, "positive cutoffs, cap >= 1 and max_nn >= 0 required");
    if (natoms == 0) return MATPL_OK;
    MATPL_REQUIRE(skin_nbr && skin_cnt && skin_vec && delta && NN_r && NN_a && NL_r && NL_a &&
                      Ri_r && Ri_a && err,
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE(aligned16(skin_vec) && aligned16(delta) && aligned16(Ri_r) && aligned16(Ri_a),
                  MATPL_ERR_INVALID, "skin_vec, delta and Ri_* must be 16-byte aligned");
    ProfScope ps("nep_skin_filter_compact", s);
    const int grid = blocks_for(natoms, 8, device_sms() * 32);
    nepnb_skin_filter_compact<<<grid, 256, 0, s>>>(
        natoms, skin_nbr, skin_cnt, skin_vec, delta, cap, (float)(rc_r * rc_r),
        (float)(rc_a * rc_a), max_r, max_a, NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a, err);
    return check_launch("matpl_nep_skin_filter_compact");
}

}  // namespace
}  // namespace matpl

using namespace matpl;

extern "C" size_t matpl_nep_neighbor_workspace_bytes(int nframes, long long natoms) {
    if (nframes <= 0 || natoms < 0) return 0;
    return workspace_layout(nframes, natoms, nullptr, nullptr);
}

extern "C" int matpl_nep_neighbor(int nframes, long long natoms, const long long *num_atom,
                                  const double *box, const double *box_orig,
                                  const long long *num_cell, const double *position,
                                  double cutoff_radial, double cutoff_angular, int max_nn_radial,
                                  int max_nn_angular, int with_rij, long long *NN_radial,
                                  long long *NN_angular, long long *NL_radial,
                                  long long *NL_angular, double *Ri_radial, double *Ri_angular,
                                  int *err_dev, void *workspace, size_t workspace_bytes,
                                  void *stream) {
    MATPL_REQUIRE_ON_DEVICE(position, "matpl_nep_neighbor");
    return run(nframes, natoms, num_atom, nullptr, 0, box, box_orig, num_cell, position,
               cutoff_radial, cutoff_angular, max_nn_radial, max_nn_angular, with_rij, false,
               false, NN_radial, NN_angular, NL_radial, NL_angular, Ri_radial, Ri_angular,
               err_dev, workspace, workspace_bytes, as_stream(stream));
}

extern "C" int matpl_nep_maxneigh(int nframes, long long natoms, const long long *num_atom,
                                  const double *box, const double *box_orig,
                                  const long long *num_cell, const double *position,
                                  double cutoff_radial, double cutoff_angular, int ntypes,
                                  const long long *type_map, int with_type, long long *NN_radial,
                                  long long *NN_angular, int *err_dev, void *workspace,
                                  size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE_ON_DEVICE(position, "matpl_nep_maxneigh");
    return run(nframes, natoms, num_atom, type_map, ntypes, box, box_orig, num_cell, position,
               cutoff_radial, cutoff_angular, 0, 0, 1, true, with_type != 0, NN_radial,
               NN_angular, nullptr, nullptr, nullptr, nullptr, err_dev, workspace,
               workspace_bytes, as_stream(stream));
}

extern "C" int matpl_nep_skin_update(int nframes, long long natoms, const long long *num_atom,
                                     const double *box, const double *box_orig,
                                     const long long *num_cell, const double *position,
                                     double r_list, double skin, int cap, int *skin_nbr,
                                     int *skin_cnt, double *x_ref, float *skin_vec,
                                     float *delta, int *gate, int *nbuild, int *err_dev,
                                     void *workspace, size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE_ON_DEVICE(position, "matpl_nep_skin_update");
    return run_skin_update(nframes, natoms, num_atom, box, box_orig, num_cell, position, r_list,
                           skin, cap, skin_nbr, skin_cnt, x_ref, (float4 *)skin_vec,
                           (float4 *)delta, gate, nbuild, err_dev, workspace, workspace_bytes,
                           as_stream(stream));
}

extern "C" int matpl_nep_skin_filter(int nframes, long long natoms, const double *position,
                                     double cutoff_radial, double cutoff_angular,
                                     int max_nn_radial, int max_nn_angular, int with_rij,
                                     int cap, const int *skin_nbr, const int *skin_cnt,
                                     long long *NN_radial, long long *NN_angular,
                                     long long *NL_radial, long long *NL_angular,
                                     double *Ri_radial, double *Ri_angular, int *err_dev,
                                     void *workspace, size_t workspace_bytes, void *stream) {
    MATPL_REQUIRE_ON_DEVICE(position, "matpl_nep_skin_filter");
    return run_skin_filter(nframes, natoms, position, cutoff_radial, cutoff_angular,
                           max_nn_radial, max_nn_angular, with_rij, cap, skin_nbr, skin_cnt,
                           NN_radial, NN_angular, NL_radial, NL_angular, Ri_radial, Ri_angular,
                           err_dev, workspace, workspace_bytes, as_stream(stream));
}

extern "C" int matpl_nep_skin_filter_compact(long long natoms, double cutoff_radial,
                                             double cutoff_angular, int max_nn_radial,
                                             int max_nn_angular, int cap, const int *skin_nbr,
                                             const int *skin_cnt, const float *skin_vec,
                                             const float *delta, int *NN_radial,
                                             int *NN_angular, int *NL_radial, int *NL_angular,
                                             float *Ri_radial, float *Ri_angular, int *err_dev,
                                             void *stream) {
    MATPL_REQUIRE_ON_DEVICE(skin_nbr, "matpl_nep_skin_filter_compact");
    return run_skin_filter_compact(natoms, cutoff_radial, cutoff_angular, max_nn_radial,
                                   max_nn_angular, cap, skin_nbr, skin_cnt,
                                   (const float4 *)skin_vec, (const float4 *)delta, NN_radial,
                                   NN_angular, NL_radial, NL_angular, (float4 *)Ri_radial,
                                   (float4 *)Ri_angular, err_dev, as_stream(stream));
}
