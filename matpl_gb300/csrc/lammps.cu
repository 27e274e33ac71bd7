// LAMMPS pair-style support for DP models, on the GPU.
//
// matpl_lammps_dp_neighbors replaces PairMATPL::generate_neighdata
// (src/lmps/lammps-libtorch/MATPL/pair_matpl.cpp:522-616), which builds on the host, every
// step, the per-type neighbor slots the TorchScript DP forward takes, from LAMMPS' full list
// over local and ghost atoms.  For every local atom i = ilist[ii] and every j of its list, in
// list order: d = x_j - x_i, rsq = dx dx + dy dy + dz dz (source operation order, no FMA);
// j is kept when rsq <= rc^2, in the block of j's model type, at the next free slot of that
// block (so slots keep the list order).  list_neigh = j + 1 (j may be a ghost atom),
// image_dr = (sqrt(rsq), dx, dy, dz), empty slots 0; type_map[ii] = model type of i; min_rsq =
// the smallest kept rsq (the reference stops the run when it is below 0.61).  One warp per
// local atom walks its list 32 entries at a time; a ballot per type gives each kept neighbor
// its slot in list order.  A block longer than m sets MATPL_KERR_NEIGHBOR_OVERFLOW (the
// reference writes past the block).
//
// The matpl_lammps_dp_* handle replaces the DP branch of PairMATPL::compute
// (pair_matpl.cpp:893-996): slot kernel, fused evaluation with ghost rows (matpl_dp_eval) and a
// pack kernel per step.  Two ways to reach LAMMPS' host arrays:
//   direct  (a GPU that reads pageable host memory through the host's page tables, as on
//           Grace): positions, types, ilist and numneigh are copied in with plain
//           cudaMemcpyAsync from LAMMPS' own arrays, the slot kernel reads every list in place
//           through firstneigh, and the pack kernel writes the forces straight into atom->f and
//           the energy / virial / Ei into mapped pinned memory.  No host-side packing.
//   staged  (elsewhere): the host packs positions, types and the list into pinned memory, one
//           host-to-device copy, one device-to-host copy of the packed results.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace matpl {
namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

constexpr double kNoPair = 1e300;

// the list of row ii (local atom i): packed rows (jstart / jflat, device) ...
struct CsrLists {
    const long long *jstart;
    const int *jflat;
    __device__ __forceinline__ const int *row(long long ii, int, long long &n) const {
        const long long a = jstart[ii];
        n = jstart[ii + 1] - a;
        return jflat + a;
    }
};
// ... or LAMMPS' own numneigh[i] / firstneigh[i] (host memory read in place)
struct LammpsLists {
    const int *numneigh;
    const int *const *firstneigh;
    __device__ __forceinline__ const int *row(long long, int i, long long &n) const {
        n = numneigh[i];
        return firstneigh[i];
    }
};

template <typename TO, typename Lists>
__global__ void __launch_bounds__(128)
lmp_neighbors(int inum, int nall, const int *__restrict__ ilist, Lists lists,
              const double *__restrict__ x, const int *__restrict__ type,
              const int *__restrict__ type_to_model, int ntypes_lmp, int nt, int m,
              unsigned long long rc2_bits, int32_t *__restrict__ list_neigh,
              TO *__restrict__ image_dr,
              int32_t *__restrict__ type_map, unsigned long long *__restrict__ min_rsq,
              int32_t *__restrict__ err, int32_t *__restrict__ num_neigh) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const long long S = (long long)nt * m;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long ii = gw; ii < inum; ii += nw) {
        const int i = ilist[ii];
        if (i < 0 || i >= inum) {  // rows are indexed by i (pair_matpl.cpp:589)
            if (lane == 0) atomicOr(err, MATPL_KERR_BAD_COUNT);
            continue;
        }
        const int til = type[i] - 1;
        const int ti = (til >= 0 && til < ntypes_lmp) ? type_to_model[til] : -1;
        if (lane == 0) {
            type_map[ii] = ti;
            if (ti < 0 || ti >= nt) atomicOr(err, MATPL_KERR_BAD_TYPE);
        }
        const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
        int cnt[16];
#pragma unroll
        for (int t = 0; t < 16; ++t) cnt[t] = 0;
        unsigned long long local_min = ubits(kNoPair);
        long long jn;
        const int *jl = lists.row(ii, i, jn);
        const long long row = (long long)i * S;
        for (long long base = 0; base < jn; base += 32) {
            const long long jj = base + lane;
            bool keep = false;
            int tj = -1, j = 0;
            double dx = 0, dy = 0, dz = 0, rsq = 0;
            if (jj < jn) {
                j = jl[jj];
                if (j >= 0 && j < nall) {
                    const int tl = type[j] - 1;
                    tj = (tl >= 0 && tl < ntypes_lmp) ? type_to_model[tl] : -1;
                    dx = da(x[3 * j], -xi);
                    dy = da(x[3 * j + 1], -yi);
                    dz = da(x[3 * j + 2], -zi);
                    rsq = da(da(dm(dx, dx), dm(dy, dy)), dm(dz, dz));
                    keep = ubits(rsq) <= rc2_bits;
                    if (keep && (tj < 0 || tj >= nt)) {
                        atomicOr(err, MATPL_KERR_BAD_TYPE);
                        keep = false;
                    }
                } else {
                    atomicOr(err, MATPL_KERR_BAD_COUNT);
                }
            }
            if (keep && ubits(rsq) < local_min) local_min = ubits(rsq);
#pragma unroll
            for (int t = 0; t < 16; ++t) {
                if (t >= nt) break;
                const bool mine = keep && tj == t;
                const unsigned mk = __ballot_sync(0xffffffffu, mine);
                if (mine) {
                    const int slot = cnt[t] + __popc(mk & lt);
                    if (slot < m) {
                        const long long s = row + (long long)t * m + slot;
                        list_neigh[s] = j + 1;
                        TO *o = image_dr + 4 * s;
                        o[0] = pair_r<TO>(rsq);
                        o[1] = conv<TO>(dx);
                        o[2] = conv<TO>(dy);
                        o[3] = conv<TO>(dz);
                    }
                }
                cnt[t] += __popc(mk);
            }
        }
        bool over = false;
#pragma unroll
        for (int t = 0; t < 16; ++t) {
            if (t >= nt) break;
            over |= cnt[t] > m;
            if (num_neigh) {       // occupied-slot form: block lengths instead of zero padding
                if (lane == 0) num_neigh[(long long)i * nt + t] = min(cnt[t], m);
                continue;
            }
            for (int s = cnt[t] + lane; s < m; s += 32) {
                const long long q = row + (long long)t * m + s;
                list_neigh[q] = 0;
                TO *o = image_dr + 4 * q;
                o[0] = o[1] = o[2] = o[3] = TO(0);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long v = __shfl_xor_sync(0xffffffffu, local_min, o);
            local_min = v < local_min ? v : local_min;
        }
        if (lane == 0) {
            if (over) atomicOr(err, MATPL_KERR_NEIGHBOR_OVERFLOW);
            if (local_min < ubits(kNoPair)) atomicMin(min_rsq, local_min);
        }
    }
}

__global__ void lmp_init_min(unsigned long long *min_rsq) {
    *min_rsq = (unsigned long long)__double_as_longlong(kNoPair);
}

template <typename Lists>
int launch_neighbors(int inum, int nall, const int *ilist, Lists lists, const double *x,
                     const int *type, const int *type_to_model, int ntypes_lmp, int nt, int m,
                     double rcut, int out_dtype, int32_t *list_neigh, void *image_dr,
                     int32_t *type_map, double *min_rsq, int32_t *err, cudaStream_t s,
                     int32_t *num_neigh = nullptr) {
    ProfScope ps("lmp_neighbors", s);
    auto *mn = reinterpret_cast<unsigned long long *>(min_rsq);
    lmp_init_min<<<1, 1, 0, s>>>(mn);
    if (inum > 0) {
        long long grid = ((long long)inum + 3) / 4;
        grid = std::min(grid, (long long)device_sms() * 16);
        const double rc2 = rcut * rcut;   // pair_matpl.cpp:536
        const unsigned long long rc2_bits = (unsigned long long)[&] {
            long long b;
            std::memcpy(&b, &rc2, 8);
            return b;
        }();
        if (out_dtype == MATPL_F64)
            lmp_neighbors<double, Lists><<<(int)grid, 128, 0, s>>>(
                inum, nall, ilist, lists, x, type, type_to_model, ntypes_lmp, nt, m, rc2_bits,
                list_neigh, (double *)image_dr, type_map, mn, err, num_neigh);
        else
            lmp_neighbors<float, Lists><<<(int)grid, 128, 0, s>>>(
                inum, nall, ilist, lists, x, type, type_to_model, ntypes_lmp, nt, m, rc2_bits,
                list_neigh, (float *)image_dr, type_map, mn, err, num_neigh);
    }
    return check_launch("matpl_lammps_dp_neighbors");
}

// fout [nall x 3] = forces; tail = [Ei (inum) | Etot, virial xx yy zz xy xz yz, min_rsq, err].
// The Voigt pairs follow the TorchScript model's upper triangle sum_pairs Rij_a f_c
// (src/model/dp_dp_script.py:417-426) mapped by pair_matpl.cpp:989-994; matpl_dp_eval's
// virial[a*3+c] = sum f_a Rij_c, so xy / xz / yz are its entries 3, 6, 7.
template <typename T>
__global__ void lmp_pack(long long nall3, int inum, const T *__restrict__ force,
                         const T *__restrict__ Ei, const double *__restrict__ Etot,
                         const double *__restrict__ virial, const double *__restrict__ min_rsq,
                         const int32_t *__restrict__ err, double *__restrict__ fout,
                         double *__restrict__ tail) {
    const long long n = nall3 + inum;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n + 9;
         k += (long long)gridDim.x * blockDim.x) {
        if (k < nall3) {
            fout[k] = (double)force[k];
            continue;
        }
        const long long q = k - nall3;
        double v;
        if (q < inum) {
            v = (double)Ei[q];
        } else {
            const int r = (int)(q - inum);
            const int voigt[6] = {0, 4, 8, 3, 6, 7};
            v = r == 0 ? Etot[0] : r <= 6 ? virial[voigt[r - 1]] : r == 7 ? *min_rsq
                                                                          : (double)*err;
        }
        tail[q] = v;
    }
}

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    bool ensure(size_t bytes) {
        if (bytes <= cap) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(align_up(bytes + bytes / 4, 256), 256);
        if (cudaMalloc(&p, want) != cudaSuccess) return false;
        cap = want;
        return true;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

// pinned, mapped host memory: p for the host, dev for kernels
struct HostBuf {
    void *p = nullptr, *dev = nullptr;
    size_t cap = 0;
    bool ensure(size_t bytes) {
        if (bytes <= cap) return true;
        if (p) cudaFreeHost(p);
        p = dev = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(align_up(bytes + bytes / 4, 256), 256);
        if (cudaHostAlloc(&p, want, cudaHostAllocMapped) != cudaSuccess) return false;
        if (cudaHostGetDevicePointer(&dev, p, 0) != cudaSuccess) {
            cudaFreeHost(p);
            p = nullptr;
            return false;
        }
        cap = want;
        return true;
    }
    ~HostBuf() {
        if (p) cudaFreeHost(p);
    }
};

}  // namespace
}  // namespace matpl

using namespace matpl;

struct matpl_lammps_dp {
    int dtype = MATPL_F64;
    matpl_dp_model model{};                 // the first model (also models[0])
    std::vector<matpl_dp_model> models;
    int ntypes_lmp = 0;
    int eatom_grouped = 0;
    int host_access = MATPL_LMP_STAGED;
    std::vector<int> t2m;
    cudaStream_t stream = nullptr;
    int32_t *err = nullptr;
    int *d_t2m = nullptr;
    DevBuf din, ln, idr, tmap, nn, Ei, Etot, force, vir, mn, out, ws;
    HostBuf hin, hout;
    ~matpl_lammps_dp() {
        if (stream) cudaStreamSynchronize(stream);
        if (err) cudaFree(err);
        if (d_t2m) cudaFree(d_t2m);
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" int matpl_lammps_dp_neighbors(int inum, int nall, const int *ilist,
                                         const long long *jstart, const int *jflat,
                                         const double *x, const int *type,
                                         const int *type_to_model, int ntypes_lmp,
                                         int model_ntypes, int m, double rcut, int out_dtype,
                                         int32_t *list_neigh, void *image_dr, int32_t *type_map,
                                         double *min_rsq, int32_t *err_dev, void *stream) {
    MATPL_REQUIRE(inum >= 0 && nall >= inum, MATPL_ERR_INVALID, "need 0 <= inum <= nall");
    MATPL_REQUIRE(model_ntypes >= 1 && model_ntypes <= 16 && m > 0 && ntypes_lmp >= 1,
                  MATPL_ERR_INVALID, "model_ntypes must be 1..16, m > 0, ntypes_lmp >= 1");
    MATPL_REQUIRE(rcut > 0, MATPL_ERR_INVALID, "rcut must be positive");
    MATPL_REQUIRE(out_dtype == MATPL_F32 || out_dtype == MATPL_F64, MATPL_ERR_DTYPE,
                  "image_dr is f32 or f64");
    MATPL_REQUIRE(ilist && jstart && x && type && type_to_model && list_neigh && image_dr &&
                      type_map && min_rsq && err_dev && (jflat || inum == 0),
                  MATPL_ERR_INVALID, "null pointer argument");
    MATPL_REQUIRE_ON_DEVICE(list_neigh, "matpl_lammps_dp_neighbors");
    return launch_neighbors(inum, nall, ilist, CsrLists{jstart, jflat}, x, type, type_to_model,
                            ntypes_lmp, model_ntypes, m, rcut, out_dtype, list_neigh, image_dr,
                            type_map, min_rsq, err_dev, as_stream(stream));
}

extern "C" int matpl_lammps_dp_create(int dtype, const matpl_dp_model *model, int ntypes_lmp,
                                      const int *type_to_model, int eatom_grouped,
                                      int host_access, matpl_lammps_dp **handle) {
    MATPL_REQUIRE(handle, MATPL_ERR_INVALID, "handle is NULL");
    *handle = nullptr;
    MATPL_REQUIRE(dtype >= MATPL_F32 && dtype <= MATPL_MIXED_TANHF, MATPL_ERR_DTYPE,
                  "unknown dtype");
    MATPL_REQUIRE(model && model->params && model->davg && model->dstd, MATPL_ERR_INVALID,
                  "model and its parameter pointers are required");
    MATPL_REQUIRE(model->ntypes >= 1 && model->ntypes <= 8 && model->m > 0, MATPL_ERR_INVALID,
                  "model ntypes must be 1..8 and m > 0");
    MATPL_REQUIRE(ntypes_lmp >= 1 && ntypes_lmp <= model->ntypes && type_to_model,
                  MATPL_ERR_INVALID, "need 1 <= LAMMPS types <= model types (pair_coeff)");
    MATPL_REQUIRE(host_access >= MATPL_LMP_AUTO && host_access <= MATPL_LMP_DIRECT,
                  MATPL_ERR_INVALID, "host_access is MATPL_LMP_AUTO, _STAGED or _DIRECT");
    std::vector<int> t2m(type_to_model, type_to_model + ntypes_lmp);
    for (int a = 0; a < ntypes_lmp; ++a) {
        MATPL_REQUIRE(t2m[a] >= 0 && t2m[a] < model->ntypes, MATPL_ERR_INVALID,
                      "type_to_model entry outside the model's types");
        for (int b = 0; b < a; ++b)
            MATPL_REQUIRE(t2m[a] != t2m[b], MATPL_ERR_INVALID,
                          "two LAMMPS types map to the same model type");
    }
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
        set_error("matpl_lammps_dp_create: no CUDA device");
        return MATPL_ERR_CUDA;
    }
    MATPL_REQUIRE(host_access != MATPL_LMP_DIRECT || pageable, MATPL_ERR_UNSUPPORTED,
                  "this GPU cannot read pageable host memory (MATPL_LMP_DIRECT)");
    auto *h = new matpl_lammps_dp();
    h->dtype = dtype;
    h->model = *model;
    // the TorchScript model gets atom_type = the pair_coeff elements in LAMMPS type order
    // (pair_matpl.cpp:913), so its image types are type_to_model in that order
    h->model.npresent = ntypes_lmp;
    for (int a = 0; a < 8; ++a) h->model.present[a] = a < ntypes_lmp ? t2m[a] : 0;
    h->ntypes_lmp = ntypes_lmp;
    h->eatom_grouped = eatom_grouped;
    h->host_access = (host_access == MATPL_LMP_DIRECT ||
                      (host_access == MATPL_LMP_AUTO && pageable))
                         ? MATPL_LMP_DIRECT
                         : MATPL_LMP_STAGED;
    h->t2m = t2m;
    bool ok = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&h->err, sizeof(int32_t)) == cudaSuccess &&
              cudaMalloc(&h->d_t2m, sizeof(int) * ntypes_lmp) == cudaSuccess &&
              cudaMemcpy(h->d_t2m, t2m.data(), sizeof(int) * ntypes_lmp,
                         cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemset(h->err, 0, sizeof(int32_t)) == cudaSuccess;
    if (!ok) {
        delete h;
        set_error("matpl_lammps_dp_create: CUDA allocation failed");
        return MATPL_ERR_CUDA;
    }
    h->model.err_dev = h->err;
    h->models.push_back(h->model);
    *handle = h;
    return MATPL_OK;
}

extern "C" int matpl_lammps_dp_add_model(matpl_lammps_dp *h, const matpl_dp_model *model) {
    MATPL_REQUIRE(h && model && model->params && model->davg && model->dstd, MATPL_ERR_INVALID,
                  "handle, model and its parameter pointers are required");
    // the slots are built once with the first model's cutoff and maxNeighborNum
    // (pair_matpl.cpp:536, 550), so every model must share them and the type count
    MATPL_REQUIRE(model->ntypes == h->model.ntypes && model->m == h->model.m &&
                      model->rmax == h->model.rmax,
                  MATPL_ERR_INVALID, "models of one pair style share ntypes, m and Rmax");
    matpl_dp_model m = *model;
    m.npresent = h->model.npresent;
    for (int a = 0; a < 8; ++a) m.present[a] = h->model.present[a];
    m.err_dev = h->err;
    h->models.push_back(m);
    return MATPL_OK;
}

extern "C" int matpl_lammps_dp_num_models(const matpl_lammps_dp *h) {
    return h ? (int)h->models.size() : -1;
}

extern "C" int matpl_lammps_dp_host_access(const matpl_lammps_dp *handle) {
    return handle ? handle->host_access : -1;
}

extern "C" void matpl_lammps_dp_destroy(matpl_lammps_dp *handle) { delete handle; }

extern "C" int matpl_lammps_dp_compute_models(matpl_lammps_dp *h, int nmodels, int nlocal,
                                              int nghost, int inum, const int *ilist,
                                              const int *numneigh, const int *const *firstneigh,
                                              const double *x, const int *type, double *f,
                                              double *eng, double *virial, double *eatom,
                                              double *min_rsq) {
    MATPL_REQUIRE(h, MATPL_ERR_INVALID, "handle is NULL");
    MATPL_REQUIRE(nmodels >= 1 && nmodels <= (int)h->models.size(), MATPL_ERR_INVALID,
                  "nmodels must be 1 .. the handle's model count");
    MATPL_REQUIRE(nlocal >= 0 && nghost >= 0 && inum == nlocal, MATPL_ERR_INVALID,
                  "a full list over the local atoms is required (inum == nlocal)");
    if (min_rsq) *min_rsq = kNoPair;
    if (inum == 0) return MATPL_OK;  // pair_matpl.cpp:906: nothing is written
    MATPL_REQUIRE(ilist && numneigh && firstneigh && x && type && f, MATPL_ERR_INVALID,
                  "null pointer argument");
    const bool direct = h->host_access == MATPL_LMP_DIRECT;
    const int nall = nlocal + nghost;
    const int nt = h->model.ntypes, m = h->model.m;
    const long long S = (long long)nt * m;
    const bool f64 = h->dtype == MATPL_F64;
    const size_t es = f64 ? 8 : 4;
    long long tot = 0;
    for (int ii = 0; ii < inum; ++ii) {
        const int i = ilist[ii];
        MATPL_REQUIRE(i >= 0 && i < inum, MATPL_ERR_INVALID, "ilist entry outside [0, inum)");
        MATPL_REQUIRE(numneigh[i] >= 0, MATPL_ERR_INVALID, "negative numneigh");
        tot += numneigh[i];
    }
    // device input: x | type | ilist | (staged: jstart | jflat, direct: numneigh)
    const size_t o_x = 0, o_ty = align_up(o_x + 24 * (size_t)nall, 16);
    const size_t o_il = align_up(o_ty + 4 * (size_t)nall, 16);
    const size_t o_js = align_up(o_il + 4 * (size_t)inum, 16);
    const size_t o_jf = align_up(o_js + 8 * ((size_t)inum + 1), 16);
    const size_t in_bytes = direct ? align_up(o_js + 4 * (size_t)inum, 16)
                                   : align_up(o_jf + 4 * (size_t)tot, 16);
    const size_t tail_n = (size_t)inum + 9;
    const size_t out_n = 3 * (size_t)nall + tail_n;
    const size_t nm = (size_t)nmodels;
    const size_t ws_bytes = matpl_dp_workspace_bytes(h->dtype, 1, inum);
    bool ok = h->din.ensure(in_bytes) && h->hout.ensure(8 * out_n * nm) &&
              (direct || (h->hin.ensure(in_bytes) && h->out.ensure(8 * out_n * nm))) &&
              h->ln.ensure(4 * S * inum) && h->idr.ensure(es * 4 * S * inum) &&
              h->tmap.ensure(4 * (size_t)inum) && h->nn.ensure(4 * (size_t)nt * inum) &&
              h->Ei.ensure(es * inum) &&
              h->Etot.ensure(8) && h->force.ensure(es * 3 * (size_t)nall) &&
              h->vir.ensure(72) && h->mn.ensure(8) && h->ws.ensure(std::max<size_t>(ws_bytes, 16));
    MATPL_REQUIRE(ok, MATPL_ERR_CUDA, "matpl_lammps_dp_compute: CUDA allocation failed");
    cudaStream_t s = h->stream;
    char *dp = (char *)h->din.p;
    const int out_dtype = f64 ? MATPL_F64 : MATPL_F32;
    int rc;
    // block lengths of rows that ilist does not name stay 0
    MATPL_REQUIRE(cudaMemsetAsync(h->nn.p, 0, 4 * (size_t)nt * inum, s) == cudaSuccess,
                  MATPL_ERR_CUDA, "matpl_lammps_dp_compute: memset failed");
    if (direct) {
        // LAMMPS' arrays as they are: positions / types / ilist / numneigh copied in, the lists
        // read in place through firstneigh
        bool c = cudaMemcpyAsync(dp + o_x, x, 24 * (size_t)nall, cudaMemcpyHostToDevice, s) ==
                     cudaSuccess &&
                 cudaMemcpyAsync(dp + o_ty, type, 4 * (size_t)nall, cudaMemcpyHostToDevice, s) ==
                     cudaSuccess &&
                 cudaMemcpyAsync(dp + o_il, ilist, 4 * (size_t)inum, cudaMemcpyHostToDevice, s) ==
                     cudaSuccess &&
                 cudaMemcpyAsync(dp + o_js, numneigh, 4 * (size_t)inum, cudaMemcpyHostToDevice,
                                 s) == cudaSuccess &&
                 cudaMemsetAsync(h->err, 0, sizeof(int32_t), s) == cudaSuccess;
        MATPL_REQUIRE(c, MATPL_ERR_CUDA, "matpl_lammps_dp_compute: host-to-device copy failed");
        rc = launch_neighbors(inum, nall, (const int *)(dp + o_il),
                              LammpsLists{(const int *)(dp + o_js), firstneigh},
                              (const double *)(dp + o_x), (const int *)(dp + o_ty), h->d_t2m,
                              h->ntypes_lmp, nt, m, h->model.rmax, out_dtype, (int32_t *)h->ln.p,
                              h->idr.p, (int32_t *)h->tmap.p, (double *)h->mn.p, h->err, s,
                              (int32_t *)h->nn.p);
    } else {
        char *hp = (char *)h->hin.p;
        std::memcpy(hp + o_x, x, 24 * (size_t)nall);
        std::memcpy(hp + o_ty, type, 4 * (size_t)nall);
        std::memcpy(hp + o_il, ilist, 4 * (size_t)inum);
        auto *js = (long long *)(hp + o_js);
        auto *jf = (int *)(hp + o_jf);
        long long off = 0;
        for (int ii = 0; ii < inum; ++ii) {
            const int i = ilist[ii];
            js[ii] = off;
            if (numneigh[i]) std::memcpy(jf + off, firstneigh[i], 4 * (size_t)numneigh[i]);
            off += numneigh[i];
        }
        js[inum] = off;
        if (cudaMemcpyAsync(dp, hp, in_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemsetAsync(h->err, 0, sizeof(int32_t), s) != cudaSuccess) {
            set_error("matpl_lammps_dp_compute: host-to-device copy failed");
            return MATPL_ERR_CUDA;
        }
        rc = launch_neighbors(inum, nall, (const int *)(dp + o_il),
                              CsrLists{(const long long *)(dp + o_js), (const int *)(dp + o_jf)},
                              (const double *)(dp + o_x), (const int *)(dp + o_ty), h->d_t2m,
                              h->ntypes_lmp, nt, m, h->model.rmax, out_dtype, (int32_t *)h->ln.p,
                              h->idr.p, (int32_t *)h->tmap.p, (double *)h->mn.p, h->err, s,
                              (int32_t *)h->nn.p);
    }
    if (rc) return rc;
    // one slot conversion, then every model (pair_matpl.cpp:945-965 runs them one by one).  The
    // slots are kept in their occupied form (per-type block lengths, no zero padding written):
    // the same pairs and arithmetic as the padded list the reference builds
    for (int k = 0; k < nmodels; ++k) {
        rc = matpl_dp_eval_occupied(h->dtype, &h->models[k], 1, inum, (int)S, nghost,
                                    (const int32_t *)h->ln.p, (const int32_t *)h->nn.p, h->idr.p,
                                    (const int32_t *)h->tmap.p, h->Ei.p, (double *)h->Etot.p,
                                    h->force.p, (double *)h->vir.p, h->ws.p, h->ws.cap, s);
        if (rc) return rc;
        // direct: forces straight into f, the rest into mapped pinned memory; staged: all into
        // one device buffer, copied back below
        double *fout = direct ? f + k * 3 * (size_t)nall : (double *)h->out.p + k * out_n;
        double *tdev = direct ? (double *)h->hout.dev + k * tail_n
                              : (double *)h->out.p + k * out_n + 3 * (size_t)nall;
        ProfScope ps("lmp_pack", s);
        const long long n = (long long)out_n;
        const int grid = (int)std::min<long long>((n + 255) / 256, (long long)device_sms() * 8);
        if (f64)
            lmp_pack<double><<<grid, 256, 0, s>>>(3LL * nall, inum, (const double *)h->force.p,
                                                  (const double *)h->Ei.p,
                                                  (const double *)h->Etot.p,
                                                  (const double *)h->vir.p,
                                                  (const double *)h->mn.p, h->err, fout, tdev);
        else
            lmp_pack<float><<<grid, 256, 0, s>>>(3LL * nall, inum, (const float *)h->force.p,
                                                 (const float *)h->Ei.p, (const double *)h->Etot.p,
                                                 (const double *)h->vir.p,
                                                 (const double *)h->mn.p, h->err, fout, tdev);
        if ((rc = check_launch("matpl_lammps_dp_compute"))) return rc;
    }
    bool c = direct || cudaMemcpyAsync(h->hout.p, h->out.p, 8 * out_n * nm,
                                       cudaMemcpyDeviceToHost, s) == cudaSuccess;
    if (!c || cudaStreamSynchronize(s) != cudaSuccess) {
        set_error(std::string("matpl_lammps_dp_compute: ") +
                  cudaGetErrorString(cudaGetLastError()));
        return MATPL_ERR_CUDA;
    }
    const double *o = (const double *)h->hout.p;
    // the error word of the last model's pack holds every kernel's flags of this call
    const double *last = direct ? o + (nm - 1) * tail_n
                                : o + (nm - 1) * out_n + 3 * (size_t)nall;
    const int kerr = (int)last[inum + 8];
    if (kerr) {
        set_error("matpl_lammps_dp_compute: kernel error code " + std::to_string(kerr) +
                  (kerr == MATPL_KERR_NEIGHBOR_OVERFLOW
                       ? " (more neighbors of one type than maxNeighborNum)"
                       : kerr == MATPL_KERR_BAD_TYPE ? " (atom type outside the pair_coeff map)"
                                                     : " (list index outside the atoms)"));
        return MATPL_ERR_INVALID;
    }
    for (int k = 0; k < nmodels; ++k) {
        const double *t = direct ? o + k * tail_n : o + k * out_n + 3 * (size_t)nall;
        const double *tail = t + inum;
        // pair_matpl.cpp:982-996: forces of local and ghost atoms are set (LAMMPS' reverse
        // communication adds the ghost rows to their owners), energy and Voigt virial
        if (!direct) std::memcpy(f + k * 3 * (size_t)nall, o + k * out_n, 24 * (size_t)nall);
        if (eng) eng[k] = tail[0];
        if (virial)
            for (int q = 0; q < 6; ++q) virial[6 * k + q] = tail[1 + q];
        if (min_rsq && k == 0) *min_rsq = tail[7];
        if (eatom) {
            double *ea = eatom + (size_t)k * inum;
            if (!h->eatom_grouped) {
                std::memcpy(ea, t, 8 * (size_t)inum);
            } else {
                // the TorchScript model returns Ei grouped by image type (dp_dp_script.py:296-311)
                // and pair_matpl.cpp:1000 stores it as is
                int j = 0;
                for (int q = 0; q < h->ntypes_lmp; ++q)
                    for (int ii = 0; ii < inum; ++ii) {
                        const int tl = type[ilist[ii]] - 1;
                        if (tl == q) ea[j++] = t[ii];
                    }
                for (; j < inum; ++j) ea[j] = 0.0;
            }
        }
    }
    return MATPL_OK;
}

extern "C" int matpl_lammps_dp_compute(matpl_lammps_dp *h, int nlocal, int nghost, int inum,
                                       const int *ilist, const int *numneigh,
                                       const int *const *firstneigh, const double *x,
                                       const int *type, double *f, double *eng, double *virial,
                                       double *eatom, double *min_rsq) {
    return matpl_lammps_dp_compute_models(h, 1, nlocal, nghost, inum, ilist, numneigh, firstneigh,
                                          x, type, f, eng, virial, eatom, min_rsq);
}
