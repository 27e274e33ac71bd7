/*
 * matpl_gb300 — C ABI of the GB300-native (sm_103a) DP / NEP evaluation path of MatPL.
 *
 * Every entry point takes raw device pointers, sizes, a dtype code and a cudaStream_t
 * (passed as void*), launches asynchronously on that stream, allocates nothing (scratch is
 * a caller-provided workspace whose size a *_workspace_bytes() query returns) and returns a
 * matpl_status.  Errors found by a kernel (neighbor overflow ...) are written to a
 * caller-provided device int32 (err_dev); the caller reads it after the stream is done.
 * matpl_last_error() gives a message for the last failing call on the calling thread.
 *
 * Layout conventions follow the reference's tensors (row-major, contiguous):
 *   B = configurations in the batch, N = local atoms, S = neighbor slots per atom
 *   (= ntypes * m, per-type blocks of m slots), nghost = ghost atoms (LAMMPS).
 */
#ifndef MATPL_GB300_H
#define MATPL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MATPL_OK = 0,
    MATPL_ERR_INVALID = 1,      /* bad size / pointer / unsupported shape */
    MATPL_ERR_DTYPE = 2,        /* dtype code not supported by this entry point */
    MATPL_ERR_WORKSPACE = 3,    /* workspace smaller than *_workspace_bytes() */
    MATPL_ERR_CUDA = 4,         /* a CUDA runtime call failed (launch, memset) */
    MATPL_ERR_UNSUPPORTED = 5   /* model shape outside the compiled kernels */
} matpl_status;

/* Codes a kernel writes to err_dev (0 = fine). */
#define MATPL_KERR_NEIGHBOR_OVERFLOW 1   /* a type block exceeds m (NeighConst.f90:75-78) */
#define MATPL_KERR_BAD_TYPE 2            /* atom type index outside [0, ntypes) */
#define MATPL_KERR_TIMEOUT 3             /* a bounded tensor-core completion wait gave up */
#define MATPL_KERR_TABLE_RANGE 6         /* compressed model: s outside the table's grid */

/* Compute forms.  MIXED*: FP32 data, embedding and fitting GEMMs on the tensor cores
 * (tcgen05, BF16 operands, FP32 accumulation in TMEM), FP64 energy / virial reductions.
 *   MATPL_MIXED         BF16x3 split operands (hi*hi + hi*lo + lo*hi), hardware tanh.approx.f32
 *   MATPL_MIXED_FAST    single BF16 embedding operands, hardware tanh.approx.f32
 *   MATPL_MIXED_TANHF   BF16x3 split operands, CUDA tanhf */
typedef enum {
    MATPL_F32 = 0,
    MATPL_F64 = 1,
    MATPL_MIXED = 2,
    MATPL_MIXED_FAST = 3,
    MATPL_MIXED_TANHF = 4
} matpl_dtype;

const char *matpl_last_error(void);
int matpl_version(void);

/* Per-kernel timing.  After matpl_profile_begin(max_launches), every kernel launch of this
 * library records a CUDA event pair on its stream (up to max_launches launches).
 * matpl_profile_collect() waits for those events, switches timing off and returns, per kernel
 * name (NUL-terminated, name_len bytes each), the summed milliseconds and launch count. */
int matpl_profile_begin(int max_launches);
int matpl_profile_collect(int max_names, char *names, int name_len, double *total_ms,
                          int *launches, int *n_out);

/* ------------------------------------------------------------------------------------
 * Force / virial custom ops.
 * Replaces CalcOps_cuda::calculateForce (src/op/src/CalcOps.cpp:6-22 -> kernel
 * src/op/kernel/calculateForce.cu:49-142) and its backward (calculateForceGrad.cu:10-90),
 * CalcOps_cuda::calculateVirial (CalcOps.cpp:170-185 -> calculateVirial.cu:19-120) and its
 * backward (calculateVirialGrad.cu:16-92).
 *   list_neigh [B,N,S] int32, 0-based neighbor index, -1 = empty slot
 *   dE         [B,N,4S]    dE/dRi of the normalised environment matrix
 *   Ri_d       [B,N,4S,3]  dRi/dr_i
 *   Rij        [B,N,S,3]   pair vectors (ImageDR[...,1:])
 * Batch stride of force / atom_virial is N+nghost (the shape of the returned tensor).
 * A pointer that a call with these sizes reads or writes is never NULL (MATPL_ERR_INVALID,
 * checked on the host); a call whose outputs are all empty returns MATPL_OK without a CUDA call.
 * ---------------------------------------------------------------------------------- */
int matpl_calc_force(int dtype, const int32_t *list_neigh, const void *dE, const void *Ri_d,
                     const void *F_center, int batch, int natoms, int nslots, int nghost,
                     void *force_out, void *stream);

int matpl_calc_virial(int dtype, const int32_t *list_neigh, const void *dE, const void *Rij,
                      const void *Ri_d, int batch, int natoms, int nslots, int nghost,
                      void *virial_out, void *atom_virial_out, void *stream);

/* grad_dE [B,N,4S] = d(force . grad_force)/d(dE); grad_force [B,N+nghost,3]. */
int matpl_calc_force_grad(int dtype, const int32_t *list_neigh, const void *Ri_d,
                          const void *grad_force, int batch, int natoms, int nslots, int nghost,
                          void *grad_dE, void *stream);

/* grad_dE [B,N,4S] = d(virial . grad_virial)/d(dE); grad_virial [B,9]. */
int matpl_calc_virial_grad(int dtype, const int32_t *list_neigh, const void *Rij,
                           const void *Ri_d, const void *grad_virial, int batch, int natoms,
                           int nslots, void *grad_dE, void *stream);

/* ------------------------------------------------------------------------------------
 * Tabulated embedding.  Replaces CalcOps_cuda::calculateCompress (src/op/src/CalcOps.cpp:331-383,
 * kernels src/op/kernel/calculateCompress.cu:3-55, calculateCompress_grad.cu:3-53):
 *   f2 [nsij] (the [nsij,1] tensor), coefficient [nsij, layer_node, coe_num] highest power first,
 *   coe_num 4 (order 3) or 6 (order 5) -> G [nsij, layer_node].
 * The backward returns grad_f2 [nsij] = sum_i grad_G[s][i] dG[s][i]/df2 directly.
 * NULL for a pointer that the sizes make read or written: MATPL_ERR_INVALID.
 * ---------------------------------------------------------------------------------- */
int matpl_calc_compress(int dtype, const void *f2, const void *coefficient, long long nsij,
                        int layer_node, int coe_num, void *G, void *stream);
int matpl_calc_compress_grad(int dtype, const void *f2, const void *coefficient,
                             const void *grad_G, long long nsij, int layer_node, int coe_num,
                             void *grad_f2, void *stream);

/* ------------------------------------------------------------------------------------
 * DP neighbor search.  Replaces the Fortran NeighConst.find_neighbore
 * (src/pre_data/gen_feature/NeighConst.f90:14-149) as called by
 * src/pre_data/dpuni_data_loader.py:595-650, plus the r column of compute_Ri (:652-716).
 *   frac_pos   [B,N,3] f64 fractional coordinates (wrapped with mod(x+10,1) internally)
 *   lattice    [B,3,3] f64 row vectors
 *   type_map   [N] int32 0-based type of each atom
 *   Rc_type    host array [ntypes] per centre-type cutoff
 * Outputs (fully written):
 *   list_neigh [B,N,ntypes*m] int32, 1-based, 0 = empty; per type ascending j (then image)
 *   image_dr   [B,N,ntypes*m,4] (r, dx, dy, dz), f64 or f32 per out_dtype
 *   num_neigh  [B,N,ntypes] int32 or NULL
 * Index sets and f64 dR are bit-identical to the restatement of the Fortran source.
 * err_dev: MATPL_KERR_NEIGHBOR_OVERFLOW (a type block needs more than m slots),
 * MATPL_KERR_BAD_TYPE, MATPL_KERR_BAD_BOX (a cell so small that natoms x periodic images
 * exceeds 2^31; its lists are left empty).  The arrays must live on the current device.
 * ---------------------------------------------------------------------------------- */
size_t matpl_neighbor_workspace_bytes(int batch, int natoms);
int matpl_neighbor_build(int batch, int natoms, int ntypes, int m_neigh, double Rc_M,
                         const double *Rc_type, const int32_t *type_map, const double *lattice,
                         const double *frac_pos, int out_dtype, int32_t *list_neigh,
                         void *image_dr, int32_t *num_neigh, int32_t *err_dev,
                         void *workspace, size_t workspace_bytes, void *stream);

/* Occupied-slot form of matpl_neighbor_build (no counterpart in the reference, which always
 * zero-fills): the same slots, but only the occupied ones (t*m + k for k < num_neigh[t]) are
 * written and the empty ones are left as they were, which saves most of the list's write
 * traffic.  num_neigh is required; readers take the block lengths from it
 * (matpl_dp_eval_occupied). */
int matpl_neighbor_build_occupied(int batch, int natoms, int ntypes, int m_neigh, double Rc_M,
                                  const double *Rc_type, const int32_t *type_map,
                                  const double *lattice, const double *frac_pos, int out_dtype,
                                  int32_t *list_neigh, void *image_dr, int32_t *num_neigh,
                                  int32_t *err_dev, void *workspace, size_t workspace_bytes,
                                  void *stream);

/* Allocation-free variant of matpl_neighbor_build.  It has no counterpart in the reference.
 * For hosts that cannot give this library device memory (an MD engine's per-step force
 * callback that owns all device memory through its own pool, or a C / Fortran host without a
 * device allocator at hand; cudaMalloc would also stall the whole device every step).  Its
 * scratch is a fixed 4 MiB array inside the library (present on every GPU that loads it, held
 * until the process exits): calls needing more (about 65,000 atoms, batch x natoms) return
 * MATPL_ERR_WORKSPACE without launching.  The first call on a device looks up that array's
 * device address (set-up), so make the first call before any stream capture.  All calls share
 * the array and it keeps the previous call's contents (the call clears what must start at
 * zero itself); calls that overlap on the GPU race on it, so serialise them.  The address
 * looked up at set-up is kept per device ordinal for the life of the process: do not call
 * cudaDeviceReset, and do not switch the device to a context other than its primary one,
 * while this entry point is in use.  Allocates no memory.  Arguments and outputs as
 * matpl_neighbor_build. */
int matpl_neighbor_build_noalloc(int batch, int natoms, int ntypes, int m_neigh, double Rc_M,
                                 const double *Rc_type, const int32_t *type_map,
                                 const double *lattice, const double *frac_pos, int out_dtype,
                                 int32_t *list_neigh, void *image_dr, int32_t *num_neigh,
                                 int32_t *err_dev, void *stream);

/* ------------------------------------------------------------------------------------
 * Environment matrix.  Replaces DP.calculate_Ri (src/model/dp_dp.py:217-302):
 *   Ri [B,N,S,4] = (Ri_raw - davg[t_i]) / dstd[t_i],  Ri_d [B,N,S,4,3] = -dRi/d(dR) / dstd
 * davg/dstd [ntypes, S*4] (the model buffers), type_map [N] 0-based model type.
 * ---------------------------------------------------------------------------------- */
int matpl_env_mat(int dtype, int batch, int natoms, int nslots, const int32_t *type_map,
                  const void *image_dr, const void *davg, const void *dstd, double rmin,
                  double rmax, void *Ri, void *Ri_d, void *stream);

/* ------------------------------------------------------------------------------------
 * Fused DP se_e2_a energy + force + virial.  Replaces DP.forward + calculate_force_virial
 * (src/model/dp_dp.py:167-215, 304-530): environment matrix, embedding nets, descriptor
 * contraction, fitting nets, the adjoint dE/dRi and the force / virial scatter, with the
 * environment matrix and all network activations kept on chip.
 *
 * Compiled network shape: embedding 1->25->25->25 (tanh, residual on equal widths),
 * M2 = 16, fitting 400->50->50->50->1 (tanh, residual layers 2-3).
 * params: device buffer in the packed layout of matpl_gb300/dp.py: pack_params, in the
 * compute dtype (f64 for MATPL_F64, f32 for MATPL_F32 and the MATPL_MIXED* forms).
 * ---------------------------------------------------------------------------------- */
typedef struct {
    int ntypes;             /* model types */
    int m;                  /* maxNeighborNum (slots per neighbor type) */
    int npresent;           /* number of image types (type_nums of dp_dp.py:197) */
    int present[8];         /* model type index of each image type, in image order */
    double rmin, rmax;      /* Rmin, Rmax (config Rm, Rc_M) */
    const void *params;     /* packed network parameters (device) */
    const void *davg;       /* [ntypes,4] per centre type (device, compute dtype) */
    const void *dstd;       /* [ntypes,4] */
    int32_t *err_dev;       /* device int32 for kernel error codes (MATPL_KERR_*), or NULL */
    /* Compressed model (src/user/ckpt_compress.py tables, evaluated like
     * calc_compress_polynomial, src/model/dp_dp.py:572-601); ctable == NULL (zero-initialise
     * the struct) keeps the embedding nets.  ctable: [ntypes^2 * ctab_rows, 25, ctab_order + 1]
     * in the compute dtype (coefficients highest power first); ctab_dx, ctab_smin, ctab_smax:
     * the grid's dx, sij_min, sij_max.  Every form: the table runs in the SIMT embedding
     * kernels (FP32 data for the MATPL_MIXED* forms, whose fitting nets stay on the tensor
     * cores); an s outside the table sets MATPL_KERR_TABLE_RANGE. */
    const void *ctable;
    int ctab_rows;
    int ctab_order;
    double ctab_dx, ctab_smin, ctab_smax;
} matpl_dp_model;

size_t matpl_dp_param_count(int ntypes);
size_t matpl_dp_workspace_bytes(int dtype, int batch, int natoms);

/* type_map [N]: model type index of each atom (atoms whose type is not in present[] get
 * Ei = 0 and contribute nothing, like dp_dp.py:304-342).  list_neigh [B,N,S] int32 1-based,
 * 0 = empty; image_dr [B,N,S,4] in the compute dtype (f32 for MIXED).
 * Outputs: Ei [B,N] (atom order, compute dtype), Etot [B] f64, force [B,N+nghost,3]
 * (compute dtype), virial [B,9] f64 with virial[a*3+c] = sum f_a * Rij_c. */
int matpl_dp_eval(int dtype, const matpl_dp_model *model, int batch, int natoms, int nslots,
                  int nghost, const int32_t *list_neigh, const void *image_dr,
                  const int32_t *type_map, void *Ei, double *Etot, void *force, double *virial,
                  void *workspace, size_t workspace_bytes, void *stream);

/* Tile shape of the MATPL_MIXED* embedding kernels, process-wide (this project's tuning
 * hook; the reference has no tensor-core path).  mixed_group_atoms = centre atoms whose pair
 * rows one CTA walks in 128-row tcgen05 tiles (1..16, capped by shared memory), and
 * mixed_ctas_per_sm = resident CTAs per SM (1..6, as shared memory and registers allow);
 * 0 = automatic (3).  Results do not depend on
 * them (same per-atom arithmetic); matpl_gb300/autotune.py picks them by timing. */
int matpl_dp_set_tuning(int mixed_group_atoms, int mixed_ctas_per_sm);
int matpl_dp_get_tuning(int *mixed_group_atoms, int *mixed_ctas_per_sm);

/* Occupied-slot form of matpl_dp_eval for lists from matpl_neighbor_build_occupied (this
 * project's fused path; the reference always hands the padded list).  num_neigh [B,N,ntypes]
 * int32 gives each type block's length: slots t*m + k with k < num_neigh[t] are read, the
 * rest of list_neigh / image_dr is never touched (it may hold anything).  Same outputs and
 * arithmetic as matpl_dp_eval on the zero-filled list. */
int matpl_dp_eval_occupied(int dtype, const matpl_dp_model *model, int batch, int natoms,
                           int nslots, int nghost, const int32_t *list_neigh,
                           const int32_t *num_neigh, const void *image_dr,
                           const int32_t *type_map, void *Ei, double *Etot, void *force,
                           double *virial, void *workspace, size_t workspace_bytes,
                           void *stream);

/* Bound of every completion wait of the MATPL_MIXED* embedding kernels (this project's own
 * hook; 0 restores the default of 2^24 polls).  A bound below 64 makes each wait a handful of
 * non-suspending checks, which is how the tests make a wait give up on purpose: the kernel
 * then records MATPL_KERR_TIMEOUT in the model's err_dev, stops issuing tensor-core work,
 * drains what it issued, frees its tensor memory and returns (the outputs are invalid). */
int matpl_dp_set_wait_limit(int polls);

/* ------------------------------------------------------------------------------------
 * Force-loss training: the embedding-net part of the second-order parameter gradient.
 * Replaces what the reference gets from torch autograd with create_graph=True through
 * DP.forward / calculate_force_virial (src/model/dp_dp.py:417-530, loss.backward() in
 * src/PWMLFF/dp_mods/dp_trainer.py:172-275).
 * For a loss with gE = dL/dEtot, gF = dL/dF [B,N,3], gV = dL/dVirial [B,9] (or NULL), the
 * force / virial part of dL/dtheta is the parameter gradient of the derivative of E along the
 * input tangent Rdot_s = Ri_d_s (gF_j - gF_i + gV r_s).
 * matpl_dp_dual_forward: per atom A = k sum_s R_s^T G_s and its tangent
 *   A_dot = k sum_s (Rdot_s^T G_s + R_s^T Gdot_s), both [B*N, 4*25] in the compute dtype,
 *   k = 1 / (m * npresent); occupied slots only (add the empty-slot term of A yourself;
 *   its tangent is zero).
 * matpl_dp_dual_backward: given A_bar = dPhi/dA and A_dot_bar = dPhi/dA_dot [B*N, 100],
 *   writes the gradient of Phi w.r.t. the embedding parameters (the first
 *   ntypes^2 * 1400 entries of the packed layout) into grad_embedding, recomputing the
 *   embedding activations slot by slot instead of storing them.
 * list_neigh [B,N,S] int32 1-based (0 = empty), image_dr [B,N,S,4], no ghost atoms;
 * dtype MATPL_F32 or MATPL_F64; model as for matpl_dp_eval (params, davg, dstd).
 * ---------------------------------------------------------------------------------- */
int matpl_dp_dual_forward(int dtype, const matpl_dp_model *model, int batch, int natoms,
                          int nslots, const int32_t *list_neigh, const void *image_dr,
                          const int32_t *type_map, const void *grad_force,
                          const void *grad_virial, void *A, void *A_dot, void *stream);
int matpl_dp_dual_backward(int dtype, const matpl_dp_model *model, int batch, int natoms,
                           int nslots, const int32_t *list_neigh, const void *image_dr,
                           const int32_t *type_map, const void *grad_force,
                           const void *grad_virial, const void *A_bar, const void *A_dot_bar,
                           void *grad_embedding, void *stream);

/* The empty-slot term of A that matpl_dp_dual_forward leaves out (this project's kernels; the
 * reference gets it from the same autograd graph, its empty slots holding the normalised zero
 * row of src/model/dp_dp.py:304-342).  For centre type t_i and each present t_j,
 *   A_pad = k sum_{t_j} n_empty(t_j) R_pad(t_i)^T G_{t_i t_j}(s_pad(t_i)),
 *   R_pad(t_i) = (0 - davg[t_i]) / dstd[t_i], s_pad = its first entry, k = 1 / (m npresent),
 * n_empty(t_j) = m - (occupied slots of type block t_j).
 * matpl_dp_pad_forward: A = A_occ + A_pad [B*N, 100] (A may alias A_occ; atoms whose type is
 *   not in present[] copy A_occ) and n_empty [B*N, npresent] int32 for the reverse.
 * matpl_dp_pad_backward: the gradient of Phi w.r.t. the embedding parameters through A_pad for
 *   A_bar = dPhi/dA: grad_embedding (the first ntypes^2 * 1400 entries of the packed layout) is
 *   written (nets of absent pairs zero).
 * workspace: matpl_dp_pad_workspace_bytes(npresent) bytes (0 for npresent outside 1..8;
 *   a shorter one is MATPL_ERR_WORKSPACE): the backward's FP64 sums over the atoms, kept in
 *   16 copies that different CTAs add into.
 * dtype MATPL_F32 or MATPL_F64; model as for matpl_dp_dual_forward. */
size_t matpl_dp_pad_workspace_bytes(int npresent);
int matpl_dp_pad_forward(int dtype, const matpl_dp_model *model, int batch, int natoms,
                         int nslots, const int32_t *list_neigh, const int32_t *type_map,
                         const void *A_occ, void *A, int32_t *n_empty, void *workspace,
                         size_t workspace_bytes, void *stream);
int matpl_dp_pad_backward(int dtype, const matpl_dp_model *model, int batch, int natoms,
                          int nslots, const int32_t *type_map, const int32_t *n_empty,
                          const void *A_bar, void *grad_embedding, void *workspace,
                          size_t workspace_bytes, void *stream);

/* matpl_dp_desc_dual: per atom the descriptor D = A^T A< and its tangent
 *   D_dot = A_dot^T A< + A^T A_dot< (A, A_dot [natoms, 4, 25], A< = first m2 columns; D, D_dot
 *   [natoms, 25, m2]) - the xyz_scater_a^T xyz_scater_b product of src/model/dp_dp.py:304-330
 *   for the training step's primal and tangent streams.  Output row r holds atom rows[r]
 *   (rows: a permutation of [0, natoms), e.g. the atoms grouped by element so that each
 *   element's fitting net reads one contiguous block; NULL = identity).
 * matpl_dp_desc_dual_grad: its transpose map: grad_A, grad_A_dot [natoms, 4, 25] (written,
 *   atom rows[r] from row r) from grad_D, grad_D_dot [natoms, 25, m2] (either may be NULL =
 *   zero).
 * dtype MATPL_F32 or MATPL_F64; 1 <= m2 <= 25.
 */
int matpl_dp_desc_dual(int dtype, long long natoms, int m2, const long long *rows, const void *A,
                       const void *A_dot, void *D, void *D_dot, void *stream);
int matpl_dp_desc_dual_grad(int dtype, long long natoms, int m2, const long long *rows,
                            const void *A, const void *A_dot, const void *grad_D,
                            const void *grad_D_dot, void *grad_A, void *grad_A_dot, void *stream);

/* matpl_dp_fit_dual: the fitting part of the same step for the rows of one element
 * (src/model/dp_embedding.py:140-163, net 400 -> 50 -> 50 -> 50 -> 1 with resnet_dt): with
 * D, D_dot [nrows, 400] (matpl_dp_desc_dual's rows) and a [nrows] = dL/dE of each row, the
 * net runs on both streams (E, E_dot) and phi = sum_r (a_r E_r + E_dot_r) is differentiated
 * once: grad_D, grad_D_dot [nrows, 400] are written; grad_params (the first B3 + 1 entries of
 * the element's packed fitting block: W0 [400][50], b0, W1 [50][50], b1, dt1, W2, b2, dt2,
 * W3 [50], b3) and *phi (f64) are accumulated (+=, zero them first).  fit_params = the
 * element's packed fitting block (with the transposed matrices).  Scratch:
 * matpl_dp_fit_dual_workspace_bytes(dtype, nrows).  dtype MATPL_F32 or MATPL_F64. */
size_t matpl_dp_fit_dual_workspace_bytes(int dtype, long long nrows);
int matpl_dp_fit_dual(int dtype, long long nrows, const void *fit_params, const void *D,
                      const void *D_dot, const void *a, void *grad_D, void *grad_D_dot,
                      void *grad_params, double *phi, void *workspace, size_t workspace_bytes,
                      void *stream);

/* ------------------------------------------------------------------------------------
 * NEP neighbor lists.  Replaces CalcOps calculate_neighbor / calculate_maxneigh
 * (src/op/src/CalcOps.cpp:1025-1172, kernels src/op/kernel/calculateNepNeighbor.cu:8-380,
 * CPU twin src/op/src/cpu_calculate_nepneighbor.cpp:6-203), bit-identical to the CPU twin.
 * Frames are concatenated: num_atom [B] int64, position [sum N, 3] f64 (cartesian),
 * box [B, 18] f64 (replicated cell h then h^-1, nep_data_loader.py:220-253), box_orig [B, 9]
 * (lattice^T), num_cell [B, 3] int64.
 * matpl_nep_neighbor writes NN_* [N] (full counts), NL_* [N, max_nn] int64 (-1 padded) and
 * Ri_* [N, max_nn, 4] f64 = (r, x, y, z) (3 wide, no r, when with_rij = 0), zero padded.
 * A list longer than max_nn sets MATPL_KERR_NEIGHBOR_OVERFLOW in err_dev (outputs invalid;
 * the reference writes past the end instead).  MATPL_KERR_BAD_BOX flags num_cell < 1.
 * matpl_nep_maxneigh writes only the counts: NN_* [N], or [N, ntypes] per neighbor element
 * when with_type (type_map [N] int64 element index).
 * ---------------------------------------------------------------------------------- */
#define MATPL_KERR_BAD_BOX 4             /* num_cell entry < 1; DP search: natoms x periodic
                                            images of one cell above 2^31 (lists left empty) */
#define MATPL_KERR_BAD_COUNT 5           /* num_atom does not sum to natoms, or a list index
                                            outside [0, natoms) */
size_t matpl_nep_neighbor_workspace_bytes(int nframes, long long natoms);
int matpl_nep_neighbor(int nframes, long long natoms, const long long *num_atom,
                       const double *box, const double *box_orig, const long long *num_cell,
                       const double *position, double cutoff_radial, double cutoff_angular,
                       int max_nn_radial, int max_nn_angular, int with_rij,
                       long long *NN_radial, long long *NN_angular, long long *NL_radial,
                       long long *NL_angular, double *Ri_radial, double *Ri_angular,
                       int *err_dev, void *workspace, size_t workspace_bytes, void *stream);
int matpl_nep_maxneigh(int nframes, long long natoms, const long long *num_atom,
                       const double *box, const double *box_orig, const long long *num_cell,
                       const double *position, double cutoff_radial, double cutoff_angular,
                       int ntypes, const long long *type_map, int with_type,
                       long long *NN_radial, long long *NN_angular, int *err_dev,
                       void *workspace, size_t workspace_bytes, void *stream);

/* Verlet-skin reuse of the NEP lists for MD-style callers (the displacement rule of
 * src/lmps/lammps-libtorch/MATPL/pair_matpl.cpp:1096-1110 applied to calculate_neighbor).
 * The drop-in calculate_neighbor above stays the exact rebuild; these two replace it for a
 * caller that steps one fixed box and passes positions that move a little per call.
 * matpl_nep_skin_update: sets *gate when some |position - x_ref| > skin / 2 (or NaN); then,
 *   only when *gate != 0 (read on the device: the sequence can be captured in a CUDA graph),
 *   rebuilds skin_nbr [natoms, cap] int32 (global n2 ascending, every pair within r_list of
 *   the frame's cell search, r_list >= max cutoff + skin), skin_cnt [natoms] and
 *   x_ref [natoms, 3] = position, clears *gate and increments *nbuild (may be NULL).  Start
 *   with *gate = 1.  A list longer than cap sets MATPL_KERR_NEIGHBOR_OVERFLOW; a frame that is
 *   not a single cell at least three r_list-wide cells thick sets MATPL_KERR_BAD_BOX (use the
 *   exact rebuild for it).  The workspace (matpl_nep_neighbor_workspace_bytes) holds the frame
 *   table of the last build and must be kept, with box / box_orig, until the next rebuild.
 *   skin_vec [natoms, cap, 4] f32 and delta [natoms, 4] f32 (both NULL, or both 16-byte
 *   aligned device arrays) add what the compact filter reads: the FP32 pair vector of every
 *   listed pair at the build, and every call's displacement position - x_ref.
 * matpl_nep_skin_filter: NN / NL / Ri exactly as matpl_nep_neighbor returns them at these
 *   positions (same pairs, same order, same bits), from the skin list and the frame table in
 *   the workspace of the last update (it also writes its per-atom FP32 scratch there).
 * matpl_nep_skin_filter_compact: the MD form, all FP32 (no FP64 pair arithmetic): pair vector
 *   = skin_vec + delta[n2] - delta[n1], kept when r^2 < rc^2; writes NN_* [natoms] int32,
 *   NL_* [natoms, max_nn] int32 (global 0-based n2, ascending) and Ri_* [natoms, max_nn, 4]
 *   f32 (r, x, y, z); slots past NN are left unwritten.  The pair vectors agree with the exact
 *   ones to a few FP32 ulps; a pair within ~1e-6 A of a cutoff may be classified the other
 *   way (its terms vanish there).  matpl_nep_eval_compact evaluates these lists. */
int matpl_nep_skin_update(int nframes, long long natoms, const long long *num_atom,
                          const double *box, const double *box_orig, const long long *num_cell,
                          const double *position, double r_list, double skin, int cap,
                          int *skin_nbr, int *skin_cnt, double *x_ref, float *skin_vec,
                          float *delta, int *gate, int *nbuild, int *err_dev, void *workspace,
                          size_t workspace_bytes, void *stream);
int matpl_nep_skin_filter(int nframes, long long natoms, const double *position,
                          double cutoff_radial, double cutoff_angular, int max_nn_radial,
                          int max_nn_angular, int with_rij, int cap, const int *skin_nbr,
                          const int *skin_cnt, long long *NN_radial, long long *NN_angular,
                          long long *NL_radial, long long *NL_angular, double *Ri_radial,
                          double *Ri_angular, int *err_dev, void *workspace,
                          size_t workspace_bytes, void *stream);
int matpl_nep_skin_filter_compact(long long natoms, double cutoff_radial, double cutoff_angular,
                                  int max_nn_radial, int max_nn_angular, int cap,
                                  const int *skin_nbr, const int *skin_cnt,
                                  const float *skin_vec, const float *delta, int *NN_radial,
                                  int *NN_angular, int *NL_radial, int *NL_angular,
                                  float *Ri_radial, float *Ri_angular, int *err_dev,
                                  void *stream);

/* ------------------------------------------------------------------------------------
 * Fused NEP energy + force + virial.  Replaces NEP.forward + calculate_force_virial
 * (src/model/nep_net.py:293-438, 486-648): descriptor (calculateNepFeat / calculateNepMbFeat,
 * CalcOps.cpp:669-1023), the per-element single-hidden-layer FittingNet
 * (src/model/nep_fitting.py:136-160), dE/dRi and calculateNepForce / calculateNepVirial.
 * Compiled shapes: n_max <= 7, basis_size <= 15, l_max = (4 or 0, 2 or 0, 1 or 0),
 * neuron <= 128, ntypes <= 64.
 * params: device buffer in the layout of matpl_gb300/nep.py: pack_params (compute dtype):
 *   c2 [T,T,n_max_r+1,basis_r+1] | c3 [T,T,n_max_a+1,basis_a+1] | q_scaler [F] |
 *   per element: W0 [F,H] | b0 [H] | W1 [H] | b1
 * ---------------------------------------------------------------------------------- */
typedef struct {
    int ntypes;
    int n_max_radial, basis_radial;     /* NepParam n_max[0], basis_size[0] */
    int n_max_angular, basis_angular;   /* n_max[1], basis_size[1] */
    int l_max_3b, l_max_4b, l_max_5b;   /* l_max */
    int neuron;                         /* hidden units */
    int train_2b;                       /* radial descriptor present */
    double cutoff_radial, cutoff_angular;
    const void *params;                 /* packed parameters (device, compute dtype) */
    int32_t *err_dev;                   /* device int32 for MATPL_KERR_* codes */
} matpl_nep_model;

size_t matpl_nep_param_count(const matpl_nep_model *model);
size_t matpl_nep_workspace_bytes(int dtype, int nframes, long long natoms);

/* dtype MATPL_F32 (FP32 arithmetic, FP64 energy / virial sums) or MATPL_F64.
 * Lists as matpl_nep_neighbor writes them (with_rij = 1); type_map [N] int64 element index.
 * Outputs: Ei [N] and force [N, 3] in the compute dtype, Etot [B] f64, virial [B, 9] f64 with
 * virial[a*3+c] = -sum_pairs (dE/dr_ij)_a (r_ij)_c (the sign NEP.forward returns). */
int matpl_nep_eval(int dtype, const matpl_nep_model *model, int nframes, long long natoms,
                   const long long *num_atom, const long long *type_map, int max_nn_radial,
                   const long long *NN_radial, const long long *NL_radial,
                   const double *Ri_radial, int max_nn_angular, const long long *NN_angular,
                   const long long *NL_angular, const double *Ri_angular, void *Ei,
                   double *Etot, void *force, double *virial, void *workspace,
                   size_t workspace_bytes, void *stream);

/* Descriptor only: feats [N, F] in the compute dtype, before q_scaler (the q of
 * NEP.calculate_qn, src/model/nep_net.py:648-670; feature order [radial n] + [l = 1..4, each
 * all n] + [4-body all n] + [5-body all n]).  Same inputs and workspace as matpl_nep_eval. */
int matpl_nep_descriptor(int dtype, const matpl_nep_model *model, int nframes, long long natoms,
                         const long long *num_atom, const long long *type_map, int max_nn_radial,
                         const long long *NN_radial, const long long *NL_radial,
                         const double *Ri_radial, int max_nn_angular,
                         const long long *NN_angular, const long long *NL_angular,
                         const double *Ri_angular, void *feats, void *workspace,
                         size_t workspace_bytes, void *stream);
/* matpl_nep_eval on the compact MD lists of matpl_nep_skin_filter_compact (int32 NN / NL,
 * 16-byte aligned f32 Ri rows of (r, x, y, z)); dtype MATPL_F32 only.  Same outputs and
 * workspace as matpl_nep_eval. */
int matpl_nep_eval_compact(int dtype, const matpl_nep_model *model, int nframes, long long natoms,
                           const long long *num_atom, const long long *type_map,
                           int max_nn_radial, const int *NN_radial, const int *NL_radial,
                           const float *Ri_radial, int max_nn_angular, const int *NN_angular,
                           const int *NL_angular, const float *Ri_angular, void *Ei,
                           double *Etot, void *force, double *virial, void *workspace,
                           size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------------------
 * Data-path statistics.  Replaces the per-image calc_stat + smooth of
 * src/pre_data/dpuni_data_loader.py:422-563 (davg / dstd of calculate_davg_dstd, :377-420).
 * list_neigh [B,N,S] int32 (1-based, 0 empty), image_dr [B,N,S,4] f64 (r, x, y, z),
 * type_map [N] model type.  sums [B, ntypes, 8] f64 (overwritten): over every slot of the atoms
 * of type t, sum Ri_c and sum Ri_c^2 for c = 0..3, Ri = vv(r) (1/r, x/r^2, y/r^2, z/r^2) with
 * the switching function of smooth (rmin, rmax); r^2 and r are formed from (x, y, z).
 * ---------------------------------------------------------------------------------- */
int matpl_env_stats(int batch, int natoms, int nslots, int ntypes, const int32_t *type_map,
                    const int32_t *list_neigh, const double *image_dr, double rmin, double rmax,
                    double *sums, int32_t *err_dev, void *stream);

/* ------------------------------------------------------------------------------------
 * NEP training operators.  Replace CalcOps calculateNepFeat (part 0, radial) and
 * calculateNepMbFeat (part 1, 3-/4-/5-body) with their Grad functions
 * (src/op/src/CalcOps.cpp:385-1023, kernels calculateNepFeat*.cu / calculateNepMbFeat*.cu).
 * coeff [T, T, n_max, n_base] (the c_param_2 / c_param_3 tensor), d12 [N, max_nn, 4] =
 * (r, x, y, z), NL [N, max_nn] int64 (-1 = empty), type_map [N] int64; dtype MATPL_F32/F64.
 * mode 0 (forward):  q [N, ldQ] = the part's features (radial n_max; angular n_max per
 *                    l = 1..l_max_3b, then the 4-body and 5-body blocks).
 * mode 1 (backward): for G [N, ldG] = dL/dq writes grad_d12 [N, max_nn, 4] = G . dq/dd12
 *                    (partials in the four columns; caller zero-fills) and W, zero-filled by
 *                    the caller: radial [N, T, n_base] = sum over neighbors of type t of
 *                    f_k(r) (dL/dc[t_i, t, n, k] = sum_i G[i, n] W[i, t, k]); angular
 *                    [N, T, n_max, n_base] (dL/dc[t_i] = sum_i W[i]).  Either output may be
 *                    NULL (not computed): the force path needs grad_d12 alone, the energy
 *                    path's coefficient gradient W alone.
 * mode 2 (second backward): for H [N, max_nn, 4] = dL/d(grad_d12) writes q = dq/dd12 . H
 *                    [N, ldQ] (= dL/dG) and W as in mode 1 for dL/dc (radial: sum of
 *                    H_r f_k'(r), to be contracted with G).
 * Compiled for n_max <= 8, n_base <= 16, l_max_3b <= 4, l_max_4b in {0, 2}, l_max_5b in {0, 1}.
 * ---------------------------------------------------------------------------------- */
int matpl_nep_feat_op(int dtype, int part, int mode, int natoms, int max_nn, int ntypes,
                      int n_max, int n_base, int l_max_3b, int l_max_4b, int l_max_5b,
                      double cutoff, const void *coeff, const void *d12, const long long *NL,
                      const long long *type_map, const void *G, long long ldG, const void *H,
                      void *q, long long ldQ, void *grad_d12, void *W, int *err_dev,
                      void *stream);

/* matpl_nep_cgrad: the coefficient gradient dL/dc [ntypes, ntypes, n_max, n_base] (zeroed,
 *   then accumulated) from the per-atom table W of matpl_nep_feat_op's backward modes, summed
 *   over the atoms of each centre type type_map[i] - the grad_coeff2 / grad_coeff3 of the
 *   reference's backward (src/op/src/CalcOps.cpp:534-538, 802-812) and the c-terms of its second
 *   backward (:618, :956).  part 0 (radial): W [natoms, ntypes, n_base],
 *   dc[t_i, tt, n, k] += G[i*ldG + n] * W[i, tt, k]; part 1 (angular): W [natoms, ntypes, n_max,
 *   n_base] already contracted with G, dc[t_i] += W[i] (G unused).  Each block of 64
 *   consecutive atoms sums its atoms of one centre type in shared memory (8 warps' partial
 *   sums), then adds each column to dc with one FP atomic per block, so the order of the
 *   atomics across blocks (and the last bits of dc) may differ between runs.  err_dev gets
 *   MATPL_KERR_BAD_TYPE for a type outside [0, ntypes).
 */
int matpl_nep_cgrad(int dtype, int part, int natoms, int ntypes, int n_max, int n_base,
                    const long long *type_map, const void *G, long long ldG, const void *W,
                    void *dc, int *err_dev, void *stream);

/* matpl_nep_zbl: the ZBL term of NEP (src/model/nep_net.py:399-408, calculate_zbl / cal_zbl
 *   :916-991) added to existing outputs.  For every angular-list slot (NL [natoms, max_nn] int64,
 *   < 0 empty; Ri [natoms, max_nn, 4] (r, x, y, z), ri_dtype MATPL_F64, or MATPL_F32 with dtype
 *   MATPL_F32) with 0 < r <= zbl: x = r s_ij 2.134563, phi = sum_k a_k exp(-b_k x) (universal ZBL
 *   screening), fc = 1 below zbl/2 and 0.5 + 0.5 cos(pi (r - zbl/2) / (zbl/2)) above,
 *   e = c_ij phi fc / r; Ei[i] += e/2, Etot[image_of[i]] += e/2 (Etot may be NULL), and with
 *   f = (1/2) de/dr (x, y, z)/r: force[i] += f, force[j] -= f, virial[image_of[i]] -= f (x) r.
 *   pair_s, pair_c [ntypes, ntypes] f64 = Z_i^0.23 + Z_j^0.23 and 14.399645 Z_i Z_j, float32
 *   values widened to f64 as the reference forms them under torch's default float32 dtype
 *   (the Python layer passes correctly rounded float32 powers).  Ei and force in
 *   dtype, Etot [nimages] and virial [nimages, 9] f64.  err_dev gets MATPL_KERR_BAD_TYPE /
 *   MATPL_KERR_BAD_COUNT.
 */
int matpl_nep_zbl(int dtype, int ri_dtype, long long natoms, int max_nn, int nimages,
                  const long long *NL, const void *Ri, const long long *type_map,
                  const long long *image_of, int ntypes, const double *pair_s,
                  const double *pair_c, double zbl, void *Ei, double *Etot, void *force,
                  double *virial, int *err_dev, void *stream);

/* matpl_nep_force_virial: forces force [natoms, 3] and per-image virial virial [nimages, 9]
 *   (both zeroed, then accumulated) of one NEP list from dE [natoms, max_nn, 4] = dE/d(r, x, y,
 *   z) and the rows Ri [natoms, max_nn, 4] = (r, x, y, z): what calculateNepForce with the centre
 *   term f0 = -sum_s dE . Ri_d and calculateNepVirial's per-image sum give
 *   (src/op/src/CalcOps.cpp:75-168, 239-330; src/model/nep_net.py:612-631) with Ri_d =
 *   calculate_Ri(Ri) (nep_net.py:440-468) formed in registers instead of read from a
 *   [natoms, max_nn, 4, 3] array.  Per slot f_a = dE_0 x_a / r + dE_(1+a) (slots with
 *   |r| <= 1e-5 give 0); force[i] -= f, force[NL] += f (NL int64, < 0 empty); virial[image_of[i]]
 *   [3a + b] += f_a x_b.  err_dev gets MATPL_KERR_BAD_COUNT for a list index >= natoms or an
 *   image index outside [0, nimages).
 * matpl_nep_force_virial_grad: g_dE [natoms, max_nn, 4] (written) from g_force [natoms, 3] and
 *   g_virial [nimages, 9] (either may be NULL = zero), the transpose of the map above.
 */
int matpl_nep_force_virial(int dtype, int natoms, int max_nn, int nimages, const long long *NL,
                           const long long *image_of, const void *dE, const void *Ri, void *force,
                           void *virial, int *err_dev, void *stream);
int matpl_nep_force_virial_grad(int dtype, int natoms, int max_nn, int nimages,
                                const long long *NL, const long long *image_of, const void *Ri,
                                const void *g_force, const void *g_virial, void *g_dE,
                                int *err_dev, void *stream);

/* ------------------------------------------------------------------------------------
 * LAMMPS pair style (DP).  Replaces PairMATPL::generate_neighdata
 * (src/lmps/lammps-libtorch/MATPL/pair_matpl.cpp:522-616) and the DP branch of
 * PairMATPL::compute (pair_matpl.cpp:893-996), which copies the expanded slot arrays to the
 * GPU and runs the TorchScript model (src/model/dp_dp_script.py:137-185) every step.
 *
 * matpl_lammps_dp_neighbors: per-type DP slots from a LAMMPS full list (device pointers).
 *   ilist [inum] local atom of each list row; the list of row ii is jflat[jstart[ii] ..
 *   jstart[ii+1]) (jstart [inum+1] int64), atom indices into x [nall, 3] f64 and
 *   type [nall] (LAMMPS types, 1-based); type_to_model [ntypes_lmp] = model type index of each
 *   LAMMPS type (pair_coeff * * <elements>).  For every j of the list with
 *   rsq = dx*dx + dy*dy + dz*dz <= rcut^2 (d = x_j - x_i, no FMA), in list order: slot
 *   i*S + t_j*m + (count of earlier kept neighbors of type t_j) gets list_neigh = j + 1 and
 *   image_dr = (sqrt(rsq), dx, dy, dz) in out_dtype (MATPL_F32 / MATPL_F64); other slots 0.
 *   type_map[ii] = model type of ilist[ii].  min_rsq (device f64) = smallest kept rsq (1e300 if
 *   none; the reference aborts when it is below 0.61).  err_dev gets
 *   MATPL_KERR_NEIGHBOR_OVERFLOW (a block longer than m; the reference writes past it),
 *   MATPL_KERR_BAD_TYPE or MATPL_KERR_BAD_COUNT (an index outside the atoms).
 *   As in the reference, the row of a list is its local atom i (not ii): LAMMPS' standard
 *   full lists have ilist[ii] = ii.
 *
 * matpl_lammps_dp_create / compute / destroy: the pair style's per-step force call.  create
 *   copies the model struct (params, davg, dstd stay owned by the caller and must outlive the
 *   handle) and sets the image types to type_to_model in LAMMPS type order (the atom_type
 *   tensor pair_matpl.cpp:913 passes).  compute takes LAMMPS' host arrays as they are (inum ==
 *   nlocal, ilist, numneigh and firstneigh indexed by atom, x = atom->x[0] [nall, 3],
 *   type = atom->type) and writes f [nall, 3] (local and ghost rows, replaced, like
 *   pair_matpl.cpp:982-987), *eng = Etot, virial[6] = xx yy zz xy xz yz (pair_matpl.cpp:989-
 *   994), eatom [inum] (or NULL; in list-row order, or grouped by LAMMPS type like the
 *   TorchScript model's Ei when eatom_grouped) and *min_rsq; it returns when they are on the
 *   host.  A kernel error returns MATPL_ERR_INVALID with its code in matpl_last_error().
 *   inum == 0 writes nothing (pair_matpl.cpp:906).
 *   host_access: MATPL_LMP_DIRECT = kernels read the lists in place through firstneigh and
 *   write f in place (needs a GPU that reads pageable host memory, cudaDevAttrPageableMemory-
 *   Access, e.g. Grace; MATPL_ERR_UNSUPPORTED otherwise); MATPL_LMP_STAGED = the host packs
 *   x / type / lists into pinned memory, one copy each way; MATPL_LMP_AUTO = direct where
 *   possible.  matpl_lammps_dp_host_access returns the form a handle uses.
 * ---------------------------------------------------------------------------------- */
int matpl_lammps_dp_neighbors(int inum, int nall, const int *ilist, const long long *jstart,
                              const int *jflat, const double *x, const int *type,
                              const int *type_to_model, int ntypes_lmp, int model_ntypes, int m,
                              double rcut, int out_dtype, int32_t *list_neigh, void *image_dr,
                              int32_t *type_map, double *min_rsq, int32_t *err_dev,
                              void *stream);

#define MATPL_LMP_AUTO 0
#define MATPL_LMP_STAGED 1
#define MATPL_LMP_DIRECT 2
typedef struct matpl_lammps_dp matpl_lammps_dp;
int matpl_lammps_dp_create(int dtype, const matpl_dp_model *model, int ntypes_lmp,
                           const int *type_to_model, int eatom_grouped, int host_access,
                           matpl_lammps_dp **handle);
int matpl_lammps_dp_host_access(const matpl_lammps_dp *handle);
int matpl_lammps_dp_compute(matpl_lammps_dp *handle, int nlocal, int nghost, int inum,
                            const int *ilist, const int *numneigh, const int *const *firstneigh,
                            const double *x, const int *type, double *f, double *eng,
                            double *virial, double *eatom, double *min_rsq);
void matpl_lammps_dp_destroy(matpl_lammps_dp *handle);

/* Model deviation (pair_style matpl with several models, pair_matpl.cpp:940-975, 1287-1320):
 * add_model appends a model (same ntypes, m and Rmax as the first: the slots are built once
 * with them); compute_models converts the list once and evaluates the first nmodels models,
 * writing f [nmodels][nall][3], eng [nmodels], virial [nmodels][6], eatom [nmodels][inum]
 * (each may be NULL but f), *min_rsq; the pair style folds the ghost rows (reverse
 * communication) and computes the deviation as before (calc_max_error, :385-483). */
int matpl_lammps_dp_add_model(matpl_lammps_dp *handle, const matpl_dp_model *model);
int matpl_lammps_dp_num_models(const matpl_lammps_dp *handle);
int matpl_lammps_dp_compute_models(matpl_lammps_dp *handle, int nmodels, int nlocal, int nghost,
                                   int inum, const int *ilist, const int *numneigh,
                                   const int *const *firstneigh, const double *x,
                                   const int *type, double *f, double *eng, double *virial,
                                   double *eatom, double *min_rsq);

/* ------------------------------------------------------------------------------------
 * Batched replica MD (one DP model, many independent periodic replicas of uneven size in one
 * ragged atom array: replica r owns atoms [rep_start[r], rep_start[r+1]); atom_rep[i] = its
 * replica; lattice / inv_lattice [nrep, 3, 3] with the cell vectors as rows).  No counterpart
 * in the reference's GPU code: it is the in-GPU form of the LAMMPS loop around the pair style
 * (velocity Verlet, and the neighbor list kept at Rc + skin and rebuilt when an atom has
 * moved more than skin / 2, the rule pair_matpl.cpp:1096-1110 defers to).  Positions x
 * [ntot, 3] FP64 Angstrom stay unwrapped.
 *
 * matpl_md_drift: x += v dt + a dt^2 / 2; sets *gate = 1 when some |x - x_ref| > skin / 2.
 *
 * matpl_md_skin_build: only when *gate != 0 (read on the device), every pair within r_list of
 * every atom, all periodic images, into nbr / img [ntot, ntypes * cap] (per type block: global
 * neighbor index, image (n_a, n_b, n_c) as three signed bytes, d = x_j - x_i + n L) and cnt
 * [ntot, ntypes]; x_ref = x; then *gate = 0 and ++*nbuild (nbuild may be NULL).  work [nwork]
 * int32 pairs (replica, first local atom) cover every replica in blocks of 128 atoms.  err_dev:
 * MATPL_KERR_NEIGHBOR_OVERFLOW (a block needs more than cap), MATPL_KERR_BAD_TYPE,
 * MATPL_KERR_BAD_BOX (a cell needing more than 63 images, or an image index past +-127).
 *
 * matpl_md_skin_filter: the pairs of the skin list with 1e-8 < r^2 < rc^2 at the current
 * positions, in list order, as the occupied-slot list matpl_dp_eval_occupied reads (B = 1,
 * N = ntot, S = ntypes * m): list_neigh 1-based global indices, image_dr (r, x_j - x_i) rows in
 * dtype (MATPL_F64 / MATPL_F32), num_neigh [ntot, ntypes]; more than m in a block sets
 * MATPL_KERR_NEIGHBOR_OVERFLOW.  Slots past the block lengths are not written.
 *
 * matpl_md_kick: mode 0 a = F inv_mass; mode 1 also v += (a_old + a) dt / 2.  Per replica,
 * ke[r] = sum conv_ke m v^2 / 2 and pe[r] = sum ei, FP64, in a fixed order (force [ntot, 3] and
 * ei [ntot] in dtype). */
int matpl_md_drift(int ntot, double dt, double skin, double *x, const double *v,
                   const double *a, const double *x_ref, int32_t *gate, void *stream);

int matpl_md_skin_build(int nrep, int ntot, int ntypes, int cap, double r_list,
                        const int32_t *rep_start, const int32_t *work, int nwork,
                        const double *lattice, const double *inv_lattice,
                        const int32_t *type_map, const double *x, int32_t *nbr, int32_t *img,
                        int32_t *cnt, double *x_ref, int32_t *gate, int32_t *nbuild,
                        int32_t *err_dev, void *stream);

int matpl_md_skin_filter(int dtype, int ntot, int ntypes, int cap, int m, double rc,
                         const int32_t *atom_rep, const double *lattice, const int32_t *nbr,
                         const int32_t *img, const int32_t *cnt, const double *x,
                         int32_t *list_neigh, void *image_dr, int32_t *num_neigh,
                         int32_t *err_dev, void *stream);

int matpl_md_kick(int dtype, int mode, int nrep, double dt, double conv_ke,
                  const int32_t *rep_start, const double *inv_mass, const double *mass,
                  const void *force, const void *ei, double *v, double *a, double *ke,
                  double *pe, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MATPL_GB300_H */
