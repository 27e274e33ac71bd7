// torch.ops.CalcOps_cuda over this library's C ABI: the operator library MatPL's Python models
// load with torch.ops.load_library (src/model/dp_dp.py:13-20, src/model/nep_net.py:17-24).
//
// The names and argument lists are those of src/op/src/CalcOps_bind.cpp:6-16 (declarations in
// src/op/include/CalcOps.h), so the schemas torch infers from them are the reference's: each op
// takes and returns tensors the same way, list returns included.  The differentiable ops are
// torch::autograd::Functions with the reference's gradient rules (CalcOps.cpp:6-72, 170-236,
// 331-383, 75-168, 238-329): calculateForce / calculateVirial / calculateNepForce /
// calculateNepVirial are differentiable in dE only, calculateCompress in f2 only.  Every
// kernel runs on the current CUDA stream of the tensors' device; a failure raises (the
// reference prints and returns zeros).  Not registered here: calculateNepFeat /
// calculateNepMbFeat / calculate_descriptor (the NEP training descriptors have their own
// autograd Functions in matpl_gb300.nep_ops).
#include <ATen/ATen.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/autograd.h>
#include <torch/library.h>

#include <vector>

#include "../../include/matpl_gb300.h"

namespace {

using at::Tensor;
using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

void check(int status, const char *what) {
    TORCH_CHECK(status == MATPL_OK, "CalcOps_cuda.", what, " failed (status ", status, "): ",
                matpl_last_error());
}

int dtype_code(const Tensor &t) {
    TORCH_CHECK(t.scalar_type() == at::kFloat || t.scalar_type() == at::kDouble,
                "CalcOps_cuda: float32 or float64 tensors expected, got ", t.scalar_type());
    return t.scalar_type() == at::kDouble ? MATPL_F64 : MATPL_F32;
}

void *stream_of(const Tensor &t) {
    return static_cast<void *>(c10::cuda::getCurrentCUDAStream(t.get_device()).stream());
}

void require_cuda(const Tensor &t, const char *what) {
    TORCH_CHECK(t.is_cuda(), "CalcOps_cuda.", what, ": CUDA tensors expected (no CPU fallback)");
}

// int64 tensor data as the C ABI's long long
long long *ll(const Tensor &t) { return reinterpret_cast<long long *>(t.data_ptr<int64_t>()); }

// list_neigh [B, N, 1, S] (or [B, N, S]) int, 0-based, -1 = empty  ->  int32 contiguous
Tensor as_list(const Tensor &ln) { return ln.to(at::kInt).contiguous(); }

// ------------------------------------------------------------------ calculateForce
struct ForceOp : public torch::autograd::Function<ForceOp> {
    static variable_list forward(AutogradContext *ctx, Tensor list_neigh, Tensor dE, Tensor Ri_d,
                                 Tensor F, Tensor nghost_tensor) {
        require_cuda(dE, "calculateForce");
        c10::cuda::CUDAGuard guard(dE.device());
        const int64_t B = list_neigh.size(0), N = list_neigh.size(1);
        const int64_t S = N > 0 ? list_neigh.numel() / (B * N) : 0;
        const int nghost = (int)nghost_tensor.item<int64_t>();
        Tensor nl = as_list(list_neigh), dEc = dE.contiguous(), Rd = Ri_d.contiguous();
        Tensor Fc = F.to(dE.scalar_type()).contiguous();
        Tensor out = at::empty({B, N + nghost, 3}, dE.options());
        check(matpl_calc_force(dtype_code(dE), nl.data_ptr<int32_t>(), dEc.data_ptr(), Rd.data_ptr(),
                               Fc.data_ptr(), (int)B, (int)N, (int)S, nghost, out.data_ptr(),
                               stream_of(dE)),
              "calculateForce");
        ctx->save_for_backward({nl, Rd});
        ctx->saved_data["nghost"] = (int64_t)nghost;
        ctx->saved_data["dE_sizes"] = dE.sizes().vec();
        return {out};
    }
    static variable_list backward(AutogradContext *ctx, variable_list grad_out) {
        auto saved = ctx->get_saved_variables();
        Tensor nl = saved[0], Rd = saved[1];
        c10::cuda::CUDAGuard guard(Rd.device());
        const int64_t B = nl.size(0), N = nl.size(1);
        const int64_t S = N > 0 ? nl.numel() / (B * N) : 0;
        const int nghost = (int)ctx->saved_data["nghost"].toInt();
        Tensor g = grad_out[0].to(Rd.scalar_type()).contiguous();
        Tensor grad = at::empty(ctx->saved_data["dE_sizes"].toIntVector(), Rd.options());
        check(matpl_calc_force_grad(dtype_code(Rd), nl.data_ptr<int32_t>(), Rd.data_ptr(),
                                    g.data_ptr(), (int)B, (int)N, (int)S, nghost, grad.data_ptr(),
                                    stream_of(Rd)),
              "calculateForce (backward)");
        return {Tensor(), grad, Tensor(), Tensor(), Tensor()};
    }
};

variable_list calculateForce(Tensor list_neigh, Tensor dE, Tensor Ri_d, Tensor F,
                             Tensor nghost_tensor) {
    return ForceOp::apply(list_neigh, dE, Ri_d, F, nghost_tensor);
}

// ------------------------------------------------------------------ calculateVirial
struct VirialOp : public torch::autograd::Function<VirialOp> {
    static variable_list forward(AutogradContext *ctx, Tensor list_neigh, Tensor dE, Tensor Rij,
                                 Tensor Ri_d, Tensor nghost_tensor) {
        require_cuda(dE, "calculateVirial");
        c10::cuda::CUDAGuard guard(dE.device());
        const int64_t B = list_neigh.size(0), N = list_neigh.size(1);
        const int64_t S = N > 0 ? list_neigh.numel() / (B * N) : 0;
        const int nghost = (int)nghost_tensor.item<int64_t>();
        Tensor nl = as_list(list_neigh), dEc = dE.contiguous(), Rd = Ri_d.contiguous();
        Tensor Rj = Rij.to(dE.scalar_type()).contiguous();
        Tensor vir = at::empty({B, 9}, dE.options());
        Tensor avir = at::empty({B, N + nghost, 9}, dE.options());
        check(matpl_calc_virial(dtype_code(dE), nl.data_ptr<int32_t>(), dEc.data_ptr(), Rj.data_ptr(),
                                Rd.data_ptr(), (int)B, (int)N, (int)S, nghost, vir.data_ptr(),
                                avir.data_ptr(), stream_of(dE)),
              "calculateVirial");
        ctx->save_for_backward({nl, Rj, Rd});
        ctx->saved_data["dE_sizes"] = dE.sizes().vec();
        ctx->mark_non_differentiable({avir});
        return {vir, avir};
    }
    static variable_list backward(AutogradContext *ctx, variable_list grad_out) {
        auto saved = ctx->get_saved_variables();
        Tensor nl = saved[0], Rj = saved[1], Rd = saved[2];
        c10::cuda::CUDAGuard guard(Rd.device());
        const int64_t B = nl.size(0), N = nl.size(1);
        const int64_t S = N > 0 ? nl.numel() / (B * N) : 0;
        Tensor g = grad_out[0].defined() ? grad_out[0].to(Rd.scalar_type()).contiguous()
                                         : at::zeros({B, 9}, Rd.options());
        Tensor grad = at::empty(ctx->saved_data["dE_sizes"].toIntVector(), Rd.options());
        check(matpl_calc_virial_grad(dtype_code(Rd), nl.data_ptr<int32_t>(), Rj.data_ptr(),
                                     Rd.data_ptr(), g.data_ptr(), (int)B, (int)N, (int)S,
                                     grad.data_ptr(), stream_of(Rd)),
              "calculateVirial (backward)");
        return {Tensor(), grad, Tensor(), Tensor(), Tensor()};
    }
};

variable_list calculateVirial(Tensor list_neigh, Tensor dE, Tensor Rij, Tensor Ri_d,
                              Tensor nghost_tensor) {
    return VirialOp::apply(list_neigh, dE, Rij, Ri_d, nghost_tensor);
}

// ------------------------------------------------------------------ calculateCompress
struct CompressOp : public torch::autograd::Function<CompressOp> {
    static variable_list forward(AutogradContext *ctx, Tensor f2, Tensor coefficient) {
        require_cuda(coefficient, "calculateCompress");
        c10::cuda::CUDAGuard guard(coefficient.device());
        Tensor c = coefficient.contiguous();
        const int64_t ns = c.size(0), nodes = c.size(1), nc = c.size(2);
        Tensor f = f2.reshape({-1}).to(c.scalar_type()).contiguous();
        Tensor G = at::empty({ns, nodes}, c.options());
        check(matpl_calc_compress(dtype_code(c), f.data_ptr(), c.data_ptr(), ns, (int)nodes,
                                  (int)nc, G.data_ptr(), stream_of(c)),
              "calculateCompress");
        ctx->save_for_backward({f, c});
        ctx->saved_data["f2_sizes"] = f2.sizes().vec();
        return {G};
    }
    static variable_list backward(AutogradContext *ctx, variable_list grad_out) {
        auto saved = ctx->get_saved_variables();
        Tensor f = saved[0], c = saved[1];
        c10::cuda::CUDAGuard guard(c.device());
        const int64_t ns = c.size(0), nodes = c.size(1), nc = c.size(2);
        Tensor g = grad_out[0].to(c.scalar_type()).contiguous();
        Tensor out = at::empty({ns}, c.options());
        check(matpl_calc_compress_grad(dtype_code(c), f.data_ptr(), c.data_ptr(), g.data_ptr(), ns,
                                       (int)nodes, (int)nc, out.data_ptr(), stream_of(c)),
              "calculateCompress (backward)");
        return {out.reshape(ctx->saved_data["f2_sizes"].toIntVector()), Tensor()};
    }
};

variable_list calculateCompress(Tensor f2, Tensor coefficient) {
    return CompressOp::apply(f2, coefficient);
}

// ------------------------------------------------------------------ calculateNepForce
// NEP lists: list_neigh [N, NN] int64 (-1 = empty), dE [N, 4 NN] (or [N, 1, 4 NN]),
// Ri_d [N, 4 NN, 3], F [N, 3] the centre term -> [force [N, 3]].
struct NepForceOp : public torch::autograd::Function<NepForceOp> {
    static variable_list forward(AutogradContext *ctx, Tensor list_neigh, Tensor dE, Tensor Ri_d,
                                 Tensor F) {
        require_cuda(dE, "calculateNepForce");
        c10::cuda::CUDAGuard guard(dE.device());
        const int64_t N = list_neigh.size(0), NN = N > 0 ? list_neigh.numel() / N : 0;
        Tensor nl = as_list(list_neigh), dEc = dE.contiguous(), Rd = Ri_d.contiguous();
        Tensor Fc = F.to(dE.scalar_type()).contiguous();
        Tensor out = at::empty({N, 3}, dE.options());
        check(matpl_calc_force(dtype_code(dE), nl.data_ptr<int32_t>(), dEc.data_ptr(), Rd.data_ptr(),
                               Fc.data_ptr(), 1, (int)N, (int)NN, 0, out.data_ptr(), stream_of(dE)),
              "calculateNepForce");
        ctx->save_for_backward({nl, Rd});
        ctx->saved_data["dE_sizes"] = dE.sizes().vec();
        return {out};
    }
    static variable_list backward(AutogradContext *ctx, variable_list grad_out) {
        auto saved = ctx->get_saved_variables();
        Tensor nl = saved[0], Rd = saved[1];
        c10::cuda::CUDAGuard guard(Rd.device());
        const int64_t N = nl.size(0), NN = N > 0 ? nl.numel() / N : 0;
        Tensor g = grad_out[0].to(Rd.scalar_type()).contiguous();
        Tensor grad = at::empty(ctx->saved_data["dE_sizes"].toIntVector(), Rd.options());
        check(matpl_calc_force_grad(dtype_code(Rd), nl.data_ptr<int32_t>(), Rd.data_ptr(),
                                    g.data_ptr(), 1, (int)N, (int)NN, 0, grad.data_ptr(),
                                    stream_of(Rd)),
              "calculateNepForce (backward)");
        return {Tensor(), grad, Tensor(), Tensor()};
    }
};

variable_list calculateNepForce(Tensor list_neigh, Tensor dE, Tensor Ri_d, Tensor F) {
    return NepForceOp::apply(list_neigh, dE, Ri_d, F);
}

// ------------------------------------------------------------------ calculateNepVirial
// -> [virial [frames, 9] (sum over each frame's atoms), atom_virial [N, 9]]
struct NepVirialOp : public torch::autograd::Function<NepVirialOp> {
    static variable_list forward(AutogradContext *ctx, Tensor list_neigh, Tensor dE, Tensor Rij,
                                 Tensor Ri_d, Tensor num_atom) {
        require_cuda(dE, "calculateNepVirial");
        c10::cuda::CUDAGuard guard(dE.device());
        const int64_t N = list_neigh.size(0), NN = N > 0 ? list_neigh.numel() / N : 0;
        Tensor nl = as_list(list_neigh), dEc = dE.contiguous(), Rd = Ri_d.contiguous();
        Tensor Rj = Rij.to(dE.scalar_type()).contiguous();
        Tensor counts = num_atom.to(at::kCPU, at::kLong).reshape({-1}).contiguous();
        const int64_t nimg = counts.numel();
        Tensor vir1 = at::empty({1, 9}, dE.options());
        Tensor avir = at::empty({N, 9}, dE.options());
        check(matpl_calc_virial(dtype_code(dE), nl.data_ptr<int32_t>(), dEc.data_ptr(), Rj.data_ptr(),
                                Rd.data_ptr(), 1, (int)N, (int)NN, 0, vir1.data_ptr(),
                                avir.data_ptr(), stream_of(dE)),
              "calculateNepVirial");
        Tensor img = at::repeat_interleave(at::arange(nimg, counts.options()), counts)
                         .to(dE.device());
        Tensor vir = at::zeros({nimg, 9}, dE.options()).index_add_(0, img, avir);
        ctx->save_for_backward({nl, Rj, Rd, counts});
        ctx->saved_data["dE_sizes"] = dE.sizes().vec();
        ctx->mark_non_differentiable({avir});
        return {vir, avir};
    }
    static variable_list backward(AutogradContext *ctx, variable_list grad_out) {
        auto saved = ctx->get_saved_variables();
        Tensor nl = saved[0], Rj = saved[1], Rd = saved[2], counts = saved[3];
        c10::cuda::CUDAGuard guard(Rd.device());
        const int64_t N = nl.size(0), NN = N > 0 ? nl.numel() / N : 0;
        Tensor grad = at::zeros({N, 4 * NN}, Rd.options());
        if (grad_out[0].defined()) {
            Tensor g = grad_out[0].to(Rd.scalar_type()).contiguous();
            const int64_t *c = counts.data_ptr<int64_t>();
            int64_t off = 0;
            for (int64_t b = 0; b < counts.numel(); ++b) {
                const int64_t n = c[b];
                if (n > 0) {
                    Tensor nl_b = nl.narrow(0, off, n), Rj_b = Rj.narrow(0, off, n);
                    Tensor Rd_b = Rd.narrow(0, off, n), gr_b = grad.narrow(0, off, n);
                    Tensor g_b = g.narrow(0, b, 1).contiguous();
                    check(matpl_calc_virial_grad(dtype_code(Rd), nl_b.data_ptr<int32_t>(),
                                                 Rj_b.data_ptr(), Rd_b.data_ptr(), g_b.data_ptr(),
                                                 1, (int)n, (int)NN, gr_b.data_ptr(),
                                                 stream_of(Rd)),
                          "calculateNepVirial (backward)");
                }
                off += n;
            }
        }
        return {Tensor(), grad.reshape(ctx->saved_data["dE_sizes"].toIntVector()), Tensor(),
                Tensor(), Tensor()};
    }
};

variable_list calculateNepVirial(Tensor list_neigh, Tensor dE, Tensor Rij, Tensor Ri_d,
                                 Tensor num_atom) {
    return NepVirialOp::apply(list_neigh, dE, Rij, Ri_d, num_atom);
}

// ------------------------------------------------------------------ NEP neighbor operators
struct Frames {
    Tensor na, bx, bo, nc, pos;
};

Frames frames_of(const Tensor &num_atoms, const Tensor &box, const Tensor &box_orig,
                 const Tensor &num_cell, const Tensor &position) {
    require_cuda(position, "calculate_neighbor");
    const auto dev = position.device();
    Frames f;
    f.na = num_atoms.to(dev, at::kLong).reshape({-1}).contiguous();
    const int64_t B = f.na.numel();
    f.bx = box.to(dev, at::kDouble).reshape({B, 18}).contiguous();
    f.bo = box_orig.to(dev, at::kDouble).reshape({B, 9}).contiguous();
    f.nc = num_cell.to(dev, at::kLong).reshape({B, 3}).contiguous();
    f.pos = position.to(at::kDouble).reshape({-1, 3}).contiguous();
    return f;
}

void kernel_error(const Tensor &err, const char *what) {
    const int code = err.item<int>();
    TORCH_CHECK(code != MATPL_KERR_NEIGHBOR_OVERFLOW, "CalcOps_cuda.", what,
                ": a neighbor list is longer than max_NN");
    TORCH_CHECK(code == 0, "CalcOps_cuda.", what, ": kernel error code ", code);
}

std::vector<Tensor> calculate_maxneigh(const Tensor &num_atoms, const Tensor &box,
                                       const Tensor &box_orig, const Tensor &num_cell,
                                       const Tensor &position, double cutoff_2b, double cutoff_3b,
                                       int64_t atom_type_num, const Tensor &atom_type_map,
                                       bool with_type) {
    Frames f = frames_of(num_atoms, box, box_orig, num_cell, position);
    c10::cuda::CUDAGuard guard(f.pos.device());
    const int64_t N = f.pos.size(0), B = f.na.numel();
    const int64_t nt = with_type ? atom_type_num : 1;
    Tensor tm = atom_type_map.to(f.pos.device(), at::kLong).contiguous();
    auto li = f.pos.options().dtype(at::kLong);
    Tensor NN_r = at::empty({N * nt}, li), NN_a = at::empty({N * nt}, li);
    Tensor err = at::zeros({1}, f.pos.options().dtype(at::kInt));
    Tensor ws = at::empty({(int64_t)matpl_nep_neighbor_workspace_bytes((int)B, N)},
                          f.pos.options().dtype(at::kByte));
    check(matpl_nep_maxneigh((int)B, N, ll(f.na), f.bx.data_ptr<double>(),
                             f.bo.data_ptr<double>(), ll(f.nc),
                             f.pos.data_ptr<double>(), cutoff_2b, cutoff_3b, (int)atom_type_num,
                             ll(tm), with_type ? 1 : 0,
                             ll(NN_r), ll(NN_a),
                             err.data_ptr<int>(), ws.data_ptr(), (size_t)ws.numel(),
                             stream_of(f.pos)),
          "calculate_maxneigh");
    kernel_error(err, "calculate_maxneigh");
    return {NN_r, NN_a};
}

std::vector<Tensor> calculate_neighbor(const Tensor &num_atoms, const Tensor &atom_type_map,
                                       const Tensor &atom_types, const Tensor &box,
                                       const Tensor &box_orig, const Tensor &num_cell,
                                       const Tensor &position, double cutoff_2b, double cutoff_3b,
                                       int64_t max_NN_radial, int64_t max_NN_angular,
                                       bool with_rij) {
    (void)atom_type_map;        // the lists do not depend on the types (signature kept)
    (void)atom_types;
    Frames f = frames_of(num_atoms, box, box_orig, num_cell, position);
    c10::cuda::CUDAGuard guard(f.pos.device());
    const int64_t N = f.pos.size(0), B = f.na.numel(), w = with_rij ? 4 : 3;
    auto li = f.pos.options().dtype(at::kLong);
    Tensor NN_r = at::empty({N}, li), NN_a = at::empty({N}, li);
    Tensor NL_r = at::empty({N, max_NN_radial}, li), NL_a = at::empty({N, max_NN_angular}, li);
    Tensor Ri_r = at::empty({N, max_NN_radial, w}, f.pos.options());
    Tensor Ri_a = at::empty({N, max_NN_angular, w}, f.pos.options());
    Tensor err = at::zeros({1}, f.pos.options().dtype(at::kInt));
    Tensor ws = at::empty({(int64_t)matpl_nep_neighbor_workspace_bytes((int)B, N)},
                          f.pos.options().dtype(at::kByte));
    check(matpl_nep_neighbor((int)B, N, ll(f.na), f.bx.data_ptr<double>(),
                             f.bo.data_ptr<double>(), ll(f.nc),
                             f.pos.data_ptr<double>(), cutoff_2b, cutoff_3b, (int)max_NN_radial,
                             (int)max_NN_angular, with_rij ? 1 : 0, ll(NN_r),
                             ll(NN_a), ll(NL_r),
                             ll(NL_a), Ri_r.data_ptr<double>(),
                             Ri_a.data_ptr<double>(), err.data_ptr<int>(), ws.data_ptr(),
                             (size_t)ws.numel(), stream_of(f.pos)),
          "calculate_neighbor");
    kernel_error(err, "calculate_neighbor");
    return {NN_r, NN_a, NL_r, NL_a, Ri_r, Ri_a};
}

}  // namespace

TORCH_LIBRARY(CalcOps_cuda, m) {
    m.def("calculateForce", calculateForce);
    m.def("calculateVirial", calculateVirial);
    m.def("calculateCompress", calculateCompress);
    m.def("calculateNepForce", calculateNepForce);
    m.def("calculateNepVirial", calculateNepVirial);
    m.def("calculate_maxneigh", calculate_maxneigh);
    m.def("calculate_neighbor", calculate_neighbor);
}
