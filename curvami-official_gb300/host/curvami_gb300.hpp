// curvami_gb300.hpp — C++17 host shim over the C ABI (include/curvami_gb300.h).
//
// Mirrors the reference's hot-path interface for C++ callers: RAII handles, exceptions
// (std::runtime_error subclass carrying the status) instead of status codes, and the
// reference's names:
//   ShapeSet::build          GlobalFRNN::execute + GlobalRKPM::solve
//                            (core/include/curvami/FRNN.h:23, GlobalRKPM.h:19)
//   NonLinearAssembler       initSparsityPattern / updateStiffness / csrMapping
//                            (plate/Assembly.h:49-59, 158), with the hinge of
//                            Meshless::assembleSystem (plate/Meshless.h:102-127)
// Data are plain std::vector (structure of arrays); INTEGRATION.md shows the adapter a
// caller holding the reference's GaussPointData / Eigen types writes around it.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/curvami_gb300.h"

namespace curvami_gb300 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

class Context {
 public:
  explicit Context(int device = 0) {
    const int rc = cgb_create(device, &h_);
    if (rc != CGB_OK) throw Error(rc, "cgb_create failed: no usable CUDA device");
  }
  ~Context() { cgb_destroy(h_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;

  void check(int rc) const {
    if (rc != CGB_OK) throw Error(rc, cgb_last_error(h_));
  }
  // Node::X_ref of every node, x y interleaved.
  void set_nodes(const std::vector<double>& xy) {
    check(cgb_set_nodes(h_, xy.data(), static_cast<int>(xy.size() / 2)));
  }
  cgb_context* get() const { return h_; }

 private:
  cgb_context* h_ = nullptr;
};

struct Crease {  // Enrichment::FoldLine
  std::vector<double> xy;
  bool extend_start = false, extend_end = false, is_closed = false;
};

struct Shapes {  // GaussPointData::neighbor_node_ids / Psi / dPsi / ddPsi, flattened
  std::vector<int64_t> nbr_ptr;
  std::vector<int32_t> nbr_idx;
  std::vector<double> psi, dpsi, ddpsi;  // 1, 2 (x y), 3 (xx yy xy) per entry
};

class ShapeSet {
 public:
  // GlobalFRNN::execute + GlobalRKPM::solve; throws Error with the reference's message
  // on a rank-deficient support. precision: CGB_SHAPE_FP64 or CGB_SHAPE_MIXED.
  static ShapeSet build(Context& ctx, const std::vector<double>& gp_xy, double rho, int order,
                        const std::vector<Crease>& creases = {}, const std::vector<double>* rho_node = nullptr,
                        int kernel = 0, int precision = CGB_SHAPE_FP64) {
    std::vector<cgb_crease> cr(creases.size());
    for (size_t k = 0; k < creases.size(); ++k)
      cr[k] = cgb_crease{creases[k].xy.data(), static_cast<int>(creases[k].xy.size() / 2),
                         creases[k].extend_start, creases[k].extend_end, creases[k].is_closed};
    cgb_shape_params prm{rho, rho_node ? rho_node->data() : nullptr, order, kernel, precision};
    cgb_shape* h = nullptr;
    const int rc = cgb_shape_build(ctx.get(), gp_xy.data(), static_cast<int>(gp_xy.size() / 2), &prm,
                                   cr.data(), static_cast<int>(cr.size()), &h);
    if (rc != CGB_OK) {
      const std::string msg = cgb_last_error(ctx.get());
      cgb_shape_destroy(h);
      throw Error(rc, msg);
    }
    return ShapeSet(ctx, h);
  }
  // Shape functions computed elsewhere (e.g. by the reference's own solve).
  static ShapeSet from_host(Context& ctx, const Shapes& s) {
    cgb_shape* h = nullptr;
    ctx.check(cgb_shape_from_host(ctx.get(), static_cast<int>(s.nbr_ptr.size()) - 1, s.nbr_ptr.data(),
                                  s.nbr_idx.data(), s.psi.empty() ? nullptr : s.psi.data(), s.dpsi.data(),
                                  s.ddpsi.data(), &h));
    return ShapeSet(ctx, h);
  }
  ShapeSet(ShapeSet&& o) noexcept : ctx_(o.ctx_), h_(std::exchange(o.h_, nullptr)) {}
  ShapeSet(const ShapeSet&) = delete;
  ~ShapeSet() { cgb_shape_destroy(h_); }

  Shapes download() const {
    int n = 0, mx = 0;
    int64_t nnz = 0;
    ctx_->check(cgb_shape_size(h_, &n, &nnz, &mx));
    Shapes s;
    s.nbr_ptr.resize(n + 1);
    s.nbr_idx.resize(nnz);
    s.psi.resize(nnz);
    s.dpsi.resize(2 * nnz);
    s.ddpsi.resize(3 * nnz);
    ctx_->check(cgb_shape_download(h_, s.nbr_ptr.data(), s.nbr_idx.data(), nullptr, s.psi.data(), s.dpsi.data(),
                                   s.ddpsi.data()));
    return s;
  }
  const cgb_shape* get() const { return h_; }
  // SetupHelper::recomputeShapeFunctions for other cuts: Phi and its derivatives
  // recomputed in place, points and neighbour lists kept (progressive creasing's rebuild).
  void rebuild(const std::vector<Crease>& creases) {
    std::vector<cgb_crease> cr(creases.size());
    for (size_t k = 0; k < creases.size(); ++k)
      cr[k] = cgb_crease{creases[k].xy.data(), static_cast<int>(creases[k].xy.size() / 2),
                         creases[k].extend_start, creases[k].extend_end, creases[k].is_closed};
    ctx_->check(cgb_shape_rebuild(h_, cr.data(), static_cast<int>(cr.size())));
  }

 private:
  ShapeSet(Context& ctx, cgb_shape* h) : ctx_(&ctx), h_(h) {}
  Context* ctx_;
  cgb_shape* h_;
};

struct FoldSpec {  // one Fold: its crease points on both sides
  const ShapeSet* left;
  const ShapeSet* right;
  std::vector<double> weight, tangent;  // n, 2n
  double Kt = 0.0, theta0 = 0.0;
  std::vector<double> theta0_gp;        // empty: theta0 everywhere
  std::vector<int8_t> active;           // empty: all active
};

class NonLinearAssembler {
 public:
  // initSparsityPattern (+ the hinge blocks Meshless::assembleSystem adds).
  NonLinearAssembler(Context& ctx, const ShapeSet& faces, const std::vector<double>& face_weight,
                     const std::vector<FoldSpec>& folds = {})
      : ctx_(&ctx) {
    std::vector<cgb_fold> f(folds.size());
    for (size_t k = 0; k < folds.size(); ++k)
      f[k] = cgb_fold{folds[k].left->get(), folds[k].right->get(), folds[k].weight.data(),
                      folds[k].tangent.data(), folds[k].Kt, folds[k].theta0,
                      folds[k].theta0_gp.empty() ? nullptr : folds[k].theta0_gp.data(),
                      folds[k].active.empty() ? nullptr : folds[k].active.data()};
    ctx.check(cgb_assembler_create(ctx.get(), faces.get(), face_weight.data(), f.data(),
                                   static_cast<int>(f.size()), &h_));
    ctx.check(cgb_assembler_pattern(h_, &n_dofs_, &nnz_));
  }
  ~NonLinearAssembler() { cgb_assembler_destroy(h_); }
  NonLinearAssembler(const NonLinearAssembler&) = delete;

  int n_dofs() const { return n_dofs_; }
  int64_t nnz() const { return nnz_; }
  // K.outerIndexPtr() / innerIndexPtr() of the reference's SparseMatrix.
  void pattern(std::vector<int32_t>& outer, std::vector<int32_t>& inner) const {
    outer.resize(n_dofs_ + 1);
    inner.resize(nnz_);
    ctx_->check(cgb_assembler_download_pattern(h_, outer.data(), inner.data()));
  }
  void set_material(const double A[9], const double B[9], const double D[9]) {
    ctx_->check(cgb_set_material(h_, A, B, D));
  }
  // Fold::gp_theta0 / gp_active of fold k (empty vectors: theta0 everywhere / all active).
  void set_fold_state(int k, double theta0, const std::vector<double>& theta0_gp,
                      const std::vector<int8_t>& active) {
    ctx_->check(cgb_assembler_set_fold_state(h_, k, theta0, theta0_gp.empty() ? nullptr : theta0_gp.data(),
                                             active.empty() ? nullptr : active.data()));
  }
  // Meshless::assembleSystem (flags CGB_TANGENT | CGB_HINGE) / assembleSystemInternalOnly
  // (CGB_HINGE): K values (nnz, block-upper CSC) and F_int (n_dofs) overwritten.
  void assemble(const std::vector<double>& x, std::vector<double>* K, std::vector<double>& F,
                int flags = CGB_TANGENT | CGB_HINGE) {
    F.resize(n_dofs_);
    if (K) K->resize(nnz_);
    ctx_->check(cgb_assemble(h_, x.data(), K ? K->data() : nullptr, F.data(), flags));
  }

 private:
  Context* ctx_;
  cgb_assembler* h_ = nullptr;
  int n_dofs_ = 0;
  int64_t nnz_ = 0;
};

}  // namespace curvami_gb300
