// capi.cu — the C ABI (include/curvami_gb300.h): handles, argument checks, status
// codes and host<->device copies around the kernels of shape.cu / pattern.cu /
// assemble.cu. Every entry point catches the library's exceptions and returns a status;
// the message is kept for cgb_last_error().
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "cgb_internal.h"

using cgb::Error;

namespace {

template <class F>
int guarded(cgb_context* ctx, F&& body) {
  try {
    body();
    if (ctx) ctx->last_error.clear();
    return CGB_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return CGB_ERR_CUDA;
  } catch (const std::exception& e) {
    if (ctx) ctx->last_error = e.what();
    return CGB_ERR_INVALID;
  }
}

void need(bool ok, const char* msg) {
  if (!ok) throw Error(CGB_ERR_INVALID, msg);
}

void bind_device(cgb_context* ctx) { CGB_CUDA(cudaSetDevice(ctx->device)); }

// The device error word after an assembly: a bounded wait of the tangent's staging
// copies gave up (the kernel left its remaining groups undone). Cleared once reported.
// Bit 8: an index in the caller-owned arrays of cgb_assemble_face_noalloc was out of range
// (the access was skipped). Bit 16: the tensor-core tangent gave up waiting for an MMA.
void check_device_word(cgb_context* ctx, int word) {
  if (word & (4 | 8 | 16)) {
    CGB_CUDA(cudaMemsetAsync(ctx->dev_err.p, 0, sizeof(int), ctx->stream));
    CGB_CUDA(cudaStreamSynchronize(ctx->stream));
    if (word & 4)
      throw Error(CGB_ERR_DEVICE, "assemble: a bulk copy of the tangent's neighbour data did not complete; "
                                  "K is incomplete");
    if (word & 16)
      throw Error(CGB_ERR_DEVICE, "assemble: a tensor-core product of the tangent did not complete in time; "
                                  "K is incomplete");
    throw Error(CGB_ERR_DEVICE, "cgb_assemble_face_noalloc: an index in the caller's arrays was out of range "
                                "(a neighbour count above max_neighbours, a node id outside [0, n_nodes), or a "
                                "block beyond nnz); K and F are incomplete");
  }
}

cudaEvent_t take_event(cgb_context* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  CGB_CUDA(cudaEventCreate(&e));
  return e;
}

void collect_marks(cgb_context* ctx) {
  for (auto& m : ctx->marks) {
    if (m.stop) {
      CGB_CUDA(cudaEventSynchronize(m.stop));
      float ms = 0.0f;
      CGB_CUDA(cudaEventElapsedTime(&ms, m.start, m.stop));
      ctx->prof_ms[m.phase] += ms;
      ctx->prof_launches[m.phase] += m.launches;
      ctx->event_pool.push_back(m.stop);
    }
    ctx->event_pool.push_back(m.start);
  }
  ctx->marks.clear();
}

}  // namespace

namespace cgb {
void prof_begin(cgb_context* ctx, int phase, cudaStream_t stream) {
  if (!ctx->profile) return;
  if (!stream) stream = ctx->stream;
  cgb_context::Mark m{phase, take_event(ctx), nullptr, 0, stream};
  CGB_CUDA(cudaEventRecord(m.start, stream));
  ctx->marks.push_back(m);
}
void prof_end(cgb_context* ctx, int phase, int launches, cudaStream_t stream) {
  if (!ctx->profile) return;
  if (!stream) stream = ctx->stream;
  for (auto it = ctx->marks.rbegin(); it != ctx->marks.rend(); ++it) {
    if (it->phase == phase && !it->stop && it->stream == stream) {
      it->stop = take_event(ctx);
      it->launches = launches;
      CGB_CUDA(cudaEventRecord(it->stop, stream));
      break;
    }
  }
  if (ctx->marks.size() > 4096) collect_marks(ctx);
}
}  // namespace cgb

extern "C" {

int cgb_profile_enable(cgb_context* ctx, int on) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    bind_device(ctx);
    if (!on) collect_marks(ctx);
    ctx->profile = on != 0;
  });
}

int cgb_profile_read(cgb_context* ctx, double* ms, int64_t* launches, int reset) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    bind_device(ctx);
    collect_marks(ctx);
    for (int p = 0; p < CGB_N_PHASES; ++p) {
      if (ms) ms[p] = ctx->prof_ms[p];
      if (launches) launches[p] = ctx->prof_launches[p];
      if (reset) { ctx->prof_ms[p] = 0.0; ctx->prof_launches[p] = 0; }
    }
  });
}

int cgb_create(int device, cgb_context** out) {
  if (!out) return CGB_ERR_INVALID;
  *out = nullptr;
  auto* ctx = new (std::nothrow) cgb_context();
  if (!ctx) return CGB_ERR_CUDA;
  const int rc = guarded(ctx, [&] {
    int n = 0;
    CGB_CUDA(cudaGetDeviceCount(&n));
    need(device >= 0 && device < n, "cgb_create: no such CUDA device");
    ctx->device = device;
    bind_device(ctx);
    CGB_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
    ctx->dev_err.alloc(1);
    CGB_CUDA(cudaMemsetAsync(ctx->dev_err.p, 0, sizeof(int), ctx->stream));
    CGB_CUDA(cudaStreamSynchronize(ctx->stream));
  });
  if (rc != CGB_OK) {
    static thread_local std::string msg;
    msg = ctx->last_error;
    delete ctx;
    return rc;
  }
  *out = ctx;
  return CGB_OK;
}

int cgb_destroy(cgb_context* ctx) {
  if (!ctx) return CGB_OK;
  ctx->closed = true;
  cgb::ctx_release(ctx);
  return CGB_OK;
}

}  // extern "C"

namespace cgb {
void ctx_retain(cgb_context* ctx) { ++ctx->refs; }
void ctx_release(cgb_context* ctx) {
  if (--ctx->refs > 0) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->node_xy.reset();
  ctx->dev_err.reset();
  for (auto& m : ctx->marks) {
    if (m.start) cudaEventDestroy(m.start);
    if (m.stop) cudaEventDestroy(m.stop);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}
}  // namespace cgb

namespace cgb {
const double* natcurv_points(const cgb_context* ctx, const cgb_shape* S, const char* what) {
  if (!ctx->natcurv.active) return nullptr;
  if (S->n_gp == 0) return nullptr;
  if (!S->has_xy || S->gp_xy.n < 2 * static_cast<size_t>(S->n_gp))
    throw Error(CGB_ERR_INVALID, std::string(what) + ": natural curvature needs the points' reference coordinates "
                                                     "(a shape set made by cgb_shape_build)");
  return S->gp_xy.p;
}
}  // namespace cgb

extern "C" {

const char* cgb_last_error(const cgb_context* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int cgb_set_stream(cgb_context* ctx, void* stream) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    bind_device(ctx);
    CGB_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) CGB_CUDA(cudaStreamDestroy(ctx->stream));
    ctx->stream = static_cast<cudaStream_t>(stream);
    ctx->own_stream = false;
  });
}

int cgb_synchronize(cgb_context* ctx) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    int dev_err = 0;
    CGB_CUDA(cudaMemcpyAsync(&dev_err, ctx->dev_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CGB_CUDA(cudaStreamSynchronize(ctx->stream));
    check_device_word(ctx, dev_err);
  });
}

int cgb_set_natural_curvature(cgb_context* ctx, const cgb_natural_curvature* nc) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    cgb::NatCurv v;
    if (nc && nc->active) {
      // main.cpp:83-95: the band's width must be positive, sense mountain (-1) or valley (+1).
      need(nc->width > 0.0, "natural_curvature.width must be > 0");
      need(nc->sign == -1.0 || nc->sign == 1.0, "natural_curvature.sense must be mountain or valley");
      v.active = 1;
      v.x0 = nc->x0;
      v.width = nc->width;
      v.amp = nc->sign * nc->theta0 / (1.7724538509055160273 * nc->width);   // sign theta0 / (sqrt(pi) w)
    }
    ctx->natcurv = v;
  });
}

int cgb_set_nodes(cgb_context* ctx, const double* node_xy, int n_nodes) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    need(n_nodes > 0 && node_xy, "cgb_set_nodes: need at least one node");
    bind_device(ctx);
    const size_t m = 2 * static_cast<size_t>(n_nodes);
    if (ctx->n_nodes != n_nodes || !std::equal(node_xy, node_xy + m, ctx->h_node_xy.begin())) ++ctx->node_gen;
    ctx->n_nodes = n_nodes;
    ctx->h_node_xy.assign(node_xy, node_xy + m);
    cgb::upload(ctx->node_xy, node_xy, 2 * static_cast<size_t>(n_nodes), ctx->stream);
    CGB_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

namespace {
std::vector<cgb::Crease> crease_list(const cgb_crease* creases, int n_creases, const char* who) {
  need(n_creases >= 0 && (n_creases == 0 || creases), (std::string(who) + ": bad crease list").c_str());
  std::vector<cgb::Crease> cr(n_creases);
  for (int c = 0; c < n_creases; ++c) {
    need(creases[c].n_vertices >= 0 && (creases[c].n_vertices == 0 || creases[c].xy),
         (std::string(who) + ": bad crease vertices").c_str());
    cr[c].xy.assign(creases[c].xy, creases[c].xy + 2 * static_cast<size_t>(creases[c].n_vertices));
    cr[c].extend_start = creases[c].extend_start;
    cr[c].extend_end = creases[c].extend_end;
    cr[c].is_closed = creases[c].is_closed;
  }
  return cr;
}
}  // namespace

int cgb_shape_build(cgb_context* ctx, const double* gp_xy, int n_gp, const cgb_shape_params* params,
                    const cgb_crease* creases, int n_creases, cgb_shape** out) {
  if (!ctx || !out) return CGB_ERR_INVALID;
  *out = nullptr;
  auto* sh = new cgb_shape();
  const int rc = guarded(ctx, [&] {
    need(params != nullptr, "cgb_shape_build: params is NULL");
    need(n_gp == 0 || gp_xy, "cgb_shape_build: gp_xy is NULL");
    const std::vector<cgb::Crease> cr = crease_list(creases, n_creases, "cgb_shape_build");
    bind_device(ctx);
    cgb::shape_build(ctx, gp_xy, n_gp, *params, cr, sh);
  });
  // A rank-deficient support still returns the (flagged) shape set, as the reference
  // has filled every array before it throws.
  if (rc == CGB_OK || rc == CGB_ERR_SINGULAR || rc == CGB_ERR_PIVOT) {
    sh->ctx = ctx;
    cgb::ctx_retain(ctx);
    *out = sh;
  } else {
    delete sh;
  }
  return rc;
}

int cgb_shape_rebuild(cgb_shape* sh, const cgb_crease* creases, int n_creases) {
  if (!sh || !sh->ctx) return CGB_ERR_INVALID;
  cgb_context* ctx = sh->ctx;
  return guarded(ctx, [&] {
    const std::vector<cgb::Crease> cr = crease_list(creases, n_creases, "cgb_shape_rebuild");
    bind_device(ctx);
    cgb::shape_rebuild(sh, cr);
  });
}

int cgb_shape_from_host(cgb_context* ctx, int n_gp, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                        const double* psi, const double* dpsi, const double* ddpsi, cgb_shape** out) {
  if (!ctx || !out) return CGB_ERR_INVALID;
  *out = nullptr;
  auto* sh = new cgb_shape();
  const int rc = guarded(ctx, [&] {
    need(n_gp >= 0 && nbr_ptr, "cgb_shape_from_host: nbr_ptr is NULL");
    bind_device(ctx);
    const int64_t nnz = nbr_ptr[n_gp];
    need(nbr_ptr[0] == 0 && nnz >= 0, "cgb_shape_from_host: nbr_ptr must start at 0");
    need(nnz == 0 || (nbr_idx && dpsi && ddpsi), "cgb_shape_from_host: neighbour arrays are NULL");
    int max_n = 0;
    for (int g = 0; g < n_gp; ++g) {
      need(nbr_ptr[g + 1] >= nbr_ptr[g], "cgb_shape_from_host: nbr_ptr must be non-decreasing");
      max_n = std::max<int64_t>(max_n, nbr_ptr[g + 1] - nbr_ptr[g]);
    }
    for (int64_t e = 0; e < nnz; ++e)
      need(nbr_idx[e] >= 0 && nbr_idx[e] < ctx->n_nodes, "cgb_shape_from_host: neighbour index out of range");
    sh->ctx = ctx;
    sh->n_gp = n_gp;
    sh->nnz = nnz;
    sh->max_n = max_n;
    cudaStream_t st = ctx->stream;
    cgb::upload(sh->nbr_ptr, nbr_ptr, n_gp + 1, st);
    cgb::upload(sh->nbr_idx, nbr_idx, nnz, st);
    if (psi) cgb::upload(sh->psi, psi, nnz, st); else sh->psi.alloc(nnz);
    cgb::upload(sh->dpsi, dpsi, 2 * nnz, st);
    cgb::upload(sh->ddpsi, ddpsi, 3 * nnz, st);
    CGB_CUDA(cudaStreamSynchronize(st));
  });
  if (rc == CGB_OK) {
    cgb::ctx_retain(ctx);
    *out = sh;
  } else {
    delete sh;
  }
  return rc;
}

int cgb_shape_size(const cgb_shape* sh, int* n_gp, int64_t* nnz, int* max_neighbours) {
  if (!sh) return CGB_ERR_INVALID;
  if (n_gp) *n_gp = sh->n_gp;
  if (nnz) *nnz = sh->nnz;
  if (max_neighbours) *max_neighbours = sh->max_n;
  return CGB_OK;
}

int cgb_shape_download(const cgb_shape* sh, int64_t* nbr_ptr, int32_t* nbr_idx, double* s, double* psi,
                       double* dpsi, double* ddpsi) {
  if (!sh) return CGB_ERR_INVALID;
  cgb_context* ctx = sh->ctx;
  return guarded(ctx, [&] {
    bind_device(ctx);
    cudaStream_t st = ctx->stream;
    auto get = [&](void* dst, const void* src, size_t bytes) {
      if (dst && bytes) CGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    };
    get(nbr_ptr, sh->nbr_ptr.p, (sh->n_gp + 1) * sizeof(int64_t));
    get(nbr_idx, sh->nbr_idx.p, sh->nnz * sizeof(int32_t));
    // s is a cache of derived data: a mixed-precision set fills it on the first request.
    if (s) cgb::shape_distances(const_cast<cgb_shape*>(sh));
    if (s && sh->s.n >= static_cast<size_t>(sh->nnz)) get(s, sh->s.p, sh->nnz * sizeof(double));
    get(psi, sh->psi.p, sh->nnz * sizeof(double));
    get(dpsi, sh->dpsi.p, 2 * sh->nnz * sizeof(double));
    get(ddpsi, sh->ddpsi.p, 3 * sh->nnz * sizeof(double));
    CGB_CUDA(cudaStreamSynchronize(st));
  });
}

int cgb_shape_device(const cgb_shape* sh, const int64_t** nbr_ptr, const int32_t** nbr_idx, const double** psi,
                     const double** dpsi, const double** ddpsi) {
  if (!sh) return CGB_ERR_INVALID;
  if (nbr_ptr) *nbr_ptr = sh->nbr_ptr.p;
  if (nbr_idx) *nbr_idx = sh->nbr_idx.p;
  if (psi) *psi = sh->psi.p;
  if (dpsi) *dpsi = sh->dpsi.p;
  if (ddpsi) *ddpsi = sh->ddpsi.p;
  return CGB_OK;
}

int cgb_shape_destroy(cgb_shape* sh) {
  if (!sh) return CGB_OK;
  cgb_context* ctx = sh->ctx;
  if (ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  delete sh;
  if (ctx) cgb::ctx_release(ctx);
  return CGB_OK;
}

namespace {
// Fold::gp_theta0 / gp_active on the device. Both arrays always exist (filled with the
// scalar rest angle and "active" when not given), so a graph captured before a later
// cgb_assembler_set_fold_state reads the new state at replay.
void set_fold_state(cgb_context* ctx, cgb_fold_dev& d, double theta0, const double* theta0_gp,
                    const int8_t* active) {
  cudaStream_t st = ctx->stream;
  const size_t n = static_cast<size_t>(d.n_gp);
  std::vector<double> t0(n, theta0);
  std::vector<int8_t> ac(n, 1);
  if (theta0_gp) std::copy(theta0_gp, theta0_gp + n, t0.begin());
  if (active) std::copy(active, active + n, ac.begin());
  d.theta0 = theta0;
  d.theta0_gp.ensure(n);
  d.active.ensure(n);
  if (n) {
    CGB_CUDA(cudaMemcpyAsync(d.theta0_gp.p, t0.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    CGB_CUDA(cudaMemcpyAsync(d.active.p, ac.data(), n, cudaMemcpyHostToDevice, st));
  }
  CGB_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
  d.has_theta0_gp = true;
  d.has_active = true;
}
}  // namespace

int cgb_assembler_create(cgb_context* ctx, const cgb_shape* faces, const double* face_weight, const cgb_fold* folds,
                         int n_folds, cgb_assembler** out) {
  if (!ctx || !out) return CGB_ERR_INVALID;
  *out = nullptr;
  auto* a = new cgb_assembler();
  const int rc = guarded(ctx, [&] {
    need(faces != nullptr && faces->ctx == ctx, "cgb_assembler_create: faces must come from this context");
    need(faces->n_gp == 0 || face_weight, "cgb_assembler_create: face_weight is NULL");
    need(n_folds >= 0 && (n_folds == 0 || folds), "cgb_assembler_create: bad fold list");
    need(ctx->n_nodes > 0, "cgb_assembler_create: nodes not set");
    bind_device(ctx);
    cudaStream_t st = ctx->stream;
    a->ctx = ctx;
    a->faces = faces;
    a->n_nodes = ctx->n_nodes;
    cgb::upload(a->weight, face_weight, faces->n_gp, st);
    a->folds.resize(n_folds);
    for (int k = 0; k < n_folds; ++k) {
      const cgb_fold& f = folds[k];
      need(f.left && f.right && f.left->ctx == ctx && f.right->ctx == ctx,
           "cgb_assembler_create: fold shape sets must come from this context");
      need(f.left->n_gp == f.right->n_gp, "cgb_assembler_create: fold left/right sizes differ");
      need(f.left->n_gp == 0 || (f.weight && f.tangent), "cgb_assembler_create: fold weight/tangent NULL");
      cgb_fold_dev& d = a->folds[k];
      d.n_gp = f.left->n_gp;
      d.Kt = f.Kt;
      d.theta0 = f.theta0;
      d.left = f.left;
      d.right = f.right;
      cgb::upload(d.weight, f.weight, d.n_gp, st);
      cgb::upload(d.tangent, f.tangent, 2 * static_cast<size_t>(d.n_gp), st);
      set_fold_state(ctx, d, f.theta0, f.theta0_gp, f.active);
    }
    cgb::pattern_build(a);
    a->F.alloc(3 * static_cast<size_t>(a->n_nodes));
    a->x.alloc(3 * static_cast<size_t>(a->n_nodes));
  });
  if (rc == CGB_OK) {
    cgb::ctx_retain(ctx);
    *out = a;
  } else {
    delete a;
  }
  return rc;
}

int cgb_assembler_set_fold_state(cgb_assembler* a, int fold, double theta0, const double* theta0_gp,
                                 const int8_t* active) {
  if (!a || !a->ctx) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(fold >= 0 && fold < static_cast<int>(a->folds.size()), "cgb_assembler_set_fold_state: no such fold");
    bind_device(a->ctx);
    set_fold_state(a->ctx, a->folds[fold], theta0, theta0_gp, active);
  });
}

int cgb_assembler_destroy(cgb_assembler* a) {
  if (!a) return CGB_OK;
  if (a->n_graphs > 0) {
    if (a->ctx) a->ctx->last_error = "cgb_assembler_destroy: destroy its graphs first";
    return CGB_ERR_INVALID;
  }
  cgb_context* ctx = a->ctx;
  if (ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  if (a->h_stage) cudaFreeHost(a->h_stage);
  if (a->side) {
    cudaStreamSynchronize(a->side);
    cudaStreamDestroy(a->side);
  }
  for (cudaEvent_t e : {a->ev_start, a->ev_done}) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : a->ev_chunk) if (e) cudaEventDestroy(e);
  delete a;
  if (ctx) cgb::ctx_release(ctx);
  return CGB_OK;
}

int cgb_assembler_pattern(const cgb_assembler* a, int* n_dofs, int64_t* nnz) {
  if (!a) return CGB_ERR_INVALID;
  if (n_dofs) *n_dofs = 3 * a->n_nodes;
  if (nnz) *nnz = 9 * a->n_blocks;
  return CGB_OK;
}

int cgb_assembler_download_pattern(const cgb_assembler* a, int32_t* outer, int32_t* inner) {
  if (!a) return CGB_ERR_INVALID;
  cgb_context* ctx = a->ctx;
  return guarded(ctx, [&] {
    bind_device(ctx);
    cudaStream_t st = ctx->stream;
    std::vector<int64_t> cp(a->n_nodes + 1);
    std::vector<int32_t> cn(std::max<int64_t>(a->n_blocks, 1));
    CGB_CUDA(cudaMemcpyAsync(cp.data(), a->col_ptr.p, cp.size() * 8, cudaMemcpyDeviceToHost, st));
    if (a->n_blocks)
      CGB_CUDA(cudaMemcpyAsync(cn.data(), a->col_nodes.p, a->n_blocks * 4, cudaMemcpyDeviceToHost, st));
    if (outer) CGB_CUDA(cudaMemcpyAsync(outer, a->outer.p, (3 * static_cast<size_t>(a->n_nodes) + 1) * 4,
                                        cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    if (inner) {
      // Column 3j+c lists rows 3i+r for the block rows i of column j (Assembly.h:84-95).
      int64_t e = 0;
      for (int j = 0; j < a->n_nodes; ++j)
        for (int c = 0; c < 3; ++c)
          for (int64_t b = cp[j]; b < cp[j + 1]; ++b)
            for (int r = 0; r < 3; ++r) inner[e++] = 3 * cn[b] + r;
    }
  });
}

int cgb_assembler_stats(cgb_assembler* a, int64_t out[4]) {
  if (!a) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(out != nullptr, "cgb_assembler_stats: out is NULL");
    bind_device(a->ctx);
    cgb::merge_prepare(a);
    out[0] = a->n_pairs;
    out[1] = a->n_blocks;
    out[2] = a->mrg_n_ent;
    out[3] = a->mrg_n_direct;
  });
}

int cgb_assembler_tensor_stats(cgb_assembler* a, int64_t out[4]) {
  if (!a) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(out != nullptr, "cgb_assembler_tensor_stats: out is NULL");
    bind_device(a->ctx);
    cgb::tc_prepare(a);
    out[0] = a->tc_n_groups;
    out[1] = static_cast<int64_t>(a->tc_fallback_h.size());
    out[2] = a->tc_point_cols;
    out[3] = a->tc_last_per_sm;
  });
}

int cgb_assembler_download_map(const cgb_assembler* a, int32_t* map, int64_t n_entries) {
  if (!a || !map) return CGB_ERR_INVALID;
  cgb_context* ctx = a->ctx;
  return guarded(ctx, [&] {
    need(n_entries == a->n_pairs, "cgb_assembler_download_map: n_entries must equal sum n(n+1)/2");
    bind_device(ctx);
    cudaStream_t st = ctx->stream;
    std::vector<int64_t> cp(a->n_nodes + 1), fptr(a->faces->n_gp + 1);
    std::vector<int32_t> fidx(std::max<int64_t>(a->faces->nnz, 1));
    CGB_CUDA(cudaMemcpyAsync(cp.data(), a->col_ptr.p, cp.size() * 8, cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaMemcpyAsync(fptr.data(), a->faces->nbr_ptr.p, fptr.size() * 8, cudaMemcpyDeviceToHost, st));
    if (a->faces->nnz)
      CGB_CUDA(cudaMemcpyAsync(fidx.data(), a->faces->nbr_idx.p, a->faces->nnz * 4, cudaMemcpyDeviceToHost, st));
    if (n_entries) CGB_CUDA(cudaMemcpyAsync(map, a->map_slot.p, n_entries * 4, cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    // Block slot -> position within column max(ni, nj) (the reference's csrMapping).
    int64_t q = 0;
    for (int g = 0; g < a->faces->n_gp; ++g) {
      const int64_t p0 = fptr[g];
      const int n = static_cast<int>(fptr[g + 1] - p0);
      for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j, ++q) {
          const int hi = std::max(fidx[p0 + i], fidx[p0 + j]);
          map[q] = static_cast<int32_t>(map[q] - cp[hi]);
        }
    }
  });
}

int cgb_set_material(cgb_assembler* a, const double* A, const double* B, const double* D) {
  if (!a) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(A && B && D, "cgb_set_material: NULL matrix");
    std::memcpy(a->A, A, sizeof a->A);
    std::memcpy(a->B, B, sizeof a->B);
    std::memcpy(a->D, D, sizeof a->D);
    a->have_material = true;
  });
}

int cgb_assemble_device(cgb_assembler* a, const double* d_x, double* d_K, double* d_F, int flags) {
  if (!a) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(d_x && d_F, "cgb_assemble_device: x and F are required");
    bind_device(a->ctx);
    cgb::assemble_device(a, d_x, (flags & CGB_TANGENT) ? d_K : nullptr, d_F, flags);
  });
}

int cgb_assemble(cgb_assembler* a, const double* x, double* K_values, double* F, int flags) {
  if (!a) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(x && F, "cgb_assemble: x and F are required");
    need(!(flags & CGB_TANGENT) || K_values, "cgb_assemble: K_values is NULL with CGB_TANGENT");
    cgb_context* ctx = a->ctx;
    bind_device(ctx);
    cudaStream_t st = ctx->stream;
    const size_t ndof = 3 * static_cast<size_t>(a->n_nodes);
    const size_t nnz = 9 * static_cast<size_t>(a->n_blocks);
    const bool want_K = (flags & CGB_TANGENT) != 0;
    if (want_K) a->K.ensure(nnz);
    cgb::prof_begin(ctx, CGB_PHASE_H2D);
    CGB_CUDA(cudaMemcpyAsync(a->x.p, x, ndof * sizeof(double), cudaMemcpyHostToDevice, st));
    cgb::prof_end(ctx, CGB_PHASE_H2D, 0);
    cgb::assemble_device(a, a->x.p, want_K ? a->K.p : nullptr, a->F.p, flags);
    cgb::prof_begin(ctx, CGB_PHASE_D2H);
    if (want_K) CGB_CUDA(cudaMemcpyAsync(K_values, a->K.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaMemcpyAsync(F, a->F.p, ndof * sizeof(double), cudaMemcpyDeviceToHost, st));
    cgb::prof_end(ctx, CGB_PHASE_D2H, 0);
    int dev_err = 0;
    CGB_CUDA(cudaMemcpyAsync(&dev_err, ctx->dev_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    check_device_word(ctx, dev_err);
  });
}

int cgb_point_state_device(cgb_context* ctx, const cgb_shape* pts, const double* d_x, const double* A,
                           const double* B, const double* D, double* d_out) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    need(pts && pts->ctx == ctx, "cgb_point_state: the shape set must come from this context");
    need(A && B && D && (pts->n_gp == 0 || (d_x && d_out)), "cgb_point_state: NULL argument");
    bind_device(ctx);
    cgb::point_state_device(ctx, pts, d_x, A, B, D, d_out);
  });
}

int cgb_point_state(cgb_context* ctx, const cgb_shape* pts, const double* x, const double* A, const double* B,
                    const double* D, double* out) {
  if (!ctx) return CGB_ERR_INVALID;
  return guarded(ctx, [&] {
    need(pts && pts->ctx == ctx, "cgb_point_state: the shape set must come from this context");
    need(A && B && D && (pts->n_gp == 0 || (x && out)), "cgb_point_state: NULL argument");
    need(ctx->n_nodes > 0, "cgb_point_state: nodes not set");
    bind_device(ctx);
    cudaStream_t st = ctx->stream;
    const size_t nx = 3 * static_cast<size_t>(ctx->n_nodes);
    const size_t no = static_cast<size_t>(pts->n_gp) * CGB_POINT_STATE_COLS;
    cgb::DevBuf<double> dx(nx), dout(std::max<size_t>(no, 1));
    CGB_CUDA(cudaMemcpyAsync(dx.p, x, nx * sizeof(double), cudaMemcpyHostToDevice, st));
    cgb::point_state_device(ctx, pts, dx.p, A, B, D, dout.p);
    if (no) CGB_CUDA(cudaMemcpyAsync(out, dout.p, no * sizeof(double), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
  });
}

int cgb_energies(cgb_assembler* a, const double* x, double* E_mem, double* E_ben, double* E_hin) {
  if (!a) return CGB_ERR_INVALID;
  return guarded(a->ctx, [&] {
    need(x != nullptr, "cgb_energies: x is NULL");
    need(a->have_material, "cgb_energies: material not set");
    cgb_context* ctx = a->ctx;
    bind_device(ctx);
    CGB_CUDA(cudaMemcpyAsync(a->x.p, x, 3 * static_cast<size_t>(a->n_nodes) * sizeof(double),
                             cudaMemcpyHostToDevice, ctx->stream));
    double e[3];
    cgb::energies_device(a, a->x.p, e);
    if (E_mem) *E_mem = e[0];
    if (E_ben) *E_ben = e[1];
    if (E_hin) *E_hin = e[2];
  });
}

}  // extern "C"
