// batch.cu — many plates as one problem, and one assembly as one CUDA graph.
//
// Independent plates of uneven size become one assembler over the union of their nodes:
// cgb_shape_concat stacks the plates' shape sets with each plate's neighbour indices
// shifted by its first node, so the union pattern is block diagonal and every kernel of
// an assembly covers the Gauss points of all plates in the same launch. cgb_graph_create
// captures one cgb_assemble_device call (memsets, the chunked residual / tangent kernels
// on their two streams, hinge, output) into a CUDA graph that a Newton iteration replays
// with a single launch. cgb_assembler_set_tuning exposes the launch shape the autotuner
// (curvami_gb300/autotune.py) searches.
#include <algorithm>
#include <vector>

#include "cgb_internal.h"

using cgb::DevBuf;
using cgb::Error;

namespace {

__global__ void offset_copy(int64_t n, const int32_t* __restrict__ in, int32_t off, int32_t* __restrict__ out) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = in[i] + off;
}

__global__ void offset_copy64(int64_t n, const int64_t* __restrict__ in, int64_t off, int64_t* __restrict__ out) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = in[i] + off;
}

unsigned blocks(int64_t n) { return static_cast<unsigned>(std::max<int64_t>(1, (n + 255) / 256)); }

template <typename T>
void copy_into(DevBuf<T>& dst, size_t at, const DevBuf<T>& src, size_t count, cudaStream_t st) {
  if (count) CGB_CUDA(cudaMemcpyAsync(dst.p + at, src.p, count * sizeof(T), cudaMemcpyDeviceToDevice, st));
}

}  // namespace

namespace cgb {

void shape_concat(cgb_context* ctx, const cgb_shape* const* sets, const int32_t* node_offset, int n_sets,
                  cgb_shape* out) {
  cudaStream_t st = ctx->stream;
  int64_t n_gp = 0, nnz = 0;
  int max_n = 0;
  bool have_s = true;
  for (int k = 0; k < n_sets; ++k) {
    const cgb_shape* s = sets[k];
    if (!s || s->ctx != ctx) throw Error(CGB_ERR_INVALID, "cgb_shape_concat: shape sets must come from this context");
    if (node_offset[k] < 0) throw Error(CGB_ERR_INVALID, "cgb_shape_concat: negative node offset");
    n_gp += s->n_gp;
    nnz += s->nnz;
    max_n = std::max(max_n, s->max_n);
    have_s = have_s && (s->nnz == 0 || s->s.n >= static_cast<size_t>(s->nnz));
  }
  if (n_gp >= (1LL << 31) - 1) throw Error(CGB_ERR_CAPACITY, "cgb_shape_concat: more than 2^31 Gauss points");
  if (nnz >= (1LL << 31)) throw Error(CGB_ERR_CAPACITY, "cgb_shape_concat: more than 2^31 neighbour entries");
  out->ctx = ctx;
  out->n_gp = static_cast<int>(n_gp);
  out->nnz = nnz;
  out->max_n = max_n;
  out->gp_xy.alloc(2 * n_gp);
  out->has_xy = true;
  for (int k = 0; k < n_sets; ++k) out->has_xy = out->has_xy && (sets[k]->has_xy || sets[k]->n_gp == 0);
  out->nbr_ptr.alloc(n_gp + 1);
  out->nbr_idx.alloc(nnz);
  if (have_s) out->s.alloc(nnz);
  out->psi.alloc(nnz);
  out->dpsi.alloc(2 * nnz);
  out->ddpsi.alloc(3 * nnz);
  int64_t g0 = 0, e0 = 0;
  for (int k = 0; k < n_sets; ++k) {
    const cgb_shape* s = sets[k];
    const int64_t e = s->nnz;
    // nbr_ptr: the set's offsets shifted by the entries before it (its last entry is the
    // next set's first, so each set writes n_gp values and the final total at the end).
    if (s->n_gp) offset_copy64<<<blocks(s->n_gp), 256, 0, st>>>(s->n_gp, s->nbr_ptr.p, e0, out->nbr_ptr.p + g0);
    if (e) offset_copy<<<blocks(e), 256, 0, st>>>(e, s->nbr_idx.p, node_offset[k], out->nbr_idx.p + e0);
    if (s->gp_xy.n >= 2 * static_cast<size_t>(s->n_gp)) copy_into(out->gp_xy, 2 * g0, s->gp_xy, 2 * s->n_gp, st);
    if (have_s) copy_into(out->s, e0, s->s, e, st);
    copy_into(out->psi, e0, s->psi, e, st);
    copy_into(out->dpsi, 2 * e0, s->dpsi, 2 * e, st);
    copy_into(out->ddpsi, 3 * e0, s->ddpsi, 3 * e, st);
    g0 += s->n_gp;
    e0 += e;
  }
  CGB_CUDA(cudaMemcpyAsync(out->nbr_ptr.p + n_gp, &nnz, sizeof(int64_t), cudaMemcpyHostToDevice, st));
  CGB_CUDA(cudaGetLastError());
  CGB_CUDA(cudaStreamSynchronize(st));
}

}  // namespace cgb

struct cgb_graph {
  cgb_assembler* a = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

template <class F>
int guarded_ctx(cgb_context* ctx, F&& body) {
  try {
    body();
    if (ctx) ctx->last_error.clear();
    return CGB_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    if (ctx) ctx->last_error = e.what();
    return CGB_ERR_INVALID;
  }
}

}  // namespace

extern "C" {

int cgb_shape_concat(cgb_context* ctx, const cgb_shape* const* sets, const int32_t* node_offset, int n_sets,
                     cgb_shape** out) {
  if (!ctx || !out) return CGB_ERR_INVALID;
  *out = nullptr;
  auto* sh = new cgb_shape();
  const int rc = guarded_ctx(ctx, [&] {
    if (n_sets < 1 || !sets || !node_offset) throw Error(CGB_ERR_INVALID, "cgb_shape_concat: empty set list");
    CGB_CUDA(cudaSetDevice(ctx->device));
    cgb::shape_concat(ctx, sets, node_offset, n_sets, sh);
  });
  if (rc == CGB_OK) {
    cgb::ctx_retain(ctx);
    *out = sh;
  } else {
    delete sh;
  }
  return rc;
}

int cgb_assembler_set_tuning(cgb_assembler* a, const cgb_tuning* t) {
  if (!a) return CGB_ERR_INVALID;
  return guarded_ctx(a->ctx, [&] {
    if (!t) throw Error(CGB_ERR_INVALID, "cgb_assembler_set_tuning: tuning is NULL");
    if (t->n_chunks < 0 || t->n_chunks > kMaxChunks) throw Error(CGB_ERR_INVALID, "cgb_assembler_set_tuning: n_chunks must be 0..16");
    if (t->residual_threads != 0 && t->residual_threads != 64 && t->residual_threads != 128 &&
        t->residual_threads != 256)
      throw Error(CGB_ERR_INVALID, "cgb_assembler_set_tuning: residual_threads must be 0, 64, 128 or 256");
    if (t->tangent_ctas_per_sm < 0 || t->tangent_ctas_per_sm > 4)
      throw Error(CGB_ERR_INVALID, "cgb_assembler_set_tuning: tangent_ctas_per_sm must be 0..4");
    if (t->tangent_kind != CGB_TANGENT_TENSOR && t->tangent_kind != CGB_TANGENT_CORES)
      throw Error(CGB_ERR_INVALID, "cgb_assembler_set_tuning: tangent_kind must be CGB_TANGENT_TENSOR or CGB_TANGENT_CORES");
    a->tuning = *t;
  });
}

int cgb_test_stage_timeout(cgb_assembler* a, int on) {
  if (!a) return CGB_ERR_INVALID;
  a->test_stage_extra_tx = on ? 16u : 0u;
  return CGB_OK;
}

int cgb_graph_create(cgb_assembler* a, const double* d_x, double* d_K, double* d_F, int flags, cgb_graph** out) {
  if (!a || !out) return CGB_ERR_INVALID;
  *out = nullptr;
  auto* g = new cgb_graph();
  cgb_context* ctx = a->ctx;
  const int rc = guarded_ctx(ctx, [&] {
    if (!d_x || !d_F) throw Error(CGB_ERR_INVALID, "cgb_graph_create: d_x and d_F are required");
    if ((flags & CGB_TANGENT) && !d_K) throw Error(CGB_ERR_INVALID, "cgb_graph_create: d_K is NULL with CGB_TANGENT");
    if (!ctx->stream) throw Error(CGB_ERR_INVALID, "cgb_graph_create: the context's stream is the legacy default stream");
    CGB_CUDA(cudaSetDevice(ctx->device));
    // One direct call first: it builds every table and buffer the call needs (merge tables,
    // deterministic lists, FP32 copies, the second stream), none of which may be created
    // while a stream is being captured.
    const bool prof = ctx->profile;
    ctx->profile = false;
    cgb::assemble_device(a, d_x, d_K, d_F, flags);
    CGB_CUDA(cudaStreamSynchronize(ctx->stream));
    CGB_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
      cgb::assemble_device(a, d_x, d_K, d_F, flags);
    } catch (...) {
      cudaGraph_t broken = nullptr;
      cudaStreamEndCapture(ctx->stream, &broken);
      if (broken) cudaGraphDestroy(broken);
      ctx->profile = prof;
      throw;
    }
    ctx->profile = prof;
    CGB_CUDA(cudaStreamEndCapture(ctx->stream, &g->graph));
    CGB_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0));
    g->a = a;
    ++a->n_graphs;
  });
  if (rc == CGB_OK) {
    *out = g;
  } else {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
  }
  return rc;
}

int cgb_graph_launch(cgb_graph* g) {
  if (!g || !g->a) return CGB_ERR_INVALID;
  cgb_context* ctx = g->a->ctx;
  return guarded_ctx(ctx, [&] {
    CGB_CUDA(cudaSetDevice(ctx->device));
    cgb::refresh_face_copies(g->a);   // the face set was rebuilt since the capture
    CGB_CUDA(cudaGraphLaunch(g->exec, ctx->stream));
  });
}

int cgb_graph_destroy(cgb_graph* g) {
  if (!g) return CGB_OK;
  if (g->a) {
    cgb_context* ctx = g->a->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    --g->a->n_graphs;
  }
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return CGB_OK;
}

}  // extern "C"
