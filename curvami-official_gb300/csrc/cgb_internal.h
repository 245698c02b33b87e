// cgb_internal.h — host-side internals shared by the CUDA translation units of the
// GB300 Gauss-point library (context, shape sets, assembler, device buffers).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/curvami_gb300.h"

namespace cgb {

// A failure inside the library: carries the C-ABI status code and the message that
// cgb_last_error() returns (the reference's exception text where one exists).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw Error(CGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CGB_CUDA(call) ::cgb::cuda_check((call), #call)

// Owning device buffer (cudaMalloc'd, freed on destruction or reset).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { reset(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { reset(); }
  void alloc(size_t count) {
    reset();
    if (count == 0) count = 1;  // keep a valid pointer for empty sets
    CGB_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void ensure(size_t count) { if (n < count || !p) alloc(count); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

template <class T>
void upload(DevBuf<T>& d, const T* h, size_t count, cudaStream_t s) {
  d.alloc(count);
  if (count) CGB_CUDA(cudaMemcpyAsync(d.p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
}

struct Crease {
  std::vector<double> xy;
  int extend_start = 0, extend_end = 0, is_closed = 0;
};

// Kinematics::NaturalCurvature (plate/Kinematics.h:21-45) as the kernels take it: the band's
// kappa_bar_XX(X) = amp * exp(-((X - x0) / width)^2), amp = sign * theta0 / (sqrt(pi) width).
struct NatCurv {
  int active = 0;
  double x0 = 0.0, width = 1.0, amp = 0.0;
};

}  // namespace cgb

// Opaque handles of the C ABI.
struct cgb_context {
  // Shape sets and assemblers keep their context alive: cgb_destroy only drops the
  // caller's reference, the context is freed when the last handle that uses it is.
  int refs = 1;
  bool closed = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string last_error;
  // Nodes (Meshless::nodes X_ref), interleaved x y.
  int n_nodes = 0;
  std::vector<double> h_node_xy;
  cgb::DevBuf<double> node_xy;
  uint64_t node_gen = 0;  // bumped whenever cgb_set_nodes changes the coordinates
  cgb::NatCurv natcurv;   // natural curvature of every constitutive evaluation (inactive by default)
  // Device-side error word written by kernels (bounds checks, capacity).
  cgb::DevBuf<int> dev_err;
  int* h_err = nullptr;  // pinned mirror
  // Tracing: event pairs per phase, summed when read.
  bool profile = false;
  struct Mark { int phase; cudaEvent_t start, stop; int launches; cudaStream_t stream; };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[CGB_N_PHASES] = {0};
  int64_t prof_launches[CGB_N_PHASES] = {0};
};

struct cgb_shape {
  cgb_context* ctx = nullptr;
  int n_gp = 0;
  int64_t nnz = 0;
  int max_n = 0;  // largest neighbour count of the set
  cgb::DevBuf<double> gp_xy;      // 2 per point
  bool has_xy = false;            // gp_xy holds the points' reference coordinates
  cgb::DevBuf<int64_t> nbr_ptr;   // n_gp + 1
  cgb::DevBuf<int32_t> nbr_idx;   // nnz
  cgb::DevBuf<double> s;          // nnz (normalised distance), may be empty
  cgb::DevBuf<double> psi;        // nnz
  cgb::DevBuf<double> dpsi;       // 2 * nnz (x, y)
  cgb::DevBuf<double> ddpsi;      // 3 * nnz (xx, yy, xy)
  // What a rebuild with other creases needs (sets made by cgb_shape_build only): the
  // shape parameters and the node coordinates the neighbour lists were found on.
  bool rebuildable = false;
  double rho = 0.0;
  int order = 0, kernel = 0;
  int precision = 0;              // CGB_SHAPE_FP64 / CGB_SHAPE_MIXED
  bool has_rho_node = false;
  cgb::DevBuf<double> rho_node;   // n_nodes (per-node radius) when has_rho_node
  uint64_t node_gen = 0;
  uint64_t version = 0;           // bumped by every rebuild (derived copies go stale)
  // Scratch of the crease / RKPM stage, kept for the next rebuild (no allocation per step).
  cgb::DevBuf<double> scr_cxy;    // crease vertices, all creases
  cgb::DevBuf<int8_t> scr_side;   // n_creases * n_nodes
  cgb::DevBuf<double> scr_gind;   // n_creases * 6 * n_gp
  cgb::DevBuf<int8_t> scr_bad;    // n_gp
  cgb::DevBuf<float4> scr_node_pair;  // 2 * n_nodes, mixed precision only
  cgb::DevBuf<float> scr_point_rec;   // point records of the mixed RKPM, n_gp x record floats
};

// Per-fold data kept by the assembler (plate/PlateData.h: Fold; Constraints.h:341).
struct cgb_fold_dev {
  int n_gp = 0;
  double Kt = 0.0, theta0 = 0.0;
  const cgb_shape* left = nullptr;
  const cgb_shape* right = nullptr;
  cgb::DevBuf<double> weight, tangent, theta0_gp;
  cgb::DevBuf<int8_t> active;
  bool has_theta0_gp = false, has_active = false;
  // Merged node list of left U right per crease point (sorted unique nodes),
  // and for every left/right entry its position in that list.
  cgb::DevBuf<int64_t> u_ptr;       // n_gp + 1
  cgb::DevBuf<int32_t> u_node;      // merged nodes
  cgb::DevBuf<int32_t> l_pos, r_pos;
  cgb::DevBuf<int64_t> pair_ptr;    // n_gp + 1, pairs P <= Q over the merged list
  cgb::DevBuf<int32_t> pair_slot;   // block slot of each pair in the union pattern
  int max_u = 0;
  int64_t n_u = 0;      // merged-node entries over all crease points (u_ptr[n_gp])
  int64_t n_pairs = 0;
};

// Most Gauss-point chunks one assembly is split into (residual / tangent overlap).
constexpr int kMaxChunks = 16;

struct cgb_assembler {
  cgb_context* ctx = nullptr;
  const cgb_shape* faces = nullptr;
  int n_nodes = 0;
  int64_t n_blocks = 0;  // 3x3 blocks of the union pattern; nnz = 9 * n_blocks
  cgb::DevBuf<double> weight;       // face Gauss-point weights
  // Union pattern (face blocks U hinge blocks), block-column CSC:
  cgb::DevBuf<int64_t> col_ptr;     // n_nodes + 1 (block offsets)
  cgb::DevBuf<int32_t> col_nodes;   // n_blocks (block rows, ascending per column)
  cgb::DevBuf<int32_t> outer;       // 3 n_nodes + 1 (scalar CSC, the reference's K layout)
  // Face Gauss point -> block slot of each local pair (i <= j) in loop order.
  cgb::DevBuf<int64_t> map_ptr;     // n_gp + 1
  cgb::DevBuf<int32_t> map_slot;    // total pairs
  int64_t n_pairs = 0;
  std::vector<cgb_fold_dev> folds;
  double A[9] = {0}, B[9] = {0}, D[9] = {0};
  bool have_material = false;
  // Accumulators.
  cgb::DevBuf<double> kacc64;       // 9 * n_blocks
  cgb::DevBuf<float> kacc32;        // 12 * n_blocks (padded for 16-byte vector atomics)
  cgb::DevBuf<double> F;            // 3 n_nodes (device scratch for host-buffer calls)
  cgb::DevBuf<double> K;            // 9 n_blocks (device scratch for host-buffer calls)
  cgb::DevBuf<double> x;            // 3 n_nodes
  cgb::DevBuf<float> dpsi32, ddpsi32; // FP32 copies of the face shape derivatives (mixed mode)
  uint64_t faces_version = 0;       // faces->version the copies (FP32, sliced-ELL) were made from
  // Merged contributions of the FP32 tangent: per group of 16 consecutive Gauss points the
  // distinct blocks ("entries", count-descending) and every pair's code in entry order.
  bool mrg_ready = false;
  cgb::DevBuf<int64_t> mrg_ent_ptr;   // n_groups + 1
  cgb::DevBuf<int32_t> mrg_ent_slot;  // block slot of each entry
  cgb::DevBuf<int32_t> mrg_ent_cstart;// (count << 16) | first contribution within its group
  cgb::DevBuf<int8_t> mrg_direct;     // 1: group too large, scatter directly
  cgb::DevBuf<uint16_t> mrg_code;     // per pair: point | i | j, grouped by entry
  // Tensor-core tangent: per face entry the index of its node in its group's sorted node
  // union, per group the union's size, per merged entry the union indices of its block's
  // row and column nodes, and the groups the tensor path does not take (union above 42
  // nodes, or too large to merge) on the device and on the host.
  bool tc_ready = false;
  cgb::DevBuf<uint8_t> tc_nbr_u;
  cgb::DevBuf<int16_t> tc_cell_U;
  cgb::DevBuf<uint16_t> tc_ent_uv;
  cgb::DevBuf<int32_t> tc_fallback;
  std::vector<int32_t> tc_fallback_h;
  int64_t tc_n_groups = 0;            // groups on the tensor path
  int64_t tc_point_cols = 0;          // sum over them of points x MMA columns (N)
  int tc_last_per_sm = 0;             // CTAs per SM of the last tensor-core tangent launch
  cgb_tuning tuning{};                // launch shape (0 = library default)
  cgb::DevBuf<int> work_ctr;          // per-chunk work counters of the residual kernel
  uint32_t test_stage_extra_tx = 0;   // failure-detection test only: bytes the staging never gets
  int n_graphs = 0;                   // live cgb_graph objects on this assembler
  int64_t mrg_n_ent = 0;              // entries over all groups
  int mrg_n_direct = 0;               // groups scattered pair by pair
  // Second stream of the chunked face launch (tangent of chunk c beside residual of c+1).
  cudaStream_t side = nullptr;
  cudaEvent_t ev_start = nullptr, ev_done = nullptr, ev_chunk[kMaxChunks] = {nullptr};
  cgb::DevBuf<float> state32;         // per-point state between the residual and tangent kernels
  cgb::DevBuf<double> state64;
  cgb::DevBuf<int64_t> sell_ptr;      // sliced-ELL copy for the FP64 phase (groups of 32 points)
  cgb::DevBuf<int32_t> sidx;
  cgb::DevBuf<double> sdpsi, sddpsi;
  // Deterministic scatter: contributions ("units") and per-block / per-node ordered lists.
  // K units are either every pair (FP64, or groups the merge cannot take) or, for the FP32
  // tangent, every merged entry (one fixed-order sum per group and block); hinge pairs follow.
  bool det_ready = false;             // F lists
  bool det_pairs_ready = false;       // K lists over pairs
  bool det_entries_ready = false;     // K lists over merged entries
  cgb::DevBuf<int64_t> blk_list_ptr;  // n_blocks + 1 (pair units)
  cgb::DevBuf<int64_t> blk_list;      // pair unit ids, ascending
  cgb::DevBuf<int64_t> ent_list_ptr;  // n_blocks + 1 (entry units)
  cgb::DevBuf<int64_t> ent_list;      // entry unit ids, ascending
  cgb::DevBuf<int64_t> node_list_ptr; // n_nodes + 1
  cgb::DevBuf<int64_t> node_list;     // F contribution ids, ascending
  cgb::DevBuf<double> contrib64;      // 9 per contribution
  cgb::DevBuf<float> contrib32;
  cgb::DevBuf<double> fcontrib;       // 3 per F contribution
  int64_t n_fcontrib = 0;
  int64_t hinge_f_base = 0;
  // Energies.
  cgb::DevBuf<double> energy;       // 3
  // Pinned staging for the host-buffer entry point.
  double* h_stage = nullptr;
  size_t h_stage_bytes = 0;
};

namespace cgb {
void ctx_retain(cgb_context* ctx);
void ctx_release(cgb_context* ctx);
// Tracing helpers (capi.cu): no-ops unless profiling is enabled on the context.
void prof_begin(cgb_context* ctx, int phase, cudaStream_t stream = nullptr);
void prof_end(cgb_context* ctx, int phase, int launches, cudaStream_t stream = nullptr);
// shape.cu
void shape_build(cgb_context* ctx, const double* gp_xy, int n_gp, const cgb_shape_params& prm,
                 const std::vector<Crease>& creases, cgb_shape* out);
// Phi and its derivatives of an existing set recomputed in place with other creases
// (same points, radius and so neighbour lists).
void shape_rebuild(cgb_shape* sh, const std::vector<Crease>& creases);
// The normalised distances s of a set built in mixed precision (which skips them), computed
// on demand with the FRNN's rounded operations; a no-op when the set has them.
void shape_distances(cgb_shape* sh);
// pattern.cu
void pattern_build(cgb_assembler* a);
void deterministic_prepare(cgb_assembler* a);
void shape_concat(cgb_context* ctx, const cgb_shape* const* sets, const int32_t* node_offset, int n_sets,
                  cgb_shape* out);
// Per-block lists of K units: pairs (units [0, n_pairs) then hinge pairs) or merged entries
// (units [0, mrg_n_ent) then hinge pairs; needs merge_prepare and no direct group).
void deterministic_pair_lists(cgb_assembler* a);
void deterministic_entry_lists(cgb_assembler* a);
void merge_prepare(cgb_assembler* a);
// The tensor-core tangent's tables (needs merge_prepare; made once per assembler).
constexpr int kTcMaxUnion = 42;
void tc_prepare(cgb_assembler* a);
// assemble.cu
void assemble_device(cgb_assembler* a, const double* d_x, double* d_K, double* d_F, int flags);
// Re-derive the assembler's copies of the face shape derivatives after a rebuild of the
// face set (no-op when they are current); enqueued on the context stream.
void refresh_face_copies(cgb_assembler* a);
void energies_device(cgb_assembler* a, const double* d_x, double* out3);
// Kinematic state rows (CGB_POINT_STATE_COLS per point) of a shape set at device x.
void point_state_device(cgb_context* ctx, const cgb_shape* S, const double* d_x, const double* A, const double* B,
                        const double* D, double* d_out);
// The shape set's point coordinates when the context's natural curvature is active (the
// kernels evaluate kappa_bar at each point's X), else null; refuses a set without them.
const double* natcurv_points(const cgb_context* ctx, const cgb_shape* S, const char* what);
// err: the context's device error word (bit 8: an index of the caller's arrays was out of
// range and the access was skipped).
void face_mixed_on_arrays(const cgb_face_problem& pr, const double* d_x, double* d_K, double* d_F,
                          float* kacc, int* err, cudaStream_t st);
}  // namespace cgb
