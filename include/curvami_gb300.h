/*
 * curvami_gb300.h — C ABI of the GB300 (sm_103a) Gauss-point hot path of Curvami.
 *
 * Stage A: RKPM shape functions per Gauss point — neighbour gather (GlobalFRNN),
 *          crease-cut visibility, moment matrix, factorisation, Phi / grad Phi /
 *          Hessian Phi (GlobalRKPM).
 * Stage B: large-rotation Kirchhoff-Love residual and tangent with the elastic-hinge
 *          terms, scattered into the reference's CSC stiffness (NonLinearAssembler,
 *          Constraints::evaluateElasticFold, Meshless::assembleSystem*).
 *
 * Plain C types only (pointers and sizes). Every call returns a status code; on a
 * non-zero status cgb_last_error() holds the message (for the reference's own error
 * conditions, the reference's exception text). One context drives one GPU and one
 * CUDA stream; it is not thread-safe. There is no CPU fallback: a missing or
 * unusable GPU is an error.
 *
 * Layout conventions (the reference's):
 *  - node / point coordinates interleaved x, y (2 doubles per point);
 *  - neighbour lists as CSR: nbr_ptr[n_gp + 1] (int64), nbr_idx[nnz] (int32), in the
 *    FRNN order of core/include/curvami/FRNN.h:57-77;
 *  - dpsi: 2 doubles per entry (d/dX, d/dY); ddpsi: 3 per entry (XX, YY, XY);
 *  - x: 3 displacement dofs per node; F: 3 per node;
 *  - K: Eigen::SparseMatrix<double> ColMajor storage of the block-upper stiffness
 *    (plate/Assembly.h:59-99): outer[3 n_nodes + 1], inner[nnz], values[nnz]. The
 *    pattern is the union of the face blocks and the hinge blocks that
 *    Meshless::assembleSystem adds (plate/Meshless.h:113-127); it is fixed once the
 *    assembler exists and values are overwritten by every assembly.
 */
#ifndef CURVAMI_GB300_H
#define CURVAMI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
enum {
  CGB_OK = 0,
  CGB_ERR_INVALID = 1,  /* bad argument or call order */
  CGB_ERR_CUDA = 2,     /* CUDA runtime error (no device, out of memory, ...) */
  CGB_ERR_SINGULAR = 3, /* RKPM: singular moment matrix (GlobalRKPM.h:241-257) */
  CGB_ERR_PIVOT = 4,    /* RKPM: Schur pivot collapsed (GlobalRKPM.h:347-359) */
  CGB_ERR_MAPPING = 5,  /* neighbour missing from the sparsity pattern (Assembly.h:146-152) */
  CGB_ERR_CAPACITY = 6, /* a documented size limit of the kernels was exceeded */
  CGB_ERR_DEVICE = 7    /* a device-side check failed (index out of range) */
};

/* ---- assembly flags ------------------------------------------------------------- */
#define CGB_TANGENT 0x1       /* form K; without it only F (residual) is produced */
#define CGB_HINGE 0x2         /* add elastic-hinge terms (the reference's flagRig == false) */
#define CGB_MIXED 0x4         /* FP64 residual, FP32-class tangent (FP32 CUDA cores or 3xTF32
                                 tensor cores, cgb_tuning.tangent_kind); default FP64 throughout */
#define CGB_DETERMINISTIC 0x8 /* fixed-order segmented-reduction scatter; default atomics */
#define CGB_HINGE_EXACT 0x10  /* hinge tangent with the dihedral Hessian (fold_exact_tangent) */

/* ---- handles --------------------------------------------------------------------- */
typedef struct cgb_context cgb_context;
typedef struct cgb_shape cgb_shape;
typedef struct cgb_assembler cgb_assembler;

/* A crease polyline. Replaces Enrichment::FoldLine
 * (core/include/curvami/Enrichment.h:10-15). */
typedef struct {
  const double* xy; /* 2 * n_vertices doubles */
  int n_vertices;
  int extend_start;
  int extend_end;
  int is_closed;
} cgb_crease;

/* Shape-stage parameters. rho / order as GlobalRKPM::solve (GlobalRKPM.h:19-21).
 * rho_node: NULL for the reference's single radius, else a per-node radius (extension).
 * kernel: 0 quartic spline (GlobalRKPM.h:15-17), 1 cubic B-spline (extension).
 * precision: CGB_SHAPE_FP64 (0, the reference's arithmetic) or CGB_SHAPE_MIXED (1: the
 * per-neighbour sums in FP32 pairs, about 48 significant bits, the moment matrix
 * factored and solved per point in FP64; same neighbours, guards and error messages).
 * Zero-initialised parameters select FP64. */
#define CGB_SHAPE_FP64 0
#define CGB_SHAPE_MIXED 1
typedef struct {
  double rho;
  const double* rho_node;
  int order;
  int kernel;
  int precision;
} cgb_shape_params;

/* One fold for the hinge. Replaces the arguments of Constraints::evaluateElasticFold
 * (plate/Constraints.h:341-347) for one Fold (plate/PlateData.h:54-76). */
typedef struct {
  const cgb_shape* left;
  const cgb_shape* right;
  const double* weight;    /* n_gp, the left Gauss-point weights */
  const double* tangent;   /* 2 * n_gp, the left Gauss-point tangents */
  double Kt;
  double theta0;
  const double* theta0_gp; /* n_gp or NULL (Fold::gp_theta0) */
  const int8_t* active;    /* n_gp or NULL (Fold::gp_active) */
} cgb_fold;

/* ---- context --------------------------------------------------------------------- */
int cgb_create(int device, cgb_context** out);
int cgb_destroy(cgb_context* ctx);
const char* cgb_last_error(const cgb_context* ctx);
/* Use the caller's cudaStream_t (passed as void*) for every launch and copy. */
int cgb_set_stream(cgb_context* ctx, void* stream);
int cgb_synchronize(cgb_context* ctx);

/* Reference node coordinates (Node::X_ref, core/include/curvami/MeshfreeData.h:7-14). */
int cgb_set_nodes(cgb_context* ctx, const double* node_xy, int n_nodes);

/* Natural curvature, Kinematics::NaturalCurvature (plate/Kinematics.h:21-45), set from the
 * config's "natural_curvature" band (main.cpp:83-95): kappa_bar(X) = sign * theta0 * g(X) eX (x) eX,
 * g(X) = exp(-((X - x0) / width)^2) / (sqrt(pi) width); sign -1 mountain, +1 valley. The
 * elastic bending strain E1_el = E1 + kappa_bar (Kinematics.h:110-111) replaces E1 in the
 * constitutive law (Constitutive.h:65) wherever this context evaluates it: the residual and
 * the tangent's resultants of every assembly, the strain energies (Meshless.h:212) and the
 * point state's N and M (its E1 columns stay the geometric curvature, as the exporter's).
 * It needs each point's reference X: shape sets made by cgb_shape_build carry it; an
 * assembly over a set made by cgb_shape_from_host is refused while it is active. Like the
 * reference's single static field, one setting per context, applied from the next call
 * (a graph captured earlier replays the setting it was captured with); active = 0 (or a
 * NULL pointer) switches it off. */
typedef struct {
  int active;
  double x0, width, theta0, sign;
} cgb_natural_curvature;
int cgb_set_natural_curvature(cgb_context* ctx, const cgb_natural_curvature* nc);

/* ---- stage A: shape functions ---------------------------------------------------- */
/* GlobalFRNN::execute + GlobalRKPM::solve for one set of Gauss points
 * (core/include/curvami/FRNN.h:23, core/include/curvami/GlobalRKPM.h:19), as called
 * per domain by SetupHelper::recomputeShapeFunctions (plate/SetupHelper.h:112-138).
 * Neighbour sets are bit-exact with the FRNN (inclusive FP64 distance test without
 * FMA contraction); Phi and its derivatives are computed in FP64.
 * Returns CGB_ERR_SINGULAR / CGB_ERR_PIVOT with the reference's message on a
 * rank-deficient support (the shape set is still created and must be destroyed). */
int cgb_shape_build(cgb_context* ctx, const double* gp_xy, int n_gp,
                    const cgb_shape_params* params, const cgb_crease* creases, int n_creases,
                    cgb_shape** out);
/* SetupHelper::recomputeShapeFunctions for one domain after the creases change
 * (plate/SetupHelper.h:112-138), as progressive creasing calls it at every tip move
 * (plate/ProgressiveCreasing.h:587-613 via main.cpp:613-616): the points, the support
 * radius and so the neighbour lists are kept (they do not depend on the creases), and
 * Phi and its derivatives are recomputed in place with the given cuts; the FRNN is not
 * repeated. Device pointers of the set stay valid. Assemblers built on the set use the
 * new values from their next assembly or graph launch. Only sets made by cgb_shape_build,
 * with the context's nodes unchanged since. Errors as cgb_shape_build (the new values
 * stand, flagged, on CGB_ERR_SINGULAR / CGB_ERR_PIVOT). */
int cgb_shape_rebuild(cgb_shape* sh, const cgb_crease* creases, int n_creases);
/* Wrap shape functions computed elsewhere (GaussPointData::neighbor_node_ids, dPsi,
 * ddPsi; core/include/curvami/MeshfreeData.h:28-34) for the assembly. psi may be NULL. */
int cgb_shape_from_host(cgb_context* ctx, int n_gp, const int64_t* nbr_ptr,
                        const int32_t* nbr_idx, const double* psi, const double* dpsi,
                        const double* ddpsi, cgb_shape** out);
int cgb_shape_size(const cgb_shape* sh, int* n_gp, int64_t* nnz, int* max_neighbours);
/* Copy results to host arrays; any pointer may be NULL. A set built with
 * CGB_SHAPE_MIXED does not keep the distances s (its RKPM does not read them); the first
 * download that asks for s computes them, bitwise equal to an FP64 build's, and needs the
 * context's nodes unchanged since the build. */
int cgb_shape_download(const cgb_shape* sh, int64_t* nbr_ptr, int32_t* nbr_idx, double* s,
                       double* psi, double* dpsi, double* ddpsi);
/* Device pointers of the shape arrays (for callers that keep data on the GPU). */
int cgb_shape_device(const cgb_shape* sh, const int64_t** nbr_ptr, const int32_t** nbr_idx,
                     const double** psi, const double** dpsi, const double** ddpsi);
int cgb_shape_destroy(cgb_shape* sh);

/* ---- stage B: assembly ----------------------------------------------------------- */
/* NonLinearAssembler::initSparsityPattern (plate/Assembly.h:59-153) for the face
 * Gauss points, widened by the hinge blocks of the folds (Meshless::assembleSystem,
 * plate/Meshless.h:113-127). face_weight: GaussPointData::weight per face point. */
int cgb_assembler_create(cgb_context* ctx, const cgb_shape* faces, const double* face_weight,
                         const cgb_fold* folds, int n_folds, cgb_assembler** out);
int cgb_assembler_destroy(cgb_assembler* a);
int cgb_assembler_pattern(const cgb_assembler* a, int* n_dofs, int64_t* nnz);
/* The K pattern (Eigen ColMajor outerIndexPtr / innerIndexPtr). */
int cgb_assembler_download_pattern(const cgb_assembler* a, int32_t* outer, int32_t* inner);
/* NonLinearAssembler::csrMapping (plate/Assembly.h:49-54) of every face Gauss point,
 * concatenated: n(n+1)/2 entries per point, the position of min(ni, nj) among the
 * block rows of column max(ni, nj). */
int cgb_assembler_download_map(const cgb_assembler* a, int32_t* map, int64_t n_entries);
/* Sizes of the assembler's work (no reference counterpart; for measurement): out[0] local
 * pairs over all face Gauss points (sum n(n+1)/2), out[1] 3x3 blocks of K, out[2] merged
 * entries of the FP32 tangent (distinct blocks per group of 16 consecutive Gauss points),
 * out[3] groups too large to merge. The first call builds the merge tables. */
int cgb_assembler_stats(cgb_assembler* a, int64_t out[4]);
/* The tensor-core tangent's share of the work (no reference counterpart; for measurement):
 * out[0] groups of 16 points formed as one tensor-core product, out[1] groups left to the
 * CUDA cores (node union above 42 nodes, or too large to merge), out[2] the sum over the
 * tensor groups of points x MMA columns N (each point is five 128 x N x 8 TF32 MMAs, so
 * the tensor pipe executes 10,240 x out[2] flops per assembly), out[3] the CTAs per SM of
 * the last tensor-core launch (0 before the first). The first call builds the tables. */
int cgb_assembler_tensor_stats(cgb_assembler* a, int64_t out[4]);
/* Fold::gp_theta0 and Fold::gp_active of fold `fold` (plate/PlateData.h:54-76), which
 * progressive creasing rewrites at every step (plate/ProgressiveCreasing.h:621-639):
 * theta0_gp NULL = every point at the scalar theta0, active NULL = every point active.
 * Inactive crease points get no hinge force, stiffness or energy (Constraints.h:350).
 * Graphs captured earlier replay with the new state. */
int cgb_assembler_set_fold_state(cgb_assembler* a, int fold, double theta0, const double* theta0_gp,
                                 const int8_t* active);
/* LaminateProperties A, B, D (plate/PlateData.h:20-35), row-major 3x3 each. */
int cgb_set_material(cgb_assembler* a, const double* A, const double* B, const double* D);

/* Meshless::assembleSystem / assembleSystemInternalOnly (plate/Meshless.h:102-127)
 * with HOST buffers: x[3 n_nodes] in, K_values[nnz] and F[3 n_nodes] out (K_values
 * may be NULL without CGB_TANGENT). Copies x in and K/F out; synchronous. */
int cgb_assemble(cgb_assembler* a, const double* x, double* K_values, double* F, int flags);
/* Same with DEVICE pointers; asynchronous on the context stream. */
int cgb_assemble_device(cgb_assembler* a, const double* d_x, double* d_K, double* d_F, int flags);

/* Meshless::computeStrainEnergies (plate/Meshless.h:204-220) and
 * computeTotalHingeEnergy (plate/Meshless.h:197-202) at x (host buffer). */
int cgb_energies(cgb_assembler* a, const double* x, double* E_mem, double* E_ben,
                 double* E_hin);

/* ---- post-processing: the kinematic state of any point set --------------------------- */
/* Kinematics::compute + Constitutive::evaluate (plate/Kinematics.h:61-120,
 * plate/Constitutive.h:57-70) and the displacement sum_I Psi_I u_I at every point of a shape
 * set (face Gauss points, crease points, or sample points built with cgb_shape_build), for
 * the step exporter (Exporter::writeBinaryStep, plate/Exporter.h:27-92) and the stress
 * sampler (StressSampler::report, plate/StressSampler.h:79-170). Row-major, per point:
 * u(3), r_X(3), r_Y(3), r_XX(3), r_YY(3), r_XY(3), b(3), E0_xx E0_yy E0_xy (tensor),
 * E1_xx E1_yy E1_xy (tensor, the curvature), N(3, Voigt), M(3, Voigt); FP64. A, B, D row-major
 * 3x3 (LaminateProperties). x: 3 n_nodes. The set must carry Psi. */
#define CGB_POINT_STATE_COLS 33
int cgb_point_state(cgb_context* ctx, const cgb_shape* pts, const double* x, const double* A, const double* B,
                    const double* D, double* out);
/* Same with device pointers, asynchronous on the context stream. */
int cgb_point_state_device(cgb_context* ctx, const cgb_shape* pts, const double* d_x, const double* A,
                           const double* B, const double* D, double* d_out);

/* ---- allocation-free face assembly -------------------------------------------------- */
/* No counterpart in the reference. It serves callers that cannot allocate GPU memory
 * while they assemble: cudaMalloc / cudaFree may synchronise the whole device (stalling
 * every other stream of the process), are not allowed while a stream is being captured,
 * and some host frameworks hand out device memory only through their own pool. Such a
 * caller keeps every input in its own device memory and calls this entry point, which
 * allocates nothing.
 *
 * It runs the mixed-precision face assembly (FP64 residual, FP32 tangent, atomic
 * scatter, faces only, no hinge; the formulas of cgb_assemble_device with CGB_TANGENT |
 * CGB_MIXED, but one warp per Gauss point and one scatter per pair, so K agrees with it to
 * FP32 summation order, not bitwise) on caller-owned arrays in the reference's own formats: the
 * neighbour lists and shape derivatives of the face Gauss points, the K column starts
 * (Eigen outerIndexPtr) and the concatenated NonLinearAssembler::csrMapping positions.
 * Its FP32 block accumulator lives in a fixed array inside the library (every GPU that
 * loads the library holds CGB_NOALLOC_MAX_BLOCKS * 48 bytes = 32 MiB of it until the
 * process exits). nnz / 9 above CGB_NOALLOC_MAX_BLOCKS is rejected with
 * CGB_ERR_CAPACITY. The first call on a device looks the array's address up for that
 * device (current device = ctx's); make that first call before any stream capture.
 * Every call shares the one array: calls whose executions overlap on the GPU (other
 * streams, other contexts of the process on the same device) race and corrupt each
 * other's K, so serialise them. All pointers in prob and the x / K / F arguments are
 * device pointers; the call is asynchronous on ctx's stream. The address of the array
 * is kept per device for the life of the process, so a device reset (cudaDeviceReset)
 * while the library is loaded is not supported.
 * With n_gp == 0 no input array is read (they may be NULL) and K and F are set to zero.
 * The sizes must describe the arrays: nnz == outer[3 n_nodes] and max_neighbours >= every
 * neighbour count. The kernels check the indices that reach the library's array or its
 * shared-memory staging (a point with more than max_neighbours neighbours, a node id
 * outside [0, n_nodes), a block beyond nnz / 9): such an access is skipped and the next
 * cgb_synchronize returns CGB_ERR_DEVICE. Other inconsistencies between the arrays (a
 * map_ptr or csr_map that does not match nbr_ptr) are undefined behaviour. */
#define CGB_NOALLOC_MAX_BLOCKS 699050
typedef struct {
  int n_gp;                /* face Gauss points */
  int n_nodes;
  int max_neighbours;      /* largest neighbour count of any Gauss point */
  int64_t nnz;             /* outer[3 n_nodes] */
  const int64_t* nbr_ptr;  /* n_gp + 1 */
  const int32_t* nbr_idx;
  const double* dpsi;      /* 2 per entry */
  const double* ddpsi;     /* 3 per entry */
  const double* weight;    /* n_gp */
  const int64_t* map_ptr;  /* n_gp + 1: sum of n(n+1)/2 over the earlier points */
  const int32_t* csr_map;  /* csrMapping positions, concatenated */
  const int32_t* outer;    /* 3 n_nodes + 1 */
  double A[9], B[9], D[9]; /* laminate stiffness, row-major, host values */
} cgb_face_problem;
int cgb_assemble_face_noalloc(cgb_context* ctx, const cgb_face_problem* prob, const double* d_x,
                              double* d_K, double* d_F);

/* ---- batching and graphs (no reference counterpart: the reference assembles one plate
 * per call on the host) ------------------------------------------------------------ */
/* The union of n_sets shape sets with the neighbour indices of set k shifted by
 * node_offset[k]: independent plates become one set over the union of their nodes
 * (call cgb_set_nodes with the union before building the assembler on it). The inputs
 * stay valid and owned by the caller. */
int cgb_shape_concat(cgb_context* ctx, const cgb_shape* const* sets, const int32_t* node_offset, int n_sets,
                     cgb_shape** out);

/* Launch shape of an assembly; 0 keeps the library's choice. n_chunks (1..16): Gauss-point
 * chunks whose residual and tangent kernels overlap on two streams (default 4 from 65,536
 * points, else 1); residual_threads (64, 128, 256): block size of the residual kernel
 * (default 256); tangent_ctas_per_sm (1..4): resident CTAs per SM of the merged FP32
 * tangent (default: as many as fit); tangent_kind, the mixed-precision tangent:
 * CGB_TANGENT_CORES (the default) every cell on the CUDA cores (FP32, merged
 * contributions); CGB_TANGENT_TENSOR forms each quadrature cell's blocks as one
 * tensor-core product (tcgen05, 3xTF32, FP32 accumulation) where the cell's neighbour union
 * has at most 42 nodes, the rest on the CUDA cores. With the quadratic basis's 20-45
 * neighbours per point the CUDA-core form is both faster (0.54 against 0.82 ms for
 * 160,000 points on one GB300) and closer to FP64 (Frobenius error of K 1e-7 against 1e-6). */
#define CGB_TANGENT_CORES 0
#define CGB_TANGENT_TENSOR 1
typedef struct cgb_tuning {
  int n_chunks;
  int residual_threads;
  int tangent_ctas_per_sm;
  int tangent_kind;
} cgb_tuning;
int cgb_assembler_set_tuning(cgb_assembler* a, const cgb_tuning* t);

/* One cgb_assemble_device call (the given device buffers and flags) captured as a CUDA
 * graph on the context's stream; cgb_graph_launch replays it (the buffers are read and
 * written at replay time). Creation runs the call once directly first. A graph must be
 * destroyed before its assembler (cgb_assembler_destroy refuses while graphs exist). */
typedef struct cgb_graph cgb_graph;
int cgb_graph_create(cgb_assembler* a, const double* d_x, double* d_K, double* d_F, int flags, cgb_graph** out);
int cgb_graph_launch(cgb_graph* g);
int cgb_graph_destroy(cgb_graph* g);

/* Failure-detection test hook (no reference counterpart): on != 0 makes every staging
 * wait of the FP32 tangent expect 16 bytes that never arrive, so the bounded wait (about
 * one second of SM clock per launch) gives up; the kernel leaves its remaining work undone
 * and the next synchronising call returns CGB_ERR_DEVICE. No fault and no hang: the
 * copies that were issued complete, only the expected count is never reached. */
int cgb_test_stage_timeout(cgb_assembler* a, int on);

/* ---- tracing (library extension; the reference only prints wall-clock times) ------ */
/* CUDA events around every phase of cgb_assemble / cgb_assemble_device and of
 * cgb_shape_build, summed per phase until read. Off by default; costs two event records
 * per phase when on. */
enum {
  CGB_PHASE_H2D = 0,    /* x host -> device (cgb_assemble only) */
  CGB_PHASE_ZERO = 1,   /* clearing of the accumulators */
  CGB_PHASE_FACE = 2,    /* face Gauss points: kinematics, resultants, residual (FP64 kernels) */
  CGB_PHASE_HINGE = 3,   /* elastic hinge */
  CGB_PHASE_REDUCE = 4,  /* block -> CSC output, or the deterministic reductions */
  CGB_PHASE_D2H = 5,     /* K, F device -> host (cgb_assemble only) */
  CGB_PHASE_TANGENT = 6, /* face tangent and its scatter (second stream, overlaps FACE) */
  CGB_PHASE_FRNN = 7,    /* shape build: neighbour count and fill (FRNN.h:23-78) */
  CGB_PHASE_CREASE = 8,  /* shape build: node sides and Gauss-point crease indicators */
  CGB_PHASE_RKPM = 9,    /* shape build: moments, inverse, Phi / grad / Hessian */
  CGB_N_PHASES = 10
};
int cgb_profile_enable(cgb_context* ctx, int on);
/* ms[CGB_N_PHASES] summed device time, launches[CGB_N_PHASES] kernels launched by the
 * library in each phase; reset != 0 clears the totals after reading. */
int cgb_profile_read(cgb_context* ctx, double* ms, int64_t* launches, int reset);

#ifdef __cplusplus
}
#endif
#endif /* CURVAMI_GB300_H */
