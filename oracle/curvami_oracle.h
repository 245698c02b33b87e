/*
 * curvami_oracle.h — CPU oracle for the Curvami Gauss-point hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain C++17 restatement (no Eigen, OpenMP,
 * built with -ffp-contract=off) of the reference's shape-function stage and of its
 * Kirchhoff–Love residual/tangent assembly. Only the tests, the smoke check and the
 * benchmark's CPU-baseline / reference arm may load it, and only as the checker or
 * as the timed CPU baseline. The GPU library never links or calls it.
 *
 * Parity status: the reference cannot be compiled here (every hot-path header needs
 * Eigen, which is absent), and it ships no golden vectors for this path. The oracle
 * is therefore pinned by the properties the reference itself relies on:
 * reproducing conditions of the RKPM basis, central-difference consistency of the
 * tangent with the residual (the reference's TangentCheck, main.cpp:651-710), of the
 * residual with the strain energy, and K symmetry. Bit-level parity with the
 * reference binary is unpinned.
 *
 * Every function cites the reference lines it restates.
 */
#ifndef CURVAMI_ORACLE_H
#define CURVAMI_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A crease polyline (Enrichment::FoldLine, core/include/curvami/Enrichment.h:10-15). */
typedef struct {
  const double* xy;   /* 2 * n_vertices doubles, x0 y0 x1 y1 ... */
  int n_vertices;
  int extend_start;
  int extend_end;
  int is_closed;
} orc_crease;

/* Window function selector. 0 = quartic spline (GlobalRKPM.h:15-17, the reference);
 * 1 = cubic B-spline (an extension the reference does not have). */
enum { ORC_KERNEL_QUARTIC = 0, ORC_KERNEL_CUBIC_BSPLINE = 1 };

/* GlobalFRNN::execute (core/include/curvami/FRNN.h:23-78).
 * Pass nbr_idx == NULL to only count: fills nbr_ptr (n_gp + 1 entries) and returns nnz.
 * With nbr_idx/s non-NULL (sized from the count) fills them too. Returns nnz. */
int64_t orc_frnn(const double* node_xy, int n_nodes, const double* gp_xy, int n_gp,
                 double rho, int64_t* nbr_ptr, int32_t* nbr_idx, double* s);

/* Per-node support radius variant of the FRNN (extension): node I is a neighbour
 * of x when |x - x_I| <= rho_node[I]; the cell grid uses cell = max(rho_node).
 * s = |x - x_I| / rho_node[I]. Same ordering rules as orc_frnn. */
int64_t orc_frnn_var(const double* node_xy, int n_nodes, const double* rho_node,
                     const double* gp_xy, int n_gp, int64_t* nbr_ptr, int32_t* nbr_idx,
                     double* s);

/* Enrichment::evaluateIndicator (core/include/curvami/Enrichment.h:23-92).
 * out[0] = f, out[1] = d, out[2..3] = grad f, out[4..6] = hess (xx, yy, xy),
 * out[7] = is_valid. */
void orc_indicator(double px, double py, const orc_crease* crease, double* out);

/* GlobalRKPM::solve (core/include/curvami/GlobalRKPM.h:19-397).
 * Inputs come from orc_frnn. rho_node may be NULL (global rho, the reference) or
 * give a per-node radius (extension; then the window uses s = |x-x_I|/rho_I and the
 * basis stays scaled by the global rho).
 * Outputs, per (Gauss point, neighbour) entry in FRNN order:
 *   psi[nnz], dpsi[2*nnz] (x, y interleaved), ddpsi[3*nnz] (xx, yy, xy interleaved).
 * gp_bad[n_gp] receives 0 / 1 (singular 3x3 block) / 2 (Schur pivot collapse).
 * Returns 0 on success, 1 or 2 when any Gauss point was flagged (the reference
 * throws at that point; outputs are still filled). */
int orc_rkpm(const double* node_xy, int n_nodes, const double* gp_xy, int n_gp,
             const int64_t* nbr_ptr, const int32_t* nbr_idx, const double* s,
             double rho, const double* rho_node, int order, int kernel,
             const orc_crease* creases, int n_creases,
             double* psi, double* dpsi, double* ddpsi, int8_t* gp_bad);

/* Classical laminate ABD (plate/Constitutive.h:10-50) for one isotropic ply as
 * main.cpp:53-61 builds it: A, B, D row-major 3x3 each. */
void orc_abd_isotropic(double E, double nu, double h, double* A, double* B, double* D);

/* NonLinearAssembler::initSparsityPattern (plate/Assembly.h:59-153), optionally
 * widened by the hinge triplet pattern that Meshless::assembleSystem adds with
 * K += K_fold (plate/Meshless.h:113-127; Constraints.h:420-433).
 * Fold Gauss points: n_fold_gp pairs, the left list in (fl_ptr, fl_idx), the right
 * list in (fr_ptr, fr_idx). Pass n_fold_gp = 0 for the face-only pattern.
 * Call 1 (inner == NULL): returns nnz and fills outer[3*n_nodes + 1].
 * Call 2 (inner != NULL): fills inner[nnz], col_ptr[n_nodes+1] / col_nodes (the block
 * rows of every node column, may be NULL), and the per-Gauss-point map
 * map[map_ptr[g] + k] (may be NULL), k over local pairs i <= j in loop order,
 * map_ptr[g] = sum_{g'<g} n(n+1)/2. Returns nnz, or -1 on a mapping miss. */
int64_t orc_pattern(int n_nodes, int n_gp, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                    int n_fold_gp, const int64_t* fl_ptr, const int32_t* fl_idx,
                    const int64_t* fr_ptr, const int32_t* fr_idx,
                    int32_t* outer, int32_t* inner, int64_t* col_ptr, int32_t* col_nodes,
                    int32_t* map);
/* The same in two steps over one column build: orc_pattern_new collects the columns and
 * returns nnz; orc_pattern_fill fills the arrays as call 2 above (outer included);
 * orc_pattern_free releases the columns. */
typedef struct orc_pattern_state orc_pattern_state;
orc_pattern_state* orc_pattern_new(int n_nodes, int n_gp, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                                   int n_fold_gp, const int64_t* fl_ptr, const int32_t* fl_idx,
                                   const int64_t* fr_ptr, const int32_t* fr_idx, int64_t* nnz);
int64_t orc_pattern_fill(const orc_pattern_state* h, int n_nodes, int n_gp, const int64_t* nbr_ptr,
                         const int32_t* nbr_idx, int32_t* outer, int32_t* inner, int64_t* col_ptr,
                         int32_t* col_nodes, int32_t* map);
void orc_pattern_free(orc_pattern_state* h);

/* Face assembly: NonLinearAssembler::updateStiffness (plate/Assembly.h:158-345) with
 * the reference's OpenMP structure (per-thread K and F scratch, guided schedule,
 * index-wise merge). n_threads <= 0 uses omp_get_max_threads().
 * x: nodal displacements (3 per node). K_values[nnz] and F[3*n_nodes] are overwritten.
 * With want_K == 0 only F is produced (the same kernel, K writes skipped). */
int orc_update_stiffness(int n_nodes, int n_gp, const double* gp_weight,
                         const int64_t* nbr_ptr, const int32_t* nbr_idx,
                         const double* dpsi, const double* ddpsi,
                         const int32_t* outer, const int32_t* map, const double* x,
                         const double* A, const double* B, const double* D, int want_K,
                         int n_threads, double* K_values, double* F, const double* gp_xy);

/* One fold (plate/PlateData.h:54-76): n_gp crease Gauss point pairs. */
typedef struct {
  int n_gp;
  const int64_t* l_ptr; const int32_t* l_idx; const double* l_dpsi;
  const int64_t* r_ptr; const int32_t* r_idx; const double* r_dpsi;
  const double* weight;    /* left-side weights (Constraints.h:368) */
  const double* tangent;   /* 2 per Gauss point (left list, Constraints.h:355) */
  double Kt, theta0;
  const double* theta0_gp; /* may be NULL */
  const int8_t* active;    /* may be NULL */
} orc_fold;

/* Constraints::evaluateElasticFold (plate/Constraints.h:341-436) for every fold,
 * scattered into the union pattern: F += hinge force; if K_values != NULL, the hinge
 * tangent triplets are summed into K (the K += K_fold of Meshless.h:119-125).
 * exact_tangent enables the finite-difference dihedral Hessian term (:394-416). */
int orc_hinge(int n_nodes, const double* x, int n_folds, const orc_fold* folds,
              int exact_tangent, const int32_t* outer, const int64_t* col_ptr,
              const int32_t* col_nodes, double* K_values, double* F);

/* Constraints::foldAngleAndGrad (plate/Constraints.h:71-119): F12 packs
 * (a1L, a2L, a1R, a2R). grad may be NULL. Returns theta. */
double orc_fold_angle(const double* F12, double tx, double ty, double* grad);

/* Constraints::computeHingeEnergy (plate/Constraints.h:310-339), summed over folds. */
double orc_hinge_energy(const double* x, int n_folds, const orc_fold* folds);

/* Meshless::computeStrainEnergies (plate/Meshless.h:204-220). */
void orc_strain_energies(int n_gp, const double* gp_weight, const int64_t* nbr_ptr,
                         const int32_t* nbr_idx, const double* dpsi, const double* ddpsi,
                         const double* x, const double* A, const double* B, const double* D,
                         double* E_mem, double* E_ben, const double* gp_xy);

/* Per-Gauss-point kinematics (plate/Kinematics.h:61-120) for inspection:
 * out[0..27] = r0X(3) r0Y(3) r0XX(3) r0YY(3) r0XY(3) b(3) C0inv(4, row-major)
 * E0(3: xx yy xy) E1(3). */
void orc_kinematics(int g, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                    const double* dpsi, const double* ddpsi, const double* x, double* out,
                    const double* X);
/* Kinematics::NaturalCurvature (plate/Kinematics.h:21-45), the one field of the run, as
 * main.cpp:83-95 sets it (sign -1 mountain, +1 valley, theta0 in radians). The functions
 * above add kappa_bar(X) to E1 (E1_el) at the points whose reference coordinates they are
 * given (gp_xy, 2 per point; X for orc_kinematics, whose out[28..30] is E1_el); with NULL
 * coordinates, or inactive, E1_el = E1. */
void orc_set_natural_curvature(int active, double x0, double width, double theta0, double sign);
/* The face assembly's OpenMP schedule: 0 the reference's schedule(guided, 8) (Assembly.h:199;
 * with several threads the per-thread sums, and so the last bits of K and F, vary from run to
 * run), 1 a static split (bitwise the same on every run with the same thread count). */
void orc_set_static_schedule(int on);

#ifdef __cplusplus
}
#endif
#endif
