// curvami_oracle.cpp — CPU oracle for the Curvami Gauss-point hot path.
//
// TEST INFRASTRUCTURE ONLY (see curvami_oracle.h): a C++17 restatement, without
// Eigen, of the reference's FRNN, crease indicator, RKPM solve, sparsity pattern,
// face assembly, elastic hinge and energies. Expressions follow the reference's
// evaluation order (left to right, as Eigen evaluates the small fixed-size products
// coefficient by coefficient), and the file is compiled with -ffp-contract=off, so a
// single-threaded run is the fixed-order sum the GPU's deterministic FP64 mode is
// compared against.
//
// Parity unpinned at the bit level against the reference binary (which cannot be
// built here: it needs Eigen); pinned by the reproducing conditions, the tangent and
// residual finite-difference checks and K symmetry (tests/test_oracle_*.py).
#include "curvami_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V2 { double x, y; };
struct V3 { double v[3]; };

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// ---------------------------------------------------------------------------------
// FRNN: core/include/curvami/FRNN.h:23-78.
// Cell size = rho; cell (x, y) = floor((p - min) / cell); cols = ceil(span_x / cell)+1;
// a flattened key y*cols + x looked up in a map of non-empty cells, so keys that wrap
// across a row behave exactly as in the reference. Scan order: dx outer, dy inner,
// node index ascending within a cell; test dist2 <= rho^2 (inclusive).
// ---------------------------------------------------------------------------------
struct CellGrid {
  double cell, minx, miny;
  int cols;
  std::unordered_map<long long, std::vector<int>> grid;
};

void build_grid(const double* node_xy, int n_nodes, double cell, CellGrid& G) {
  G.cell = cell;
  double minx = node_xy[0], miny = node_xy[1], maxx = node_xy[0];
  for (int i = 0; i < n_nodes; ++i) {
    minx = std::min(minx, node_xy[2 * i]);
    miny = std::min(miny, node_xy[2 * i + 1]);
    maxx = std::max(maxx, node_xy[2 * i]);
  }
  G.minx = minx; G.miny = miny;
  G.cols = static_cast<int>(std::ceil((maxx - minx) / cell)) + 1;
  G.grid.clear();
  for (int i = 0; i < n_nodes; ++i) {
    int cx = static_cast<int>(std::floor((node_xy[2 * i] - minx) / cell));
    int cy = static_cast<int>(std::floor((node_xy[2 * i + 1] - miny) / cell));
    G.grid[static_cast<long long>(cy) * G.cols + cx].push_back(i);
  }
}

template <class Accept>
int64_t frnn_impl(const double* node_xy, int n_nodes, const double* gp_xy, int n_gp, double cell,
                  int64_t* nbr_ptr, int32_t* nbr_idx, double* s, Accept accept) {
  if (n_nodes <= 0 || n_gp <= 0) {
    if (nbr_ptr) for (int g = 0; g <= std::max(n_gp, 0); ++g) nbr_ptr[g] = 0;
    return 0;
  }
  CellGrid G;
  build_grid(node_xy, n_nodes, cell, G);
  int64_t nnz = 0;
  for (int g = 0; g < n_gp; ++g) {
    nbr_ptr[g] = nnz;
    const double gx = gp_xy[2 * g], gy = gp_xy[2 * g + 1];
    int qx = static_cast<int>(std::floor((gx - G.minx) / G.cell));
    int qy = static_cast<int>(std::floor((gy - G.miny) / G.cell));
    for (int dx = -1; dx <= 1; ++dx) {
      for (int dy = -1; dy <= 1; ++dy) {
        auto it = G.grid.find(static_cast<long long>(qy + dy) * G.cols + (qx + dx));
        if (it == G.grid.end()) continue;
        for (int j : it->second) {
          const double ddx = node_xy[2 * j] - gx;
          const double ddy = node_xy[2 * j + 1] - gy;
          const double dist2 = ddx * ddx + ddy * ddy;
          double sv;
          if (accept(j, dist2, sv)) {
            if (nbr_idx) { nbr_idx[nnz] = j; s[nnz] = sv; }
            ++nnz;
          }
        }
      }
    }
  }
  nbr_ptr[n_gp] = nnz;
  return nnz;
}

// ---------------------------------------------------------------------------------
// Crease indicator: core/include/curvami/Enrichment.h:23-92.
// ---------------------------------------------------------------------------------
struct Indicator {
  double f = 0, d = std::numeric_limits<double>::infinity();
  double gx = 0, gy = 0, hxx = 0, hyy = 0, hxy = 0;
  bool valid = false;
};

Indicator indicator(double px, double py, const orc_crease& fold) {
  Indicator out;
  const size_t N = static_cast<size_t>(fold.n_vertices);
  if (N < 2) return out;
  double Cx = 0, Cy = 0, t_best = 0.0, snx = 0, sny = 0;
  size_t idx_best = 0;
  const double inf = std::numeric_limits<double>::infinity();
  for (size_t i = 0; i < N - 1; ++i) {
    const double Ax = fold.xy[2 * i], Ay = fold.xy[2 * i + 1];
    const double Bx = fold.xy[2 * i + 2], By = fold.xy[2 * i + 3];
    const double vx = Bx - Ax, vy = By - Ay;
    const double v_sq = vx * vx + vy * vy;
    if (v_sq == 0) continue;
    const double wx = px - Ax, wy = py - Ay;
    const double t = (wx * vx + wy * vy) / v_sq;
    const double t_min = (i == 0 && fold.extend_start) ? -inf : 0.0;
    const double t_max = (i == N - 2 && fold.extend_end) ? inf : 1.0;
    const double tc = std::max(t_min, std::min(t_max, t));
    const double cx = Ax + tc * vx, cy = Ay + tc * vy;
    const double ex = px - cx, ey = py - cy;
    const double cur = ex * ex + ey * ey;
    if (cur < out.d * out.d) {
      out.d = std::sqrt(cur);
      Cx = cx; Cy = cy; idx_best = i; t_best = tc;
      const double L = std::sqrt(v_sq);
      snx = -vy / L; sny = vx / L;
    }
  }
  out.valid = (out.d > 1e-12);
  if (!out.valid) { out.f = 0.0; return out; }
  const double ux = (px - Cx) / out.d, uy = (py - Cy) / out.d;
  const double dp = ux * snx + uy * sny;
  const bool start_cap = (idx_best == 0 && t_best == 0.0 && !fold.extend_start && !fold.is_closed);
  const bool end_cap = (idx_best == N - 2 && t_best == 1.0 && !fold.extend_end && !fold.is_closed);
  if (start_cap || end_cap) {
    out.f = dp;
    out.gx = (snx - out.f * ux) / out.d;
    out.gy = (sny - out.f * uy) / out.d;
    const double d2 = out.d * out.d;
    out.hxx = (3 * out.f * ux * ux - 2 * snx * ux - out.f) / d2;
    out.hyy = (3 * out.f * uy * uy - 2 * sny * uy - out.f) / d2;
    out.hxy = (3 * out.f * ux * uy - (snx * uy + ux * sny)) / d2;
  } else {
    out.f = (dp >= 0.0) ? 1.0 : -1.0;
  }
  return out;
}

// ---------------------------------------------------------------------------------
// Window functions. Quartic spline: GlobalRKPM.h:15-17 (dw cut off below 1e-14).
// Cubic B-spline: extension, same cut-offs.
// ---------------------------------------------------------------------------------
inline void window(int kernel, double s, double& w, double& dw, double& d2w) {
  if (kernel == ORC_KERNEL_QUARTIC) {
    if (s >= 1.0) { w = 0.0; } else { double s2 = s * s; w = 1.0 - 6.0 * s2 + 8.0 * s2 * s - 3.0 * s2 * s2; }
    if (s >= 1.0 || s < 1e-14) dw = 0.0; else dw = -12.0 * s + 24.0 * s * s - 12.0 * s * s * s;
    if (s >= 1.0) d2w = 0.0; else d2w = -12.0 + 48.0 * s - 36.0 * s * s;
  } else {
    if (s >= 1.0) { w = 0.0; dw = 0.0; d2w = 0.0; return; }
    if (s <= 0.5) {
      w = 2.0 / 3.0 - 4.0 * s * s + 4.0 * s * s * s;
      dw = (s < 1e-14) ? 0.0 : -8.0 * s + 12.0 * s * s;
      d2w = -8.0 + 24.0 * s;
    } else {
      const double r = 1.0 - s;
      w = 4.0 / 3.0 * r * r * r;
      dw = -4.0 * r * r;
      d2w = 8.0 * r;
    }
  }
}

// Packed symmetric index K[i][j] (GlobalRKPM.h:29-36): row-major over i <= j.
struct Packed {
  int np, nm;
  std::vector<int> K;
  explicit Packed(int np_) : np(np_), nm(0), K(np_ * np_) {
    for (int i = 0; i < np; ++i)
      for (int j = i; j < np; ++j) { K[i * np + j] = K[j * np + i] = nm++; }
  }
  int operator()(int i, int j) const { return K[i * np + j]; }
};

using M3 = double[3][3];

// Eigen's 3x3 inverse (cofactors, det from the first column).
void inverse3(const M3 m, M3 inv) {
  const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  const double c10 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  const double c20 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  const double det = m[0][0] * c00 + m[0][1] * c10 + m[0][2] * c20;
  const double id = 1.0 / det;
  inv[0][0] = c00 * id;
  inv[1][0] = c10 * id;
  inv[2][0] = c20 * id;
  inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
  inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
  inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
  inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
  inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
  inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
}

void mul3(const M3 a, const M3 b, M3 c) {
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) c[r][k] = a[r][0] * b[0][k] + a[r][1] * b[1][k] + a[r][2] * b[2][k];
}

// ---------------------------------------------------------------------------------
// Kinematics::NaturalCurvature (plate/Kinematics.h:21-45): one field for the whole run
// (the reference's function-local static), set by orc_set_natural_curvature.
// ---------------------------------------------------------------------------------
struct NaturalCurvature {
  bool active = false;
  double x0 = 0.0, width = 1.0, theta0 = 0.0, sign = -1.0;
  double g(double X) const {
    const double t = (X - x0) / width;
    return std::exp(-t * t) / (1.7724538509055160273 * width);
  }
  double kappa_xx(double X) const { return active ? sign * theta0 * g(X) : 0.0; }
};
NaturalCurvature g_natural;
// The face assembly's loop schedule: the reference's guided one (rounding varies from run to
// run with more than one thread), or static (the same rounding on every run).
bool g_static_schedule = false;

// ---------------------------------------------------------------------------------
// Kinematics::compute (plate/Kinematics.h:61-120). X: the point's reference coordinates
// (for the natural curvature; NULL when the caller has none, then E1_el = E1).
// ---------------------------------------------------------------------------------
struct Kin {
  double r0X[3], r0Y[3], r0XX[3], r0YY[3], r0XY[3];
  double C0inv[2][2];
  double b[3];
  double E0[2][2], E1[2][2];
  double E1el[2][2];  // E1 + kappa_bar (Kinematics.h:110-111)
};

void kinematics(int64_t p0, int64_t p1, const int32_t* nbr_idx, const double* dpsi,
                const double* ddpsi, const double* x, Kin& k, const double* X = nullptr) {
  double r0X[3] = {1.0, 0.0, 0.0}, r0Y[3] = {0.0, 1.0, 0.0};
  double r0XX[3] = {0, 0, 0}, r0YY[3] = {0, 0, 0}, r0XY[3] = {0, 0, 0};
  for (int64_t e = p0; e < p1; ++e) {
    const double* u = x + 3 * static_cast<int64_t>(nbr_idx[e]);
    const double dx = dpsi[2 * e], dy = dpsi[2 * e + 1];
    const double dxx = ddpsi[3 * e], dyy = ddpsi[3 * e + 1], dxy = ddpsi[3 * e + 2];
    for (int c = 0; c < 3; ++c) {
      r0X[c] += u[c] * dx;
      r0Y[c] += u[c] * dy;
      r0XX[c] += u[c] * dxx;
      r0YY[c] += u[c] * dyy;
      r0XY[c] += u[c] * dxy;
    }
  }
  std::memcpy(k.r0X, r0X, sizeof r0X); std::memcpy(k.r0Y, r0Y, sizeof r0Y);
  std::memcpy(k.r0XX, r0XX, sizeof r0XX); std::memcpy(k.r0YY, r0YY, sizeof r0YY);
  std::memcpy(k.r0XY, r0XY, sizeof r0XY);
  const double C00 = dot3(r0X, r0X), C11 = dot3(r0Y, r0Y), C01 = dot3(r0X, r0Y);
  // Eigen 2x2 inverse: det = m00*m11 - m10*m01, entries scaled by 1/det.
  const double det = C00 * C11 - C01 * C01;
  const double id = 1.0 / det;
  k.C0inv[0][0] = C11 * id;
  k.C0inv[1][0] = -C01 * id;
  k.C0inv[0][1] = -C01 * id;
  k.C0inv[1][1] = C00 * id;
  double n[3];
  cross3(r0X, r0Y, n);
  const double area = std::sqrt(dot3(n, n));
  for (int c = 0; c < 3; ++c) k.b[c] = n[c] / area;
  k.E0[0][0] = 0.5 * (C00 - 1.0);
  k.E0[1][1] = 0.5 * (C11 - 1.0);
  k.E0[0][1] = k.E0[1][0] = 0.5 * (C01 - 0.0);
  k.E1[0][0] = -dot3(r0XX, k.b);
  k.E1[1][1] = -dot3(r0YY, k.b);
  k.E1[0][1] = k.E1[1][0] = -dot3(r0XY, k.b);
  std::memcpy(k.E1el, k.E1, sizeof k.E1);
  if (g_natural.active && X) k.E1el[0][0] += g_natural.kappa_xx(X[0]);
}

// Constitutive::evaluate (plate/Constitutive.h:57-70): N = A e0 + B e1, M = B^T e0 + D e1,
// e1 from E1_el (Constitutive.h:65).
void resultants(const Kin& k, const double* A, const double* B, const double* D, double* N, double* M) {
  const double e0[3] = {k.E0[0][0], k.E0[1][1], 2.0 * k.E0[0][1]};
  const double e1[3] = {k.E1el[0][0], k.E1el[1][1], 2.0 * k.E1el[0][1]};
  for (int r = 0; r < 3; ++r) {
    const double Ae = A[3 * r] * e0[0] + A[3 * r + 1] * e0[1] + A[3 * r + 2] * e0[2];
    const double Be = B[3 * r] * e1[0] + B[3 * r + 1] * e1[1] + B[3 * r + 2] * e1[2];
    N[r] = Ae + Be;
    const double Bt = B[r] * e0[0] + B[3 + r] * e0[1] + B[6 + r] * e0[2];
    const double De = D[3 * r] * e1[0] + D[3 * r + 1] * e1[1] + D[3 * r + 2] * e1[2];
    M[r] = Bt + De;
  }
}

}  // namespace

extern "C" {

int64_t orc_frnn(const double* node_xy, int n_nodes, const double* gp_xy, int n_gp, double rho,
                 int64_t* nbr_ptr, int32_t* nbr_idx, double* s) {
  const double rho2 = rho * rho;
  return frnn_impl(node_xy, n_nodes, gp_xy, n_gp, rho, nbr_ptr, nbr_idx, s,
                   [&](int, double dist2, double& sv) {
                     if (dist2 <= rho2) { sv = std::sqrt(dist2) / rho; return true; }
                     return false;
                   });
}

int64_t orc_frnn_var(const double* node_xy, int n_nodes, const double* rho_node, const double* gp_xy,
                     int n_gp, int64_t* nbr_ptr, int32_t* nbr_idx, double* s) {
  double cell = 0.0;
  for (int i = 0; i < n_nodes; ++i) cell = std::max(cell, rho_node[i]);
  return frnn_impl(node_xy, n_nodes, gp_xy, n_gp, cell, nbr_ptr, nbr_idx, s,
                   [&](int j, double dist2, double& sv) {
                     const double r = rho_node[j];
                     if (dist2 <= r * r) { sv = std::sqrt(dist2) / r; return true; }
                     return false;
                   });
}

void orc_indicator(double px, double py, const orc_crease* crease, double* out) {
  Indicator I = indicator(px, py, *crease);
  out[0] = I.f; out[1] = I.d; out[2] = I.gx; out[3] = I.gy;
  out[4] = I.hxx; out[5] = I.hyy; out[6] = I.hxy; out[7] = I.valid ? 1.0 : 0.0;
}

// GlobalRKPM::solve (core/include/curvami/GlobalRKPM.h:19-397), one Gauss point at a
// time (the reference runs the same per-point arithmetic phase by phase over all
// points; per point the operations and their order are the same).
int orc_rkpm(const double* node_xy, int n_nodes, const double* gp_xy, int n_gp,
             const int64_t* nbr_ptr, const int32_t* nbr_idx, const double* s, double rho,
             const double* rho_node, int order, int kernel, const orc_crease* creases, int n_creases,
             double* psi_out, double* dpsi_out, double* ddpsi_out, int8_t* gp_bad) {
  (void)n_nodes;
  const int np = (order + 1) * (order + 2) / 2;
  const Packed K(np);
  const int nm = K.nm;
  int worst = 0;

  // Per-node crease side (Enrichment.h:23-92 evaluated at the node; GlobalRKPM.h:92-93).
  // Depends only on the node, so it is hoisted out of the per-pair loop; identical values.
  #pragma omp parallel
  {
    std::vector<double> PSI, dPx, dPy, d2Pxx, d2Pyy, d2Pxy, CSI, ETA;
    std::vector<double> P, dPdX, dPdY, d2PdX2, d2PdY2, d2PdXDY;
    std::vector<double> Mm(6 * nm), Mi(6 * nm);
    std::vector<Indicator> gind(n_creases);
    std::vector<double> xp(order + 1), yp(order + 1);
    int local_worst = 0;
    #pragma omp for schedule(static)
    for (int g = 0; g < n_gp; ++g) {
      const int64_t p0 = nbr_ptr[g], p1 = nbr_ptr[g + 1];
      const int n = static_cast<int>(p1 - p0);
      const double gx = gp_xy[2 * g], gy = gp_xy[2 * g + 1];
      PSI.assign(n, 0); dPx.assign(n, 0); dPy.assign(n, 0);
      d2Pxx.assign(n, 0); d2Pyy.assign(n, 0); d2Pxy.assign(n, 0);
      CSI.assign(n, 0); ETA.assign(n, 0);
      // Weight jets, GlobalRKPM.h:59-84 (with the reference's d2x/d2y as written).
      for (int a = 0; a < n; ++a) {
        const int64_t e = p0 + a;
        const int j = nbr_idx[e];
        const double xi = (gx - node_xy[2 * j]) / rho;
        const double eta = (gy - node_xy[2 * j + 1]) / rho;
        CSI[a] = xi; ETA[a] = eta;
        // Window in the node's own normalised offset (identity for a global rho).
        const double fac = rho_node ? rho / rho_node[j] : 1.0;
        const double zx = rho_node ? xi * fac : xi, zy = rho_node ? eta * fac : eta;
        const double si = s[e];
        double wi, d, dd;
        window(kernel, si, wi, d, dd);
        const double dx = (si == 0.0) ? 0.0 : zx / si;
        const double dy = (si == 0.0) ? 0.0 : zy / si;
        PSI[a] = wi;
        dPx[a] = d * dx;
        dPy[a] = d * dy;
        const double si3 = si * si * si;
        const double d2x = (si == 0.0) ? dd : (zx * zx) / si3;
        const double d2y = (si == 0.0) ? dd : (zy * zy) / si3;
        d2Pxx[a] = dd * dx * dx + d * d2x;
        d2Pyy[a] = dd * dy * dy + d * d2y;
        d2Pxy[a] = (si == 0.0) ? 0.0 : dd * dx * dy + d * (-(zx * zy) / si3);
        if (rho_node) {
          dPx[a] *= fac; dPy[a] *= fac;
          const double f2 = fac * fac;
          d2Pxx[a] *= f2; d2Pyy[a] *= f2; d2Pxy[a] *= f2;
        }
      }
      // Crease visibility, GlobalRKPM.h:87-112.
      for (int c = 0; c < n_creases; ++c) gind[c] = indicator(gx, gy, creases[c]);
      for (int a = 0; a < n; ++a) {
        const int j = nbr_idx[p0 + a];
        for (int c = 0; c < n_creases; ++c) {
          const Indicator& iG = gind[c];
          const Indicator iN = indicator(node_xy[2 * j], node_xy[2 * j + 1], creases[c]);
          const double sn = (iN.f >= 0.0) ? 1.0 : -1.0;
          const double W = 0.5 * (1.0 + sn * iG.f);
          const double dWx = 0.5 * sn * iG.gx * rho, dWy = 0.5 * sn * iG.gy * rho;
          const double ddWxx = 0.5 * sn * iG.hxx * rho * rho;
          const double ddWyy = 0.5 * sn * iG.hyy * rho * rho;
          const double ddWxy = 0.5 * sn * iG.hxy * rho * rho;
          const double oW = PSI[a], ox = dPx[a], oy = dPy[a];
          const double oxx = d2Pxx[a], oyy = d2Pyy[a], oxy = d2Pxy[a];
          PSI[a] *= W;
          dPx[a] = ox * W + oW * dWx;
          dPy[a] = oy * W + oW * dWy;
          d2Pxx[a] = oxx * W + 2.0 * ox * dWx + oW * ddWxx;
          d2Pyy[a] = oyy * W + 2.0 * oy * dWy + oW * ddWyy;
          d2Pxy[a] = oxy * W + ox * dWy + oy * dWx + oW * ddWxy;
        }
      }
      // Basis jets, GlobalRKPM.h:114-152 (np rows per entry, degree-major, p_y ascending).
      P.assign(np * n, 0); dPdX.assign(np * n, 0); dPdY.assign(np * n, 0);
      d2PdX2.assign(np * n, 0); d2PdY2.assign(np * n, 0); d2PdXDY.assign(np * n, 0);
      for (int a = 0; a < n; ++a) {
        const double xx = CSI[a], yy = ETA[a];
        xp[0] = 1.0; yp[0] = 1.0;
        for (int p = 1; p <= order; ++p) { xp[p] = xp[p - 1] * xx; yp[p] = yp[p - 1] * yy; }
        int idx = 0;
        for (int d = 0; d <= order; ++d) {
          for (int py = 0; py <= d; ++py) {
            const int px = d - py;
            double* at = &P[idx * n + a];
            *at = xp[px] * yp[py];
            if (px > 0) dPdX[idx * n + a] = static_cast<double>(px) * xp[px - 1] * yp[py];
            if (py > 0) dPdY[idx * n + a] = static_cast<double>(py) * xp[px] * yp[py - 1];
            if (px > 1) d2PdX2[idx * n + a] = static_cast<double>(px * (px - 1)) * xp[px - 2] * yp[py];
            if (py > 1) d2PdY2[idx * n + a] = static_cast<double>(py * (py - 1)) * xp[px] * yp[py - 2];
            if (px > 0 && py > 0) d2PdXDY[idx * n + a] = static_cast<double>(px * py) * xp[px - 1] * yp[py - 1];
            ++idx;
          }
        }
      }
      // Moments, GlobalRKPM.h:161-189.  Mm[m*nm + k], m = M, dMx, dMy, d2Mxx, d2Myy, d2Mxy.
      std::fill(Mm.begin(), Mm.end(), 0.0);
      double* M = &Mm[0]; double* dMx = &Mm[nm]; double* dMy = &Mm[2 * nm];
      double* d2Mxx = &Mm[3 * nm]; double* d2Myy = &Mm[4 * nm]; double* d2Mxy = &Mm[5 * nm];
      for (int a = 0; a < n; ++a) {
        for (int ip = 0; ip < np; ++ip) {
          for (int jp = ip; jp < np; ++jp) {
            const int k = K(ip, jp);
            const double pi = P[ip * n + a], pj = P[jp * n + a];
            const double dpix = dPdX[ip * n + a], dpjx = dPdX[jp * n + a];
            const double dpiy = dPdY[ip * n + a], dpjy = dPdY[jp * n + a];
            M[k] += pi * pj * PSI[a];
            dMx[k] += pi * pj * dPx[a] + (dpix * pj + pi * dpjx) * PSI[a];
            dMy[k] += pi * pj * dPy[a] + (dpiy * pj + pi * dpjy) * PSI[a];
            d2Mxx[k] += d2Pxx[a] * pi * pj + 2.0 * dPx[a] * (dpix * pj + pi * dpjx)
                        + PSI[a] * (d2PdX2[ip * n + a] * pj + 2.0 * dpix * dpjx + pi * d2PdX2[jp * n + a]);
            d2Myy[k] += d2Pyy[a] * pi * pj + 2.0 * dPy[a] * (dpiy * pj + pi * dpjy)
                        + PSI[a] * (d2PdY2[ip * n + a] * pj + 2.0 * dpiy * dpjy + pi * d2PdY2[jp * n + a]);
            d2Mxy[k] += d2Pxy[a] * pi * pj + dPx[a] * (dpiy * pj + pi * dpjy) + dPy[a] * (dpix * pj + pi * dpjx)
                        + PSI[a] * (d2PdXDY[ip * n + a] * pj + dpix * dpjy + dpiy * dpjx + pi * d2PdXDY[jp * n + a]);
          }
        }
      }
      // 3x3 leading block inverse with derivatives, GlobalRKPM.h:203-239.
      std::fill(Mi.begin(), Mi.end(), 0.0);
      double* Minv = &Mi[0]; double* dMinvx = &Mi[nm]; double* dMinvy = &Mi[2 * nm];
      double* d2Minvxx = &Mi[3 * nm]; double* d2Minvyy = &Mi[4 * nm]; double* d2Minvxy = &Mi[5 * nm];
      int bad = 0;
      {
        M3 m3, dmx3, dmy3, d2mxx3, d2myy3, d2mxy3;
        auto fill3 = [&](const double* S, M3 D) {
          for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) D[r][c] = S[K(r, c)];
        };
        fill3(M, m3); fill3(dMx, dmx3); fill3(dMy, dmy3);
        fill3(d2Mxx, d2mxx3); fill3(d2Myy, d2myy3); fill3(d2Mxy, d2mxy3);
        M3 inv;
        inverse3(m3, inv);
        M3 chk;
        mul3(m3, inv, chk);
        bool finite = true;
        double res = 0.0;
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            if (!std::isfinite(inv[r][c])) finite = false;
            res = std::max(res, std::fabs(chk[r][c] - (r == c ? 1.0 : 0.0)));
          }
        if (!finite || res > 1e-8) bad = 1;
        M3 ninv, t1, invx, invy, invxx, invyy, invxy;
        for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) ninv[r][c] = -inv[r][c];
        mul3(ninv, dmx3, t1); mul3(t1, inv, invx);
        mul3(ninv, dmy3, t1); mul3(t1, inv, invy);
        // invxx = inv * (2 dmx inv dmx - d2mxx) * inv
        // inv * (2 dm inv dm - d2m) * inv, with 2.0 * dm * inv * dm evaluated as
        // ((2.0 * dm) * inv) * dm and the outer product as (inv * inner) * inv.
        auto second = [&](const M3 dm, const M3 d2m, M3 out) {
          M3 a2, p, q, inner, r;
          for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) a2[i][j] = 2.0 * dm[i][j];
          mul3(a2, inv, p);
          mul3(p, dm, q);
          for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) inner[i][j] = q[i][j] - d2m[i][j];
          mul3(inv, inner, r);
          mul3(r, inv, out);
        };
        second(dmx3, d2mxx3, invxx);
        second(dmy3, d2myy3, invyy);
        {
          // inv * (dmx inv dmy + dmy inv dmx - d2mxy) * inv
          M3 p, q1, q2, inner, r;
          mul3(dmx3, inv, p); mul3(p, dmy3, q1);
          mul3(dmy3, inv, p); mul3(p, dmx3, q2);
          for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) inner[i][j] = q1[i][j] + q2[i][j] - d2mxy3[i][j];
          mul3(inv, inner, r);
          mul3(r, inv, invxy);
        }
        for (int r = 0; r < 3; ++r)
          for (int c = r; c < 3; ++c) {
            const int k = K(r, c);
            Minv[k] = inv[r][c]; dMinvx[k] = invx[r][c]; dMinvy[k] = invy[r][c];
            d2Minvxx[k] = invxx[r][c]; d2Minvyy[k] = invyy[r][c]; d2Minvxy[k] = invxy[r][c];
          }
      }
      // Bordered (Schur) inversion for np > 3, GlobalRKPM.h:259-345.
      for (int it = 3; it < np; ++it) {
        double b[16], dbx[16], dby[16], d2bxx[16], d2byy[16], d2bxy[16];
        double v[16], vx[16], vy[16], vxx[16], vyy[16], vxy[16];
        for (int j = 0; j < it; ++j) {
          const int k = K(j, it);
          b[j] = M[k]; dbx[j] = dMx[k]; dby[j] = dMy[k];
          d2bxx[j] = d2Mxx[k]; d2byy[j] = d2Myy[k]; d2bxy[j] = d2Mxy[k];
        }
        for (int r = 0; r < it; ++r) {
          double sv = 0, sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
          // v = aI b; vx = daIx b + aI dbx; ... each product a row-dot, then the sums.
          double aIb = 0, daxb = 0, aIdbx = 0, dayb = 0, aIdby = 0;
          double d2xxb = 0, daxdbx = 0, aId2bxx = 0, d2yyb = 0, daydby = 0, aId2byy = 0;
          double d2xyb = 0, daxdby = 0, daydbx = 0, aId2bxy = 0;
          for (int c = 0; c < it; ++c) {
            const int k = K(r, c);
            aIb += Minv[k] * b[c];
            daxb += dMinvx[k] * b[c]; aIdbx += Minv[k] * dbx[c];
            dayb += dMinvy[k] * b[c]; aIdby += Minv[k] * dby[c];
            d2xxb += d2Minvxx[k] * b[c]; daxdbx += dMinvx[k] * dbx[c]; aId2bxx += Minv[k] * d2bxx[c];
            d2yyb += d2Minvyy[k] * b[c]; daydby += dMinvy[k] * dby[c]; aId2byy += Minv[k] * d2byy[c];
            d2xyb += d2Minvxy[k] * b[c]; daxdby += dMinvx[k] * dby[c]; daydbx += dMinvy[k] * dbx[c];
            aId2bxy += Minv[k] * d2bxy[c];
          }
          sv = aIb;
          sx = daxb + aIdbx;
          sy = dayb + aIdby;
          sxx = d2xxb + 2.0 * daxdbx + aId2bxx;
          syy = d2yyb + 2.0 * daydby + aId2byy;
          sxy = d2xyb + daxdby + daydbx + aId2bxy;
          v[r] = sv; vx[r] = sx; vy[r] = sy; vxx[r] = sxx; vyy[r] = syy; vxy[r] = sxy;
        }
        auto dot = [&](const double* a, const double* c) {
          double t = 0; for (int j = 0; j < it; ++j) t += a[j] * c[j]; return t;
        };
        const int kii = K(it, it);
        const double q = M[kii] - dot(b, v);
        const double qx = dMx[kii] - (dot(dbx, v) + dot(b, vx));
        const double qy = dMy[kii] - (dot(dby, v) + dot(b, vy));
        const double qxx = d2Mxx[kii] - (dot(d2bxx, v) + 2.0 * dot(dbx, vx) + dot(b, vxx));
        const double qyy = d2Myy[kii] - (dot(d2byy, v) + 2.0 * dot(dby, vy) + dot(b, vyy));
        const double qxy = d2Mxy[kii] - (dot(d2bxy, v) + dot(dbx, vy) + dot(dby, vx) + dot(b, vxy));
        // A point flagged singular keeps that flag (the reference throws on the singular
        // set before the bordering, GlobalRKPM.h:241-257).
        if (!(std::fabs(q) > 1e-12 * std::max(std::fabs(M[kii]), 1.0)) && bad == 0) bad = 2;
        const double iQ = 1.0 / q, iQ2 = iQ * iQ, iQ3 = iQ2 * iQ;
        for (int r = 0; r < it; ++r) {
          for (int c = r; c < it; ++c) {
            const int k = K(r, c);
            Minv[k] += v[r] * v[c] * iQ;
            dMinvx[k] += (vx[r] * v[c] + v[r] * vx[c]) * iQ - v[r] * v[c] * qx * iQ2;
            dMinvy[k] += (vy[r] * v[c] + v[r] * vy[c]) * iQ - v[r] * v[c] * qy * iQ2;
            d2Minvxx[k] += (vxx[r] * v[c] + 2.0 * vx[r] * vx[c] + v[r] * vxx[c]) * iQ
                           - (vx[r] * v[c] + v[r] * vx[c]) * qx * iQ2 * 2.0
                           + v[r] * v[c] * (2.0 * qx * qx * iQ3 - qxx * iQ2);
            d2Minvyy[k] += (vyy[r] * v[c] + 2.0 * vy[r] * vy[c] + v[r] * vyy[c]) * iQ
                           - (vy[r] * v[c] + v[r] * vy[c]) * qy * iQ2 * 2.0
                           + v[r] * v[c] * (2.0 * qy * qy * iQ3 - qyy * iQ2);
            d2Minvxy[k] += (vxy[r] * v[c] + vx[r] * vy[c] + vy[r] * vx[c] + v[r] * vxy[c]) * iQ
                           - (vx[r] * v[c] + v[r] * vx[c]) * qy * iQ2
                           - (vy[r] * v[c] + v[r] * vy[c]) * qx * iQ2
                           + v[r] * v[c] * (2.0 * qx * qy * iQ3 - qxy * iQ2);
          }
        }
        for (int j = 0; j < it; ++j) {
          const int k = K(j, it);
          Minv[k] = -v[j] * iQ;
          dMinvx[k] = -vx[j] * iQ + v[j] * qx * iQ2;
          dMinvy[k] = -vy[j] * iQ + v[j] * qy * iQ2;
          d2Minvxx[k] = -vxx[j] * iQ + 2.0 * vx[j] * qx * iQ2 + v[j] * (qxx * iQ2 - 2.0 * qx * qx * iQ3);
          d2Minvyy[k] = -vyy[j] * iQ + 2.0 * vy[j] * qy * iQ2 + v[j] * (qyy * iQ2 - 2.0 * qy * qy * iQ3);
          d2Minvxy[k] = -vxy[j] * iQ + vx[j] * qy * iQ2 + vy[j] * qx * iQ2 + v[j] * (qxy * iQ2 - 2.0 * qx * qy * iQ3);
        }
        Minv[kii] = iQ;
        dMinvx[kii] = -qx * iQ2;
        dMinvy[kii] = -qy * iQ2;
        d2Minvxx[kii] = 2.0 * qx * qx * iQ3 - qxx * iQ2;
        d2Minvyy[kii] = 2.0 * qy * qy * iQ3 - qyy * iQ2;
        d2Minvxy[kii] = 2.0 * qx * qy * iQ3 - qxy * iQ2;
      }
      if (gp_bad) gp_bad[g] = static_cast<int8_t>(bad);
      local_worst = std::max(local_worst, bad);
      // Shape functions, GlobalRKPM.h:363-396.
      const double rho2 = rho * rho;
      for (int a = 0; a < n; ++a) {
        double C = 0.0, dCx = 0.0, dCy = 0.0, d2Cxx = 0.0, d2Cyy = 0.0, d2Cxy = 0.0;
        for (int jp = 0; jp < np; ++jp) {
          const int k = K(0, jp);
          const double v = Minv[k], vx = dMinvx[k], vy = dMinvy[k];
          const double vxx = d2Minvxx[k], vyy = d2Minvyy[k], vxy = d2Minvxy[k];
          const double p = P[jp * n + a], px = dPdX[jp * n + a], py = dPdY[jp * n + a];
          C += v * p;
          dCx += vx * p + v * px;
          dCy += vy * p + v * py;
          d2Cxx += vxx * p + 2.0 * vx * px + v * d2PdX2[jp * n + a];
          d2Cyy += vyy * p + 2.0 * vy * py + v * d2PdY2[jp * n + a];
          d2Cxy += vxy * p + vx * py + vy * px + v * d2PdXDY[jp * n + a];
        }
        const int64_t e = p0 + a;
        psi_out[e] = C * PSI[a];
        dpsi_out[2 * e] = (dCx * PSI[a] + C * dPx[a]) / rho;
        dpsi_out[2 * e + 1] = (dCy * PSI[a] + C * dPy[a]) / rho;
        ddpsi_out[3 * e] = (d2Cxx * PSI[a] + 2.0 * dCx * dPx[a] + C * d2Pxx[a]) / rho2;
        ddpsi_out[3 * e + 1] = (d2Cyy * PSI[a] + 2.0 * dCy * dPy[a] + C * d2Pyy[a]) / rho2;
        ddpsi_out[3 * e + 2] = (d2Cxy * PSI[a] + dCx * dPy[a] + dCy * dPx[a] + C * d2Pxy[a]) / rho2;
      }
    }
    #pragma omp critical
    worst = std::max(worst, local_worst);
  }
  return worst;
}

void orc_abd_isotropic(double E, double nu, double h, double* A, double* B, double* D) {
  // main.cpp:53-61 (one ply, E1 = E2 = E, G12 = E / (2 (1 + nu)), angle 0) and
  // Constitutive::computeABD (plate/Constitutive.h:10-50).
  const double E1 = E, E2 = E, nu12 = nu, G12 = E / (2.0 * (1.0 + nu));
  const double nu21 = (E2 / E1) * nu12;
  const double den = 1.0 - nu12 * nu21;
  double Q[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  Q[0][0] = E1 / den; Q[1][1] = E2 / den; Q[0][1] = Q[1][0] = (nu12 * E2) / den; Q[2][2] = G12;
  const double theta = 0.0 * M_PI / 180.0;
  const double m = std::cos(theta), n = std::sin(theta);
  const double m2 = m * m, n2 = n * n, m4 = m2 * m2, n4 = n2 * n2;
  double Qb[3][3];
  Qb[0][0] = Q[0][0] * m4 + 2.0 * (Q[0][1] + 2.0 * Q[2][2]) * m2 * n2 + Q[1][1] * n4;
  Qb[1][1] = Q[0][0] * n4 + 2.0 * (Q[0][1] + 2.0 * Q[2][2]) * m2 * n2 + Q[1][1] * m4;
  Qb[0][1] = Qb[1][0] = (Q[0][0] + Q[1][1] - 4.0 * Q[2][2]) * m2 * n2 + Q[0][1] * (m4 + n4);
  Qb[0][2] = Qb[2][0] = (Q[0][0] - Q[0][1] - 2.0 * Q[2][2]) * n * m * m2 + (Q[0][1] - Q[1][1] + 2.0 * Q[2][2]) * n2 * n * m;
  Qb[1][2] = Qb[2][1] = (Q[0][0] - Q[0][1] - 2.0 * Q[2][2]) * m * n * n2 + (Q[0][1] - Q[1][1] + 2.0 * Q[2][2]) * m2 * m * n;
  Qb[2][2] = (Q[0][0] + Q[1][1] - 2.0 * Q[0][1] - 2.0 * Q[2][2]) * m2 * n2 + Q[2][2] * (m4 + n4);
  const double z0 = -h / 2.0, z1 = z0 + h;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      A[3 * r + c] = 0.0 + Qb[r][c] * (z1 - z0);
      B[3 * r + c] = 0.0 + 0.5 * Qb[r][c] * (z1 * z1 - z0 * z0);
      D[3 * r + c] = 0.0 + (1.0 / 3.0) * Qb[r][c] * (z1 * z1 * z1 - z0 * z0 * z0);
    }
}

namespace {

// plate/Assembly.h:62-82: col_nodes[nj] = sorted unique {ni <= nj} over every pair of
// neighbours of every Gauss point; plus the hinge triplets (Constraints.h:376-433): every
// ordered pair of the concatenated left+right neighbour lists with node_k <= node_m, since
// K += K_fold widens the pattern. The reference collects the pairs in one thread; here
// each thread collects its share of the Gauss points and the per-column lists are then
// merged, sorted and made unique column by column. A sorted unique set does not depend on
// the order its members were collected in, so the columns are the reference's.
std::vector<std::vector<int>> pattern_columns(int n_nodes, int n_gp, const int64_t* nbr_ptr,
                                              const int32_t* nbr_idx, int n_fold_gp, const int64_t* fl_ptr,
                                              const int32_t* fl_idx, const int64_t* fr_ptr,
                                              const int32_t* fr_idx) {
  int T = 1;
#ifdef _OPENMP
  T = omp_get_max_threads();
#endif
  std::vector<std::vector<std::vector<int>>> loc(T, std::vector<std::vector<int>>(n_nodes));
#pragma omp parallel num_threads(T)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    auto& L = loc[t];
#pragma omp for schedule(static)
    for (int g = 0; g < n_gp; ++g)
      for (int64_t a = nbr_ptr[g]; a < nbr_ptr[g + 1]; ++a)
        for (int64_t b = nbr_ptr[g]; b < nbr_ptr[g + 1]; ++b)
          if (nbr_idx[a] <= nbr_idx[b]) L[nbr_idx[b]].push_back(nbr_idx[a]);
  }
  std::vector<int> ids;
  for (int g = 0; g < n_fold_gp; ++g) {
    ids.clear();
    for (int64_t a = fl_ptr[g]; a < fl_ptr[g + 1]; ++a) ids.push_back(fl_idx[a]);
    for (int64_t a = fr_ptr[g]; a < fr_ptr[g + 1]; ++a) ids.push_back(fr_idx[a]);
    for (int a : ids)
      for (int b : ids)
        if (a <= b) loc[0][b].push_back(a);
  }
  std::vector<std::vector<int>> cols(n_nodes);
#pragma omp parallel for schedule(dynamic, 64) num_threads(T)
  for (int j = 0; j < n_nodes; ++j) {
    auto& c = cols[j];
    for (int t = 0; t < T; ++t) {
      c.insert(c.end(), loc[t][j].begin(), loc[t][j].end());
      std::vector<int>().swap(loc[t][j]);
    }
    std::sort(c.begin(), c.end());
    c.erase(std::unique(c.begin(), c.end()), c.end());
  }
  return cols;
}

int64_t pattern_fill(const std::vector<std::vector<int>>& cols, int n_nodes, int n_gp, const int64_t* nbr_ptr,
                     const int32_t* nbr_idx, int32_t* outer, int32_t* inner, int64_t* col_ptr,
                     int32_t* col_nodes, int32_t* map);

}  // namespace

struct orc_pattern_state {
  std::vector<std::vector<int>> cols;
};

orc_pattern_state* orc_pattern_new(int n_nodes, int n_gp, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                                   int n_fold_gp, const int64_t* fl_ptr, const int32_t* fl_idx,
                                   const int64_t* fr_ptr, const int32_t* fr_idx, int64_t* nnz) {
  auto* h = new orc_pattern_state;
  h->cols = pattern_columns(n_nodes, n_gp, nbr_ptr, nbr_idx, n_fold_gp, fl_ptr, fl_idx, fr_ptr, fr_idx);
  int64_t blocks = 0;
  for (const auto& c : h->cols) blocks += static_cast<int64_t>(c.size());
  *nnz = 9 * blocks;
  return h;
}

int64_t orc_pattern_fill(const orc_pattern_state* h, int n_nodes, int n_gp, const int64_t* nbr_ptr,
                         const int32_t* nbr_idx, int32_t* outer, int32_t* inner, int64_t* col_ptr,
                         int32_t* col_nodes, int32_t* map) {
  return pattern_fill(h->cols, n_nodes, n_gp, nbr_ptr, nbr_idx, outer, inner, col_ptr, col_nodes, map);
}

void orc_pattern_free(orc_pattern_state* h) { delete h; }

int64_t orc_pattern(int n_nodes, int n_gp, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                    int n_fold_gp, const int64_t* fl_ptr, const int32_t* fl_idx,
                    const int64_t* fr_ptr, const int32_t* fr_idx,
                    int32_t* outer, int32_t* inner, int64_t* col_ptr, int32_t* col_nodes,
                    int32_t* map) {
  const auto cols = pattern_columns(n_nodes, n_gp, nbr_ptr, nbr_idx, n_fold_gp, fl_ptr, fl_idx, fr_ptr, fr_idx);
  return pattern_fill(cols, n_nodes, n_gp, nbr_ptr, nbr_idx, outer, inner, col_ptr, col_nodes, map);
}

namespace {

int64_t pattern_fill(const std::vector<std::vector<int>>& cols, int n_nodes, int n_gp, const int64_t* nbr_ptr,
                     const int32_t* nbr_idx, int32_t* outer, int32_t* inner, int64_t* col_ptr,
                     int32_t* col_nodes, int32_t* map) {
  int64_t nnz = 0;
  int64_t off = 0;
  for (int j = 0; j < n_nodes; ++j) {
    for (int c = 0; c < 3; ++c) {
      outer[3 * j + c] = static_cast<int32_t>(off);
      off += 3 * static_cast<int64_t>(cols[j].size());
    }
  }
  outer[3 * n_nodes] = static_cast<int32_t>(off);
  nnz = off;
  if (!inner) return nnz;
  int64_t e = 0;
  for (int j = 0; j < n_nodes; ++j)
    for (int c = 0; c < 3; ++c)
      for (int i : cols[j])
        for (int r = 0; r < 3; ++r) inner[e++] = 3 * i + r;
  if (col_ptr) {
    int64_t cp = 0;
    for (int j = 0; j < n_nodes; ++j) {
      col_ptr[j] = cp;
      if (col_nodes) for (int i : cols[j]) col_nodes[cp++] = i; else cp += cols[j].size();
    }
    col_ptr[n_nodes] = cp;
  }
  bool ok = true;
  if (map) {
    // plate/Assembly.h:112-144 (an OpenMP loop over the Gauss points there too): per
    // local pair (i <= j) the position of min(ni, nj) in col_nodes[max(ni, nj)].
    std::vector<int64_t> mptr(static_cast<size_t>(n_gp) + 1, 0);
    for (int g = 0; g < n_gp; ++g) {
      const int64_t n = nbr_ptr[g + 1] - nbr_ptr[g];
      mptr[g + 1] = mptr[g] + n * (n + 1) / 2;
    }
    int miss = 0;
#pragma omp parallel for schedule(guided, 64) reduction(| : miss)
    for (int g = 0; g < n_gp; ++g) {
      const int64_t p0 = nbr_ptr[g];
      const int n = static_cast<int>(nbr_ptr[g + 1] - p0);
      int64_t mo = mptr[g];
      for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
          const int ni = nbr_idx[p0 + i], nj = nbr_idx[p0 + j];
          const int lo = std::min(ni, nj), hi = std::max(ni, nj);
          const auto& ch = cols[hi];
          auto it = std::lower_bound(ch.begin(), ch.end(), lo);
          if (it == ch.end() || *it != lo) { map[mo++] = -1; miss = 1; }
          else map[mo++] = static_cast<int32_t>(it - ch.begin());
        }
    }
    ok = miss == 0;
  }
  return ok ? nnz : -1;
}

}  // namespace

void orc_set_static_schedule(int on) { g_static_schedule = on != 0; }

void orc_set_natural_curvature(int active, double x0, double width, double theta0, double sign) {
  g_natural.active = active != 0;
  g_natural.x0 = x0;
  g_natural.width = width;
  g_natural.theta0 = theta0;
  g_natural.sign = sign;
}

int orc_update_stiffness(int n_nodes, int n_gp, const double* gp_weight, const int64_t* nbr_ptr,
                         const int32_t* nbr_idx, const double* dpsi, const double* ddpsi,
                         const int32_t* outer, const int32_t* map, const double* x,
                         const double* A, const double* B, const double* D, int want_K, int n_threads,
                         double* K_values, double* F, const double* gp_xy) {
  // plate/Assembly.h:158-345.
  int max_threads = 1;
#ifdef _OPENMP
  max_threads = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  (void)n_threads;
#endif
  const int64_t nnz = outer[3 * n_nodes];
  const int64_t ndof = 3 * static_cast<int64_t>(n_nodes);
  std::vector<std::vector<double>> lf(max_threads), lk(max_threads);
  // Map offsets per Gauss point (the reference keeps one vector per point).
  std::vector<int64_t> map_ptr(n_gp + 1);
  map_ptr[0] = 0;
  for (int g = 0; g < n_gp; ++g) {
    const int64_t n = nbr_ptr[g + 1] - nbr_ptr[g];
    map_ptr[g + 1] = map_ptr[g] + n * (n + 1) / 2;
  }
  #pragma omp parallel for schedule(static) num_threads(max_threads)
  for (int t = 0; t < max_threads; ++t) {
    lf[t].assign(ndof, 0.0);
    if (want_K) lk[t].assign(nnz, 0.0);
  }
#ifdef _OPENMP
  omp_set_schedule(g_static_schedule ? omp_sched_static : omp_sched_guided, g_static_schedule ? 0 : 8);
#endif
  #pragma omp parallel num_threads(max_threads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    std::vector<double> Bm, Bb, P, Q, Db, N2, C0d, Tu;
    // schedule(guided, 8) as the reference (Assembly.h:199); with g_static_schedule a static
    // split, which fixes every thread's share and so the rounding for a given thread count.
    #pragma omp for schedule(runtime)
    for (int g = 0; g < n_gp; ++g) {
      const int64_t p0 = nbr_ptr[g], p1 = nbr_ptr[g + 1];
      const int n = static_cast<int>(p1 - p0);
      if (n == 0) continue;
      Kin k;
      kinematics(p0, p1, nbr_idx, dpsi, ddpsi, x, k, gp_xy ? gp_xy + 2 * static_cast<int64_t>(g) : nullptr);
      double Nr[3], Mr[3];
      resultants(k, A, B, D, Nr, Mr);
      const double W = gp_weight[g];
      // V = F0 * C0inv (3x2)
      double V[3][2];
      for (int r = 0; r < 3; ++r) {
        const double f0 = k.r0X[r], f1 = k.r0Y[r];
        V[r][0] = f0 * k.C0inv[0][0] + f1 * k.C0inv[1][0];
        V[r][1] = f0 * k.C0inv[0][1] + f1 * k.C0inv[1][1];
      }
      const double N2x2[2][2] = {{Nr[0], Nr[2]}, {Nr[2], Nr[1]}};
      double vc[3];
      for (int r = 0; r < 3; ++r) vc[r] = k.r0XX[r] * Mr[0] + 2.0 * k.r0XY[r] * Mr[2] + k.r0YY[r] * Mr[1];
      // p_XY = (C0inv * F0^T) * v_curv
      double CF[2][3];
      for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 3; ++c) CF[a][c] = k.C0inv[a][0] * k.r0X[c] + k.C0inv[a][1] * k.r0Y[c];
      double pXY[2];
      for (int a = 0; a < 2; ++a) pXY[a] = CF[a][0] * vc[0] + CF[a][1] * vc[1] + CF[a][2] * vc[2];
      double bbT[3][3];
      for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) bbT[r][c] = k.b[r] * k.b[c];
      const double bdv = dot3(k.b, vc);
      Bm.resize(9 * n); Bb.resize(9 * n); P.resize(9 * n); Q.resize(9 * n); Db.resize(9 * n);
      N2.resize(2 * n); C0d.resize(2 * n); Tu.resize(n);
      double* Fl = lf[tid].data();
      for (int i = 0; i < n; ++i) {
        const int64_t e = p0 + i;
        const int node = nbr_idx[e];
        const double dx = dpsi[2 * e], dy = dpsi[2 * e + 1];
        const double dxx = ddpsi[3 * e], dyy = ddpsi[3 * e + 1], dxy = ddpsi[3 * e + 2];
        double* bm = &Bm[9 * i]; double* bb = &Bb[9 * i];
        for (int c = 0; c < 3; ++c) {
          bm[0 * 3 + c] = k.r0X[c] * dx;
          bm[1 * 3 + c] = k.r0Y[c] * dy;
          bm[2 * 3 + c] = k.r0X[c] * dy + k.r0Y[c] * dx;
        }
        double gI[3];
        for (int r = 0; r < 3; ++r) gI[r] = V[r][0] * dx + V[r][1] * dy;
        const double SXX = dot3(k.r0XX, gI), SYY = dot3(k.r0YY, gI), SXY = dot3(k.r0XY, gI);
        const double c0 = -dxx + SXX, c1 = -dyy + SYY, c2 = 2.0 * (-dxy + SXY);
        for (int c = 0; c < 3; ++c) { bb[c] = c0 * k.b[c]; bb[3 + c] = c1 * k.b[c]; bb[6 + c] = c2 * k.b[c]; }
        for (int c = 0; c < 3; ++c) {
          const double fm = bm[c] * Nr[0] + bm[3 + c] * Nr[1] + bm[6 + c] * Nr[2];
          const double fb = bb[c] * Mr[0] + bb[3 + c] * Mr[1] + bb[6 + c] * Mr[2];
          Fl[3 * static_cast<int64_t>(node) + c] += (fm + fb) * W;
        }
        double* p = &P[9 * i]; double* q = &Q[9 * i];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            const double am = A[3 * r] * bm[c] + A[3 * r + 1] * bm[3 + c] + A[3 * r + 2] * bm[6 + c];
            const double bbv = B[3 * r] * bb[c] + B[3 * r + 1] * bb[3 + c] + B[3 * r + 2] * bb[6 + c];
            p[3 * r + c] = am + bbv;
            const double bmv = B[3 * r] * bm[c] + B[3 * r + 1] * bm[3 + c] + B[3 * r + 2] * bm[6 + c];
            const double db = D[3 * r] * bb[c] + D[3 * r + 1] * bb[3 + c] + D[3 * r + 2] * bb[6 + c];
            q[3 * r + c] = bmv + db;
          }
        double* dbm = &Db[9 * i];
        for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) dbm[3 * r + c] = (-gI[r]) * k.b[c];
        N2[2 * i] = N2x2[0][0] * dx + N2x2[0][1] * dy;
        N2[2 * i + 1] = N2x2[1][0] * dx + N2x2[1][1] * dy;
        C0d[2 * i] = k.C0inv[0][0] * dx + k.C0inv[0][1] * dy;
        C0d[2 * i + 1] = k.C0inv[1][0] * dx + k.C0inv[1][1] * dy;
        const double HM = dxx * Mr[0] + 2.0 * dxy * Mr[2] + dyy * Mr[1];
        const double Gp = dx * pXY[0] + dy * pXY[1];
        Tu[i] = Gp - HM;
      }
      if (!want_K) continue;
      double* Kl = lk[tid].data();
      int64_t mo = map_ptr[g];
      for (int i = 0; i < n; ++i) {
        const double* bmi = &Bm[9 * i]; const double* bbi = &Bb[9 * i]; const double* dbi = &Db[9 * i];
        const double dxi = dpsi[2 * (p0 + i)], dyi = dpsi[2 * (p0 + i) + 1];
        const double Tui = Tu[i];
        for (int j = i; j < n; ++j) {
          const double* pj = &P[9 * j]; const double* qj = &Q[9 * j]; const double* dbj = &Db[9 * j];
          const double geo = dxi * N2[2 * j] + dyi * N2[2 * j + 1];
          const double T3s = bdv * (dxi * C0d[2 * j] + dyi * C0d[2 * j + 1]);
          double KIJ[3][3];
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
              const double km = bmi[r] * pj[c] + bmi[3 + r] * pj[3 + c] + bmi[6 + r] * pj[6 + c];
              const double kb = bbi[r] * qj[c] + bbi[3 + r] * qj[3 + c] + bbi[6 + r] * qj[6 + c];
              const double kmat = km + kb;
              const double kgeo = (r == c) ? geo : 0.0;
              const double t12 = Tui * dbj[3 * r + c] + Tu[j] * dbi[3 * c + r];
              const double t3 = T3s * bbT[r][c];
              KIJ[r][c] = (((kmat + kgeo) + t12) + t3) * W;
            }
          const int ni = nbr_idx[p0 + i], nj = nbr_idx[p0 + j];
          const int64_t pos3 = 3 * static_cast<int64_t>(map[mo++]);
          const bool flip = ni > nj;
          const int64_t hi3 = 3 * static_cast<int64_t>(flip ? ni : nj);
          for (int c = 0; c < 3; ++c) {
            double* dst = Kl + outer[hi3 + c] + pos3;
            if (!flip) { dst[0] += KIJ[0][c]; dst[1] += KIJ[1][c]; dst[2] += KIJ[2][c]; }
            else { dst[0] += KIJ[c][0]; dst[1] += KIJ[c][1]; dst[2] += KIJ[c][2]; }
          }
        }
      }
    }
  }
  // Merge, plate/Assembly.h:327-344.
  for (int64_t d = 0; d < ndof; ++d) {
    double s = 0.0;
    for (int t = 0; t < max_threads; ++t) s += lf[t][d];
    F[d] = s;
  }
  if (want_K) {
    #pragma omp parallel for schedule(static) num_threads(max_threads)
    for (int64_t idx = 0; idx < nnz; ++idx) {
      double s = 0.0;
      for (int t = 0; t < max_threads; ++t) s += lk[t][idx];
      K_values[idx] = s;
    }
  }
  return 0;
}

double orc_fold_angle(const double* F, double tx, double ty, double* grad) {
  // plate/Constraints.h:54-119.
  const double *a1L = F, *a2L = F + 3, *a1R = F + 6, *a2R = F + 9;
  double nL[3], nR[3];
  cross3(a1L, a2L, nL); cross3(a1R, a2R, nR);
  const double normL = std::sqrt(dot3(nL, nL)), normR = std::sqrt(dot3(nR, nR));
  double bL[3], bR[3];
  for (int c = 0; c < 3; ++c) { bL[c] = nL[c] / normL; bR[c] = nR[c] / normR; }
  double aT[3];
  for (int c = 0; c < 3; ++c) aT[c] = a1L[c] * tx + a2L[c] * ty;
  const double naT = std::sqrt(dot3(aT, aT));
  double t[3];
  for (int c = 0; c < 3; ++c) t[c] = aT[c] / naT;
  const double cth = dot3(bL, bR);
  double bxb[3];
  cross3(bL, bR, bxb);
  const double sth = dot3(bxb, t);
  const double theta = std::atan2(-sth, cth);
  if (grad) {
    // db/dF = (I - b b^T)/|n| * dn/dF, dn/dF cols: e_i x a2 (i<3), a1 x e_i.
    auto dbdF = [](const double* a1, const double* a2, const double* b, double nn, double out[3][6]) {
      double dn[3][6];
      for (int i = 0; i < 3; ++i) {
        double e[3] = {0, 0, 0}; e[i] = 1.0;
        double c1[3], c2[3];
        cross3(e, a2, c1); cross3(a1, e, c2);
        for (int r = 0; r < 3; ++r) { dn[r][i] = c1[r]; dn[r][i + 3] = c2[r]; }
      }
      double Pm[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Pm[r][c] = ((r == c ? 1.0 : 0.0) - b[r] * b[c]) / nn;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 6; ++c) out[r][c] = Pm[r][0] * dn[0][c] + Pm[r][1] * dn[1][c] + Pm[r][2] * dn[2][c];
    };
    double dbL[3][6], dbR[3][6];
    dbdF(a1L, a2L, bL, normL, dbL);
    dbdF(a1R, a2R, bR, normR, dbR);
    double daT[3][6] = {{tx, 0, 0, ty, 0, 0}, {0, tx, 0, 0, ty, 0}, {0, 0, tx, 0, 0, ty}};
    double Pt[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) Pt[r][c] = ((r == c ? 1.0 : 0.0) - t[r] * t[c]) / naT;
    double dt[3][6];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 6; ++c) dt[r][c] = Pt[r][0] * daT[0][c] + Pt[r][1] * daT[1][c] + Pt[r][2] * daT[2][c];
    double bRxt[3], txbL[3];
    cross3(bR, t, bRxt); cross3(t, bL, txbL);
    double dcL[6], dcR[6], dsL[6], dsR[6];
    for (int c = 0; c < 6; ++c) {
      dcL[c] = bR[0] * dbL[0][c] + bR[1] * dbL[1][c] + bR[2] * dbL[2][c];
      dcR[c] = bL[0] * dbR[0][c] + bL[1] * dbR[1][c] + bL[2] * dbR[2][c];
      const double s1 = bRxt[0] * dbL[0][c] + bRxt[1] * dbL[1][c] + bRxt[2] * dbL[2][c];
      const double s2 = bxb[0] * dt[0][c] + bxb[1] * dt[1][c] + bxb[2] * dt[2][c];
      dsL[c] = s1 + s2;
      dsR[c] = txbL[0] * dbR[0][c] + txbL[1] * dbR[1][c] + txbL[2] * dbR[2][c];
    }
    const double denom = cth * cth + sth * sth;
    const double inv = (denom > 1e-14) ? 1.0 / denom : 0.0;
    for (int c = 0; c < 6; ++c) {
      grad[c] = -(cth * dsL[c] - sth * dcL[c]) * inv;
      grad[6 + c] = -(cth * dsR[c] - sth * dcR[c]) * inv;
    }
  }
  return theta;
}

int orc_hinge(int n_nodes, const double* x, int n_folds, const orc_fold* folds, int exact_tangent,
              const int32_t* outer, const int64_t* col_ptr, const int32_t* col_nodes, double* K_values,
              double* F) {
  // plate/Constraints.h:341-436, folds in order, crease points in order; triplets are
  // summed into K in the order they are generated (setFromTriplets sums duplicates,
  // then K += K_fold, Meshless.h:119-125).
  // The pattern is read only when K is wanted (F-only calls pass no pattern).
  const int64_t nnz = (K_values && outer) ? outer[3 * n_nodes] : 0;
  std::vector<double> Kf(nnz, 0.0);
  for (int f = 0; f < n_folds; ++f) {
    const orc_fold& fd = folds[f];
    for (int i = 0; i < fd.n_gp; ++i) {
      if (fd.active && fd.active[i] == 0) continue;
      // Only F0 = (r0,X, r0,Y) of each side is needed (Kinematics.h:64-81); the curvature
      // terms Kinematics::compute also forms do not enter the hinge.
      double F12[12];
      auto grad_sum = [&](const int64_t* ptr, const int32_t* idx, const double* dps, double* a1, double* a2) {
        a1[0] = 1.0; a1[1] = 0.0; a1[2] = 0.0;
        a2[0] = 0.0; a2[1] = 1.0; a2[2] = 0.0;
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
          const double* u = x + 3 * static_cast<int64_t>(idx[e]);
          for (int c = 0; c < 3; ++c) { a1[c] += u[c] * dps[2 * e]; a2[c] += u[c] * dps[2 * e + 1]; }
        }
      };
      grad_sum(fd.l_ptr, fd.l_idx, fd.l_dpsi, F12, F12 + 3);
      grad_sum(fd.r_ptr, fd.r_idx, fd.r_dpsi, F12 + 6, F12 + 9);
      const double tx = fd.tangent[2 * i], ty = fd.tangent[2 * i + 1];
      double gradF[12];
      const double theta = orc_fold_angle(F12, tx, ty, gradF);
      const double th0 = fd.theta0_gp ? fd.theta0_gp[i] : fd.theta0;
      const double moment = fd.Kt * (theta - th0);
      const double W = fd.weight[i];
      const double Wm = W * moment, WK = W * fd.Kt;
      std::vector<int> ids;
      std::vector<double> gr;
      std::vector<std::array<double, 2>> Bv;  // (dX, dY) of each dof
      std::vector<int> blk;                   // block offset (0 left, 6 right) + d
      auto extract = [&](int block, const int64_t* ptr, const int32_t* idx, const double* dps) {
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
          const double dX = dps[2 * e], dY = dps[2 * e + 1];
          for (int d = 0; d < 3; ++d) {
            ids.push_back(3 * idx[e] + d);
            gr.push_back(gradF[block + d] * dX + gradF[block + d + 3] * dY);
            Bv.push_back({dX, dY});
            blk.push_back(block + d);
          }
        }
      };
      extract(0, fd.l_ptr, fd.l_idx, fd.l_dpsi);
      extract(6, fd.r_ptr, fd.r_idx, fd.r_dpsi);
      double H[12][12];
      const bool use_hess = exact_tangent && K_values && std::fabs(Wm) > 0.0;
      if (use_hess) {
        double mx = 0.0;
        for (int k = 0; k < 12; ++k) mx = std::max(mx, std::fabs(F12[k]));
        const double hs = 1e-6 * std::max(1.0, mx);
        for (int k = 0; k < 12; ++k) {
          double Fp[12], Fm[12], gp[12], gm[12];
          std::memcpy(Fp, F12, sizeof Fp); std::memcpy(Fm, F12, sizeof Fm);
          Fp[k] += hs; Fm[k] -= hs;
          orc_fold_angle(Fp, tx, ty, gp);
          orc_fold_angle(Fm, tx, ty, gm);
          for (int r = 0; r < 12; ++r) H[r][k] = (gp[r] - gm[r]) / (2.0 * hs);
        }
        double Hs[12][12];
        for (int r = 0; r < 12; ++r) for (int c = 0; c < 12; ++c) Hs[r][c] = 0.5 * (H[r][c] + H[c][r]);
        std::memcpy(H, Hs, sizeof H);
      }
      const size_t nd = ids.size();
      for (size_t k = 0; k < nd; ++k) {
        F[ids[k]] += gr[k] * Wm;
        if (!K_values) continue;
        for (size_t m = 0; m < nd; ++m) {
          double val = gr[k] * gr[m] * WK;
          if (use_hess) {
            // B[k] . (H B[m]): B[k] has dX at blk[k] and dY at blk[k]+3.
            const int bk = blk[k], bm = blk[m];
            const double hbm_k = H[bk][bm] * Bv[m][0] + H[bk][bm + 3] * Bv[m][1];
            const double hbm_k3 = H[bk + 3][bm] * Bv[m][0] + H[bk + 3][bm + 3] * Bv[m][1];
            val += Wm * (Bv[k][0] * hbm_k + Bv[k][1] * hbm_k3);
          }
          const int nk = ids[k] / 3, nm = ids[m] / 3;
          if (nk <= nm) {
            const int32_t* c0 = col_nodes + col_ptr[nm];
            const int32_t* c1 = col_nodes + col_ptr[nm + 1];
            const int32_t* it = std::lower_bound(c0, c1, nk);
            if (it == c1 || *it != nk) return -1;
            const int64_t pos = it - c0;
            Kf[outer[ids[m]] + 3 * pos + (ids[k] % 3)] += val;
          }
        }
      }
    }
  }
  if (K_values)
    for (int64_t e = 0; e < nnz; ++e) K_values[e] = K_values[e] + Kf[e];
  return 0;
}

double orc_hinge_energy(const double* x, int n_folds, const orc_fold* folds) {
  // plate/Constraints.h:310-339.
  double E = 0.0;
  for (int f = 0; f < n_folds; ++f) {
    const orc_fold& fd = folds[f];
    for (int i = 0; i < fd.n_gp; ++i) {
      if (fd.active && fd.active[i] == 0) continue;
      double F12[12];
      auto grad_sum = [&](const int64_t* ptr, const int32_t* idx, const double* dps, double* a1, double* a2) {
        a1[0] = 1.0; a1[1] = 0.0; a1[2] = 0.0;
        a2[0] = 0.0; a2[1] = 1.0; a2[2] = 0.0;
        for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) {
          const double* u = x + 3 * static_cast<int64_t>(idx[e]);
          for (int c = 0; c < 3; ++c) { a1[c] += u[c] * dps[2 * e]; a2[c] += u[c] * dps[2 * e + 1]; }
        }
      };
      grad_sum(fd.l_ptr, fd.l_idx, fd.l_dpsi, F12, F12 + 3);
      grad_sum(fd.r_ptr, fd.r_idx, fd.r_dpsi, F12 + 6, F12 + 9);
      const double theta = orc_fold_angle(F12, fd.tangent[2 * i], fd.tangent[2 * i + 1], nullptr);
      const double th0 = fd.theta0_gp ? fd.theta0_gp[i] : fd.theta0;
      const double d = theta - th0;
      E += fd.weight[i] * (0.5 * fd.Kt * (d * d));
    }
  }
  return E;
}

void orc_strain_energies(int n_gp, const double* gp_weight, const int64_t* nbr_ptr, const int32_t* nbr_idx,
                         const double* dpsi, const double* ddpsi, const double* x, const double* A,
                         const double* B, const double* D, double* E_mem, double* E_ben, const double* gp_xy) {
  // plate/Meshless.h:204-220 (e1 from E1_el, Meshless.h:212).
  double em = 0.0, eb = 0.0;
  for (int g = 0; g < n_gp; ++g) {
    Kin k;
    kinematics(nbr_ptr[g], nbr_ptr[g + 1], nbr_idx, dpsi, ddpsi, x, k, gp_xy ? gp_xy + 2 * g : nullptr);
    double Nr[3], Mr[3];
    resultants(k, A, B, D, Nr, Mr);
    const double e0[3] = {k.E0[0][0], k.E0[1][1], 2.0 * k.E0[0][1]};
    const double e1[3] = {k.E1el[0][0], k.E1el[1][1], 2.0 * k.E1el[0][1]};
    em += 0.5 * gp_weight[g] * dot3(e0, Nr);
    eb += 0.5 * gp_weight[g] * dot3(e1, Mr);
  }
  *E_mem = em;
  *E_ben = eb;
}

void orc_kinematics(int g, const int64_t* nbr_ptr, const int32_t* nbr_idx, const double* dpsi,
                    const double* ddpsi, const double* x, double* out, const double* X) {
  Kin k;
  kinematics(nbr_ptr[g], nbr_ptr[g + 1], nbr_idx, dpsi, ddpsi, x, k, X);
  std::memcpy(out, k.r0X, 24); std::memcpy(out + 3, k.r0Y, 24);
  std::memcpy(out + 6, k.r0XX, 24); std::memcpy(out + 9, k.r0YY, 24);
  std::memcpy(out + 12, k.r0XY, 24); std::memcpy(out + 15, k.b, 24);
  out[18] = k.C0inv[0][0]; out[19] = k.C0inv[0][1]; out[20] = k.C0inv[1][0]; out[21] = k.C0inv[1][1];
  out[22] = k.E0[0][0]; out[23] = k.E0[1][1]; out[24] = k.E0[0][1];
  out[25] = k.E1[0][0]; out[26] = k.E1[1][1]; out[27] = k.E1[0][1];
  out[28] = k.E1el[0][0]; out[29] = k.E1el[1][1]; out[30] = k.E1el[0][1];
}

}  // extern "C"
