// shape.cu — stage A on sm_103a: neighbour gather (GlobalFRNN) and RKPM shape
// functions with crease visibility (GlobalRKPM), FP64.
//
// Reference: core/include/curvami/FRNN.h:23-78, core/include/curvami/Enrichment.h:23-92,
// core/include/curvami/GlobalRKPM.h:15-397.
//
// Design: the node cell grid is a dense array over the reference's flattened cell key
// (y * cols + x, so keys that wrap across a row resolve to the same cells as the
// reference's hash map). One thread per Gauss point gathers its neighbours in the
// reference's order (dx outer, dy inner, node index ascending in a cell) with an FP64
// distance test written without FMA contraction, so the neighbour sets and their order
// are bit-exact. The RKPM solve is FP64-pipe bound on GB300 (the FP64 rate is 1/62 of
// the FP32 rate), so it also runs one Gauss point per thread: two passes over the
// neighbours (moments, then shape functions) recompute the per-neighbour jets instead
// of storing them, and per-node crease sides are hoisted into a per-node array.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>

#include "cgb_device.cuh"
#include "cgb_internal.h"

namespace cgb {
namespace {

constexpr int kThreads = 128;

struct GridDev {
  double minx, miny, cell;
  int cols;
  long long ncells;
  const int32_t* cell_start;  // ncells + 1
  const int32_t* cell_nodes;
};

// Thread per Gauss point: count (out_idx == nullptr) or fill the neighbour list.
__global__ void frnn_kernel(int n_gp, const double* __restrict__ gp_xy,
                            const double* __restrict__ node_xy, const double* __restrict__ rho_node,
                            double rho, double rho2, GridDev G, const int64_t* __restrict__ ptr,
                            int32_t* __restrict__ count, int32_t* __restrict__ out_idx,
                            double* __restrict__ out_s) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gp) return;
  const double gx = gp_xy[2 * g], gy = gp_xy[2 * g + 1];
  const int qx = static_cast<int>(floor(__ddiv_rn(__dsub_rn(gx, G.minx), G.cell)));
  const int qy = static_cast<int>(floor(__ddiv_rn(__dsub_rn(gy, G.miny), G.cell)));
  int64_t pos = out_idx ? ptr[g] : 0;
  int cnt = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    for (int dy = -1; dy <= 1; ++dy) {
      const long long key = static_cast<long long>(qy + dy) * G.cols + (qx + dx);
      if (key < 0 || key >= G.ncells) continue;
      const int k0 = G.cell_start[key], k1 = G.cell_start[key + 1];
      for (int k = k0; k < k1; ++k) {
        const int j = G.cell_nodes[k];
        const double ddx = __dsub_rn(node_xy[2 * j], gx);
        const double ddy = __dsub_rn(node_xy[2 * j + 1], gy);
        const double dist2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
        double r = rho, r2 = rho2;
        if (rho_node) { r = rho_node[j]; r2 = __dmul_rn(r, r); }
        if (dist2 <= r2) {
          if (out_idx) {
            out_idx[pos] = j;
            out_s[pos] = __ddiv_rn(__dsqrt_rn(dist2), r);
            ++pos;
          }
          ++cnt;
        }
      }
    }
  }
  if (!out_idx) count[g] = cnt;
}

// Per-node crease side sn = (f >= 0 ? +1 : -1) (GlobalRKPM.h:92-93).
__global__ void node_side_kernel(int n_nodes, const double* __restrict__ node_xy, DevCrease cr,
                                 int8_t* __restrict__ side) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_nodes) return;
  const DevIndicator I = eval_indicator(node_xy[2 * j], node_xy[2 * j + 1], cr);
  side[j] = (I.f >= 0.0) ? 1 : -1;
}

// Gauss-point indicators, 6 doubles per point per crease.
// Crease c's indicator at every Gauss point, written in place into the [g][crease][6]
// layout the RKPM kernel reads (n_creases values per point).
__global__ void gp_indicator_kernel(int n_gp, const double* __restrict__ gp_xy, DevCrease cr, int c, int n_creases,
                                    double* __restrict__ out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gp) return;
  const DevIndicator I = eval_indicator(gp_xy[2 * g], gp_xy[2 * g + 1], cr);
  double* o = out + 6 * (static_cast<int64_t>(g) * n_creases + c);
  o[0] = I.f; o[1] = I.gx; o[2] = I.gy; o[3] = I.hxx; o[4] = I.hyy; o[5] = I.hxy;
}

__device__ __forceinline__ void window(int kernel, double s, double& w, double& dw, double& d2w) {
  if (kernel == 0) {  // quartic spline, GlobalRKPM.h:15-17
    if (s >= 1.0) { w = 0.0; } else { const double s2 = s * s; w = 1.0 - 6.0 * s2 + 8.0 * s2 * s - 3.0 * s2 * s2; }
    dw = (s >= 1.0 || s < 1e-14) ? 0.0 : -12.0 * s + 24.0 * s * s - 12.0 * s * s * s;
    d2w = (s >= 1.0) ? 0.0 : -12.0 + 48.0 * s - 36.0 * s * s;
  } else {  // cubic B-spline (extension), same cut-offs
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

struct Jets { double w, x, y, xx, yy, xy; };

// Weight jets with crease visibility for one (Gauss point, neighbour) entry:
// GlobalRKPM.h:59-84 (including the reference's d2x = xi^2/s^3, d2y = eta^2/s^3) and
// the visibility product of GlobalRKPM.h:87-112.
__device__ __forceinline__ Jets weight_jets(int kernel, double xi, double eta, double si, double fac,
                                            int n_creases, const double* gind,
                                            const int8_t* node_side, int n_nodes, int j,
                                            double rho) {
  const double zx = xi * fac, zy = eta * fac;
  double wi, d, dd;
  window(kernel, si, wi, d, dd);
  const double dx = (si == 0.0) ? 0.0 : zx / si;
  const double dy = (si == 0.0) ? 0.0 : zy / si;
  Jets J;
  J.w = wi;
  J.x = d * dx;
  J.y = d * dy;
  const double si3 = si * si * si;
  const double d2x = (si == 0.0) ? dd : (zx * zx) / si3;
  const double d2y = (si == 0.0) ? dd : (zy * zy) / si3;
  J.xx = dd * dx * dx + d * d2x;
  J.yy = dd * dy * dy + d * d2y;
  J.xy = (si == 0.0) ? 0.0 : dd * dx * dy + d * (-(zx * zy) / si3);
  if (fac != 1.0) {
    const double f2 = fac * fac;
    J.x *= fac; J.y *= fac; J.xx *= f2; J.yy *= f2; J.xy *= f2;
  }
  for (int c = 0; c < n_creases; ++c) {
    const double* I = gind + 6 * c;
    const double sn = static_cast<double>(node_side[static_cast<int64_t>(c) * n_nodes + j]);
    const double W = 0.5 * (1.0 + sn * I[0]);
    const double dWx = 0.5 * sn * I[1] * rho, dWy = 0.5 * sn * I[2] * rho;
    const double ddWxx = 0.5 * sn * I[3] * rho * rho;
    const double ddWyy = 0.5 * sn * I[4] * rho * rho;
    const double ddWxy = 0.5 * sn * I[5] * rho * rho;
    const Jets o = J;
    J.w = o.w * W;
    J.x = o.x * W + o.w * dWx;
    J.y = o.y * W + o.w * dWy;
    J.xx = o.xx * W + 2.0 * o.x * dWx + o.w * ddWxx;
    J.yy = o.yy * W + 2.0 * o.y * dWy + o.w * ddWyy;
    J.xy = o.xy * W + o.x * dWy + o.y * dWx + o.w * ddWxy;
  }
  return J;
}

// Monomial basis jets (GlobalRKPM.h:114-152): degree-major, p_y ascending.
template <int ORDER>
struct Basis {
  static constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  double p[NP], px[NP], py[NP], pxx[NP], pyy[NP], pxy[NP];
  __device__ __forceinline__ explicit Basis(double x, double y) {
    double xp[ORDER + 1], yp[ORDER + 1];
    xp[0] = 1.0; yp[0] = 1.0;
#pragma unroll
    for (int q = 1; q <= ORDER; ++q) { xp[q] = xp[q - 1] * x; yp[q] = yp[q - 1] * y; }
    int idx = 0;
#pragma unroll
    for (int d = 0; d <= ORDER; ++d) {
#pragma unroll
      for (int qy = 0; qy <= d; ++qy) {
        const int qx = d - qy;
        p[idx] = xp[qx] * yp[qy];
        px[idx] = qx > 0 ? static_cast<double>(qx) * xp[qx > 0 ? qx - 1 : 0] * yp[qy] : 0.0;
        py[idx] = qy > 0 ? static_cast<double>(qy) * xp[qx] * yp[qy > 0 ? qy - 1 : 0] : 0.0;
        pxx[idx] = qx > 1 ? static_cast<double>(qx * (qx - 1)) * xp[qx > 1 ? qx - 2 : 0] * yp[qy] : 0.0;
        pyy[idx] = qy > 1 ? static_cast<double>(qy * (qy - 1)) * xp[qx] * yp[qy > 1 ? qy - 2 : 0] : 0.0;
        pxy[idx] = (qx > 0 && qy > 0)
                       ? static_cast<double>(qx * qy) * xp[qx > 0 ? qx - 1 : 0] * yp[qy > 0 ? qy - 1 : 0]
                       : 0.0;
        ++idx;
      }
    }
  }
};

template <int NP>
struct PackedIdx {
  // K[i][j] of GlobalRKPM.h:29-36, row-major over i <= j.
  __device__ __forceinline__ static int k(int i, int j) {
    const int a = i < j ? i : j, b = i < j ? j : i;
    return a * NP - a * (a - 1) / 2 + (b - a);
  }
};

__device__ __forceinline__ void inv3(const double m[3][3], double r[3][3]) {
  const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  const double c10 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  const double c20 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  const double det = m[0][0] * c00 + m[0][1] * c10 + m[0][2] * c20;
  const double id = 1.0 / det;
  r[0][0] = c00 * id; r[1][0] = c10 * id; r[2][0] = c20 * id;
  r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
  r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
  r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
  r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
  r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
  r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
}

__device__ __forceinline__ void mm3(const double a[3][3], const double b[3][3], double c[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) c[r][k] = a[r][0] * b[0][k] + a[r][1] * b[1][k] + a[r][2] * b[2][k];
}

// Raw moments xi^a eta^b, a + b <= 2 ORDER, degree-major with b ascending; basis
// function i of Basis<ORDER> is the monomial xi^bx(i) eta^by(i).
template <int ORDER>
struct RawIdx {
  static constexpr int D = 2 * ORDER;
  static constexpr int NR = (D + 1) * (D + 2) / 2;
  __host__ __device__ static constexpr int r(int a, int b) { return (a + b) * (a + b + 1) / 2 + b; }
  __host__ __device__ static constexpr int deg(int i) {
    int d = 0;
    while ((d + 1) * (d + 2) / 2 <= i) ++d;
    return d;
  }
  __host__ __device__ static constexpr int by(int i) { return i - deg(i) * (deg(i) + 1) / 2; }
  __host__ __device__ static constexpr int bx(int i) { return deg(i) - by(i); }
};

struct RkpmArgs {
  int n_gp, n_nodes, kernel, n_creases;
  double rho;
  const double* gp_xy;
  const double* node_xy;
  const double* rho_node;
  const int64_t* ptr;
  const int32_t* idx;
  const double* s;
  const double* gind;        // 6 * n_creases per Gauss point
  const int8_t* node_side;   // n_creases * n_nodes
  double* psi;
  double* dpsi;
  double* ddpsi;
  int8_t* bad;
};

// One Gauss point per thread: GlobalRKPM.h:59-397 for that point.
template <int ORDER>
__global__ void __launch_bounds__(kThreads) rkpm_kernel(RkpmArgs a) {
  constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  constexpr int NM = NP * (NP + 1) / 2;
  using PI = PackedIdx<NP>;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n_gp) return;
  const int64_t p0 = a.ptr[g], p1 = a.ptr[g + 1];
  const double gx = a.gp_xy[2 * g], gy = a.gp_xy[2 * g + 1];
  double gind[6 * 4];
  const int nc = a.n_creases < 4 ? a.n_creases : 4;
  for (int c = 0; c < 6 * nc; ++c) gind[c] = a.gind[static_cast<int64_t>(g) * 6 * a.n_creases + c];

  // Moments (GlobalRKPM.h:161-189): M, dMx, dMy, d2Mxx, d2Myy, d2Mxy. Every entry of
  // M = sum_I w_I p_I p_I^T is a raw moment mu_ab = sum_I w_I xi^a eta^b with
  // a + b <= 2 ORDER, and the jets follow from the weight jets by the product rule,
  //   D_x mu_ab = S^x_ab + a S_{a-1,b},   D_xx mu_ab = S^xx_ab + 2a S^x_{a-1,b} + a(a-1) S_{a-2,b},
  //   D_xy mu_ab = S^xy_ab + b S^x_{a,b-1} + a S^y_{a-1,b} + ab S_{a-1,b-1}   (y alike),
  // with S^g_ab = sum_I (D^g w_I) xi^a eta^b. Accumulating the 6 x NR sums S per neighbour
  // (90 FMA for ORDER 2) replaces the 6 x NM jets of p_i p_j (about 6x the FP64 work);
  // M and its jets are formed once per point.
  using RI = RawIdx<ORDER>;
  constexpr int NR = RI::NR;
  double S0[NR], Sx[NR], Sy[NR], Sxx[NR], Syy[NR], Sxy[NR];
#pragma unroll
  for (int k = 0; k < NR; ++k) { S0[k] = 0; Sx[k] = 0; Sy[k] = 0; Sxx[k] = 0; Syy[k] = 0; Sxy[k] = 0; }
  for (int64_t e = p0; e < p1; ++e) {
    const int j = a.idx[e];
    const double xi = (gx - a.node_xy[2 * j]) / a.rho;
    const double eta = (gy - a.node_xy[2 * j + 1]) / a.rho;
    const double fac = a.rho_node ? a.rho / a.rho_node[j] : 1.0;
    const Jets J = weight_jets(a.kernel, xi, eta, a.s[e], fac, nc, gind, a.node_side, a.n_nodes, j, a.rho);
    double xp[RI::D + 1], yp[RI::D + 1];
    xp[0] = 1.0; yp[0] = 1.0;
#pragma unroll
    for (int q = 1; q <= RI::D; ++q) { xp[q] = xp[q - 1] * xi; yp[q] = yp[q - 1] * eta; }
#pragma unroll
    for (int d = 0; d <= RI::D; ++d) {
#pragma unroll
      for (int b = 0; b <= d; ++b) {
        const int k = RI::r(d - b, b);
        const double m = xp[d - b] * yp[b];
        S0[k] += J.w * m; Sx[k] += J.x * m; Sy[k] += J.y * m;
        Sxx[k] += J.xx * m; Syy[k] += J.yy * m; Sxy[k] += J.xy * m;
      }
    }
  }
  double M[NM], Mx[NM], My[NM], Mxx[NM], Myy[NM], Mxy[NM];
  {
    auto at = [](const double* S, int aa, int bb) { return (aa < 0 || bb < 0) ? 0.0 : S[RI::r(aa, bb)]; };
#pragma unroll
    for (int ip = 0; ip < NP; ++ip) {
#pragma unroll
      for (int jp = ip; jp < NP; ++jp) {
        const int k = PI::k(ip, jp);
        const int A = RI::bx(ip) + RI::bx(jp), Bq = RI::by(ip) + RI::by(jp);
        const double fa = static_cast<double>(A), fb = static_cast<double>(Bq);
        M[k] = at(S0, A, Bq);
        Mx[k] = at(Sx, A, Bq) + fa * at(S0, A - 1, Bq);
        My[k] = at(Sy, A, Bq) + fb * at(S0, A, Bq - 1);
        Mxx[k] = at(Sxx, A, Bq) + 2.0 * fa * at(Sx, A - 1, Bq) + fa * (fa - 1.0) * at(S0, A - 2, Bq);
        Myy[k] = at(Syy, A, Bq) + 2.0 * fb * at(Sy, A, Bq - 1) + fb * (fb - 1.0) * at(S0, A, Bq - 2);
        Mxy[k] = at(Sxy, A, Bq) + fb * at(Sx, A, Bq - 1) + fa * at(Sy, A - 1, Bq) + fa * fb * at(S0, A - 1, Bq - 1);
      }
    }
  }

  // The reference inverts M by blocks (GlobalRKPM.h:197-345): the leading 3x3 block with
  // a residual guard, then one bordering step per further basis function with a Schur-pivot
  // guard, carrying the five derivative jets of the whole inverse along. The shape
  // functions only use row 0 of M^-1 and its jets, i.e. b = M^-1 e0 and
  //   b_x = -M^-1 (M_x b),  b_xx = -M^-1 (M_xx b + 2 M_x b_x),
  //   b_xy = -M^-1 (M_xy b + M_x b_y + M_y b_x)   (y alike),
  // so M is factored once (LDL^T, no pivoting: M is symmetric positive semi-definite) and
  // six solves give b and its jets - about a quarter of the FP64 work of the full inverse
  // jets. The guards are evaluated as the reference does: the 3x3 residual test on the
  // leading block, and the pivot test on the Schur complements, which are the LDL^T pivots
  // d_k for k >= 3.
  int bad = 0;
  {
    double m3[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) m3[r][c] = M[PI::k(r, c)];
    double inv[3][3], chk[3][3];
    inv3(m3, inv);
    mm3(m3, inv, chk);
    bool finite = true;
    double res = 0.0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (!isfinite(inv[r][c])) finite = false;
        res = fmax(res, fabs(chk[r][c] - (r == c ? 1.0 : 0.0)));
      }
    if (!finite || res > 1e-8) bad = 1;
  }
  // LDL^T of M: L unit lower (packed like M, strictly lower part used), D diagonal.
  double Lf[NP][NP], Dg[NP], iD[NP];
#pragma unroll
  for (int j = 0; j < NP; ++j) {
    double d = M[PI::k(j, j)];
#pragma unroll
    for (int q = 0; q < j; ++q) d -= Lf[j][q] * Lf[j][q] * Dg[q];
    Dg[j] = d;
    iD[j] = 1.0 / d;
    if (j >= 3 && !(fabs(d) > 1e-12 * fmax(fabs(M[PI::k(j, j)]), 1.0)) && bad == 0) bad = 2;
#pragma unroll
    for (int i = j + 1; i < NP; ++i) {
      double v = M[PI::k(i, j)];
#pragma unroll
      for (int q = 0; q < j; ++q) v -= Lf[i][q] * Lf[j][q] * Dg[q];
      Lf[i][j] = v * iD[j];
    }
  }
  a.bad[g] = static_cast<int8_t>(bad);
  // x <- M^-1 x in place.
  auto solve = [&](double* x) {
#pragma unroll
    for (int i = 1; i < NP; ++i)
#pragma unroll
      for (int q = 0; q < i; ++q) x[i] -= Lf[i][q] * x[q];
#pragma unroll
    for (int i = 0; i < NP; ++i) x[i] *= iD[i];
#pragma unroll
    for (int i = NP - 2; i >= 0; --i)
#pragma unroll
      for (int q = i + 1; q < NP; ++q) x[i] -= Lf[q][i] * x[q];
  };
  // y += alpha * S x for a packed symmetric S.
  auto symv = [&](const double* S, const double* x, double alpha, double* y) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < NP; ++q) t += S[PI::k(i, q)] * x[q];
      y[i] += alpha * t;
    }
  };
  double c0[NP], c0x[NP], c0y[NP], c0xx[NP], c0yy[NP], c0xy[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    c0[i] = i == 0 ? 1.0 : 0.0;
    c0x[i] = 0.0; c0y[i] = 0.0; c0xx[i] = 0.0; c0yy[i] = 0.0; c0xy[i] = 0.0;
  }
  solve(c0);
  symv(Mx, c0, -1.0, c0x); solve(c0x);
  symv(My, c0, -1.0, c0y); solve(c0y);
  symv(Mxx, c0, -1.0, c0xx); symv(Mx, c0x, -2.0, c0xx); solve(c0xx);
  symv(Myy, c0, -1.0, c0yy); symv(My, c0y, -2.0, c0yy); solve(c0yy);
  symv(Mxy, c0, -1.0, c0xy); symv(Mx, c0y, -1.0, c0xy); symv(My, c0x, -1.0, c0xy); solve(c0xy);
  // Shape functions (GlobalRKPM.h:363-396).
  const double rho2 = a.rho * a.rho;
  for (int64_t e = p0; e < p1; ++e) {
    const int j = a.idx[e];
    const double xi = (gx - a.node_xy[2 * j]) / a.rho;
    const double eta = (gy - a.node_xy[2 * j + 1]) / a.rho;
    const double fac = a.rho_node ? a.rho / a.rho_node[j] : 1.0;
    const Jets J = weight_jets(a.kernel, xi, eta, a.s[e], fac, nc, gind, a.node_side, a.n_nodes, j, a.rho);
    const Basis<ORDER> B(xi, eta);
    double C = 0.0, Cx = 0.0, Cy = 0.0, Cxx = 0.0, Cyy = 0.0, Cxy = 0.0;
#pragma unroll
    for (int jp = 0; jp < NP; ++jp) {
      C += c0[jp] * B.p[jp];
      Cx += c0x[jp] * B.p[jp] + c0[jp] * B.px[jp];
      Cy += c0y[jp] * B.p[jp] + c0[jp] * B.py[jp];
      Cxx += c0xx[jp] * B.p[jp] + 2.0 * c0x[jp] * B.px[jp] + c0[jp] * B.pxx[jp];
      Cyy += c0yy[jp] * B.p[jp] + 2.0 * c0y[jp] * B.py[jp] + c0[jp] * B.pyy[jp];
      Cxy += c0xy[jp] * B.p[jp] + c0x[jp] * B.py[jp] + c0y[jp] * B.px[jp] + c0[jp] * B.pxy[jp];
    }
    a.psi[e] = C * J.w;
    a.dpsi[2 * e] = (Cx * J.w + C * J.x) / a.rho;
    a.dpsi[2 * e + 1] = (Cy * J.w + C * J.y) / a.rho;
    a.ddpsi[3 * e] = (Cxx * J.w + 2.0 * Cx * J.x + C * J.xx) / rho2;
    a.ddpsi[3 * e + 1] = (Cyy * J.w + 2.0 * Cy * J.y + C * J.yy) / rho2;
    a.ddpsi[3 * e + 2] = (Cxy * J.w + Cx * J.y + Cy * J.x + C * J.xy) / rho2;
  }
}

inline unsigned blocks_for(int64_t n, int t = kThreads) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

void shape_values(cgb_context* ctx, cgb_shape* out, const std::vector<Crease>& creases);

void shape_build(cgb_context* ctx, const double* gp_xy, int n_gp, const cgb_shape_params& prm,
                 const std::vector<Crease>& creases, cgb_shape* out) {
  cudaStream_t st = ctx->stream;
  const int n_nodes = ctx->n_nodes;
  if (n_nodes <= 0) throw Error(CGB_ERR_INVALID, "cgb_shape_build: nodes not set (cgb_set_nodes)");
  if (n_gp < 0) throw Error(CGB_ERR_INVALID, "cgb_shape_build: n_gp < 0");
  if (prm.order < 1 || prm.order > 3)
    throw Error(CGB_ERR_INVALID, "cgb_shape_build: order must be 1, 2 or 3");
  if (!(prm.rho > 0.0)) throw Error(CGB_ERR_INVALID, "cgb_shape_build: rho must be > 0");
  if (creases.size() > 4) throw Error(CGB_ERR_CAPACITY, "cgb_shape_build: at most 4 creases per call");
  out->ctx = ctx;
  out->n_gp = n_gp;
  out->rho = prm.rho;
  out->order = prm.order;
  out->kernel = prm.kernel;
  out->node_gen = ctx->node_gen;

  // ---- node cell grid (FRNN.h:33-44), host side, O(n_nodes) ----
  const double* nxy = ctx->h_node_xy.data();
  double cell = prm.rho;
  std::vector<double> rn;
  if (prm.rho_node) {
    rn.assign(prm.rho_node, prm.rho_node + n_nodes);
    cell = 0.0;
    for (double r : rn) {
      if (!(r > 0.0)) throw Error(CGB_ERR_INVALID, "cgb_shape_build: rho_node must be > 0");
      cell = std::max(cell, r);
    }
  }
  double minx = nxy[0], miny = nxy[1], maxx = nxy[0];
  for (int i = 0; i < n_nodes; ++i) {
    minx = std::min(minx, nxy[2 * i]);
    miny = std::min(miny, nxy[2 * i + 1]);
    maxx = std::max(maxx, nxy[2 * i]);
  }
  const int cols = static_cast<int>(std::ceil((maxx - minx) / cell)) + 1;
  std::vector<long long> key(n_nodes);
  long long kmax = 0;
  for (int i = 0; i < n_nodes; ++i) {
    const int cx = static_cast<int>(std::floor((nxy[2 * i] - minx) / cell));
    const int cy = static_cast<int>(std::floor((nxy[2 * i + 1] - miny) / cell));
    key[i] = static_cast<long long>(cy) * cols + cx;
    kmax = std::max(kmax, key[i]);
  }
  const long long ncells = kmax + 1;
  if (ncells > (1LL << 28))
    throw Error(CGB_ERR_CAPACITY, "cgb_shape_build: the node cell grid exceeds 2^28 cells (rho too small for the node extent)");
  std::vector<int32_t> cstart(ncells + 1, 0), cnodes(n_nodes);
  for (int i = 0; i < n_nodes; ++i) cstart[key[i] + 1]++;
  for (long long c = 0; c < ncells; ++c) cstart[c + 1] += cstart[c];
  {
    std::vector<int32_t> cur(cstart.begin(), cstart.end() - 1);
    for (int i = 0; i < n_nodes; ++i) cnodes[cur[key[i]]++] = i;  // ascending node index per cell
  }
  DevBuf<int32_t> d_cstart, d_cnodes;
  upload(d_cstart, cstart.data(), cstart.size(), st);
  upload(d_cnodes, cnodes.data(), cnodes.size(), st);
  out->has_rho_node = prm.rho_node != nullptr;
  if (prm.rho_node) upload(out->rho_node, rn.data(), rn.size(), st);
  const double* d_rn = prm.rho_node ? out->rho_node.p : nullptr;
  GridDev G{minx, miny, cell, cols, ncells, d_cstart.p, d_cnodes.p};

  upload(out->gp_xy, gp_xy, 2 * static_cast<size_t>(n_gp), st);
  const double rho2 = prm.rho * prm.rho;
  DevBuf<int32_t> d_cnt(n_gp);
  prof_begin(ctx, CGB_PHASE_FRNN);
  if (n_gp > 0)
    frnn_kernel<<<blocks_for(n_gp), kThreads, 0, st>>>(n_gp, out->gp_xy.p, ctx->node_xy.p,
                                                        d_rn, prm.rho, rho2, G,
                                                        nullptr, d_cnt.p, nullptr, nullptr);
  CGB_CUDA(cudaGetLastError());
  prof_end(ctx, CGB_PHASE_FRNN, n_gp > 0 ? 1 : 0);
  std::vector<int32_t> cnt(n_gp);
  if (n_gp > 0)
    CGB_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt.p, sizeof(int32_t) * n_gp, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> ptr(n_gp + 1, 0);
  int max_n = 0;
  for (int g = 0; g < n_gp; ++g) {
    ptr[g + 1] = ptr[g] + cnt[g];
    max_n = std::max(max_n, cnt[g]);
  }
  const int64_t nnz = ptr[n_gp];
  if (nnz >= (1LL << 31)) throw Error(CGB_ERR_CAPACITY, "cgb_shape_build: more than 2^31 neighbour entries");
  out->nnz = nnz;
  out->max_n = max_n;
  upload(out->nbr_ptr, ptr.data(), ptr.size(), st);
  out->nbr_idx.alloc(nnz);
  out->s.alloc(nnz);
  prof_begin(ctx, CGB_PHASE_FRNN);
  if (n_gp > 0)
    frnn_kernel<<<blocks_for(n_gp), kThreads, 0, st>>>(n_gp, out->gp_xy.p, ctx->node_xy.p,
                                                        d_rn, prm.rho, rho2, G,
                                                        out->nbr_ptr.p, nullptr, out->nbr_idx.p, out->s.p);
  prof_end(ctx, CGB_PHASE_FRNN, n_gp > 0 ? 1 : 0);
  CGB_CUDA(cudaGetLastError());

  out->rebuildable = true;
  shape_values(ctx, out, creases);
}

// Crease indicators, RKPM and the reference's guards for the points and neighbour lists
// already in `out` (SetupHelper::recomputeShapeFunctions after the FRNN). The value
// arrays keep their allocation when they have one, so device pointers handed out
// earlier (assemblers, captured graphs) stay valid across rebuilds.
void shape_values(cgb_context* ctx, cgb_shape* out, const std::vector<Crease>& creases) {
  cudaStream_t st = ctx->stream;
  const int n_nodes = ctx->n_nodes;
  const int n_gp = out->n_gp;
  const int64_t nnz = out->nnz;
  if (creases.size() > 4) throw Error(CGB_ERR_CAPACITY, "cgb_shape_build: at most 4 creases per call");
  const int nc = static_cast<int>(creases.size());
  std::vector<double> all_xy;
  std::vector<size_t> off(nc + 1, 0);
  for (int c = 0; c < nc; ++c) {
    all_xy.insert(all_xy.end(), creases[c].xy.begin(), creases[c].xy.end());
    off[c + 1] = all_xy.size();
  }
  out->scr_cxy.ensure(std::max<size_t>(all_xy.size(), 1));
  out->scr_side.ensure(static_cast<size_t>(std::max(nc, 1)) * n_nodes);
  out->scr_gind.ensure(static_cast<size_t>(std::max(nc, 1)) * 6 * std::max(n_gp, 1));
  out->scr_bad.ensure(std::max(n_gp, 1));
  if (!all_xy.empty())
    CGB_CUDA(cudaMemcpyAsync(out->scr_cxy.p, all_xy.data(), all_xy.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  int8_t* side = out->scr_side.p;
  double* gind = out->scr_gind.p;
  std::vector<DevCrease> dcr(nc);
  prof_begin(ctx, CGB_PHASE_CREASE);
  for (int c = 0; c < nc; ++c) {
    dcr[c] = DevCrease{out->scr_cxy.p + off[c], static_cast<int>(creases[c].xy.size() / 2), creases[c].extend_start,
                       creases[c].extend_end, creases[c].is_closed};
    node_side_kernel<<<blocks_for(n_nodes), kThreads, 0, st>>>(n_nodes, ctx->node_xy.p, dcr[c],
                                                                 side + static_cast<int64_t>(c) * n_nodes);
  }
  // Gauss-point indicators laid out [g][c][6].
  if (nc > 0 && n_gp > 0)
    for (int c = 0; c < nc; ++c)
      gp_indicator_kernel<<<blocks_for(n_gp), kThreads, 0, st>>>(n_gp, out->gp_xy.p, dcr[c], c, nc, gind);
  prof_end(ctx, CGB_PHASE_CREASE, nc * (1 + (n_gp > 0 ? 1 : 0)));
  CGB_CUDA(cudaGetLastError());

  // ---- RKPM ----
  if (out->psi.n < static_cast<size_t>(std::max<int64_t>(nnz, 1))) out->psi.alloc(nnz);
  if (out->dpsi.n < static_cast<size_t>(std::max<int64_t>(2 * nnz, 1))) out->dpsi.alloc(2 * nnz);
  if (out->ddpsi.n < static_cast<size_t>(std::max<int64_t>(3 * nnz, 1))) out->ddpsi.alloc(3 * nnz);
  int8_t* bad = out->scr_bad.p;
  RkpmArgs ra{n_gp, n_nodes, out->kernel, nc, out->rho, out->gp_xy.p, ctx->node_xy.p,
              out->has_rho_node ? out->rho_node.p : nullptr, out->nbr_ptr.p, out->nbr_idx.p, out->s.p, gind,
              side, out->psi.p, out->dpsi.p, out->ddpsi.p, bad};
  prof_begin(ctx, CGB_PHASE_RKPM);
  if (n_gp > 0) {
    switch (out->order) {
      case 1: rkpm_kernel<1><<<blocks_for(n_gp), kThreads, 0, st>>>(ra); break;
      case 2: rkpm_kernel<2><<<blocks_for(n_gp), kThreads, 0, st>>>(ra); break;
      default: rkpm_kernel<3><<<blocks_for(n_gp), kThreads, 0, st>>>(ra); break;
    }
  }
  prof_end(ctx, CGB_PHASE_RKPM, n_gp > 0 ? 1 : 0);
  CGB_CUDA(cudaGetLastError());
  std::vector<int8_t> hbad(n_gp);
  if (n_gp > 0) CGB_CUDA(cudaMemcpyAsync(hbad.data(), bad, n_gp, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  // The reference's guards (GlobalRKPM.h:241-257 after the 3x3 block, 347-359 after
  // the bordering): singular first, then pivot collapse.
  size_t n1 = 0, f1 = 0, n2 = 0, f2 = 0;
  for (int g = 0; g < n_gp; ++g) {
    if (hbad[g] == 1) { if (!n1) f1 = g; ++n1; }
    if (hbad[g] == 2) { if (!n2) f2 = g; ++n2; }
  }
  auto count_of = [&](size_t g) {
    int64_t pr[2];
    CGB_CUDA(cudaMemcpy(pr, out->nbr_ptr.p + g, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost));
    return pr[1] - pr[0];
  };
  if (n1) {
    throw Error(CGB_ERR_SINGULAR,
                "RKPM: singular moment matrix at " + std::to_string(n1) + " of " + std::to_string(n_gp) +
                    " Gauss points (first is index " + std::to_string(f1) + " with " +
                    std::to_string(count_of(f1)) +
                    " neighbours). The support is rank-deficient for the requested "
                    "basis order - typically too few visible nodes, which happens "
                    "where a crease cuts most of a support away. Increase the support "
                    "radius, refine the mesh there, or lower the order.");
  }
  if (n2) {
    throw Error(CGB_ERR_PIVOT,
                "RKPM: moment-matrix pivot collapsed during block inversion at " + std::to_string(n2) +
                    " of " + std::to_string(n_gp) + " Gauss points (first is index " + std::to_string(f2) +
                    " with " + std::to_string(count_of(f2)) +
                    " neighbours). Same cause and remedies as a singular moment matrix.");
  }
}

void shape_rebuild(cgb_shape* sh, const std::vector<Crease>& creases) {
  cgb_context* ctx = sh->ctx;
  if (!sh->rebuildable)
    throw Error(CGB_ERR_INVALID, "cgb_shape_rebuild: the set was not made by cgb_shape_build (wrapped or concatenated)");
  if (ctx->node_gen != sh->node_gen)
    throw Error(CGB_ERR_INVALID, "cgb_shape_rebuild: the nodes changed since the set was built (cgb_set_nodes)");
  // The new values stand even when a guard fires, as the reference's arrays do.
  ++sh->version;
  shape_values(ctx, sh, creases);
}

}  // namespace cgb
