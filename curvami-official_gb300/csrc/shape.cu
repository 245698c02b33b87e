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
#include "cgb_pair.cuh"

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

// FP32 pre-test of the FRNN distance test. Coordinates relative to the grid's lower corner
// are rounded to float (node32, per node; the point's in the kernel), the squared distance
// is formed in float, and `margin` bounds its difference from the exact squared distance
// (coordinate rounding, float arithmetic, the float radius; computed on the host from the
// extent of the nodes and points). A candidate beyond r^2 + margin is outside and one
// below r^2 - margin inside whatever FP64 gives; only those within the margin take the
// exact FP64 test, so every decision is the FP64 one.
struct FrnnPre {
  const float2* node32;   // per node, (x - minx, y - miny) in float
  const float* r2n32;     // per node r^2 in float, or nullptr for the single radius
  float r2f;              // the single radius squared, in float
  float margin;
};

// Thread per Gauss point: count (out_idx == nullptr) or fill the neighbour list.
__global__ void frnn_kernel(int n_gp, const double* __restrict__ gp_xy,
                            const double* __restrict__ node_xy, const double* __restrict__ rho_node,
                            double rho, double rho2, GridDev G, FrnnPre pre, const int64_t* __restrict__ ptr,
                            int32_t* __restrict__ count, int32_t* __restrict__ out_idx,
                            double* __restrict__ out_s) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gp) return;
  const double gx = gp_xy[2 * g], gy = gp_xy[2 * g + 1];
  const float gxf = __double2float_rn(gx - G.minx), gyf = __double2float_rn(gy - G.miny);
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
        const float2 nf = pre.node32[j];
        const float fdx = nf.x - gxf, fdy = nf.y - gyf;
        const float d2f = fdx * fdx + fdy * fdy;
        const float r2f = pre.r2n32 ? pre.r2n32[j] : pre.r2f;
        if (d2f > r2f + pre.margin) continue;          // outside, whatever FP64 gives
        bool inside = d2f < r2f - pre.margin;          // inside, whatever FP64 gives
        double dist2 = 0.0, r = rho;
        if (!inside || out_s) {
          const double ddx = __dsub_rn(node_xy[2 * j], gx);
          const double ddy = __dsub_rn(node_xy[2 * j + 1], gy);
          dist2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
          double r2 = rho2;
          if (rho_node) { r = rho_node[j]; r2 = __dmul_rn(r, r); }
          if (!inside) inside = dist2 <= r2;
        }
        if (inside) {
          if (out_idx) {
            out_idx[pos] = j;
            if (out_s) out_s[pos] = __ddiv_rn(__dsqrt_rn(dist2), r);
            ++pos;
          }
          ++cnt;
        }
      }
    }
  }
  if (!out_idx) count[g] = cnt;
}

// Normalised distances s of an existing neighbour list, with the FRNN's own rounded
// operations (so bitwise equal to what frnn_kernel writes); sets built in mixed
// precision skip s in the FRNN and compute it here when a caller downloads it.
__global__ void distance_kernel(int n_gp, const double* __restrict__ gp_xy, const double* __restrict__ node_xy,
                                const double* __restrict__ rho_node, double rho, const int64_t* __restrict__ ptr,
                                const int32_t* __restrict__ idx, double* __restrict__ out_s) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gp) return;
  const double gx = gp_xy[2 * g], gy = gp_xy[2 * g + 1];
  for (int64_t e = ptr[g]; e < ptr[g + 1]; ++e) {
    const int j = idx[e];
    const double ddx = __dsub_rn(node_xy[2 * j], gx);
    const double ddy = __dsub_rn(node_xy[2 * j + 1], gy);
    const double dist2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
    const double r = rho_node ? rho_node[j] : rho;
    out_s[e] = __ddiv_rn(__dsqrt_rn(dist2), r);
  }
}

// Neighbour counts -> CSR offsets on the device: ptr[g + 1] = sum of cnt[0..g], plus the
// total and the largest count for the host (two numbers instead of the whole array).
constexpr int kScanThreads = 1024;

__global__ void scan_local_kernel(int n, const int32_t* __restrict__ cnt, int64_t* __restrict__ ptr,
                                  int64_t* __restrict__ block_sum, int32_t* __restrict__ block_max) {
  __shared__ int64_t sv[kScanThreads];
  __shared__ int32_t mv[kScanThreads];
  const int t = threadIdx.x;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanThreads + t;
  const int32_t c = i < n ? cnt[i] : 0;
  sv[t] = c;
  mv[t] = c;
  __syncthreads();
  for (int off = 1; off < kScanThreads; off <<= 1) {   // Hillis-Steele inclusive scan
    const int64_t a = t >= off ? sv[t - off] : 0;
    const int32_t m = t >= off ? mv[t - off] : 0;
    __syncthreads();
    sv[t] += a;
    mv[t] = max(mv[t], m);
    __syncthreads();
  }
  if (i < n) ptr[i + 1] = sv[t];
  if (t == kScanThreads - 1) {
    block_sum[blockIdx.x] = sv[t];
    block_max[blockIdx.x] = mv[t];
  }
}

// One thread: block totals -> exclusive block offsets (in place); totals[0] = nnz, [1] = max.
__global__ void scan_blocks_kernel(int nb, int64_t* __restrict__ block_sum, const int32_t* __restrict__ block_max,
                                   int64_t* __restrict__ totals) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int64_t run = 0;
  int32_t mx = 0;
  for (int b = 0; b < nb; ++b) {
    const int64_t v = block_sum[b];
    block_sum[b] = run;
    run += v;
    mx = max(mx, block_max[b]);
  }
  totals[0] = run;
  totals[1] = mx;
}

__global__ void scan_add_kernel(int n, int64_t* __restrict__ ptr, const int64_t* __restrict__ block_off) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanThreads + threadIdx.x;
  if (i < n) ptr[i + 1] += block_off[blockIdx.x];
  if (i == 0) ptr[0] = 0;
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

// Row 0 of M^-1 and its five jets at one point.
template <int ORDER>
struct RowJets {
  static constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  double c0[NP], c0x[NP], c0y[NP], c0xx[NP], c0yy[NP], c0xy[NP];
};

// The per-point part of GlobalRKPM::solve (GlobalRKPM.h:161-359) from the raw-moment sums
// S^g_ab of the six weight jets (FP64): M and its jets, the reference's guards, and row 0
// of M^-1 with its jets. Returns the guard code (0 fine, 1 singular, 2 pivot collapse).
//
// Moments (GlobalRKPM.h:161-189): M, dMx, dMy, d2Mxx, d2Myy, d2Mxy. Every entry of
// M = sum_I w_I p_I p_I^T is a raw moment mu_ab = sum_I w_I xi^a eta^b with
// a + b <= 2 ORDER, and the jets follow from the weight jets by the product rule,
//   D_x mu_ab = S^x_ab + a S_{a-1,b},   D_xx mu_ab = S^xx_ab + 2a S^x_{a-1,b} + a(a-1) S_{a-2,b},
//   D_xy mu_ab = S^xy_ab + b S^x_{a,b-1} + a S^y_{a-1,b} + ab S_{a-1,b-1}   (y alike),
// with S^g_ab = sum_I (D^g w_I) xi^a eta^b.
template <int ORDER>
__device__ __forceinline__ int point_solve(const double* S0, const double* Sx, const double* Sy,
                                           const double* Sxx, const double* Syy, const double* Sxy,
                                           RowJets<ORDER>& R) {
  constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  constexpr int NM = NP * (NP + 1) / 2;
  using PI = PackedIdx<NP>;
  using RI = RawIdx<ORDER>;
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
  double(&c0)[NP] = R.c0;
  double(&c0x)[NP] = R.c0x;
  double(&c0y)[NP] = R.c0y;
  double(&c0xx)[NP] = R.c0xx;
  double(&c0yy)[NP] = R.c0yy;
  double(&c0xy)[NP] = R.c0xy;
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
  return bad;
}

struct RkpmArgs {
  int n_gp, n_nodes, kernel, n_creases;
  double rho;
  const float4* node_pair;   // mixed kernel: 2 per node (node_pair_kernel)
  fp2 irho, irho2;           // mixed kernel: 1 / rho and 1 / rho^2 as pairs
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
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n_gp) return;
  const int64_t p0 = a.ptr[g], p1 = a.ptr[g + 1];
  const double gx = a.gp_xy[2 * g], gy = a.gp_xy[2 * g + 1];
  // The point's crease indicators: a local copy for up to 4 creases, read in place beyond.
  double gloc[6 * 4];
  const int nc = a.n_creases;
  const double* gind = a.gind + static_cast<int64_t>(g) * 6 * nc;
  if (nc <= 4) {
    for (int c = 0; c < 6 * nc; ++c) gloc[c] = gind[c];
    gind = gloc;
  }

  // Raw-moment sums S^g_ab of the six weight jets (see point_solve). Accumulating the
  // 6 x NR sums per neighbour (90 FMA for ORDER 2) replaces the 6 x NM jets of p_i p_j
  // (about 6x the FP64 work); M and its jets are formed once per point.
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
  RowJets<ORDER> R;
  a.bad[g] = static_cast<int8_t>(point_solve<ORDER>(S0, Sx, Sy, Sxx, Syy, Sxy, R));
  const double(&c0)[NP] = R.c0;
  const double(&c0x)[NP] = R.c0x;
  const double(&c0y)[NP] = R.c0y;
  const double(&c0xx)[NP] = R.c0xx;
  const double(&c0yy)[NP] = R.c0yy;
  const double(&c0xy)[NP] = R.c0xy;
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


// ---- mixed precision: the per-neighbour work in FP32 pairs ----------------------------
//
// The FP64 kernel spends about 650 FP64 operations per neighbour (differences and
// divisions by rho, the window jets with their divisions by s, the crease product, the
// 90 moment FMAs, then the jets again and the shape-function sums), and GB300 issues FP64
// at 1/62 of the FP32 rate. The mixed kernels do all of that per-neighbour arithmetic in
// FP32 pairs (cgb_pair.cuh, about 48 significant bits) on the FP32 pipe, and keep FP64
// for the per-point part: the raw-moment sums are rounded to FP64 and point_solve forms
// M and its jets, applies the reference's guards, factors M (LDL^T) and solves for row 0
// of M^-1 and its jets exactly as the FP64 kernel does. Only the per-point factorisation
// is FP64, which is 1/n of the work; the shape functions are then summed in pairs from the
// FP64 row jets and rounded to FP64 once.
//
// Coordinates: node and point coordinates are split into three floats each (72 bits, so
// the split of a double is exact) and differenced in pairs, so xi = (x - x_I) / rho is
// accurate to the pair precision relative to xi itself, not to the coordinates' size.

__device__ __forceinline__ void split3(double v, float& a, float& b, float& c) {
  a = __double2float_rn(v);
  const double r = v - static_cast<double>(a);
  b = __double2float_rn(r);
  c = __double2float_rn(r - static_cast<double>(b));
}

// Per node: {x0, x1, x2, y0}, {y1, y2, fac.hi, fac.lo} with x = x0 + x1 + x2 and
// fac = rho / rho_I (1 for the single radius).
__global__ void node_pair_kernel(int n_nodes, const double* __restrict__ node_xy,
                                 const double* __restrict__ rho_node, double rho, float4* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_nodes) return;
  float x0, x1, x2, y0, y1, y2;
  split3(node_xy[2 * j], x0, x1, x2);
  split3(node_xy[2 * j + 1], y0, y1, y2);
  const fp2 fac = rho_node ? fp2_from_double(rho / rho_node[j]) : fp2{1.0f, 0.0f};
  out[2 * j] = make_float4(x0, x1, x2, y0);
  out[2 * j + 1] = make_float4(y1, y2, fac.hi, fac.lo);
}

// (a0 + a1 + a2) - (b0 + b1 + b2) as a pair.
__device__ __forceinline__ fp2 diff3(float a0, float a1, float a2, float b0, float b1, float b2) {
  const fp2 h = fp2_two_sum(a0, -b0);
  const fp2 m = fp2_two_sum(a1, -b1);
  return fp2_add_exact(h, m) + __fsub_rn(a2, b2);
}

constexpr float kTwoThirdsHi = static_cast<float>(2.0 / 3.0);
constexpr float kTwoThirdsLo = static_cast<float>(2.0 / 3.0 - static_cast<double>(kTwoThirdsHi));
constexpr float kFourThirdsHi = static_cast<float>(4.0 / 3.0);
constexpr float kFourThirdsLo = static_cast<float>(4.0 / 3.0 - static_cast<double>(kFourThirdsHi));

// window() in pairs, same branches and cut-offs, polynomials in Horner form.
__device__ __forceinline__ void window_pair(int kernel, fp2 s, fp2& w, fp2& dw, fp2& d2w) {
  const fp2 z{0.0f, 0.0f};
  if (fp2_ge(s, 1.0f)) { w = z; dw = z; d2w = z; return; }
  const bool tiny = s.hi < 1e-14f;
  if (kernel == 0) {  // 1 - 6 s^2 + 8 s^3 - 3 s^4
    const fp2 s2 = fp2_sqr(s);
    w = 1.0f + s2 * (-6.0f + s * (8.0f - 3.0f * s));
    dw = tiny ? z : s * (-12.0f + s * (24.0f - 12.0f * s));
    d2w = -12.0f + s * (48.0f - 36.0f * s);
  } else if (fp2_le(s, 0.5f)) {  // 2/3 - 4 s^2 + 4 s^3
    const fp2 s2 = fp2_sqr(s);
    w = fp2{kTwoThirdsHi, kTwoThirdsLo} + s2 * (-4.0f + 4.0f * s);
    dw = tiny ? z : s * (-8.0f + 12.0f * s);
    d2w = -8.0f + 24.0f * s;
  } else {  // 4/3 (1 - s)^3
    const fp2 r = 1.0f - s;
    const fp2 r2 = fp2_sqr(r);
    w = fp2{kFourThirdsHi, kFourThirdsLo} * (r2 * r);
    dw = -4.0f * r2;
    d2w = 8.0f * r;
  }
}

// weight_jets() in pairs: jets v = {w, x, y, xx, yy, xy}. gc holds per crease
// 0.5 I_f, 0.5 I_gx rho, 0.5 I_gy rho, 0.5 I_hxx rho^2, 0.5 I_hyy rho^2, 0.5 I_hxy rho^2.
struct JetsP {
  fp2 v[6];
};
__device__ __forceinline__ JetsP weight_jets_pair(int kernel, fp2 xi, fp2 eta, fp2 fac, bool scaled, int nc,
                                                  const fp2* gc, const int8_t* __restrict__ node_side,
                                                  int n_nodes, int j) {
  const fp2 zx = scaled ? xi * fac : xi, zy = scaled ? eta * fac : eta;
  const fp2 si = fp2_sqrt(fp2_sqr(zx) + fp2_sqr(zy));
  fp2 wi, d, dd;
  window_pair(kernel, si, wi, d, dd);
  JetsP J;
  J.v[0] = wi;
  if (fp2_is_zero(si)) {  // s == 0: dx = dy = 0, d2x = d2y = d2w, no cross term
    const fp2 z{0.0f, 0.0f};
    J.v[1] = z; J.v[2] = z;
    J.v[3] = d * dd; J.v[4] = d * dd; J.v[5] = z;
  } else {
    const fp2 is = fp2_recip(si);
    const fp2 dx = zx * is, dy = zy * is;
    const fp2 is3 = fp2_sqr(is) * is;
    J.v[1] = d * dx;
    J.v[2] = d * dy;
    J.v[3] = dd * fp2_sqr(dx) + d * (fp2_sqr(zx) * is3);  // the reference's d2x = xi^2 / s^3
    J.v[4] = dd * fp2_sqr(dy) + d * (fp2_sqr(zy) * is3);  // and d2y = eta^2 / s^3
    J.v[5] = dd * (dx * dy) - d * ((zx * zy) * is3);
  }
  if (scaled) {
    const fp2 f2 = fp2_sqr(fac);
    J.v[1] = J.v[1] * fac; J.v[2] = J.v[2] * fac;
    J.v[3] = J.v[3] * f2; J.v[4] = J.v[4] * f2; J.v[5] = J.v[5] * f2;
  }
  for (int c = 0; c < nc; ++c) {
    const fp2* G = gc + 6 * c;
    const float sn = node_side[static_cast<int64_t>(c) * n_nodes + j] > 0 ? 1.0f : -1.0f;
    const fp2 W = G[0] * sn + 0.5f;
    const fp2 dWx = G[1] * sn, dWy = G[2] * sn;
    const fp2 ddWxx = G[3] * sn, ddWyy = G[4] * sn, ddWxy = G[5] * sn;
    const JetsP o = J;
    J.v[0] = o.v[0] * W;
    J.v[1] = o.v[1] * W + o.v[0] * dWx;
    J.v[2] = o.v[2] * W + o.v[0] * dWy;
    J.v[3] = o.v[3] * W + 2.0f * (o.v[1] * dWx) + o.v[0] * ddWxx;
    J.v[4] = o.v[4] * W + 2.0f * (o.v[2] * dWy) + o.v[0] * ddWyy;
    J.v[5] = o.v[5] * W + o.v[1] * dWy + o.v[2] * dWx + o.v[0] * ddWxy;
  }
  return J;
}

// Monomial basis jets in pairs (Basis<ORDER> above).
template <int ORDER>
struct BasisPair {
  static constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  fp2 p[NP], px[NP], py[NP], pxx[NP], pyy[NP], pxy[NP];
  __device__ __forceinline__ static fp2 mono(const fp2* xp, const fp2* yp, int a, int b) {
    return a == 0 ? yp[b] : (b == 0 ? xp[a] : xp[a] * yp[b]);
  }
  __device__ __forceinline__ explicit BasisPair(fp2 x, fp2 y) {
    fp2 xp[ORDER + 1], yp[ORDER + 1];
    xp[0] = fp2{1.0f, 0.0f}; yp[0] = fp2{1.0f, 0.0f};
#pragma unroll
    for (int q = 1; q <= ORDER; ++q) { xp[q] = q == 1 ? x : xp[q - 1] * x; yp[q] = q == 1 ? y : yp[q - 1] * y; }
    const fp2 z{0.0f, 0.0f};
    int idx = 0;
#pragma unroll
    for (int d = 0; d <= ORDER; ++d) {
#pragma unroll
      for (int qy = 0; qy <= d; ++qy) {
        const int qx = d - qy;
        p[idx] = mono(xp, yp, qx, qy);
        px[idx] = qx > 0 ? static_cast<float>(qx) * mono(xp, yp, qx - 1, qy) : z;
        py[idx] = qy > 0 ? static_cast<float>(qy) * mono(xp, yp, qx, qy - 1) : z;
        pxx[idx] = qx > 1 ? static_cast<float>(qx * (qx - 1)) * mono(xp, yp, qx - 2, qy) : z;
        pyy[idx] = qy > 1 ? static_cast<float>(qy * (qy - 1)) * mono(xp, yp, qx, qy - 2) : z;
        pxy[idx] = (qx > 0 && qy > 0) ? static_cast<float>(qx * qy) * mono(xp, yp, qx - 1, qy - 1) : z;
        ++idx;
      }
    }
  }
};

// Per-point inputs of the pair passes.
struct PairPoint {
  float gx0, gx1, gx2, gy0, gy1, gy2;
  int nc;
  bool scaled;
  fp2 gc[6 * 4];    // scaled crease indicators, up to 4 creases
  const fp2* gcp;   // gc, or the point record's copy when there are more creases
};

__device__ __forceinline__ void pair_xi(const RkpmArgs& a, const PairPoint& P, int j, fp2& xi, fp2& eta, fp2& fac) {
  const float4 n0 = __ldg(a.node_pair + 2 * j), n1 = __ldg(a.node_pair + 2 * j + 1);
  xi = diff3(P.gx0, P.gx1, P.gx2, n0.x, n0.y, n0.z) * a.irho;
  eta = diff3(P.gy0, P.gy1, P.gy2, n0.w, n1.x, n1.y) * a.irho;
  fac = fp2{n1.z, n1.w};
}

// Raw-moment sums of weight jets J0 .. J0 + NJ - 1 over the point's neighbours, in pairs
// (Dot2 accumulation), rounded to FP64 into Sd[J0 + jj][k].
template <int ORDER, int J0, int NJ>
__device__ __forceinline__ void pair_moment_sums(const RkpmArgs& a, const PairPoint& P, int64_t p0, int64_t p1,
                                                 double (&Sd)[6][RawIdx<ORDER>::NR]) {
  using RI = RawIdx<ORDER>;
  constexpr int NR = RI::NR;
  fp2 S[NJ][NR];
#pragma unroll
  for (int q = 0; q < NJ; ++q)
#pragma unroll
    for (int k = 0; k < NR; ++k) S[q][k] = fp2{0.0f, 0.0f};
  for (int64_t e = p0; e < p1; ++e) {
    const int j = a.idx[e];
    fp2 xi, eta, fac;
    pair_xi(a, P, j, xi, eta, fac);
    const JetsP J = weight_jets_pair(a.kernel, xi, eta, fac, P.scaled, P.nc, P.gcp, a.node_side, a.n_nodes, j);
    fp2 xp[RI::D + 1], yp[RI::D + 1];
    xp[0] = fp2{1.0f, 0.0f}; yp[0] = fp2{1.0f, 0.0f};
#pragma unroll
    for (int q = 1; q <= RI::D; ++q) { xp[q] = q == 1 ? xi : xp[q - 1] * xi; yp[q] = q == 1 ? eta : yp[q - 1] * eta; }
#pragma unroll
    for (int d = 0; d <= RI::D; ++d) {
#pragma unroll
      for (int b = 0; b <= d; ++b) {
        const int k = RI::r(d - b, b);
        const fp2 m = BasisPair<ORDER>::mono(xp, yp, d - b, b);
#pragma unroll
        for (int q = 0; q < NJ; ++q) fp2_fma_acc(S[q][k], J.v[J0 + q], m);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NJ; ++q)
#pragma unroll
    for (int k = 0; k < NR; ++k) Sd[J0 + q][k] = fp2_to_double(S[q][k]);
}

// The mixed RKPM runs as two kernels:
//  - rkpm_pair_point_kernel, one Gauss point per thread: the raw-moment sums in pairs over
//    the point's neighbours, the per-point FP64 solve, and a point record for the second
//    kernel (the point's coordinates split in three floats, its crease indicators scaled
//    for the visibility product, and row 0 of M^-1 with its five jets, all as pairs);
//  - rkpm_pair_value_kernel, one (point, neighbour) pair per thread: the weight and basis
//    jets of that neighbour and Phi, grad Phi, Hessian Phi from the point record.
// Split this way the per-pair half runs at full occupancy instead of inside a thread
// that holds 90 pair accumulators, and each kernel's code fits the instruction cache.
//
// Launch shape of the point kernel, measured on the 1,000,000-point stage (order 2; RKPM
// phase of both kernels): 2 blocks per SM (255 registers) 8.24 ms, 3 blocks (168 registers,
// more spills) 8.80 ms; the jets summed in two passes of three (half the accumulators, the
// weight jets computed twice) 9.4 ms at 3 and 9.2 ms at 4 blocks per SM; before the split,
// one kernel doing both passes took 11.3 ms. Order 3 (28 raw moments) needs the two passes
// to keep the accumulators in registers.
constexpr int kPairMinBlocks = 2;
constexpr int kPairSplitOrder = 3;
constexpr int kPairValueThreads = 256;

// Floats per point record: 6 coordinate parts, 12 per crease (6 pairs), 12 per basis
// function (6 jets x 1 pair), rounded up to 4 so every record starts on 16 bytes.
__host__ __device__ constexpr int pair_record_floats(int order, int n_creases) {
  return (6 + 12 * n_creases + 6 * (order + 1) * (order + 2) + 3) & ~3;
}

template <int ORDER>
__global__ void __launch_bounds__(kThreads, kPairMinBlocks) rkpm_pair_point_kernel(RkpmArgs a, float* __restrict__ rec,
                                                                                   int RS) {
  constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  using RI = RawIdx<ORDER>;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n_gp) return;
  const int64_t p0 = a.ptr[g], p1 = a.ptr[g + 1];
  PairPoint P;
  split3(a.gp_xy[2 * g], P.gx0, P.gx1, P.gx2);
  split3(a.gp_xy[2 * g + 1], P.gy0, P.gy1, P.gy2);
  P.nc = a.n_creases;
  P.scaled = a.rho_node != nullptr;
  const double r1 = 0.5 * a.rho, r2 = 0.5 * a.rho * a.rho;
  float* out = rec + static_cast<int64_t>(g) * RS;
  // The scaled indicators go to the point record first; with more than 4 creases the
  // moment sums read them back from there (this thread's own writes).
  for (int c = 0; c < P.nc; ++c) {
    const double* I = a.gind + (static_cast<int64_t>(g) * a.n_creases + c) * 6;
    const fp2 v[6] = {fp2_from_double(0.5 * I[0]), fp2_from_double(r1 * I[1]), fp2_from_double(r1 * I[2]),
                      fp2_from_double(r2 * I[3]), fp2_from_double(r2 * I[4]), fp2_from_double(r2 * I[5])};
    for (int q = 0; q < 6; ++q) {
      if (c < 4) P.gc[6 * c + q] = v[q];
      out[6 + 2 * (6 * c + q)] = v[q].hi;
      out[7 + 2 * (6 * c + q)] = v[q].lo;
    }
  }
  P.gcp = P.nc <= 4 ? P.gc : reinterpret_cast<const fp2*>(out + 6);
  double Sd[6][RI::NR];
  if constexpr (ORDER < kPairSplitOrder) {
    pair_moment_sums<ORDER, 0, 6>(a, P, p0, p1, Sd);
  } else {
    pair_moment_sums<ORDER, 0, 3>(a, P, p0, p1, Sd);
    pair_moment_sums<ORDER, 3, 3>(a, P, p0, p1, Sd);
  }
  RowJets<ORDER> R;
  a.bad[g] = static_cast<int8_t>(point_solve<ORDER>(Sd[0], Sd[1], Sd[2], Sd[3], Sd[4], Sd[5], R));
  out[0] = P.gx0; out[1] = P.gx1; out[2] = P.gx2;
  out[3] = P.gy0; out[4] = P.gy1; out[5] = P.gy2;
  float2* cj = reinterpret_cast<float2*>(out + 6 + 12 * P.nc);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    fp2 v = fp2_from_double(R.c0[i]);   cj[i] = make_float2(v.hi, v.lo);
    v = fp2_from_double(R.c0x[i]);      cj[NP + i] = make_float2(v.hi, v.lo);
    v = fp2_from_double(R.c0y[i]);      cj[2 * NP + i] = make_float2(v.hi, v.lo);
    v = fp2_from_double(R.c0xx[i]);     cj[3 * NP + i] = make_float2(v.hi, v.lo);
    v = fp2_from_double(R.c0yy[i]);     cj[4 * NP + i] = make_float2(v.hi, v.lo);
    v = fp2_from_double(R.c0xy[i]);     cj[5 * NP + i] = make_float2(v.hi, v.lo);
  }
}

// Shape functions (GlobalRKPM.h:363-396) of one (point, neighbour) pair per thread. The
// point of pair e is the last g with ptr[g] <= e: lane 0 of each warp finds it for the
// warp's first pair by bisection, the other lanes step forward from there.
template <int ORDER>
__global__ void __launch_bounds__(kPairValueThreads) rkpm_pair_value_kernel(RkpmArgs a, const float* __restrict__ rec,
                                                                            int RS, int64_t nnz) {
  constexpr int NP = (ORDER + 1) * (ORDER + 2) / 2;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int g0 = 0;
  if (lane == 0) {
    const int64_t ef = e < nnz ? e : nnz - 1;
    int lo = 0, hi = a.n_gp;             // ptr[lo] <= ef < ptr[hi]
    while (hi - lo > 1) {
      const int mid = lo + (hi - lo) / 2;
      if (__ldg(a.ptr + mid) <= ef) lo = mid; else hi = mid;
    }
    g0 = lo;
  }
  g0 = __shfl_sync(0xffffffffu, g0, 0);
  if (e >= nnz) return;
  int g = g0;
  while (__ldg(a.ptr + g + 1) <= e) ++g;
  const float* R = rec + static_cast<int64_t>(g) * RS;
  const int nc = a.n_creases;
  const fp2* gc = reinterpret_cast<const fp2*>(R + 6);
  const fp2* cj = reinterpret_cast<const fp2*>(R + 6 + 12 * nc);
  const int j = a.idx[e];
  const float4 n0 = __ldg(a.node_pair + 2 * j), n1 = __ldg(a.node_pair + 2 * j + 1);
  const fp2 xi = diff3(__ldg(R), __ldg(R + 1), __ldg(R + 2), n0.x, n0.y, n0.z) * a.irho;
  const fp2 eta = diff3(__ldg(R + 3), __ldg(R + 4), __ldg(R + 5), n0.w, n1.x, n1.y) * a.irho;
  const fp2 fac{n1.z, n1.w};
  const JetsP J = weight_jets_pair(a.kernel, xi, eta, fac, a.rho_node != nullptr, nc, gc, a.node_side, a.n_nodes, j);
  const BasisPair<ORDER> B(xi, eta);
  const fp2 z{0.0f, 0.0f};
  fp2 C = z, Cx = z, Cy = z, Cxx = z, Cyy = z, Cxy = z;
#pragma unroll
  for (int jp = 0; jp < NP; ++jp) {
    const fp2 c0 = cj[jp], c0x = cj[NP + jp], c0y = cj[2 * NP + jp];
    const fp2 c0xx = cj[3 * NP + jp], c0yy = cj[4 * NP + jp], c0xy = cj[5 * NP + jp];
    const fp2 c0x2 = c0x * 2.0f, c0y2 = c0y * 2.0f;
    fp2_fma_acc(C, c0, B.p[jp]);
    fp2_fma_acc(Cx, c0x, B.p[jp]); fp2_fma_acc(Cx, c0, B.px[jp]);
    fp2_fma_acc(Cy, c0y, B.p[jp]); fp2_fma_acc(Cy, c0, B.py[jp]);
    fp2_fma_acc(Cxx, c0xx, B.p[jp]); fp2_fma_acc(Cxx, c0x2, B.px[jp]); fp2_fma_acc(Cxx, c0, B.pxx[jp]);
    fp2_fma_acc(Cyy, c0yy, B.p[jp]); fp2_fma_acc(Cyy, c0y2, B.py[jp]); fp2_fma_acc(Cyy, c0, B.pyy[jp]);
    fp2_fma_acc(Cxy, c0xy, B.p[jp]); fp2_fma_acc(Cxy, c0x, B.py[jp]);
    fp2_fma_acc(Cxy, c0y, B.px[jp]); fp2_fma_acc(Cxy, c0, B.pxy[jp]);
  }
  C = fp2_norm(C); Cx = fp2_norm(Cx); Cy = fp2_norm(Cy);
  Cxx = fp2_norm(Cxx); Cyy = fp2_norm(Cyy); Cxy = fp2_norm(Cxy);
  const fp2* w = J.v;
  fp2 gx = z, gy = z, hxx = z, hyy = z, hxy = z;
  fp2_fma_acc(gx, Cx, w[0]); fp2_fma_acc(gx, C, w[1]);
  fp2_fma_acc(gy, Cy, w[0]); fp2_fma_acc(gy, C, w[2]);
  const fp2 Cx2 = Cx * 2.0f, Cy2 = Cy * 2.0f;
  fp2_fma_acc(hxx, Cxx, w[0]); fp2_fma_acc(hxx, Cx2, w[1]); fp2_fma_acc(hxx, C, w[3]);
  fp2_fma_acc(hyy, Cyy, w[0]); fp2_fma_acc(hyy, Cy2, w[2]); fp2_fma_acc(hyy, C, w[4]);
  fp2_fma_acc(hxy, Cxy, w[0]); fp2_fma_acc(hxy, Cx, w[2]); fp2_fma_acc(hxy, Cy, w[1]); fp2_fma_acc(hxy, C, w[5]);
  a.psi[e] = fp2_to_double(C * w[0]);
  a.dpsi[2 * e] = fp2_to_double(fp2_norm(gx) * a.irho);
  a.dpsi[2 * e + 1] = fp2_to_double(fp2_norm(gy) * a.irho);
  a.ddpsi[3 * e] = fp2_to_double(fp2_norm(hxx) * a.irho2);
  a.ddpsi[3 * e + 1] = fp2_to_double(fp2_norm(hyy) * a.irho2);
  a.ddpsi[3 * e + 2] = fp2_to_double(fp2_norm(hxy) * a.irho2);
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
  out->ctx = ctx;
  out->n_gp = n_gp;
  out->rho = prm.rho;
  out->order = prm.order;
  out->kernel = prm.kernel;
  if (prm.precision != CGB_SHAPE_FP64 && prm.precision != CGB_SHAPE_MIXED)
    throw Error(CGB_ERR_INVALID, "cgb_shape_build: precision must be CGB_SHAPE_FP64 or CGB_SHAPE_MIXED");
  out->precision = prm.precision;
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
  out->has_xy = true;
  const double rho2 = prm.rho * prm.rho;
  // The FP32 pre-test (FrnnPre): float coordinates relative to (minx, miny) and the margin.
  // e = 2^-23 X (X the largest relative coordinate) bounds the rounding of one coordinate
  // with room to spare; c = cell = the largest radius. A candidate at distance d >= 2c (the
  // wrapped cell keys can bring far nodes) is outside under both tests: its float distance
  // is off by a relative 2^-22 at most, far above r^2 + margin. Every other candidate has
  // |dx|, |dy| < 2c and d^2 < 8 c^2; its float differences are off by eps <= 2e + 2^-24 2c
  // each, so the float d^2 is off by <= 2 (|dx| + |dy|) eps + 2 eps^2 <= 16 c e + 8 e^2 +
  // 2^-20 c^2 (+ lower order), its arithmetic by <= 2 ulp(8 c^2) = 2^-20 c^2 and the float
  // radius by <= 2^-24 c^2: below 16 c e + 8 e^2 + 64 2^-24 c^2.
  // X may be taken over the node box widened by two cells: a point farther out is more than
  // 2c from every node, truly outside, and its float distance (off by a relative 2^-23) stays
  // above 4 c^2 (1 - 2^-22)^2 > r^2 + margin, so it is classified outside too.
  double maxy = miny;
  for (int i = 0; i < n_nodes; ++i) maxy = std::max(maxy, nxy[2 * i + 1]);
  const double ext = std::max(maxx - minx, maxy - miny) + 2.0 * cell;
  const double e = std::ldexp(ext, -23), fu = std::ldexp(1.0, -24);
  const double margin = 16.0 * cell * e + 8.0 * e * e + 64.0 * fu * cell * cell;
  std::vector<float> n32(2 * static_cast<size_t>(n_nodes)), r32;
  for (int i = 0; i < n_nodes; ++i) {
    n32[2 * i] = static_cast<float>(nxy[2 * i] - minx);
    n32[2 * i + 1] = static_cast<float>(nxy[2 * i + 1] - miny);
  }
  DevBuf<float> d_n32, d_r32;
  upload(d_n32, n32.data(), n32.size(), st);
  if (prm.rho_node) {
    r32.resize(n_nodes);
    for (int i = 0; i < n_nodes; ++i) r32[i] = static_cast<float>(rn[i] * rn[i]);
    upload(d_r32, r32.data(), r32.size(), st);
  }
  const FrnnPre pre{reinterpret_cast<const float2*>(d_n32.p), prm.rho_node ? d_r32.p : nullptr,
                    static_cast<float>(rho2), static_cast<float>(margin)};
  DevBuf<int32_t> d_cnt(n_gp);
  prof_begin(ctx, CGB_PHASE_FRNN);
  if (n_gp > 0)
    frnn_kernel<<<blocks_for(n_gp), kThreads, 0, st>>>(n_gp, out->gp_xy.p, ctx->node_xy.p,
                                                        d_rn, prm.rho, rho2, G, pre,
                                                        nullptr, d_cnt.p, nullptr, nullptr);
  CGB_CUDA(cudaGetLastError());
  prof_end(ctx, CGB_PHASE_FRNN, n_gp > 0 ? 1 : 0);
  // CSR offsets on the device; only the total and the largest count come back.
  out->nbr_ptr.alloc(static_cast<size_t>(n_gp) + 1);
  int64_t totals[2] = {0, 0};
  if (n_gp > 0) {
    const int nb = static_cast<int>((static_cast<int64_t>(n_gp) + kScanThreads - 1) / kScanThreads);
    DevBuf<int64_t> bsum(nb), tot(2);
    DevBuf<int32_t> bmax(nb);
    scan_local_kernel<<<nb, kScanThreads, 0, st>>>(n_gp, d_cnt.p, out->nbr_ptr.p, bsum.p, bmax.p);
    scan_blocks_kernel<<<1, 1, 0, st>>>(nb, bsum.p, bmax.p, tot.p);
    scan_add_kernel<<<nb, kScanThreads, 0, st>>>(n_gp, out->nbr_ptr.p, bsum.p);
    CGB_CUDA(cudaGetLastError());
    CGB_CUDA(cudaMemcpyAsync(totals, tot.p, sizeof(totals), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
  } else {
    CGB_CUDA(cudaMemsetAsync(out->nbr_ptr.p, 0, sizeof(int64_t), st));
  }
  const int64_t nnz = totals[0];
  if (nnz >= (1LL << 31)) throw Error(CGB_ERR_CAPACITY, "cgb_shape_build: more than 2^31 neighbour entries");
  out->nnz = nnz;
  out->max_n = static_cast<int>(totals[1]);
  out->nbr_idx.alloc(nnz);
  // The mixed RKPM recomputes distances in FP32 pairs and does not read s, so a mixed set
  // skips the FRNN's rounded square roots and divisions; cgb_shape_download computes s on
  // demand (shape_distances), bitwise equal.
  const bool want_s = prm.precision != CGB_SHAPE_MIXED;
  if (want_s) out->s.alloc(nnz); else out->s.reset();
  prof_begin(ctx, CGB_PHASE_FRNN);
  if (n_gp > 0)
    frnn_kernel<<<blocks_for(n_gp), kThreads, 0, st>>>(n_gp, out->gp_xy.p, ctx->node_xy.p,
                                                        d_rn, prm.rho, rho2, G, pre,
                                                        out->nbr_ptr.p, nullptr, out->nbr_idx.p,
                                                        want_s ? out->s.p : nullptr);
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
  const double* d_rn = out->has_rho_node ? out->rho_node.p : nullptr;
  const bool mixed = out->precision == CGB_SHAPE_MIXED;
  auto pair_of = [](double v) {
    const float hi = static_cast<float>(v);
    return fp2{hi, static_cast<float>(v - static_cast<double>(hi))};
  };
  RkpmArgs ra{n_gp, n_nodes, out->kernel, nc, out->rho, nullptr, pair_of(1.0 / out->rho),
              pair_of(1.0 / (out->rho * out->rho)), out->gp_xy.p, ctx->node_xy.p, d_rn, out->nbr_ptr.p,
              out->nbr_idx.p, out->s.p, gind, side, out->psi.p, out->dpsi.p, out->ddpsi.p, bad};
  prof_begin(ctx, CGB_PHASE_RKPM);
  if (mixed && n_nodes > 0) {
    out->scr_node_pair.ensure(2 * static_cast<size_t>(n_nodes));
    node_pair_kernel<<<blocks_for(n_nodes), kThreads, 0, st>>>(n_nodes, ctx->node_xy.p, d_rn, out->rho,
                                                                 out->scr_node_pair.p);
    ra.node_pair = out->scr_node_pair.p;
  }
  if (n_gp > 0) {
    if (mixed) {
      const int RS = pair_record_floats(out->order, nc);
      out->scr_point_rec.ensure(static_cast<size_t>(n_gp) * RS);
      float* rec = out->scr_point_rec.p;
      const unsigned vb = blocks_for(std::max<int64_t>(nnz, 1), kPairValueThreads);
      switch (out->order) {
        case 1:
          rkpm_pair_point_kernel<1><<<blocks_for(n_gp), kThreads, 0, st>>>(ra, rec, RS);
          if (nnz > 0) rkpm_pair_value_kernel<1><<<vb, kPairValueThreads, 0, st>>>(ra, rec, RS, nnz);
          break;
        case 2:
          rkpm_pair_point_kernel<2><<<blocks_for(n_gp), kThreads, 0, st>>>(ra, rec, RS);
          if (nnz > 0) rkpm_pair_value_kernel<2><<<vb, kPairValueThreads, 0, st>>>(ra, rec, RS, nnz);
          break;
        default:
          rkpm_pair_point_kernel<3><<<blocks_for(n_gp), kThreads, 0, st>>>(ra, rec, RS);
          if (nnz > 0) rkpm_pair_value_kernel<3><<<vb, kPairValueThreads, 0, st>>>(ra, rec, RS, nnz);
          break;
      }
    } else {
      switch (out->order) {
        case 1: rkpm_kernel<1><<<blocks_for(n_gp), kThreads, 0, st>>>(ra); break;
        case 2: rkpm_kernel<2><<<blocks_for(n_gp), kThreads, 0, st>>>(ra); break;
        default: rkpm_kernel<3><<<blocks_for(n_gp), kThreads, 0, st>>>(ra); break;
      }
    }
  }
  prof_end(ctx, CGB_PHASE_RKPM, (n_gp > 0 ? 1 : 0) + (mixed && n_nodes > 0 ? 1 : 0) + (mixed && nnz > 0 ? 1 : 0));
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

void shape_distances(cgb_shape* sh) {
  cgb_context* ctx = sh->ctx;
  // Only sets built here in mixed precision lack s; wrapped or concatenated sets without
  // distances keep returning none, as before.
  if (sh->nnz == 0 || sh->s.n >= static_cast<size_t>(sh->nnz) || !sh->rebuildable) return;
  if (ctx->node_gen != sh->node_gen)
    throw Error(CGB_ERR_INVALID, "cgb_shape_download: s is computed on demand for mixed-precision sets and the "
                                 "nodes changed since the set was built (cgb_set_nodes)");
  sh->s.alloc(sh->nnz);
  distance_kernel<<<blocks_for(sh->n_gp), kThreads, 0, ctx->stream>>>(
      sh->n_gp, sh->gp_xy.p, ctx->node_xy.p, sh->has_rho_node ? sh->rho_node.p : nullptr, sh->rho, sh->nbr_ptr.p,
      sh->nbr_idx.p, sh->s.p);
  CGB_CUDA(cudaGetLastError());
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
