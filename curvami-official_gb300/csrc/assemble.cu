// assemble.cu — stage B on sm_103a: the Kirchhoff-Love residual and tangent of every
// face Gauss point, the elastic hinge, and their scatter into the block-upper CSC K.
//
// Reference: NonLinearAssembler::updateStiffness (plate/Assembly.h:158-345),
// Kinematics::compute (plate/Kinematics.h:61-120), Constitutive::evaluate
// (plate/Constitutive.h:57-70), Constraints::evaluateElasticFold / foldAngleAndGrad
// (plate/Constraints.h:54-119, 341-436), Meshless::assembleSystem* (plate/Meshless.h:102-127)
// and the energies (plate/Meshless.h:197-220, Constraints.h:310-339).
//
// One warp per Gauss point. Lanes first reduce the kinematic sums (r0,a and r0,ab over
// the neighbours) with shuffles, every lane then holds the point's frame a1, a2, b,
// C0^-1 and the resultants N, M. Per neighbour (lane-strided) the FP64 residual
// contribution is formed and scattered, and a record of the neighbour's factors is
// staged in shared memory. The pair loop then spreads the n(n+1)/2 blocks over the
// lanes. Each block is written in the rank-3 form
//     K_IJ = a1 (x) Y1 + a2 (x) Y2 + b (x) Y3 + geo I,
// which follows from Bm_I = a1 (x) (dx, 0, dy) + a2 (x) (0, dy, dx) in strain space,
// Bb_I = beta_I (x) b, Db_J = -(a1 c_J0 + a2 c_J1) (x) b with c_J = C0^-1 grad Phi_J:
//     Y1 = dx_I P_J0 + dy_I P_J2 - Tu_I c_J0 b
//     Y2 = dy_I P_J1 + dx_I P_J2 - Tu_I c_J1 b
//     Y3 = beta_I . Q_J - Tu_J (a1 c_I0 + a2 c_I1) + bv (dPhi_I . c_J) b
//     geo = dPhi_I . N dPhi_J,
// the same terms as K_mat + K_geo_m + T12 + T3 of Assembly.h:290-300 (70 FMA per block
// against the reference's ~90), with the Gauss weight folded into the J-side factors.
//
// Precision modes: FP64 throughout, or "mixed" (FP64 kinematics, resultants and
// residual; the per-neighbour factors and the pair loop in FP32, accumulated into an
// FP32 block array that is widened to FP64 on output).
// Scatter modes: atomics into a block array (BSR, one 3x3 block per pattern slot), or
// deterministic: every block value goes to a contribution array and a second kernel
// sums each block's contributions in ascending Gauss-point order.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>

#include "cgb_device.cuh"
#include "cgb_internal.h"
#include "cgb_umma.cuh"

namespace cgb {
namespace {

constexpr int kFaceWarps = 4;
constexpr int kRecI = 9;   // dx dy beta0 beta1 beta2 Tu g0 g1 g2
constexpr int kRecJ = 23;  // P(9) Q(9) cW0 cW1 nW0 nW1 TuW
constexpr int kRec = kRecI + kRecJ;
// Device error word bit: an index of caller-owned arrays was out of range (allocation-free
// entry point); the access was skipped.
constexpr int kErrIndex = 8;

struct Material {
  double A[9], B[9], D[9];
  // FP32 copies for the FP32 tangent: a double -> float conversion issues on the FP64 pipe,
  // which the records loop would otherwise pay for 9-27 times per record.
  float Af[9], Bf[9], Df[9];
  template <class T> __device__ __forceinline__ T Ai(int i) const { if constexpr (sizeof(T) == 4) return Af[i]; else return A[i]; }
  template <class T> __device__ __forceinline__ T Bi(int i) const { if constexpr (sizeof(T) == 4) return Bf[i]; else return B[i]; }
  template <class T> __device__ __forceinline__ T Di(int i) const { if constexpr (sizeof(T) == 4) return Df[i]; else return D[i]; }
};

inline Material make_material(const double* A, const double* B, const double* D) {
  Material m;
  for (int i = 0; i < 9; ++i) {
    m.A[i] = A[i]; m.B[i] = B[i]; m.D[i] = D[i];
    m.Af[i] = static_cast<float>(A[i]); m.Bf[i] = static_cast<float>(B[i]); m.Df[i] = static_cast<float>(D[i]);
  }
  return m;
}

struct FaceArgs {
  int n_gp;
  int g_begin, g_end;  // the Gauss points [g_begin, g_end) of this launch (multiples of 32 apart)
  int nmax;
  const int64_t* ptr;
  const int32_t* idx;
  const double* dpsi;
  const double* ddpsi;
  const void* dpsi_t;   // grad / Hessian Phi in the tangent's precision (FP32 copies in mixed mode)
  const void* ddpsi_t;
  const double* weight;
  const double* x;
  const int64_t* map_ptr;
  const int32_t* map_slot;
  const int32_t* outer;  // scalar CSC column starts (POS_MAP only)
  // POS_MAP only (caller-owned arrays): the bounds every index is checked against, and
  // the error word that records a violation (the access is skipped).
  int64_t n_blocks;
  int n_nodes;
  int* err;
  // Phase-1 copy of the neighbour data in sliced-ELL order: Gauss point 32 W + l, entry
  // q at sell_ptr[W] + 32 q + l (null: read the CSR arrays).
  const int64_t* sell_ptr;
  const int32_t* sidx;
  const double* sdpsi;
  const double* sddpsi;
  Material mat;
  NatCurv nc;               // natural curvature (inactive by default)
  const double* gp_xy;      // the points' reference coordinates (set when nc is active)
  double* F;         // atomic F (3 n_nodes)
  double* Fc;        // deterministic F contributions (3 per entry)
  void* Kacc;        // atomic block accumulator
  void* Kc;          // deterministic contributions (9 per pair)
};

// Per-point kinematics and resultants (Kinematics.h:61-120, Constitutive.h:57-70).
struct PointState {
  double a1[3], a2[3], rxx[3], ryy[3], rxy[3], b[3];
  double Ci[4];   // C0^-1 row-major
  double N[3], M[3];
  double pXY[2];
  double bv;
  double e0[3], e1[3];
  double e1el[3];  // elastic bending strain E1_el = E1 + kappa_bar (Voigt), what N and M see
};

// kappa_bar_XX of the natural-curvature band at reference X (plate/Kinematics.h:25-34).
__device__ __forceinline__ double natcurv_kappa(const NatCurv& nc, double X) {
  if (!nc.active) return 0.0;
  const double t = (X - nc.x0) / nc.width;
  return nc.amp * exp(-t * t);
}

// kbar: the natural curvature's kappa_bar_XX at the point (0 without one); it enters E1_el
// only (Kinematics.h:110-111, Constitutive.h:65).
__device__ __forceinline__ void point_state(const double s[15], const Material& m, PointState& P,
                                            double kbar = 0.0) {
  P.a1[0] = 1.0 + s[0]; P.a1[1] = s[1]; P.a1[2] = s[2];
  P.a2[0] = s[3]; P.a2[1] = 1.0 + s[4]; P.a2[2] = s[5];
#pragma unroll
  for (int c = 0; c < 3; ++c) { P.rxx[c] = s[6 + c]; P.ryy[c] = s[9 + c]; P.rxy[c] = s[12 + c]; }
  const double C00 = P.a1[0] * P.a1[0] + P.a1[1] * P.a1[1] + P.a1[2] * P.a1[2];
  const double C11 = P.a2[0] * P.a2[0] + P.a2[1] * P.a2[1] + P.a2[2] * P.a2[2];
  const double C01 = P.a1[0] * P.a2[0] + P.a1[1] * P.a2[1] + P.a1[2] * P.a2[2];
  const double det = C00 * C11 - C01 * C01;
  const double id = 1.0 / det;
  P.Ci[0] = C11 * id; P.Ci[1] = -C01 * id; P.Ci[2] = -C01 * id; P.Ci[3] = C00 * id;
  double n[3] = {P.a1[1] * P.a2[2] - P.a1[2] * P.a2[1], P.a1[2] * P.a2[0] - P.a1[0] * P.a2[2],
                 P.a1[0] * P.a2[1] - P.a1[1] * P.a2[0]};
  const double inv_area = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);   // one division, not three
#pragma unroll
  for (int c = 0; c < 3; ++c) P.b[c] = n[c] * inv_area;
  P.e0[0] = 0.5 * (C00 - 1.0);
  P.e0[1] = 0.5 * (C11 - 1.0);
  P.e0[2] = 2.0 * (0.5 * C01);
  P.e1[0] = -(P.rxx[0] * P.b[0] + P.rxx[1] * P.b[1] + P.rxx[2] * P.b[2]);
  P.e1[1] = -(P.ryy[0] * P.b[0] + P.ryy[1] * P.b[1] + P.ryy[2] * P.b[2]);
  P.e1[2] = 2.0 * -(P.rxy[0] * P.b[0] + P.rxy[1] * P.b[1] + P.rxy[2] * P.b[2]);
  P.e1el[0] = P.e1[0] + kbar; P.e1el[1] = P.e1[1]; P.e1el[2] = P.e1[2];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    P.N[r] = m.A[3 * r] * P.e0[0] + m.A[3 * r + 1] * P.e0[1] + m.A[3 * r + 2] * P.e0[2] +
             (m.B[3 * r] * P.e1el[0] + m.B[3 * r + 1] * P.e1el[1] + m.B[3 * r + 2] * P.e1el[2]);
    P.M[r] = m.B[r] * P.e0[0] + m.B[3 + r] * P.e0[1] + m.B[6 + r] * P.e0[2] +
             (m.D[3 * r] * P.e1el[0] + m.D[3 * r + 1] * P.e1el[1] + m.D[3 * r + 2] * P.e1el[2]);
  }
  double vc[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) vc[c] = P.rxx[c] * P.M[0] + 2.0 * P.rxy[c] * P.M[2] + P.ryy[c] * P.M[1];
  P.bv = P.b[0] * vc[0] + P.b[1] * vc[1] + P.b[2] * vc[2];
  const double fa = P.a1[0] * vc[0] + P.a1[1] * vc[1] + P.a1[2] * vc[2];
  const double fb = P.a2[0] * vc[0] + P.a2[1] * vc[1] + P.a2[2] * vc[2];
  P.pXY[0] = P.Ci[0] * fa + P.Ci[1] * fb;
  P.pXY[1] = P.Ci[2] * fa + P.Ci[3] * fb;
}

// Kinematic sums over the neighbours, lane-strided, reduced across the warp.
__device__ __forceinline__ void kin_sums(int lane, int64_t p0, int n, const int32_t* idx, const double* dpsi,
                                         const double* ddpsi, const double* x, double s[15]) {
#pragma unroll
  for (int k = 0; k < 15; ++k) s[k] = 0.0;
  for (int a = lane; a < n; a += 32) {
    const int64_t e = p0 + a;
    const int64_t j = idx[e];
    const double u0 = x[3 * j], u1 = x[3 * j + 1], u2 = x[3 * j + 2];
    const double2 d = reinterpret_cast<const double2*>(dpsi)[e];
    const double dxx = ddpsi[3 * e], dyy = ddpsi[3 * e + 1], dxy = ddpsi[3 * e + 2];
    s[0] += u0 * d.x; s[1] += u1 * d.x; s[2] += u2 * d.x;
    s[3] += u0 * d.y; s[4] += u1 * d.y; s[5] += u2 * d.y;
    s[6] += u0 * dxx; s[7] += u1 * dxx; s[8] += u2 * dxx;
    s[9] += u0 * dyy; s[10] += u1 * dyy; s[11] += u2 * dyy;
    s[12] += u0 * dxy; s[13] += u1 * dxy; s[14] += u2 * dxy;
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) s[k] = warp_sum(s[k]);
}

// Scatter of one block into the accumulators. v is row-major in the local (I, J)
// orientation; the stored block is (min node, max node), transposed when flipped.
template <typename TK>
__device__ __forceinline__ void scatter_atomic(void* acc, int32_t slot, bool flip, const TK v[9]);

template <>
__device__ __forceinline__ void scatter_atomic<double>(void* acc, int32_t slot, bool flip, const double v[9]) {
  double* d = static_cast<double*>(acc) + 9 * static_cast<int64_t>(slot);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(d + 3 * r + c, flip ? v[3 * c + r] : v[3 * r + c]);
}

template <>
__device__ __forceinline__ void scatter_atomic<float>(void* acc, int32_t slot, bool flip, const float v[9]) {
  // 12 floats per block: three 16-byte vector atomics.
  float4* d = reinterpret_cast<float4*>(static_cast<float*>(acc) + 12 * static_cast<int64_t>(slot));
  float t[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) t[3 * r + c] = flip ? v[3 * c + r] : v[3 * r + c];
  atomicAdd(d, make_float4(t[0], t[1], t[2], t[3]));
  atomicAdd(d + 1, make_float4(t[4], t[5], t[6], t[7]));
  atomicAdd(d + 2, make_float4(t[8], 0.0f, 0.0f, 0.0f));
}

template <typename TK>
__device__ __forceinline__ void store_contrib(void* cbuf, int64_t q, bool flip, const TK v[9]) {
  TK* d = static_cast<TK*>(cbuf) + 9 * q;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) d[3 * r + c] = flip ? v[3 * c + r] : v[3 * r + c];
}

// Per-point state handed from the FP64 phase to the pair phase, [field][32] in shared
// memory: a1(3) a2(3) b(3) r0XX(3) r0YY(3) r0XY(3) C0^-1(4) N(3) M(3) pXY(2) bv W.
constexpr int kState = 32;
enum : int { S_A1 = 0, S_A2 = 3, S_B = 6, S_RXX = 9, S_RYY = 12, S_RXY = 15, S_CI = 18, S_N = 22,
             S_M = 25, S_P = 28, S_BV = 30, S_W = 31 };

// TIN: element type of the grad / Hessian Phi arrays the pair phase reads (TK, or FP64
// read and rounded in the kernel). POS_MAP: map_slot holds the reference's csrMapping
// positions and the block slot is outer[3 max(ni, nj)] / 9 + position.
// BZERO: the laminate coupling matrix B is zero (every symmetric laminate, and the
// single isotropic ply of the reference's app, whose B = Q (z1^2 - z0^2) / 2 is exactly
// 0). Then P = A Bm = a1 (x) pa + a2 (x) pb and Q = D Bb = b (x) qc, and the J-side
// record shrinks from 23 to 14 values.
// Phase 1 for the Gauss point g0 + lane (g0 a multiple of 32): FP64 kinematics,
// resultants and residual (F atomics, or per-entry contributions when DET); when st is
// not null the point's state goes to st[field * st_stride + st_idx] in TK.
// CHECK (caller-owned arrays only): a neighbour id outside [0, n_nodes) is flagged in the
// error word and the neighbour is left out.
template <typename TK, bool DET, bool CHECK = false>
__device__ __forceinline__ void phase1_point(const FaceArgs& a, int g0, int lane, TK* st, int64_t st_stride,
                                             int64_t st_idx) {
  const Material& m = a.mat;
  const int g = g0 + lane;
  if (g < a.g_end) {
      const int64_t p0 = a.ptr[g];
      const int n = static_cast<int>(a.ptr[g + 1] - p0);
      // Entry q of this lane's point: CSR p0 + q, or sliced-ELL sb + 32 q (coalesced
      // across the warp: the 32 lanes read 32 consecutive entries per q).
      const bool sell = a.sell_ptr != nullptr;
      const int64_t sb = sell ? a.sell_ptr[g0 >> 5] + lane : p0;
      const int64_t stride = sell ? 32 : 1;
      const int32_t* Ix = sell ? a.sidx : a.idx;
      const double* Dp = sell ? a.sdpsi : a.dpsi;
      const double* Ddp = sell ? a.sddpsi : a.ddpsi;
      double s[15];
#pragma unroll
      for (int k = 0; k < 15; ++k) s[k] = 0.0;
#pragma unroll 4
      for (int q = 0; q < n; ++q) {
        const int64_t e = sb + q * stride;
        const int64_t j = Ix[e];
        if (CHECK && (j < 0 || j >= a.n_nodes)) {
          atomicOr(a.err, kErrIndex);
          continue;
        }
        const double u0 = a.x[3 * j], u1 = a.x[3 * j + 1], u2 = a.x[3 * j + 2];
        const double2 d = reinterpret_cast<const double2*>(Dp)[e];
        const double dxx = Ddp[3 * e], dyy = Ddp[3 * e + 1], dxy = Ddp[3 * e + 2];
        s[0] += u0 * d.x; s[1] += u1 * d.x; s[2] += u2 * d.x;
        s[3] += u0 * d.y; s[4] += u1 * d.y; s[5] += u2 * d.y;
        s[6] += u0 * dxx; s[7] += u1 * dxx; s[8] += u2 * dxx;
        s[9] += u0 * dyy; s[10] += u1 * dyy; s[11] += u2 * dyy;
        s[12] += u0 * dxy; s[13] += u1 * dxy; s[14] += u2 * dxy;
      }
      PointState P;
      point_state(s, m, P, a.gp_xy ? natcurv_kappa(a.nc, a.gp_xy[2 * static_cast<int64_t>(g)]) : 0.0);
      const double W = a.weight[g];
      // The state the tangent needs goes out first, so that only the residual's coefficients
      // stay live through the neighbour loop.
      if (st) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          st[(S_A1 + c) * st_stride + st_idx] = static_cast<TK>(P.a1[c]);
          st[(S_A2 + c) * st_stride + st_idx] = static_cast<TK>(P.a2[c]);
          st[(S_B + c) * st_stride + st_idx] = static_cast<TK>(P.b[c]);
          st[(S_RXX + c) * st_stride + st_idx] = static_cast<TK>(P.rxx[c]);
          st[(S_RYY + c) * st_stride + st_idx] = static_cast<TK>(P.ryy[c]);
          st[(S_RXY + c) * st_stride + st_idx] = static_cast<TK>(P.rxy[c]);
          st[(S_N + c) * st_stride + st_idx] = static_cast<TK>(P.N[c]);
          st[(S_M + c) * st_stride + st_idx] = static_cast<TK>(P.M[c]);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) st[(S_CI + c) * st_stride + st_idx] = static_cast<TK>(P.Ci[c]);
        st[(S_P + 0) * st_stride + st_idx] = static_cast<TK>(P.pXY[0]);
        st[(S_P + 1) * st_stride + st_idx] = static_cast<TK>(P.pXY[1]);
        st[S_BV * st_stride + st_idx] = static_cast<TK>(P.bv);
        st[S_W * st_stride + st_idx] = static_cast<TK>(W);
      }
      // f_I = W (Bm_I^T N + Bb_I^T M) (Assembly.h:249) = W (a1 u1 + a2 u2 + b Tu_I), since
      // beta_I . M = dPhi_I . pXY - (Phi_XX M0 + 2 Phi_XY M2 + Phi_YY M1) = Tu_I, with
      // u1 = Phi_X N0 + Phi_Y N2 and u2 = Phi_Y N1 + Phi_X N2. It is linear in the five
      // derivatives of Phi_I, so per point f_I[c] = Gx[c] Phi_X + Gy[c] Phi_Y + Hxx[c] Phi_XX +
      // Hyy[c] Phi_YY + Hxy[c] Phi_XY: five FP64 FMAs per component and neighbour (GB300's
      // FP64 pipe bounds this kernel).
      double Gx[3], Gy[3], Hxx[3], Hyy[3], Hxy[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Gx[c] = W * (P.a1[c] * P.N[0] + P.a2[c] * P.N[2] + P.b[c] * P.pXY[0]);
        Gy[c] = W * (P.a1[c] * P.N[2] + P.a2[c] * P.N[1] + P.b[c] * P.pXY[1]);
        Hxx[c] = -W * P.b[c] * P.M[0];
        Hyy[c] = -W * P.b[c] * P.M[1];
        Hxy[c] = -2.0 * W * P.b[c] * P.M[2];
      }
      if (n > 0) {
#pragma unroll 2
        for (int q = 0; q < n; ++q) {
          const int64_t es = sb + q * stride;
          const int64_t e = p0 + q;
          const double2 d = reinterpret_cast<const double2*>(Dp)[es];
          const double dxx = Ddp[3 * es], dyy = Ddp[3 * es + 1], dxy = Ddp[3 * es + 2];
          double f[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) f[c] = Gx[c] * d.x + Gy[c] * d.y + Hxx[c] * dxx + Hyy[c] * dyy + Hxy[c] * dxy;
          if (DET) {
#pragma unroll
            for (int c = 0; c < 3; ++c) a.Fc[3 * e + c] = f[c];
          } else {
            const int64_t node = Ix[es];
            if (CHECK && (node < 0 || node >= a.n_nodes)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) atomicAdd(a.F + 3 * node + c, f[c]);
          }
        }
      }
    }
}

// Phase 2 for the Gauss points g0 .. g0 + 31 across the warp, in the tangent's precision:
// per-neighbour records in shared memory, then the pair loop and the scatter. st holds
// the 32 points' states as [field][32].
template <typename TK, bool DET, typename TIN, bool POS_MAP, bool BZERO>
__device__ __forceinline__ void phase2_group(const FaceArgs& a, int g0, int lane, const TK* st, TK* rec, int* nid) {
  const Material& m = a.mat;
  const int nmax = a.nmax;
  const TIN* dpsi_t = static_cast<const TIN*>(a.dpsi_t);
  const TIN* ddpsi_t = static_cast<const TIN*>(a.ddpsi_t);
  const int kend = min(32, a.g_end - g0);
  for (int k = 0; k < kend; ++k) {
    const int gg = g0 + k;
    const int64_t p0 = a.ptr[gg];
    const int n = static_cast<int>(a.ptr[gg + 1] - p0);
    if (n == 0) continue;  // Assembly.h:208
    if (POS_MAP && n > nmax) {  // the records are staged for nmax neighbours
      if (lane == 0) atomicOr(a.err, kErrIndex);
      continue;
    }
    TK a1t[3], a2t[3], bt[3], rxx[3], ryy[3], rxy[3], Nt[3], Mt[3], Ci[4];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      a1t[c] = st[(S_A1 + c) * 32 + k]; a2t[c] = st[(S_A2 + c) * 32 + k]; bt[c] = st[(S_B + c) * 32 + k];
      rxx[c] = st[(S_RXX + c) * 32 + k]; ryy[c] = st[(S_RYY + c) * 32 + k]; rxy[c] = st[(S_RXY + c) * 32 + k];
      Nt[c] = st[(S_N + c) * 32 + k]; Mt[c] = st[(S_M + c) * 32 + k];
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) Ci[c] = st[(S_CI + c) * 32 + k];
    const TK pX = st[S_P * 32 + k], pY = st[(S_P + 1) * 32 + k];
    const TK bv = st[S_BV * 32 + k], Wt = st[S_W * 32 + k];

    // Records of the neighbours (lane per neighbour).
    for (int i = lane; i < n; i += 32) {
      const int64_t e = p0 + i;
      const TK dx = static_cast<TK>(dpsi_t[2 * e]), dy = static_cast<TK>(dpsi_t[2 * e + 1]);
      const TK dxx = static_cast<TK>(ddpsi_t[3 * e]), dyy = static_cast<TK>(ddpsi_t[3 * e + 1]);
      const TK dxy = static_cast<TK>(ddpsi_t[3 * e + 2]);
      const TK c0 = Ci[0] * dx + Ci[1] * dy;
      const TK c1 = Ci[2] * dx + Ci[3] * dy;
      TK gI[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) gI[r] = a1t[r] * c0 + a2t[r] * c1;
      const TK b0 = -dxx + (rxx[0] * gI[0] + rxx[1] * gI[1] + rxx[2] * gI[2]);
      const TK b1 = -dyy + (ryy[0] * gI[0] + ryy[1] * gI[1] + ryy[2] * gI[2]);
      const TK b2 = TK(2) * (-dxy + (rxy[0] * gI[0] + rxy[1] * gI[1] + rxy[2] * gI[2]));
      const TK Tu = dx * pX + dy * pY - (dxx * Mt[0] + TK(2) * dxy * Mt[2] + dyy * Mt[1]);
      TK* R = rec + i;
      R[0 * nmax] = dx; R[1 * nmax] = dy;
      R[2 * nmax] = b0; R[3 * nmax] = b1; R[4 * nmax] = b2;
      R[5 * nmax] = Tu;
#pragma unroll
      for (int r = 0; r < 3; ++r) R[(6 + r) * nmax] = gI[r];
      if constexpr (BZERO) {
        // J side: pa(3) pb(3) qc(3) cW(2) nW(2) TuW, all times W.
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const TK Ar0 = m.Ai<TK>(3 * r), Ar1 = m.Ai<TK>(3 * r + 1), Ar2 = m.Ai<TK>(3 * r + 2);
          const TK Dr0 = m.Di<TK>(3 * r), Dr1 = m.Di<TK>(3 * r + 1), Dr2 = m.Di<TK>(3 * r + 2);
          R[(kRecI + r) * nmax] = (Ar0 * dx + Ar2 * dy) * Wt;
          R[(kRecI + 3 + r) * nmax] = (Ar1 * dy + Ar2 * dx) * Wt;
          R[(kRecI + 6 + r) * nmax] = (Dr0 * b0 + Dr1 * b1 + Dr2 * b2) * Wt;
        }
        R[(kRecI + 9) * nmax] = c0 * Wt;
        R[(kRecI + 10) * nmax] = c1 * Wt;
        R[(kRecI + 11) * nmax] = (Nt[0] * dx + Nt[2] * dy) * Wt;
        R[(kRecI + 12) * nmax] = (Nt[2] * dx + Nt[1] * dy) * Wt;
        R[(kRecI + 13) * nmax] = Tu * Wt;
      } else {
      // P = A Bm + B Bb, Q = B Bm + D Bb (Assembly.h:255-256), times W:
      //   P(r,c) = a1_c pa_r + a2_c pb_r + b_c pc_r.
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const TK Ar0 = m.Ai<TK>(3 * r), Ar1 = m.Ai<TK>(3 * r + 1), Ar2 = m.Ai<TK>(3 * r + 2);
        const TK Br0 = m.Bi<TK>(3 * r), Br1 = m.Bi<TK>(3 * r + 1), Br2 = m.Bi<TK>(3 * r + 2);
        const TK Dr0 = m.Di<TK>(3 * r), Dr1 = m.Di<TK>(3 * r + 1), Dr2 = m.Di<TK>(3 * r + 2);
        const TK pa = (Ar0 * dx + Ar2 * dy) * Wt;
        const TK pb = (Ar1 * dy + Ar2 * dx) * Wt;
        const TK pc = (Br0 * b0 + Br1 * b1 + Br2 * b2) * Wt;
        const TK qa = (Br0 * dx + Br2 * dy) * Wt;
        const TK qb = (Br1 * dy + Br2 * dx) * Wt;
        const TK qc = (Dr0 * b0 + Dr1 * b1 + Dr2 * b2) * Wt;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          R[(kRecI + 3 * r + c) * nmax] = a1t[c] * pa + a2t[c] * pb + bt[c] * pc;
          R[(kRecI + 9 + 3 * r + c) * nmax] = a1t[c] * qa + a2t[c] * qb + bt[c] * qc;
        }
      }
      R[(kRecI + 18) * nmax] = c0 * Wt;
      R[(kRecI + 19) * nmax] = c1 * Wt;
      R[(kRecI + 20) * nmax] = (Nt[0] * dx + Nt[2] * dy) * Wt;
      R[(kRecI + 21) * nmax] = (Nt[2] * dx + Nt[1] * dy) * Wt;
      R[(kRecI + 22) * nmax] = Tu * Wt;
      }
      nid[i] = a.idx[e];
    }
    __syncwarp();

    // Pair loop: the n(n+1)/2 blocks of this point spread over the lanes.
    const int64_t np = static_cast<int64_t>(n) * (n + 1) / 2;
    const int64_t m0 = a.map_ptr[gg];
    int i = 0, off = lane;
    while (i < n && off >= n - i) { off -= n - i; ++i; }
    for (int64_t p = lane; p < np; p += 32) {
      const int j = i + off;
      const TK* RI = rec + i;
      const TK* RJ = rec + j;
      const TK dxi = RI[0], dyi = RI[nmax], be0 = RI[2 * nmax], be1 = RI[3 * nmax], be2 = RI[4 * nmax];
      const TK Tui = RI[5 * nmax], gi0 = RI[6 * nmax], gi1 = RI[7 * nmax], gi2 = RI[8 * nmax];
      TK v[9];
      if constexpr (BZERO) {
        const TK pa0 = RJ[kRecI * nmax], pa1 = RJ[(kRecI + 1) * nmax], pa2 = RJ[(kRecI + 2) * nmax];
        const TK pb0 = RJ[(kRecI + 3) * nmax], pb1 = RJ[(kRecI + 4) * nmax], pb2 = RJ[(kRecI + 5) * nmax];
        const TK qc0 = RJ[(kRecI + 6) * nmax], qc1 = RJ[(kRecI + 7) * nmax], qc2 = RJ[(kRecI + 8) * nmax];
        const TK cj0 = RJ[(kRecI + 9) * nmax], cj1 = RJ[(kRecI + 10) * nmax];
        const TK nj0 = RJ[(kRecI + 11) * nmax], nj1 = RJ[(kRecI + 12) * nmax];
        const TK TuWj = RJ[(kRecI + 13) * nmax];
        const TK s1 = Tui * cj0, s2 = Tui * cj1;
        const TK geo = dxi * nj0 + dyi * nj1;
        const TK z11 = dxi * pa0 + dyi * pa2, z12 = dxi * pb0 + dyi * pb2;
        const TK z21 = dyi * pa1 + dxi * pa2, z22 = dyi * pb1 + dxi * pb2;
        const TK z33 = be0 * qc0 + be1 * qc1 + be2 * qc2 + bv * (dxi * cj0 + dyi * cj1);
        TK Y1[3], Y2[3], Y3[3];
        const TK gi[3] = {gi0, gi1, gi2};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          Y1[c] = a1t[c] * z11 + a2t[c] * z12 - s1 * bt[c];
          Y2[c] = a1t[c] * z21 + a2t[c] * z22 - s2 * bt[c];
          Y3[c] = bt[c] * z33 - TuWj * gi[c];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            v[3 * r + c] = a1t[r] * Y1[c] + a2t[r] * Y2[c] + bt[r] * Y3[c] + (r == c ? geo : TK(0));
      } else {
      const TK cj0 = RJ[(kRecI + 18) * nmax], cj1 = RJ[(kRecI + 19) * nmax];
      const TK nj0 = RJ[(kRecI + 20) * nmax], nj1 = RJ[(kRecI + 21) * nmax];
      const TK TuWj = RJ[(kRecI + 22) * nmax];
      const TK s1 = Tui * cj0, s2 = Tui * cj1;
      const TK t3 = bv * (dxi * cj0 + dyi * cj1);
      const TK geo = dxi * nj0 + dyi * nj1;
      TK Y1[3], Y2[3], Y3[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const TK P0 = RJ[(kRecI + c) * nmax], P1 = RJ[(kRecI + 3 + c) * nmax], P2 = RJ[(kRecI + 6 + c) * nmax];
        const TK Q0 = RJ[(kRecI + 9 + c) * nmax], Q1 = RJ[(kRecI + 12 + c) * nmax], Q2 = RJ[(kRecI + 15 + c) * nmax];
        const TK gic = c == 0 ? gi0 : (c == 1 ? gi1 : gi2);
        Y1[c] = dxi * P0 + dyi * P2 - s1 * bt[c];
        Y2[c] = dyi * P1 + dxi * P2 - s2 * bt[c];
        Y3[c] = be0 * Q0 + be1 * Q1 + be2 * Q2 + t3 * bt[c] - TuWj * gic;
      }
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          v[3 * r + c] = a1t[r] * Y1[c] + a2t[r] * Y2[c] + bt[r] * Y3[c] + (r == c ? geo : TK(0));
      }
      const bool flip = nid[i] > nid[j];
      if (DET) {
        store_contrib<TK>(a.Kc, m0 + p, flip, v);
      } else if (POS_MAP) {
        const int hi = flip ? nid[i] : nid[j];
        const int64_t slot = hi >= 0 && hi < a.n_nodes
                                 ? a.outer[3 * static_cast<int64_t>(hi)] / 9 + a.map_slot[m0 + p] : -1;
        if (slot >= 0 && slot < a.n_blocks) scatter_atomic<TK>(a.Kacc, static_cast<int32_t>(slot), flip, v);
        else atomicOr(a.err, kErrIndex);
      } else {
        scatter_atomic<TK>(a.Kacc, a.map_slot[m0 + p], flip, v);
      }
      off += 32;
      while (i < n && off >= n - i) { off -= n - i; ++i; }
    }
    __syncwarp();
  }
}

template <typename TK, bool DET, bool WANT_K, typename TIN = TK, bool POS_MAP = false, bool BZERO = false>
__global__ void __launch_bounds__(32 * kFaceWarps, sizeof(TK) == 4 ? 5 : 3) face_kernel(FaceArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nmax = a.nmax;
  TK* base_w = reinterpret_cast<TK*>(smem_raw) + static_cast<size_t>(w) * (kState * 32 + kRec * nmax);
  TK* st = base_w;                 // [kState][32]
  TK* rec = base_w + kState * 32;  // [kRec][nmax]
  int* nid = reinterpret_cast<int*>(reinterpret_cast<TK*>(smem_raw) +
                                    static_cast<size_t>(kFaceWarps) * (kState * 32 + kRec * nmax)) + w * nmax;
  // Each warp owns 32 consecutive Gauss points per round.
  for (int g0 = (blockIdx.x * kFaceWarps + w) * 32; g0 < a.n_gp; g0 += gridDim.x * kFaceWarps * 32) {
    // Phase 1: one Gauss point per lane, FP64. Every lane does distinct work, so no FP64
    // issue slot is spent on a redundant or masked copy (on GB300 an FP64 warp
    // instruction costs the same with 1 or 32 lanes).
    phase1_point<TK, DET, POS_MAP>(a, g0, lane, WANT_K ? st : static_cast<TK*>(nullptr), 32, lane);
    if (!WANT_K) continue;
    __syncwarp();
    phase2_group<TK, DET, TIN, POS_MAP, BZERO>(a, g0, lane, st, rec, nid);
  }
}

// The same work as two kernels, each sized for its own occupancy: the residual kernel
// (phase 1, one Gauss point per thread, FP64 bound) writes the per-point state to
// global memory ([field][n_gp]); the tangent kernel (phase 2) stages 32 points' states
// in shared memory and runs the pair loop.
// Work is handed out 32 points at a time from a counter (zeroed per assembly), so the
// warps of a launch finish together whatever the grid: when the tangent kernel of the
// previous chunk holds most of each SM, only one residual CTA fits beside it, and a
// fixed split into CTAs would leave a partial last wave.
template <typename TK, bool DET, bool STORE>
__global__ void __launch_bounds__(256) face_residual_kernel(FaceArgs a, TK* gstate, int* __restrict__ work) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    int unit = 0;
    if (lane == 0) unit = atomicAdd(work, 1);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    const int64_t g0 = a.g_begin + 32 * static_cast<int64_t>(unit);
    if (g0 >= a.g_end) break;
    phase1_point<TK, DET>(a, static_cast<int>(g0), lane, STORE ? gstate : static_cast<TK*>(nullptr), a.n_gp,
                          g0 + lane);
  }
}

constexpr int kTanWarps = 4;

template <typename TK, bool DET, bool BZERO>
__global__ void __launch_bounds__(32 * kTanWarps) face_tangent_kernel(FaceArgs a, const TK* __restrict__ gstate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nmax = a.nmax;
  TK* base_w = reinterpret_cast<TK*>(smem_raw) + static_cast<size_t>(w) * (kState * 32 + kRec * nmax);
  TK* st = base_w;
  TK* rec = base_w + kState * 32;
  int* nid = reinterpret_cast<int*>(reinterpret_cast<TK*>(smem_raw) +
                                    static_cast<size_t>(kTanWarps) * (kState * 32 + kRec * nmax)) + w * nmax;
  for (int g0 = a.g_begin + (blockIdx.x * kTanWarps + w) * 32; g0 < a.g_end; g0 += gridDim.x * kTanWarps * 32) {
    const int g = g0 + lane;
#pragma unroll 4
    for (int f = 0; f < kState; ++f) st[f * 32 + lane] = g < a.g_end ? gstate[static_cast<int64_t>(f) * a.n_gp + g] : TK(0);
    __syncwarp();
    phase2_group<TK, DET, TK, false, BZERO>(a, g0, lane, st, rec, nid);
  }
}

// ---- hinge (FP64) -----------------------------------------------------------------

struct HingeArgs {
  int n_gp;
  int max_u;
  const int64_t* lptr; const int32_t* lidx; const double* ldpsi;
  const int64_t* rptr; const int32_t* ridx; const double* rdpsi;
  const double* weight; const double* tangent;
  double Kt, theta0;
  const double* theta0_gp; const int8_t* active;
  const int64_t* u_ptr; const int32_t* u_node; const int32_t* l_pos; const int32_t* r_pos;
  const int64_t* pair_ptr; const int32_t* pair_slot;
  const double* x;
  int exact;
  int want_K;
  int tk_float;      // accumulator type
  double* F; void* Kacc;              // atomic mode
  double* Fc; void* Kc;               // deterministic mode
  int64_t f_base, k_base;             // contribution id offsets of this fold
};

__device__ __forceinline__ void cross(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Constraints::foldAngleAndGrad (plate/Constraints.h:54-119).
__device__ double fold_angle(const double* F, double tx, double ty, double* grad) {
  const double *a1L = F, *a2L = F + 3, *a1R = F + 6, *a2R = F + 9;
  double nL[3], nR[3];
  cross(a1L, a2L, nL); cross(a1R, a2R, nR);
  const double normL = sqrt(dot(nL, nL)), normR = sqrt(dot(nR, nR));
  double bL[3], bR[3], aT[3], t[3];
  for (int c = 0; c < 3; ++c) { bL[c] = nL[c] / normL; bR[c] = nR[c] / normR; aT[c] = a1L[c] * tx + a2L[c] * ty; }
  const double naT = sqrt(dot(aT, aT));
  for (int c = 0; c < 3; ++c) t[c] = aT[c] / naT;
  const double cth = dot(bL, bR);
  double bxb[3];
  cross(bL, bR, bxb);
  const double sth = dot(bxb, t);
  const double theta = atan2(-sth, cth);
  if (grad) {
    double dbL[3][6], dbR[3][6];
    for (int side = 0; side < 2; ++side) {
      const double* a1 = side ? a1R : a1L;
      const double* a2 = side ? a2R : a2L;
      const double* b = side ? bR : bL;
      const double nn = side ? normR : normL;
      double (*out)[6] = side ? dbR : dbL;
      double dn[3][6];
      for (int i = 0; i < 3; ++i) {
        double e[3] = {0, 0, 0};
        e[i] = 1.0;
        double c1[3], c2[3];
        cross(e, a2, c1); cross(a1, e, c2);
        for (int r = 0; r < 3; ++r) { dn[r][i] = c1[r]; dn[r][i + 3] = c2[r]; }
      }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 6; ++c) {
          double acc = 0.0;
          for (int k = 0; k < 3; ++k) acc += (((r == k) ? 1.0 : 0.0) - b[r] * b[k]) / nn * dn[k][c];
          out[r][c] = acc;
        }
    }
    double dt[3][6];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 6; ++c) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) {
          const double daT = (c < 3) ? ((c == k) ? tx : 0.0) : ((c - 3 == k) ? ty : 0.0);
          acc += (((r == k) ? 1.0 : 0.0) - t[r] * t[k]) / naT * daT;
        }
        dt[r][c] = acc;
      }
    double bRxt[3], txbL[3];
    cross(bR, t, bRxt); cross(t, bL, txbL);
    const double denom = cth * cth + sth * sth;
    const double inv = (denom > 1e-14) ? 1.0 / denom : 0.0;
    for (int c = 0; c < 6; ++c) {
      const double dcL = bR[0] * dbL[0][c] + bR[1] * dbL[1][c] + bR[2] * dbL[2][c];
      const double dcR = bL[0] * dbR[0][c] + bL[1] * dbR[1][c] + bL[2] * dbR[2][c];
      const double dsL = (bRxt[0] * dbL[0][c] + bRxt[1] * dbL[1][c] + bRxt[2] * dbL[2][c]) +
                         (bxb[0] * dt[0][c] + bxb[1] * dt[1][c] + bxb[2] * dt[2][c]);
      const double dsR = txbL[0] * dbR[0][c] + txbL[1] * dbR[1][c] + txbL[2] * dbR[2][c];
      grad[c] = -(cth * dsL - sth * dcL) * inv;
      grad[6 + c] = -(cth * dsR - sth * dcR) * inv;
    }
  }
  return theta;
}

constexpr int kHingeWarps = 2;

// One warp per crease Gauss point (Constraints.h:349-435). The left and right
// entries are merged per node: with G_u = sum of the dof gradients of node u over both
// sides, the reference's triplets (all k, m with node_k <= node_m) sum to
// W Kt G_P (x) G_Q (+ W moment B_P^T H B_Q) on block (P, Q) of the merged list.
__global__ void __launch_bounds__(32 * kHingeWarps) hinge_kernel(HingeArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Per warp: G[3*max_u], Bsum[4*max_u], H[144] (+16 spare).
  double* base = reinterpret_cast<double*>(smem_raw) + static_cast<size_t>(w) * (7 * a.max_u + 144 + 16);
  double* G = base;
  double* Bs = base + 3 * a.max_u;
  double* H = base + 7 * a.max_u;
  for (int g = blockIdx.x * kHingeWarps + w; g < a.n_gp; g += gridDim.x * kHingeWarps) {
    if (a.active && a.active[g] == 0) continue;  // Constraints.h:350
    double sL[6] = {0, 0, 0, 0, 0, 0}, sR[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t e = a.lptr[g] + lane; e < a.lptr[g + 1]; e += 32) {
      const int64_t j = a.lidx[e];
      const double dX = a.ldpsi[2 * e], dY = a.ldpsi[2 * e + 1];
      for (int c = 0; c < 3; ++c) { sL[c] += a.x[3 * j + c] * dX; sL[3 + c] += a.x[3 * j + c] * dY; }
    }
    for (int64_t e = a.rptr[g] + lane; e < a.rptr[g + 1]; e += 32) {
      const int64_t j = a.ridx[e];
      const double dX = a.rdpsi[2 * e], dY = a.rdpsi[2 * e + 1];
      for (int c = 0; c < 3; ++c) { sR[c] += a.x[3 * j + c] * dX; sR[3 + c] += a.x[3 * j + c] * dY; }
    }
    double F12[12];
    for (int k = 0; k < 6; ++k) { F12[k] = warp_sum(sL[k]); F12[6 + k] = warp_sum(sR[k]); }
    F12[0] += 1.0; F12[4] += 1.0; F12[6] += 1.0; F12[10] += 1.0;
    const double tx = a.tangent[2 * g], ty = a.tangent[2 * g + 1];
    double grad[12];
    const double theta = fold_angle(F12, tx, ty, grad);
    const double th0 = a.theta0_gp ? a.theta0_gp[g] : a.theta0;
    const double W = a.weight[g];
    const double Wm = W * (a.Kt * (theta - th0));
    const double WK = W * a.Kt;
    const bool use_hess = a.exact && a.want_K && fabs(Wm) > 0.0;
    if (use_hess) {
      // Central differences of the analytic gradient (Constraints.h:402-413), one
      // perturbed evaluation per lane (24 lanes), then symmetrised.
      double mx = 0.0;
      for (int k = 0; k < 12; ++k) mx = fmax(mx, fabs(F12[k]));
      const double hs = 1e-6 * fmax(1.0, mx);
      if (lane < 24) {
        const int k = lane >> 1;
        double Fp[12];
        for (int q = 0; q < 12; ++q) Fp[q] = F12[q];
        Fp[k] += (lane & 1) ? -hs : hs;
        double gp[12];
        fold_angle(Fp, tx, ty, gp);
        // H[r][k] = (g+ - g-)/(2h): the '+' lane stores g+, the '-' lane subtracts it.
        if ((lane & 1) == 0) for (int r = 0; r < 12; ++r) H[r * 12 + k] = gp[r];
        __syncwarp(0x00ffffffu);
        if (lane & 1) for (int r = 0; r < 12; ++r) H[r * 12 + k] = (H[r * 12 + k] - gp[r]) / (2.0 * hs);
      }
      __syncwarp();
      if (lane < 12) {
        double row[12];
        for (int c = 0; c < 12; ++c) row[c] = 0.5 * (H[lane * 12 + c] + H[c * 12 + lane]);
        __syncwarp(0x00000fffu);
        for (int c = 0; c < 12; ++c) H[lane * 12 + c] = row[c];
      }
      __syncwarp();
    }
    // Per merged node: G_u (3) and the summed (dX, dY) of each side (4).
    const int64_t u0 = a.u_ptr[g];
    const int mu = static_cast<int>(a.u_ptr[g + 1] - u0);
    for (int u = lane; u < mu; u += 32) {
      G[3 * u] = 0.0; G[3 * u + 1] = 0.0; G[3 * u + 2] = 0.0;
      Bs[4 * u] = 0.0; Bs[4 * u + 1] = 0.0; Bs[4 * u + 2] = 0.0; Bs[4 * u + 3] = 0.0;
    }
    __syncwarp();
    // Left then right: within a side every node occurs once, so no two lanes collide.
    for (int64_t e = a.lptr[g] + lane; e < a.lptr[g + 1]; e += 32) {
      const int u = a.l_pos[e];
      const double dX = a.ldpsi[2 * e], dY = a.ldpsi[2 * e + 1];
      for (int d = 0; d < 3; ++d) G[3 * u + d] += grad[d] * dX + grad[d + 3] * dY;
      Bs[4 * u] += dX; Bs[4 * u + 1] += dY;
    }
    __syncwarp();
    for (int64_t e = a.rptr[g] + lane; e < a.rptr[g + 1]; e += 32) {
      const int u = a.r_pos[e];
      const double dX = a.rdpsi[2 * e], dY = a.rdpsi[2 * e + 1];
      for (int d = 0; d < 3; ++d) G[3 * u + d] += grad[6 + d] * dX + grad[9 + d] * dY;
      Bs[4 * u + 2] += dX; Bs[4 * u + 3] += dY;
    }
    __syncwarp();
    for (int u = lane; u < mu; u += 32) {
      const int node = a.u_node[u0 + u];
      for (int d = 0; d < 3; ++d) {
        const double f = G[3 * u + d] * Wm;
        if (a.Fc) a.Fc[3 * (a.f_base + u0 + u) + d] = f;
        else atomicAdd(a.F + 3 * static_cast<int64_t>(node) + d, f);
      }
    }
    if (a.want_K) {
      const int64_t np = static_cast<int64_t>(mu) * (mu + 1) / 2;
      const int64_t q0 = a.pair_ptr[g];
      int P = 0, off = lane;
      while (P < mu && off >= mu - P) { off -= mu - P; ++P; }
      for (int64_t p = lane; p < np; p += 32) {
        const int Q = P + off;
        double v[9];
        for (int dk = 0; dk < 3; ++dk)
          for (int dm = 0; dm < 3; ++dm) {
            double val = WK * (G[3 * P + dk] * G[3 * Q + dm]);
            if (use_hess) {
              // B_P(dk) has dX_L at dk, dY_L at dk+3, dX_R at 6+dk, dY_R at 9+dk.
              const int ik[4] = {dk, dk + 3, 6 + dk, 9 + dk};
              const int im[4] = {dm, dm + 3, 6 + dm, 9 + dm};
              double hb = 0.0;
              for (int s1 = 0; s1 < 4; ++s1) {
                double row = 0.0;
                for (int s2 = 0; s2 < 4; ++s2) row += H[ik[s1] * 12 + im[s2]] * Bs[4 * Q + s2];
                hb += Bs[4 * P + s1] * row;
              }
              val += Wm * hb;
            }
            v[3 * dk + dm] = val;
          }
        if (a.Kc) {
          if (a.tk_float) { float t[9]; for (int k = 0; k < 9; ++k) t[k] = static_cast<float>(v[k]); store_contrib<float>(a.Kc, a.k_base + q0 + p, false, t); }
          else store_contrib<double>(a.Kc, a.k_base + q0 + p, false, v);
        } else {
          const int32_t slot = a.pair_slot[q0 + p];
          if (a.tk_float) { float t[9]; for (int k = 0; k < 9; ++k) t[k] = static_cast<float>(v[k]); scatter_atomic<float>(a.Kacc, slot, false, t); }
          else scatter_atomic<double>(a.Kacc, slot, false, v);
        }
        off += 32;
        while (P < mu && off >= mu - P) { off -= mu - P; ++P; }
      }
    }
    __syncwarp();
  }
}

// ---- output: blocks -> the reference's CSC -------------------------------------------
// Column node j holds len_j block rows; scalar column 3j+c starts at 9 col_ptr[j] +
// 3 c len_j and lists rows 3i+r for the block rows i ascending (Assembly.h:103-107).
template <typename TA, int STRIDE>
__global__ void blocks_to_csc(int n_nodes, const int64_t* __restrict__ col_ptr, const TA* __restrict__ acc,
                              double* __restrict__ K) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t j = warp; j < n_nodes; j += nw) {
    const int64_t b0 = col_ptr[j];
    const int len = static_cast<int>(col_ptr[j + 1] - b0);
    double* col = K + 9 * b0;
    for (int t = lane; t < 9 * len; t += 32) {
      // t enumerates the column's output in storage order: c major, then (pos, r).
      const int c = t / (3 * len), rem = t - c * 3 * len, pos = rem / 3, r = rem - 3 * pos;
      col[t] = static_cast<double>(acc[(b0 + pos) * STRIDE + 3 * r + c]);
    }
  }
}

// The same output step with the block columns taken from the scalar CSC outer index:
// column node j starts at block outer[3j] / 9 and holds (outer[3j+1] - outer[3j]) / 3 blocks.
// A column whose blocks would fall outside [0, n_blocks) is skipped and flagged.
template <typename TA, int STRIDE>
__global__ void blocks_to_csc_outer(int n_nodes, int64_t n_blocks, const int32_t* __restrict__ outer,
                                    const TA* __restrict__ acc, double* __restrict__ K, int* err) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t j = warp; j < n_nodes; j += nw) {
    const int64_t o = outer[3 * j];
    const int64_t b0 = o / 9;
    const int len = (outer[3 * j + 1] - outer[3 * j]) / 3;
    if (o < 0 || o % 9 != 0 || len < 0 || b0 + len > n_blocks) {
      if (lane == 0) atomicOr(err, kErrIndex);
      continue;
    }
    double* col = K + o;
    for (int t = lane; t < 9 * len; t += 32) {
      const int c = t / (3 * len), rem = t - c * 3 * len, pos = rem / 3, r = rem - 3 * pos;
      col[t] = static_cast<double>(acc[(b0 + pos) * STRIDE + 3 * r + c]);
    }
  }
}

// Deterministic: each block sums its contributions in ascending id order.
template <typename TC>
__global__ void det_reduce_blocks(int n_nodes, const int64_t* __restrict__ col_ptr,
                                  const int64_t* __restrict__ lptr, const int64_t* __restrict__ list,
                                  const TC* __restrict__ contrib, double* __restrict__ K) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t j = warp; j < n_nodes; j += nw) {
    const int64_t b0 = col_ptr[j];
    const int len = static_cast<int>(col_ptr[j + 1] - b0);
    double* col = K + 9 * b0;
    for (int pos = lane; pos < len; pos += 32) {
      TC s[9];
      for (int k = 0; k < 9; ++k) s[k] = TC(0);
      for (int64_t q = lptr[b0 + pos]; q < lptr[b0 + pos + 1]; ++q) {
        const TC* v = contrib + 9 * list[q];
        for (int k = 0; k < 9; ++k) s[k] += v[k];
      }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) col[3 * c * len + 3 * pos + r] = static_cast<double>(s[3 * r + c]);
    }
  }
}

__global__ void det_reduce_F(int n_nodes, const int64_t* __restrict__ lptr, const int64_t* __restrict__ list,
                             const double* __restrict__ fc, double* __restrict__ F) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_nodes) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int64_t q = lptr[j]; q < lptr[j + 1]; ++q) {
    const double* v = fc + 3 * list[q];
    s0 += v[0]; s1 += v[1]; s2 += v[2];
  }
  F[3 * j] = s0; F[3 * j + 1] = s1; F[3 * j + 2] = s2;
}

// ---- energies -----------------------------------------------------------------------
__global__ void __launch_bounds__(128) face_energy_kernel(int n_gp, const int64_t* ptr, const int32_t* idx,
                                                          const double* dpsi, const double* ddpsi,
                                                          const double* weight, const double* x, Material m,
                                                          NatCurv nc, const double* gp_xy, double* out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  double em = 0.0, eb = 0.0;
  for (int64_t g = warp; g < n_gp; g += nw) {
    const int64_t p0 = ptr[g];
    const int n = static_cast<int>(ptr[g + 1] - p0);
    double s[15];
    kin_sums(lane, p0, n, idx, dpsi, ddpsi, x, s);
    PointState P;
    point_state(s, m, P, gp_xy ? natcurv_kappa(nc, gp_xy[2 * g]) : 0.0);
    if (lane == 0) {   // Meshless.h:204-220, with E1_el (Meshless.h:212)
      em += 0.5 * weight[g] * (P.e0[0] * P.N[0] + P.e0[1] * P.N[1] + P.e0[2] * P.N[2]);
      eb += 0.5 * weight[g] * (P.e1el[0] * P.M[0] + P.e1el[1] * P.M[1] + P.e1el[2] * P.M[2]);
    }
  }
  if (lane == 0) { atomicAdd(out, em); atomicAdd(out + 1, eb); }
}

// ---- kinematic state of arbitrary points (post-processing) ---------------------------
// One thread per point: the displacement sum_I Psi_I u_I and Kinematics::compute /
// Constitutive::evaluate (plate/Kinematics.h:61-120, Constitutive.h:57-70) in FP64, one row
// of kPointStateCols per point: u(3) r_X(3) r_Y(3) r_XX(3) r_YY(3) r_XY(3) b(3)
// E0 (xx yy xy, tensor) E1 (xx yy xy, tensor) N (Voigt) M (Voigt).
constexpr int kPointStateCols = 33;
__global__ void __launch_bounds__(128) point_state_kernel(int n, const int64_t* __restrict__ ptr,
                                                          const int32_t* __restrict__ idx,
                                                          const double* __restrict__ psi,
                                                          const double* __restrict__ dpsi,
                                                          const double* __restrict__ ddpsi,
                                                          const double* __restrict__ x, Material m,
                                                          NatCurv nc, const double* __restrict__ gp_xy,
                                                          double* __restrict__ out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  double s[15], u[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < 15; ++k) s[k] = 0.0;
  for (int64_t e = ptr[g]; e < ptr[g + 1]; ++e) {
    const int64_t j = idx[e];
    const double u0 = x[3 * j], u1 = x[3 * j + 1], u2 = x[3 * j + 2];
    const double p = psi[e], dx = dpsi[2 * e], dy = dpsi[2 * e + 1];
    const double dxx = ddpsi[3 * e], dyy = ddpsi[3 * e + 1], dxy = ddpsi[3 * e + 2];
    u[0] += p * u0; u[1] += p * u1; u[2] += p * u2;
    s[0] += u0 * dx; s[1] += u1 * dx; s[2] += u2 * dx;
    s[3] += u0 * dy; s[4] += u1 * dy; s[5] += u2 * dy;
    s[6] += u0 * dxx; s[7] += u1 * dxx; s[8] += u2 * dxx;
    s[9] += u0 * dyy; s[10] += u1 * dyy; s[11] += u2 * dyy;
    s[12] += u0 * dxy; s[13] += u1 * dxy; s[14] += u2 * dxy;
  }
  PointState P;
  point_state(s, m, P, gp_xy ? natcurv_kappa(nc, gp_xy[2 * static_cast<int64_t>(g)]) : 0.0);
  double* o = out + static_cast<int64_t>(g) * kPointStateCols;
  for (int c = 0; c < 3; ++c) {
    o[c] = u[c];
    o[3 + c] = P.a1[c]; o[6 + c] = P.a2[c];
    o[9 + c] = P.rxx[c]; o[12 + c] = P.ryy[c]; o[15 + c] = P.rxy[c];
    o[18 + c] = P.b[c];
    o[27 + c] = P.N[c]; o[30 + c] = P.M[c];
  }
  o[21] = P.e0[0]; o[22] = P.e0[1]; o[23] = 0.5 * P.e0[2];
  o[24] = P.e1[0]; o[25] = P.e1[1]; o[26] = 0.5 * P.e1[2];
}

__global__ void hinge_energy_kernel(HingeArgs a, double* out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.n_gp) return;
  if (a.active && a.active[g] == 0) return;
  double F12[12] = {1, 0, 0, 0, 1, 0, 1, 0, 0, 0, 1, 0};
  for (int64_t e = a.lptr[g]; e < a.lptr[g + 1]; ++e) {
    const int64_t j = a.lidx[e];
    for (int c = 0; c < 3; ++c) { F12[c] += a.x[3 * j + c] * a.ldpsi[2 * e]; F12[3 + c] += a.x[3 * j + c] * a.ldpsi[2 * e + 1]; }
  }
  for (int64_t e = a.rptr[g]; e < a.rptr[g + 1]; ++e) {
    const int64_t j = a.ridx[e];
    for (int c = 0; c < 3; ++c) { F12[6 + c] += a.x[3 * j + c] * a.rdpsi[2 * e]; F12[9 + c] += a.x[3 * j + c] * a.rdpsi[2 * e + 1]; }
  }
  const double theta = fold_angle(F12, a.tangent[2 * g], a.tangent[2 * g + 1], nullptr);
  const double th0 = a.theta0_gp ? a.theta0_gp[g] : a.theta0;
  const double d = theta - th0;
  atomicAdd(out, a.weight[g] * (0.5 * a.Kt * (d * d)));
}

// ---- FP32 tangent with merged contributions ------------------------------------------
// One CTA per group of kMG consecutive Gauss points. The CTA builds the group's
// per-neighbour records (AoS, 16-byte rows) and point frames in shared memory, then each
// thread takes distinct blocks ("entries") of the group, sums every contribution to its
// block in registers (in a fixed order: point, then local pair) and scatters it once with
// three 16-byte vector atomics. On GB300 a scattered 48-byte block costs ~14 ns of L2
// atomic throughput per SM-slot (~70 G blocks/s for the chip); merging the ~7.5
// contributions per block of a 4x4 quadrature cell divides that traffic accordingly.
constexpr int kMG = 16;          // points per group (the setup kernel uses the same)
constexpr int kMrgThreads = 256;

struct MergeArgs {
  const int64_t* ent_ptr;
  const int32_t* ent_slot;
  const int32_t* ent_cstart;  // (count << 16) | first contribution
  const int8_t* direct;
  const uint16_t* code;       // point (4) | i (6) | j (6)
  int* err;                   // set to kErrStage when a staging copy never completes
  uint32_t extra_tx;          // 0; the failure-detection test expects bytes that never arrive
  // The merged kernel's groups: glist[0 .. gcount) when glist is set (the groups the tensor
  // tangent does not take), else every group of [g_begin, g_end).
  const int32_t* glist;
  int gcount;
};

// ---- bulk-copy (TMA) staging --------------------------------------------------------
// One elected thread copies a group's contiguous ranges of grad / Hessian Phi and ids
// into shared memory with cp.async.bulk, completing on an mbarrier the CTA waits on.
constexpr int kErrStage = 4;
constexpr long long kStageCycles = 1LL << 31;  // SM clock cycles (~1 s) before a wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait: false if the phase did not complete within kStageCycles SM cycles.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity))
    if (clock64() - t0 > kStageCycles) return false;
  return true;
}

// L2 prefetch of the bytes [lo, hi) of a global array whose base is 16-byte aligned: a
// hint, so the window shrinks to the whole 16-byte units inside it (the bulk prefetch's
// rule) and nothing outside the range is touched.
__device__ __forceinline__ void l2_prefetch(const void* base, int64_t lo, int64_t hi) {
  const int64_t b = (lo + 15) & ~static_cast<int64_t>(15), e = hi & ~static_cast<int64_t>(15);
  if (e > b)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;"
                 :: "l"(static_cast<const char*>(base) + b), "r"(static_cast<uint32_t>(e - b)) : "memory");
}

// Byte window [lo, lo + len) of the element range [q0, q1) of an array with `es`-byte
// elements, widened to 16-byte boundaries (the bulk copy's alignment rule).
struct StageWin { int64_t lo; uint32_t len, skip; };
__device__ __forceinline__ StageWin stage_window(int64_t q0, int64_t q1, int es) {
  const int64_t b0 = q0 * es, b1 = q1 * es;
  StageWin w;
  w.lo = b0 & ~static_cast<int64_t>(15);
  w.len = static_cast<uint32_t>(((b1 + 15) & ~static_cast<int64_t>(15)) - w.lo);
  w.skip = static_cast<uint32_t>(b0 - w.lo);
  return w;
}

// The block of the local pair (i, j) of one point from the frame (fr[0..1]: a1 | b.v,
// a2), the I-side record (ri[0..1]) and the J-side record (rj), as in phase2_group, added
// to v (the three rank-1 terms of each entry as one FMA chain onto it). The unit normal
// b = a1 x a2 / |a1 x a2| and g_I = a1 c0_I + a2 c1_I are rebuilt from the frame here
// rather than read: the kernel is bound by shared-memory wavefronts, not FMAs.
template <bool BZERO>
__device__ __forceinline__ void merged_pair(const float4* fr, const float4* ri, const float4* rj, float v[9]) {
  const float4 f0 = fr[0], f1 = fr[1];
  const float a1t[3] = {f0.x, f0.y, f0.z}, a2t[3] = {f1.x, f1.y, f1.z};
  float bt[3] = {a1t[1] * a2t[2] - a1t[2] * a2t[1], a1t[2] * a2t[0] - a1t[0] * a2t[2],
                 a1t[0] * a2t[1] - a1t[1] * a2t[0]};
  const float rn = rsqrtf(bt[0] * bt[0] + bt[1] * bt[1] + bt[2] * bt[2]);
  bt[0] *= rn; bt[1] *= rn; bt[2] *= rn;
  const float bv = f0.w;
  const float4 i0 = ri[0], i1 = ri[1];
  const float dxi = i0.x, dyi = i0.y, be0 = i0.z, be1 = i0.w, be2 = i1.x, Tui = i1.y;
  const float gi[3] = {a1t[0] * i1.z + a2t[0] * i1.w, a1t[1] * i1.z + a2t[1] * i1.w, a1t[2] * i1.z + a2t[2] * i1.w};
  float Y1[3], Y2[3], Y3[3], geo;
  if constexpr (BZERO) {
    const float4 j0 = rj[0], j1 = rj[1], j2 = rj[2], j3 = rj[3];
    const float pa0 = j0.x, pa1 = j0.y, pa2 = j0.z, pb0 = j0.w, pb1 = j1.x, pb2 = j1.y;
    const float qc0 = j1.z, qc1 = j1.w, qc2 = j2.x, cj0 = j2.y, cj1 = j2.z, nj0 = j2.w, nj1 = j3.x, TuWj = j3.y;
    const float s1 = Tui * cj0, s2 = Tui * cj1;
    geo = dxi * nj0 + dyi * nj1;
    const float z11 = dxi * pa0 + dyi * pa2, z12 = dxi * pb0 + dyi * pb2;
    const float z21 = dyi * pa1 + dxi * pa2, z22 = dyi * pb1 + dxi * pb2;
    const float z33 = be0 * qc0 + be1 * qc1 + be2 * qc2 + bv * (dxi * cj0 + dyi * cj1);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Y1[c] = a1t[c] * z11 + a2t[c] * z12 - s1 * bt[c];
      Y2[c] = a1t[c] * z21 + a2t[c] * z22 - s2 * bt[c];
      Y3[c] = bt[c] * z33 - TuWj * gi[c];
    }
  } else {
    float J[24];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const float4 t = rj[q];
      J[4 * q] = t.x; J[4 * q + 1] = t.y; J[4 * q + 2] = t.z; J[4 * q + 3] = t.w;
    }
    const float cj0 = J[18], cj1 = J[19], nj0 = J[20], nj1 = J[21], TuWj = J[22];
    const float s1 = Tui * cj0, s2 = Tui * cj1;
    const float t3 = bv * (dxi * cj0 + dyi * cj1);
    geo = dxi * nj0 + dyi * nj1;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Y1[c] = dxi * J[c] + dyi * J[6 + c] - s1 * bt[c];
      Y2[c] = dyi * J[3 + c] + dxi * J[6 + c] - s2 * bt[c];
      Y3[c] = be0 * J[9 + c] + be1 * J[12 + c] + be2 * J[15 + c] + t3 * bt[c] - TuWj * gi[c];
    }
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
      v[3 * r + c] = fmaf(bt[r], Y3[c], fmaf(a2t[r], Y2[c], fmaf(a1t[r], Y1[c], v[3 * r + c])));
    v[4 * r] += geo;
  }
}

// DET: every entry's sum is stored (9 floats at unit e0 + e of a.Kc) for the ordered
// per-block reduction instead of being added atomically; it needs no direct group.
template <bool BZERO, bool DET>
__global__ void __launch_bounds__(kMrgThreads, 4) face_tangent_merged_kernel(FaceArgs a, const float* __restrict__ gstate,
                                                                            MergeArgs mg) {
  // One record per (point, neighbour): the I side (2 float4) then the J side (4 float4, 6
  // when B != 0), with an odd stride RW in float4. A warp reads the records of 32
  // different (point, neighbour) pairs at once, and with an even stride of 2^m float4
  // those addresses fall into only 8 / 2^m of the 8 four-bank groups (a stride of 4
  // serialises a float4 load into ~16 wavefronts instead of ~4).
  constexpr int RW = BZERO ? 7 : 9;  // float4 rows of a record (6 or 8 used)
  constexpr int FW = 3;              // float4 rows of a point frame (2 used)
  extern __shared__ __align__(16) float msm[];
  __shared__ uint64_t stage_bar;
  __shared__ int64_t sptr[kMG + 1];
  const int nmax = a.nmax;
  const int E = kMG * nmax;                                 // most entries of a group
  float* st = msm;                                          // [kState][kMG]
  float4* fr = reinterpret_cast<float4*>(st + kState * kMG); // [kMG][FW]
  float4* rec = fr + FW * kMG;                              // [kMG * nmax][RW]
  // Staging windows (16-byte aligned): grad Phi, Hessian Phi of the group's entries.
  unsigned char* s_d = reinterpret_cast<unsigned char*>(rec + RW * E);
  unsigned char* s_dd = s_d + 8 * E + 32;
  const unsigned char* dpsi_b = static_cast<const unsigned char*>(a.dpsi_t);
  const unsigned char* ddpsi_b = static_cast<const unsigned char*>(a.ddpsi_t);
  const Material& m = a.mat;
  // Groups of this launch: [g_begin, g_end) are multiples of kMG apart (chunk bounds are
  // multiples of 32), so a group never straddles two launches.
  const int G0 = a.g_begin / kMG;
  const int nG = mg.glist ? mg.gcount : (a.g_end + kMG - 1) / kMG - G0;
  auto group = [&](int gi) { return mg.glist ? mg.glist[gi] : G0 + gi; };
  // Thread 0 starts the copies of group G's ranges; every thread later waits on the phase.
  auto stage = [&](int G) {
    const int g0 = G * kMG, g1 = min(g0 + kMG, a.g_end);
    const int64_t q0 = a.ptr[g0], q1 = a.ptr[g1];
    const StageWin wd = stage_window(q0, q1, 8), wdd = stage_window(q0, q1, 12);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect(&stage_bar, wd.len + wdd.len + mg.extra_tx);
    if (wd.len) bulk_load(s_d, dpsi_b + wd.lo, wd.len, &stage_bar);
    if (wdd.len) bulk_load(s_dd, ddpsi_b + wdd.lo, wdd.len, &stage_bar);
    // The group's pair codes and entry tables are read once per step from DRAM, one code per
    // contribution: bring them into L2 now, a group ahead of their use.
    l2_prefetch(mg.code, 2 * a.map_ptr[g0], 2 * a.map_ptr[g1]);
    const int64_t e0 = mg.ent_ptr[G], e1 = mg.ent_ptr[G + 1];
    l2_prefetch(mg.ent_cstart, 4 * e0, 4 * e1);
    l2_prefetch(mg.ent_slot, 4 * e0, 4 * e1);
  };
  if (threadIdx.x == 0) {
    mbar_init(&stage_bar);
    if (static_cast<int>(blockIdx.x) < nG) stage(group(blockIdx.x));
  }
  __syncthreads();
  uint32_t phase = 0;
  for (int gi = blockIdx.x; gi < nG; gi += gridDim.x) {
    const int G = group(gi);
    const int g0 = G * kMG;
    const int kn = min(kMG, a.g_end - g0);
    for (int t = threadIdx.x; t < kState * kMG; t += blockDim.x) {
      const int f = t / kMG, k = t - f * kMG;
      st[t] = k < kn ? gstate[static_cast<int64_t>(f) * a.n_gp + g0 + k] : 0.0f;
    }
    if (threadIdx.x <= kn) sptr[threadIdx.x] = a.ptr[g0 + threadIdx.x];
    // Every thread waits on the copies of this group, then the CTA agrees on the outcome
    // so that no thread leaves while another waits at a barrier.
    const bool ok = mbar_wait(&stage_bar, phase);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicOr(mg.err, kErrStage);
        mbar_wait(&stage_bar, phase);   // let copies still in flight land before leaving
      }
      return;
    }
    phase ^= 1u;
    const int64_t q0 = sptr[0];
    const float* sdp = reinterpret_cast<const float*>(s_d + (q0 * 8 - ((q0 * 8) & ~static_cast<int64_t>(15))));
    const float* sddp = reinterpret_cast<const float*>(s_dd + (q0 * 12 - ((q0 * 12) & ~static_cast<int64_t>(15))));
    if (threadIdx.x < kn) {
      const int k = threadIdx.x;
      fr[FW * k] = make_float4(st[(S_A1) * kMG + k], st[(S_A1 + 1) * kMG + k], st[(S_A1 + 2) * kMG + k], st[S_BV * kMG + k]);
      fr[FW * k + 1] = make_float4(st[(S_A2) * kMG + k], st[(S_A2 + 1) * kMG + k], st[(S_A2 + 2) * kMG + k], 0.0f);
    }
    // Records of every (point, neighbour) of the group (the same formulas as phase2_group),
    // from the staged copies.
    for (int t = threadIdx.x; t < kMG * nmax; t += blockDim.x) {
      const int k = t / nmax, i = t - k * nmax;
      if (k >= kn) continue;
      const int64_t p0 = sptr[k];
      if (i >= sptr[k + 1] - p0) continue;
      const int64_t e = p0 + i - q0;   // entry within the group's staged range
      const float a1t[3] = {st[S_A1 * kMG + k], st[(S_A1 + 1) * kMG + k], st[(S_A1 + 2) * kMG + k]};
      const float a2t[3] = {st[S_A2 * kMG + k], st[(S_A2 + 1) * kMG + k], st[(S_A2 + 2) * kMG + k]};
      const float bt[3] = {st[S_B * kMG + k], st[(S_B + 1) * kMG + k], st[(S_B + 2) * kMG + k]};
      float rxx[3], ryy[3], rxy[3], Nt[3], Mt[3], Ci[4];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        rxx[c] = st[(S_RXX + c) * kMG + k]; ryy[c] = st[(S_RYY + c) * kMG + k]; rxy[c] = st[(S_RXY + c) * kMG + k];
        Nt[c] = st[(S_N + c) * kMG + k]; Mt[c] = st[(S_M + c) * kMG + k];
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) Ci[c] = st[(S_CI + c) * kMG + k];
      const float pX = st[S_P * kMG + k], pY = st[(S_P + 1) * kMG + k], Wt = st[S_W * kMG + k];
      const float dx = sdp[2 * e], dy = sdp[2 * e + 1];
      const float dxx = sddp[3 * e], dyy = sddp[3 * e + 1], dxy = sddp[3 * e + 2];
      const float c0 = Ci[0] * dx + Ci[1] * dy, c1 = Ci[2] * dx + Ci[3] * dy;
      float gI[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) gI[r] = a1t[r] * c0 + a2t[r] * c1;
      const float b0 = -dxx + (rxx[0] * gI[0] + rxx[1] * gI[1] + rxx[2] * gI[2]);
      const float b1 = -dyy + (ryy[0] * gI[0] + ryy[1] * gI[1] + ryy[2] * gI[2]);
      const float b2 = 2.0f * (-dxy + (rxy[0] * gI[0] + rxy[1] * gI[1] + rxy[2] * gI[2]));
      const float Tu = dx * pX + dy * pY - (dxx * Mt[0] + 2.0f * dxy * Mt[2] + dyy * Mt[1]);
      float4* RI = rec + RW * t;
      RI[0] = make_float4(dx, dy, b0, b1);
      RI[1] = make_float4(b2, Tu, c0, c1);
      float4* RJ = rec + RW * t + 2;
      if constexpr (BZERO) {
        float pa[3], pb[3], qc[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          pa[r] = (m.Ai<float>(3 * r) * dx + m.Ai<float>(3 * r + 2) * dy) * Wt;
          pb[r] = (m.Ai<float>(3 * r + 1) * dy + m.Ai<float>(3 * r + 2) * dx) * Wt;
          qc[r] = (m.Di<float>(3 * r) * b0 + m.Di<float>(3 * r + 1) * b1 +
                   m.Di<float>(3 * r + 2) * b2) * Wt;
        }
        RJ[0] = make_float4(pa[0], pa[1], pa[2], pb[0]);
        RJ[1] = make_float4(pb[1], pb[2], qc[0], qc[1]);
        RJ[2] = make_float4(qc[2], c0 * Wt, c1 * Wt, (Nt[0] * dx + Nt[2] * dy) * Wt);
        RJ[3] = make_float4((Nt[2] * dx + Nt[1] * dy) * Wt, Tu * Wt, 0.0f, 0.0f);
      } else {
        float J[24];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const float Ar0 = m.Ai<float>(3 * r), Ar1 = m.Ai<float>(3 * r + 1), Ar2 = m.Ai<float>(3 * r + 2);
          const float Br0 = m.Bi<float>(3 * r), Br1 = m.Bi<float>(3 * r + 1), Br2 = m.Bi<float>(3 * r + 2);
          const float Dr0 = m.Di<float>(3 * r), Dr1 = m.Di<float>(3 * r + 1), Dr2 = m.Di<float>(3 * r + 2);
          const float pa = (Ar0 * dx + Ar2 * dy) * Wt, pb = (Ar1 * dy + Ar2 * dx) * Wt, pc = (Br0 * b0 + Br1 * b1 + Br2 * b2) * Wt;
          const float qa = (Br0 * dx + Br2 * dy) * Wt, qb = (Br1 * dy + Br2 * dx) * Wt, qc = (Dr0 * b0 + Dr1 * b1 + Dr2 * b2) * Wt;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            J[3 * r + c] = a1t[c] * pa + a2t[c] * pb + bt[c] * pc;
            J[9 + 3 * r + c] = a1t[c] * qa + a2t[c] * qb + bt[c] * qc;
          }
        }
        J[18] = c0 * Wt; J[19] = c1 * Wt;
        J[20] = (Nt[0] * dx + Nt[2] * dy) * Wt; J[21] = (Nt[2] * dx + Nt[1] * dy) * Wt;
        J[22] = Tu * Wt; J[23] = 0.0f;
#pragma unroll
        for (int q = 0; q < 6; ++q) RJ[q] = make_float4(J[4 * q], J[4 * q + 1], J[4 * q + 2], J[4 * q + 3]);
      }
    }
    __syncthreads();
    // The staging buffers are free again: start the next group's copies, which land while
    // this group's entries are summed.
    if (threadIdx.x == 0 && gi + static_cast<int>(gridDim.x) < nG) stage(group(gi + gridDim.x));
    float4* acc4 = static_cast<float4*>(a.Kacc);
    const int64_t cbase = a.map_ptr[g0];
    if (!DET && mg.direct[G]) {
      // Too many pairs for the setup's shared-memory sort: scatter pair by pair.
      for (int k = 0; k < kn; ++k) {
        const int64_t p0k = a.ptr[g0 + k];
        const int n = static_cast<int>(a.ptr[g0 + k + 1] - p0k);
        const int np = n * (n + 1) / 2;
        const int64_t m0 = a.map_ptr[g0 + k];
        for (int p = threadIdx.x; p < np; p += blockDim.x) {
          int i = 0, off = p;
          while (off >= n - i) { off -= n - i; ++i; }
          const int j = i + off;
          float v[9] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
          merged_pair<BZERO>(fr + FW * k, rec + RW * (k * nmax + i), rec + RW * (k * nmax + j) + 2, v);
          scatter_atomic<float>(a.Kacc, a.map_slot[m0 + p], a.idx[p0k + i] > a.idx[p0k + j], v);
        }
      }
    } else {
      const int64_t e0 = mg.ent_ptr[G];
      const int ne = static_cast<int>(mg.ent_ptr[G + 1] - e0);
      // Entries are count-descending; thread t takes one entry per round of blockDim.x, in
      // ascending order on even rounds and descending on odd ones, so that every warp's
      // rounds add up to about the same work before the group's closing barrier. Each
      // thread's entries are software-pipelined: the next entry's (count, first) word and its
      // first code are fetched while this entry's contributions are summed, so that no entry
      // starts on two dependent global loads.
      const int step = static_cast<int>(blockDim.x);
      const int t = threadIdx.x;
      auto entry_of = [&](int r) {
        const int base = r * step, rem = min(step, ne - base);
        return t < rem ? base + ((r & 1) ? rem - 1 - t : t) : ne;
      };
      const uint16_t* gcodes = mg.code + cbase;
      int r = 0;
      int e = entry_of(0);
      int cs = e < ne ? mg.ent_cstart[e0 + e] : 0;
      unsigned first = (e < ne && (cs >> 16) > 0) ? gcodes[cs & 0xffff] : 0u;
      for (; e < ne; e = entry_of(++r)) {
        const int cnt = cs >> 16, c0 = cs & 0xffff;
        const int en = entry_of(r + 1);
        const int cs_n = en < ne ? mg.ent_cstart[e0 + en] : 0;
        const int32_t slot = DET ? 0 : mg.ent_slot[e0 + e];
        float acc[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = 0.0f;
        // Codes are in the block's stored orientation (row node first); the next code (after
        // the last one, the next entry's first) is fetched while the current contribution is
        // computed.
        const uint16_t* codes = gcodes + c0;
        unsigned next = first;
        for (int c = 0; c < cnt; ++c) {
          const unsigned code = next;
          if (c + 1 < cnt) next = codes[c + 1];
          else next = (cs_n >> 16) > 0 ? gcodes[cs_n & 0xffff] : 0u;
          const int k = code >> 12, i = (code >> 6) & 63, j = code & 63;
          merged_pair<BZERO>(fr + FW * k, rec + RW * (k * nmax + i), rec + RW * (k * nmax + j) + 2, acc);
        }
        first = cnt > 0 ? next : ((cs_n >> 16) > 0 ? gcodes[cs_n & 0xffff] : 0u);
        cs = cs_n;
        if constexpr (DET) {
          float* d = static_cast<float*>(a.Kc) + 9 * (e0 + e);
#pragma unroll
          for (int q = 0; q < 9; ++q) d[q] = acc[q];
        } else {
          float4* d = acc4 + 3 * static_cast<int64_t>(slot);
          atomicAdd(d, make_float4(acc[0], acc[1], acc[2], acc[3]));
          atomicAdd(d + 1, make_float4(acc[4], acc[5], acc[6], acc[7]));
          atomicAdd(d + 2, make_float4(acc[8], 0.0f, 0.0f, 0.0f));
        }
      }
    }
    __syncthreads();
  }
}

#include "tangent_tc.cuh"

inline unsigned nb(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// SM count per device ordinal, looked up once per device (grids are sized from it).
int sm_count(int device) {
  constexpr int kMaxDev = 64;
  static std::atomic<int> cached[kMaxDev];
  if (device < 0 || device >= kMaxDev) {
    int v = 0;
    CGB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device));
    return v;
  }
  int v = cached[device].load(std::memory_order_relaxed);
  if (v <= 0) {
    CGB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device));
    cached[device].store(v, std::memory_order_relaxed);
  }
  return v;
}

HingeArgs hinge_args(cgb_assembler* a, cgb_fold_dev& f, const double* d_x, int flags) {
  HingeArgs h{};
  h.n_gp = f.n_gp;
  h.max_u = std::max(f.max_u, 1);
  h.lptr = f.left->nbr_ptr.p; h.lidx = f.left->nbr_idx.p; h.ldpsi = f.left->dpsi.p;
  h.rptr = f.right->nbr_ptr.p; h.ridx = f.right->nbr_idx.p; h.rdpsi = f.right->dpsi.p;
  h.weight = f.weight.p; h.tangent = f.tangent.p;
  h.Kt = f.Kt; h.theta0 = f.theta0;
  h.theta0_gp = f.has_theta0_gp ? f.theta0_gp.p : nullptr;
  h.active = f.has_active ? f.active.p : nullptr;
  h.u_ptr = f.u_ptr.p; h.u_node = f.u_node.p; h.l_pos = f.l_pos.p; h.r_pos = f.r_pos.p;
  h.pair_ptr = f.pair_ptr.p; h.pair_slot = f.pair_slot.p;
  h.x = d_x;
  h.exact = (flags & CGB_HINGE_EXACT) ? 1 : 0;
  h.want_K = (flags & CGB_TANGENT) ? 1 : 0;
  h.tk_float = (flags & CGB_MIXED) ? 1 : 0;
  (void)a;
  return h;
}

__global__ void to_float(int64_t n, const double* __restrict__ src, float* __restrict__ dst) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n) dst[i] = static_cast<float>(src[i]);
}

// FP32 copies of grad / Hessian Phi for the FP32 pair phase (made once per assembler).
// FP32 copies of grad / Hessian Phi, each followed by kStagePad zero elements: the
// tangent stages a group's range of these arrays with bulk copies whose ends are rounded
// out to 16 bytes, which may read up to 15 bytes past the last entry.
constexpr int kStagePad = 16;

void ensure_fp32_shapes(cgb_assembler* a) {
  if (a->dpsi32.p) return;
  const cgb_shape* S = a->faces;
  a->faces_version = S->version;
  cudaStream_t st = a->ctx->stream;
  a->dpsi32.alloc(2 * S->nnz + kStagePad);
  a->ddpsi32.alloc(3 * S->nnz + kStagePad);
  CGB_CUDA(cudaMemsetAsync(a->dpsi32.p, 0, a->dpsi32.bytes(), st));
  CGB_CUDA(cudaMemsetAsync(a->ddpsi32.p, 0, a->ddpsi32.bytes(), st));
  if (S->nnz) {
    to_float<<<nb(2 * S->nnz, 256), 256, 0, st>>>(2 * S->nnz, S->dpsi.p, a->dpsi32.p);
    to_float<<<nb(3 * S->nnz, 256), 256, 0, st>>>(3 * S->nnz, S->ddpsi.p, a->ddpsi32.p);
  }
  CGB_CUDA(cudaGetLastError());
}

// Sliced-ELL copy of the face neighbour data for phase 1: groups of 32 consecutive Gauss
// points, each group padded to its longest list; entry q of point 32 W + l at
// sell_ptr[W] + 32 q + l. Padding entries are never read (q < n of the point).
__global__ void fill_sell(int n_gp, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                          const double* __restrict__ dpsi, const double* __restrict__ ddpsi,
                          const int64_t* __restrict__ sell_ptr, int32_t* __restrict__ sidx,
                          double* __restrict__ sdpsi, double* __restrict__ sddpsi) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_gp) return;
  const int64_t base = sell_ptr[g >> 5] + (g & 31);
  for (int64_t e = ptr[g], q = 0; e < ptr[g + 1]; ++e, ++q) {
    const int64_t d = base + 32 * q;
    sidx[d] = idx[e];
    sdpsi[2 * d] = dpsi[2 * e];
    sdpsi[2 * d + 1] = dpsi[2 * e + 1];
    sddpsi[3 * d] = ddpsi[3 * e];
    sddpsi[3 * d + 1] = ddpsi[3 * e + 1];
    sddpsi[3 * d + 2] = ddpsi[3 * e + 2];
  }
}

void ensure_sell(cgb_assembler* a) {
  if (a->sell_ptr.p) return;
  const cgb_shape* S = a->faces;
  a->faces_version = S->version;
  cudaStream_t st = a->ctx->stream;
  std::vector<int64_t> ptr(S->n_gp + 1);
  CGB_CUDA(cudaMemcpyAsync(ptr.data(), S->nbr_ptr.p, ptr.size() * 8, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  const int ngroups = (S->n_gp + 31) / 32;
  std::vector<int64_t> sp(ngroups + 1, 0);
  for (int W = 0; W < ngroups; ++W) {
    int64_t mx = 0;
    for (int g = 32 * W; g < std::min(S->n_gp, 32 * W + 32); ++g) mx = std::max(mx, ptr[g + 1] - ptr[g]);
    sp[W + 1] = sp[W] + 32 * mx;
  }
  upload(a->sell_ptr, sp.data(), sp.size(), st);
  a->sidx.alloc(sp[ngroups]);
  a->sdpsi.alloc(2 * sp[ngroups]);
  a->sddpsi.alloc(3 * sp[ngroups]);
  CGB_CUDA(cudaMemsetAsync(a->sidx.p, 0, a->sidx.bytes(), st));
  if (S->n_gp)
    fill_sell<<<nb(S->n_gp, 128), 128, 0, st>>>(S->n_gp, S->nbr_ptr.p, S->nbr_idx.p, S->dpsi.p, S->ddpsi.p,
                                                a->sell_ptr.p, a->sidx.p, a->sdpsi.p, a->sddpsi.p);
  CGB_CUDA(cudaGetLastError());
}

}  // namespace

void refresh_face_copies(cgb_assembler* a) {
  const cgb_shape* S = a->faces;
  if (a->faces_version == S->version) return;
  cudaStream_t st = a->ctx->stream;
  if (a->dpsi32.p && S->nnz) {
    to_float<<<nb(2 * S->nnz, 256), 256, 0, st>>>(2 * S->nnz, S->dpsi.p, a->dpsi32.p);
    to_float<<<nb(3 * S->nnz, 256), 256, 0, st>>>(3 * S->nnz, S->ddpsi.p, a->ddpsi32.p);
  }
  if (a->sell_ptr.p && S->n_gp)
    fill_sell<<<nb(S->n_gp, 128), 128, 0, st>>>(S->n_gp, S->nbr_ptr.p, S->nbr_idx.p, S->dpsi.p, S->ddpsi.p,
                                                a->sell_ptr.p, a->sidx.p, a->sdpsi.p, a->sddpsi.p);
  CGB_CUDA(cudaGetLastError());
  a->faces_version = S->version;
}

namespace {

constexpr int kChunks = 4;

// The second stream and the events of the chunked face launch (created once per
// assembler; the stream is non-blocking and joined back into the context stream).
void ensure_side_stream(cgb_assembler* a) {
  if (a->side) return;
  CGB_CUDA(cudaStreamCreateWithFlags(&a->side, cudaStreamNonBlocking));
  CGB_CUDA(cudaEventCreateWithFlags(&a->ev_start, cudaEventDisableTiming));
  CGB_CUDA(cudaEventCreateWithFlags(&a->ev_done, cudaEventDisableTiming));
  for (int c = 0; c < kMaxChunks; ++c) CGB_CUDA(cudaEventCreateWithFlags(&a->ev_chunk[c], cudaEventDisableTiming));
}

}  // namespace

// Dynamic shared memory of the merged FP32 tangent for neighbour lists of up to nmax
// entries: per-point state and frames of the 16 points, one record per (point, neighbour)
// (RW float4, odd), and the staging windows of grad / Hessian Phi (20 bytes per entry + 64).
constexpr size_t kMergedSmemMax = 220 * 1024;
size_t merged_smem_bytes(int nmax, bool bzero) {
  const size_t RW = bzero ? 7 : 9, FW = 3;
  const size_t E = static_cast<size_t>(kMG) * nmax;
  return (static_cast<size_t>(kState) * kMG + 4 * FW * kMG + 4 * RW * E) * sizeof(float) + (20 * E + 64);
}

void assemble_device(cgb_assembler* a, const double* d_x, double* d_K, double* d_F, int flags) {
  cgb_context* ctx = a->ctx;
  cudaStream_t st = ctx->stream;
  const cgb_shape* S = a->faces;
  const bool want_K = (flags & CGB_TANGENT) != 0;
  const bool mixed = (flags & CGB_MIXED) != 0;
  const bool det = (flags & CGB_DETERMINISTIC) != 0;
  const bool hinge = (flags & CGB_HINGE) != 0;
  if (!a->have_material) throw Error(CGB_ERR_INVALID, "assemble: material not set (cgb_set_material)");
  if (want_K && !d_K) throw Error(CGB_ERR_INVALID, "assemble: K output missing with CGB_TANGENT");
  refresh_face_copies(a);
  if (det) deterministic_prepare(a);
  bool bzero = true;
  for (double v : a->B) bzero = bzero && (v == 0.0);
  // The FP32 tangent merges each group's contributions per block; in deterministic mode the
  // merged sums become the K units, unless a group is too large to merge. The merged kernel
  // stages a group's records in shared memory: supports too wide for that (the reference
  // app's cubic basis at rho = 6h has over 100 neighbours) take the per-point FP32 tangent.
  const size_t msm = merged_smem_bytes(std::max(S->max_n, 1), bzero);
  bool merged = false;
  if (mixed && want_K && msm <= kMergedSmemMax) {
    merge_prepare(a);
    merged = !det || a->mrg_n_direct == 0;
  }
  // The tensor-core tangent takes the merged path's cells whose node union fits one
  // 128-row tile (its entries are the merged entries, so the deterministic lists are the
  // same).
  const size_t tcsm = tc_smem_bytes(std::max(S->max_n, 1), bzero);
  const bool use_tc = merged && a->tuning.tangent_kind == CGB_TANGENT_TENSOR && tcsm <= kMergedSmemMax;
  if (use_tc) tc_prepare(a);
  if (det && want_K) {
    if (merged) deterministic_entry_lists(a);
    else deterministic_pair_lists(a);
  }
  const int64_t k_face_units = merged ? a->mrg_n_ent : a->n_pairs;

  const int64_t ndof = 3 * static_cast<int64_t>(a->n_nodes);
  // Accumulators.
  prof_begin(ctx, CGB_PHASE_ZERO);
  if (!det) CGB_CUDA(cudaMemsetAsync(d_F, 0, ndof * sizeof(double), st));
  if (want_K && !det) {
    if (mixed) {
      a->kacc32.ensure(12 * a->n_blocks);
      CGB_CUDA(cudaMemsetAsync(a->kacc32.p, 0, 12 * a->n_blocks * sizeof(float), st));
    } else {
      a->kacc64.ensure(9 * a->n_blocks);
      CGB_CUDA(cudaMemsetAsync(a->kacc64.p, 0, 9 * a->n_blocks * sizeof(double), st));
    }
  }
  const int64_t n_contrib = k_face_units + [&] { int64_t s = 0; for (auto& f : a->folds) s += f.n_pairs; return s; }();
  if (det) {
    a->fcontrib.ensure(3 * std::max<int64_t>(a->n_fcontrib, 1));
    if (want_K) {
      if (mixed) a->contrib32.ensure(9 * std::max<int64_t>(n_contrib, 1));
      else a->contrib64.ensure(9 * std::max<int64_t>(n_contrib, 1));
    }
    // Hinge entries of inactive crease points contribute zero.
    if (a->n_fcontrib > S->nnz)
      CGB_CUDA(cudaMemsetAsync(a->fcontrib.p + 3 * S->nnz, 0, 3 * (a->n_fcontrib - S->nnz) * sizeof(double), st));
    if (want_K && n_contrib > k_face_units) {
      if (mixed) CGB_CUDA(cudaMemsetAsync(a->contrib32.p + 9 * k_face_units, 0, 9 * (n_contrib - k_face_units) * sizeof(float), st));
      else CGB_CUDA(cudaMemsetAsync(a->contrib64.p + 9 * k_face_units, 0, 9 * (n_contrib - k_face_units) * sizeof(double), st));
    }
  }

  prof_end(ctx, CGB_PHASE_ZERO, 0);

  // Face kernel.
  FaceArgs fa{};
  fa.n_gp = S->n_gp;
  fa.g_begin = 0;
  fa.g_end = S->n_gp;
  fa.nmax = std::max(S->max_n, 1);
  fa.ptr = S->nbr_ptr.p; fa.idx = S->nbr_idx.p; fa.dpsi = S->dpsi.p; fa.ddpsi = S->ddpsi.p;
  fa.weight = a->weight.p; fa.x = d_x;
  fa.map_ptr = a->map_ptr.p; fa.map_slot = a->map_slot.p;
  ensure_sell(a);
  fa.sell_ptr = a->sell_ptr.p; fa.sidx = a->sidx.p; fa.sdpsi = a->sdpsi.p; fa.sddpsi = a->sddpsi.p;
  fa.mat = make_material(a->A, a->B, a->D);
  fa.nc = ctx->natcurv;
  fa.gp_xy = natcurv_points(ctx, S, "assemble");
  fa.F = d_F;
  fa.Fc = a->fcontrib.p;
  fa.Kacc = mixed ? static_cast<void*>(a->kacc32.p) : static_cast<void*>(a->kacc64.p);
  fa.Kc = mixed ? static_cast<void*>(a->contrib32.p) : static_cast<void*>(a->contrib64.p);
  const size_t tk = mixed ? sizeof(float) : sizeof(double);
  const size_t smem = want_K ? static_cast<size_t>(kFaceWarps) * ((kState * 32 + kRec * fa.nmax) * tk +
                                                                 fa.nmax * sizeof(int)) : 0;
  if (mixed && want_K) {
    ensure_fp32_shapes(a);
    fa.dpsi_t = a->dpsi32.p;
    fa.ddpsi_t = a->ddpsi32.p;
  } else {
    fa.dpsi_t = S->dpsi.p;
    fa.ddpsi_t = S->ddpsi.p;
  }
  if (smem > 200 * 1024)
    throw Error(CGB_ERR_CAPACITY, "assemble: " + std::to_string(S->max_n) + " neighbours per Gauss point exceed the shared-memory staging");
  const int sms = sm_count(ctx->device);
  const unsigned grid = std::max(1u, std::min(nb(S->n_gp, 32 * kFaceWarps), static_cast<unsigned>(sms * 8)));
  (void)grid;
  // Residual kernel (phase 1) then tangent kernel (phase 2), each at its own occupancy.
  const size_t state_bytes = static_cast<size_t>(kState) * std::max(S->n_gp, 1) * tk;
  if (want_K) {
    if (mixed) a->state32.ensure(state_bytes / sizeof(float));
    else a->state64.ensure(state_bytes / sizeof(double));
  }
  float* st32 = a->state32.p;
  double* st64 = a->state64.p;
  // The residual kernel of chunk c + 1 (FP64 pipe) runs beside the tangent kernel of
  // chunk c (FP32 pipe, L2 atomics) on a second stream; chunks are multiples of 32 points.
  ensure_side_stream(a);
  const int n_chunks = a->tuning.n_chunks > 0 ? a->tuning.n_chunks : (S->n_gp >= 65536 ? kChunks : 1);
  const int rthreads = a->tuning.residual_threads > 0 ? a->tuning.residual_threads : 256;
  const int chunk = ((S->n_gp + n_chunks - 1) / n_chunks + 31) / 32 * 32;
  // Chunk c covers [cb(c), cb(c + 1)). The first chunk is a quarter of the others: the
  // tangent stream waits for its residual, and from then on the tangent stream is the
  // longer of the two, so a short first chunk shortens the step; the rest share the
  // remaining points evenly. All bounds are multiples of 32 points.
  const int first = n_chunks > 1 ? std::max(32, (chunk / 4 + 31) / 32 * 32) : chunk;
  const int rest = n_chunks > 1 ? ((std::max(S->n_gp - first, 0) + n_chunks - 2) / (n_chunks - 1) + 31) / 32 * 32 : 0;
  auto cb = [&](int c) {
    const int64_t b = c == 0 ? 0 : static_cast<int64_t>(first) + static_cast<int64_t>(c - 1) * rest;
    return static_cast<int>(std::min<int64_t>(b, S->n_gp));
  };
  int nface = 0;
  const size_t tsm = static_cast<size_t>(kTanWarps) * ((kState * 32 + kRec * fa.nmax) * tk + fa.nmax * sizeof(int));
  // Work counters of the chunks' residual launches.
  a->work_ctr.ensure(kMaxChunks);
  CGB_CUDA(cudaMemsetAsync(a->work_ctr.p, 0, kMaxChunks * sizeof(int), st));
  if (want_K) {
    CGB_CUDA(cudaEventRecord(a->ev_start, st));
    CGB_CUDA(cudaStreamWaitEvent(a->side, a->ev_start, 0));
  }
  for (int c = 0; c < n_chunks && S->n_gp > 0; ++c) {
    int* work = a->work_ctr.p + c;
    fa.g_begin = cb(c);
    fa.g_end = cb(c + 1);
    if (fa.g_begin >= fa.g_end) break;
    const int ncg = fa.g_end - fa.g_begin;
    const unsigned rgrid = std::max(1u, std::min(nb(ncg, rthreads), static_cast<unsigned>(sms * 16 * (256 / rthreads))));
    prof_begin(ctx, CGB_PHASE_FACE);
    if (mixed) {
      if (det) { if (want_K) face_residual_kernel<float, true, true><<<rgrid, rthreads, 0, st>>>(fa, st32, work);
                 else face_residual_kernel<float, true, false><<<rgrid, rthreads, 0, st>>>(fa, st32, work); }
      else { if (want_K) face_residual_kernel<float, false, true><<<rgrid, rthreads, 0, st>>>(fa, st32, work);
             else face_residual_kernel<float, false, false><<<rgrid, rthreads, 0, st>>>(fa, st32, work); }
    } else {
      if (det) { if (want_K) face_residual_kernel<double, true, true><<<rgrid, rthreads, 0, st>>>(fa, st64, work);
                 else face_residual_kernel<double, true, false><<<rgrid, rthreads, 0, st>>>(fa, st64, work); }
      else { if (want_K) face_residual_kernel<double, false, true><<<rgrid, rthreads, 0, st>>>(fa, st64, work);
             else face_residual_kernel<double, false, false><<<rgrid, rthreads, 0, st>>>(fa, st64, work); }
    }
    ++nface;
    prof_end(ctx, CGB_PHASE_FACE, 1);
    CGB_CUDA(cudaGetLastError());
    if (!want_K) continue;
    CGB_CUDA(cudaEventRecord(a->ev_chunk[c], st));
    CGB_CUDA(cudaStreamWaitEvent(a->side, a->ev_chunk[c], 0));
    prof_begin(ctx, CGB_PHASE_TANGENT, a->side);
    const unsigned tgrid = std::max(1u, std::min(nb(ncg, 32 * kTanWarps), static_cast<unsigned>(sms * 16)));
    auto tl = [&](auto kern, auto* stp) {
      if (tsm > 48 * 1024) CGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tsm)));
      kern<<<tgrid, 32 * kTanWarps, tsm, a->side>>>(fa, stp);
    };
    int ntan = 1;
    if (merged) {
      MergeArgs mg{a->mrg_ent_ptr.p, a->mrg_ent_slot.p, a->mrg_ent_cstart.p, a->mrg_direct.p, a->mrg_code.p,
                   ctx->dev_err.p, a->test_stage_extra_tx, nullptr, 0};
      auto kern = det ? (bzero ? face_tangent_merged_kernel<true, true> : face_tangent_merged_kernel<false, true>)
                      : (bzero ? face_tangent_merged_kernel<true, false> : face_tangent_merged_kernel<false, false>);
      CGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(msm)));
      int per_sm = 0;
      CGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMrgThreads, msm));
      const int Gb = fa.g_begin / kMG, Ge = (fa.g_end + kMG - 1) / kMG;
      const int groups = Ge - Gb;
      if (a->tuning.tangent_ctas_per_sm > 0) per_sm = std::min(per_sm, a->tuning.tangent_ctas_per_sm);
      if (use_tc) {
        // Cells whose node union fits one 128-row tile: one tensor-core product each; the
        // others (sorted group list, this chunk's part) on the CUDA cores.
        TcArgs tca{a->tc_nbr_u.p, a->tc_cell_U.p, a->tc_ent_uv.p};
        auto tk = det ? (bzero ? face_tangent_tc_kernel<true, true> : face_tangent_tc_kernel<false, true>)
                      : (bzero ? face_tangent_tc_kernel<true, false> : face_tangent_tc_kernel<false, false>);
        CGB_CUDA(cudaFuncSetAttribute(tk, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(tcsm)));
        CGB_CUDA(cudaFuncSetAttribute(tk, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        // Each CTA holds 256 of the SM's 512 tensor-memory columns: two CTAs per SM at most,
        // when the shared memory of two (dynamic + static + the 1 KB the runtime reserves per
        // CTA) fits the SM's.
        cudaFuncAttributes fat{};
        CGB_CUDA(cudaFuncGetAttributes(&fat, tk));
        int smem_sm = 0;
        CGB_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
        int tc_per_sm = 2 * (tcsm + fat.sharedSizeBytes + 1024) <= static_cast<size_t>(smem_sm) ? 2 : 1;
        if (a->tuning.tangent_ctas_per_sm > 0) tc_per_sm = std::min(tc_per_sm, a->tuning.tangent_ctas_per_sm);
        a->tc_last_per_sm = tc_per_sm;
        const unsigned tgrid2 = static_cast<unsigned>(std::max(1, std::min(groups, tc_per_sm * sms)));
        tk<<<tgrid2, kTcThreads, tcsm, a->side>>>(fa, st32, mg, tca);
        const auto& fb = a->tc_fallback_h;
        const int lo = static_cast<int>(std::lower_bound(fb.begin(), fb.end(), Gb) - fb.begin());
        const int hi = static_cast<int>(std::lower_bound(fb.begin(), fb.end(), Ge) - fb.begin());
        ntan = 1;
        if (hi > lo) {
          MergeArgs mf = mg;
          mf.glist = a->tc_fallback.p + lo;
          mf.gcount = hi - lo;
          const unsigned fgrid = static_cast<unsigned>(std::max(1, std::min(hi - lo, std::max(per_sm, 1) * sms)));
          kern<<<fgrid, kMrgThreads, msm, a->side>>>(fa, st32, mf);
          ntan = 2;
        }
      } else {
        const unsigned mgrid = static_cast<unsigned>(std::max(1, std::min(groups, std::max(per_sm, 1) * sms)));
        kern<<<mgrid, kMrgThreads, msm, a->side>>>(fa, st32, mg);
      }
    } else if (mixed) {
      if (det) { if (bzero) tl(face_tangent_kernel<float, true, true>, st32); else tl(face_tangent_kernel<float, true, false>, st32); }
      else { if (bzero) tl(face_tangent_kernel<float, false, true>, st32); else tl(face_tangent_kernel<float, false, false>, st32); }
    } else {
      if (det) { if (bzero) tl(face_tangent_kernel<double, true, true>, st64); else tl(face_tangent_kernel<double, true, false>, st64); }
      else { if (bzero) tl(face_tangent_kernel<double, false, true>, st64); else tl(face_tangent_kernel<double, false, false>, st64); }
    }
    ++nface;
    prof_end(ctx, CGB_PHASE_TANGENT, ntan, a->side);
    CGB_CUDA(cudaGetLastError());
  }
  (void)nface;

  // Hinge, on the context stream beside the last tangent chunks: it reads x, its shape sets
  // and the fold state and adds into F and the block accumulator with atomics (or into its
  // own contribution slots in deterministic mode), none of which the tangent reads.
  if (hinge) {
    prof_begin(ctx, CGB_PHASE_HINGE);
    int nl = 0;
    int64_t kb = k_face_units, fb = a->hinge_f_base;
    for (auto& f : a->folds) {
      if (f.n_gp == 0) continue;
      HingeArgs h = hinge_args(a, f, d_x, flags);
      h.F = d_F;
      h.Kacc = mixed ? static_cast<void*>(a->kacc32.p) : static_cast<void*>(a->kacc64.p);
      if (det) {
        h.Fc = a->fcontrib.p;
        h.Kc = mixed ? static_cast<void*>(a->contrib32.p) : static_cast<void*>(a->contrib64.p);
        h.f_base = fb; h.k_base = kb;
      }
      const size_t hs = static_cast<size_t>(kHingeWarps) * (7 * h.max_u + 144 + 16) * sizeof(double);
      if (hs > 48 * 1024) CGB_CUDA(cudaFuncSetAttribute(hinge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(hs)));
      hinge_kernel<<<nb(f.n_gp, kHingeWarps), 32 * kHingeWarps, hs, st>>>(h);
      CGB_CUDA(cudaGetLastError());
      ++nl;
      kb += f.n_pairs;
      fb += f.n_u;
    }
    prof_end(ctx, CGB_PHASE_HINGE, nl);
  }
  if (want_K) {
    CGB_CUDA(cudaEventRecord(a->ev_done, a->side));
    CGB_CUDA(cudaStreamWaitEvent(st, a->ev_done, 0));
  }

  // Reductions / output.
  const unsigned cg = std::max(1u, std::min(nb(a->n_nodes, 4), static_cast<unsigned>(sms * 32)));
  prof_begin(ctx, CGB_PHASE_REDUCE);
  int nred = 0;
  if (det) {
    nred = want_K ? 2 : 1;
    det_reduce_F<<<nb(a->n_nodes, 128), 128, 0, st>>>(a->n_nodes, a->node_list_ptr.p, a->node_list.p, a->fcontrib.p, d_F);
    if (want_K) {
      if (merged) det_reduce_blocks<float><<<cg, 128, 0, st>>>(a->n_nodes, a->col_ptr.p, a->ent_list_ptr.p, a->ent_list.p, a->contrib32.p, d_K);
      else if (mixed) det_reduce_blocks<float><<<cg, 128, 0, st>>>(a->n_nodes, a->col_ptr.p, a->blk_list_ptr.p, a->blk_list.p, a->contrib32.p, d_K);
      else det_reduce_blocks<double><<<cg, 128, 0, st>>>(a->n_nodes, a->col_ptr.p, a->blk_list_ptr.p, a->blk_list.p, a->contrib64.p, d_K);
    }
  } else if (want_K) {
    nred = 1;
    if (mixed) blocks_to_csc<float, 12><<<cg, 128, 0, st>>>(a->n_nodes, a->col_ptr.p, a->kacc32.p, d_K);
    else blocks_to_csc<double, 9><<<cg, 128, 0, st>>>(a->n_nodes, a->col_ptr.p, a->kacc64.p, d_K);
  }
  prof_end(ctx, CGB_PHASE_REDUCE, nred);
  CGB_CUDA(cudaGetLastError());
}

// Mixed-precision face assembly on caller-owned device arrays, with the FP32 block
// accumulator supplied by the caller (the allocation-free entry point, noalloc.cu).
void face_mixed_on_arrays(const cgb_face_problem& pr, const double* d_x, double* d_K, double* d_F,
                          float* kacc, int* err, cudaStream_t st) {
  FaceArgs fa{};
  fa.n_gp = pr.n_gp;
  fa.g_begin = 0;
  fa.g_end = pr.n_gp;
  fa.nmax = std::max(pr.max_neighbours, 1);
  fa.ptr = pr.nbr_ptr; fa.idx = pr.nbr_idx; fa.dpsi = pr.dpsi; fa.ddpsi = pr.ddpsi;
  fa.dpsi_t = pr.dpsi; fa.ddpsi_t = pr.ddpsi;
  fa.weight = pr.weight; fa.x = d_x;
  fa.map_ptr = pr.map_ptr; fa.map_slot = pr.csr_map; fa.outer = pr.outer;
  fa.mat = make_material(pr.A, pr.B, pr.D);
  fa.F = d_F;
  fa.Kacc = kacc;
  const int64_t n_blocks = static_cast<int64_t>(pr.nnz / 9);
  fa.n_blocks = n_blocks;
  fa.n_nodes = pr.n_nodes;
  fa.err = err;
  CGB_CUDA(cudaMemsetAsync(d_F, 0, 3 * static_cast<size_t>(pr.n_nodes) * sizeof(double), st));
  if (pr.n_gp == 0) {  // no face point: K is zero, and outer is not needed
    if (pr.nnz > 0) CGB_CUDA(cudaMemsetAsync(d_K, 0, static_cast<size_t>(pr.nnz) * sizeof(double), st));
    return;
  }
  CGB_CUDA(cudaMemsetAsync(kacc, 0, 12 * static_cast<size_t>(n_blocks) * sizeof(float), st));
  const size_t smem = static_cast<size_t>(kFaceWarps) * ((kState * 32 + kRec * fa.nmax) * sizeof(float) +
                                                        fa.nmax * sizeof(int));
  auto kern = face_kernel<float, false, true, double, true>;
  if (smem > 48 * 1024) CGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int dev = 0;
  CGB_CUDA(cudaGetDevice(&dev));
  const int sms = sm_count(dev);
  const unsigned grid = std::max(1u, std::min(nb(pr.n_gp, 32 * kFaceWarps), static_cast<unsigned>(sms * 8)));
  kern<<<grid, 32 * kFaceWarps, smem, st>>>(fa);
  const unsigned cg = std::max(1u, std::min(nb(pr.n_nodes, 4), static_cast<unsigned>(sms * 32)));
  blocks_to_csc_outer<float, 12><<<cg, 128, 0, st>>>(pr.n_nodes, n_blocks, pr.outer, kacc, d_K, err);
  CGB_CUDA(cudaGetLastError());
}

void point_state_device(cgb_context* ctx, const cgb_shape* S, const double* d_x, const double* A, const double* B,
                        const double* D, double* d_out) {
  if (S->n_gp == 0) return;
  if (!S->psi.p || S->psi.n < static_cast<size_t>(std::max<int64_t>(S->nnz, 1)))
    throw Error(CGB_ERR_INVALID, "point state: the shape set has no Psi");
  const Material m = make_material(A, B, D);
  const double* xy = natcurv_points(ctx, S, "point state");
  point_state_kernel<<<nb(S->n_gp, 128), 128, 0, ctx->stream>>>(S->n_gp, S->nbr_ptr.p, S->nbr_idx.p, S->psi.p,
                                                                S->dpsi.p, S->ddpsi.p, d_x, m, ctx->natcurv, xy,
                                                                d_out);
  CGB_CUDA(cudaGetLastError());
}

void energies_device(cgb_assembler* a, const double* d_x, double* out3) {
  cgb_context* ctx = a->ctx;
  cudaStream_t st = ctx->stream;
  a->energy.ensure(3);
  CGB_CUDA(cudaMemsetAsync(a->energy.p, 0, 3 * sizeof(double), st));
  const Material m = make_material(a->A, a->B, a->D);
  const cgb_shape* S = a->faces;
  if (S->n_gp)
    face_energy_kernel<<<std::max(1u, std::min(nb(S->n_gp, 4), static_cast<unsigned>(sm_count(ctx->device) * 32))), 128, 0, st>>>(
        S->n_gp, S->nbr_ptr.p, S->nbr_idx.p, S->dpsi.p, S->ddpsi.p, a->weight.p, d_x, m, ctx->natcurv,
        natcurv_points(ctx, S, "energies"), a->energy.p);
  for (auto& f : a->folds) {
    if (!f.n_gp) continue;
    HingeArgs h = hinge_args(a, f, d_x, 0);
    hinge_energy_kernel<<<nb(f.n_gp, 128), 128, 0, st>>>(h, a->energy.p + 2);
  }
  CGB_CUDA(cudaGetLastError());
  CGB_CUDA(cudaMemcpyAsync(out3, a->energy.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
}

}  // namespace cgb
