// tangent_tc.cuh — the FP32-class tangent of one quadrature cell (16 consecutive Gauss
// points) as one tensor-core product on sm_103a (tcgen05, 3xTF32 with FP32 accumulation
// in tensor memory). Included by assemble.cu after the merged CUDA-core tangent, whose
// per-point state, staging and merge tables it shares.
//
// The pair loop of NonLinearAssembler::updateStiffness (plate/Assembly.h:282-324) gives,
// per Gauss point and local pair (i, j), the 3x3 block
//     K_ij = a1 (x) Y1 + a2 (x) Y2 + b (x) Y3 + geo I        (see the top of assemble.cu)
// which is the frame form  K_ij = F T(i, j) F^T  with F = [a1 a2 b] and, since the frame's
// metric inverse G = (F^T F)^-1 = diag(C0^-1, 1) gives I = F G F^T, the geometric term
// folded into T. Every entry of T is a sum of products of a scalar of neighbour i
// (dx, dy, Tu, c0, c1, beta0, beta1, beta2) and a coefficient of neighbour j, so
//     K_ij[r][c] = sum_{m<13} L_m(i)[r] R_m(j)[c]
// with the 13 I-side rows L_m(i) = F_p[r] phi_f(i) and J-side vectors R_m(j). Over the
// union of the cell's neighbour nodes (U <= 42 nodes, 3U <= 126 rows) the cell's blocks are
//     K_cell = sum_k A_k B_k^T,   A_k, B_k: 128 x 13, rows (node u, component r),
// zero where node u is not a neighbour of point k: a 128 x 3U x (16 x 13) product. It runs
// as 3xTF32 (A = Ah + Al, B = Bh + Bl, each part rounded to TF32, Ah Bh + Ah Bl + Al Bh, the
// Al Bl term dropped: FP32-class accuracy), i.e. K = 40 per point (13 + 13 + 13 + one zero),
// five 128 x N x 8 MMAs.
//
// Per CTA (256 threads), per cell:
//  - the cell's point states (from the FP64 residual kernel) and, staged by a bulk copy
//    (TMA) completing on an mbarrier, its FP32 grad / Hessian Phi; then the records of all
//    the cell's (point, neighbour) entries, every thread taking a share;
//  - per point k, in one of two operand stages: warps 0-3 write the 128 rows of A_k (hi /
//    lo split) into tensor memory with tcgen05.st (row = lane), warps 4-7 the rows of B_k
//    into shared memory in the canonical K-major no-swizzle layout; after one barrier, one
//    thread issues the five MMAs (A from tensor memory, B from shared memory) and commits
//    them to the stage's mbarrier; the stage is rewritten two points later, after it;
//  - after the last point: the accumulator (128 lanes x 3U columns of tensor memory) goes to
//    a dense matrix in shared memory (over the B stages and the records), and each merged
//    entry of the cell (a distinct 3x3 block of K, from the merge tables) is read from it and
//    scattered with three 16-byte FP32 vector atomics (or stored, deterministic mode).
// Every wait is bounded (about one second of SM clock); a CTA that gives up records bit 16
// (or bit 4 for the staging copy) in the device error word, lets its copies and MMAs land
// (bounded), frees its tensor memory and returns.

constexpr int kTcThreads = 256;              // rows 0-127 of A (warps 0-3) and of B (warps 4-7)
constexpr int kTcMaxU = kTcMaxUnion;         // 42: 3 U <= 126 rows of one M = 128 tile
constexpr int kTcK = 40;                     // per point: 13 + 13 + 13 values + one zero
constexpr int kTcChunks = kTcK / 4;          // 16-byte chunks of a B row
constexpr int kTcOpBytes = 128 * kTcK * 4;   // B of one point: 20,480 bytes
constexpr int kTcDStride = 132;              // floats per row of the epilogue's dense matrix
constexpr int kTcDBytes = 128 * kTcDStride * 4;
constexpr int kErrTensor = 16;               // device error word: an MMA completion never came
// Tensor memory: the accumulator in columns [0, 128), A of the two operand stages in
// [128, 168) and [168, 208).
constexpr uint32_t kTcCols = 256;
constexpr uint32_t kTcACol = 128;

struct TcArgs {
  const uint8_t* nbr_u;    // per face entry: its node's index in the cell's sorted union
  const int16_t* cell_U;   // per group: union size (above kTcMaxU: not on this path)
  const uint16_t* ent_uv;  // per merged entry: union index of its row node | its column node << 8
};

// Floats of one neighbour record: the I side (dx dy Tu c0 c1 beta0 beta1 beta2) and the
// J side, the frame coefficients (on a1, a2, b) of the 13 R vectors; with B = 0 only their
// nonzero coefficients.
__host__ __device__ constexpr int tc_rec_floats(bool bzero) { return bzero ? 24 : 36; }

__host__ __device__ inline size_t tc_region_bytes(int nmax, bool bzero) {
  const size_t ops_rec = 2 * static_cast<size_t>(kTcOpBytes) +
                         static_cast<size_t>(kMG) * nmax * tc_rec_floats(bzero) * sizeof(float);
  return ops_rec > static_cast<size_t>(kTcDBytes) ? ops_rec : static_cast<size_t>(kTcDBytes);
}
__host__ __device__ inline size_t tc_smem_bytes(int nmax, bool bzero) {
  return tc_region_bytes(nmax, bzero) + static_cast<size_t>(kState) * kMG * sizeof(float) +
         (20 * static_cast<size_t>(kMG) * nmax + 64);
}

// The record of one (point, neighbour) entry (the reference's per-neighbour quantities of
// Assembly.h:233-268 in the rank-3 frame form; W = Gauss weight folded into the J side).
template <bool BZERO>
__device__ __forceinline__ void tc_record(const float* st, int k, const Material& m, float dx, float dy, float dxx,
                                          float dyy, float dxy, float* R) {
  auto S = [&](int f) { return st[f * kMG + k]; };
  const float a1t[3] = {S(S_A1), S(S_A1 + 1), S(S_A1 + 2)};
  const float a2t[3] = {S(S_A2), S(S_A2 + 1), S(S_A2 + 2)};
  const float Ci[4] = {S(S_CI), S(S_CI + 1), S(S_CI + 2), S(S_CI + 3)};
  const float Nt[3] = {S(S_N), S(S_N + 1), S(S_N + 2)};
  const float Mt[3] = {S(S_M), S(S_M + 1), S(S_M + 2)};
  const float pX = S(S_P), pY = S(S_P + 1), bv = S(S_BV), Wt = S(S_W);
  const float c0 = Ci[0] * dx + Ci[1] * dy, c1 = Ci[2] * dx + Ci[3] * dy;
  float gI[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) gI[r] = a1t[r] * c0 + a2t[r] * c1;
  const float b0 = -dxx + (S(S_RXX) * gI[0] + S(S_RXX + 1) * gI[1] + S(S_RXX + 2) * gI[2]);
  const float b1 = -dyy + (S(S_RYY) * gI[0] + S(S_RYY + 1) * gI[1] + S(S_RYY + 2) * gI[2]);
  const float b2 = 2.0f * (-dxy + (S(S_RXY) * gI[0] + S(S_RXY + 1) * gI[1] + S(S_RXY + 2) * gI[2]));
  const float Tu = dx * pX + dy * pY - (dxx * Mt[0] + 2.0f * dxy * Mt[2] + dyy * Mt[1]);
  float pa[3], pb[3], qc[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    pa[r] = (m.Ai<float>(3 * r) * dx + m.Ai<float>(3 * r + 2) * dy) * Wt;
    pb[r] = (m.Ai<float>(3 * r + 1) * dy + m.Ai<float>(3 * r + 2) * dx) * Wt;
    qc[r] = (m.Di<float>(3 * r) * b0 + m.Di<float>(3 * r + 1) * b1 + m.Di<float>(3 * r + 2) * b2) * Wt;
  }
  const float cW0 = c0 * Wt, cW1 = c1 * Wt;
  const float nW0 = (Nt[0] * dx + Nt[2] * dy) * Wt, nW1 = (Nt[2] * dx + Nt[1] * dy) * Wt;
  R[0] = dx; R[1] = dy; R[2] = Tu; R[3] = c0; R[4] = c1; R[5] = b0; R[6] = b1; R[7] = b2;
  // T(i, j) with the geometric term folded in through G = diag(C0^-1, 1):
  //   (a1, dx): P0 + geo G(0, .)   (a1, dy): P2 + geo G(0, .)
  //   (a2, dx): P2 + geo G(1, .)   (a2, dy): P1 + geo G(1, .)   (b, beta_r): Q_r
  if constexpr (BZERO) {   // P_r = a1 pa_r + a2 pb_r, Q_r = b qc_r
    R[8] = pa[0] + Ci[0] * nW0;  R[9] = pb[0] + Ci[1] * nW0;
    R[10] = pa[2] + Ci[0] * nW1; R[11] = pb[2] + Ci[1] * nW1;
    R[12] = pa[2] + Ci[2] * nW0; R[13] = pb[2] + Ci[3] * nW0;
    R[14] = pa[1] + Ci[2] * nW1; R[15] = pb[1] + Ci[3] * nW1;
    R[16] = qc[0]; R[17] = qc[1]; R[18] = qc[2];
    R[19] = -cW0; R[20] = -cW1;
    R[21] = bv * cW0 + nW0; R[22] = bv * cW1 + nW1;
    R[23] = -Tu * Wt;
  } else {                 // P_r = a1 pa_r + a2 pb_r + b pc_r, Q_r = a1 qa_r + a2 qb_r + b qc_r
    float pc[3], qa[3], qb[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      pc[r] = (m.Bi<float>(3 * r) * b0 + m.Bi<float>(3 * r + 1) * b1 + m.Bi<float>(3 * r + 2) * b2) * Wt;
      qa[r] = (m.Bi<float>(3 * r) * dx + m.Bi<float>(3 * r + 2) * dy) * Wt;
      qb[r] = (m.Bi<float>(3 * r + 1) * dy + m.Bi<float>(3 * r + 2) * dx) * Wt;
    }
    R[8] = pa[0] + Ci[0] * nW0;  R[9] = pb[0] + Ci[1] * nW0;  R[10] = pc[0];
    R[11] = pa[2] + Ci[0] * nW1; R[12] = pb[2] + Ci[1] * nW1; R[13] = pc[2];
    R[14] = pa[2] + Ci[2] * nW0; R[15] = pb[2] + Ci[3] * nW0; R[16] = pc[2];
    R[17] = pa[1] + Ci[2] * nW1; R[18] = pb[1] + Ci[3] * nW1; R[19] = pc[1];
#pragma unroll
    for (int r = 0; r < 3; ++r) { R[20 + 3 * r] = qa[r]; R[21 + 3 * r] = qb[r]; R[22 + 3 * r] = qc[r]; }
    R[29] = -cW0; R[30] = -cW1;
    R[31] = bv * cW0 + nW0; R[32] = bv * cW1 + nW1;
    R[33] = -Tu * Wt;
  }
}

// 3xTF32 split of 13 values into the 40 K-values of one operand row: hi parts first, then
// (A) hi again and lo, or (B) lo and hi again, then one zero; every part rounded to TF32
// here (the tensor core would otherwise truncate the low parts' mantissas: a one-signed
// error of up to 2^-21 of the value).
template <bool IS_A>
__device__ __forceinline__ void tc_split(const float (&v)[13], float (&out)[kTcK]) {
#pragma unroll
  for (int q = 0; q < 13; ++q) {
    const float hi = umma::to_tf32(v[q]);
    const float lo = umma::to_tf32(v[q] - hi);
    out[q] = hi;
    out[13 + q] = IS_A ? hi : lo;
    out[26 + q] = IS_A ? lo : hi;
  }
  out[39] = 0.0f;
}

// Row (u, r) of A: F_p[r] phi_f(i) for the 13 I-side features of neighbour i (R: its record).
__device__ __forceinline__ void tc_a_values(const float* R, float a1r, float a2r, float br, float (&av)[13]) {
  const float dx = R[0], dy = R[1], Tu = R[2];
  av[0] = a1r * dx; av[1] = a1r * dy; av[2] = a1r * Tu;
  av[3] = a2r * dx; av[4] = a2r * dy; av[5] = a2r * Tu;
  av[6] = br * R[3]; av[7] = br * R[4];
  av[8] = br * R[5]; av[9] = br * R[6]; av[10] = br * R[7];
  av[11] = br * dx; av[12] = br * dy;
}

// Row (v, c) of B: component c of the 13 R vectors of neighbour j.
template <bool BZERO>
__device__ __forceinline__ void tc_b_values(const float* R, float a1r, float a2r, float br, float (&bv)[13]) {
  if constexpr (BZERO) {
    bv[0] = R[8] * a1r + R[9] * a2r;
    bv[1] = R[10] * a1r + R[11] * a2r;
    bv[2] = R[19] * br;
    bv[3] = R[12] * a1r + R[13] * a2r;
    bv[4] = R[14] * a1r + R[15] * a2r;
    bv[5] = R[20] * br;
    bv[6] = R[23] * a1r;
    bv[7] = R[23] * a2r;
    bv[8] = R[16] * br; bv[9] = R[17] * br; bv[10] = R[18] * br;
    bv[11] = R[21] * br;
    bv[12] = R[22] * br;
  } else {
    bv[0] = R[8] * a1r + R[9] * a2r + R[10] * br;
    bv[1] = R[11] * a1r + R[12] * a2r + R[13] * br;
    bv[2] = R[29] * br;
    bv[3] = R[14] * a1r + R[15] * a2r + R[16] * br;
    bv[4] = R[17] * a1r + R[18] * a2r + R[19] * br;
    bv[5] = R[30] * br;
    bv[6] = R[33] * a1r;
    bv[7] = R[33] * a2r;
    bv[8] = R[20] * a1r + R[21] * a2r + R[22] * br;
    bv[9] = R[23] * a1r + R[24] * a2r + R[25] * br;
    bv[10] = R[26] * a1r + R[27] * a2r + R[28] * br;
    bv[11] = R[31] * br;
    bv[12] = R[32] * br;
  }
}

template <bool BZERO, bool DET>
__global__ void __launch_bounds__(kTcThreads, 2) face_tangent_tc_kernel(FaceArgs a, const float* __restrict__ gstate,
                                                                       MergeArgs mg, TcArgs tc) {
  constexpr int RS = tc_rec_floats(BZERO);
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ __align__(8) uint64_t stage_bar;
  __shared__ __align__(8) uint64_t mma_bar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int64_t sptr[kMG + 1];
  __shared__ int16_t pos[kMG][kTcMaxU + 2];   // (point, union node) -> entry within the cell, or -1
  __shared__ int s_next;
  const int t = threadIdx.x, w = t >> 5;
  const bool a_role = t < 128;
  const int row = t & 127;                     // operand row (u, r): u = row / 3, r = row % 3
  const int nmax = a.nmax;
  const int E = kMG * nmax;
  unsigned char* opsB = tsm;                                   // 2 stages of B
  float* rec = reinterpret_cast<float*>(tsm + 2 * kTcOpBytes); // [entry of the cell][RS]
  float* Dm = reinterpret_cast<float*>(tsm);                   // epilogue, over B and the records
  const size_t region = tc_region_bytes(nmax, BZERO);
  float* st = reinterpret_cast<float*>(tsm + region);          // [kState][kMG]
  unsigned char* s_d = reinterpret_cast<unsigned char*>(st + kState * kMG);
  unsigned char* s_dd = s_d + 8 * E + 32;
  const unsigned char* dpsi_b = static_cast<const unsigned char*>(a.dpsi_t);
  const unsigned char* ddpsi_b = static_cast<const unsigned char*>(a.ddpsi_t);
  const Material& m = a.mat;
  const int G1 = (a.g_end + kMG - 1) / kMG;
  const int stride = static_cast<int>(gridDim.x);
  auto eligible = [&](int G) { return !mg.direct[G] && tc.cell_U[G] <= kTcMaxU; };
  auto next_from = [&](int G) {
    while (G < G1 && !eligible(G)) G += stride;
    return G;
  };
  auto stage = [&](int G) {
    const int g0 = G * kMG, g1 = min(g0 + kMG, a.g_end);
    const int64_t q0 = a.ptr[g0], q1 = a.ptr[g1];
    const StageWin wd = stage_window(q0, q1, 8), wdd = stage_window(q0, q1, 12);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect(&stage_bar, wd.len + wdd.len + mg.extra_tx);
    if (wd.len) bulk_load(s_d, dpsi_b + wd.lo, wd.len, &stage_bar);
    if (wdd.len) bulk_load(s_dd, ddpsi_b + wdd.lo, wdd.len, &stage_bar);
  };
  if (w == 0) umma::tmem_alloc(&tmem_base, kTcCols);
  if (t == 0) {
    mbar_init(&stage_bar);
    mbar_init(&mma_bar[0]);
    mbar_init(&mma_bar[1]);
    const int G = next_from(a.g_begin / kMG + static_cast<int>(blockIdx.x));
    s_next = G;
    if (G < G1) stage(G);
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tb = tmem_base;
  const uint32_t lane_base = static_cast<uint32_t>(32 * (w & 3)) << 16;
  uint32_t sphase = 0, mphase0 = 0, mphase1 = 0;
  bool pend0 = false, pend1 = false;   // a commit on the stage's mbarrier not waited for yet
  bool dirty0 = true, dirty1 = true;   // (B rows) this thread's row of the stage may be nonzero
  bool stage_in_flight = s_next < G1;
  int err = 0;
  auto wait_stage = [&](int s) -> bool {  // the MMAs that read operand stage s are done
    bool ok = true;
    if (s == 0 && pend0) { ok = mbar_wait(&mma_bar[0], mphase0); mphase0 ^= 1u; pend0 = false; }
    if (s == 1 && pend1) { ok = mbar_wait(&mma_bar[1], mphase1); mphase1 ^= 1u; pend1 = false; }
    return ok;
  };

  for (int G = s_next; G < G1;) {
    const int g0 = G * kMG;
    const int kn = min(kMG, a.g_end - g0);
    const int U = tc.cell_U[G];
    for (int i = t; i < kState * kMG; i += kTcThreads) {
      const int f = i / kMG, k = i - f * kMG;
      st[i] = k < kn ? gstate[static_cast<int64_t>(f) * a.n_gp + g0 + k] : 0.0f;
    }
    if (t <= kn) sptr[t] = a.ptr[g0 + t];
    for (int i = t; i < kMG * (kTcMaxU + 2); i += kTcThreads) (&pos[0][0])[i] = -1;
    __syncthreads();
    const int64_t q0 = sptr[0], q1 = sptr[kn];
    const int items = static_cast<int>(q1 - q0);
    for (int e = t; e < items; e += kTcThreads) {
      int k = 0;
      while (k + 1 < kn && sptr[k + 1] - q0 <= e) ++k;
      const int u = tc.nbr_u[q0 + e];
      if (u < kTcMaxU) pos[k][u] = static_cast<int16_t>(e);
    }
    // The cell's grad / Hessian Phi (bulk copies issued during the previous cell).
    const bool sok = mbar_wait(&stage_bar, sphase);
    if (__syncthreads_or(!sok)) { err = kErrStage; break; }
    sphase ^= 1u;
    stage_in_flight = false;
    {
      const float* sdp = reinterpret_cast<const float*>(s_d + (q0 * 8 - ((q0 * 8) & ~static_cast<int64_t>(15))));
      const float* sddp = reinterpret_cast<const float*>(s_dd + (q0 * 12 - ((q0 * 12) & ~static_cast<int64_t>(15))));
      // Records of every entry of the cell.
      for (int e = t; e < items; e += kTcThreads) {
        int k = 0;
        while (k + 1 < kn && sptr[k + 1] - q0 <= e) ++k;
        tc_record<BZERO>(st, k, m, sdp[2 * e], sdp[2 * e + 1], sddp[3 * e], sddp[3 * e + 1], sddp[3 * e + 2],
                         rec + e * RS);
      }
    }
    __syncthreads();
    // The staging buffers are free: start the next cell's copies.
    if (t == 0) {
      const int Gn = next_from(G + stride);
      s_next = Gn;
      if (Gn < G1) stage(Gn);
    }
    const int n3 = 3 * U;
    const int N = max(16, (n3 + 15) & ~15);
    const uint32_t idesc = umma::idesc_tf32(128, N);
    const int u_row = row / 3, r_row = row - 3 * (row / 3);
    bool failed = false;
    for (int k = 0; k < kn; ++k) {
      const int s = k & 1;
      // Operand stage s is free once the MMAs of point k - 2 are done.
      const bool ok = wait_stage(s);
      const int e = row < n3 ? pos[k][u_row] : -1;
      const float a1r = st[(S_A1 + r_row) * kMG + k], a2r = st[(S_A2 + r_row) * kMG + k];
      const float br = st[(S_B + r_row) * kMG + k];
      if (a_role) {
        // A row into tensor memory (every lane writes: zeros outside the point's support).
        float av[13];
        if (e >= 0) {
          tc_a_values(rec + e * RS, a1r, a2r, br, av);
        } else {
#pragma unroll
          for (int q = 0; q < 13; ++q) av[q] = 0.0f;
        }
        float A2[kTcK];
        tc_split<true>(av, A2);
        const uint32_t ta = tb + lane_base + kTcACol + static_cast<uint32_t>(kTcK * s);
#pragma unroll
        for (int c = 0; c < kTcK / 8; ++c) {
          const float v8[8] = {A2[8 * c], A2[8 * c + 1], A2[8 * c + 2], A2[8 * c + 3],
                               A2[8 * c + 4], A2[8 * c + 5], A2[8 * c + 6], A2[8 * c + 7]};
          umma::tmem_st8(ta + 8 * c, v8);
        }
        umma::tmem_st_wait();
      } else if (row < n3) {
        // B row into shared memory (rows outside the support zeroed once).
        bool& dirty = s == 0 ? dirty0 : dirty1;
        unsigned char* opB = opsB + s * kTcOpBytes;
        if (e >= 0 || dirty) {
          float bvals[13];
          if (e >= 0) {
            tc_b_values<BZERO>(rec + e * RS, a1r, a2r, br, bvals);
          } else {
#pragma unroll
            for (int q = 0; q < 13; ++q) bvals[q] = 0.0f;
          }
          float B2[kTcK];
          tc_split<false>(bvals, B2);
          const int base = ((row >> 3) * kTcChunks) * 128 + (row & 7) * 16;
#pragma unroll
          for (int c = 0; c < kTcChunks; ++c)
            *reinterpret_cast<float4*>(opB + base + c * 128) =
                make_float4(B2[4 * c], B2[4 * c + 1], B2[4 * c + 2], B2[4 * c + 3]);
          dirty = e >= 0;
        }
        umma::fence_proxy_async();
      }
      umma::fence_before_sync();
      if (__syncthreads_or(!ok)) { failed = true; break; }
      if (t == 0) {
        umma::fence_after_sync();
        const uint32_t b0 = umma::saddr(opsB + s * kTcOpBytes);
#pragma unroll
        for (int q = 0; q < kTcK / 8; ++q) {
          const uint64_t bd = umma::smem_desc(b0 + q * 256, 128, kTcChunks * 128);
          umma::mma_tf32_ta(tb, tb + kTcACol + static_cast<uint32_t>(kTcK * s + 8 * q), bd, idesc, k > 0 || q > 0);
        }
        umma::mma_commit(&mma_bar[s]);
      }
      if (s == 0) pend0 = true; else pend1 = true;
    }
    const bool d0 = wait_stage(0), d1 = wait_stage(1);
    const bool bad = __syncthreads_or(failed || !(d0 && d1));
    const int Gn = s_next;
    stage_in_flight = Gn < G1;
    if (bad) { err = kErrTensor; break; }
    umma::fence_after_sync();
    // Accumulator -> dense block matrix (rows of this warp's lanes, its half of the columns
    // [0, 3U)) in shared memory, over the B stages and the records (both dead now).
    {
      const int drow = 32 * (w & 3) + (t & 31);
      for (int c = 2 * (w >> 2); c < 2 * (w >> 2) + 2; ++c) {
        if (32 * c >= n3) break;   // warp-uniform
        uint32_t v[32];
        umma::tmem_ld32(tb + lane_base + static_cast<uint32_t>(32 * c), v);
        float4* dst = reinterpret_cast<float4*>(Dm + drow * kTcDStride + 32 * c);
#pragma unroll
        for (int q = 0; q < 8; ++q)
          dst[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]),
                               __uint_as_float(v[4 * q + 2]), __uint_as_float(v[4 * q + 3]));
      }
    }
    umma::fence_before_sync();
    __syncthreads();
    // Merged entries: block (row node, column node) = D[3 ul + r][3 uh + c].
    const int64_t e0 = mg.ent_ptr[G];
    const int ne = static_cast<int>(mg.ent_ptr[G + 1] - e0);
    float4* acc4 = static_cast<float4*>(a.Kacc);
    for (int e = t; e < ne; e += kTcThreads) {
      const unsigned uv = tc.ent_uv[e0 + e];
      const int ul = uv & 255u, uh = uv >> 8;
      const float* d0p = Dm + (3 * ul) * kTcDStride + 3 * uh;
      float v[9];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[3 * r + c] = d0p[r * kTcDStride + c];
      if constexpr (DET) {
        float* d = static_cast<float*>(a.Kc) + 9 * (e0 + e);
#pragma unroll
        for (int q = 0; q < 9; ++q) d[q] = v[q];
      } else {
        float4* d = acc4 + 3 * static_cast<int64_t>(mg.ent_slot[e0 + e]);
        atomicAdd(d, make_float4(v[0], v[1], v[2], v[3]));
        atomicAdd(d + 1, make_float4(v[4], v[5], v[6], v[7]));
        atomicAdd(d + 2, make_float4(v[8], 0.0f, 0.0f, 0.0f));
      }
    }
    __syncthreads();
    // The epilogue overwrote the B stages.
    dirty0 = true;
    dirty1 = true;
    G = Gn;
  }
  if (err) {
    // Let this CTA's copies and MMAs land (bounded) before its tensor memory is freed.
    if (t == 0) atomicOr(mg.err, err);
    wait_stage(0);
    wait_stage(1);
    if (t == 0 && stage_in_flight) mbar_wait(&stage_bar, sphase);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (w == 0) umma::tmem_dealloc(tb, kTcCols);
}
