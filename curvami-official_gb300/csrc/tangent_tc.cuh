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
// as 3xTF32 (A = Ah + Al, B = Bh + Bl, Ah Bh + Ah Bl + Al Bh, the Al Bl term dropped: about
// FP32 accuracy), i.e. K = 40 per point (13 + 13 + 13 + one zero), five 128 x N x 8 MMAs.
//
// Per CTA (128 threads, one per operand row, two CTAs per SM), per cell:
//  - the cell's point states (from the FP64 residual kernel) and, staged by a bulk copy
//    (TMA) completing on an mbarrier, its FP32 grad / Hessian Phi;
//  - per point k: the neighbour records (threads i < n), then every thread writes its row
//    of A_k and B_k (hi / lo split) into one of two operand stages in the canonical K-major
//    no-swizzle layout, and one thread issues the five MMAs and commits them to the stage's
//    mbarrier; the stage is rewritten two points later, after that mbarrier;
//  - after the last point: the accumulator (128 lanes x 3U columns of tensor memory) goes to
//    a dense matrix in shared memory (over the operand stages), and each merged entry of the
//    cell (a distinct 3x3 block of K, from the merge tables) is read from it and scattered
//    with three 16-byte FP32 vector atomics (or stored, deterministic mode).
// Every wait is bounded (about one second of SM clock); a CTA that gives up records bit 16
// (or bit 4 for the staging copy) in the device error word, lets its copies and MMAs land
// (bounded), frees its tensor memory and returns.

constexpr int kTcThreads = 128;
constexpr int kTcMaxU = kTcMaxUnion;         // 42: 3 U <= 126 rows of one M = 128 tile
constexpr int kTcK = 40;                     // per point: 13 + 13 + 13 values + one zero
constexpr int kTcChunks = kTcK / 4;          // 16-byte chunks of an operand row
constexpr int kTcOpBytes = 128 * kTcK * 4;   // one operand of one point: 20,480 bytes
constexpr int kTcOpsBytes = 4 * kTcOpBytes;  // two stages x (A, B)
constexpr int kTcRec = 36;                   // floats per neighbour record (34 used)
constexpr int kTcDStride = 132;              // floats per row of the epilogue's dense matrix
constexpr int kErrTensor = 16;               // device error word: an MMA completion never came
constexpr uint32_t kTcCols = 128;            // tensor-memory columns of the accumulator

static_assert(128 * kTcDStride * 4 <= kTcOpsBytes, "the epilogue matrix must fit over the operand stages");

struct TcArgs {
  const uint8_t* nbr_u;    // per face entry: its node's index in the cell's sorted union
  const int16_t* cell_U;   // per group: union size (above kTcMaxU: not on this path)
  const uint16_t* ent_uv;  // per merged entry: union index of its row node | its column node << 8
};

__host__ __device__ inline size_t tc_smem_bytes(int nmax) {
  const size_t E = static_cast<size_t>(kMG) * nmax;
  return kTcOpsBytes + (static_cast<size_t>(kState) * kMG + 2 * static_cast<size_t>(nmax) * kTcRec) * sizeof(float) +
         (20 * E + 64);
}

// One neighbour record: I side dx dy Tu c0 c1 beta0 beta1 beta2; J side the frame
// coefficients (on a1, a2, b) of the R vectors paired with (a1,dx) (a1,dy) (a2,dx) (a2,dy),
// Q0 Q1 Q2, then -cW0, -cW1, bv cW0 + nW0, bv cW1 + nW1, -TuW (W = Gauss weight).
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
  float pa[3], pb[3], pc[3], qa[3], qb[3], qc[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    pa[r] = (m.Ai<float>(3 * r) * dx + m.Ai<float>(3 * r + 2) * dy) * Wt;
    pb[r] = (m.Ai<float>(3 * r + 1) * dy + m.Ai<float>(3 * r + 2) * dx) * Wt;
    qc[r] = (m.Di<float>(3 * r) * b0 + m.Di<float>(3 * r + 1) * b1 + m.Di<float>(3 * r + 2) * b2) * Wt;
    if constexpr (BZERO) {
      pc[r] = 0.0f; qa[r] = 0.0f; qb[r] = 0.0f;
    } else {
      pc[r] = (m.Bi<float>(3 * r) * b0 + m.Bi<float>(3 * r + 1) * b1 + m.Bi<float>(3 * r + 2) * b2) * Wt;
      qa[r] = (m.Bi<float>(3 * r) * dx + m.Bi<float>(3 * r + 2) * dy) * Wt;
      qb[r] = (m.Bi<float>(3 * r + 1) * dy + m.Bi<float>(3 * r + 2) * dx) * Wt;
    }
  }
  const float cW0 = c0 * Wt, cW1 = c1 * Wt;
  const float nW0 = (Nt[0] * dx + Nt[2] * dy) * Wt, nW1 = (Nt[2] * dx + Nt[1] * dy) * Wt;
  R[0] = dx; R[1] = dy; R[2] = Tu; R[3] = c0; R[4] = c1; R[5] = b0; R[6] = b1; R[7] = b2;
  // (a1, dx): P0 + geo G(0, .)    (a1, dy): P2 + geo G(0, .)
  R[8] = pa[0] + Ci[0] * nW0;  R[9] = pb[0] + Ci[1] * nW0;  R[10] = pc[0];
  R[11] = pa[2] + Ci[0] * nW1; R[12] = pb[2] + Ci[1] * nW1; R[13] = pc[2];
  // (a2, dx): P2 + geo G(1, .)    (a2, dy): P1 + geo G(1, .)
  R[14] = pa[2] + Ci[2] * nW0; R[15] = pb[2] + Ci[3] * nW0; R[16] = pc[2];
  R[17] = pa[1] + Ci[2] * nW1; R[18] = pb[1] + Ci[3] * nW1; R[19] = pc[1];
  // (b, beta_r): Q_r
#pragma unroll
  for (int r = 0; r < 3; ++r) { R[20 + 3 * r] = qa[r]; R[21 + 3 * r] = qb[r]; R[22 + 3 * r] = qc[r]; }
  R[29] = -cW0; R[30] = -cW1;
  R[31] = bv * cW0 + nW0; R[32] = bv * cW1 + nW1;
  R[33] = -Tu * Wt;
}

// Row t of A_k and B_k: node u = t / 3 of the union, component r = t % 3, neighbour i of
// point k (or none: zeros), written as 10 chunks of 16 bytes into the core-matrix layout
// (core matrix (t / 8, chunk) at ((t / 8) * 10 + chunk) * 128 bytes, row t % 8 within it).
__device__ __forceinline__ void tc_write_row(unsigned char* opA, unsigned char* opB, int t, const float* R, float a1r,
                                             float a2r, float br) {
  float av[13], bv[13];
  if (R) {
    const float dx = R[0], dy = R[1], Tu = R[2];
    av[0] = a1r * dx; av[1] = a1r * dy; av[2] = a1r * Tu;
    av[3] = a2r * dx; av[4] = a2r * dy; av[5] = a2r * Tu;
    av[6] = br * R[3]; av[7] = br * R[4];
    av[8] = br * R[5]; av[9] = br * R[6]; av[10] = br * R[7];
    av[11] = br * dx; av[12] = br * dy;
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
  } else {
#pragma unroll
    for (int q = 0; q < 13; ++q) { av[q] = 0.0f; bv[q] = 0.0f; }
  }
  // 3xTF32: A' = [Ah | Ah | Al | 0], B' = [Bh | Bl | Bh | 0].
  float A2[kTcK], B2[kTcK];
#pragma unroll
  for (int q = 0; q < 13; ++q) {
    const float ah = umma::to_tf32(av[q]), bh = umma::to_tf32(bv[q]);
    A2[q] = ah; A2[13 + q] = ah; A2[26 + q] = av[q] - ah;
    B2[q] = bh; B2[13 + q] = bv[q] - bh; B2[26 + q] = bh;
  }
  A2[39] = 0.0f; B2[39] = 0.0f;
  const int base = ((t >> 3) * kTcChunks) * 128 + (t & 7) * 16;
#pragma unroll
  for (int c = 0; c < kTcChunks; ++c) {
    *reinterpret_cast<float4*>(opA + base + c * 128) = make_float4(A2[4 * c], A2[4 * c + 1], A2[4 * c + 2], A2[4 * c + 3]);
    *reinterpret_cast<float4*>(opB + base + c * 128) = make_float4(B2[4 * c], B2[4 * c + 1], B2[4 * c + 2], B2[4 * c + 3]);
  }
}

template <bool BZERO, bool DET>
__global__ void __launch_bounds__(kTcThreads, 2) face_tangent_tc_kernel(FaceArgs a, const float* __restrict__ gstate,
                                                                       MergeArgs mg, TcArgs tc) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ __align__(8) uint64_t stage_bar;
  __shared__ __align__(8) uint64_t mma_bar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int64_t sptr[kMG + 1];
  __shared__ int8_t pos[kMG][kTcMaxU + 2];
  __shared__ int s_next;
  const int t = threadIdx.x, w = t >> 5;
  const int nmax = a.nmax;
  const int E = kMG * nmax;
  unsigned char* ops = tsm;
  float* st = reinterpret_cast<float*>(tsm + kTcOpsBytes);  // [kState][kMG]
  float* rec = st + kState * kMG;                           // [2][nmax][kTcRec]
  unsigned char* s_d = reinterpret_cast<unsigned char*>(rec + 2 * nmax * kTcRec);
  unsigned char* s_dd = s_d + 8 * E + 32;
  float* Dm = reinterpret_cast<float*>(tsm);                // epilogue, over the operand stages
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
  uint32_t sphase = 0, mphase0 = 0, mphase1 = 0;
  bool pend0 = false, pend1 = false;   // a commit on the stage's mbarrier not waited for yet
  bool dirty0 = true, dirty1 = true;   // this thread's row of the stage may hold nonzeros
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
    for (int64_t e = q0 + t; e < q1; e += kTcThreads) {
      int k = 0;
      while (k + 1 < kn && sptr[k + 1] <= e) ++k;
      const int u = tc.nbr_u[e];
      if (u < kTcMaxU) pos[k][u] = static_cast<int8_t>(e - sptr[k]);
    }
    // The cell's grad / Hessian Phi (bulk copies issued during the previous cell).
    const bool sok = mbar_wait(&stage_bar, sphase);
    if (__syncthreads_or(!sok)) { err = kErrStage; break; }
    sphase ^= 1u;
    stage_in_flight = false;
    const float* sdp = reinterpret_cast<const float*>(s_d + (q0 * 8 - ((q0 * 8) & ~static_cast<int64_t>(15))));
    const float* sddp = reinterpret_cast<const float*>(s_dd + (q0 * 12 - ((q0 * 12) & ~static_cast<int64_t>(15))));
    const int n3 = 3 * U;
    const int N = max(16, (n3 + 15) & ~15);
    const uint32_t idesc = umma::idesc_tf32(128, N);
    const int u_row = t / 3, r_row = t - 3 * (t / 3);
    bool failed = false;
    for (int k = 0; k < kn; ++k) {
      const int s = k & 1;
      float* R = rec + s * nmax * kTcRec;
      const int64_t p0 = sptr[k];
      const int n = static_cast<int>(sptr[k + 1] - p0);
      for (int i = t; i < n; i += kTcThreads) {
        const int64_t e = p0 + i - q0;
        tc_record<BZERO>(st, k, m, sdp[2 * e], sdp[2 * e + 1], sddp[3 * e], sddp[3 * e + 1], sddp[3 * e + 2],
                         R + i * kTcRec);
      }
      // Operand stage s is free once the MMAs of point k - 2 are done.
      const bool ok = wait_stage(s);
      if (__syncthreads_or(!ok)) { failed = true; break; }
      unsigned char* opA = ops + s * 2 * kTcOpBytes;
      unsigned char* opB = opA + kTcOpBytes;
      bool& dirty = s == 0 ? dirty0 : dirty1;
      if (t < n3) {
        const int i = pos[k][u_row];
        if (i >= 0) {
          const float a1r = st[(S_A1 + r_row) * kMG + k], a2r = st[(S_A2 + r_row) * kMG + k];
          const float br = st[(S_B + r_row) * kMG + k];
          tc_write_row(opA, opB, t, R + i * kTcRec, a1r, a2r, br);
          dirty = true;
        } else if (dirty) {
          tc_write_row(opA, opB, t, nullptr, 0.0f, 0.0f, 0.0f);
          dirty = false;
        }
      }
      umma::fence_proxy_async();
      __syncthreads();
      if (t == 0) {
        umma::fence_after_sync();
        const uint32_t a0 = umma::saddr(opA), b0 = umma::saddr(opB);
#pragma unroll
        for (int q = 0; q < kTcK / 8; ++q) {
          const uint64_t ad = umma::smem_desc(a0 + q * 256, 128, kTcChunks * 128);
          const uint64_t bd = umma::smem_desc(b0 + q * 256, 128, kTcChunks * 128);
          umma::mma_tf32(tb, ad, bd, idesc, k > 0 || q > 0);
        }
        umma::mma_commit(&mma_bar[s]);
      }
      if (s == 0) pend0 = true; else pend1 = true;
    }
    if (failed) { err = kErrTensor; break; }
    // The staging buffers are free: start the next cell's copies.
    if (t == 0) {
      const int Gn = next_from(G + stride);
      s_next = Gn;
      if (Gn < G1) stage(Gn);
    }
    const bool d0 = wait_stage(0), d1 = wait_stage(1);
    const bool bad = __syncthreads_or(!(d0 && d1));
    const int Gn = s_next;
    stage_in_flight = Gn < G1;
    if (bad) { err = kErrTensor; break; }
    umma::fence_after_sync();
    // Accumulator -> dense block matrix (rows t, columns [0, 3U)) in shared memory.
    const int nch = (n3 + 31) / 32;
    for (int c = 0; c < nch; ++c) {
      uint32_t v[32];
      umma::tmem_ld32(tb + (static_cast<uint32_t>(32 * w) << 16) + static_cast<uint32_t>(32 * c), v);
      float4* drow = reinterpret_cast<float4*>(Dm + t * kTcDStride + 32 * c);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        drow[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]), __uint_as_float(v[4 * q + 2]),
                              __uint_as_float(v[4 * q + 3]));
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
    // The epilogue overwrote the operand stages.
    dirty0 = true;
    dirty1 = true;
    umma::fence_after_sync();
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
