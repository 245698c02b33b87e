// pattern.cu — symbolic phase on sm_103a: the block-upper sparsity pattern of K, the
// Gauss-point -> block-slot map, and the ordered contribution lists of the
// deterministic scatter.
//
// Reference: NonLinearAssembler::initSparsityPattern (plate/Assembly.h:59-153) and the
// pattern growth of K += K_fold (plate/Meshless.h:113-127, Constraints.h:420-433).
//
// Column j of the block pattern is the sorted set of nodes i <= j that share a
// neighbour list with j. "Neighbour lists" are the face Gauss points' lists plus, for
// the hinge, each crease point's merged left/right node list (the hinge couples every
// node pair of that merged list). One warp builds one column: it walks the lists that
// contain j (node -> list inverse index), inserts every i <= j into a shared-memory hash
// set, then sorts the set by ranks. The result is the same sorted unique set the
// reference builds with sort + unique, so the pattern is bit-exact.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>

#include "cgb_device.cuh"
#include "cgb_internal.h"

namespace cgb {
namespace {

constexpr int kWarps = 2;
constexpr int kCap = 2048;        // hash slots per warp (8 KB)
constexpr int kMaxColumn = 1536;  // largest column the hash set accepts (75 % load)

enum : int { kErrCapacity = CGB_ERR_CAPACITY, kErrMapping = CGB_ERR_MAPPING };

// A set of lists in CSR form (face Gauss points, then crease points).
struct Lists {
  int n;
  const int64_t* ptr;
  const int32_t* idx;
};

__global__ void count_per_node(int64_t n, const int32_t* __restrict__ idx, int32_t* __restrict__ cnt) {
  const int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (e < n) atomicAdd(&cnt[idx[e]], 1);
}

// inv[cursor[node]++] = list id (+ base), one thread per list.
__global__ void fill_inverse(Lists L, int base, int64_t* __restrict__ cursor, int32_t* __restrict__ inv) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= L.n) return;
  for (int64_t e = L.ptr[g]; e < L.ptr[g + 1]; ++e) {
    const int64_t at = atomicAdd(reinterpret_cast<unsigned long long*>(&cursor[L.idx[e]]), 1ULL);
    inv[at] = base + g;
  }
}

__device__ __forceinline__ unsigned hash32(unsigned x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}

// Column sets. Phase 0 counts, phase 1 writes the sorted column into col_nodes.
__global__ void __launch_bounds__(32 * kWarps) column_kernel(int n_nodes, Lists A, Lists B,
                                                              const int64_t* __restrict__ inv_ptr,
                                                              const int32_t* __restrict__ inv,
                                                              int phase, int32_t* __restrict__ col_len,
                                                              const int64_t* __restrict__ col_ptr,
                                                              int32_t* __restrict__ col_nodes, int* err) {
  __shared__ int table[kWarps][kCap];
  __shared__ int keys[kWarps][kMaxColumn];
  __shared__ int count[kWarps];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* T = table[w];
  for (int j = blockIdx.x * kWarps + w; j < n_nodes; j += gridDim.x * kWarps) {
    for (int s = lane; s < kCap; s += 32) T[s] = -1;
    if (lane == 0) count[w] = 0;
    __syncwarp();
    bool overflow = false;
    for (int64_t q = inv_ptr[j]; q < inv_ptr[j + 1]; ++q) {
      const int lid = inv[q];
      const Lists& L = lid < A.n ? A : B;
      const int li = lid < A.n ? lid : lid - A.n;
      const int64_t e0 = L.ptr[li], e1 = L.ptr[li + 1];
      for (int64_t e = e0 + lane; e < e1; e += 32) {
        const int i = L.idx[e];
        if (i > j) continue;
        unsigned h = hash32(static_cast<unsigned>(i)) & (kCap - 1);
        for (int probe = 0; probe < kCap; ++probe) {
          const int prev = atomicCAS(&T[h], -1, i);
          if (prev == -1) {
            const int at = atomicAdd(&count[w], 1);
            if (at < kMaxColumn) keys[w][at] = i; else overflow = true;
            break;
          }
          if (prev == i) break;
          h = (h + 1) & (kCap - 1);
        }
      }
    }
    __syncwarp();
    const int m = count[w];
    if (__any_sync(0xffffffffu, overflow) || m > kMaxColumn) {
      if (lane == 0) dev_fail(err, kErrCapacity);
      continue;
    }
    if (phase == 0) {
      if (lane == 0) col_len[j] = m;
    } else {
      const int64_t base = col_ptr[j];
      for (int a = lane; a < m; a += 32) {
        const int v = keys[w][a];
        int rank = 0;
        for (int b = 0; b < m; ++b) rank += (keys[w][b] < v);
        col_nodes[base + rank] = v;
      }
    }
    __syncwarp();
  }
}

// Face Gauss point -> block slot of each local pair (i <= j), in the reference's loop
// order (plate/Assembly.h:128-143). One warp per Gauss point.
__global__ void slot_map_kernel(int n_gp, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                const int64_t* __restrict__ map_ptr, const int64_t* __restrict__ col_ptr,
                                const int32_t* __restrict__ col_nodes, int32_t* __restrict__ slot, int* err) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t g = warp; g < n_gp; g += nwarps) {
    const int64_t p0 = ptr[g];
    const int n = static_cast<int>(ptr[g + 1] - p0);
    const int64_t np = static_cast<int64_t>(n) * (n + 1) / 2;
    const int64_t m0 = map_ptr[g];
    // pair p -> (i, j): walk rows of length n - i.
    int i = 0, off = lane;
    while (i < n && off >= n - i) { off -= n - i; ++i; }
    for (int64_t p = lane; p < np; p += 32) {
      const int j = i + off;
      const int ni = idx[p0 + i], nj = idx[p0 + j];
      const int lo = ni < nj ? ni : nj, hi = ni < nj ? nj : ni;
      int64_t a = col_ptr[hi], b = col_ptr[hi + 1];
      while (a < b) {
        const int64_t mid = (a + b) >> 1;
        if (col_nodes[mid] < lo) a = mid + 1; else b = mid;
      }
      int32_t s = -1;
      if (a < col_ptr[hi + 1] && col_nodes[a] == lo) s = static_cast<int32_t>(a);
      else dev_fail(err, kErrMapping);
      slot[m0 + p] = s;
      off += 32;
      while (i < n && off >= n - i) { off -= n - i; ++i; }
    }
  }
}

// CSR fill of the deterministic lists: one thread per contribution id.
__global__ void count_slots(int64_t n, const int32_t* __restrict__ key, int64_t* __restrict__ cnt) {
  const int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (q < n) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[key[q]]), 1ULL);
}
__global__ void fill_slots(int64_t n, int64_t base, const int32_t* __restrict__ key, int64_t* __restrict__ cursor,
                           int64_t* __restrict__ list) {
  const int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (q < n) {
    const int64_t at = atomicAdd(reinterpret_cast<unsigned long long*>(&cursor[key[q]]), 1ULL);
    list[at] = base + q;
  }
}
// Sort each list ascending (insertion sort: lists are short and this runs once).
__global__ void sort_lists(int64_t n, const int64_t* __restrict__ lptr, int64_t* __restrict__ list) {
  const int64_t b = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (b >= n) return;
  const int64_t s = lptr[b], e = lptr[b + 1];
  for (int64_t k = s + 1; k < e; ++k) {
    const int64_t v = list[k];
    int64_t m = k - 1;
    while (m >= s && list[m] > v) { list[m + 1] = list[m]; --m; }
    list[m + 1] = v;
  }
}

// ---- merged contributions for the FP32 tangent ---------------------------------------
// A group is kMergeGroup consecutive face Gauss points (one quadrature cell with a 4x4 rule).
// Its pairs are sorted by (block slot, point, i, j); each distinct slot is an entry whose
// contributions are summed in registers before one scatter. Entries are ordered by
// contribution count, descending (stable), so the threads of a warp get similar loops.
// Contribution code: point k (4 bits) | local i (6 bits) | local j (6 bits).
constexpr int kMergeGroup = 16;
constexpr int kMergeItems = 16384;  // sortable pairs per group (8-byte keys, 128 KB)

__global__ void __launch_bounds__(256) merge_groups_kernel(int n_gp, const int64_t* __restrict__ ptr,
                                                          const int32_t* __restrict__ idx,
                                                          const int64_t* __restrict__ map_ptr,
                                                          const int32_t* __restrict__ map_slot, int phase,
                                                          int32_t* __restrict__ ent_count,
                                                          const int64_t* __restrict__ ent_ptr,
                                                          int32_t* __restrict__ ent_slot,
                                                          int32_t* __restrict__ ent_cstart,
                                                          uint16_t* __restrict__ con_code) {
  extern __shared__ unsigned long long mkeys[];
  __shared__ int hist[kMergeGroup + 2];
  __shared__ int n_ent;
  const int G = blockIdx.x;
  const int g0 = G * kMergeGroup, g1 = min(n_gp, g0 + kMergeGroup);
  const int64_t q0 = map_ptr[g0], q1 = map_ptr[g1];
  const int items = static_cast<int>(q1 - q0);
  bool ok = items <= kMergeItems;
  for (int k = 0; k < g1 - g0; ++k) ok = ok && (ptr[g0 + k + 1] - ptr[g0 + k] <= 64);
  if (!ok) {  // the group scatters directly (count -1)
    if (phase == 0 && threadIdx.x == 0) ent_count[G] = -1;
    return;
  }
  // Keys: slot (high 32 bits) | k i j (low 16 bits); pairs walked point by point. The
  // local pair is written row node first (i and j swapped when node(i) > node(j)), so the
  // tangent evaluates the block in its stored orientation, K_{min,max}, and needs no
  // transpose (the pair blocks are symmetric: K_ji = K_ij^T).
  for (int k = 0; k < g1 - g0; ++k) {
    const int64_t p0 = ptr[g0 + k];
    const int n = static_cast<int>(ptr[g0 + k + 1] - p0);
    const int64_t m0 = map_ptr[g0 + k] - q0;
    const int np = n * (n + 1) / 2;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
      int i = 0, off = p;
      while (off >= n - i) { off -= n - i; ++i; }
      int j = i + off;
      int ii = i;
      if (idx[p0 + i] > idx[p0 + j]) { ii = j; j = i; }
      const unsigned code = (static_cast<unsigned>(k) << 12) | (static_cast<unsigned>(ii) << 6) | static_cast<unsigned>(j);
      mkeys[m0 + p] = (static_cast<unsigned long long>(static_cast<unsigned>(map_slot[q0 + m0 + p])) << 16) | code;
    }
  }
  int n2 = 1;
  while (n2 < items) n2 <<= 1;
  for (int t = items + threadIdx.x; t < n2; t += blockDim.x) mkeys[t] = ~0ULL;
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const bool up = (t & k) == 0;
          const unsigned long long a = mkeys[t], b = mkeys[u];
          if ((a > b) == up) { mkeys[t] = b; mkeys[u] = a; }
        }
      }
      __syncthreads();
    }
  }
  // Entry heads: position t starts an entry when its slot differs from t - 1.
  if (threadIdx.x == 0) n_ent = 0;
  __syncthreads();
  for (int t = threadIdx.x; t < items; t += blockDim.x)
    if (t == 0 || (mkeys[t] >> 16) != (mkeys[t - 1] >> 16)) atomicAdd(&n_ent, 1);
  __syncthreads();
  const int m = n_ent;
  if (phase == 0) {
    if (threadIdx.x == 0) ent_count[G] = m;
    return;
  }
  if (ent_ptr[G + 1] - ent_ptr[G] != m) return;
  // Per entry: start (rank among heads, by a serial scan over the sorted keys is avoided:
  // each head counts the heads before it with a parallel prefix over positions).
  // Reuse the key array's tail (beyond n2) is not possible in general, so write the codes
  // in sorted order first, then the entry table.
  const int64_t c0 = q0;  // contribution base of this group
  for (int t = threadIdx.x; t < items; t += blockDim.x) con_code[c0 + t] = static_cast<uint16_t>(mkeys[t] & 0xffff);
  // Entry start positions and counts, then a stable counting sort of the entries by count.
  // Thread 0 walks the sorted keys (items <= 16384): the entry table is small.
  if (threadIdx.x == 0) {
    for (int c = 0; c < kMergeGroup + 2; ++c) hist[c] = 0;
    int e = 0, start = 0;
    for (int t = 1; t <= items; ++t) {
      if (t == items || (mkeys[t] >> 16) != (mkeys[t - 1] >> 16)) {
        const int cnt = t - start;
        hist[cnt > kMergeGroup ? kMergeGroup : cnt]++;  // counts <= points per group
        // temporarily store (start, slot) at the entry's unsorted index
        ent_cstart[ent_ptr[G] + e] = start;
        ent_slot[ent_ptr[G] + e] = static_cast<int32_t>(mkeys[start] >> 16);
        ++e;
        start = t;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // Descending count order: offsets for count = 16, 15, ..., 1.
    int acc = 0;
    int off[kMergeGroup + 1];
    for (int c = kMergeGroup; c >= 1; --c) { off[c] = acc; acc += hist[c]; }
    // Stable placement needs the unsorted table; copy it through the key array (no longer used).
    int* tmp = reinterpret_cast<int*>(mkeys);
    for (int e = 0; e < m; ++e) { tmp[2 * e] = ent_cstart[ent_ptr[G] + e]; tmp[2 * e + 1] = ent_slot[ent_ptr[G] + e]; }
    for (int e = 0; e < m; ++e) {
      const int start = tmp[2 * e];
      const int end = (e + 1 < m) ? tmp[2 * e + 2] : items;
      int cnt = end - start;
      if (cnt > kMergeGroup) cnt = kMergeGroup;
      const int at = off[cnt]++;
      ent_cstart[ent_ptr[G] + at] = (cnt << 16) | start;  // count in the high half
      ent_slot[ent_ptr[G] + at] = tmp[2 * e + 1];
    }
  }
}

inline unsigned nb(int64_t n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

int read_err(cgb_context* ctx) {
  int e = 0;
  CGB_CUDA(cudaMemcpyAsync(&e, ctx->dev_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CGB_CUDA(cudaStreamSynchronize(ctx->stream));
  return e;
}

}  // namespace

void pattern_build(cgb_assembler* a) {
  cgb_context* ctx = a->ctx;
  cudaStream_t st = ctx->stream;
  const cgb_shape* F = a->faces;
  const int n_nodes = a->n_nodes;
  CGB_CUDA(cudaMemsetAsync(ctx->dev_err.p, 0, sizeof(int), st));

  // ---- hinge lists: merged sorted node lists of every crease point (host) ----
  std::vector<int64_t> hptr(1, 0);
  std::vector<int32_t> hidx;
  for (auto& f : a->folds) {
    std::vector<int64_t> lp(f.n_gp + 1), rp(f.n_gp + 1);
    CGB_CUDA(cudaMemcpyAsync(lp.data(), f.left->nbr_ptr.p, lp.size() * 8, cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaMemcpyAsync(rp.data(), f.right->nbr_ptr.p, rp.size() * 8, cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    std::vector<int32_t> li(std::max<int64_t>(lp.back(), 1)), ri(std::max<int64_t>(rp.back(), 1));
    if (lp.back()) CGB_CUDA(cudaMemcpyAsync(li.data(), f.left->nbr_idx.p, lp.back() * 4, cudaMemcpyDeviceToHost, st));
    if (rp.back()) CGB_CUDA(cudaMemcpyAsync(ri.data(), f.right->nbr_idx.p, rp.back() * 4, cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    std::vector<int64_t> uptr(f.n_gp + 1, 0);
    std::vector<int32_t> unode, lpos(std::max<int64_t>(lp.back(), 1)), rpos(std::max<int64_t>(rp.back(), 1));
    std::vector<int32_t> tmp;
    f.max_u = 0;
    for (int g = 0; g < f.n_gp; ++g) {
      tmp.clear();
      for (int64_t e = lp[g]; e < lp[g + 1]; ++e) tmp.push_back(li[e]);
      for (int64_t e = rp[g]; e < rp[g + 1]; ++e) tmp.push_back(ri[e]);
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      for (int64_t e = lp[g]; e < lp[g + 1]; ++e)
        lpos[e] = static_cast<int32_t>(std::lower_bound(tmp.begin(), tmp.end(), li[e]) - tmp.begin());
      for (int64_t e = rp[g]; e < rp[g + 1]; ++e)
        rpos[e] = static_cast<int32_t>(std::lower_bound(tmp.begin(), tmp.end(), ri[e]) - tmp.begin());
      unode.insert(unode.end(), tmp.begin(), tmp.end());
      uptr[g + 1] = uptr[g] + static_cast<int64_t>(tmp.size());
      f.max_u = std::max<int>(f.max_u, static_cast<int>(tmp.size()));
      hidx.insert(hidx.end(), tmp.begin(), tmp.end());
      hptr.push_back(hptr.back() + static_cast<int64_t>(tmp.size()));
    }
    f.n_u = uptr[f.n_gp];
    upload(f.u_ptr, uptr.data(), uptr.size(), st);
    upload(f.u_node, unode.data(), unode.size(), st);
    upload(f.l_pos, lpos.data(), lpos.size(), st);
    upload(f.r_pos, rpos.data(), rpos.size(), st);
    CGB_CUDA(cudaStreamSynchronize(st));
  }
  const int n_hl = static_cast<int>(hptr.size() - 1);
  DevBuf<int64_t> d_hptr;
  DevBuf<int32_t> d_hidx;
  upload(d_hptr, hptr.data(), hptr.size(), st);
  upload(d_hidx, hidx.data(), hidx.size(), st);

  // ---- node -> list inverse index ----
  DevBuf<int32_t> cnt(n_nodes);
  CGB_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), st));
  if (F->nnz) count_per_node<<<nb(F->nnz, 256), 256, 0, st>>>(F->nnz, F->nbr_idx.p, cnt.p);
  if (!hidx.empty()) count_per_node<<<nb(hidx.size(), 256), 256, 0, st>>>(hidx.size(), d_hidx.p, cnt.p);
  CGB_CUDA(cudaGetLastError());
  std::vector<int32_t> hc(n_nodes);
  CGB_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, cnt.bytes(), cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> inv_ptr(n_nodes + 1, 0);
  for (int j = 0; j < n_nodes; ++j) inv_ptr[j + 1] = inv_ptr[j] + hc[j];
  DevBuf<int64_t> d_inv_ptr, cursor;
  upload(d_inv_ptr, inv_ptr.data(), inv_ptr.size(), st);
  upload(cursor, inv_ptr.data(), n_nodes, st);
  DevBuf<int32_t> inv(inv_ptr.back());
  Lists LA{F->n_gp, F->nbr_ptr.p, F->nbr_idx.p};
  Lists LB{n_hl, d_hptr.p, d_hidx.p};
  if (LA.n) fill_inverse<<<nb(LA.n, 128), 128, 0, st>>>(LA, 0, cursor.p, inv.p);
  if (LB.n) fill_inverse<<<nb(LB.n, 128), 128, 0, st>>>(LB, LA.n, cursor.p, inv.p);
  CGB_CUDA(cudaGetLastError());

  // ---- columns: count, scan, fill ----
  DevBuf<int32_t> col_len(n_nodes);
  const unsigned cgrid = std::max(1u, std::min(nb(n_nodes, kWarps), 152u * 16u));
  column_kernel<<<cgrid, 32 * kWarps, 0, st>>>(n_nodes, LA, LB, d_inv_ptr.p, inv.p, 0, col_len.p, nullptr,
                                              nullptr, ctx->dev_err.p);
  CGB_CUDA(cudaGetLastError());
  if (int e = read_err(ctx))
    throw Error(e, "initSparsityPattern: a column of the node pattern has more than 1536 block rows");
  std::vector<int32_t> hl(n_nodes);
  CGB_CUDA(cudaMemcpyAsync(hl.data(), col_len.p, col_len.bytes(), cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> cptr(n_nodes + 1, 0);
  for (int j = 0; j < n_nodes; ++j) cptr[j + 1] = cptr[j] + hl[j];
  a->n_blocks = cptr[n_nodes];
  if (9 * a->n_blocks >= (1LL << 31))
    throw Error(CGB_ERR_CAPACITY, "initSparsityPattern: nnz(K) exceeds the int32 index range of the reference's K");
  upload(a->col_ptr, cptr.data(), cptr.size(), st);
  a->col_nodes.alloc(a->n_blocks);
  column_kernel<<<cgrid, 32 * kWarps, 0, st>>>(n_nodes, LA, LB, d_inv_ptr.p, inv.p, 1, col_len.p, a->col_ptr.p,
                                              a->col_nodes.p, ctx->dev_err.p);
  CGB_CUDA(cudaGetLastError());
  // Scalar CSC outer index (Assembly.h:103-107): column 3j+c starts at
  // 9 col_ptr[j] + 3 c len_j.
  std::vector<int32_t> outer(3 * static_cast<size_t>(n_nodes) + 1);
  for (int j = 0; j < n_nodes; ++j)
    for (int c = 0; c < 3; ++c) outer[3 * j + c] = static_cast<int32_t>(9 * cptr[j] + 3 * c * hl[j]);
  outer[3 * n_nodes] = static_cast<int32_t>(9 * cptr[n_nodes]);
  upload(a->outer, outer.data(), outer.size(), st);

  // ---- face slot map ----
  std::vector<int64_t> fptr(F->n_gp + 1);
  CGB_CUDA(cudaMemcpyAsync(fptr.data(), F->nbr_ptr.p, fptr.size() * 8, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> mptr(F->n_gp + 1, 0);
  for (int g = 0; g < F->n_gp; ++g) {
    const int64_t n = fptr[g + 1] - fptr[g];
    mptr[g + 1] = mptr[g] + n * (n + 1) / 2;
  }
  a->n_pairs = mptr[F->n_gp];
  upload(a->map_ptr, mptr.data(), mptr.size(), st);
  a->map_slot.alloc(a->n_pairs);
  if (F->n_gp)
    slot_map_kernel<<<std::min<int64_t>(nb(F->n_gp, 8), 152 * 64), 256, 0, st>>>(
        F->n_gp, F->nbr_ptr.p, F->nbr_idx.p, a->map_ptr.p, a->col_ptr.p, a->col_nodes.p, a->map_slot.p,
        ctx->dev_err.p);
  CGB_CUDA(cudaGetLastError());
  if (int e = read_err(ctx)) {
    if (e == CGB_ERR_MAPPING)
      throw Error(e, "Assembly: Gauss-point neighbour missing from the sparsity pattern; "
                     "CSR mapping is inconsistent.");
    throw Error(e, "initSparsityPattern: device check failed");
  }

  // ---- hinge pair slots (host: crease points are few) ----
  if (!a->folds.empty()) {
    std::vector<int32_t> hcn(a->n_blocks);
    CGB_CUDA(cudaMemcpyAsync(hcn.data(), a->col_nodes.p, hcn.size() * 4, cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaStreamSynchronize(st));
    int64_t hoff = 0;
    for (auto& f : a->folds) {
      std::vector<int64_t> pp(f.n_gp + 1, 0);
      std::vector<int32_t> ps;
      for (int g = 0; g < f.n_gp; ++g) {
        const int64_t u0 = hptr[hoff + g], u1 = hptr[hoff + g + 1];
        for (int64_t P = u0; P < u1; ++P)
          for (int64_t Q = P; Q < u1; ++Q) {
            const int lo = hidx[P], hi = hidx[Q];
            auto b0 = hcn.begin() + cptr[hi], b1 = hcn.begin() + cptr[hi + 1];
            auto it = std::lower_bound(b0, b1, lo);
            if (it == b1 || *it != lo)
              throw Error(CGB_ERR_MAPPING, "Assembly: hinge block missing from the sparsity pattern");
            ps.push_back(static_cast<int32_t>(it - hcn.begin()));
          }
        pp[g + 1] = static_cast<int64_t>(ps.size());
      }
      hoff += f.n_gp;
      f.n_pairs = static_cast<int64_t>(ps.size());
      upload(f.pair_ptr, pp.data(), pp.size(), st);
      upload(f.pair_slot, ps.data(), ps.size(), st);
      CGB_CUDA(cudaStreamSynchronize(st));
    }
  }
  CGB_CUDA(cudaStreamSynchronize(st));
}

// ---- tables of the tensor-core tangent --------------------------------------------------
// One CTA per group of kMergeGroup points: the group's neighbour ids sorted and made unique
// (the group's node union, ascending ids), every face entry's index in it, the union's size,
// and for every merged entry (from its first contribution code, written row node first) the
// union indices of the block's row and column nodes. Groups with more than kTcItems entries
// get the size 32767 (not on the tensor path).
constexpr int kTcItems = 1024;

__global__ void __launch_bounds__(128) tc_cells_kernel(int n_gp, const int64_t* __restrict__ ptr,
                                                       const int32_t* __restrict__ idx,
                                                       const int64_t* __restrict__ map_ptr,
                                                       const int64_t* __restrict__ ent_ptr,
                                                       const int32_t* __restrict__ ent_cstart,
                                                       const uint16_t* __restrict__ code, uint8_t* __restrict__ nbr_u,
                                                       int16_t* __restrict__ cell_U, uint16_t* __restrict__ ent_uv) {
  __shared__ int ids[kTcItems];
  __shared__ int s_nu;
  const int G = blockIdx.x, t = threadIdx.x;
  const int g0 = G * kMergeGroup, g1 = min(n_gp, g0 + kMergeGroup);
  const int64_t q0 = ptr[g0], q1 = ptr[g1];
  const int items = static_cast<int>(q1 - q0);
  if (items > kTcItems) {
    for (int64_t e = q0 + t; e < q1; e += blockDim.x) nbr_u[e] = 255;
    if (t == 0) cell_U[G] = 32767;
    return;
  }
  int n2 = 1;
  while (n2 < items) n2 <<= 1;
  for (int i = t; i < n2; i += blockDim.x) ids[i] = i < items ? idx[q0 + i] : 0x7fffffff;
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = t; i < n2; i += blockDim.x) {
        const int u = i ^ j;
        if (u > i) {
          const bool up = (i & k) == 0;
          const int x = ids[i], y = ids[u];
          if ((x > y) == up) { ids[i] = y; ids[u] = x; }
        }
      }
      __syncthreads();
    }
  }
  if (t == 0) {  // unique, in place (items <= 1024)
    int m = 0;
    for (int i = 0; i < items; ++i)
      if (m == 0 || ids[i] != ids[m - 1]) ids[m++] = ids[i];
    s_nu = m;
  }
  __syncthreads();
  const int U = s_nu;
  if (t == 0) cell_U[G] = static_cast<int16_t>(U);
  auto find = [&](int node) {
    int lo = 0, hi = U;  // first position with ids[pos] >= node
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (ids[mid] < node) lo = mid + 1; else hi = mid;
    }
    return lo < 255 ? lo : 255;
  };
  for (int64_t e = q0 + t; e < q1; e += blockDim.x) nbr_u[e] = static_cast<uint8_t>(find(idx[e]));
  const int64_t e0 = ent_ptr[G], e1 = ent_ptr[G + 1];
  const int64_t cbase = map_ptr[g0];
  for (int64_t e = e0 + t; e < e1; e += blockDim.x) {
    const unsigned cd = code[cbase + (ent_cstart[e] & 0xffff)];
    const int k = cd >> 12, i = (cd >> 6) & 63, j = cd & 63;
    const int64_t p0 = ptr[g0 + k];
    ent_uv[e] = static_cast<uint16_t>(find(idx[p0 + i]) | (find(idx[p0 + j]) << 8));
  }
}

void tc_prepare(cgb_assembler* a) {
  if (a->tc_ready) return;
  merge_prepare(a);
  cudaStream_t st = a->ctx->stream;
  const cgb_shape* S = a->faces;
  const int n_gp = S->n_gp;
  const int ng = (n_gp + kMergeGroup - 1) / kMergeGroup;
  a->tc_nbr_u.alloc(std::max<int64_t>(S->nnz, 1));
  a->tc_cell_U.alloc(std::max(ng, 1));
  a->tc_ent_uv.alloc(std::max<int64_t>(a->mrg_n_ent, 1));
  if (ng > 0)
    tc_cells_kernel<<<ng, 128, 0, st>>>(n_gp, S->nbr_ptr.p, S->nbr_idx.p, a->map_ptr.p, a->mrg_ent_ptr.p,
                                        a->mrg_ent_cstart.p, a->mrg_code.p, a->tc_nbr_u.p, a->tc_cell_U.p,
                                        a->tc_ent_uv.p);
  CGB_CUDA(cudaGetLastError());
  std::vector<int16_t> cu(std::max(ng, 1));
  std::vector<int8_t> direct(std::max(ng, 1));
  if (ng > 0) {
    CGB_CUDA(cudaMemcpyAsync(cu.data(), a->tc_cell_U.p, ng * sizeof(int16_t), cudaMemcpyDeviceToHost, st));
    CGB_CUDA(cudaMemcpyAsync(direct.data(), a->mrg_direct.p, ng * sizeof(int8_t), cudaMemcpyDeviceToHost, st));
  }
  CGB_CUDA(cudaStreamSynchronize(st));
  a->tc_fallback_h.clear();
  a->tc_n_groups = 0;
  a->tc_point_cols = 0;
  for (int G = 0; G < ng; ++G) {
    if (direct[G] || cu[G] > kTcMaxUnion) {
      a->tc_fallback_h.push_back(G);
    } else {
      const int n_cols = std::max(16, (3 * cu[G] + 15) & ~15);
      ++a->tc_n_groups;
      a->tc_point_cols += static_cast<int64_t>(std::min(kMergeGroup, n_gp - G * kMergeGroup)) * n_cols;
    }
  }
  upload(a->tc_fallback, a->tc_fallback_h.data(), a->tc_fallback_h.size(), st);
  CGB_CUDA(cudaStreamSynchronize(st));
  a->tc_ready = true;
}

void merge_prepare(cgb_assembler* a) {
  if (a->mrg_ready) return;
  cudaStream_t st = a->ctx->stream;
  const cgb_shape* S = a->faces;
  const int n_gp = S->n_gp;
  const int ng = (n_gp + kMergeGroup - 1) / kMergeGroup;
  const size_t smem = kMergeItems * sizeof(unsigned long long);
  CGB_CUDA(cudaFuncSetAttribute(merge_groups_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)));
  DevBuf<int32_t> counts(ng);
  if (ng > 0)
    merge_groups_kernel<<<ng, 256, smem, st>>>(n_gp, S->nbr_ptr.p, S->nbr_idx.p, a->map_ptr.p, a->map_slot.p, 0, counts.p,
                                               nullptr, nullptr, nullptr, nullptr);
  CGB_CUDA(cudaGetLastError());
  std::vector<int32_t> hc(std::max(ng, 1));
  if (ng > 0) CGB_CUDA(cudaMemcpyAsync(hc.data(), counts.p, ng * 4, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> ep(ng + 1, 0);
  std::vector<int8_t> direct(std::max(ng, 1), 0);
  for (int G = 0; G < ng; ++G) {
    if (hc[G] < 0) { direct[G] = 1; ep[G + 1] = ep[G]; }
    else ep[G + 1] = ep[G] + hc[G];
  }
  upload(a->mrg_ent_ptr, ep.data(), ep.size(), st);
  upload(a->mrg_direct, direct.data(), direct.size(), st);
  a->mrg_ent_slot.alloc(ep[ng]);
  a->mrg_ent_cstart.alloc(ep[ng]);
  a->mrg_code.alloc(a->n_pairs);
  a->mrg_n_ent = ep[ng];
  a->mrg_n_direct = 0;
  for (int G = 0; G < ng; ++G) a->mrg_n_direct += direct[G];
  if (ng > 0)
    merge_groups_kernel<<<ng, 256, smem, st>>>(n_gp, S->nbr_ptr.p, S->nbr_idx.p, a->map_ptr.p, a->map_slot.p, 1, nullptr,
                                               a->mrg_ent_ptr.p, a->mrg_ent_slot.p, a->mrg_ent_cstart.p,
                                               a->mrg_code.p);
  CGB_CUDA(cudaGetLastError());
  CGB_CUDA(cudaStreamSynchronize(st));
  a->mrg_ready = true;
}

// Ordered lists for the deterministic scatter. F contribution ids: face entries
// [0, nnz_face), then hinge merged-node entries fold by fold. K unit ids: the face units
// (pairs, or merged entries), then hinge pairs fold by fold. Each K block and each node sums
// its units in ascending id order, i.e. Gauss point (or group of Gauss points) by Gauss
// point in the reference's loop order.
namespace {

// Per-block ascending lists of K units: n_face face units whose block slots are face_slot,
// then every fold's pairs.
void block_lists(cgb_assembler* a, int64_t n_face, const int32_t* face_slot, DevBuf<int64_t>& ptr,
                 DevBuf<int64_t>& list) {
  cudaStream_t st = a->ctx->stream;
  int64_t nq = n_face;
  for (auto& f : a->folds) nq += f.n_pairs;
  DevBuf<int64_t> cnt(a->n_blocks + 1);
  CGB_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), st));
  if (n_face) count_slots<<<nb(n_face, 256), 256, 0, st>>>(n_face, face_slot, cnt.p);
  for (auto& f : a->folds)
    if (f.n_pairs) count_slots<<<nb(f.n_pairs, 256), 256, 0, st>>>(f.n_pairs, f.pair_slot.p, cnt.p);
  std::vector<int64_t> hc(a->n_blocks);
  CGB_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, hc.size() * 8, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> lp(a->n_blocks + 1, 0);
  for (int64_t b = 0; b < a->n_blocks; ++b) lp[b + 1] = lp[b] + hc[b];
  upload(ptr, lp.data(), lp.size(), st);
  DevBuf<int64_t> cur;
  upload(cur, lp.data(), a->n_blocks, st);
  list.alloc(std::max<int64_t>(nq, 1));
  if (n_face) fill_slots<<<nb(n_face, 256), 256, 0, st>>>(n_face, 0, face_slot, cur.p, list.p);
  int64_t base = n_face;
  for (auto& f : a->folds) {
    if (f.n_pairs) fill_slots<<<nb(f.n_pairs, 256), 256, 0, st>>>(f.n_pairs, base, f.pair_slot.p, cur.p, list.p);
    base += f.n_pairs;
  }
  sort_lists<<<nb(a->n_blocks, 128), 128, 0, st>>>(a->n_blocks, ptr.p, list.p);
  CGB_CUDA(cudaGetLastError());
  CGB_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

void deterministic_pair_lists(cgb_assembler* a) {
  if (a->det_pairs_ready) return;
  block_lists(a, a->n_pairs, a->map_slot.p, a->blk_list_ptr, a->blk_list);
  a->det_pairs_ready = true;
}

void deterministic_entry_lists(cgb_assembler* a) {
  if (a->det_entries_ready) return;
  merge_prepare(a);
  if (a->mrg_n_direct) throw Error(CGB_ERR_INVALID, "deterministic entry lists need every group merged");
  block_lists(a, a->mrg_n_ent, a->mrg_ent_slot.p, a->ent_list_ptr, a->ent_list);
  a->det_entries_ready = true;
}

void deterministic_prepare(cgb_assembler* a) {
  if (a->det_ready) return;
  cgb_context* ctx = a->ctx;
  cudaStream_t st = ctx->stream;
  int64_t n_hf = 0;
  std::vector<int64_t> fnum;  // merged-node entries per fold
  for (auto& f : a->folds) {
    fnum.push_back(f.n_u);
    n_hf += f.n_u;
  }
  a->hinge_f_base = a->faces->nnz;
  a->n_fcontrib = a->faces->nnz + n_hf;

  // F lists (node of each contribution: face entries then hinge merged nodes).
  DevBuf<int64_t> fc(a->n_nodes + 1);
  CGB_CUDA(cudaMemsetAsync(fc.p, 0, fc.bytes(), st));
  if (a->faces->nnz) count_slots<<<nb(a->faces->nnz, 256), 256, 0, st>>>(a->faces->nnz, a->faces->nbr_idx.p, fc.p);
  for (size_t k = 0; k < a->folds.size(); ++k)
    if (fnum[k]) count_slots<<<nb(fnum[k], 256), 256, 0, st>>>(fnum[k], a->folds[k].u_node.p, fc.p);
  std::vector<int64_t> hf(a->n_nodes);
  CGB_CUDA(cudaMemcpyAsync(hf.data(), fc.p, hf.size() * 8, cudaMemcpyDeviceToHost, st));
  CGB_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> np(a->n_nodes + 1, 0);
  for (int j = 0; j < a->n_nodes; ++j) np[j + 1] = np[j] + hf[j];
  upload(a->node_list_ptr, np.data(), np.size(), st);
  DevBuf<int64_t> fcur;
  upload(fcur, np.data(), a->n_nodes, st);
  a->node_list.alloc(a->n_fcontrib);
  if (a->faces->nnz)
    fill_slots<<<nb(a->faces->nnz, 256), 256, 0, st>>>(a->faces->nnz, 0, a->faces->nbr_idx.p, fcur.p, a->node_list.p);
  int64_t base = a->faces->nnz;
  for (size_t k = 0; k < a->folds.size(); ++k) {
    if (fnum[k]) fill_slots<<<nb(fnum[k], 256), 256, 0, st>>>(fnum[k], base, a->folds[k].u_node.p, fcur.p, a->node_list.p);
    base += fnum[k];
  }
  sort_lists<<<nb(a->n_nodes, 128), 128, 0, st>>>(a->n_nodes, a->node_list_ptr.p, a->node_list.p);
  CGB_CUDA(cudaGetLastError());
  CGB_CUDA(cudaStreamSynchronize(st));
  a->det_ready = true;
}

}  // namespace cgb
