// cgb_device.cuh — device helpers shared by the kernels of the GB300 Gauss-point library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace cgb {

// Device error word: the first failing check stores its code; the host reads it back.
__device__ __forceinline__ void dev_fail(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Device-side crease polyline: vertices packed in one array for all creases.
struct DevCrease {
  const double* xy;  // 2 * n_vertices
  int n_vertices;
  int extend_start, extend_end, is_closed;
};

// Enrichment::evaluateIndicator (core/include/curvami/Enrichment.h:23-92). The
// geometric decisions (closest segment with a strict '<', clamping of t, the 1e-12
// validity distance, the end caps, the side test) are evaluated with explicitly
// rounded operations, so they are taken exactly as a non-contracted FP64 CPU run
// takes them.
struct DevIndicator {
  double f, gx, gy, hxx, hyy, hxy;
};

__device__ __forceinline__ DevIndicator eval_indicator(double px, double py, const DevCrease& c) {
  DevIndicator out{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const int N = c.n_vertices;
  if (N < 2) return out;
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  double d = inf;
  double Cx = 0, Cy = 0, t_best = 0, snx = 0, sny = 0;
  int idx_best = 0;
  for (int i = 0; i < N - 1; ++i) {
    const double Ax = c.xy[2 * i], Ay = c.xy[2 * i + 1];
    const double Bx = c.xy[2 * i + 2], By = c.xy[2 * i + 3];
    const double vx = __dsub_rn(Bx, Ax), vy = __dsub_rn(By, Ay);
    const double v_sq = __dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy));
    if (v_sq == 0.0) continue;
    const double wx = __dsub_rn(px, Ax), wy = __dsub_rn(py, Ay);
    const double t = __ddiv_rn(__dadd_rn(__dmul_rn(wx, vx), __dmul_rn(wy, vy)), v_sq);
    const double t_min = (i == 0 && c.extend_start) ? -inf : 0.0;
    const double t_max = (i == N - 2 && c.extend_end) ? inf : 1.0;
    const double tm = (t < t_max) ? t : t_max;     // std::min(t_max, t)
    const double tc = (t_min < tm) ? tm : t_min;   // std::max(t_min, .)
    const double cx = __dadd_rn(Ax, __dmul_rn(tc, vx)), cy = __dadd_rn(Ay, __dmul_rn(tc, vy));
    const double ex = __dsub_rn(px, cx), ey = __dsub_rn(py, cy);
    const double cur = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
    if (cur < __dmul_rn(d, d)) {
      d = __dsqrt_rn(cur);
      Cx = cx; Cy = cy; idx_best = i; t_best = tc;
      const double L = __dsqrt_rn(v_sq);
      snx = __ddiv_rn(-vy, L);
      sny = __ddiv_rn(vx, L);
    }
  }
  if (!(d > 1e-12)) return out;  // invalid: f = 0, no derivatives
  const double ux = __ddiv_rn(__dsub_rn(px, Cx), d), uy = __ddiv_rn(__dsub_rn(py, Cy), d);
  const double dp = __dadd_rn(__dmul_rn(ux, snx), __dmul_rn(uy, sny));
  const bool start_cap = (idx_best == 0 && t_best == 0.0 && !c.extend_start && !c.is_closed);
  const bool end_cap = (idx_best == N - 2 && t_best == 1.0 && !c.extend_end && !c.is_closed);
  if (start_cap || end_cap) {
    out.f = dp;
    out.gx = (snx - out.f * ux) / d;
    out.gy = (sny - out.f * uy) / d;
    const double d2 = d * d;
    out.hxx = (3 * out.f * ux * ux - 2 * snx * ux - out.f) / d2;
    out.hyy = (3 * out.f * uy * uy - 2 * sny * uy - out.f) / d2;
    out.hxy = (3 * out.f * ux * uy - (snx * uy + ux * sny)) / d2;
  } else {
    out.f = (dp >= 0.0) ? 1.0 : -1.0;
  }
  return out;
}

}  // namespace cgb
