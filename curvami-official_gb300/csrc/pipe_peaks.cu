// pipe_peaks.cu — measures the FP64 and FP32 FMA throughput of the current GPU, the
// roofline denominators of the compute-bound kernels (the machine's measured peaks file
// covers only HBM copy bandwidth and bf16 tensor throughput). Built as its own small library
// (libcgb_peaks.so) used by the benchmark; it is not part of the hot-path ABI.
#include <cuda_runtime.h>

namespace {

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  // Eight independent chains per thread keep the pipe full; the result is written only
  // under a condition that never holds, so the loop is not optimised away.
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-12345.0) out[0] = s;
}

template <typename T>
double measure(int sms, int iters, cudaStream_t st) {
  T* d = nullptr;
  if (cudaMalloc(&d, 64) != cudaSuccess) return -1.0;
  const dim3 grid(sms * 8), block(256);
  fma_chains<T><<<grid, block, 0, st>>>(d, 4, (T)0.999, (T)0.001);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, st);
    fma_chains<T><<<grid, block, 0, st>>>(d, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8 * 16 * static_cast<double>(iters) * grid.x * block.x;
    const double tf = flops / (ms * 1e-3) / 1e12;
    if (tf > best) best = tf;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return best;
}

}  // namespace

extern "C" int cgb_measure_fma_peaks(int device, double* fp64_tflops, double* fp32_tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaStream_t st;
  if (cudaStreamCreate(&st) != cudaSuccess) return 2;
  if (fp64_tflops) *fp64_tflops = measure<double>(sms, 2000, st);
  if (fp32_tflops) *fp32_tflops = measure<float>(sms, 20000, st);
  cudaStreamDestroy(st);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
