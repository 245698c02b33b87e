// noalloc.cu — the allocation-free entry point cgb_assemble_face_noalloc.
//
// For callers that may not allocate GPU memory during assembly (cudaMalloc / cudaFree
// can synchronise the device, are illegal during stream capture, or are reserved to a
// host framework's own pool). The only scratch the mixed face assembly needs beyond
// its inputs and outputs is the FP32 block accumulator; here it is a file-scope device
// array of fixed size, present on every GPU that loads the library until the process
// exits. Nothing in this file calls cudaMalloc, cudaFree or an allocating routine.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "cgb_internal.h"

namespace {

constexpr size_t kScratchFloats = static_cast<size_t>(CGB_NOALLOC_MAX_BLOCKS) * 12;  // 32 MiB

// The block accumulator (12 floats per 3x3 block, 16-byte vector atomics). Shared by
// every call of the process on the same device: overlapping calls race.
static __device__ __align__(256) float g_block_scratch[kScratchFloats];

// Device address of g_block_scratch per device ordinal, looked up once per device. In
// host code the array's name is only a host-side stand-in, so the kernels get this
// address, never &g_block_scratch. The address is kept for the life of the process:
// resetting a device (cudaDeviceReset) while the library is loaded is not supported.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_scratch_addr[kMaxDevices] = {nullptr};

float* scratch_for_current_device() {
  int dev = 0;
  CGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw cgb::Error(CGB_ERR_INVALID, "cgb_assemble_face_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_block_scratch);
    if (e != cudaSuccess || !p)
      throw cgb::Error(CGB_ERR_CUDA, std::string("cgb_assemble_face_noalloc: cudaGetSymbolAddress failed: ") +
                                         cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<float*>(p);
  }
  return g_scratch_addr[dev];
}

}  // namespace

extern "C" int cgb_assemble_face_noalloc(cgb_context* ctx, const cgb_face_problem* prob, const double* d_x,
                                         double* d_K, double* d_F) {
  if (!ctx) return CGB_ERR_INVALID;
  try {
    if (!prob || !d_x || !d_K || !d_F) throw cgb::Error(CGB_ERR_INVALID, "cgb_assemble_face_noalloc: NULL argument");
    const cgb_face_problem& pr = *prob;
    if (pr.n_gp < 0 || pr.n_nodes <= 0 || pr.nnz < 0 || pr.nnz % 9 != 0 || pr.max_neighbours < 0)
      throw cgb::Error(CGB_ERR_INVALID, "cgb_assemble_face_noalloc: inconsistent sizes");
    // Without face points K and F are zero and no input array is read.
    if (pr.n_gp > 0 && (!pr.nbr_ptr || !pr.nbr_idx || !pr.dpsi || !pr.ddpsi || !pr.weight || !pr.map_ptr ||
                        !pr.csr_map || !pr.outer))
      throw cgb::Error(CGB_ERR_INVALID, "cgb_assemble_face_noalloc: NULL input array");
    if (pr.nnz / 9 > CGB_NOALLOC_MAX_BLOCKS)
      throw cgb::Error(CGB_ERR_CAPACITY, "cgb_assemble_face_noalloc: nnz(K) = " + std::to_string(pr.nnz) +
                                             " exceeds the fixed accumulator (" +
                                             std::to_string(static_cast<long long>(CGB_NOALLOC_MAX_BLOCKS) * 9) +
                                             " values); use cgb_assemble_device");
    // The kernel stages 32 floats and one index per neighbour, for 4 warps, in shared
    // memory (plus 32 x 32 floats of per-point state per warp).
    if (4 * ((32 * 32 + 32 * static_cast<size_t>(pr.max_neighbours)) * sizeof(float) +
             static_cast<size_t>(pr.max_neighbours) * sizeof(int)) > 200 * 1024)
      throw cgb::Error(CGB_ERR_CAPACITY, "cgb_assemble_face_noalloc: too many neighbours per Gauss point");
    if (ctx->natcurv.active)
      throw cgb::Error(CGB_ERR_INVALID, "cgb_assemble_face_noalloc: natural curvature needs the Gauss points' "
                                        "coordinates, which this entry point does not take; use cgb_assemble_device");
    CGB_CUDA(cudaSetDevice(ctx->device));
    float* scratch = scratch_for_current_device();
    cgb::face_mixed_on_arrays(pr, d_x, d_K, d_F, scratch, ctx->dev_err.p, ctx->stream);
    ctx->last_error.clear();
    return CGB_OK;
  } catch (const cgb::Error& e) {
    ctx->last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    ctx->last_error = e.what();
    return CGB_ERR_INVALID;
  }
}
