// noalloc.cu -- the logistic-regression potential without any device allocation.
//
// Some callers cannot call cudaMalloc at the moment they need a potential evaluated:
//   * a JAX/XLA FFI custom-call handler: XLA owns every device buffer of the
//     computation and, with its default preallocation, leaves little memory
//     that cudaMalloc could still hand out, so a handler must not allocate per call;
//   * host frameworks that route all device memory through their own pool
//     and forbid allocations behind their back.
// gbn_logreg_potential_noalloc serves them: the caller passes the data, the
// positions and the outputs as device pointers, and the kernel's scratch (the
// per-row-group partial gradients and log-likelihoods of the FP32 logistic
// potential) lives in the file-scope device arrays below, of a fixed size that
// every GPU loading this library holds until the process exits.
//
// The first call on a device (with that device current) looks up the device
// addresses of the arrays with cudaGetSymbolAddress and raises the kernel's
// shared-memory limit on that device; make that first call before any stream
// capture.  All calls share the arrays: calls that overlap on the GPU (on
// different streams, or from different threads) race on them and must be
// serialised by the caller.  Nothing needs clearing between calls, because every
// scratch word the kernels read is written earlier in the same call.
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/gbnuts.h"
#include "internal.h"

namespace gbn {

cudaError_t launch_logreg_simt_scratch(const float* x, const float* y, int64_t n, int p, double prior_scale,
                                       const float* Q, int npts, int row_groups, float* part_g, double* part_ll,
                                       double* PE, float* G, cudaStream_t st);
cudaError_t logreg_simt_smem_attr();

namespace {

constexpr int kRowGroups = 16;  // row groups of the scratch layout (one CTA row per group)
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_part_g[kRowGroups * GBN_NOALLOC_MAX_POINTS * 64];
static __device__ __align__(256) double g_noalloc_part_ll[kRowGroups * GBN_NOALLOC_MAX_POINTS];

struct DeviceScratch {
  float* part_g = nullptr;
  double* part_ll = nullptr;
};
DeviceScratch g_scratch[kMaxDevices];
std::mutex g_scratch_mutex;
thread_local std::string g_noalloc_error;

int noalloc_fail(int code, const std::string& msg) {
  g_noalloc_error = msg;
  return code;
}

}  // namespace
}  // namespace gbn

using namespace gbn;

extern "C" const char* gbn_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

extern "C" int gbn_logreg_potential_noalloc(void* stream, const float* d_x, const float* d_y, int64_t n, int32_t p,
                                            double prior_scale, const float* d_z, int32_t num_points, double* d_pe,
                                            float* d_grad) {
  if (!d_x || !d_y || !d_z || !d_pe || !d_grad)
    return noalloc_fail(GBN_ERR_INVALID_ARG, "gbn_logreg_potential_noalloc: null pointer");
  if (n < 1 || p < 1 || p > 64)
    return noalloc_fail(GBN_ERR_INVALID_ARG, "gbn_logreg_potential_noalloc: need n >= 1 and 1 <= p <= 64");
  if (!(prior_scale > 0.0) || !std::isfinite(prior_scale))
    return noalloc_fail(GBN_ERR_INVALID_ARG, "gbn_logreg_potential_noalloc: prior_scale must be finite and > 0");
  if (num_points < 1 || num_points > GBN_NOALLOC_MAX_POINTS)
    return noalloc_fail(GBN_ERR_INVALID_ARG,
                        "gbn_logreg_potential_noalloc: num_points must be in [1, GBN_NOALLOC_MAX_POINTS = " +
                            std::to_string(GBN_NOALLOC_MAX_POINTS) + "]; got " + std::to_string(num_points));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(GBN_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(GBN_ERR_UNSUPPORTED, "device index out of range");
  DeviceScratch s;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch[dev].part_g) {  // once per device, with that device current
      void* pg = nullptr;
      void* pl = nullptr;
      e = cudaGetSymbolAddress(&pg, g_noalloc_part_g);
      if (e != cudaSuccess)
        return noalloc_fail(GBN_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      e = cudaGetSymbolAddress(&pl, g_noalloc_part_ll);
      if (e != cudaSuccess)
        return noalloc_fail(GBN_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      e = logreg_simt_smem_attr();
      if (e != cudaSuccess)
        return noalloc_fail(GBN_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
      g_scratch[dev].part_g = static_cast<float*>(pg);
      g_scratch[dev].part_ll = static_cast<double*>(pl);
    }
    s = g_scratch[dev];
  }
  int64_t ntiles = (n + 63) / 64;
  int row_groups = (int)(ntiles < kRowGroups ? ntiles : kRowGroups);
  e = launch_logreg_simt_scratch(d_x, d_y, n, p, prior_scale, d_z, num_points, row_groups,
                                 s.part_g, s.part_ll, d_pe, d_grad, (cudaStream_t)stream);
  if (e != cudaSuccess) return noalloc_fail(GBN_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return GBN_OK;
}
