// ps_noalloc.cu -- binning of given half-complex fields without any device
// allocation on the call path.
//
// Who needs it: a code that measures P_l(k) in situ, between the kernels of
// its own time step (an N-body or hydro solver, a mock pipeline), usually
// owns the device memory through its own pool.  A cudaMalloc there
// synchronises the whole device, breaking the solver's stream overlap, and
// fails outright once the pool has taken the free memory.  Such a caller
// creates the estimator context once at start-up (that allocates its
// geometry tables) and then needs a per-step call that allocates nothing.
//
// The call runs the same kernels as ps_gpu_bin_fields_host (k_bin_fields,
// then the ordered reduce of the per-CTA partial sums).  The partials live in
// the file-scope array below instead of the context's cudaMalloc'd buffer.
#include <cuda_runtime.h>
#include <stdint.h>

#include "powspec_gpu.h"
#include "ps_internal.h"

namespace ps {
namespace {

constexpr int kNoAllocMaxCtas = 160;     // partial-sum rows (one per CTA)
constexpr int kNoAllocMaxWidth = 3200;   // npole * nbin
constexpr size_t kNoAllocScratchBytes =  // 4,096,000 bytes
    (size_t)kNoAllocMaxCtas * kNoAllocMaxWidth * sizeof(float2);

// Per-CTA partial sums [grid][npole * nbin] of every call on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// With the context's device current: the scratch array's device address and
// the SM count.  Looked up on every call rather than cached, so that an
// address never outlives the CUDA context it belongs to (a caller may reset
// the device between calls); the lookup is cheap once the module is loaded.
cudaError_t scratch_of_current_device(int dev, void** ptr, int* nsm) {
  cudaError_t e = cudaGetSymbolAddress(ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  return cudaDeviceGetAttribute(nsm, cudaDevAttrMultiProcessorCount, dev);
}

}  // namespace

// Called by ps_gpu_create with the context's device current: the first
// lookup of the array loads this file's module, which is when the driver
// places the array in device memory.  Doing it at context creation keeps
// that one-time placement off the per-step call.  Returns the CUDA status;
// the caller clears a failure, which the entry point then reports.
cudaError_t noalloc_prepare(int dev) {
  void* p = nullptr;
  int nsm = 0;
  return scratch_of_current_device(dev, &p, &nsm);
}

}  // namespace ps

using namespace ps;

extern "C" int ps_gpu_bin_fields_noalloc(ps_gpu_ctx* c, const float* f1, const float* f2,
                                         double* pl, void* stream) {
  CtxView v;
  if (ctx_view(c, &v)) return PS_GPU_ERR_ARG;
  if (!f1 || !f2 || !pl)
    return ctx_fail(c, PS_GPU_ERR_ARG, "bin_fields_noalloc: null field or output pointer");
  if (((uintptr_t)f1 | (uintptr_t)f2 | (uintptr_t)pl) & 7)
    return ctx_fail(c, PS_GPU_ERR_ARG, "bin_fields_noalloc: pointers must be 8-byte aligned");
  const int width = v.geom.npole * v.geom.nbin;
  if (width > kNoAllocMaxWidth)
    return ctx_fail(c, PS_GPU_ERR_RANGE,
                    "bin_fields_noalloc: npole * nbin = %d exceeds the scratch limit %d", width,
                    kNoAllocMaxWidth);
  // the caller's current device is given back on return (DeviceScope)
  DeviceScope dev_scope(v.device);
  cudaError_t e = dev_scope.err;
  void* scratch = nullptr;
  int nsm = 0;
  if (e == cudaSuccess) e = scratch_of_current_device(v.device, &scratch, &nsm);
  if (e != cudaSuccess)
    return ctx_fail(c, PS_GPU_ERR_CUDA, "bin_fields_noalloc set-up: %s", cudaGetErrorString(e));
  const int grid = nsm < kNoAllocMaxCtas ? nsm : kNoAllocMaxCtas;
  cudaStream_t s = (cudaStream_t)stream;
  float2* part = (float2*)scratch;  // FP32-pair partials
  // the kernel adds its tile sums into the partials: they start at zero
  e = cudaMemsetAsync(part, 0, (size_t)grid * width * sizeof(float2), s);
  if (e != cudaSuccess)
    return ctx_fail(c, PS_GPU_ERR_CUDA, "bin_fields_noalloc memset: %s", cudaGetErrorString(e));
  BinFieldArgs b;
  b.ng = v.ng;
  b.f1 = (const float2*)f1;
  b.f2 = (const float2*)f2;
  b.geom = v.geom;
  b.geom.nmu = 1;
  b.partials = part;
  b.grid = grid;
  launch_bin_fields(b, s);
  launch_reduce(part, grid, width, pl, s);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return ctx_fail(c, PS_GPU_ERR_CUDA, "bin_fields_noalloc launch: %s", cudaGetErrorString(e));
  return 0;
}
