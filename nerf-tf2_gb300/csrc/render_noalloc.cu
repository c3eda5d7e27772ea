// nerfgb_render_rays_noalloc: the fused render for callers that cannot
// allocate device memory.
//
// Who needs it: code embedded in a host framework that owns the GPU's memory.
// TensorFlow, the reference's runtime, reserves nearly all device memory for
// its own allocator when it starts, so a raw cudaMalloc from a custom op or a
// py_function can fail; other hosts (real-time renderers, plugins with a fixed
// device budget) forbid allocation on their render threads. Such a caller can
// still pass its own inputs and outputs but has nowhere to get the
// intermediate buffers nerfgb_render_rays needs as `workspace`.
//
// This entry point takes that workspace from a file-scope device array of
// NERFGB_NOALLOC_SCRATCH_BYTES (16 MiB), reserved when this module is loaded
// on a device and held until the process exits. It calls no cudaMalloc,
// cudaFree or other allocating routine.
//
// Set-up: the first call in each CUDA context (normally once per device: the
// device's primary context) looks up the array's device address with
// cudaGetSymbolAddress while that device is current (host code cannot use
// the array's name as a device address) and caches it under the context's
// unique id. Make that first call before any stream capture. A context that
// is destroyed and created again (cudaDeviceReset, or another driver
// context) loads this module again, possibly at another address; its new id
// misses the cache, so the address is looked up again rather than reused.
//
// Sharing: every call on a device uses the same array and leaves the last
// call's intermediates in it. Nothing in it has to start at zero: each
// region is fully written before it is read. Calls that overlap on the GPU
// (different streams or host threads) race on the array; serialise them.
#include <cuda.h>

#include <mutex>
#include <unordered_map>

#include "common.cuh"

namespace nerfgb {

static __device__ __align__(256) unsigned char g_render_scratch[NERFGB_NOALLOC_SCRATCH_BYTES];

static std::mutex g_scratch_mu;
// context id (cuCtxGetId) -> device address of g_render_scratch in that context
static std::unordered_map<unsigned long long, void *> g_scratch_ptr;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// The unique id of the calling thread's current context, through the driver
// entry points the runtime hands out (no link against libcuda). 0 if none.
static unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of g_render_scratch in the current context (looked up once
// per context).
static int scratch_for_current_context(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return NERFGB_E_DEVICE;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = current_context_id();
  if (id != 0) {
    auto hit = g_scratch_ptr.find(id);
    if (hit != g_scratch_ptr.end()) {
      *out = hit->second;
      return NERFGB_OK;
    }
  }
  // First call in this context (or none is current yet: the lookup makes the
  // runtime set up the device's primary context).
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_render_scratch) != cudaSuccess || !p) return NERFGB_E_CUDA;
  if (id == 0) id = current_context_id();
  if (id == 0) return NERFGB_E_DEVICE;
  g_scratch_ptr[id] = p;
  *out = p;
  return NERFGB_OK;
}

}  // namespace nerfgb

extern "C" int nerfgb_render_rays_noalloc(const void *packed_coarse, const void *packed_fine, int precision,
                                          const float *rays_o, const float *rays_d, const float *near,
                                          const float *far, const float *u_coarse, const float *u_fine,
                                          unsigned long long seed, int n_rays, int n_coarse, int n_fine,
                                          int perturb, int lin_inv_depth, int white_bg, int trans_mode,
                                          float *rgb_coarse, float *depth_coarse, float *acc_coarse,
                                          float *rgb_fine, float *depth_fine, float *acc_fine, int *err_word,
                                          void *stream) {
  if (n_rays < 0 || n_coarse < 2 || n_fine < 1) return NERFGB_E_INVALID_ARG;
  const long long need = nerfgb_render_workspace_bytes(n_rays, n_coarse, n_fine);
  if (need < 0) return NERFGB_E_INVALID_ARG;
  if (need > (long long)NERFGB_NOALLOC_SCRATCH_BYTES) return NERFGB_E_SCRATCH_LIMIT;
  if (n_rays == 0) return NERFGB_OK;
  void *ws = nullptr;
  const int rc = nerfgb::scratch_for_current_context(&ws);
  if (rc != NERFGB_OK) return rc;
  return nerfgb_render_rays(packed_coarse, packed_fine, precision, rays_o, rays_d, near, far, u_coarse, u_fine,
                            seed, n_rays, n_coarse, n_fine, perturb, lin_inv_depth, white_bg, trans_mode,
                            rgb_coarse, depth_coarse, acc_coarse, rgb_fine, depth_fine, acc_fine, ws, err_word,
                            stream);
}
