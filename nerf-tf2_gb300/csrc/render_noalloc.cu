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
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current (host code cannot
// use the array's name as a device address) and caches it. Make that first
// call before any stream capture.
//
// Sharing: every call on a device uses the same array and leaves the last
// call's intermediates in it. Nothing in it has to start at zero: each
// region is fully written before it is read. Calls that overlap on the GPU
// (different streams or host threads) race on the array; serialise them.
#include <mutex>

#include "common.cuh"

namespace nerfgb {

static __device__ __align__(256) unsigned char g_render_scratch[NERFGB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static std::mutex g_scratch_mu;
static void *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_render_scratch on the current device (looked up once).
static int scratch_for_current_device(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NERFGB_E_DEVICE;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_render_scratch) != cudaSuccess || !p) return NERFGB_E_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
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
  const int rc = nerfgb::scratch_for_current_device(&ws);
  if (rc != NERFGB_OK) return rc;
  return nerfgb_render_rays(packed_coarse, packed_fine, precision, rays_o, rays_d, near, far, u_coarse, u_fine,
                            seed, n_rays, n_coarse, n_fine, perturb, lin_inv_depth, white_bg, trans_mode,
                            rgb_coarse, depth_coarse, acc_coarse, rgb_fine, depth_fine, acc_fine, ws, err_word,
                            stream);
}
