// Training-side kernels: compositing backward, losses, Adam.
//
// The reference differentiates NeRF.forward with tf.GradientTape and applies
// Keras Adam (nerf/core/model.py:148-171, :413-418). These kernels are the
// hand-written counterparts.
#include <math.h>

#include "common.cuh"
#include "mlp_internal.cuh"

namespace nerfgb {

// ---------------------------------------------------------------------------
// Compositing backward (ray_utils.py:408-551). One warp per ray; lane l owns
// samples [l*k, (l+1)*k). With w_i = a_i T_i, T_i = prod_{j<i} f_j,
// f_j = (1 - a_j) + 1e-10, a_j = 1 - exp(-s_j d_j):
//   dL/da_k = g_k T_k - (1/f_k) sum_{i>k} g_i w_i
//   dL/ds_k = dL/da_k * d_k * exp(-s_k d_k)
// where g_i = dL/dw_i (given) + sum_c G_c c_ic - white_bg * sum_c G_c, and
// dL/dc_ic = w_i G_c, G = dL/dpred_rgb.
// ---------------------------------------------------------------------------
constexpr int kCbWarps = 4;

__global__ void __launch_bounds__(32 * kCbWarps)
    composite_bwd_kernel(const float *__restrict__ sigma, const float *__restrict__ t,
                         const float *__restrict__ rgb, const float *__restrict__ grad_map,
                         const float *__restrict__ grad_w, int R, int S, int white_bg, float last_delta,
                         float *__restrict__ grad_sigma, float *__restrict__ grad_rgb) {
  extern __shared__ float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *s_t = smem + warp * 4 * (S + 1);  // t
  float *s_sig = s_t + (S + 1);            // sigma
  float *s_T = s_sig + (S + 1);            // transmittance T_i
  float *s_g = s_T + (S + 1);              // g_i = dL/dw_i
  const int k = (S + 31) >> 5;
  for (int r = blockIdx.x * kCbWarps + warp; r < R; r += gridDim.x * kCbWarps) {
    const long long base = (long long)r * S;
    for (int j = lane; j < S; j += 32) {
      s_t[j] = t[base + j];
      s_sig[j] = sigma[base + j];
    }
    __syncwarp();
    float G0 = 0.f, G1 = 0.f, G2 = 0.f;
    if (grad_map) {
      G0 = grad_map[3 * r];
      G1 = grad_map[3 * r + 1];
      G2 = grad_map[3 * r + 2];
    }
    const float Gbg = white_bg ? (G0 + G1 + G2) : 0.0f;
    const int j0 = min(lane * k, S), j1 = min(j0 + k, S);
    const float dlast = last_delta >= 0.0f ? last_delta : (S > 1 ? s_t[S - 1] - s_t[S - 2] : 1e10f);
    // Exclusive transmittance product across lanes.
    float loc = 1.0f;
    for (int j = j0; j < j1; ++j) {
      const float d = (j < S - 1) ? s_t[j + 1] - s_t[j] : dlast;
      loc *= expf(-s_sig[j] * d) + 1e-10f;  // (1 - a) + 1e-10 with 1 - a = exp(-s d)
    }
    float inc = loc;
    for (int off = 1; off < 32; off <<= 1) {
      float o = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc *= o;
    }
    float Tr = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) Tr = 1.0f;
    // Forward sweep: T_i, g_i and the lane's sum of g_i w_i.
    float gw_sum = 0.0f;
    for (int j = j0; j < j1; ++j) {
      const float d = (j < S - 1) ? s_t[j + 1] - s_t[j] : dlast;
      const float e = expf(-s_sig[j] * d);
      float g = grad_w ? grad_w[base + j] : 0.0f;
      if (grad_map) {
        const float *c = rgb + 3 * (base + j);
        g += G0 * c[0] + G1 * c[1] + G2 * c[2] - Gbg;
      }
      s_T[j] = Tr;
      s_g[j] = g;
      gw_sum += g * (1.0f - e) * Tr;
      Tr *= e + 1e-10f;
    }
    // Sum of g w over the lanes after this one.
    float suf = gw_sum;
    for (int off = 1; off < 32; off <<= 1) {
      float o = __shfl_down_sync(0xffffffffu, suf, off);
      if (lane + off < 32) suf += o;
    }
    float after = __shfl_down_sync(0xffffffffu, suf, 1);
    if (lane == 31) after = 0.0f;
    // Backward sweep over the segment.
    for (int j = j1 - 1; j >= j0; --j) {
      const float d = (j < S - 1) ? s_t[j + 1] - s_t[j] : dlast;
      const float e = expf(-s_sig[j] * d);
      const float w = (1.0f - e) * s_T[j];
      const float g = s_g[j];
      const float da = g * s_T[j] - after / (e + 1e-10f);
      grad_sigma[base + j] = da * d * e;
      if (grad_rgb) {
        float *gr = grad_rgb + 3 * (base + j);
        gr[0] = w * G0;
        gr[1] = w * G1;
        gr[2] = w * G2;
      }
      after += g * w;
    }
    __syncwarp();
  }
}

// MSE (keras.losses.MeanSquaredError, model.py:32,157-168): loss += scale *
// mean((p - y)^2); grad = scale * 2 (p - y) / n.
// The loss kernels run as one block of kLossThreads so that the loss is
// reproducible bit for bit: each thread sums a fixed stride of the elements
// in order, warps reduce by a fixed shuffle tree, and thread 0 adds the
// warps' sums in order to *loss (one add).
constexpr int kLossThreads = 1024;

__device__ __forceinline__ float block_sum_ordered(float part) {
  __shared__ float warp_sums[kLossThreads / 32];
  for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = part;
  __syncthreads();
  float total = 0.0f;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += warp_sums[w];
  return total;  // thread 0
}

__global__ void __launch_bounds__(kLossThreads)
    mse_kernel(const float *__restrict__ pred, const float *__restrict__ target, long long n, float scale,
               float *__restrict__ loss, float *__restrict__ grad) {
  float part = 0.0f;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float d = pred[i] - target[i];
    part += d * d;
    if (grad) grad[i] = scale * 2.0f * d / (float)n;
  }
  const float total = block_sum_ordered(part);
  if (threadIdx.x == 0 && loss) *loss += scale * total / (float)n;
}

// Envelope loss of the proposal sampler on weight histograms [R,S]:
// sum (1 + lam [w_p < w_t]) (w_p - w_t)^2 / R.
__global__ void __launch_bounds__(kLossThreads)
    envelope_loss_kernel(const float *__restrict__ wp, const float *__restrict__ wt, long long n, int R, float lam,
                         float *__restrict__ loss, float *__restrict__ grad) {
  float part = 0.0f;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float d = wp[i] - wt[i];
    const float rho = d < 0.0f ? 1.0f + lam : 1.0f;
    part += rho * d * d;
    grad[i] = 2.0f * rho * d / (float)R;
  }
  const float total = block_sum_ordered(part);
  if (threadIdx.x == 0 && loss) *loss += total / (float)R;
}

// TensorFlow ApplyAdam (Keras Adam, model.py:418): m += (g - m)(1 - b1);
// v += (g^2 - v)(1 - b2); var -= lr_t m / (sqrt(v) + eps).
__global__ void adam_kernel(float *__restrict__ var, float *__restrict__ m, float *__restrict__ v,
                            const float *__restrict__ g, long long n, float lr_t, float b1, float b2, float eps) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = m[i] + (gi - m[i]) * (1.0f - b1);
    const float vi = v[i] + (gi * gi - v[i]) * (1.0f - b2);
    m[i] = mi;
    v[i] = vi;
    var[i] -= lr_t * mi / (sqrtf(vi) + eps);
  }
}

static int grid_cap(long long n, int block) {
  long long g = (n + block - 1) / block;
  int sms = num_sms();
  long long cap = (long long)(sms > 0 ? sms : 148) * 32;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

int launch_composite_bwd(const float *sigma, const float *t, const float *rgb, const float *grad_map,
                         const float *grad_w, int R, int S, int white_bg, float last_delta, float *grad_sigma,
                         float *grad_rgb, cudaStream_t stream) {
  size_t smem = (size_t)kCbWarps * 4 * (S + 1) * sizeof(float);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(composite_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return NERFGB_E_CUDA;
  int sms = num_sms();
  int blocks = (R + kCbWarps - 1) / kCbWarps;
  int cap = (sms > 0 ? sms : 148) * 16;
  composite_bwd_kernel<<<blocks < cap ? blocks : cap, 32 * kCbWarps, smem, stream>>>(
      sigma, t, rgb, grad_map, grad_w, R, S, white_bg, last_delta, grad_sigma, grad_rgb);
  return launch_status();
}

}  // namespace nerfgb

using namespace nerfgb;

extern "C" int nerfgb_composite_backward(const float *sigma, const float *t_vals, const float *sample_rgb,
                                         const float *grad_rgb_map, const float *grad_weights, int n_rays,
                                         int n_samples, int white_bg, float *grad_sigma,
                                         float *grad_sample_rgb, void *stream) {
  if (n_rays < 0 || n_samples < 1) return NERFGB_E_INVALID_ARG;
  if (n_samples > 2048) return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!sigma || !t_vals || !grad_sigma || (!grad_rgb_map && !grad_weights) ||
      (grad_rgb_map && !sample_rgb))
    return NERFGB_E_INVALID_ARG;
  return launch_composite_bwd(sigma, t_vals, sample_rgb, grad_rgb_map, grad_weights, n_rays, n_samples,
                              white_bg, 1e10f, grad_sigma, grad_sample_rgb, as_stream(stream));
}

extern "C" int nerfgb_mse_loss(const float *pred, const float *target, long long n, float scale, float *loss,
                               float *grad, void *stream) {
  if (n < 0) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!pred || !target || (!loss && !grad)) return NERFGB_E_INVALID_ARG;
  mse_kernel<<<1, kLossThreads, 0, as_stream(stream)>>>(pred, target, n, scale, loss, grad);
  return launch_status();
}

extern "C" int nerfgb_envelope_loss(const float *w_prop, const float *w_target, int n_rays, int n_bins,
                                    float lam, float *loss, float *grad, void *stream) {
  if (n_rays < 0 || n_bins < 1) return NERFGB_E_INVALID_ARG;
  if (n_rays == 0) return NERFGB_OK;
  if (!w_prop || !w_target || !grad) return NERFGB_E_INVALID_ARG;
  long long n = (long long)n_rays * n_bins;
  envelope_loss_kernel<<<1, kLossThreads, 0, as_stream(stream)>>>(w_prop, w_target, n, n_rays, lam, loss, grad);
  return launch_status();
}

extern "C" int nerfgb_adam_step(float *params, float *m, float *v, const float *grads, long long n, float lr,
                                float beta1, float beta2, float eps, long long step, void *stream) {
  if (n < 0 || step < 1) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!params || !m || !v || !grads) return NERFGB_E_INVALID_ARG;
  const double lr_t = (double)lr * sqrt(1.0 - pow((double)beta2, (double)step)) / (1.0 - pow((double)beta1, (double)step));
  adam_kernel<<<grid_cap(n, 256), 256, 0, as_stream(stream)>>>(params, m, v, grads, n, (float)lr_t, beta1, beta2,
                                                                eps);
  return launch_status();
}
