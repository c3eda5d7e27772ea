// Launchers shared between the MLP translation units.
#pragma once
#include <cuda_runtime.h>

namespace nerfgb {

// FP32 SIMT forward (mlp.cu).
int launch_mlp_fp32(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                    float *rgb, float *sigma, cudaStream_t stream);

// FP32 SIMT forward that also stores every layer's activations (mlp.cu).
int launch_mlp_fp32_store(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                          float *rgb, float *sigma, float *acts, cudaStream_t stream);

// BF16 tcgen05 forward (mlp_tc.cu).
int launch_mlp_bf16(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                    float *rgb, float *sigma, int *err_word, cudaStream_t stream);

// FP8-e4m3 tcgen05 forward (mlp_tc.cu).
int launch_mlp_fp8(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                   float *rgb, float *sigma, int *err_word, cudaStream_t stream);

// Proposal network forward (proposal.cu).
int launch_proposal_forward(const float *params, const float *xyz, long long n, float *sigma, cudaStream_t stream);

// Compositing with a chosen last interval (ray_ops.cu): last_delta >= 0 is
// used as is (the reference uses 1e10), < 0 means the previous spacing.
// sample_rgb and the map outputs may be NULL.
int launch_composite(const float *sample_rgb, const float *sigma, const float *t_vals, int n_rays, int n_samples,
                     int white_bg, int trans_mode, float last_delta, float *weights, float *pred_rgb,
                     float *pred_depth, float *acc_map, cudaStream_t stream);
int launch_composite_bwd(const float *sigma, const float *t, const float *rgb, const float *grad_map,
                         const float *grad_w, int R, int S, int white_bg, float last_delta, float *grad_sigma,
                         float *grad_rgb, cudaStream_t stream);

}  // namespace nerfgb
