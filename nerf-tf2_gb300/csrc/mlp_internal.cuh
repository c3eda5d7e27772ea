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

// Proposal network forward (proposal.cu).
int launch_proposal_forward(const float *params, const float *xyz, long long n, float *sigma, cudaStream_t stream);

}  // namespace nerfgb
