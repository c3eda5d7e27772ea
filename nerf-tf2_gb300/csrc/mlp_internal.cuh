// Launchers shared between the MLP translation units.
#pragma once
#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's entry-point query)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "nerfgb.h"

namespace nerfgb {

// Optional indirection of an MLP launch's rows. Logical row k in [0, n) is
// physical row map[k] of xyz, of the outputs and (divided by rows_per_dir)
// of dirs; with n_dev the row count is read on the device as
// min(*n_dev, n), so a compaction kernel can feed the MLP without a host
// round trip. Both NULL: the identity and the host count.
struct RowMap {
  const int *map = nullptr;
  const int *n_dev = nullptr;
};

// A tensor map of 16-bit elements over `base` (mlp_tc.cu): rank dims
// (innermost first), the byte strides of dims 1.. (multiples of 16), box
// sizes; no interleave, zero fill outside the dims; no swizzle, or with
// swizzle128 the 128-byte swizzle (box rows of 128 bytes land with their
// 16-byte chunks permuted by the row within each 8-row, 1024-byte block).
int encode_tensor_map_u16(CUtensorMap *map, const void *base, int rank, const unsigned long long *dims,
                          const unsigned long long *strides, const unsigned *box, bool swizzle128 = false);

// FP32 SIMT forward (mlp.cu).
int launch_mlp_fp32(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                    float *rgb, float *sigma, cudaStream_t stream, const RowMap &rm = RowMap());

// FP32 SIMT forward that also stores every layer's activations (mlp.cu).
int launch_mlp_fp32_store(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                          float *rgb, float *sigma, float *acts, cudaStream_t stream);

// BF16 tcgen05 forward (mlp_tc.cu).
int launch_mlp_bf16(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                    float *rgb, float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm = RowMap());

// BF16 tcgen05 forward that also writes the BF16 activation tape (kActsLd
// values per row, the FP32 tape's columns) for the BF16 backward (mlp_tc.cu).
int launch_mlp_bf16_train(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                          float *rgb, float *sigma, uint16_t *tape, int *err_word, cudaStream_t stream);

// Backward of the sigma and rgb heads (mlp_train.cu) from an FP32 or a BF16
// activation tape: dz9 [n][256] (128 used) = dL/d(dense_9 pre-activation),
// dsp [n] = dL/d(sigma pre-activation), head gradients into grads.
int launch_head_bwd(const float *table, const float *tape, long long n, const float *d_rgb, const float *d_sigma,
                    float *dz9, float *dsp, float *grads, cudaStream_t stream);
int launch_head_bwd(const float *table, const uint16_t *tape, long long n, const float *d_rgb,
                    const float *d_sigma, float *dz9, float *dsp, float *grads, cudaStream_t stream);

// Tensor-core GEMMs of the BF16 backward (gemm_tc.cu). dX [M][256] (BF16) =
// dZ [M][n_out] (BF16, row stride 256) W^T with W the layer's BF16 weights
// [k_in][n_out] (rows 0..255 used).
int launch_gemm_dx(const __nv_bfloat16 *dz, long long M, int n_out, const __nv_bfloat16 *W, __nv_bfloat16 *dx,
                   int *err, cudaStream_t stream);
// grads [k][n] (row stride n_out) += sum_m In[m][k] dZ[m][n], k < k_in <= 256,
// In BF16 with row stride ld_in, dZ BF16 with row stride 256; the rows are
// reduced in `splits` parts whose partial sums go to `part`
// (gemm_dw_partial_floats(splits) floats) before they are added.
int launch_gemm_dw(const __nv_bfloat16 *in, long long ld_in, int k_in, const __nv_bfloat16 *dz, int n_out,
                   long long M, float *grads, float *part, int splits, int *err, cudaStream_t stream);
long long gemm_dw_partial_floats(int splits);
// The BF16 (pair) or FP8 tensor-core forward with a chosen limit on every
// bounded wait (ns) and the weight chunk at position `withhold` of the load
// sequence of the (even) CTA left unloaded, so that a wait runs out: the
// failure path's test hook (mlp_tc.cu).
int launch_mlp_wait_test(const void *packed, bool fp8, const float *xyz, const float *dirs, long long n, int rpd,
                         float *rgb, float *sigma, int *err_word, cudaStream_t stream, unsigned long long wait_ns,
                         long long withhold);

// FP8-e4m3 tcgen05 forward (mlp_tc.cu).
int launch_mlp_fp8(const void *packed, const float *xyz, const float *dirs, long long n, int rows_per_dir,
                   float *rgb, float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm = RowMap());

// Dispatch on precision (render.cu).
int launch_mlp(const void *packed, int precision, const float *xyz, const float *dirs, long long n, int rpd,
               float *rgb, float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm = RowMap());

// Sample gates (gate.cu). Coarse: sample (r, j) is on where w[r*S + j] > tau;
// writes mask[r*S + j] (0/1), appends the on samples' indices r*S + j to
// row_map (rays in any order, samples of a ray in order) and adds their
// number to *count. Fine: sample (r, j) of the sorted union is on where it is
// a coarse sample whose mask is on, or a fine draw (perm >= Sc); with the
// draws' bins (piece [R, S - Sc], not NULL) only a fine draw whose bin's mask
// is on.
int launch_gate_coarse(const float *w, int R, int S, float tau, unsigned char *mask, int *row_map, int *count,
                       cudaStream_t stream);
int launch_gate_fine(const int *perm, const unsigned char *mask_c, const int *piece, int R, int Sc, int S,
                     int *row_map, int *count, cudaStream_t stream);

// Proposal network forward (proposal.cu).
int launch_proposal_forward(const float *params, const float *xyz, long long n, float *sigma, cudaStream_t stream);
// The same network on tensor cores: BF16 operands, FP32 accumulation (proposal.cu).
int launch_proposal_forward_bf16(const float *params, const float *xyz, long long n, float *sigma,
                                 cudaStream_t stream);

// Compositing with a chosen last interval (ray_ops.cu): last_delta >= 0 is
// used as is (the reference uses 1e10), < 0 means the previous spacing.
// sample_rgb and the map outputs may be NULL.
// Optional gate on the compositor's weights (the coarse gate of the gated
// render): sample j of a ray is on where w > tau (NaN: off); mask [R*S]
// (0/1, may be NULL), the on samples' indices appended to row_map at slots
// taken from *count, sig_zero (may be NULL) zeroed at the off samples.
struct CompositeGate {
  float tau = 0.0f;
  unsigned char *mask = nullptr;
  int *row_map = nullptr, *count = nullptr;
  float *sig_zero = nullptr;
};
int launch_composite(const float *sample_rgb, const float *sigma, const float *t_vals, int n_rays, int n_samples,
                     int white_bg, int trans_mode, float last_delta, float *weights, float *pred_rgb,
                     float *pred_depth, float *acc_map, cudaStream_t stream,
                     const CompositeGate &gate = CompositeGate());

// Stratified coarse sampler (ray_ops.cu); u_vals NULL with perturb: the
// Philox draws of nerfgb_uniform(seed, 0, R*S) are made in the kernel.
int launch_coarse_sample(const float *rays_o, const float *rays_d, const float *near, const float *far,
                         const float *u_vals, unsigned long long seed, int R, int S, int perturb, int lin_inv,
                         float *xyz, float *dirs, float *t_vals, float *edges, float *widths, cudaStream_t stream);

// What the fine sampler (ray_ops.cu) fuses around the sampling, all fields
// optional: the coarse pass's compositing (the bin weights from sigma_c
// [R*Sc] instead of bin_weights; with rgb_c [R*Sc,3] and map_* also the
// coarse maps; w_c receives the weights), the fine gate of the gated render
// (a member of the sorted union is on where it is a fine draw or its coarse
// sample's mask_c entry is on; on members appended to row_map at slots from
// *count, sig_zero / rgb_zero zeroed at the off members), and the Philox
// draws of nerfgb_uniform(seed, R*Sc, R*Sf) when u_vals is NULL.
struct FineFuse {
  const float *sigma_c = nullptr, *rgb_c = nullptr;
  int mode = NERFGB_TRANS_LOGSUM, white_bg = 0;
  float *w_c = nullptr;
  float *map_rgb = nullptr, *map_depth = nullptr, *map_acc = nullptr;
  const unsigned char *mask_c = nullptr;
  int *row_map = nullptr, *count = nullptr;
  float *sig_zero = nullptr, *rgb_zero = nullptr;
  int gate_draws = 0;  // 1: a fine draw is on only where its coarse bin's gate is
  unsigned long long seed = 0;
};
int launch_fine_sample(const float *rays_o, const float *rays_d, const float *bin_weights, const float *left_edges,
                       int ld_left, const float *bin_widths, const float *t_vals_coarse, const float *u_vals,
                       int n_rays, int n_coarse, int n_fine, float *xyz, float *dirs, float *t_vals,
                       int *piece_idxs, int *sort_perm, cudaStream_t stream, const FineFuse &fz);
int launch_composite_bwd(const float *sigma, const float *t, const float *rgb, const float *grad_map,
                         const float *grad_w, int R, int S, int white_bg, float last_delta, float *grad_sigma,
                         float *grad_rgb, cudaStream_t stream);

// The BF16/FP8 proposal paths' front end (proposal.cu), one warp per ray:
// stratified samples (xyz, t_vals, edges [R, S+1], widths), the BF16
// proposal density at them, its weights over the bins (to w_out when not
// NULL) and, with gate.row_map, the coarse gate.
int launch_prop_front(const float *params, const float *rays_o, const float *rays_d, const float *near,
                      const float *far, const float *u, unsigned long long seed, int R, int S, int perturb,
                      int lin_inv, int mode, float *xyz, float *t_vals, float *edges, float *widths, float *w_out,
                      const CompositeGate &gate, cudaStream_t stream);

#ifdef NERF_BOUNDS_CHECK
// Error words of the bounds-check build, one per translation unit (common.cuh).
int bounds_read_ray_ops(int reset);
int bounds_read_gate(int reset);
int bounds_read_mlp(int reset);
int bounds_read_proposal(int reset);
int bounds_read_mlp_tc(int reset);
#endif

}  // namespace nerfgb
