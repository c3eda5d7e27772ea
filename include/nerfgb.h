/*
 * nerfgb.h - C ABI of libnerfgb.so, the GB300 (sm_103a) render path of
 * nerf-tf2: stratified sampling, positional encoding, the coarse/fine
 * 8x256 MLP, alpha compositing and the inverse-transform fine sampler.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless stated otherwise.
 *    Tensors are dense, row-major, float32 (int32 for indices).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream). Every call is enqueued on it and returns without a host sync.
 *  - The caller allocates every output and workspace; no entry point
 *    allocates device memory. One exception holds memory for the life of
 *    the process: the 16 MiB scratch array of
 *    nerfgb_render_rays_noalloc (a static device array, reserved when the
 *    library's module loads on a device).
 *  - Every entry point returns NERFGB_OK (0) or a negative NERFGB_E_* code.
 *    None aborts, throws or exits.
 *  - Kernels with bounded device-side waits report a timeout through
 *    `err_word` (a caller-zeroed device int32). Read it after a sync and
 *    decode it with nerfgb_status_string().
 *
 * The reference (thatbrguy/nerf-tf2, TensorFlow 2.6) has no native code and no
 * FFI. Each entry point below names the Python function it replaces; the
 * Python mirror in the package binds them with ctypes under the reference's
 * names.
 */
#ifndef NERFGB_H_
#define NERFGB_H_

#ifdef __cplusplus
extern "C" {
#endif

#define NERFGB_ABI_VERSION 2

/* Status codes. */
#define NERFGB_OK 0
#define NERFGB_E_INVALID_ARG (-1) /* null pointer, negative size, misaligned  */
#define NERFGB_E_UNSUPPORTED (-2) /* size or flag outside the kernels' range  */
#define NERFGB_E_CUDA (-3)        /* CUDA launch or runtime error              */
#define NERFGB_E_TIMEOUT (-4)     /* a bounded device wait ran out            */
#define NERFGB_E_DEVICE (-5)      /* no usable sm_103 device                  */
#define NERFGB_E_SCRATCH_LIMIT (-6) /* request needs more than the built-in scratch */

/* Flags of nerfgb_render_rays_gated. */
#define NERFGB_GATE_FINE_DRAWS 1 /* gate the fine draws by their coarse bins too */

/* MLP arithmetic precision. */
#define NERFGB_PREC_FP32 0 /* FP32 SIMT, FP32 accumulate                      */
#define NERFGB_PREC_BF16 1 /* BF16 tcgen05 GEMMs, FP32 accumulate (TMEM)      */
#define NERFGB_PREC_FP8 2  /* FP8-e4m3 tcgen05 GEMMs (per-output-channel weight
                              scales), FP32 accumulate (TMEM)               */

/* Transmittance evaluation in the compositor. */
#define NERFGB_TRANS_CUMPROD 0 /* sequential FP32 product, as written          */
#define NERFGB_TRANS_LOGSUM 1  /* exp of a compensated FP32 log-sum            */

int nerfgb_abi_version(void);
const char *nerfgb_status_string(int status);

/* ---- parameters of one coarse or fine network ------------------------ */

/* Number of float32 values in the flat parameter blob of one network:
 * dense_0..dense_7, sigma, dense_8, dense_9, rgb; per layer the Keras kernel
 * [in,out] row-major followed by the bias [out]. The layers are those built
 * by get_coarse_or_fine_model (nerf/core/model.py:334-394). */
long long nerfgb_mlp_param_count(void);

/* Bytes of the packed device layout that the MLP kernels read for
 * `precision`. */
long long nerfgb_mlp_packed_bytes(int precision);

/* Packs a device float32 parameter blob into `packed`
 * (nerfgb_mlp_packed_bytes(precision) bytes, 256-byte aligned). */
int nerfgb_mlp_pack(const float *params, int precision, void *packed,
                    void *stream);

/* ---- ray operators ----------------------------------------------------- */

/* Replaces ray_utils.create_input_batch_coarse_model
 * (nerf/utils/ray_utils.py:137-274). Inputs rays_o, rays_d [R,3]; near, far
 * [R,1]; u_vals [R,S] uniforms in [0,1) (read only when perturb != 0; they
 * stand in for tf.random.uniform at :230). Outputs xyz, dirs [R*S,3]
 * (dirs may be NULL), t_vals [R,S], bin_edges [R,S+1], bin_widths [R,S].
 * left_edges/right_edges are views of bin_edges. 1 <= S <= 1024. */
int nerfgb_coarse_sample(const float *rays_o, const float *rays_d,
                         const float *near, const float *far,
                         const float *u_vals, int n_rays, int n_coarse,
                         int perturb, int lin_inv_depth, float *xyz,
                         float *dirs, float *t_vals, float *bin_edges,
                         float *bin_widths, void *stream);

/* Replaces ray_utils.create_input_batch_fine_model
 * (nerf/utils/ray_utils.py:276-406). bin_weights, bin_widths, t_vals_coarse
 * [R,Sc]; left_edges rows of length Sc at row stride ld_left (Sc+1 when it
 * is a view of bin_edges); u_vals [R,Sf] stand in for tf.random.uniform at
 * :355. Outputs xyz, dirs [R*(Sc+Sf),3] (dirs may be NULL), t_vals
 * [R,Sc+Sf] sorted ascending; optional piece_idxs [R,Sf] (the searchsorted
 * result) and sort_perm [R,Sc+Sf] (stable argsort of concat(t_c, t_f)).
 * 2 <= Sc <= 256, 1 <= Sf <= 512. */
int nerfgb_fine_sample(const float *rays_o, const float *rays_d,
                       const float *bin_weights, const float *left_edges,
                       int ld_left, const float *bin_widths,
                       const float *t_vals_coarse, const float *u_vals,
                       int n_rays, int n_coarse, int n_fine, float *xyz,
                       float *dirs, float *t_vals, int *piece_idxs,
                       int *sort_perm, void *stream);

/* Replaces ray_utils.post_process_model_output (ray_utils.py:484-551) with
 * compute_weights (:426-482) and sigma_to_alpha (:408-424) inside.
 * sample_rgb [R*S,3], sigma [R*S], t_vals [R,S] -> weights [R,S] (may be
 * NULL), pred_rgb [R,3], pred_depth [R], acc_map [R]. 1 <= S <= 2048. */
int nerfgb_composite(const float *sample_rgb, const float *sigma,
                     const float *t_vals, int n_rays, int n_samples,
                     int white_bg, int trans_mode, float *weights,
                     float *pred_rgb, float *pred_depth, float *acc_map,
                     void *stream);

/* Replaces ray_utils.sigma_to_alpha (ray_utils.py:408-424):
 * alpha = 1 - exp(-sigma * diffs), n elements. */
int nerfgb_sigma_to_alpha(const float *sigma, const float *diffs,
                          long long n, float *alpha, void *stream);

/* Replaces PositionalEncoder(L).call (nerf/core/model.py:319-331):
 * x [n,3] -> out [n, 3 + 6L]. 1 <= L <= 16. */
int nerfgb_positional_encode(const float *x, long long n, int L, float *out,
                             void *stream);

/* Replaces the Keras model returned by get_coarse_or_fine_model
 * (nerf/core/model.py:334-394) called on (xyz, dirs): xyz [n,3]; dirs
 * [ceil(n/rows_per_dir), 3] (row i uses dirs[i / rows_per_dir]; 1 = one
 * direction per sample as in the reference). Outputs rgb [n,3], sigma [n].
 * `packed` comes from nerfgb_mlp_pack with the same precision. err_word:
 * caller-zeroed device int32 (may be NULL for FP32). */
int nerfgb_mlp_forward(const void *packed, int precision, const float *xyz,
                       const float *dirs, long long n_rows, int rows_per_dir,
                       float *rgb, float *sigma, int *err_word, void *stream);

/* nerfgb_mlp_forward through a row map: logical row k in [0, n) reads xyz
 * row row_map[k] and dirs row row_map[k] / rows_per_dir and writes rgb/sigma
 * row row_map[k]; n = min(*n_rows_dev, n_rows_max) read on the device (the
 * count a gate kernel left there). row_map NULL: the identity; n_rows_dev
 * NULL: n = n_rows_max. Rows not mapped are left untouched. */
int nerfgb_mlp_forward_mapped(const void *packed, int precision,
                              const float *xyz, const float *dirs,
                              long long n_rows_max, int rows_per_dir,
                              const int *row_map, const int *n_rows_dev,
                              float *rgb, float *sigma, int *err_word,
                              void *stream);

/* Diagnostic of the tensor-core kernels' failure path (no counterpart in the
 * reference, which surfaces TensorFlow's errors): nerfgb_mlp_forward at
 * precision BF16 or FP8 with every bounded device wait limited to wait_ns
 * (1e3 .. 1e10 ns; the default kernels use 2 s) and, when withhold_chunk >=
 * 0, the weight chunk at that position of the (even) CTA's load sequence
 * left unloaded, so that the MMA issuer's wait runs out. The kernel then
 * writes NERFGB_E_TIMEOUT to *err_word, drains its copies and MMAs, frees
 * its tensor memory and returns; the outputs are unspecified. */
int nerfgb_mlp_forward_wait_test(const void *packed, int precision,
                                 const float *xyz, const float *dirs,
                                 long long n_rows, int rows_per_dir,
                                 float *rgb, float *sigma, int *err_word,
                                 unsigned long long wait_ns,
                                 long long withhold_chunk, void *stream);

/* Status of the bounds-check build (compiled with -DNERF_BOUNDS_CHECK, as
 * libnerfgb_bounds.so): every index the kernels compute from data (the fine
 * sampler's searchsorted bins and sort positions, the gates' sort-permutation
 * entries and row-map slots, the MLP's row-map rows) is checked against its
 * buffer; an index out of range is clamped to 0 and the first failing
 * check's site code (1..9, see csrc/common.cuh) is recorded. Returns 0 when
 * no check failed, the site code otherwise, NERFGB_E_UNSUPPORTED in the
 * normal build. Synchronises the device; reset != 0 clears the record. No
 * counterpart in the reference. */
int nerfgb_bounds_check_status(int reset);

/* ---- ray generation ------------------------------------------------- */

/* Replaces get_rays_tf (nerf/utils/ray_utils.py:53-106): rays_o, rays_d
 * [H*W, 3] for pixel p = v*W + u of a pinhole camera, intrinsic [3,3] and
 * c2w [4,4] row-major float32 device arrays. d = R (x, y, 1) with
 * x = (u - cx)/fx, y = (v - cy)/fy, normalised by sqrt(d.d) + 1e-8; the
 * rotation and the norm are sequential float32 sums. */
int nerfgb_get_rays(int H, int W, const float *intrinsic, const float *c2w,
                    float *rays_o, float *rays_d, void *stream);

/* Replaces the sample-mode map function (nerf/core/base_dataset.py:555-621)
 * for one image: ray b of the batch is get_rays_tf's ray of pixel idxs[b]
 * (device int32 [batch], drawn by the caller, e.g. nerfgb_uniform_int; the
 * reference draws them with tf.random.uniform), with near/far and
 * rgb = image / 255 (image: uint8 [H, W, 3] on the device). Outputs rays_o,
 * rays_d, rgb [batch, 3], near_out, far_out [batch]. An index outside
 * [0, H*W) yields zeros. */
int nerfgb_sample_rays(const unsigned char *image, int H, int W,
                       const float *intrinsic, const float *c2w, float near,
                       float far, const int *idxs, int batch, float *rays_o,
                       float *rays_d, float *near_out, float *far_out,
                       float *rgb, void *stream);

/* Replaces create_depth_map (nerf/utils/ray_utils.py:108-135): out [n] =
 * pred_depth / scale_factor (map_type 1) or the camera-frame z of
 * rays_o + rays_d * pred_depth / scale_factor under w2c [4,4] (map_type 2;
 * the rays of the frame, e.g. from nerfgb_get_rays). */
int nerfgb_depth_map(const float *pred_depth, long long n, float scale_factor,
                     int map_type, const float *rays_o, const float *rays_d,
                     const float *w2c, float *out, void *stream);

/* ---- uniforms -------------------------------------------------------- */

/* Fills out[0..n) with uniforms in [0,1) from Philox4x32-10 keyed by seed;
 * element i uses counter (offset + i). Used when the caller supplies no
 * jitter uniforms (the reference draws them with tf.random.uniform). */
int nerfgb_uniform(unsigned long long seed, unsigned long long offset,
                   long long n, float *out, void *stream);

/* Integers in [0, maxval): out[i] = (w * maxval) >> 32 for the 32-bit word
 * w = offset + i of the same Philox4x32-10 stream. */
int nerfgb_uniform_int(unsigned long long seed, unsigned long long offset,
                       long long n, int maxval, int *out, void *stream);

/* ---- fused render --------------------------------------------------- */

/* Workspace bytes that nerfgb_render_rays needs for n_rays rays. */
long long nerfgb_render_workspace_bytes(int n_rays, int n_coarse, int n_fine);

/* Replaces NeRF.forward (nerf/core/model.py:57-125) for inference: coarse
 * sample -> coarse MLP -> composite -> fine sample -> fine MLP -> composite.
 * rays_o, rays_d [R,3]; near, far [R,1]; u_coarse [R,Sc] and u_fine [R,Sf]
 * may be NULL, in which case uniforms come from Philox keyed by `seed`.
 * Outputs [R,3] rgb and [R] depth/acc of the coarse pass (may be NULL) and
 * of the fine pass. `workspace` holds nerfgb_render_workspace_bytes bytes. */
int nerfgb_render_rays(const void *packed_coarse, const void *packed_fine,
                       int precision, const float *rays_o,
                       const float *rays_d, const float *near,
                       const float *far, const float *u_coarse,
                       const float *u_fine, unsigned long long seed,
                       int n_rays, int n_coarse, int n_fine, int perturb,
                       int lin_inv_depth, int white_bg, int trans_mode,
                       float *rgb_coarse, float *depth_coarse,
                       float *acc_coarse, float *rgb_fine, float *depth_fine,
                       float *acc_fine, void *workspace, int *err_word,
                       void *stream);

/* ---- learned proposal sampler (not in the reference) ------------------- */

/* Parameters of the proposal network: a 2x64 ReLU MLP on the L=6 positional
 * encoding of xyz (39 inputs) with a softplus density output. Flat float32
 * blob of 6,785 values: W1 [39,64], b1 [64], W2 [64,64], b2 [64], W3 [64],
 * b3 [1]. */
long long nerfgb_proposal_param_count(void);

/* sigma [n] = proposal density at xyz [n,3]. */
int nerfgb_proposal_forward(const float *params, const float *xyz, long long n,
                            float *sigma, void *stream);

/* nerfgb_proposal_forward on tensor cores: BF16 operands, FP32 accumulation
 * (the encoding and the last layer in FP32). The render paths use it with a
 * BF16 or FP8 NeRF MLP, and nerfgb_proposal_forward with an FP32 one. */
int nerfgb_proposal_forward_bf16(const float *params, const float *xyz,
                                 long long n, float *sigma, void *stream);

/* grad_params [6785] += d/dparams of sum_i grad_sigma[i] * sigma_i
 * (accumulates; zero it first). */
int nerfgb_proposal_backward(const float *params, const float *xyz,
                             const float *grad_sigma, long long n,
                             float *grad_params, void *stream);

/* Volume-rendering weights [R, n_bins] of the proposal's densities sigma
 * [R*n_bins] at t_vals [R, n_bins]: compute_weights (ray_utils.py:426-482)
 * except that the last interval is the previous spacing instead of 1e10,
 * so the last bin's weight stays differentiable and can be 0. */
int nerfgb_proposal_weights(const float *sigma, const float *t_vals,
                            int n_rays, int n_bins, int trans_mode,
                            float *weights, void *stream);

/* dL/dsigma [R*n_bins] of nerfgb_proposal_weights given dL/dweights. */
int nerfgb_proposal_weights_backward(const float *sigma, const float *t_vals,
                                     const float *grad_weights, int n_rays,
                                     int n_bins, float *grad_sigma,
                                     void *stream);

/* nerfgb_render_rays with the proposal network in place of the coarse MLP:
 * its density at the Sc stratified samples, composited as the coarse pass
 * is, gives the PDF of the fine sampler; the fine MLP then runs on the
 * Sc + Sf sorted samples. The proposal's weights are those of
 * nerfgb_proposal_weights; the proposal runs in FP32 with an FP32 MLP and
 * in BF16 (nerfgb_proposal_forward_bf16) otherwise. Outputs the fine
 * rgb/depth/acc maps. Same workspace size as nerfgb_render_rays. */
int nerfgb_render_rays_proposal(const float *proposal_params,
                                const void *packed_fine, int precision,
                                const float *rays_o, const float *rays_d,
                                const float *near, const float *far,
                                const float *u_coarse, const float *u_fine,
                                unsigned long long seed, int n_rays,
                                int n_coarse, int n_fine, int perturb,
                                int lin_inv_depth, int white_bg,
                                int trans_mode, float *rgb_fine,
                                float *depth_fine, float *acc_fine,
                                void *workspace, int *err_word, void *stream);

/* Coarse sample gate: sample (r, j) is on where weights[r*S + j] > tau (NaN:
 * off). Writes mask [R*S] (0/1), appends the on samples' indices r*S + j to
 * row_map (rays in any order, each ray's samples in order) and adds their
 * number to *count (device; zero it first). */
int nerfgb_gate_coarse(const float *weights, int n_rays, int n_samples,
                       float tau, unsigned char *mask, int *row_map,
                       int *count, void *stream);

/* Fine sample gate over the sorted coarse+fine union [R, n_samples]: member
 * j is on where it is a coarse sample whose mask is on, or a fine draw
 * (sort_perm >= n_coarse). With piece_idxs (the fine sampler's bin of each
 * draw, [R, n_samples - n_coarse]; NULL: every draw on) a fine draw is on
 * only where its bin's coarse mask is on. Appends r*n_samples + j to
 * row_map, adds to *count. */
int nerfgb_gate_fine(const int *sort_perm, const unsigned char *mask_coarse,
                     const int *piece_idxs, int n_rays, int n_coarse,
                     int n_samples, int *row_map, int *count, void *stream);

/* Workspace bytes of nerfgb_render_rays_gated (more than
 * nerfgb_render_workspace_bytes: the gates' masks and row maps). */
long long nerfgb_render_gated_workspace_bytes(int n_rays, int n_coarse,
                                              int n_fine);

/* The proposal-gated render: the coarse -> fine chain of nerfgb_render_rays,
 * with the proposal (FP32 with an FP32 MLP, BF16 otherwise) deciding which
 * samples the NeRF MLP evaluates. Coarse
 * samples whose proposal weight (nerfgb_proposal_weights of the proposal
 * density at the stratified samples) is at most gate_tau get sigma = 0 and
 * are not evaluated, in the coarse pass and again in the fine pass's sorted
 * union. The fine draws are evaluated unless gate_flags has
 * NERFGB_GATE_FINE_DRAWS: then a draw whose coarse bin is off is not
 * evaluated either (sigma = 0; a ray whose bins are all off costs no MLP
 * rows). gate_tau < 0 evaluates every sample and reproduces
 * nerfgb_render_rays' fine maps bit for bit. */
int nerfgb_render_rays_gated(const float *proposal_params,
                             const void *packed_coarse,
                             const void *packed_fine, int precision,
                             const float *rays_o, const float *rays_d,
                             const float *near, const float *far,
                             const float *u_coarse, const float *u_fine,
                             unsigned long long seed, int n_rays,
                             int n_coarse, int n_fine, int perturb,
                             int lin_inv_depth, int white_bg, int trans_mode,
                             float gate_tau, int gate_flags, float *rgb_fine,
                             float *depth_fine, float *acc_fine,
                             void *workspace, int *err_word, void *stream);

/* ---- training --------------------------------------------------------- */

/* Gradient of compositing (ray_utils.py:408-551, differentiated as
 * tf.GradientTape does at nerf/core/model.py:148-170): given dL/dpred_rgb
 * [R,3] and/or dL/dweights [R,S] (either may be NULL, not both), writes
 * dL/dsigma [R*S] and, when grad_sample_rgb is not NULL, dL/dsample_rgb
 * [R*S,3]. sample_rgb is needed only with grad_rgb_map. */
int nerfgb_composite_backward(const float *sigma, const float *t_vals,
                              const float *sample_rgb,
                              const float *grad_rgb_map,
                              const float *grad_weights, int n_rays,
                              int n_samples, int white_bg, float *grad_sigma,
                              float *grad_sample_rgb, void *stream);

/* keras.losses.MeanSquaredError (nerf/core/model.py:32, :157-168) over n
 * elements, times `scale`: *loss += scale * mean((pred - target)^2) (loss may
 * be NULL), grad[i] = scale * 2 (pred - target) / n (grad may be NULL). */
int nerfgb_mse_loss(const float *pred, const float *target, long long n,
                    float scale, float *loss, float *grad, void *stream);

/* Envelope loss of the proposal on weight histograms [R, n_bins]:
 * *loss += sum (1 + lam [w_prop < w_target]) (w_prop - w_target)^2 / R;
 * grad = dloss/dw_prop. */
int nerfgb_envelope_loss(const float *w_prop, const float *w_target,
                         int n_rays, int n_bins, float lam, float *loss,
                         float *grad, void *stream);

/* One Adam step as TensorFlow's ApplyAdam computes it for Keras Adam
 * (nerf/core/model.py:413-418): lr_t = lr sqrt(1 - b2^step) / (1 - b1^step);
 * m += (g - m)(1 - b1); v += (g^2 - v)(1 - b2); p -= lr_t m / (sqrt(v) + eps).
 * step >= 1. */
int nerfgb_adam_step(float *params, float *m, float *v, const float *grads,
                     long long n, float lr, float beta1, float beta2,
                     float eps, long long step, void *stream);

/* Floats of stored activations per MLP row (enc_xyz, h0..h7, bottleneck,
 * enc_dir, h9) written by nerfgb_mlp_forward_train. */
long long nerfgb_mlp_acts_floats_per_row(void);

/* The FP32 MLP forward of nerfgb_mlp_forward that also stores every layer's
 * activations in acts [n_rows, nerfgb_mlp_acts_floats_per_row()] for the
 * backward (the tape that tf.GradientTape keeps, nerf/core/model.py:148).
 * `packed` is an FP32 pack. */
int nerfgb_mlp_forward_train(const void *packed, const float *xyz,
                             const float *dirs, long long n_rows,
                             int rows_per_dir, float *rgb, float *sigma,
                             float *acts, void *stream);

/* Workspace bytes of nerfgb_mlp_backward for n_rows rows. */
long long nerfgb_mlp_backward_workspace_bytes(long long n_rows);

/* Gradient of sum(d_rgb * rgb + d_sigma * sigma) of the MLP w.r.t. its flat
 * parameter blob (Keras layout, nerfgb_mlp_param_count floats), ACCUMULATED
 * into grad_params. acts from nerfgb_mlp_forward_train on the same rows with
 * the same FP32 pack. d_sigma may be NULL. FP32 throughout. */
int nerfgb_mlp_backward(const void *packed, const float *acts, long long n_rows,
                        const float *d_rgb, const float *d_sigma,
                        float *grad_params, void *workspace, void *stream);

/* ---- BF16 training (tensor cores, FP32 master weights) ------------------ */

/* nerfgb_mlp_forward with the BF16 pack that also writes the BF16 activation
 * tape: [n_rows][nerfgb_mlp_acts_floats_per_row()] BF16 values (uint16
 * bits) at the FP32 tape's columns, each the operand the next layer's GEMM
 * read; tape 16-byte aligned. err_word: caller-zeroed device int32. */
int nerfgb_mlp_forward_train_bf16(const void *packed_bf16, const float *xyz,
                                  const float *dirs, long long n_rows,
                                  int rows_per_dir, float *rgb, float *sigma,
                                  void *tape, int *err_word, void *stream);

/* Workspace bytes of nerfgb_mlp_backward_bf16 for n_rows rows. */
long long nerfgb_mlp_backward_bf16_workspace_bytes(long long n_rows);

/* nerfgb_mlp_backward from a BF16 tape: every dX and dW product is a BF16
 * tensor-core GEMM (tcgen05) with FP32 accumulation, against a BF16 copy of
 * the FP32 master weights in packed_fp32 (the FP32 pack); bias and head
 * gradients in FP32. grad_params accumulates (zero it first). err_word:
 * caller-zeroed device int32 for the GEMMs' bounded waits. */
int nerfgb_mlp_backward_bf16(const void *packed_fp32, const void *tape,
                             long long n_rows, const float *d_rgb,
                             const float *d_sigma, float *grad_params,
                             void *workspace, int *err_word, void *stream);

/* ---- fused render without allocation --------------------------------- */

/* Size of the built-in scratch array of nerfgb_render_rays_noalloc: 16 MiB,
 * enough for 1,700 rays per call at 64 coarse + 128 fine samples
 * (nerfgb_render_workspace_bytes gives the need of a request). */
#define NERFGB_NOALLOC_SCRATCH_BYTES (16u << 20)

/* No counterpart in the reference. nerfgb_render_rays for callers that
 * cannot allocate device memory (for example code running inside a framework
 * that has reserved the GPU's memory for its own allocator, as TensorFlow
 * does): same arguments without `workspace`. The intermediates live in a
 * library-owned device array of NERFGB_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this code holds until the process exits; the call allocates
 * nothing. Requests needing more return NERFGB_E_SCRATCH_LIMIT (render in
 * smaller chunks). The first call in each CUDA context (once per device for
 * the runtime's primary context, and again after cudaDeviceReset, which
 * reloads the module) looks up the array's address; make it before any
 * stream capture. All calls share the array: calls that overlap on the GPU
 * race and must be serialised. */
int nerfgb_render_rays_noalloc(const void *packed_coarse,
                               const void *packed_fine, int precision,
                               const float *rays_o, const float *rays_d,
                               const float *near, const float *far,
                               const float *u_coarse, const float *u_fine,
                               unsigned long long seed, int n_rays,
                               int n_coarse, int n_fine, int perturb,
                               int lin_inv_depth, int white_bg,
                               int trans_mode, float *rgb_coarse,
                               float *depth_coarse, float *acc_coarse,
                               float *rgb_fine, float *depth_fine,
                               float *acc_fine, int *err_word, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NERFGB_H_ */
