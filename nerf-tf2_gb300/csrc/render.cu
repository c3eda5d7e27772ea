// Fused render: the inference body of NeRF.forward (nerf/core/model.py:57-125)
// as one C-ABI call over caller-provided workspace. The chain is the one the
// reference runs: coarse sample -> coarse MLP -> composite -> fine sample ->
// fine MLP -> composite. Directions are read per ray (rows_per_dir = samples
// per ray), so the broadcast dir_inputs tensor is never materialised.
#include "common.cuh"
#include "mlp_internal.cuh"

namespace nerfgb {

struct RenderWs {
  float *u_c, *u_f, *xyz_c, *t_c, *edges, *widths, *rgb_c, *sig_c, *w_c, *xyz_f, *t_f, *rgb_f, *sig_f;
  float *map_rgb_c, *map_depth_c, *map_acc_c;
  long long bytes;
};

static long long align256(long long b) { return (b + 255) / 256 * 256; }

static RenderWs carve(void *base, int R, int Sc, int Sf) {
  RenderWs w{};
  const long long r = R, S = Sc + Sf;
  const long long sizes[16] = {r * Sc, r * Sf, r * Sc * 3, r * Sc, r * (Sc + 1), r * Sc, r * Sc * 3, r * Sc,
                               r * Sc, r * S * 3, r * S,    r * S * 3, r * S,       r * 3,  r,          r};
  float **slots[16] = {&w.u_c,   &w.u_f,  &w.xyz_c, &w.t_c,   &w.edges,     &w.widths,
                       &w.rgb_c, &w.sig_c, &w.w_c,  &w.xyz_f, &w.t_f,       &w.rgb_f,
                       &w.sig_f, &w.map_rgb_c, &w.map_depth_c, &w.map_acc_c};
  long long off = 0;
  for (int i = 0; i < 16; ++i) {
    if (base) *slots[i] = reinterpret_cast<float *>(static_cast<char *>(base) + off);
    off += align256(sizes[i] * (long long)sizeof(float));
  }
  w.bytes = off;
  return w;
}

// The proposal runs at the render's precision class: FP32 with an FP32 MLP,
// BF16 operands (tensor cores, FP32 accumulation) with a BF16 or FP8 MLP.
static int launch_proposal(int precision, const float *params, const float *xyz, long long n, float *sigma,
                           cudaStream_t stream) {
  return precision == NERFGB_PREC_FP32 ? launch_proposal_forward(params, xyz, n, sigma, stream)
                                       : launch_proposal_forward_bf16(params, xyz, n, sigma, stream);
}

int launch_mlp(const void *packed, int precision, const float *xyz, const float *dirs, long long n, int rpd,
               float *rgb, float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm) {
  if (precision == NERFGB_PREC_FP32) return launch_mlp_fp32(packed, xyz, dirs, n, rpd, rgb, sigma, stream, rm);
  if (precision == NERFGB_PREC_FP8)
    return launch_mlp_fp8(packed, xyz, dirs, n, rpd, rgb, sigma, err_word, stream, rm);
  return launch_mlp_bf16(packed, xyz, dirs, n, rpd, rgb, sigma, err_word, stream, rm);
}

}  // namespace nerfgb

using namespace nerfgb;

extern "C" int nerfgb_bounds_check_status(int reset) {
#ifdef NERF_BOUNDS_CHECK
  const int v[5] = {bounds_read_ray_ops(reset), bounds_read_gate(reset), bounds_read_mlp(reset),
                    bounds_read_mlp_tc(reset), bounds_read_proposal(reset)};
  for (int i = 0; i < 5; ++i)
    if (v[i] < 0) return NERFGB_E_CUDA;
  for (int i = 0; i < 5; ++i)
    if (v[i] != 0) return v[i];
  return NERFGB_OK;
#else
  (void)reset;
  return NERFGB_E_UNSUPPORTED;
#endif
}

extern "C" long long nerfgb_render_workspace_bytes(int n_rays, int n_coarse, int n_fine) {
  if (n_rays < 0 || n_coarse < 1 || n_fine < 0) return -1;
  return carve(nullptr, n_rays, n_coarse, n_fine).bytes;
}

extern "C" int nerfgb_render_rays(const void *packed_coarse, const void *packed_fine, int precision,
                                  const float *rays_o, const float *rays_d, const float *near, const float *far,
                                  const float *u_coarse, const float *u_fine, unsigned long long seed,
                                  int n_rays, int n_coarse, int n_fine, int perturb, int lin_inv_depth,
                                  int white_bg, int trans_mode, float *rgb_coarse, float *depth_coarse,
                                  float *acc_coarse, float *rgb_fine, float *depth_fine, float *acc_fine,
                                  void *workspace, int *err_word, void *stream) {
  if (n_rays < 0 || n_coarse < 2 || n_fine < 1) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8)
    return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!packed_coarse || !packed_fine || !rays_o || !rays_d || !near || !far || !rgb_fine || !depth_fine ||
      !acc_fine || !workspace || !aligned(workspace, 256))
    return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && !err_word) return NERFGB_E_INVALID_ARG;
  cudaStream_t st = as_stream(stream);
  const int R = n_rays, Sc = n_coarse, Sf = n_fine, S = Sc + Sf;
  RenderWs w = carve(workspace, R, Sc, Sf);
  int rc;
  // Uniforms not supplied are drawn in the samplers from Philox keyed by
  // seed: coarse draws use counters [0, R*Sc), fine draws [R*Sc, R*S).
  if (trans_mode != NERFGB_TRANS_CUMPROD && trans_mode != NERFGB_TRANS_LOGSUM) return NERFGB_E_UNSUPPORTED;
  if ((rc = launch_coarse_sample(rays_o, rays_d, near, far, u_coarse, seed, R, Sc, perturb, lin_inv_depth, w.xyz_c,
                                 nullptr, w.t_c, w.edges, w.widths, st)) != NERFGB_OK)
    return rc;
  if ((rc = launch_mlp(packed_coarse, precision, w.xyz_c, rays_d, (long long)R * Sc, Sc, w.rgb_c, w.sig_c,
                       err_word, st)) != NERFGB_OK)
    return rc;
  // the coarse pass's compositing (and its maps, when asked for) inside the fine sampler
  FineFuse fz;
  fz.sigma_c = w.sig_c;
  fz.mode = trans_mode;
  fz.white_bg = white_bg;
  fz.seed = seed;
  if (rgb_coarse || depth_coarse || acc_coarse) {
    fz.rgb_c = w.rgb_c;
    fz.map_rgb = rgb_coarse ? rgb_coarse : w.map_rgb_c;
    fz.map_depth = depth_coarse ? depth_coarse : w.map_depth_c;
    fz.map_acc = acc_coarse ? acc_coarse : w.map_acc_c;
  }
  if ((rc = launch_fine_sample(rays_o, rays_d, nullptr, w.edges, Sc + 1, w.widths, w.t_c, u_fine, R, Sc, Sf, w.xyz_f,
                               nullptr, w.t_f, nullptr, nullptr, st, fz)) != NERFGB_OK)
    return rc;
  if ((rc = launch_mlp(packed_fine, precision, w.xyz_f, rays_d, (long long)R * S, S, w.rgb_f, w.sig_f, err_word,
                       st)) != NERFGB_OK)
    return rc;
  return nerfgb_composite(w.rgb_f, w.sig_f, w.t_f, R, S, white_bg, trans_mode, nullptr, rgb_fine, depth_fine,
                          acc_fine, stream);
}

extern "C" int nerfgb_render_rays_proposal(const float *proposal_params, const void *packed_fine, int precision,
                                           const float *rays_o, const float *rays_d, const float *near,
                                           const float *far, const float *u_coarse, const float *u_fine,
                                           unsigned long long seed, int n_rays, int n_coarse, int n_fine,
                                           int perturb, int lin_inv_depth, int white_bg, int trans_mode,
                                           float *rgb_fine, float *depth_fine, float *acc_fine, void *workspace,
                                           int *err_word, void *stream) {
  if (n_rays < 0 || n_coarse < 2 || n_fine < 1) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8)
    return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!proposal_params || !packed_fine || !rays_o || !rays_d || !near || !far || !rgb_fine || !depth_fine ||
      !acc_fine || !workspace || !aligned(workspace, 256))
    return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && !err_word) return NERFGB_E_INVALID_ARG;
  cudaStream_t st = as_stream(stream);
  const int R = n_rays, Sc = n_coarse, Sf = n_fine, S = Sc + Sf;
  RenderWs w = carve(workspace, R, Sc, Sf);
  int rc;
  // The proposal density at the stratified samples replaces the coarse MLP;
  // its weights are the fine sampler's PDF.
  if (precision == NERFGB_PREC_FP32) {
    if ((rc = launch_coarse_sample(rays_o, rays_d, near, far, u_coarse, seed, R, Sc, perturb, lin_inv_depth,
                                   w.xyz_c, nullptr, w.t_c, w.edges, w.widths, st)) != NERFGB_OK)
      return rc;
    if ((rc = launch_proposal(precision, proposal_params, w.xyz_c, (long long)R * Sc, w.sig_c, st)) != NERFGB_OK)
      return rc;
    if ((rc = nerfgb_proposal_weights(w.sig_c, w.t_c, R, Sc, trans_mode, w.w_c, stream)) != NERFGB_OK) return rc;
  } else if ((rc = launch_prop_front(proposal_params, rays_o, rays_d, near, far, u_coarse, seed, R, Sc, perturb,
                                     lin_inv_depth, trans_mode, w.xyz_c, w.t_c, w.edges, w.widths, w.w_c,
                                     CompositeGate(), st)) != NERFGB_OK) {
    return rc;
  }
  FineFuse fz;
  fz.seed = seed;
  if ((rc = launch_fine_sample(rays_o, rays_d, w.w_c, w.edges, Sc + 1, w.widths, w.t_c, u_fine, R, Sc, Sf, w.xyz_f,
                               nullptr, w.t_f, nullptr, nullptr, st, fz)) != NERFGB_OK)
    return rc;
  if ((rc = launch_mlp(packed_fine, precision, w.xyz_f, rays_d, (long long)R * S, S, w.rgb_f, w.sig_f, err_word,
                       st)) != NERFGB_OK)
    return rc;
  return nerfgb_composite(w.rgb_f, w.sig_f, w.t_f, R, S, white_bg, trans_mode, nullptr, rgb_fine, depth_fine,
                          acc_fine, stream);
}

// ---------------------------------------------------------------------------
// Proposal-gated render: the plain coarse -> fine chain, with the learned
// proposal deciding which samples the NeRF MLP evaluates. Coarse samples
// whose proposal weight (finite-bin compositing of the proposal density) is
// at most gate_tau get sigma = 0 and are not evaluated, in the coarse pass
// and again as members of the fine pass's sorted union; the fine draws are
// evaluated unless NERFGB_GATE_FINE_DRAWS gates them by their coarse bins'
// decisions as well. With gate_tau < 0 every sample is evaluated and the
// result equals nerfgb_render_rays bit for bit.
// ---------------------------------------------------------------------------
namespace nerfgb {

struct GateWs {
  float *sig_p, *w_p;
  unsigned char *mask_c;
  int *map_c, *map_f, *perm, *counts;
  long long bytes;
};

static GateWs carve_gate(void *base, int R, int Sc, int Sf) {
  GateWs g{};
  const long long r = R, S = Sc + Sf;
  long long off = carve(nullptr, R, Sc, Sf).bytes;
  auto take = [&](long long bytes) -> char * {
    char *p = base ? static_cast<char *>(base) + off : nullptr;
    off += align256(bytes);
    return p;
  };
  g.sig_p = reinterpret_cast<float *>(take(r * Sc * 4));
  g.w_p = reinterpret_cast<float *>(take(r * Sc * 4));
  g.mask_c = reinterpret_cast<unsigned char *>(take(r * Sc));
  g.map_c = reinterpret_cast<int *>(take(r * Sc * 4));
  g.map_f = reinterpret_cast<int *>(take(r * S * 4));
  g.perm = reinterpret_cast<int *>(take(r * S * 4));
  g.counts = reinterpret_cast<int *>(take(2 * 4));
  g.bytes = off;
  return g;
}

}  // namespace nerfgb

extern "C" long long nerfgb_render_gated_workspace_bytes(int n_rays, int n_coarse, int n_fine) {
  if (n_rays < 0 || n_coarse < 1 || n_fine < 0) return -1;
  return carve_gate(nullptr, n_rays, n_coarse, n_fine).bytes;
}

extern "C" int nerfgb_render_rays_gated(const float *proposal_params, const void *packed_coarse,
                                        const void *packed_fine, int precision, const float *rays_o,
                                        const float *rays_d, const float *near, const float *far,
                                        const float *u_coarse, const float *u_fine, unsigned long long seed,
                                        int n_rays, int n_coarse, int n_fine, int perturb, int lin_inv_depth,
                                        int white_bg, int trans_mode, float gate_tau, int gate_flags,
                                        float *rgb_fine,
                                        float *depth_fine, float *acc_fine, void *workspace, int *err_word,
                                        void *stream) {
  if (n_rays < 0 || n_coarse < 2 || n_fine < 1) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8)
    return NERFGB_E_UNSUPPORTED;
  if ((long long)n_rays * (n_coarse + n_fine) > 0x7fffffffLL) return NERFGB_E_INVALID_ARG;
  if (n_rays == 0) return NERFGB_OK;
  if (!proposal_params || !packed_coarse || !packed_fine || !rays_o || !rays_d || !near || !far || !rgb_fine ||
      !depth_fine || !acc_fine || !workspace || !aligned(workspace, 256))
    return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && !err_word) return NERFGB_E_INVALID_ARG;
  cudaStream_t st = as_stream(stream);
  const int R = n_rays, Sc = n_coarse, Sf = n_fine, S = Sc + Sf;
  if (trans_mode != NERFGB_TRANS_CUMPROD && trans_mode != NERFGB_TRANS_LOGSUM) return NERFGB_E_UNSUPPORTED;
  if (gate_flags & ~NERFGB_GATE_FINE_DRAWS) return NERFGB_E_INVALID_ARG;
  RenderWs w = carve(workspace, R, Sc, Sf);
  GateWs g = carve_gate(workspace, R, Sc, Sf);
  int rc;
  // Uniforms: the counters of nerfgb_render_rays (drawn in the samplers), so
  // equal seeds give equal draws.
  if (cudaMemsetAsync(g.counts, 0, 2 * sizeof(int), st) != cudaSuccess) return NERFGB_E_CUDA;
  // Proposal weights over the coarse bins and the coarse gate in one pass:
  // the off samples' sigma is zeroed (the row-mapped MLP writes the others).
  CompositeGate cg;
  cg.tau = gate_tau;
  cg.mask = g.mask_c;
  cg.row_map = g.map_c;
  cg.count = g.counts;
  cg.sig_zero = w.sig_c;
  if (precision == NERFGB_PREC_FP32) {
    if ((rc = launch_coarse_sample(rays_o, rays_d, near, far, u_coarse, seed, R, Sc, perturb, lin_inv_depth,
                                   w.xyz_c, nullptr, w.t_c, w.edges, w.widths, st)) != NERFGB_OK)
      return rc;
    if ((rc = launch_proposal(precision, proposal_params, w.xyz_c, (long long)R * Sc, g.sig_p, st)) != NERFGB_OK)
      return rc;
    if ((rc = launch_composite(nullptr, g.sig_p, w.t_c, R, Sc, 0, trans_mode, -1.0f, nullptr, nullptr, nullptr,
                               nullptr, st, cg)) != NERFGB_OK)
      return rc;
  } else if ((rc = launch_prop_front(proposal_params, rays_o, rays_d, near, far, u_coarse, seed, R, Sc, perturb,
                                     lin_inv_depth, trans_mode, w.xyz_c, w.t_c, w.edges, w.widths, nullptr, cg,
                                     st)) != NERFGB_OK) {
    // BF16/FP8: samples, proposal density, weights and gate in one kernel
    return rc;
  }
  RowMap rm_c;
  rm_c.map = g.map_c;
  rm_c.n_dev = g.counts;
  if ((rc = launch_mlp(packed_coarse, precision, w.xyz_c, rays_d, (long long)R * Sc, Sc, w.rgb_c, w.sig_c,
                       err_word, st, rm_c)) != NERFGB_OK)
    return rc;
  // The fine sampler composites the coarse weights as the plain chain does
  // (last interval 1e10), samples, sorts and gates the sorted union.
  FineFuse fz;
  fz.sigma_c = w.sig_c;
  fz.mode = trans_mode;
  fz.white_bg = white_bg;
  fz.mask_c = g.mask_c;
  fz.row_map = g.map_f;
  fz.count = g.counts + 1;
  fz.sig_zero = w.sig_f;
  fz.rgb_zero = w.rgb_f;
  fz.gate_draws = (gate_flags & NERFGB_GATE_FINE_DRAWS) ? 1 : 0;
  fz.seed = seed;
  if ((rc = launch_fine_sample(rays_o, rays_d, nullptr, w.edges, Sc + 1, w.widths, w.t_c, u_fine, R, Sc, Sf, w.xyz_f,
                               nullptr, w.t_f, nullptr, nullptr, st, fz)) != NERFGB_OK)
    return rc;
  RowMap rm_f;
  rm_f.map = g.map_f;
  rm_f.n_dev = g.counts + 1;
  if ((rc = launch_mlp(packed_fine, precision, w.xyz_f, rays_d, (long long)R * S, S, w.rgb_f, w.sig_f, err_word,
                       st, rm_f)) != NERFGB_OK)
    return rc;
  return nerfgb_composite(w.rgb_f, w.sig_f, w.t_f, R, S, white_bg, trans_mode, nullptr, rgb_fine, depth_fine,
                          acc_fine, stream);
}
