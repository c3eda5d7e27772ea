// Per-ray device functions shared by the render path's kernels (ray_ops.cu,
// proposal.cu): the stratified sample of one bin, one ray's compositing by a
// warp, and the gate's compaction of one ray's samples into a row map.
#pragma once

#include "common.cuh"

namespace nerfgb {

// Point i of tf.linspace(a, b, num): a at 0, b at num-1, else a + delta*i with
// delta = (b - a) / (num - 1), each step rounded (TF's linspace_nd).
__device__ __forceinline__ float linspace_at(float a, float b, int num, int i) {
  if (i == 0) return a;
  if (i == num - 1) return b;
  float delta = fdiv(fsub(b, a), (float)(num - 1));
  return fadd(a, fmul(delta, (float)i));
}

// Bin edge i of S bins (ray_utils.py:183-203).
__device__ __forceinline__ float bin_edge(float nr, float fr, int S, int i, int lin_inv) {
  if (!lin_inv) return linspace_at(nr, fr, S + 1, i);
  return fdiv(1.0f, linspace_at(fdiv(1.0f, nr), fdiv(1.0f, fr), S + 1, i));
}

// Sample i of ray r's S stratified bins (ray_utils.py:183-253): the bin's
// edges e0, e1, width, depth t (jittered by u when perturb) and the point
// o + t d. gid = r * S + i is also the sample's Philox counter when u is
// NULL.
struct BinSample {
  float e0, e1, w, t, x[3];
};
__device__ __forceinline__ BinSample coarse_bin_sample(const float *__restrict__ rays_o,
                                                       const float *__restrict__ rays_d, float nr, float fr,
                                                       const float *__restrict__ u, unsigned long long seed, int r,
                                                       int S, int i, int perturb, int lin_inv) {
  BinSample b;
  const long long gid = (long long)r * S + i;
  b.e0 = bin_edge(nr, fr, S, i, lin_inv);
  b.e1 = bin_edge(nr, fr, S, i + 1, lin_inv);
  b.w = fsub(b.e1, b.e0);                                        // :226
  const float ug = perturb ? (u ? u[gid] : philox_uniform(seed, (unsigned long long)gid)) : 0.0f;
  b.t = perturb ? fadd(b.e0, fmul(ug, b.w))                      // :234
                : fmul(0.5f, fadd(b.e0, b.e1));                  // :243
#pragma unroll
  for (int c = 0; c < 3; ++c) b.x[c] = fadd(rays_o[3 * r + c], fmul(b.t, rays_d[3 * r + c]));  // :251
  return b;
}

struct CSum {
  float s, c;
};
__device__ __forceinline__ CSum two_sum_add(CSum a, CSum b) {
  float s = fadd(a.s, b.s);
  float bp = fsub(s, a.s);
  float e = fadd(fsub(a.s, fsub(s, bp)), fsub(b.s, bp));
  return CSum{s, fadd(fadd(a.c, b.c), e)};
}

// One ray's compositing by one warp from shared copies: s_t, s_sig [S],
// s_rgb [3S] or NULL. Writes the weights to w_out[0..S) (may be NULL) and
// returns (r, g, b, depth, acc) in every lane (white_bg not applied). Lane l
// owns the contiguous segment [l*k, (l+1)*k), k = ceil(S/32).
__device__ __forceinline__ void composite_ray(int lane, const float *s_t, const float *s_sig, const float *s_rgb,
                                              int S, int mode, float last_delta, float *w_out, float (&out)[5]) {
  const int k = (S + 31) >> 5;
  const int j0 = min(lane * k, S), j1 = min(j0 + k, S);
  // Per-sample alpha and transmittance factor.
  float loc_prod = 1.0f;
  CSum loc{0.0f, 0.0f};
  // Last interval: 1e10 as the reference (:462-468), or (last_delta < 0)
  // the previous spacing.
  const float dlast = last_delta >= 0.0f ? last_delta : (S > 1 ? fsub(s_t[S - 1], s_t[S - 2]) : 1e10f);
  for (int j = j0; j < j1; ++j) {
    float delta = (j < S - 1) ? fsub(s_t[j + 1], s_t[j]) : dlast;   // :462-468
    float alpha = fsub(1.0f, expf(fmul(-s_sig[j], delta)));         // :423
    float fac = fadd(fsub(1.0f, alpha), 1e-10f);                    // :480
    if (mode == NERFGB_TRANS_CUMPROD) {
      loc_prod = fmul(loc_prod, fac);
    } else {
      loc = two_sum_add(loc, CSum{logf(fac), 0.0f});
    }
  }
  // Exclusive scan across lanes.
  float ex_prod = 1.0f;
  CSum ex{0.0f, 0.0f};
  if (mode == NERFGB_TRANS_CUMPROD) {
    float inc = loc_prod;
    for (int off = 1; off < 32; off <<= 1) {
      float o = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc = fmul(o, inc);
    }
    ex_prod = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) ex_prod = 1.0f;
  } else {
    CSum inc = loc;
    for (int off = 1; off < 32; off <<= 1) {
      float os = __shfl_up_sync(0xffffffffu, inc.s, off);
      float oc = __shfl_up_sync(0xffffffffu, inc.c, off);
      if (lane >= off) inc = two_sum_add(CSum{os, oc}, inc);
    }
    ex.s = __shfl_up_sync(0xffffffffu, inc.s, 1);
    ex.c = __shfl_up_sync(0xffffffffu, inc.c, 1);
    if (lane == 0) ex = CSum{0.0f, 0.0f};
  }
  // Weights and partial sums.
  float pr = 0.f, pg = 0.f, pb = 0.f, pd = 0.f, pa = 0.f;
  float run_prod = ex_prod;
  CSum run = ex;
  for (int j = j0; j < j1; ++j) {
    float delta = (j < S - 1) ? fsub(s_t[j + 1], s_t[j]) : dlast;
    float alpha = fsub(1.0f, expf(fmul(-s_sig[j], delta)));
    float fac = fadd(fsub(1.0f, alpha), 1e-10f);
    float T;
    if (mode == NERFGB_TRANS_CUMPROD) {
      T = run_prod;
      run_prod = fmul(run_prod, fac);
    } else {
      T = expf(fadd(run.s, run.c));
      run = two_sum_add(run, CSum{logf(fac), 0.0f});
    }
    float w = fmul(alpha, T);                                       // :480
    if (w_out) w_out[j] = w;
    if (s_rgb) {
      const float *c = s_rgb + 3 * j;
      pr = fadd(pr, fmul(w, c[0]));                                 // :534
      pg = fadd(pg, fmul(w, c[1]));
      pb = fadd(pb, fmul(w, c[2]));
    }
    pd = fadd(pd, fmul(s_t[j], w));                                 // :537
    pa = fadd(pa, w);                                               // :540
  }
  for (int off = 16; off > 0; off >>= 1) {
    pr = fadd(pr, __shfl_xor_sync(0xffffffffu, pr, off));
    pg = fadd(pg, __shfl_xor_sync(0xffffffffu, pg, off));
    pb = fadd(pb, __shfl_xor_sync(0xffffffffu, pb, off));
    pd = fadd(pd, __shfl_xor_sync(0xffffffffu, pd, off));
    pa = fadd(pa, __shfl_xor_sync(0xffffffffu, pa, off));
  }
  out[0] = pr;
  out[1] = pg;
  out[2] = pb;
  out[3] = pd;
  out[4] = pa;
}

// The maps of lane 0's sums: rgb (+ 1 - acc with white_bg, :542-544), depth, acc.
__device__ __forceinline__ void store_maps(int r, int white_bg, const float (&m)[5], float *pred_rgb,
                                           float *pred_depth, float *acc_map) {
  float pr = m[0], pg = m[1], pb = m[2];
  if (white_bg) {
    float bg = fsub(1.0f, m[4]);
    pr = fadd(pr, bg);
    pg = fadd(pg, bg);
    pb = fadd(pb, bg);
  }
  pred_rgb[3 * r + 0] = pr;
  pred_rgb[3 * r + 1] = pg;
  pred_rgb[3 * r + 2] = pb;
  pred_depth[r] = m[3];
  acc_map[r] = m[4];
}

// Appends the ray's on samples (in order) to row_map at a slot taken by one
// atomic on *count, writes mask (0/1) when given, and zeroes sig_zero (and
// rgb_zero, 3 values) at the off samples, which the row-mapped MLP leaves
// untouched. on(j) is the warp's predicate for sample j of the ray.
template <typename On>
__device__ __forceinline__ void gate_ray(int lane, long long row0, int S, int R, On on, unsigned char *mask,
                                         int *row_map, int *count, float *sig_zero, float *rgb_zero, int site) {
  int total = 0;
  for (int j0 = 0; j0 < S; j0 += 32) total += __popc(__ballot_sync(0xffffffffu, j0 + lane < S && on(j0 + lane)));
  int base = 0;
  if (lane == 0 && total > 0) base = atomicAdd(count, total);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int j0 = 0; j0 < S; j0 += 32) {
    const int j = j0 + lane;
    const bool o = j < S && on(j);
    const unsigned b = __ballot_sync(0xffffffffu, o);
    if (j < S) {
      if (mask) mask[row0 + j] = o ? 1 : 0;
      if (!o) {
        if (sig_zero) sig_zero[row0 + j] = 0.0f;
        if (rgb_zero) {
          rgb_zero[3 * (row0 + j)] = 0.0f;
          rgb_zero[3 * (row0 + j) + 1] = 0.0f;
          rgb_zero[3 * (row0 + j) + 2] = 0.0f;
        }
      }
    }
    if (o) row_map[NG_IDX(base + __popc(b & ((1u << lane) - 1u)), (long long)R * S, site)] = (int)(row0 + j);
    base += __popc(b);
  }
}

}  // namespace nerfgb
