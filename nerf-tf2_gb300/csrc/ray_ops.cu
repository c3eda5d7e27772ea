// Ray operators of the render path: stratified coarse sampler, positional
// encoder, compositor and inverse-transform fine sampler.
//
// Layout in HBM: rays [R,3]/[R,1] float32; per-sample tensors [R,S] or
// [R*S,3] row-major, the layouts the reference's TensorFlow tensors have.
#include <math.h>

#include "common.cuh"
#include "mlp_internal.cuh"
#include "ray_device.cuh"

namespace nerfgb {

// ---------------------------------------------------------------------------
// Stratified coarse sampler (ray_utils.py:137-274). One thread per (ray, bin).
// ---------------------------------------------------------------------------

// u NULL with perturb: the uniform of (ray r, bin i) is element r*S + i of
// the Philox stream keyed by seed (nerfgb_uniform's element), drawn here.
__global__ void coarse_sample_kernel(const float *__restrict__ rays_o, const float *__restrict__ rays_d,
                                     const float *__restrict__ near, const float *__restrict__ far,
                                     const float *__restrict__ u, unsigned long long seed, int R, int S,
                                     int perturb, int lin_inv, float *__restrict__ xyz, float *__restrict__ dirs,
                                     float *__restrict__ t_out, float *__restrict__ edges,
                                     float *__restrict__ widths) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long long)R * S) return;
  int r = (int)(gid / S), i = (int)(gid - (long long)r * S);
  const BinSample b = coarse_bin_sample(rays_o, rays_d, near[r], far[r], u, seed, r, S, i, perturb, lin_inv);
  t_out[gid] = b.t;
  widths[gid] = b.w;
  edges[(long long)r * (S + 1) + i] = b.e0;
  if (i == S - 1) edges[(long long)r * (S + 1) + S] = b.e1;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    xyz[3 * gid + c] = b.x[c];
    if (dirs) dirs[3 * gid + c] = rays_d[3 * r + c];              // :253
  }
}

// ---------------------------------------------------------------------------
// Positional encoder (model.py:319-331): out[n, 3+6L] =
// [x, sin(x_c m_l), cos(x_c m_l)] at index 3 + c*2L + 2l + {0,1}.
// ---------------------------------------------------------------------------
__global__ void encode_kernel(const float *__restrict__ x, long long n, int L, float *__restrict__ out) {
  long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per = 3 + 3 * L;  // 3 copies + 3L (c,l) pairs
  if (gid >= n * per) return;
  long long row = gid / per;
  int j = (int)(gid - row * per);
  int D = 3 + 6 * L;
  if (j < 3) {
    out[row * D + j] = x[row * 3 + j];
    return;
  }
  j -= 3;
  int c = j / L, l = j - c * L;
  float arg = fmul(x[row * 3 + c], enc_multiplier(l));
  float s, co;
  sincosf(arg, &s, &co);
  out[row * D + 3 + c * 2 * L + 2 * l] = s;
  out[row * D + 3 + c * 2 * L + 2 * l + 1] = co;
}

// ---------------------------------------------------------------------------
// Compositor (ray_utils.py:408-551). One warp per ray. Lane l owns the
// contiguous segment [l*k, (l+1)*k) of the S samples, k = ceil(S/32).
// Transmittance T_i = prod_{j<i} ((1 - alpha_j) + 1e-10) (:480), either as a
// product or as exp of a compensated log-sum (Neumaier per lane, TwoSum
// across lanes).
// ---------------------------------------------------------------------------
constexpr int kCompWarps = 4;

// Compositor (ray_utils.py:408-551), one warp per ray: t, sigma and rgb are
// staged in shared memory with coalesced loads, the weights written back
// from there. With gate_map != NULL the weights also gate the samples
// (sample j on where w > tau, NaN off; gate_ray).
__global__ void __launch_bounds__(32 * kCompWarps)
    composite_kernel(const float *__restrict__ rgb, const float *__restrict__ sigma,
                     const float *__restrict__ t, int R, int S, int white_bg, int mode, float last_delta,
                     float *__restrict__ weights, float *__restrict__ pred_rgb,
                     float *__restrict__ pred_depth, float *__restrict__ acc_map, float tau,
                     unsigned char *__restrict__ gate_mask, int *__restrict__ gate_map, int *__restrict__ gate_count,
                     float *__restrict__ gate_sig_zero) {
  extern __shared__ float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *s_t = smem + warp * (6 * S + 1);
  float *s_sig = s_t + (S + 1);
  float *s_w = s_sig + S;
  float *s_rgb = s_w + S;  // 3S
  for (int r = blockIdx.x * kCompWarps + warp; r < R; r += gridDim.x * kCompWarps) {
    const long long base = (long long)r * S;
    for (int j = lane; j < S; j += 32) {
      s_t[j] = t[base + j];
      s_sig[j] = sigma[base + j];
    }
    if (rgb)
      for (int j = lane; j < 3 * S; j += 32) s_rgb[j] = rgb[3 * base + j];
    __syncwarp();
    float m[5];
    composite_ray(lane, s_t, s_sig, rgb ? s_rgb : nullptr, S, mode, last_delta, s_w, m);
    __syncwarp();
    if (weights)
      for (int j = lane; j < S; j += 32) weights[base + j] = s_w[j];
    if (lane == 0 && pred_rgb) store_maps(r, white_bg, m, pred_rgb, pred_depth, acc_map);
    if (gate_map)
      gate_ray(lane, base, S, R, [&](int j) { return s_w[j] > tau; }, gate_mask, gate_map, gate_count,
               gate_sig_zero, nullptr, kSiteGateCoarse);
    __syncwarp();
  }
}

__global__ void sigma_to_alpha_kernel(const float *__restrict__ sigma, const float *__restrict__ diffs,
                                      long long n, float *__restrict__ alpha) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) alpha[i] = fsub(1.0f, expf(fmul(-sigma[i], diffs[i])));
}

// ---------------------------------------------------------------------------
// Inverse-transform fine sampler (ray_utils.py:276-406). One warp per ray.
// The two reductions that feed the CDF (denominator :338, cumsum :342) run
// left to right in one lane, in fp32 without FMA, so the CDF, the
// searchsorted indices and the sorted t are bit-identical to the sequential
// restatement.
// ---------------------------------------------------------------------------
constexpr int kFineWarps = 4;

// Strict weak order of numpy's stable sort: NaN after every number, ties by
// original index.
__device__ __forceinline__ bool sort_before(float a, int ia, float b, int ib) {
  bool na = isnan(a), nb = isnan(b);
  if (na || nb) return (!na && nb) || (na && nb && ia < ib);
  return a < b || (a == b && ia < ib);
}

// Bitonic sort of P = 32 E (key, index) pairs held E per lane (element i =
// lane E + e), ascending by key, ties by index (keys not NaN): the
// compare-exchange of elements i and i ^ j runs in registers for j < E and
// through shuffles (lane ^ j / E) otherwise. Both sides of a pair compute
// the same min and max, each keeping its own.
__device__ __forceinline__ bool key_before(float a, int ia, float b, int ib) { return a < b || (a == b && ia < ib); }
template <int E>
__device__ __forceinline__ void warp_bitonic_sort(float (&key)[E], int (&idx)[E], int lane) {
  constexpr int P = 32 * E;
#pragma unroll
  for (int k = 2; k <= P; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= E) {
        const int m = j / E;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int i = lane * E + e;
          const float pk = __shfl_xor_sync(0xffffffffu, key[e], m);
          const int pi = __shfl_xor_sync(0xffffffffu, idx[e], m);
          const bool take_min = ((i & j) == 0) == ((i & k) == 0);
          const bool other_first = key_before(pk, pi, key[e], idx[e]);
          if (other_first == take_min) {
            key[e] = pk;
            idx[e] = pi;
          }
        }
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
          if (e & j) continue;  // e is the pair's lower element, e + j the upper
          const int i = lane * E + e;
          const bool asc = (i & k) == 0;
          if (key_before(key[e + j], idx[e + j], key[e], idx[e]) == asc) {
            const float tk = key[e];
            const int ti = idx[e];
            key[e] = key[e + j];
            idx[e] = idx[e + j];
            key[e + j] = tk;
            idx[e + j] = ti;
          }
        }
      }
    }
  }
}

// The fine draws (s_t[Sc .. Sc + Sf)) padded to P = 32 E with (+inf, index
// >= Sf), sorted by warp_bitonic_sort into s_fk (keys) and s_fi (indices).
template <int E>
__device__ __forceinline__ void sort_fine_draws(const float *s_t, int Sc, int Sf, float *s_fk, int *s_fi, int lane) {
  float key[E];
  int idx[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int i = lane * E + e;
    key[e] = i < Sf ? s_t[Sc + i] : INFINITY;
    idx[e] = i;
  }
  warp_bitonic_sort<E>(key, idx, lane);
#pragma unroll
  for (int e = 0; e < E; ++e) {
    s_fk[lane * E + e] = key[e];
    s_fi[lane * E + e] = idx[e];
  }
}

// Shared-memory words per warp of fine_sample_kernel: w, pdf, left edges,
// widths (4 Sc), the CDF (Sc + 1), concat and sorted t (2 S), the bitonic
// keys and indices (2 P), the permutation (S), rgb_c (3 Sc), the draws'
// bins (Sf).
__host__ __device__ __forceinline__ int fine_smem_floats(int Sc, int Sf, int P) {
  const int S = Sc + Sf;
  return 4 * Sc + (Sc + 1) + 2 * S + 2 * P + S + 3 * Sc + Sf;
}

__global__ void __launch_bounds__(32 * kFineWarps, 8)
    fine_sample_kernel(const float *__restrict__ rays_o, const float *__restrict__ rays_d,
                       const float *__restrict__ bin_weights, const float *__restrict__ left_edges,
                       int ld_left, const float *__restrict__ bin_widths,
                       const float *__restrict__ t_coarse, const float *__restrict__ u, int R, int Sc,
                       int Sf, float *__restrict__ xyz, float *__restrict__ dirs,
                       float *__restrict__ t_out, int *__restrict__ piece_idxs,
                       int *__restrict__ sort_perm, int P, FineFuse fz) {
  extern __shared__ float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = Sc + Sf;
  const int per_warp = fine_smem_floats(Sc, Sf, P);
  float *s_w = smem + warp * per_warp;  // w + 1e-5, then pdf * width
  float *s_pdf = s_w + Sc;
  float *s_left = s_pdf + Sc;
  float *s_wid = s_left + Sc;
  float *s_agg = s_wid + Sc;      // Sc + 1
  float *s_t = s_agg + Sc + 1;    // concat(t_c, t_f), S
  float *s_srt = s_t + S;         // sorted, S (first holds sigma_c for the fused compositing)
  float *s_fk = s_srt + S;        // fast path: fine keys (P, a power of two >= Sf) ...
  int *s_fi = reinterpret_cast<int *>(s_fk + P);  // ... and their fine indices
  int *s_perm = s_fi + P;         // the sort permutation, S
  float *s_rgbc = reinterpret_cast<float *>(s_perm + S);  // rgb_c of the ray, 3 Sc
  int *s_pc = reinterpret_cast<int *>(s_rgbc + 3 * Sc);   // each fine draw's coarse bin, Sf
  for (int r = blockIdx.x * kFineWarps + warp; r < R; r += gridDim.x * kFineWarps) {
    const long long rb = (long long)r * Sc;
    if (fz.sigma_c) {
      // the coarse pass's compositing (ray_utils.py:426-482) of this ray
      for (int j = lane; j < Sc; j += 32) {
        s_wid[j] = bin_widths[rb + j];
        s_left[j] = left_edges[(long long)r * ld_left + j];
        s_t[j] = t_coarse[rb + j];
        s_srt[j] = fz.sigma_c[rb + j];
      }
      const bool maps = fz.rgb_c && fz.map_rgb;
      if (maps)
        for (int j = lane; j < 3 * Sc; j += 32) s_rgbc[j] = fz.rgb_c[3 * rb + j];
      __syncwarp();
      float m[5];
      composite_ray(lane, s_t, s_srt, maps ? s_rgbc : nullptr, Sc, fz.mode, 1e10f, s_w, m);
      __syncwarp();
      if (lane == 0 && maps) store_maps(r, fz.white_bg, m, fz.map_rgb, fz.map_depth, fz.map_acc);
      for (int j = lane; j < Sc; j += 32) {
        if (fz.w_c) fz.w_c[rb + j] = s_w[j];
        float w = fadd(s_w[j], 1e-5f);                                // :335
        s_w[j] = w;
        s_pdf[j] = fmul(w, s_wid[j]);
      }
    } else {
      for (int j = lane; j < Sc; j += 32) {
        float w = fadd(bin_weights[rb + j], 1e-5f);                   // :335
        float wd = bin_widths[rb + j];
        s_w[j] = w;
        s_pdf[j] = fmul(w, wd);
        s_wid[j] = wd;
        s_left[j] = left_edges[(long long)r * ld_left + j];
        s_t[j] = t_coarse[rb + j];
      }
    }
    __syncwarp();
    float denom = 0.0f;
    if (lane == 0)
      for (int j = 0; j < Sc; ++j) denom = fadd(denom, s_pdf[j]);     // :338
    denom = __shfl_sync(0xffffffffu, denom, 0);
    __syncwarp();
    for (int j = lane; j < Sc; j += 32) {
      float p = fdiv(s_w[j], denom);                                  // :339
      s_pdf[j] = p;
      s_w[j] = fmul(p, s_wid[j]);
    }
    __syncwarp();
    if (lane == 0) {                                                  // :342-345
      float acc = 0.0f;
      s_agg[0] = 0.0f;
      for (int j = 0; j < Sc; ++j) {
        acc = fadd(acc, s_w[j]);
        s_agg[j + 1] = acc;
      }
    }
    __syncwarp();
    const long long ub = (long long)r * Sf;
    for (int k = lane; k < Sf; k += 32) {
      // u NULL: element R*Sc + r*Sf + k of the Philox stream (after the coarse draws)
      float uk = u ? u[ub + k] : philox_uniform(fz.seed, (unsigned long long)R * Sc + ub + k);
      // upper_bound over the inner edges agg[1..Sc-1] (:363).
      int first = 0, count = Sc - 1;
      while (count > 0) {
        int step = count >> 1, it = first + step;
        if (!(uk < s_agg[1 + it])) {
          first = it + 1;
          count -= step + 1;
        } else {
          count = step;
        }
      }
      first = (int)NG_IDX(first, Sc, kSiteFinePiece);
      float a_ = s_agg[first], p_ = s_pdf[first], l_ = s_left[first];  // :366-368
      float mask = (p_ < 1e-8f) ? 0.0f : 1.0f;                          // :372
      p_ = fmaxf(p_, 1e-8f);                                            // :373
      s_t[Sc + k] = fadd(fmul(fdiv(fsub(uk, a_), p_), mask), l_);       // :376
      if (piece_idxs) piece_idxs[ub + k] = first;
      s_pc[k] = first;
    }
    __syncwarp();
    // Stable sort of concat(t_c, t_f) (:380-385).
    const long long sb = (long long)r * S;
    bool fast = false;
    if (P > 0) {
      // t_c non-decreasing and no NaN anywhere: the stable order is t_c in
      // place merged with the sorted fine draws, a t_c element first on a tie.
      bool ok = true;
      for (int j = lane; j < Sc; j += 32) ok = ok && !isnan(s_t[j]) && (j + 1 >= Sc || s_t[j] <= s_t[j + 1]);
      for (int k = lane; k < Sf; k += 32) ok = ok && !isnan(s_t[Sc + k]);
      fast = __all_sync(0xffffffffu, ok);
    }
    if (fast) {
      // Bitonic sort of (t_f[k], k), padded to P with (+inf, k >= Sf): in
      // registers and shuffles up to P = 128, through shared memory above
      // (the same network; more keys per lane would cost the kernel's
      // occupancy in registers).
      if (P == 32) {
        sort_fine_draws<1>(s_t, Sc, Sf, s_fk, s_fi, lane);
      } else if (P == 64) {
        sort_fine_draws<2>(s_t, Sc, Sf, s_fk, s_fi, lane);
      } else if (P == 128) {
        sort_fine_draws<4>(s_t, Sc, Sf, s_fk, s_fi, lane);
      } else {
        for (int k = lane; k < P; k += 32) {
          s_fk[k] = k < Sf ? s_t[Sc + k] : INFINITY;
          s_fi[k] = k;
        }
        __syncwarp();
        for (int size = 2; size <= P; size <<= 1) {
          for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int q = lane; q < P / 2; q += 32) {
              const int lo = 2 * stride * (q / stride) + (q % stride), hi = lo + stride;
              const float a = s_fk[lo], b = s_fk[hi];
              const int ia = s_fi[lo], ib = s_fi[hi];
              // ascending block: b first -> swap; descending: a first -> swap
              if (key_before(b, ib, a, ia) == ((lo & size) == 0)) {
                s_fk[lo] = b;
                s_fk[hi] = a;
                s_fi[lo] = ib;
                s_fi[hi] = ia;
              }
            }
            __syncwarp();
          }
        }
      }
      __syncwarp();
      // t_c[i] lands after the fine draws strictly below it; the j-th
      // sorted draw after the coarse samples at or below it.
      for (int i = lane; i < Sc; i += 32) {
        const float v = s_t[i];
        int first = 0, count = Sf;  // lower_bound over s_fk[0, Sf)
        while (count > 0) {
          const int step = count >> 1, it = first + step;
          if (s_fk[it] < v) {
            first = it + 1;
            count -= step + 1;
          } else {
            count = step;
          }
        }
        const int pos = (int)NG_IDX(i + first, S, kSiteSortCoarse);
        s_srt[pos] = v;
        s_perm[pos] = i;
      }
      for (int j = lane; j < Sf; j += 32) {
        const float v = s_fk[j];
        int first = 0, count = Sc;  // upper_bound over t_c
        while (count > 0) {
          const int step = count >> 1, it = first + step;
          if (!(v < s_t[it])) {
            first = it + 1;
            count -= step + 1;
          } else {
            count = step;
          }
        }
        const int pos = (int)NG_IDX(j + first, S, kSiteSortFine);
        s_srt[pos] = v;
        s_perm[pos] = Sc + s_fi[j];
      }
    } else {
      // Rank sort: rank = number of elements that precede e in the stable order.
      for (int e = lane; e < S; e += 32) {
        float v = s_t[e];
        int rank = 0;
        for (int q = 0; q < S; ++q) rank += sort_before(s_t[q], q, v, e) ? 1 : 0;
        rank = (int)NG_IDX(rank, S, kSiteSortRank);
        s_srt[rank] = v;
        s_perm[rank] = e;
      }
    }
    __syncwarp();
    float o0 = rays_o[3 * r], o1 = rays_o[3 * r + 1], o2 = rays_o[3 * r + 2];
    float d0 = rays_d[3 * r], d1 = rays_d[3 * r + 1], d2 = rays_d[3 * r + 2];
    if (sort_perm)
      for (int p = lane; p < S; p += 32) sort_perm[sb + p] = s_perm[p];
    if (fz.row_map) {
      // the fine gate (the gated render): a coarse sample whose gate is on,
      // or a fine draw (with gate_draws: one whose coarse bin's gate is on)
      const unsigned char *mc = fz.mask_c + rb;
      const bool draws = fz.gate_draws != 0;
      gate_ray(lane, sb, S, R,
               [&](int j) {
                 const int q = (int)NG_IDX(s_perm[j], S, kSiteGateFinePerm);
                 return q >= Sc ? (!draws || mc[s_pc[q - Sc]] != 0) : mc[q] != 0;
               },
               nullptr, fz.row_map, fz.count, fz.sig_zero, fz.rgb_zero, kSiteGateFine);
    }
    for (int p = lane; p < S; p += 32) {
      float tv = s_srt[p];
      t_out[sb + p] = tv;
      float *x = xyz + 3 * (sb + p);                                  // :389
      x[0] = fadd(o0, fmul(tv, d0));
      x[1] = fadd(o1, fmul(tv, d1));
      x[2] = fadd(o2, fmul(tv, d2));
      if (dirs) {
        float *dd = dirs + 3 * (sb + p);
        dd[0] = d0;
        dd[1] = d1;
        dd[2] = d2;
      }
    }
    __syncwarp();
  }
}

// get_rays_tf (ray_utils.py:53-106) for pixel (u, v): x = (u - cx) / fx,
// y = (v - cy) / fy, z = 1; d = R (x, y, z) as a sequential three-term sum
// per component (TF leaves the matmul's order open); d /= sqrt(d.d) + 1e-8
// with d.d summed in order; o = c2w[:3, 3]. Plain IEEE float32 operations
// without contraction, as the oracle does.
__device__ __forceinline__ void pixel_ray(float u, float v, const float *__restrict__ K,
                                          const float *__restrict__ c2w, float (&o)[3], float (&d)[3]) {
  const float x = fdiv(fsub(u, K[2]), K[0]);
  const float y = fdiv(fsub(v, K[5]), K[4]);
#pragma unroll
  for (int i = 0; i < 3; ++i) d[i] = fadd(fadd(fmul(x, c2w[4 * i]), fmul(y, c2w[4 * i + 1])), c2w[4 * i + 2]);
  const float m = fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2]));
  const float den = fadd(__fsqrt_rn(m), 1e-8f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    d[i] = fdiv(d[i], den);
    o[i] = c2w[4 * i + 3];
  }
}

// One thread per pixel p = v * W + u.
__global__ void get_rays_kernel(int H, int W, const float *__restrict__ K, const float *__restrict__ c2w,
                                float *__restrict__ rays_o, float *__restrict__ rays_d) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (long long)H * W) return;
  float o[3], d[3];
  pixel_ray((float)(p % W), (float)(p / W), K, c2w, o, d);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    rays_d[3 * p + i] = d[i];
    rays_o[3 * p + i] = o[i];
  }
}

// Sample-mode batch (base_dataset.py:555-621): ray idxs[b] of the image's
// get_rays_tf rays with near/far = bounds and rgb = image / 255 (uint8 HWC).
// Indices outside [0, H*W) give a zero ray, zero rgb and bounds.
__global__ void sample_rays_kernel(const unsigned char *__restrict__ img, int H, int W,
                                   const float *__restrict__ K, const float *__restrict__ c2w, float near,
                                   float far, const int *__restrict__ idxs, int B, float *__restrict__ rays_o,
                                   float *__restrict__ rays_d, float *__restrict__ near_out,
                                   float *__restrict__ far_out, float *__restrict__ rgb) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const long long p = idxs[b];
  float o[3] = {0.f, 0.f, 0.f}, d[3] = {0.f, 0.f, 0.f}, c[3] = {0.f, 0.f, 0.f};
  const bool in = p >= 0 && p < (long long)H * W;
  if (in) {
    pixel_ray((float)(p % W), (float)(p / W), K, c2w, o, d);
#pragma unroll
    for (int i = 0; i < 3; ++i) c[i] = fdiv((float)img[3 * p + i], 255.0f);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    rays_o[3 * b + i] = o[i];
    rays_d[3 * b + i] = d[i];
    rgb[3 * b + i] = c[i];
  }
  near_out[b] = in ? near : 0.0f;
  far_out[b] = in ? far : 0.0f;
}

// Uniform integers in [0, maxval): (word * maxval) >> 32 of the Philox
// stream's words offset .. offset + n - 1.
__global__ void uniform_int_kernel(unsigned long long seed, unsigned long long offset, long long n, int maxval,
                                   int *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int)(((unsigned long long)philox_word(seed, offset + (unsigned long long)i) * (unsigned)maxval) >> 32);
}

// create_depth_map (ray_utils.py:108-135): type 1 = depth * (1 / scale);
// type 2 = the camera-frame z of o + d * depth * (1 / scale) under w2c.
__global__ void depth_map_kernel(const float *__restrict__ depth, long long n, float inv_scale, int type,
                                 const float *__restrict__ rays_o, const float *__restrict__ rays_d,
                                 const float *__restrict__ w2c, float *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ds = fmul(depth[i], inv_scale);
  if (type == 1) {
    out[i] = ds;
    return;
  }
  float z = w2c[11];
#pragma unroll
  for (int k = 0; k < 3; ++k) z = fadd(z, fmul(w2c[8 + k], fadd(rays_o[3 * i + k], fmul(rays_d[3 * i + k], ds))));
  out[i] = z;
}

__global__ void uniform_kernel(unsigned long long seed, unsigned long long offset, long long n,
                               float *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = philox_uniform(seed, offset + (unsigned long long)i);
}

static int grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (int)(g > 0x7fffffffLL ? 0x7fffffff : g);
}

}  // namespace nerfgb

using namespace nerfgb;

extern "C" int nerfgb_abi_version(void) { return NERFGB_ABI_VERSION; }

extern "C" const char *nerfgb_status_string(int s) {
  switch (s) {
    case NERFGB_OK: return "NERFGB_OK";
    case NERFGB_E_INVALID_ARG: return "NERFGB_E_INVALID_ARG";
    case NERFGB_E_UNSUPPORTED: return "NERFGB_E_UNSUPPORTED";
    case NERFGB_E_CUDA: return "NERFGB_E_CUDA";
    case NERFGB_E_TIMEOUT: return "NERFGB_E_TIMEOUT";
    case NERFGB_E_DEVICE: return "NERFGB_E_DEVICE";
    case NERFGB_E_SCRATCH_LIMIT: return "NERFGB_E_SCRATCH_LIMIT";
    default: return "NERFGB_E_UNKNOWN";
  }
}

namespace nerfgb {
int launch_coarse_sample(const float *rays_o, const float *rays_d, const float *near, const float *far,
                         const float *u_vals, unsigned long long seed, int R, int S, int perturb, int lin_inv,
                         float *xyz, float *dirs, float *t_vals, float *edges, float *widths, cudaStream_t stream) {
  const long long n = (long long)R * S;
  if (n == 0) return NERFGB_OK;
  coarse_sample_kernel<<<grid_for(n, 256), 256, 0, stream>>>(rays_o, rays_d, near, far, u_vals, seed, R, S,
                                                             perturb, lin_inv, xyz, dirs, t_vals, edges, widths);
  return launch_status();
}
}  // namespace nerfgb

extern "C" int nerfgb_coarse_sample(const float *rays_o, const float *rays_d, const float *near,
                                    const float *far, const float *u_vals, int n_rays, int n_coarse,
                                    int perturb, int lin_inv_depth, float *xyz, float *dirs,
                                    float *t_vals, float *bin_edges, float *bin_widths, void *stream) {
  if (n_rays < 0 || n_coarse < 1) return NERFGB_E_INVALID_ARG;
  if (n_coarse > 1024) return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!rays_o || !rays_d || !near || !far || !xyz || !t_vals || !bin_edges || !bin_widths ||
      (perturb && !u_vals))
    return NERFGB_E_INVALID_ARG;
  return launch_coarse_sample(rays_o, rays_d, near, far, u_vals, 0, n_rays, n_coarse, perturb, lin_inv_depth, xyz,
                              dirs, t_vals, bin_edges, bin_widths, as_stream(stream));
}

extern "C" int nerfgb_positional_encode(const float *x, long long n, int L, float *out, void *stream) {
  if (n < 0 || L < 1) return NERFGB_E_INVALID_ARG;
  if (L > 16) return NERFGB_E_UNSUPPORTED;
  if (n == 0) return NERFGB_OK;
  if (!x || !out) return NERFGB_E_INVALID_ARG;
  long long work = n * (3 + 3 * L);
  encode_kernel<<<grid_for(work, 256), 256, 0, as_stream(stream)>>>(x, n, L, out);
  return launch_status();
}

namespace nerfgb {
int launch_composite(const float *sample_rgb, const float *sigma, const float *t_vals, int n_rays, int n_samples,
                     int white_bg, int trans_mode, float last_delta, float *weights, float *pred_rgb,
                     float *pred_depth, float *acc_map, cudaStream_t stream, const CompositeGate &gate) {
  size_t smem = (size_t)kCompWarps * (6 * n_samples + 1) * sizeof(float);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(composite_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return NERFGB_E_CUDA;
  int sms = num_sms();
  int blocks = (n_rays + kCompWarps - 1) / kCompWarps;
  int cap = (sms > 0 ? sms : 148) * 16;
  composite_kernel<<<blocks < cap ? blocks : cap, 32 * kCompWarps, smem, stream>>>(
      sample_rgb, sigma, t_vals, n_rays, n_samples, white_bg, trans_mode, last_delta, weights, pred_rgb,
      pred_depth, acc_map, gate.tau, gate.mask, gate.row_map, gate.count, gate.sig_zero);
  return launch_status();
}
}  // namespace nerfgb

extern "C" int nerfgb_composite(const float *sample_rgb, const float *sigma, const float *t_vals,
                                int n_rays, int n_samples, int white_bg, int trans_mode,
                                float *weights, float *pred_rgb, float *pred_depth, float *acc_map,
                                void *stream) {
  if (n_rays < 0 || n_samples < 1) return NERFGB_E_INVALID_ARG;
  if (n_samples > 2048) return NERFGB_E_UNSUPPORTED;
  if (trans_mode != NERFGB_TRANS_CUMPROD && trans_mode != NERFGB_TRANS_LOGSUM)
    return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!sample_rgb || !sigma || !t_vals || !pred_rgb || !pred_depth || !acc_map)
    return NERFGB_E_INVALID_ARG;
  return launch_composite(sample_rgb, sigma, t_vals, n_rays, n_samples, white_bg, trans_mode, 1e10f, weights,
                          pred_rgb, pred_depth, acc_map, as_stream(stream));
}

extern "C" int nerfgb_sigma_to_alpha(const float *sigma, const float *diffs, long long n, float *alpha,
                                     void *stream) {
  if (n < 0) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!sigma || !diffs || !alpha) return NERFGB_E_INVALID_ARG;
  sigma_to_alpha_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(sigma, diffs, n, alpha);
  return launch_status();
}

extern "C" int nerfgb_fine_sample(const float *rays_o, const float *rays_d, const float *bin_weights,
                                  const float *left_edges, int ld_left, const float *bin_widths,
                                  const float *t_vals_coarse, const float *u_vals, int n_rays,
                                  int n_coarse, int n_fine, float *xyz, float *dirs, float *t_vals,
                                  int *piece_idxs, int *sort_perm, void *stream) {
  if (n_rays < 0 || n_coarse < 2 || n_fine < 1 || ld_left < n_coarse) return NERFGB_E_INVALID_ARG;
  if (n_coarse > 256 || n_fine > 512) return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!rays_o || !rays_d || !bin_weights || !left_edges || !bin_widths || !t_vals_coarse ||
      !u_vals || !xyz || !t_vals)
    return NERFGB_E_INVALID_ARG;
  return launch_fine_sample(rays_o, rays_d, bin_weights, left_edges, ld_left, bin_widths, t_vals_coarse, u_vals,
                            n_rays, n_coarse, n_fine, xyz, dirs, t_vals, piece_idxs, sort_perm, as_stream(stream),
                            FineFuse());
}

namespace nerfgb {
int launch_fine_sample(const float *rays_o, const float *rays_d, const float *bin_weights, const float *left_edges,
                       int ld_left, const float *bin_widths, const float *t_vals_coarse, const float *u_vals,
                       int n_rays, int n_coarse, int n_fine, float *xyz, float *dirs, float *t_vals,
                       int *piece_idxs, int *sort_perm, cudaStream_t stream, const FineFuse &fz) {
  if (n_rays == 0) return NERFGB_OK;
  int S = n_coarse + n_fine;
  // Fast stable sort for up to 512 fine draws: keys padded to a power of two.
  int P = 0;
  if (n_fine <= 512) {
    P = 32;
    while (P < n_fine) P <<= 1;
  }
  size_t smem = (size_t)kFineWarps * fine_smem_floats(n_coarse, n_fine, P) * sizeof(float);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(fine_sample_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return NERFGB_E_CUDA;
  int sms = num_sms();
  int blocks = (n_rays + kFineWarps - 1) / kFineWarps;
  int cap = (sms > 0 ? sms : 148) * 16;
  fine_sample_kernel<<<blocks < cap ? blocks : cap, 32 * kFineWarps, smem, stream>>>(
      rays_o, rays_d, bin_weights, left_edges, ld_left, bin_widths, t_vals_coarse, u_vals, n_rays, n_coarse,
      n_fine, xyz, dirs, t_vals, piece_idxs, sort_perm, P, fz);
  return launch_status();
}
}  // namespace nerfgb

extern "C" int nerfgb_uniform(unsigned long long seed, unsigned long long offset, long long n, float *out,
                              void *stream) {
  if (n < 0) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!out) return NERFGB_E_INVALID_ARG;
  uniform_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(seed, offset, n, out);
  return launch_status();
}

extern "C" int nerfgb_get_rays(int H, int W, const float *intrinsic, const float *c2w, float *rays_o,
                               float *rays_d, void *stream) {
  if (H < 0 || W < 0) return NERFGB_E_INVALID_ARG;
  const long long n = (long long)H * W;
  if (n == 0) return NERFGB_OK;
  if (!intrinsic || !c2w || !rays_o || !rays_d) return NERFGB_E_INVALID_ARG;
  get_rays_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(H, W, intrinsic, c2w, rays_o, rays_d);
  return launch_status();
}

extern "C" int nerfgb_sample_rays(const unsigned char *image, int H, int W, const float *intrinsic,
                                  const float *c2w, float near, float far, const int *idxs, int batch,
                                  float *rays_o, float *rays_d, float *near_out, float *far_out, float *rgb,
                                  void *stream) {
  if (H < 0 || W < 0 || batch < 0) return NERFGB_E_INVALID_ARG;
  if (batch == 0) return NERFGB_OK;
  if (!image || !intrinsic || !c2w || !idxs || !rays_o || !rays_d || !near_out || !far_out || !rgb)
    return NERFGB_E_INVALID_ARG;
  sample_rays_kernel<<<(batch + 255) / 256, 256, 0, as_stream(stream)>>>(image, H, W, intrinsic, c2w, near, far,
                                                                          idxs, batch, rays_o, rays_d, near_out,
                                                                          far_out, rgb);
  return launch_status();
}

extern "C" int nerfgb_uniform_int(unsigned long long seed, unsigned long long offset, long long n, int maxval,
                                  int *out, void *stream) {
  if (n < 0 || maxval < 1) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!out) return NERFGB_E_INVALID_ARG;
  uniform_int_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(seed, offset, n, maxval, out);
  return launch_status();
}

extern "C" int nerfgb_depth_map(const float *pred_depth, long long n, float scale_factor, int map_type,
                                const float *rays_o, const float *rays_d, const float *w2c, float *out,
                                void *stream) {
  if (n < 0 || (map_type != 1 && map_type != 2) || !(scale_factor != 0.0f)) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!pred_depth || !out || (map_type == 2 && (!rays_o || !rays_d || !w2c))) return NERFGB_E_INVALID_ARG;
  depth_map_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(pred_depth, n, 1.0f / scale_factor, map_type,
                                                                    rays_o, rays_d, w2c, out);
  return launch_status();
}

#ifdef NERF_BOUNDS_CHECK
namespace nerfgb {
NG_BOUNDS_READER(bounds_read_ray_ops)
}  // namespace nerfgb
#endif
