// Learned proposal sampler (not in the reference): a 2x64 ReLU MLP on the
// L=6 positional encoding of xyz (39 inputs, the concatenation convention of
// nerf/core/model.py:323-330) with a softplus density output. Its weights
// are composited over finite bins: the last interval is the previous
// spacing, not the reference's 1e10 (ray_utils.py:465-468). With 1e10, any
// positive density in the last bin takes all remaining transmittance and
// d(alpha_last)/d(sigma) vanishes, so a learned density could neither avoid
// nor be taught to avoid piling every ray's fine samples into that bin. At inference
// its density at the 64 stratified samples, composited exactly as the coarse
// pass is (ray_utils.py:426-482), replaces the coarse MLP's weights as the
// PDF of the inverse-transform fine sampler (ray_utils.py:276-406).
//
// Parameters (flat float32, 6,785 values): W1 [39,64], b1 [64], W2 [64,64],
// b2 [64], W3 [64], b3 [1].
//
// Forward: one thread per sample, weights broadcast from shared memory.
// Backward: recompute per 128-sample tile; per-sample vectors go to shared
// memory (odd row strides, conflict-free), then each thread reduces its own
// slice of dW over the tile in registers and adds it to the CTA's gradient
// in shared memory; one atomicAdd per parameter per CTA at the end.
#include <cuda_bf16.h>
#include <math.h>

#include "common.cuh"
#include "mlp_internal.cuh"
#include "ray_device.cuh"

namespace nerfgb {
namespace prop {

constexpr int kIn = 39, kH = 64;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kH, kW2 = kB1 + kH, kB2 = kW2 + kH * kH, kW3 = kB2 + kH, kB3 = kW3 + kH;
constexpr int kParams = kB3 + 1;  // 6785
constexpr int kThreads = 128;
constexpr int kEncLd = 41, kRowLd = 65;

__device__ __forceinline__ void encode6(const float x[3], float enc[kIn]) {
  enc[0] = x[0];
  enc[1] = x[1];
  enc[2] = x[2];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      float s, co;
      sincosf(fmul(x[c], enc_multiplier(l)), &s, &co);
      enc[3 + c * 12 + 2 * l] = s;
      enc[3 + c * 12 + 2 * l + 1] = co;
    }
}

__device__ __forceinline__ float softplus(float z) { return fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z))); }

__device__ __forceinline__ void load_params(const float *__restrict__ p, float *sw) {
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) sw[i] = p[i];
}

// h1 = ReLU(enc W1 + b1), z2 = h1 W2 + b2.
__device__ __forceinline__ void hidden(const float *sw, const float enc[kIn], float h1[kH], float z2[kH]) {
#pragma unroll
  for (int j = 0; j < kH; ++j) h1[j] = sw[kB1 + j];
#pragma unroll
  for (int k = 0; k < kIn; ++k) {
    const float e = enc[k];
#pragma unroll
    for (int j = 0; j < kH; j += 4) {
      const float4 w = *reinterpret_cast<const float4 *>(sw + kW1 + k * kH + j);
      h1[j] = fmaf(e, w.x, h1[j]);
      h1[j + 1] = fmaf(e, w.y, h1[j + 1]);
      h1[j + 2] = fmaf(e, w.z, h1[j + 2]);
      h1[j + 3] = fmaf(e, w.w, h1[j + 3]);
    }
  }
#pragma unroll
  for (int j = 0; j < kH; ++j) h1[j] = fmaxf(h1[j], 0.0f);
#pragma unroll
  for (int j = 0; j < kH; ++j) z2[j] = sw[kB2 + j];
#pragma unroll 4
  for (int k = 0; k < kH; ++k) {
    const float h = h1[k];
#pragma unroll
    for (int j = 0; j < kH; j += 4) {
      const float4 w = *reinterpret_cast<const float4 *>(sw + kW2 + k * kH + j);
      z2[j] = fmaf(h, w.x, z2[j]);
      z2[j + 1] = fmaf(h, w.y, z2[j + 1]);
      z2[j + 2] = fmaf(h, w.z, z2[j + 2]);
      z2[j + 3] = fmaf(h, w.w, z2[j + 3]);
    }
  }
}

__global__ void __launch_bounds__(kThreads)
    prop_fwd_kernel(const float *__restrict__ params, const float *__restrict__ xyz, long long n,
                    float *__restrict__ sigma) {
  __shared__ __align__(16) float sw[kParams + 3];
  load_params(params, sw);
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float x[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    float enc[kIn], h1[kH], z2[kH];
    encode6(x, enc);
    hidden(sw, enc, h1, z2);
    float z3 = sw[kB3];
#pragma unroll
    for (int j = 0; j < kH; ++j) z3 = fmaf(fmaxf(z2[j], 0.0f), sw[kW3 + j], z3);
    sigma[i] = softplus(z3);
  }
}

// ---------------------------------------------------------------------------
// Inference forward on tensor cores: BF16 operands, FP32 accumulation
// (mma.sync m16n8k16; at 6,656 MAC per sample the kernel is bound by the
// encoding and its memory traffic, not by the tensor pipe). One warp per 16
// samples: layer 1's accumulator fragments are layer 2's A fragments (the
// m16n8 C layout of two n-tiles is the m16k16 A layout), so h1 never leaves
// registers. Weights sit in shared memory transposed ([n][k], k contiguous),
// rows padded by 8 BF16 so that a B-fragment load is conflict-free.
// ---------------------------------------------------------------------------
constexpr int kK1 = 48;              // 39 inputs padded to 3 k-steps of 16
constexpr int kLd1 = kK1 + 8, kLd2 = kH + 8;
constexpr int kFwdWarps = 4;
constexpr int kEncLdB = kK1 + 8;     // per-warp encoding rows (BF16), padded

__device__ __forceinline__ uint32_t bf16x2_relu(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// The proposal's weights in shared memory for the BF16 forward.
struct PropSmemBf16 {
  __nv_bfloat16 W1[kH * kLd1];
  __nv_bfloat16 W2[kH * kLd2];
  float B1[kH], B2[kH], W3[kH], B3;
};

// All threads of the block; the caller synchronises. Weights transposed into
// [n][k] (reads follow the [k][n] source, coalesced).
__device__ __forceinline__ void stage_weights_bf16(const float *__restrict__ params, PropSmemBf16 &sp) {
  for (int e = threadIdx.x; e < kLd1 * kH; e += blockDim.x) {
    const int k = e / kH, nn = e % kH;
    sp.W1[nn * kLd1 + k] = __float2bfloat16_rn(k < kIn ? params[kW1 + k * kH + nn] : 0.0f);
  }
  for (int e = threadIdx.x; e < kLd2 * kH; e += blockDim.x) {
    const int k = e / kH, nn = e % kH;
    sp.W2[nn * kLd2 + k] = __float2bfloat16_rn(k < kH ? params[kW2 + k * kH + nn] : 0.0f);
  }
  for (int j = threadIdx.x; j < kH; j += blockDim.x) {
    sp.B1[j] = params[kB1 + j];
    sp.B2[j] = params[kB2 + j];
    sp.W3[j] = params[kW3 + j];
  }
  if (threadIdx.x == 0) sp.B3 = params[kB3];
}

// Octaves l0 .. l1-1 of coordinate c of the encoding (sin, cos of
// x * 2^l pi) from one sincosf at octave l0: the angle doubles exactly from
// one octave to the next, and sin 2a = (2 sin a) cos a, cos 2a = cos a cos a
// - sin a sin a, each operation rounded in FP32 (no FMA). Five doublings put
// an absolute error of a few 1e-6 on a value that is then rounded to BF16.
__device__ __forceinline__ void encode_octaves_bf16(__nv_bfloat16 *er, float xc, int c, int l0, int l1) {
  float sn, cs;
  sincosf(fmul(xc, enc_multiplier(l0)), &sn, &cs);
  for (int l = l0; l < l1; ++l) {
    if (l > l0) {
      const float s2 = fmul(fmul(2.0f, sn), cs);
      cs = fsub(fmul(cs, cs), fmul(sn, sn));
      sn = s2;
    }
    er[3 + c * 12 + 2 * l] = __float2bfloat16_rn(sn);
    er[3 + c * 12 + 2 * l + 1] = __float2bfloat16_rn(cs);
  }
}

// One 16-row tile's encodings (BF16) into the warp's buffer: two lanes per
// row (row = lane / 2). Lane h = 0 writes the three coordinates, coordinate
// 0's six octaves and coordinate 2's octaves 0-2; lane h = 1 the zero
// padding, coordinate 1's octaves and coordinate 2's octaves 3-5 (two
// sincosf per lane, encode_octaves_bf16). x: the lane's row's point.
__device__ __forceinline__ void encode_row_bf16(__nv_bfloat16 *enc, int lane, const float (&x)[3]) {
  const int row = lane >> 1, h = lane & 1;
  __nv_bfloat16 *er = enc + row * kEncLdB;
  if (h == 0) {
    er[0] = __float2bfloat16_rn(x[0]);
    er[1] = __float2bfloat16_rn(x[1]);
    er[2] = __float2bfloat16_rn(x[2]);
    encode_octaves_bf16(er, x[0], 0, 0, 6);
    encode_octaves_bf16(er, x[2], 2, 0, 3);
  } else {
#pragma unroll
    for (int k = kIn; k < kK1; ++k) er[k] = __float2bfloat16_rn(0.0f);
    encode_octaves_bf16(er, x[1], 1, 0, 6);
    encode_octaves_bf16(er, x[2], 2, 3, 6);
  }
}

// The densities of the tile's rows g = lane / 4 (s0) and g + 8 (s1), valid
// in the lanes with lane % 4 == 0, from the encodings in the warp's buffer.
__device__ __forceinline__ void tile_sigma_bf16(const PropSmemBf16 &sp, const __nv_bfloat16 *enc, int lane,
                                                float &s0, float &s1) {
  const int g = lane >> 2, t = lane & 3;
  // layer 1: [16 x 48] enc x [48 x 64] W1, accumulators start at b1
  float d1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    d1[j][0] = d1[j][2] = sp.B1[8 * j + 2 * t];
    d1[j][1] = d1[j][3] = sp.B1[8 * j + 2 * t + 1];
  }
#pragma unroll
  for (int ks = 0; ks < kK1 / 16; ++ks) {
    const int k0 = 16 * ks + 2 * t;
    const uint32_t *e0 = reinterpret_cast<const uint32_t *>(enc + g * kEncLdB + k0);
    const uint32_t *e1 = reinterpret_cast<const uint32_t *>(enc + (g + 8) * kEncLdB + k0);
    const uint32_t a[4] = {e0[0], e1[0], e0[4], e1[4]};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const __nv_bfloat16 *b = sp.W1 + (8 * j + g) * kLd1 + k0;
      mma_bf16(d1[j], a, *reinterpret_cast<const uint32_t *>(b), *reinterpret_cast<const uint32_t *>(b + 8));
    }
  }
  // layer 2: relu(h1) as BF16 A fragments straight from the layer-1 accumulators
  float d2[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    d2[j][0] = d2[j][2] = sp.B2[8 * j + 2 * t];
    d2[j][1] = d2[j][3] = sp.B2[8 * j + 2 * t + 1];
  }
#pragma unroll
  for (int ks = 0; ks < kH / 16; ++ks) {
    const uint32_t a[4] = {bf16x2_relu(d1[2 * ks][0], d1[2 * ks][1]), bf16x2_relu(d1[2 * ks][2], d1[2 * ks][3]),
                           bf16x2_relu(d1[2 * ks + 1][0], d1[2 * ks + 1][1]),
                           bf16x2_relu(d1[2 * ks + 1][2], d1[2 * ks + 1][3])};
    const int k0 = 16 * ks + 2 * t;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const __nv_bfloat16 *b = sp.W2 + (8 * j + g) * kLd2 + k0;
      mma_bf16(d2[j], a, *reinterpret_cast<const uint32_t *>(b), *reinterpret_cast<const uint32_t *>(b + 8));
    }
  }
  // layer 3 (FP32): relu(z2) . w3 over this thread's 16 columns, then the quad
  float p0 = 0.0f, p1 = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float w0 = sp.W3[8 * j + 2 * t], w1 = sp.W3[8 * j + 2 * t + 1];
    p0 = fmaf(fmaxf(d2[j][0], 0.0f), w0, fmaf(fmaxf(d2[j][1], 0.0f), w1, p0));
    p1 = fmaf(fmaxf(d2[j][2], 0.0f), w0, fmaf(fmaxf(d2[j][3], 0.0f), w1, p1));
  }
  p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
  p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
  p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
  p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
  s0 = softplus(sp.B3 + p0);
  s1 = softplus(sp.B3 + p1);
}

__global__ void __launch_bounds__(32 * kFwdWarps)
    prop_fwd_bf16_kernel(const float *__restrict__ params, const float *__restrict__ xyz, long long n,
                         float *__restrict__ sigma) {
  __shared__ __align__(16) PropSmemBf16 sp;
  __shared__ __align__(16) __nv_bfloat16 sEnc[kFwdWarps][16 * kEncLdB];
  stage_weights_bf16(params, sp);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long ntiles = (n + 15) / 16;
  const long long wstride = (long long)gridDim.x * kFwdWarps;
  __nv_bfloat16 *enc = sEnc[threadIdx.x >> 5];
  for (long long tile = (long long)blockIdx.x * kFwdWarps + (threadIdx.x >> 5); tile < ntiles; tile += wstride) {
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    {
      const long long gr = tile * 16 + (lane >> 1);
      float x[3] = {0.f, 0.f, 0.f};
      if (gr < n) {
        x[0] = xyz[3 * gr];
        x[1] = xyz[3 * gr + 1];
        x[2] = xyz[3 * gr + 2];
      }
      encode_row_bf16(enc, lane, x);
    }
    __syncwarp();
    float s0, s1;
    tile_sigma_bf16(sp, enc, lane, s0, s1);
    if (t == 0) {
      if (r0 < n) sigma[r0] = s0;
      if (r1 < n) sigma[r1] = s1;
    }
    __syncwarp();  // the buffer is rewritten by the next tile
  }
}

// ---------------------------------------------------------------------------
// Front end of the BF16/FP8 proposal paths, one warp per ray: the ray's S
// stratified samples (coarse_sample_kernel's arithmetic: Philox draws
// inside, t, bin edges, widths, points written out), the proposal density
// at them (prop_fwd_bf16_kernel's arithmetic, 16 samples per tile), the
// proposal weights over the bins (composite_ray with the finite last
// interval, nerfgb_proposal_weights' arithmetic) written to w_out when
// given, and with gate_map the coarse gate (sample j on where its weight >
// tau; gate_ray zeroes the coarse sigma at the off samples). Replaces the
// coarse sampler, proposal forward and proposal compositing launches.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kFwdWarps)
    prop_front_kernel(const float *__restrict__ params, const float *__restrict__ rays_o,
                      const float *__restrict__ rays_d, const float *__restrict__ near,
                      const float *__restrict__ far, const float *__restrict__ u, unsigned long long seed, int R,
                      int S, int perturb, int lin_inv, int mode, float *__restrict__ xyz, float *__restrict__ t_out,
                      float *__restrict__ edges, float *__restrict__ widths, float *__restrict__ w_out, float tau,
                      unsigned char *__restrict__ gate_mask, int *__restrict__ gate_map,
                      int *__restrict__ gate_count, float *__restrict__ gate_sig_zero) {
  __shared__ __align__(16) PropSmemBf16 sp;
  __shared__ __align__(16) __nv_bfloat16 sEnc[kFwdWarps][16 * kEncLdB];
  extern __shared__ float fsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
  float *s_t = fsm + warp * 6 * S;  // t [S], sigma [S], weights [S], points [3S]
  float *s_sig = s_t + S;
  float *s_w = s_sig + S;
  float *s_x = s_w + S;
  __nv_bfloat16 *enc = sEnc[warp];
  stage_weights_bf16(params, sp);
  __syncthreads();
  for (int r = blockIdx.x * kFwdWarps + warp; r < R; r += gridDim.x * kFwdWarps) {
    const long long base = (long long)r * S;
    const float nr = near[r], fr = far[r];
    for (int i = lane; i < S; i += 32) {
      const BinSample b = coarse_bin_sample(rays_o, rays_d, nr, fr, u, seed, r, S, i, perturb, lin_inv);
      t_out[base + i] = b.t;
      widths[base + i] = b.w;
      edges[(long long)r * (S + 1) + i] = b.e0;
      if (i == S - 1) edges[(long long)r * (S + 1) + S] = b.e1;
      s_t[i] = b.t;
#pragma unroll
      for (int c = 0; c < 3; ++c) s_x[3 * i + c] = b.x[c];
    }
    __syncwarp();
    for (int j = lane; j < 3 * S; j += 32) xyz[3 * base + j] = s_x[j];
    for (int i0 = 0; i0 < S; i0 += 16) {
      const int i = i0 + (lane >> 1);
      float x[3] = {0.f, 0.f, 0.f};
      if (i < S) {
        x[0] = s_x[3 * i];
        x[1] = s_x[3 * i + 1];
        x[2] = s_x[3 * i + 2];
      }
      encode_row_bf16(enc, lane, x);
      __syncwarp();
      float s0, s1;
      tile_sigma_bf16(sp, enc, lane, s0, s1);
      if (t4 == 0) {
        if (i0 + g < S) s_sig[i0 + g] = s0;
        if (i0 + g + 8 < S) s_sig[i0 + g + 8] = s1;
      }
      __syncwarp();  // the buffer is rewritten by the next tile; s_sig complete
    }
    float m[5];
    composite_ray(lane, s_t, s_sig, nullptr, S, mode, -1.0f, s_w, m);
    __syncwarp();
    if (w_out)
      for (int j = lane; j < S; j += 32) w_out[base + j] = s_w[j];
    if (gate_map)
      gate_ray(lane, base, S, R, [&](int j) { return s_w[j] > tau; }, gate_mask, gate_map, gate_count,
               gate_sig_zero, nullptr, kSiteGateCoarse);
    __syncwarp();
  }
}

constexpr size_t kBwdSmem =
    (size_t)(2 * (kParams + 3) + kThreads * kEncLd + 4 * kThreads * kRowLd + kThreads) * sizeof(float);

// grads += d/dparams sum_i dsigma_i * sigma_i.
__global__ void __launch_bounds__(kThreads)
    prop_bwd_kernel(const float *__restrict__ params, const float *__restrict__ xyz, const float *__restrict__ dsig,
                    long long n, float *__restrict__ grads) {
  extern __shared__ __align__(16) float sm[];
  float *sw = sm;
  float *sacc = sw + kParams + 3;  // this CTA's gradient, one slice per thread
  float *sENC = sacc + kParams + 3;
  float *sH1 = sENC + kThreads * kEncLd;
  float *sH2 = sH1 + kThreads * kRowLd;
  float *sDZ2 = sH2 + kThreads * kRowLd;
  float *sDZ1 = sDZ2 + kThreads * kRowLd;
  float *sDZ3 = sDZ1 + kThreads * kRowLd;
  const int tid = threadIdx.x, j = tid & 63, half = tid >> 6;
  load_params(params, sw);
  for (int q = tid; q < kParams; q += kThreads) sacc[q] = 0.0f;
  __syncthreads();
  const long long ntiles = (n + kThreads - 1) / kThreads;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long i = tile * kThreads + tid;
    const bool valid = i < n;
    float x[3] = {0.f, 0.f, 0.f};
    if (valid) {
      x[0] = xyz[3 * i];
      x[1] = xyz[3 * i + 1];
      x[2] = xyz[3 * i + 2];
    }
    float enc[kIn], h1[kH], z2[kH];
    encode6(x, enc);
    hidden(sw, enc, h1, z2);
#pragma unroll
    for (int k = 0; k < kIn; ++k) sENC[tid * kEncLd + k] = enc[k];
#pragma unroll
    for (int k = 0; k < kH; ++k) sH1[tid * kRowLd + k] = h1[k];
    float z3 = sw[kB3];
#pragma unroll
    for (int q = 0; q < kH; ++q) z3 = fmaf(fmaxf(z2[q], 0.0f), sw[kW3 + q], z3);
    const float dz3 = valid ? dsig[i] / (1.0f + expf(-z3)) : 0.0f;  // softplus' = sigmoid
    sDZ3[tid] = dz3;
#pragma unroll
    for (int q = 0; q < kH; ++q) {
      sH2[tid * kRowLd + q] = fmaxf(z2[q], 0.0f);
      z2[q] = z2[q] > 0.0f ? sw[kW3 + q] * dz3 : 0.0f;  // z2 now holds dz2
      sDZ2[tid * kRowLd + q] = z2[q];
    }
    // dz1 = (W2 dz2) * [h1 > 0]
#pragma unroll 4
    for (int k = 0; k < kH; ++k) {
      float acc = 0.0f;
#pragma unroll
      for (int q = 0; q < kH; q += 4) {
        const float4 w = *reinterpret_cast<const float4 *>(sw + kW2 + k * kH + q);
        acc = fmaf(w.x, z2[q], acc);
        acc = fmaf(w.y, z2[q + 1], acc);
        acc = fmaf(w.z, z2[q + 2], acc);
        acc = fmaf(w.w, z2[q + 3], acc);
      }
      sDZ1[tid * kRowLd + k] = sH1[tid * kRowLd + k] > 0.0f ? acc : 0.0f;
    }
    __syncthreads();
    // Reduce this tile into the thread's slice: column j, rows of its half.
    float aW2[32], aW1[20], aB1 = 0.f, aB2 = 0.f, aW3 = 0.f, aB3 = 0.f;
#pragma unroll
    for (int q = 0; q < 32; ++q) aW2[q] = 0.f;
#pragma unroll
    for (int q = 0; q < 20; ++q) aW1[q] = 0.f;
    for (int t = 0; t < kThreads; ++t) {
      const float d2 = sDZ2[t * kRowLd + j], d1 = sDZ1[t * kRowLd + j];
#pragma unroll
      for (int q = 0; q < 32; ++q) aW2[q] = fmaf(sH1[t * kRowLd + half * 32 + q], d2, aW2[q]);
#pragma unroll
      for (int q = 0; q < 20; ++q)
        if (half * 20 + q < kIn) aW1[q] = fmaf(sENC[t * kEncLd + half * 20 + q], d1, aW1[q]);
      if (half == 0) {
        aB1 += d1;
        aB2 += d2;
        aW3 = fmaf(sH2[t * kRowLd + j], sDZ3[t], aW3);
        if (j == 0) aB3 += sDZ3[t];
      }
    }
#pragma unroll
    for (int q = 0; q < 32; ++q) sacc[kW2 + (half * 32 + q) * kH + j] += aW2[q];
#pragma unroll
    for (int q = 0; q < 20; ++q)
      if (half * 20 + q < kIn) sacc[kW1 + (half * 20 + q) * kH + j] += aW1[q];
    if (half == 0) {
      sacc[kB1 + j] += aB1;
      sacc[kB2 + j] += aB2;
      sacc[kW3 + j] += aW3;
      if (j == 0) sacc[kB3] += aB3;
    }
    __syncthreads();
  }
  for (int q = tid; q < kParams; q += kThreads) atomicAdd(grads + q, sacc[q]);
}

static int grid_for(long long n, int per_cta_items) {
  long long g = (n + per_cta_items - 1) / per_cta_items;
  int sms = num_sms();
  long long cap = (long long)(sms > 0 ? sms : 148) * 8;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

}  // namespace prop

int launch_proposal_forward(const float *params, const float *xyz, long long n, float *sigma, cudaStream_t stream) {
  prop::prop_fwd_kernel<<<prop::grid_for(n, prop::kThreads), prop::kThreads, 0, stream>>>(params, xyz, n, sigma);
  return launch_status();
}

int launch_proposal_forward_bf16(const float *params, const float *xyz, long long n, float *sigma,
                                 cudaStream_t stream) {
  // persistent: two CTAs per SM, so that each converts the weights once for
  // many 16-sample tiles
  const long long tiles = (n + 16 * prop::kFwdWarps - 1) / (16 * prop::kFwdWarps);
  const int sms = num_sms();
  const long long cap = (long long)(sms > 0 ? sms : 148) * 2;
  prop::prop_fwd_bf16_kernel<<<(unsigned)(tiles < cap ? tiles : cap), 32 * prop::kFwdWarps, 0, stream>>>(
      params, xyz, n, sigma);
  return launch_status();
}

int launch_prop_front(const float *params, const float *rays_o, const float *rays_d, const float *near,
                      const float *far, const float *u, unsigned long long seed, int R, int S, int perturb,
                      int lin_inv, int mode, float *xyz, float *t_vals, float *edges, float *widths, float *w_out,
                      const CompositeGate &gate, cudaStream_t stream) {
  if (R == 0) return NERFGB_OK;
  const size_t smem = (size_t)prop::kFwdWarps * 6 * S * sizeof(float);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(prop::prop_front_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return NERFGB_E_CUDA;
  // persistent: each CTA converts the weights once for many rays
  const long long blocks = (R + prop::kFwdWarps - 1) / prop::kFwdWarps;
  const int sms = num_sms();
  const long long cap = (long long)(sms > 0 ? sms : 148) * 4;
  prop::prop_front_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 32 * prop::kFwdWarps, smem, stream>>>(
      params, rays_o, rays_d, near, far, u, seed, R, S, perturb, lin_inv, mode, xyz, t_vals, edges, widths, w_out,
      gate.tau, gate.mask, gate.row_map, gate.count, gate.sig_zero);
  return launch_status();
}

}  // namespace nerfgb

using namespace nerfgb;

extern "C" long long nerfgb_proposal_param_count(void) { return prop::kParams; }

extern "C" int nerfgb_proposal_weights(const float *sigma, const float *t_vals, int n_rays, int n_bins, int trans_mode,
                                       float *weights, void *stream) {
  if (n_rays < 0 || n_bins < 2) return NERFGB_E_INVALID_ARG;
  if (n_bins > 2048) return NERFGB_E_UNSUPPORTED;
  if (trans_mode != NERFGB_TRANS_CUMPROD && trans_mode != NERFGB_TRANS_LOGSUM) return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!sigma || !t_vals || !weights) return NERFGB_E_INVALID_ARG;
  return launch_composite(nullptr, sigma, t_vals, n_rays, n_bins, 0, trans_mode, -1.0f, weights, nullptr, nullptr,
                          nullptr, as_stream(stream));
}

extern "C" int nerfgb_proposal_weights_backward(const float *sigma, const float *t_vals, const float *grad_weights,
                                                int n_rays, int n_bins, float *grad_sigma, void *stream) {
  if (n_rays < 0 || n_bins < 2) return NERFGB_E_INVALID_ARG;
  if (n_bins > 2048) return NERFGB_E_UNSUPPORTED;
  if (n_rays == 0) return NERFGB_OK;
  if (!sigma || !t_vals || !grad_weights || !grad_sigma) return NERFGB_E_INVALID_ARG;
  return launch_composite_bwd(sigma, t_vals, nullptr, nullptr, grad_weights, n_rays, n_bins, 0, -1.0f, grad_sigma,
                              nullptr, as_stream(stream));
}

extern "C" int nerfgb_proposal_forward_bf16(const float *params, const float *xyz, long long n, float *sigma,
                                            void *stream) {
  if (n < 0) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!params || !xyz || !sigma) return NERFGB_E_INVALID_ARG;
  return launch_proposal_forward_bf16(params, xyz, n, sigma, as_stream(stream));
}

extern "C" int nerfgb_proposal_forward(const float *params, const float *xyz, long long n, float *sigma,
                                       void *stream) {
  if (n < 0) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!params || !xyz || !sigma) return NERFGB_E_INVALID_ARG;
  return launch_proposal_forward(params, xyz, n, sigma, as_stream(stream));
}

extern "C" int nerfgb_proposal_backward(const float *params, const float *xyz, const float *grad_sigma, long long n,
                                        float *grad_params, void *stream) {
  if (n < 0) return NERFGB_E_INVALID_ARG;
  if (n == 0) return NERFGB_OK;
  if (!params || !xyz || !grad_sigma || !grad_params) return NERFGB_E_INVALID_ARG;
  if (cudaFuncSetAttribute(prop::prop_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)prop::kBwdSmem) != cudaSuccess)
    return NERFGB_E_CUDA;
  const long long ntiles = (n + prop::kThreads - 1) / prop::kThreads;
  int sms = num_sms();
  int grid = (int)(ntiles < sms ? ntiles : sms);
  prop::prop_bwd_kernel<<<grid, prop::kThreads, prop::kBwdSmem, as_stream(stream)>>>(params, xyz, grad_sigma, n,
                                                                                      grad_params);
  return launch_status();
}

#ifdef NERF_BOUNDS_CHECK
namespace nerfgb {
NG_BOUNDS_READER(bounds_read_proposal)
}  // namespace nerfgb
#endif
