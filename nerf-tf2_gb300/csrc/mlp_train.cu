// Backward pass of the NeRF MLP (nerf/core/model.py:334-394), the gradient
// tf.GradientTape takes at model.py:148-170, in FP32 with FP32 master
// weights.
//
// The forward (mlp.cu, STORE variant) writes every layer's post-activation
// rows to `acts` (kActsLd floats per row). The backward then runs layer by
// layer from the heads down:
//   head kernel   rgb = sigmoid(h9 Wr + br), sigma = ReLU(h7 ws + bs):
//                 dZ9 = (dpre_rgb Wr^T) * [h9 > 0], dpre_sigma, head grads
//   dW kernel     dW[k][n] += sum_m In[m][k] dZ[m][n]  (split over m, atomics)
//   dX kernel     dZ_prev[m][k] = (sum_n dZ[m][n] W[k][n] + dpre_sigma[m] ws[k])
//                                 * [h_prev[m][k] > 0]
// Gradients land in the flat Keras layout of the parameter blob.
#include "common.cuh"
#include "mlp_internal.cuh"

namespace nerfgb {
namespace train {

constexpr int kTM = 64;
constexpr int kDzLd = 256;  // row stride of the dZ buffers

// ---------------------------------------------------------------------------
// Heads
// ---------------------------------------------------------------------------
// Four tape values as FP32: the FP32 tape, or the BF16 tape of the
// tensor-core training forward.
__device__ __forceinline__ float4 tape4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ float4 tape4(const uint16_t *p) {
  const uint2 u = *reinterpret_cast<const uint2 *>(p);
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                     __uint_as_float(u.y & 0xffff0000u));
}

// Eight tape values as FP32 (16-byte BF16 load, or two of FP32).
__device__ __forceinline__ void tape8(const float *p, float (&v)[8]) {
  const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 4);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void tape8(const uint16_t *p, float (&v)[8]) {
  const uint4 u = *reinterpret_cast<const uint4 *>(p);
  const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[2 * i] = __uint_as_float(w[i] << 16);
    v[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

// One warp per row at a time, kHeadRows rows loaded before any is used:
// lane l owns h9 columns 4l..4l+3 and h7 columns 8l..8l+7 (coalesced tape
// loads), the head dot products are lane partials summed by a shuffle
// butterfly (every lane ends with the sums), dZ9 is written 16 bytes per
// lane, and the head weights' gradients accumulate in the lanes' registers
// over all of the warp's rows; they reach the blob once per block (shared
// atomics, then one global atomic per parameter).
constexpr int kHeadWarps = 8;
constexpr int kHeadRows = 2;

template <typename T>
__global__ void __launch_bounds__(32 * kHeadWarps, 2)
    head_bwd_kernel(const float *__restrict__ table, const T *__restrict__ acts, long long n,
                    const float *__restrict__ d_rgb, const float *__restrict__ d_sigma, float *__restrict__ dz9,
                    float *__restrict__ dsp_out, float *__restrict__ grads) {
  __shared__ float sAcc[644];  // dWr [128][3], dbr [3], dws [256], dbs [1]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < 644; e += blockDim.x) sAcc[e] = 0.0f;
  float wr[4][3], wsg[8];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) wr[j][c] = table[kRgbWOff + (4 * lane + j) * 3 + c];
#pragma unroll
  for (int j = 0; j < 8; ++j) wsg[j] = table[kSigmaWOff + 8 * lane + j];
  const float br[3] = {table[kRgbBOff], table[kRgbBOff + 1], table[kRgbBOff + 2]};
  const float bs = table[kSigmaBOff];
  float gwr[4][3], gws[8], gbr[3] = {0.f, 0.f, 0.f}, gbs = 0.0f;
#pragma unroll
  for (int j = 0; j < 4; ++j) gwr[j][0] = gwr[j][1] = gwr[j][2] = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) gws[j] = 0.0f;
  __syncthreads();
  const long long wstep = (long long)gridDim.x * kHeadWarps * kHeadRows;
  for (long long r0 = ((long long)blockIdx.x * kHeadWarps + warp) * kHeadRows; r0 < n; r0 += wstep) {
    float h9[kHeadRows][4], h7[kHeadRows][8], drgb[kHeadRows][3], dsg[kHeadRows];
#pragma unroll
    for (int q = 0; q < kHeadRows; ++q) {
      const long long r = r0 + q;
      if (r < n) {
        const float4 a = tape4(acts + r * kActsLd + acts_offset(9) + 4 * lane);
        h9[q][0] = a.x; h9[q][1] = a.y; h9[q][2] = a.z; h9[q][3] = a.w;
        tape8(acts + r * kActsLd + acts_offset(7) + 8 * lane, h7[q]);
#pragma unroll
        for (int c = 0; c < 3; ++c) drgb[q][c] = d_rgb[r * 3 + c];
        dsg[q] = d_sigma ? d_sigma[r] : 0.0f;
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) h9[q][j] = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j) h7[q][j] = 0.0f;
        drgb[q][0] = drgb[q][1] = drgb[q][2] = dsg[q] = 0.0f;
      }
    }
#pragma unroll
    for (int q = 0; q < kHeadRows; ++q) {
      const long long r = r0 + q;
      const bool valid = r < n;
      float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f, sp = 0.0f;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        p0 = fmaf(h9[q][j], wr[j][0], p0);
        p1 = fmaf(h9[q][j], wr[j][1], p1);
        p2 = fmaf(h9[q][j], wr[j][2], p2);
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) sp = fmaf(h7[q][j], wsg[j], sp);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        p0 += __shfl_xor_sync(0xffffffffu, p0, o);
        p1 += __shfl_xor_sync(0xffffffffu, p1, o);
        p2 += __shfl_xor_sync(0xffffffffu, p2, o);
        sp += __shfl_xor_sync(0xffffffffu, sp, o);
      }
      // rgb = sigmoid(h9 Wr + br), sigma = ReLU(h7 ws + bs) (model.py:374-386)
      const float pre[3] = {br[0] + p0, br[1] + p1, br[2] + p2};
      float drp[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float y = 1.0f / (1.0f + expf(-pre[c]));
        drp[c] = valid ? drgb[q][c] * y * (1.0f - y) : 0.0f;
      }
      const float dsp = (valid && sp + bs > 0.0f) ? dsg[q] : 0.0f;
      if (valid) {
        if (lane == 0) dsp_out[r] = dsp;
        float o[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float g = drp[0] * wr[j][0] + drp[1] * wr[j][1] + drp[2] * wr[j][2];
          o[j] = h9[q][j] > 0.0f ? g : 0.0f;
        }
        *reinterpret_cast<float4 *>(dz9 + r * kDzLd + 4 * lane) = make_float4(o[0], o[1], o[2], o[3]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) gwr[j][c] = fmaf(h9[q][j], drp[c], gwr[j][c]);
#pragma unroll
      for (int j = 0; j < 8; ++j) gws[j] = fmaf(h7[q][j], dsp, gws[j]);
#pragma unroll
      for (int c = 0; c < 3; ++c) gbr[c] += drp[c];
      gbs += dsp;
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(&sAcc[(4 * lane + j) * 3 + c], gwr[j][c]);
#pragma unroll
  for (int j = 0; j < 8; ++j) atomicAdd(&sAcc[387 + 8 * lane + j], gws[j]);
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(&sAcc[384 + c], gbr[c]);
    atomicAdd(&sAcc[643], gbs);
  }
  __syncthreads();
  float *gWr = grads + flat_offset(11), *gbr_out = gWr + 128 * 3;
  float *gws_out = grads + flat_offset(8), *gbs_out = gws_out + 256;
  for (int e = threadIdx.x; e < 644; e += blockDim.x) {
    float *dst = e < 384 ? gWr + e : e < 387 ? gbr_out + (e - 384) : e < 643 ? gws_out + (e - 387) : gbs_out;
    atomicAdd(dst, sAcc[e]);
  }
}

// ---------------------------------------------------------------------------
// dX: dz_out[m][k] = (sum_n dz_in[m][n] W[k][n] + dsp[m] ws[k]) * mask, k < 256
// ---------------------------------------------------------------------------
constexpr int kNC = 32;
constexpr size_t kDxSmem = (size_t)(kTM * (kNC + 4) + kNC * (256 + 4)) * sizeof(float);

__global__ void __launch_bounds__(256)
    dx_kernel(const float *__restrict__ W, int N, const float *__restrict__ dz_in, long long n,
              const float *__restrict__ dsp, const float *__restrict__ ws, const float *__restrict__ acts, int mask_off,
              float *__restrict__ dz_out) {
  extern __shared__ __align__(16) float sm[];
  float *sA = sm;                      // [kTM][kNC + 4]
  float *sB = sm + kTM * (kNC + 4);    // [kNC][256 + 4]: sB[nn][k] = W[k][n0 + nn]
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const long long ntiles = (n + kTM - 1) / kTM;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long row0 = tile * kTM;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    for (int n0 = 0; n0 < N; n0 += kNC) {
      __syncthreads();
      for (int e = tid; e < kTM * (kNC / 4); e += 256) {
        const int r = e / (kNC / 4), q = e % (kNC / 4);
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (row0 + r < n) v = *reinterpret_cast<const float4 *>(dz_in + (row0 + r) * kDzLd + n0 + 4 * q);
        *reinterpret_cast<float4 *>(sA + r * (kNC + 4) + 4 * q) = v;
      }
      {
        const int k = tid;  // one W row per thread
#pragma unroll
        for (int q = 0; q < kNC / 4; ++q) {
          const float4 v = *reinterpret_cast<const float4 *>(W + (long long)k * N + n0 + 4 * q);
          sB[(4 * q) * (256 + 4) + k] = v.x;
          sB[(4 * q + 1) * (256 + 4) + k] = v.y;
          sB[(4 * q + 2) * (256 + 4) + k] = v.z;
          sB[(4 * q + 3) * (256 + 4) + k] = v.w;
        }
      }
      __syncthreads();
#pragma unroll 4
      for (int nn = 0; nn < kNC; ++nn) {
        float a[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = sA[(ty * 8 + i) * (kNC + 4) + nn];
        const float4 b0 = *reinterpret_cast<const float4 *>(sB + nn * (256 + 4) + tx * 4);
        const float4 b1 = *reinterpret_cast<const float4 *>(sB + nn * (256 + 4) + 128 + tx * 4);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          acc[i][0] = fmaf(a[i], b0.x, acc[i][0]);
          acc[i][1] = fmaf(a[i], b0.y, acc[i][1]);
          acc[i][2] = fmaf(a[i], b0.z, acc[i][2]);
          acc[i][3] = fmaf(a[i], b0.w, acc[i][3]);
          acc[i][4] = fmaf(a[i], b1.x, acc[i][4]);
          acc[i][5] = fmaf(a[i], b1.y, acc[i][5]);
          acc[i][6] = fmaf(a[i], b1.z, acc[i][6]);
          acc[i][7] = fmaf(a[i], b1.w, acc[i][7]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const long long m = row0 + ty * 8 + i;
      if (m >= n) continue;
      const float ds = dsp ? dsp[m] : 0.0f;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = h * 128 + tx * 4;
        float4 v = make_float4(acc[i][4 * h], acc[i][4 * h + 1], acc[i][4 * h + 2], acc[i][4 * h + 3]);
        if (dsp) {
          v.x = fmaf(ds, ws[k], v.x);
          v.y = fmaf(ds, ws[k + 1], v.y);
          v.z = fmaf(ds, ws[k + 2], v.z);
          v.w = fmaf(ds, ws[k + 3], v.w);
        }
        if (mask_off >= 0) {
          const float4 hm = *reinterpret_cast<const float4 *>(acts + m * kActsLd + mask_off + k);
          v.x = hm.x > 0.0f ? v.x : 0.0f;
          v.y = hm.y > 0.0f ? v.y : 0.0f;
          v.z = hm.z > 0.0f ? v.z : 0.0f;
          v.w = hm.w > 0.0f ? v.w : 0.0f;
        }
        *reinterpret_cast<float4 *>(dz_out + m * kDzLd + k) = v;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// dW: dW[(k_dst0 + k) * out + n] += sum_m In[m][k] dZ[m][n]; db[n] += sum dZ.
// grid (N/64, ceil(K/64), m-slices); 4x4 outputs per thread.
// ---------------------------------------------------------------------------
constexpr int kMC = 32;
constexpr long long kMSlice = 8192;

__global__ void __launch_bounds__(256)
    dw_kernel(const float *__restrict__ acts, int in_off, int K, const float *__restrict__ dz, int N, long long n,
              float *__restrict__ dW, int out, int k_dst0, float *__restrict__ db) {
  __shared__ __align__(16) float sA[kMC][64 + 4];
  __shared__ __align__(16) float sB[kMC][64 + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int n0 = blockIdx.x * 64, k0 = blockIdx.y * 64;
  const long long m_begin = (long long)blockIdx.z * kMSlice;
  const long long m_end = m_begin + kMSlice < n ? m_begin + kMSlice : n;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
  float bacc[4] = {0.f, 0.f, 0.f, 0.f};
  const bool do_bias = db && blockIdx.y == 0 && ty == 0;
  for (long long m0 = m_begin; m0 < m_end; m0 += kMC) {
    __syncthreads();
    for (int e = tid; e < kMC * 64; e += 256) {
      const int mm = e >> 6, c = e & 63;
      const long long m = m0 + mm;
      sA[mm][c] = (m < m_end && k0 + c < K) ? acts[m * kActsLd + in_off + k0 + c] : 0.0f;
      sB[mm][c] = (m < m_end && n0 + c < N) ? dz[m * kDzLd + n0 + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll 8
    for (int mm = 0; mm < kMC; ++mm) {
      const float4 a = *reinterpret_cast<const float4 *>(&sA[mm][ty * 4]);
      const float4 b = *reinterpret_cast<const float4 *>(&sB[mm][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
      if (do_bias) {
#pragma unroll
        for (int j = 0; j < 4; ++j) bacc[j] += bv[j];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int k = k0 + ty * 4 + i;
    if (k >= K) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int nn = n0 + tx * 4 + j;
      if (nn < N) atomicAdd(dW + (long long)(k_dst0 + k) * out + nn, acc[i][j]);
    }
  }
  if (do_bias) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (n0 + tx * 4 + j < N) atomicAdd(db + n0 + tx * 4 + j, bacc[j]);
  }
}

static int persistent_grid(long long n) {
  const long long tiles = (n + kTM - 1) / kTM;
  const int sms = num_sms();
  const long long cap = (long long)(sms > 0 ? sms : 148) * 2;
  return (int)(tiles < cap ? tiles : cap);
}

}  // namespace train

template <typename T>
static int launch_head_bwd_t(const float *table, const T *tape, long long n, const float *d_rgb,
                             const float *d_sigma, float *dz9, float *dsp, float *grads, cudaStream_t st) {
  using namespace train;
  if (n == 0) return NERFGB_OK;
  const long long rows_per_block = (long long)kHeadWarps * kHeadRows;
  const long long blocks = (n + rows_per_block - 1) / rows_per_block;
  const int sms = num_sms();
  const long long cap = (long long)(sms > 0 ? sms : 148) * 2;  // two blocks per SM (launch bounds)
  head_bwd_kernel<T><<<(unsigned)(blocks < cap ? blocks : cap), 32 * kHeadWarps, 0, st>>>(table, tape, n, d_rgb,
                                                                                        d_sigma, dz9, dsp, grads);
  return launch_status();
}

int launch_head_bwd(const float *table, const float *tape, long long n, const float *d_rgb, const float *d_sigma,
                    float *dz9, float *dsp, float *grads, cudaStream_t st) {
  return launch_head_bwd_t(table, tape, n, d_rgb, d_sigma, dz9, dsp, grads, st);
}

int launch_head_bwd(const float *table, const uint16_t *tape, long long n, const float *d_rgb,
                    const float *d_sigma, float *dz9, float *dsp, float *grads, cudaStream_t st) {
  return launch_head_bwd_t(table, tape, n, d_rgb, d_sigma, dz9, dsp, grads, st);
}

namespace train {

static int launch_dw(const float *acts, int in_off, int K, const float *dz, int N, long long n, float *grads,
                     int flat_layer, int k_dst0, bool bias, cudaStream_t st) {
  const int out = flat_out(flat_layer);
  float *dW = grads + flat_offset(flat_layer);
  float *db = bias ? dW + (long long)flat_in(flat_layer) * out : nullptr;
  dim3 grid((N + 63) / 64, (K + 63) / 64, (unsigned)((n + kMSlice - 1) / kMSlice));
  dw_kernel<<<grid, 256, 0, st>>>(acts, in_off, K, dz, N, n, dW, out, k_dst0, db);
  return launch_status();
}

static int launch_dx(const float *table_base_W, int g, const float *dz_in, long long n, const float *dsp,
                     const float *ws, const float *acts, int mask_off, float *dz_out, cudaStream_t st) {
  if (cudaFuncSetAttribute(dx_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDxSmem) != cudaSuccess)
    return NERFGB_E_CUDA;
  dx_kernel<<<persistent_grid(n), 256, kDxSmem, st>>>(table_base_W + gemm_w_offset(g), gemm_n(g), dz_in, n, dsp,
                                                      ws, acts, mask_off, dz_out);
  return launch_status();
}

}  // namespace train
}  // namespace nerfgb

using namespace nerfgb;

extern "C" long long nerfgb_mlp_acts_floats_per_row(void) { return kActsLd; }

extern "C" long long nerfgb_mlp_backward_workspace_bytes(long long n_rows) {
  if (n_rows < 0) return -1;
  return (2 * n_rows * train::kDzLd + n_rows) * (long long)sizeof(float);
}

extern "C" int nerfgb_mlp_forward_train(const void *packed, const float *xyz, const float *dirs, long long n_rows,
                                        int rows_per_dir, float *rgb, float *sigma, float *acts, void *stream) {
  if (n_rows < 0 || rows_per_dir < 1) return NERFGB_E_INVALID_ARG;
  if (n_rows == 0) return NERFGB_OK;
  if (!packed || !xyz || !dirs || !rgb || !sigma || !acts || !aligned(packed, 256) || !aligned(acts, 16))
    return NERFGB_E_INVALID_ARG;
  return launch_mlp_fp32_store(packed, xyz, dirs, n_rows, rows_per_dir, rgb, sigma, acts, as_stream(stream));
}

extern "C" int nerfgb_mlp_backward(const void *packed, const float *acts, long long n_rows, const float *d_rgb,
                                   const float *d_sigma, float *grad_params, void *workspace, void *stream) {
  using namespace train;
  if (n_rows < 0) return NERFGB_E_INVALID_ARG;
  if (n_rows == 0) return NERFGB_OK;
  if (!packed || !acts || !d_rgb || !grad_params || !workspace || !aligned(packed, 256) || !aligned(acts, 16) ||
      !aligned(workspace, 16))
    return NERFGB_E_INVALID_ARG;
  cudaStream_t st = as_stream(stream);
  const long long n = n_rows;
  const float *W = reinterpret_cast<const float *>(packed);  // FP32 pack: padded [Kp][N] blocks
  const float *table = W + kFp32TableOff;
  float *bufA = reinterpret_cast<float *>(workspace);
  float *bufB = bufA + n * kDzLd;
  float *dsp = bufB + n * kDzLd;
  int rc;
  if ((rc = launch_head_bwd(table, acts, n, d_rgb, d_sigma, bufA, dsp, grad_params, st)) != NERFGB_OK) return rc;
  // dense_9 (flat 10): input [bottleneck | enc_dir], output 128.
  if ((rc = launch_dw(acts, acts_offset(8), 256, bufA, 128, n, grad_params, 10, 0, true, st)) != NERFGB_OK) return rc;
  if ((rc = launch_dw(acts, kActsEncDir, 27, bufA, 128, n, grad_params, 10, 256, false, st)) != NERFGB_OK) return rc;
  // dBottleneck = dZ9 W9[0:256]^T (dense_8 is linear: no mask).
  if ((rc = launch_dx(W, 9, bufA, n, nullptr, nullptr, acts, -1, bufB, st)) != NERFGB_OK) return rc;
  // dense_8 (flat 9): input h7.
  if ((rc = launch_dw(acts, acts_offset(7), 256, bufB, 256, n, grad_params, 9, 0, true, st)) != NERFGB_OK) return rc;
  // dZ7 = (dBott W8^T + dpre_sigma ws) * [h7 > 0]
  if ((rc = launch_dx(W, 8, bufB, n, dsp, table + kSigmaWOff, acts, acts_offset(7), bufA, st)) != NERFGB_OK)
    return rc;
  float *cur = bufA, *nxt = bufB;
  for (int l = 7; l >= 0; --l) {
    if (l == 0) {
      if ((rc = launch_dw(acts, kActsEncXyz, 63, cur, 256, n, grad_params, 0, 0, true, st)) != NERFGB_OK) return rc;
      break;
    }
    if (l == 5) {
      if ((rc = launch_dw(acts, acts_offset(4), 256, cur, 256, n, grad_params, 5, 0, true, st)) != NERFGB_OK)
        return rc;
      if ((rc = launch_dw(acts, kActsEncXyz, 63, cur, 256, n, grad_params, 5, 256, false, st)) != NERFGB_OK)
        return rc;
    } else {
      if ((rc = launch_dw(acts, acts_offset(l - 1), 256, cur, 256, n, grad_params, l, 0, true, st)) != NERFGB_OK)
        return rc;
    }
    if ((rc = launch_dx(W, l, cur, n, nullptr, nullptr, acts, acts_offset(l - 1), nxt, st)) != NERFGB_OK) return rc;
    float *t = cur;
    cur = nxt;
    nxt = t;
  }
  return NERFGB_OK;
}
