// BF16 backward of the NeRF MLP (nerf/core/model.py:334-394; the gradient
// tf.GradientTape takes at model.py:148-170) with FP32 master weights.
//
// The forward is the tensor-core BF16 kernel with its tape (mlp_tc.cu,
// STORE): each layer's BF16 activations are exactly the operands its
// successor's MMAs read. The backward runs the layers of mlp_train.cu from
// the heads down, with every product a BF16 tensor-core GEMM accumulating in
// FP32 (gemm_tc.cu):
//   prep    z = dX (+ dpre_sigma * ws at dense_7) * [h > 0]  (dX in BF16
//           from the GEMM, z in FP32), dz = bf16(z), db += column sums of z
//   dW      grads[k][n] += sum_m In[m][k] dz[m][n]   (In = the tape's BF16 input columns)
//   dX      dX[m][k] = sum_n dz[m][n] W[k][n], k < 256 (W = BF16 copy of the FP32
//           master weights, resident in shared memory for the launch)
#include <cuda_bf16.h>

#include "common.cuh"
#include "mlp_internal.cuh"

namespace nerfgb {
namespace train16 {

constexpr int kDzLd = 256;                    // row stride of the dZ buffers
constexpr int kMaxSplits = 160;               // row splits of a dW GEMM (partial sums in the workspace)
constexpr int kPrepBlocksPerSm = 4;          // persistent prep grid (resident at 54 registers)

__global__ void to_bf16_kernel(const float *__restrict__ src, __nv_bfloat16 *__restrict__ dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

// z = raw (+ dsp * ws) (* [tape act > 0]) over N columns (N = 128 or 256);
// dz = bf16(z); db[n] += sum_m z. Eight columns per thread (16-byte loads
// and stores), N / 8 threads per row; the blocks stride over the rows (a
// persistent grid of several blocks per SM, for the loads in flight), each
// thread keeping its columns' sums in registers over all of its rows; the
// sums are reduced in shared memory, one atomic per column per block.
__device__ __forceinline__ void load8(const float *p, float (&v)[8]) {
  const float4 a = *reinterpret_cast<const float4 *>(p), b = *reinterpret_cast<const float4 *>(p + 4);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void load8(const __nv_bfloat16 *p, float (&v)[8]) {
  const uint4 u = *reinterpret_cast<const uint4 *>(p);
  const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[2 * i] = __uint_as_float(w[i] << 16);
    v[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

template <typename Tin, bool MASK, bool SIG>
__global__ void __launch_bounds__(256)
    prep_kernel(const Tin *__restrict__ raw, long long M, int N, const uint16_t *__restrict__ tape, int act_off,
                const float *__restrict__ dsp, const float *__restrict__ ws, __nv_bfloat16 *__restrict__ dz,
                float *__restrict__ db) {
  __shared__ float red[256 * 8];
  const int tpr = N / 8;                    // threads per row
  const int rpp = 256 / tpr;                // rows per pass
  const int t = threadIdx.x, c0 = (t % tpr) * 8, rsub = t / tpr;
  const long long mstep = (long long)gridDim.x * rpp;
  float w[8], sum[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    w[i] = SIG ? ws[c0 + i] : 0.0f;
    sum[i] = 0.0f;
  }
#pragma unroll 4
  for (long long m = (long long)blockIdx.x * rpp + rsub; m < M; m += mstep) {
    float z[8];
    load8(raw + m * kDzLd + c0, z);
    if (SIG) {
      const float d = dsp[m];
#pragma unroll
      for (int i = 0; i < 8; ++i) z[i] = fmaf(d, w[i], z[i]);
    }
    if (MASK) {
      const uint4 a = *reinterpret_cast<const uint4 *>(tape + m * kActsLd + act_off + c0);
      const uint32_t aw[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t lo = aw[i] & 0xffffu, hi = aw[i] >> 16;  // ReLU outputs: > 0 unless 0 (or -0)
        if (lo == 0 || (lo & 0x8000u)) z[2 * i] = 0.0f;
        if (hi == 0 || (hi & 0x8000u)) z[2 * i + 1] = 0.0f;
      }
    }
    uint4 o;
    __nv_bfloat162 p0 = __floats2bfloat162_rn(z[0], z[1]), p1 = __floats2bfloat162_rn(z[2], z[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(z[4], z[5]), p3 = __floats2bfloat162_rn(z[6], z[7]);
    o.x = *reinterpret_cast<uint32_t *>(&p0);
    o.y = *reinterpret_cast<uint32_t *>(&p1);
    o.z = *reinterpret_cast<uint32_t *>(&p2);
    o.w = *reinterpret_cast<uint32_t *>(&p3);
    *reinterpret_cast<uint4 *>(dz + m * kDzLd + c0) = o;
#pragma unroll
    for (int i = 0; i < 8; ++i) sum[i] += z[i];
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) red[rsub * N + c0 + i] = sum[i];
  __syncthreads();
  for (int c = t; c < N; c += 256) {
    float a = 0.0f;
    for (int r = 0; r < rpp; ++r) a += red[r * N + c];
    atomicAdd(db + c, a);
  }
}

struct Ws {
  float *f32, *dsp;                  // dZ9 from the heads (FP32), dpre_sigma
  __nv_bfloat16 *raw, *dz, *wb;      // dX output, masked dZ (GEMM operand), BF16 weights
  float *part;                       // dW split partials
  long long bytes;
};

static long long a256(long long b) { return (b + 255) / 256 * 256; }

static Ws carve(void *base, long long n) {
  Ws w{};
  long long off = 0;
  auto take = [&](long long bytes) -> char * {
    char *p = base ? static_cast<char *>(base) + off : nullptr;
    off += a256(bytes);
    return p;
  };
  w.f32 = reinterpret_cast<float *>(take(n * kDzLd * 4));
  w.dsp = reinterpret_cast<float *>(take(n * 4));
  w.raw = reinterpret_cast<__nv_bfloat16 *>(take(n * kDzLd * 2));
  w.dz = reinterpret_cast<__nv_bfloat16 *>(take(n * kDzLd * 2));
  w.wb = reinterpret_cast<__nv_bfloat16 *>(take(kGemmWElems * 2));
  w.part = reinterpret_cast<float *>(take(gemm_dw_partial_floats(kMaxSplits) * 4));
  w.bytes = off;
  return w;
}

template <bool MASK, bool SIG, typename Tin>
static int prep(const Tin *raw, long long M, int N, const uint16_t *tape, int act_off, const float *dsp,
                const float *ws, __nv_bfloat16 *dz, float *db, cudaStream_t st) {
  const long long rpp = 256 / (N / 8);  // rows per block pass
  const long long passes = (M + rpp - 1) / rpp;
  const int sms = num_sms();
  const long long cap = (long long)(sms > 0 ? sms : 148) * kPrepBlocksPerSm;
  prep_kernel<Tin, MASK, SIG><<<(unsigned)(passes < cap ? passes : cap), 256, 0, st>>>(raw, M, N, tape, act_off, dsp,
                                                                                     ws, dz, db);
  return launch_status();
}

// grads (flat layer fl, rows [k_dst0, k_dst0 + K)) += In^T dz, In = tape
// columns [in_off, in_off + K).
static int dW(const uint16_t *tape, int in_off, int K, const __nv_bfloat16 *dz, int N, long long M, float *grads,
              int fl, int k_dst0, float *part, int *err, cudaStream_t st) {
  const int sms = num_sms();
  if (sms <= 0) return NERFGB_E_DEVICE;
  const long long chunks = (M + 63) / 64;
  int splits = sms < kMaxSplits ? sms : kMaxSplits;
  if (chunks < splits) splits = (int)chunks;
  return launch_gemm_dw(reinterpret_cast<const __nv_bfloat16 *>(tape) + in_off, kActsLd, K, dz, N, M,
                        grads + flat_offset(fl) + (long long)k_dst0 * N, part, splits, err, st);
}

// out [M][256] (BF16) = dz [M][N] W_g[0:256][N]^T.
static int dX(const __nv_bfloat16 *wb, int g, const __nv_bfloat16 *dz, long long M, __nv_bfloat16 *out, int *err,
              cudaStream_t st) {
  return launch_gemm_dx(dz, M, gemm_n(g), wb + gemm_w_offset(g), out, err, st);
}

static float *bias_grad(float *grads, int fl) { return grads + flat_offset(fl) + (long long)flat_in(fl) * flat_out(fl); }

}  // namespace train16
}  // namespace nerfgb

using namespace nerfgb;

extern "C" long long nerfgb_mlp_backward_bf16_workspace_bytes(long long n_rows) {
  if (n_rows < 0) return -1;
  return train16::carve(nullptr, n_rows).bytes;
}

extern "C" int nerfgb_mlp_forward_train_bf16(const void *packed_bf16, const float *xyz, const float *dirs,
                                             long long n_rows, int rows_per_dir, float *rgb, float *sigma,
                                             void *tape, int *err_word, void *stream) {
  if (n_rows < 0 || rows_per_dir < 1) return NERFGB_E_INVALID_ARG;
  if (n_rows == 0) return NERFGB_OK;
  if (!packed_bf16 || !xyz || !dirs || !rgb || !sigma || !tape || !err_word || !aligned(packed_bf16, 256) ||
      !aligned(tape, 16))
    return NERFGB_E_INVALID_ARG;
  return launch_mlp_bf16_train(packed_bf16, xyz, dirs, n_rows, rows_per_dir, rgb, sigma,
                               reinterpret_cast<uint16_t *>(tape), err_word, as_stream(stream));
}

extern "C" int nerfgb_mlp_backward_bf16(const void *packed_fp32, const void *tape, long long n_rows,
                                        const float *d_rgb, const float *d_sigma, float *grad_params,
                                        void *workspace, int *err_word, void *stream) {
  using namespace train16;
  if (n_rows < 0) return NERFGB_E_INVALID_ARG;
  if (n_rows == 0) return NERFGB_OK;
  if (!packed_fp32 || !tape || !d_rgb || !grad_params || !workspace || !err_word || !aligned(packed_fp32, 256) ||
      !aligned(tape, 16) || !aligned(workspace, 256))
    return NERFGB_E_INVALID_ARG;
  int *err = err_word;
  cudaStream_t st = as_stream(stream);
  const long long M = n_rows;
  const float *W = reinterpret_cast<const float *>(packed_fp32);  // FP32 pack: [Kp][N] blocks, then the table
  const float *table = W + kFp32TableOff;
  const uint16_t *tp = reinterpret_cast<const uint16_t *>(tape);
  Ws w = carve(workspace, M);
  int rc;
  to_bf16_kernel<<<(unsigned)((kGemmWElems + 255) / 256), 256, 0, st>>>(W, w.wb, kGemmWElems);
  if ((rc = launch_status()) != NERFGB_OK) return rc;
  // heads -> dZ9 (masked by [h9 > 0], FP32) and dpre_sigma
  if ((rc = launch_head_bwd(table, tp, M, d_rgb, d_sigma, w.f32, w.dsp, grad_params, st)) != NERFGB_OK) return rc;
  // dense_9 (flat 10): input [bottleneck | enc_dir], 128 outputs
  if ((rc = prep<false, false>(w.f32, M, 128, tp, 0, nullptr, nullptr, w.dz, bias_grad(grad_params, 10), st)) !=
      NERFGB_OK)
    return rc;
  if ((rc = dW(tp, acts_offset(8), 256, w.dz, 128, M, grad_params, 10, 0, w.part, err, st)) != NERFGB_OK) return rc;
  if ((rc = dW(tp, kActsEncDir, 27, w.dz, 128, M, grad_params, 10, 256, w.part, err, st)) != NERFGB_OK) return rc;
  if ((rc = dX(w.wb, 9, w.dz, M, w.raw, err, st)) != NERFGB_OK) return rc;
  // dense_8 (flat 9): linear, input h7
  if ((rc = prep<false, false>(w.raw, M, 256, tp, 0, nullptr, nullptr, w.dz, bias_grad(grad_params, 9), st)) !=
      NERFGB_OK)
    return rc;
  if ((rc = dW(tp, acts_offset(7), 256, w.dz, 256, M, grad_params, 9, 0, w.part, err, st)) != NERFGB_OK) return rc;
  if ((rc = dX(w.wb, 8, w.dz, M, w.raw, err, st)) != NERFGB_OK) return rc;
  // dense_7 .. dense_0
  for (int l = 7; l >= 0; --l) {
    float *db = bias_grad(grad_params, l);
    rc = (l == 7) ? prep<true, true>(w.raw, M, 256, tp, acts_offset(7), w.dsp, table + kSigmaWOff, w.dz, db, st)
                  : prep<true, false>(w.raw, M, 256, tp, acts_offset(l), nullptr, nullptr, w.dz, db, st);
    if (rc != NERFGB_OK) return rc;
    if (l == 0) {
      if ((rc = dW(tp, kActsEncXyz, 63, w.dz, 256, M, grad_params, 0, 0, w.part, err, st)) != NERFGB_OK) return rc;
      break;
    }
    if (l == 5) {
      if ((rc = dW(tp, acts_offset(4), 256, w.dz, 256, M, grad_params, 5, 0, w.part, err, st)) != NERFGB_OK) return rc;
      if ((rc = dW(tp, kActsEncXyz, 63, w.dz, 256, M, grad_params, 5, 256, w.part, err, st)) != NERFGB_OK) return rc;
    } else {
      if ((rc = dW(tp, acts_offset(l - 1), 256, w.dz, 256, M, grad_params, l, 0, w.part, err, st)) != NERFGB_OK)
        return rc;
    }
    if ((rc = dX(w.wb, l, w.dz, M, w.raw, err, st)) != NERFGB_OK) return rc;
  }
  return NERFGB_OK;
}
