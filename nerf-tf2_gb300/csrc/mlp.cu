// NeRF MLP (nerf/core/model.py:334-394): weight packing, the FP32 SIMT
// forward (the plain path) and the precision dispatcher.
//
// FP32 SIMT forward: one CTA of 256 threads owns a 64-row tile. The tile's
// activations stay in shared memory for all ten GEMM layers
// (X[64][320]: hidden state in columns 0..255, enc_xyz in 256..319, later
// enc_dir in 256..287). Weights stream from L2 in K-chunks of 32 rows,
// double-buffered with cp.async. Each thread accumulates an 8x8 register
// block: 8 rows x (4 + 4) columns.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include "common.cuh"
#include "mlp_internal.cuh"

namespace nerfgb {

// ---------------------------------------------------------------------------
// Packing
// ---------------------------------------------------------------------------
__global__ void pack_kernel(const float *__restrict__ flat, int precision, unsigned char *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kGemmWElems) {
    int g = 0;
    while (g + 1 < kNumGemm && i >= gemm_w_offset(g + 1)) ++g;
    long long e = i - gemm_w_offset(g);
    const int N = gemm_n(g);
    int k = (int)(e / N), n = (int)(e - (long long)k * N);
    const int L = flat_idx_of_gemm(g);
    float v = (k < gemm_k(g)) ? flat[flat_offset(L) + (long long)k * N + n] : 0.0f;
    if (precision == NERFGB_PREC_FP32) {
      reinterpret_cast<float *>(out)[i] = v;
    } else if (precision == NERFGB_PREC_FP8) {
      const float sc = reinterpret_cast<const float *>(out + kFp8ScaleOff)[bias_offset(g) + n];
      int c = k >> 5, kk = k & 31;
      long long byte = gemm_w_offset(g) + (long long)c * (32 * N) + (kk >> 4) * (N * 16) + n * 16 + (kk & 15);
      __nv_fp8_e4m3 q(sc > 0.0f ? v / sc : 0.0f);
      out[byte] = *reinterpret_cast<unsigned char *>(&q);
    } else {
      int c = k >> 5, kk = k & 31;
      long long byte = gemm_w_offset(g) * 2 + (long long)c * (32 * N * 2) + (kk >> 3) * (N * 16) + n * 16 +
                       (kk & 7) * 2;
      *reinterpret_cast<__nv_bfloat16 *>(out + byte) = __float2bfloat16_rn(v);
      *reinterpret_cast<__nv_bfloat16 *>(out + pair_w_byte(g, k, n)) = __float2bfloat16_rn(v);
    }
    return;
  }
  long long t = i - kGemmWElems;
  if (t >= kTableElems) return;
  float v = 0.0f;
  if (t < kBiasElems) {
    int g = 0;
    while (g + 1 < kNumGemm && t >= bias_offset(g + 1)) ++g;
    int n = (int)t - bias_offset(g);
    const int L = flat_idx_of_gemm(g);
    v = flat[flat_offset(L) + (long long)flat_in(L) * flat_out(L) + n];
  } else if (t < kSigmaBOff) {
    v = flat[flat_offset(8) + (t - kSigmaWOff)];
  } else if (t == kSigmaBOff) {
    v = flat[flat_offset(8) + 256];
  } else if (t >= kRgbWOff && t < kRgbBOff) {
    v = flat[flat_offset(11) + (t - kRgbWOff)];
  } else if (t >= kRgbBOff && t < kRgbBOff + 3) {
    v = flat[flat_offset(11) + 128 * 3 + (t - kRgbBOff)];
  }
  float *table = reinterpret_cast<float *>(
      out + (precision == NERFGB_PREC_FP32 ? kFp32TableOff * 4
                                            : precision == NERFGB_PREC_BF16 ? kBf16TableOff : kFp8TableOff));
  table[t] = v;
}

// FP8 per-output-channel scales: scale[g][n] = max_k |W_g[k][n]| / 448.
__global__ void fp8_scale_kernel(const float *__restrict__ flat, unsigned char *__restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kBiasElems) return;
  int g = 0;
  while (g + 1 < kNumGemm && e >= bias_offset(g + 1)) ++g;
  const int n = e - bias_offset(g), N = gemm_n(g), L = flat_idx_of_gemm(g);
  float m = 0.0f;
  for (int k = 0; k < gemm_k(g); ++k) m = fmaxf(m, fabsf(flat[flat_offset(L) + (long long)k * N + n]));
  reinterpret_cast<float *>(out + kFp8ScaleOff)[e] = m / kE4M3Max;
}

// ---------------------------------------------------------------------------
// FP32 SIMT forward
// ---------------------------------------------------------------------------
constexpr int kTM = 64;    // rows per tile
constexpr int kKC = 32;    // K rows per weight chunk
constexpr int kXLD = 320;  // X row stride (floats)
constexpr int kChunksPerTile = (64 + 256 * 4 + 320 + 256 * 3 + 288) / kKC;  // 77
constexpr size_t kFp32Smem = (size_t)(kTM * kXLD + 2 * kKC * 256) * sizeof(float);

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }

// Chunk q of the per-tile sequence -> (layer, chunk-in-layer).
__device__ __forceinline__ void chunk_of(int q, int &g, int &c) {
  g = 0;
  int base = 0;
  while (true) {
    int nch = gemm_kp(g) / kKC;
    if (q < base + nch) break;
    base += nch;
    ++g;
  }
  c = q - base;
}

__device__ __forceinline__ void load_chunk(const float *__restrict__ W, float *dst, int q, int tid) {
  int g, c;
  chunk_of(q, g, c);
  const int N = gemm_n(g);
  const float *src = W + gemm_w_offset(g) + (long long)c * kKC * N;
  const int pieces = kKC * N / 4;
  for (int p = tid; p < pieces; p += 256) cp_async16(dst + 4 * p, src + 4 * p);
}

__device__ __forceinline__ float f4c(const float4 &v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

template <int NCH>
__device__ __forceinline__ void fp32_chunk(const float *__restrict__ Xr, const float *__restrict__ Wc,
                                           int tx, float (&acc)[8][8]) {
  constexpr int N = 128 * NCH;
#pragma unroll
  for (int kk = 0; kk < kKC; kk += 4) {
    float4 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = *reinterpret_cast<const float4 *>(Xr + i * kXLD + kk);
#pragma unroll
    for (int kq = 0; kq < 4; ++kq) {
      float4 b0 = *reinterpret_cast<const float4 *>(Wc + (kk + kq) * N + tx * 4);
      float4 b1 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (NCH == 2) b1 = *reinterpret_cast<const float4 *>(Wc + (kk + kq) * N + 128 + tx * 4);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float av = f4c(a[i], kq);
        acc[i][0] = fmaf(av, b0.x, acc[i][0]);
        acc[i][1] = fmaf(av, b0.y, acc[i][1]);
        acc[i][2] = fmaf(av, b0.z, acc[i][2]);
        acc[i][3] = fmaf(av, b0.w, acc[i][3]);
        if (NCH == 2) {
          acc[i][4] = fmaf(av, b1.x, acc[i][4]);
          acc[i][5] = fmaf(av, b1.y, acc[i][5]);
          acc[i][6] = fmaf(av, b1.z, acc[i][6]);
          acc[i][7] = fmaf(av, b1.w, acc[i][7]);
        }
      }
    }
  }
}

// Copies columns [c0, c0 + nc) of the tile's X rows to acts[row][off ..].
__device__ __forceinline__ void store_cols(float *__restrict__ acts, long long row0, long long n, const float *X,
                                           int c0, int nc, int off, int tid) {
  const int per_row = nc / 4;
  for (int e = tid; e < kTM * per_row; e += 256) {
    const int r = e / per_row, q = e - r * per_row;
    if (row0 + r < n)
      *reinterpret_cast<float4 *>(acts + (row0 + r) * kActsLd + off + 4 * q) =
          *reinterpret_cast<const float4 *>(X + r * kXLD + c0 + 4 * q);
  }
}

// STORE: also write every layer's post-activation rows to `acts` (training).
// rm: optional row map (logical row k reads and writes physical row
// rm.map[k]) and device row count; not used with STORE.
template <bool STORE>
__global__ void __launch_bounds__(256, 1)
    mlp_fp32_kernel(const float *__restrict__ pk, const float *__restrict__ xyz,
                    const float *__restrict__ dirs, long long n_max, int rpd, float *__restrict__ rgb,
                    float *__restrict__ sigma, float *__restrict__ acts, RowMap rm) {
  extern __shared__ __align__(16) float sm[];
  float *X = sm;
  float *Wb = sm + kTM * kXLD;
  const float *table = pk + kFp32TableOff;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const long long n = rm.n_dev ? min((long long)*rm.n_dev, n_max) : n_max;
  const long long ntiles = (n + kTM - 1) / kTM;
  auto phys = [&](long long k) -> long long {
    return rm.map ? (long long)NG_IDX(rm.map[k], n_max, kSiteMlpRowMapFp32) : k;
  };

  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long row0 = tile * kTM;
    // First weight chunk of the tile.
    load_chunk(pk, Wb, 0, tid);
    cp_async_commit();
    // enc_xyz -> X[:, 256..319] (model.py:319-331), column 319 = 0.
    for (int e = tid; e < kTM * 33; e += 256) {
      int r = e / 33, j = e - r * 33;
      long long gr = row0 + r;
      bool valid = gr < n;
      const long long pr = valid ? phys(gr) : 0;
      float *xr = X + r * kXLD + 256;
      if (j < 3) {
        xr[j] = valid ? xyz[pr * 3 + j] : 0.0f;
      } else {
        int jj = j - 3, c = jj / 10, l = jj - c * 10;
        float xv = valid ? xyz[pr * 3 + c] : 0.0f;
        float s, co;
        sincosf(fmul(xv, enc_multiplier(l)), &s, &co);
        xr[3 + c * 20 + 2 * l] = s;
        xr[3 + c * 20 + 2 * l + 1] = co;
      }
    }
    if (tid < kTM) X[tid * kXLD + 319] = 0.0f;

    int q = 0;
    for (int g = 0; g < kNumGemm; ++g) {
      const int N = gemm_n(g);
      const int nch = gemm_kp(g) / kKC;
      const int kin = (g == 0) ? 256 : 0;
      float acc[8][8];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
      for (int c = 0; c < nch; ++c, ++q) {
        if (q + 1 < kChunksPerTile) load_chunk(pk, Wb + ((q + 1) & 1) * kKC * 256, q + 1, tid);
        cp_async_commit();
        cp_async_wait1();
        __syncthreads();
        const float *Xr = X + (ty * 8) * kXLD + kin + c * kKC;
        const float *Wc = Wb + (q & 1) * kKC * 256;
        if (N == 256)
          fp32_chunk<2>(Xr, Wc, tx, acc);
        else
          fp32_chunk<1>(Xr, Wc, tx, acc);
        __syncthreads();
      }
      // Epilogue: bias (+ReLU) into X[:, 0..N).
      const float *bias = table + bias_offset(g);
      const bool relu = gemm_relu(g);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h == 1 && N != 256) break;
        int col = h * 128 + tx * 4;
        float4 bv = *reinterpret_cast<const float4 *>(bias + col);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          float4 v = make_float4(acc[i][4 * h] + bv.x, acc[i][4 * h + 1] + bv.y, acc[i][4 * h + 2] + bv.z,
                                 acc[i][4 * h + 3] + bv.w);
          if (relu) {
            v.x = fmaxf(v.x, 0.f);
            v.y = fmaxf(v.y, 0.f);
            v.z = fmaxf(v.z, 0.f);
            v.w = fmaxf(v.w, 0.f);
          }
          *reinterpret_cast<float4 *>(X + (ty * 8 + i) * kXLD + col) = v;
        }
      }
      if (g == 8) {
        // enc_dir -> X[:, 256..287] (enc_xyz is dead after dense_5).
        for (int e = tid; e < kTM * 15; e += 256) {
          int r = e / 15, j = e - r * 15;
          long long gr = row0 + r;
          long long dr = phys(gr < n ? gr : n - 1) / rpd;
          float *xr = X + r * kXLD + 256;
          if (j < 3) {
            xr[j] = dirs[dr * 3 + j];
          } else {
            int jj = j - 3, c = jj / 4, l = jj - c * 4;
            float s, co;
            sincosf(fmul(dirs[dr * 3 + c], enc_multiplier(l)), &s, &co);
            xr[3 + c * 8 + 2 * l] = s;
            xr[3 + c * 8 + 2 * l + 1] = co;
          }
        }
        for (int e = tid; e < kTM * 5; e += 256) X[(e / 5) * kXLD + 283 + e % 5] = 0.0f;
      }
      __syncthreads();
      if (STORE) {
        store_cols(acts, row0, n, X, 0, N, acts_offset(g), tid);
        if (g == 0) store_cols(acts, row0, n, X, 256, 64, kActsEncXyz, tid);
        if (g == 8) store_cols(acts, row0, n, X, 256, 32, kActsEncDir, tid);
      }
      if (g == 7) {
        // sigma = ReLU(h7 . w + b) (model.py:374-375).
        int r = tid >> 2, part = tid & 3;
        const float *sw = table + kSigmaWOff;
        float s = 0.0f;
        for (int k = part * 64; k < part * 64 + 64; ++k) s = fmaf(X[r * kXLD + k], sw[k], s);
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (part == 0 && row0 + r < n) sigma[phys(row0 + r)] = fmaxf(s + table[kSigmaBOff], 0.0f);
        __syncthreads();
      }
    }
    // rgb = sigmoid(h9 . W + b) (model.py:386-387).
    for (int e = tid; e < kTM * 3; e += 256) {
      int r = e / 3, c = e - r * 3;
      const float *rw = table + kRgbWOff;
      float s = 0.0f;
      for (int k = 0; k < 128; ++k) s = fmaf(X[r * kXLD + k], rw[k * 3 + c], s);
      s += table[kRgbBOff + c];
      if (row0 + r < n) rgb[phys(row0 + r) * 3 + c] = 1.0f / (1.0f + expf(-s));
    }
    __syncthreads();
  }
}

}  // namespace nerfgb

using namespace nerfgb;

extern "C" long long nerfgb_mlp_param_count(void) { return kParamCount; }

extern "C" long long nerfgb_mlp_packed_bytes(int precision) {
  if (precision == NERFGB_PREC_FP32) return kFp32PackBytes;
  if (precision == NERFGB_PREC_BF16) return kBf16PackBytes;
  if (precision == NERFGB_PREC_FP8) return kFp8PackBytes;
  return -1;
}

extern "C" int nerfgb_mlp_pack(const float *params, int precision, void *packed, void *stream) {
  if (precision != NERFGB_PREC_FP32 && precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8)
    return NERFGB_E_UNSUPPORTED;
  if (!params || !packed || !aligned(packed, 256) || !aligned(params, 4)) return NERFGB_E_INVALID_ARG;
  if (precision == NERFGB_PREC_FP8) {
    fp8_scale_kernel<<<(kBiasElems + 255) / 256, 256, 0, as_stream(stream)>>>(
        params, reinterpret_cast<unsigned char *>(packed));
    if (launch_status() != NERFGB_OK) return NERFGB_E_CUDA;
  }
  long long total = kGemmWElems + kTableElems;
  pack_kernel<<<(int)((total + 255) / 256), 256, 0, as_stream(stream)>>>(
      params, precision, reinterpret_cast<unsigned char *>(packed));
  return launch_status();
}

namespace nerfgb {
int launch_mlp_fp32(const void *packed, const float *xyz, const float *dirs, long long n, int rpd,
                    float *rgb, float *sigma, cudaStream_t stream, const RowMap &rm) {
  if (cudaFuncSetAttribute(mlp_fp32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFp32Smem) !=
      cudaSuccess)
    return NERFGB_E_CUDA;
  long long ntiles = (n + kTM - 1) / kTM;
  int sms = num_sms();
  if (sms <= 0) return NERFGB_E_DEVICE;
  int grid = (int)(ntiles < sms ? ntiles : sms);
  mlp_fp32_kernel<false><<<grid, 256, kFp32Smem, stream>>>(reinterpret_cast<const float *>(packed), xyz, dirs,
                                                            n, rpd, rgb, sigma, nullptr, rm);
  return launch_status();
}

int launch_mlp_fp32_store(const void *packed, const float *xyz, const float *dirs, long long n, int rpd,
                          float *rgb, float *sigma, float *acts, cudaStream_t stream) {
  if (cudaFuncSetAttribute(mlp_fp32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFp32Smem) !=
      cudaSuccess)
    return NERFGB_E_CUDA;
  long long ntiles = (n + kTM - 1) / kTM;
  int sms = num_sms();
  if (sms <= 0) return NERFGB_E_DEVICE;
  int grid = (int)(ntiles < sms ? ntiles : sms);
  mlp_fp32_kernel<true><<<grid, 256, kFp32Smem, stream>>>(reinterpret_cast<const float *>(packed), xyz, dirs, n,
                                                           rpd, rgb, sigma, acts, RowMap());
  return launch_status();
}
}  // namespace nerfgb

extern "C" int nerfgb_mlp_forward(const void *packed, int precision, const float *xyz, const float *dirs,
                                  long long n_rows, int rows_per_dir, float *rgb, float *sigma,
                                  int *err_word, void *stream) {
  if (n_rows < 0 || rows_per_dir < 1) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8)
    return NERFGB_E_UNSUPPORTED;
  if (n_rows == 0) return NERFGB_OK;
  if (!packed || !xyz || !dirs || !rgb || !sigma || !aligned(packed, 256)) return NERFGB_E_INVALID_ARG;
  if (precision == NERFGB_PREC_FP32)
    return launch_mlp_fp32(packed, xyz, dirs, n_rows, rows_per_dir, rgb, sigma, as_stream(stream));
  if (!err_word) return NERFGB_E_INVALID_ARG;
  if (precision == NERFGB_PREC_FP8)
    return launch_mlp_fp8(packed, xyz, dirs, n_rows, rows_per_dir, rgb, sigma, err_word, as_stream(stream));
  return launch_mlp_bf16(packed, xyz, dirs, n_rows, rows_per_dir, rgb, sigma, err_word, as_stream(stream));
}

extern "C" int nerfgb_mlp_forward_wait_test(const void *packed, int precision, const float *xyz, const float *dirs,
                                            long long n_rows, int rows_per_dir, float *rgb, float *sigma,
                                            int *err_word, unsigned long long wait_ns, long long withhold_chunk,
                                            void *stream) {
  if (n_rows < 0 || rows_per_dir < 1) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8) return NERFGB_E_UNSUPPORTED;
  if (wait_ns < 1000ull || wait_ns > 10000000000ull) return NERFGB_E_INVALID_ARG;
  if (n_rows == 0) return NERFGB_OK;
  if (!packed || !xyz || !dirs || !rgb || !sigma || !err_word || !aligned(packed, 256)) return NERFGB_E_INVALID_ARG;
  return launch_mlp_wait_test(packed, precision == NERFGB_PREC_FP8, xyz, dirs, n_rows, rows_per_dir, rgb, sigma,
                              err_word, as_stream(stream), wait_ns, withhold_chunk);
}

extern "C" int nerfgb_mlp_forward_mapped(const void *packed, int precision, const float *xyz, const float *dirs,
                                         long long n_rows_max, int rows_per_dir, const int *row_map,
                                         const int *n_rows_dev, float *rgb, float *sigma, int *err_word,
                                         void *stream) {
  if (n_rows_max < 0 || rows_per_dir < 1) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && precision != NERFGB_PREC_BF16 && precision != NERFGB_PREC_FP8)
    return NERFGB_E_UNSUPPORTED;
  if (n_rows_max == 0) return NERFGB_OK;
  if (!packed || !xyz || !dirs || !rgb || !sigma || !aligned(packed, 256)) return NERFGB_E_INVALID_ARG;
  if (precision != NERFGB_PREC_FP32 && !err_word) return NERFGB_E_INVALID_ARG;
  RowMap rm;
  rm.map = row_map;
  rm.n_dev = n_rows_dev;
  return launch_mlp(packed, precision, xyz, dirs, n_rows_max, rows_per_dir, rgb, sigma, err_word,
                    as_stream(stream), rm);
}

#ifdef NERF_BOUNDS_CHECK
namespace nerfgb {
NG_BOUNDS_READER(bounds_read_mlp)
}  // namespace nerfgb
#endif
