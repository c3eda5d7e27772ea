// Shared definitions of libnerfgb: parameter layouts, exact-rounding float
// helpers, Philox4x32-10, argument checks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "nerfgb.h"

namespace nerfgb {

// ---------------------------------------------------------------------------
// Network shape (nerf/core/model.py:334-394). GEMM layers in execution order:
// dense_0..dense_7, dense_8, dense_9. K is padded to a multiple of 32 with
// zero rows: dense_0 63->64, dense_5 319->320 ([h | enc_xyz]), dense_9
// 283->288 ([bottleneck | enc_dir]).
// ---------------------------------------------------------------------------
constexpr int kNumGemm = 10;
#define NG_HD __host__ __device__ __forceinline__ constexpr
NG_HD int gemm_k(int g) { return g == 0 ? 63 : g == 5 ? 319 : g == 9 ? 283 : 256; }
NG_HD int gemm_kp(int g) { return g == 0 ? 64 : g == 5 ? 320 : g == 9 ? 288 : 256; }
NG_HD int gemm_n(int g) { return g == 9 ? 128 : 256; }
NG_HD bool gemm_relu(int g) { return g != 8; }  // dense_8 (model.py:377-378) is linear
constexpr int kW = 256;          // hidden width
constexpr int kEncXyz = 63;      // 3 + 3*2*10
constexpr int kEncDir = 27;      // 3 + 3*2*4

// Flat blob (nerfgb_mlp_param_count): Keras order dense_0..7, sigma, dense_8,
// dense_9, rgb; per layer kernel [in,out] row-major then bias [out].
// GEMM layer g sits at flat index flat_idx_of_gemm(g).
NG_HD int flat_idx_of_gemm(int g) { return g < 8 ? g : g + 1; }
NG_HD int flat_in(int l) { return l == 0 ? 63 : l == 5 ? 319 : l == 10 ? 283 : l == 11 ? 128 : 256; }
NG_HD int flat_out(int l) { return l == 8 ? 1 : l == 10 ? 128 : l == 11 ? 3 : 256; }

NG_HD long long flat_offset(int layer) {
  long long off = 0;
  for (int i = 0; i < layer; ++i) off += (long long)flat_in(i) * flat_out(i) + flat_out(i);
  return off;
}
constexpr long long kParamCount = flat_offset(12);  // 595,844

// Padded GEMM weights: offset (elements) of layer g's [Kp][N] block.
NG_HD long long gemm_w_offset(int g) {
  long long off = 0;
  for (int i = 0; i < g; ++i) off += (long long)gemm_kp(i) * gemm_n(i);
  return off;
}
constexpr long long kGemmWElems = gemm_w_offset(kNumGemm);  // 593,920

// FP32 side tables shared by both packs (float offsets inside the table).
NG_HD int bias_offset(int g) {
  int off = 0;
  for (int i = 0; i < g; ++i) off += gemm_n(i);
  return off;
}
constexpr int kBiasElems = bias_offset(kNumGemm);     // 2,432
constexpr int kSigmaWOff = kBiasElems;                // [256]
constexpr int kSigmaBOff = kSigmaWOff + 256;          // [1] (+3 pad)
constexpr int kRgbWOff = kSigmaBOff + 4;              // [128][3]
constexpr int kRgbBOff = kRgbWOff + 128 * 3;          // [3] (+1 pad)
constexpr int kTableElems = kRgbBOff + 4;

// FP32 pack: padded W blocks [Kp][N] fp32, then the table.
constexpr long long kFp32TableOff = kGemmWElems;  // floats
constexpr long long kFp32PackBytes = (kGemmWElems + kTableElems) * 4;

// BF16 pack: per GEMM layer, K chunks of 32; chunk (n, k) byte offset
// (k/8)*(N*16) + n*16 + (k%8)*2 (K-major core matrices, no swizzle). Then
// the fp32 table at a 1 KB aligned offset, then the same weights in the
// CTA-pair layout (pair_w_byte).
constexpr long long kBf16WBytes = kGemmWElems * 2;
constexpr long long kBf16TableOff = (kBf16WBytes + 1023) / 1024 * 1024;  // bytes

// CTA-pair layout, for the 2-SM MMA in which each CTA of a pair holds one
// N-half of every weight chunk: per GEMM layer, chunks of kPairKch K-rows
// (the last may be shorter, kc rows); per chunk N-half 0 then N-half 1, each
// (k/8)*(N/2*16) + n'*16 + (k%8)*2 with n' = n mod N/2, so that a CTA's half
// of a chunk is one contiguous copy.
constexpr int kPairKch = 64;
constexpr long long kBf16PairOff = (kBf16TableOff + (long long)kTableElems * 4 + 1023) / 1024 * 1024;
constexpr long long kBf16PackBytes = kBf16PairOff + kBf16WBytes;
NG_HD long long pair_w_byte(int g, int k, int n) {
  const int N = gemm_n(g), H = N / 2, c = k / kPairKch, kk = k % kPairKch;
  const int kc = gemm_kp(g) - c * kPairKch < kPairKch ? gemm_kp(g) - c * kPairKch : kPairKch;
  return kBf16PairOff + gemm_w_offset(g) * 2 + (long long)c * (kPairKch * N * 2) + (long long)(n / H) * (kc * H * 2) +
         (kk / 8) * (H * 16) + (n % H) * 16 + (kk % 8) * 2;
}

// Stored activations of one row for training (floats): enc_xyz [64] | h0..h7
// [8 x 256] | bottleneck [256] | enc_dir [32] | h9 [128].
constexpr int kActsEncXyz = 0;
constexpr int kActsEncDir = 64 + 9 * 256;     // 2368
constexpr int kActsLd = kActsEncDir + 32 + 128;  // 2528
NG_HD int acts_offset(int g) { return g < 9 ? 64 + 256 * g : kActsEncDir + 32; }

// FP8 pack: the same chunks as BF16 with one byte per weight, e4m3 of
// W[k][n] / scale[n] (per output channel, scale = max_k |W[k][n]| / 448);
// core matrices hold 16 K-elements: chunk (n, k) byte offset
// (k/16)*(N*16) + n*16 + (k%16). Then the FP32 table, then the scales
// [kBiasElems] (same indexing as the biases).
constexpr long long kFp8WBytes = kGemmWElems;
constexpr long long kFp8TableOff = (kFp8WBytes + 1023) / 1024 * 1024;  // bytes
constexpr long long kFp8ScaleOff = kFp8TableOff + (long long)kTableElems * 4;
constexpr long long kFp8PackBytes = kFp8ScaleOff + (long long)kBiasElems * 4;
constexpr float kE4M3Max = 448.0f;

// ---------------------------------------------------------------------------
// Correctly rounded fp32 arithmetic, never fused into FMA. The reference's
// TensorFlow ops are separate elementwise kernels, so each step rounds.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// fp32(2^l) * fp32(pi): PositionalEncoder multipliers (model.py:309-311).
__device__ __forceinline__ float enc_multiplier(int l) {
  return fmul((float)(1u << l), 3.14159265358979323846f);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As
// Easy as 1, 2, 3", SC 2011): multipliers and Weyl key increments as
// published there.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 ctr, uint2 key) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
    uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
    ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
    key.x += W0;
    key.y += W1;
  }
  return ctr;
}

// Top 24 bits scaled to [0, 1).
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Uniform for flat element index e of the stream keyed by seed.
// Word e of the stream keyed by seed: output (e mod 4) of counter (e div 4).
__device__ __forceinline__ uint32_t philox_word(unsigned long long seed, unsigned long long e) {
  unsigned long long c = e >> 2;
  uint4 r = philox4x32_10(make_uint4((uint32_t)c, (uint32_t)(c >> 32), 0u, 0u),
                          make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  return (e & 3) == 0 ? r.x : (e & 3) == 1 ? r.y : (e & 3) == 2 ? r.z : r.w;
}

__device__ __forceinline__ float philox_uniform(unsigned long long seed, unsigned long long e) {
  return u01(philox_word(seed, e));
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NERFGB_OK : NERFGB_E_CUDA;
}

inline int num_sms() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return n;
}

inline bool aligned(const void *p, unsigned a) { return ((uintptr_t)p % a) == 0; }

// ---------------------------------------------------------------------------
// Bounds-check build (-DNERF_BOUNDS_CHECK): every index computed from data
// (searchsorted results, sort ranks, sort permutations, gate row maps and
// counts, MLP row maps) goes through NG_IDX(i, n, site). Out of [0, n) the
// first failing site's code is recorded in this translation unit's device
// word and the index is clamped to 0, so that the access stays in bounds;
// nerfgb_bounds_check_status() reads and clears the words. Without the flag
// NG_IDX(i, n, site) is i.
// ---------------------------------------------------------------------------
#ifdef NERF_BOUNDS_CHECK
static __device__ int g_bounds_err;  // one per translation unit
__device__ __forceinline__ long long ng_checked(long long i, long long n, int site) {
  if (i < 0 || i >= n) {
    atomicCAS(&g_bounds_err, 0, site);
    return 0;
  }
  return i;
}
#define NG_IDX(i, n, site) ::nerfgb::ng_checked((long long)(i), (long long)(n), (site))
// Reads (and with reset, clears) this translation unit's error word.
#define NG_BOUNDS_READER(fn)                                                         \
  int fn(int reset) {                                                                \
    int v = 0;                                                                       \
    if (cudaMemcpyFromSymbol(&v, g_bounds_err, sizeof(int)) != cudaSuccess) return -1; \
    if (reset) {                                                                     \
      const int z = 0;                                                               \
      if (cudaMemcpyToSymbol(g_bounds_err, &z, sizeof(int)) != cudaSuccess) return -1; \
    }                                                                                \
    return v;                                                                        \
  }
#else
#define NG_IDX(i, n, site) (i)
#endif

// Site codes of NG_IDX (reported by nerfgb_bounds_check_status).
enum BoundsSite {
  kSiteFinePiece = 1,     // fine sampler: searchsorted bin of a draw
  kSiteSortCoarse = 2,    // fine sampler: merged position of a coarse depth
  kSiteSortFine = 3,      // fine sampler: merged position of a fine draw
  kSiteSortRank = 4,      // fine sampler: rank-sort position
  kSiteGateCoarse = 5,    // coarse gate: row-map slot
  kSiteGateFinePerm = 6,  // fine gate: sort permutation entry
  kSiteGateFine = 7,      // fine gate: row-map slot
  kSiteMlpRowMap = 8,     // MLP: physical row of a row-map entry (tensor-core kernels)
  kSiteMlpRowMapFp32 = 9,  // MLP: physical row of a row-map entry (FP32 kernel)
  kSiteGateFinePiece = 10  // fine gate: coarse bin of a fine draw
};

}  // namespace nerfgb
