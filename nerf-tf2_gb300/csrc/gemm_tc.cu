// Tensor-core BF16 GEMMs of the MLP backward (the gradient tf.GradientTape
// takes at nerf/core/model.py:148-170 through the Dense layers of
// model.py:366-387), FP32 accumulation in TMEM:
//
//   C[M][N] = sum_k A[m][k] B[n][k]        (tcgen05.mma.cta_group::1.kind::f16)
//
// The streamed operands come from row-major global memory by tensor copies
// (TMA) in the 128-byte swizzled layout, so that the copy engine fetches
// whole 128-byte rows (boxes whose innermost extent is 16 bytes cost one
// request per 16 bytes and held these kernels near 4 TB/s):
//   K-major A (the reduction along the row, dX's dZ): 2-D boxes of 64
//            columns by 128 rows, row r at r*128 bytes (smem_desc_sw128);
//   MN-major A and B (the reduction along the rows, dW's In and dZ): 3-D
//            boxes of 64-element atoms by kKc rows by the atoms of the tile,
//            atom a at a*8 KB, row k at k*128 bytes (smem_desc_mn_sw128,
//            the instruction descriptor's transpose bit set);
// rows and atoms past the bounds are zero-filled, and within every 1024-byte
// block the 16-byte chunks of row k sit permuted by k % 8, as the swizzled
// descriptors read them. dX's resident B (W) is copied once by cp.async in
// the no-swizzle core-matrix layout (8 rows x 16 bytes; K-major, LBO = the
// stride between 8-column groups, SBO = 128).
// The backward uses:
//   dX = dZ W^T   A = dZ [rows][n_out] (K-major), B = W [k_in][n_out]
//                 (K-major, resident), C = dX [rows][k_in] stored as BF16;
//   dW = In^T dZ  A = In [rows][k_in] (MN-major: M = k_in), B = dZ
//                 [rows][n_out] (MN-major: N = n_out), reduced over rows in
//                 splits; each split's FP32 partial goes to a workspace and a
//                 reduction kernel adds the splits into the gradient blob.
//
// Warp roles (9 warps): 0-3 epilogue (TMEM lane quadrant = warp), 4-7
// loaders (warp 4's first lane issues the tensor copies of an NST-stage
// ring, full/empty mbarriers; all four warps copy a resident B once with
// cp.async), 8 TMEM allocation and the MMA issuer (one thread). Work items (an M tile, a split
// of K) are taken persistently: item = blockIdx.x + i * gridDim.x. With one
// 128-row M tile per item the accumulator is double-buffered in TMEM, so an
// item's epilogue overlaps the next item's MMAs.
//
// Every mbarrier wait is bounded (tc::wait_bar): on a timeout the kernel
// writes NERFGB_E_TIMEOUT to *err, every role stops, loaders drain their
// copies, the issuer drains its MMAs, TMEM is freed and the kernel returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"
#include "mlp_internal.cuh"
#include "tcgen05.cuh"

namespace nerfgb {
namespace gemm {

using namespace tc;

constexpr int kKc = 64;                    // K per stage (4 MMAs of K = 16)
constexpr int kEpiWarps = 4;
constexpr int kLoadWarps = 4;
constexpr int kLoadThreads = kLoadWarps * 32;
constexpr int kIssuerWarp = kEpiWarps + kLoadWarps;
constexpr int kThreads = (kIssuerWarp + 1) * 32;  // 288
constexpr uint32_t kPad = 16;              // bytes added to a group stride (bank spread of the copies)

enum Epi { kEpiBf16 = 0, kEpiF32 = 1 };

// Tensor maps of the streamed operands (A, and B unless resident).
struct Maps {
  CUtensorMap a, b;
};

struct Args {
  const __nv_bfloat16 *A;  // K-major: [M][K] row stride lda; MN-major: [K][M] row stride lda
  const __nv_bfloat16 *B;  // K-major: [N][K] row stride ldb; MN-major: [K][N] row stride ldb
  long long lda, ldb;
  long long M, N, K;       // N = the MMA's N (128 or 256); M and N rows past the operand bounds read 0
  long long m_valid;       // rows of C written
  long long k_split;       // K per work item (a multiple of kKc)
  int m_tiles, k_splits;
  void *C;                 // kEpiBf16: bf16 [M][ldc]; kEpiF32: float [k_splits][m_tiles * MT * 128][ldc]
  long long ldc;
  int *err;
};

// Stage geometry for MT 128-row M tiles per item. B_RES: B (K-major, all of
// K <= 256) is loaded once per CTA into its own region after the ring and
// the stages hold A alone.
template <bool A_MN, bool B_MN, int MT, bool B_RES = false>
struct Geo {
  // bytes per 8 columns of a streamed stage (A; B streamed MN-major), which
  // size the stages; the resident B's group stride (padded for the
  // cp.async copies' banks)
  static constexpr uint32_t kSA = A_MN ? kKc * 16 : MT * 128 * 16;
  static constexpr uint32_t kSB = B_MN ? kKc * 16 : 256 * 16 + kPad;
  static constexpr uint32_t kABytes = A_MN ? (MT * 128 / 8) * kSA : (kKc / 8) * kSA;
  static constexpr uint32_t kBBytes = B_RES ? 0 : B_MN ? (256 / 8) * kSB : (kKc / 8) * kSB;
  static constexpr uint32_t kStage = (kABytes + kBBytes + 127) / 128 * 128;
  static constexpr int kNst = B_RES ? 4 : MT == 1 ? 4 : 3;
  static constexpr uint32_t kRing = kNst * kStage;
  static constexpr uint32_t kBRes = kRing;                               // resident B: 32 column groups
  static constexpr uint32_t kBar0 = kRing + (B_RES ? 32 * kSB : 0);
  static constexpr uint32_t kBarFull = kBar0;            // [kNst]
  static constexpr uint32_t kBarEmpty = kBar0 + 64;      // [kNst]
  static constexpr uint32_t kBarAcc = kBar0 + 128;       // [2]
  static constexpr uint32_t kBarTmem = kBar0 + 144;      // [2]
  static constexpr uint32_t kBarDrain = kBar0 + 160;
  static constexpr uint32_t kBarB = kBar0 + 168;
  static constexpr uint32_t kTmemSlot = kBar0 + 176;
  static constexpr uint32_t kAbort = kBar0 + 184;        // int, then the wait limit (u64) at +8
  static constexpr uint32_t kSmem = kBar0 + 200;
  static constexpr int kBufs = MT == 1 ? 2 : 1;          // TMEM accumulators (256 columns per 128-row tile)
  static_assert(kNst <= 8 && kSmem <= 227 * 1024, "ring");
  static_assert(!B_RES || (!B_MN && MT == 1), "resident B: K-major, one M tile");
};

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One box of a 3-D tensor map into shared memory at dst, completing on the
// mbarrier bar (coordinates innermost first).
__device__ __forceinline__ void tma_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

// One box of a 2-D tensor map (coordinates innermost first).
__device__ __forceinline__ void tma_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// Descriptor of a K-major operand in the 128-byte swizzled layout: rows of
// 64 BF16 (128 bytes) at a 128-byte pitch, each 1024-byte block of 8 rows
// with its 16-byte chunks permuted by the row (as the 128-byte-swizzle
// tensor copy writes them; the block must start 1024-byte aligned). SBO =
// 1024 (between 8-row blocks), LBO unused, swizzle mode 2 (bits 61-63); a
// K step of 16 elements advances the start address by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// Descriptor of an MN-major operand in the 128-byte swizzled layout: atoms
// of 64 MN-elements (128-byte rows, one per K row), 64 K rows each (8 KB),
// each 1024-byte block of 8 K rows with its 16-byte chunks permuted by the
// row (as the 128-byte-swizzle tensor copy of a box of 64 elements x 64
// rows x atoms writes them; blocks 1024-byte aligned). LBO = 8192 (between
// MN atoms), SBO = 1024 (between 8-row K blocks), swizzle mode 2; a K step
// of 16 rows advances the start address by 2048 bytes.
__device__ __forceinline__ uint64_t smem_desc_mn_sw128(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(8192u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
         (1ull << 46) | (2ull << 61);
}

template <bool A_MN, bool B_MN, int MT, int EPI, bool B_RES = false>
__global__ void __launch_bounds__(kThreads, 1) gemm_kernel(Args a, const __grid_constant__ Maps maps) {
  using G = Geo<A_MN, B_MN, MT, B_RES>;
  static_assert(A_MN || (MT == 1 && G::kABytes == 128u * 128u && G::kStage % 1024u == 0),
                "a K-major A is one 128-row tile of 128-byte swizzled rows per stage");
  extern __shared__ __align__(1024) uint8_t smem[];
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + G::kAbort);
  const long long items = (long long)a.m_tiles * a.k_splits;
  constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((A_MN ? 1u : 0u) << 15) |
                              ((B_MN ? 1u : 0u) << 16) | ((128u >> 4) << 24);
  const uint32_t idesc = kIdesc | ((uint32_t)(a.N >> 3) << 17);
  // Chunks of item it: [k_begin, k_end) in steps of kKc.
  auto item_range = [&](long long it, long long &mt, long long &kb, long long &ke) {
    mt = it % a.m_tiles;
    const long long ks = it / a.m_tiles;
    kb = ks * a.k_split;
    ke = kb + a.k_split < a.K ? kb + a.k_split : a.K;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < G::kNst; ++s) {
      mbar_init(sbase + G::kBarFull + 8 * s, 1);  // the copying thread's arrive, then the bytes
      mbar_init(sbase + G::kBarEmpty + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(sbase + G::kBarAcc + 8 * b, 1);
      mbar_init(sbase + G::kBarTmem + 8 * b, kEpiWarps);
    }
    mbar_init(sbase + G::kBarDrain, 1);
    mbar_init(sbase + G::kBarB, kLoadThreads);
    *abort_flag = 0;
    set_wait_limit(abort_flag, kWaitNs);
    if ((sbase & 1023u) != 0) {
      // the swizzled stages need 1024-byte alignment: nothing is copied
      atomicExch(a.err, NERFGB_E_UNSUPPORTED);
      *abort_flag = 1;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kIssuerWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + G::kTmemSlot),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(smem + G::kTmemSlot);

  if (warp >= kEpiWarps && warp < kIssuerWarp) {
    // ---------------- loaders ----------------
    const int t = threadIdx.x - kEpiWarps * 32;
    if (B_RES) {
      // all of B (K <= 256 columns): piece (n, 8-column group g) -> g*SB + n*16
      const int ng = (int)((a.K + 7) / 8);
      for (int p = t; p < 256 * ng; p += kLoadThreads) {
        const int g = p % ng, n = p / ng;
        const bool ok = n < a.N;
        cp_async16(sbase + G::kBRes + (uint32_t)g * G::kSB + (uint32_t)n * 16u,
                   ok ? a.B + (long long)n * a.ldb + 8 * g : a.B, ok ? 16u : 0u);
      }
      cp_async_commit();
      cp_async_wait<0>();
      fence_proxy_async();
      mbar_arrive(sbase + G::kBarB);
    }
    if (t == 0) {
      // One thread issues each stage's tensor copies: A (MT*128 rows or
      // kKc rows of MN-major groups) and a streamed B; the stage completes
      // on their bytes.
      constexpr uint32_t kBytes = G::kABytes + G::kBBytes;
      long long q = 0;
      bool ok = true;
      for (long long it = blockIdx.x; it < items && ok; it += gridDim.x) {
        long long mt, kb, ke;
        item_range(it, mt, kb, ke);
        const int m0 = (int)(mt * MT * 128);
        for (long long k0 = kb; k0 < ke; k0 += kKc, ++q) {
          const int st = (int)(q % G::kNst);
          const uint32_t ph = (uint32_t)((q / G::kNst) & 1);
          if (!wait_bar(sbase + G::kBarEmpty + 8 * st, ph ^ 1u, abort_flag, a.err)) {
            ok = false;
            break;
          }
          if (*abort_flag) {
            ok = false;
            break;
          }
          const uint32_t full = sbase + G::kBarFull + 8 * st, sa = sbase + st * G::kStage;
          mbar_expect_tx(full, kBytes);
          // MN-major: rows = the reduction (k0 ..), groups = M columns (m0 / 8 ..);
          // K-major: rows = M (m0 ..), groups = the reduction columns (k0 / 8 ..)
          if (A_MN)
            tma_3d(sa, &maps.a, 0, (int)k0, m0 / 64, full);  // 64-element atoms x kKc rows, swizzled
          else
            tma_2d(sa, &maps.a, (int)k0, m0, full);  // 64 columns x 128 rows, 128-byte swizzle
          if (!B_RES) tma_3d(sa + G::kABytes, &maps.b, 0, (int)k0, 0, full);
        }
      }
      if (!ok) {
        // Drain: wait (bounded) for the copies of the stages still in flight.
        const uint64_t t0 = globaltimer();
        for (long long d = q > G::kNst ? q - G::kNst : 0; d < q; ++d)
          while (!mbar_try(sbase + G::kBarFull + 8 * (int)(d % G::kNst), (uint32_t)((d / G::kNst) & 1)) &&
                 globaltimer() - t0 < 10000000ull) {
          }
      }
    }
  } else if (warp == kIssuerWarp) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      long long q = 0, n_items = 0;
      bool issued = false;
      if (B_RES) {
        if (wait_bar(sbase + G::kBarB, 0, abort_flag, a.err)) tc_fence_after();
      }
      for (long long it = blockIdx.x; it < items; it += gridDim.x, ++n_items) {
        if (*abort_flag) break;
        long long mt, kb, ke;
        item_range(it, mt, kb, ke);
        const int b = G::kBufs == 2 ? (int)(n_items & 1) : 0;
        if (n_items >= G::kBufs) {
          // the epilogue has read this buffer's previous accumulator
          const uint32_t ph = (uint32_t)(((n_items - G::kBufs) / G::kBufs) & 1);
          if (!wait_bar(sbase + G::kBarTmem + 8 * b, ph, abort_flag, a.err)) break;
          tc_fence_after();
        }
        const uint32_t d0 = tmem + (uint32_t)(b * MT) * 256u;
        bool first = true;
        for (long long k0 = kb; k0 < ke; k0 += kKc, ++q) {
          const int st = (int)(q % G::kNst);
          if (!wait_bar(sbase + G::kBarFull + 8 * st, (uint32_t)((q / G::kNst) & 1), abort_flag, a.err)) break;
          tc_fence_after();
          const uint32_t sa = (sbase + st * G::kStage) & 0x3FFFFu;
          // resident B: this chunk's column groups start at k0 / 8
          const uint32_t sb = B_RES ? ((sbase + G::kBRes) & 0x3FFFFu) + (uint32_t)(k0 / 8) * G::kSB
                                    : sa + G::kABytes;
#pragma unroll
          for (int s = 0; s < kKc / 16; ++s) {
            // B: K-major k-step s = 2 column groups (2s * SB); MN-major = 2 row groups (2s * 128)
            const uint64_t bdesc =
                B_MN ? smem_desc_mn_sw128(sb + 2048u * s) : smem_desc(sb + 2u * s * G::kSB, G::kSB, 128u);
#pragma unroll
            for (int h = 0; h < MT; ++h) {
              const uint64_t adesc = A_MN ? smem_desc_mn_sw128(sa + (uint32_t)h * 16384u + 2048u * s)
                                          : smem_desc_sw128(sa + 32u * s);
              tc_mma(d0 + (uint32_t)h * 256u, adesc, bdesc, idesc, (first && s == 0) ? 0u : 1u);
            }
          }
          first = false;
          issued = true;
          tc_commit(sbase + G::kBarEmpty + 8 * st);
        }
        if (*abort_flag) break;
        tc_commit(sbase + G::kBarAcc + 8 * b);
      }
      if (issued) {
        tc_commit(sbase + G::kBarDrain);
        const uint64_t t0 = globaltimer();
        while (!mbar_try(sbase + G::kBarDrain, 0) && globaltimer() - t0 < 100000000ull) {
        }
      }
    }
  } else {
    // ---------------- epilogue ----------------
    long long n_items = 0;
    for (long long it = blockIdx.x; it < items; it += gridDim.x, ++n_items) {
      long long mt, kb, ke;
      item_range(it, mt, kb, ke);
      const int b = G::kBufs == 2 ? (int)(n_items & 1) : 0;
      const uint32_t ph = (uint32_t)((n_items / G::kBufs) & 1);
      if (!__all_sync(0xffffffffu, wait_bar(sbase + G::kBarAcc + 8 * b, ph, abort_flag, a.err))) break;
      tc_fence_after();
      const long long ks = it / a.m_tiles;
#pragma unroll 1
      for (int h = 0; h < MT; ++h) {
        const long long r = mt * MT * 128 + h * 128 + 32 * warp + lane;  // row of C (= TMEM lane)
        const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(b * MT + h) * 256u;
#pragma unroll 1
        for (int j = 0; j < (int)(a.N / 32); ++j) {
          uint32_t raw[32];
          tmem_ld32(tl + 32u * j, raw);
          tmem_wait32(raw);
          if (EPI == kEpiBf16) {
            if (r < a.m_valid) {
              uint4 *dst = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(a.C) + r * a.ldc + 32 * j);
#pragma unroll
              for (int q4 = 0; q4 < 4; ++q4)
                dst[q4] = make_uint4(pack_bf16(__uint_as_float(raw[8 * q4]), __uint_as_float(raw[8 * q4 + 1])),
                                     pack_bf16(__uint_as_float(raw[8 * q4 + 2]), __uint_as_float(raw[8 * q4 + 3])),
                                     pack_bf16(__uint_as_float(raw[8 * q4 + 4]), __uint_as_float(raw[8 * q4 + 5])),
                                     pack_bf16(__uint_as_float(raw[8 * q4 + 6]), __uint_as_float(raw[8 * q4 + 7])));
            }
          } else {
            // this split's partial (every row of the tile; the reduction reads the valid ones)
            float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float *>(a.C) +
                                                     (ks * a.m_tiles * MT * 128 + r) * a.ldc + 32 * j);
#pragma unroll
            for (int q4 = 0; q4 < 8; ++q4)
              dst[q4] = make_float4(__uint_as_float(raw[4 * q4]), __uint_as_float(raw[4 * q4 + 1]),
                                    __uint_as_float(raw[4 * q4 + 2]), __uint_as_float(raw[4 * q4 + 3]));
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(sbase + G::kBarTmem + 8 * b);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == kIssuerWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

// grads[r][c] += sum_s part[s][r][c] for r < rows, c < cols (part row stride
// ld, split stride split_rows * ld); grads row stride gld. A block takes 64
// elements; its four warp pairs sum the splits s = g, g + 4, ... (g = the
// pair) in order, and the four sums are added in order: the same result
// whatever the launch.
constexpr int kRedElems = 64, kRedGroups = 4;
__global__ void __launch_bounds__(kRedElems *kRedGroups)
    reduce_splits_kernel(const float *__restrict__ part, int splits, long long split_rows, int ld, int rows, int cols,
                         float *__restrict__ grads, int gld) {
  __shared__ float sums[kRedGroups][kRedElems];
  const int t = threadIdx.x % kRedElems, grp = threadIdx.x / kRedElems;
  const long long e = (long long)blockIdx.x * kRedElems + t;
  const bool ok = e < (long long)rows * cols;
  const int r = ok ? (int)(e / cols) : 0, c = ok ? (int)(e % cols) : 0;
  float s = 0.0f;
  if (ok)
    for (int k = grp; k < splits; k += kRedGroups) s += part[(k * split_rows + r) * ld + c];
  sums[grp][t] = s;
  __syncthreads();
  if (grp == 0 && ok) grads[(long long)r * gld + c] += ((sums[0][t] + sums[1][t]) + sums[2][t]) + sums[3][t];
}

// An MN-major operand [rows][cols] (cols contiguous, row stride ld) as 3-D
// (64 elements, rows, 64-element atoms; strides 2 B, ld * 2, 128 B) with the
// 128-byte swizzle: boxes of kKc rows by box_atoms atoms (atoms past the
// bounds zero-filled) land as smem_desc_mn_sw128 reads them.
static int operand_map_mn_sw128(CUtensorMap *m, const __nv_bfloat16 *X, long long ld, long long rows, long long atoms,
                                unsigned box_atoms) {
  if (reinterpret_cast<uintptr_t>(X) % 16 != 0 || (ld * 2) % 16 != 0 || atoms < 1) return NERFGB_E_INVALID_ARG;
  const unsigned long long dims[3] = {64, (unsigned long long)rows, (unsigned long long)atoms};
  const unsigned long long strides[2] = {(unsigned long long)(ld * 2), 128};
  const unsigned box[3] = {64, kKc, box_atoms};
  return encode_tensor_map_u16(m, X, 3, dims, strides, box, true);
}

template <bool A_MN, bool B_MN, int MT, int EPI, bool B_RES = false>
static int launch(const Args &a, cudaStream_t st) {
  using G = Geo<A_MN, B_MN, MT, B_RES>;
  auto kern = gemm_kernel<A_MN, B_MN, MT, EPI, B_RES>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kSmem) != cudaSuccess)
    return NERFGB_E_CUDA;
  const int sms = num_sms();
  if (sms <= 0) return NERFGB_E_DEVICE;
  const long long items = (long long)a.m_tiles * a.k_splits;
  if (items == 0) return NERFGB_OK;
  const int grid = (int)(items < sms ? items : sms);
  Maps maps{};
  int rc;
  // A: MN-major [K rows][M cols] in kKc-row boxes of all MT*128 columns;
  // K-major [M rows][K cols] in 128-row boxes of kKc columns
  if (A_MN) {
    rc = operand_map_mn_sw128(&maps.a, a.A, a.lda, a.K, a.M / 64, MT * 128 / 64);
  } else {
    // K-major [M rows][K cols]: boxes of kKc columns (128 bytes) by 128 rows,
    // 128-byte swizzle (one TMA row request per 128 bytes)
    if (reinterpret_cast<uintptr_t>(a.A) % 16 != 0 || (a.lda * 2) % 16 != 0) return NERFGB_E_INVALID_ARG;
    const unsigned long long dims[2] = {(unsigned long long)a.K, (unsigned long long)a.M};
    const unsigned long long strides[1] = {(unsigned long long)(a.lda * 2)};
    const unsigned box[2] = {kKc, 128};
    rc = encode_tensor_map_u16(&maps.a, a.A, 2, dims, strides, box, true);
  }
  if (rc != NERFGB_OK) return rc;
  if (!B_RES) {
    static_assert(B_RES || B_MN, "a streamed B is MN-major");
    // [K rows][N cols] in kKc-row boxes of 256 columns (past N: zeros)
    if ((rc = operand_map_mn_sw128(&maps.b, a.B, a.ldb, a.K, a.N / 64, 256 / 64)) != NERFGB_OK) return rc;
  }
  kern<<<grid, kThreads, G::kSmem, st>>>(a, maps);
  return launch_status();
}

}  // namespace gemm

// dX [M][256] (BF16, row stride 256) = dZ [M][n_out] (BF16, row stride 256)
// times W^T, W = the layer's BF16 weights [k_in][n_out] (rows 0..255 used).
int launch_gemm_dx(const __nv_bfloat16 *dz, long long M, int n_out, const __nv_bfloat16 *W, __nv_bfloat16 *dx,
                   int *err, cudaStream_t st) {
  gemm::Args a{};
  a.A = dz;
  a.lda = 256;
  a.B = W;
  a.ldb = n_out;
  a.M = M;
  a.N = 256;
  a.K = n_out;
  a.m_valid = M;
  a.k_split = ((n_out + gemm::kKc - 1) / gemm::kKc) * gemm::kKc;
  a.m_tiles = (int)((M + 127) / 128);
  a.k_splits = 1;
  a.C = dx;
  a.ldc = 256;
  a.err = err;
  // W^T (at most 256 x 256 BF16) stays in shared memory for the whole launch
  return gemm::launch<false, false, 1, gemm::kEpiBf16, true>(a, st);
}

// Rows of split partials the dW GEMM writes for M rows (workspace sizing).
long long gemm_dw_partial_floats(int splits) { return (long long)splits * 256 * 256; }

// grads (row stride n_out) [k][n] += sum_m In[m][k] dZ[m][n] for k < k_in
// (In: BF16, row stride ld_in; k_in <= 256: 128 or 256-row M tiles), with
// `splits` partial sums in `part` (gemm_dw_partial_floats(splits) floats).
int launch_gemm_dw(const __nv_bfloat16 *in, long long ld_in, int k_in, const __nv_bfloat16 *dz, int n_out,
                   long long M, float *grads, float *part, int splits, int *err, cudaStream_t st) {
  if (k_in < 1 || k_in > 256 || (n_out != 128 && n_out != 256) || splits < 1) return NERFGB_E_UNSUPPORTED;
  gemm::Args a{};
  a.A = in;
  a.lda = ld_in;
  a.B = dz;
  a.ldb = 256;
  a.M = k_in <= 128 ? 128 : 256;
  a.N = n_out;
  a.K = M;
  a.m_valid = k_in;
  const long long chunks = (M + gemm::kKc - 1) / gemm::kKc;
  const long long per = (chunks + splits - 1) / splits;
  a.k_split = per * gemm::kKc;
  a.k_splits = (int)((chunks + per - 1) / per);
  a.m_tiles = 1;
  a.C = part;
  a.ldc = 256;
  a.err = err;
  const int rc = k_in <= 128 ? gemm::launch<true, true, 1, gemm::kEpiF32>(a, st)
                             : gemm::launch<true, true, 2, gemm::kEpiF32>(a, st);
  if (rc != NERFGB_OK) return rc;
  const long long n = (long long)k_in * n_out;
  gemm::reduce_splits_kernel<<<(unsigned)((n + gemm::kRedElems - 1) / gemm::kRedElems),
                               gemm::kRedElems * gemm::kRedGroups, 0, st>>>(part, a.k_splits, a.M, 256, k_in, n_out,
                                                                            grads, n_out);
  return launch_status();
}

}  // namespace nerfgb
