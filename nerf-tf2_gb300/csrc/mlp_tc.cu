// Tensor-core forward of the NeRF MLP (nerf/core/model.py:334-394) on
// sm_103a: tcgen05.mma with FP32 accumulators in TMEM, operands in shared
// memory, weights streamed by the bulk-copy (TMA) engine.
//
// CTA tile: 256 sample rows = two 128-row sub-tiles (A, B). The tensor core
// runs layer g of A, then of B (ping-pong), so each sub-tile's epilogue
// overlaps the other's MMAs; a lockstep schedule (A and B consume every
// weight chunk together) is compiled from the same source. The whole 10-GEMM
// chain runs on chip: activations never leave shared memory and only
// xyz/dirs (in) and rgb/sigma (out) touch HBM.
//
// Two kernels share this source:
//   pair (BF16): CTAs run as cluster pairs. The even CTA issues 2-SM MMAs
//     (tcgen05.mma.cta_group::2, M = 256: sub-tile s of both CTAs, B split
//     by N between them), so each SM streams only half of every weight chunk
//     and a 4-stage ring of 16 KB halves holds a whole 256-K layer for both
//     sub-tiles. All 16 epilogue warps serve one sub-tile at a time.
//   single CTA (FP8): tcgen05.mma.cta_group::1, M = 128 per sub-tile, every
//     weight chunk streamed once per sub-tile, 8 epilogue warps per sub-tile.
//
// Warp roles (18 warps; 19 with the tape):
//   warp 0      weight producer: bulk copies of KCH-row weight chunks into
//               an NST-stage ring (full/empty mbarriers); pair: one thread in
//               ring order issuing 2-SM tensor copies that complete on the
//               even CTA's barrier, single CTA: one lane per stage
//   warp 1      TMEM allocator and MMA issuer (one thread; its issue code is
//               generated per layer at compile time, see issue_run); in the
//               odd CTA of a pair only the allocator
//   warps 2-17  epilogue: compute the positional encodings, then per layer
//               read the accumulator (tcgen05.ld), add bias, apply ReLU,
//               round to BF16 (or E4M3) and write the next layer's A operand;
//               the sigma and rgb heads run in FP32.
//   warp 18     (the pair kernel that writes the training tape only) one
//               thread storing each written operand region to the tape by a
//               3-D tensor store, then releasing the region to the epilogue.
//
// Shared memory (bytes, BF16): ring [0,64K) | encA [64K,80K) | encB
// [80K,96K) | actA [96K,160K) | actB [160K,224K) | barriers, sigma partials.
// FP8 halves every operand region and takes a 112K ring plus the bias/head
// table and scales. Operand layout: K-major, no swizzle, 8x16-byte core
// matrices. Element (r, k) of a 128-row operand sits at (k/8)*2048 + r*16 +
// (k%8)*2; weights (n, k) of an N-row chunk at (k/8)*(N*16) + n*16 + (k%8)*2
// (pair: of each N/2-row half).
//
// Every mbarrier wait is bounded (globaltimer). On a timeout the kernel sets
// *err_word = NERFGB_E_TIMEOUT, raises an abort flag that every role polls,
// drains its own bulk copies and MMAs (bounded), frees TMEM and returns (a
// pair meets at a cluster barrier first, so that neither CTA leaves while
// the other's MMAs or arrivals may still touch it).
#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's entry-point query)
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

#include <mutex>
#include <unordered_map>

#include "common.cuh"
#include "mlp_internal.cuh"
#include "tcgen05.cuh"

namespace nerfgb {
namespace tc {

constexpr int kRows = 256;          // rows per CTA tile
constexpr int kThreads = 18 * 32;
// The pair kernel that writes the activation tape has a 19th warp whose
// first lane stores each written operand region to the tape.
constexpr int kTapeWarp = 18;
__host__ __device__ constexpr int threads_of(bool tape_warp) { return tape_warp ? (kTapeWarp + 1) * 32 : kThreads; }

// Tensor maps of the pair pack's weights (2-D, 256-byte rows of 128 BF16),
// one per weight-half size: 64 rows (16 KB), 32 (8 KB), 16 (4 KB). With the
// tape: the tape (kActsLd BF16 per row) as 3-D (8 elements, rows, 8-element
// column groups; strides 2 B, the row stride, 16 B), whose 128-row boxes
// have the operand regions' image (element (r, k) at (k/8)*2048 + r*16 +
// (k%8)*2), so a region is stored to its tape columns as one box: tape[0]
// 32 groups (a 256-wide activation), tape[1] 8 (enc_xyz), tape[2] 4 (enc_dir).
struct PairMaps {
  CUtensorMap map[3];
  CUtensorMap tape[3];
};
__host__ __device__ constexpr int pair_map_of(uint32_t bytes) { return bytes == 16384u ? 0 : bytes == 8192u ? 1 : 2; }

// Shared-memory layout. Operands take E = 2 (BF16) or 1 (FP8) bytes per
// element. TSMEM: the bias/head table (and, for FP8, the per-channel weight
// scales) live in shared memory; otherwise they are read through L1.
template <bool TSMEM, bool F8>
struct Layout {
  static constexpr uint32_t kE = F8 ? 1 : 2;
  static constexpr uint32_t kEncBytes = 128 * 64 * kE;   // per sub-tile
  static constexpr uint32_t kActBytes = 128 * 256 * kE;  // per sub-tile
  static constexpr uint32_t kTableBytes =
      TSMEM ? ((kTableElems + (F8 ? kBiasElems : 0)) * 4 + 127) / 128 * 128 : 0;
  static constexpr uint32_t kRingBytes = F8 ? 112 * 1024 : TSMEM ? 48 * 1024 : 64 * 1024;
  static constexpr uint32_t kRingOff = 0;
  static constexpr uint32_t kEncOff = kRingBytes;               // + s * kEncBytes
  static constexpr uint32_t kActOff = kEncOff + 2 * kEncBytes;  // + s * kActBytes
  static constexpr uint32_t kTableOff = kActOff + 2 * kActBytes;
  static constexpr uint32_t kMiscOff = kTableOff + kTableBytes;
  static constexpr uint32_t kBarFull = kMiscOff;         // [16]
  static constexpr uint32_t kBarEmpty = kMiscOff + 128;  // [16]
  static constexpr uint32_t kBarAccf = kMiscOff + 256;   // [2]
  static constexpr uint32_t kBarActr = kMiscOff + 272;   // [2]
  static constexpr uint32_t kBarDrain = kMiscOff + 288;
  static constexpr uint32_t kTmemSlot = kMiscOff + 296;
  static constexpr uint32_t kAbort = kMiscOff + 304;    // int, then the wait limit (u64) at +8
  static constexpr uint32_t kBarHead = kMiscOff + 320;  // [2]
  static constexpr uint32_t kBarTapeRdy = kMiscOff + 336;   // [2] (the pair kernel with the tape)
  static constexpr uint32_t kBarTapeDone = kMiscOff + 352;  // [2]
  static constexpr uint32_t kSigPart = kMiscOff + 384;  // float [2][128] (single-CTA epilogue)
  static constexpr uint32_t kSmemBytes = kSigPart + 2 * 128 * 4;
  // Pair epilogue: head partial sums (float), in regions idle at the time: sigma's [4][128]
  // in the upper half of the sub-tile's encoding region (enc_xyz's columns
  // 32-63, last read by dense_5, rewritten by the next tile), rgb's
  // [3][4][128] at the start of the sub-tile's activation region (last read
  // by dense_9, rewritten by the next tile's dense_0 epilogue).
  static constexpr uint32_t kSigPartOff = kEncBytes / 2;
  static_assert(4 * 128 * 4 <= kEncBytes / 2 && 3 * 4 * 128 * 4 <= kActBytes, "head partials fit");
};

// ---------------------------------------------------------------------------
// Positional encodings written as BF16 A-operand rows.
// ---------------------------------------------------------------------------
// The tensor-core kernels' positional encoding (model.py:319-331): octave
// l of a coordinate from one sincosf at octave 4*floor(l/4) and l % 4 angle
// doublings (the FP32 angle doubles exactly from one octave to the next;
// sin 2a = (2 sin a) cos a, cos 2a = cos a cos a - sin a sin a, each
// operation rounded in FP32): at most three doublings, ~5e-7 from sincosf at
// every octave, below the BF16 (or E4M3) rounding the value then gets. The
// value of an octave does not depend on which warp computes it.
template <int NP, int L, int W, int Q>
__device__ __forceinline__ void encode_pairs_q(const float (&x)[3], float (&v)[W]) {
  float sn = 0.0f, cs = 1.0f;
  int cur_c = -1, cur_l = -1;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int ks = 3 + 2 * p;  // sin at ks, cos at ks + 1
    if (ks + 1 < W * Q || ks >= W * Q + W) continue;
    const int c = p / L, l = p % L;
    if (c != cur_c || (l & 3) == 0 || cur_l != l - 1) {
      // a chain starts at octave 4*floor(l/4)
      const int l0 = l & ~3;
      sincosf(fmul(x[c], enc_multiplier(l0)), &sn, &cs);
      for (int d = l0; d < l; ++d) {
        const float s2 = fmul(fmul(2.0f, sn), cs);
        cs = fsub(fmul(cs, cs), fmul(sn, sn));
        sn = s2;
      }
    } else {
      const float s2 = fmul(fmul(2.0f, sn), cs);
      cs = fsub(fmul(cs, cs), fmul(sn, sn));
      sn = s2;
    }
    cur_c = c;
    cur_l = l;
    if (ks >= W * Q && ks < W * Q + W) v[ks - W * Q] = sn;
    if (ks + 1 >= W * Q && ks + 1 < W * Q + W) v[ks + 1 - W * Q] = cs;
  }
}

// enc_xyz columns [32*HF, 32*HF + 32) of row r (63 values, column 63 = 0).
// tape_dst (BF16 path only, may be NULL): the same 32 values to the tape.
template <int HF, bool F8>
__device__ __forceinline__ void write_enc_xyz(uint32_t enc, int r, const float (&x)[3], uint16_t *tape_dst) {
  float v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = 0.0f;
  if (HF == 0) {
    v[0] = x[0];
    v[1] = x[1];
    v[2] = x[2];
  }
  encode_pairs_q<30, 10, 32, HF>(x, v);
  if (!F8 && tape_dst) {
    uint32_t u[16];
    pack32_bf16(v, u);
    tape_store32(tape_dst, u);
  }
  store_row32<F8, false>(enc, r, 32 * HF, v);
}

// enc_dir (27 values, 5 zero pad) into K-elements 0..31 of the enc region.
template <bool F8>
__device__ __forceinline__ void write_enc_dir(uint32_t enc, int r, const float (&d)[3], uint16_t *tape_dst) {
  float v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = 0.0f;
  v[0] = d[0];
  v[1] = d[1];
  v[2] = d[2];
  encode_pairs_q<12, 4, 32, 0>(d, v);
  if (!F8 && tape_dst) {
    uint32_t u[16];
    pack32_bf16(v, u);
    tape_store32(tape_dst, u);
  }
  store_row32<F8, false>(enc, r, 0, v);
}

// Stores v[0..16) as the K-elements [k0, k0+16) of row r of a 128-row
// operand region (k0 a multiple of 16).
template <bool F8>
__device__ __forceinline__ void store_row16(uint32_t region, int r, int k0, const float (&v)[16]) {
  if (F8) {
    st_shared_v4(region + (uint32_t)(k0 / 16) * 2048u + r * 16, pack_e4m3x4(v[0], v[1], v[2], v[3]),
                 pack_e4m3x4(v[4], v[5], v[6], v[7]), pack_e4m3x4(v[8], v[9], v[10], v[11]),
                 pack_e4m3x4(v[12], v[13], v[14], v[15]));
  } else {
#pragma unroll
    for (int g = 0; g < 2; ++g)
      st_shared_v4(region + (uint32_t)(k0 / 8 + g) * 2048u + r * 16, pack_bf16(v[8 * g], v[8 * g + 1]),
                   pack_bf16(v[8 * g + 2], v[8 * g + 3]), pack_bf16(v[8 * g + 4], v[8 * g + 5]),
                   pack_bf16(v[8 * g + 6], v[8 * g + 7]));
  }
}
// The same for 8 K-elements [k0, k0+8) (k0 a multiple of 8).
template <bool F8>
__device__ __forceinline__ void store_row8(uint32_t region, int r, int k0, const float (&v)[8]) {
  if (F8) {
    asm volatile("st.shared.v2.b32 [%0], {%1,%2};" ::"r"(region + (uint32_t)(k0 / 16) * 2048u + r * 16 + (k0 % 16)),
                 "r"(pack_e4m3x4(v[0], v[1], v[2], v[3])), "r"(pack_e4m3x4(v[4], v[5], v[6], v[7]))
                 : "memory");
  } else {
    st_shared_v4(region + (uint32_t)(k0 / 8) * 2048u + r * 16, pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]),
                 pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
  }
}

// enc_xyz columns [16*Q, 16*Q + 16) of row r (63 values, column 63 = 0).
// tape_dst (BF16 path only, may be NULL): the same 16 values to the tape.
template <int Q, bool F8>
__device__ __forceinline__ void write_enc_xyz_q(uint32_t enc, int r, const float (&x)[3], uint16_t *tape_dst) {
  float v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = 0.0f;
  if (Q == 0) {
    v[0] = x[0];
    v[1] = x[1];
    v[2] = x[2];
  }
  encode_pairs_q<30, 10, 16, Q>(x, v);
  if (!F8 && tape_dst) {
    uint4 *t = reinterpret_cast<uint4 *>(tape_dst);
    t[0] = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
    t[1] = make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]),
                      pack_bf16(v[14], v[15]));
  }
  store_row16<F8>(enc, r, 16 * Q, v);
}

// enc_dir (27 values, 5 zero pad in K-elements 0..31 of the enc region):
// columns [8*Q, 8*Q + 8) of row r.
template <int Q, bool F8>
__device__ __forceinline__ void write_enc_dir_q(uint32_t enc, int r, const float (&d)[3], uint16_t *tape_dst) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = (8 * Q + i < 3) ? d[8 * Q + i] : 0.0f;
  encode_pairs_q<12, 4, 8, Q>(d, v);
  if (!F8 && tape_dst)
    *reinterpret_cast<uint4 *>(tape_dst) =
        make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
  store_row8<F8>(enc, r, 8 * Q, v);
}

// ---------------------------------------------------------------------------
// MMA issue
// ---------------------------------------------------------------------------
// tcgen05.mma is issued by one thread, and the tensor pipe runs ahead of it
// by little: every instruction the issuing thread executes between two MMAs
// is latency on the pipe (measured: a 128x256x16 MMA takes 128 cycles; with
// run-time layer shapes, operand selects and 64-bit descriptor assembly per
// MMA the issue loop took ~164 cycles per MMA). So the issue code is shaped
// at compile time per layer: descriptors are two 32-bit words, the high word
// a constant (SBO = 128 B, version bit 46) and the low word a base plus
// immediates (start address >> 4 in bits 0-13, LBO >> 4 in bits 16-29).
constexpr uint32_t kDescHi = (128u >> 4) | (1u << 14);

__device__ __forceinline__ uint64_t desc_lo(uint32_t lo) { return ((uint64_t)kDescHi << 32) | lo; }

// Out-of-line slow path of a full-barrier wait: spins until the phase
// completes, the CTA aborts, or the wait limit passes (then raises the abort).
__device__ __noinline__ void wait_slow(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try(bar, parity)) {
    if (*abort_flag) return;
    if (globaltimer() - t0 > wait_limit(abort_flag)) {
      atomicExch(err, NERFGB_E_TIMEOUT);
      *abort_flag = 1;
      return;
    }
  }
}

__device__ __forceinline__ void wait_fast(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err) {
  if (!mbar_try(bar, parity)) wait_slow(bar, parity, abort_flag, err);
}

template <bool F8, bool PAIR>
__device__ __forceinline__ void mma_any(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  static_assert(!(F8 && PAIR), "the pair path is BF16");
  if (PAIR)
    tc_mma_pair(d, a, b, idesc, acc);
  else if (F8)
    tc_mma_f8(d, a, b, idesc, acc);
  else
    tc_mma(d, a, b, idesc, acc);
}

// Ring position of the MMA issuer.
struct RingPos {
  int stage;
  uint32_t phase;
};

// NC chunks of KC K-rows: A from the sub-tiles' regions (descriptor low words
// a_lo0/a_lo1 at the run's first K-group), B from successive ring stages.
// FIRST: the run starts the layer (its first MMA overwrites the accumulator).
// WAIT: wait for each stage's weights (a run over stages another run has
// already waited for skips it). FREE: release each stage once its MMAs
// complete. PAIR: 2-SM MMAs (M = 256 over the pair, each ring stage holds
// this CTA's N/2 weight rows), commits to both CTAs.
template <int NC, int KC, int N, bool F8, int NST, uint32_t kStageBytes, int S_LO, int S_HI, bool FIRST,
          bool PAIR = false, bool WAIT = true, bool FREE = true>
__device__ __forceinline__ void issue_run(uint32_t bar_full, uint32_t bar_empty, uint32_t ring_lo, uint32_t a_lo0,
                                          uint32_t a_lo1, uint32_t tmem, uint32_t idesc, RingPos &rp,
                                          volatile int *abort_flag, int *err) {
  constexpr int KM = F8 ? 32 : 16;   // K per MMA
  constexpr int KW = F8 ? 16 : 8;    // K per 16-byte core-matrix row
  constexpr uint32_t kAStep = 2048u >> 4;                    // one A K-group
  constexpr uint32_t kAChunk = (uint32_t)(KC / KW) * kAStep;  // one chunk of A
  constexpr uint32_t kBStep = (uint32_t)(PAIR ? N / 2 : N);  // one B K-group: rows*16 B >> 4
  static_assert(KC % KM == 0, "chunk is a whole number of MMAs");
#pragma unroll 1
  for (int c = 0; c < NC; ++c) {
    if (WAIT) {
      wait_fast(bar_full + 8 * rp.stage, rp.phase, abort_flag, err);
      tc_fence_after();
    }
    const uint32_t b_lo = ring_lo + (uint32_t)rp.stage * (kStageBytes >> 4);
    const uint32_t a0 = a_lo0 + (uint32_t)c * kAChunk, a1 = a_lo1 + (uint32_t)c * kAChunk;
#pragma unroll
    for (int ks = 0; ks < KC / KM; ++ks) {
      const uint64_t bdesc = desc_lo(b_lo + (uint32_t)(2 * ks) * kBStep);
      const uint32_t acc = (FIRST && ks == 0) ? (c > 0 ? 1u : 0u) : 1u;
      if (S_LO == 0) mma_any<F8, PAIR>(tmem, desc_lo(a0 + (uint32_t)(2 * ks) * kAStep), bdesc, idesc, acc);
      if (S_HI == 1) mma_any<F8, PAIR>(tmem + 256, desc_lo(a1 + (uint32_t)(2 * ks) * kAStep), bdesc, idesc, acc);
    }
    if (FREE) commit_any<PAIR>(bar_empty + 8 * rp.stage);
    if (++rp.stage == NST) {
      rp.stage = 0;
      rp.phase ^= 1;
    }
  }
}

// The MMAs of GEMM layer G for sub-tiles [S_LO, S_HI]: its K rows are
// [activation (256) | encoding (the rest)] for dense_5 and dense_9, the
// encoding alone for dense_0 and the activation alone otherwise; chunks
// never straddle the two (KCH divides 256), the last may be short.
template <int G, int KCH, int NST, bool TSMEM, bool F8, int S_LO, int S_HI, bool PAIR = false, bool WAIT = true,
          bool FREE = true>
__device__ __forceinline__ void issue_gemm(uint32_t sbase, uint32_t tmem, RingPos &rp, volatile int *abort_flag,
                                           int *err) {
  using L = Layout<TSMEM, F8>;
  constexpr int N = gemm_n(G), Kp = gemm_kp(G);
  constexpr int KA = G == 0 ? 0 : 256, KE = Kp - KA;
  constexpr int NB = PAIR ? N / 2 : N;  // weight rows (output channels) per ring stage
  constexpr uint32_t kStageBytes = (PAIR ? 128 : 256) * KCH * L::kE;
  constexpr uint32_t idesc = F8 ? idesc_e4m3(128, N) : idesc_bf16(PAIR ? 256 : 128, N);
  static_assert(256 % KCH == 0, "chunks must not straddle the activation/encoding split");
  const uint32_t bar_full = sbase + L::kBarFull, bar_empty = sbase + L::kBarEmpty;
  // Descriptor start addresses are 18-bit shared-window offsets (a CTA's
  // window address may carry bits above them, as in a cluster launch).
  const uint32_t sw = sbase & 0x3FFFFu;
  const uint32_t ring_lo = ((sw + L::kRingOff) >> 4) | ((uint32_t)NB << 16);
  constexpr uint32_t kALbo = (2048u >> 4) << 16;
  if constexpr (KA > 0) {
    const uint32_t act_lo = ((sw + L::kActOff) >> 4) | kALbo;
    issue_run<KA / KCH, KCH, N, F8, NST, kStageBytes, S_LO, S_HI, true, PAIR, WAIT, FREE>(
        bar_full, bar_empty, ring_lo, act_lo, act_lo + (L::kActBytes >> 4), tmem, idesc, rp, abort_flag, err);
  }
  const uint32_t enc_lo = ((sw + L::kEncOff) >> 4) | kALbo;
  if constexpr (KE / KCH > 0)
    issue_run<KE / KCH, KCH, N, F8, NST, kStageBytes, S_LO, S_HI, KA == 0, PAIR, WAIT, FREE>(
        bar_full, bar_empty, ring_lo, enc_lo, enc_lo + (L::kEncBytes >> 4), tmem, idesc, rp, abort_flag, err);
  if constexpr (KE % KCH > 0) {
    constexpr int KR = KE % KCH;
    constexpr int KW = F8 ? 16 : 8;
    const uint32_t off = (uint32_t)(KE / KCH) * (uint32_t)(KCH / KW) * (2048u >> 4);
    issue_run<1, KR, N, F8, NST, kStageBytes, S_LO, S_HI, KA == 0 && KE / KCH == 0, PAIR, WAIT, FREE>(
        bar_full, bar_empty, ring_lo, enc_lo + off, enc_lo + off + (L::kEncBytes >> 4), tmem, idesc, rp, abort_flag,
        err);
  }
}

// Weight chunks of GEMM layer G, and whether the pair schedule streams them
// once per tile (they all fit the ring: sub-tile A's MMAs leave them in place
// for sub-tile B's, which release them) or once per sub-tile.
template <int G, int KCH>
constexpr int layer_chunks() {
  return (gemm_kp(G) + KCH - 1) / KCH;
}
__host__ __device__ constexpr bool pair_stream_once(int nch, int nst) { return nch <= nst; }

// One layer: wait until the epilogue has written the A operands (and read
// the accumulators), issue, then signal the accumulators full.
template <int G, int KCH, int NST, bool PINGPONG, bool TSMEM, bool F8, bool PAIR = false>
__device__ __forceinline__ void issue_layer(uint32_t sbase, uint32_t tmem, RingPos &rp, uint32_t &actr_phase,
                                            volatile int *abort_flag, int *err) {
  using L = Layout<TSMEM, F8>;
  const uint32_t actr = sbase + L::kBarActr, accf = sbase + L::kBarAccf;
  if constexpr (PAIR) {
    // Ping-pong over the pair: M = 256 rows (128 from each CTA) per MMA.
    constexpr bool once = pair_stream_once(layer_chunks<G, KCH>(), NST);
    wait_fast(actr, actr_phase, abort_flag, err);
    tc_fence_after();
    const RingPos start = rp;
    issue_gemm<G, KCH, NST, TSMEM, F8, 0, 0, true, true, !once>(sbase, tmem, rp, abort_flag, err);
    tc_commit_pair(accf);
    wait_fast(actr + 8, actr_phase, abort_flag, err);
    tc_fence_after();
    if (once) rp = start;
    issue_gemm<G, KCH, NST, TSMEM, F8, 1, 1, true, !once, true>(sbase, tmem, rp, abort_flag, err);
    tc_commit_pair(accf + 8);
  } else if constexpr (PINGPONG) {
    wait_fast(actr, actr_phase, abort_flag, err);
    tc_fence_after();
    issue_gemm<G, KCH, NST, TSMEM, F8, 0, 0>(sbase, tmem, rp, abort_flag, err);
    tc_commit(accf);
    wait_fast(actr + 8, actr_phase, abort_flag, err);
    tc_fence_after();
    issue_gemm<G, KCH, NST, TSMEM, F8, 1, 1>(sbase, tmem, rp, abort_flag, err);
    tc_commit(accf + 8);
  } else {
    wait_fast(actr, actr_phase, abort_flag, err);
    wait_fast(actr + 8, actr_phase, abort_flag, err);
    tc_fence_after();
    issue_gemm<G, KCH, NST, TSMEM, F8, 0, 1>(sbase, tmem, rp, abort_flag, err);
    tc_commit(accf);
    tc_commit(accf + 8);
  }
  actr_phase ^= 1;
}

template <int KCH, int NST, bool PINGPONG, bool TSMEM, bool F8, bool PAIR>
__device__ __forceinline__ void issue_tile(uint32_t sbase, uint32_t tmem, RingPos &rp, uint32_t &actr_phase,
                                           volatile int *abort_flag, int *err) {
  issue_layer<0, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<1, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<2, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<3, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<4, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<5, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<6, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<7, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<8, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  issue_layer<9, KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
  static_assert(kNumGemm == 10, "one issue_layer per GEMM");
}

// The CTA's weight-chunk loads in ring order: per tile, per GEMM layer, the
// layer's chunks once or (ping-pong, unless the pair schedule keeps the layer
// in the ring) once per sub-tile. f(g, c) returns false to stop.
template <int KCH, int NST, bool PINGPONG, bool PAIR, typename F>
__device__ __forceinline__ void for_each_load(long long t_first, long long t_step, long long ntiles, F &&f) {
  for (long long tile = t_first; tile < ntiles; tile += t_step)
    for (int g = 0; g < kNumGemm; ++g) {
      const int nch = (gemm_kp(g) + KCH - 1) / KCH;
      const int reps = PAIR ? (pair_stream_once(nch, NST) ? 1 : 2) : (PINGPONG ? 2 : 1);
      for (int s = 0; s < reps; ++s)
        for (int c = 0; c < nch; ++c)
          if (!f(g, c)) return;
    }
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
// KCH: K rows per weight chunk; NST: ring stages. PINGPONG: the tensor core
// runs A(g) then B(g), each streaming the layer's weights (epilogues overlap
// MMAs); otherwise A and B share every chunk in lockstep (half the weight
// traffic, epilogues exposed).
// F8: E4M3 operands (kind::f8f6f4, K = 32 per MMA) with per-output-channel
// weight scales applied in the epilogue; else BF16 (kind::f16, K = 16).
// STORE (BF16 only, training): every layer's BF16 activations (the operands
// the next layer's MMAs read) and the encodings also go to `tape`, kActsLd
// BF16 values per row at the columns of the FP32 tape (acts_offset).
// PAIR (BF16, ping-pong): CTAs run as cluster pairs on 512-row tiles, 256
// rows per CTA as above. The even CTA's issuer drives 2-SM MMAs (M = 256:
// sub-tile s of both CTAs) and each CTA streams only its N/2 half of every
// weight chunk (kBf16PairOff layout), halving the bytes an SM takes in; with
// half chunks of 16 KB a 4-stage ring holds a whole 256-K layer, so such a
// layer is streamed once for both sub-tiles. Both CTAs' halves are 2-SM
// tensor copies (maps: the pair pack as 256-byte rows) completing on the even
// CTA's full barrier; the odd CTA's epilogue warps arrive on the even CTA's
// operand barriers; commits reach both CTAs.
template <int KCH, int NST, bool PINGPONG, bool TSMEM, bool F8, bool STORE, bool PAIR = false>
__global__ void __launch_bounds__(threads_of(STORE && PAIR), 1)
    mlp_tc_kernel(const uint8_t *__restrict__ packed, const float *__restrict__ xyz,
                    const float *__restrict__ dirs, long long n_max, int rpd, float *__restrict__ rgb_out,
                    float *__restrict__ sigma_out, int *__restrict__ err, RowMap rm, uint16_t *__restrict__ tape,
                    unsigned long long wait_ns, long long withhold, const __grid_constant__ PairMaps maps) {
  static_assert(!(STORE && F8), "the activation tape is BF16");
  static_assert(kActsLd % 8 == 0 && kActsEncXyz % 8 == 0 && kActsEncDir % 8 == 0, "tape columns in 8-element groups");
  static_assert(!PAIR || (!F8 && PINGPONG && KCH == kPairKch), "pair path: BF16 ping-pong, the pair pack's chunks");
  using L = Layout<TSMEM, F8>;
  constexpr uint32_t kE = L::kE;           // bytes per operand element
  constexpr uint32_t kRingOff = L::kRingOff, kEncOff = L::kEncOff, kActOff = L::kActOff;
  constexpr uint32_t kBarFull = L::kBarFull, kBarEmpty = L::kBarEmpty, kBarAccf = L::kBarAccf;
  constexpr uint32_t kBarActr = L::kBarActr, kBarDrain = L::kBarDrain, kTmemSlot = L::kTmemSlot;
  constexpr uint32_t kAbort = L::kAbort, kSigPart = L::kSigPart;
  constexpr uint32_t kStageBytes = (PAIR ? 128 : 256) * KCH * kE;
  static_assert(NST * kStageBytes <= L::kRingBytes && NST <= 16, "ring does not fit");
  constexpr long long kTileRows = PAIR ? 2 * kRows : kRows;
  extern __shared__ __align__(1024) uint8_t smem[];
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kAbort);
  // Tiles: this CTA (or pair) takes first, first + step, ...; rank = the
  // CTA's place in its pair (its rows follow the even CTA's 256).
  // (Single CTA: blockIdx.x and gridDim.x, read at each use rather than
  // kept live across the roles' code.)
  const uint32_t crank = PAIR ? cluster_rank() : 0u;
  const long long pair_first = PAIR ? (long long)cluster_id() : 0ll;
  const long long pair_step = PAIR ? (long long)cluster_count() : 0ll;
#define t_first (PAIR ? pair_first : (long long)blockIdx.x)
#define t_step (PAIR ? pair_step : (long long)gridDim.x)
  constexpr long long kTabOff = F8 ? kFp8TableOff : kBf16TableOff;
  const float *table = TSMEM ? reinterpret_cast<const float *>(smem + L::kTableOff)
                             : reinterpret_cast<const float *>(packed + kTabOff);
  // FP8 scales follow the table (shared) or sit at kFp8ScaleOff (global).
  const float *scales = TSMEM ? table + kTableElems : reinterpret_cast<const float *>(packed + kFp8ScaleOff);
  // Row count (device-side with a row map from a compaction kernel) and the
  // physical row of logical row k.
  const long long n = rm.n_dev ? min((long long)*rm.n_dev, n_max) : n_max;
  const long long ntiles = (n + kTileRows - 1) / kTileRows;
  auto phys = [&](long long k) -> long long {
    return rm.map ? (long long)NG_IDX(rm.map[k], n_max, kSiteMlpRowMap) : k;
  };

  if (TSMEM) {  // bias and head table (and scales) -> shared memory
    const float4 *src = reinterpret_cast<const float4 *>(packed + kTabOff);
    float4 *dst = reinterpret_cast<float4 *>(smem + L::kTableOff);
    for (int i = threadIdx.x; i < kTableElems / 4; i += kThreads) dst[i] = src[i];
    if (F8) {
      const float4 *ssrc = reinterpret_cast<const float4 *>(packed + kFp8ScaleOff);
      for (int i = threadIdx.x; i < kBiasElems / 4; i += kThreads) dst[kTableElems / 4 + i] = ssrc[i];
    }
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      // pair: the even CTA's stage completes on its producer's arrival and
      // the bytes of both CTAs' copies (the odd CTA's signal it directly)
      mbar_init(sbase + kBarFull + 8 * s, 1);
      mbar_init(sbase + kBarEmpty + 8 * s, 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(sbase + kBarAccf + 8 * s, 1);
      // pair: one arrival per epilogue warp of both CTAs; single CTA: one
      // per thread of the sub-tile's eight epilogue warps
      mbar_init(sbase + kBarActr + 8 * s, PAIR ? 32 : 256);
      // head partial sums: one arrival per epilogue warp of the sub-tile's
      // other half (single CTA: 4) or of all four column quarters (pair: 16)
      mbar_init(sbase + L::kBarHead + 8 * s, PAIR ? 16 : 4);
    }
    mbar_init(sbase + kBarDrain, 1);
    if (STORE && PAIR) {
      for (int s = 0; s < 2; ++s) {
        // one arrival per epilogue warp of this CTA; the tape writer's
        mbar_init(sbase + L::kBarTapeRdy + 8 * s, 16);
        mbar_init(sbase + L::kBarTapeDone + 8 * s, 1);
      }
    }
    *abort_flag = 0;
    set_wait_limit(abort_flag, wait_ns);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    // pair: one warp of each CTA allocates collectively (same address in both)
    if (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + kTmemSlot),
                   "r"(512));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + kTmemSlot),
                   "r"(512));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
  }
  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync_all();  // the peer's barriers exist before any arrival reaches them
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(smem + kTmemSlot);

  const uint8_t *wsrc = packed + (PAIR ? kBf16PairOff : 0);
  // Bytes and source of this CTA's part of chunk c of GEMM layer g (pair:
  // its N-half, contiguous in the pair pack).
  auto chunk_src = [&](int g, int c, uint32_t &bytes) -> const uint8_t * {
    const int N = gemm_n(g), Kp = gemm_kp(g);
    const int kc = Kp - c * KCH < KCH ? Kp - c * KCH : KCH;  // the last chunk may be short
    bytes = (uint32_t)(PAIR ? N / 2 : N) * kc * kE;
    return wsrc + gemm_w_offset(g) * kE + (long long)c * KCH * N * kE + crank * bytes;
  };
  if (warp == 0) {
    // ---------------- weight producer ----------------
    if (PAIR) {
      // One thread issues the loads in ring order (stage q % NST): a stage
      // frees once per chunk of MMAs, and the copies of one thread complete
      // at a few hundred cycles' spacing, so one thread keeps pace without
      // lanes of one warp spinning on different barriers. Each CTA copies
      // its N-half with a 2-SM tensor copy that completes on the even CTA's
      // full barrier, whose producer expects both halves' bytes.
      if (lane == 0) {
        uint32_t used = 0;  // bit st: parity of the copies issued into stage st
        int st = 0;
        bool ok = true;
        long long nq = 0;  // chunks of this CTA's load sequence
        for_each_load<KCH, NST, PINGPONG, PAIR>(t_first, t_step, ntiles, [&](int g, int c) {
          if (!wait_bar(sbase + kBarEmpty + 8 * st, ((used >> st) & 1u) ^ 1u, abort_flag, err)) {
            ok = false;
            return false;
          }
          // test hook of the failure path: the even CTA leaves chunk `withhold` unloaded
          if (!(nq++ == withhold && crank == 0)) {
            uint32_t bytes;
            const uint8_t *src = chunk_src(g, c, bytes);
            const uint32_t full = sbase + kBarFull + 8 * st;
            if (crank == 0) mbar_expect_tx(full, 2 * bytes);
            tma_2d_pair(sbase + kRingOff + st * kStageBytes, &maps.map[pair_map_of(bytes)], 0,
                        (int)((src - packed - kBf16PairOff) >> 8), crank == 0 ? full : peer_addr(full, 0));
          }
          used ^= 1u << st;
          if (++st == NST) st = 0;
          return true;
        });
        if (!ok && crank == 0) {
          // Drain: wait (bounded) for the stages' last copies (both CTAs';
          // the odd CTA's own drain is at the kernel's end).
          const uint64_t t0 = globaltimer();
          for (int k = 0; k < NST; ++k)
            while (!mbar_try(sbase + kBarFull + 8 * k, ((used >> k) & 1u) ^ 1u) && globaltimer() - t0 < 10000000ull) {
            }
        }
      }
    } else if (lane < NST) {
      // Lane l owns ring stage l and issues every NST-th chunk: bulk copies
      // issued by one thread complete one after another, copies issued by
      // different threads overlap.
      const int st = lane;
      const uint32_t full = sbase + kBarFull + 8 * st;
      uint32_t phase = 0;
      long long q = 0;  // chunk counter over the CTA's whole sequence
      bool ok = true, issued = false;
      for (long long tile = t_first; tile < ntiles && ok; tile += t_step) {
        for (int g = 0; g < kNumGemm && ok; ++g) {
          const int nch = (gemm_kp(g) + KCH - 1) / KCH;  // the last chunk may be 32 K
          for (int s = 0; s < (PINGPONG ? 2 : 1) && ok; ++s) {
            for (int c = 0; c < nch; ++c, ++q) {
              if ((int)(q % NST) != st) continue;
              if (!wait_bar(sbase + kBarEmpty + 8 * st, phase ^ 1, abort_flag, err)) {
                ok = false;
                break;
              }
              if (q != withhold) {  // test hook of the failure path: chunk `withhold` left unloaded
                const int N = gemm_n(g), Kp = gemm_kp(g);
                const int kc = Kp - c * KCH < KCH ? Kp - c * KCH : KCH;
                const uint32_t bytes = (uint32_t)N * kc * kE;
                mbar_expect_tx(full, bytes);
                bulk_g2s(sbase + kRingOff + st * kStageBytes,
                         packed + gemm_w_offset(g) * kE + (long long)c * KCH * N * kE, bytes, full);
              }
              issued = true;
              phase ^= 1;
            }
          }
        }
      }
      if (!ok && issued) {
        // Drain: wait (bounded) for this stage's copy still in flight.
        uint64_t t0 = globaltimer();
        while (!mbar_try(full, phase ^ 1) && globaltimer() - t0 < 10000000ull) {
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    // pair: the even CTA issues for both (the odd CTA's warp 1 only holds
    // the TMEM allocation).
    const bool issued_any = t_first < ntiles;
    if (lane == 0 && crank == 0) {
      if (PAIR) {
        // both CTAs must hold the same TMEM columns (the collective
        // allocation gives them); otherwise issue nothing
        uint32_t peer_tmem;
        asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(peer_tmem) : "r"(peer_addr(sbase + kTmemSlot, 1))
                     : "memory");
        if (peer_tmem != tmem) {
          atomicExch(err, NERFGB_E_UNSUPPORTED);
          *abort_flag = 1;
        }
      }
      // After an abort every wait returns at once: the remaining MMAs of the
      // tile read stale (in-bounds) shared memory and the tile loop ends.
      RingPos rp{0, 0u};
      uint32_t actr_phase = 0;
      for (long long tile = t_first; tile < ntiles; tile += t_step) {
        if (*abort_flag) break;
        issue_tile<KCH, NST, PINGPONG, TSMEM, F8, PAIR>(sbase, tmem, rp, actr_phase, abort_flag, err);
      }
      if (issued_any) {
        // Drain every MMA issued by this thread before TMEM is released
        // (pair: in both CTAs).
        commit_any<PAIR>(sbase + kBarDrain);
        uint64_t t0 = globaltimer();
        while (!mbar_try(sbase + kBarDrain, 0) && globaltimer() - t0 < 100000000ull) {
        }
      }
    }
  } else if (STORE && PAIR && warp == kTapeWarp) {
    // ---------------- tape writer (pair kernel with the tape) ----------------
    // Per tile and sub-tile the epilogue signals ten regions on tape_rdy, in
    // order: enc_xyz (written for the tile's dense_0), then h0 .. h8 (each
    // layer's output, the next layer's operand; with h8 the enc_dir of
    // dense_9). Each goes to its tape columns of the sub-tile's 128 rows as
    // one tensor store (rows past n are not written); once the store has read
    // shared memory, tape_done tells the epilogue that the region may be
    // rewritten. h9 (never an operand) is stored by the epilogue itself.
    if (lane == 0) {
      uint32_t rdy_phase[2] = {0u, 0u};
      bool ok = true;
      for (long long tile = t_first; tile < ntiles && ok; tile += t_step) {
        for (int e = 0; e < 10 && ok; ++e) {
          for (int s = 0; s < 2; ++s) {
            if (!wait_bar(sbase + L::kBarTapeRdy + 8 * s, rdy_phase[s], abort_flag, err)) {
              ok = false;
              break;
            }
            rdy_phase[s] ^= 1u;
            const long long row = tile * kTileRows + (long long)crank * kRows + s * 128;
            const uint32_t enc = sbase + kEncOff + s * L::kEncBytes, act = sbase + kActOff + s * L::kActBytes;
            if (row < n) {  // (a box from row n on would write nothing)
              if (e == 0) {
                tma_store_3d(&maps.tape[1], enc, 0, (int)row, kActsEncXyz / 8);
              } else {
                tma_store_3d(&maps.tape[0], act, 0, (int)row, acts_offset(e - 1) / 8);
                if (e == 9) tma_store_3d(&maps.tape[2], enc, 0, (int)row, kActsEncDir / 8);
              }
              bulk_commit();
              bulk_wait_read();
            }
            mbar_arrive(sbase + L::kBarTapeDone + 8 * s);
          }
        }
      }
      bulk_wait_all();  // no store still reads this CTA's shared memory or writes the tape
    }
  } else {
    if constexpr (PAIR) {
      // ---------------- epilogue warps (pair) ----------------
      // All 16 warps serve whichever sub-tile's accumulators are ready (A, then
      // B, every layer), so that one sub-tile's epilogue runs on every warp
      // while the tensor core runs the other's MMAs. Warp w reads TMEM lane
      // quadrant qd = w % 4 (rows 32*qd ..) and column quarter cq: 64 columns
      // (32 of dense_9's 128); the heads' partial sums over the quarters meet
      // in shared memory behind the head barrier (one arrival per warp).
      const int ew = warp - 2;
      const int qd = warp & 3, cq = ew >> 2;
      const int r = 32 * qd + lane;  // row within a sub-tile (= TMEM lane)
      const uint32_t tlane = tmem + ((uint32_t)(32 * qd) << 16);
      // With the tape: a region signalled to the tape writer is not rewritten
      // before its store has read it (tape_done; at most one pending per
      // sub-tile, so a parity wait cannot miss a phase).
      bool tape_pending[2] = {false, false};
      uint32_t tape_phase[2] = {0u, 0u};
      auto tape_settle = [&](int s) -> bool {
        if (!STORE || !tape_pending[s]) return true;
        tape_pending[s] = false;
        const bool done = __all_sync(0xffffffffu, wait_bar(sbase + L::kBarTapeDone + 8 * s, tape_phase[s], abort_flag,
                                                           err));
        tape_phase[s] ^= 1u;
        return done;
      };
      // The operands of sub-tile s's next MMAs are written (and its
      // accumulators read): one arrival per warp, on the even CTA's barrier
      // for a pair (with the tape, also on this CTA's tape_rdy).
      auto operands_ready = [&](int s) {
        fence_proxy_async();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if (PAIR)
            mbar_arrive_remote(peer_addr(sbase + kBarActr + 8 * s, 0));
          else
            mbar_arrive(sbase + kBarActr + 8 * s);
          if (STORE) mbar_arrive(sbase + L::kBarTapeRdy + 8 * s);
        }
        if (STORE) tape_pending[s] = true;
      };
      auto head_arrive = [&](int s) {
        __syncwarp();
        if (lane == 0) mbar_arrive(sbase + L::kBarHead + 8 * s);
      };
      // Row state of sub-tile s in tile t, and its enc_xyz quarter written as
      // the operand of dense_0 (the first tile's at the start, each later
      // tile's as soon as the sub-tile's dense_9 of the tile before is done).
      long long prow[2];
      bool valid[2];
      uint16_t *trow_tape[2];
      auto start_rows = [&](long long t, int s) {
        const long long grow = t * kTileRows + (long long)crank * kRows + s * 128 + r;
        valid[s] = grow < n;
        prow[s] = phys(valid[s] ? grow : n - 1);
        trow_tape[s] = (STORE && valid[s]) ? tape + grow * kActsLd : nullptr;
        const uint32_t enc = sbase + kEncOff + s * L::kEncBytes;
        float x[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = valid[s] ? xyz[prow[s] * 3 + c] : 0.0f;
        // (with the tape, the encoding reaches it by the tape writer's store)
        uint16_t *const tt = nullptr;
        tape_settle(s);  // nothing pending here: the sub-tile's dense_9 epilogue settled it
        if (cq == 0)
          write_enc_xyz_q<0, F8>(enc, r, x, tt);
        else if (cq == 1)
          write_enc_xyz_q<1, F8>(enc, r, x, tt);
        else if (cq == 2)
          write_enc_xyz_q<2, F8>(enc, r, x, tt);
        else
          write_enc_xyz_q<3, F8>(enc, r, x, tt);
        operands_ready(s);
      };
      uint32_t accf_phase = 0;  // both sub-tiles' accumulator barriers, per layer
      bool ok = true;
      if (t_first < ntiles) {
        start_rows(t_first, 0);
        start_rows(t_first, 1);
      }
      for (long long tile = t_first; tile < ntiles && ok; tile += t_step) {
        const bool has_next = tile + t_step < ntiles;
        for (int g = 0; g < kNumGemm && ok; ++g) {
          const float *bias = table + bias_offset(g);
          const int nj = g == 9 ? 1 : 2;                    // 32-column pieces of this warp
          const int cbase = g == 9 ? 32 * cq : 64 * cq;     // first column
          for (int s = 0; s < 2; ++s) {
            const uint32_t bar_accf = sbase + kBarAccf + 8 * s;
            // warp-uniform outcome, so that the warp leaves together
            if (!__all_sync(0xffffffffu, wait_bar(bar_accf, accf_phase, abort_flag, err))) {
              ok = false;
              break;
            }
            tc_fence_after();
            // the sub-tile's regions are rewritten below (the next operand,
            // head partials, encodings) once the tape has them
            if (!tape_settle(s)) {
              ok = false;
              break;
            }
            const uint32_t enc = sbase + kEncOff + s * L::kEncBytes;
            const uint32_t act = sbase + kActOff + s * L::kActBytes;
            float sig = 0.0f;
            float rgb_acc[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
            for (int j = 0; j < nj; ++j) {
              const int col0 = cbase + j * 32;
              uint32_t raw[32];
              tmem_ld32(tlane + s * 256 + col0, raw);
              float v[32];
              if (F8) {
                // acc * scale[col] + bias[col] (per-output-channel weight scale)
                tmem_wait32(raw);
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                  const float4 b4 = *reinterpret_cast<const float4 *>(bias + col0 + i);
                  const float4 s4 = *reinterpret_cast<const float4 *>(scales + bias_offset(g) + col0 + i);
                  fma_f32x2(v[i], v[i + 1], __uint_as_float(raw[i]), __uint_as_float(raw[i + 1]), s4.x, s4.y, b4.x,
                            b4.y);
                  fma_f32x2(v[i + 2], v[i + 3], __uint_as_float(raw[i + 2]), __uint_as_float(raw[i + 3]), s4.z, s4.w,
                            b4.z, b4.w);
                }
              } else {
                float b[32];
#pragma unroll
                for (int i = 0; i < 32; i += 4)
                  *reinterpret_cast<float4 *>(b + i) = *reinterpret_cast<const float4 *>(bias + col0 + i);
                tmem_wait32(raw);
#pragma unroll
                for (int i = 0; i < 32; i += 2)
                  add_f32x2(v[i], v[i + 1], __uint_as_float(raw[i]), __uint_as_float(raw[i + 1]), b[i], b[i + 1]);
              }
              if (g == 7) {
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                  const float4 w4 = *reinterpret_cast<const float4 *>(table + kSigmaWOff + col0 + i);
                  sig = fmaf(fmaxf(v[i], 0.0f), w4.x, sig);
                  sig = fmaf(fmaxf(v[i + 1], 0.0f), w4.y, sig);
                  sig = fmaf(fmaxf(v[i + 2], 0.0f), w4.z, sig);
                  sig = fmaf(fmaxf(v[i + 3], 0.0f), w4.w, sig);
                }
              }
              if (g == 9) {
                if (STORE && trow_tape[s]) {
                  uint32_t u[16];
#pragma unroll
                  for (int i = 0; i < 16; ++i) u[i] = pack_bf16_relu(v[2 * i], v[2 * i + 1]);
                  tape_store32(trow_tape[s] + acts_offset(9) + col0, u);
                }
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                  // rows col0+i .. col0+i+3 of the [128][3] rgb kernel: 12 floats
                  const float *wr = table + kRgbWOff + (col0 + i) * 3;
                  const float4 a4 = *reinterpret_cast<const float4 *>(wr);
                  const float4 b4 = *reinterpret_cast<const float4 *>(wr + 4);
                  const float4 c4 = *reinterpret_cast<const float4 *>(wr + 8);
                  const float w12[12] = {a4.x, a4.y, a4.z, a4.w, b4.x, b4.y, b4.z, b4.w, c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                  for (int q = 0; q < 4; ++q) {
                    const float h = fmaxf(v[i + q], 0.0f);
                    rgb_acc[0] = fmaf(h, w12[3 * q], rgb_acc[0]);
                    rgb_acc[1] = fmaf(h, w12[3 * q + 1], rgb_acc[1]);
                    rgb_acc[2] = fmaf(h, w12[3 * q + 2], rgb_acc[2]);
                  }
                }
              } else if (F8) {
                if (g == 8)  // dense_8 is linear (model.py:377-378)
                  store_row32<true, false>(act, r, col0, v);
                else
                  store_row32<true, true>(act, r, col0, v);
              } else if (STORE) {
                // BF16 operands of the next layer (the tape writer stores them)
                uint32_t u[16];
                if (g == 8) {  // dense_8 is linear (model.py:377-378)
#pragma unroll
                  for (int i = 0; i < 16; ++i) u[i] = pack_bf16(v[2 * i], v[2 * i + 1]);
                } else {
#pragma unroll
                  for (int i = 0; i < 16; ++i) u[i] = pack_bf16_relu(v[2 * i], v[2 * i + 1]);
                }
#pragma unroll
                for (int kg = 0; kg < 4; ++kg)
                  st_shared_v4(act + (uint32_t)(col0 / 8 + kg) * 2048u + r * 16, u[4 * kg], u[4 * kg + 1],
                               u[4 * kg + 2], u[4 * kg + 3]);
              } else if (g == 8) {  // dense_8 is linear (model.py:377-378)
#pragma unroll
                for (int kg = 0; kg < 4; ++kg)
                  st_shared_v4(act + (uint32_t)(col0 / 8 + kg) * 2048u + r * 16, pack_bf16(v[8 * kg], v[8 * kg + 1]),
                               pack_bf16(v[8 * kg + 2], v[8 * kg + 3]), pack_bf16(v[8 * kg + 4], v[8 * kg + 5]),
                               pack_bf16(v[8 * kg + 6], v[8 * kg + 7]));
              } else {
#pragma unroll
                for (int kg = 0; kg < 4; ++kg)
                  st_shared_v4(act + (uint32_t)(col0 / 8 + kg) * 2048u + r * 16,
                               pack_bf16_relu(v[8 * kg], v[8 * kg + 1]), pack_bf16_relu(v[8 * kg + 2], v[8 * kg + 3]),
                               pack_bf16_relu(v[8 * kg + 4], v[8 * kg + 5]),
                               pack_bf16_relu(v[8 * kg + 6], v[8 * kg + 7]));
              }
            }
            const uint32_t bar_head = sbase + L::kBarHead + 8 * s;
            if (g == 7) {
              // sigma = ReLU(h7 . w + b) (model.py:374-375): quarter sums in FP32
              float *part = reinterpret_cast<float *>(smem + kEncOff + s * L::kEncBytes + L::kSigPartOff);
              part[cq * 128 + r] = sig;
              head_arrive(s);
              // h7 is written: dense_8 may start while the quarter sums meet
              // (they sit in the enc region's upper half, which nothing
              // rewrites before the next tile's encoding)
              operands_ready(s);
              if (cq == 0) {
                // the head barrier completes twice per tile (sigma, rgb): parity 0, then 1
                if (!__all_sync(0xffffffffu, wait_bar(bar_head, 0, abort_flag, err))) {
                  ok = false;
                  break;
                }
                if (valid[s])
                  sigma_out[prow[s]] =
                      fmaxf(((part[r] + part[128 + r]) + (part[256 + r] + part[384 + r])) + table[kSigmaBOff], 0.0f);
              }
            }
            if (g == 8) {
              // enc_dir into the enc region (enc_xyz was last read by dense_5).
              const long long dr = prow[s] / rpd;
              float d[3];
#pragma unroll
              for (int c = 0; c < 3; ++c) d[c] = dirs[dr * 3 + c];
              uint16_t *const tt = nullptr;  // (the tape writer stores it with h8)
              if (cq == 0)
                write_enc_dir_q<0, F8>(enc, r, d, tt);
              else if (cq == 1)
                write_enc_dir_q<1, F8>(enc, r, d, tt);
              else if (cq == 2)
                write_enc_dir_q<2, F8>(enc, r, d, tt);
              else
                write_enc_dir_q<3, F8>(enc, r, d, tt);
            }
            if (g == 9) {
              // rgb = sigmoid(h9 . W + b) (model.py:385-386): quarter sums in FP32
              float *part = reinterpret_cast<float *>(smem + kActOff + s * L::kActBytes);
#pragma unroll
              for (int c = 0; c < 3; ++c) part[(c * 4 + cq) * 128 + r] = rgb_acc[c];
              head_arrive(s);
              if (cq == 0) {
                if (!__all_sync(0xffffffffu, wait_bar(bar_head, 1, abort_flag, err))) {
                  ok = false;
                  break;
                }
                if (valid[s]) {
#pragma unroll
                  for (int c = 0; c < 3; ++c) {
                    const float z = ((part[c * 512 + r] + part[c * 512 + 128 + r]) +
                                     (part[c * 512 + 256 + r] + part[c * 512 + 384 + r])) +
                                    table[kRgbBOff + c];
                    rgb_out[prow[s] * 3 + c] = 1.0f / (1.0f + expf(-z));
                  }
                }
              }
              // the enc region is free (dense_9 done); the rgb partials are
              // read before this warp's arrival lets dense_0 overwrite them
              if (has_next) start_rows(tile + t_step, s);
            } else if (g != 7) {
              operands_ready(s);
            }
          }
          accf_phase ^= 1;
        }
      }
    } else {
      // ---------------- epilogue warps (single CTA) ----------------
      const int ew = warp - 2;
      const int s = ew >> 3, hf = (ew >> 2) & 1, qd = warp & 3;
      const int r = 32 * qd + lane;  // row within the sub-tile (= TMEM lane)
      const uint32_t enc = sbase + kEncOff + s * L::kEncBytes;
      const uint32_t act = sbase + kActOff + s * L::kActBytes;
      const uint32_t trow = tmem + ((uint32_t)(32 * qd) << 16) + s * 256 + hf * 128;
      const uint32_t bar_accf = sbase + kBarAccf + 8 * s, bar_actr = sbase + kBarActr + 8 * s;
      float *sig_part = reinterpret_cast<float *>(smem + kSigPart) + s * 128;
      const uint32_t bar_head = sbase + L::kBarHead + 8 * s;
      uint32_t accf_phase = 0, head_phase = 0;
      bool ok = true;
      for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long grow = tile * kRows + s * 128 + r;
        const bool valid = grow < n;
        const long long prow = phys(valid ? grow : n - 1);
        float x[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = valid ? xyz[prow * 3 + c] : 0.0f;
        uint16_t *trow_tape = (STORE && valid) ? tape + grow * kActsLd : nullptr;
        if (hf == 0)
          write_enc_xyz<0, F8>(enc, r, x, trow_tape ? trow_tape + kActsEncXyz : nullptr);
        else
          write_enc_xyz<1, F8>(enc, r, x, trow_tape ? trow_tape + kActsEncXyz + 32 : nullptr);
        fence_proxy_async();
        tc_fence_before();
        mbar_arrive(bar_actr);
        float rgb_acc[3] = {0.f, 0.f, 0.f};
        for (int g = 0; g < kNumGemm; ++g) {
          // warp-uniform outcome, so that the warp's tcgen05.ld stay convergent
          if (!__all_sync(0xffffffffu, wait_bar(bar_accf, accf_phase, abort_flag, err))) {
            ok = false;
            break;
          }
          accf_phase ^= 1;
          tc_fence_after();
          const float *bias = table + bias_offset(g);
          float sig = 0.0f;
          if (!(g == 9 && hf == 1)) {
#pragma unroll 1
            for (int j = 0; j < 4; ++j) {
              uint32_t raw[32];
              tmem_ld32(trow + j * 32, raw);
              const int col0 = hf * 128 + j * 32;
              float v[32];
              if (F8) {
                // acc * scale[col] + bias[col] (per-output-channel weight scale)
                tmem_wait32(raw);
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                  const float4 b4 = *reinterpret_cast<const float4 *>(bias + col0 + i);
                  const float4 s4 = *reinterpret_cast<const float4 *>(scales + bias_offset(g) + col0 + i);
                  fma_f32x2(v[i], v[i + 1], __uint_as_float(raw[i]), __uint_as_float(raw[i + 1]), s4.x, s4.y, b4.x,
                            b4.y);
                  fma_f32x2(v[i + 2], v[i + 3], __uint_as_float(raw[i + 2]), __uint_as_float(raw[i + 3]), s4.z, s4.w,
                            b4.z, b4.w);
                }
              } else {
                float b[32];
#pragma unroll
                for (int i = 0; i < 32; i += 4) *reinterpret_cast<float4 *>(b + i) = *reinterpret_cast<const float4 *>(bias + col0 + i);
                tmem_wait32(raw);
#pragma unroll
                for (int i = 0; i < 32; i += 2)
                  add_f32x2(v[i], v[i + 1], __uint_as_float(raw[i]), __uint_as_float(raw[i + 1]), b[i], b[i + 1]);
              }
              if (g == 7) {
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                  const float4 w4 = *reinterpret_cast<const float4 *>(table + kSigmaWOff + col0 + i);
                  sig = fmaf(fmaxf(v[i], 0.0f), w4.x, sig);
                  sig = fmaf(fmaxf(v[i + 1], 0.0f), w4.y, sig);
                  sig = fmaf(fmaxf(v[i + 2], 0.0f), w4.z, sig);
                  sig = fmaf(fmaxf(v[i + 3], 0.0f), w4.w, sig);
                }
              }
              if (g == 9) {
                if (STORE && trow_tape) {
                  uint32_t u[16];
#pragma unroll
                  for (int i = 0; i < 16; ++i) u[i] = pack_bf16_relu(v[2 * i], v[2 * i + 1]);
                  tape_store32(trow_tape + acts_offset(9) + col0, u);
                }
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                  // rows col0+i .. col0+i+3 of the [128][3] rgb kernel: 12 floats
                  const float *wr = table + kRgbWOff + (col0 + i) * 3;
                  const float4 a4 = *reinterpret_cast<const float4 *>(wr);
                  const float4 b4 = *reinterpret_cast<const float4 *>(wr + 4);
                  const float4 c4 = *reinterpret_cast<const float4 *>(wr + 8);
                  const float w12[12] = {a4.x, a4.y, a4.z, a4.w, b4.x, b4.y, b4.z, b4.w, c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                  for (int q = 0; q < 4; ++q) {
                    const float h = fmaxf(v[i + q], 0.0f);
                    rgb_acc[0] = fmaf(h, w12[3 * q], rgb_acc[0]);
                    rgb_acc[1] = fmaf(h, w12[3 * q + 1], rgb_acc[1]);
                    rgb_acc[2] = fmaf(h, w12[3 * q + 2], rgb_acc[2]);
                  }
                }
              } else if (F8) {
                if (g == 8)  // dense_8 is linear (model.py:377-378)
                  store_row32<true, false>(act, r, col0, v);
                else
                  store_row32<true, true>(act, r, col0, v);
              } else if (STORE) {
                // BF16 operands of the next layer, to shared memory and the tape
                uint32_t u[16];
                if (g == 8) {  // dense_8 is linear (model.py:377-378)
#pragma unroll
                  for (int i = 0; i < 16; ++i) u[i] = pack_bf16(v[2 * i], v[2 * i + 1]);
                } else {
#pragma unroll
                  for (int i = 0; i < 16; ++i) u[i] = pack_bf16_relu(v[2 * i], v[2 * i + 1]);
                }
#pragma unroll
                for (int kg = 0; kg < 4; ++kg)
                  st_shared_v4(act + (uint32_t)(col0 / 8 + kg) * 2048u + r * 16, u[4 * kg], u[4 * kg + 1],
                               u[4 * kg + 2], u[4 * kg + 3]);
                if (trow_tape) tape_store32(trow_tape + acts_offset(g) + col0, u);
              } else if (g == 8) {  // dense_8 is linear (model.py:377-378)
#pragma unroll
                for (int kg = 0; kg < 4; ++kg)
                  st_shared_v4(act + (uint32_t)(col0 / 8 + kg) * 2048u + r * 16, pack_bf16(v[8 * kg], v[8 * kg + 1]),
                               pack_bf16(v[8 * kg + 2], v[8 * kg + 3]), pack_bf16(v[8 * kg + 4], v[8 * kg + 5]),
                               pack_bf16(v[8 * kg + 6], v[8 * kg + 7]));
              } else {
#pragma unroll
                for (int kg = 0; kg < 4; ++kg)
                  st_shared_v4(act + (uint32_t)(col0 / 8 + kg) * 2048u + r * 16,
                               pack_bf16_relu(v[8 * kg], v[8 * kg + 1]), pack_bf16_relu(v[8 * kg + 2], v[8 * kg + 3]),
                               pack_bf16_relu(v[8 * kg + 4], v[8 * kg + 5]),
                               pack_bf16_relu(v[8 * kg + 6], v[8 * kg + 7]));
              }
            }
          }
          if (g == 7) {
            // sigma = ReLU(h7 . w + b) (model.py:374-375), halves summed in FP32:
            // the second half's warps publish theirs behind the head barrier
            // (a bounded wait, so that an abort cannot strand a warp at it)
            if (hf == 1) {
              sig_part[r] = sig;
              __syncwarp();
              if (lane == 0) mbar_arrive(bar_head);
            } else {
              if (!__all_sync(0xffffffffu, wait_bar(bar_head, head_phase, abort_flag, err))) {
                ok = false;
                break;
              }
              head_phase ^= 1;
              if (valid) sigma_out[prow] = fmaxf(sig + sig_part[r] + table[kSigmaBOff], 0.0f);
            }
          }
          if (g == 8 && hf == 0) {
            // enc_dir into the enc region (enc_xyz was last read by dense_5).
            const long long dr = prow / rpd;
            float d[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) d[c] = dirs[dr * 3 + c];
            write_enc_dir<F8>(enc, r, d, trow_tape ? trow_tape + kActsEncDir : nullptr);
          }
          if (g == 9) {
            if (hf == 0 && valid) {
#pragma unroll
              for (int c = 0; c < 3; ++c)
                rgb_out[prow * 3 + c] = 1.0f / (1.0f + expf(-(rgb_acc[c] + table[kRgbBOff + c])));
            }
          } else {
            fence_proxy_async();
            tc_fence_before();
            mbar_arrive(bar_actr);
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (PAIR) {
    if (crank == 1 && warp == 1 && lane == 0 && t_first < ntiles) {
      // the even CTA's last commit (after every MMA on this CTA's data) has
      // reached this CTA
      uint64_t t0 = globaltimer();
      while (!mbar_try(sbase + kBarDrain, 0) && globaltimer() - t0 < 100000000ull) {
      }
      // Without a timeout every copy of this CTA was waited for by the even
      // CTA's issuer. After one (in either CTA) copies may still be in
      // flight, and they complete on the even CTA's barriers, which this CTA
      // cannot wait on: give them 100 us (copies from L2 take microseconds).
      uint32_t peer_abort;
      asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(peer_abort) : "r"(peer_addr(sbase + kAbort, 0))
                   : "memory");
      if (*abort_flag || peer_abort) {
        t0 = globaltimer();
        while (globaltimer() - t0 < 100000ull) {
        }
      }
    }
    __syncwarp();
    cluster_sync_all();  // no MMA or arrival of the pair touches either CTA any more
  }
  if (warp == 1) {
    tc_fence_after();
    if (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
#undef t_first
#undef t_step
}

}  // namespace tc

// cuTensorMapEncodeTiled, looked up once through the runtime (the library
// does not link the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  });
  return fn;
}

int encode_tensor_map_u16(CUtensorMap *map, const void *base, int rank, const unsigned long long *dims,
                          const unsigned long long *strides, const unsigned *box, bool swizzle128) {
  const EncodeTiledFn enc = encode_tiled();
  if (!enc || rank < 1 || rank > 5) return NERFGB_E_CUDA;
  cuuint64_t d[5], st[4];
  cuuint32_t b[5], e[5];
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
    e[i] = 1;
    if (i > 0) st[i - 1] = strides[i - 1];
  }
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, (cuuint32_t)rank, const_cast<void *>(base), d, st, b, e,
             CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS
             ? NERFGB_OK
             : NERFGB_E_CUDA;
}

// The pair pack's weights (kBf16WBytes from kBf16PairOff) as a 2-D tensor of
// 256-byte rows (128 16-bit elements), boxes of 64, 32 and 16 rows: every
// weight half of the pair layout starts on a row (its byte offset is a
// multiple of 256) and is one such box.
static int pair_maps(const uint8_t *packed, tc::PairMaps &m) {
  static_assert(kBf16PairOff % 1024 == 0 && kBf16WBytes % 256 == 0, "pair pack rows");
  if (reinterpret_cast<uintptr_t>(packed) % 256 != 0) return NERFGB_E_INVALID_ARG;
  const unsigned long long dims[2] = {128, (unsigned long long)(kBf16WBytes / 256)};
  const unsigned long long strides[1] = {256};
  const unsigned rows[3] = {64, 32, 16};
  for (int i = 0; i < 3; ++i) {
    const unsigned box[2] = {128, rows[i]};
    const int rc = encode_tensor_map_u16(&m.map[i], packed + kBf16PairOff, 2, dims, strides, box);
    if (rc != NERFGB_OK) return rc;
  }
  return NERFGB_OK;
}

template <int KCH, int NST, bool PP, bool TSMEM, bool F8, bool STORE = false, bool PAIR = false>
static int launch_variant(const void *packed, const float *xyz, const float *dirs, long long n, int rpd,
                          float *rgb, float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm,
                          uint16_t *tape = nullptr, unsigned long long wait_ns = tc::kWaitNs,
                          long long withhold = -1) {
  constexpr uint32_t smem = tc::Layout<TSMEM, F8>::kSmemBytes;
  static_assert(smem <= 227 * 1024, "shared memory");
  auto kern = tc::mlp_tc_kernel<KCH, NST, PP, TSMEM, F8, STORE, PAIR>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return NERFGB_E_CUDA;
  const int sms = num_sms();
  if (sms <= 0) return NERFGB_E_DEVICE;
  const uint8_t *pk = reinterpret_cast<const uint8_t *>(packed);
  if constexpr (PAIR) {
    // Cluster pairs on 512-row tiles; as many pairs as the device
    // co-schedules (one CTA per SM), at most one per tile.
    const long long ntiles = (n + 2 * tc::kRows - 1) / (2 * tc::kRows);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3((unsigned)tc::threads_of(STORE));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // Co-resident pairs of this kernel, per device (asked once per device;
    // concurrent first calls are serialised).
    static std::mutex mu;
    static std::unordered_map<int, int> pairs_of_device;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return NERFGB_E_DEVICE;
    int max_pairs;
    {
      std::lock_guard<std::mutex> lock(mu);
      auto hit = pairs_of_device.find(dev);
      if (hit == pairs_of_device.end()) {
        cfg.gridDim = dim3((unsigned)(sms / 2 * 2));
        int m = 0;
        if (cudaOccupancyMaxActiveClusters(&m, kern, &cfg) != cudaSuccess) return NERFGB_E_CUDA;
        hit = pairs_of_device.emplace(dev, m).first;
      }
      max_pairs = hit->second;
    }
    if (max_pairs < 1) return NERFGB_E_UNSUPPORTED;
    const long long pairs = ntiles < max_pairs ? (ntiles > 0 ? ntiles : 1) : max_pairs;
    cfg.gridDim = dim3((unsigned)(2 * pairs));
    tc::PairMaps maps{};
    int rc = pair_maps(pk, maps);
    if (rc != NERFGB_OK) return rc;
    if constexpr (STORE) {
      // the tape [n][kActsLd] BF16 as 3-D (8 elements, rows, 8-element
      // groups), boxes of 128 rows by 32, 8 and 4 groups (tc::PairMaps)
      if (reinterpret_cast<uintptr_t>(tape) % 16 != 0) return NERFGB_E_INVALID_ARG;
      const unsigned long long dims[3] = {8, (unsigned long long)(n > 0 ? n : 1), kActsLd / 8};
      const unsigned long long strides[2] = {(unsigned long long)kActsLd * 2, 16};
      const unsigned groups[3] = {32, 8, 4};
      for (int i = 0; i < 3; ++i) {
        const unsigned box[3] = {8, 128, groups[i]};
        if ((rc = encode_tensor_map_u16(&maps.tape[i], tape, 3, dims, strides, box)) != NERFGB_OK) return rc;
      }
    }
    if (cudaLaunchKernelEx(&cfg, kern, pk, xyz, dirs, n, rpd, rgb, sigma, err_word, rm, tape, wait_ns, withhold,
                           maps) != cudaSuccess)
      return NERFGB_E_CUDA;
    return launch_status();
  } else {
    const long long ntiles = (n + tc::kRows - 1) / tc::kRows;
    const int grid = (int)(ntiles < sms ? ntiles : sms);
    tc::PairMaps none{};  // the single-CTA kernels copy with cp.async.bulk
    kern<<<grid, tc::kThreads, smem, stream>>>(pk, xyz, dirs, n, rpd, rgb, sigma, err_word, rm, tape, wait_ns,
                                               withhold, none);
    return launch_status();
  }
}

// Ring stages of the pair kernel: kPairKch-K chunks (one N-half each per CTA),
// a whole 256-K layer. Eight stages of 32-K chunks ran 1.21 ms against 0.91
// on the 786,432-row fine pass: per-chunk barrier and copy overheads.
constexpr int kPairNst = 4;

int launch_mlp_bf16(const void *packed, const float *xyz, const float *dirs, long long n, int rpd, float *rgb,
                    float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm) {
  // Cluster pairs with 2-SM MMAs: ping-pong, 64-K chunks, each CTA's ring 4
  // stages of 16 KB N-halves (a whole 256-K layer), bias/head table read
  // through L1.
  return launch_variant<kPairKch, kPairNst, true, false, false, false, true>(packed, xyz, dirs, n, rpd, rgb, sigma,
                                                                            err_word, stream, rm);
}

int launch_mlp_bf16_train(const void *packed, const float *xyz, const float *dirs, long long n, int rpd, float *rgb,
                          float *sigma, uint16_t *tape, int *err_word, cudaStream_t stream) {
  // The inference kernel plus the tape stores (the same outputs bit for bit).
  return launch_variant<kPairKch, kPairNst, true, false, false, true, true>(packed, xyz, dirs, n, rpd, rgb, sigma,
                                                                           err_word, stream, RowMap(), tape);
}

int launch_mlp_fp8(const void *packed, const float *xyz, const float *dirs, long long n, int rpd, float *rgb,
                   float *sigma, int *err_word, cudaStream_t stream, const RowMap &rm) {
  // FP8 halves every operand: 112 KB of ring, 7 stages of 64-K chunks
  // (16 KB per bulk copy). Ping-pong: 0.68 ms on 786,432 rows against 0.83
  // for lockstep; at half the weight bytes the doubled stream fits the ring.
  return launch_variant<64, 7, true, true, true>(packed, xyz, dirs, n, rpd, rgb, sigma, err_word, stream, rm);
}

int launch_mlp_wait_test(const void *packed, bool fp8, const float *xyz, const float *dirs, long long n, int rpd,
                         float *rgb, float *sigma, int *err_word, cudaStream_t stream, unsigned long long wait_ns,
                         long long withhold) {
  // the kernels of launch_mlp_bf16 / launch_mlp_fp8 with the given wait limit and withheld chunk
  if (fp8)
    return launch_variant<64, 7, true, true, true>(packed, xyz, dirs, n, rpd, rgb, sigma, err_word, stream,
                                                   RowMap(), nullptr, wait_ns, withhold);
  return launch_variant<kPairKch, kPairNst, true, false, false, false, true>(packed, xyz, dirs, n, rpd, rgb, sigma,
                                                                            err_word, stream, RowMap(), nullptr,
                                                                            wait_ns, withhold);
}

}  // namespace nerfgb

#ifdef NERF_BOUNDS_CHECK
namespace nerfgb {
NG_BOUNDS_READER(bounds_read_mlp_tc)
}  // namespace nerfgb
#endif
