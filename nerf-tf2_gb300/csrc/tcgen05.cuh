// sm_103a PTX wrappers shared by the tensor-core kernels (mlp_tc.cu,
// gemm_tc.cu): mbarriers with bounded waits, cluster-pair helpers, bulk
// copies, tcgen05 MMA / commit / TMEM loads, shared-memory matrix and
// instruction descriptors, BF16/E4M3 packing.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <stdint.h>

#include "common.cuh"

namespace nerfgb {
namespace tc {

constexpr unsigned long long kWaitNs = 2000000000ull;  // default limit of one wait: 2 s

// The kernels keep their wait limit (ns, 64-bit) in shared memory 8 bytes
// after their abort flag (an int at an 8-byte aligned offset), so that the
// bounded waits can read it without a register of their own.
__device__ __forceinline__ unsigned long long wait_limit(volatile int *abort_flag) {
  return *reinterpret_cast<volatile unsigned long long *>(reinterpret_cast<volatile char *>(abort_flag) + 8);
}
__device__ __forceinline__ void set_wait_limit(volatile int *abort_flag, unsigned long long ns) {
  *reinterpret_cast<volatile unsigned long long *>(reinterpret_cast<volatile char *>(abort_flag) + 8) = ns;
}

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Cluster-pair helpers. The address of a variable of CTA `rank` at this
// CTA's shared offset `addr`, and an arrive on a barrier of another CTA
// (default semantics, as for local arrivals; the writer's data in shared
// memory is published to the tensor core by fence.proxy.async before).
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t peer_addr(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// 2-D tensor copy (TMA) of one box into this CTA's shared memory at dst,
// completing on the mbarrier at cluster address bar: with .cta_group::2 the
// barrier may be the pair's other CTA's (the one that issues the 2-SM MMAs
// reading this data). map: the generic address of a CUtensorMap kernel
// parameter; (x, y) the box's first element.
__device__ __forceinline__ void tma_2d_pair(uint32_t dst, const void *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// A 3-D box from shared memory at src to global memory by a tensor store
// (the box's image in shared memory: innermost dimension first), in the
// thread's bulk async-group. Writes to src by other threads must have been
// made visible to the async proxy (fence.proxy.async, then a barrier).
__device__ __forceinline__ void tma_store_3d(const void *map, uint32_t src, int c0, int c1, int c2) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(src), "r"(c0), "r"(c1), "r"(c2)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// until the thread's bulk groups have read their shared-memory sources
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// until the thread's bulk groups have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The 2-SM forms. The MMA is issued by one thread of the pair's even CTA: A
// is M/2 rows from each CTA's shared memory at the same offset (rows
// [0, M/2) from the even CTA), B is N/2 columns from each (columns [0, N/2)
// from the even CTA), and each CTA's TMEM receives its own M/2 rows of D at
// the same address. The commit arrives on the barrier at the same offset in
// both CTAs.
__device__ __forceinline__ void tc_mma_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit_pair(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
      "h"((uint16_t)3)
      : "memory");
}
template <bool PAIR>
__device__ __forceinline__ void commit_any(uint32_t bar) {
  if (PAIR)
    tc_commit_pair(bar);
  else
    tc_commit(bar);
}
__device__ __forceinline__ void tc_mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void named_sync(int id, int threads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// 32 lanes x 32 columns of FP32 from TMEM; thread t gets lane (addr.lane + t).
// The load is asynchronous until tmem_wait32, which also ties the registers
// so no use can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait32(uint32_t (&r)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                 "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                 "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
}

// (x0 + y0, x1 + y1) in one paired FP32 add (round to nearest even, as two
// FADDs).
__device__ __forceinline__ void add_f32x2(float &d0, float &d1, float x0, float x1, float y0, float y1) {
  asm("{\n.reg .b64 a, b, d;\nmov.b64 a, {%2, %3};\nmov.b64 b, {%4, %5};\nadd.rn.f32x2 d, a, b;\n"
      "mov.b64 {%0, %1}, d;\n}"
      : "=f"(d0), "=f"(d1)
      : "f"(x0), "f"(x1), "f"(y0), "f"(y1));
}

// (x0 * y0 + z0, x1 * y1 + z1) in one paired FP32 FMA (each rounded once,
// as fmaf).
__device__ __forceinline__ void fma_f32x2(float &d0, float &d1, float x0, float x1, float y0, float y1, float z0,
                                          float z1) {
  asm("{\n.reg .b64 a, b, c, d;\nmov.b64 a, {%2, %3};\nmov.b64 b, {%4, %5};\nmov.b64 c, {%6, %7};\n"
      "fma.rn.f32x2 d, a, b, c;\nmov.b64 {%0, %1}, d;\n}"
      : "=f"(d0), "=f"(d1)
      : "f"(x0), "f"(x1), "f"(y0), "f"(y1), "f"(z0), "f"(z1));
}

// Shared-memory matrix descriptor: K-major, no swizzle (layout type 0),
// descriptor version 1 at bit 46. lbo = byte stride between core matrices
// adjacent in K, sbo = byte stride between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor of kind::f8f6f4: E4M3 A and B (format 0, K-major),
// FP32 D.
__host__ __device__ constexpr uint32_t idesc_e4m3(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Four floats to four E4M3 bytes (round to nearest, saturate to +-448),
// v0 in the lowest byte.
__device__ __forceinline__ uint32_t pack_e4m3x4(float v0, float v1, float v2, float v3) {
  const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(v0, v1), __NV_SATFINITE, __NV_E4M3);
  const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(v2, v3), __NV_SATFINITE, __NV_E4M3);
  return lo | (hi << 16);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&p);
}
// max(x, 0) of both values, rounded to BF16 and packed (lo in the low half).
__device__ __forceinline__ uint32_t pack_bf16_relu(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
// 32 BF16 values (16 packed pairs) to 64 contiguous bytes of the activation
// tape (16-byte aligned).
__device__ __forceinline__ void tape_store32(uint16_t *dst, const uint32_t (&u)[16]) {
  uint4 *p = reinterpret_cast<uint4 *>(dst);
#pragma unroll
  for (int q = 0; q < 4; ++q) p[q] = make_uint4(u[4 * q], u[4 * q + 1], u[4 * q + 2], u[4 * q + 3]);
}
__device__ __forceinline__ void pack32_bf16(const float (&v)[32], uint32_t (&u)[16]) {
#pragma unroll
  for (int i = 0; i < 16; ++i) u[i] = pack_bf16(v[2 * i], v[2 * i + 1]);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// Stores v[0..32) as the K-elements [k0, k0+32) of row r of a 128-row operand
// region (K-major core matrices of 16 bytes: 8 BF16 or 16 E4M3 elements;
// element (r, k) at (k / KW) * 2048 + r * 16 + (k % KW) * E).
template <bool F8, bool RELU>
__device__ __forceinline__ void store_row32(uint32_t region, int r, int k0, float (&v)[32]) {
  if (RELU) {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i], 0.0f);
  }
  if (F8) {
#pragma unroll
    for (int g = 0; g < 2; ++g)
      st_shared_v4(region + (uint32_t)(k0 / 16 + g) * 2048u + r * 16,
                   pack_e4m3x4(v[16 * g], v[16 * g + 1], v[16 * g + 2], v[16 * g + 3]),
                   pack_e4m3x4(v[16 * g + 4], v[16 * g + 5], v[16 * g + 6], v[16 * g + 7]),
                   pack_e4m3x4(v[16 * g + 8], v[16 * g + 9], v[16 * g + 10], v[16 * g + 11]),
                   pack_e4m3x4(v[16 * g + 12], v[16 * g + 13], v[16 * g + 14], v[16 * g + 15]));
  } else {
#pragma unroll
    for (int g = 0; g < 4; ++g)
      st_shared_v4(region + (uint32_t)(k0 / 8 + g) * 2048u + r * 16, pack_bf16(v[8 * g], v[8 * g + 1]),
                   pack_bf16(v[8 * g + 2], v[8 * g + 3]), pack_bf16(v[8 * g + 4], v[8 * g + 5]),
                   pack_bf16(v[8 * g + 6], v[8 * g + 7]));
  }
}

// Bounded wait: returns false (after flagging) on timeout or abort.
__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err) {
  if (mbar_try(bar, parity)) return true;
  uint64_t t0 = globaltimer();
  while (true) {
    if (mbar_try(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > wait_limit(abort_flag)) {
      atomicExch(err, NERFGB_E_TIMEOUT);
      *abort_flag = 1;
      return false;
    }
  }
}


}  // namespace tc
}  // namespace nerfgb
