// Batched DB x queries product over Z_{2^32} on the 5th-generation tensor
// cores (tcgen05 + TMEM + TMA), exact.
//
// Reference: the per-request GEMVs Matrix<uint16_t>::Multiply and
// Matrix<int32_t>::Multiply (crypto/matrix.cc:261-374) called by
// PirServer::ProcessResponse (crypto/pir/server/pir_server.cc:215-248). A
// batch of B requests turns the two GEMVs into one GEMM:
//   out[q][r] = sum_c DB[r][c] * q1[q][c] + sum_j P[r][j] * y_g[q][j]  mod 2^32
//
// Exactness with fp16 operands and fp32 accumulators. Every operand is split
// into balanced base-256 digits, exact fp16 values:
//   * a query word q (mod 2^32) into y0..y3 in [-128, 127], with
//     q = y0 + 2^8 y1 + 2^16 y2 + 2^24 y3 mod 2^32 (the top carry drops);
//   * a pack entry (its u32 two's complement, mod 2^32) into p0..p3 likewise;
//   * a DB entry x in [0, 2^16) as x - 2^15 = x0 + 2^8 x1 with x0 in
//     [-128, 127], x1 in [-128, 128]; the offset comes back as
//     2^15 * sum_c q1[c], one word per request added in the epilogue.
// Only digit pairs whose weight 2^(8s), s = i + j, is below 2^32 matter. The
// accumulator of a CTA holds four blocks of 64 fp32 columns, block s
// collecting every pair of weight 2^(8s):
//   MMA(X0, [Y0 Y1 Y2 Y3]) -> blocks 0..3,  MMA(X1, [Y0 Y1 Y2]) -> blocks 1..3
// so each accumulator element receives at most two digit products per K
// index, each of magnitude <= 128 * 128 = 2^14. A unit of K = 128 therefore
// keeps every partial sum v in [-2^22, 2^22]: exact fp32 integers, decoded
// exactly as bits(v + 1.5 * 2^23) - 0x4B400000 (v + 1.5 * 2^23 lies in
// [2^23, 2^24], where consecutive integers are consecutive encodings) before
// being added, shifted by 8s, into a u32 register accumulator. Signed digits
// halve the decode work per MAC against unsigned bytes, whose K = 64 units
// already reach 2^23. The pack matrix runs as two units per K block (p0,p1
// like the DB; then p2 -> blocks 2..3 and p3 -> block 3).
//
// Kernel structure. Each CTA covers two 128-row blocks that share one
// 64-request tile (fewer operand bytes moved from L2 per MAC). Every operand
// tile has 128-byte rows (128-byte swizzle): an A box row holds two digit
// planes of a 32-wide K chunk, a request row 64 K of one plane. Shared
// memory (224 KB) holds one ring of A boxes per row block (4 x 16 KB, one
// per K=32 step of a unit, filled and released in pairs) and 3 request
// slots of 32 KB (K = 64 x 4 planes x 64 requests). The MMA pipe runs row
// block 0 over a unit, then row block 1, so a row block's boxes are
// refilled a whole row-block pass before they are read again. 12 warps:
//   warp 0     TMA producer, issuing loads in the order the MMA pipe frees
//              their buffers
//   warp 1     MMA issuer: one thread issues tcgen05.mma (M=128, K=16,
//              N=256/192 or 128/64) with descriptors that are the ring
//              base plus compile-time offsets, row block 0 into TMEM
//              columns 0..255, then row block 1 into columns 256..511, so
//              one epilogue group drains a block while the other is filled
//   warp 2     TMEM allocator (512 columns)
//   warps 4-7  epilogue for row block 0, warps 8-11 for row block 1:
//              tcgen05.ld, decode, accumulate
// The K range can be split over several CTAs (split-K) to balance the grid
// over the SMs; split partial sums are added with 32-bit atomics, which are
// exact mod 2^32. Every mbarrier wait is bounded; on a timeout the kernel
// raises an error flag, drains its own copies with bounded waits, frees TMEM
// and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <type_traits>

#include "internal.h"
#include "limb_gemm.h"

namespace inspire {
namespace {

constexpr int kBlockRows = 128;    // rows per MMA (M)
constexpr int kRowBlocks = 2;      // row blocks per CTA sharing a request tile
constexpr int kTileRows = kBlockRows * kRowBlocks;
constexpr int kStageK = 32;        // K per A stage (two planes: 128-byte rows)
constexpr int kUnitK = 128;        // K per exact accumulation unit
constexpr int kStagesPerUnit = kUnitK / kStageK;
constexpr int kATileBytes = kBlockRows * kStageK * 2;      // 8 KB per plane
constexpr int kABoxBytes = 2 * kATileBytes;                // both planes: 16 KB
// One ring of A boxes per row block, one box per step of a unit (so the box
// of step h is h), filled and released in pairs of steps, and a ring of
// request slots: the digit planes load K = 64 at a time (128-byte rows),
// slot n serving steps 2n and 2n + 1 of both row blocks.
constexpr int kAStages = kStagesPerUnit;
constexpr int kAPairs = kAStages / 2;
constexpr int kARingBytes = kAStages * kABoxBytes;         // 64 KB per row block
constexpr int kBSlotK = 2 * kStageK;
constexpr int kBRows = 256;        // request-tile rows of the B operand
constexpr int kBSlotBytes = kBRows * kBSlotK * 2;          // 32 KB
constexpr int kBSlots = 3;
constexpr int kBHalves = kStagesPerUnit / 2;               // request slots per unit
constexpr int kRingBytes = kRowBlocks * kARingBytes + kBSlots * kBSlotBytes;  // 224 KB
constexpr int kThreads = 384;
// The converting form (a u16 DB read as it is stored): a fourth warpgroup
// (warps 12-15) turns each raw 128-row x 32-column u16 tile, loaded by TMA
// into a staging ring, into its A box's two fp16 digit planes.
constexpr int kConvThreads = 128;
constexpr int kThreadsConv = kThreads + kConvThreads;
constexpr int kRawTileBytes = kBlockRows * kStageK * 2;    // 8 KB
// Register split of the converting form, per warpgroup (128 threads each):
// producer / MMA / allocator, two epilogue groups, converter. The launch
// holds 512 threads x 128 registers = 65536; the split sums to the same.
constexpr int kRegsCtl = 56, kRegsEpi = 176, kRegsConv = 104;
static_assert(kRegsCtl + 2 * kRegsEpi + kRegsConv == 4 * 128,
              "register split of the converting form");
constexpr int kTmemCols = 512;     // one 256-column accumulator per row block
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kBarrierBytes = 512;
constexpr size_t kSmemBytes = kRingBytes + 1024 + kBarrierBytes;
static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");

// Shared-memory plan of one kernel form within the kRingBytes budget: the
// two A rings, the request slots (NQ planes x TQ requests x 64 K of fp16;
// three, or two for full tiles in the converting form) and, in the
// converting form, a staging ring of raw u16 tiles (8 KB each, as many as
// fit: 9 with narrow request tiles) that
// the producer fills ahead of the converter, so that a raw tile is already
// on chip when its box frees up.
// Full request tiles leave no room for staging: their converting form loads
// each raw tile into the first half of its own box (once the MMA pipe has
// freed it) and the converter expands it in place.
constexpr int kMaxStages = 16;  // staging slots the barrier region provides for
template <int NQ, bool CONV, int TQ>
struct RingPlan {
  static constexpr int kBSlotB = NQ * TQ * kBSlotK * 2;
  static constexpr bool kStaged = CONV && NQ * TQ < kBRows;
  static constexpr int kBS = kBSlots;
  static constexpr int kBBase = kRowBlocks * kARingBytes;
  static constexpr int kStageBase = kBBase + kBS * kBSlotB;
  static constexpr int kFree = (kRingBytes - kStageBase) / kRawTileBytes;
  static constexpr int kStages = kStaged ? (kFree < kMaxStages ? kFree : kMaxStages) : 0;
  static_assert(!kStaged || kStages >= 4, "raw staging ring");
  // The converter warps' parity waits on the staging slots are exact when
  // each warp owns its slots (a multiple of 4) or, waiting for the freed box
  // first, when the ring holds at least two row blocks' tiles (8).
  static_assert(!kStaged || kStages % 4 == 0 || kStages >= 8, "staging ring size");
  static_assert(kStageBase + kStages * kRawTileBytes <= kRingBytes, "ring budget");
};

// Request words split into NQ balanced base-256 digit planes: NQ = 4 for
// Z_2^32 words, 8 for Z_2^64. A full request tile holds TQ = 256 / NQ
// requests, so its B operand has 256 rows (NQ planes x TQ requests), the DB
// / low-pack MMA has N = 256 and the accumulator of a row block NQ weight
// blocks of TQ columns (256 TMEM columns). The narrow tile (kNarrowTQ = 16
// requests) cuts the MMA work of small batches by 256 / (16 NQ): the DB is
// then streamed once per 16 requests instead of once per 64 (or 32) padded
// ones, with N = 16 NQ, ..., 16 (NQ - 3), all multiples of 16 as M = 128
// needs.
template <int NQ>
struct LimbShape {
  using Acc = typename std::conditional<NQ == 4, uint32_t, unsigned long long>::type;
};
constexpr int kNarrowTQ = 16;

// ------------------------------------------------------------------ PTX --
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false on timeout or when another role has raised the flag.
// With err == nullptr (draining after an error) it only bounds the wait.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          int* err) {
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u) {
      if (err != nullptr && *reinterpret_cast<volatile int*>(err) != 0) {
        return false;
      }
      if (i > kSpinLimit) {
        if (err != nullptr) atomicExch(err, 1);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map,
                                            uint64_t* bar, void* dst, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::"
      "bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(bar)), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t cols) {
  asm volatile(
      "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
          smem_addr(dst)),
      "r"(cols)
      : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
                   : "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
               "r"(cols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
      "[%0];" ::"r"(smem_addr(bar))
      : "memory");
}

#define INSPIRE_R32(i) "=r"(v[i])
__device__ __forceinline__ void tmem_ld_x32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : INSPIRE_R32(0), INSPIRE_R32(1), INSPIRE_R32(2), INSPIRE_R32(3),
        INSPIRE_R32(4), INSPIRE_R32(5), INSPIRE_R32(6), INSPIRE_R32(7),
        INSPIRE_R32(8), INSPIRE_R32(9), INSPIRE_R32(10), INSPIRE_R32(11),
        INSPIRE_R32(12), INSPIRE_R32(13), INSPIRE_R32(14), INSPIRE_R32(15),
        INSPIRE_R32(16), INSPIRE_R32(17), INSPIRE_R32(18), INSPIRE_R32(19),
        INSPIRE_R32(20), INSPIRE_R32(21), INSPIRE_R32(22), INSPIRE_R32(23),
        INSPIRE_R32(24), INSPIRE_R32(25), INSPIRE_R32(26), INSPIRE_R32(27),
        INSPIRE_R32(28), INSPIRE_R32(29), INSPIRE_R32(30), INSPIRE_R32(31)
      : "r"(taddr));
}
#undef INSPIRE_R32

#define INSPIRE_R16(i) "=r"(v[i])
__device__ __forceinline__ void tmem_ld_x16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : INSPIRE_R16(0), INSPIRE_R16(1), INSPIRE_R16(2), INSPIRE_R16(3),
        INSPIRE_R16(4), INSPIRE_R16(5), INSPIRE_R16(6), INSPIRE_R16(7),
        INSPIRE_R16(8), INSPIRE_R16(9), INSPIRE_R16(10), INSPIRE_R16(11),
        INSPIRE_R16(12), INSPIRE_R16(13), INSPIRE_R16(14), INSPIRE_R16(15)
      : "r"(taddr));
}
#undef INSPIRE_R16

// tcgen05.ld of N consecutive 32-bit columns (N = 16 or 32) of the warp's
// 32 TMEM lanes.
template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&v)[N]) {
  if constexpr (N == 32) {
    tmem_ld_x32(taddr, v);
  } else {
    static_assert(N == 16, "tcgen05.ld width");
    tmem_ld_x16(taddr, v);
  }
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Generic-proxy shared-memory writes become visible to the async proxy (the
// tensor core's operand reads).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint4 lds128(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}

__device__ __forceinline__ void sts128(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x),
               "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

// Two u16 DB entries x (one per 16-bit half of w) -> their balanced digits
// x - 2^15 = x0 + 2^8 x1 as half2 pairs. With b0, b1 the bytes of x:
// x0 + 128 = b0 ^ 0x80 in [0, 255] and x1 + 128 = b1 + (b0 >> 7) in
// [0, 256]; 0x6400 | v is the fp16 encoding of 1024 + v for v < 1024, so
// one fp16 subtraction of 1152 = 1024 + 128 gives each digit exactly.
__device__ __forceinline__ void u16_digits(uint32_t w, uint32_t& d0,
                                           uint32_t& d1) {
  const uint32_t h0 = (w & 0x00FF00FFu) ^ 0x64806480u;
  const uint32_t h1 = __byte_perm(w, 0u, 0x4341) + ((w >> 7) & 0x00010001u) +
                      0x64006400u;
  const __half2 off = __halves2half2(__ushort_as_half(0x6480),
                                     __ushort_as_half(0x6480));
  const __half2 x0 = __hsub2(*reinterpret_cast<const __half2*>(&h0), off);
  const __half2 x1 = __hsub2(*reinterpret_cast<const __half2*>(&h1), off);
  d0 = *reinterpret_cast<const uint32_t*>(&x0);
  d1 = *reinterpret_cast<const uint32_t*>(&x1);
}

// Instruction descriptor of kind::f16: fp16 A/B, fp32 D, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int n, int m) {
  return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

struct LimbArgs {
  int rows;          // R (multiple of 256)
  int n_db_units;    // DB columns / kUnitK
  int n_pk_blocks;   // pack columns / kUnitK
  int qcap;          // request rows per byte plane in the request maps
  int batch;         // valid requests
  int ksplit;        // CTAs sharing one (row pair, request tile)
  int64_t out_stride;
};

__device__ __forceinline__ int unit_kind(int u, int n_db_units) {
  return u < n_db_units ? 0 : 1 + ((u - n_db_units) & 1);
}

// Shared-memory matrix descriptors, K-major and swizzled: bits 0-13 the
// address >> 4, 16-29 LBO >> 4 (1: unused when swizzled), 32-45 SBO >> 4
// (the distance of 8-row groups), bit 46 the version, 61-63 the swizzle.
// Every operand tile has 128-byte rows (128-byte swizzle, SBO 1024): an A
// row holds two digit planes of a 32-wide K chunk, a request row 64 K of one
// plane. The upper word is therefore one constant; the lower word is
// (address >> 4) | 1 << 16, so every descriptor of the ring is a fixed
// offset from the lower word of the ring base.
constexpr uint32_t kDescHi128 = (1024 >> 4) | (1u << 14) | (2u << 29);

__device__ __forceinline__ void mma_f16_w(uint32_t d_tmem, uint32_t a_lo,
                                          uint32_t b_lo, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
      "mov.b64 da, {%1, %2};\n\t"
      "mov.b64 db, {%3, %4};\n\t"
      "setp.ne.b32 p, %6, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %5, p;\n\t}" ::"r"(d_tmem),
      "r"(a_lo), "r"(kDescHi128), "r"(b_lo), "r"(kDescHi128), "r"(idesc),
      "r"(accumulate)
      : "memory");
}

// Where the operands of unit u live: the A map and its x coordinate for
// step 0 (A rows interleave the digit planes per 32-wide K chunk: the DB as
// [x0 | x1], the pack matrix as [p0 | p1 | p2 | p3]), the request map and
// its x for step 0, and how many request planes the unit reads.
struct UnitSrc {
  const CUtensorMap* am;
  const CUtensorMap* bm;
  int ax, a_step, bx, nb;
  int kind;  // 0: DB unit, 1 / 2: low / high pack planes
  int rx;    // DB column of step 0 (raw u16 tiles of the converting form)
};

template <int NW>
__device__ __forceinline__ UnitSrc unit_src(int u, int n_db_units,
                                            const CUtensorMap* tm_db,
                                            const CUtensorMap* tm_pk,
                                            const CUtensorMap* tm_q,
                                            const CUtensorMap* tm_y) {
  const int kind = unit_kind(u, n_db_units);
  const int kb = kind == 0 ? u : (u - n_db_units) >> 1;
  UnitSrc r;
  r.am = kind == 0 ? tm_db : tm_pk;
  r.bm = kind == 0 ? tm_q : tm_y;
  r.a_step = kind == 0 ? 2 * kStageK : 4 * kStageK;
  r.ax = kb * kStagesPerUnit * r.a_step + (kind == 2 ? 2 * kStageK : 0);
  r.bx = kb * kUnitK;
  r.nb = kind == 2 ? NW - 2 : NW;
  r.kind = kind;
  r.rx = kb * kUnitK;
  return r;
}

// CONV = false: the DB comes as resident fp16 digit planes (tm_db). CONV =
// true: the DB comes as stored, u16 (tm_raw), and the converter warpgroup
// writes each A box's digit planes from its raw tile (pack units keep
// their planes in both forms). NW <= NQ: the weight blocks computed, so the
// products are exact mod 2^(8 NW) (NW = 7 when the caller reads only the
// low 56 bits of a Z_2^64 word: q <= 2^56, LowBits after the product).
template <int NQ, bool CONV, int TQ, int NW = NQ>
__global__ void __launch_bounds__(CONV ? kThreadsConv : kThreads, 1)
limb_gemm_kernel(const __grid_constant__ CUtensorMap tm_db,
                 const __grid_constant__ CUtensorMap tm_raw,
                 const __grid_constant__ CUtensorMap tm_pk,
                 const __grid_constant__ CUtensorMap tm_q,
                 const __grid_constant__ CUtensorMap tm_y, LimbArgs a,
                 const typename LimbShape<NQ>::Acc* __restrict__ qsum,
                 typename LimbShape<NQ>::Acc* __restrict__ out, int* __restrict__ err) {
  using Acc = typename LimbShape<NQ>::Acc;
  constexpr int kTileQ = TQ;
  constexpr int kBPlaneBytes = TQ * kBSlotK * 2;  // rows of 128 bytes
  static_assert(NQ * TQ <= kBRows && ((NQ - 3) * TQ) % 16 == 0 && TQ % 16 == 0,
                "request tile: N of every MMA a multiple of 16, at most 256");
  static_assert(NW <= NQ && NW >= 4 && ((NW - 3) * TQ) % 16 == 0, "weight blocks");
  using Plan = RingPlan<NQ, CONV, TQ>;
  constexpr int kBS = Plan::kBS;            // request slots
  constexpr int kBSlotB = Plan::kBSlotB;    // bytes per request slot
  constexpr int kNS = Plan::kStages;        // raw staging slots (converting form)
  constexpr bool kStaged = Plan::kStaged;   // else raw tiles convert in place
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* a_full = reinterpret_cast<uint64_t*>(smem + kRingBytes);  // [rb][pair]
  uint64_t* a_empty = a_full + kRowBlocks * kAPairs;
  uint64_t* b_full = a_empty + kRowBlocks * kAPairs;                     // [slot]
  uint64_t* b_empty = b_full + kBSlots;
  uint64_t* acc_full = b_empty + kBSlots;
  uint64_t* acc_empty = acc_full + kRowBlocks;
  uint64_t* mma_done = acc_empty + kRowBlocks;
  // Staged: st_full / st_empty per staging slot. In place: st_full[pair]
  // is the pair's raw-tiles-landed barrier.
  uint64_t* st_full = mma_done + 1;
  uint64_t* st_empty = st_full + kMaxStages;
  // Staged: the converter warps are done with the DB units (one arrival
  // each).
  uint64_t* conv_done = st_empty + kMaxStages;
  uint32_t* tmem_base_slot = reinterpret_cast<uint32_t*>(conv_done + 1);
  static_assert((3 * kRowBlocks * 2 + 2 * kBSlots + 2 + 2 * kMaxStages) * 8 + 4 <= kBarrierBytes,
                "barrier region");

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int nqt = (a.batch + kTileQ - 1) / kTileQ;
  // CTA order: request tile fastest (the tiles of a row pair read the same
  // A boxes at about the same time), then row pair, then K slice: the
  // resident CTAs all read one K slice of the request planes, which stays
  // in L2 while every row pair passes over it.
  const int n_pairs = a.rows / kTileRows;
  const int qt = blockIdx.x % nqt;
  const int rest = blockIdx.x / nqt;
  const int ks = rest / n_pairs;
  const int row0 = (rest % n_pairs) * kTileRows;
  const int q0 = qt * kTileQ;
  const int n_units = a.n_db_units + 2 * a.n_pk_blocks;
  const int per = (n_units + a.ksplit - 1) / a.ksplit;
  const int u0 = ks * per;
  const int nu = max(0, min(n_units, u0 + per) - u0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kRowBlocks * kAPairs; ++s) {
      // The converting form fills a DB box pair from two converter warps
      // (one arrival each); the producer's pack-unit loads arrive twice.
      mbar_init(&a_full[s], CONV ? 2 : 1);
      mbar_init(&a_empty[s], 1);
    }
    for (int s = 0; s < kBS; ++s) {
      mbar_init(&b_full[s], 1);
      mbar_init(&b_empty[s], 1);
    }
    for (int b = 0; b < kRowBlocks; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);
    }
    mbar_init(mma_done, 1);
    mbar_init(conv_done, kConvThreads / 32);
    for (int s = 0; s < (kStaged ? kNS : kRowBlocks * kAPairs); ++s) {
      mbar_init(&st_full[s], 1);
      mbar_init(&st_empty[s], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) tmem_alloc(tmem_base_slot, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_base_slot;

  // The MMA pipe runs row block 0 over a unit, then row block 1 over it. A
  // box pair (rb, p) is refilled once row block rb has used it, a whole
  // row-block pass before it is read again; request half n of unit i (steps
  // 2n, 2n+1) lives in slot (kBHalves * i + n) % kBSlots, refilled after
  // row block 1 has read its previous half.
  // In the converting form registers move from the control and converter
  // warpgroups to the two epilogue groups (kRegsCtl / kRegsEpi /
  // kRegsConv), each warpgroup at the top of its role.
  if (warp < 4) {
  if constexpr (CONV) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kRegsCtl));
  }
  if (warp == 0 && lane == 0) {
    // ---------------------------------------------------- TMA producer --
    // Loads go out in the order the MMA pipe frees their buffers: the row
    // block 0 boxes of the unit, then per pair its request half and its row
    // block 1 boxes.
    int a_last[kRowBlocks * kAPairs];
    bool a_raw[kRowBlocks * kAPairs];  // in place: last load was raw tiles
    int b_last[kBSlots];
    int st_last[kMaxStages];
    for (int s = 0; s < kRowBlocks * kAPairs; ++s) {
      a_last[s] = -1;
      a_raw[s] = false;
    }
    for (int s = 0; s < kBSlots; ++s) b_last[s] = -1;
    for (int s = 0; s < kMaxStages; ++s) st_last[s] = -1;
    bool ok = true;
    bool conv_seen = false;  // staged: conv_done observed
    int seq = 0;  // raw tiles issued (converting form), in the MMA's box order
    auto load_pair = [&](int rb, int p, const UnitSrc& src, int i) {
      if constexpr (kStaged) {
        if (src.kind == 0) {
          // Raw u16 tiles into the staging ring; the converter writes the
          // boxes once the MMA pipe has freed them.
          for (int hh = 0; hh < 2; ++hh, ++seq) {
            const int j = seq % kNS;
            if (!mbar_wait(&st_empty[j], ((seq / kNS) & 1) ^ 1, err)) return false;
            mbar_expect_tx(&st_full[j], kRawTileBytes);
            tma_load_2d(&tm_raw, &st_full[j], smem + Plan::kStageBase + j * kRawTileBytes,
                        src.rx + (2 * p + hh) * kStageK, row0 + rb * kBlockRows);
            st_last[j] = seq;
          }
          return true;
        }
        // A pack unit's boxes: this thread waited on no A barrier during
        // the DB units, and a parity wait cannot tell phases two apart, so
        // it first waits until the converter warps are done with the DB
        // units (the MMA pipe has then freed all but the last DB unit's
        // boxes, and the wait below is for the next phase). With three
        // request slots the request-slot waits already keep this thread
        // within one unit of the MMA pipe; this wait does not depend on
        // that depth.
        if (!conv_seen) {
          if (!mbar_wait(conv_done, 0, err)) return false;
          conv_seen = true;
        }
      }
      const int s = rb * kAPairs + p;
      if (!mbar_wait(&a_empty[s], (i & 1) ^ 1, err)) return false;
      if constexpr (CONV && !kStaged) {
        if (src.kind == 0) {
          // Raw u16 tiles into the first half of each box of the pair.
          mbar_expect_tx(&st_full[s], 2 * kRawTileBytes);
          for (int hh = 0; hh < 2; ++hh) {
            const int h = 2 * p + hh;
            tma_load_2d(&tm_raw, &st_full[s], smem + rb * kARingBytes + h * kABoxBytes,
                        src.rx + h * kStageK, row0 + rb * kBlockRows);
          }
          a_last[s] = i;
          a_raw[s] = true;
          return true;
        }
      }
      if (CONV) mbar_arrive(&a_full[s]);
      mbar_expect_tx(&a_full[s], 2 * kABoxBytes);
      for (int hh = 0; hh < 2; ++hh) {
        const int h = 2 * p + hh;
        tma_load_2d(src.am, &a_full[s], smem + rb * kARingBytes + h * kABoxBytes,
                    src.ax + h * src.a_step, row0 + rb * kBlockRows);
      }
      a_last[s] = i;
      a_raw[s] = false;
      return true;
    };
    for (int i = 0; i < nu && ok; ++i) {
      const UnitSrc src = unit_src<NW>(u0 + i, a.n_db_units, &tm_db, &tm_pk, &tm_q, &tm_y);
      for (int p = 0; p < kAPairs && ok; ++p) ok = load_pair(0, p, src, i);
      for (int p = 0; p < kAPairs && ok; ++p) {
        const int n = kBHalves * i + p;
        const int slot = n % kBS;
        if (!mbar_wait(&b_empty[slot], ((n / kBS) & 1) ^ 1, err)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&b_full[slot], src.nb * kBPlaneBytes);
        unsigned char* bs = smem + Plan::kBBase + slot * kBSlotB;
        for (int j = 0; j < src.nb; ++j) {
          tma_load_2d(src.bm, &b_full[slot], bs + j * kBPlaneBytes, src.bx + p * kBSlotK,
                      j * a.qcap + q0);
        }
        b_last[slot] = n;
        ok = load_pair(1, p, src, i);
      }
    }
    // Drain: every copy this thread issued has landed before the CTA exits.
    for (int s = 0; s < kRowBlocks * kAPairs; ++s) {
      if (a_last[s] >= 0) {
        mbar_wait(a_raw[s] ? &st_full[s] : &a_full[s], a_last[s] & 1, nullptr);
      }
    }
    for (int s = 0; s < kBS; ++s) {
      if (b_last[s] >= 0) mbar_wait(&b_full[s], (b_last[s] / kBS) & 1, nullptr);
    }
    for (int s = 0; s < kNS; ++s) {
      if (st_last[s] >= 0) {
        mbar_wait(&st_full[s], (st_last[s] / (kNS > 0 ? kNS : 1)) & 1, nullptr);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ------------------------------------------------------ MMA issuer --
    // The A descriptors are the ring base plus compile-time offsets and the
    // request descriptors one slot offset per half: straight-line MMAs,
    // which keep the one issuing thread ahead of the tensor pipe. The ring
    // waits need no tcgen05 fence (the copies and the MMAs are both in the
    // async proxy, ordered by the mbarrier); the accumulator hand-off does.
    // N of the four MMA shapes: the NW request planes that reach a
    // computed weight block (DB x0, pack p0), one fewer (x1, p1), and for
    // the high pack planes NW-2 (p2), NW-3 (p3).
    constexpr uint32_t id_n0 = instr_desc(NW * kTileQ, kBlockRows);
    constexpr uint32_t id_n1 = instr_desc((NW - 1) * kTileQ, kBlockRows);
    constexpr uint32_t id_n2 = instr_desc((NW - 2) * kTileQ, kBlockRows);
    constexpr uint32_t id_n3 = instr_desc((NW - 3) * kTileQ, kBlockRows);
    const uint32_t lo0 = (smem_addr(smem) >> 4) | (1u << 16);
    bool ok = true;
    for (int i = 0; i < nu && ok; ++i) {
      // DB and low pack units: x0 * [y0..y_{NW-1}] -> weight blocks
      // 0..NW-1, then x1 * [y0..y_{NW-2}] -> blocks 1..NW-1; high pack
      // units: p2 * [y0..y_{NW-3}] -> blocks 2.., then p3 -> blocks 3..
      const bool high = unit_kind(u0 + i, a.n_db_units) == 2;
      const uint32_t id_0 = high ? id_n2 : id_n0, id_1 = high ? id_n3 : id_n1;
      const uint32_t c_0 = high ? 2u * kTileQ : 0u, c_1 = high ? 3u * kTileQ : 1u * kTileQ;
      int slot[kBHalves];
      uint32_t b_lo[kBHalves];
#pragma unroll
      for (int p = 0; p < kBHalves; ++p) {
        slot[p] = (kBHalves * i + p) % kBS;
        b_lo[p] = lo0 + ((Plan::kBBase + slot[p] * kBSlotB) >> 4);
      }
#pragma unroll
      for (int rb = 0; rb < kRowBlocks; ++rb) {
        ok = ok && mbar_wait(&acc_empty[rb], (i & 1) ^ 1, err);
        tc_fence_after();
        const uint32_t d = tmem + rb * 256;
#pragma unroll
        for (int p = 0; p < kAPairs; ++p) {
          if (rb == 0) {
            const int n = kBHalves * i + p;
            ok = ok && mbar_wait(&b_full[slot[p]], (n / kBS) & 1, err);
          }
          ok = ok && mbar_wait(&a_full[rb * kAPairs + p], i & 1, err);
          if (ok) {
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
              const int h = 2 * p + hh;
              const uint32_t ab = lo0 + ((rb * kARingBytes + h * kABoxBytes) >> 4);
              // Odd steps read the second 64 bytes of the request rows.
              const uint32_t bs = b_lo[p] + ((hh * 64) >> 4);
#pragma unroll
              for (int kk = 0; kk < kStageK / 16; ++kk) {
                // An A box: 128 rows of 128 bytes, plane 0 in the first 64
                // bytes of each row, plane 1 in the last.
                const uint32_t a0 = ab + ((kk * 32) >> 4);
                const uint32_t bq = bs + ((kk * 32) >> 4);
                mma_f16_w(d + c_0, a0, bq, id_0, (h | kk) != 0 ? 1u : 0u);
                mma_f16_w(d + c_1, a0 + (64 >> 4), bq, id_1, 1u);
              }
            }
            mma_commit(&a_empty[rb * kAPairs + p]);
            if (rb == kRowBlocks - 1) mma_commit(&b_empty[slot[p]]);
          }
        }
        if (ok) mma_commit(&acc_full[rb]);
      }
    }
    mma_commit(mma_done);
    mbar_wait(mma_done, 0, nullptr);
  }
  } else if (CONV && warp >= 12) {
    if constexpr (CONV) {
      asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kRegsConv));
    }
    // ------------------------------------------------------- converter --
    // Converter warp w (0..3) owns box w of every DB unit's step ring, in
    // the order the MMA pipe reads the boxes: row block 0, then row block
    // 1. Warps 0 and 1 fill box pair 0, warps 2 and 3 pair 1, so four boxes
    // are converted at once and each pair's a_full completes on its two
    // warps' arrivals. Staged (narrow tiles): the box's raw tile is staging
    // slot seq % kNS, where seq = 8 i + 4 rb + w counts the DB boxes in the
    // producer's order; in place (full tiles): the first half of the box.
    // Per box: lane 0 waits (bounded) for the raw tile (staged: first for
    // the MMA pipe to have freed the box, then for the tile) and the warp
    // shares the outcome;
    // every lane loads its 16 raw units (16 bytes, eight K values each), the
    // warp meets (and lane 0 frees the staging slot); then the lanes write
    // the units' x0 and
    // x1 digits into the box, fence them for the tensor core, meet again
    // and lane 0 arrives. Lane l takes the units g = 32 k + l: row
    // r = (l & 7) | k << 3, unit u = (l >> 3) & 3. Eight consecutive lanes
    // cover eight consecutive rows of one unit, so the raw reads (64-byte
    // rows, 64-byte swizzle: unit u at u ^ ((r >> 1) & 3)) and the plane
    // writes (128-byte rows, 128-byte swizzle: unit v at v ^ (r & 7); x0 in
    // units 0-3, x1 in 4-7) hit eight different bank groups.
    if constexpr (CONV) {
    const int cw = warp - 12;
    const int p = cw >> 1;
    const uint32_t ring = smem_addr(smem);
    const int u = (lane >> 3) & 3;
    bool ok = true;
    for (int i = 0; i < nu && ok; ++i) {
      if (unit_kind(u0 + i, a.n_db_units) != 0) break;  // DB units come first
      for (int rb = 0; rb < kRowBlocks; ++rb) {
        const int s = rb * kAPairs + p;
        const int sq = 8 * i + 4 * rb + cw;
        const int j = kStaged ? sq % kNS : 0;
        const uint32_t box = ring + rb * kARingBytes + cw * kABoxBytes;
        bool ready = false;
        if (lane == 0) {
          if constexpr (kStaged) {
            // The box first: once the MMA pipe has freed unit i - 1's box,
            // the staging slot's previous tile (sq - kNS, another warp's
            // when kNS is not a multiple of 4) has been read, so the parity
            // wait on the slot is for the right phase even when copies land
            // out of order.
            ready = mbar_wait(&a_empty[s], (i & 1) ^ 1, err) &&
                    mbar_wait(&st_full[j], (sq / kNS) & 1, err);
          } else {
            ready = mbar_wait(&st_full[s], i & 1, err);
          }
        }
        if (__shfl_sync(0xffffffffu, ready ? 1 : 0, 0) == 0) {
          ok = false;
          break;
        }
        // Staged: the slot's tile; in place: the first half of the box.
        const uint32_t stage =
            kStaged ? ring + Plan::kStageBase + j * kRawTileBytes : box;
        uint4 raw[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const int r = (lane & 7) | (k << 3);
          raw[k] = lds128(stage + r * 64 + ((u ^ ((r >> 1) & 3)) << 4));
        }
        __syncwarp();
        if (kStaged && lane == 0) mbar_arrive(&st_empty[j]);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const int r = (lane & 7) | (k << 3);
          uint4 x0, x1;
          u16_digits(raw[k].x, x0.x, x1.x);
          u16_digits(raw[k].y, x0.y, x1.y);
          u16_digits(raw[k].z, x0.z, x1.z);
          u16_digits(raw[k].w, x0.w, x1.w);
          sts128(box + r * 128 + ((u ^ (r & 7)) << 4), x0);
          sts128(box + r * 128 + (((4 + u) ^ (r & 7)) << 4), x1);
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&a_full[s]);
      }
    }
    if (lane == 0) mbar_arrive(conv_done);
    }
  } else {
    if constexpr (CONV) {
      asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kRegsEpi));
    }
    // -------------------------------------------------------- epilogue --
    const int e = (warp - 4) / 4;   // row block
    const int ew = (warp - 4) % 4;  // TMEM lanes 32*ew .. 32*ew+31
    Acc acc[kTileQ];
#pragma unroll
    for (int i = 0; i < kTileQ; ++i) acc[i] = 0;
    bool ok = true;
    uint32_t n01 = 0, n23 = 0;
    for (int i = 0; i < nu; ++i) {
      // Warp-uniform outcome: the TMEM loads below are .sync.aligned.
      if (!__all_sync(0xffffffffu, mbar_wait(&acc_full[e], i & 1, err))) {
        ok = false;
        break;
      }
      tc_fence_after();
      const int kind = unit_kind(u0 + i, a.n_db_units);
      n23 += 1;
      n01 += kind != 2 ? 1 : 0;
      const uint32_t base =
          tmem + (static_cast<uint32_t>(ew * 32) << 16) + e * 256;
#pragma unroll
      for (int sblk = 0; sblk < NW; ++sblk) {
        if (kind == 2 && sblk < 2) continue;
        constexpr int kLd = kTileQ < 32 ? kTileQ : 32;  // columns per load
        uint32_t v[kTileQ / kLd][kLd];
#pragma unroll
        for (int c = 0; c < kTileQ / kLd; ++c) {
          tmem_ld<kLd>(base + sblk * kTileQ + kLd * c, v[c]);
        }
        tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < kTileQ / kLd; ++c) {
#pragma unroll
          for (int j = 0; j < kLd; ++j) {
            acc[kLd * c + j] +=
                static_cast<Acc>(__float_as_uint(__uint_as_float(v[c][j]) + 12582912.0f))
                << (8 * sblk);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[e]);
    }
    if (ok && *reinterpret_cast<volatile int*>(err) == 0) {
      // Every decoded value carried 0x4B400000 (the bits of 1.5 * 2^23),
      // shifted by its block weight: remove them all at once, mod 2^w.
      const Acc m = 0x4B400000u;
      Acc corr = 0;
#pragma unroll
      for (int sblk = 0; sblk < NW; ++sblk) {
        corr += static_cast<Acc>(sblk < 2 ? n01 : n23) * (m << (8 * sblk));
      }
      const int row = row0 + e * kBlockRows + ew * 32 + lane;
#pragma unroll
      for (int j = 0; j < kTileQ; ++j) {
        const int q = q0 + j;
        if (q < a.batch) {
          Acc* o = out + q * a.out_stride + row;
          // The DB offset 2^15 * sum_c q1[c], once per output word.
          const Acc v = acc[j] - corr + (ks == 0 ? __ldg(qsum + q) << 15 : Acc{0});
          if (a.ksplit == 1) {
            *o = v;
          } else {
            atomicAdd(o, v);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 2) tmem_dealloc(tmem, kTmemCols);
}

// Digit planes of a u16 matrix: x - 2^15 = x0 + 2^8 x1 (x0 in [-128, 127],
// x1 in [-128, 128]) as fp16, interleaved per 32-wide K chunk so that one
// 128-byte row carries both planes of a chunk: [rows][cols_pad/32][2][32];
// zero past cols (padding columns meet zero query words).
__global__ void split_u16_kernel(const uint16_t* __restrict__ src,
                                 int64_t rows, int64_t cols,
                                 int64_t cols_pad, __half* __restrict__ dst) {
  const int64_t total = rows * cols_pad;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       i < total; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / cols_pad, c = i % cols_pad;
    const int v = c < cols ? static_cast<int>(src[r * cols + c]) - 32768 : 0;
    const int x0 = ((v + 128) & 255) - 128;
    const int x1 = (v - x0) / 256;
    const int64_t o = r * 2 * cols_pad + (c / 32) * 64 + (c % 32);
    dst[o] = __int2half_rn(x0);
    dst[o + 32] = __int2half_rn(x1);
  }
}

// Balanced base-256 digits of a word (mod 2^(8 NQ): the top carry drops)
// as fp16 values.
template <int NQ, typename T>
__device__ __forceinline__ void word_digits(T x, __half (&h)[NQ]) {
  int carry = 0;
#pragma unroll
  for (int j = 0; j < NQ; ++j) {
    int b = static_cast<int>((x >> (8 * j)) & 255u) + carry;
    carry = b >= 128 ? 1 : 0;
    b -= carry << 8;
    h[j] = __int2half_rn(b);
  }
}

// The requests' first-dimension words as the NQ digit planes (plane j at
// j * plane_rows rows, cols_pad columns, zero past cols and for requests
// batch..rows_pad) and their sums mod 2^w (the DB offset term; qsum must
// be zeroed). Each thread takes 4 consecutive columns of one request:
// 16-byte loads when the rows allow them, 8-byte stores per plane.
// grid = (ceil(cols_pad / 1024), rows_pad), block = 256.
template <typename T, int NQ>
__global__ void split_queries_kernel(const T* __restrict__ q1, int64_t cols,
                                     int64_t stride, int batch, int64_t plane_rows,
                                     int64_t cols_pad, __half* __restrict__ dst,
                                     T* __restrict__ qsum) {
  __shared__ T part[8];
  const int q = blockIdx.y;
  const int64_t c0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * 4;
  T x[4] = {0, 0, 0, 0};
  if (q < batch && c0 < cols) {
    const T* row = q1 + q * stride;
    if (c0 + 4 <= cols && ((reinterpret_cast<uintptr_t>(row + c0) & 15) == 0)) {
      constexpr int kVec = 16 / sizeof(T);
#pragma unroll
      for (int v = 0; v < 4; v += kVec) {
        const uint4 w = *reinterpret_cast<const uint4*>(row + c0 + v);
        const T* e = reinterpret_cast<const T*>(&w);
#pragma unroll
        for (int i = 0; i < kVec; ++i) x[v + i] = e[i];
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) x[i] = c0 + i < cols ? row[c0 + i] : T{0};
    }
  }
  if (c0 < cols_pad) {
    __half h[4][NQ];  // [column][plane]
#pragma unroll
    for (int i = 0; i < 4; ++i) word_digits<NQ>(x[i], h[i]);
    const int64_t plane = plane_rows * cols_pad;
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
      __half2 lo = __halves2half2(h[0][j], h[1][j]);
      __half2 hi = __halves2half2(h[2][j], h[3][j]);
      uint2 w;
      w.x = *reinterpret_cast<uint32_t*>(&lo);
      w.y = *reinterpret_cast<uint32_t*>(&hi);
      *reinterpret_cast<uint2*>(dst + j * plane + q * cols_pad + c0) = w;
    }
  }
  if (q >= batch) return;  // uniform per block
  T sum = x[0] + x[1] + x[2] + x[3];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    T t = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += part[w];
    atomicAdd(qsum + q, t);
  }
}

// The same NQ digit planes of any request-word matrix (the packing keys' y_g
// words), one word per iteration. Planes plane_rows x cols_pad apart.
template <typename T, int NQ>
__global__ void split_words_kernel(const T* __restrict__ src, int64_t rows, int64_t cols,
                                   int64_t stride, int64_t rows_pad, int64_t plane_rows,
                                   int64_t cols_pad, __half* __restrict__ dst) {
  const int64_t total = rows_pad * cols_pad;
  const int64_t plane = plane_rows * cols_pad;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       i < total; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / cols_pad, c = i % cols_pad;
    const T x = r < rows && c < cols ? src[r * stride + c] : T{0};
    __half h[NQ];
    word_digits<NQ>(x, h);
#pragma unroll
    for (int j = 0; j < NQ; ++j) dst[j * plane + i] = h[j];
  }
}

// Balanced base-256 digit planes (each in [-128, 127], the top carry
// dropped: mod 2^32) of the u32 two's complement of a matrix of `kind`:
// plane j holds rows_pad x cols_pad fp16 (zero outside rows x cols) and
// starts at row j * plane_rows.
// With interleave (the pack matrix, an A operand) the planes share rows
// instead: [rows][cols_pad/32][4][32].
__global__ void split_u32_kernel(const void* __restrict__ src, int kind,
                                 int64_t rows, int64_t cols, int64_t stride,
                                 int64_t rows_pad, int64_t plane_rows,
                                 int64_t cols_pad, __half* __restrict__ dst,
                                 int interleave = 0, int exact_top = 0) {
  const int64_t total = rows_pad * cols_pad;
  const int64_t plane = plane_rows * cols_pad;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       i < total; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / cols_pad, c = i % cols_pad;
    uint32_t x = 0;
    if (r < rows && c < cols) {
      const int64_t o = r * stride + c;
      switch (kind) {
        case kI16: x = static_cast<uint32_t>(static_cast<int32_t>(
                       static_cast<const int16_t*>(src)[o])); break;
        case kI32: x = static_cast<uint32_t>(static_cast<const int32_t*>(src)[o]); break;
        default: x = static_cast<const uint32_t*>(src)[o]; break;
      }
    }
    // With exact_top the signed entry itself is the sum of its digits (the
    // top digit takes the remainder, in [-128, 128]): products with 64-bit
    // request words need the integer, not its value mod 2^32.
    const int64_t sv = static_cast<int32_t>(x);
    int64_t low = 0;
    int carry = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int b = static_cast<int>((x >> (8 * j)) & 255u) + carry;
      carry = b >= 128 ? 1 : 0;
      b -= carry << 8;
      if (exact_top && j == 3) b = static_cast<int>((sv - low) >> 24);
      low += static_cast<int64_t>(b) << (8 * j);
      const int64_t o = interleave ? r * 4 * cols_pad + (c / 32) * 128 + j * 32 + (c % 32)
                                   : j * plane + i;
      dst[o] = __int2half_rn(b);
    }
  }
}

// ------------------------------------------------------------ host side --
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess) {
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
  });
  return fn;
}

// 2-D fp16 tensor [rows][cols], box box_rows x 32, 64-byte swizzle.
// Box box_rows x box_cols with 128-byte rows and the 128-byte swizzle.
bool make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols,
              uint32_t box_rows, uint32_t box_cols) {
  auto fn = encode_fn();
  if (fn == nullptr) return false;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t elem[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base),
                  dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The u16 DB as stored, [rows][cols]: boxes of 128 rows x 32 columns
// (64-byte rows, 64-byte swizzle), zero fill past the last column. Needs
// rows of a multiple of 16 bytes (cols % 8 == 0).
bool make_raw_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols) {
  auto fn = encode_fn();
  if (fn == nullptr || cols % 8 != 0 ||
      (reinterpret_cast<uintptr_t>(base) & 15) != 0) {
    return false;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * 2};
  cuuint32_t box[2] = {static_cast<cuuint32_t>(kStageK), static_cast<cuuint32_t>(kBlockRows)};
  cuuint32_t elem[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(base), dims,
                  strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

class LimbScratchImpl : public LimbScratch {
 public:
  ~LimbScratchImpl() override {
    if (q_planes) cudaFree(q_planes);
    if (y_planes) cudaFree(y_planes);
    if (qsum) cudaFree(qsum);
  }
  int64_t qcap = 0;
  __half* q_planes = nullptr;
  __half* y_planes = nullptr;
  void* qsum = nullptr;  // sum_c q1[q][c] per request (coefficient words)
  CUtensorMap tm_q{}, tm_y{};      // boxes of a full request tile
  CUtensorMap tm_qn{}, tm_yn{};    // boxes of a narrow tile
};

class LimbGemmImpl : public LimbGemm {
 public:
  ~LimbGemmImpl() override {
    for (void* p : {db_planes_, pk_planes_})
      if (p) cudaFree(p);
    if (err_) cudaFree(err_);
  }

  // planes: also keep the DB's fp16 digit planes resident (2x the DB's
  // bytes), so that both forms of the kernel can run and the autotuner
  // picks per batch size. Without them the DB is read as stored.
  bool Init(int nq, const void* db, int64_t rows, int64_t db_cols, int mat_kind,
            const void* pack, int64_t pack_cols, bool planes) {
    nq_ = nq;
    tq_ = kBRows / nq;
    word_ = nq == 4 ? 4 : 8;
    rows_ = rows;
    db_cols_ = db_cols;
    pk_cols_ = pack_cols;
    cpad_ = round_up(db_cols, kUnitK);
    kpad_ = round_up(pack_cols, kUnitK);
    // The converting form and the narrow tiles serve Z_2^32 words; over
    // Z_2^64 the engine keeps the resident planes and full tiles (the form
    // the 64-bit tests and benchmarks were validated with).
    conv_ = nq == 4 && make_raw_map(&tm_raw_, db, rows, db_cols);
    if (!conv_) planes = true;  // rows not 16-byte multiples: planes only
    if (cudaMalloc(&err_, sizeof(int)) != cudaSuccess) return false;
    if (cudaMemset(err_, 0, sizeof(int)) != cudaSuccess) return false;
    if (planes) {
      if (cudaMalloc(&db_planes_, 2ull * rows * cpad_ * 2) != cudaSuccess) return false;
      split_u16_kernel<<<152 * 16, 256>>>(static_cast<const uint16_t*>(db), rows,
                                          db_cols, cpad_, db_planes_);
    }
    if (cudaMalloc(&pk_planes_, 4ull * rows * kpad_ * 2) != cudaSuccess) return false;
    split_u32_kernel<<<152 * 16, 256>>>(pack, mat_kind, rows, pack_cols, pack_cols,
                                        rows, rows, kpad_, pk_planes_, 1, nq == 8 ? 1 : 0);
    if (cudaDeviceSynchronize() != cudaSuccess) return false;
    if (planes &&
        !make_map(&tm_db_, db_planes_, rows, 2ull * cpad_, kBlockRows, 2 * kStageK)) {
      return false;
    }
    if (!make_map(&tm_pk_, pk_planes_, rows, 4ull * kpad_, kBlockRows, 2 * kStageK)) return false;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev);
    const int smem = static_cast<int>(kSmemBytes);
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t fe = cudaSuccess;
    auto allow = [&](const void* fn) {
      if (fe == cudaSuccess) fe = cudaFuncSetAttribute(fn, attr, smem);
    };
    if (nq == 4) {
      allow(reinterpret_cast<const void*>(limb_gemm_kernel<4, false, 64>));
      allow(reinterpret_cast<const void*>(limb_gemm_kernel<4, false, kNarrowTQ>));
      if (conv_) {
        allow(reinterpret_cast<const void*>(limb_gemm_kernel<4, true, 64>));
        allow(reinterpret_cast<const void*>(limb_gemm_kernel<4, true, kNarrowTQ>));
      }
    } else {
      allow(reinterpret_cast<const void*>(limb_gemm_kernel<8, false, 32>));
      allow(reinterpret_cast<const void*>(limb_gemm_kernel<8, false, 32, 7>));
    }
    return fe == cudaSuccess;
  }

  // Resident device bytes of the engine (digit planes).
  int64_t ResidentBytes() const override {
    return (db_planes_ ? 2 * rows_ * cpad_ * 2 : 0) + 4 * rows_ * kpad_ * 2;
  }

  std::unique_ptr<LimbScratch> NewScratch() override {
    return std::unique_ptr<LimbScratch>(new LimbScratchImpl());
  }

  int64_t ScratchBytes(int batch) const override {
    const int64_t need = round_up(batch, tq_);
    return nq_ * need * (cpad_ + kpad_) * 2 + word_ * need;
  }

  cudaError_t Reserve(LimbScratch* scratch, int batch) override {
    return EnsureQueries(static_cast<LimbScratchImpl*>(scratch), batch);
  }

  cudaError_t EnsureQueries(LimbScratchImpl* sc, int batch) {
    const int64_t need = round_up(batch, tq_);
    if (need <= sc->qcap) return cudaSuccess;
    if (sc->q_planes) cudaFree(sc->q_planes);
    if (sc->y_planes) cudaFree(sc->y_planes);
    if (sc->qsum) cudaFree(sc->qsum);
    sc->q_planes = sc->y_planes = nullptr;
    sc->qsum = nullptr;
    sc->qcap = 0;
    cudaError_t e = cudaMalloc(&sc->q_planes, static_cast<size_t>(nq_) * need * cpad_ * 2);
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&sc->y_planes, static_cast<size_t>(nq_) * need * kpad_ * 2);
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&sc->qsum, static_cast<size_t>(word_) * need);
    if (e != cudaSuccess) return e;
    if (!make_map(&sc->tm_q, sc->q_planes, static_cast<uint64_t>(nq_) * need, cpad_, tq_,
                  kBSlotK) ||
        !make_map(&sc->tm_y, sc->y_planes, static_cast<uint64_t>(nq_) * need, kpad_, tq_,
                  kBSlotK) ||
        !make_map(&sc->tm_qn, sc->q_planes, static_cast<uint64_t>(nq_) * need, cpad_,
                  kNarrowTQ, kBSlotK) ||
        !make_map(&sc->tm_yn, sc->y_planes, static_cast<uint64_t>(nq_) * need, kpad_,
                  kNarrowTQ, kBSlotK)) {
      return cudaErrorInvalidValue;
    }
    sc->qcap = need;
    return cudaSuccess;
  }

  cudaError_t Run(int batch, const void* q1, int64_t q1_stride, const void* yg,
                  int64_t yg_stride, void* out, LimbScratch* scratch,
                  cudaStream_t st, int out_bits) override {
    return Launch(batch, q1, q1_stride, yg, yg_stride, out, scratch, st,
                  Chosen(batch), WeightBlocks(out_bits));
  }

  cudaError_t RunForm(int batch, const void* q1, int64_t q1_stride, const void* yg,
                      int64_t yg_stride, void* out, LimbScratch* scratch,
                      cudaStream_t st, int form, int split, int out_bits) override {
    Choice c = Chosen(batch);
    c.form = form & 1;
    c.narrow = (form >> 1) & 1;
    if (split > 0) c.split = split;
    if (!Available(c)) return cudaErrorNotSupported;
    return Launch(batch, q1, q1_stride, yg, yg_stride, out, scratch, st, c,
                  WeightBlocks(out_bits));
  }

  // Weight blocks (base-256 digit positions) of the product words the
  // caller reads: all of them, or for Z_2^64 words read mod 2^b with
  // b <= 56 only the seven below 2^56.
  int WeightBlocks(int out_bits) const {
    return nq_ == 8 && out_bits > 0 && out_bits <= 56 ? 7 : nq_;
  }

  // One configuration of the product: split-K factor, DB form and request
  // tile (1: the narrow 16-request tile).
  struct Choice {
    int split, form, narrow;
  };

  bool Available(const Choice& c) const {
    if (c.narrow && nq_ != 4) return false;
    return (c.form == kFormRaw && conv_) || (c.form == kFormPlanes && db_planes_);
  }

  // Tuned choices are kept per batch size rounded up to the narrow tile.
  static int64_t TuneKey(int batch) { return round_up(batch, kNarrowTQ); }

  // Autotuner: times every available (form, request tile, split-K factor)
  // with at least 8 K units per CTA and 80 % of the last wave busy (plus the
  // heuristic factor) on this batch size, and keeps the fastest for later
  // launches of the same size. The narrow tile is tried up to 64 requests.
  // Synchronises `st`.
  cudaError_t Tune(int batch, const void* q1, int64_t q1_stride, const void* yg,
                   int64_t yg_stride, void* out, LimbScratch* scratch,
                   cudaStream_t st, int out_bits, int* chosen, int* chosen_form,
                   float* best_ms) override {
    if (batch <= 0) return cudaErrorInvalidValue;
    const int nw = WeightBlocks(out_bits);
    const int n_units = static_cast<int>((cpad_ + 2 * kpad_) / kUnitK);
    const int sms = sms_ > 0 ? sms_ : 148;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      return e;
    }
    Choice best = Heuristic(batch);
    float best_t = 0;
    for (int narrow = 0; narrow <= (batch <= 64 && nq_ == 4 ? 1 : 0) && e == cudaSuccess;
         ++narrow) {
      const int tq = narrow ? kNarrowTQ : tq_;
      const int64_t tiles = (rows_ / kTileRows) * ((batch + tq - 1) / tq);
      const int heuristic = ChooseSplit(tiles, n_units);
      for (int form = kFormPlanes; form <= kFormRaw && e == cudaSuccess; ++form) {
        for (int k = 1; k <= 16 && e == cudaSuccess; ++k) {
          const Choice c{k, form, narrow};
          if (!Available(c)) break;
          if (n_units / k < 8) break;
          const int64_t items = tiles * k;
          const int64_t waves = (items + sms - 1) / sms;
          const double eff = static_cast<double>(items) / (waves * sms);
          if (k != heuristic && eff < 0.8) continue;
          e = Launch(batch, q1, q1_stride, yg, yg_stride, out, scratch, st, c, nw);
          if (e == cudaSuccess) e = cudaEventRecord(e0, st);
          for (int r = 0; r < 2 && e == cudaSuccess; ++r) {
            e = Launch(batch, q1, q1_stride, yg, yg_stride, out, scratch, st, c, nw);
          }
          if (e == cudaSuccess) e = cudaEventRecord(e1, st);
          if (e == cudaSuccess) e = cudaEventSynchronize(e1);
          float ms = 0;
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
          if (e == cudaSuccess && (best_t == 0 || ms < best_t)) {
            best_t = ms;
            best = c;
          }
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return e;
    {
      std::lock_guard<std::mutex> lk(tune_mu_);
      tuned_[TuneKey(batch)] = best;
    }
    if (chosen) *chosen = best.split;
    if (chosen_form) *chosen_form = best.form + 2 * best.narrow;
    if (best_ms) *best_ms = best_t / 2;
    return cudaSuccess;
  }

  // Without a tuned choice: the full tile, the resident planes when there
  // are some (the form measured fastest for large batches), else the DB as
  // stored, and the split-K factor that fills the SMs.
  Choice Heuristic(int batch) const {
    const int64_t tiles = (rows_ / kTileRows) * ((batch + tq_ - 1) / tq_);
    return {ChooseSplit(tiles, static_cast<int>((cpad_ + 2 * kpad_) / kUnitK)),
            db_planes_ ? kFormPlanes : kFormRaw, 0};
  }

  Choice Chosen(int batch) {
    {
      std::lock_guard<std::mutex> lk(tune_mu_);
      auto it = tuned_.find(TuneKey(batch));
      if (it != tuned_.end()) return it->second;
    }
    return Heuristic(batch);
  }

  cudaError_t Launch(int batch, const void* q1, int64_t q1_stride, const void* yg,
                     int64_t yg_stride, void* out, LimbScratch* scratch,
                     cudaStream_t st, const Choice& c, int nw) {
    if (batch <= 0) return cudaSuccess;
    if (!Available(c)) return cudaErrorNotSupported;
    LimbScratchImpl* sc = static_cast<LimbScratchImpl*>(scratch);
    cudaError_t e = EnsureQueries(sc, batch);
    if (e != cudaSuccess) return e;
    const int64_t bpad = round_up(batch, tq_);
    // Byte planes of the requests, qcap rows apart; rows batch..bpad are 0.
    e = cudaMemsetAsync(sc->qsum, 0, static_cast<size_t>(word_) * batch, st);
    if (e != cudaSuccess) return e;
    const dim3 qgrid(static_cast<unsigned>((cpad_ + 1023) / 1024), static_cast<unsigned>(bpad));
    if (nq_ == 4) {
      split_queries_kernel<uint32_t, 4><<<qgrid, 256, 0, st>>>(
          static_cast<const uint32_t*>(q1), db_cols_, q1_stride, batch, sc->qcap, cpad_,
          sc->q_planes, static_cast<uint32_t*>(sc->qsum));
      split_words_kernel<uint32_t, 4><<<152 * 8, 256, 0, st>>>(
          static_cast<const uint32_t*>(yg), batch, pk_cols_, yg_stride, bpad, sc->qcap, kpad_,
          sc->y_planes);
    } else {
      using U = unsigned long long;
      split_queries_kernel<U, 8><<<qgrid, 256, 0, st>>>(
          static_cast<const U*>(q1), db_cols_, q1_stride, batch, sc->qcap, cpad_, sc->q_planes,
          static_cast<U*>(sc->qsum));
      split_words_kernel<U, 8><<<152 * 8, 256, 0, st>>>(
          static_cast<const U*>(yg), batch, pk_cols_, yg_stride, bpad, sc->qcap, kpad_,
          sc->y_planes);
    }
    LimbArgs a;
    a.rows = static_cast<int>(rows_);
    a.n_db_units = static_cast<int>(cpad_ / kUnitK);
    a.n_pk_blocks = static_cast<int>(kpad_ / kUnitK);
    a.qcap = static_cast<int>(sc->qcap);
    a.batch = batch;
    a.out_stride = rows_;
    a.ksplit = c.split;
    const int tq = c.narrow ? kNarrowTQ : tq_;
    const int64_t tiles = (rows_ / kTileRows) * ((batch + tq - 1) / tq);
    if (a.ksplit > 1) {
      e = cudaMemsetAsync(out, 0, static_cast<size_t>(batch) * rows_ * word_, st);
      if (e != cudaSuccess) return e;
    }
    const unsigned grid = static_cast<unsigned>(tiles * a.ksplit);
    const CUtensorMap& mq = c.narrow ? sc->tm_qn : sc->tm_q;
    const CUtensorMap& my = c.narrow ? sc->tm_yn : sc->tm_y;
    using U = unsigned long long;
    const uint32_t* qs4 = static_cast<const uint32_t*>(sc->qsum);
    const U* qs8 = static_cast<const U*>(sc->qsum);
    uint32_t* o4 = static_cast<uint32_t*>(out);
    U* o8 = static_cast<U*>(out);
    const bool raw = c.form == kFormRaw;
    const int nt = raw ? kThreadsConv : kThreads;
#define INSPIRE_LIMB_LAUNCH(NQ, CONV, TQ, NW, QS, OUT)                              \
  limb_gemm_kernel<NQ, CONV, TQ, NW><<<grid, nt, kSmemBytes, st>>>(                 \
      tm_db_, tm_raw_, tm_pk_, mq, my, a, QS, OUT, err_)
    if (nq_ == 4) {
      if (!raw && !c.narrow) INSPIRE_LIMB_LAUNCH(4, false, 64, 4, qs4, o4);
      if (!raw && c.narrow) INSPIRE_LIMB_LAUNCH(4, false, kNarrowTQ, 4, qs4, o4);
      if (raw && !c.narrow) INSPIRE_LIMB_LAUNCH(4, true, 64, 4, qs4, o4);
      if (raw && c.narrow) INSPIRE_LIMB_LAUNCH(4, true, kNarrowTQ, 4, qs4, o4);
    } else if (nw == 7) {
      // Available(): planes, full tiles; products read mod 2^56.
      INSPIRE_LIMB_LAUNCH(8, false, 32, 7, qs8, o8);
    } else {
      INSPIRE_LIMB_LAUNCH(8, false, 32, 8, qs8, o8);
    }
#undef INSPIRE_LIMB_LAUNCH
    return cudaGetLastError();
  }

  // Split-K factor that fills the SMs in whole waves (one CTA per SM), with
  // at least 16 accumulation units per K slice (small products, e.g. a
  // 2048-row pack matrix: 64 units, 32 tiles at B = 256, split 4).
  int ChooseSplit(int64_t tiles, int n_units) const {
    const int sms = sms_ > 0 ? sms_ : 148;
    int best = 1;
    double best_eff = 0;
    for (int k = 1; k <= 8; ++k) {
      if (n_units / k < 16) break;
      const int64_t items = tiles * k;
      const int64_t waves = (items + sms - 1) / sms;
      const double eff = static_cast<double>(items) / (waves * sms);
      if (eff > best_eff + 0.02) {
        best_eff = eff;
        best = k;
      }
    }
    return best;
  }

  int CheckError() override {
    int h = 0;
    if (cudaMemcpy(&h, err_, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return -1;
    if (h != 0) cudaMemset(err_, 0, sizeof(int));
    return h;
  }

 private:
  int64_t rows_ = 0, db_cols_ = 0, pk_cols_ = 0, cpad_ = 0, kpad_ = 0;
  int sms_ = 0;
  int nq_ = 4, tq_ = 64, word_ = 4;  // request digit planes, requests per tile, word bytes
  __half *db_planes_ = nullptr, *pk_planes_ = nullptr;
  bool conv_ = false;  // the raw-DB (converting) form can run
  int* err_ = nullptr;
  CUtensorMap tm_db_{}, tm_raw_{}, tm_pk_{};
  std::mutex tune_mu_;
  std::map<int64_t, Choice> tuned_;  // TuneKey(batch) -> tuned configuration
};

}  // namespace

void LimbGemm::Create(int coeff_bits, int db_kind, const void* db, int64_t rows,
                      int64_t db_cols, int mat_kind, const void* pack,
                      int64_t pack_cols, bool db_planes, std::unique_ptr<LimbGemm>* out) {
  out->reset();
  // A u16 DB over Z_{2^32} (4 request digit planes; int16, int32 or u32
  // pack matrices) or Z_{2^64} (8 planes; int16 or int32 pack matrices,
  // split into digits whose sum is the entry itself).
  if (db_kind != kU16) return;
  if (coeff_bits == 32) {
    if (mat_kind != kI16 && mat_kind != kI32 && mat_kind != kU32) return;
  } else if (coeff_bits == 64) {
    if (mat_kind != kI16 && mat_kind != kI32) return;
  } else {
    return;
  }
  if (rows % kTileRows != 0 || db_cols <= 0 || pack_cols <= 0) return;
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10) return;
  std::unique_ptr<LimbGemmImpl> impl(new LimbGemmImpl());
  if (!impl->Init(coeff_bits == 32 ? 4 : 8, db, rows, db_cols, mat_kind, pack, pack_cols,
                  db_planes)) {
    cudaGetLastError();
    return;
  }
  *out = std::move(impl);
}

}  // namespace inspire
