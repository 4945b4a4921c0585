// One-pass split-precision grouped GEMM on the 5th-generation tensor cores
// (tcgen05 + TMEM), for the groups of a step whose whole K fits one exact
// pass (1 <= K <= 256 slots).
//
// Arithmetic (exact model: tests/split_model.py).  Every FP64 element of a
// row i of A (column j of B) is cut relative to the row's (column's) largest
// biased exponent over the group's whole K into four balanced 8-bit digits
// (X = d0 2^24 + d1 2^16 + d2 2^8 + d3 = |x| / 2^(E-1053) rounded, <= 2^31,
// |digit| <= 128, the element's sign on every digit), held as bf16 planes.
// The tensor cores form the level sums
//   L_l = sum_{s+t=l} A_s B_t^T,  l = 0..3  (10 digit products),
// in FP32 in tensor memory; a digit product is at most 2^14 and a level takes
// at most four per slot, so for K <= 256 every level is an exact integer
// below 2^24.  The epilogue combines the levels once per tile into the exact
// integer S = L0 2^24 + L1 2^16 + L2 2^8 + L3 (< 2^48) and writes
// S 2^(Ea_i + Eb_j - 2082) as FP64 with integer operations.  The result is
// a deterministic function of the inputs, bit-identical to the model.
//
// Two phases per step.
//  1. Prepare kernels (k_prep_a, k_prep_b) cut every operand tile once: an A
//     tile is 128 rows of a group over its whole K, a B tile is a column tile
//     of 16 / 32 / 64 columns.  Each tile record in the plane buffer is the
//     exact shared-memory image the tensor cores read (K-major, 64-byte
//     swizzle, k blocks of 32 slots) followed by the exponents (and, for B,
//     the output offset and row stride of every column).  These are plain
//     streaming kernels with many warps per SM, so the gathers of the
//     block-sparse operands run with enough loads in flight.
//  2. k_step_umma moves records into shared memory with bulk copies
//     (cp.async.bulk, completion counted on mbarriers) and multiplies:
//       warps 0-15 epilogue: warp w reads TMEM lanes 32(w%4).. (one output
//                  row per thread) and every fourth 8-column chunk from
//                  column 8(w/4), folds the levels and stores the tile;
//       warp 16    producer: lane 0 issues the bulk copies (B tile of the
//                  work item, per row tile its exponents and column map, A
//                  k blocks through a ring of stages);
//       warp 17    TMEM allocation; lane 0 issues the MMAs and commits.
//     Level products: the B planes of a column tile of TN columns are stacked
//     along N as B' = [B0 | B1 | B2 | B3] (4 TN rows of a K-major operand)
//     and the four level accumulators of a row tile lie side by side in TMEM
//     ([L0 | L1 | L2 | L3], TN columns each), so per 16-slot k step four MMAs
//     A_a x B'[0, (4-a) TN) -> TMEM columns [a TN, 4 TN) (N = 4TN, 3TN, 2TN,
//     TN) issue all ten products.  Two TMEM accumulator buffers let the
//     epilogue of one row tile overlap the MMAs of the next.
// Every wait is bounded in time (2 s): on expiry the kernel records an error
// code (zmpo_device_status), every role stops at its next item boundary,
// the producer waits (bounded) for the bulk copies it issued, the MMA
// issuer's outstanding work is waited for (bounded) and the tensor memory is
// released before the kernel returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zmpo_gb300.h"
#include "device_common.cuh"
#include "engine.h"

namespace zmpo {

__device__ int g_umma_error = 0;

namespace umma {

// ----------------------------------------------------------- constants
constexpr int TM = kUmmaTM;                   // rows per tile (TMEM lanes)
constexpr int KMAX = kUmmaMaxK;               // slots of one exact pass
constexpr int KB_SLOTS = kUmmaKB;             // slots per k block (one 64-byte swizzle row)
constexpr int NKB_MAX = KMAX / KB_SLOTS;
constexpr int ROW_BYTES = 64;                 // K-major rows of 32 bf16, 64-byte swizzle
constexpr int A_PLANE = TM * ROW_BYTES;       // 8 KB: one digit plane of a k block
constexpr int A_STAGE = 4 * A_PLANE;          // 32 KB: four planes
constexpr int NTHREADS = 576;
constexpr int EPI_WARPS = 16, PROD_WARP = 16, MMA_WARP = 17;
constexpr int EPI_GROUPS = EPI_WARPS / 4;       // epilogue warps per TMEM lane quarter
constexpr int CHUNK_STEP = 8 * EPI_GROUPS;      // column step between a warp's 8-column chunks
constexpr int STG_BYTES = EPI_WARPS * 32 * 4 * 8;  // per epilogue warp: 32 rows x 4 float64
constexpr int PREP_THREADS = 256;
constexpr int BIAS = 2082;
constexpr uint64_t WAIT_NS = 2000000000ull;   // 2 s bound on every wait
static_assert(A_PLANE == kUmmaAPlane && A_STAGE == kUmmaAKB, "plane record layout");

// error codes recorded in g_umma_error (first one wins)
constexpr int ERR_TIMEOUT_BASE = 100;         // + site of the wait
constexpr int ERR_B_TILE = 90;                // a one-pass item's B tile exceeds its launch's B region

// barrier indices (A ring after the fixed ones)
enum {
  BAR_T_FULL = 0,    // [2] MMA commit (tile done) -> epilogue
  BAR_T_EMPTY = 2,   // [2] epilogue (128) -> MMA
  BAR_E_FULL = 4,    // [2] tile record copied (+ producer's arrival) -> epilogue
  BAR_E_EMPTY = 6,   // [2] tile record read, epilogue (128) -> producer
  BAR_B_FULL = 8,    // [2] B tile of the item copied -> MMA (one per B buffer)
  BAR_B_FREE = 10,   // [2] MMA commit after the item -> producer
  BAR_DONE = 12,     // MMA commit at the end (teardown)
  BAR_A_FULL = 13    // [NSTAGE] A k block copied -> MMA; then [NSTAGE] A_EMPTY (MMA commit -> producer)
};

// Shared memory of the one-pass kernel for column tiles of TN and items whose
// B tile has at most NKBB k blocks: two B buffers when two fit next to a ring
// of at least two A stages (the next item's B tile is copied while the
// current item's row tiles run), else one; then a ring of A k blocks as deep
// as the rest of the 227 KB allows (at most 6 stages), so the A blocks of the
// next row tiles are copied while the current one is multiplied and folded.
template <int TN, int NKBB>
struct Layout {
  static constexpr int B_KB = 4 * TN * ROW_BYTES;         // one k block of the four B planes
  // tile record (one per TMEM buffer): row exponents (copied from the A
  // tile), column exponents, output offsets of (row 0, column c) and row
  // strides (copied from the B tile, in that order), then m0, M, cbuf
  static constexpr int REC_EA = 0;
  static constexpr int REC_EB = REC_EA + TM * 4;
  static constexpr int REC_CB = REC_EB + TN * 4;          // int64 colbase[TN]
  static constexpr int REC_RS = REC_CB + TN * 8;          // int64 rowstride[TN]
  static constexpr int REC_INFO = REC_RS + TN * 8;        // int m0, M, cbuf, pad
  static constexpr int REC_BYTES = REC_INFO + 16;
  static constexpr int FREE_BYTES = 232448 - 1024 - 2 * REC_BYTES - STG_BYTES - 16 - 8 * (BAR_A_FULL + 2 * 6);
  static constexpr int NBB = FREE_BYTES - 2 * NKBB * B_KB >= 2 * A_STAGE ? 2 : 1;  // B buffers
  static constexpr int RING_BYTES = FREE_BYTES - NBB * NKBB * B_KB;
  static constexpr int NSTAGE = RING_BYTES / A_STAGE < 6 ? RING_BYTES / A_STAGE : 6;  // A k-block ring
  static constexpr int OFF_B = 0;                         // buffer b at OFF_B + b * NKBB * B_KB
  static constexpr int OFF_A = OFF_B + NBB * NKBB * B_KB;
  static constexpr int OFF_REC = OFF_A + NSTAGE * A_STAGE;
  static constexpr int OFF_STG = OFF_REC + 2 * REC_BYTES;  // epilogue staging, 1 KB per warp
  static constexpr int OFF_BAR = OFF_STG + STG_BYTES;
  static constexpr int BAR_A_EMPTY = BAR_A_FULL + NSTAGE;
  static constexpr int NBAR = BAR_A_FULL + 2 * NSTAGE;
  static constexpr int OFF_MISC = OFF_BAR + NBAR * 8;     // tmem base, abort flag
  static constexpr int BYTES = OFF_MISC + 16;
  static constexpr int SMEM = BYTES + 1024;               // + alignment of the base to 1024
  static constexpr int TMEM_COLS = 8 * TN;                // two buffers of four levels
  static_assert(TN == 16 || TN == 32 || TN == 64, "column tile");
  static_assert(NKBB == 2 || NKBB == 4 || NKBB == NKB_MAX, "B k blocks of a launch");
  static_assert(NSTAGE >= 2, "A ring of at least two stages");
  static_assert(B_KB == umma_b_kb_bytes(TN), "plane record layout");
  static_assert(OFF_A % 1024 == 0 && A_STAGE % 1024 == 0 && B_KB % 1024 == 0, "swizzle atoms");
  static_assert(OFF_REC % 16 == 0 && REC_EB % 16 == 0 && REC_BYTES % 16 == 0, "bulk-copy alignment");
  static_assert(REC_INFO - REC_EB == TN * 20 && REC_CB % 16 == 0, "exponents + column map of a tile record");
  static_assert(SMEM <= 232448, "shared memory");
};

// ------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void bar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void bar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// one arrival that also expects `bytes` of bulk-copy completions this phase
__device__ __forceinline__ void bar_arrive_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// global -> shared bulk copy (16-byte aligned, size a multiple of 16), its
// bytes counted on `bar`
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ bool bar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P1;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase of parity `parity` of barrier `bar` to complete, at most
// WAIT_NS.  Returns false (at once) when the kernel is aborting, or after
// recording a timeout at `site` and raising the abort flag.
__device__ __noinline__ bool wait_bounded(uint32_t bar, uint32_t parity, volatile int *abort_flag, int site,
                                          bool heed_abort = true) {
  if (bar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  while (true) {
    if (bar_try_wait(bar, parity)) return true;
    if (heed_abort && *abort_flag) return false;
    if (globaltimer() - t0 > WAIT_NS) {
      *abort_flag = 1;
      atomicCAS(&g_umma_error, 0, ERR_TIMEOUT_BASE + site);
      return false;
    }
  }
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// barrier of the epilogue warps (id 2) that also returns the OR of `v` over
// the participating threads
__device__ __forceinline__ bool role_sync_or(int id, int nthreads, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}

// Shared-memory matrix descriptor: K-major, 64-byte swizzle (8-row groups of
// 64-byte rows, 512 bytes apart), version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) | ((uint64_t)(512u >> 4) << 32) |
         ((uint64_t)1u << 46) | ((uint64_t)4u << 61);
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major,
// M = 128, N = n.
__device__ __forceinline__ uint32_t idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(dtmem), "l"(ad), "l"(bd), "r"(id), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t *v) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr)
               : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ------------------------------------------------------------ digit cut
__device__ __forceinline__ int dexp(double x) { return (int)(((unsigned)__double2hiint(x) >> 20) & 0x7ffu); }

// Y = X + 0x808080 with X = |x| / 2^(E-1053) rounded to the nearest integer
// (halves up; E >= exponent of x, so X <= 2^31): the bytes of Y are d0, d1+128,
// d2+128, d3+128.  From the 53-bit significand m: X = (m + 2^(s-1)) >> s with
// s = E - e + 22 (capped at 63, where X is 0 for any m < 2^53).
__device__ __forceinline__ uint32_t balanced(double x, int E) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffu);
  const unsigned long long m = (b & 0xfffffffffffffull) | 0x10000000000000ull;
  const int s = min(E - e + 22, 63);
  const uint32_t X = e ? (uint32_t)((m + (1ull << (s - 1))) >> s) : 0u;
  return X + 0x808080u;
}

// byte K of Y minus OFF as the bit pattern of an exact float (PRMT + FADD)
template <int K, int OFF>
__device__ __forceinline__ float byte_f(uint32_t Y) {
  return __uint_as_float(__byte_perm(Y, 0x4B000000u, 0x7440u | K)) - (8388608.0f + (float)OFF);
}

// digit planes of two elements (k, k+1) as packed bf16 pairs: the bf16 of a
// small integer-valued float is its upper half; the sign flips every digit
__device__ __forceinline__ void cut_pair(double x0, double x1, int E, uint32_t d[4]) {
  const uint32_t Y0 = balanced(x0, E), Y1 = balanced(x1, E);
  const uint32_t sg = ((unsigned)__double2hiint(x0) >> 16 & 0x8000u) | ((unsigned)__double2hiint(x1) & 0x80000000u);
  d[0] = __byte_perm(__float_as_uint(byte_f<3, 0>(Y0)), __float_as_uint(byte_f<3, 0>(Y1)), 0x7632u) ^ sg;
  d[1] = __byte_perm(__float_as_uint(byte_f<2, 128>(Y0)), __float_as_uint(byte_f<2, 128>(Y1)), 0x7632u) ^ sg;
  d[2] = __byte_perm(__float_as_uint(byte_f<1, 128>(Y0)), __float_as_uint(byte_f<1, 128>(Y1)), 0x7632u) ^ sg;
  d[3] = __byte_perm(__float_as_uint(byte_f<0, 128>(Y0)), __float_as_uint(byte_f<0, 128>(Y1)), 0x7632u) ^ sg;
}

// Cut 8 consecutive slots (one 16-byte chunk per plane) of one row of a
// K-major plane set: plane0 = row 0 of plane 0 of the k block, planes
// plane_bytes apart, chunk = slot / 8 within the k block.  The 16-byte chunk
// index is XORed with bits 1-2 of the row (the 64-byte swizzle of an image
// whose 8-row groups start at multiples of 512 bytes).
__device__ __forceinline__ void cut8_store(const double *v, int E, unsigned char *plane0, int plane_bytes, int row,
                                           int chunk) {
  uint32_t d[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t p[4];
    cut_pair(v[2 * i], v[2 * i + 1], E, p);
#pragma unroll
    for (int s = 0; s < 4; ++s) d[s][i] = p[s];
  }
  const int off = row * ROW_BYTES + ((chunk ^ ((row >> 1) & 3)) << 4);
#pragma unroll
  for (int s = 0; s < 4; ++s)
    *reinterpret_cast<uint4 *>(plane0 + s * plane_bytes + off) = make_uint4(d[s][0], d[s][1], d[s][2], d[s][3]);
}

// S 2^e as FP64 with integer operations (|S| < 2^53: exact); results below
// the normal range are flushed to zero
__device__ __forceinline__ double scaled_int_to_double(long long S, int e) {
  if (S == 0) return 0.0;
  const unsigned long long sign = S < 0 ? 0x8000000000000000ull : 0ull;
  const unsigned long long A = (unsigned long long)(S < 0 ? -S : S);
  const int n = 63 - __clzll((long long)A);
  const int be = n + e + 1023;
  if (be <= 0) return 0.0;
  const unsigned long long mant = (A << (52 - n)) & 0xfffffffffffffull;
  return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | mant));
}

__device__ __forceinline__ int lvl(uint32_t bits) { return __float2int_rz(__uint_as_float(bits)); }

// S = L0 2^24 + L1 2^16 + L2 2^8 + L3 from the four level sums (FP32 bit
// patterns of exact integers: |L0| <= 2^22, |L1| <= 2^23, |L2| <= 3 2^22,
// |L3| <= 2^24 for a pass of at most 256 slots of balanced digits, |d| <=
// 128): L0 2^8 + L1 fits 32 bits, the rest is summed in 64 bits.
__device__ __forceinline__ long long fold_levels(uint32_t b0, uint32_t b1, uint32_t b2, uint32_t b3) {
  const int hi = lvl(b0) * 256 + lvl(b1);
  return (long long)hi * 65536 + (long long)lvl(b2) * 256 + (long long)lvl(b3);
}

// The epilogue warp's 32 x 8 chunk (lane = row row0 + lane, val[i] =
// column i) stored through the warp's 1 KB staging area, four columns at a
// time: each store instruction then writes 8 rows x 4 consecutive columns
// (32 contiguous bytes per row when the columns are in one output block).
// The chunk's columns are cb[i] (output offset of row 0, < 0: none) and
// rs[i] (row stride).  The staging index is XOR-swizzled by bits 2-3 of the
// row, so the 16 lanes of a half warp touch 16 different 8-byte bank pairs
// (no bank conflicts).  Called by every lane of the warp.
__device__ __forceinline__ void store_chunk(double *stg, const double *val, int lane, int row0, int M,
                                            const long long *cb, const long long *rs, double *out, bool ok) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
#pragma unroll
    for (int i = 0; i < 4; ++i) stg[lane * 4 + (i ^ ((lane >> 2) & 3))] = val[4 * h + i];
    __syncwarp();
    if (ok) {
      const int col = lane & 3;
      const long long base = cb[4 * h + col], stride = rs[4 * h + col];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = k * 8 + (lane >> 2);
        const double x = stg[r * 4 + (col ^ ((r >> 2) & 3))];
        if (row0 + r < M && base >= 0) out[base + (long long)(row0 + r) * stride] = x;
      }
    }
    __syncwarp();
  }
}

// Slot table of the slots k0 .. k0+kc-1 of a group (one warp; kc <= KMAX):
// lanes take segments 32 at a time, an inclusive scan places each segment's
// k range, and the part of it inside the window is written.  Returns the
// number of slots in the window; sets *scaled when one of them has a weight
// other than 1.
__device__ int build_slots_window(const Group &g, const Seg *__restrict__ segs, const Bufs &bufs, Slot *slots,
                                  int lane, int k0, int kc, int *scaled) {
  kc = min(kc, KMAX);
  const int k1 = k0 + kc;
  int base = 0;
  unsigned sc = 0;
  for (int s0 = 0; s0 < g.nseg && base < k1; s0 += 32) {
    const int sidx = s0 + lane;
    Seg sg;
    int k = 0;
    if (sidx < g.nseg) {
      sg = segs[g.seg0 + sidx];
      k = sg.K;
    }
    int incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int first = base + incl - k;  // global slot of the segment's k = 0
    const int lo = max(first, k0), hi = min(first + k, k1);
    const bool in = k > 0 && lo < hi;
    if (in) {
      const double *A = bufs.p[sg.abuf] + sg.a_off;
      const double *B = g.ncb ? bufs.p[sg.bbuf] : bufs.p[sg.bbuf] + sg.b_off;
      for (int gj = lo; gj < hi; ++gj) {
        const int j = gj - first;
        Slot &sl = slots[gj - k0];
        sl.a = A + (int64_t)j * sg.sak;
        sl.b = g.ncb ? B : B + (int64_t)j * sg.sbk;
        sl.sam = sg.sam;
        sl.sbn = sg.sbn;
        sl.alpha = sg.alpha;
        sl.scaled = sg.alpha != 1.0;
        sl.seg = sidx;
        sl.kk = j;
      }
    }
    sc |= __ballot_sync(0xffffffffu, in && sg.alpha != 1.0);
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
  *scaled = sc != 0u;
  return max(0, min(kc, base - k0));
}

// rows of a row tile rounded up to 8 (the rows an A record holds)
__device__ __forceinline__ int tile_rows8(int M, int m0) { return (min(TM, M - m0) + 7) & ~7; }

// A(row, slot j), with the slot's weight when the group has weights
__device__ __forceinline__ double load_a(const Slot &sl, int row, bool scaled) {
  double x = __ldg(sl.a + (int64_t)row * sl.sam);
  if (scaled && sl.scaled) x *= sl.alpha;
  return x;
}

}  // namespace umma

// ------------------------------------------------------------ prepare kernels
// One A record per item (rows m0 .. m0+tm8-1, slots k0 .. k0+kc-1 of the
// group), a block of 4096 elements at a time: the raw FP64 values are copied
// into shared memory with asynchronous 8-byte copies (cp.async, zero-filled
// past the rows and slots of the item), the row exponents are taken there,
// and the rows are cut from there into the four digit planes of every k
// block (a warp writes 8 rows x 4 chunks = 512 contiguous bytes of each
// plane); the 128 exponents follow the planes.  Every value is read once.
//
// A block is RB rows x W slots with W = the window's slots rounded up to a
// power of two (32 .. 256) and RB = 4096 / W (128 .. 16 rows), so items with
// a short K take many rows per block.  The copies run along the rows when a
// slot's rows are contiguous (unit row stride), else along the slots.  The
// copies hold no registers, so many blocks per SM keep enough copies in
// flight.  The slot table keeps what the copies need: the address of row 0,
// the row stride and the weight of every slot of the window (weights are
// applied when the staged values are read).
constexpr int PREP_ELEMS = 4096;              // elements of a staging block
constexpr int PREP_LOADS = PREP_ELEMS / umma::PREP_THREADS;  // 16 per thread and block
// staging row pitch in float64: W + 2 (= 2 mod 16), so the 16 lanes of a half
// warp reading (4 rows x 4 chunks) in the cut meet at most 2-way bank
// conflicts; the largest block is 128 rows x (32 + 2)
constexpr int PREP_STAGE = 128 * (32 + 2);
static_assert(umma::PREP_THREADS == 256 && PREP_LOADS == 16, "prepare-kernel thread map");
static_assert(PREP_STAGE >= 16 * (umma::KMAX + 2) && PREP_STAGE >= 64 * (64 + 2) && PREP_STAGE >= 32 * (128 + 2),
              "staging buffer of every block shape");

namespace umma {
struct ASlotTable {
  const double *a[KMAX];   // A(row 0, slot)
  int64_t sam[KMAX];       // row stride
  double alpha[KMAX];      // weight
};

// The table of the slots k0 .. k0+kc-1 of a group, written by one warp
// (kc <= KMAX): lanes take segments 32 at a time, an inclusive scan places
// each segment's k range, then the warp writes the window part of each of
// the 32 segments in turn, one slot per lane.  Returns the number of slots
// in the window; sets *scaled when one of them has a weight other than 1.
__device__ int build_a_slots(const Group &g, const Seg *__restrict__ segs, const Bufs &bufs, ASlotTable &t,
                             int lane, int k0, int kc, int *scaled) {
  kc = min(kc, KMAX);
  const int k1 = k0 + kc;
  int base = 0;
  unsigned sc = 0;
  for (int s0 = 0; s0 < g.nseg && base < k1; s0 += 32) {
    const int sidx = s0 + lane;
    Seg sg;
    int k = 0;
    if (sidx < g.nseg) {
      sg = segs[g.seg0 + sidx];
      k = sg.K;
    }
    int incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int first = base + incl - k;  // global slot of the segment's k = 0
    const int lo = max(first, k0), hi = min(first + k, k1);
    const bool in = k > 0 && lo < hi;
    const unsigned inmask = __ballot_sync(0xffffffffu, in);
    sc |= __ballot_sync(0xffffffffu, in && sg.alpha != 1.0);
    const double *A = in ? bufs.p[sg.abuf] + sg.a_off : nullptr;
    const long long sak = in ? sg.sak : 0, sam = in ? sg.sam : 0;
    const double alpha = in ? sg.alpha : 1.0;
    for (unsigned m = inmask; m; m &= m - 1) {
      const int src = __ffs(m) - 1;
      const int slo = __shfl_sync(0xffffffffu, lo, src), shi = __shfl_sync(0xffffffffu, hi, src);
      const int sfirst = __shfl_sync(0xffffffffu, first, src);
      const double *sA = reinterpret_cast<const double *>(
          __shfl_sync(0xffffffffu, reinterpret_cast<long long>(A), src));
      const long long ssak = __shfl_sync(0xffffffffu, sak, src), ssam = __shfl_sync(0xffffffffu, sam, src);
      const double salpha = __shfl_sync(0xffffffffu, alpha, src);
      for (int gj = slo + lane; gj < shi; gj += 32) {
        t.a[gj - k0] = sA + (int64_t)(gj - sfirst) * ssak;
        t.sam[gj - k0] = ssam;
        t.alpha[gj - k0] = salpha;
      }
    }
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
  *scaled = sc != 0u;
  return max(0, min(kc, base - k0));
}
}  // namespace umma

__global__ void __launch_bounds__(umma::PREP_THREADS, 4)
k_prep_a(const PrepA *__restrict__ items, int64_t nitems, const Group *__restrict__ groups,
         const Seg *__restrict__ segs, Bufs bufs, unsigned char *__restrict__ planes) {
  using namespace umma;
  __shared__ ASlotTable tab;
  __shared__ int s_ctl[2];
  __shared__ int s_ea[TM];
  extern __shared__ double stage[];  // PREP_STAGE: RB rows x (W + 2)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t stage_s = smem_u32(stage);
  for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const PrepA p = items[it];
    const Group g = groups[p.group];
    if (warp == 0) {
      int sc;
      const int K = build_a_slots(g, segs, bufs, tab, lane, p.k0, p.kc, &sc);
      if (lane == 0) {
        s_ctl[0] = K;
        s_ctl[1] = sc;
      }
    }
    if (tid < TM) s_ea[tid] = 0;
    __syncthreads();
    const int K = s_ctl[0];
    const bool scaled = s_ctl[1] != 0;
    const int nkb = (K + KB_SLOTS - 1) / KB_SLOTS, kpad = nkb * KB_SLOTS;
    const int tm8 = tile_rows8(g.M, p.m0), PL = tm8 * ROW_BYTES;
    // block shape: W = kpad rounded up to a power of two, RB = 4096 / W rows
    const int lw = nkb <= 1 ? 5 : (nkb <= 2 ? 6 : (nkb <= 4 ? 7 : 8));  // log2 W
    const int W = 1 << lw, lrb = 12 - lw, RB = 1 << lrb, pitch = W + 2;
    // rows contiguous for a slot (unit row stride): copies along the rows
    const bool rows_fast = K > 0 && tab.sam[0] == 1;
    // element e = tid + 256 i of a block: along the rows, the thread's row is
    // tid mod RB and its slots tid / RB + (256 / RB) i; along the slots, its
    // slot is tid mod W and its rows tid / W + (256 / W) i
    const int t_r = rows_fast ? (tid & (RB - 1)) : (tid >> lw);
    const int t_j = rows_fast ? (tid >> lrb) : (tid & (W - 1));
    const int step = rows_fast ? (PREP_THREADS >> lrb) : (PREP_THREADS >> lw);
    unsigned char *rec = planes + p.rec;
    for (int rb = 0; rb < tm8; rb += RB) {
#pragma unroll 4
      for (int i = 0; i < PREP_LOADS; ++i) {
        const int r = rows_fast ? t_r : t_r + step * i;
        const int j = rows_fast ? t_j + step * i : t_j;
        if (j >= kpad) continue;
        const int grow = p.m0 + rb + r;
        const bool ok = j < K && grow < g.M;
        // an empty element copies nothing (source size 0, zero fill) from a valid address
        const double *src = ok ? tab.a[j] + (int64_t)grow * tab.sam[j] : reinterpret_cast<const double *>(planes);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(stage_s + 8u * (uint32_t)(r * pitch + j)),
                     "l"(src), "r"(ok ? 8 : 0)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      __syncthreads();
      {  // row exponents: 256 / RB threads per row
        const int ltpr = 8 - lrb, tpr = 1 << ltpr;
        const int r = tid >> ltpr, part = tid & (tpr - 1);
        int em = 0;
        for (int j = part; j < kpad; j += tpr) {
          double x = stage[r * pitch + j];
          if (scaled) x *= tab.alpha[j < K ? j : 0];
          em = max(em, dexp(x));
        }
        for (int o = tpr >> 1; o >= 1; o >>= 1) em = max(em, __shfl_xor_sync(0xffffffffu, em, o));
        if (rb + r < tm8 && part == 0) s_ea[rb + r] = em;
      }
      __syncthreads();
      for (int u = tid; u < (nkb << (lrb + 2)); u += PREP_THREADS) {
        const int ch = u & 3, r = (u >> 2) & (RB - 1), kb = u >> (lrb + 2);
        if (rb + r >= tm8) continue;
        double x[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int j = kb * KB_SLOTS + ch * 8 + i;
          x[i] = stage[r * pitch + j];
          if (scaled) x[i] *= tab.alpha[j < K ? j : 0];
        }
        cut8_store(x, s_ea[rb + r], rec + (int64_t)kb * 4 * PL, PL, rb + r, ch);
      }
      __syncthreads();  // the staging block is refilled
    }
    if (tid < TM) reinterpret_cast<int *>(rec + (int64_t)nkb * 4 * PL)[tid] = s_ea[tid];
    __syncthreads();  // the slot table and the exponents are rewritten by the next item
  }
}

// One B record per item (columns n0 .. n0+tn-1, slots k0 .. k0+kc-1): the
// column exponents over the window (column-block look-ups once per column),
// the four digit planes of every k block (plane s holds rows s*tn + c), then
// the exponents after the planes.
__global__ void __launch_bounds__(umma::PREP_THREADS)
k_prep_b(const PrepB *__restrict__ items, int64_t nitems, const Group *__restrict__ groups,
         const Seg *__restrict__ segs, const ColBlock *__restrict__ cbl, const SegB *__restrict__ segb, Bufs bufs,
         unsigned char *__restrict__ planes) {
  using namespace umma;
  __shared__ Slot slots[KMAX];
  __shared__ int s_ctl[2];
  __shared__ int s_eb[64], s_jb[64], s_rel[64];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const PrepB p = items[it];
    const Group g = groups[p.group];
    const int tn = p.tn;
    if (warp == 0) {
      int sc;
      const int K = build_slots_window(g, segs, bufs, slots, lane, p.k0, p.kc, &sc);
      if (lane == 0) {
        s_ctl[0] = K;
        s_ctl[1] = sc;
      }
    }
    for (int c = tid; c < tn; c += PREP_THREADS) {
      int rel = 0;
      s_jb[c] = g.ncb ? find_cblock(cbl, g, p.n0 + c, rel) : -1;
      s_rel[c] = rel;
      s_eb[c] = 0;
    }
    __syncthreads();
    const int K = s_ctl[0];
    const int nkb = (K + KB_SLOTS - 1) / KB_SLOTS;
    auto load_b = [&](int j, int c) -> double {
      const int col = p.n0 + c;
      if (j >= K || col >= g.N) return 0.0;
      return g.ncb ? load_b_cb(slots[j], segb, g, s_jb[c], s_rel[c])
                   : __ldg(slots[j].b + (int64_t)col * slots[j].sbn);
    };
    for (int u = tid; u < tn * nkb * 4; u += PREP_THREADS) {
      const int c = u % tn, g8 = u / tn;
      double v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = load_b(g8 * 8 + i, c);
      int em = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) em = max(em, dexp(v[i]));
      if (em) atomicMax(s_eb + c, em);
    }
    __syncthreads();
    unsigned char *rec = planes + p.rec;
    unsigned char *tail = rec + (int64_t)nkb * umma_b_kb_bytes(tn);
    for (int c = tid; c < tn; c += PREP_THREADS) reinterpret_cast<int *>(tail)[c] = s_eb[c];
    for (int u = tid; u < nkb * tn * 4; u += PREP_THREADS) {
      const int kb = u / (tn * 4), c = (u >> 2) % tn, ch = u & 3;
      double v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = load_b(kb * KB_SLOTS + ch * 8 + i, c);
      cut8_store(v, s_eb[c], rec + (int64_t)kb * umma_b_kb_bytes(tn), tn * ROW_BYTES, c, ch);
    }
    __syncthreads();  // the slot table and the column arrays are rewritten by the next item
  }
}

// ------------------------------------------------------------------ kernel
template <int TN, int NKBB>
__global__ void __launch_bounds__(umma::NTHREADS, 1)
k_step_umma(const UWork *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
            const unsigned char *__restrict__ planes, const int64_t *__restrict__ cmaps, Bufs bufs) {
  using namespace umma;
  using LY = Layout<TN, NKBB>;
  constexpr int NSTAGE = LY::NSTAGE;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw_s = smem_u32(smem_raw);
  const uint32_t base_s = (raw_s + 1023u) & ~1023u;
  unsigned char *sm = smem_raw + (base_s - raw_s);
  unsigned char *rec0 = sm + LY::OFF_REC;
  const uint32_t bar0 = base_s + LY::OFF_BAR;
  uint32_t *misc = reinterpret_cast<uint32_t *>(sm + LY::OFF_MISC);  // [0] tmem, [1] abort
  volatile int *abort_flag = reinterpret_cast<volatile int *>(misc + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };

  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(misc)),
                 "r"(LY::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      bar_init(bar(BAR_T_FULL + s), 1);
      bar_init(bar(BAR_T_EMPTY + s), EPI_WARPS * 32);
      bar_init(bar(BAR_E_FULL + s), 1);
      bar_init(bar(BAR_E_EMPTY + s), EPI_WARPS * 32);
    }
    for (int s = 0; s < 2; ++s) {
      bar_init(bar(BAR_B_FULL + s), 1);
      bar_init(bar(BAR_B_FREE + s), 1);
    }
    bar_init(bar(BAR_DONE), 1);
    for (int s = 0; s < NSTAGE; ++s) {
      bar_init(bar(BAR_A_FULL + s), 1);
      bar_init(bar(LY::BAR_A_EMPTY + s), 1);
    }
    misc[1] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = misc[0];

  if (warp == PROD_WARP) {
    // ================================================================ producer
    if (lane == 0) {
      uint32_t t = 0, q = 0, item = 0;
      uint32_t nA[NSTAGE], nE[2] = {0u, 0u}, nB[2] = {0u, 0u};  // phases armed per barrier (for the drain)
#pragma unroll
      for (int s = 0; s < NSTAGE; ++s) nA[s] = 0;
      bool ok = true;
      for (int64_t w = blockIdx.x; ok && w < nwork; w += gridDim.x, ++item) {
        if (*abort_flag) break;
        const UWork wk = work[w];
        const Group g = groups[wk.group];
        const int nrt = wk.nrt_k & 0xff, K = wk.nrt_k >> 8;
        const int nkb = (K + KB_SLOTS - 1) / KB_SLOTS;
        const unsigned char *brec = planes + wk.b_rec;
        if (nkb > NKBB) {  // the planner routes every item to a launch whose B region holds it
          *abort_flag = 1;
          atomicCAS(&g_umma_error, 0, ERR_B_TILE);
          break;
        }
        // B buffer of the item and its earlier uses
        const uint32_t bb = LY::NBB == 2 ? (item & 1) : 0, ub = LY::NBB == 2 ? (item >> 1) : item;
        if (!(ok = wait_bounded(bar(BAR_B_FREE + bb), (ub & 1) ^ 1, abort_flag, 1))) break;
        bar_arrive_tx(bar(BAR_B_FULL + bb), (uint32_t)(nkb * LY::B_KB));
        bulk_g2s(base_s + LY::OFF_B + bb * (NKBB * LY::B_KB), brec, (uint32_t)(nkb * LY::B_KB),
                 bar(BAR_B_FULL + bb));
        ++nB[bb];
        const unsigned char *arec = planes + wk.a_rec;
        for (int r = 0; r < nrt; ++r, ++t) {
          const uint32_t b = t & 1, u = t >> 1;
          const int m0 = wk.m0 + r * TM, akb = 4 * tile_rows8(g.M, m0) * ROW_BYTES;  // bytes of an A k block
          if (!(ok = wait_bounded(bar(BAR_E_EMPTY + b), (u & 1) ^ 1, abort_flag, 2))) break;
          unsigned char *rec = rec0 + b * LY::REC_BYTES;
          const uint32_t rec_s = base_s + LY::OFF_REC + b * LY::REC_BYTES;
          int *info = reinterpret_cast<int *>(rec + LY::REC_INFO);
          info[0] = m0;
          info[1] = g.M;
          info[2] = g.cbuf;
          bar_arrive_tx(bar(BAR_E_FULL + b), (uint32_t)(TM * 4 + TN * 20));
          bulk_g2s(rec_s + LY::REC_EA, arec + (int64_t)nkb * akb, TM * 4, bar(BAR_E_FULL + b));
          bulk_g2s(rec_s + LY::REC_EB, brec + (int64_t)nkb * LY::B_KB, TN * 4, bar(BAR_E_FULL + b));
          bulk_g2s(rec_s + LY::REC_CB, cmaps + wk.cmap, TN * 16, bar(BAR_E_FULL + b));
          ++nE[b];
          for (int kb = 0; kb < nkb; ++kb, ++q) {
            const uint32_t s = q % NSTAGE, use = q / NSTAGE;
            if (!(ok = wait_bounded(bar(LY::BAR_A_EMPTY + s), (use & 1) ^ 1, abort_flag, 3))) break;
            bar_arrive_tx(bar(BAR_A_FULL + s), (uint32_t)akb);
            bulk_g2s(base_s + LY::OFF_A + s * A_STAGE, arec + (int64_t)kb * akb, (uint32_t)akb, bar(BAR_A_FULL + s));
            ++nA[s];
          }
          if (!ok) break;
          arec += (int64_t)nkb * akb + TM * 4;
        }
      }
      // drain: every bulk copy issued has landed before the CTA may exit
#pragma unroll
      for (int s = 0; s < NSTAGE; ++s)
        if (nA[s]) wait_bounded(bar(BAR_A_FULL + s), (nA[s] - 1) & 1, abort_flag, 10, false);
      for (int b = 0; b < 2; ++b)
        if (nE[b]) wait_bounded(bar(BAR_E_FULL + b), (nE[b] - 1) & 1, abort_flag, 11, false);
      for (int b = 0; b < 2; ++b)
        if (nB[b]) wait_bounded(bar(BAR_B_FULL + b), (nB[b] - 1) & 1, abort_flag, 12, false);
    }
    __syncwarp();
  } else if (warp == MMA_WARP) {
    // ====================================================================== MMA
    if (lane == 0) {
      uint32_t q = 0, t = 0, item = 0;
      for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x, ++item) {
        if (*abort_flag) break;
        const UWork wk = work[w];
        const int M = groups[wk.group].M;
        const int nrt = wk.nrt_k & 0xff, K = wk.nrt_k >> 8;
        const int nkb = (K + KB_SLOTS - 1) / KB_SLOTS;
        const uint32_t bb = LY::NBB == 2 ? (item & 1) : 0, ub = LY::NBB == 2 ? (item >> 1) : item;
        const bool okb = wait_bounded(bar(BAR_B_FULL + bb), ub & 1, abort_flag, 4);
        tc_fence_after();
        for (int r = 0; r < nrt; ++r, ++t) {
          const uint32_t b = t & 1, u = t >> 1;
          // planes of the A record are tm8 rows apart; the MMA reads 128 rows
          // from each (rows past tm8 land in TMEM lanes the epilogue skips)
          const uint32_t PL = (uint32_t)(tile_rows8(M, wk.m0 + r * TM) * ROW_BYTES);
          wait_bounded(bar(BAR_T_EMPTY + b), (u & 1) ^ 1, abort_flag, 5);
          tc_fence_after();
          for (int kb = 0; kb < nkb; ++kb, ++q) {
            const uint32_t s = q % NSTAGE, use = q / NSTAGE;
            const bool ok = wait_bounded(bar(BAR_A_FULL + s), use & 1, abort_flag, 6);
            tc_fence_after();
            if (ok && okb && !*abort_flag) {
              const uint32_t a_s = base_s + LY::OFF_A + s * A_STAGE;
              const uint32_t b_s = base_s + LY::OFF_B + bb * (NKBB * LY::B_KB) + kb * LY::B_KB;
#pragma unroll
              for (int k16 = 0; k16 < 2; ++k16) {
                if (kb * KB_SLOTS + k16 * 16 >= K) break;
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                  const uint32_t d = tmem + b * (4 * TN) + a * TN;
                  mma(d, sdesc(a_s + a * PL + k16 * 32), sdesc(b_s + k16 * 32), idesc((4 - a) * TN),
                      (kb | k16 | a) != 0);
                }
              }
            }
            commit(bar(LY::BAR_A_EMPTY + s));
          }
          commit(bar(BAR_T_FULL + b));
        }
        commit(bar(BAR_B_FREE + bb));
      }
      commit(bar(BAR_DONE));
    }
    __syncwarp();
  } else {
    // ================================================================= epilogue
    // warp w reads TMEM lanes 32(w%4).. (tile rows) and every fourth 8-column
    // chunk (from column 8(w/4))
    const int quarter = warp & 3, group = warp >> 2;
    const int e = quarter * 32 + lane;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    double *stg = reinterpret_cast<double *>(sm + LY::OFF_STG) + warp * 128;
    uint32_t t = 0;
    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
      if (role_sync_or(2, EPI_WARPS * 32, *abort_flag != 0)) break;
      const UWork wk = work[w];
      const int nrt = wk.nrt_k & 0xff;
      for (int r = 0; r < nrt; ++r, ++t) {
        const uint32_t b = t & 1, u = t >> 1;
        const bool ok_rec = wait_bounded(bar(BAR_E_FULL + b), u & 1, abort_flag, 7);
        const unsigned char *rec = rec0 + b * LY::REC_BYTES;
        const int *info = reinterpret_cast<const int *>(rec + LY::REC_INFO);
        const int m0 = info[0], M = info[1], cbuf = info[2];
        const int ea = reinterpret_cast<const int *>(rec + LY::REC_EA)[e];
        const int *eb = reinterpret_cast<const int *>(rec + LY::REC_EB);
        const long long *cb = reinterpret_cast<const long long *>(rec + LY::REC_CB);
        const long long *rs = reinterpret_cast<const long long *>(rec + LY::REC_RS);
        // stores only when the tile record and the accumulators are both this
        // tile's (an aborting MMA issuer commits without having multiplied)
        const bool ok_acc = wait_bounded(bar(BAR_T_FULL + b), u & 1, abort_flag, 8);
        const bool ok = ok_rec && ok_acc && *abort_flag == 0;
        tc_fence_after();
        double *out = bufs.p[ok ? cbuf : 0];
#pragma unroll 1
        for (int c0 = 8 * group; c0 < TN; c0 += CHUNK_STEP) {
          uint32_t v[4][8];
          const uint32_t ta = tmem + lane_base + b * (4 * TN) + c0;
#pragma unroll
          for (int l = 0; l < 4; ++l) tmem_ld8(ta + l * TN, v[l]);
          tmem_ld_wait();
          double val[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const long long S = fold_levels(v[0][i], v[1][i], v[2][i], v[3][i]);
            val[i] = scaled_int_to_double(S, ea + eb[c0 + i] - BIAS);
          }
          store_chunk(stg, val, lane, m0 + quarter * 32, M, cb + c0, rs + c0, out, ok);
        }
        tc_fence_before();
        bar_arrive(bar(BAR_T_EMPTY + b));
        bar_arrive(bar(BAR_E_EMPTY + b));
      }
    }
  }

  // ---- teardown: wait for the MMA issuer's last commit, release TMEM
  tc_fence_before();
  __syncthreads();
  if (warp == MMA_WARP) {
    tc_fence_after();
    // the issuer's last commit completes once every MMA it issued has
    // finished writing TMEM (waited for even when aborting)
    if (lane == 0) wait_bounded(bar(BAR_DONE), 0, abort_flag, 9, false);
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(LY::TMEM_COLS)
                 : "memory");
  }
}

// ------------------------------------------------------------- long kernel
// Groups with a longer K than one pass (at most kUmmaLongMaxK slots: the
// split-K parts of longer groups): a work item is one row tile and one
// column tile over every pass of 256 slots.  Each pass has its own A and B
// records (own exponents), so a stage of the ring carries one k block of
// both; the tile's result of a pass, exact as in the one-pass kernel, is
// added in FP64 (pass order) to the epilogue's per-thread accumulators, and
// the sum is stored once after the last pass.
template <int TN>
struct LongLayout {
  static constexpr int NSTAGE = 4;
  static constexpr int B_KB = 4 * TN * umma::ROW_BYTES;
  static constexpr int STAGE = umma::A_STAGE + B_KB;      // A k block (128-row planes) + B k block
  static constexpr int OFF_S = 0;
  static constexpr int OFF_REC = OFF_S + NSTAGE * STAGE;
  static constexpr int REC_EA = 0;
  static constexpr int REC_EB = REC_EA + umma::TM * 4;
  static constexpr int REC_CB = REC_EB + TN * 4;
  static constexpr int REC_RS = REC_CB + TN * 8;
  static constexpr int REC_INFO = REC_RS + TN * 8;
  static constexpr int REC_BYTES = REC_INFO + 16;
  static constexpr int OFF_STG = OFF_REC + 2 * REC_BYTES;  // epilogue staging, 2 KB per warp
  static constexpr int OFF_BAR = OFF_STG + umma::STG_BYTES;
  // barriers: T_FULL[2], T_EMPTY[2], E_FULL[2], E_EMPTY[2], DONE, S_FULL[NSTAGE], S_EMPTY[NSTAGE]
  static constexpr int BAR_DONE = 8, BAR_S_FULL = 9, BAR_S_EMPTY = BAR_S_FULL + NSTAGE;
  static constexpr int NBAR = BAR_S_EMPTY + NSTAGE;
  static constexpr int OFF_MISC = OFF_BAR + NBAR * 8;
  static constexpr int BYTES = OFF_MISC + 16;
  static constexpr int SMEM = BYTES + 1024;
  static constexpr int TMEM_COLS = 8 * TN;
  static_assert(TN == 16 || TN == 32 || TN == 64, "column tile");
  static_assert(STAGE % 1024 == 0 && B_KB % 1024 == 0, "swizzle atoms");
  static_assert(OFF_REC % 16 == 0 && REC_EB % 16 == 0 && REC_BYTES % 16 == 0, "bulk-copy alignment");
  static_assert(SMEM <= 232448, "shared memory");
};

template <int TN>
__global__ void __launch_bounds__(umma::NTHREADS, 1)
k_step_umma_long(const UWork *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
                 const unsigned char *__restrict__ planes, const int64_t *__restrict__ cmaps, Bufs bufs) {
  using namespace umma;
  using LY = LongLayout<TN>;
  constexpr int NSTAGE = LY::NSTAGE;
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw_s = smem_u32(smem_raw);
  const uint32_t base_s = (raw_s + 1023u) & ~1023u;
  unsigned char *sm = smem_raw + (base_s - raw_s);
  unsigned char *rec0 = sm + LY::OFF_REC;
  const uint32_t bar0 = base_s + LY::OFF_BAR;
  uint32_t *misc = reinterpret_cast<uint32_t *>(sm + LY::OFF_MISC);  // [0] tmem, [1] abort
  volatile int *abort_flag = reinterpret_cast<volatile int *>(misc + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };

  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(misc)),
                 "r"(LY::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      bar_init(bar(BAR_T_FULL + s), 1);
      bar_init(bar(BAR_T_EMPTY + s), EPI_WARPS * 32);
      bar_init(bar(BAR_E_FULL + s), 1);
      bar_init(bar(BAR_E_EMPTY + s), EPI_WARPS * 32);
    }
    bar_init(bar(LY::BAR_DONE), 1);
    for (int s = 0; s < NSTAGE; ++s) {
      bar_init(bar(LY::BAR_S_FULL + s), 1);
      bar_init(bar(LY::BAR_S_EMPTY + s), 1);
    }
    misc[1] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = misc[0];

  if (warp == PROD_WARP) {
    // ================================================================ producer
    if (lane == 0) {
      uint32_t t = 0, q = 0;
      uint32_t nS[NSTAGE], nE[2] = {0u, 0u};  // phases armed per barrier (for the drain)
#pragma unroll
      for (int s = 0; s < NSTAGE; ++s) nS[s] = 0;
      bool ok = true;
      for (int64_t w = blockIdx.x; ok && w < nwork; w += gridDim.x) {
        if (*abort_flag) break;
        const UWork wk = work[w];
        const Group g = groups[wk.group];
        const int K = wk.nrt_k >> 8, npass = (K + KMAX - 1) / KMAX;
        const int akb = 4 * tile_rows8(g.M, wk.m0) * ROW_BYTES;
        const unsigned char *arec = planes + wk.a_rec, *brec = planes + wk.b_rec;
        for (int j = 0; j < npass; ++j, ++t) {
          const int kc = min(KMAX, K - j * KMAX), nkb = (kc + KB_SLOTS - 1) / KB_SLOTS;
          const uint32_t b = t & 1, u = t >> 1;
          if (!(ok = wait_bounded(bar(BAR_E_EMPTY + b), (u & 1) ^ 1, abort_flag, 2))) break;
          unsigned char *rec = rec0 + b * LY::REC_BYTES;
          const uint32_t rec_s = base_s + LY::OFF_REC + b * LY::REC_BYTES;
          int *info = reinterpret_cast<int *>(rec + LY::REC_INFO);
          info[0] = wk.m0;
          info[1] = g.M;
          info[2] = g.cbuf;
          info[3] = j == npass - 1;
          bar_arrive_tx(bar(BAR_E_FULL + b), (uint32_t)(TM * 4 + TN * 20));
          bulk_g2s(rec_s + LY::REC_EA, arec + (int64_t)nkb * akb, TM * 4, bar(BAR_E_FULL + b));
          bulk_g2s(rec_s + LY::REC_EB, brec + (int64_t)nkb * LY::B_KB, TN * 4, bar(BAR_E_FULL + b));
          bulk_g2s(rec_s + LY::REC_CB, cmaps + wk.cmap, TN * 16, bar(BAR_E_FULL + b));
          ++nE[b];
          for (int kb = 0; kb < nkb; ++kb, ++q) {
            const uint32_t s = q % NSTAGE, use = q / NSTAGE;
            if (!(ok = wait_bounded(bar(LY::BAR_S_EMPTY + s), (use & 1) ^ 1, abort_flag, 3))) break;
            const uint32_t st = base_s + LY::OFF_S + s * LY::STAGE;
            bar_arrive_tx(bar(LY::BAR_S_FULL + s), (uint32_t)(akb + LY::B_KB));
            bulk_g2s(st, arec + (int64_t)kb * akb, (uint32_t)akb, bar(LY::BAR_S_FULL + s));
            bulk_g2s(st + A_STAGE, brec + (int64_t)kb * LY::B_KB, LY::B_KB, bar(LY::BAR_S_FULL + s));
            ++nS[s];
          }
          if (!ok) break;
          arec += (int64_t)nkb * akb + TM * 4;
          brec += (int64_t)nkb * LY::B_KB + TN * 4;
        }
      }
      // drain: every bulk copy issued has landed before the CTA may exit
#pragma unroll
      for (int s = 0; s < NSTAGE; ++s)
        if (nS[s]) wait_bounded(bar(LY::BAR_S_FULL + s), (nS[s] - 1) & 1, abort_flag, 10, false);
      for (int b = 0; b < 2; ++b)
        if (nE[b]) wait_bounded(bar(BAR_E_FULL + b), (nE[b] - 1) & 1, abort_flag, 11, false);
    }
    __syncwarp();
  } else if (warp == MMA_WARP) {
    // ====================================================================== MMA
    if (lane == 0) {
      uint32_t q = 0, t = 0;
      for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
        if (*abort_flag) break;
        const UWork wk = work[w];
        const int K = wk.nrt_k >> 8, npass = (K + KMAX - 1) / KMAX;
        const uint32_t PL = (uint32_t)(tile_rows8(groups[wk.group].M, wk.m0) * ROW_BYTES);
        for (int j = 0; j < npass; ++j, ++t) {
          const int kc = min(KMAX, K - j * KMAX), nkb = (kc + KB_SLOTS - 1) / KB_SLOTS;
          const uint32_t b = t & 1, u = t >> 1;
          wait_bounded(bar(BAR_T_EMPTY + b), (u & 1) ^ 1, abort_flag, 5);
          tc_fence_after();
          for (int kb = 0; kb < nkb; ++kb, ++q) {
            const uint32_t s = q % NSTAGE, use = q / NSTAGE;
            const bool ok = wait_bounded(bar(LY::BAR_S_FULL + s), use & 1, abort_flag, 6);
            tc_fence_after();
            if (ok && !*abort_flag) {
              const uint32_t a_s = base_s + LY::OFF_S + s * LY::STAGE, b_s = a_s + A_STAGE;
#pragma unroll
              for (int k16 = 0; k16 < 2; ++k16) {
                if (kb * KB_SLOTS + k16 * 16 >= kc) break;
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                  const uint32_t d = tmem + b * (4 * TN) + a * TN;
                  mma(d, sdesc(a_s + a * PL + k16 * 32), sdesc(b_s + k16 * 32), idesc((4 - a) * TN),
                      (kb | k16 | a) != 0);
                }
              }
            }
            commit(bar(LY::BAR_S_EMPTY + s));
          }
          commit(bar(BAR_T_FULL + b));
        }
      }
      commit(bar(LY::BAR_DONE));
    }
    __syncwarp();
  } else {
    // ================================================================= epilogue
    // warp w reads TMEM lanes 32(w%4).. and every fourth 8-column chunk (from
    // column 8(w/4)); its sums (at most NCH chunks) stay in registers over
    // the passes
    constexpr int NCH = (TN / 8 + EPI_GROUPS - 1) / EPI_GROUPS;
    const int quarter = warp & 3, group = warp >> 2;
    const int e = quarter * 32 + lane;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    double *stg = reinterpret_cast<double *>(sm + LY::OFF_STG) + warp * 128;
    uint32_t t = 0;
    for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
      if (role_sync_or(2, EPI_WARPS * 32, *abort_flag != 0)) break;
      const UWork wk = work[w];
      const int K = wk.nrt_k >> 8, npass = (K + KMAX - 1) / KMAX;
      double acc[8 * NCH];
#pragma unroll
      for (int c = 0; c < 8 * NCH; ++c) acc[c] = 0.0;
      for (int j = 0; j < npass; ++j, ++t) {
        const uint32_t b = t & 1, u = t >> 1;
        const bool ok_rec = wait_bounded(bar(BAR_E_FULL + b), u & 1, abort_flag, 7);
        const unsigned char *rec = rec0 + b * LY::REC_BYTES;
        const int *info = reinterpret_cast<const int *>(rec + LY::REC_INFO);
        const int ea = reinterpret_cast<const int *>(rec + LY::REC_EA)[e];
        const int *eb = reinterpret_cast<const int *>(rec + LY::REC_EB);
        const bool ok_acc = wait_bounded(bar(BAR_T_FULL + b), u & 1, abort_flag, 8);
        const bool ok = __all_sync(0xffffffffu, ok_rec && ok_acc && *abort_flag == 0);
        tc_fence_after();
#pragma unroll
        for (int jc = 0; jc < NCH; ++jc) {
          const int c0 = 8 * group + CHUNK_STEP * jc;
          if (c0 >= TN) break;
          uint32_t v[4][8];
          const uint32_t ta = tmem + lane_base + b * (4 * TN) + c0;
#pragma unroll
          for (int l = 0; l < 4; ++l) tmem_ld8(ta + l * TN, v[l]);
          tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const long long S = fold_levels(v[0][i], v[1][i], v[2][i], v[3][i]);
            acc[8 * jc + i] += scaled_int_to_double(S, ea + eb[c0 + i] - BIAS);
          }
        }
        // the last pass stores the sums (its tile record has the column map)
        if (ok && info[3]) {
          double *out = bufs.p[info[2]];
          const long long *cb = reinterpret_cast<const long long *>(rec + LY::REC_CB);
          const long long *rs = reinterpret_cast<const long long *>(rec + LY::REC_RS);
#pragma unroll
          for (int jc = 0; jc < NCH; ++jc) {
            const int c0 = 8 * group + CHUNK_STEP * jc;
            if (c0 >= TN) break;
            store_chunk(stg, acc + 8 * jc, lane, info[0] + quarter * 32, info[1], cb + c0, rs + c0, out, true);
          }
        }
        tc_fence_before();
        bar_arrive(bar(BAR_T_EMPTY + b));
        bar_arrive(bar(BAR_E_EMPTY + b));
      }
    }
  }

  // ---- teardown: wait for the MMA issuer's last commit, release TMEM
  tc_fence_before();
  __syncthreads();
  if (warp == MMA_WARP) {
    tc_fence_after();
    if (lane == 0) wait_bounded(bar(LY::BAR_DONE), 0, abort_flag, 9, false);
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(LY::TMEM_COLS)
                 : "memory");
  }
}

template <int TN>
static int launch_umma_long_t(const UWork *work, int64_t nwork, const Step &s, const Bufs &b,
                              const unsigned char *planes, int nsm, void *stream) {
  if (nwork == 0) return ZMPO_OK;
  constexpr int smem = LongLayout<TN>::SMEM;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_step_umma_long<TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return record_cuda_error("k_step_umma_long: shared memory attribute", (int)e);
    attr = true;
  }
  const int grid = (int)(nwork < nsm ? nwork : nsm);
  k_step_umma_long<TN><<<grid, umma::NTHREADS, smem, (cudaStream_t)stream>>>(work, nwork, s.d_groups, planes,
                                                                             s.d_cmap, b);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ZMPO_OK : record_cuda_error("k_step_umma_long", (int)e);
}

template <int TN, int NKBB>
static int launch_umma_k(const UWork *work, int64_t nwork, const Step &s, const Bufs &b,
                         const unsigned char *planes, int nsm, void *stream) {
  if (nwork == 0) return ZMPO_OK;
  constexpr int smem = umma::Layout<TN, NKBB>::SMEM;
  static bool attr = false;
  if (!attr) {
    cudaError_t e =
        cudaFuncSetAttribute(k_step_umma<TN, NKBB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return record_cuda_error("k_step_umma: shared memory attribute", (int)e);
    attr = true;
  }
  const int grid = (int)(nwork < nsm ? nwork : nsm);
  k_step_umma<TN, NKBB><<<grid, umma::NTHREADS, smem, (cudaStream_t)stream>>>(work, nwork, s.d_groups, planes,
                                                                              s.d_cmap, b);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ZMPO_OK : record_cuda_error("k_step_umma", (int)e);
}

// The one-pass items of a column tile lie in the list by the k blocks of
// their B tile (more than 4, 3-4, at most 2): one launch per class, with the
// A ring its B tile leaves room for.
template <int TN>
static int launch_umma_t(const UWork *work, const int64_t *ncls, const Step &s, const Bufs &b,
                         const unsigned char *planes, int nsm, void *stream) {
  int rc;
  if ((rc = launch_umma_k<TN, umma::NKB_MAX>(work, ncls[0], s, b, planes, nsm, stream))) return rc;
  if ((rc = launch_umma_k<TN, 4>(work + ncls[0], ncls[1], s, b, planes, nsm, stream))) return rc;
  return launch_umma_k<TN, 2>(work + ncls[0] + ncls[1], ncls[2], s, b, planes, nsm, stream);
}

int launch_step_umma(const Step &s, const Bufs &b, unsigned char *planes, bool cut_kept, void *stream) {
  if (s.nprep_a == 0 && s.nprep_b == 0) return ZMPO_OK;
  if (!planes) return record_arg_error("tensor-core groups without a plane buffer");
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t cap = (int64_t)nsm * 8;
  // the kept records (first items of each list) are cut unless the caller
  // reuses those of the previous call
  const int64_t a0 = cut_kept ? 0 : s.nprep_a_kept, b0 = cut_kept ? 0 : s.nprep_b_kept;
  const int64_t na = s.nprep_a - a0, nb = s.nprep_b - b0;
  if (na > 0) {
    constexpr int stage_bytes = PREP_STAGE * (int)sizeof(double);
    k_prep_a<<<(int)(na < cap ? na : cap), umma::PREP_THREADS, stage_bytes, (cudaStream_t)stream>>>(
        s.d_prep_a + a0, na, s.d_groups, s.d_segs, b, planes);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_cuda_error("k_prep_a", (int)e);
  }
  if (nb > 0) {
    k_prep_b<<<(int)(nb < cap ? nb : cap), umma::PREP_THREADS, 0, (cudaStream_t)stream>>>(
        s.d_prep_b + b0, nb, s.d_groups, s.d_segs, s.d_cblocks, s.d_segb, b, planes);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_cuda_error("k_prep_b", (int)e);
  }
  int rc;
  if ((rc = launch_umma_long_t<64>(s.d_work_ul[2], s.nwork_ul[2], s, b, planes, nsm, stream))) return rc;
  if ((rc = launch_umma_long_t<32>(s.d_work_ul[1], s.nwork_ul[1], s, b, planes, nsm, stream))) return rc;
  if ((rc = launch_umma_long_t<16>(s.d_work_ul[0], s.nwork_ul[0], s, b, planes, nsm, stream))) return rc;
  if ((rc = launch_umma_t<64>(s.d_work_um[2], s.nwork_um_cls[2], s, b, planes, nsm, stream))) return rc;
  if ((rc = launch_umma_t<32>(s.d_work_um[1], s.nwork_um_cls[1], s, b, planes, nsm, stream))) return rc;
  return launch_umma_t<16>(s.d_work_um[0], s.nwork_um_cls[0], s, b, planes, nsm, stream);
}

int umma_device_status(int *code, int reset) {
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_umma_error, sizeof(int));
  if (e != cudaSuccess) return record_cuda_error("device_status", (int)e);
  if (code) *code = v;
  if (reset && v) {
    const int z = 0;
    e = cudaMemcpyToSymbol(g_umma_error, &z, sizeof(int));
    if (e != cudaSuccess) return record_cuda_error("device_status reset", (int)e);
  }
  return ZMPO_OK;
}

}  // namespace zmpo
