// Device kernels of the GB300 DMRG engine.
//
// A "step" is one grouped launch over many block products (see engine.h):
// every output sub-matrix (group) is owned by one CTA tile, which loops over
// the group's segments (strided GEMMs) and writes the result once.  Two
// arithmetic paths share the task lists:
//
//   k_step_fp64   FP64 FMA on the CUDA cores (reference arithmetic).
//   k_step_tc     the split path: FP64 operands cut into S exact digit planes
//   k_step_tcb    per K-chunk (a shared power-of-two scale per row of A and
//                 per column of B, Ozaki-style), digit products on the BF16
//                 tensor cores (mma.sync m16n8k16, FP32 accumulate, exact:
//                 every per-level sum stays below 2^24), per-chunk results
//                 scaled by powers of two and summed in a two-float (hi+lo)
//                 accumulator on the FP32 pipes; FP64 only for the final
//                 store.  S = 4 (balanced digits of 31 bits, |digit| <= 128)
//                 keeps the level pairs s+t <= 3 (10 products, ~2^-31
//                 relative to the row/column maximum); S = 7 (unsigned
//                 bytes) keeps 28 products (~2^-56).  k_step_tcb is the
//                 B-resident variant for groups whose K fits one pass.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zmpo_gb300.h"
#include "device_common.cuh"
#include "engine.h"

namespace zmpo {

static int launch_error(const char *where) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return ZMPO_OK;
  return record_cuda_error(where, (int)e);
}

static int grid_for(int64_t nwork, int per_sm) {
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int64_t g = (int64_t)nsm * per_sm;
  if (nwork < g) g = nwork;
  return (int)(g < 1 ? 1 : g);
}

// C(r, c) of a group; column-block groups use the tile's map (c - n0 indexes it)
__device__ __forceinline__ void store_c(const Bufs &bufs, const ColBlock *__restrict__ cbl, const Group &g,
                                        int r, int c, int n0, const int *cbj, const int *cbrel, double v) {
  if (g.ncb == 0) {
    bufs.p[g.cbuf][g.c_off + (int64_t)r * g.scm + (int64_t)c * g.scn] = v;
    return;
  }
  const int j = cbj[c - n0];
  if (j < 0) return;
  const ColBlock cb = cbl[g.cb0 + j];
  bufs.p[g.cbuf][cb.c_off + (int64_t)r * cb.scm + (int64_t)cbrel[c - n0] * cb.scn] = v;
}

// ------------------------------------------------------------------ FP64
constexpr int F_TM = 32, F_TN = 32, F_TK = 16, F_NT = 256;

__global__ void __launch_bounds__(F_NT)
k_step_fp64(const Work *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
            const Seg *__restrict__ segs, const ColBlock *__restrict__ cbl, const SegB *__restrict__ segb,
            Bufs bufs) {
  __shared__ double As[F_TK][F_TM + 1];
  __shared__ double Bs[F_TK][F_TN + 1];
  __shared__ int cbj[F_TN], cbrel[F_TN];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
    const Work wk = work[w];
    const Group g = groups[wk.group];
    const int m0 = wk.mt, n0 = wk.nt;
    if (g.ncb) tile_cblocks(cbl, g, n0, F_TN, cbj, cbrel);
    __syncthreads();
    double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
    for (int si = 0; si < g.nseg; ++si) {
      const Seg s = segs[g.seg0 + si];
      const double *A = bufs.p[s.abuf] + s.a_off;
      const double *B = bufs.p[s.bbuf] + s.b_off;
      const bool a_kfast = s.sak == 1, b_nfast = s.sbn == 1;
      const bool scaled = s.alpha != 1.0;
      for (int k0 = 0; k0 < s.K; k0 += F_TK) {
        for (int e = tid; e < F_TM * F_TK; e += F_NT) {
          int r, k;
          if (a_kfast) { r = e / F_TK; k = e % F_TK; } else { r = e % F_TM; k = e / F_TM; }
          double v = 0.0;
          if (m0 + r < g.M && k0 + k < s.K) {
            v = A[(int64_t)(m0 + r) * s.sam + (int64_t)(k0 + k) * s.sak];
            if (scaled) v *= s.alpha;
          }
          As[k][r] = v;
        }
        for (int e = tid; e < F_TK * F_TN; e += F_NT) {
          int k, c;
          if (b_nfast) { k = e / F_TN; c = e % F_TN; } else { c = e / F_TK; k = e % F_TK; }
          double v = 0.0;
          if (n0 + c < g.N && k0 + k < s.K) {
            if (g.ncb == 0) {
              v = B[(int64_t)(k0 + k) * s.sbk + (int64_t)(n0 + c) * s.sbn];
            } else {
              const int j = cbj[c];
              if (j >= 0) {
                const SegB sb = segb[g.sb0 + (int64_t)si * g.ncb + j];
                if (sb.b_off >= 0)
                  v = bufs.p[s.bbuf][sb.b_off + (int64_t)(k0 + k) * sb.sbk + (int64_t)cbrel[c] * sb.sbn];
              }
            }
          }
          Bs[k][c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < F_TK; ++k) {
          const double a0 = As[k][ty], a1 = As[k][ty + 16];
          const double b0 = Bs[k][tx], b1 = Bs[k][tx + 16];
          c00 = fma(a0, b0, c00);
          c01 = fma(a0, b1, c01);
          c10 = fma(a1, b0, c10);
          c11 = fma(a1, b1, c11);
        }
        __syncthreads();
      }
    }
    const int r0 = m0 + ty, r1 = m0 + ty + 16, q0 = n0 + tx, q1 = n0 + tx + 16;
    if (r0 < g.M && q0 < g.N) store_c(bufs, cbl, g, r0, q0, n0, cbj, cbrel, c00);
    if (r0 < g.M && q1 < g.N) store_c(bufs, cbl, g, r0, q1, n0, cbj, cbrel, c01);
    if (r1 < g.M && q0 < g.N) store_c(bufs, cbl, g, r1, q0, n0, cbj, cbrel, c10);
    if (r1 < g.M && q1 < g.N) store_c(bufs, cbl, g, r1, q1, n0, cbj, cbrel, c11);
    __syncthreads();  // the column map is rewritten by the next tile
  }
}

int launch_step_fp64(const Step &s, const Bufs &b, void *stream) {
  if (s.nwork_fp64 == 0) return ZMPO_OK;
  k_step_fp64<<<grid_for(s.nwork_fp64, 8), F_NT, 0, (cudaStream_t)stream>>>(
      s.d_work_fp64, s.nwork_fp64, s.d_groups, s.d_segs, s.d_cblocks, s.d_segb, b);
  return launch_error("k_step_fp64");
}

// ------------------------------------------------------- split (tensor core)
// Tiles of TM x TN outputs (TcShape), K packed in chunks of TK slots:
// consecutive segments of the group fill the slots of a chunk (a short block
// product does not waste a whole chunk).  Per chunk: shared power-of-two
// scale per row of A / column of B over the chunk, S exact digit planes in
// shared memory, digit products per level on the BF16 tensor cores (exact in
// FP32: level sums < 2^24), level sums scaled and added to a two-float
// accumulator.  Integer->float conversions stay 32-bit: 64-bit conversions
// issue on the FP64 pipe, which is narrow on GB300.

// biased exponent of a double (0 for zero / denormal)
__device__ __forceinline__ int dexp(double x) {
  return (int)(((unsigned)__double2hiint(x) >> 20) & 0x7ffu);
}

// small non-negative integer (< 2^23) to float without a conversion unit
__device__ __forceinline__ float small_u2f(unsigned d) {
  return __uint_as_float(0x4B000000u | d) - 8388608.0f;
}

// S = 7: S unsigned 8-bit digits of |x| / 2^(E-1022), most significant
// first, the element's sign on each, packed as bf16 (exact: |digit| <= 255).
template <int S>
__device__ __forceinline__ void digits_bf16(double x, int E, __nv_bfloat16 *d, int stride) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7ffu);
  unsigned long long X = 0ull;
  if (e != 0) {
    const unsigned long long mant = ((unsigned long long)((hi & 0xfffffu) | 0x100000u) << 32) | lo;
    const int sh = e - E + 8 * S - 53;
    if (sh >= 0)
      X = mant << sh;
    else if (sh > -64)
      X = mant >> (-sh);
  }
  const unsigned sgn = hi & 0x80000000u;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const unsigned dig = (unsigned)(X >> (8 * (S - 1 - s))) & 0xffu;
    const float f = __uint_as_float(__float_as_uint(small_u2f(dig)) | sgn);
    d[s * stride] = __float2bfloat16_rn(f);
  }
}

// S = 4: the 32 most significant bits of |x|'s significand aligned to the
// chunk exponent E (E >= exponent of x), truncated, using 32-bit integer
// operations only (balanced31 below recodes its top 31 bits into digits).
__device__ __forceinline__ uint32_t aligned32(double x, int E) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7ffu);
  const uint32_t top = e ? ((((hi & 0xfffffu) | 0x100000u) << 11) | (lo >> 21)) : 0u;
  return __funnelshift_rc(top, 0u, (unsigned)(E - e));
}

// byte k of X as the bit pattern of the float 2^23 + byte (PRMT), then the
// exact float value of the byte minus OFF (one FADD)
template <int K, int OFF>
__device__ __forceinline__ float byte_to_float(uint32_t X) {
  return __uint_as_float(__byte_perm(X, 0x4B000000u, 0x7440u | K)) - (8388608.0f + (float)OFF);
}

// S = 4 digits, balanced: the 31 most significant bits X of |x| aligned to
// the chunk exponent E are written X = d0 2^24 + d1 2^16 + d2 2^8 + d3 with
// d1..d3 in [-128, 127] and d0 in [0, 128]: Y = X + 0x808080 has the bytes
// d1+128, d2+128, d3+128 and d0 on top (X < 2^31, so d0 <= 128).  Every
// digit is an integer of magnitude <= 128 (exact in bf16); a digit product
// is at most 2^14 in magnitude, so a level (at most four products per k)
// stays exact in FP32 (< 2^24) for up to 256 slots.  The element's sign
// flips every digit.
__device__ __forceinline__ uint32_t balanced31(double x, int E) { return (aligned32(x, E) >> 1) + 0x808080u; }

// bf16 digit planes of two neighbouring elements (same row, k and k+1) as
// packed pairs: the bf16 of a small integer-valued float is its upper half
__device__ __forceinline__ void digits4_pair(double x0, double x1, int E, uint32_t *d, int stride_u32) {
  const uint32_t Y0 = balanced31(x0, E), Y1 = balanced31(x1, E);
  const uint32_t sg = ((unsigned)__double2hiint(x0) >> 16 & 0x8000u) | ((unsigned)__double2hiint(x1) & 0x80000000u);
  d[0] = __byte_perm(__float_as_uint(byte_to_float<3, 0>(Y0)), __float_as_uint(byte_to_float<3, 0>(Y1)), 0x7632u) ^ sg;
  d[stride_u32] =
      __byte_perm(__float_as_uint(byte_to_float<2, 128>(Y0)), __float_as_uint(byte_to_float<2, 128>(Y1)), 0x7632u) ^ sg;
  d[2 * stride_u32] =
      __byte_perm(__float_as_uint(byte_to_float<1, 128>(Y0)), __float_as_uint(byte_to_float<1, 128>(Y1)), 0x7632u) ^ sg;
  d[3 * stride_u32] =
      __byte_perm(__float_as_uint(byte_to_float<0, 128>(Y0)), __float_as_uint(byte_to_float<0, 128>(Y1)), 0x7632u) ^ sg;
}

// single element variant (one bf16 per plane)
__device__ __forceinline__ void digits4_one(double x, int E, __nv_bfloat16 *d, int stride) {
  const uint32_t Y = balanced31(x, E);
  const unsigned short sg = (unsigned short)((unsigned)__double2hiint(x) >> 16 & 0x8000u);
  unsigned short *u = reinterpret_cast<unsigned short *>(d);
  u[0] = (unsigned short)(__float_as_uint(byte_to_float<3, 0>(Y)) >> 16) ^ sg;
  u[stride] = (unsigned short)(__float_as_uint(byte_to_float<2, 128>(Y)) >> 16) ^ sg;
  u[2 * stride] = (unsigned short)(__float_as_uint(byte_to_float<1, 128>(Y)) >> 16) ^ sg;
  u[3 * stride] = (unsigned short)(__float_as_uint(byte_to_float<0, 128>(Y)) >> 16) ^ sg;
}

// 2^k as a float for k in the float range (subnormal powers of two are exact;
// below 2^-149 the contribution is dropped)
__device__ __forceinline__ float pow2f(int k) {
  if (k > 127) k = 127;
  if (k >= -126) return __int_as_float((k + 127) << 23);
  if (k >= -149) return __int_as_float(1 << (k + 149));
  return 0.f;
}

// hi + lo (two floats) as a double with integer operations only: both become
// signed fixed-point numbers on the larger exponent (29 guard bits), are added
// in 64 bits and the sum is normalised into the double's fields (bits below
// the 53rd are truncated).  The FP64 pipe, narrow on GB300, is not used.
__device__ __forceinline__ double two_float_to_double(float hi, float lo) {
  const uint32_t bh = __float_as_uint(hi), bl = __float_as_uint(lo);
  int eh = (int)((bh >> 23) & 0xffu), el = (int)((bl >> 23) & 0xffu);
  long long mh = (long long)((bh & 0x7fffffu) | (eh ? 0x800000u : 0u));
  long long ml = (long long)((bl & 0x7fffffu) | (el ? 0x800000u : 0u));
  eh = eh ? eh : 1;  // subnormal floats: exponent 1 without the leading bit
  el = el ? el : 1;
  if (bh >> 31) mh = -mh;
  if (bl >> 31) ml = -ml;
  const int E = max(eh, el);
  const int dh = min(E - eh, 63), dl = min(E - el, 63);
  const long long S = ((mh << 29) >> dh) + ((ml << 29) >> dl);  // value S * 2^(E - 150 - 29)
  if (S == 0) return 0.0;
  const unsigned long long sign = S < 0 ? 0x8000000000000000ull : 0ull;
  const unsigned long long A = (unsigned long long)(S < 0 ? -S : S);
  const int n = 63 - __clzll((long long)A);  // position of the leading bit (<= 53)
  const unsigned long long mant = n >= 52 ? (A >> (n - 52)) : (A << (52 - n));
  const long long ebits = (long long)(E - 150 - 29 + n + 1023);  // always a normal double here
  return __longlong_as_double((long long)(sign | ((unsigned long long)ebits << 52) |
                                          (mant & 0xfffffffffffffull)));
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float z = s - a;
  e = (a - (s - z)) + (b - z);
}

// exact power of two 2^k times v (two steps below the normal range)
__device__ __forceinline__ float scale_pow2(float v, int k) {
  if (k >= -126) {
    if (k > 127) k = 127;
    return v * __int_as_float((k + 127) << 23);
  }
  if (k < -250) return 0.f;
  return (v * __int_as_float((k + 100 + 127) << 23)) * __int_as_float((-100 + 127) << 23);
}

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
  const float s = hi + x;
  const float z = s - hi;
  const float e = (hi - (s - z)) + (x - z);
  hi = s;
  lo += e;
}

// ldmatrix: four (two) 8x8 b16 matrices from shared memory in mma fragment
// order; lane l gives the address of row l & 7 of matrix l >> 3 (16-byte
// aligned rows)
__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2(uint32_t addr, uint32_t &r0, uint32_t &r1) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Slot tables of up to NCH chunks in one pass of warp 0 (lane l looks at
// segment cur+l; the inclusive scan places every segment's k range in the
// slot sequence, chunk c holding slots [c*TK, (c+1)*TK)).  A chunk may be
// shorter than TK (end of the 32 segments a pass sees): sums are unchanged.
// nslot[c] = slots of chunk c; *nchunk = chunks filled (0 = done);
// *scaled = some slot of the pass has a weight other than 1.
template <int TK, int NCH>
__device__ __forceinline__ void build_slots_multi(const Group &g, const Seg *__restrict__ segs,
                                                  const Bufs &bufs, Slot *slots, int *cursor,
                                                  int *nslot, int *nchunk, int *scaled, int lane) {
  constexpr int CAP = TK * NCH;
  const int cur = cursor[0], curk = cursor[1];
  if (cur >= g.nseg) {
    if (lane == 0) *nchunk = 0;
    return;
  }
  const int sidx = cur + lane;
  Seg sg;
  int avail = 0;
  if (sidx < g.nseg) {
    sg = segs[g.seg0 + sidx];
    avail = sg.K - (lane == 0 ? curk : 0);
  }
  int incl = avail;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int excl = incl - avail;
  if (avail > 0 && excl < CAP) {
    const double *A = bufs.p[sg.abuf] + sg.a_off;
    const double *B = g.ncb ? bufs.p[sg.bbuf] : bufs.p[sg.bbuf] + sg.b_off;
    const int k0 = lane == 0 ? curk : 0;
    const int jend = min(incl, CAP);
    for (int j = excl; j < jend; ++j) {
      const int kk = k0 + (j - excl);
      Slot &sl = slots[j];
      sl.a = A + (int64_t)kk * sg.sak;
      sl.b = g.ncb ? B : B + (int64_t)kk * sg.sbk;
      sl.sam = sg.sam;
      sl.sbn = sg.sbn;
      sl.alpha = sg.alpha;
      sl.scaled = sg.alpha != 1.0;
      sl.seg = sidx;
      sl.kk = kk;
    }
  }
  const unsigned wscaled = __ballot_sync(0xffffffffu, avail > 0 && excl < CAP && sg.alpha != 1.0);
  const unsigned reach = __ballot_sync(0xffffffffu, incl >= CAP && avail > 0);
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int lstop = reach ? (__ffs(reach) - 1) : -1;
  const int stop_incl = __shfl_sync(0xffffffffu, incl, lstop < 0 ? 31 : lstop);
  const int stop_excl = __shfl_sync(0xffffffffu, excl, lstop < 0 ? 31 : lstop);
  if (lane == 0) {
    int filled;
    if (lstop < 0) {  // every segment the lanes saw fits
      filled = min(total, CAP);
      cursor[0] = cur + min(32, g.nseg - cur);
      cursor[1] = 0;
    } else {
      filled = CAP;
      const int used = CAP - stop_excl;  // slots taken from segment cur+lstop
      const int base = lstop == 0 ? curk : 0;
      if (stop_incl == CAP) {
        cursor[0] = cur + lstop + 1;
        cursor[1] = 0;
      } else {
        cursor[0] = cur + lstop;
        cursor[1] = base + used;
      }
    }
    const int nch = (filled + TK - 1) / TK;
    for (int c = 0; c < nch; ++c) nslot[c] = min(TK, filled - c * TK);
    *nchunk = nch;
    *scaled = wscaled != 0u;
  }
}

// One CTA per output tile of TM rows x TN columns; warps tile it in m16 x n8
// pieces (TM/16 x TN/8 warps), so each thread holds one m16n8 accumulator
// per digit level.  A chunk of 32 k slots is cut by TPR threads per row of A
// and TPC threads per column of B.  Per chunk: slot table (warp 0), operands
// to digit planes, digit products, scaled sums; three barriers.
template <int S, int TM, int TN>
struct TcShape {
  // k slots per chunk.  S = 4 (balanced digits, |digit| <= 128, at most 4
  // products per level and k) stays exact in FP32 (< 2^24) up to 256 slots;
  // S = 7 (digits 0..255, at most 7 products) up to 32.  The 64-column tiles
  // take 64-slot chunks with S = 4 (half the barriers and level folds per
  // k); the narrower tiles keep 32 (64 slots there mean more registers per
  // thread, measured slower).  128-slot chunks in 64 x 64 tiles measured
  // slower too (more registers; the last chunk of a group wastes more).
  static constexpr int TK = (S == 4 && TN == 64) ? 64 : 32;
  static constexpr int PAD = TK + 8;          // bf16 per plane row in shared memory
  static constexpr int NCH = 8;               // chunks per slot-table pass (4, 8, 16 measured: 8 best)
  static constexpr int WM = TM / 16, WN = TN / 8;
  static constexpr int NT = 32 * WM * WN;     // threads per CTA
  static constexpr int TPR = NT / TM;         // threads per row of A
  static constexpr int KPA = TK / TPR;        // A slots per thread
  static constexpr int TPC = NT / TN;         // threads per column of B
  static constexpr int KPB = TK / TPC;        // B slots per thread
  // resident threads per SM the register budget is sized for (16 A slots
  // per thread need more registers than 8)
  static constexpr int THREADS_SM = (KPA > 8 && NT < 512) ? 768 : 1024;
  static_assert(TPR >= 1 && KPA >= 1 && TPC >= 1 && KPB >= 1, "tile shape");
};

// Cut of one chunk of A: TPR threads per row, KPA slots each; the row's
// chunk exponent (max over its TPR threads) and its S digit planes.  Slot
// weights other than 1 are applied only in passes that have one (scaled is
// the same for the whole CTA: the other passes issue no FP64 multiply -- the
// FP64 pipe is narrow on GB300).
template <int S, int TM, int TPR, int KPA, int T_PAD>
__device__ __forceinline__ void cut_a(const Slot *slt, int ns, int rowa, int M, __nv_bfloat16 *Ap, int *Ea,
                                      int ra, int parta, bool scaled) {
  double v[KPA];
  int emax = 0;
#pragma unroll
  for (int t = 0; t < KPA; ++t) {
    const int j = parta * KPA + t;
    double x = 0.0;
    if (j < ns && rowa < M) {
      const Slot &sl = slt[j];
      x = __ldg(sl.a + (int64_t)rowa * sl.sam);
    }
    v[t] = x;
  }
  if (scaled) {
#pragma unroll
    for (int t = 0; t < KPA; ++t) {
      const int j = parta * KPA + t;
      if (j < ns && slt[j].scaled) v[t] *= slt[j].alpha;
    }
  }
#pragma unroll
  for (int t = 0; t < KPA; ++t) emax = max(emax, dexp(v[t]));
#pragma unroll
  for (int o = 1; o < TPR; o <<= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  if (parta == 0) Ea[ra] = emax;
  if constexpr (S == 4 && KPA % 2 == 0) {
    uint32_t *ap = reinterpret_cast<uint32_t *>(Ap + ra * T_PAD + parta * KPA);
#pragma unroll
    for (int t = 0; t < KPA; t += 2) digits4_pair(v[t], v[t + 1], emax, ap + t / 2, TM * T_PAD / 2);
  } else if constexpr (S == 4) {
#pragma unroll
    for (int t = 0; t < KPA; ++t) digits4_one(v[t], emax, Ap + ra * T_PAD + parta * KPA + t, TM * T_PAD);
  } else {
#pragma unroll
    for (int t = 0; t < KPA; ++t) digits_bf16<S>(v[t], emax, Ap + ra * T_PAD + parta * KPA + t, TM * T_PAD);
  }
}

// Cut of one chunk of B: TPC threads per column, KPB slots each.
template <int S, int TN, int TPC, int KPB, int T_PAD>
__device__ __forceinline__ void cut_b(const Slot *slt, int ns, int colb, const Group &g,
                                      const SegB *__restrict__ segb, int jb, int colrel, __nv_bfloat16 *Bp,
                                      int *Eb, int cb, int partb) {
  double v[KPB];
  int emax = 0;
#pragma unroll
  for (int t = 0; t < KPB; ++t) {
    const int j = partb * KPB + t;
    double x = 0.0;
    if (j < ns && colb < g.N)
      x = g.ncb ? load_b_cb(slt[j], segb, g, jb, colrel) : __ldg(slt[j].b + (int64_t)colb * slt[j].sbn);
    v[t] = x;
    emax = max(emax, dexp(x));
  }
#pragma unroll
  for (int o = 1; o < TPC; o <<= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  if (partb == 0) Eb[cb] = emax;
  if constexpr (S == 4 && KPB % 2 == 0) {
    uint32_t *bp = reinterpret_cast<uint32_t *>(Bp + cb * T_PAD + partb * KPB);
#pragma unroll
    for (int t = 0; t < KPB; t += 2) digits4_pair(v[t], v[t + 1], emax, bp + t / 2, TN * T_PAD / 2);
  } else if constexpr (S == 4) {
#pragma unroll
    for (int t = 0; t < KPB; ++t) digits4_one(v[t], emax, Bp + cb * T_PAD + partb * KPB + t, TN * T_PAD);
  } else {
#pragma unroll
    for (int t = 0; t < KPB; ++t) digits_bf16<S>(v[t], emax, Bp + cb * T_PAD + partb * KPB + t, TN * T_PAD);
  }
}

// Digit products of one chunk of ns slots for this warp's m16 x n8 piece
// (exact in FP32 per level; k steps past the chunk's slots are skipped), then
// the levels scaled by 2^(Ea + Eb - 2044 - 8(l+2)) (S = 7) or
// 2^(Ea + Eb - 2058 - 8l) (S = 4, 31-bit balanced digits) into the two-float
// sums.
template <int S, int TM, int TN, int TK, int T_PAD>
__device__ __forceinline__ void mma_fold(const __nv_bfloat16 *Ap, const __nv_bfloat16 *Bp, const int *Ea,
                                         const int *Eb, int ns, int wm, int wn, int gq, int tq, float *hi,
                                         float *lo) {
  float acc[S][4];
#pragma unroll
  for (int l = 0; l < S; ++l)
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[l][i] = 0.f;
  // ldmatrix row addresses of this lane: lane l points at row l & 7 of 8x8
  // matrix l >> 3.  A (x4): matrices (rows 0-7 | 8-15) x (k 0-7 | 8-15) in
  // fragment order; B (x4 over two levels): (level sb | sb+1) x (k 0-7 | 8-15).
  const int lane = gq * 4 + tq;
  const uint32_t a_base = (uint32_t)__cvta_generic_to_shared(
      Ap + (wm + (lane & 7) + ((lane >> 3) & 1) * 8) * T_PAD + (lane >> 4) * 8);
  const uint32_t b_base = (uint32_t)__cvta_generic_to_shared(
      Bp + ((lane >> 4) * TN + wn + (lane & 7)) * T_PAD + ((lane >> 3) & 1) * 8);
  constexpr uint32_t A_LEVEL = TM * T_PAD * 2, B_LEVEL = TN * T_PAD * 2;  // bytes per plane
#pragma unroll
  for (int kk = 0; kk < TK; kk += 16) {
    if (kk >= ns) break;  // the same for the whole CTA
    uint32_t bf[S][2];
#pragma unroll
    for (int sb = 0; sb + 1 < S; sb += 2)
      ldsm_x4(b_base + sb * B_LEVEL + kk * 2, bf[sb][0], bf[sb][1], bf[sb + 1][0], bf[sb + 1][1]);
    if constexpr (S % 2 == 1) ldsm_x2(b_base + (S - 1) * B_LEVEL + kk * 2, bf[S - 1][0], bf[S - 1][1]);
#pragma unroll
    for (int sa = 0; sa < S; ++sa) {
      uint32_t af[4];
      ldsm_x4(a_base + sa * A_LEVEL + kk * 2, af[0], af[1], af[2], af[3]);
#pragma unroll
      for (int sb = 0; sb + sa < S; ++sb) mma_bf16(acc[sa + sb], af, bf[sb]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = wm + gq + (i >> 1) * 8;
    const int c = wn + 2 * tq + (i & 1);
    const int ea = Ea[r], eb = Eb[c];
    if (ea == 0 || eb == 0) continue;
    const int base = ea + eb - 2044;
    if constexpr (S == 4) {
      // levels are exact integers below 2^24: level 0 + level 1 / 2^8 as an
      // exact pair, levels 2 and 3 into its low part, one scale
      float h, e;
      two_sum(acc[0][i], acc[1][i] * 0x1p-8f, h, e);
      e = fmaf(acc[2][i], 0x1p-16f, e);
      e = fmaf(acc[3][i], 0x1p-24f, e);
      const float sc = pow2f(base - 14);  // 31-bit X: one more power of two than 32
      float s2, e2;
      two_sum(hi[i], h * sc, s2, e2);
      hi[i] = s2;
      lo[i] += e2 + e * sc;
    } else {
#pragma unroll
      for (int l = 0; l < S; ++l) two_sum_acc(hi[i], lo[i], scale_pow2(acc[l][i], base - 8 * (l + 2)));
    }
  }
}

template <int S, int TM, int TN>
__global__ void __launch_bounds__(TcShape<S, TM, TN>::NT, TcShape<S, TM, TN>::THREADS_SM / TcShape<S, TM, TN>::NT)
k_step_tc(const Work *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
          const Seg *__restrict__ segs, const ColBlock *__restrict__ cbl, const SegB *__restrict__ segb,
          Bufs bufs) {
  using Sh = TcShape<S, TM, TN>;
  constexpr int TPR = Sh::TPR, KPA = Sh::KPA, TPC = Sh::TPC, KPB = Sh::KPB;
  constexpr int TK = Sh::TK, T_PAD = Sh::PAD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *Ap = reinterpret_cast<__nv_bfloat16 *>(smem_raw);  // [S][TM][PAD]
  __nv_bfloat16 *Bp = Ap + S * TM * T_PAD;                          // [S][TN][PAD]
  int *Ea = reinterpret_cast<int *>(Bp + S * TN * T_PAD);           // [TM]
  int *Eb = Ea + TM;                                                // [TN]
  Slot *slots = reinterpret_cast<Slot *>(Eb + (TN < 16 ? 16 : TN));  // [NCH][TK] (Eb holds TN ints)
  int *ctl = reinterpret_cast<int *>(slots + Sh::NCH * TK);  // cursor[2], nchunk, nslot[NCH], scaled

  __shared__ int cbj[TN], cbrel[TN];  // column-block map of the tile
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp % Sh::WM) * 16, wn = (warp / Sh::WM) * 8;  // this warp's m16n8 piece
  const int gq = lane >> 2, tq = lane & 3;
  const int ra = tid / TPR, parta = tid % TPR;  // A: row, part of the chunk
  const int cb = tid / TPC, partb = tid % TPC;  // B: column, part of the chunk

  for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
    const Work wk = work[w];
    const Group g = groups[wk.group];
    const int m0 = wk.mt, n0 = wk.nt;
    const int rowa = m0 + ra, colb = n0 + cb;
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    if (tid == 0) {
      ctl[0] = 0;
      ctl[1] = 0;
    }
    if (g.ncb) tile_cblocks(cbl, g, n0, TN, cbj, cbrel);
    __syncthreads();
    const int jb = g.ncb ? cbj[cb] : -1, colrel = g.ncb ? cbrel[cb] : 0;
    while (true) {
      if (warp == 0)
        build_slots_multi<TK, Sh::NCH>(g, segs, bufs, slots, ctl, ctl + 3, ctl + 2, ctl + 3 + Sh::NCH, lane);
      __syncthreads();
      const int nch = ctl[2];
      if (nch == 0) break;
      const bool scaled = ctl[3 + Sh::NCH] != 0;
      for (int ch = 0; ch < nch; ++ch) {
        const int ns = ctl[3 + ch];
        const Slot *slt = slots + ch * TK;
        cut_a<S, TM, TPR, KPA, T_PAD>(slt, ns, rowa, g.M, Ap, Ea, ra, parta, scaled);
        cut_b<S, TN, TPC, KPB, T_PAD>(slt, ns, colb, g, segb, jb, colrel, Bp, Eb, cb, partb);
        __syncthreads();
        mma_fold<S, TM, TN, TK, T_PAD>(Ap, Bp, Ea, Eb, ns, wm, wn, gq, tq, hi, lo);
        __syncthreads();
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = m0 + wm + gq + (i >> 1) * 8;
      const int c = n0 + wn + 2 * tq + (i & 1);
      if (r < g.M && c < g.N) store_c(bufs, cbl, g, r, c, n0, cbj, cbrel, two_float_to_double(hi[i], lo[i]));
    }
    __syncthreads();  // the column map is rewritten by the next tile
  }
}

// B-resident variant for groups whose whole K fits in CHB chunks of one
// slot-table pass (at most 32 segments): a work item is one column tile and
// a run of up to MB row tiles (Work::pad of them).  The column tile's B is cut
// into digit planes once, for every chunk, and stays in shared memory while
// the row tiles stream through: B is cut once per run instead of once per row
// tile.
template <int TM, int TN>
struct TcbShape {
  using Sh = TcShape<4, TM, TN>;
  static constexpr int CHB = 256 / Sh::TK;      // K up to 256
  static constexpr int EBN = TN < 16 ? 16 : TN;
  static constexpr size_t smem() {
    return (size_t)4 * TM * Sh::PAD * 2 + (size_t)CHB * 4 * TN * Sh::PAD * 2 + (size_t)TM * 4 +
           (size_t)CHB * EBN * 4 + (size_t)CHB * Sh::TK * sizeof(Slot) + (4 + CHB) * 4 + 16;
  }
};

// Barrier of the NTH threads of one part of the CTA (ids 1 .. NPART; id 0 is
// __syncthreads): all parts run the same number of row-tile chunks, so every
// part barrier is reached by all of its threads.
__device__ __forceinline__ void bar_part(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}

// The CTA's NPART parts (256 threads each) take TM/NPART rows of each row
// tile against the same resident B planes, each with its own A planes and
// its own barrier: the parts drift apart, so one part's digit products
// overlap another part's loads and cuts (the phases of a single 1024-thread
// loop are otherwise in lockstep).  2 parts: -3 % sigma time, 4: -7 %.
constexpr int NPART = 4;

template <int TM, int TN>
__global__ void __launch_bounds__(TcShape<4, TM, TN>::NT, TcShape<4, TM, TN>::THREADS_SM / TcShape<4, TM, TN>::NT)
k_step_tcb(const Work *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
           const Seg *__restrict__ segs, const ColBlock *__restrict__ cbl, const SegB *__restrict__ segb,
           Bufs bufs) {
  constexpr int S = 4;
  using Sh = TcShape<S, TM, TN>;
  using Bh = TcbShape<TM, TN>;
  constexpr int TPC = Sh::TPC, KPB = Sh::KPB;
  constexpr int TK = Sh::TK, T_PAD = Sh::PAD, CHB = Bh::CHB, EBN = Bh::EBN;
  constexpr int BPL = S * TN * T_PAD;  // bf16 per chunk of B planes
  // one of NPART parts: TMH rows, NTH threads, warps WMH x WN of m16 x n8 pieces
  constexpr int TMH = TM / NPART, NTH = Sh::NT / NPART, WMH = TMH / 16;
  constexpr int TPRH = NTH / TMH, KPAH = TK / TPRH;
  static_assert(WMH * Sh::WN * 32 == NTH && TPRH * KPAH == TK && TPRH <= 32, "part shape");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *Ap = reinterpret_cast<__nv_bfloat16 *>(smem_raw);  // [NPART][S][TMH][PAD]
  __nv_bfloat16 *Bp = Ap + S * TM * T_PAD;                          // [CHB][S][TN][PAD]
  int *Ea = reinterpret_cast<int *>(Bp + CHB * BPL);                // [NPART][TMH]
  int *Eb = Ea + TM;                                                // [CHB][EBN]
  Slot *slots = reinterpret_cast<Slot *>(Eb + CHB * EBN);          // [CHB][TK]
  int *ctl = reinterpret_cast<int *>(slots + CHB * TK);             // cursor[2], nchunk, nslot[CHB], scaled

  __shared__ int cbj[TN], cbrel[TN];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int part = tid / NTH, tidh = tid % NTH, warph = tidh >> 5;
  const int wm = (warph % WMH) * 16, wn = (warph / WMH) * 8;
  const int gq = lane >> 2, tq = lane & 3;
  const int ra = tidh / TPRH, parta = tidh % TPRH;
  const int cb = tid / TPC, partb = tid % TPC;
  __nv_bfloat16 *Aph = Ap + part * S * TMH * T_PAD;
  int *Eah = Ea + part * TMH;

  for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
    const Work wk = work[w];
    const Group g = groups[wk.group];
    const int n0 = wk.nt, colb = n0 + cb;
    if (tid == 0) {
      ctl[0] = 0;
      ctl[1] = 0;
    }
    if (g.ncb) tile_cblocks(cbl, g, n0, TN, cbj, cbrel);
    __syncthreads();
    const int jb = g.ncb ? cbj[cb] : -1, colrel = g.ncb ? cbrel[cb] : 0;
    if (warp == 0) build_slots_multi<TK, CHB>(g, segs, bufs, slots, ctl, ctl + 3, ctl + 2, ctl + 3 + CHB, lane);
    __syncthreads();
    const int nch = ctl[2];  // the planner routes only groups that one pass covers
    const bool scaled = ctl[3 + CHB] != 0;
    for (int ch = 0; ch < nch; ++ch)
      cut_b<S, TN, TPC, KPB, T_PAD>(slots + ch * TK, ctl[3 + ch], colb, g, segb, jb, colrel, Bp + ch * BPL,
                                    Eb + ch * EBN, cb, partb);
    __syncthreads();  // B planes of every chunk ready for all parts
    for (int mi = 0; mi < wk.pad; ++mi) {
      const int m0 = wk.mt + mi * TM + part * TMH, rowa = m0 + ra;
      float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
      for (int ch = 0; ch < nch; ++ch) {
        cut_a<S, TMH, TPRH, KPAH, T_PAD>(slots + ch * TK, ctl[3 + ch], rowa, g.M, Aph, Eah, ra, parta, scaled);
        bar_part(1 + part, NTH);
        mma_fold<S, TMH, TN, TK, T_PAD>(Aph, Bp + ch * BPL, Eah, Eb + ch * EBN, ctl[3 + ch], wm, wn, gq, tq,
                                        hi, lo);
        bar_part(1 + part, NTH);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = m0 + wm + gq + (i >> 1) * 8;
        const int c = n0 + wn + 2 * tq + (i & 1);
        if (r < g.M && c < g.N) store_c(bufs, cbl, g, r, c, n0, cbj, cbrel, two_float_to_double(hi[i], lo[i]));
      }
    }
    __syncthreads();  // slot tables, B planes and the column map are rewritten by the next item
  }
}

template <int TM, int TN>
static int launch_tcb_t(const Work *work, int64_t nwork, const Step &s, const Bufs &b, void *stream) {
  if (nwork == 0) return ZMPO_OK;
  const size_t smem = TcbShape<TM, TN>::smem();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_step_tcb<TM, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  constexpr int NT = TcShape<4, TM, TN>::NT;
  k_step_tcb<TM, TN><<<grid_for(nwork, TcShape<4, TM, TN>::THREADS_SM / NT), NT, smem, (cudaStream_t)stream>>>(
      work, nwork, s.d_groups, s.d_segs, s.d_cblocks, s.d_segb, b);
  return launch_error("k_step_tcb");
}

template <int S, int TM, int TN>
static int launch_tc_t(const Work *work, int64_t nwork, const Step &s, const Bufs &b, void *stream) {
  if (nwork == 0) return ZMPO_OK;
  using Sh = TcShape<S, TM, TN>;
  const size_t smem = (size_t)S * (TM + TN) * Sh::PAD * sizeof(__nv_bfloat16) +
                      (size_t)(TM + (TN < 16 ? 16 : TN)) * sizeof(int) + Sh::NCH * Sh::TK * sizeof(Slot) +
                      (4 + Sh::NCH) * sizeof(int) + 16;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_step_tc<S, TM, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  constexpr int NT = TcShape<S, TM, TN>::NT;
  k_step_tc<S, TM, TN><<<grid_for(nwork, TcShape<S, TM, TN>::THREADS_SM / NT), NT, smem, (cudaStream_t)stream>>>(
      work, nwork, s.d_groups, s.d_segs, s.d_cblocks, s.d_segb, b);
  return launch_error("k_step_tc");
}

template <int S>
static int launch_split_all(const Step &s, const Bufs &b, void *stream, bool cut_kept) {
  int rc;
  // S = 4: the groups routed to the B-resident kernel are not in the S = 4
  // lists; S = 7 (no B-resident variant) uses the lists of every group
  Work *const(*wl)[4] = S == 4 ? s.d_work_tc4 : s.d_work_tc;
  const int64_t(*nw)[4] = S == 4 ? s.nwork_tc4 : s.nwork_tc;
  if (S == 4) {
    if ((rc = launch_step_umma(s, b, step_planes(s, b), cut_kept, stream))) return rc;
    if ((rc = launch_tcb_t<64, 64>(s.d_work_tcb[0], s.nwork_tcb[0], s, b, stream))) return rc;
    if ((rc = launch_tcb_t<128, 32>(s.d_work_tcb[1], s.nwork_tcb[1], s, b, stream))) return rc;
  }
  if ((rc = launch_tc_t<S, 128, 8>(wl[2][0], nw[2][0], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 128, 16>(wl[2][1], nw[2][1], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 64, 8>(wl[1][0], nw[1][0], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 64, 16>(wl[1][1], nw[1][1], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 32, 8>(wl[0][0], nw[0][0], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 32, 16>(wl[0][1], nw[0][1], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 128, 32>(wl[2][2], nw[2][2], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 64, 32>(wl[1][2], nw[1][2], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 32, 32>(wl[0][2], nw[0][2], s, b, stream))) return rc;
  if ((rc = launch_tc_t<S, 64, 64>(wl[1][3], nw[1][3], s, b, stream))) return rc;
  return launch_tc_t<S, 32, 64>(wl[0][3], nw[0][3], s, b, stream);
}

int launch_step_split(const Step &s, const Bufs &b, int nslices, void *stream, bool cut_kept) {
  if (nslices == 4) return launch_split_all<4>(s, b, stream, cut_kept);
  if (nslices == 7) return launch_split_all<7>(s, b, stream, true);
  return record_arg_error("unsupported slice count");
}

// ------------------------------------------------------------- split-K sum
__global__ void __launch_bounds__(256)
k_reduce(const Reduction *__restrict__ reds, int nred, int64_t total, Bufs bufs) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nred - 1;
    while (lo < hi) {  // last reduction with elem0 <= i
      const int mid = (lo + hi + 1) >> 1;
      if (reds[mid].elem0 <= i) lo = mid; else hi = mid - 1;
    }
    const Reduction r = reds[lo];
    const int64_t e = i - r.elem0;
    const int m = (int)(e / r.N), n = (int)(e % r.N);
    const double *P = bufs.p[kPartialBuf] + r.part_off + e;
    const int64_t stride = (int64_t)r.M * r.N;
    double acc = 0.0;
    for (int t = 0; t < r.nparts; ++t) acc += P[t * stride];
    bufs.p[r.cbuf][r.c_off + (int64_t)m * r.scm + (int64_t)n * r.scn] = acc;
  }
}

int launch_reduce(const Step &s, const Bufs &b, void *stream) {
  if (s.red_elems == 0) return ZMPO_OK;
  Bufs bb = b;
  bb.p[kPartialBuf] = s.d_part;
  const int64_t blocks = (s.red_elems + 255) / 256;
  k_reduce<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, (cudaStream_t)stream>>>(
      s.d_reds, (int)s.reds.size(), s.red_elems, bb);
  return launch_error("k_reduce");
}

// ----------------------------------------------------------------- HDiag
constexpr int D_NT = 256, D_EPT = 8;  // up to D_NT * D_EPT elements per pass

__global__ void __launch_bounds__(D_NT)
k_hdiag(const DiagBlock *__restrict__ blocks, int64_t nblocks, const DiagTerm *__restrict__ terms,
        Bufs bufs, double *__restrict__ out, int max_ac, int max_ar) {
  extern __shared__ double sm[];
  double *V = sm;            // [da][dc]
  double *Y = sm + max_ac;   // [da][dr]
  const double *Lb = bufs.p[0], *Rb = bufs.p[1], *Wb = bufs.p[2];
  for (int64_t bi = blockIdx.x; bi < nblocks; bi += gridDim.x) {
    const DiagBlock db = blocks[bi];
    const int nel = db.dl * db.dr;
    for (int p0 = 0; p0 < nel; p0 += D_NT * D_EPT) {
      double acc[D_EPT];
#pragma unroll
      for (int j = 0; j < D_EPT; ++j) acc[j] = 0.0;
      for (int ti = 0; ti < db.nt; ++ti) {
        const DiagTerm t = terms[db.t0 + ti];
        __syncthreads();
        for (int e = threadIdx.x; e < t.da * t.dc; e += D_NT) {
          const int a = e / t.dc, c = e % t.dc;
          double v;
          if (t.ncsite == 2) {
            v = 0.0;
            for (int b = 0; b < t.db; ++b)
              v += Wb[t.wi_off + a * t.wi_sa + b * t.wi_sb] * Wb[t.wj_off + b * t.wj_sb + c * t.wj_sc];
          } else {
            v = Wb[t.wi_off + a * t.wi_sa + c * t.wi_sb];
          }
          V[e] = v;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < t.da * db.dr; e += D_NT) {
          const int a = e / db.dr, r = e % db.dr;
          double y = 0.0;
          for (int c = 0; c < t.dc; ++c) y += V[a * t.dc + c] * Rb[t.r_off + c * t.r_sc + r * t.r_sr];
          Y[e] = y;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < D_EPT; ++j) {
          const int e = p0 + j * D_NT + threadIdx.x;
          if (e < nel) {
            const int l = e / db.dr, r = e % db.dr;
            double s = 0.0;
            for (int a = 0; a < t.da; ++a) s += Lb[t.l_off + a * t.l_sa + l * t.l_sl] * Y[a * db.dr + r];
            acc[j] += t.alpha * s;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < D_EPT; ++j) {
        const int e = p0 + j * D_NT + threadIdx.x;
        if (e < nel) out[db.out_off + e] = acc[j];
      }
    }
  }
}

int launch_hdiag(const DiagBlock *blocks, int64_t nblocks, const DiagTerm *terms, const Bufs &b,
                 double *out, int max_ac, int max_ar, void *stream) {
  if (nblocks == 0) return ZMPO_OK;
  const size_t smem = (size_t)(max_ac + max_ar) * sizeof(double);
  if (smem > 200 * 1024) return record_arg_error("hdiag: MPO sector too large for shared memory");
  cudaFuncSetAttribute(k_hdiag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_hdiag<<<grid_for(nblocks, 4), D_NT, smem, (cudaStream_t)stream>>>(blocks, nblocks, terms, b, out,
                                                                       max_ac, max_ar);
  return launch_error("k_hdiag");
}

}  // namespace zmpo

// =================================================== allocation-free variant
// zmpo_contract_exec_noalloc: the split-K partial sums of a contraction live in
// this fixed device array instead of memory the plan allocates, for callers
// that must not allocate device memory at the time of the call (see the
// declaration in include/zmpo_gb300.h).  Every device that loads the library
// holds the array until the process exits.
namespace zmpo {
int contract_step_for(zmpo_engine *e, int plan_id, int precision, Step **out);
}

constexpr int64_t kNoAllocScratchElems = int64_t(1) << 20;  // 8 MiB of float64
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchElems];
constexpr int kNoAllocMaxDevices = 64;
static double *g_noalloc_ptr[kNoAllocMaxDevices];  // device address of the array, per device

// split-K sum that reads the partials from the scratch pointer it is given
static int launch_reduce_given_scratch(const zmpo::Step &s, const zmpo::Bufs &b, void *stream) {
  if (s.red_elems == 0) return ZMPO_OK;
  const int64_t blocks = (s.red_elems + 255) / 256;
  zmpo::k_reduce<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, (cudaStream_t)stream>>>(
      s.d_reds, (int)s.reds.size(), s.red_elems, b);
  return zmpo::launch_error("k_reduce (static scratch)");
}

extern "C" int zmpo_contract_exec_noalloc(zmpo_engine *e, int plan_id, const double *d_a,
                                          const double *d_b, double *d_out, int precision,
                                          void *stream) {
  zmpo::Step *st = nullptr;
  int rc = zmpo::contract_step_for(e, plan_id, precision, &st);
  if (rc) return rc;
  if (precision == ZMPO_PREC_SPLIT && st->plane_bytes > 0 && st->plane_ws_off < 0 && !st->d_planes_own)
    return zmpo::record_arg_error(
        "contract_exec_noalloc: run the plan once with the split precision through zmpo_contract_exec "
        "during set-up (that call makes the plan's digit-plane buffer)");
  if (st->part_elems > kNoAllocScratchElems)
    return zmpo::record_size_error(
        "contract_exec_noalloc: the plan needs more split-K scratch than the fixed 8 MiB "
        "(1048576 float64) array holds; use zmpo_contract_exec");
  int dev = -1;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return zmpo::record_cuda_error("contract_exec_noalloc: cudaGetDevice", (int)ce);
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return zmpo::record_size_error("contract_exec_noalloc: device ordinal beyond 63");
  if (g_noalloc_ptr[dev] == nullptr) {
    // one-time set-up on this device (the device is current): the array's
    // name is a host-side stand-in, the kernels need its device address
    void *p = nullptr;
    ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (ce != cudaSuccess)
      return zmpo::record_cuda_error("contract_exec_noalloc: cudaGetSymbolAddress", (int)ce);
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  zmpo::Bufs b{};
  b.p[0] = const_cast<double *>(d_a);
  b.p[1] = const_cast<double *>(d_b);
  b.p[4] = d_out;
  b.p[zmpo::kPartialBuf] = g_noalloc_ptr[dev];
  if (precision == ZMPO_PREC_FP64)
    rc = zmpo::launch_step_fp64(*st, b, stream);
  else if (precision == ZMPO_PREC_SPLIT)
    rc = zmpo::launch_step_split(*st, b, 4, stream);
  else if (precision == ZMPO_PREC_EMU64)
    rc = zmpo::launch_step_split(*st, b, 7, stream);
  else
    return zmpo::record_arg_error("contract_exec_noalloc: unknown precision");
  if (rc) return rc;
  return launch_reduce_given_scratch(*st, b, stream);
}
