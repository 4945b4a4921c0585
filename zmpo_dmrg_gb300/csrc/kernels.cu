// Device kernels of the GB300 DMRG engine.
//
// A "step" is one grouped launch over many block products (see engine.h):
// every output sub-matrix (group) is owned by one CTA tile, which loops over
// the group's segments (strided GEMMs) and writes the result once.  Two
// arithmetic paths share the task lists:
//
//   k_step_fp64   FP64 FMA on the CUDA cores (reference arithmetic).
//   k_step_split  FP64 operands cut into S exact 8-bit digit planes per
//                 K-chunk (a shared power-of-two scale per row of A and per
//                 column of B, Ozaki-style), digit products on the BF16
//                 tensor cores (mma.sync m16n8k16, FP32 accumulate, exact:
//                 every per-level sum stays below 2^24), per-chunk results
//                 scaled by powers of two and summed in a two-float (hi+lo)
//                 accumulator on the FP32 pipes; FP64 only for the final
//                 store.  S = 4 keeps pairs s+t <= 5 (10 products, ~2^-32
//                 relative to the row/column maximum); S = 7 keeps 28
//                 products (~2^-56).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zmpo_gb300.h"
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

// ------------------------------------------------------------------ FP64
constexpr int F_TM = 32, F_TN = 32, F_TK = 16, F_NT = 256;

__global__ void __launch_bounds__(F_NT)
k_step_fp64(const Work *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
            const Seg *__restrict__ segs, Bufs bufs) {
  __shared__ double As[F_TK][F_TM + 1];
  __shared__ double Bs[F_TK][F_TN + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
    const Work wk = work[w];
    const Group g = groups[wk.group];
    const int m0 = wk.mt * F_TM, n0 = wk.nt * F_TN;
    double c00 = 0.0, c01 = 0.0, c10 = 0.0, c11 = 0.0;
    for (int si = 0; si < g.nseg; ++si) {
      const Seg s = segs[g.seg0 + si];
      const double *A = bufs.p[s.abuf] + s.a_off;
      const double *B = bufs.p[s.bbuf] + s.b_off;
      const bool a_kfast = s.sak == 1, b_nfast = s.sbn == 1;
      for (int k0 = 0; k0 < s.K; k0 += F_TK) {
        for (int e = tid; e < F_TM * F_TK; e += F_NT) {
          int r, k;
          if (a_kfast) { r = e / F_TK; k = e % F_TK; } else { r = e % F_TM; k = e / F_TM; }
          double v = 0.0;
          if (m0 + r < g.M && k0 + k < s.K) v = s.alpha * A[(int64_t)(m0 + r) * s.sam + (int64_t)(k0 + k) * s.sak];
          As[k][r] = v;
        }
        for (int e = tid; e < F_TK * F_TN; e += F_NT) {
          int k, c;
          if (b_nfast) { k = e / F_TN; c = e % F_TN; } else { c = e / F_TK; k = e % F_TK; }
          double v = 0.0;
          if (n0 + c < g.N && k0 + k < s.K) v = B[(int64_t)(k0 + k) * s.sbk + (int64_t)(n0 + c) * s.sbn];
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
    double *C = bufs.p[g.cbuf] + g.c_off;
    const int r0 = m0 + ty, r1 = m0 + ty + 16, q0 = n0 + tx, q1 = n0 + tx + 16;
    if (r0 < g.M && q0 < g.N) C[(int64_t)r0 * g.scm + (int64_t)q0 * g.scn] = c00;
    if (r0 < g.M && q1 < g.N) C[(int64_t)r0 * g.scm + (int64_t)q1 * g.scn] = c01;
    if (r1 < g.M && q0 < g.N) C[(int64_t)r1 * g.scm + (int64_t)q0 * g.scn] = c10;
    if (r1 < g.M && q1 < g.N) C[(int64_t)r1 * g.scm + (int64_t)q1 * g.scn] = c11;
  }
}

int launch_step_fp64(const Step &s, const Bufs &b, void *stream) {
  if (s.nwork_fp64 == 0) return ZMPO_OK;
  k_step_fp64<<<grid_for(s.nwork_fp64, 8), F_NT, 0, (cudaStream_t)stream>>>(
      s.d_work_fp64, s.nwork_fp64, s.d_groups, s.d_segs, b);
  return launch_error("k_step_fp64");
}

// ------------------------------------------------------- split (tensor core)
constexpr int S_TM = 32, S_TN = 32, S_TK = 32, S_NT = 128;
constexpr int S_PAD = 40;  // bf16 row stride of a digit plane (bank-conflict free)

// biased exponent of a double (0 for zero / denormal)
__device__ __forceinline__ int dexp(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}

// 8-bit digits of |x| * 2^(8S - (E - 1022)) where E >= biased exponent of x;
// returns the signed digits (most significant first) as floats.
template <int S>
__device__ __forceinline__ void digits(double x, int E, float *d) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  const float sg = (bits >> 63) ? -1.f : 1.f;
  unsigned long long X = 0ull;
  if (e != 0) {
    const unsigned long long mant = (bits & 0xfffffffffffffull) | (1ull << 52);
    const int sh = e - E + 8 * S - 53;  // X = mant * 2^sh, X < 2^(8S)
    if (sh >= 0)
      X = mant << sh;
    else if (sh > -64)
      X = mant >> (-sh);
  }
#pragma unroll
  for (int s = 0; s < S; ++s) d[s] = sg * (float)((X >> (8 * (S - 1 - s))) & 0xffull);
}

// exact power of two 2^k as a float scale applied in two steps
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

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int S>
__global__ void __launch_bounds__(S_NT)
k_step_split(const Work *__restrict__ work, int64_t nwork, const Group *__restrict__ groups,
             const Seg *__restrict__ segs, Bufs bufs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double *Ad = reinterpret_cast<double *>(smem_raw);            // [TM][TK]
  double *Bd = Ad + S_TM * S_TK;                                // [TN][TK]
  __nv_bfloat16 *Ap = reinterpret_cast<__nv_bfloat16 *>(Bd + S_TN * S_TK);  // [S][TM][PAD]
  __nv_bfloat16 *Bp = Ap + S * S_TM * S_PAD;                    // [S][TN][PAD]
  int *Ea = reinterpret_cast<int *>(Bp + S * S_TN * S_PAD);     // [TM]
  int *Eb = Ea + S_TM;                                          // [TN]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 16, wn = (warp & 1) * 16;  // warp tile origin
  const int gq = lane >> 2, tq = lane & 3;

  for (int64_t w = blockIdx.x; w < nwork; w += gridDim.x) {
    const Work wk = work[w];
    const Group g = groups[wk.group];
    const int m0 = wk.mt * S_TM, n0 = wk.nt * S_TN;
    // two-float accumulators: [ntile 0..1][c 0..3]
    float hi[8], lo[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) hi[i] = lo[i] = 0.f;

    for (int si = 0; si < g.nseg; ++si) {
      const Seg s = segs[g.seg0 + si];
      const double *A = bufs.p[s.abuf] + s.a_off;
      const double *B = bufs.p[s.bbuf] + s.b_off;
      const bool a_kfast = s.sak == 1, b_nfast = s.sbn == 1;
      const bool unit_alpha = s.alpha == 1.0;
      const float ahi = (float)s.alpha;
      const float alo = (float)(s.alpha - (double)ahi);
      for (int k0 = 0; k0 < s.K; k0 += S_TK) {
        // 1. stage FP64 operands
        for (int e = tid; e < S_TM * S_TK; e += S_NT) {
          int r, k;
          if (a_kfast) { r = e / S_TK; k = e % S_TK; } else { r = e % S_TM; k = e / S_TM; }
          double v = 0.0;
          if (m0 + r < g.M && k0 + k < s.K) v = A[(int64_t)(m0 + r) * s.sam + (int64_t)(k0 + k) * s.sak];
          Ad[r * S_TK + k] = v;
        }
        for (int e = tid; e < S_TN * S_TK; e += S_NT) {
          int c, k;
          if (b_nfast) { k = e / S_TN; c = e % S_TN; } else { c = e / S_TK; k = e % S_TK; }
          double v = 0.0;
          if (n0 + c < g.N && k0 + k < s.K) v = B[(int64_t)(k0 + k) * s.sbk + (int64_t)(n0 + c) * s.sbn];
          Bd[c * S_TK + k] = v;
        }
        __syncthreads();
        // 2. shared exponent per row of A / column of B (4 threads per line)
        {
          const int line = tid >> 2, part = tid & 3;
          int ea = 0, eb = 0;
#pragma unroll
          for (int k = part * 8; k < part * 8 + 8; ++k) {
            ea = max(ea, dexp(Ad[line * S_TK + k]));
            eb = max(eb, dexp(Bd[line * S_TK + k]));
          }
          ea = max(ea, __shfl_xor_sync(0xffffffffu, ea, 1));
          ea = max(ea, __shfl_xor_sync(0xffffffffu, ea, 2));
          eb = max(eb, __shfl_xor_sync(0xffffffffu, eb, 1));
          eb = max(eb, __shfl_xor_sync(0xffffffffu, eb, 2));
          if (part == 0) {
            Ea[line] = ea;
            Eb[line] = eb;
          }
        }
        __syncthreads();
        // 3. digit planes
        for (int e = tid; e < S_TM * S_TK; e += S_NT) {
          const int r = e / S_TK, k = e % S_TK;
          float d[S];
          digits<S>(Ad[e], Ea[r], d);
#pragma unroll
          for (int p = 0; p < S; ++p) Ap[(p * S_TM + r) * S_PAD + k] = __float2bfloat16_rn(d[p]);
          digits<S>(Bd[e], Eb[r], d);
#pragma unroll
          for (int p = 0; p < S; ++p) Bp[(p * S_TN + r) * S_PAD + k] = __float2bfloat16_rn(d[p]);
        }
        __syncthreads();
        // 4. digit products per level l = s + t (levels 0..S-1 here), exact
        float acc[S][8];
#pragma unroll
        for (int l = 0; l < S; ++l)
#pragma unroll
          for (int i = 0; i < 8; ++i) acc[l][i] = 0.f;
#pragma unroll
        for (int kk = 0; kk < S_TK; kk += 16) {
#pragma unroll
          for (int sa = 0; sa < S; ++sa) {
            uint32_t af[4];
            const __nv_bfloat16 *ap = Ap + (sa * S_TM + wm) * S_PAD + kk;
            af[0] = *reinterpret_cast<const uint32_t *>(ap + gq * S_PAD + 2 * tq);
            af[1] = *reinterpret_cast<const uint32_t *>(ap + (gq + 8) * S_PAD + 2 * tq);
            af[2] = *reinterpret_cast<const uint32_t *>(ap + gq * S_PAD + 2 * tq + 8);
            af[3] = *reinterpret_cast<const uint32_t *>(ap + (gq + 8) * S_PAD + 2 * tq + 8);
#pragma unroll
            for (int sb = 0; sb + sa < S; ++sb) {
#pragma unroll
              for (int nt = 0; nt < 2; ++nt) {
                uint32_t bf[2];
                const __nv_bfloat16 *bp = Bp + (sb * S_TN + wn + nt * 8 + gq) * S_PAD + kk;
                bf[0] = *reinterpret_cast<const uint32_t *>(bp + 2 * tq);
                bf[1] = *reinterpret_cast<const uint32_t *>(bp + 2 * tq + 8);
                mma_bf16(&acc[sa + sb][nt * 4], af, bf);
              }
            }
          }
        }
        // 5. scale each level by 2^(Ea + Eb - 2044 - 8(l+2)) and accumulate
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int r = wm + gq + (i >> 1) * 8;
            const int c = wn + nt * 8 + 2 * tq + (i & 1);
            const int base = Ea[r] + Eb[c] - 2044;
            if (Ea[r] == 0 || Eb[c] == 0) continue;
#pragma unroll
            for (int l = 0; l < S; ++l) {
              const float x = scale_pow2(acc[l][nt * 4 + i], base - 8 * (l + 2));
              if (unit_alpha) {
                two_sum_acc(hi[nt * 4 + i], lo[nt * 4 + i], x);
              } else {
                const float p = x * ahi;
                const float pe = fmaf(x, ahi, -p) + x * alo;
                two_sum_acc(hi[nt * 4 + i], lo[nt * 4 + i], p);
                lo[nt * 4 + i] += pe;
              }
            }
          }
        }
        __syncthreads();
      }
    }
    double *C = bufs.p[g.cbuf] + g.c_off;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = m0 + wm + gq + (i >> 1) * 8;
        const int c = n0 + wn + nt * 8 + 2 * tq + (i & 1);
        if (r < g.M && c < g.N)
          C[(int64_t)r * g.scm + (int64_t)c * g.scn] = (double)hi[nt * 4 + i] + (double)lo[nt * 4 + i];
      }
    }
  }
}

template <int S>
static int launch_split_t(const Step &s, const Bufs &b, void *stream) {
  const size_t smem = (size_t)(S_TM + S_TN) * S_TK * sizeof(double) +
                      (size_t)S * (S_TM + S_TN) * S_PAD * sizeof(__nv_bfloat16) +
                      (size_t)(S_TM + S_TN) * sizeof(int);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_step_split<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_step_split<S><<<grid_for(s.nwork_tc, 8), S_NT, smem, (cudaStream_t)stream>>>(
      s.d_work_tc, s.nwork_tc, s.d_groups, s.d_segs, b);
  return launch_error("k_step_split");
}

int launch_step_split(const Step &s, const Bufs &b, int nslices, void *stream) {
  if (s.nwork_tc == 0) return ZMPO_OK;
  if (nslices == 4) return launch_split_t<4>(s, b, stream);
  if (nslices == 7) return launch_split_t<7>(s, b, stream);
  return record_arg_error("unsupported slice count");
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
