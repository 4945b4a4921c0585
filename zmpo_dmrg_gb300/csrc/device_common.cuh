// Device-side helpers shared by the grouped GEMM kernels (kernels.cu,
// kernels_umma.cu): the slot record of a K slot of a group and the lookups
// of column-block groups.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace zmpo {

// column block of column col of a column-block group, and col relative to it
// (binary search: the blocks of a group are in ascending n0)
__device__ __forceinline__ int find_cblock(const ColBlock *__restrict__ cbl, const Group &g, int col,
                                           int &colrel) {
  colrel = 0;
  if (g.ncb <= 0 || col < 0 || col >= g.N) return -1;
  int lo = 0, hi = g.ncb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cbl[g.cb0 + mid].n0 <= col) lo = mid; else hi = mid - 1;
  }
  const ColBlock c = cbl[g.cb0 + lo];
  if (col < c.n0 || col >= c.n0 + c.n) return -1;
  colrel = col - c.n0;
  return lo;
}

// column-block map of the tile's columns n0 .. n0+tn-1 into shared memory
// (one binary search per column instead of one per access); needs a barrier
// before use
__device__ __forceinline__ void tile_cblocks(const ColBlock *__restrict__ cbl, const Group &g, int n0, int tn,
                                             int *cbj, int *cbrel) {
  for (int c = threadIdx.x; c < tn; c += blockDim.x) {
    int rel;
    cbj[c] = find_cblock(cbl, g, n0 + c, rel);
    cbrel[c] = rel;
  }
}

struct Slot {
  const double *a;  // A(row 0, k) of the slot's segment
  const double *b;  // B(k, col 0); column-block groups: B buffer base
  int64_t sam, sbn;
  double alpha;
  int scaled;       // alpha != 1 (decided once per slot, not per element)
  int seg;          // column-block groups: segment index inside the group
  int kk;           // and k inside the segment
  int pad;
};

// B(k, col) of a column-block group for the thread's column block jb
// (jb < 0: column outside the group) -- zero where the pair has no B part
__device__ __forceinline__ double load_b_cb(const Slot &sl, const SegB *__restrict__ segb, const Group &g,
                                            int jb, int colrel) {
  if (jb < 0) return 0.0;
  const SegB sb = segb[g.sb0 + (int64_t)sl.seg * g.ncb + jb];
  if (sb.b_off < 0) return 0.0;
  return __ldg(sl.b + sb.b_off + (int64_t)sl.kk * sb.sbk + (int64_t)colrel * sb.sbn);
}


}  // namespace zmpo
