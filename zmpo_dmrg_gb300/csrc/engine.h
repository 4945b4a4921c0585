// Internal declarations shared by the host-side planner (planner.cpp) and the
// device kernels (kernels.cu) of the GB300 DMRG engine.
#pragma once
#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace zmpo {

// Allocator whose resize() leaves new elements default-initialised (no zero
// fill for the plain record types): the planner sizes its record arrays and
// then fills them in place, part by part on several threads.
template <class T>
struct NoInitAllocator : std::allocator<T> {
  using value_type = T;
  template <class U>
  struct rebind {
    using other = NoInitAllocator<U>;
  };
  NoInitAllocator() noexcept = default;
  template <class U>
  NoInitAllocator(const NoInitAllocator<U> &) noexcept {}
  template <class U>
  void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new (static_cast<void *>(p)) U;
  }
  template <class U, class... A>
  void construct(U *p, A &&...a) {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};
template <class T>
using rec_vector = std::vector<T, NoInitAllocator<T>>;

// Device task records.  A "group" is one dense output sub-matrix
// C[m*scm + n*scn] (m < M, n < N) of an output block; it is the sum of its
// segments, each a strided GEMM alpha * A(m,k) B(k,n) with k < K.  All
// contributions to an output region live in one group, so every output
// element has exactly one writer and the sum order is fixed.
struct Seg {
  int64_t a_off, b_off;
  int64_t sam, sak, sbk, sbn;
  double alpha;
  int32_t K;
  int8_t abuf, bbuf, pad0, pad1;
};

struct Group {
  int64_t c_off;
  int64_t scm, scn;
  int32_t M, N;
  int32_t seg0, nseg;
  int32_t cbuf;
  // ncb = 0: one output block (c_off, scm, scn; B part in each Seg).
  // ncb > 0: "column-block group": the output blocks that share the same A
  // rows are side by side in N (ColBlock cb0 .. cb0+ncb-1), the segments are
  // the union of their A parts, and SegB[sb0 + s * ncb + j] is the B part of
  // segment s for column block j (b_off < 0: that pair does not exist, zero).
  // A is then cut into digit planes once per column tile of the whole row
  // instead of once per output block.
  int32_t ncb;
  int32_t cb0, sb0;
};

struct ColBlock {
  int64_t c_off, scm, scn;  // output block (buffer Group::cbuf)
  int32_t n0, n;            // its columns inside the group
};

struct SegB {
  int64_t b_off, sbk, sbn;
};

// Split-K: a long group is cut into parts written to plan-owned scratch and
// summed in part order by k_reduce (deterministic).
struct Reduction {
  int64_t c_off;        // destination (buffer cbuf)
  int64_t scm, scn;
  int64_t part_off;     // first partial (scratch), parts consecutive, M*N each
  int32_t M, N;
  int32_t nparts, cbuf;
  int64_t elem0;        // prefix of M*N over reductions (thread mapping)
};
static_assert(sizeof(Reduction) == 56, "Reduction record layout (zmpo_plan_step_tasks)");

struct Work {
  int32_t group;
  int32_t mt, nt;   // first row and first column of the tile inside the group
  int32_t pad;      // B-resident kernel: row tiles of the item (from row mt)
};

// tcgen05 path (kernels_umma.cu), split precision.  Groups whose whole K
// fits one exact pass (1 <= K <= 256, at least 64 rows) are multiplied in one
// pass per tile; groups with 256 < K <= 2048 and the split-K parts of longer
// groups in passes of 256 slots, each pass exact with its own exponents,
// summed in FP64 in pass order.  Prepare kernels cut the operand tiles of
// every pass once per launch into records that are the shared-memory image
// the tensor cores read (K-major, 64-byte swizzle), in a plane buffer:
//   A record (row tile of tm8 rows, tm8 = the tile's rows rounded up to 8, one
//     pass): nkb k blocks of 32 slots, each four planes of tm8 rows x 64
//     bytes, then 128 int32 row exponents;
//   B record (column tile of tn columns, one pass): nkb k blocks, each four
//     planes of tn rows x 64 bytes (plane s holds rows s*tn .. s*tn+tn-1),
//     then tn int32 column exponents.  Groups whose B parts in the pass are
//     the same share one B record.
// The output column map of a (group, column tile) -- tn int64 output offsets
// of (row 0, column c) (-1: no such column), then tn int64 output row strides
// -- is made by the planner (an array uploaded with the task lists).
// Every record size is a multiple of 16 bytes (bulk-copy granularity).
constexpr int kUmmaTM = 128, kUmmaMaxK = 256, kUmmaKB = 32;
constexpr int kUmmaLongMaxK = 2048;                 // K of a long item (passes of kUmmaMaxK)
constexpr int64_t kUmmaAPlane = 128 * 64;           // one 128-row digit plane of a k block
constexpr int64_t kUmmaAKB = 4 * kUmmaAPlane;       // four planes (shared-memory stage)
constexpr int64_t umma_a_rec_bytes(int nkb, int tm8) { return (int64_t)nkb * 256 * tm8 + kUmmaTM * 4; }
constexpr int64_t umma_b_kb_bytes(int tn) { return 4 * (int64_t)tn * 64; }
constexpr int64_t umma_b_rec_bytes(int nkb, int tn) { return nkb * umma_b_kb_bytes(tn) + (int64_t)tn * 4; }

struct PrepA {      // cut one A record: rows m0 .., slots k0 .. k0+kc-1 of the group
  int64_t rec;      // byte offset of the record in the plane buffer
  int32_t group, m0, k0, kc;
};
struct PrepB {      // cut one B record: columns n0 .. n0+tn-1, slots k0 .. k0+kc-1
  int64_t rec;
  int32_t group, n0, tn, k0, kc, pad;
};
struct UWork {      // tcgen05 work item: one column tile, a run of row tiles (one-pass)
  int64_t a_rec;    // or one row tile and every pass of its K (long); first A record
  int64_t b_rec;    // first B record of the column tile (one per pass, consecutive)
  int64_t cmap;     // its column map (element offset into the column-map array)
  int32_t group, m0;
  int32_t nrt_k;    // row tiles of the run (1 for long items) | K << 8
  int32_t pad;
};

constexpr int kMaxBufs = 8;
constexpr int kPartialBuf = 6;   // buffer slot of the split-K scratch
constexpr int kWorkspaceBuf = 5; // buffer slot of a sigma / renorm plan's workspace
struct Bufs {
  double *p[kMaxBufs];
};

// One launch worth of tasks (device copies + host mirror of sizes).
struct Step {
  int idx = 0;                   // position in its plan's chain
  rec_vector<Seg> segs;
  rec_vector<Group> groups;
  rec_vector<ColBlock> cblocks;
  rec_vector<SegB> segb;
  Seg *d_segs = nullptr;
  Group *d_groups = nullptr;
  ColBlock *d_cblocks = nullptr;
  SegB *d_segb = nullptr;
  Work *d_work_fp64 = nullptr;   // tiles of kTileFP64
  // tensor-core tiles of every group (7 digit slices)
  Work *d_work_tc[3][4] = {};  // [row tile 32/64/128][column tile 8/16/32/64]
  // 4 digit slices: the groups of the B-resident kernel (Work: column tile
  // nt, row tiles mt .. mt+pad-1) and the tiles of all other groups
  Work *d_work_tcb[2] = {};    // [64 x 64 tiles, 128 x 32 tiles]
  Work *d_work_tc4[3][4] = {};
  // 4 digit slices, the tcgen05 groups: the prepare items (A and B records)
  // and the work items of the one-pass kernel by column tile 16 / 32 / 64
  PrepA *d_prep_a = nullptr;
  PrepB *d_prep_b = nullptr;
  int64_t nprep_a = 0, nprep_b = 0;
  UWork *d_work_um[3] = {};
  int64_t nwork_um[3] = {};
  // one-pass items of each column tile by the k blocks of their B tile
  // (more than 4, 3-4, at most 2), in that order in d_work_um
  int64_t nwork_um_cls[3][3] = {};
  UWork *d_work_ul[3] = {};         // long items (passes), by column tile 16 / 32 / 64
  int64_t *d_cmap = nullptr;        // column maps of the tcgen05 work items
  int64_t nwork_ul[3] = {};
  int64_t nprep_a_kept = 0, nprep_b_kept = 0;  // the first items cut kept records
  // plane buffer of the step: a kept area (records of the operand sides in
  // keep_side -- bit 0 A, bit 1 B -- which stay fixed between calls) and a
  // per-call area, byte offsets from the buffer's base
  uint8_t keep_side = 0;
  int64_t plane_keep_off = 0, plane_keep_bytes = 0;
  int64_t plane_call_off = 0, plane_call_bytes = 0;
  int64_t plane_bytes = 0;          // the whole buffer
  // where the plane buffer lives: a byte offset into the workspace buffer
  // (sigma plans; every step of a plan shares one region), or step-owned
  // memory (plane_ws_off < 0: renormalisation and contraction plans,
  // allocated at the step's first split-precision run)
  int64_t plane_ws_off = -1;
  unsigned char *d_planes_own = nullptr;
  int64_t nwork_fp64 = 0;
  int64_t nwork_tc[3][4] = {};
  int64_t nwork_tcb[2] = {};
  int64_t nwork_tc4[3][4] = {};
  double flops = 0.0;            // sum of 2*m*n*k of the reference tasks
  // multiply-adds the tiles of the step issue (tile padding included, K of a
  // group rounded up to the 16-slot MMA step): FP64 tiles, 4-slice and
  // 7-slice tensor-core tiles (times the digit products per multiply-add)
  double mma_macs[3] = {0.0, 0.0, 0.0};
  int64_t ntasks = 0;
  // Work lists by precision family, made on the host (the split lists of a
  // sigma plan at plan time, every other list at the first run that needs
  // it) and copied to the device in one allocation per family: the common
  // records (segments, groups, column blocks, B parts, split-K sums), the
  // 4-slice lists (tcgen05 items, column maps, mma.sync tiles), the FP64
  // tiles, the 7-slice tiles.  gk: each group's K (the lists other than the
  // 4-slice ones need no segments).
  struct HostLists {
    std::vector<Work> w64, wtc[3][4], wtc4[3][4], wtcb[2];
    std::vector<UWork> um[3], ul[3];
    std::vector<PrepA> prep_a;   // kept items first
    std::vector<PrepB> prep_b;
    std::vector<int64_t> cmap;
  } hl;
  std::vector<int64_t> gk;
  int64_t nsegs = 0;             // segments (the host copy is freed at the first upload)
  bool lists_split = false, lists_fp64 = false, lists_emu = false;
  bool up_common = false, up_split = false, up_fp64 = false, up_emu = false;
  int64_t area_b0[2] = {0, 0};   // B records' offset in the per-call [0] / kept [1] area
  void *d_lists = nullptr, *d_lists_split = nullptr, *d_lists_fp64 = nullptr, *d_lists_emu = nullptr;
  std::vector<Reduction> reds;   // split-K reductions (host)
  Reduction *d_reds = nullptr;
  int64_t red_elems = 0;         // total output elements of the reductions
  int64_t part_elems = 0;        // scratch size (doubles)
  double *d_part = nullptr;      // split-K scratch, owned by the step
  double alg_bytes = 0.0;        // each operand tensor read once + output written once
  // profiling (zmpo_profile): events around the launch, accumulated time
  void *ev0 = nullptr, *ev1 = nullptr;
  bool ev_pending = false;
  double ms_total = 0.0;
  int64_t ncalls = 0;
};

// the prepared-plane buffer of a step for the buffers of this call
inline unsigned char *step_planes(const Step &s, const Bufs &b) {
  return s.plane_ws_off >= 0 ? reinterpret_cast<unsigned char *>(b.p[kWorkspaceBuf]) + s.plane_ws_off
                             : s.d_planes_own;
}

// Launchers (kernels.cu)
int launch_step_fp64(const Step &s, const Bufs &b, void *stream);
int launch_step_split(const Step &s, const Bufs &b, int nslices, void *stream, bool cut_kept = true);
int launch_reduce(const Step &s, const Bufs &b, void *stream);
// tcgen05 one-pass kernels (kernels_umma.cu) and their error word: the
// prepare kernels cut the step's one-pass operand tiles into `planes`, then
// the tensor-core kernels multiply them
int launch_step_umma(const Step &s, const Bufs &b, unsigned char *planes, bool cut_kept, void *stream);
int umma_device_status(int *code, int reset);

// Diagonal terms for HDiag: out[l, r] += alpha * sum_{a,b,c} Ld[a,l] Wi[a,b]
// Wj[b,c] Rd[c,r] for one psi block; Ld/Rd are diagonal blocks of the
// environments (strided), Wi/Wj scalars per (a,b) / (b,c) sector pair.
struct DiagTerm {
  int64_t l_off, r_off, wi_off, wj_off;  // element offsets of the blocks
  int64_t l_sa, l_sl;                     // L block strides for (a, l)
  int64_t r_sc, r_sr;                     // R block strides for (c, r)
  int64_t wi_sa, wi_sb;                   // Wi strides for (a, b)
  int64_t wj_sb, wj_sc;                   // Wj strides for (b, c)
  double alpha;
  int32_t da, db, dc;
  int32_t ncsite;                         // 1: no Wj factor (dc unused)
};
struct DiagBlock {
  int64_t out_off;
  int32_t dl, dr;
  int32_t t0, nt;
};
int launch_hdiag(const DiagBlock *blocks, int64_t nblocks, const DiagTerm *terms,
                 const Bufs &b, double *out, int max_ac, int max_ar, void *stream);

// error recording shared by both translation units
int record_cuda_error(const char *where, int cuda_err);
int record_arg_error(const char *msg);
int record_size_error(const char *msg);

}  // namespace zmpo
