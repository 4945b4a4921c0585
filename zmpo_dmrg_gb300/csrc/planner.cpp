// Host side of the GB300 DMRG engine: block layouts, symbolic block-sparse
// contraction (task lists), GEMM mapping of each block task, sigma / renorm /
// HDiag plans and the C ABI declared in include/zmpo_gb300.h.
//
// The symbolic part restates the reference's qtensor.fromQsyms
// (source/qtensor/qtensor.py:272-346), the C rule symAllowed
// (ctypes/qsym.c:5-480) and qtensor.tensordotSYM (qtensor.py:563-637) as
// plain C++ over integer sector indices.  The numeric part (tensordotCAL,
// qtensor.py:642-659) becomes grouped GEMM launches in kernels.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <unordered_map>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>
#include "../../include/zmpo_gb300.h"
#include "engine.h"

namespace zmpo {

static thread_local std::string g_err;


static int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int record_cuda_error(const char *where, int cuda_err) {
  return fail(ZMPO_E_CUDA, std::string(where) + ": " + cudaGetErrorString((cudaError_t)cuda_err));
}

int record_arg_error(const char *msg) { return fail(ZMPO_E_ARG, msg); }

int record_size_error(const char *msg) { return fail(ZMPO_E_SIZE, msg); }

#define CUDA_TRY(x)                                                      \
  do {                                                                   \
    cudaError_t _e = (x);                                                \
    if (_e != cudaSuccess)                                               \
      return fail(_e == cudaErrorMemoryAllocation ? ZMPO_E_NOMEM         \
                                                  : ZMPO_E_CUDA,         \
                  std::string(#x) + ": " + cudaGetErrorString(_e));      \
  } while (0)

// ------------------------------------------------------------------ layouts
struct Packing {
  int64_t nblks = 0;
  int64_t size = 0;
  std::vector<int64_t> flat;     // allowed blocks, ascending flat index
  std::vector<int64_t> off;      // packed offset of each allowed block
  std::vector<int32_t> lookup;   // flat -> ordinal, -1 if not allowed
  std::vector<int32_t> bsec;     // [ordinal][leg] sector of each allowed block
  std::vector<int64_t> bdim;     // [ordinal][leg] dimension of each allowed block
};

struct Layout {
  int rank = 0, nq = 0;
  std::vector<int> nsec;
  std::vector<std::vector<double>> q;     // [leg][sec*nq + k]
  std::vector<std::vector<int64_t>> dim;  // [leg][sec]
  std::vector<int> status;
  std::shared_ptr<Packing> pk;

  int64_t secstride(int leg) const {
    int64_t s = 1;
    for (int j = rank - 1; j > leg; --j) s *= nsec[j];
    return s;
  }
  void sectors(int64_t flat, int *sec) const {
    for (int j = rank - 1; j >= 0; --j) {
      sec[j] = (int)(flat % nsec[j]);
      flat /= nsec[j];
    }
  }
  int64_t ravel(const int *sec) const {
    int64_t f = 0;
    for (int j = 0; j < rank; ++j) f = f * nsec[j] + sec[j];
    return f;
  }
  // sectors and dimensions of an allowed block (tables made with the packing)
  void block_sectors(int64_t ord, int *sec) const {
    const int32_t *p = pk->bsec.data() + (size_t)ord * rank;
    for (int j = 0; j < rank; ++j) sec[j] = p[j];
  }
  void block_dims(int64_t ord, int64_t *d) const {
    const int64_t *p = pk->bdim.data() + (size_t)ord * rank;
    for (int j = 0; j < rank; ++j) d[j] = p[j];
  }
};

// allowed iff sum_k |sum_{status 0} q_k - sum_{status 1} q_k| < 1e-10.
// Blocks are visited in ascending flat order by an odometer over legs
// 0 .. rank-2 that keeps the signed charge sums and the dimension products of
// the leading legs (accumulated leg by leg in the same order as a direct sum,
// so the test is bit-for-bit the direct one), with the last leg innermost.
// The sectors and dimensions of every allowed block are tabulated.
static void build_packing(Layout &L) {
  auto pk = std::make_shared<Packing>();
  int64_t nb = 1;
  for (int j = 0; j < L.rank; ++j) nb *= L.nsec[j];
  pk->nblks = nb;
  pk->lookup.assign((size_t)nb, -1);
  const int R = L.rank, nq = L.nq;
  if (R == 0) {
    pk->lookup[0] = 0;
    pk->flat.push_back(0);
    pk->off.push_back(0);
    pk->size = 1;
    L.pk = pk;
    return;
  }
  for (int j = 0; j < R; ++j)
    if (L.nsec[j] == 0) {
      L.pk = pk;
      return;
    }
  std::vector<int> sec(R, 0);
  std::vector<double> part((size_t)R * nq, 0.0);  // part[j] = signed charge sum of legs < j
  std::vector<int64_t> dprod(R, 1);               // dprod[j] = dimension product of legs < j
  auto set_leg = [&](int j) {  // part[j+1], dprod[j+1] from leg j's sector
    const double sg = L.status[j] ? -1.0 : 1.0;
    const double *qq = &L.q[j][(size_t)sec[j] * nq];
    for (int k = 0; k < nq; ++k) part[(size_t)(j + 1) * nq + k] = part[(size_t)j * nq + k] + sg * qq[k];
    dprod[j + 1] = dprod[j] * L.dim[j][sec[j]];
  };
  for (int j = 0; j + 1 < R; ++j) set_leg(j);
  const int last = R - 1;
  const double sgl = L.status[last] ? -1.0 : 1.0;
  int64_t f = 0, off = 0;
  while (true) {
    const double *pre = &part[(size_t)last * nq];
    for (int s = 0; s < L.nsec[last]; ++s, ++f) {
      const double *qq = &L.q[last][(size_t)s * nq];
      double dtot = 0.0;
      for (int k = 0; k < nq; ++k) dtot += std::fabs(pre[k] + sgl * qq[k]);
      if (dtot < 1e-10) {
        pk->lookup[(size_t)f] = (int32_t)pk->flat.size();
        pk->flat.push_back(f);
        pk->off.push_back(off);
        off += dprod[last] * L.dim[last][s];
        for (int j = 0; j < last; ++j) {
          pk->bsec.push_back(sec[j]);
          pk->bdim.push_back(L.dim[j][sec[j]]);
        }
        pk->bsec.push_back(s);
        pk->bdim.push_back(L.dim[last][s]);
      }
    }
    int j = last - 1;
    while (j >= 0 && ++sec[j] == L.nsec[j]) sec[j--] = 0;
    if (j < 0) break;
    for (int t = j; t < last; ++t) set_leg(t);
  }
  pk->size = off;
  L.pk = pk;
}

// ------------------------------------------------------------ contractions
struct Task {
  int32_t ob, ab, bb;
};

struct Contraction {
  int lay_a = -1, lay_b = -1, lay_out = -1;
  std::vector<int> e1, i1, e2, i2;
  std::vector<Task> tasks;  // sorted by output block
  std::vector<int64_t> task_start;  // [nout+1] CSR over output blocks
};

// Steps are built from "output works": one output block region and the list
// of block products that sum into it.
struct TaskRef {
  const Contraction *c;
  const Layout *la, *lb, *lo;
  int32_t ab, bb;
  int64_t a_base, b_base;
  int abuf, bbuf;
  double alpha;
};
struct OutWork {
  const Layout *lo;
  int32_t ob;
  int64_t c_base;
  int cbuf;
  std::vector<TaskRef> tasks;
};

struct Plan {
  int kind = 0;  // 1 contract, 2 sigma, 3 renorm
  std::vector<Step> steps;
  int64_t ws_elems = 0;
  double flops = 0.0;       // reference work F_ref (its task lists)
  double exec_flops = 0.0;  // work of the executed task lists
  int64_t ntasks = 0;
  // contract
  int lay_out = -1;
  // renorm
  std::vector<int> out_lay;
  std::vector<int64_t> out_off;
  int64_t out_total = 0;
  int status = 0;
  // sigma: kept records (records of the environments and the MPO in the
  // workspace's plane region) and whether the next call may reuse them
  bool reuse_next = false, kept_ready = false;
  const void *kept_ws = nullptr, *kept_L = nullptr, *kept_R = nullptr, *kept_W = nullptr;
  // sigma: the psi size (checked at call time) and HDiag tables
  int64_t ndim0 = 0;
  std::vector<DiagBlock> dblocks;
  std::vector<DiagTerm> dterms;
  DiagBlock *d_dblocks = nullptr;
  DiagTerm *d_dterms = nullptr;
  int64_t max_ac = 0, max_ar = 0;
  bool diag_uploaded = false;
};

}  // namespace zmpo

using namespace zmpo;

struct zmpo_engine {
  int device = 0;
  std::vector<std::unique_ptr<Layout>> layouts;
  std::vector<std::unique_ptr<Contraction>> contractions;
  std::vector<std::unique_ptr<Plan>> plans;
  // the sigma plan that last ran on each workspace buffer (a plan's kept
  // records in a workspace are valid only while no other plan used it)
  std::unordered_map<const void *, int> ws_user;
};

namespace zmpo {

static Layout *get_layout(zmpo_engine *e, int id) {
  if (!e || id < 0 || id >= (int)e->layouts.size() || !e->layouts[id]) return nullptr;
  return e->layouts[id].get();
}

static int add_layout(zmpo_engine *e, std::unique_ptr<Layout> L) {
  e->layouts.push_back(std::move(L));
  return (int)e->layouts.size() - 1;
}

// A plan keeps only its task lists: the symbolic contractions and the
// intermediate layouts made while building it are dropped afterwards (layout
// ids handed to the caller are kept), so long sweeps do not accumulate them.
static void drop_internal(zmpo_engine *e, size_t c0, size_t l0, const std::vector<int> &keep) {
  for (size_t i = c0; i < e->contractions.size(); ++i) e->contractions[i].reset();
  for (size_t i = l0; i < e->layouts.size(); ++i)
    if (std::find(keep.begin(), keep.end(), (int)i) == keep.end()) e->layouts[i].reset();
}

static bool same_q(const Layout &A, int la, const Layout &B, int lb) {
  if (A.nsec[la] != B.nsec[lb] || A.nq != B.nq) return false;
  for (size_t i = 0; i < A.q[la].size(); ++i)
    if (A.q[la][i] != B.q[lb][i]) return false;
  for (int s = 0; s < A.nsec[la]; ++s)
    if (A.dim[la][s] != B.dim[lb][s]) return false;
  return true;
}

// tensordotSYM: output layout + task list (qtensor.py:563-637)
// The output layout and the contraction go to the given (existing, empty)
// slots of the engine's tables, so several contractions can be built at
// once on different threads into slots reserved in advance.
static int build_contraction_at(zmpo_engine *e, int ia, int ib, int naxes, const int *ax_a,
                                const int *ax_b, int lay_slot, int contr_slot) {
  Layout *A = get_layout(e, ia), *B = get_layout(e, ib);
  if (!A || !B) return fail(ZMPO_E_ID, "contract: unknown layout");
  auto C = std::make_unique<Contraction>();
  C->lay_a = ia;
  C->lay_b = ib;
  std::vector<char> ina(A->rank, 0), inb(B->rank, 0);
  for (int k = 0; k < naxes; ++k) {
    if (ax_a[k] < 0 || ax_a[k] >= A->rank || ax_b[k] < 0 || ax_b[k] >= B->rank)
      return fail(ZMPO_E_ARG, "contract: axis out of range");
    ina[ax_a[k]] = 1;
    inb[ax_b[k]] = 1;
    C->i1.push_back(ax_a[k]);
    C->i2.push_back(ax_b[k]);
    if (!same_q(*A, ax_a[k], *B, ax_b[k]))
      return fail(ZMPO_E_SYM, "contract: contracted legs have different sectors");
  }
  for (int j = 0; j < A->rank; ++j)
    if (!ina[j]) C->e1.push_back(j);
  for (int j = 0; j < B->rank; ++j)
    if (!inb[j]) C->e2.push_back(j);
  std::vector<int> exts2;
  for (int j : C->e2) exts2.push_back(B->status[j]);
  if (naxes > 0) {
    bool flip = A->status[C->i1[0]] == B->status[C->i2[0]];
    for (int k = 0; k < naxes; ++k) {
      int s2 = B->status[C->i2[k]] ^ (flip ? 1 : 0);
      if (A->status[C->i1[k]] == s2)
        return fail(ZMPO_E_SYM, "contract: inconsistent leg directions");
    }
    if (flip)
      for (auto &s : exts2) s ^= 1;
  }
  auto O = std::make_unique<Layout>();
  O->nq = A->nq;
  for (int j : C->e1) {
    O->nsec.push_back(A->nsec[j]);
    O->q.push_back(A->q[j]);
    O->dim.push_back(A->dim[j]);
    O->status.push_back(A->status[j]);
  }
  for (size_t t = 0; t < C->e2.size(); ++t) {
    int j = C->e2[t];
    O->nsec.push_back(B->nsec[j]);
    O->q.push_back(B->q[j]);
    O->dim.push_back(B->dim[j]);
    O->status.push_back(exts2[t]);
  }
  O->rank = (int)O->nsec.size();
  build_packing(*O);
  // index A's allowed blocks by their external sector tuple
  const int ne1 = (int)C->e1.size(), ne2 = (int)C->e2.size();
  std::unordered_map<int64_t, std::vector<std::pair<int64_t, int32_t>>> amap;
  {
    int sec[16];
    for (size_t ob = 0; ob < A->pk->flat.size(); ++ob) {
      A->block_sectors((int64_t)ob, sec);
      int64_t ef = 0, inf = 0;
      for (int j : C->e1) ef = ef * A->nsec[j] + sec[j];
      for (int j : C->i1) inf = inf * A->nsec[j] + sec[j];
      amap[ef].push_back({inf, (int32_t)ob});
    }
    for (auto &kv : amap) std::sort(kv.second.begin(), kv.second.end());
  }
  C->task_start.assign(O->pk->flat.size() + 1, 0);
  int osec[16], bsec[16], isec[16];
  for (size_t ob = 0; ob < O->pk->flat.size(); ++ob) {
    C->task_start[ob] = (int64_t)C->tasks.size();
    O->block_sectors((int64_t)ob, osec);
    int64_t ef = 0;
    for (int t = 0; t < ne1; ++t) ef = ef * A->nsec[C->e1[t]] + osec[t];
    auto it = amap.find(ef);
    if (it == amap.end()) continue;
    for (auto &pr : it->second) {
      // internal sector indices from the A internal flat
      int64_t inf = pr.first;
      for (int k = naxes - 1; k >= 0; --k) {
        isec[k] = (int)(inf % A->nsec[C->i1[k]]);
        inf /= A->nsec[C->i1[k]];
      }
      for (int k = 0; k < naxes; ++k) bsec[C->i2[k]] = isec[k];
      for (int t = 0; t < ne2; ++t) bsec[C->e2[t]] = osec[ne1 + t];
      int64_t bf = B->ravel(bsec);
      int32_t bo = B->pk->lookup[(size_t)bf];
      if (bo < 0) continue;
      C->tasks.push_back({(int32_t)ob, pr.second, bo});
    }
  }
  C->task_start[O->pk->flat.size()] = (int64_t)C->tasks.size();
  e->layouts[lay_slot] = std::move(O);
  C->lay_out = lay_slot;
  e->contractions[contr_slot] = std::move(C);
  return ZMPO_OK;
}

static int build_contraction(zmpo_engine *e, int ia, int ib, int naxes, const int *ax_a,
                             const int *ax_b, int *out_layout, int *out_contr) {
  e->layouts.emplace_back();
  e->contractions.emplace_back();
  const int ls = (int)e->layouts.size() - 1, cs = (int)e->contractions.size() - 1;
  const int rc = build_contraction_at(e, ia, ib, naxes, ax_a, ax_b, ls, cs);
  if (rc) {
    e->layouts.pop_back();
    e->contractions.pop_back();
    return rc;
  }
  *out_layout = ls;
  *out_contr = cs;
  return ZMPO_OK;
}

// 2*m*n*k summed over the block tasks of a contraction (the reference's
// tensordotCAL work on the same task list)
static double contraction_flops(zmpo_engine *e, const Contraction *C) {
  const Layout *A = get_layout(e, C->lay_a), *B = get_layout(e, C->lay_b);
  double f = 0.0;
  int64_t ad[16], bd[16];
  for (const auto &t : C->tasks) {
    A->block_dims(t.ab, ad);
    B->block_dims(t.bb, bd);
    double m = 1, n = 1, k = 1;
    for (int j : C->e1) m *= (double)ad[j];
    for (int j : C->e2) n *= (double)bd[j];
    for (int j : C->i1) k *= (double)ad[j];
    f += 2.0 * m * n * k;
  }
  return f;
}

// ------------------------------------------------------------ GEMM mapping
struct Leg2 {
  int64_t d, s0, s1;
};

static void rowmajor_strides(const int64_t *d, int r, int64_t *st) {
  int64_t s = 1;
  for (int j = r - 1; j >= 0; --j) {
    st[j] = s;
    s *= d[j];
  }
}

// Expand all output works of one launch into groups / segments.
constexpr int64_t kSplitK = 2048;
static_assert(kSplitK == kUmmaLongMaxK, "a split-K part is one long tcgen05 item");

// Column-block groups: output blocks of one step whose groups read the same A
// rows (same output layout, same row-leg sectors, same A tensor and term) are
// joined side by side in N.  Their segments become the union of the A parts;
// each (segment, column block) pair keeps its own B part, or none.  Only
// groups made of one region with one segment per task take part, and only
// while the joined K stays below the split-K length.
// Key of the A rows an output block reads: output layout, A tensor (layout,
// buffer, base), output buffer, M and the row-leg sectors (fixed size, no
// heap allocation per group).
struct MergeKey {
  int64_t w[6 + 16];
  int n = 0;
  bool operator==(const MergeKey &o) const {
    if (n != o.n) return false;
    for (int i = 0; i < n; ++i)
      if (w[i] != o.w[i]) return false;
    return true;
  }
};
struct MergeKeyHash {
  size_t operator()(const MergeKey &k) const {
    uint64_t h = 0x9e3779b97f4a7c15ull ^ (uint64_t)k.n;
    for (int i = 0; i < k.n; ++i) {
      uint64_t x = (uint64_t)k.w[i] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
      h ^= x ^ (x >> 31);
    }
    return (size_t)h;
  }
};
struct MergeInfo {
  bool ok = false;
  MergeKey key;
};
// Merge keys of a part's groups in build order: only groups that may be
// joined keep a key (most groups of some steps never can, and a key is
// 184 bytes)
struct MergeTable {
  std::vector<int32_t> idx;     // per group: its key, or -1
  std::vector<MergeKey> keys;
  bool ok(size_t g) const { return idx[g] >= 0; }
  const MergeKey &key(size_t g) const { return keys[(size_t)idx[g]]; }
  void push(const MergeInfo &mi) {
    if (mi.ok) {
      idx.push_back((int32_t)keys.size());
      keys.push_back(mi.key);
    } else {
      idx.push_back(-1);
    }
  }
  void push_none() { idx.push_back(-1); }
  void pop() {
    if (idx.back() >= 0) keys.pop_back();
    idx.pop_back();
  }
};

// threads of one step's group build, and the block tasks per thread below
// which fewer are used
constexpr int kBuildThreads = 4;
constexpr int64_t kTasksPerThread = 8000;

template <class StepLike>
static void merge_column_blocks(StepLike &st, const MergeTable &info) {
  std::unordered_map<MergeKey, std::vector<int>, MergeKeyHash> buckets;
  buckets.reserve(st.groups.size());
  for (size_t g = 0; g < st.groups.size(); ++g)
    if (info.ok(g)) buckets[info.key(g)].push_back((int)g);
  bool any = false;
  for (const auto &kv : buckets) any = any || kv.second.size() >= 2;
  if (!any) return;  // nothing to join: the groups stay as they are
  rec_vector<Group> groups;
  rec_vector<Seg> segs;
  groups.reserve(st.groups.size());
  segs.reserve(st.segs.size());
  std::vector<char> done(st.groups.size(), 0);
  auto emit_plain = [&](int gi) {
    Group g = st.groups[gi];
    const int32_t s0 = g.seg0;
    g.seg0 = (int32_t)segs.size();
    for (int i = 0; i < g.nseg; ++i) segs.push_back(st.segs[s0 + i]);
    groups.push_back(g);
  };
  for (size_t gi = 0; gi < st.groups.size(); ++gi) {
    if (done[gi]) continue;
    if (!info.ok(gi)) {
      emit_plain((int)gi);
      continue;
    }
    const std::vector<int> &bk = buckets[info.key(gi)];
    for (int x : bk) done[x] = 1;
    if (bk.size() < 2) {
      emit_plain((int)gi);
      continue;
    }
    // union of A parts, in first-seen order (parts with the same A offset
    // are chained from a hash of that offset; the full part is compared)
    auto same_part = [](const Seg &x, const Seg &y) {
      return x.a_off == y.a_off && x.sam == y.sam && x.sak == y.sak && x.alpha == y.alpha && x.K == y.K &&
             x.abuf == y.abuf;
    };
    std::unordered_map<int64_t, int> first_part;
    std::vector<int> next_part;
    std::vector<Seg> parts;
    struct Use {
      int part, blk;
      SegB b;
    };
    std::vector<Use> uses;
    bool ok = true;
    int64_t ntot = 0, ktot = 0;
    const Group &G0 = st.groups[bk[0]];
    const int8_t bbuf = st.segs[G0.seg0].bbuf;
    for (size_t j = 0; j < bk.size() && ok; ++j) {
      const Group &G = st.groups[bk[j]];
      if (G.M != G0.M || G.cbuf != G0.cbuf) ok = false;
      ntot += G.N;
      for (int i = 0; i < G.nseg && ok; ++i) {
        const Seg &sg = st.segs[G.seg0 + i];
        if (sg.bbuf != bbuf) {
          ok = false;
          break;
        }
        int p = -1;
        auto it = first_part.find(sg.a_off);
        if (it != first_part.end())
          for (int q = it->second; q >= 0; q = next_part[q])
            if (same_part(parts[q], sg)) {
              p = q;
              break;
            }
        if (p < 0) {
          p = (int)parts.size();
          next_part.push_back(it != first_part.end() ? it->second : -1);
          first_part[sg.a_off] = p;
          parts.push_back(sg);
          ktot += sg.K;
        }
        uses.push_back({p, (int)j, {sg.b_off, sg.sbk, sg.sbn}});
      }
    }
    if (!ok || ktot > kSplitK || ntot > INT32_MAX) {
      for (int x : bk) emit_plain(x);
      continue;
    }
    Group mg{};
    mg.c_off = 0;
    mg.scm = mg.scn = 0;
    mg.M = G0.M;
    mg.N = (int32_t)ntot;
    mg.seg0 = (int32_t)segs.size();
    mg.nseg = (int32_t)parts.size();
    mg.cbuf = G0.cbuf;
    mg.ncb = (int32_t)bk.size();
    mg.cb0 = (int32_t)st.cblocks.size();
    mg.sb0 = (int32_t)st.segb.size();
    int32_t n0 = 0;
    for (int x : bk) {
      const Group &G = st.groups[x];
      st.cblocks.push_back({G.c_off, G.scm, G.scn, n0, G.N});
      n0 += G.N;
    }
    const size_t sb_base = st.segb.size();
    st.segb.resize(sb_base + parts.size() * bk.size(), SegB{-1, 0, 0});
    for (auto &u : uses) st.segb[sb_base + (size_t)u.part * bk.size() + u.blk] = u.b;
    for (auto &p : parts) {
      Seg sg = p;
      sg.b_off = -1;
      sg.sbk = sg.sbn = 0;
      segs.push_back(sg);
    }
    groups.push_back(mg);
  }
  st.groups.swap(groups);
  st.segs.swap(segs);
}

// Groups and segments of a range of output works (one part of a step, built
// on its own thread; the parts are joined in order).
struct GroupPart {
  rec_vector<Seg> segs;
  rec_vector<Group> groups;
  rec_vector<ColBlock> cblocks;
  rec_vector<SegB> segb;
  MergeTable minfo;
  std::vector<Reduction> reds;   // offsets (part_off, elem0, part groups' c_off) local to the part
  int64_t part_elems = 0, red_elems = 0;
  double flops = 0.0;
  int64_t ntasks = 0;
  std::vector<Seg> tmp;
};

// A group longer than kSplitK slots (the last one built) becomes parts of
// kSplitK slots (cut at segment boundaries or inside a segment), written to
// the split-K scratch (buffer kPartialBuf, M x N each, row-major) and summed
// in order into the group's output by a split-K reduction.
static void split_last_group(GroupPart &out) {
  const Group G = out.groups.back();
  int64_t ktot = 0;
  for (int i = 0; i < G.nseg; ++i) ktot += out.segs[G.seg0 + i].K;
  if (ktot <= kSplitK || G.M == 0 || G.N == 0) return;
  out.groups.pop_back();
  out.minfo.pop();
  out.tmp.assign(out.segs.begin() + G.seg0, out.segs.begin() + G.seg0 + G.nseg);
  out.segs.resize(G.seg0);
  Reduction r;
  r.c_off = G.c_off;
  r.scm = G.scm;
  r.scn = G.scn;
  r.M = G.M;
  r.N = G.N;
  r.cbuf = G.cbuf;
  r.part_off = out.part_elems;
  r.nparts = 0;
  const int64_t mn = (int64_t)G.M * G.N;
  Group cur{};
  auto open_part = [&]() {
    cur = Group{};
    cur.c_off = out.part_elems;
    cur.scm = G.N;
    cur.scn = 1;
    cur.M = G.M;
    cur.N = G.N;
    cur.cbuf = kPartialBuf;
    cur.seg0 = (int32_t)out.segs.size();
    cur.nseg = 0;
    out.part_elems += mn;
    r.nparts += 1;
  };
  auto close_part = [&]() {
    out.groups.push_back(cur);
    out.minfo.push_none();  // parts are never joined
  };
  open_part();
  int64_t kin = 0;
  for (const Seg &sgm : out.tmp) {
    int64_t k0 = 0;
    while (k0 < sgm.K) {
      if (kin >= kSplitK) {
        close_part();
        open_part();
        kin = 0;
      }
      const int64_t take = std::min<int64_t>(sgm.K - k0, kSplitK - kin);
      Seg piece = sgm;
      piece.a_off = sgm.a_off + k0 * sgm.sak;
      piece.b_off = sgm.b_off + k0 * sgm.sbk;
      piece.K = (int32_t)take;
      out.segs.push_back(piece);
      cur.nseg += 1;
      kin += take;
      k0 += take;
    }
  }
  close_part();
  r.elem0 = out.red_elems;
  out.red_elems += mn;
  out.reds.push_back(r);
}

// Per-task geometry of one output work, independent of its sub-regions:
// block dimensions and strides of both operands, the block offsets, the
// primary M / N / K strides, the K loops left after merging contiguous K
// legs, and the stride each sub-region loop adds to the A or B offset.
struct TaskGeo {
  int64_t ad[16], as[16], bd[16], bs[16];
  int64_t a0, b0, sam, sbn, sak, sbk, K, nk;
  int nkloop;
  Leg2 kloops[16];
  int64_t ls[16];
};

static int build_groups(std::vector<OutWork> &works, size_t w0, size_t w1, GroupPart &out) {
  std::vector<TaskGeo> geo;                          // reused across the works
  std::vector<std::pair<int, int>> mr, nr, loops;    // merged M / N legs, sub-region loops (range, isM)
  std::vector<int64_t> lidx;
  for (size_t wi = w0; wi < w1; ++wi) {
    OutWork &w = works[wi];
    const Layout &O = *w.lo;
    int64_t od[16], ost[16];
    O.block_dims(w.ob, od);
    rowmajor_strides(od, O.rank, ost);
    const int64_t c0 = w.c_base + O.pk->off[w.ob];
    // legs of the output block; M legs are e1 of each task's contraction, N
    // legs e2.  All tasks of one output work share the split (ne1 fixed).
    int ne1 = w.tasks.empty() ? O.rank : (int)w.tasks[0].c->e1.size();
    for (auto &t : w.tasks)
      if ((int)t.c->e1.size() != ne1) return fail(ZMPO_E_ARG, "mixed contraction split");
    geo.resize(w.tasks.size());
    for (size_t ti = 0; ti < w.tasks.size(); ++ti) {
      const TaskRef &tk = w.tasks[ti];
      TaskGeo &gt = geo[ti];
      tk.la->block_dims(tk.ab, gt.ad);
      tk.lb->block_dims(tk.bb, gt.bd);
      rowmajor_strides(gt.ad, tk.la->rank, gt.as);
      rowmajor_strides(gt.bd, tk.lb->rank, gt.bs);
    }
    // Determine M decomposition valid for C and every task's A; likewise N.
    // Represent each merged leg by its range of original legs.
    auto decompose = [&](int j0, int j1, bool isM, std::vector<std::pair<int, int>> &ranges) {
      ranges.clear();
      int start = -1;
      for (int j = j0; j < j1; ++j) {
        if (od[j] == 1) continue;
        if (start < 0) {
          start = j;
          ranges.push_back({j, j + 1});
          continue;
        }
        auto &rg = ranges.back();
        int outer = rg.second - 1;
        // find previous non-unit leg in the range
        while (outer >= rg.first && od[outer] == 1) --outer;
        bool ok = ost[outer] == od[j] * ost[j];
        for (size_t ti = 0; ti < w.tasks.size() && ok; ++ti) {
          const TaskRef &t = w.tasks[ti];
          const int64_t *xs = isM ? geo[ti].as : geo[ti].bs;
          const std::vector<int> &ex = isM ? t.c->e1 : t.c->e2;
          int jo = isM ? outer : outer - ne1, ji = isM ? j : j - ne1;
          ok = xs[ex[jo]] == od[j] * xs[ex[ji]];
        }
        if (ok)
          rg.second = j + 1;
        else
          ranges.push_back({j, j + 1});
      }
    };
    decompose(0, ne1, true, mr);
    decompose(ne1, O.rank, false, nr);
    auto rdim = [&](const std::pair<int, int> &r) {
      int64_t d = 1;
      for (int j = r.first; j < r.second; ++j) d *= od[j];
      return d;
    };
    auto innermost = [&](const std::pair<int, int> &r) {
      int j = r.second - 1;
      while (j > r.first && od[j] == 1) --j;
      return j;
    };
    // primary M / N range = largest; the others become sub-region loops
    int pm = -1, pn = -1;
    for (int i = 0; i < (int)mr.size(); ++i)
      if (pm < 0 || rdim(mr[i]) > rdim(mr[pm])) pm = i;
    for (int i = 0; i < (int)nr.size(); ++i)
      if (pn < 0 || rdim(nr[i]) > rdim(nr[pn])) pn = i;
    loops.clear();
    for (int i = 0; i < (int)mr.size(); ++i)
      if (i != pm) loops.push_back({i, 1});
    for (int i = 0; i < (int)nr.size(); ++i)
      if (i != pn) loops.push_back({i, 0});
    int64_t nsub = 1;
    for (auto &lp : loops) nsub *= rdim(lp.second ? mr[lp.first] : nr[lp.first]);
    const int64_t M = pm >= 0 ? rdim(mr[pm]) : 1;
    const int64_t N = pn >= 0 ? rdim(nr[pn]) : 1;
    const int64_t scm = pm >= 0 ? ost[innermost(mr[pm])] : 0;
    const int64_t scn = pn >= 0 ? ost[innermost(nr[pn])] : 0;
    if (M > INT32_MAX || N > INT32_MAX) return fail(ZMPO_E_SIZE, "block too large");
    // key of the A rows this output block reads (column-block groups)
    MergeInfo mi;
    mi.ok = nsub == 1 && !w.tasks.empty();
    if (mi.ok) {
      int sec[16];
      O.block_sectors(w.ob, sec);
      const auto &t0 = w.tasks[0];
      int64_t *kw = mi.key.w;
      kw[0] = (int64_t)(intptr_t)w.lo;
      kw[1] = (int64_t)(intptr_t)t0.la;
      kw[2] = t0.abuf;
      kw[3] = w.cbuf;
      kw[4] = t0.a_base;
      kw[5] = M;
      for (int j = 0; j < ne1; ++j) kw[6 + j] = sec[j];
      mi.key.n = 6 + ne1;
      for (auto &t : w.tasks)
        if (t.la != t0.la || t.abuf != t0.abuf || t.a_base != t0.a_base) mi.ok = false;
    }
    // the rest of each task's geometry (the reference work unit 2 m n k of
    // the full block product is counted here, once per task)
    for (size_t ti = 0; ti < w.tasks.size(); ++ti) {
      const TaskRef &tk = w.tasks[ti];
      TaskGeo &gt = geo[ti];
      const int64_t *ad = gt.ad, *as = gt.as, *bd = gt.bd, *bs = gt.bs;
      const auto &e1 = tk.c->e1, &e2 = tk.c->e2, &i1 = tk.c->i1, &i2 = tk.c->i2;
      {
        double m = 1, n = 1, k = 1;
        for (int j : e1) m *= (double)ad[j];
        for (int j : e2) n *= (double)bd[j];
        for (int j : i1) k *= (double)ad[j];
        out.flops += 2.0 * m * n * k;
        out.ntasks += 1;
      }
      gt.a0 = tk.a_base + tk.la->pk->off[tk.ab];
      gt.b0 = tk.b_base + tk.lb->pk->off[tk.bb];
      for (size_t i = 0; i < loops.size(); ++i) {
        auto &rg = loops[i].second ? mr[loops[i].first] : nr[loops[i].first];
        int jj = innermost(rg);
        gt.ls[i] = loops[i].second ? as[e1[jj]] : bs[e2[jj - ne1]];
      }
      gt.sam = pm >= 0 ? as[e1[innermost(mr[pm])]] : 0;
      gt.sbn = pn >= 0 ? bs[e2[innermost(nr[pn]) - ne1]] : 0;
      // K legs: sort by A stride (descending), merge where contiguous in both
      Leg2 kraw[16], kl[16];
      int nraw = 0, nkl = 0;
      for (size_t k = 0; k < i1.size(); ++k) kraw[nraw++] = {ad[i1[k]], as[i1[k]], bs[i2[k]]};
      std::sort(kraw, kraw + nraw, [](const Leg2 &x, const Leg2 &y) { return x.s0 > y.s0; });
      for (int i = 0; i < nraw; ++i) {
        const Leg2 &l = kraw[i];
        if (l.d == 1) continue;
        if (nkl > 0) {
          Leg2 &o = kl[nkl - 1];
          if (o.s0 == l.d * l.s0 && o.s1 == l.d * l.s1) {
            o.d *= l.d;
            o.s0 = l.s0;
            o.s1 = l.s1;
            continue;
          }
        }
        kl[nkl++] = l;
      }
      int pk = -1;
      for (int i = 0; i < nkl; ++i)
        if (pk < 0 || kl[i].d > kl[pk].d) pk = i;
      gt.K = pk >= 0 ? kl[pk].d : 1;
      gt.sak = pk >= 0 ? kl[pk].s0 : 0;
      gt.sbk = pk >= 0 ? kl[pk].s1 : 0;
      gt.nkloop = 0;
      for (int i = 0; i < nkl; ++i)
        if (i != pk) gt.kloops[gt.nkloop++] = kl[i];
      gt.nk = 1;
      for (int i = 0; i < gt.nkloop; ++i) gt.nk *= gt.kloops[i].d;
      if (gt.nk != 1) mi.ok = false;
    }
    lidx.assign(loops.size(), 0);
    auto sub_index = [&](int64_t sub) {
      int64_t t = sub;
      for (int i = (int)loops.size() - 1; i >= 0; --i) {
        int64_t d = rdim(loops[i].second ? mr[loops[i].first] : nr[loops[i].first]);
        lidx[i] = t % d;
        t /= d;
      }
    };
    for (int64_t sub = 0; sub < nsub; ++sub) {
      // multi-index of the sub-region over the loop ranges; each range is a
      // merged leg so its index maps linearly with the innermost stride
      sub_index(sub);
      int64_t coff = c0;
      for (size_t i = 0; i < loops.size(); ++i) {
        auto &rg = loops[i].second ? mr[loops[i].first] : nr[loops[i].first];
        coff += lidx[i] * ost[innermost(rg)];
      }
      Group g;
      g.c_off = coff;
      g.scm = scm;
      g.scn = scn;
      g.M = (int32_t)M;
      g.N = (int32_t)N;
      g.seg0 = (int32_t)out.segs.size();
      g.cbuf = w.cbuf;
      g.ncb = g.cb0 = g.sb0 = 0;
      for (size_t ti = 0; ti < w.tasks.size(); ++ti) {
        const TaskRef &tk = w.tasks[ti];
        const TaskGeo &gt = geo[ti];
        int64_t a0 = gt.a0, b0 = gt.b0;
        for (size_t i = 0; i < loops.size(); ++i) {
          if (loops[i].second)
            a0 += lidx[i] * gt.ls[i];
          else
            b0 += lidx[i] * gt.ls[i];
        }
        for (int64_t ki = 0; ki < gt.nk; ++ki) {
          int64_t aa = a0, bb = b0, tt = ki;
          for (int i = gt.nkloop - 1; i >= 0; --i) {
            int64_t x = tt % gt.kloops[i].d;
            tt /= gt.kloops[i].d;
            aa += x * gt.kloops[i].s0;
            bb += x * gt.kloops[i].s1;
          }
          Seg s;
          s.a_off = aa;
          s.b_off = bb;
          s.sam = gt.sam;
          s.sak = gt.sak;
          s.sbk = gt.sbk;
          s.sbn = gt.sbn;
          s.alpha = tk.alpha;
          s.K = (int32_t)gt.K;
          s.abuf = (int8_t)tk.abuf;
          s.bbuf = (int8_t)tk.bbuf;
          s.pad0 = s.pad1 = 0;
          out.segs.push_back(s);
        }
      }
      g.nseg = (int32_t)out.segs.size() - g.seg0;
      out.groups.push_back(g);
      out.minfo.push(mi);
      split_last_group(out);
    }
  }
  return ZMPO_OK;
}

static int build_step(std::vector<OutWork> &works, Step &st) {
  st.segs.clear();
  st.groups.clear();
  {
    // algorithmic traffic: every distinct operand tensor once, every output block once
    struct Operand {
      const Layout *l;
      int64_t base;
      int buf;
      bool operator<(const Operand &o) const { return std::tie(l, base, buf) < std::tie(o.l, o.base, o.buf); }
      bool operator==(const Operand &o) const { return l == o.l && base == o.base && buf == o.buf; }
    };
    std::vector<Operand> seen;
    Operand lastA{nullptr, -1, -1}, lastB{nullptr, -1, -1};
    double out_elems = 0.0;
    for (auto &w : works) {
      int64_t od[16];
      w.lo->block_dims(w.ob, od);
      double n = 1;
      for (int j = 0; j < w.lo->rank; ++j) n *= (double)od[j];
      out_elems += n;
      for (auto &t : w.tasks) {
        const Operand a{t.la, t.a_base, t.abuf}, b{t.lb, t.b_base, t.bbuf};
        // consecutive tasks mostly read the same tensors: skip repeats early
        // (the sort below removes the rest)
        if (!(a == lastA)) seen.push_back(lastA = a);
        if (!(b == lastB)) seen.push_back(lastB = b);
      }
    }
    std::sort(seen.begin(), seen.end());
    seen.erase(std::unique(seen.begin(), seen.end()), seen.end());
    double in_elems = 0.0;
    for (auto &o : seen) in_elems += (double)o.l->pk->size;
    st.alg_bytes = 8.0 * (in_elems + out_elems);
  }
  // parts of about equal task counts on their own threads (large steps)
  int64_t ntask_all = 0;
  for (auto &w : works) ntask_all += (int64_t)w.tasks.size();
  const int nparts = (int)std::max<int64_t>(1, std::min<int64_t>(kBuildThreads, ntask_all / kTasksPerThread));
  std::vector<size_t> cut(nparts + 1, works.size());
  cut[0] = 0;
  {
    int64_t acc = 0;
    int p = 1;
    for (size_t i = 0; i < works.size() && p < nparts; ++i) {
      acc += (int64_t)works[i].tasks.size();
      if (acc * nparts >= ntask_all * p) cut[p++] = i + 1;
    }
    // column-block groups join output blocks that read the same A tensor of
    // one term: a part ends where the term of single-term works changes, so
    // every join happens inside one part (and each part joins its own)
    auto term = [&](size_t i, int64_t &base, const Layout *&la) {
      const auto &t = works[i].tasks;
      if (t.empty() || t.front().a_base != t.back().a_base || t.front().la != t.back().la) return false;
      base = t.front().a_base;
      la = t.front().la;
      return true;
    };
    for (int q = 1; q < nparts; ++q) {
      if (cut[q] < cut[q - 1]) cut[q] = cut[q - 1];
      int64_t b0, b1;
      const Layout *l0, *l1;
      while (cut[q] > 0 && cut[q] < works.size() && term(cut[q] - 1, b0, l0) && term(cut[q], b1, l1) && b0 == b1 &&
             l0 == l1)
        ++cut[q];
    }
  }
  std::vector<GroupPart> parts(nparts);
  std::vector<int> rcs(nparts, ZMPO_OK);
  std::vector<std::string> msgs(nparts);
  if (nparts == 1) {
    rcs[0] = build_groups(works, 0, works.size(), parts[0]);
    if (rcs[0]) return rcs[0];
    merge_column_blocks(parts[0], parts[0].minfo);
  } else {
    std::vector<std::thread> pool;
    for (int p = 0; p < nparts; ++p)
      pool.emplace_back([&, p]() {
        rcs[p] = build_groups(works, cut[p], cut[p + 1], parts[p]);
        if (rcs[p] == ZMPO_OK) merge_column_blocks(parts[p], parts[p].minfo);
        if (rcs[p]) msgs[p] = g_err;
      });
    for (auto &t : pool) t.join();
    for (int p = 0; p < nparts; ++p)
      if (rcs[p]) return fail(rcs[p], msgs[p]);
  }
  // join the parts in order: segment, column-block, B-part and scratch
  // offsets shift by what the parts before hold
  st.reds.clear();
  st.cblocks.clear();
  st.segb.clear();
  st.red_elems = st.part_elems = 0;
  for (auto &p : parts) {
    for (Reduction r : p.reds) {
      r.part_off += st.part_elems;
      r.elem0 += st.red_elems;
      st.reds.push_back(r);
    }
    if (st.part_elems > 0)
      for (Group &g : p.groups)
        if (g.cbuf == kPartialBuf) g.c_off += st.part_elems;
    st.part_elems += p.part_elems;
    st.red_elems += p.red_elems;
  }
  if (nparts == 1) {
    st.segs.swap(parts[0].segs);
    st.groups.swap(parts[0].groups);
    st.cblocks.swap(parts[0].cblocks);
    st.segb.swap(parts[0].segb);
    st.flops += parts[0].flops;
    st.ntasks += parts[0].ntasks;
    return ZMPO_OK;
  }
  size_t ns = 0, ng = 0, nc = 0, nb = 0;
  for (auto &p : parts) {
    ns += p.segs.size();
    ng += p.groups.size();
    nc += p.cblocks.size();
    nb += p.segb.size();
  }
  // each part's records go to their place in the joined arrays on the
  // part's own thread
  st.segs.resize(ns);
  st.groups.resize(ng);
  st.cblocks.resize(nc);
  st.segb.resize(nb);
  struct Off {
    size_t s, g, c, b;
  };
  std::vector<Off> offs(nparts);
  {
    Off o{0, 0, 0, 0};
    for (int q = 0; q < nparts; ++q) {
      offs[q] = o;
      o.s += parts[q].segs.size();
      o.g += parts[q].groups.size();
      o.c += parts[q].cblocks.size();
      o.b += parts[q].segb.size();
      st.flops += parts[q].flops;
      st.ntasks += parts[q].ntasks;
    }
  }
  std::vector<std::thread> pool;
  for (int q = 0; q < nparts; ++q)
    pool.emplace_back([&st, &parts, &offs, q]() {
      GroupPart &p = parts[q];
      const Off o = offs[q];
      std::copy(p.segs.begin(), p.segs.end(), st.segs.begin() + o.s);
      std::copy(p.cblocks.begin(), p.cblocks.end(), st.cblocks.begin() + o.c);
      std::copy(p.segb.begin(), p.segb.end(), st.segb.begin() + o.b);
      Group *out = st.groups.data() + o.g;
      for (Group g : p.groups) {
        g.seg0 += (int32_t)o.s;
        if (g.ncb > 0) {
          g.cb0 += (int32_t)o.c;
          g.sb0 += (int32_t)o.b;
        }
        *out++ = g;
      }
      // the part's records are released on its thread
      rec_vector<Seg>().swap(p.segs);
      rec_vector<SegB>().swap(p.segb);
    });
  for (auto &t : pool) t.join();
  return ZMPO_OK;
}

// tile sizes of the two kernels (must match kernels.cu)
constexpr int kTileFP64M = 32, kTileFP64N = 32;
// B-resident kernel (kernels.cu, k_step_tcb): largest K it holds (four
// 64-slot or eight 32-slot chunks) and the row tiles of one work item
constexpr int kBresMaxK = 256, kBresRun = 16;


// Groups the one-pass tensor-core kernel (kernels_umma.cu) takes in the
// 4-slice path: the whole K in one exact pass, at least half a row tile.
// ZMPO_SPLIT_LEGACY=1 in the environment keeps every group on the mma.sync
// kernels (for comparisons).
constexpr int kUmmaMinM = 64;
static bool umma_enabled() {
  static const bool on = [] {
    const char *v = std::getenv("ZMPO_SPLIT_LEGACY");
    return !(v && v[0] == '1');
  }();
  return on;
}

// The tcgen05 routes of the split path: one-pass groups (the whole K in one
// exact pass, at least 64 rows, not a split-K part) and long groups (K up to
// kUmmaLongMaxK in passes of kUmmaMaxK slots: groups with a longer K than one
// pass, and every split-K part).
static bool umma_one_pass(const Group &G, int64_t ktot) {
  return umma_enabled() && ktot >= 1 && ktot <= kUmmaMaxK && G.M >= kUmmaMinM && G.N >= 1 &&
         G.cbuf != kPartialBuf;
}
static bool umma_long(const Group &G, int64_t ktot) {
  return umma_enabled() && ktot >= 1 && ktot <= kUmmaLongMaxK && G.M >= 1 && G.N >= 1 &&
         (ktot > kUmmaMaxK || G.cbuf == kPartialBuf);
}

// column tiles: full 64-column tiles, then the smallest of 16 / 32 / 64 that
// holds the rest
static int umma_tn(int rem) { return rem >= 64 ? 64 : (rem <= 16 ? 16 : (rem <= 32 ? 32 : 64)); }
static int umma_ti(int tn) { return tn == 16 ? 0 : (tn == 32 ? 1 : 2); }
static int umma_tm8(int M, int m0) { return (std::min(kUmmaTM, M - m0) + 7) & ~7; }

static int64_t group_k(const Step &st, const Group &G) {
  int64_t k = 0;
  for (int i = 0; i < G.nseg; ++i) k += st.segs[G.seg0 + i].K;
  return k;
}

// Records and work items of the tcgen05 groups of a step.  A group side
// (A or B) that the step's keep_side marks (bit 0: A, bit 1: B) has its
// records in the step's kept area (records of operands that stay fixed
// between calls, which a caller may let the next call reuse), every other
// side in the per-call area.  Each area holds its A records, then (from a
// 256-byte aligned offset) its B records.
struct UmmaLists {
  std::vector<PrepA> pa[2];          // [per-call, kept]; rec relative to its part
  std::vector<PrepB> pb[2];
  std::vector<UWork> w1[3], wl[3];   // one-pass / long items by column tile; pad = kept sides
  std::vector<int64_t> cmap;         // column maps (tn output offsets, then tn row strides each)
  // B-record sequences (all passes of a column tile) of plain groups, by a
  // hash of the tile and its B parts (candidates compared in full): groups
  // reading the same B parts share them
  struct BSeq {
    int32_t g, n0, tn, ncol;
    int64_t K, rec;
  };
  std::unordered_map<uint64_t, std::vector<BSeq>> bseq[2];
  int64_t abytes[2] = {0, 0}, bbytes[2] = {0, 0};
  double macs = 0.0;                 // multiply-adds the MMAs issue (x10 digit products)
};

// The B records of a column tile (columns n0 .. n0+tn-1, all K slots) of a
// plain group are fixed by the tile (n0, tn, its columns inside the group),
// K and the B part of every segment with slots (buffer, offset of its first
// slot, strides, length).  Equal tiles of two groups have equal records.
static uint64_t b_parts_hash(const Step &st, const Group &G) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (int i = 0; i < G.nseg; ++i) {
    const Seg &sg = st.segs[G.seg0 + i];
    if (sg.K <= 0) continue;
    for (int64_t v : {(int64_t)sg.bbuf, sg.b_off, sg.sbk, sg.sbn, (int64_t)sg.K}) h = (h ^ (uint64_t)v) * 0x100000001b3ull;
  }
  return h;
}
static bool same_b_parts(const Step &st, const Group &X, const Group &Y) {
  int i = 0, j = 0;
  while (true) {
    while (i < X.nseg && st.segs[X.seg0 + i].K <= 0) ++i;
    while (j < Y.nseg && st.segs[Y.seg0 + j].K <= 0) ++j;
    if (i == X.nseg || j == Y.nseg) return i == X.nseg && j == Y.nseg;
    const Seg &a = st.segs[X.seg0 + i], &b = st.segs[Y.seg0 + j];
    if (a.bbuf != b.bbuf || a.b_off != b.b_off || a.sbk != b.sbk || a.sbn != b.sbn || a.K != b.K) return false;
    ++i;
    ++j;
  }
}

// Output column map of columns n0 .. n0+tn-1 of a group: tn offsets of
// (row 0, column) (-1: none), then tn row strides
static void column_map(const Step &st, const Group &G, int n0, int tn, std::vector<int64_t> &out) {
  const size_t base = out.size();
  out.resize(base + 2 * (size_t)tn);
  // column blocks lie side by side in order of n0: find the first one that
  // ends after n0, then walk along with the columns
  int j = 0;
  if (G.ncb > 0) {
    int lo = 0, hi = G.ncb - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const ColBlock &cb = st.cblocks[G.cb0 + mid];
      if (cb.n0 + cb.n <= n0) lo = mid + 1; else hi = mid;
    }
    j = lo;
  }
  for (int c = 0; c < tn; ++c) {
    const int col = n0 + c;
    int64_t cbase = -1, rs = 0;
    if (col < G.N) {
      if (G.ncb == 0) {
        cbase = G.c_off + (int64_t)col * G.scn;
        rs = G.scm;
      } else {
        while (j < G.ncb && st.cblocks[G.cb0 + j].n0 + st.cblocks[G.cb0 + j].n <= col) ++j;
        if (j < G.ncb) {
          const ColBlock &cb = st.cblocks[G.cb0 + j];
          if (col >= cb.n0) {
            cbase = cb.c_off + (int64_t)(col - cb.n0) * cb.scn;
            rs = cb.scm;
          }
        }
      }
    }
    out[base + c] = cbase;
    out[base + tn + c] = rs;
  }
}

constexpr int kUmmaRunMax = 16;      // row tiles of a one-pass work item

static bool side_kept(const Step &st, bool a_side) { return (st.keep_side >> (a_side ? 0 : 1)) & 1u; }

// kbase: the group's first slot in G's segments (a split-K part counted
// before the split: G is the whole group)
static void umma_add_group(UmmaLists &L, const Step &st, int g, const Group &G, int64_t kbase, int64_t K,
                           bool keep_a, bool keep_b) {
  const bool one = umma_one_pass(G, K);
  if (!one && !umma_long(G, K)) return;
  const int ka = keep_a ? 1 : 0, kb = keep_b ? 1 : 0;
  const int nrt = (G.M + kUmmaTM - 1) / kUmmaTM;
  const int npass = (int)((K + kUmmaMaxK - 1) / kUmmaMaxK);
  const double k16 = (double)((K + 15) / 16 * 16);
  // A records: per row tile, per pass (one pass for one-pass groups)
  std::vector<int64_t> arec(nrt);
  for (int r = 0; r < nrt; ++r) {
    const int m0 = r * kUmmaTM, tm8 = umma_tm8(G.M, m0);
    arec[r] = L.abytes[ka];
    for (int j = 0; j < npass; ++j) {
      const int k0 = j * kUmmaMaxK, kc = (int)std::min<int64_t>(kUmmaMaxK, K - k0);
      L.pa[ka].push_back({L.abytes[ka], g, m0, k0, kc});
      L.abytes[ka] += umma_a_rec_bytes((kc + kUmmaKB - 1) / kUmmaKB, tm8);
    }
  }
  const int nruns = (nrt + kUmmaRunMax - 1) / kUmmaRunMax;
  const int len = (nrt + nruns - 1) / nruns;
  const int32_t sides = ka | (kb << 1);
  const uint64_t hparts = G.ncb == 0 ? b_parts_hash(st, G) : 0;
  for (int n0 = 0; n0 < G.N;) {
    // long groups wider than one tile take 64-column tiles only, so their
    // tiles run in one launch next to each other (A re-read from L2)
    const int tn = (!one && G.N > 64) ? 64 : umma_tn(G.N - n0), ti = umma_ti(tn);
    int64_t brec = -1;
    uint64_t kh = 0;
    const int ncol = std::min(tn, G.N - n0);
    if (G.ncb == 0 && kbase == 0) {
      kh = hparts;
      for (int64_t v : {(int64_t)n0, (int64_t)tn, (int64_t)ncol, K}) kh = (kh ^ (uint64_t)v) * 0x100000001b3ull;
      auto it = L.bseq[kb].find(kh);
      if (it != L.bseq[kb].end())
        for (const auto &c : it->second)
          if (c.n0 == n0 && c.tn == tn && c.ncol == ncol && c.K == K && same_b_parts(st, st.groups[c.g], G)) {
            brec = c.rec;
            break;
          }
    }
    if (brec < 0) {
      brec = L.bbytes[kb];
      if (G.ncb == 0 && kbase == 0) L.bseq[kb][kh].push_back({g, n0, tn, ncol, K, brec});
      for (int j = 0; j < npass; ++j) {
        const int k0 = j * kUmmaMaxK, kc = (int)std::min<int64_t>(kUmmaMaxK, K - k0);
        L.pb[kb].push_back({L.bbytes[kb], g, n0, tn, k0, kc, 0});
        L.bbytes[kb] += umma_b_rec_bytes((kc + kUmmaKB - 1) / kUmmaKB, tn);
      }
    }
    {
      const int64_t cm = (int64_t)L.cmap.size();
      column_map(st, G, n0, tn, L.cmap);
      if (one) {
        for (int r = 0; r < nrt; r += len)
          L.w1[ti].push_back({arec[r], brec, cm, g, r * kUmmaTM, std::min(len, nrt - r) | (int32_t)(K << 8), sides});
      } else {
        for (int r = 0; r < nrt; ++r)
          L.wl[ti].push_back({arec[r], brec, cm, g, r * kUmmaTM, 1 | (int32_t)(K << 8), sides});
      }
    }
    L.macs += (double)nrt * kUmmaTM * tn * k16;
    n0 += tn;
  }
}

static int64_t area_bytes(const UmmaLists &L, int k, int64_t *b0) {
  const int64_t a = (L.abytes[k] + 255) & ~int64_t(255);
  if (b0) *b0 = a;
  return L.abytes[k] + L.bbytes[k] > 0 ? ((a + L.bbytes[k] + 255) & ~int64_t(255)) : 0;
}

// Where a step's kept and per-call record areas lie in its plane buffer,
// and the record offsets of its prepare and work items from area-relative
// to buffer offsets (after build_split_lists).  Kept prepare items come
// first in their lists; a work item's pad holds its kept sides until then.
static void place_records(Step &st) {
  const int64_t abase[2] = {st.plane_call_off, st.plane_keep_off};
  const int64_t bbase[2] = {st.plane_call_off + st.area_b0[0], st.plane_keep_off + st.area_b0[1]};
  for (size_t i = 0; i < st.hl.prep_a.size(); ++i)
    st.hl.prep_a[i].rec += abase[(int64_t)i < st.nprep_a_kept ? 1 : 0];
  for (size_t i = 0; i < st.hl.prep_b.size(); ++i)
    st.hl.prep_b[i].rec += bbase[(int64_t)i < st.nprep_b_kept ? 1 : 0];
  for (int i = 0; i < 3; ++i)
    for (auto *wv : {&st.hl.um[i], &st.hl.ul[i]})
      for (auto &w : *wv) {
        w.a_rec += abase[w.pad & 1];
        w.b_rec += bbase[(w.pad >> 1) & 1];
        w.pad = 0;
      }
}

// A step-owned plane buffer: the kept area, then the per-call area
// (renormalisation and contraction plans: allocated at the step's first
// split-precision run).
static void place_step_owned(Step &st) {
  st.plane_ws_off = -1;
  st.plane_keep_off = 0;
  st.plane_call_off = st.plane_keep_bytes;
  st.plane_bytes = st.plane_keep_bytes + st.plane_call_bytes;
  place_records(st);
}

// Sigma plans: one plane region at the end of the workspace: the kept
// areas of the steps one after another, then one per-call area shared by
// the steps (they run one after another).  The records of operands that
// stay fixed while a Davidson solve calls the plan are kept: the
// environments, the MPO and, two-site, the MPO product O that step 0
// writes (keep_side per step, bit 0 = A, bit 1 = B; two-site: O = Wi Wj,
// T1 = L psi, T3 = T1 O, sigma = T3 R; one-site: T1 = L psi, T2 = T1 W,
// sigma = T2 R).  Other plans (renormalisation, which runs in FP64 or the
// 7-slice emulation, and contractions) keep nothing.
static uint8_t sigma_keep_side(int ncsite, int idx) {
  static const uint8_t kTwo[4] = {3, 1, 2, 2}, kOne[3] = {1, 2, 2};
  return ncsite == 2 ? (idx < 4 ? kTwo[idx] : 0) : (idx < 3 ? kOne[idx] : 0);
}

static void reserve_plane_region(Plan *P) {
  int64_t keep_total = 0, call_max = 0;
  for (auto &st : P->steps) {
    st.plane_keep_off = keep_total;
    keep_total += st.plane_keep_bytes;
    call_max = std::max(call_max, st.plane_call_bytes);
  }
  if (keep_total + call_max == 0) {
    for (auto &st : P->steps) place_step_owned(st);
    return;
  }
  const int64_t off = ((P->ws_elems * (int64_t)sizeof(double)) + 255) & ~int64_t(255);
  for (auto &st : P->steps) {
    st.plane_ws_off = off;
    st.plane_call_off = keep_total;
    st.plane_bytes = keep_total + call_max;
    place_records(st);
  }
  P->ws_elems = ((off + keep_total + call_max + 255) & ~int64_t(255)) / (int64_t)sizeof(double);
}

static void free_step(Step &st);

// Each group's K after the split-K parts, and the groups in order of cost
// (longest first, for load balance).
static void step_group_k(Step &st) {
  st.gk.assign(st.groups.size(), 0);
  for (size_t g = 0; g < st.groups.size(); ++g) {
    int64_t k = 0;
    for (int s = 0; s < st.groups[g].nseg; ++s) k += st.segs[st.groups[g].seg0 + s].K;
    st.gk[g] = k;
  }
  st.nsegs = (int64_t)st.segs.size();
}

static std::vector<int> cost_order(const Step &st) {
  std::vector<int> order(st.groups.size());
  std::iota(order.begin(), order.end(), 0);
  std::vector<int64_t> cost(st.groups.size());
  for (size_t g = 0; g < st.groups.size(); ++g) cost[g] = st.gk[g] + 16 * (int64_t)st.groups[g].nseg;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  return order;
}

// The structure every precision shares: per-group K.
static void finish_step_structure(Step &st) { step_group_k(st); }

// Column tiles of the mma.sync kernels.  Columns: full pieces of the widest
// tile, then one narrower tile for the rest (the smallest of 8/16/32/64 that
// holds it), so a group of 74 columns takes 64 + 16 instead of 64 + 64.
// 64-column tiles cut K in 64-slot chunks: a group with K <= 32 would leave
// half of every chunk empty, so it takes 32-column tiles (32-slot chunks)
// instead.  Rows: likewise with 128-row tiles (64 under 64-column tiles,
// 1024 threads at most) and a 32/64/128-row tile for the rest.
template <class F>
static void mma_sync_tiles(const Group &G, int64_t ktot, F &&tile) {
  const int wmax = ktot <= 32 ? 32 : 64;
  std::vector<std::pair<int, int>> rows;  // (first row, tile height)
  for (int n0 = 0; n0 < G.N;) {
    const int rem = G.N - n0;
    const int tn = rem >= wmax ? wmax : (rem <= 8 ? 8 : (rem <= 16 ? 16 : (rem <= 32 ? 32 : 64)));
    const int hmax = tn == 64 ? 64 : 128;
    rows.clear();
    for (int m0 = 0; m0 < G.M;) {
      const int rm = G.M - m0;
      const int tm = rm >= hmax ? hmax : (rm <= 32 ? 32 : (rm <= 64 ? 64 : 128));
      rows.push_back({m0, tm});
      m0 += tm;
    }
    tile(n0, tn, hmax, rows);
    n0 += tn;
  }
}

static int tile_index_n(int tn) { return tn == 8 ? 0 : (tn == 16 ? 1 : (tn == 32 ? 2 : 3)); }
static int tile_index_m(int tm) { return tm == 32 ? 0 : (tm == 64 ? 1 : 2); }

// 4-slice lists (needs the segments): the tcgen05 prepare and work items
// (record offsets relative to their area until place_records), the column
// maps, the sizes of the kept and per-call record areas, and the mma.sync
// tiles (B-resident and plain) of the groups the tcgen05 kernels do not take.
static void build_split_lists(Step &st) {
  auto &wtc4 = st.hl.wtc4;
  auto &wtcb = st.hl.wtcb;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 4; ++j) wtc4[i][j].clear();
  wtcb[0].clear();
  wtcb[1].clear();
  UmmaLists UL;
  st.mma_macs[1] = 0.0;
  auto order = cost_order(st);
  {
    // the column maps' final size (tcgen05 groups: 2 tn entries per column
    // tile), so the array is filled without regrowing
    size_t ncm = 0;
    for (size_t g = 0; g < st.groups.size(); ++g) {
      const Group &G = st.groups[g];
      const bool one = umma_one_pass(G, st.gk[g]);
      if (!one && !umma_long(G, st.gk[g])) continue;
      for (int n0 = 0; n0 < G.N;) {
        const int tn = (!one && G.N > 64) ? 64 : umma_tn(G.N - n0);
        ncm += 2 * (size_t)tn;
        n0 += tn;
      }
    }
    UL.cmap.reserve(ncm);
  }
  for (int g : order) {
    const Group &G = st.groups[g];
    const int64_t kt = st.gk[g];
    const double k16 = (double)((kt + 15) / 16 * 16);
    const double macs0 = UL.macs;
    umma_add_group(UL, st, g, G, 0, kt, side_kept(st, true), side_kept(st, false));
    if (UL.macs != macs0) {
      st.mma_macs[1] += UL.macs - macs0;
      continue;
    }
    mma_sync_tiles(G, kt, [&](int n0, int tn, int hmax, const std::vector<std::pair<int, int>> &rows) {
      // B-resident kernel: 64 x 64 or 128 x 32 tiles, a run of at least two
      // full-height row tiles, the whole K in one slot-table pass (at most
      // 32 segments, K <= kBresMaxK)
      const int bres = tn == 64 ? 0 : (tn == 32 ? 1 : -1);
      size_t nfull = 0;
      if (bres >= 0 && G.nseg <= 32 && kt <= kBresMaxK)
        while (nfull < rows.size() && rows[nfull].second == hmax) ++nfull;
      if (nfull < 2) nfull = 0;
      if (nfull) {
        const int nruns = (int)((nfull + kBresRun - 1) / kBresRun);
        const int len = (int)((nfull + nruns - 1) / nruns);
        for (int r = 0; r < (int)nfull; r += len)
          wtcb[bres].push_back({g, rows[r].first, n0, std::min(len, (int)nfull - r)});
      }
      for (size_t r = 0; r < rows.size(); ++r) {
        if (r >= nfull) wtc4[tile_index_m(rows[r].second)][tile_index_n(tn)].push_back({g, rows[r].first, n0, 0});
        st.mma_macs[1] += (double)rows[r].second * tn * k16;  // the same tiles, B-resident or not
      }
    });
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 4; ++j) st.nwork_tc4[i][j] = (int64_t)wtc4[i][j].size();
  for (int i = 0; i < 2; ++i) st.nwork_tcb[i] = (int64_t)wtcb[i].size();
  // area sizes; record offsets stay area-relative until place_records
  st.plane_call_bytes = area_bytes(UL, 0, &st.area_b0[0]);
  st.plane_keep_bytes = area_bytes(UL, 1, &st.area_b0[1]);
  // long items: groups whose first column tile shares a B-record sequence
  // run one after another, and a group's column tiles next to each other (the
  // repeated reads of a shared B sequence, and of a group's A records, come
  // from L2)
  {
    std::unordered_map<int, int64_t> first_b;
    for (int i = 2; i >= 0; --i)
      for (const UWork &w : UL.wl[i]) {
        auto it = first_b.find(w.group);
        if (it == first_b.end() || w.b_rec < it->second) first_b[w.group] = w.b_rec;
      }
    for (int i = 0; i < 3; ++i)
      std::stable_sort(UL.wl[i].begin(), UL.wl[i].end(), [&](const UWork &x, const UWork &y) {
        const int64_t bx = first_b[x.group], by = first_b[y.group];
        return bx != by ? bx < by : x.group < y.group;
      });
  }
  // prepare items: kept ones first (a call that reuses them skips them)
  st.hl.prep_a = UL.pa[1];
  st.hl.prep_a.insert(st.hl.prep_a.end(), UL.pa[0].begin(), UL.pa[0].end());
  st.hl.prep_b = UL.pb[1];
  st.hl.prep_b.insert(st.hl.prep_b.end(), UL.pb[0].begin(), UL.pb[0].end());
  st.nprep_a = (int64_t)st.hl.prep_a.size();
  st.nprep_b = (int64_t)st.hl.prep_b.size();
  st.nprep_a_kept = (int64_t)UL.pa[1].size();
  st.nprep_b_kept = (int64_t)UL.pb[1].size();
  for (int i = 0; i < 3; ++i) {
    // one-pass items by the k blocks of their B tile (more than 4, 3-4, at
    // most 2; the kernel of each class keeps a deeper A ring for a smaller B)
    auto cls = [](const UWork &w) {
      const int nkb = ((w.nrt_k >> 8) + kUmmaKB - 1) / kUmmaKB;
      return nkb > 4 ? 0 : (nkb > 2 ? 1 : 2);
    };
    std::stable_sort(UL.w1[i].begin(), UL.w1[i].end(),
                     [&](const UWork &x, const UWork &y) { return cls(x) < cls(y); });
    for (int c = 0; c < 3; ++c) st.nwork_um_cls[i][c] = 0;
    for (const UWork &w : UL.w1[i]) st.nwork_um_cls[i][cls(w)] += 1;
    st.nwork_um[i] = (int64_t)UL.w1[i].size();
    st.nwork_ul[i] = (int64_t)UL.wl[i].size();
    st.hl.um[i].swap(UL.w1[i]);
    st.hl.ul[i].swap(UL.wl[i]);
  }
  st.hl.cmap.swap(UL.cmap);
  st.lists_split = true;
}

// FP64 tiles (kTileFP64M x kTileFP64N) of every group.
static void build_fp64_list(Step &st) {
  st.hl.w64.clear();
  st.mma_macs[0] = 0.0;
  for (int g : cost_order(st)) {
    const Group &G = st.groups[g];
    const double k16 = (double)((st.gk[g] + 15) / 16 * 16);
    for (int m0 = 0; m0 < G.M; m0 += kTileFP64M)
      for (int n0 = 0; n0 < G.N; n0 += kTileFP64N) {
        st.hl.w64.push_back({g, m0, n0, 0});
        st.mma_macs[0] += (double)kTileFP64M * kTileFP64N * k16;
      }
  }
  st.nwork_fp64 = (int64_t)st.hl.w64.size();
  st.lists_fp64 = true;
}

// 7-slice mma.sync tiles of every group.
static void build_emu_lists(Step &st) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 4; ++j) st.hl.wtc[i][j].clear();
  st.mma_macs[2] = 0.0;
  for (int g : cost_order(st)) {
    const Group &G = st.groups[g];
    const double k16 = (double)((st.gk[g] + 15) / 16 * 16);
    mma_sync_tiles(G, st.gk[g], [&](int n0, int tn, int, const std::vector<std::pair<int, int>> &rows) {
      for (const auto &r : rows) {
        st.hl.wtc[tile_index_m(r.second)][tile_index_n(tn)].push_back({g, r.first, n0, 0});
        st.mma_macs[2] += (double)r.second * tn * k16;
      }
    });
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 4; ++j) st.nwork_tc[i][j] = (int64_t)st.hl.wtc[i][j].size();
  st.lists_emu = true;
}

// One device allocation for several host lists, each at a 256-byte aligned
// offset; *dptr of each list points into it (nullptr for an empty list).
struct ListUpload {
  struct Part {
    void **dst;
    const void *src;
    size_t bytes, off;
  };
  std::vector<Part> parts;
  size_t total = 0;
  template <class T, class A>
  void add(T **dptr, const std::vector<T, A> &v) {
    *dptr = nullptr;
    if (v.empty()) return;
    const size_t bytes = v.size() * sizeof(T);
    parts.push_back({(void **)dptr, v.data(), bytes, total});
    total += (bytes + 255) & ~size_t(255);
  }
  int run(void **dbuf) {
    if (total == 0) return ZMPO_OK;
    CUDA_TRY(cudaMalloc(dbuf, total));
    unsigned char *base = static_cast<unsigned char *>(*dbuf);
    for (const Part &p : parts) {
      CUDA_TRY(cudaMemcpy(base + p.off, p.src, p.bytes, cudaMemcpyHostToDevice));
      *p.dst = base + p.off;
    }
    return ZMPO_OK;
  }
};

// The host segments again (after the first upload freed them): the 4-slice
// lists of a plan other than a sigma plan are made at its first 4-slice run.
static int host_segments(Step &st) {
  if (!st.segs.empty() || st.nsegs == 0) return ZMPO_OK;
  if (!st.d_segs) return fail(ZMPO_E_ARG, "task lists: segments neither on the host nor on the device");
  st.segs.resize((size_t)st.nsegs);
  CUDA_TRY(cudaMemcpy(st.segs.data(), st.d_segs, st.segs.size() * sizeof(Seg), cudaMemcpyDeviceToHost));
  return ZMPO_OK;
}

// Host lists of a precision (made when missing).
static int host_lists(Step &st, int precision) {
  if (precision == ZMPO_PREC_SPLIT && !st.lists_split) {
    int rc = host_segments(st);
    if (rc) return rc;
    build_split_lists(st);
    place_step_owned(st);
    if (st.up_common) rec_vector<Seg>().swap(st.segs);
  } else if (precision == ZMPO_PREC_FP64 && !st.lists_fp64) {
    build_fp64_list(st);
  } else if (precision == ZMPO_PREC_EMU64 && !st.lists_emu) {
    build_emu_lists(st);
  }
  return ZMPO_OK;
}

// Device copies of the lists a run at this precision needs, made on first
// use (the common records, then the precision's family).  After the common
// upload the host segments are freed; the groups stay (sizes, the test
// interfaces).
static int upload_lists(Step &st, int precision) {
  if (!st.up_common) {
    ListUpload U;
    U.add(&st.d_segs, st.segs);
    U.add(&st.d_groups, st.groups);
    U.add(&st.d_cblocks, st.cblocks);
    U.add(&st.d_segb, st.segb);
    U.add(&st.d_reds, st.reds);
    int rc = U.run(&st.d_lists);
    if (rc) return rc;
    if (st.part_elems > 0) CUDA_TRY(cudaMalloc((void **)&st.d_part, st.part_elems * sizeof(double)));
    st.up_common = true;
    rec_vector<Seg>().swap(st.segs);
  }
  int rc = host_lists(st, precision);
  if (rc) return rc;
  if (precision == ZMPO_PREC_SPLIT && !st.up_split) {
    ListUpload U;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) U.add(&st.d_work_tc4[i][j], st.hl.wtc4[i][j]);
    for (int i = 0; i < 2; ++i) U.add(&st.d_work_tcb[i], st.hl.wtcb[i]);
    for (int i = 0; i < 3; ++i) {
      U.add(&st.d_work_um[i], st.hl.um[i]);
      U.add(&st.d_work_ul[i], st.hl.ul[i]);
    }
    U.add(&st.d_prep_a, st.hl.prep_a);
    U.add(&st.d_prep_b, st.hl.prep_b);
    U.add(&st.d_cmap, st.hl.cmap);
    rc = U.run(&st.d_lists_split);
    if (rc) return rc;
    st.up_split = true;
  } else if (precision == ZMPO_PREC_FP64 && !st.up_fp64) {
    ListUpload U;
    U.add(&st.d_work_fp64, st.hl.w64);
    rc = U.run(&st.d_lists_fp64);
    if (rc) return rc;
    std::vector<Work>().swap(st.hl.w64);
    st.up_fp64 = true;
  } else if (precision == ZMPO_PREC_EMU64 && !st.up_emu) {
    ListUpload U;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) U.add(&st.d_work_tc[i][j], st.hl.wtc[i][j]);
    rc = U.run(&st.d_lists_emu);
    if (rc) return rc;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) std::vector<Work>().swap(st.hl.wtc[i][j]);
    st.up_emu = true;
  }
  return ZMPO_OK;
}

// A failed upload (out of device memory, say) frees every device copy of
// the step, so a later call can try again from the host lists.
static int upload_step(Step &st, int precision) {
  const int rc = upload_lists(st, precision);
  if (rc != ZMPO_OK) free_step(st);
  return rc;
}

// Frees the device copies of every list family not (completely) uploaded.
static void free_step(Step &st) {
  if (!st.up_common) {
    cudaFree(st.d_lists);
    st.d_lists = nullptr;
    st.d_segs = nullptr;
    st.d_groups = nullptr;
    st.d_cblocks = nullptr;
    st.d_segb = nullptr;
    st.d_reds = nullptr;
    cudaFree(st.d_part);
    st.d_part = nullptr;
  }
  if (!st.up_split) {
    cudaFree(st.d_lists_split);
    st.d_lists_split = nullptr;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) st.d_work_tc4[i][j] = nullptr;
    for (int i = 0; i < 2; ++i) st.d_work_tcb[i] = nullptr;
    for (int i = 0; i < 3; ++i) st.d_work_um[i] = st.d_work_ul[i] = nullptr;
    st.d_prep_a = nullptr;
    st.d_prep_b = nullptr;
    st.d_cmap = nullptr;
  }
  if (!st.up_fp64) {
    cudaFree(st.d_lists_fp64);
    st.d_lists_fp64 = nullptr;
    st.d_work_fp64 = nullptr;
  }
  if (!st.up_emu) {
    cudaFree(st.d_lists_emu);
    st.d_lists_emu = nullptr;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) st.d_work_tc[i][j] = nullptr;
  }
}

// Every device allocation of the step (plan destruction).
static void release_step(Step &st) {
  if (st.ev0) cudaEventDestroy((cudaEvent_t)st.ev0);
  if (st.ev1) cudaEventDestroy((cudaEvent_t)st.ev1);
  st.ev0 = st.ev1 = nullptr;
  st.up_common = st.up_split = st.up_fp64 = st.up_emu = false;
  free_step(st);
  cudaFree(st.d_planes_own);
  st.d_planes_own = nullptr;
}

static bool g_profile = false;

static void profile_collect(Step &st) {
  if (!st.ev_pending) return;
  cudaEventSynchronize((cudaEvent_t)st.ev1);
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, (cudaEvent_t)st.ev0, (cudaEvent_t)st.ev1) == cudaSuccess) {
    st.ms_total += ms;
    st.ncalls += 1;
  }
  st.ev_pending = false;
}

static int run_step(Step &st, const Bufs &b, int precision, void *stream, bool cut_kept = true) {
  int rc = upload_step(st, precision);
  if (rc) return rc;
  // one NVTX range per step ("zmpo.step<i>"), so a profiler can select the
  // launches of one step of a chain
  static const char *kRange[] = {"zmpo.step0", "zmpo.step1", "zmpo.step2", "zmpo.step3",
                                 "zmpo.step4", "zmpo.step5", "zmpo.step6", "zmpo.step7"};
  nvtxRangePushA(kRange[st.idx & 7]);
  struct Pop {
    ~Pop() { nvtxRangePop(); }
  } pop;
  if (g_profile) {
    profile_collect(st);
    if (!st.ev0) {
      cudaEventCreate((cudaEvent_t *)&st.ev0);
      cudaEventCreate((cudaEvent_t *)&st.ev1);
    }
    cudaEventRecord((cudaEvent_t)st.ev0, (cudaStream_t)stream);
  }
  Bufs bb = b;
  bb.p[kPartialBuf] = st.d_part;
  if (precision == ZMPO_PREC_SPLIT && st.plane_bytes > 0 && st.plane_ws_off < 0 && !st.d_planes_own)
    CUDA_TRY(cudaMalloc((void **)&st.d_planes_own, st.plane_bytes));
  if (precision == ZMPO_PREC_FP64)
    rc = launch_step_fp64(st, bb, stream);
  else if (precision == ZMPO_PREC_SPLIT)
    rc = launch_step_split(st, bb, 4, stream, cut_kept);
  else if (precision == ZMPO_PREC_EMU64)
    rc = launch_step_split(st, bb, 7, stream);
  else
    return fail(ZMPO_E_ARG, "unknown precision");
  if (rc == ZMPO_OK) rc = launch_reduce(st, bb, stream);
  if (g_profile && rc == ZMPO_OK) {
    cudaEventRecord((cudaEvent_t)st.ev1, (cudaStream_t)stream);
    st.ev_pending = true;
  }
  return rc;
}

static Plan *get_plan(zmpo_engine *e, int id, int kind) {
  if (!e || id < 0 || id >= (int)e->plans.size() || !e->plans[id]) return nullptr;
  if (kind && e->plans[id]->kind != kind) return nullptr;
  return e->plans[id].get();
}

// per-class chain of contractions, instantiated per operator
struct ChainStep {
  int contr;  // contraction id
  int lay;    // output layout
};

}  // namespace zmpo

namespace zmpo {
// The single launch of a contraction plan whose device task lists exist
// (used by the allocation-free entry point in kernels.cu).
int contract_step_for(zmpo_engine *e, int plan_id, int precision, Step **out) {
  Plan *P = get_plan(e, plan_id, 1);
  if (!P) return fail(ZMPO_E_ID, "contract_exec_noalloc: unknown contraction plan");
  const Step &st = P->steps[0];
  const bool ready = st.up_common && (precision == ZMPO_PREC_SPLIT ? st.up_split
                                      : precision == ZMPO_PREC_FP64 ? st.up_fp64
                                                                    : st.up_emu);
  if (!ready)
    return fail(ZMPO_E_ARG,
                "contract_exec_noalloc: the plan has no device task lists for this precision yet; run it "
                "once at this precision through zmpo_contract_exec during set-up");
  *out = &P->steps[0];
  return ZMPO_OK;
}
}  // namespace zmpo

// ====================================================================== C ABI
extern "C" {

int zmpo_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return ZMPO_E_ARG;
  std::snprintf(buf, len, "%s", g_err.c_str());
  return ZMPO_OK;
}

int zmpo_version(void) { return 1; }

int symAllowed(int rank, int nqnum, int *ndims, int *status, int *allowed, double *a0,
               double *a1, double *a2, double *a3, double *a4, double *a5, double *a6,
               double *a7) {
  if (rank < 1 || rank > 8 || nqnum < 1 || !ndims || !status || !allowed)
    return fail(ZMPO_E_ARG, "symAllowed: rank must be 1..8");
  double *qs[8] = {a0, a1, a2, a3, a4, a5, a6, a7};
  int64_t nb = 1;
  for (int j = 0; j < rank; ++j) {
    if (!qs[j] || ndims[j] < 0) return fail(ZMPO_E_ARG, "symAllowed: missing leg");
    nb *= ndims[j];
  }
  int sec[8] = {0};
  std::vector<double> diff(nqnum);
  for (int64_t f = 0; f < nb; ++f) {
    int64_t t = f;
    for (int j = rank - 1; j >= 0; --j) {
      sec[j] = (int)(t % ndims[j]);
      t /= ndims[j];
    }
    std::fill(diff.begin(), diff.end(), 0.0);
    for (int j = 0; j < rank; ++j) {
      const double *q = qs[j] + (size_t)sec[j] * nqnum;
      for (int k = 0; k < nqnum; ++k) diff[k] += status[j] == 0 ? q[k] : -q[k];
    }
    double dtot = 0.0;
    for (int k = 0; k < nqnum; ++k) dtot += std::fabs(diff[k]);
    allowed[f] = dtot < 1.e-10;
  }
  return ZMPO_OK;
}

int zmpo_engine_create(zmpo_engine **out, int device) {
  if (!out) return fail(ZMPO_E_ARG, "engine_create: null out");
  *out = new zmpo_engine();
  (*out)->device = device;
  return ZMPO_OK;
}

int zmpo_engine_destroy(zmpo_engine *e) {
  if (!e) return ZMPO_OK;
  for (auto &p : e->plans) {
    if (!p) continue;
    for (auto &s : p->steps) release_step(s);
    cudaFree(p->d_dblocks);
    cudaFree(p->d_dterms);
  }
  delete e;
  return ZMPO_OK;
}

int zmpo_layout_create(zmpo_engine *e, int rank, int nqnum, const int *nsec,
                       const double *qsyms, const int64_t *dims, const int *status,
                       int *layout_id) {
  if (!e || !layout_id || rank < 0 || rank > 12 || nqnum < 1 || (rank > 0 && (!nsec || !qsyms || !dims || !status)))
    return fail(ZMPO_E_ARG, "layout_create: bad arguments");
  auto L = std::make_unique<Layout>();
  L->rank = rank;
  L->nq = nqnum;
  size_t qo = 0, dof = 0;
  int64_t nb = 1;
  for (int j = 0; j < rank; ++j) {
    if (nsec[j] < 1) return fail(ZMPO_E_ARG, "layout_create: empty leg");
    L->nsec.push_back(nsec[j]);
    L->q.emplace_back(qsyms + qo, qsyms + qo + (size_t)nsec[j] * nqnum);
    L->dim.emplace_back(dims + dof, dims + dof + nsec[j]);
    for (int s = 0; s < nsec[j]; ++s)
      if (dims[dof + s] < 1) return fail(ZMPO_E_ARG, "layout_create: sector dim < 1");
    L->status.push_back(status[j] ? 1 : 0);
    qo += (size_t)nsec[j] * nqnum;
    dof += nsec[j];
    nb *= nsec[j];
    if (nb > (int64_t)1 << 31) return fail(ZMPO_E_SIZE, "layout_create: too many blocks");
  }
  build_packing(*L);
  *layout_id = add_layout(e, std::move(L));
  return ZMPO_OK;
}

int zmpo_layout_derive(zmpo_engine *e, int src, const double *qsyms, const int *status,
                       int *layout_id) {
  Layout *S = get_layout(e, src);
  if (!S || !qsyms || !status || !layout_id) return fail(ZMPO_E_ARG, "layout_derive: bad arguments");
  auto L = std::make_unique<Layout>(*S);
  size_t qo = 0;
  for (int j = 0; j < L->rank; ++j) {
    L->q[j].assign(qsyms + qo, qsyms + qo + (size_t)L->nsec[j] * L->nq);
    qo += (size_t)L->nsec[j] * L->nq;
    L->status[j] = status[j] ? 1 : 0;
  }
  *layout_id = add_layout(e, std::move(L));
  return ZMPO_OK;
}

int zmpo_layout_info(zmpo_engine *e, int id, int64_t *size_allowed, int64_t *nblocks, int *rank) {
  Layout *L = get_layout(e, id);
  if (!L) return fail(ZMPO_E_ID, "layout_info: unknown layout");
  if (size_allowed) *size_allowed = L->pk->size;
  if (nblocks) *nblocks = (int64_t)L->pk->flat.size();
  if (rank) *rank = L->rank;
  return ZMPO_OK;
}

int zmpo_layout_blocks(zmpo_engine *e, int id, int64_t *flat, int64_t *off) {
  Layout *L = get_layout(e, id);
  if (!L) return fail(ZMPO_E_ID, "layout_blocks: unknown layout");
  for (size_t i = 0; i < L->pk->flat.size(); ++i) {
    if (flat) flat[i] = L->pk->flat[i];
    if (off) off[i] = L->pk->off[i];
  }
  return ZMPO_OK;
}

int zmpo_contract_plan(zmpo_engine *e, int lay_a, int lay_b, int naxes, const int *axes_a,
                       const int *axes_b, int *lay_out, int *plan_id) {
  if (!e || !lay_out || !plan_id || naxes < 0 || (naxes > 0 && (!axes_a || !axes_b)))
    return fail(ZMPO_E_ARG, "contract_plan: bad arguments");
  int lo = -1, ci = -1;
  const size_t c0 = e->contractions.size(), l0 = e->layouts.size();
  int rc = build_contraction(e, lay_a, lay_b, naxes, axes_a, axes_b, &lo, &ci);
  if (rc) return rc;
  auto P = std::make_unique<Plan>();
  P->kind = 1;
  P->lay_out = lo;
  const Contraction *C = e->contractions[ci].get();
  const Layout *A = get_layout(e, lay_a), *B = get_layout(e, lay_b), *O = get_layout(e, lo);
  std::vector<OutWork> works(O->pk->flat.size());
  for (size_t ob = 0; ob < O->pk->flat.size(); ++ob) {
    OutWork &w = works[ob];
    w.lo = O;
    w.ob = (int32_t)ob;
    w.c_base = 0;
    w.cbuf = 4;
    for (int64_t t = C->task_start[ob]; t < C->task_start[ob + 1]; ++t)
      w.tasks.push_back({C, A, B, O, C->tasks[t].ab, C->tasks[t].bb, 0, 0, 0, 1, 1.0});
  }
  P->steps.emplace_back();
  P->steps.back().idx = (int)P->steps.size() - 1;
  rc = build_step(works, P->steps.back());
  if (rc) return rc;
  finish_step_structure(P->steps.back());
  P->flops = P->steps.back().flops;
  P->ntasks = P->steps.back().ntasks;
  e->plans.push_back(std::move(P));
  drop_internal(e, c0, l0, {lo});
  *lay_out = lo;
  *plan_id = (int)e->plans.size() - 1;
  return ZMPO_OK;
}

int zmpo_contract_exec(zmpo_engine *e, int plan_id, const double *d_a, const double *d_b,
                       double *d_out, int precision, void *stream) {
  Plan *P = get_plan(e, plan_id, 1);
  if (!P) return fail(ZMPO_E_ID, "contract_exec: unknown plan");
  Bufs b{};
  b.p[0] = const_cast<double *>(d_a);
  b.p[1] = const_cast<double *>(d_b);
  b.p[4] = d_out;
  return run_step(P->steps[0], b, precision, stream);
}

// The steps of a chain have independent task lists: their GEMM mappings are
// built on one host thread per step (error text is per thread, so it is
// carried back to the caller's thread).
// The steps of a plan, one host thread per step: groups and segments, then
// the work lists.  keep_ncsite > 0: a sigma plan of that many dot sites (its
// steps keep the records of the operands fixed during a solve); 0: nothing
// kept.
extern "C++" {
template <class MakeWorks>
static int build_steps_parallel(Plan *P, int nstep, MakeWorks &&make_works, int keep_ncsite) {
  P->steps.resize(nstep);
  std::vector<int> rcs(nstep, ZMPO_OK);
  std::vector<std::string> msgs(nstep);
  std::vector<std::thread> pool;
  for (int s = 0; s < nstep; ++s) {
    P->steps[s].idx = s;
    P->steps[s].keep_side = keep_ncsite > 0 ? sigma_keep_side(keep_ncsite, s) : 0;
    pool.emplace_back([&, s]() {
      std::vector<OutWork> works;
      make_works(s, works);
      rcs[s] = build_step(works, P->steps[s]);
      if (rcs[s] == ZMPO_OK) {
        finish_step_structure(P->steps[s]);
        // sigma plans: the 4-slice lists now (their record areas are placed
        // in the workspace); other plans at their first 4-slice run
        if (keep_ncsite > 0) build_split_lists(P->steps[s]);
      }
      if (rcs[s]) msgs[s] = g_err;
    });
  }
  for (auto &t : pool) t.join();
  for (int s = 0; s < nstep; ++s)
    if (rcs[s]) return fail(rcs[s], msgs[s]);
  return ZMPO_OK;
}
}  // extern "C++"

int zmpo_sigma_plan(zmpo_engine *e, const zmpo_sigma_desc *d, int *plan_id) {
  if (!e || !d || !plan_id || d->nop < 0 || d->nclass < 1 || (d->ncsite != 1 && d->ncsite != 2))
    return fail(ZMPO_E_ARG, "sigma_plan: bad descriptor");
  const Layout *Psi = get_layout(e, d->lay_psi);
  if (!Psi) return fail(ZMPO_E_ID, "sigma_plan: unknown psi layout");
  const size_t c0 = e->contractions.size(), l0 = e->layouts.size();
  // Per-class symbolic chains (the reference caches the same per icase0,
  // mpo_dmrg_kernelQt.py:199-204).  The reference's two-site chain is
  //   T1 = L.psi, T2 = T1.Wi, T3 = T2.Wj, sigma = T3.R   (kernelQt.py:270-306)
  // and its tasks define the reported work F_ref.  The engine executes
  //   O = Wi.Wj (over the shared MPO bond), T1 = L.psi, T3 = T1.O, sigma = T3.R
  // which gives the same T3 layout without materialising T2.
  struct ClassChain {
    bool built = false;
    std::vector<ChainStep> c;  // executed steps
    double ref_flops = 0.0;
  };
  std::vector<ClassChain> chains(d->nclass);
  static const int ax1a[1] = {2}, ax1b[1] = {0};
  static const int ax2a[2] = {0, 2}, ax2b[2] = {0, 3};
  static const int ax3a[2] = {1, 3}, ax3b[2] = {3, 0};
  static const int ax4a[2] = {1, 3}, ax4b[2] = {2, 0};
  static const int ax3a1[2] = {1, 2}, ax3b1[2] = {2, 0};
  static const int axOa[1] = {1}, axOb[1] = {0};
  static const int axTa[3] = {0, 2, 3}, axTb[3] = {0, 2, 5};
  // classes in order of first appearance; each class's chain (a fixed
  // number of contractions) is built on its own thread into table slots
  // reserved for it, in the order a one-thread build would use them
  std::vector<int> cls_order;
  {
    std::vector<char> seen(d->nclass, 0);
    for (int op = 0; op < d->nop; ++op) {
      const int c = d->op_class[op];
      if (c < 0 || c >= d->nclass) return fail(ZMPO_E_ARG, "sigma_plan: bad class");
      if (!seen[c]) {
        seen[c] = 1;
        cls_order.push_back(c);
      }
    }
  }
  const int per_chain = d->ncsite == 2 ? 6 : 3;
  e->layouts.resize(l0 + cls_order.size() * per_chain);
  e->contractions.resize(c0 + cls_order.size() * per_chain);
  std::vector<int> chain_rc(cls_order.size(), ZMPO_OK);
  std::vector<std::string> chain_msg(cls_order.size());
  auto build_chain = [&](size_t k) -> int {
    const int c = cls_order[k];
    ClassChain &ch = chains[c];
    ch.built = true;
    int next_l = (int)(l0 + k * per_chain), next_c = (int)(c0 + k * per_chain);
    auto contract = [&](int ia, int ib, int n, const int *aa, const int *ab, int *lo_, int *ci_) {
      *lo_ = next_l++;
      *ci_ = next_c++;
      return build_contraction_at(e, ia, ib, n, aa, ab, *lo_, *ci_);
    };
    int lo = -1, ci = -1, rc = 0, l1 = -1, c1 = -1;
    rc = contract(d->lay_L[c], d->lay_psi, 1, ax1a, ax1b, &l1, &c1);
    if (rc) return rc;
    ch.ref_flops += contraction_flops(e, e->contractions[c1].get());
    if (d->ncsite == 2) {
      int l2, c2, l3, c3;
      rc = contract(l1, d->lay_Wi[c], 2, ax2a, ax2b, &l2, &c2);
      if (rc) return rc;
      rc = contract(l2, d->lay_Wj[c], 2, ax3a, ax3b, &l3, &c3);
      if (rc) return rc;
      ch.ref_flops += contraction_flops(e, e->contractions[c2].get()) +
                      contraction_flops(e, e->contractions[c3].get());
      int lO, cO;
      rc = contract(d->lay_Wi[c], d->lay_Wj[c], 1, axOa, axOb, &lO, &cO);
      if (rc) return rc;
      ch.c.push_back({cO, lO});
      ch.c.push_back({c1, l1});
      rc = contract(l1, lO, 3, axTa, axTb, &lo, &ci);
      if (rc) return rc;
      const Layout *T3a = get_layout(e, l3), *T3b = get_layout(e, lo);
      if (T3a->pk->flat != T3b->pk->flat || T3a->pk->size != T3b->pk->size)
        return fail(ZMPO_E_SYM, "sigma_plan: fused MPO step layout differs");
      ch.c.push_back({ci, lo});
      rc = contract(lo, d->lay_Rf[c], 2, ax4a, ax4b, &lo, &ci);
    } else {
      ch.c.push_back({c1, l1});
      rc = contract(l1, d->lay_Wi[c], 2, ax2a, ax2b, &lo, &ci);
      if (rc) return rc;
      ch.ref_flops += contraction_flops(e, e->contractions[ci].get());
      ch.c.push_back({ci, lo});
      rc = contract(lo, d->lay_Rf[c], 2, ax3a1, ax3b1, &lo, &ci);
    }
    if (rc) return rc;
    ch.ref_flops += contraction_flops(e, e->contractions[ci].get());
    ch.c.push_back({ci, lo});
    const Layout *Out = get_layout(e, lo);
    if (Out->pk->flat != Psi->pk->flat || Out->pk->size != Psi->pk->size)
      return fail(ZMPO_E_SYM, "sigma_plan: H.psi layout differs from psi layout");
    return ZMPO_OK;
  };
  {
    std::vector<std::thread> pool;
    for (size_t k = 0; k < cls_order.size(); ++k)
      pool.emplace_back([&, k]() {
        chain_rc[k] = build_chain(k);
        if (chain_rc[k]) chain_msg[k] = g_err;
      });
    for (auto &t : pool) t.join();
    for (size_t k = 0; k < cls_order.size(); ++k)
      if (chain_rc[k]) return fail(chain_rc[k], chain_msg[k]);
  }
  auto P = std::make_unique<Plan>();
  P->kind = 2;
  P->ndim0 = Psi->pk->size;
  const int nstep = (int)chains[d->op_class[0 < d->nop ? 0 : 0]].c.size();
  // workspace: per op, outputs of steps 0..nstep-2
  std::vector<std::vector<int64_t>> ws_off(d->nop, std::vector<int64_t>(nstep, 0));
  int64_t ws = 0;
  for (int op = 0; op < d->nop; ++op) {
    const ClassChain &ch = chains[d->op_class[op]];
    for (int s = 0; s < nstep - 1; ++s) {
      ws_off[op][s] = ws;
      ws += get_layout(e, ch.c[s].lay)->pk->size;
      ws = (ws + 31) & ~int64_t(31);
    }
    P->flops += ch.ref_flops;
  }
  P->ws_elems = ws;
  // Structurally zero intermediate blocks: an output block of an
  // intermediate step whose every task reads such a block (or that has no
  // task) is zero for any operand values.  It is neither written nor read:
  // its works are dropped and so are the tasks that read it.  src_step[s] =
  // the steps whose outputs step s reads as A and B (-1: a caller operand).
  static const int src2[4][2] = {{-1, -1}, {-1, -1}, {1, 0}, {2, -1}};
  static const int src1[3][2] = {{-1, -1}, {0, -1}, {1, -1}};
  auto src_step = [&](int s, int which) { return d->ncsite == 2 ? src2[s][which] : src1[s][which]; };
  std::vector<std::vector<std::vector<char>>> alive(d->nclass);
  for (int c = 0; c < d->nclass; ++c) {
    if (!chains[c].built) continue;
    alive[c].resize(nstep);
    for (int s = 0; s < nstep - 1; ++s) {
      const Contraction *C = e->contractions[chains[c].c[s].contr].get();
      const int sa = src_step(s, 0), sb = src_step(s, 1);
      const size_t nob = C->task_start.size() - 1;
      alive[c][s].assign(nob, 0);
      for (size_t ob = 0; ob < nob; ++ob)
        for (int64_t t = C->task_start[ob]; t < C->task_start[ob + 1]; ++t)
          if ((sa < 0 || alive[c][sa][C->tasks[t].ab]) && (sb < 0 || alive[c][sb][C->tasks[t].bb])) {
            alive[c][s][ob] = 1;
            break;
          }
    }
  }
  auto live_task = [&](int c, int s, const Task &t) {
    const int sa = src_step(s, 0), sb = src_step(s, 1);
    return (sa < 0 || alive[c][sa][t.ab]) && (sb < 0 || alive[c][sb][t.bb]);
  };
  // buffers: 0 L, 1 R, 2 W, 3 x, 4 y, 5 workspace
  // operand sources per executed step (two-site: O, T1, T3, sigma).  The
  // steps' task lists are independent: each step's output works and GEMM
  // mappings are built on a host thread of its own.
  auto make_works = [&](int s, std::vector<OutWork> &works) {
    auto src = [&](int op, bool isA, int &buf, int64_t &base) {
      if (d->ncsite == 2) {
        switch (s) {
          case 0: buf = 2; base = isA ? d->off_Wi[op] : d->off_Wj[op]; return;
          case 1: if (isA) { buf = 0; base = d->off_L[op]; } else { buf = 3; base = 0; } return;
          case 2: buf = 5; base = isA ? ws_off[op][1] : ws_off[op][0]; return;
          default: if (isA) { buf = 5; base = ws_off[op][2]; } else { buf = 1; base = d->off_R[op]; } return;
        }
      }
      switch (s) {
        case 0: if (isA) { buf = 0; base = d->off_L[op]; } else { buf = 3; base = 0; } return;
        case 1: if (isA) { buf = 5; base = ws_off[op][0]; } else { buf = 2; base = d->off_Wi[op]; } return;
        default: if (isA) { buf = 5; base = ws_off[op][1]; } else { buf = 1; base = d->off_R[op]; } return;
      }
    };
    if (s < nstep - 1) {
      for (int op = 0; op < d->nop; ++op) {
        const ClassChain &ch = chains[d->op_class[op]];
        const Contraction *C = e->contractions[ch.c[s].contr].get();
        const Layout *A = get_layout(e, C->lay_a), *B = get_layout(e, C->lay_b),
                     *O = get_layout(e, C->lay_out);
        int abuf, bbuf;
        int64_t abase, bbase;
        src(op, true, abuf, abase);
        src(op, false, bbuf, bbase);
        for (size_t ob = 0; ob < O->pk->flat.size(); ++ob) {
          if (!alive[d->op_class[op]][s][ob]) continue;
          OutWork w;
          w.lo = O;
          w.ob = (int32_t)ob;
          w.c_base = ws_off[op][s];
          w.cbuf = 5;
          // the term weight goes on the per-term MPO product O = w Wi.Wj
          // (two-site), so the sum over terms reads unscaled operands
          const double wgt = (d->ncsite == 2 && s == 0) ? d->wts[op] : 1.0;
          for (int64_t t = C->task_start[ob]; t < C->task_start[ob + 1]; ++t)
            if (live_task(d->op_class[op], s, C->tasks[t]))
              w.tasks.push_back({C, A, B, O, C->tasks[t].ab, C->tasks[t].bb, abase, bbase, abuf, bbuf, wgt});
          works.push_back(std::move(w));
        }
      }
    } else {
      // last step: every op contributes to the same psi blocks
      works.resize(Psi->pk->flat.size());
      for (size_t ob = 0; ob < works.size(); ++ob) {
        works[ob].lo = Psi;
        works[ob].ob = (int32_t)ob;
        works[ob].c_base = 0;
        works[ob].cbuf = 4;
      }
      for (int op = 0; op < d->nop; ++op) {
        const ClassChain &ch = chains[d->op_class[op]];
        const Contraction *C = e->contractions[ch.c[s].contr].get();
        const Layout *A = get_layout(e, C->lay_a), *B = get_layout(e, C->lay_b),
                     *O = get_layout(e, C->lay_out);
        int abuf, bbuf;
        int64_t abase, bbase;
        src(op, true, abuf, abase);
        src(op, false, bbuf, bbase);
        for (size_t ob = 0; ob < O->pk->flat.size(); ++ob)
          for (int64_t t = C->task_start[ob]; t < C->task_start[ob + 1]; ++t)
            if (live_task(d->op_class[op], s, C->tasks[t]))
              works[ob].tasks.push_back({C, A, B, O, C->tasks[t].ab, C->tasks[t].bb, abase, bbase, abuf,
                                         bbuf, d->ncsite == 2 ? 1.0 : d->wts[op]});
      }
    }
  };
  {
    int rc = build_steps_parallel(P.get(), nstep, make_works, d->ncsite);
    if (rc) return rc;
    for (auto &st : P->steps) {
      P->exec_flops += st.flops;
      P->ntasks += st.ntasks;
    }
    reserve_plane_region(P.get());
  }
  // ---- HDiag terms: out[l,r] += w * sum Ld[a,l] Wi[a,b] (Wj[b,c]) Rd[c,r]
  {
    int psec[16];
    for (size_t ob = 0; ob < Psi->pk->flat.size(); ++ob) {
      Psi->block_sectors((int64_t)ob, psec);
      DiagBlock db;
      db.out_off = Psi->pk->off[ob];
      db.dl = (int32_t)Psi->dim[0][psec[0]];
      db.dr = (int32_t)Psi->dim[Psi->rank - 1][psec[Psi->rank - 1]];
      db.t0 = (int32_t)P->dterms.size();
      const int sl = psec[0], sr = psec[Psi->rank - 1];
      const int n1 = psec[1], n2 = d->ncsite == 2 ? psec[2] : -1;
      for (int op = 0; op < d->nop; ++op) {
        int c = d->op_class[op];
        const Layout *L = get_layout(e, d->lay_L[c]), *R = get_layout(e, d->lay_Rf[c]);
        const Layout *Wi = get_layout(e, d->lay_Wi[c]);
        const Layout *Wj = d->ncsite == 2 ? get_layout(e, d->lay_Wj[c]) : nullptr;
        for (int sa = 0; sa < L->nsec[0]; ++sa) {
          int ls[3] = {sa, sl, sl};
          int32_t lb = L->pk->lookup[(size_t)L->ravel(ls)];
          if (lb < 0) continue;
          for (int sb = 0; sb < Wi->nsec[1]; ++sb) {
            int ws1[4] = {sa, sb, n1, n1};
            int32_t wib = Wi->pk->lookup[(size_t)Wi->ravel(ws1)];
            if (wib < 0) continue;
            int nsc = d->ncsite == 2 ? Wj->nsec[1] : 1;
            for (int sc = 0; sc < nsc; ++sc) {
              int32_t wjb = -1;
              int rs0 = sb;
              if (d->ncsite == 2) {
                int ws2[4] = {sb, sc, n2, n2};
                wjb = Wj->pk->lookup[(size_t)Wj->ravel(ws2)];
                if (wjb < 0) continue;
                rs0 = sc;
              }
              int rsec[3] = {rs0, sr, sr};
              int32_t rb = R->pk->lookup[(size_t)R->ravel(rsec)];
              if (rb < 0) continue;
              DiagTerm t;
              int64_t ld[3], rd[3], wid[4], wjd[4];
              L->block_dims(lb, ld);
              R->block_dims(rb, rd);
              Wi->block_dims(wib, wid);
              t.l_off = d->off_L[op] + L->pk->off[lb];
              t.l_sa = ld[1] * ld[2];
              t.l_sl = ld[2] + 1;
              t.r_off = d->off_R[op] + R->pk->off[rb];
              t.r_sc = rd[1] * rd[2];
              t.r_sr = rd[2] + 1;
              t.wi_off = d->off_Wi[op] + Wi->pk->off[wib];
              t.wi_sa = wid[1];
              t.wi_sb = 1;
              t.da = (int32_t)ld[0];
              t.db = (int32_t)wid[1];
              if (d->ncsite == 2) {
                Wj->block_dims(wjb, wjd);
                t.wj_off = d->off_Wj[op] + Wj->pk->off[wjb];
                t.wj_sb = wjd[1];
                t.wj_sc = 1;
                t.dc = (int32_t)wjd[1];
              } else {
                t.wj_off = 0;
                t.wj_sb = t.wj_sc = 0;
                t.dc = (int32_t)wid[1];
              }
              t.alpha = d->wts[op];
              t.ncsite = d->ncsite;
              P->dterms.push_back(t);
            }
          }
        }
      }
      db.nt = (int32_t)P->dterms.size() - db.t0;
      P->dblocks.push_back(db);
    }
    for (const auto &t : P->dterms) {
      P->max_ac = std::max<int64_t>(P->max_ac, (int64_t)t.da * t.dc);
    }
    for (const auto &b : P->dblocks) {
      int64_t mda = 0;
      for (int i = 0; i < b.nt; ++i) mda = std::max<int64_t>(mda, P->dterms[b.t0 + i].da);
      P->max_ar = std::max<int64_t>(P->max_ar, mda * b.dr);
    }
  }
  e->plans.push_back(std::move(P));
  drop_internal(e, c0, l0, {});
  *plan_id = (int)e->plans.size() - 1;
  return ZMPO_OK;
}

int zmpo_sigma_workspace(zmpo_engine *e, int plan_id, int64_t *bytes) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P || !bytes) return fail(ZMPO_E_ID, "workspace: unknown plan");
  *bytes = P->ws_elems * (int64_t)sizeof(double);
  return ZMPO_OK;
}

int zmpo_plan_stats(zmpo_engine *e, int plan_id, double *flops, int64_t *ntasks, int *nlaunch) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P) return fail(ZMPO_E_ID, "plan_stats: unknown plan");
  if (flops) *flops = P->flops;
  if (ntasks) *ntasks = P->ntasks;
  if (nlaunch) *nlaunch = (int)P->steps.size();
  return ZMPO_OK;
}

int zmpo_plan_kernel_count(zmpo_engine *e, int plan_id, int precision, int *count) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P) return fail(ZMPO_E_ID, "plan_kernel_count: unknown plan");
  if (!count) return fail(ZMPO_E_ARG, "plan_kernel_count: null output");
  int n = 0;
  for (auto &s : P->steps) {
    int rc = host_lists(s, precision);
    if (rc) return rc;
    if (precision == ZMPO_PREC_FP64) {
      n += s.nwork_fp64 > 0;
    } else {
      const bool s4 = precision == ZMPO_PREC_SPLIT;
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 4; ++c) n += (s4 ? s.nwork_tc4[a][c] : s.nwork_tc[a][c]) > 0;
      if (s4) {
        n += (s.nwork_tcb[0] > 0) + (s.nwork_tcb[1] > 0) + (s.nprep_a > 0) + (s.nprep_b > 0);
        for (int i = 0; i < 3; ++i) {
          n += s.nwork_ul[i] > 0;
          for (int c = 0; c < 3; ++c) n += s.nwork_um_cls[i][c] > 0;
        }
      }
    }
    n += s.red_elems > 0;
  }
  *count = n;
  return ZMPO_OK;
}

int zmpo_plan_mma_macs(zmpo_engine *e, int plan_id, int precision, int nmax, double *macs) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P) return fail(ZMPO_E_ID, "plan_mma_macs: unknown plan");
  if (!macs || nmax < 0) return fail(ZMPO_E_ARG, "plan_mma_macs: bad output");
  const int which = precision == ZMPO_PREC_FP64 ? 0 : (precision == ZMPO_PREC_SPLIT ? 1 : 2);
  for (int i = 0; i < nmax; ++i) macs[i] = 0.0;
  for (size_t i = 0; i < P->steps.size(); ++i) {
    int rc = host_lists(P->steps[i], precision);
    if (rc) return rc;
    if ((int)i < nmax) macs[i] = P->steps[i].mma_macs[which];
  }
  return ZMPO_OK;
}

int zmpo_sigma(zmpo_engine *e, int plan_id, const double *d_L, const double *d_R,
               const double *d_W, const double *d_x, double *d_y, void *d_workspace,
               int precision, void *stream) {
  Plan *P = get_plan(e, plan_id, 2);
  if (!P) return fail(ZMPO_E_ID, "sigma: unknown plan");
  if (P->ws_elems > 0 && !d_workspace) return fail(ZMPO_E_ARG, "sigma: workspace required");
  Bufs b{};
  b.p[0] = const_cast<double *>(d_L);
  b.p[1] = const_cast<double *>(d_R);
  b.p[2] = const_cast<double *>(d_W);
  b.p[3] = const_cast<double *>(d_x);
  b.p[4] = d_y;
  b.p[5] = (double *)d_workspace;
  // the kept records are reused when the caller asked for it and they are
  // this plan's, from its last split call on the same buffers, with no other
  // plan run on this workspace since
  const bool reuse = P->reuse_next && P->kept_ready && P->kept_ws == d_workspace && P->kept_L == d_L &&
                     P->kept_R == d_R && P->kept_W == d_W && e->ws_user[d_workspace] == plan_id;
  P->reuse_next = false;
  e->ws_user[d_workspace] = plan_id;
  if (precision == ZMPO_PREC_SPLIT) P->kept_ready = false;
  for (auto &s : P->steps) {
    int rc = run_step(s, b, precision, stream, !reuse);
    if (rc) return rc;
  }
  if (precision == ZMPO_PREC_SPLIT) {
    P->kept_ready = true;
    P->kept_ws = d_workspace;
    P->kept_L = d_L;
    P->kept_R = d_R;
    P->kept_W = d_W;
  }
  return ZMPO_OK;
}

int zmpo_sigma_reuse_kept(zmpo_engine *e, int plan_id, int reuse) {
  Plan *P = get_plan(e, plan_id, 2);
  if (!P) return fail(ZMPO_E_ID, "sigma_reuse_kept: unknown plan");
  P->reuse_next = reuse != 0;
  return ZMPO_OK;
}

int zmpo_hdiag(zmpo_engine *e, int plan_id, const double *d_L, const double *d_R,
               const double *d_W, double *d_diag, void *stream) {
  Plan *P = get_plan(e, plan_id, 2);
  if (!P) return fail(ZMPO_E_ID, "hdiag: unknown plan");
  if (!P->diag_uploaded) {
    if (!P->dblocks.empty()) {
      CUDA_TRY(cudaMalloc((void **)&P->d_dblocks, P->dblocks.size() * sizeof(DiagBlock)));
      CUDA_TRY(cudaMemcpy(P->d_dblocks, P->dblocks.data(), P->dblocks.size() * sizeof(DiagBlock),
                          cudaMemcpyHostToDevice));
    }
    if (!P->dterms.empty()) {
      CUDA_TRY(cudaMalloc((void **)&P->d_dterms, P->dterms.size() * sizeof(DiagTerm)));
      CUDA_TRY(cudaMemcpy(P->d_dterms, P->dterms.data(), P->dterms.size() * sizeof(DiagTerm),
                          cudaMemcpyHostToDevice));
    }
    std::vector<DiagTerm>().swap(P->dterms);
    P->diag_uploaded = true;
  }
  Bufs b{};
  b.p[0] = const_cast<double *>(d_L);
  b.p[1] = const_cast<double *>(d_R);
  b.p[2] = const_cast<double *>(d_W);
  return launch_hdiag(P->d_dblocks, (int64_t)P->dblocks.size(), P->d_dterms, b, d_diag,
                      (int)P->max_ac, (int)P->max_ar, stream);
}

int zmpo_renorm_plan(zmpo_engine *e, const zmpo_renorm_desc *d, int *plan_id) {
  if (!e || !d || !plan_id || d->nop < 0 || d->nclass < 1 || (d->status != 0 && d->status != 1))
    return fail(ZMPO_E_ARG, "renorm_plan: bad descriptor");
  const size_t c0 = e->contractions.size(), l0 = e->layouts.size();
  // reference chains (mpo_dmrg_kernelQt.py:665-667 for 'L', 727-729 for 'R')
  static const int La1[1] = {0}, Lb1[1] = {1};
  static const int La2[2] = {0, 2}, Lb2[2] = {2, 0};
  static const int La3[2] = {1, 3}, Lb3[2] = {1, 0};
  static const int Ra1[1] = {2}, Rb1[1] = {1};
  static const int Ra2[2] = {1, 2}, Rb2[2] = {2, 1};
  static const int Ra3[2] = {1, 3}, Rb3[2] = {1, 2};
  struct Ch {
    bool built = false;
    int c1 = -1, c2 = -1, c3 = -1, l1 = -1, l2 = -1, l3 = -1;
  };
  std::vector<Ch> ch(d->nclass);
  for (int op = 0; op < d->nop; ++op) {
    int c = d->op_class[op];
    if (c < 0 || c >= d->nclass) return fail(ZMPO_E_ARG, "renorm_plan: bad class");
    if (ch[c].built) continue;
    ch[c].built = true;
    int rc;
    if (d->status == 0) {
      rc = build_contraction(e, d->lay_site, d->lay_env[c], 1, La1, Lb1, &ch[c].l1, &ch[c].c1);
      if (rc) return rc;
      rc = build_contraction(e, d->lay_W[c], ch[c].l1, 2, La2, Lb2, &ch[c].l2, &ch[c].c2);
      if (rc) return rc;
      rc = build_contraction(e, ch[c].l2, d->lay_site, 2, La3, Lb3, &ch[c].l3, &ch[c].c3);
    } else {
      rc = build_contraction(e, d->lay_site, d->lay_env[c], 1, Ra1, Rb1, &ch[c].l1, &ch[c].c1);
      if (rc) return rc;
      rc = build_contraction(e, d->lay_W[c], ch[c].l1, 2, Ra2, Rb2, &ch[c].l2, &ch[c].c2);
      if (rc) return rc;
      rc = build_contraction(e, ch[c].l2, d->lay_site, 2, Ra3, Rb3, &ch[c].l3, &ch[c].c3);
    }
    if (rc) return rc;
  }
  auto P = std::make_unique<Plan>();
  P->kind = 3;
  P->status = d->status;
  P->out_lay.assign(d->nclass, -1);
  P->out_off.assign(d->nop, -1);
  for (int c = 0; c < d->nclass; ++c)
    if (ch[c].built && get_layout(e, ch[c].l3)->pk->size > 0) P->out_lay[c] = ch[c].l3;
  int64_t tot = 0, ws = 0;
  std::vector<int64_t> w1(d->nop, 0), w2(d->nop, 0);
  for (int op = 0; op < d->nop; ++op) {
    int c = d->op_class[op];
    if (P->out_lay[c] < 0) continue;
    P->out_off[op] = tot;
    tot += get_layout(e, ch[c].l3)->pk->size;
    w1[op] = ws;
    ws += get_layout(e, ch[c].l1)->pk->size;
    ws = (ws + 31) & ~int64_t(31);
    w2[op] = ws;
    ws += get_layout(e, ch[c].l2)->pk->size;
    ws = (ws + 31) & ~int64_t(31);
  }
  P->out_total = tot;
  P->ws_elems = ws;
  // structurally zero blocks of T1 and T2 (as in the sigma plan): step 1
  // reads T1 as B, step 2 reads T2 as A
  std::vector<std::array<std::vector<char>, 2>> alive(d->nclass);
  for (int c = 0; c < d->nclass; ++c) {
    if (!ch[c].built) continue;
    const Contraction *C1 = e->contractions[ch[c].c1].get(), *C2 = e->contractions[ch[c].c2].get();
    alive[c][0].assign(C1->task_start.size() - 1, 0);
    for (size_t ob = 0; ob + 1 < C1->task_start.size(); ++ob)
      alive[c][0][ob] = C1->task_start[ob + 1] > C1->task_start[ob];
    alive[c][1].assign(C2->task_start.size() - 1, 0);
    for (size_t ob = 0; ob + 1 < C2->task_start.size(); ++ob)
      for (int64_t t = C2->task_start[ob]; t < C2->task_start[ob + 1]; ++t)
        if (alive[c][0][C2->tasks[t].bb]) {
          alive[c][1][ob] = 1;
          break;
        }
  }
  // the reference's work: every task of the three contractions per term
  for (int op = 0; op < d->nop; ++op) {
    const int c = d->op_class[op];
    if (P->out_lay[c] < 0) continue;
    for (int ci : {ch[c].c1, ch[c].c2, ch[c].c3}) P->flops += contraction_flops(e, e->contractions[ci].get());
  }
  // buffers: 0 env, 2 W, 3 site, 4 out, 5 workspace (the works of each step
  // are made on that step's thread)
  auto make_works = [&](int s, std::vector<OutWork> &works) {
    for (int op = 0; op < d->nop; ++op) {
      int c = d->op_class[op];
      if (P->out_lay[c] < 0) continue;
      int ci = s == 0 ? ch[c].c1 : (s == 1 ? ch[c].c2 : ch[c].c3);
      const Contraction *C = e->contractions[ci].get();
      const Layout *A = get_layout(e, C->lay_a), *B = get_layout(e, C->lay_b),
                   *O = get_layout(e, C->lay_out);
      int abuf, bbuf, cbuf;
      int64_t abase, bbase, cbase;
      if (s == 0) {
        abuf = 3; abase = 0; bbuf = 0; bbase = d->off_env[op]; cbuf = 5; cbase = w1[op];
      } else if (s == 1) {
        abuf = 2; abase = d->off_W[op]; bbuf = 5; bbase = w1[op]; cbuf = 5; cbase = w2[op];
      } else {
        abuf = 5; abase = w2[op]; bbuf = 3; bbase = 0; cbuf = 4; cbase = P->out_off[op];
      }
      for (size_t ob = 0; ob < O->pk->flat.size(); ++ob) {
        if (s < 2 && !alive[c][s][ob]) continue;  // zero intermediate block
        OutWork w;
        w.lo = O;
        w.ob = (int32_t)ob;
        w.c_base = cbase;
        w.cbuf = cbuf;
        for (int64_t t = C->task_start[ob]; t < C->task_start[ob + 1]; ++t) {
          const Task &tk = C->tasks[t];
          if ((s == 1 && !alive[c][0][tk.bb]) || (s == 2 && !alive[c][1][tk.ab])) continue;
          w.tasks.push_back({C, A, B, O, tk.ab, tk.bb, abase, bbase, abuf, bbuf, 1.0});
        }
        works.push_back(std::move(w));
      }
    }
  };
  {
    int rc = build_steps_parallel(P.get(), 3, make_works, 0);
    if (rc) return rc;
    for (auto &st : P->steps) {
      P->exec_flops += st.flops;
      P->ntasks += st.ntasks;
    }
  }
  e->plans.push_back(std::move(P));
  {
    std::vector<int> keep;  // the output layouts go back to the caller
    for (int c = 0; c < d->nclass; ++c)
      if (ch[c].built) keep.push_back(ch[c].l3);
    drop_internal(e, c0, l0, keep);
  }
  *plan_id = (int)e->plans.size() - 1;
  return ZMPO_OK;
}

int zmpo_renorm_outputs(zmpo_engine *e, int plan_id, int *lay_out, int64_t *off_out, int64_t *total) {
  Plan *P = get_plan(e, plan_id, 3);
  if (!P) return fail(ZMPO_E_ID, "renorm_outputs: unknown plan");
  if (lay_out)
    for (size_t c = 0; c < P->out_lay.size(); ++c) lay_out[c] = P->out_lay[c];
  if (off_out)
    for (size_t i = 0; i < P->out_off.size(); ++i) off_out[i] = P->out_off[i];
  if (total) *total = P->out_total;
  return ZMPO_OK;
}

int zmpo_renorm_workspace(zmpo_engine *e, int plan_id, int64_t *bytes) {
  return zmpo_sigma_workspace(e, plan_id, bytes);
}

int zmpo_renorm(zmpo_engine *e, int plan_id, const double *d_env, const double *d_W,
                const double *d_site, double *d_out, void *d_workspace, int precision,
                void *stream) {
  Plan *P = get_plan(e, plan_id, 3);
  if (!P) return fail(ZMPO_E_ID, "renorm: unknown plan");
  if (P->ws_elems > 0 && !d_workspace) return fail(ZMPO_E_ARG, "renorm: workspace required");
  Bufs b{};
  b.p[0] = const_cast<double *>(d_env);
  b.p[2] = const_cast<double *>(d_W);
  b.p[3] = const_cast<double *>(d_site);
  b.p[4] = d_out;
  b.p[5] = (double *)d_workspace;
  for (auto &s : P->steps) {
    int rc = run_step(s, b, precision, stream);
    if (rc) return rc;
  }
  return ZMPO_OK;
}

int zmpo_profile(zmpo_engine *e, int on) {
  if (!e) return fail(ZMPO_E_ARG, "profile: null engine");
  g_profile = on != 0;
  return ZMPO_OK;
}

int zmpo_plan_launch_times(zmpo_engine *e, int plan_id, int nmax, double *ms_avg, double *alg_bytes,
                           int64_t *ncalls) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P) return fail(ZMPO_E_ID, "launch_times: unknown plan");
  for (int s = 0; s < (int)P->steps.size() && s < nmax; ++s) {
    Step &st = P->steps[s];
    profile_collect(st);
    if (ms_avg) ms_avg[s] = st.ncalls ? st.ms_total / (double)st.ncalls : 0.0;
    if (alg_bytes) alg_bytes[s] = st.alg_bytes;
    if (ncalls) ncalls[s] = st.ncalls;
    st.ms_total = 0.0;
    st.ncalls = 0;
  }
  return ZMPO_OK;
}

int zmpo_plan_groups(zmpo_engine *e, int plan_id, int step, int64_t *ngroups, int32_t *M,
                     int32_t *N, int32_t *nseg, int64_t *ktot) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P || step < 0 || step >= (int)P->steps.size() || !ngroups)
    return fail(ZMPO_E_ID, "plan_groups: unknown plan or step");
  const Step &st = P->steps[step];
  *ngroups = (int64_t)st.groups.size();
  if (!M) return ZMPO_OK;
  for (size_t g = 0; g < st.groups.size(); ++g) {
    const Group &G = st.groups[g];
    M[g] = G.M;
    N[g] = G.N;
    if (nseg) nseg[g] = G.nseg;
    if (ktot) {
      const int64_t k = st.gk[g];
      ktot[g] = k;
    }
  }
  return ZMPO_OK;
}

int zmpo_plan_step_tasks(zmpo_engine *e, int plan_id, int step, int64_t *counts, void *groups, void *segs,
                         void *cblocks, void *segb, void *reds) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P || step < 0 || step >= (int)P->steps.size() || !counts)
    return fail(ZMPO_E_ID, "plan_step_tasks: unknown plan or step");
  const Step &st = P->steps[step];
  if (st.up_common) return fail(ZMPO_E_ARG, "plan_step_tasks: task lists already moved to the device");
  counts[0] = (int64_t)st.groups.size();
  counts[1] = (int64_t)st.segs.size();
  counts[2] = (int64_t)st.cblocks.size();
  counts[3] = (int64_t)st.segb.size();
  counts[4] = (int64_t)st.reds.size();
  if (groups) memcpy(groups, st.groups.data(), st.groups.size() * sizeof(Group));
  if (segs) memcpy(segs, st.segs.data(), st.segs.size() * sizeof(Seg));
  if (cblocks) memcpy(cblocks, st.cblocks.data(), st.cblocks.size() * sizeof(ColBlock));
  if (segb) memcpy(segb, st.segb.data(), st.segb.size() * sizeof(SegB));
  if (reds) memcpy(reds, st.reds.data(), st.reds.size() * sizeof(Reduction));
  return ZMPO_OK;
}

int zmpo_device_status(zmpo_engine *e, int *code, int reset) {
  if (!e || !code) return fail(ZMPO_E_ARG, "device_status: null argument");
  return umma_device_status(code, reset);
}

int zmpo_plan_destroy(zmpo_engine *e, int plan_id) {
  Plan *P = get_plan(e, plan_id, 0);
  if (!P) return fail(ZMPO_E_ID, "plan_destroy: unknown plan");
  for (auto &s : P->steps) release_step(s);
  cudaFree(P->d_dblocks);
  cudaFree(P->d_dterms);
  e->plans[plan_id].reset();
  return ZMPO_OK;
}

}  // extern "C"
