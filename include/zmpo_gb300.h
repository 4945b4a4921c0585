/*
 * zmpo_gb300.h -- C ABI of the GB300 engine for the DMRG sigma-vector and
 * environment-renormalisation path of zhendongli2008/zmpo_dmrg.
 *
 * Conventions
 *   - Every entry point returns int: 0 = ok, negative = error kind
 *     (ZMPO_E_*); zmpo_last_error() gives the message of the last failure
 *     on the calling thread.  Nothing calls exit().
 *   - Pointers named `d_*` are CUDA device pointers (e.g. from torch
 *     tensors); `stream` is a cudaStream_t passed as void*.
 *   - Block-sparse tensors use the reference's packing: allowed blocks in
 *     row-major order of their sector multi-index, each block row-major
 *     (source/qtensor/qtensor.py:272-346).  A device array of a tensor is
 *     therefore bit-for-bit the reference's qtensor `value` array.
 *   - Calls on one engine are not re-entrant; one host thread drives one
 *     engine and its stream.
 */
#ifndef ZMPO_GB300_H
#define ZMPO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZMPO_OK 0
#define ZMPO_E_ARG (-1)      /* invalid argument / shape mismatch         */
#define ZMPO_E_CUDA (-2)     /* CUDA runtime error                         */
#define ZMPO_E_SYM (-3)      /* quantum numbers of contracted legs differ  */
#define ZMPO_E_ID (-4)       /* unknown engine object id                   */
#define ZMPO_E_NOMEM (-5)    /* device allocation failed                   */
#define ZMPO_E_SIZE (-6)     /* request exceeds a documented limit         */

/* Precision of the block contractions (argument `precision`). */
#define ZMPO_PREC_FP64 0     /* FP64 FMA on the CUDA cores                 */
#define ZMPO_PREC_SPLIT 1    /* BF16 tensor cores, 4 exact digit slices;
                                groups whose whole K fits one exact pass
                                (K <= 256) run on tcgen05 with exponents
                                per row / column over that K              */
#define ZMPO_PREC_EMU64 2    /* BF16 tensor cores, 7 exact digit slices    */

typedef struct zmpo_engine zmpo_engine;

/* Message of the last failed call on this thread (always NUL-terminated). */
int zmpo_last_error(char *buf, size_t len);
/* ABI version of this library. */
int zmpo_version(void);

/* Drop-in for the reference's native block rule `symAllowed`
 * (ctypes/qsym.c:5, bound by source/qtensor/qtensor_util.py:79-84): same
 * arguments.  allowed[blk] = sum_k |sum_{status=0} q - sum_{status=1} q| < 1e-10
 * over the row-major enumeration of sector multi-indices.  Ranks 1..8.
 * (The reference's rank-8 loop bound reads ndims[6] for the last leg,
 * qsym.c:436; this implementation uses ndims[7].) */
int symAllowed(int rank, int nqnum, int *ndims, int *status, int *allowed,
               double *a0, double *a1, double *a2, double *a3,
               double *a4, double *a5, double *a6, double *a7);

/* Engine: owns block layouts, contraction plans and their device task
 * lists.  `device` is the CUDA ordinal the engine's allocations use. */
int zmpo_engine_create(zmpo_engine **out, int device);
int zmpo_engine_destroy(zmpo_engine *e);

/* Block layout of a qtensor (restates qtensor.fromQsyms, qtensor.py:272).
 *   nsec[rank]        number of sectors per leg
 *   qsyms[...]        concatenated per leg, nsec[leg] x nqnum, float64
 *   dims[...]         concatenated per leg, nsec[leg] sector dimensions
 *   status[rank]      0/1 leg direction (qtensor.status)                 */
int zmpo_layout_create(zmpo_engine *e, int rank, int nqnum, const int *nsec,
                       const double *qsyms, const int64_t *dims,
                       const int *status, int *layout_id);
/* Same packing as `src`, new quantum numbers / status for symbolic
 * matching (the reference's in-place `rop.qsyms = [...]` flips,
 * mpo_dmrg_kernelQt.py:301 and 737-741). */
int zmpo_layout_derive(zmpo_engine *e, int src, const double *qsyms,
                       const int *status, int *layout_id);
int zmpo_layout_info(zmpo_engine *e, int layout_id, int64_t *size_allowed,
                     int64_t *nblocks, int *rank);
/* flat[i] = row-major sector index of allowed block i, off[i] its offset. */
int zmpo_layout_blocks(zmpo_engine *e, int layout_id, int64_t *flat,
                       int64_t *off);

/* Block-sparse tensordot (qtensor.tensordotSYM + tensordotCAL,
 * qtensor.py:563-659): plan = output layout + task list; exec computes
 * d_out = tensordot(d_a, d_b, axes) in the chosen precision. */
int zmpo_contract_plan(zmpo_engine *e, int lay_a, int lay_b, int naxes,
                       const int *axes_a, const int *axes_b,
                       int *lay_out, int *plan_id);
int zmpo_contract_exec(zmpo_engine *e, int plan_id, const double *d_a,
                       const double *d_b, double *d_out, int precision,
                       void *stream);

/* Allocation-free variant of zmpo_contract_exec (no counterpart in the
 * reference).  For callers that cannot allocate device memory when they run
 * a contraction -- code recorded into a CUDA graph by stream capture, where
 * cudaMalloc is not allowed, or a host framework that hands out all device
 * memory itself -- the split-K partial sums go to a fixed 8 MiB array
 * (1048576 float64) compiled into this library instead of memory the plan
 * allocates.  Every GPU that loads the library holds that array until the
 * process exits.  The call allocates nothing: the plan must have run once
 * through zmpo_contract_exec during set-up, with the precision of the later
 * calls (that call builds the plan's device task lists of that precision
 * and, for the split precision, the plan's own buffer of prepared digit
 * planes), and a plan that
 * needs more scratch than the array holds is rejected with ZMPO_E_SIZE.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress, with that device current); make that
 * first call before any stream capture.  All calls share the one array and it
 * keeps the last call's contents (every partial is overwritten before it is
 * read, nothing needs clearing); calls whose launches overlap on the GPU race
 * on it, so order them on one stream. */
int zmpo_contract_exec_noalloc(zmpo_engine *e, int plan_id, const double *d_a,
                               const double *d_b, double *d_out, int precision,
                               void *stream);

/* Sigma vector H.psi over all operator terms p of one dot
 * (replaces mpo_dmrg_kernelQt.HVecQt, mpo_dmrg_kernelQt.py:153-319, and the
 * Reduce over ranks, tools/pdvdson.py:75).  Operators of one class share
 * layouts (qtensor_opers.case, qtensor_opers.py:72-90). */
typedef struct {
  int ncsite;            /* 1 or 2 sites in the dot                      */
  int nop;               /* number of operator terms p                   */
  int nclass;            /* number of layout classes                     */
  const int *op_class;   /* [nop] class of each term                     */
  const int *lay_L;      /* [nclass] left environment layouts [a,bra,ket] */
  const int *lay_Wi;     /* [nclass] MPO site isite  [a,b,n',n]           */
  const int *lay_Wj;     /* [nclass] MPO site isite+1 (ncsite == 2)       */
  const int *lay_Rf;     /* [nclass] right environments with the reference's
                            quantum-number flip [-q0, qkey-q1, qkey-q2]  */
  int lay_psi;           /* wavefunction layout (dmrg.qtmp)              */
  const int64_t *off_L;  /* [nop] element offset of L_p in d_L           */
  const int64_t *off_R;  /* [nop] element offset of R_p in d_R           */
  const int64_t *off_Wi; /* [nop] offset of W_p(isite) in d_W            */
  const int64_t *off_Wj; /* [nop] offset of W_p(isite+1) in d_W          */
  const double *wts;     /* [nop] hpwts                                  */
} zmpo_sigma_desc;

int zmpo_sigma_plan(zmpo_engine *e, const zmpo_sigma_desc *desc, int *plan_id);
/* Bytes of device workspace zmpo_sigma needs for this plan. */
int zmpo_sigma_workspace(zmpo_engine *e, int plan_id, int64_t *bytes);
/* Algorithmic FP64 work of one sigma (sum of 2*m*n*k over the reference's
 * task lists), and the number of tasks / launches. */
int zmpo_plan_stats(zmpo_engine *e, int plan_id, double *flops,
                    int64_t *ntasks, int *nlaunch);
/* Host copy of one step's task records before the plan's first execution
 * (afterwards they live on the device): counts[5] = groups, segments, column
 * blocks, per-(segment, column block) B parts, split-K sums; each output
 * pointer may be NULL and receives the records in the engine's internal
 * layout (csrc/engine.h: Group 56 bytes, Seg 64, ColBlock 32, SegB 24,
 * Reduction 56).  Groups longer than the split-K length appear as their
 * parts, which write scratch buffer 6; a split-K sum adds its parts in order
 * into its destination.  For inspection and tests; no reference
 * counterpart. */
int zmpo_plan_step_tasks(zmpo_engine *e, int plan_id, int step, int64_t *counts,
                         void *groups, void *segs, void *cblocks, void *segb, void *reds);
/* Number of kernel launches one execution of the plan issues at this
 * precision (grouped GEMM launches per tile shape plus split-K sums).  No
 * reference counterpart: it reports what the engine will launch. */
int zmpo_plan_kernel_count(zmpo_engine *e, int plan_id, int precision, int *count);
/* Multiply-adds the tiles of each step issue at this precision (tile padding
 * included, a group's K rounded up to 16), macs[step] for step < nmax; the
 * tensor-core paths issue 10 (split) or 28 (emu64) digit products per
 * multiply-add.  No reference counterpart: the roofline of the executed work. */
int zmpo_plan_mma_macs(zmpo_engine *e, int plan_id, int precision, int nmax, double *macs);
/* y = H x (ndim0 = size of lay_psi).  d_x, d_y device vectors. */
int zmpo_sigma(zmpo_engine *e, int plan_id, const double *d_L,
               const double *d_R, const double *d_W, const double *d_x,
               double *d_y, void *d_workspace, int precision, void *stream);
/* Lets the next zmpo_sigma call of this plan (split precision) skip
 * re-cutting the tensor-core digit planes of the operands that stay fixed
 * during a Davidson solve (the environments L, R and the MPO W): they are
 * reused from the plan's previous split-precision call when that call had
 * the same d_L, d_R, d_W and d_workspace and no other sigma plan ran on
 * d_workspace since; otherwise the call cuts them as usual.  The caller
 * guarantees that the contents of d_L, d_R and d_W did not change since that
 * call.  Applies to the next call only.  No reference counterpart (the
 * reference has no prepared operands). */
int zmpo_sigma_reuse_kept(zmpo_engine *e, int plan_id, int reuse);
/* Davidson preconditioner diag(H) in the packed psi order (replaces
 * HDiagQt, mpo_dmrg_kernelQt.py:30-127). */
int zmpo_hdiag(zmpo_engine *e, int plan_id, const double *d_L,
               const double *d_R, const double *d_W, double *d_diag,
               void *stream);

/* Environment renormalisation for all p (replaces renormQt_H00,
 * mpo_dmrg_kernelQt.py:633-768).  status 0 = 'L' (new left environment
 * from site [l,n,r] status [F,F,T]); 1 = 'R' (site status [T,F,F]).
 * lay_W holds, for 'R', the reference's flipped MPO layout. */
typedef struct {
  int status;
  int nop;
  int nclass;
  const int *op_class;
  const int *lay_env;    /* [nclass] input environment layouts          */
  const int *lay_W;      /* [nclass] MPO layouts                         */
  int lay_site;          /* renormalised site tensor                    */
  const int64_t *off_env;/* [nop] */
  const int64_t *off_W;  /* [nop] */
} zmpo_renorm_desc;

int zmpo_renorm_plan(zmpo_engine *e, const zmpo_renorm_desc *desc,
                     int *plan_id);
/* Output layouts per class (-1 when the class has no allowed block),
 * output offset per op (-1 when empty) and total output elements. */
int zmpo_renorm_outputs(zmpo_engine *e, int plan_id, int *lay_out,
                        int64_t *off_out, int64_t *total);
int zmpo_renorm_workspace(zmpo_engine *e, int plan_id, int64_t *bytes);
int zmpo_renorm(zmpo_engine *e, int plan_id, const double *d_env,
                const double *d_W, const double *d_site, double *d_out,
                void *d_workspace, int precision, void *stream);

/* Tracing: when on, every launch of a plan is bracketed by CUDA events on
 * its stream; zmpo_plan_launch_times returns, per launch of the plan, the
 * average device time (ms) since the last read, the algorithmic bytes of
 * that launch (each operand tensor read once, each output written once) and
 * the number of timed calls, then resets the counters. */
int zmpo_profile(zmpo_engine *e, int on);
int zmpo_plan_launch_times(zmpo_engine *e, int plan_id, int nmax, double *ms_avg,
                           double *alg_bytes, int64_t *ncalls);

/* Introspection of a launch of a plan: number of output groups (groups
 * longer than the split-K length as their parts) and, when M is non-NULL,
 * per group its rows, columns, number of block products and summed K. */
int zmpo_plan_groups(zmpo_engine *e, int plan_id, int step, int64_t *ngroups,
                     int32_t *M, int32_t *N, int32_t *nseg, int64_t *ktot);

/* Error word of the device kernels (no reference counterpart).  The
 * tensor-core kernels bound every wait between their warps in time; a wait
 * that runs out records a code here (100 + the wait's site) and the kernel
 * returns early without hanging the GPU, leaving its output incomplete.
 * *code = 0 when no kernel has reported an error; reset != 0 clears it.
 * Synchronises with the device. */
int zmpo_device_status(zmpo_engine *e, int *code, int reset);

/* Release a contraction / sigma / renorm plan. */
int zmpo_plan_destroy(zmpo_engine *e, int plan_id);

#ifdef __cplusplus
}
#endif
#endif /* ZMPO_GB300_H */
