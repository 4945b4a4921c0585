"""Benchmark of the DMRG sigma-vector hot path on one GB300.

One step = one two-site H.psi over every operator term H_p (48 terms) at the
middle dot of K=24 spatial orbitals, 24 electrons, Sz=0, bond dimension
D=512, (N,Sz) block-sparse, in the split-precision tensor-core path.  Inputs
are seeded synthetic integrals (the configuration's generator) and a seeded
random block-sparse MPS with realistic sector sizes; the environments of all
terms are built on the GPU by the engine's renormalisation.

Printed (one JSON line, rank 0): ``value`` = F_ref / t with F_ref the
reference's algorithmic FLOPs of one H.psi (sum of 2mnk over its block task
lists) and t the device time per step with inputs resident in HBM; ``e2e`` =
the same through the C ABI with host input/output vectors (H2D + D2H inside
the timed region); ``roofline`` for the dominant launch; ``cpu_baseline`` =
the oracle (the reference's NumPy kernel restated) on a bounded sample of the
same workload; ``parity_vs_oracle`` = the engine's sigma against the oracle's
over that sample.  ``--impl reference`` times only the oracle, on a dot built
on the host without any engine code.
"""
import argparse
import collections
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOAD = dict(K=24, nelec=24, D=512, isite=11, seed=2024)
SMALL = dict(K=12, nelec=12, D=128, isite=5, seed=2024)
MEDIUM = dict(K=16, nelec=16, D=256, isite=7, seed=2024)
# the large batched configuration (hopping 0.7), run with a workspace budget
LARGE = dict(K=36, nelec=36, D=1024, isite=17, seed=2024, hop=0.7)
LARGE_WORKSPACE = 64e9
# the spin-projected configuration: singlet projection with 8 Gauss-Legendre
# points (320 terms [p, g]), H.psi with the N-only relabelling
SPCFG = dict(K=20, nelec=20, D=512, isite=9, seed=2024, npts=8, sval=0.0)
METRIC = "sweep s & sigma-vec TFLOP/s, split-BF16 vs FP64 on 1 GB300 at ΔE≤1e-8 Eh"


def peaks():
    """HBM GB/s and bf16 TFLOP/s: the measured copies (the sustained GEMM rate:
    the kernels are timed inside a step of tens of ms), else the fallback."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p.get("bf16_tflops_sustained", p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1700.0, "fallback"


class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        # raw samples; the summary goes into the JSON line
        self.path = os.environ.get("ZMPO_CLOCKS_CSV",
                                   os.path.join(tempfile.gettempdir(), "zmpo_clocks_bench.csv"))

    @staticmethod
    def device_id():
        """nvidia-smi ignores CUDA_VISIBLE_DEVICES: select the GPU this process
        runs on by its UUID (read-only query)."""
        try:
            import torch
            u = str(torch.cuda.get_device_properties(torch.cuda.current_device()).uuid)
            return u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            return "0"

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                       "-i", self.device_id(), "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(numpy.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_problem(with_oracle=False, small=False, medium=False, large=False, sp=False):
    from tests.problems import random_problem
    t0 = time.perf_counter()
    cfg = SMALL if small else (MEDIUM if medium else (LARGE if large else (SPCFG if sp else WORKLOAD)))
    P = random_problem(device=True, with_oracle=with_oracle, **cfg)
    return P, time.perf_counter() - t0


def oracle_rate(m, terms_per_step, nsteps, isite, x):
    """The oracle's HVecQt (the reference's NumPy algorithm, all host cores
    through BLAS) over rotating subsets of ``terms_per_step`` operator terms,
    ``nsteps`` times: step i takes terms i*s .. i*s+s-1 (mod the term count),
    so enough steps visit every term.  Returns per-step (F_ref, seconds) and
    the set of terms visited; F_ref counts 2mnk over the reference's task
    lists of the terms evaluated."""
    from oracle import kernel as ok, qtensor as oq
    fL, fR = m.flst[0][0:2]
    allops = list(range(m.fhop['nops']))
    out, seen = [], set()
    for i in range(nsteps):
        chosen = [allops[(i * terms_per_step + j) % len(allops)] for j in range(terms_per_step)]
        seen.update(chosen)
        sub = _oracle_view(m, chosen)
        oq.reset_flops()
        t0 = time.perf_counter()
        ok.HVecQt(x, [sub, isite, 2, sub.flst, 'L', True], sub.qtmp.size_allowed, None)
        dt = time.perf_counter() - t0
        out.append((float(oq.FLOPS["count"]), dt))
    return out, seen


def _oracle_view(m, chosen):
    """Oracle driver restricted to the terms ``chosen`` (same environments,
    MPO sites and packed wavefunction layout)."""
    import copy
    sub = copy.copy(m)
    fL, fR = m.flst[0][0:2]
    sub.opers = [m.opers[i] for i in chosen]
    sub.hpwts = numpy.asarray([m.hpwts[i] for i in chosen])
    sub.fhop = {'nops': len(chosen)}
    fLo, fRo = {}, {}
    for k, i in enumerate(chosen):
        fLo['opers%d' % k] = fL['opers%d' % i]
        fRo['opers%d' % k] = fR['opers%d' % i]
        for st in (m._dot_isite, m._dot_isite + 1):
            sub.fhop['site%d/op%d' % (st, k)] = m.fhop['site%d/op%d' % (st, i)]
    sub.flst = [[fLo, fRo]]
    sub._hvec_templates = None
    return sub


def reference_dot(cfg):
    """The dot of ``cfg`` for the reference arm, built on the host by the
    oracle alone (no engine code): the same seeded integrals and random MPS as
    the engine arm, environments of every operator term renormalised site by
    site with the oracle's renormQt_H00 (the reference's algorithm), so both
    arms contract the same environments (to FP64 rounding)."""
    from tests.problems import random_problem
    P = random_problem(device=False, with_oracle=True, **cfg)
    m = P.o
    m._dot_isite = P.isite
    return m


def cpu_leg(P, cfg, budget_terms=12):
    """Engine arm, rank 0: (1) ``cpu_baseline`` = the oracle's HVecQt on the
    host cores over a bounded sample of the dot's terms (``budget_terms``, two
    per operator class), fed the environments the engine built; (2)
    ``parity_vs_oracle`` = the engine's sigma over the same terms against that
    oracle sigma, FP64 / split / 56-bit emulation, relative norm error."""
    from tests.problems import class_covering_terms, oracle_subset_driver, product_sigma_subset
    from oracle import kernel as ok, qtensor as oq
    terms, classes = class_covering_terms(P, 2)
    terms = terms[:budget_terms]
    m = oracle_subset_driver(P, terms)
    x = numpy.random.default_rng(6).standard_normal(P.ndim0)
    oq.reset_flops()
    t0 = time.perf_counter()
    ref = ok.HVecQt(x, [m, P.isite, 2, m.flst, 'L', True], m.qtmp.size_allowed, None)
    dt = time.perf_counter() - t0
    fl = float(oq.FLOPS["count"])
    base = {"value": fl / dt / 1e12, "unit": "TFLOP/s", "cores": cpu_threads(), "kind": "port",
            "sample": "oracle HVecQt over %d of the %d operator terms (two per operator class, %d classes), "
                      "environments copied from the engine's dot, %.1f s, F_ref/t" %
                      (len(terms), P.p.nops, len(classes), dt),
            "mpi": MPI_NOTE}
    par = {"terms": terms, "classes": classes}
    for prec in ("fp64", "split", "emu64"):
        y = product_sigma_subset(P, terms, x, prec)
        par[prec] = float(numpy.linalg.norm(y - ref) / numpy.linalg.norm(ref))
    par["tolerance"] = {"fp64": 1e-10, "split": 1e-8, "emu64": 1e-10}
    return base, par


def workload_config(cfg, ndim0, nterms):
    """``config`` of both arms' JSON lines (identical for the same workload)."""
    w = "two-site H.psi, K=%d N=%d Sz=0 D=%d, %d terms, (N,Sz) blocks" % (cfg["K"], cfg["nelec"], cfg["D"], nterms)
    if cfg.get("npts"):
        w += ", spin-projected S=0 with %d quadrature points (N-only terms)" % cfg["npts"]
    return {"workload": w, "ndim0": int(ndim0), "terms": int(nterms), "middle_dot": int(cfg["isite"])}


MPI_NOTE = ("the reference's MPI operator partition (mpirun over mpi4py) is unavailable on this box: "
            "mpi4py and an MPI launcher are absent; one process with multithreaded BLAS on every host core")


def gradient_metrics(K=16, nelec=16, D=256, seed=2024):
    """Energy gradient (dE/dh1e, dE/d(pq|rs)) at a seeded random left-canonical
    MPS of K=16, 16 electrons, D=256 (the adjoint configuration's sizes; the
    cost does not depend on convergence): seconds for the site gradients
    (engine contractions) and for the chain rule, and a central-difference
    check (step 1e-5) of the fixed-MPS energy along a random symmetric direction."""
    import torch
    from tests.problems import bond_structure, random_left_site, QPHYS
    from zmpo_dmrg_gb300 import integrals as I, adjoint
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.qtensor import qtensor
    rng = numpy.random.default_rng(seed)
    h, eri, _ = I.synthetic(K, seed)
    m = mpo_dmrg(seed=1)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.partition()
    m.loadInts(I.spin_orbital(h, eri))
    m.dumpMPO()
    qnuml, _ = bond_structure(K, nelec, 0.0, D, rng)
    qnuml[K] = numpy.array([[float(nelec), 0.0]])   # one state at the right end
    fmps = {'nsite': K}
    for i in range(K):
        t = qtensor([False, False, True])
        t.fromDenseTensor(random_left_site(qnuml[i], qnuml[i + 1], rng), [qnuml[i], QPHYS, qnuml[i + 1]])
        fmps['site%d' % i] = t
    for i in range(K + 1):
        fmps['qnum%d' % i] = qnuml[i]
    m.flmps = fmps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grads, energy, _ = adjoint.site_gradients(m)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    dh, dg = adjoint.integral_gradients(m, h, eri, grads)
    t2 = time.perf_counter()
    dH = rng.standard_normal((K, K))
    dH = dH + dH.T
    dG = adjoint.symmetrize_eri_gradient(rng.standard_normal((K, K, K, K)))
    eps = 1e-5
    es = []
    for sgn in (1, -1):
        m.loadInts(I.spin_orbital(h + sgn * eps * dH, eri + sgn * eps * dG))
        m.dumpMPO()
        es.append(m.checkMPS()[0])
    fd = (es[0] - es[1]) / (2 * eps)
    an = float((dh * dH).sum() + (dg * dG).sum())
    return {"workload": "K=%d N=%d D=%d random left-canonical MPS, %d terms" % (K, nelec, D, m.nops),
            "s_site_gradients": t1 - t0, "s_chain_rule": t2 - t1, "energy": energy,
            "fd_directional": fd, "adjoint_directional": an, "abs_diff": abs(fd - an)}


def sweep_converged(K=24, nelec=24, D=512, seed=2024, maxiter=14, tol=1e-8, hop=1.0, phases=True):
    """Sweep seconds of the split path against the FP64 path at the same
    converged state (K=24, 24 electrons, Sz=0, D=512 by default).

    Phase 1: the reference's default two-site schedule (mpo_dmrg_schedule
    normal(2): bond dimension ramp from 1.5 sqrt(D), density-matrix noise
    1e-4 in the ramp, Davidson tolerance 1e-4 down to 1e-9) from the
    occupation-number state, split precision, until the schedule's
    convergence test (energy change below ``tol`` after the ramp) or
    ``maxiter`` sweep pairs.  Phase 2: from that MPS (environments rebuilt
    from it for each arm, so both arms start from identical states), one FP64
    sweep pair and one split sweep pair at D, Davidson 1e-9, no noise, each
    timed alone: seconds per sweep pair and half sweep, matvecs, energies,
    their difference, the difference of each arm from the phase-1 energy,
    and whether each arm's pair is converged: its right and left half sweeps
    end within ``tol`` of each other (the schedule's own test compares whole
    sweeps; its last sweeps can still be above the fixed point, which the
    noise-free pair at Davidson 1e-9 then reaches).  (The noisy ramp
    amplifies any perturbation, even one of 1e-15 in an environment, into a
    different truncation, so two runs of the whole schedule are compared
    only through this common state.)"""
    import torch
    from zmpo_dmrg_gb300 import integrals as I
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.mpo_dmrg_schedule import schedule
    h, eri, _ = I.synthetic(K, seed, hop)
    m = mpo_dmrg(seed=1)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.occun = I.closed_shell_occun(K, nelec)
    m.qsectors = {str([float(nelec), 0.0]): 1}
    m.precision, m.precision_renorm = "split", "emu64"
    m.partition()
    m.loadInts(I.spin_orbital(h, eri))
    m.dumpMPO()
    out = {"workload": "K=%d N=%d Sz=0 D=%d: default two-site schedule from the occupation-number state (split "
                       "precision), then one sweep pair (right + left, %d dots each, Davidson 1e-9, no noise) per "
                       "arm from the same converged MPS" % (K, nelec, D, K - 1)}
    sc = schedule(maxM=D, tol=tol, maxiter=maxiter)
    sc.normal(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m.default(sc)
    torch.cuda.synchronize()
    out["converge"] = {"s": time.perf_counter() - t0, "sweeps": m.nsweep, "converged": bool(m.ifconv),
                       "energy": float(m.Energy), "energies": [float(e) for e in m.eav],
                       "matvecs": int(sum(m.nmvp))}
    e_conv = float(m.Energy)
    mps = {k: v for k, v in m.flmps.items() if k.startswith('site') or k.startswith('qnum')}
    mps['nsite'] = K
    fixed = schedule(maxM=D, tol=1e-9, maxiter=1)
    fixed.fixed(ncsite=2, maxM=D, tol=1e-9, maxiter=1, noise=0.0)
    for prec in ("fp64", "split"):
        m.precision = prec
        m.precision_renorm = "emu64" if prec == "split" else "fp64"
        m.flmps = {'nsite': K, 'qnum0': m.qnuml[0]}
        m.frmps = {'nsite': K, 'qnum%d' % K: m.qnumr[-1]}
        m.qnuml = [numpy.asarray(mps['qnum%d' % i]) for i in range(K + 1)]
        m.flmps.update(mps)
        m.initOps(mps)
        m.psi0 = None
        fixed.getParameters(m, 0)
        m.crit_e = 1e-9
        m.plan_counts = collections.Counter()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r1 = m.sweep(list(range(K)), 2, 'R')
        r2 = m.sweep(list(range(K)), 2, 'L')
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        e = min(float(r1[2]), float(r2[2]))
        out[prec] = {"s_per_sweep": dt, "s_per_half_sweep": dt / 2, "energy": e, "matvecs": int(r1[0] + r2[0]),
                     "converged": abs(float(r1[2]) - float(r2[2])) < tol,
                     "dE_half_sweeps": float(r2[2]) - float(r1[2]),
                     "dE_vs_converged": e - e_conv}
        # plans built for structures not met before, and plans reused
        out[prec]["plans"] = dict(m.plan_counts)
        if phases and prec == "split":
            # the same sweep pair again with seconds per phase of the dots
            # (plan building, diagonal, Davidson, final Rayleigh quotient,
            # decimation, guess, renormalisation ...); each phase boundary
            # synchronises the device, so the phases add up to more than the
            # timed pair, where the GPU work of one dot overlaps the host
            # work of the next
            m.flmps = {'nsite': K, 'qnum0': m.qnuml[0]}
            m.frmps = {'nsite': K, 'qnum%d' % K: m.qnumr[-1]}
            m.qnuml = [numpy.asarray(mps['qnum%d' % i]) for i in range(K + 1)]
            m.flmps.update(mps)
            m.initOps(mps)
            m.psi0 = None
            # the plans of the timed pair would all be reused: start empty
            from zmpo_dmrg_gb300.mpo_dmrg_kernel import _release_all
            for name in ("_sigma_cache", "_renorm_cache"):
                if name in m.__dict__:
                    _release_all(m.__dict__[name])
            m._sigma_plan = None
            m.phase_times = {}
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m.sweep(list(range(K)), 2, 'R')
            m.sweep(list(range(K)), 2, 'L')
            torch.cuda.synchronize()
            out[prec]["phases_s"] = {k: round(v, 4) for k, v in sorted(m.phase_times.items(), key=lambda kv: -kv[1])}
            out[prec]["phases_s"]["total"] = round(time.perf_counter() - t0, 4)
            m.phase_times = None
    out["dE_split_fp64"] = abs(out["split"]["energy"] - out["fp64"]["energy"])
    out["sweep_speedup_split_vs_fp64"] = out["fp64"]["s_per_sweep"] / out["split"]["s_per_sweep"]
    del m
    torch.cuda.empty_cache()
    return out


def section(name, fn):
    """Run one optional section of the benchmark: its result, or, when it
    raises, {"error": "<type>: <message>"} (also printed on stderr), so the
    result line is printed whatever happens in the section."""
    try:
        return fn()
    except Exception as ex:  # noqa: BLE001 -- reported in the result line
        print("bench: %s failed: %r" % (name, ex), file=sys.stderr)
        return {"error": "%s: %s" % (type(ex).__name__, ex)}


def cpu_threads():
    return os.cpu_count() or 1


def run_reference(args):
    """--impl reference: the reference's algorithm (the oracle's restatement
    of HVecQt, NumPy/BLAS FP64) on the host cores, on the same workload.  No
    engine code is imported: the dot is built on the host (``reference_dot``)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cfg = WORKLOAD
    t0 = time.perf_counter()
    m = reference_dot(cfg)
    t_setup = time.perf_counter() - t0
    n = m.qtmp.size_allowed
    x = numpy.random.default_rng(5).standard_normal(n)
    nops = m.fhop['nops']
    # three terms a step: the driver's 20 timed steps visit all 48 terms
    per = 3
    oracle_rate(m, per, args.warmup, cfg["isite"], x)
    res, seen = oracle_rate(m, per, args.steps, cfg["isite"], x)
    fl = sum(r[0] for r in res)
    tt = sum(r[1] for r in res)
    v = fl / tt / 1e12
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt / len(res),
           "higher_is_better": True, "config": workload_config(cfg, n, nops),
           "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cpu_threads(), "kind": "port",
                            "sample": "oracle HVecQt (the reference's NumPy algorithm, FP64) over %d of the %d "
                                      "operator terms per step, rotating (%d distinct terms timed), F_ref/t; "
                                      "environments built by the oracle's renormalisation on the host "
                                      "(%.0f s)" % (per, nops, len(seen), t_setup),
                            "mpi": MPI_NOTE, "setup_s": t_setup},
           "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine")
    ap.add_argument("--precision", default="split")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--small", action="store_true", help="K=12, D=128 case (profiling)")
    ap.add_argument("--medium", action="store_true", help="K=16, D=256 case (profiling)")
    ap.add_argument("--no-gradient", action="store_true",
                    help="skip the energy-gradient timing at K=16, D=256 (adjoint configuration)")
    ap.add_argument("--sp", action="store_true",
                    help="spin-projected H.psi, K=20, D=512, 8 quadrature points (terms in batches)")
    ap.add_argument("--large", action="store_true",
                    help="K=36, D=1024, hopping 0.7 (terms in batches under a 64 GB workspace)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from zmpo_dmrg_gb300 import build as _b
    _b.build()
    from zmpo_dmrg_gb300 import engine as E
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HVec, _sigma_plan

    P, t_build = build_problem(small=args.small, medium=args.medium, large=args.large, sp=args.sp)
    cfg = SMALL if args.small else (MEDIUM if args.medium else (LARGE if args.large else
                                                                 (SPCFG if args.sp else WORKLOAD)))
    pm = P.p
    if args.large or args.sp:
        pm.workspace_budget = LARGE_WORKSPACE
        pm._sigma_plan = None
    flst = pm.flst
    if world > 1:
        # the operator terms partitioned over the ranks (the reference's
        # partitionSites): each rank's plan covers its block of terms and the
        # partial vectors are summed with one NCCL all-reduce per step
        from zmpo_dmrg_gb300.mpo_dmrg_kernel import EnvSet
        from zmpo_dmrg_gb300.parallel import partition_ops
        mine = [o[0] for o in partition_ops(pm.sbas, world, rank)]
        keep = numpy.zeros(pm.nops, dtype=bool)
        keep[mine] = True
        flst = [[EnvSet(env.buf, numpy.where(keep, env.off, -1), env.layouts, env.tensors)
                 for env in pm.flst[0][0:2]] + list(pm.flst[0][2:])]
    info = [pm, P.isite, 2, flst, 'L', True]
    eng = E.get()
    plan = _sigma_plan(info)
    flops = plan.flops
    n = P.ndim0
    x_host = numpy.random.default_rng(5).standard_normal(n)
    x = torch.from_numpy(x_host).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def step(prec):
        plan.run(pm, x, y, prec)
        if dist:
            dist.all_reduce(y)

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            step(prec)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step(prec)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return e0.elapsed_time(e1) / 1e3 / steps

    # accuracy of both paths against FP64 on this workload
    step("fp64")
    y64 = y.clone()
    step(args.precision)
    err_split = float(torch.linalg.norm(y - y64) / torch.linalg.norm(y64))

    clocks = Clocks()
    clocks.start()
    t_split = timed(args.precision, args.steps, max(args.warmup, 3))
    clocks_rec = clocks.stop()
    t_fp64 = timed("fp64", max(2, args.steps // 10), 1)

    # the first H.psi of a Davidson solve also cuts the digit planes of the
    # environments and the MPO (later ones reuse them, as the timed steps do)
    def cold_step():
        plan._kept_token = None
        step(args.precision)

    for _ in range(2):
        cold_step()
    torch.cuda.synchronize()
    ncold = max(3, args.steps // 4)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(ncold):
        cold_step()
    c1.record(stream)
    torch.cuda.synchronize()
    t_cold = c0.elapsed_time(c1) / 1e3 / ncold

    # per-launch durations (engine tracing: CUDA events around each launch on
    # its stream) and the algorithmic bytes of each launch
    L = plan.fL.buf
    R = plan.fR.buf
    W = pm.mpo_store.buf
    eng.profile(True)
    for pid in plan.pids:
        eng.launch_times(pid)
    nprof = max(5, args.steps // 2)
    for _ in range(nprof):
        step(args.precision)
    torch.cuda.synchronize()
    ms, abytes, ncalls = eng.launch_times(plan.pid)
    for pid in plan.pids[1:]:   # term batches: the same steps, summed
        ms2, ab2, _ = eng.launch_times(pid)
        ms, abytes = ms + ms2, abytes + ab2
    eng.profile(False)
    launches = [{"launch": i, "ms": float(ms[i]), "alg_bytes": float(abytes[i]),
                 "GBs": float(abytes[i] / (ms[i] * 1e-3) / 1e9) if ms[i] > 0 else None}
                for i in range(plan.nlaunch)]
    top = max(range(plan.nlaunch), key=lambda i: ms[i])
    # multiply-adds the tiles of each step issue (tile padding included)
    macs = sum(eng.mma_macs(pid, args.precision, plan.nlaunch) for pid in plan.pids)
    products = {"split": 10, "emu64": 28, "fp64": 1}[args.precision]
    # e2e through the C ABI with host vectors
    xh = torch.from_numpy(x_host).pin_memory()
    yh = torch.empty(n, dtype=torch.float64).pin_memory()
    for _ in range(3):
        xd = xh.cuda(non_blocking=True)
        plan.run(pm, xd, y, args.precision)
        yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ne2e = max(3, args.steps // 2)
    for _ in range(ne2e):
        xd = xh.cuda(non_blocking=True)
        plan.run(pm, xd, y, args.precision)
        yh.copy_(y, non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / ne2e

    # algorithmic bytes of one step: every operand block read once, outputs written once
    hbm, bf16, peak_kind = peaks()
    value = flops / t_split / 1e12
    tmax = t_split
    if dist:
        tt = torch.tensor([t_split], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tmax = float(tt.item())
        ft = torch.tensor([flops], dtype=torch.float64, device="cuda")
        dist.all_reduce(ft)  # the whole dot's F_ref: every rank's terms
        flops = float(ft.item())
        value = flops / tmax / 1e12
    result = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": tmax * 1e3, "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
        "dtype": "f64 (bf16 digit slices, fp32 accumulate)",
        "data": "synthetic (seeded integrals + seeded random block-sparse MPS)",
        "config": workload_config(cfg, n, pm.nops),
        "plan": {"F_ref_flops": flops, "tasks": plan.ntasks, "precision": args.precision,
                 "term_batches": len(plan.pids),
                 "l2": "inputs larger than L2 (environments %.2f GB)" % ((L.numel() + R.numel()) * 8 / 1e9),
                 "build_s": t_build},
        "fp64": {"value": flops / t_fp64 / 1e12, "ms_per_step": t_fp64 * 1e3},
        "first_of_solve": {"value": flops / t_cold / 1e12, "ms_per_step": t_cold * 1e3,
                           "note": "an H.psi that also cuts the digit planes of the environments and the MPO "
                                   "(the first of a Davidson solve); the timed steps reuse them, as every later "
                                   "H.psi of a solve does"},
        "split_vs_fp64_rel_err": err_split,
        "e2e": {"value": flops / t_e2e / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 8},
        "gpu_launches": args.steps * sum(eng.kernel_count(pid, args.precision) for pid in plan.pids),
        "clocks": clocks_rec,
        "launches": launches,
        "roofline": {"bound": "hbm",
                     "kernel": "step %d of %d: prepare kernels (k_prep_a / k_prep_b), tcgen05 kernels "
                               "(k_step_umma / k_step_umma_long), split-K sum" % (top, plan.nlaunch),
                     "achieved": launches[top]["GBs"], "peak": hbm, "unit": "GB/s",
                     "frac": (launches[top]["GBs"] or 0.0) / hbm,
                     "traffic": None,
                     "traffic_note": "DRAM bytes of the step's kernels: see the ncu summaries (profiles/); the "
                                     "algorithmic bytes count every operand tensor read once and every output "
                                     "written once",
                     "peak_source": peak_kind},
        # the tensor-pipe view of the same step: BF16 digit products the
        # tcgen05 MMAs issue (10 per FP64 multiply-add, 128-row tiles and
        # 16-slot steps included) over the measured sustained bf16 GEMM rate
        "roofline_tensor": {"bound": "tensor", "kernel": "tcgen05 kernels of step %d" % top,
                            "achieved": 2.0 * products * macs[top] / (ms[top] * 1e-3) / 1e12 if ms[top] > 0 else None,
                            "peak": bf16, "unit": "TFLOP/s",
                            "frac": (2.0 * products * macs[top] / (ms[top] * 1e-3) / 1e12 / bf16) if ms[top] > 0 else None,
                            "executed_flops_per_launch": 2.0 * products * macs[top] / len(plan.pids),
                            "note": "tcgen05.mma kind::f16 BF16 digit products (%d per FP64 multiply-add), tile "
                                    "padding included, over the step's whole time (prepare kernels included); "
                                    "peak = cuBLAS bf16 sustained" % products,
                            "peak_source": peak_kind} if args.precision != "fp64" else None,
    }
    if world > 1:
        result["config"]["parallelism"] = ("operator terms partitioned over %d ranks (contiguous blocks), one NCCL "
                                           "all-reduce of sigma per step" % world)
    # the split path multiplies on the tensor cores: its headline roofline is
    # the tensor-pipe view of the dominant step; the HBM view stays beside it
    if result.get("roofline_tensor"):
        rt = result.pop("roofline_tensor")
        rt.setdefault("traffic", None)
        rt["traffic_note"] = result["roofline"]["traffic_note"]
        result["roofline_hbm"] = result["roofline"]
        result["roofline"] = rt
    # the sections after the sigma measurement each record their own failure
    # (the JSON line is printed whatever happens in them)
    if rank == 0 and not args.no_sweep:
        result["sweep"] = section("sweep", sweep_converged)
        result["sweep_k10"] = section("sweep_k10", lambda: sweep_converged(K=10, nelec=10, D=64, maxiter=16))
    if rank == 0 and not args.no_gradient and not (args.small or args.medium or args.large or args.sp):
        result["gradient"] = section("gradient", gradient_metrics)
    if rank == 0 and not args.no_cpu and not (args.large or args.sp):
        leg = section("cpu_baseline", lambda: cpu_leg(P, cfg))
        if isinstance(leg, dict):
            result["cpu_baseline"], result["parity_vs_oracle"] = leg, leg
        else:
            result["cpu_baseline"], result["parity_vs_oracle"] = leg
    if rank == 0:
        print(json.dumps(result))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
