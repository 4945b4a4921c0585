"""The allocation-free contraction entry point (``zmpo_contract_exec_noalloc``).

Callers that cannot allocate device memory while they run -- work recorded into
a CUDA graph by stream capture, or a host framework that owns the device
memory budget -- use this variant: its split-K partial sums live in a fixed
8 MiB array inside the library.  The tests call it through the C ABI twice in
a row and checks both results against the regular ``zmpo_contract_exec`` on
the same plan, for the FP64 and the split tensor-core path, replay it from a
CUDA graph recorded by stream capture, and check that a plan needing more
scratch than the array holds, or a precision the set-up run did not use, is
refused.  This file is
collected last so that a failure here does not stop the other tests."""

import numpy
import pytest

pytestmark = pytest.mark.gpu


def _layouts(eng, mdims, kdims, ndims):
    """A[m,k] and B[k,n] with one-label sectors; blocks on the diagonal."""
    q = lambda n: numpy.arange(n, dtype=float).reshape(n, 1)
    la = eng.layout([q(len(mdims)), q(len(kdims))], [mdims, kdims], [False, True])
    lb = eng.layout([q(len(kdims)), q(len(ndims))], [kdims, ndims], [False, True])
    return la, lb


def _run(gpu, mdims, kdims, ndims, precision, seed):
    import torch
    from zmpo_dmrg_gb300 import engine as E, _lib
    eng = E.get()
    la, lb = _layouts(eng, mdims, kdims, ndims)
    lo, pid = eng.contract_plan(la, lb, ([1], [0]))
    na = eng.layout_blocks(la)[0]
    nb = eng.layout_blocks(lb)[0]
    no = eng.layout_blocks(lo)[0]
    g = torch.Generator(device="cuda").manual_seed(seed)
    a = torch.randn(na, dtype=torch.float64, device="cuda", generator=g)
    b = torch.randn(nb, dtype=torch.float64, device="cuda", generator=g)
    ref = torch.empty(no, dtype=torch.float64, device="cuda")
    eng.contract_exec(pid, a, b, ref, precision)  # set-up run: builds the device task lists
    outs = []
    for _ in range(2):
        out = torch.full((no,), float("nan"), dtype=torch.float64, device="cuda")
        rc = _lib.lib().zmpo_contract_exec_noalloc(eng.h, pid, E.device_ptr(a), E.device_ptr(b),
                                                   E.device_ptr(out), _lib.PREC[precision],
                                                   E.current_stream())
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        outs.append(out)
    return ref, outs, eng, pid, a, b


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("split", 1e-12)])
def test_noalloc_matches_regular_entry_point(gpu, precision, tol):
    # K = 5000 and 3000 exceed the split-K threshold: the partials are used
    ref, outs, *_ = _run(gpu, [40, 24], [5000, 3000], [30, 20], precision, seed=3)
    import torch
    for out in outs:
        assert torch.isfinite(out).all()
        err = float(torch.linalg.norm(out - ref) / torch.linalg.norm(ref))
        assert err <= tol


def test_noalloc_refuses_oversized_scratch(gpu):
    import torch
    from zmpo_dmrg_gb300 import engine as E, _lib
    eng = E.get()
    la, lb = _layouts(eng, [1100], [5000], [1000])   # 3 parts x 1.1e6 > 1048576
    lo, pid = eng.contract_plan(la, lb, ([1], [0]))
    a = torch.ones(1100 * 5000, dtype=torch.float64, device="cuda")
    b = torch.ones(5000 * 1000, dtype=torch.float64, device="cuda")
    out = torch.empty(1100 * 1000, dtype=torch.float64, device="cuda")
    eng.contract_exec(pid, a, b, out, "fp64")
    rc = _lib.lib().zmpo_contract_exec_noalloc(eng.h, pid, E.device_ptr(a), E.device_ptr(b),
                                               E.device_ptr(out), _lib.PREC["fp64"], E.current_stream())
    assert rc == -6
    assert "8 MiB" in _lib.last_error()


def test_noalloc_under_stream_capture(gpu):
    """The use the entry point is for: after a set-up run and one warm call,
    the call is recorded into a CUDA graph by stream capture and replayed; the
    replay equals the regular entry point."""
    import torch
    from zmpo_dmrg_gb300 import engine as E, _lib
    ref, outs, eng, pid, a, b = _run(gpu, [40, 24], [5000, 3000], [30, 20], "split", seed=5)
    out = torch.full_like(ref, float("nan"))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rc = _lib.lib().zmpo_contract_exec_noalloc(eng.h, pid, E.device_ptr(a), E.device_ptr(b),
                                                   E.device_ptr(out), _lib.PREC["split"], E.current_stream())
    assert rc == 0, _lib.last_error()
    for _ in range(2):
        out.fill_(float("nan"))
        graph.replay()
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert float(torch.linalg.norm(out - ref) / torch.linalg.norm(ref)) <= 1e-12


def test_noalloc_needs_a_set_up_run_at_its_precision(gpu):
    """Device task lists are made per precision at the first run: a call at a
    precision the set-up did not use is refused before any launch."""
    import torch
    from zmpo_dmrg_gb300 import engine as E, _lib
    eng = E.get()
    la, lb = _layouts(eng, [40], [300], [30])
    lo, pid = eng.contract_plan(la, lb, ([1], [0]))
    a = torch.ones(40 * 300, dtype=torch.float64, device="cuda")
    b = torch.ones(300 * 30, dtype=torch.float64, device="cuda")
    out = torch.empty(40 * 30, dtype=torch.float64, device="cuda")
    eng.contract_exec(pid, a, b, out, "fp64")
    rc = _lib.lib().zmpo_contract_exec_noalloc(eng.h, pid, E.device_ptr(a), E.device_ptr(b),
                                               E.device_ptr(out), _lib.PREC["split"], E.current_stream())
    assert rc != 0 and "this precision" in _lib.last_error()
