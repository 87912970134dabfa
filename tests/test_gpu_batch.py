"""Many-spectra sets and the persistent batched kernel against the oracle.

ps_mcm_set_device: K windows x spin cases on one grid, in window groups.
ps_batch_*: uneven problems (different lmax, K, spin cases) in one persistent
launch, directly and replayed from a CUDA graph; and the autotuner.
"""
import numpy as np
import pytest

from gpu_util import cond_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _W(nW, seed, cutoff=None):
    from powerspectra_gpu import synthetic as syn
    return syn.mask_spectrum(nW, 0.4 + 0.05 * (seed % 8), cutoff or max(nW / 3.0, 5.0), seed=seed)


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), device="cuda")


@pytest.mark.parametrize("mode,tol,cases", [("plain", 1e-12, 0xF), ("chosen", 1e-6, 0xF), ("chosen", 1e-6, 0xC),
                                            ("chosen", 1e-6, 0x4), ("chosen", 1e-6, 0x2), ("chosen", 1e-6, 0x9)])
def test_mcm_set_device(ctx, mode, tol, cases):
    L, K = 90, 5
    Ws = [_W(2 * L + 1, seed=k) for k in range(K)]
    dW = [_dev(w) for w in Ws]
    n = L + 1
    dM = {(k, s): torch.zeros((n, n), dtype=torch.float64, device="cuda") for k in range(K) for s in range(4)}
    ptrs = [dM[k, s].data_ptr() for k in range(K) for s in range(4)]
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.mcm_set_device(cases, [d.data_ptr() for d in dW], 2 * L + 1, 0, L, ptrs, n, mode=mode)
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(0)
    for k in range(K):
        for s in range(4):
            if not cases & (1 << s):
                continue
            got = dM[k, s].cpu().numpy().T
            ref = o.inner_mcm(s, Ws[k], 0, L)
            assert max_err_scaled(got, ref, cond_scale(s, Ws[k], 0, L)) < tol, (k, s)


def _batch_problems(seed=3):
    rng = np.random.default_rng(seed)
    probs, refs = [], []
    for i in range(7):
        L = int(rng.choice([40, 77, 128, 200, 255]))
        K = int(rng.integers(1, 6))
        cases = [0x1, 0xC, 0xF, 0x2, 0x4, 0x8, 0x3][i]  # every batch body, and a split combination
        lmin = [0, 0, 2, 0, 5, 0, 0][i]
        n = L - lmin + 1
        Ws = [_W(2 * L + 1, seed=100 * i + k) for k in range(K)]
        dW = [_dev(w) for w in Ws]
        dM = [torch.zeros((n, n), dtype=torch.float64, device="cuda") if cases & (1 << s) else None
              for k in range(K) for s in range(4)]
        probs.append({"lmin": lmin, "lmax": L, "cases": cases, "nW": 2 * L + 1, "ldm": n,
                      "W": [d.data_ptr() for d in dW], "M": [m.data_ptr() if m is not None else 0 for m in dM],
                      "_keep": (dW, dM)})
        refs.append((Ws, lmin, L, cases, dM))
    return probs, refs


def _check(refs, tol=1e-6):
    for Ws, lmin, L, cases, dM in refs:
        for k, W in enumerate(Ws):
            for s in range(4):
                if cases & (1 << s):
                    got = dM[4 * k + s].cpu().numpy().T
                    ref = o.inner_mcm(s, W, lmin, L)
                    assert max_err_scaled(got, ref, cond_scale(s, W, lmin, L)) < tol, (L, k, s)


def test_batch_run_and_graph(ctx):
    probs, refs = _batch_problems()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.batch_prepare(probs)
        ctx.batch_run()
        torch.cuda.synchronize()
        _check(refs)
        for _, _, _, _, dM in refs:
            for m in dM:
                if m is not None:
                    m.zero_()
        ctx.batch_graph_launch()  # capture + replay
        ctx.batch_graph_launch()  # replay
        torch.cuda.synchronize()
        _check(refs)
    finally:
        ctx.set_stream(0)


def test_batch_autotune_and_group_sizes(ctx):
    probs, refs = _batch_problems(seed=9)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        best = ctx.batch_autotune(probs)
        assert best["group_slots"] in (2, 4, 8) and best["blocks_per_sm"] != 0 and best["ms"] > 0
        for gs in (2, 4, 8):
            for bps in (0, -1):  # persistent kernel, and one launch per group
                for _, _, _, _, dM in refs:
                    for m in dM:
                        if m is not None:
                            m.fill_(float("nan"))
                ctx.batch_prepare(probs, group_slots=gs, blocks_per_sm=bps)
                ctx.batch_run()
                torch.cuda.synchronize()
                _check(refs)
    finally:
        ctx.set_stream(0)


def test_batch_argument_errors(ctx):
    import powerspectra_gpu as pg
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.batch_run() if False else ctx.batch_prepare([{"lmin": 5, "lmax": 3, "cases": 1, "nW": 10, "ldm": 10,
                                                           "W": [1], "M": [1, 0, 0, 0]}])
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.batch_prepare([{"lmin": 0, "lmax": 10, "cases": 1, "nW": 10, "ldm": 11, "W": [0], "M": [1, 0, 0, 0]}])
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.batch_prepare([{"lmin": 0, "lmax": 10, "cases": 1, "nW": 21, "ldm": 11, "W": [1], "M": [1, 0, 0, 0]}],
                          group_slots=3)


@pytest.mark.parametrize("cases", [0xF, 0xC, 0x1])
def test_mcm_set_host(ctx, cases):
    """ps_mcm_set: host spectra in, host matrices out (some page-locked, written in place)."""
    L, K, lmin = 70, 3, 2
    Ws = [_W(2 * L + 1, seed=40 + k) for k in range(K)]
    n = L - lmin + 1
    outs = {}
    for k in range(K):
        for s in range(4):
            if cases & (1 << s):
                if (k + s) % 2:
                    outs[k, s] = torch.empty((n, n), dtype=torch.float64).pin_memory().numpy().T
                else:
                    outs[k, s] = np.empty((n, n), dtype=np.float64, order="F")
    got = ctx.mcm_set(cases, Ws, lmin, L, mode="chosen", outs=outs)
    for (k, s), m in got.items():
        assert m is outs[k, s]
        ref = o.inner_mcm(s, Ws[k], lmin, L)
        assert max_err_scaled(m, ref, cond_scale(s, Ws[k], lmin, L)) < 1e-6, (k, s)


def _routed_problems():
    """Problems whose TT slots or ++/-- slots (9 or more at these sizes) take the tensor-core
    kernels, next to ones that stay on the CUDA cores."""
    specs = [(97, 0, 0x1, 9), (130, 3, 0xC, 5), (64, 0, 0xF, 5), (77, 2, 0x1, 3), (50, 0, 0x3, 4)]
    probs, refs = [], []
    for i, (L, lmin, cases, K) in enumerate(specs):
        n = L - lmin + 1
        Ws = [_W(2 * L + 1, seed=700 + 10 * i + k) for k in range(K)]
        dW = [_dev(w) for w in Ws]
        dM = [torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda") if cases & (1 << s) else None
              for k in range(K) for s in range(4)]
        probs.append({"lmin": lmin, "lmax": L, "cases": cases, "nW": 2 * L + 1, "ldm": n,
                      "W": [d.data_ptr() for d in dW], "M": [m.data_ptr() if m is not None else 0 for m in dM],
                      "_keep": (dW, dM)})
        refs.append((Ws, lmin, L, cases, dM))
    return probs, refs


@pytest.mark.parametrize("bps,graph", [(0, False), (-1, False), (0, True), (-1, True)])
def test_batch_tensor_core_routing(ctx, bps, graph):
    """The batch routes each problem's TT slots and ++/-- slots to the tensor-core kernels when
    there are enough for its lmax, like ps_mcm_set_device: every output against the oracle (NaN sentinels),
    in the persistent and the launch form, directly and from a CUDA graph; with the tensor cores
    switched off the routed slots change in their last bits, and problems 3 and 4 (TT and TE
    slots on the CUDA cores, grouped the same either way) not at all.  Problem 2's TT and TE slots
    stay on the CUDA cores but in other groups once its ++/-- slots leave, so only their tolerance
    is checked."""
    probs, refs = _routed_problems()
    routed = {(0, 0), (1, 2), (1, 3), (2, 2), (2, 3)}  # (problem, spin case)
    same_groups = {(3, 0), (4, 0), (4, 1)}
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        outs = {}
        for tc in (True, False):
            ctx.set_tensor_cores(tc)
            for _, _, _, _, dM in refs:
                for m in dM:
                    if m is not None:
                        m.fill_(float("nan"))
            ctx.batch_prepare(probs, group_slots=4, blocks_per_sm=bps)
            for _ in range(2 if graph else 1):
                ctx.batch_graph_launch() if graph else ctx.batch_run()
            torch.cuda.synchronize()
            ctx.synchronize()  # reports a tensor-core wait that gave up
            _check(refs)
            outs[tc] = [[m.cpu().numpy() if m is not None else None for m in dM] for _, _, _, _, dM in refs]
        for i, (Ws, _, _, cases, _) in enumerate(refs):
            for k in range(len(Ws)):
                for s in range(4):
                    if cases & (1 << s):
                        same = np.array_equal(outs[True][i][4 * k + s], outs[False][i][4 * k + s])
                        if (i, s) in routed:
                            assert not same, (i, k, s)
                        elif (i, s) in same_groups:
                            assert same, (i, k, s)
    finally:
        ctx.set_tensor_cores(True)
        ctx.set_stream(0)


def test_batch_launch_form_in_a_graph(ctx):
    """blocks_per_sm = -1: one launch per window group, captured into a CUDA graph and replayed."""
    probs, refs = _batch_problems(seed=5)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.batch_prepare(probs, group_slots=8, blocks_per_sm=-1)
        for _ in range(2):
            for _, _, _, _, dM in refs:
                for m in dM:
                    if m is not None:
                        m.fill_(float("nan"))
            ctx.batch_graph_launch()
            torch.cuda.synchronize()
            _check(refs)
    finally:
        ctx.set_stream(0)


@pytest.mark.parametrize("mode,tol", [("plain", 1e-12), ("chosen", 1e-6)])
def test_mcm_set_sparse_slots(ctx, mode, tol):
    """A set where each spectrum gets only some spin cases (NULL outputs skip their slots), like
    the large set: TT of spectra 0, 3, ..., ++ of 1, 4, ..., -- of 2, 5, ..., and one TE slot.
    The skipped outputs stay untouched."""
    L, K = 70, 10
    Ws = [_W(2 * L + 1, seed=20 + k) for k in range(K)]
    dW = [_dev(w) for w in Ws]
    n = L + 1
    want = {(k, (0, 2, 3)[k % 3]) for k in range(K)} | {(4, 1)}
    dM = {(k, s): torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
          for k in range(K) for s in range(4)}
    ptrs = [dM[k, s].data_ptr() if (k, s) in want else 0 for k in range(K) for s in range(4)]
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.mcm_set_device(0xF, [d.data_ptr() for d in dW], 2 * L + 1, 0, L, ptrs, n, mode=mode)
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(0)
    for k in range(K):
        for s in range(4):
            got = dM[k, s].cpu().numpy().T
            if (k, s) not in want:
                assert np.isnan(got).all(), (k, s)
                continue
            ref = o.inner_mcm(s, Ws[k], 0, L)
            assert max_err_scaled(got, ref, cond_scale(s, Ws[k], 0, L)) < tol, (k, s)


def test_mcm_set_host_sparse_slots(ctx):
    """ps_mcm_set with a slot filter: only the chosen (window, case) slots are returned."""
    L, K = 60, 4
    Ws = [_W(2 * L + 1, seed=40 + k) for k in range(K)]
    slots = {(0, 0), (1, 2), (2, 3), (3, 2), (3, 3)}
    got = ctx.mcm_set(0xD, Ws, 0, L, mode="chosen", slots=slots)
    assert set(got) == slots
    for (k, s), M in got.items():
        ref = o.inner_mcm(s, Ws[k], 0, L)
        assert max_err_scaled(M, ref, cond_scale(s, Ws[k], 0, L)) < 1e-6, (k, s)


def test_mcm_set_all_slots_null_is_an_error(ctx):
    import powerspectra_gpu as pg
    L = 10
    dW = [_dev(_W(2 * L + 1, seed=1))]
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.mcm_set_device(0x1, [d.data_ptr() for d in dW], 2 * L + 1, 0, L, [0, 0, 0, 0], L + 1)
