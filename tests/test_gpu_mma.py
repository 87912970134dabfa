"""The tensor-core coupling kernels (k_coupling_mma): the TT slots of a
chosen-mode set and its ++ / -- slots when there are enough of them for the
lmax (9 below lmax 768; TT 5 from lmax 768 and 4 from 3072, ++/-- 5 from lmax
1536); one (0 0 0) or (2 -2 0) family generation for up to 15 windows
(the (0 0 0) sweeps two points per time step), the window contraction as BF16
tcgen05 MMAs (three-part split, fresh FP32 accumulator per 16 steps,
float-float totals).

Bar: the chosen form's 1e-6 max relative error against FP64 (the oracle at
small sizes, the plain FP64 kernel or the oracle on sampled rows at large
sizes), relative to the sum of |terms| of each element.  Every output element
is written (NaN sentinels, a leading dimension larger than the matrix).
"""
import numpy as np
import pytest

from gpu_util import cond_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 1e-6


def _W(nW, seed, fsky=0.6, cutoff=None):
    from powerspectra_gpu import synthetic as syn
    return syn.mask_spectrum(nW, fsky, cutoff or max(nW / 3.0, 5.0), seed=seed)


def _run_set(ctx, Ws, slots, lmin, lmax, pad=3, tensor_cores=True, mode="chosen"):
    """ps_mcm_set_device over (window, case) `slots`; returns {slot: host matrix (l1, l2)}."""
    n = lmax - lmin + 1
    ld = n + pad
    dW = [torch.tensor(np.ascontiguousarray(w), device="cuda") for w in Ws]
    mats = {sl: torch.full((n, ld), float("nan"), dtype=torch.float64, device="cuda") for sl in slots}
    ptrs = [0] * (4 * len(Ws))
    cases = 0
    for (k, s), m in mats.items():
        ptrs[4 * k + s] = m.data_ptr()
        cases |= 1 << s
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    ctx.set_tensor_cores(tensor_cores)
    try:
        ctx.mcm_set_device(cases, [d.data_ptr() for d in dW], min(len(w) for w in Ws), lmin, lmax, ptrs, ld,
                           mode=mode)
        torch.cuda.synchronize()
        ctx.synchronize()  # reports a tensor-core wait that gave up
    finally:
        ctx.set_tensor_cores(True)
        ctx.set_stream(0)
    out = {}
    for sl, m in mats.items():
        a = m.cpu().numpy()
        assert np.all(np.isnan(a[:, n:])), sl  # the padding stays untouched
        out[sl] = a[:, :n].T  # column-major storage: the transpose is M[l1, l2]
    return out


@pytest.mark.parametrize("L,lmin,nWk", [(40, 0, "2L1"), (97, 3, "2L1"), (64, 0, "short"), (200, 0, "L1"),
                                        (5, 0, "2L1"), (1, 0, "2L1"), (0, 0, "L1"), (33, 2, "2L1")])
def test_mma_vs_oracle_small(ctx, L, lmin, nWk):
    nW = {"2L1": 2 * L + 1, "L1": L + 1, "short": max(L // 2, 1)}[nWk]
    Ws = [_W(nW, seed=10 + k, fsky=0.4 + 0.04 * k) for k in range(10)]
    slots = [(k, s) for k in range(5) for s in (2, 3)] + [(k, 0) for k in range(1, 10)]
    got = _run_set(ctx, Ws, slots, lmin, L)
    for (k, s), G in got.items():
        assert np.all(np.isfinite(G)), (k, s)
        R = o.inner_mcm(s, Ws[k], lmin, L)
        assert max_err_scaled(G, R, cond_scale(s, Ws[k], lmin, L)) < TOL, (k, s)


def test_mma_fifteen_windows_and_a_second_launch(ctx):
    """17 slots: 15 in one tensor-core launch, 2 more in a second one."""
    L = 120
    Ws = [_W(2 * L + 1, seed=40 + k, fsky=0.3 + 0.03 * k) for k in range(9)]
    slots = [(k, s) for k in range(9) for s in (2, 3)][:17]
    got = _run_set(ctx, Ws, slots, 0, L)
    for (k, s), G in got.items():
        R = o.inner_mcm(s, Ws[k], 0, L)
        assert max_err_scaled(G, R, cond_scale(s, Ws[k], 0, L)) < TOL, (k, s)


def test_mma_negative_windows(ctx):
    """Windows with negative entries: the sums cancel; measured against the sum of |terms|."""
    L = 150
    Ws = [_W(2 * L + 1, seed=60 + k) * np.where(np.arange(2 * L + 1) % (5 + k) == 0, -1.0, 1.0) for k in range(9)]
    slots = [(k, s) for k in range(5) for s in (2, 3)] + [(k, 0) for k in range(9)]
    got = _run_set(ctx, Ws, slots, 0, L)
    for (k, s), G in got.items():
        R = o.inner_mcm(s, Ws[k], 0, L)
        assert max_err_scaled(G, R, cond_scale(s, Ws[k], 0, L)) < TOL, (k, s)


def test_mma_wide_dynamic_range(ctx):
    """Windows spanning ~1e-97 (beyond FP32's range): the block scale keeps relative precision."""
    L = 1500
    l = np.arange(2 * L + 1, dtype=np.float64)
    base = 1e-3 * (l + 1) ** -2 * np.exp(-l * (l + 1) / (2 * 150.0 ** 2))
    Ws = []
    for k in range(9):
        W = base * (1.0 + 0.1 * k)
        W[0] += 4 * np.pi * (0.3 + 0.05 * k)
        Ws.append(W)
    assert Ws[0][-1] < 1e-90
    slots = [(k, s) for k in range(5) for s in (2, 3)] + [(k, 0) for k in range(9)]
    got = _run_set(ctx, Ws, slots, 0, L)
    ref = _run_set(ctx, Ws, slots, 0, L, mode="plain")
    for sl in slots:
        assert max_err_scaled(got[sl], ref[sl], np.abs(ref[sl])) < TOL, sl


def test_mma_matches_plain_fp64_full_size(ctx):
    """lmax 2047, the large set's mix (20 spectra: 7 TT, 7 ++, 6 --): every element against FP64."""
    from powerspectra_gpu import synthetic as syn
    big = syn.large_set(lmax=2047, K=20, seed=9)
    slots = [(k, (0, 2, 3)[k % 3]) for k in range(20)]
    got = _run_set(ctx, big["W"], slots, 0, 2047)
    ref = _run_set(ctx, big["W"], slots, 0, 2047, mode="plain")
    errs = {sl: max_err_scaled(got[sl], ref[sl], np.abs(ref[sl])) for sl in slots}
    assert max(errs.values()) < TOL, errs


def test_mma_agrees_with_cuda_core_path(ctx):
    """The same set with the tensor-core kernels switched off: both within 2e-6 of each other,
    and the routing itself: the 10 ++/-- slots (9 or more below lmax 1536) and the 5 TT slots (5
    or more from lmax 768) take the tensor-core kernels, so their results differ from the
    CUDA-core kernels' in the last bits."""
    L = 800
    Ws = [_W(2 * L + 1, seed=80 + k, fsky=0.5 + 0.05 * k) for k in range(5)]
    slots = [(k, s) for k in range(5) for s in (0, 2, 3)]
    a = _run_set(ctx, Ws, slots, 2, L)
    b = _run_set(ctx, Ws, slots, 2, L, tensor_cores=False)
    for sl in slots:
        assert max_err_scaled(a[sl], b[sl], np.abs(b[sl])) < 2 * TOL, sl
        assert not np.array_equal(a[sl], b[sl]), sl


@pytest.mark.parametrize("K,routed", [(4, False), (5, True)])
def test_mma_tt_routing_threshold(ctx, K, routed):
    """TT sets at lmax 1001: 4 slots stay on the CUDA cores (the same bits with the tensor cores
    switched off), 5 take the tensor-core kernel (odd lmin and lmax, lmin > 0)."""
    L = 1001
    Ws = [_W(2 * L + 1, seed=120 + k, fsky=0.45 + 0.05 * k) for k in range(K)]
    slots = [(k, 0) for k in range(K)]
    a = _run_set(ctx, Ws, slots, 5, L)
    b = _run_set(ctx, Ws, slots, 5, L, tensor_cores=False)
    for (k, s) in slots:  # against the CUDA-core kernels (the oracle checks are the other tests')
        assert max_err_scaled(a[k, s], b[k, s], np.abs(b[k, s])) < 2 * TOL, (k, s)
        assert np.array_equal(a[k, s], b[k, s]) != routed, (k, s)


def test_mma_lmax_8191_sampled_rows(ctx):
    """lmax 8191, nW 16383: 13 ++/-- and 9 TT slots, sampled rows and columns against the oracle."""
    from powerspectra_gpu import synthetic as syn
    big = syn.large_set(K=13)
    L, Ws = big["lmax"], big["W"]
    slots = [(k, 2 if k % 2 == 0 else 3) for k in range(13)] + [(k, 0) for k in range(9)]
    got = _run_set(ctx, Ws, slots, 0, L, pad=0)
    rows = [0, 1, 2, 701, 4094, 8000, 8191]
    for (k, s) in [(0, 2), (1, 3), (12, 2), (0, 0), (8, 0)]:
        R = o.inner_mcm(s, Ws[k], 0, L, rows=rows)
        G = got[k, s]
        for r in rows:
            assert max_err_scaled(G[r, r:], R[r, r:], np.abs(R[r, r:])) < TOL, (k, s, r)
            assert max_err_scaled(G[r:, r], R[r:, r], np.abs(R[r:, r])) < TOL, (k, s, r)


def test_mma_at_the_largest_lmax(ctx):
    """lmax 16383 (the largest the library accepts), nW 32767: 5 TT slots and 10 ++/-- slots on the
    tensor-core kernels; sampled rows and columns against the oracle (sampled on the device)."""
    from powerspectra_gpu import synthetic as syn
    L = 16383
    n = L + 1
    Ws = [syn.mask_spectrum(2 * L + 1, 0.5 + 0.05 * k, 1500.0 + 100.0 * k, seed=16000 + k) for k in range(5)]
    slots = [(k, s) for k in range(5) for s in (0, 2, 3)]
    dW = [torch.tensor(w, device="cuda") for w in Ws]
    mats = {sl: torch.empty((n, n), dtype=torch.float64, device="cuda") for sl in slots}
    ptrs = [0] * (4 * len(Ws))
    for (k, s), m in mats.items():
        ptrs[4 * k + s] = m.data_ptr()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.mcm_set_device(0xD, [d.data_ptr() for d in dW], 2 * L + 1, 0, L, ptrs, n, mode="chosen")
        torch.cuda.synchronize()
        ctx.synchronize()
    finally:
        ctx.set_stream(0)
    rows = [2, 9000, 16383]
    for (k, s) in [(0, 0), (4, 0), (1, 2), (3, 3)]:
        R = o.inner_mcm(s, Ws[k], 0, L, rows=rows)
        m = mats[k, s]  # column-major storage: m[l2, l1] = M[l1, l2]
        for r in rows:
            row, col = m[r:, r].cpu().numpy(), m[r, r:].cpu().numpy()  # M[r, r:] and M[r:, r]
            assert max_err_scaled(row, R[r, r:], np.abs(R[r, r:])) < TOL, (k, s, r)
            assert max_err_scaled(col, R[r:, r], np.abs(R[r:, r])) < TOL, (k, s, r)
    del mats
    torch.cuda.empty_cache()


def test_mma_host_entry_point(ctx):
    """ps_mcm_set (host spectra, page-locked and pageable outputs) through the tensor-core kernels."""
    L = 300
    Ws = [_W(2 * L + 1, seed=90 + k) for k in range(9)]
    slots = {(k, s) for k in range(5) for s in (2, 3)} | {(k, 0) for k in range(9)}
    n = L + 1
    outs = {}
    for i, sl in enumerate(sorted(slots)):
        t = torch.empty((n, n), dtype=torch.float64, pin_memory=(i % 2 == 0))
        outs[sl] = t.numpy().T  # F-ordered view
    got = ctx.mcm_set(0xD, Ws, 0, L, mode="chosen", outs=outs, slots=slots)
    for (k, s), G in got.items():
        R = o.inner_mcm(s, Ws[k], 0, L)
        assert max_err_scaled(G, R, cond_scale(s, Ws[k], 0, L)) < TOL, (k, s)
