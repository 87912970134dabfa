"""ps_coupledcov_set_device: several covariance blocks of one grid in one call.

In chosen mode the Xi of all the blocks' windows are computed grouped across
the blocks by family product and parity (the squared (0 0 0) windows by the
tensor-core kernel, and the squared (2 -2 0) ones, when there are enough of them
for the lmax, the rest by the CUDA-core kernel in groups of up to 8),
and each block is formed from its windows' Xi.  Plain FP64, or the tensor cores
switched off, runs the fused covariance kernel block by block.
"""
import numpy as np
import pytest

from gpu_util import cov_scale, max_err_scaled
from oracle import oracle as o

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SET6 = ["TTTT", "EEEE", "TETE", "TTTE", "TTEE", "TEEE"]
ROUTED = {"TTTT", "TTTE", "TTEE"}  # at lmax 180 all their 15 windows on the tensor-core kernel


def _inputs(L, kinds, seed=0):
    from powerspectra_gpu import synthetic as syn
    spectra, noise = syn.signal_spectra(L)
    f = syn.FIELDS
    S = [spectra["TT", f[0], f[2]], spectra["EE", f[1], f[3]], spectra["TE", f[0], f[3]], spectra["TE", f[1], f[2]]]
    R = [noise["TT", f[0], f[0]], noise["EE", f[1], f[1]], noise["TT", f[0], f[2]], noise["EE", f[1], f[3]]]
    blocks = []
    for b, kind in enumerate(kinds):
        Ws = [syn.mask_spectrum(2 * L + 1, 0.4 + 0.03 * ((b * 8 + k) % 13), 60.0 + 7 * k, seed=seed + 10 * b + k)
              for k in range(o.COV_NWINDOWS[kind])]
        blocks.append((kind, S, R[:o.COV_NRATIOS[kind]], Ws))
    return blocks


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), device="cuda")


def _run(ctx, blocks, lmin, L, mode="chosen", per_block=False, tensor_cores=True, pad=3):
    n = L - lmin + 1
    ld = n + pad
    keep, spec, outs = [], [], []
    for kind, S, R, Ws in blocks:
        dS, dR, dW = [_dev(x) for x in S], [_dev(x) for x in R], [_dev(x) for x in Ws]
        C = torch.full((n, ld), float("nan"), dtype=torch.float64, device="cuda")
        keep.append((dS, dR, dW, C))
        spec.append((kind, [x.data_ptr() for x in dS], [x.data_ptr() for x in dR], [x.data_ptr() for x in dW],
                     C.data_ptr()))
        outs.append(C)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    ctx.set_tensor_cores(tensor_cores)
    try:
        nW = 2 * L + 1
        if per_block:
            for kind, dS, dR, dW, dC in spec:
                ctx.coupledcov_device(kind, dS, dR, dW, nW, lmin, L, dC, ld, mode=mode)
        else:
            ctx.coupledcov_set_device(spec, nW, lmin, L, ld, mode=mode)
        torch.cuda.synchronize()
        ctx.synchronize()  # reports a tensor-core wait that gave up
    finally:
        ctx.set_tensor_cores(True)
        ctx.set_stream(0)
    res = []
    for C in outs:
        a = C.cpu().numpy()
        assert np.all(np.isnan(a[:, n:]))  # the padding stays untouched
        res.append(a[:, :n].T)
    return res


@pytest.mark.parametrize("L,lmin", [(150, 0), (97, 2)])
def test_cov_set_vs_oracle(ctx, L, lmin):
    blocks = _inputs(L, SET6 + ["TEEE_PLANCK"])
    got = _run(ctx, blocks, lmin, L)
    for (kind, S, R, Ws), C in zip(blocks, got):
        assert np.all(np.isfinite(C)), kind
        ref = o.loop_cov(kind, S, R, Ws, lmin, L)
        assert max_err_scaled(C, ref, cov_scale(kind, S, R, Ws, lmin, L)) < 1e-6, kind
        assert np.array_equal(C, C.T), kind


def test_cov_set_against_per_block_calls(ctx):
    """Every block within 2e-6 (of the sum of |terms|) of the fused kernel's; the blocks whose
    windows all take the tensor-core kernel differ in the last bits; with the tensor cores off
    every block is the fused kernel's, bit for bit."""
    L = 180
    blocks = _inputs(L, SET6, seed=5)
    a = _run(ctx, blocks, 0, L)
    b = _run(ctx, blocks, 0, L, per_block=True)
    c = _run(ctx, blocks, 0, L, tensor_cores=False)
    for (kind, S, R, Ws), x, y, z in zip(blocks, a, b, c):
        assert max_err_scaled(x, y, cov_scale(kind, S, R, Ws, 0, L)) < 2e-6, kind
        if kind in ROUTED:
            assert not np.array_equal(x, y), kind
        assert np.array_equal(z, y), kind


def test_cov_set_plain_fp64(ctx):
    L = 60
    blocks = _inputs(L, SET6, seed=9)
    got = _run(ctx, blocks, 1, L, mode="plain")
    for (kind, S, R, Ws), C in zip(blocks, got):
        ref = o.loop_cov(kind, S, R, Ws, 1, L)
        assert max_err_scaled(C, ref, cov_scale(kind, S, R, Ws, 1, L)) < 1e-12, kind


def test_cov_set_below_the_thresholds(ctx):
    """TTEE's 2 squared (0 0 0) windows and TEEE_PLANCK's 4 squared (2 -2 0) ones (fewer than
    the 9 needed at lmax 120) take the CUDA-core kernel for their Xi: the same arithmetic as the fused kernel,
    so the blocks agree with it to FP64 rounding of the final formula."""
    L = 120
    blocks = _inputs(L, ["TTEE", "TEEE_PLANCK"], seed=3)
    a = _run(ctx, blocks, 0, L)
    b = _run(ctx, blocks, 0, L, per_block=True)
    for (kind, S, R, Ws), x, y in zip(blocks, a, b):
        assert max_err_scaled(x, y, cov_scale(kind, S, R, Ws, 0, L)) < 1e-13, kind


def test_cov_set_argument_errors(ctx):
    from powerspectra_gpu._lib import PowerSpectraArgumentError
    L = 20
    d = torch.zeros(2 * L + 1, dtype=torch.float64, device="cuda")
    C = torch.zeros((L + 1, L + 1), dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    with pytest.raises(PowerSpectraArgumentError):  # not a kind
        ctx.coupledcov_set_device([(99, [p] * 4, [p] * 4, [p] * 8, C.data_ptr())], 2 * L + 1, 0, L, L + 1)
    with pytest.raises(PowerSpectraArgumentError):  # a NULL window
        ctx.coupledcov_set_device([("TTTT", [p] * 4, [p] * 4, [p] * 7 + [0], C.data_ptr())], 2 * L + 1, 0, L, L + 1)
    with pytest.raises(PowerSpectraArgumentError):  # a NULL output
        ctx.coupledcov_set_device([("TTEE", [p] * 4, [], [p] * 2, 0)], 2 * L + 1, 0, L, L + 1)
    with pytest.raises(PowerSpectraArgumentError):  # ldc too small
        ctx.coupledcov_set_device([("TTEE", [p] * 4, [], [p] * 2, C.data_ptr())], 2 * L + 1, 0, L, L)
