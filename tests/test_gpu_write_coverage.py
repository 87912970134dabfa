"""Write coverage of the device entry points: every output element is written, and nothing
outside the matrices is.  Outputs start as NaN with a leading dimension larger than the matrix;
afterwards the matrix holds no NaN and the padding rows are still all NaN.  This is the
NaN-sentinel check that stands in for a race/bounds sanitizer on this GPU pool."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PAD = 5


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), device="cuda")


def _sentinel(n):
    """Column-major n x n matrix with leading dimension n + PAD, as a (n, n + PAD) row-major tensor."""
    return torch.full((n, n + PAD), float("nan"), dtype=torch.float64, device="cuda")


def _check(t, n):
    a = t.cpu().numpy()
    assert not np.isnan(a[:, :n]).any(), "an element of the matrix was not written"
    assert np.isnan(a[:, n:]).all(), "a write landed outside the matrix"


@pytest.mark.parametrize("mode", ["plain", "chosen"])
@pytest.mark.parametrize("lmin,lmax", [(0, 70), (2, 129), (5, 33)])
def test_mcm_multi_device(ctx, mode, lmin, lmax):
    from powerspectra_gpu import synthetic as syn
    c = syn.all_spins(lmax)
    dW = {0: _dev(c["WT"]), 1: _dev(c["WTP"]), 2: _dev(c["WP"]), 3: _dev(c["WP"])}
    n = lmax - lmin + 1
    out = {s: _sentinel(n) for s in range(4)}
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.mcm_multi_device({s: d.data_ptr() for s, d in dW.items()}, len(c["WT"]), lmin, lmax,
                             {s: t.data_ptr() for s, t in out.items()}, n + PAD, mode=mode)
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(0)
    for s in range(4):
        _check(out[s], n)


@pytest.mark.parametrize("kind", ["TTTT", "EEEE", "TETE", "TTTE", "TEEE", "TEEE_PLANCK", "TTEE"])
def test_coupledcov_device(ctx, kind):
    from oracle import oracle as o
    from powerspectra_gpu import synthetic as syn
    L = 90
    rng = np.random.default_rng(3)
    S = [_dev(1.0 + rng.random(L + 1)) for _ in range(4)]
    R = [_dev(1.0 + rng.random(L + 1)) for _ in range(o.COV_NRATIOS[kind])]
    Ws = [_dev(syn.mask_spectrum(2 * L + 1, 0.5, 40.0, seed=k)) for k in range(o.COV_NWINDOWS[kind])]
    n = L + 1
    C = _sentinel(n)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.coupledcov_device(kind, [x.data_ptr() for x in S], [x.data_ptr() for x in R], [w.data_ptr() for w in Ws],
                              2 * L + 1, 0, L, C.data_ptr(), n + PAD, mode="chosen")
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(0)
    _check(C, n)


def test_batch_run(ctx):
    from powerspectra_gpu import synthetic as syn
    probs, outs = [], []
    for i, (lmin, lmax, cases) in enumerate([(0, 64, 0xF), (3, 100, 0xC), (0, 45, 0x1), (1, 80, 0x2)]):
        n = lmax - lmin + 1
        Ws = [_dev(syn.mask_spectrum(lmax + 1, 0.5, 30.0, seed=10 * i + k)) for k in range(2)]
        M = [_sentinel(n) if cases & (1 << s) else None for k in range(2) for s in range(4)]
        probs.append({"lmin": lmin, "lmax": lmax, "cases": cases, "nW": lmax + 1, "ldm": n + PAD,
                      "W": [w.data_ptr() for w in Ws], "M": [m.data_ptr() if m is not None else 0 for m in M],
                      "_keep": (Ws, M)})
        outs.append((n, M))
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        ctx.batch_prepare(probs)
        ctx.batch_run()
        torch.cuda.synchronize()
    finally:
        ctx.set_stream(0)
    for n, M in outs:
        for m in M:
            if m is not None:
                _check(m, n)
