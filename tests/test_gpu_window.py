"""Mask spectra from harmonic coefficients (alm2cl / window_function_W!,
src/workspace.jl:174-213) on the GPU against the oracle's alm2cl restatement.

FP64 sums of products: the bar is 1e-12 relative to the sum of |terms| of each
l (cross-spectra of random coefficients cancel)."""
import numpy as np
import pytest

from oracle import oracle as o

pytestmark = pytest.mark.gpu


def _alm(lmax, mmax, seed):
    rng = np.random.default_rng(seed)
    n = o.n_alms(lmax, mmax)
    a = rng.normal(size=n) + 1j * rng.normal(size=n)
    a[:lmax + 1] = a[:lmax + 1].real  # m = 0 coefficients of a real field are real
    return a * np.exp(-np.arange(n) % (lmax + 1) / 200.0)


def _abs_scale(A, B, lmax, mmax, lout):
    """The same mean on |a| |b|: no cancellation, so it bounds the sum of |terms|."""
    Aa = [None if a is None else np.abs(a).astype(complex) for a in A]
    Ba = [None if b is None else np.abs(b).astype(complex) for b in B]
    return o.window_function_W(Aa, Ba, lmax, mmax, lout)


@pytest.mark.parametrize("lmax,mmax,lout", [(0, 0, 0), (1, 1, 1), (127, 127, 127), (300, 300, 250), (513, 100, 513),
                                            (1000, 1000, 1000)])
def test_alm2cl_cross_and_auto(ctx, lmax, mmax, lout):
    a, b = _alm(lmax, mmax, 1), _alm(lmax, mmax, 2)
    for A, B in (([a], [b]), ([a], [a])):
        got = ctx.window_W(A, B, lmax, mmax, lout)
        ref = o.window_function_W(A, B, lmax, mmax, lout)
        sc = _abs_scale(A, B, lmax, mmax, lout)
        assert np.max(np.abs(got - ref) / sc) < 1e-12


def test_window_function_W_terms(ctx):
    """PP x PP: four (QQ/UU) x (QQ/UU) terms, the cross-field ones zero sets (None), mean over all four."""
    lmax = 400
    q, u, q2, u2 = (_alm(lmax, lmax, s) for s in (3, 4, 5, 6))
    A = [q, q, u, None]
    B = [q2, u2, q2, u2]
    got = ctx.window_W(A, B, lmax)
    ref = o.window_function_W(A, B, lmax)
    sc = _abs_scale(A, B, lmax, lmax, lmax)
    assert np.max(np.abs(got - ref) / sc) < 1e-12
    # all-zero terms count in the mean
    half = ctx.window_W([q, None], [q2, q2], lmax)
    np.testing.assert_allclose(half, 0.5 * ctx.window_W([q], [q2], lmax), rtol=1e-15, atol=0)


def test_known_answer_all_ones(ctx):
    """a_lm = 1 everywhere: cl[l] = (1 + 2 min(l, mmax)) / (2l + 1)."""
    lmax, mmax = 700, 300
    a = np.ones(o.n_alms(lmax, mmax), dtype=complex)
    l = np.arange(lmax + 1)
    np.testing.assert_allclose(ctx.window_W([a], [a], lmax, mmax),
                               (1.0 + 2.0 * np.minimum(l, mmax)) / (2.0 * l + 1.0), rtol=1e-14)


def test_device_variant_and_reproducible(ctx):
    import torch
    lmax = 2047
    a, b = _alm(lmax, lmax, 7), _alm(lmax, lmax, 8)
    da = torch.from_numpy(a.view(np.float64)).cuda()
    db = torch.from_numpy(b.view(np.float64)).cuda()
    dW = torch.empty(lmax + 1, dtype=torch.float64, device="cuda")
    ctx.window_W_device([da.data_ptr(), da.data_ptr()], [db.data_ptr(), None], lmax, lmax, lmax, dW.data_ptr())
    ctx.synchronize()
    got = dW.cpu().numpy()
    ref = o.window_function_W([a, a], [b, None], lmax)
    sc = _abs_scale([a, a], [b, None], lmax, lmax, lmax)
    assert np.max(np.abs(got - ref) / sc) < 1e-12
    ctx.window_W_device([da.data_ptr(), da.data_ptr()], [db.data_ptr(), None], lmax, lmax, lmax, dW.data_ptr())
    ctx.synchronize()
    assert np.array_equal(dW.cpu().numpy(), got)  # fixed summation order: bit-identical


def test_argument_errors(ctx):
    import powerspectra_gpu as pg
    import torch
    a = _alm(10, 10, 0)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.window_W([], [], 10)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.window_W([a] * 17, [a] * 17, 10)
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.window_W([a], [a], 10, 11)  # mmax > lmax
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.window_W([a], [a], 10, 10, 11)  # lout > lmax
    with pytest.raises(pg.PowerSpectraArgumentError):
        ctx.window_W([a[:-1]], [a], 10)
    buf = torch.zeros(2 * o.n_alms(10, 10) + 2, dtype=torch.float64, device="cuda")
    dW = torch.empty(11, dtype=torch.float64, device="cuda")
    with pytest.raises(pg.PowerSpectraArgumentError, match="aligned"):  # rejected on the host, nothing launched
        ctx.window_W_device([buf.data_ptr() + 8], [buf.data_ptr()], 10, 10, 10, dW.data_ptr())
    assert np.allclose(ctx.window_W([a], [a], 10), o.alm2cl(a, a, 10), rtol=1e-13)  # context still usable


def test_alm_workspace_feeds_coupledcov(ctx):
    """coupledcov with windows from coefficient sets (AlmWindowWorkspace) equals coupledcov with the
    oracle's window_function_W of the same sets; the cache returns the same array on a repeat."""
    import powerspectra_gpu as pg
    from gpu_util import cov_scale, max_err_scaled
    from powerspectra_gpu import synthetic as syn
    L = 96
    _, spectra, noise = syn.covariance_inputs(L)
    names = syn.FIELDS
    sets = {}

    def ew(A, i, j, alpha):
        if A not in ("∅∅", "II", "QQ", "UU") or (A != "∅∅" and i != j):
            return None  # effective_weight_alm!'s zero Alm for cross-field weights
        key = (A, i, j, alpha)
        if key not in sets:
            a = _alm(L, L, syn._key_seed(key) % 100000)
            a[0] = 4.0 + abs(a[0])  # a monopole-dominated mask-like spectrum
            sets[key] = a
        return sets[key]

    ws = pg.AlmWindowWorkspace(names, L, ew, ctx=ctx)
    W1 = ws.window_function_W("TT", "TT", names[0], names[2], "TT", names[1], names[3], "TT")
    assert ws.window_function_W("TT", "TT", names[0], names[2], "TT", names[1], names[3], "TT") is W1
    ref_ws = pg.WindowWorkspace(names, L, lambda X, Y, i, j, a, p, q, b: o.window_function_W(
        [ew(wx, i, j, a) for wx in pg.wterms(X) for wy in pg.wterms(Y)],
        [ew(wy, p, q, b) for wx in pg.wterms(X) for wy in pg.wterms(Y)], L))
    for ch in (("TT", "TT"), ("EE", "EE"), ("TE", "TE")):
        C = pg.coupledcov(*ch, ws, spectra, noise, mode="plain", ctx=ctx)
        kind, S, R, Ws = pg.covariance.gather(*ch, ref_ws, spectra, noise)
        ref = o.loop_cov(kind, S, R, Ws, 0, L)
        assert max_err_scaled(C.parent, ref, cov_scale(kind, S, R, Ws, 0, L)) < 1e-11, ch


def test_pinned_host_sets_read_in_place(ctx):
    """Page-locked coefficient sets are read by the kernel where they lie; same bits as copied sets."""
    import torch
    lmax = 700
    a, b = _alm(lmax, lmax, 21), _alm(lmax, lmax, 22)
    ref = ctx.window_W([a, a], [b, None], lmax)
    pa = torch.from_numpy(a.view(np.float64).copy()).pin_memory().numpy().view(np.complex128)
    pb = torch.from_numpy(b.view(np.float64).copy()).pin_memory().numpy().view(np.complex128)
    got = ctx.window_W([pa, pa], [pb, None], lmax)
    assert np.array_equal(got, ref)
    mixed = ctx.window_W([pa, a], [b, pb], lmax)  # one pinned and one pageable set per term
    np.testing.assert_allclose(mixed, 0.5 * (ctx.window_W([a], [b], lmax) + ctx.window_W([a], [b], lmax)), rtol=1e-15)
