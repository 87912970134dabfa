"""The allocation-free entry point, checked against the context-based one.

ps_mcm_multi_device_noalloc exists for callers that may not allocate device
memory (their GPU memory is owned by another allocator, or they cannot take
the synchronisation that cudaMalloc/cudaFree may cause).  It must produce the
same matrices as ps_mcm_multi_device in chosen mode.  Two calls in a row with
different sizes and windows check that the shared fixed scratch carries
nothing from one call into the next.  The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import max_err_scaled

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-12  # same kernel as the context path: results agree to rounding (they are in fact identical)


def _noalloc_fn():
    import powerspectra_gpu._lib as L
    lib = L.load()
    fn = lib.ps_mcm_multi_device_noalloc
    fn.argtypes = [ctypes.c_uint, L._DPP, ctypes.c_int64, ctypes.c_int, ctypes.c_int, L._DPP, ctypes.c_int64,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn, L


def _case(L, lmin, seed, cases=0xF):
    from powerspectra_gpu import synthetic as syn
    nW = 2 * L + 1
    Ws = [syn.mask_spectrum(nW, 0.5 + 0.1 * s, 0.3 * L + 20, seed=seed + s) for s in range(4)]
    n = L - lmin + 1
    dW = [torch.tensor(w, device="cuda") for w in Ws]
    used = [s for s in range(4) if cases & (1 << s)]
    outs_new = {s: torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda") for s in used}
    outs_ref = {s: torch.zeros((n, n), dtype=torch.float64, device="cuda") for s in used}
    return nW, n, dW, outs_new, outs_ref


def _compare(fn, L, ctx, stream, lmax, lmin, seed, cases):
    nW, n, dW, new, ref = _case(lmax, lmin, seed, cases)
    ptr = lambda d: L.dptr_array([d[s].data_ptr() if s in d else 0 for s in range(4)])
    st = fn(cases, L.dptr_array([d.data_ptr() for d in dW]), nW, lmin, lmax, ptr(new), n,
            ctypes.c_void_p(stream.cuda_stream))
    assert st == 0
    ctx.mcm_multi_device({s: dW[s].data_ptr() for s in new}, nW, lmin, lmax, {s: ref[s].data_ptr() for s in ref}, n,
                         mode="chosen")
    torch.cuda.synchronize()
    for s in new:
        a, b = new[s].cpu().numpy(), ref[s].cpu().numpy()
        assert np.all(np.isfinite(a)), (lmax, lmin, s)  # every element written (NaN sentinel)
        assert max_err_scaled(a, b, np.abs(b)) < TOL, (lmax, lmin, s)


def test_noalloc_matches_context_path_twice(ctx):
    fn, L = _noalloc_fn()
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    try:
        for (lmax, lmin, seed) in ((300, 0, 11), (173, 2, 29)):
            _compare(fn, L, ctx, stream, lmax, lmin, seed, 0xF)
    finally:
        ctx.set_stream(0)


@pytest.mark.parametrize("lmin", [0, 37])
def test_noalloc_at_its_largest_lmax(ctx, lmin):
    """lmax 4095, the limit of the fixed scratch: with lmin = 0 the windows, their split copies
    and the task list fill their regions completely (264192 tasks)."""
    fn, L = _noalloc_fn()
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    try:
        _compare(fn, L, ctx, stream, 4095, lmin, 3 + lmin, 0x1)
    finally:
        ctx.set_stream(0)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    fn, L = _noalloc_fn()
    dW = [torch.zeros(10, dtype=torch.float64, device="cuda") for _ in range(4)]
    M = [torch.zeros(1, dtype=torch.float64, device="cuda") for _ in range(4)]
    st = fn(0x1, L.dptr_array([d.data_ptr() for d in dW]), 10, 0, 4096, L.dptr_array([m.data_ptr() for m in M]),
            4097, None)
    assert st == 1  # PS_ERR_ARG, before any GPU work
    st = fn(0x1, L.dptr_array([d.data_ptr() for d in dW]), 10, 5, 4, L.dptr_array([m.data_ptr() for m in M]), 1, None)
    assert st == 1
