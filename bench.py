#!/usr/bin/env python
"""Benchmark of the mode-coupling hot path: coupling elements per second.

Workload (default, --config large_8191): the large coupling set at lmax 8191,
nW 16383 -- 20 seeded mask spectra, spectrum k giving TT (M00, k % 3 == 0),
EE (M++, k % 3 == 1) or BB (M--, k % 3 == 2): 20 matrices of 8192 x 8192 FP64
(10.7 GB) per step, computed by ONE ps_mcm_set_device call (the (window, case)
slots not wanted are NULL).  --config all_spins_3071 is the secondary headline:
every spin case of one grid at lmax 3071 (M00, M02, M++, M--) through one
ps_mcm_multi_device call.

  value     whole-job elements/s with the spectra resident in HBM
  e2e       the same through the host-pointer C ABI call (ps_mcm_set /
            ps_mcm_multi): pinned host spectra in, pinned host matrices out,
            copies inside the timed region
  roofline  the coupling kernels: algorithmic flops per step / their
            CUDA-event time, against this GPU's FMA-pipe peak measured live by
            the library's probe kernel
  plain_fp64  the plain FP64 kernels on the same workload, the chosen/plain
            ratio, and the max relative error of every chosen matrix against
            its FP64 counterpart (relative to |FP64| -- all terms are >= 0 -- or,
            for TE, to the Cauchy-Schwarz bound of its sum of |terms|; no floor)
  decoupled  max relative error of the decoupled spectrum M \\ pCl solved with
            the chosen M against the FP64 M (ps_solve), pCl = M_fp64 C_true
  cpu_baseline  the C/OpenMP oracle (the reference algorithm restated) on a
            row sample of the same workload, on the host cores

Multi-GPU (torchrun, one rank per GPU): every rank computes its own
independent problem (weak scaling); no collective touches the data path.
--impl reference times the CPU restatement of the reference algorithm.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "powerspectra.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "coupling elements/sec (l1,l2 pairs×spectra), chosen vs plain FP64 GPU, at ≤1e-6 rel err"
UNIT = "elements/s"
# Canonical algorithmic flops per l3-term (fixed accounting, sqrt and division count as one flop):
FLOP_SPIN0 = 8 + 1          # two-term 00 recurrence
FLOP_SPIN2 = 14 + 1 + 1     # three-term 22 recurrence
FLOP_CONTRACT = 3           # per mask spectrum: product/square, (2 l3 + 1) weight, FMA
L2_FLUSH_BYTES = 256 << 20  # > 126 MB L2


def l3_terms(lmin, lmax, nW):
    """l3-terms of one family summed over the pairs lmin <= l1 <= l2 <= lmax, l3 <= nW - 1."""
    import numpy as np
    tot = 0
    for l1 in range(lmin, lmax + 1):
        l2 = np.arange(l1, lmax + 1)
        hi = np.minimum(l1 + l2, nW - 1)
        tot += int(np.clip(hi - (l2 - l1) + 1, 0, None).sum())
    return tot


def workload(name, rank=0):
    """The headline workloads.  kind "multi": one ps_mcm_multi call, spin case s on window Ws[s];
    kind "set": one ps_mcm_set call over `windows` with the (window, case) `slots`."""
    from powerspectra_gpu import synthetic as syn
    if name.startswith("all_spins_"):
        L = int(name.rsplit("_", 1)[1])  # all_spins_3071 is configuration 2; smaller ones are profiling cases
        c = syn.all_spins(L, seed=1 + 10 * rank)
        Ws = {0: c["WT"], 1: c["WTP"], 2: c["WP"], 3: c["WP"]}
        return {"name": name, "kind": "multi", "lmin": 0, "lmax": L, "nW": c["nW"], "Ws": Ws, "spectra": 3,
                "slots": [(s, s) for s in range(4)], "windows": [Ws[s] for s in range(4)],
                "cases": ["TT (M00, W_T)", "TE (M02, W_TxP)", "EE/BB diagonal (M++, W_P)",
                          "EE/BB off-diagonal (M--, W_P)"]}
    if name == "tt_767":
        c = syn.tt_767(seed=rank)
        return {"name": name, "kind": "multi", "lmin": 0, "lmax": 767, "nW": len(c["W"]), "Ws": {0: c["W"]},
                "spectra": 1, "slots": [(0, 0)], "windows": [c["W"]], "cases": ["TT (M00)"]}
    if name.startswith("large_"):
        L = int(name.rsplit("_", 1)[1])  # large_8191 is configuration 5; smaller ones are profiling cases
        big = syn.large_set(lmax=L, seed=5 + 10 * rank)
        slots = [(k, (0, 2, 3)[k % 3]) for k in range(len(big["W"]))]
        return {"name": name, "kind": "set", "lmin": 0, "lmax": L, "nW": big["nW"], "windows": big["W"],
                "spectra": len(big["W"]), "slots": slots, "cases_mask": 0xD,
                "cases": ["%d spectra: TT (M00) for k %% 3 == 0, EE (M++) for k %% 3 == 1, BB (M--) for k %% 3 == 2"
                          % len(big["W"])]}
    raise SystemExit("unknown --config %s" % name)


CASE_NAMES = {0: "TT", 1: "TE", 2: "EE_pp", 3: "BB_mm"}


def flops_per_step(wl, terms):
    """Canonical flops of one step: each family the slots need once per l3-term, and the contraction
    once per distinct spectrum (++ and -- of one spectrum split its terms by parity)."""
    spins = set(s for _, s in wl["slots"])
    f = 0
    if spins & {0, 1}:
        f += FLOP_SPIN0
    if spins & {1, 2, 3}:
        f += FLOP_SPIN2
    f += FLOP_CONTRACT * wl["spectra"]
    return f * terms


def _profile_traffic(workload_name, mode):
    """DRAM bytes per step of the coupling kernels from a committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        rec = json.load(open(path)).get(workload_name, {}).get(mode)
    except (OSError, ValueError):
        return None, None
    if not rec:
        return None, None
    return rec["bytes_per_step"], "profiles/dram_traffic.json: " + rec["command"]


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline(wl, stride, nthreads=0, offset=0):
    """Oracle (reference algorithm: one family fill + dot per pair and (window, spin case) slot,
    OpenMP dynamic rows) on every stride-th l1 row from lmin + offset; elements/s scaled by the
    l3-term share of the sampled rows."""
    from oracle import oracle as o
    lmin, lmax, nW = wl["lmin"], wl["lmax"], wl["nW"]
    rows = list(range(lmin + offset % stride, lmax + 1, stride))
    t0 = time.perf_counter()
    for k, s in wl["slots"]:
        o.inner_mcm(s, wl["windows"][k], lmin, lmax, rows=rows, nthreads=nthreads)
    dt = time.perf_counter() - t0
    share = o.l3_terms(lmin, lmax, nW, rows) / o.l3_terms(lmin, lmax, nW)
    n = lmax - lmin + 1
    elements = len(wl["slots"]) * n * n
    threads = nthreads or o.max_threads()
    return {"value": elements * share / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "seconds": dt, "sampled_fraction": share,
            "sample": "every %d-th l1 row (%d rows, %.3f%% of the l3-terms), %d (window, spin case) slots as "
                      "separate passes, %.1f s, scaled by l3-term share" % (stride, len(rows), 100 * share,
                                                                          len(wl["slots"]), dt)}


# l1-row stride of the oracle samples: (cpu_baseline leg of our arm, one step of the reference arm)
CPU_STRIDE = {"tt_767": (1, 2), "all_spins_3071": (3, 16), "large_8191": (512, 2048)}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference algorithm on the same workload.
    Each step times a bounded row sample (the sampled rows rotate from step to step); `value` is
    the sampled elements/s scaled by the l3-term share, and `ms_per_step` is the time a step
    actually took.  The full-step time is extrapolated and marked so."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = workload(args.config)
    stride = CPU_STRIDE.get(args.config, (3, 16))[1]
    for i in range(args.warmup):
        cpu_baseline(wl, stride, offset=7 * i)
    vals = [cpu_baseline(wl, stride, offset=7 * (args.warmup + i)) for i in range(args.steps)]
    value = statistics.median(v["value"] for v in vals)
    n = wl["lmax"] - wl["lmin"] + 1
    timed_s = sum(v["seconds"] for v in vals)
    cb = dict(vals[-1])
    cb["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": timed_s / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["name"], "lmax": wl["lmax"], "nW": wl["nW"], "cases": wl["cases"],
                       "implementation": "C/OpenMP restatement of the reference algorithm (Julia is not installed)"},
            "timed_seconds": timed_s, "extrapolated": True,
            "sampled_fraction": statistics.mean(v["sampled_fraction"] for v in vals),
            "ms_per_full_step_extrapolated": len(wl["slots"]) * n * n / value * 1e3,
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _accuracy(ctx, wl, got, ref):
    """Max elementwise relative error of `got` (chosen) against `ref` (plain FP64), per (window,
    case) slot, on the device, with no floor: relative to |ref| (every term of a squared family
    on a non-negative window is >= 0, so |ref| is the sum of |terms|), and for TE to the
    Cauchy-Schwarz bound of its sum of |terms|, sqrt(M00(|W|) (M++(|W|) + M--(|W|))), in FP64."""
    import numpy as np
    import torch
    out = {}
    n = wl["lmax"] - wl["lmin"] + 1
    for slot in wl["slots"]:
        k, s = slot
        den = ref[slot].abs()
        if s == 1 or (wl["windows"][k] < 0).any():
            A = np.abs(wl["windows"][k])
            m = ctx.mcm_multi({0: A, 2: A, 3: A}, wl["lmin"], wl["lmax"], mode="plain")
            b = m[s] if s != 1 else np.sqrt(np.abs(m[0] * (m[2] + m[3])))
            den = torch.maximum(den, torch.from_numpy(b.T.copy()).to(ref[slot].device).reshape(n, n))
        den = torch.where(den == 0, torch.ones_like(den), den)
        out[slot] = float(((got[slot] - ref[slot]).abs() / den).max().item())
    return out


def _decoupled(ctx, wl, got, ref, extra):
    """Max relative error of decoupled spectra: pCl = M_fp64 C_true, then M \\ pCl by ps_solve
    (FP64 LU on the GPU) with the chosen M and with the FP64 M (src/modecoupling.jl:358,
    src/blockspectralmatrix.jl:124-129).  TT: M00 of the first TT slot.  EE/BB: the block
    [[M++, M--], [M--, M++]] of one spectrum on l >= 2 (the 2x2 block of mcm(:EE_BB),
    src/modecoupling.jl:210-216).  TE: M02 on l >= 2.  `extra(k, s, mode)` supplies a missing
    block of spectrum k as a device tensor."""
    import numpy as np
    lmin, lmax = wl["lmin"], wl["lmax"]
    ls = np.arange(lmin, lmax + 1, dtype=np.float64)
    base = ((ls + 2.0) / 80.0) ** -2.4
    C = {"TT": 1000.0 * base, "EE": 40.0 * base, "BB": 4.0 * base, "TE": 0.3 * np.sqrt(1000.0 * 40.0) * base}

    def host(t):  # the device tensor holds the column-major matrix: its transpose is M
        return np.asfortranarray(t.cpu().numpy().T)

    def err(Mc, Mp, c):
        p = Mp @ c
        xc, xp = ctx.solve(Mc, p), ctx.solve(Mp, p)
        return {"max_rel_err_chosen_vs_fp64": float(np.max(np.abs(xc - xp) / np.abs(xp))),
                "max_rel_err_fp64_vs_truth": float(np.max(np.abs(xp - c) / np.abs(c)))}

    res = {}
    tt = [sl for sl in wl["slots"] if sl[1] == 0]
    if tt:
        r = err(host(got[tt[0]]), host(ref[tt[0]]), C["TT"])
        r["system"] = "M00 of spectrum %d, l = %d..%d" % (tt[0][0], lmin, lmax)
        res["TT"] = r
    cut = max(0, 2 - lmin)
    te = [sl for sl in wl["slots"] if sl[1] == 1]
    if te:
        r = err(host(got[te[0]])[cut:, cut:], host(ref[te[0]])[cut:, cut:], C["TE"][cut:])
        r["system"] = "M02 of spectrum %d, l = %d..%d" % (te[0][0], lmin + cut, lmax)
        res["TE"] = r
    pp = [sl for sl in wl["slots"] if sl[1] == 2]
    if pp:
        k = pp[0][0]
        mats = {}
        for mode, src in (("chosen", got), ("plain", ref)):
            Mpp = host(src[k, 2])[cut:, cut:]
            Mmm = host(src[k, 3] if (k, 3) in src else extra(k, 3, mode))[cut:, cut:]
            mats[mode] = np.block([[Mpp, Mmm], [Mmm, Mpp]])
        c = np.concatenate([C["EE"][cut:], C["BB"][cut:]])
        r = err(np.asfortranarray(mats["chosen"]), np.asfortranarray(mats["plain"]), c)
        m = len(c) // 2
        p = mats["plain"] @ c
        xc, xp = ctx.solve(np.asfortranarray(mats["chosen"]), p), ctx.solve(np.asfortranarray(mats["plain"]), p)
        rel = np.abs(xc - xp) / np.abs(xp)
        r.update({"EE": float(rel[:m].max()), "BB": float(rel[m:].max()),
                  "system": "[[M++, M--], [M--, M++]] of spectrum %d, l = %d..%d" % (k, lmin + cut, lmax)})
        res["EE_BB"] = r
    return res


def run_ours(args):
    import numpy as np
    import torch
    import powerspectra_gpu as pg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        tt = torch.tensor([x], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        return float(tt.item())

    wl = workload(args.config, rank)
    lmin, lmax, nW = wl["lmin"], wl["lmax"], wl["nW"]
    n = lmax - lmin + 1
    slots = wl["slots"]
    K = len(wl["windows"])
    mode = args.mode
    ctx = pg.Context(local)
    # one real (non-default) stream shared by torch and the library, so the CUDA
    # events below bracket the library's kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    dW = [torch.tensor(w, device="cuda") for w in wl["windows"]]
    dM = {sl: torch.empty((n, n), dtype=torch.float64, device="cuda") for sl in slots}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def ptrs(mats):
        if wl["kind"] == "multi":
            return {s: mats[k, s].data_ptr() for k, s in slots}
        out = [0] * (4 * K)
        for k, s in slots:
            out[4 * k + s] = mats[k, s].data_ptr()
        return out

    def step(m=mode, mats=dM, outp=None):
        outp = outp or ptrs(mats)
        if wl["kind"] == "multi":
            ctx.mcm_multi_device({s: dW[k].data_ptr() for k, s in slots}, nW, lmin, lmax, outp, n, mode=m)
        else:
            ctx.mcm_set_device(wl["cases_mask"], [d.data_ptr() for d in dW], nW, lmin, lmax, outp, n, mode=m)

    mptr = ptrs(dM)
    peak64 = ctx.fma_peak(fp64=True)
    peak32 = ctx.fma_peak(fp64=False)
    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        step(outp=mptr)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    kernel_ms = []
    n_launch0 = ctx.launch_count()
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        flush.zero_()
        step(outp=mptr)
        kernel_ms.append(ctx.last_kernel_ms())  # the coupling kernels of this call, events on this stream
    t1.record(stream)
    barrier()
    launches = ctx.launch_count() - n_launch0
    clk = clocks.stop()
    elapsed = max_over_ranks(t0.elapsed_time(t1) / 1e3)
    elements = len(slots) * n * n
    value = world * elements * args.steps / elapsed

    # the same chosen-mode call with the tensor-core kernels switched off (CUDA-core contraction in
    # groups of up to 8 slots): two timed steps, for the comparison of the two contraction paths
    cuda_cores = None
    if mode == "chosen" and wl["kind"] == "set" and not args.no_plain:
        ctx.set_tensor_cores(False)
        step(outp=mptr)
        ck = []
        barrier()
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        for _ in range(2):
            flush.zero_()
            step(outp=mptr)
            ck.append(ctx.last_kernel_ms())
        c1.record(stream)
        barrier()
        ctx.set_tensor_cores(True)
        cel = max_over_ranks(c0.elapsed_time(c1) / 1e3)
        cuda_cores = {"value": world * elements * 2 / cel, "unit": UNIT, "ms_per_step": cel / 2 * 1e3,
                      "kernel_ms_per_step": statistics.mean(ck), "steps": 2,
                      "what": "the same ps_mcm_set_device call with ps_set_tensor_cores(ctx, 0)"}
        step(outp=mptr)  # the timed path's results again, for the accuracy legs below
        torch.cuda.synchronize()

    # the plain FP64 kernels on the same workload (the chosen form's comparison point): one timed
    # step (the kernels run for seconds, so no warm-up), then every chosen matrix against it
    plain = decoupled = None
    if mode == "chosen" and not args.no_plain:
        pM = {sl: torch.empty((n, n), dtype=torch.float64, device="cuda") for sl in slots}
        pptr = ptrs(pM)
        ksteps = 1 if lmax > 4095 else max(1, min(args.steps, 2))
        pk = []
        barrier()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(ksteps):
            flush.zero_()
            step("plain", outp=pptr)
            pk.append(ctx.last_kernel_ms())
        p1.record(stream)
        barrier()
        pel = max_over_ranks(p0.elapsed_time(p1) / 1e3)
        plain = {"value": world * elements * ksteps / pel, "unit": UNIT, "kernel_ms_per_step": statistics.mean(pk),
                 "ms_per_step": pel / ksteps * 1e3, "steps": ksteps}
        plain["chosen_over_plain"] = value / plain["value"]
        if rank == 0:
            acc = _accuracy(ctx, wl, dM, pM)
            per_case = {}
            for (k, s), e in acc.items():
                per_case[CASE_NAMES[s]] = max(per_case.get(CASE_NAMES[s], 0.0), e)
            plain["max_rel_err_chosen_vs_fp64"] = per_case
            plain["max_rel_err_per_matrix"] = [{"spectrum": k, "case": CASE_NAMES[s], "max_rel_err": acc[k, s]}
                                               for k, s in slots]
            plain["error_measure"] = ("max over all elements of |chosen - fp64| / |fp64| (TE: / Cauchy-Schwarz "
                                      "bound of the sum of |terms|); no floor")
            if not args.no_decoupled:
                def extra(k, s, m):
                    t = torch.empty((n, n), dtype=torch.float64, device="cuda")
                    ctx.mcm_multi_device({s: dW[k].data_ptr()}, nW, lmin, lmax, {s: t.data_ptr()}, n, mode=m)
                    torch.cuda.synchronize()
                    return t
                decoupled = _decoupled(ctx, wl, dM, pM, extra)
        del pM

    # end to end through the host-pointer ABI: pinned spectra in, pinned matrices out, every step
    e2e = None
    if args.no_e2e:
        pass
    else:
        e2e = _run_e2e(ctx, wl, args, barrier, max_over_ranks, world, elements)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    return _finish(ctx, wl, args, mode, kernel_ms, peak64, peak32, world, elapsed, value, clk, launches, plain,
                   decoupled, e2e, dist, cuda_cores)


def _run_e2e(ctx, wl, args, barrier, max_over_ranks, world, elements):
    """e2e leg: the host-pointer ABI call with pinned spectra in and pinned matrices out."""
    import numpy as np
    import torch
    lmin, lmax, nW = wl["lmin"], wl["lmax"], wl["nW"]
    n = lmax - lmin + 1
    slots = wl["slots"]
    mode = args.mode
    hW = [torch.from_numpy(np.ascontiguousarray(w)).pin_memory().numpy() for w in wl["windows"]]
    hM = {sl: torch.empty((n, n), dtype=torch.float64, pin_memory=True).numpy().T for sl in slots}  # F-ordered
    ctx.set_stream(0)

    def host_step():
        if wl["kind"] == "multi":
            ctx.mcm_multi({s: hW[k] for k, s in slots}, lmin, lmax, mode=mode, outs={s: hM[k, s] for k, s in slots})
        else:
            ctx.mcm_set(wl["cases_mask"], hW, lmin, lmax, mode=mode, outs=hM, slots=set(slots))
    host_step()  # warm the host path
    barrier()
    kms = 0.0
    e0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
        kms += ctx.last_kernel_ms()  # the call has synchronised: its coupling kernels' CUDA-event time
    barrier()
    e_el = max_over_ranks(time.perf_counter() - e0)
    nuse = min(nW, 2 * lmax + 1)
    e2e = {"value": world * elements * args.steps / e_el, "unit": UNIT,
           "h2d_bytes_per_step": int(len(set(k for k, _ in slots)) * nuse * 8),
           "d2h_bytes_per_step": int(elements * 8),
           "call": "ps_mcm_multi" if wl["kind"] == "multi" else "ps_mcm_set",
           "how": "pinned host spectra in; pinned host matrices out, written by the kernel in place",
           "kernel_ms_per_step": kms / args.steps}
    del hM
    return e2e


def _finish(ctx, wl, args, mode, kernel_ms, peak64, peak32, world, elapsed, value, clk, launches, plain, decoupled,
            e2e, dist, cuda_cores=None):
    lmin, lmax, nW = wl["lmin"], wl["lmax"], wl["nW"]
    slots = wl["slots"]
    terms = l3_terms(lmin, lmax, nW)
    fl = flops_per_step(wl, terms)
    kms = statistics.mean(kernel_ms)
    peak = peak64 if mode == "plain" else peak32
    achieved = fl / (kms * 1e-3)
    traffic, traffic_src = _profile_traffic(wl["name"], mode)
    roofline = {"bound": "fp64_fma_pipe" if mode == "plain" else "fp32_fma_pipe",
                "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": traffic_src,
                "peak_source": "measured live by the library's FMA-chain probe kernel (MEASURED_PEAKS.json has no "
                               "CUDA-core FP64/FP32 figure)",
                "algorithmic_flops_per_step": fl, "l3_terms_per_family": terms,
                "flops_per_l3_term": fl / terms, "kernel_ms_per_step": kms,
                "kernels": "the coupling kernels of one call (CUDA events around them on the launching stream)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if mode == "plain" else "f32",
            "data": "synthetic",
            "config": {"workload": wl["name"], "lmax": lmax, "nW": nW, "matrices_per_step": len(slots),
                       "cases": wl["cases"], "mode": mode, "per_rank": "independent problem per GPU",
                       "call": "ps_mcm_multi_device" if wl["kind"] == "multi" else "ps_mcm_set_device",
                       "l2": "256 MiB buffer written between timed steps"},
            "roofline": roofline, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
            "fma_peaks_tflops": {"fp64": peak64 / 1e12, "fp32": peak32 / 1e12}}
    if cuda_cores is not None:
        line["cuda_core_contraction"] = cuda_cores
        line["cuda_core_contraction"]["tensor_core_over_cuda_core"] = value / cuda_cores["value"]
    if plain is not None:
        line["plain_fp64"] = plain
    if decoupled is not None:
        line["decoupled"] = decoupled
    if world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(wl, CPU_STRIDE.get(args.config, (3, 16))[0])
    print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


SET_CONFIGS = ("batched_64", "batched_small_256", "large_set", "cov_2508")


def _set_problems(name, lmax=0):
    """Host-side definition of the multi-matrix configurations.

    batched_64: 64 problems, lmax drawn from {511, ..., 6143}, K in 1..16 seeded mask
      spectra each, spin 0 (M00 per spectrum) or spin 2 (M++ and M-- per spectrum).
    batched_small_256: 256 small problems, lmax drawn from {64, ..., 1023}, K in 1..4, spin 0
      or 2: the persistent queue against one launch per window group and per-problem calls.
    large_set: the large_8191 workload (lmax 8191, nW 16383, K = 20 spectra; spectrum k gives
      TT (k % 3 == 0), EE = M++ (k % 3 == 1) or BB = M-- (k % 3 == 2): 20 matrices of 8192^2,
      10.7 GB) as one ps_mcm_set_device call per spin case, against the persistent batch graph.
    """
    from powerspectra_gpu import synthetic as syn
    if name in ("batched_64", "batched_small_256"):
        out = []
        for pr in (syn.batched_problems() if name == "batched_64" else syn.small_batch()):
            out.append({"lmin": 0, "lmax": pr["lmax"], "cases": 0x1 if pr["spin"] == 0 else 0xC,
                        "nW": pr["lmax"] + 1, "W": pr["W"]})
        return out
    if name == "large_set":
        big = syn.large_set(lmax=lmax or 8191)
        groups = {0x1: [], 0x4: [], 0x8: []}
        for k, W in enumerate(big["W"]):
            groups[(0x1, 0x4, 0x8)[k % 3]].append(W)
        return [{"lmin": 0, "lmax": big["lmax"], "cases": c, "nW": big["nW"], "W": Ws} for c, Ws in groups.items()]
    raise SystemExit("unknown set config %s" % name)


def run_set(args):
    """Secondary configurations (parity-test cases, measured on request): the chosen path
    against the plain FP64 path on the same device-resident inputs, plus the max relative
    error of every chosen matrix against its FP64 counterpart."""
    import numpy as np
    import torch
    import powerspectra_gpu as pg
    from powerspectra_gpu import synthetic as syn

    torch.cuda.set_device(0)
    ctx = pg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    keep = []

    def dev(a):
        t = torch.tensor(np.ascontiguousarray(a), device="cuda")
        keep.append(t)
        return t

    def ev_time(fn, steps):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / steps

    line = {"config": {"workload": args.config if not args.lmax else "%s (lmax %d)" % (args.config, args.lmax)},
            "unit": UNIT}
    if args.config == "cov_2508":
        L = 2508
        ws, spectra, noise = syn.covariance_inputs(L)
        blocks = syn.COV_BLOCKS
        n = L + 1
        jobs, outs_c, outs_p, outs_b = [], [], [], []
        windows = set()
        for (a, b) in blocks:
            kind, S, R, Ws = pg.covariance.gather(a, b, ws, spectra, noise)
            windows.update(hash(np.ascontiguousarray(w).tobytes()) for w in Ws)  # distinct spectra by content
            jobs.append((kind, [dev(x) for x in S], [dev(x) for x in R], [dev(x) for x in Ws]))
            outs_c.append(torch.empty((n, n), dtype=torch.float64, device="cuda"))
            outs_p.append(torch.empty((n, n), dtype=torch.float64, device="cuda"))
            outs_b.append(torch.empty((n, n), dtype=torch.float64, device="cuda"))

        def run_set(mode, outs):  # one ps_coupledcov_set_device call for the six blocks
            ctx.coupledcov_set_device([(kind, [x.data_ptr() for x in S], [x.data_ptr() for x in R],
                                        [x.data_ptr() for x in Ws], C.data_ptr())
                                       for (kind, S, R, Ws), C in zip(jobs, outs)], n, 0, L, n, mode=mode)

        def run_blocks(mode, outs):  # one ps_coupledcov_device call per block
            for (kind, S, R, Ws), C in zip(jobs, outs):
                ctx.coupledcov_device(kind, [x.data_ptr() for x in S], [x.data_ptr() for x in R],
                                      [x.data_ptr() for x in Ws], n, 0, L, C.data_ptr(), n, mode=mode)
        elements = len(jobs) * n * n
        line["config"].update({"lmax": L, "blocks": ["%s%s" % bl for bl in blocks],
                               "windows": sum(len(j[3]) for j in jobs), "distinct_windows": len(windows),
                               "call": "ps_coupledcov_set_device"})
        chosen = lambda: run_set("chosen", outs_c)
        plain = lambda: run_set("plain", outs_p)
        mats = list(zip(outs_c, outs_p))
    else:
        probs = _set_problems(args.config, args.lmax)
        prob_dev, mats = [], []
        for pr in probs:
            n = pr["lmax"] - pr["lmin"] + 1
            dW = [dev(w) for w in pr["W"]]
            Mc, Mp, pc, pp = [], [], [], []
            for k in range(len(dW)):
                for s_ in range(4):
                    if pr["cases"] & (1 << s_):
                        c = torch.empty((n, n), dtype=torch.float64, device="cuda")
                        q = torch.empty((n, n), dtype=torch.float64, device="cuda") if not args.no_plain else None
                        Mc.append(c)
                        mats.append((c, q))
                        pc.append(c.data_ptr())
                        pp.append(q.data_ptr() if q is not None else 0)
                    else:
                        pc.append(0)
                        pp.append(0)
            keep.extend(Mc)
            prob_dev.append({"lmin": pr["lmin"], "lmax": pr["lmax"], "cases": pr["cases"], "nW": pr["nW"],
                             "ldm": n, "W": [d.data_ptr() for d in dW], "M": pc, "Mp": pp})
        elements = sum(int(c.shape[0]) ** 2 for c, _ in mats)
        tune = ctx.batch_autotune(prob_dev[:min(len(prob_dev), 8)]) if args.config == "batched_64" else None
        if args.config == "batched_small_256":
            # the persistent kernel (4-slot groups, full occupancy) against the launch form
            # (one launch per window group) on the same problems, each replayed from a CUDA graph
            forms = {}
            for name, bps in (("persistent", 0), ("launch_form", -1)):
                ctx.batch_prepare(prob_dev, group_slots=4, blocks_per_sm=bps)
                for _ in range(max(args.warmup, 3)):
                    ctx.batch_graph_launch()
                forms[name] = {"ms_per_step": ev_time(ctx.batch_graph_launch, args.steps) * 1e3}
                forms[name]["rows"] = [c[[0, c.shape[0] // 2, c.shape[0] - 1]].clone() for c, _ in mats]
            dd = 0.0
            for a, b in zip(forms["persistent"]["rows"], forms["launch_form"]["rows"]):
                den = torch.where(b == 0, torch.ones_like(b), b.abs())
                dd = max(dd, float(((a - b).abs() / den).max().item()))
            line["batch_forms"] = {k: {"ms_per_step": v["ms_per_step"]} for k, v in forms.items()}
            line["batch_forms"]["persistent_over_launch_form"] = (forms["launch_form"]["ms_per_step"]
                                                                  / forms["persistent"]["ms_per_step"])
            line["batch_forms"]["max_rel_diff"] = dd
            ctx.batch_prepare(prob_dev, group_slots=4, blocks_per_sm=0)
        else:
            ctx.batch_prepare(prob_dev)

        def plain():
            for pr in prob_dev:
                ctx.mcm_set_device(pr["cases"], pr["W"], pr["nW"], pr["lmin"], pr["lmax"], pr["Mp"], pr["ldm"],
                                   mode="plain")

        def sequential_chosen():
            for pr in prob_dev:
                ctx.mcm_set_device(pr["cases"], pr["W"], pr["nW"], pr["lmin"], pr["lmax"], pr["M"], pr["ldm"],
                                   mode="chosen")
        line["config"].update({"problems": len(probs), "matrices": len(mats),
                               "lmax": sorted(set(p["lmax"] for p in probs)), "autotune": tune})
        # the set of spectra on one grid (large_set) runs as one ps_mcm_set_device call per spin case;
        # the uneven batch (batched_64) as one persistent launch replayed from a CUDA graph, with
        # the per-problem ps_mcm_set_device calls timed beside it
        chosen = sequential_chosen if args.config == "large_set" else ctx.batch_graph_launch
        other = ctx.batch_graph_launch if args.config == "large_set" else sequential_chosen
        other_name = "batched_graph" if args.config == "large_set" else "sequential_chosen"
        line["config"]["chosen_path"] = ("ps_mcm_set_device per spin case" if args.config == "large_set"
                                         else "ps_batch_graph_launch (persistent kernel)")
        for _ in range(args.warmup):
            other()
        line[other_name] = {"value": elements / ev_time(other, args.steps), "unit": UNIT}
        # three rows of every matrix from the other path, to check the timed path's results against
        seq_rows = [c[[0, c.shape[0] // 2, c.shape[0] - 1]].clone() for c, _ in mats]
    for _ in range(max(args.warmup, 3)):
        chosen()
    t_c = ev_time(chosen, args.steps)
    if args.config == "cov_2508":
        # the same blocks as six separate ps_coupledcov_device calls (fused kernels only)
        blk = lambda: run_blocks("chosen", outs_b)
        blk()
        t_b = ev_time(blk, 2)
        # both chosen paths against each other, per block relative to its largest element (the
        # strict per-element error against FP64 is the plain_fp64 leg's)
        d = {}
        for (kind, _, _, _), c, q in zip(jobs, outs_c, outs_b):
            d[kind] = float(((c - q).abs().max() / q.abs().max()).item())
        line["per_block_calls"] = {"ms_per_step": t_b * 1e3, "steps": 2, "set_over_per_block": t_b / t_c,
                                   "max_abs_diff_over_block_max_vs_timed_path": d}
    else:
        d = 0.0
        for (c, _), r in zip(mats, seq_rows):
            b = c[[0, c.shape[0] // 2, c.shape[0] - 1]]
            den = torch.where(r == 0, torch.ones_like(r), r.abs())
            d = max(d, float(((b - r).abs() / den).max().item()))
        line[other_name]["max_rel_diff_vs_timed_path"] = d
    line.update({"metric": METRIC, "value": elements / t_c, "ms_per_step": t_c * 1e3, "steps": args.steps,
                 "elements_per_step": elements, "mode": "chosen"})
    if not args.no_plain:
        plain()
        t_p = ev_time(plain, 1)
        # strict error, no floor: |fp64| where every term is >= 0 (squared families on non-negative
        # windows, and the covariance blocks whose windows all use squared families); the TETE
        # block's 00x22 windows cancel, so it is measured on sampled rows against the oracle's
        # sum of |terms| of each element
        errs = []
        for i, (c, q) in enumerate(mats):
            if args.config == "cov_2508" and jobs[i][0] == "TETE":
                from oracle import oracle as o
                kind, S, R, Ws = jobs[i]
                rows = [0, 1, 2, 300, 1254, 2000, 2508]
                h = lambda t: t.cpu().numpy()
                sc = o.loop_cov(kind, [h(x) for x in S], [h(x) for x in R], [h(x) for x in Ws], 0, L, rows=rows,
                                absolute=True)
                cc, qq = h(c).T, h(q).T
                e = 0.0
                for r in rows:  # the oracle fills row r from the diagonal on
                    den = np.maximum(np.abs(qq[r, r:]), sc[r, r:])
                    den = np.where(den == 0, 1.0, den)
                    e = max(e, float(np.max(np.abs(cc[r, r:] - qq[r, r:]) / den)))
                errs.append(e)
                continue
            den = torch.where(q == 0, torch.ones_like(q), q.abs())
            errs.append(float(((c - q).abs() / den).max().item()))
        line["plain_fp64"] = {"value": elements / t_p, "ms_per_step": t_p * 1e3, "steps": 1,
                              "chosen_over_plain": t_p / t_c, "max_rel_err_chosen_vs_fp64": max(errs),
                              "error_measure": "|chosen - fp64| / |fp64| per element, no floor (TETE: sampled "
                                               "rows against the oracle's sum of |terms|)"}
    print(json.dumps(line))
    ctx.close()
    return 0


# dram__bytes_read.sum + dram__bytes_write.sum of k_alm2cl_partial for one cross spectrum at lmax 8191
# (ncu, one capture of this workload): 1.07 GB read + 10.7 MB partial sums written
WINDOW_TRAFFIC = 1.0807e9


def run_window(args):
    """window_W_8191: mask spectra W_l from harmonic coefficients (alm2cl, window_function_W!).

    8 seeded coefficient sets at lmax = mmax = 8191 (33.6M complex coefficients, 537 MB each,
    a mask-like envelope in l) and the 36 spectra of all pairs i <= j, one ps_window_W_device
    call each: one step reads 8 auto sets once and 28 cross pairs twice, 34.4 GB.  The
    reduction is HBM-bound; the roofline is coefficient bytes read / kernel time against the
    measured HBM copy bandwidth."""
    import numpy as np
    import torch
    import powerspectra_gpu as pg
    from oracle import oracle as o

    L, nsets = args.lmax or 8191, 8
    torch.cuda.set_device(0)
    ctx = pg.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    nalm = o.n_alms(L, L)
    ls = torch.cat([torch.arange(m, L + 1, device="cuda", dtype=torch.float64) for m in range(L + 1)])
    env = torch.exp(-ls / 3000.0) / (ls + 1.0)
    gen = torch.Generator(device="cuda").manual_seed(8191)
    sets = []
    for _ in range(nsets):
        a = torch.randn((nalm, 2), dtype=torch.float64, device="cuda", generator=gen) * env[:, None]
        a[:L + 1, 1] = 0.0  # m = 0 coefficients of a real field are real
        sets.append(a)
    del ls, env
    pairs = [(i, j) for i in range(nsets) for j in range(i, nsets)]
    out = torch.empty((len(pairs), L + 1), dtype=torch.float64, device="cuda")
    bytes_step = sum((1 if i == j else 2) * nalm * 16 for i, j in pairs)

    def step():
        for q, (i, j) in enumerate(pairs):
            ctx.window_W_device([sets[i].data_ptr()], [sets[j].data_ptr()], L, L, L, out[q].data_ptr())

    def ev_time(fn, steps):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / steps

    for _ in range(max(args.warmup, 3)):
        step()
    clk = ClockSampler(0)
    launches0 = ctx.launch_count()
    t = ev_time(step, args.steps)
    launches = (ctx.launch_count() - launches0) // args.steps
    clocks = clk.stop()
    # one partial-sum launch alone, for the roofline (its share is nearly all of a call)
    probe = torch.empty(L + 1, dtype=torch.float64, device="cuda")
    t1s = []
    for _ in range(3):  # the partial-sum kernel alone, timed by the library's events on this stream
        ctx.window_W_device([sets[2].data_ptr()], [sets[3].data_ptr()], L, L, L, probe.data_ptr())
        torch.cuda.synchronize()
        t1s.append(ctx.last_kernel_ms() / 1e3)
    t1 = statistics.median(t1s)
    peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    ach = 2 * nalm * 16 / t1 / 1e9
    # parity at full size: one auto and one cross spectrum against the oracle (numpy, host)
    host = [sets[k].cpu().numpy().view(np.complex128).ravel() for k in (0, 1)]
    got = out.cpu().numpy()
    t0 = time.perf_counter()
    ref_cross = o.alm2cl(host[0], host[1], L)
    cpu_dt = time.perf_counter() - t0
    ref_auto = o.alm2cl(host[0], host[0], L)
    sc_cross = o.alm2cl(np.abs(host[0]).astype(complex), np.abs(host[1]).astype(complex), L)
    err = max(float(np.max(np.abs(got[1] - ref_cross) / sc_cross)),
              float(np.max(np.abs(got[0] - ref_auto) / np.abs(ref_auto))))
    # e2e: the host-pointer entry point, pinned host sets in, spectra out (each call copies its sets)
    hsets = [torch.empty((nalm, 2), dtype=torch.float64, pin_memory=True) for _ in range(3)]
    for k in range(3):
        hsets[k].copy_(sets[k])
    hw = np.empty(L + 1)
    e2e_pairs = [(0, 0), (0, 1), (1, 2)]
    t0 = time.perf_counter()
    for i, j in e2e_pairs:
        ctx.window_W([hsets[i].numpy().view(np.complex128).ravel()], [hsets[j].numpy().view(np.complex128).ravel()],
                     L)
    e2e_dt = time.perf_counter() - t0
    e2e_bytes = sum((1 if i == j else 2) * nalm * 16 for i, j in e2e_pairs)
    line = {"metric": "alm2cl coefficient bytes/s (window_function_W! mask spectra)", "value": bytes_step / t / 1e9,
            "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "window_W_%d" % L, "lmax": L, "mmax": L, "sets": nsets,
                                            "spectra_per_step": len(pairs), "bytes_per_step": bytes_step,
                                            "l2": "inputs (537 MB per set) larger than L2"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": WINDOW_TRAFFIC * nalm / o.n_alms(8191, 8191),  # scaled by the coefficients
                         "kernel": "k_alm2cl_partial, one cross spectrum",
                         "kernel_ms": t1 * 1e3, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
            "e2e": {"value": e2e_bytes / e2e_dt / 1e9, "unit": "GB/s", "h2d_bytes_per_step": e2e_bytes,
                    "d2h_bytes_per_step": 8 * (L + 1) * len(e2e_pairs),
                    "what": "ps_window_W on pinned host sets: 1 auto and 2 cross spectra"},
            "max_rel_err_vs_oracle": err, "clocks": clocks, "gpu_launches": launches,
            "cpu_baseline": {"value": 2 * nalm * 16 / cpu_dt / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                             "sample": "one cross spectrum at lmax %d with the oracle's numpy alm2cl, %.1f s"
                                       % (L, cpu_dt)}}
    print(json.dumps(line))
    ctx.close()
    return 0


QUICKPOL_REF_S = 3.951  # quickpolXi!, 1000 x 1000, band 100, nu = 0, s = 2: 20 Julia threads (reference notebook)


def run_quickpol(args):
    """quickpol_999: quickpolXi!(Xi, 0, 0, 2, 2, omega, omega) for a 1000 x 1000 Xi (l 0..999) with
    band (100, 100) and a scan-weight coefficient set of lmax = mmax = 30000 -- the configuration
    of the reference's QuickPol notebook.  The set is a 7.2 GB host array; only its rows with
    l <= 2 * 999 enter Xi (the 3j support), and those are seeded random values with a decaying
    envelope while the rest stay zero.  One step is one host call of ps_quickpol_xi_alm: packing
    of the used rows, the copy, quickpolW and Xi on the GPU, and the copy back into a page-locked Xi
    (allocated once, as a caller registers its output matrix)."""
    import numpy as np
    import powerspectra_gpu as pg
    from oracle import oracle as o

    lmax, band, alm_lmax = 999, 100, 30000
    nalm = o.n_alms(alm_lmax, alm_lmax)
    lw = 2 * lmax
    omega = np.zeros(nalm, dtype=np.complex128)  # untouched pages stay unallocated
    rng = np.random.default_rng(30000)
    for m in range(lw + 1):
        i0 = o.alm_index(m, m, alm_lmax)
        ls = np.arange(m, lw + 1)
        omega[i0:i0 + len(ls)] = (rng.normal(size=len(ls)) + 1j * rng.normal(size=len(ls))) * np.exp(-ls / 600.0) \
            / (1.0 + m)
    omega[:lw + 1] = omega[:lw + 1].real
    ctx = pg.Context(0)
    import torch
    Xout = torch.empty((lmax + 1, lmax + 1), dtype=torch.float64).pin_memory().numpy().T  # F-ordered, page-locked

    def timed(mode):
        for _ in range(max(args.warmup, 3)):
            ctx.quickpol_xi_alm(0, 0, 2, 2, omega, omega, alm_lmax, lmax, band, band, mode=mode, out=Xout)
        ts, ks = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            X = ctx.quickpol_xi_alm(0, 0, 2, 2, omega, omega, alm_lmax, lmax, band, band, mode=mode, out=Xout)
            ts.append(time.perf_counter() - t0)
            ks.append(ctx.last_kernel_ms())
        return X.copy(), statistics.median(ts), statistics.median(ks)

    Xp, t_plain, k_plain = timed("plain")
    clk = ClockSampler(0)
    launches0 = ctx.launch_count()
    X, t, k_chosen = timed(args.mode)
    clocks = clk.stop()
    launches = (ctx.launch_count() - launches0) // (args.steps + max(args.warmup, 3))
    # CPU: the oracle (quickpolW over the used rows in numpy, Xi in C/OpenMP on all host threads)
    packed = np.concatenate([omega[o.alm_index(m, m, alm_lmax):o.alm_index(m, m, alm_lmax) + lw + 1 - m]
                             for m in range(lw + 1)])
    t0 = time.perf_counter()
    W = o.quickpolW(packed, packed, lw)
    R = o.quickpol_xi(0, 0, 2, 2, W, lmax, band, band)
    cpu_dt = time.perf_counter() - t0
    scale = o.quickpol_xi(0, 0, 2, 2, W, lmax, band, band, absolute=True)  # sum of |terms| per element
    mask = scale > 0
    err = float(np.max(np.abs(X - R)[mask] / scale[mask]))
    err_plain = float(np.max(np.abs(Xp - R)[mask] / scale[mask]))
    line = {"metric": "quickpolXi! wall time per call (1000 x 1000, band 100, nu = 0, s = 2)", "value": t,
            "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": t * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": t / QUICKPOL_REF_S,
            "dtype": "f32" if args.mode == "chosen" else "f64", "data": "synthetic",
            "config": {"workload": "quickpol_999", "lmax": lmax, "band": [band, band], "nu": [0, 0], "s": [2, 2],
                       "alm_lmax": alm_lmax, "alm_mmax": alm_lmax,
                       "used_rows": "l <= %d (the 3j support); the rest of the set is zero" % lw,
                       "step": "ps_quickpol_xi_alm on host arrays: pack, copy, quickpolW + Xi kernels, copy back "
                               "into a page-locked Xi"},
            "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": 16 * o.n_alms(lw, lw),
                    "d2h_bytes_per_step": 8 * (lmax + 1) ** 2},
            "mode": args.mode, "kernel_ms": k_chosen,
            "max_err_vs_oracle": err, "err_scale": "sum of |W f1 f2| behind each element",
            "plain_fp64": {"value": t_plain, "unit": "s", "kernel_ms": k_plain, "max_err_vs_oracle": err_plain,
                           "chosen_over_plain": t_plain / t},
            "clocks": clocks,
            "gpu_launches": launches,
            "reference_published_s": QUICKPOL_REF_S,
            "cpu_baseline": {"value": cpu_dt, "unit": "s", "cores": o.max_threads(), "kind": "port",
                             "sample": "the whole configuration: oracle quickpolW (numpy) + Xi (C, OpenMP)"}}
    print(json.dumps(line))
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", default="large_8191")
    ap.add_argument("--mode", default="chosen", choices=("plain", "chosen"),
                    help="chosen: FP32-pipe recurrence with compensation (the product path); plain: FP64")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain FP64 kernel")
    ap.add_argument("--no-decoupled", action="store_true", help="skip the decoupled-spectrum error leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--lmax", type=int, default=0,
                    help="window_W_8191 and large_8191: another lmax (a smaller case for profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config in SET_CONFIGS:
        return run_set(args)
    if args.config == "window_W_8191":
        return run_window(args)
    if args.config == "quickpol_999":
        return run_quickpol(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
