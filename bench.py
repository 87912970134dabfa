#!/usr/bin/env python
"""Benchmark of the mode-coupling hot path: coupling elements per second.

Workload (default, --config all_spins_3071): every spin case of one (l1, l2)
grid at lmax 3071 with nW = 6143 -- M00 (TT) on the temperature mask spectrum,
M02 (TE) on the TxP cross-spectrum, M++ and M-- (EE/BB blocks) on the
polarisation mask spectrum: 4 matrices of 3072 x 3072 FP64 per step.  One step
is one pass of the hot path over that workload (one ps_mcm_multi_device call).

  value     whole-job elements/s with the spectra resident in HBM
  e2e       the same through the host-pointer C ABI call (ps_mcm_multi):
            pinned host spectra in, pinned host matrices out, copies timed
  roofline  the coupling kernel: algorithmic flops per launch / its CUDA-event
            time, against this GPU's FMA-pipe peak measured live by the
            library's probe kernel
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
    from powerspectra_gpu import synthetic as syn
    if name.startswith("all_spins_"):
        L = int(name.rsplit("_", 1)[1])  # all_spins_3071 is the benchmark; smaller ones are profiling cases
        c = syn.all_spins(L, seed=1 + 10 * rank)
        Ws = {0: c["WT"], 1: c["WTP"], 2: c["WP"], 3: c["WP"]}
        return {"name": name, "lmin": 0, "lmax": L, "nW": c["nW"], "Ws": Ws, "spectra": 3,
                "cases": ["TT (M00, W_T)", "TE (M02, W_TxP)", "EE/BB diagonal (M++, W_P)", "EE/BB off-diagonal (M--, W_P)"]}
    if name == "tt_767":
        c = syn.tt_767(seed=rank)
        return {"name": name, "lmin": 0, "lmax": 767, "nW": len(c["W"]), "Ws": {0: c["W"]}, "spectra": 1,
                "cases": ["TT (M00)"]}
    raise SystemExit("unknown --config %s" % name)


def flops_per_launch(wl, terms):
    spins = set(wl["Ws"])
    f = 0
    if spins & {0, 1}:
        f += FLOP_SPIN0
    if spins & {1, 2, 3}:
        f += FLOP_SPIN2
    f += FLOP_CONTRACT * wl["spectra"]
    return f * terms


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


def cpu_baseline(wl, budget_rows_stride, nthreads=0):
    """Oracle (reference algorithm: one family fill + dot per pair and spin case, OpenMP
    dynamic rows) on every stride-th l1 row; elements/s extrapolated by l3-term share."""
    from oracle import oracle as o
    lmin, lmax, nW = wl["lmin"], wl["lmax"], wl["nW"]
    rows = list(range(lmin, lmax + 1, budget_rows_stride))
    t0 = time.perf_counter()
    for s, W in wl["Ws"].items():
        o.inner_mcm(s, W, lmin, lmax, rows=rows, nthreads=nthreads)
    dt = time.perf_counter() - t0
    share = o.l3_terms(lmin, lmax, nW, rows) / o.l3_terms(lmin, lmax, nW)
    n = lmax - lmin + 1
    elements = len(wl["Ws"]) * n * n
    threads = nthreads or o.max_threads()
    return {"value": elements * share / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "every %d-th l1 row (%d rows, %.2f%% of the l3-terms), %d spin cases as separate passes, "
                      "%.1f s, scaled by l3-term share" % (budget_rows_stride, len(rows), 100 * share,
                                                            len(wl["Ws"]), dt)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = workload(args.config)
    stride = {"tt_767": 2}.get(args.config, 16)
    for _ in range(args.warmup):
        cpu_baseline(wl, stride)
    vals = [cpu_baseline(wl, stride) for _ in range(args.steps)]
    value = statistics.median(v["value"] for v in vals)
    n = wl["lmax"] - wl["lmin"] + 1
    ms = len(wl["Ws"]) * n * n / value * 1e3
    cb = dict(vals[-1])
    cb["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl["name"], "lmax": wl["lmax"], "nW": wl["nW"], "cases": wl["cases"],
                       "implementation": "C/OpenMP restatement of the reference algorithm (Julia is not installed)"},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _accuracy(ctx, wl, got, ref):
    """Max elementwise relative error of `got` (chosen) against `ref` (plain FP64) per spin
    case, on the device.  TE elements are measured against the Cauchy-Schwarz bound of
    their sum of |terms|, sqrt(M00(|W|) (M++(|W|) + M--(|W|))), computed in FP64."""
    import torch
    out = {}
    names = {0: "TT", 1: "TE", 2: "EE_BB_pp", 3: "EE_BB_mm"}
    for s in sorted(got):
        den = ref[s].abs()
        if s == 1:
            import numpy as np
            A = np.abs(wl["Ws"][1])
            n = wl["lmax"] - wl["lmin"] + 1
            m = ctx.mcm_multi({0: A, 2: A, 3: A}, wl["lmin"], wl["lmax"], mode="plain")
            b = torch.from_numpy(np.sqrt(np.abs(m[0] * (m[2] + m[3]))).T.copy()).to(ref[s].device)
            den = torch.maximum(den, b.reshape(n, n))
        den = torch.where(den == 0, torch.ones_like(den), den)
        out[names[s]] = float(((got[s] - ref[s]).abs() / den).max().item())
    return out


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
    spins = sorted(wl["Ws"])
    mode = args.mode
    ctx = pg.Context(local)
    # one real (non-default) stream shared by torch and the library, so the CUDA
    # events below bracket the library's kernels
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    dW = {s: torch.tensor(wl["Ws"][s], device="cuda") for s in spins}
    dM = {s: torch.empty((n, n), dtype=torch.float64, device="cuda") for s in spins}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    wptr = {s: dW[s].data_ptr() for s in spins}
    mptr = {s: dM[s].data_ptr() for s in spins}

    def step(m=mode, outp=mptr):
        ctx.mcm_multi_device(wptr, nW, lmin, lmax, outp, n, mode=m)

    peak64 = ctx.fma_peak(fp64=True)
    peak32 = ctx.fma_peak(fp64=False)
    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        step()
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
        step()
        kernel_ms.append(ctx.last_kernel_ms())  # coupling kernel only, events on this stream
    t1.record(stream)
    barrier()
    launches = ctx.launch_count() - n_launch0
    clk = clocks.stop()
    elapsed = max_over_ranks(t0.elapsed_time(t1) / 1e3)
    elements = len(spins) * n * n
    value = world * elements * args.steps / elapsed

    # the plain FP64 kernel on the same workload (the chosen form's comparison point)
    plain = None
    if mode == "chosen" and not args.no_plain:
        pM = {s: torch.empty((n, n), dtype=torch.float64, device="cuda") for s in spins}
        pptr = {s: pM[s].data_ptr() for s in spins}
        step("plain", pptr)
        torch.cuda.synchronize()
        ksteps = max(1, min(args.steps, 2))
        pk = []
        barrier()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(ksteps):
            flush.zero_()
            step("plain", pptr)
            pk.append(ctx.last_kernel_ms())
        p1.record(stream)
        barrier()
        pel = max_over_ranks(p0.elapsed_time(p1) / 1e3)
        acc = _accuracy(ctx, wl, dM, pM) if rank == 0 else None
        plain = {"value": world * elements * ksteps / pel, "unit": UNIT, "kernel_ms_per_launch": statistics.mean(pk),
                 "steps": ksteps}
        plain["chosen_over_plain"] = value / plain["value"]
        plain["max_rel_err_chosen_vs_fp64"] = acc
        del pM

    # end to end through the host-pointer ABI: pinned spectra in, pinned matrices out
    hW = {s: torch.from_numpy(np.ascontiguousarray(wl["Ws"][s])).pin_memory().numpy() for s in spins}
    hM = {s: torch.empty((n, n), dtype=torch.float64).pin_memory().numpy().T for s in spins}  # F-ordered views
    ctx.set_stream(0)
    ctx.mcm_multi(hW, lmin, lmax, mode=mode, outs=hM)  # warm the host path
    barrier()
    e0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.mcm_multi(hW, lmin, lmax, mode=mode, outs=hM)
    barrier()
    e_el = max_over_ranks(time.perf_counter() - e0)
    e2e = {"value": world * elements * args.steps / e_el, "unit": UNIT,
           "h2d_bytes_per_step": int(sum(min(len(hW[s]), 2 * lmax + 1) * 8 for s in spins)),
           "d2h_bytes_per_step": int(elements * 8)}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    terms = l3_terms(lmin, lmax, nW)
    fl = flops_per_launch(wl, terms)
    kms = statistics.mean(kernel_ms)
    peak = peak64 if mode == "plain" else peak32
    achieved = fl / (kms * 1e-3)
    # DRAM bytes per launch from one ncu capture of this kernel at this size
    # (profiles/coupling_chosen_all_spins_3071_dram.md); bench.py cannot run ncu itself
    traffic = 2.468e8 if (wl["name"] == "all_spins_3071" and mode == "chosen") else None
    roofline = {"bound": "fp64_fma_pipe" if mode == "plain" else "fp32_fma_pipe",
                "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one capture of the same kernel "
                                  "and workload" if traffic else None,
                "peak_source": "measured live by the library's FMA-chain probe kernel (MEASURED_PEAKS.json has no "
                               "CUDA-core FP64/FP32 figure)",
                "algorithmic_flops_per_launch": fl, "l3_terms_per_family": terms,
                "flops_per_l3_term": fl / terms, "kernel_ms_per_launch": kms}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if mode == "plain" else "f32",
            "data": "synthetic",
            "config": {"workload": wl["name"], "lmax": lmax, "nW": nW, "matrices_per_step": len(spins),
                       "cases": wl["cases"], "mode": mode, "per_rank": "independent problem per GPU",
                       "l2": "256 MiB buffer written between timed steps"},
            "roofline": roofline, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
            "fma_peaks_tflops": {"fp64": peak64 / 1e12, "fp32": peak32 / 1e12}}
    if plain is not None:
        line["plain_fp64"] = plain
    if world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(wl, {"tt_767": 1}.get(args.config, 3))
    print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


SET_CONFIGS = ("batched_64", "large_8191", "cov_2508")


def _set_problems(name, lmax=0):
    """Host-side definition of the multi-matrix configurations.

    batched_64: 64 problems, lmax drawn from {511, ..., 6143}, K in 1..16 seeded mask
      spectra each, spin 0 (M00 per spectrum) or spin 2 (M++ and M-- per spectrum).
    large_8191: lmax 8191, nW 16383, K = 20 spectra; spectrum k gives TT (k % 3 == 0),
      EE = M++ (k % 3 == 1) or BB = M-- (k % 3 == 2): 20 matrices of 8192^2, 10.7 GB.
    """
    from powerspectra_gpu import synthetic as syn
    if name == "batched_64":
        out = []
        for pr in syn.batched_problems():
            out.append({"lmin": 0, "lmax": pr["lmax"], "cases": 0x1 if pr["spin"] == 0 else 0xC,
                        "nW": pr["lmax"] + 1, "W": pr["W"]})
        return out
    if name == "large_8191":
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
        jobs, outs_c, outs_p = [], [], []
        windows = set()
        for (a, b) in blocks:
            kind, S, R, Ws = pg.covariance.gather(a, b, ws, spectra, noise)
            windows.update(id(w) for w in Ws)
            jobs.append((kind, [dev(x) for x in S], [dev(x) for x in R], [dev(x) for x in Ws]))
            outs_c.append(torch.empty((n, n), dtype=torch.float64, device="cuda"))
            outs_p.append(torch.empty((n, n), dtype=torch.float64, device="cuda"))

        def run(mode, outs):
            for (kind, S, R, Ws), C in zip(jobs, outs):
                ctx.coupledcov_device(kind, [x.data_ptr() for x in S], [x.data_ptr() for x in R],
                                      [x.data_ptr() for x in Ws], n, 0, L, C.data_ptr(), n, mode=mode)
        elements = len(jobs) * n * n
        line["config"].update({"lmax": L, "blocks": ["%s%s" % bl for bl in blocks],
                               "windows": sum(len(j[3]) for j in jobs), "distinct_windows": len(windows)})
        chosen = lambda: run("chosen", outs_c)
        plain = lambda: run("plain", outs_p)
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
        # the set of spectra on one grid (large_8191) runs as one ps_mcm_set_device call per spin case;
        # the uneven batch (batched_64) as one persistent launch replayed from a CUDA graph, with
        # the per-problem ps_mcm_set_device calls timed beside it
        chosen = sequential_chosen if args.config == "large_8191" else ctx.batch_graph_launch
        other = ctx.batch_graph_launch if args.config == "large_8191" else sequential_chosen
        other_name = "batched_graph" if args.config == "large_8191" else "sequential_chosen"
        line["config"]["chosen_path"] = ("ps_mcm_set_device per spin case" if args.config == "large_8191"
                                         else "ps_batch_graph_launch (persistent kernel)")
        for _ in range(args.warmup):
            other()
        line[other_name] = {"value": elements / ev_time(other, args.steps), "unit": UNIT}
        # three rows of every matrix from the other path, to check the timed path's results against
        seq_rows = [c[[0, c.shape[0] // 2, c.shape[0] - 1]].clone() for c, _ in mats]
    for _ in range(max(args.warmup, 3)):
        chosen()
    t_c = ev_time(chosen, args.steps)
    if args.config != "cov_2508":
        d = 0.0
        for (c, _), r in zip(mats, seq_rows):
            b = c[[0, c.shape[0] // 2, c.shape[0] - 1]]
            den = torch.maximum(r.abs(), 1e-9 * r.abs().max())
            den = torch.where(den == 0, torch.ones_like(den), den)
            d = max(d, float(((b - r).abs() / den).max().item()))
        line[other_name]["max_rel_diff_vs_timed_path"] = d
    line.update({"metric": METRIC, "value": elements / t_c, "ms_per_step": t_c * 1e3, "steps": args.steps,
                 "elements_per_step": elements, "mode": "chosen"})
    if not args.no_plain:
        plain()
        t_p = ev_time(plain, 1)
        errs = []
        for c, q in mats:
            den = torch.maximum(q.abs(), 1e-9 * q.abs().max())
            den = torch.where(den == 0, torch.ones_like(den), den)
            errs.append(float(((c - q).abs() / den).max().item()))
        line["plain_fp64"] = {"value": elements / t_p, "ms_per_step": t_p * 1e3, "steps": 1,
                              "chosen_over_plain": t_p / t_c, "max_rel_err_chosen_vs_fp64": max(errs)}
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
    ap.add_argument("--config", default="all_spins_3071")
    ap.add_argument("--mode", default="chosen", choices=("plain", "chosen"),
                    help="chosen: FP32-pipe recurrence with compensation (the product path); plain: FP64")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain FP64 kernel")
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
