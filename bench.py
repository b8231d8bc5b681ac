"""Benchmark of the EnKF-C analysis cycle (calc + update) on GB300.

Workload (default): workload 3, the largest that fits one GPU -- a 1000x1000
grid, 10 layers x 2 fields, 96 members, 2M uniform observations, ETKF,
radius 25 cells, stride 2 (250,000 local analyses per cycle; about 30 GB
resident).  --config 2 runs the 600x900 batched DEnKF workload (60,000
analyses).  Synthetic, seeded inputs (enkf-c_gb300/synth.py).

One step = one full cycle on the device with every input resident in HBM:
spatial index build, innovations (das_calcinnandspread), standardisation,
local-analysis transforms for all points, and the X5 update of all
field-layers.  `value` = local analyses per second of that cycle.

`e2e` = the same cycle through the host-buffer C ABI (HE, fields in pinned
host memory; T, w and the updated fields copied back), timed on the host.

Multi-GPU: the cycle does not exchange data between GPUs, so --gpus N runs N
independent replicas (one process per GPU); value = all analyses / max time.

--impl reference times the CPU restatement of the reference (oracle/) on the
host cores over a bounded random sample of the same workload, the threads
taking work units from a shared queue.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "enkf-c_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "local analyses/s (calc + update cycle)"

# DRAM bytes per local analysis from ncu captures of the current version of
# a kernel:
#   k_update_cells, workload 2 at half edge length (15,000 analyses):
#     462.6 MB (dram__bytes.sum.per_second x duration);
#   k_transforms_mixed, workload 3 at full size, three launches of one solve
#     batch (19,456 analyses each): 820.2 MB read + 1,450.1 MB written on
#     average (dram__bytes_read.sum, dram__bytes_write.sum).
# Traffic grows with the analyses (and, for the update, with the cells they
# cover), so a full launch scales by the analyses.  A kernel without a
# capture of its current version reports no traffic.
TRAFFIC_PER_ANALYSIS = {
    (2, "k_update_cells"): 462.6e6 / 15000,
    (3, "k_transforms_mixed"): (820.2e6 + 1450.1e6) / 19456,
}
UNIT = "analyses/s"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 6:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def aggregate(local_ms: float, local_units: int, world: int, device=None):
    """Replica aggregation across ranks: the job time is the slowest rank's
    time (all-reduce MAX), the work is the sum of every rank's units (all-
    reduce SUM).  Returns (max_ms, total_units).  Single process: identity."""
    if world <= 1:
        return local_ms, local_units
    import torch
    import torch.distributed as dist
    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), int(round(u.item()))


def workload(cfg: int, scale: float):
    import synth
    return synth.make(cfg, scale=scale)


def obs_tables(w):
    nl = np.ones(w.ntypes, np.int32)
    lr = np.zeros((w.ntypes, 8))
    lr[:, 0] = w.locrad
    lw = np.zeros((w.ntypes, 8))
    lw[:, 0] = 1.0
    return nl, lr, lw


def update_bytes(w, nfl):
    m = w.nmem
    cells = w.nj * w.ni
    fields = 2 * nfl * m * cells * 4
    x5 = w.nanalyses * (w.nmem_dynamic * m + m) * 4
    return fields + x5, fields, x5


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args, rank, world, local_rank):
    import torch

    import build as _b
    _b.build()
    import enkfg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    w = workload(args.config, args.scale)
    nfl = w.nfields * w.nlayers
    m = w.nmem
    path = enkfg.PATH_BATCHED if args.path == "batched" else enkfg.PATH_PLAIN
    prec = enkfg.PREC_MIXED if args.precision == "mixed" else enkfg.PREC_FP64

    ctx = enkfg.Enkfg(local_rank)
    nl, lr, lw = obs_tables(w)
    ctx.set_obstypes(nl, lr, lw, np.ones(w.ntypes))
    ctx.set_obs(w.lon, w.lat, w.otype, w.status, w.estd, w.value)
    ctx.set_grid(w.x, w.y, stride=w.stride)

    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    HE_d = torch.from_numpy(w.HE).to(dev)
    fields_h = np.ascontiguousarray(w.fields.reshape(nfl, m, w.nj, w.ni))
    fields_d = torch.from_numpy(fields_h).to(dev)
    numlev_d = torch.from_numpy(w.numlevels.astype(np.int32)).to(dev)
    levels = np.tile(np.arange(w.nlayers, dtype=np.int32), w.nfields)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # 256 MB > L2 (129 MB)
    torch.cuda.synchronize()

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def step(timed_parts=None, path=path, prec=prec):
        with torch.cuda.stream(stream):
            flush.zero_()
            if timed_parts is not None:
                timed_parts[0].record(stream)
            ctx.rebuild_index()
            ctx.set_HE_dev(HE_d.data_ptr(), m, w.nmem_dynamic)
            ctx.calcinnandspread(want=False)
            ctx.standardise()
            ctx.calctransforms_dev(mode=w.mode, scheme=w.scheme, alpha=w.alpha, path=path, precision=prec)
            if timed_parts is not None:
                timed_parts[1].record(stream)
            ctx.updatefields_dev(fields_d.data_ptr(), numlev_d.data_ptr(), nfl, levels, mode=w.mode, nmem=m,
                                 nmem_dynamic=w.nmem_dynamic, inflation=w.inflation, inf_ratio=w.inf_ratio,
                                 precision=prec)
            if timed_parts is not None:
                timed_parts[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    calc_ms, upd_ms, kern_ms, ukern_ms, fin_ms = [], [], [], [], []
    l0 = ctx.launches
    with ClockSampler(local_rank) as clk:
        ev[0].record(stream)
        for k in range(args.steps):
            parts = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            step(parts)
            stream.synchronize()
            calc_ms.append(parts[0].elapsed_time(parts[1]))
            upd_ms.append(parts[1].elapsed_time(parts[2]))
            # the library's CUDA events on the launching stream, summed over
            # the transform stage's batches: the transform kernels
            # (kernel_times [0]), the solve kernels after them ([1]); the
            # update kernel(s) (stage_times [3])
            st_ms = ctx.stage_times()
            kt = ctx.kernel_times()
            kern_ms.append(kt[0])
            fin_ms.append(kt[1])
            ukern_ms.append(st_ms[3])
        ev[1].record(stream)
        torch.cuda.synchronize()
    launches = ctx.launches - l0
    total_ms, units = aggregate(ev[0].elapsed_time(ev[1]), w.nanalyses * args.steps, world, dev)

    # the same cycle replayed from a CUDA graph: everything after the index
    # build (HE copy, innovations, standardisation, gather, transforms,
    # update) captured once on the context's stream; the index build (host
    # round trips for the bucket grid) stays eager before each replay
    graph = None
    if args.graph:
        def cycle():
            ctx.set_HE_dev(HE_d.data_ptr(), m, w.nmem_dynamic)
            ctx.calcinnandspread(want=False)
            ctx.standardise()
            ctx.calctransforms_dev(mode=w.mode, scheme=w.scheme, alpha=w.alpha, path=path, precision=prec)
            ctx.updatefields_dev(fields_d.data_ptr(), numlev_d.data_ptr(), nfl, levels, mode=w.mode, nmem=m,
                                 nmem_dynamic=w.nmem_dynamic, inflation=w.inflation, inf_ratio=w.inf_ratio,
                                 precision=prec)
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(stream):
                ctx.rebuild_index()
            stream.synchronize()
            with torch.cuda.graph(g, stream=stream):
                cycle()
            gl0 = ctx.launches
            for _ in range(args.warmup):
                with torch.cuda.stream(stream):
                    flush.zero_()
                    ctx.rebuild_index()
                    g.replay()
            torch.cuda.synchronize()
            ge = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ge[0].record(stream)
            for _ in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                    ctx.rebuild_index()
                    g.replay()
            ge[1].record(stream)
            torch.cuda.synchronize()
            gms, gunits = aggregate(ge[0].elapsed_time(ge[1]), w.nanalyses * args.steps, world, dev)
            graph = {"value": gunits / (gms / 1e3), "ms_per_step": gms / args.steps,
                     "captured": "HE copy, innovations, standardisation, gather, transforms, update",
                     "eager": "index build"}
            del g
        except Exception as exc:   # report, do not hide: the eager numbers stand
            graph = {"error": str(exc)[:300]}
    # the plain GPU FP64 path (one CTA per analysis, in-kernel eigensolver)
    # on the same cycle, for the batched-mixed vs plain comparison
    plain64 = None
    if args.compare_fp64 and not (path == enkfg.PATH_PLAIN and prec == enkfg.PREC_FP64):
        step(path=enkfg.PATH_PLAIN, prec=enkfg.PREC_FP64)
        torch.cuda.synchronize()
        pe = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        npl = 1
        pe[0].record(stream)
        for _ in range(npl):
            step(path=enkfg.PATH_PLAIN, prec=enkfg.PREC_FP64)
        pe[1].record(stream)
        torch.cuda.synchronize()
        pms = pe[0].elapsed_time(pe[1]) / npl
        plain64 = {"value": w.nanalyses / (pms / 1e3), "ms_per_step": pms, "path": "plain", "precision": "fp64",
                   "steps": npl}
        step()   # back to the measured path's state for what follows
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms_per_step = total_ms / args.steps
    value = units / (total_ms / 1e3)

    # rooflines.  Transform kernel (the dominant one): algorithmic FLOPs =
    # sum over points of 2 m^2 p + 2 m p (S'S as a full m x m product and
    # S's), over the kernel's own CUDA-event time.  FP64 path: against the
    # nominal FP64 rate (FP64 is not among the measured peaks).  Mixed path:
    # against the measured bf16 rate / 2 (dense TF32); the tensor work it
    # issues per algorithmic flop is reported beside it (per group of 8
    # observations: 4 MMAs of 128 x N x 8 in the stacked form, N <= 64,
    # else 6).  Update kernel: fields read + written and X5 read once, over
    # its CUDA-event time, against the measured HBM copy bandwidth.
    # traffic: DRAM bytes (read + write) per analysis from an ncu capture of
    # the kernel (TRAFFIC_PER_ANALYSIS), scaled to the launch's analyses.
    peaks, peak_src = load_peaks()
    calc_t = statistics.median(calc_ms) / 1e3
    upd_t = statistics.median(upd_ms) / 1e3
    kern_t = statistics.median(kern_ms) / 1e3
    ukern_t = statistics.median(ukern_ms) / 1e3
    ub, _, _ = update_bytes(w, nfl)
    counts = ctx.findlocal(lists=False).astype(np.float64)
    flops = float((2.0 * m * m * counts + 2.0 * m * counts).sum())
    kname = "k_transforms_mixed" if prec == enkfg.PREC_MIXED else "k_transforms"
    if prec == enkfg.PREC_MIXED:
        N = (m + 15) // 16 * 16
        nmma = 4 if N <= 64 else 6
        issued = float((nmma * 2.0 * 128 * N * 8 * np.ceil(counts / 8.0)).sum())
        roof = {"kernel": kname, "bound": "tensor", "achieved": flops / kern_t / 1e12,
                "peak": peaks["bf16_tflops"] / 2.0, "unit": "TFLOP/s",
                "peak_source": f"{peak_src} bf16 {peaks['bf16_tflops']} / 2 (dense TF32)",
                "mma_per_8_obs": nmma, "issued_per_algorithmic_flop": issued / flops,
                "issued_tflops": issued / kern_t / 1e12}
    else:
        roof = {"kernel": kname, "bound": "fp64", "achieved": flops / kern_t / 1e12, "peak": 1.25,
                "unit": "TFLOP/s", "peak_source": "GB300 nominal FP64 (FP64 is not among the measured peaks)"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    tpa = TRAFFIC_PER_ANALYSIS.get((w.cfg, kname))
    roof["traffic"] = tpa * w.nanalyses if tpa else None
    if tpa is None:
        roof["traffic_note"] = "no ncu capture of this version of the kernel"
    roof["kernel_ms"] = kern_t * 1e3
    roof["solve_kernels_ms"] = statistics.median(fin_ms)
    roof["flops_per_launch"] = flops
    ukname = "k_update_cells" if m <= 64 else "k_update_v3"
    upa = TRAFFIC_PER_ANALYSIS.get((w.cfg, ukname))
    uroof = {"kernel": ukname, "bound": "hbm",
             "traffic": upa * w.nanalyses if upa else None,
             "achieved": ub / ukern_t / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
             "frac": ub / ukern_t / 1e9 / peaks["hbm_gbs"], "bytes_per_launch": ub, "kernel_ms": ukern_t * 1e3,
             "peak_source": peak_src}

    # the forward operator on the device (das_getHE; H_surf_standard with
    # bilinear interpolation): HE [m][nobs] of the observed layer (field 0,
    # layer 0) from the resident ensemble, one launch per observation type.
    # Algorithmic bytes: the observed layer read once and HE written once.
    def measure_he():
        ctx.set_obs_positions(w.lon.astype(np.float64), w.lat.astype(np.float64))
        layer = fields_d[0]                                  # [m][nj][ni]
        hb = layer.numel() * 4 + m * w.nobs * 4

        def he_pass(evs=None):
            ctx.begin_HE(m, w.nmem_dynamic)
            with torch.cuda.stream(stream):
                flush.zero_()
            if evs:
                evs[0].record(stream)
            for t in range(w.ntypes):
                ctx.map_obs_dev(t, layer.data_ptr(), m, w.ni, w.nj, numlev_d.data_ptr(), stream=stream.cuda_stream)
            if evs:
                evs[1].record(stream)
            ctx.finish_HE()

        for _ in range(3):
            he_pass()
        he_ms = []
        for _ in range(5):
            evs = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            he_pass(evs)
            torch.cuda.synchronize()
            he_ms.append(evs[0].elapsed_time(evs[1]))
        ht = statistics.median(he_ms) / 1e3
        return {"kernel": "k_map_obs", "ms": ht * 1e3, "launches_per_pass": w.ntypes,
                "obs_member_values_per_s": w.nobs * m / ht, "bytes_per_pass": hb, "achieved_gbs": hb / ht / 1e9,
                "peak_gbs": peaks["hbm_gbs"], "frac": hb / ht / 1e9 / peaks["hbm_gbs"]}

    # the observation-impact adjoint on workload 4 (the grid and observations
    # of workload 2, 64 members, J = sum over wet cells of (analysis mean -
    # verifying field)^2): the forward transforms (batched mixed, as the
    # cycle runs them), then the adjoint of the mean update and of the
    # transforms -- the FP32 production form and the FP64 form
    def measure_adjoint():
        w4 = workload(4, args.scale)
        c4 = enkfg.Enkfg(local_rank)
        try:
            nl4, lr4, lw4 = obs_tables(w4)
            c4.set_obstypes(nl4, lr4, lw4, np.ones(w4.ntypes))
            c4.set_obs(w4.lon, w4.lat, w4.otype, w4.status, w4.estd, w4.value)
            c4.set_HE(w4.HE)
            c4.calcinnandspread(want=False)
            c4.standardise()
            c4.set_grid(w4.x, w4.y, stride=w4.stride)
            layer = w4.fields[0, 0]
            wet = w4.numlevels > 0
            g = np.where(wet, 2.0 * (layer.astype(np.float64).mean(axis=0) - w4.verify), 0.0)
            res = {}
            for k in range(2):
                t0 = time.perf_counter()
                out = c4.calctransforms(mode=w4.mode, scheme=w4.scheme, path=enkfg.PATH_BATCHED,
                                        precision=enkfg.PREC_MIXED, want64=True, want_diag=False)
                t1 = time.perf_counter()
                wbar = c4.adjoint_mean(layer, g)
                t2 = time.perf_counter()
                g32 = c4.adjoint_transforms(wbar, mode=w4.mode, scheme=w4.scheme, precision=enkfg.PREC_MIXED)
                t3 = time.perf_counter()
                g64 = c4.adjoint_transforms(wbar, mode=w4.mode, scheme=w4.scheme, precision=enkfg.PREC_FP64)
                t4 = time.perf_counter()
                res = {"workload": workload_name(w4), "forward_ms": (t1 - t0) * 1e3, "adjoint_mean_ms": (t2 - t1) * 1e3,
                       "adjoint_fp32_ms": (t3 - t2) * 1e3, "adjoint_fp64_ms": (t4 - t3) * 1e3,
                       "fp32_vs_fp64_innov": float(np.linalg.norm(g32[0] - g64[0]) / np.linalg.norm(g64[0])),
                       "fp32_vs_fp64_var": float(np.linalg.norm(g32[1] - g64[1]) / np.linalg.norm(g64[1])),
                       "timing": "host wall clock around each call (host-buffer entry points, copies included), "
                                 "second of two runs"}
            return res
        finally:
            c4.close()

    adjoint = None
    if args.adjoint:
        try:
            adjoint = measure_adjoint()
        except Exception as exc:   # report, do not hide: the cycle's numbers stand
            adjoint = {"error": str(exc)[:300]}

    he_stage = None
    if args.he:
        try:
            he_stage = measure_he()
        except Exception as exc:   # report, do not hide: the cycle's numbers stand
            he_stage = {"error": str(exc)[:300]}

    # end to end through the host-buffer C ABI (pinned host memory)
    e2e = None
    if rank == 0 or world > 1:
        HE_pin = torch.from_numpy(w.HE).pin_memory().numpy()
        f_pin = torch.from_numpy(fields_h).pin_memory().numpy()
        ctx.set_stream(None)
        # caller-owned pinned outputs (as a host application would keep its
        # transform and field buffers); the fields are updated in place
        T_h = torch.empty((w.nj_s, w.ni_s, w.nmem_dynamic, m), dtype=torch.float32).pin_memory().numpy()
        W_h = torch.empty((w.nj_s, w.ni_s, m), dtype=torch.float32).pin_memory().numpy()

        def e2e_step():
            ctx.rebuild_index()
            ctx.set_HE(HE_pin, w.nmem_dynamic)
            ctx.calcinnandspread(want=False)
            ctx.standardise()
            out = ctx.calctransforms(mode=w.mode, scheme=w.scheme, alpha=w.alpha, path=path, precision=prec,
                                     want_diag=False, T_out=T_h if w.mode != enkfg.MODE_ENOI else None, w_out=W_h)
            res = ctx.updatefields(f_pin, w.numlevels, levels, mode=w.mode, nmem=m, nmem_dynamic=w.nmem_dynamic,
                                   inflation=w.inflation, inf_ratio=w.inf_ratio, precision=prec, inplace=True)
            return out, res

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ne = max(1, min(args.steps, 3))
        for _ in range(ne):
            out, res = e2e_step()
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / ne
        h2d = w.HE.nbytes + fields_h.nbytes + w.numlevels.size * 4
        d2h = out["w"].nbytes + (out["T"].nbytes if out["T"] is not None else 0) + res.nbytes
        e2e = {"value": w.nanalyses / te, "unit": UNIT, "ms_per_step": te * 1e3, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
        del T_h, W_h

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(w, args.cpu_units)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == enkfg.PREC_FP64 else "f32/tf32-split",
            "data": "synthetic (seeded, enkf-c_gb300/synth.py)",
            "config": {"workload": workload_name(w),
                       "local_analyses": w.nanalyses, "path": args.path, "precision": args.precision,
                       "parallelism": f"replicas x{world}",
                       "l2": f"256 MB flush before every step; fields ({fields_h.nbytes / 1e9:.2f} GB) exceed L2"},
            "stages_ms": {"calc": statistics.median(calc_ms), "update": statistics.median(upd_ms)},
            "update_gbs": ub / upd_t / 1e9,
            "calc_algorithmic_tflops": flops / calc_t / 1e12,
            "roofline": roof, "roofline_update": uroof, "graph": graph, "e2e": e2e, "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "plain_gpu_fp64": plain64,
            "he_stage": he_stage,
            "adjoint": adjoint,
            "speedup_vs_plain_gpu_fp64": (value / plain64["value"]) if plain64 else None,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    ctx.close()


# ---------------------------------------------------------------------------
# CPU (oracle) side
# ---------------------------------------------------------------------------
UNIT_COLS = 50   # strided columns in one CPU work unit (one queue item)


def cpu_sample(w, per_worker, threads, seed=0):
    """The calc + update cycle of the CPU restatement on a bounded sample:
    per-cycle set-up (kd-trees, innovations, standardisation) on the whole
    domain; the transforms of `per_worker` x `threads` work units (pieces of
    UNIT_COLS strided columns of one strided row, drawn at random over the
    domain) taken from a shared queue by the threads as they come free (the
    reference's dynamic mpiqueue schedule); and the update of the model rows
    of the sampled strided rows, all field-layers.  Returns a dict with the
    sample's analyses, model rows updated and the times (s)."""
    import concurrent.futures as cf

    import oracle
    t0 = time.perf_counter()
    nl, lr, lw = oracle.locrad_table(w.ntypes, w.locrad)
    obs = oracle.ObsSet(w.lon, w.lat, w.otype, w.status, w.ntypes, nl, lr, lw)
    S, s = oracle.prepare(w.HE, w.value, w.status, w.estd, w.otype, np.ones(w.ntypes))
    t_setup = time.perf_counter() - t0
    allu = [(jj, i0, min(i0 + UNIT_COLS, w.ni_s)) for jj in range(w.nj_s) for i0 in range(0, w.ni_s, UNIT_COLS)]
    rng = np.random.default_rng(seed)
    k = min(len(allu), max(1, per_worker * threads))
    units = [allu[i] for i in sorted(rng.choice(len(allu), k, replace=False))]
    n_an = sum(u[2] - u[1] for u in units)
    t0 = time.perf_counter()
    out = oracle.calctransforms(obs, mode=w.mode, scheme=w.scheme, nmem=w.nmem, nmem_dynamic=w.nmem_dynamic,
                                alpha=w.alpha, stride=w.stride, x=w.x, y=w.y, S=S, s=s, threads=threads,
                                want_diag=False, units=units)
    t_calc = time.perf_counter() - t0
    nfl = w.nfields * w.nlayers
    fl = w.fields.reshape(nfl, w.nmem, w.nj, w.ni)
    T = out["T"] if out["T"] is not None else np.zeros((w.nj_s, w.ni_s, 1, w.nmem), np.float32)
    rows = sorted({u[0] for u in units})

    def upd(args_):
        jj, f = args_
        j1 = jj * w.stride
        j2 = min(w.nj - 1, j1 + w.stride - 1)
        return oracle.updatefields(fl[f][:, j1:j2 + 1], T, out["w"], w.numlevels, mode=w.mode, nmem=w.nmem,
                                   nmem_dynamic=w.nmem_dynamic, stride=w.stride, level=f % w.nlayers,
                                   inflation=w.inflation, inf_ratio=w.inf_ratio, j1=j1, j2=j2)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(upd, [(jj, f) for jj in rows for f in range(nfl)]))
    t_upd = time.perf_counter() - t0
    return dict(analyses=n_an, units=len(units), rows=len(rows), setup=t_setup, calc=t_calc, update=t_upd)


def cpu_rate(w, smp):
    """Analyses/s of a full cycle from a sample: set-up once, the transforms
    scaled by analyses, the update by strided rows."""
    full = smp["setup"] + smp["calc"] * (w.nanalyses / smp["analyses"]) + smp["update"] * (w.nj_s / smp["rows"])
    return w.nanalyses / full, full


def cpu_sample_text(w, smp, threads, full):
    return (f"{smp['units']} work units of {UNIT_COLS} strided columns ({smp['analyses']} of {w.nanalyses} local "
            f"analyses, {threads} threads pulling from a shared queue) and the model rows of {smp['rows']} strided "
            f"rows x {w.nfields * w.nlayers} field-layers; set-up {smp['setup']:.2f} s, calc {smp['calc']:.2f} s, "
            f"update {smp['update']:.2f} s; scaled to the full cycle ({full:.1f} s): calc by analyses, update by "
            f"rows; C restatement of the reference (oracle/) + OpenBLAS, one thread per worker")


def cpu_baseline(w, per_worker):
    threads = os.cpu_count() or 1
    smp = cpu_sample(w, per_worker, threads)
    v, full = cpu_rate(w, smp)
    return {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": cpu_sample_text(w, smp, threads, full)}


def run_reference(args, rank, world):
    """The CPU restatement of the reference on the host cores.  Each step
    runs the per-cycle set-up on the whole domain and a bounded random sample
    of the transforms and the update (cpu_sample); value = the full cycle's
    analyses / its time scaled from the samples, ms_per_step = the measured
    wall time of a step (the sample)."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    w = workload(args.config, args.scale)
    threads = os.cpu_count() or 1
    for k in range(args.warmup):
        cpu_sample(w, 1, threads, seed=1000 + k)
    fulls, walls, smp = [], [], None
    for k in range(args.steps):
        t0 = time.perf_counter()
        smp = cpu_sample(w, args.cpu_units, threads, seed=k)
        walls.append(time.perf_counter() - t0)
        fulls.append(cpu_rate(w, smp)[1])
    value = w.nanalyses * len(fulls) / sum(fulls)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": workload_name(w), "path": "cpu", "parallelism": f"{threads} host threads"},
            "full_cycle_s": statistics.mean(fulls),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": cpu_sample_text(w, smp, threads, statistics.mean(fulls)) +
                             "; the reference's own build needs MPI and NetCDF, absent here"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_name(w):
    return (f"workload {w.cfg}: {w.ni}x{w.nj} grid, {w.nlayers} layers x {w.nfields} fields, m={w.nmem}"
            f"{f' ({w.nmem_dynamic} dynamic)' if w.nmem_dynamic < w.nmem else ''}, {w.nobs} obs, "
            f"{'DEnKF' if w.scheme == 0 else 'ETKF'}, radius {w.locrad:g}, stride {w.stride}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--path", default="batched", choices=["plain", "batched"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-units", type=int, default=8, help="CPU work units per host thread in a sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--graph", type=int, default=1, help="also time the cycle replayed from a CUDA graph")
    ap.add_argument("--compare-fp64", type=int, default=1, help="also time the plain GPU FP64 path")
    ap.add_argument("--he", type=int, default=1, help="also time the device forward operator (HE stage)")
    ap.add_argument("--adjoint", type=int, default=1, help="also time the observation-impact adjoint (workload 4)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_gpu(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
