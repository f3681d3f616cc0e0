"""Benchmark of the scalar-advection stage (MakeUtrans, VelPred, MakeEdgeScal, fluxes,
UpdateScal; MAC projection skipped) on the 3-D single-level workload: 256^3 cells in 64
boxes of 64^3, NumSpec = 13, ppm_type 1, w0 != 0 (seeded synthetic atmosphere).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` is advected cell-updates per second over all GPUs with the
inputs resident in HBM; ``e2e`` is the same metric through the public API with host
buffers copied in and the result copied out every step.  ``--impl reference`` times the
CPU restatement of the reference stage (the oracle) on this host's cores.  With torchrun
(N > 1) every rank advances its own independent copy of the workload (replicas: the stage
is single-GPU) and the value is the total over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "advected cell-updates/s (FP64, <=1e-12 rel) batched vs per-box; %HBM; adj/fwd"
UNIT = "cell-updates/s"
HBM_PEAK_FALLBACK = 6792.7

# Per-cell work of the kernels that bound the stage, counted by ncu on one batched stage of
# 128^3 cells in 8 boxes of 64^3, NumSpec 13, ppm_type 1 (the counts per valid cell do not
# depend on how many 64^3 boxes there are; summaries under profiles/):
#   fp64: FP64 warp instructions (smsp__inst_executed_pipe_fp64.sum) per valid cell, one launch
#   dram: DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per valid cell, one launch
KERNEL_WORK = {
    "k_ppm_cell<0,1,1>": {"fp64": 0.6582, "dram": 50.7},
    "k_ppm_cell<1,1,1>": {"fp64": 0.6467, "dram": 51.3},
    "k_ppm_cell<2,1,1>": {"fp64": 0.6482, "dram": 51.9},
    "k_ppm_cell<0,1,0>": {"fp64": 0.7034, "dram": 50.4},
    "k_ppm_cell<1,1,0>": {"fp64": 0.6736, "dram": 50.8},
    "k_ppm_cell<2,1,0>": {"fp64": 0.6502, "dram": 50.9},
    "k_update_rhox": {"fp64": 9.0, "dram": 675.0},
    "k_ppm_face<0,1>": {"fp64": 0.4189, "dram": 18.4},
    "k_ppm_face<1,1>": {"fp64": 0.4188, "dram": 19.0},
    "k_ppm_face<2,1>": {"fp64": 0.4287, "dram": 19.0},
    "k_es_edges<0,0,1>": {"fp64": 0.4433, "dram": 62.4},
    "k_es_edges<1,0,1>": {"fp64": 0.4191, "dram": 63.7},
    "k_es_edges<2,0,1>": {"fp64": 0.3989, "dram": 64.0},
}
STAGE_FP64_PER_CELL = 146.50  # FP64 warp instructions per valid cell, whole stage


def jsonable(o):
    """json.dumps default: numpy scalars and arrays as Python numbers and lists."""
    if isinstance(o, np.generic):
        return o.item()
    if isinstance(o, np.ndarray):
        return o.tolist()
    raise TypeError(f"not JSON serialisable: {type(o).__name__}")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


def demangle(name):
    """Short form of a madv kernel symbol: _ZN4madv10k_ppm_cellILi1ELi1ELi1EEEv... -> k_ppm_cell<1,1,1>."""
    import re
    m = re.match(r"_ZN4madv(\d+)", name)
    if not m:
        return name
    n = int(m.group(1))
    base = name[m.end():m.end() + n]
    pos = m.end() + n
    if name[pos:pos + 1] != "I":
        return base
    pos += 1
    args = []
    while True:
        a = re.match(r"L[ib](n?\d+)E", name[pos:])
        if not a:
            break
        args.append(a.group(1).replace("n", "-"))
        pos += a.end()
    return f"{base}<{','.join(args)}>"


def roofline(kern, ncell, stage_ms, fp64_tflops_probe, peaks, peak_kind):
    """FP64-issue roofline of the dominant kernel: the kernel (all its template instances:
    directions, PPM type, face or cell tracing velocity) with the most device time in one
    batched stage.

    achieved = FP64 warp instructions of its launches (per-cell counts x valid cells, from
    ncu) / their summed launch time (CUDA events around each launch); peak = the FP64 issue
    rate of the DFMA-chain probe run in this process (1 DFMA = 2 flops, so issue rate = probe
    TFLOP/s / 2).  Units: 10^12 FP64 lane-instructions per second (warp instructions x 32).
    """
    inst_of = {}
    fam = {}
    for k, (n, ms) in kern.items():
        d = demangle(k)
        inst_of.setdefault(d, [0, 0.0])
        inst_of[d][0] += n
        inst_of[d][1] += ms
        base = d.split("<")[0]
        fam.setdefault(base, {})[d] = inst_of[d]
    name, members = max(fam.items(), key=lambda kv: sum(v[1] for v in kv[1].values()))
    launches = sum(v[0] for v in members.values())
    ms = sum(v[1] for v in members.values())
    issue_peak = fp64_tflops_probe / 2.0  # T lane-instructions/s
    r = {"bound": "fp64", "kernel": name, "instances": sorted(members), "unit": "T FP64 lane-inst/s",
         "launches": launches, "mean_launch_ms": ms / launches, "peak": issue_peak,
         "peak_kind": "measured in this run (DFMA-chain probe, %.3f TFLOP/s)" % fp64_tflops_probe}
    if any(m not in KERNEL_WORK for m in members):
        r.update({"achieved": None, "frac": None, "traffic": None,
                  "note": "no ncu instruction count recorded for " +
                          ", ".join(m for m in members if m not in KERNEL_WORK)})
        return r
    inst = sum(KERNEL_WORK[m]["fp64"] * 32 * ncell * v[0] for m, v in members.items())
    r["achieved"] = inst / (ms * 1e-3) / 1e12
    r["frac"] = r["achieved"] / issue_peak
    r["algorithmic_per_launch"] = {"fp64_lane_inst": inst / launches,
                                   "per_valid_cell": inst / launches / ncell}
    dram = [KERNEL_WORK[m]["dram"] for m in members]
    if all(x is not None for x in dram):
        r["traffic"] = sum(KERNEL_WORK[m]["dram"] * ncell * v[0] for m, v in members.items()) / launches
        hbm = peaks.get("hbm_gbs", HBM_PEAK_FALLBACK)
        r["hbm"] = {"achieved_gbs": r["traffic"] / (ms / launches * 1e-3) / 1e9, "peak_gbs": hbm,
                    "peak_kind": peak_kind}
    else:
        r["traffic"] = None
    st_inst = STAGE_FP64_PER_CELL * 32 * ncell
    r["stage"] = {"fp64_lane_inst": st_inst, "achieved": st_inst / (stage_ms * 1e-3) / 1e12,
                  "frac": st_inst / (stage_ms * 1e-3) / 1e12 / issue_peak}
    return r


def max_over_ranks(x, ws, device="cuda"):
    """The slowest rank's time: every rank times its own replica of the workload, and the
    job's step time is the maximum (all-reduce MAX over the process group)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(ncell_per_rank, ws, ms):
    """Whole-job throughput of N replicas: all ranks' cells over the slowest rank's time."""
    return ws * ncell_per_rank / (ms * 1e-3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.tmp.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.tmp.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample_config(nspec, n=128, box=64):
    """CPU sample with the workload's box shape: n^3 in boxes of box^3 (128^3 in 8 boxes of
    64^3 for the bounded baseline next to the GPU line; the whole workload for the
    reference arm)."""
    from maestroex_gb300 import configs
    return configs.planar_config(n=(n, n, n), nspec=nspec, ppm_type=1, max_grid=box,
                                 seed=20261203 + 1, w0_amp=1.0e4, cfl=0.7)


def run_cpu_baseline(steps, warmup, nthreads=0, nspec=13, n=128, box=64):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    cfg = cpu_sample_config(nspec, n, box)
    ncell = int(np.prod(cfg["n"]))
    want = ("snew",)
    for _ in range(warmup):
        pyoracle.run_stage(cfg, nthreads=nthreads, want=want)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        res = pyoracle.run_stage(cfg, nthreads=nthreads, want=want)
        times.append(time.perf_counter() - t0)
    dt = float(np.median(times))
    cores = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    return {"value": ncell / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"oracle on {n}^3 cells in {len(cfg['boxes'])} boxes of {box}^3, NumSpec {nspec}, ppm_type 1 "
                      f"(same box shape and per-cell work as the GPU workload), median of {steps} timed runs after "
                      f"{warmup}",
            "s_per_sample": dt, "cfg": cfg, "snew": res["snew"]}


def state_parity(gpu_levels, ref_levels, nspec):
    """Largest relative difference of the updated state from the oracle's, per component:
    max |gpu - ref| over the valid cells of every level divided by the component's max |ref|
    (the benchmark's error definition), and the pointwise relative difference over the cells
    where |ref| > 1e-3 max |ref|; `bitwise` when every value is identical."""
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    names = {RHO: "rho", RHOH: "rhoh"}
    names.update({FIRSTSPEC + s: f"rhoX{s + 1}" for s in range(nspec)})
    per, point, bitwise = {}, 0.0, True
    for c, name in names.items():
        g = np.concatenate([np.asarray(x)[c][np.isfinite(np.asarray(r)[c])] for x, r in zip(gpu_levels, ref_levels)])
        r = np.concatenate([np.asarray(r)[c][np.isfinite(np.asarray(r)[c])] for r in ref_levels])
        scale = float(np.abs(r).max())
        d = np.abs(g - r)
        per[name] = float(d.max() / scale) if scale > 0 else float(d.max())
        big = np.abs(r) > 1e-3 * scale
        if big.any():
            point = max(point, float((d[big] / np.abs(r[big])).max()))
        bitwise &= bool(np.array_equal(g, r))
    return {"max_rel_err_vs_oracle": max(per.values()), "pointwise_rel_err": point, "bitwise": bitwise,
            "per_component": per, "tolerance": 1e-12}


def run_parity(headline_ref, args):
    """The GPU stage against the oracle on the benchmark workloads' shapes: the headline
    layout (the CPU-baseline sample, whose oracle result is reused), the two-level AMR shape
    and the spherical two-level shape, each at a size the oracle runs in seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    import torch
    from maestroex_gb300 import capi, configs
    from maestroex_gb300.stage import run_amr_stage_gpu, run_stage_gpu
    out = {}
    cfg = headline_ref["cfg"]
    gpu = run_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    out["headline_layout"] = {"sample": f"{cfg['n'][0]}^3 in {len(cfg['boxes'])} boxes of 64^3, NumSpec "
                                        f"{cfg['nspec']}, ppm_type 1, w0 != 0 (the CPU-baseline sample), graph mode",
                              **state_parity([gpu["snew"]], [headline_ref["snew"]], cfg["nspec"])}
    cfg = configs.two_level_sample(nspec=args.nspec)
    t0 = time.perf_counter()
    ref = pyoracle.run_stage_levels(cfg, want=("snew",))
    t_or = time.perf_counter() - t0
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    l1 = cfg["levels"][1]["boxes"]
    out["amr"] = {"sample": f"two levels: level 0 64^3 in {len(cfg['levels'][0]['boxes'])} uneven boxes, level 1 "
                            f"{len(l1)} boxes of 16-32 cells around 3 bubbles, NumSpec {args.nspec}, ppm_type 2, "
                            "w0 != 0, graph mode", "oracle_s": t_or,
                  **state_parity([g["snew"] for g in gpu], [r["snew"] for r in ref], args.nspec)}
    cfg = configs.spherical_two_level_sample()
    t0 = time.perf_counter()
    ref = pyoracle.run_stage_levels(cfg, want=("snew",))
    t_or = time.perf_counter() - t0
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    out["spherical"] = {"sample": f"spherical full star, two levels: level 0 48^3 in "
                                  f"{len(cfg['levels'][0]['boxes'])} uneven boxes, level 1 "
                                  f"{len(cfg['levels'][1]['boxes'])} boxes, NumSpec 21, ppm_type 2, w0 1e5, "
                                  "graph mode", "oracle_s": t_or,
                        **state_parity([g["snew"] for g in gpu], [r["snew"] for r in ref], 21)}
    torch.cuda.empty_cache()
    return out


def run_amr(args, ws, steps, warmup, barrier):
    """Two-level AMR workload: the batched path replayed as a CUDA graph against
    one launch per box, same inputs, same results (bitwise; checked here)."""
    import torch
    from maestroex_gb300 import capi, configs
    from maestroex_gb300.stage import amr_buffers, make_amr_stage
    cfg = configs.workload_amr(n0=args.amr_n, nspec=args.nspec)
    st = make_amr_stage(cfg)
    if args.component_streams >= 0:
        st.set_option("component_streams", args.component_streams)
    if args.es_inline >= 0:
        st.set_option("es_inline", args.es_inline)
    bufs = amr_buffers(cfg)
    names = ("uold", "sold", "gpi")
    snap = [{n: [t.clone() for t in getattr(b, n).fabs] for n in names} for b in bufs]

    def reset():
        for b, sn in zip(bufs, snap):
            for n, ts in sn.items():
                for dst, src in zip(getattr(b, n).fabs, ts):
                    dst.copy_(src)

    def timed(mode, k, warm):
        for _ in range(warm):
            reset()
            st.stage_forward_levels(bufs, mode=mode)
        barrier()
        total = 0.0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(k):
            reset()
            torch.cuda.synchronize()
            e0.record()
            st.stage_forward_levels(bufs, mode=mode)
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        barrier()
        return total / k

    ms_graph_untuned = timed(capi.MODE_GRAPH, steps, warmup)
    tuned = st.autotune(lambda: (reset(), st.stage_forward_levels(bufs, mode=capi.MODE_BATCHED)))
    ms_graph = timed(capi.MODE_GRAPH, steps, warmup)
    launches_graph = st.launch_count()
    out_graph = [torch.cat([f.flatten() for f in b.snew.fabs]) for b in bufs]
    ms_batched = timed(capi.MODE_BATCHED, steps, 1)
    ms_perbox = timed(capi.MODE_PER_BOX, steps, 1)
    launches_perbox = st.launch_count()
    same = all(torch.equal(a, torch.cat([f.flatten() for f in b.snew.fabs])) for a, b in zip(out_graph, bufs))
    cells = [int(np.prod(L["n"])) if l == 0 else
             sum((b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in L["boxes"])
             for l, L in enumerate(cfg["levels"])]
    ncell = sum(cells)
    st.close()
    del bufs, snap
    torch.cuda.empty_cache()
    return {
        "workload": f"two-level AMR: level 0 {args.amr_n}^3 in {len(cfg['levels'][0]['boxes'])} uneven boxes "
                    f"(edges 16-128), level 1 (ratio 2) {len(cfg['levels'][1]['boxes'])} boxes of 16-64 cells "
                    f"around 3 bubbles ({cells[1] / 8 / cells[0]:.3f} of the domain), NumSpec {args.nspec}, "
                    "ppm_type 2; level-1 state injected from level 0",
        "cells_per_level": cells, "unit": UNIT,
        "graph": {"value": ws * ncell / (ms_graph * 1e-3), "ms_per_step": ms_graph, "gpu_launches": launches_graph,
                  "autotuned": True},
        "graph_untuned": {"value": ws * ncell / (ms_graph_untuned * 1e-3), "ms_per_step": ms_graph_untuned},
        "autotuner_choices_per_level": [{str(t): sum(1 for k, v in tuned.items()
                                                     if k.startswith(f"L{lev} ") and not k.endswith("ppm_form") and v == t)
                                         for t in sorted({v for k, v in tuned.items() if not k.endswith("ppm_form")})}
                                        for lev in range(2)],
        "autotuner_ppm_form_per_level": [tuned.get(f"L{lev} ppm_form") for lev in range(2)],
        "batched_no_graph": {"value": ws * ncell / (ms_batched * 1e-3), "ms_per_step": ms_batched},
        "per_box": {"value": ws * ncell / (ms_perbox * 1e-3), "ms_per_step": ms_perbox,
                    "gpu_launches": launches_perbox},
        "speedup_graph_vs_per_box": ms_perbox / ms_graph,
        "identical_results_graph_vs_per_box": bool(same),
    }


def fd_check(grad_of, jdiff, draw, want, max_tries, skip_tol=1e-7):
    """Central-difference check of adjoint gradient entries.

    draw() -> (field, comp, cell, x): a seeded random entry and its magnitude scale;
    jdiff(field, comp, cell, h) = J(x + h) - J(x - h), the states differenced before the
    weights are applied; grad_of(field, comp, cell) = the adjoint's entry.  Each entry is
    differenced with h = 1e-6 x and h/2.  A limiter or upwind switch inside [x - h, x + h]
    shows as a difference between the two quotients far above their O(h^2) truncation
    error: such entries are skipped when the quotients differ by more than skip_tol
    (1e-7, below the 1e-6 pass bar).  The error of an accepted entry is taken against the
    Richardson extrapolation (4 D(h/2) - D(h)) / 3.  Stops after `want` accepted entries or
    `max_tries` drawn ones."""
    errs, skipped, tries = [], 0, 0  # errors as Python floats
    while len(errs) < want and tries < max_tries:
        tries += 1
        field, comp, cell, x = draw()
        d = [jdiff(field, comp, cell, rel * x) / (2 * rel * x) for rel in (1e-6, 0.5e-6)]
        scale = max(abs(d[0]), abs(d[1]), 1e-300)
        if abs(d[0] - d[1]) > skip_tol * scale:
            skipped += 1
            continue
        rich = (4.0 * d[1] - d[0]) / 3.0
        errs.append(float(abs(grad_of(field, comp, cell) - rich) / scale))
    return {"entries": len(errs), "skipped_limiter_switch": skipped,
            "worst_rel_err": max(errs) if errs else None, "median_rel_err": float(np.median(errs)) if errs else None,
            "pass_bar": 1e-6, "passed": bool(errs) and bool(max(errs) <= 1e-6),
            "h": "1e-6 max(|x|, rms/10) and h/2; entries whose two quotients differ by more than "
                 f"{skip_tol:g} (a limiter switch inside [x - h, x + h]) are skipped; error against the Richardson "
                 "extrapolation (4 D(h/2) - D(h)) / 3"}


def run_adjoint(args, barrier):
    """Multi-step adjoint workload: 128^3 in 8 boxes of 64^3, NumSpec 3, ppm_type 1, 16 steps
    at CFL 0.5 with the velocity held fixed, J = sum(w rhoX + v rhoh) with w, v ~ N(0, 1),
    stored states every 4 steps.  Times the forward alone, the adjoint for dJ/d(state) and
    the adjoint for dJ/d(state, velocity) (each call runs its own forward), and checks
    --fd-entries gradient entries at random cells against central differences of the same
    forward (fd_check)."""
    import torch
    from maestroex_gb300 import configs
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    from maestroex_gb300.stage import MultiFab, make_stage
    n, nsteps, ckpt = args.adj_n, args.adj_steps, args.adj_ckpt
    cfg = configs.adjoint_config(n=(n, n, n), max_grid=min(64, n), nspec=3)
    st = make_stage(cfg)
    boxes, nscal = cfg["boxes"], 4 + cfg["nspec"]
    u = MultiFab(boxes, 3, 0).from_domain(cfg["uold"])
    s0 = MultiFab(boxes, nscal, 0).from_domain(cfg["sold"])
    rng = np.random.default_rng(20261203 + 40)
    w = np.zeros_like(cfg["sold"])
    w[RHOH] = rng.normal(size=w[RHOH].shape)
    w[FIRSTSPEC:] = rng.normal(size=w[FIRSTSPEC:].shape)
    wt = MultiFab(boxes, nscal, 0).from_domain(w)
    gs, gu, sf = MultiFab(boxes, nscal, 0), MultiFab(boxes, 3, 0), MultiFab(boxes, nscal, 0)

    if args.profile_adjoint:
        call_kw = dict(grad_s=gs, grad_u=gu)
        st.stage_adjoint(u, s0, wt, nsteps, ckpt, **call_kw)
        torch.cuda.synchronize()
        print(json.dumps({"profile_adjoint": True, "launches": st.launch_count()}))
        return None

    def call(kind, uu=None, ss=None):
        return st.stage_adjoint(u if uu is None else uu, s0 if ss is None else ss, wt, nsteps, ckpt,
                                grad_s=gs if kind != "fwd" else None, grad_u=gu if kind == "full" else None,
                                sfinal=sf)

    def timed(kind, reps):
        call(kind)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for _ in range(reps):
            torch.cuda.synchronize()
            e0.record()
            J, nbytes = call(kind)
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps, J, nbytes

    reps = max(1, args.steps // 2)
    ms_fwd, J, _ = timed("fwd", reps)
    ms_state, _, bytes_state = timed("state", reps)
    ms_full, J_full, bytes_full = timed("full", reps)
    call("full")
    G = gs.to_domain(cfg["n"]).cpu().numpy()
    GU = gu.to_domain(cfg["n"]).cpu().numpy()
    S, U = cfg["sold"], cfg["uold"]

    def perturbed(src, comp, cell, h):
        m = MultiFab(boxes, src.ncomp, 0)
        for a, b in zip(m.fabs, src.fabs):
            a.copy_(b)
        i, j, k = cell
        for bi, bx in enumerate(boxes):
            if bx[0] <= i <= bx[3] and bx[1] <= j <= bx[4] and bx[2] <= k <= bx[5]:
                m.fabs[bi][comp, k - bx[2], j - bx[1], i - bx[0]] += h
        return m

    def final(uu, ss):
        out = MultiFab(boxes, nscal, 0)
        st.stage_adjoint(uu, ss, wt, nsteps, ckpt, sfinal=out)
        return out

    def dJ(a, b):
        return sum(float((x * (p - q)).sum()) for x, p, q in zip(wt.fabs, a.fabs, b.fabs))

    rms_s = np.sqrt((S ** 2).mean(axis=(1, 2, 3)))
    rms_u = np.sqrt((U ** 2).mean(axis=(1, 2, 3)))
    kinds = [("s", RHOH), ("s", FIRSTSPEC), ("s", FIRSTSPEC + 1), ("s", FIRSTSPEC + 2), ("s", RHO),
             ("u", 0), ("u", 1), ("u", 2)]

    def draw():
        field, comp = kinds[int(rng.integers(0, len(kinds)))]
        cell = tuple(int(v) for v in rng.integers(0, n, size=3))
        X, R = (S, rms_s) if field == "s" else (U, rms_u)
        i, j, k = cell
        return field, comp, cell, max(abs(X[comp, k, j, i]), 0.1 * R[comp])

    def jdiff(field, comp, cell, h):
        if field == "s":
            return dJ(final(u, perturbed(s0, comp, cell, h)), final(u, perturbed(s0, comp, cell, -h)))
        return dJ(final(perturbed(u, comp, cell, h), s0), final(perturbed(u, comp, cell, -h), s0))

    def grad_of(field, comp, cell):
        i, j, k = cell
        return (G if field == "s" else GU)[comp, k, j, i]

    fd = fd_check(grad_of, jdiff, draw, args.fd_entries, 2 * args.fd_entries)
    st.close()
    torch.cuda.empty_cache()
    return {
        "workload": f"3-D single level {n}^3 in {len(boxes)} boxes of {min(64, n)}^3, NumSpec 3, ppm_type 1, "
                    f"periodic, {nsteps} steps at CFL 0.5 with the velocity held fixed, stored states every {ckpt} "
                    "steps; J = sum(w rhoX + v rhoh_final), w, v ~ N(0,1)",
        "fwd_ms": ms_fwd, "adj_state_ms": ms_state, "adj_state_velocity_ms": ms_full,
        "adj_over_fwd_state": ms_state / ms_fwd, "adj_over_fwd_state_velocity": ms_full / ms_fwd,
        "device_bytes_state": bytes_state, "device_bytes_state_velocity": bytes_full,
        "J": J_full,
        "fd_check": fd,
    }


def run_mac_projection(args, barrier):
    """MAC projection (Maestro::MacProj, plane-parallel, one level) on the headline layout:
    256^3 in 64 boxes of 64^3, periodic x / y, slip wall below and outflow above (Dirichlet
    phi = 0 there), the seeded atmosphere's density, beta0 = rho0, a MAC velocity of the
    workload's magnitude with a seeded perturbation and macrhs = beta0 (S - Sbar) of 1e-3 of
    it, solved to the reference's tolerance (1e-10 of max|rhs|, max norm).  Times one call:
    gathers, multigrid V-cycles, correction and ghost refill."""
    import torch
    from maestroex_gb300 import configs
    from maestroex_gb300.params import INTERIOR, OUTFLOW, RHO, SLIPWALL
    from maestroex_gb300.stage import MultiFab, make_stage
    n = args.n
    cfg = configs.planar_config(n=(n, n, n), nspec=2, ppm_type=1, max_grid=min(64, n),
                                bc_lo=(INTERIOR, INTERIOR, SLIPWALL), bc_hi=(INTERIOR, INTERIOR, OUTFLOW),
                                rho_pert=1e-3, w0_amp=0.0, seed=20261203 + 80)
    rng = np.random.default_rng(20261203 + 81)
    st = make_stage(cfg)
    boxes = cfg["boxes"]
    umax = float(np.abs(cfg["uold"]).max())
    shapes = [(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]
    um = [MultiFab(boxes, 1, 1, nodal=d) for d in range(3)]
    snap = []
    for d in range(3):
        u = umax * (0.5 + 0.1 * rng.standard_normal(shapes[d]))
        if d == 2:
            u[0] = 0.0  # the wall
        else:
            np.moveaxis(u, 2 - d, -1)[..., -1] = np.moveaxis(u, 2 - d, -1)[..., 0]
        um[d].from_domain(torch.from_numpy(u[None]))
        snap.append([t.clone() for t in um[d].fabs])
    beta0 = cfg["rho0_old"]
    rh = MultiFab(boxes, 1, 0).from_domain(
        torch.from_numpy((1e-3 * umax / cfg["dx"][0] * beta0[:, None, None] * rng.standard_normal((n, n, n)))[None]))
    ro = MultiFab(boxes, 1, 0).from_domain(torch.from_numpy(cfg["sold"][RHO][None].copy()))
    phi = MultiFab(boxes, 1, 0)

    def reset():
        for d in range(3):
            for dst, src in zip(um[d].fabs, snap[d]):
                dst.copy_(src)

    for _ in range(2):
        reset()
        st.mac_project(um, rh, ro, beta0, macphi=phi)
    barrier()
    reps = max(1, args.steps // 2)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tot, it, ratio = 0.0, 0, 0.0
    for _ in range(reps):
        reset()
        torch.cuda.synchronize()
        e0.record()
        it, ratio = st.mac_project(um, rh, ro, beta0, macphi=phi)
        e1.record()
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    launches = st.launch_count()
    st.close()
    del um, snap, rh, ro, phi
    torch.cuda.empty_cache()
    ms = tot / reps
    return {"workload": f"MAC projection, {n}^3 in {len(boxes)} boxes of {min(64, n)}^3, periodic x/y, slip wall "
                        "below, outflow above, seeded atmosphere density, beta0 = rho0, tolerance 1e-10 of max|rhs|",
            "ms_per_call": ms, "v_cycles": it, "resid_ratio": ratio, "gpu_launches": launches,
            "value": n ** 3 / (ms * 1e-3), "unit": "cells/s"}


def run_spherical_adjoint(args, barrier):
    """Spherical multi-step adjoint: a full star on one level, n^3 in boxes of 64^3, NumSpec
    21, ppm_type 2, outflow faces, w0 of amplitude 1e5 cm/s, the cell velocity held fixed, 8
    steps with the state stored every 4.  Gravity: the star's, scaled by --sph-adj-gravity
    (default 1e-3: the MAC velocity takes the density's buoyancy through MakeVelForce, and
    the steps -- no MAC projection, no force-limited dt -- stay above the cutoff density;
    0: no gravity, the MAC velocity independent of the state).  Times the forward alone and
    the adjoint for dJ/d(state) (which runs its own forward) at --sph-adj-n, and checks
    --sph-fd-entries gradient entries inside the star against central differences of the
    same forward (fd_check, a third of them density entries) on the same star at
    --sph-fd-n cells a side (each entry costs four 8-step forwards)."""
    import torch
    from maestroex_gb300 import configs
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    from maestroex_gb300.stage import MultiFab, make_stage
    nsteps, ckpt = 8, 4
    gscale = args.sph_adj_gravity

    def case(n):
        # a smooth 1% perturbation of density and enthalpy, so that the star's symmetry ties
        # no limiter decision within the finite-difference step
        cfg = configs.spherical_config(n=n, nspec=21, ppm_type=2, max_grid=min(64, n), w0_amp=1.0e5, pert=1.0e-2)
        cfg["grav_cell"] = cfg["grav_cell"] * gscale
        boxes, nscal = cfg["boxes"], 4 + cfg["nspec"]
        rng = np.random.default_rng(20261203 + 60)
        w = np.zeros_like(cfg["sold"])
        w[RHOH] = rng.normal(size=w[RHOH].shape)
        w[FIRSTSPEC:] = rng.normal(size=w[FIRSTSPEC:].shape)
        return dict(cfg=cfg, st=make_stage(cfg), boxes=boxes, nscal=nscal, n=n,
                    u=MultiFab(boxes, 3, 0).from_domain(cfg["uold"]),
                    s0=MultiFab(boxes, nscal, 0).from_domain(cfg["sold"]),
                    wt=MultiFab(boxes, nscal, 0).from_domain(w),
                    gs=MultiFab(boxes, nscal, 0), sf=MultiFab(boxes, nscal, 0))

    def call(c, grad):
        return c["st"].stage_adjoint(c["u"], c["s0"], c["wt"], nsteps, ckpt, grad_s=c["gs"] if grad else None,
                                     sfinal=c["sf"])

    def timed(c, grad, reps):
        call(c, grad)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for _ in range(reps):
            torch.cuda.synchronize()
            e0.record()
            J, nbytes = call(c, grad)
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps, J, nbytes

    big = case(args.sph_adj_n)
    reps = max(1, args.steps // 2)
    ms_fwd, _, _ = timed(big, False, reps)
    ms_adj, J, nbytes = timed(big, True, reps)
    nboxes = len(big["boxes"])
    big["st"].close()
    del big
    torch.cuda.empty_cache()

    c = case(args.sph_fd_n)
    call(c, True)
    torch.cuda.synchronize()
    n, boxes, nscal, cfg = c["n"], c["boxes"], c["nscal"], c["cfg"]
    G = c["gs"].to_domain(cfg["n"]).cpu().numpy()
    S = cfg["sold"]
    rng = np.random.default_rng(20261203 + 61)

    def final(ss):
        out = MultiFab(boxes, nscal, 0)
        c["st"].stage_adjoint(c["u"], ss, c["wt"], nsteps, ckpt, sfinal=out)
        return out

    def perturbed(comp, cell, h):
        m = MultiFab(boxes, nscal, 0)
        for a, b in zip(m.fabs, c["s0"].fabs):
            a.copy_(b)
        i, j, k = cell
        for bi, bx in enumerate(boxes):
            if bx[0] <= i <= bx[3] and bx[1] <= j <= bx[4] and bx[2] <= k <= bx[5]:
                m.fabs[bi][comp, k - bx[2], j - bx[1], i - bx[0]] += h
        return m

    rms = np.sqrt((S ** 2).mean(axis=(1, 2, 3)))
    comps = [RHOH, RHO] + [FIRSTSPEC + q for q in range(21)]

    def draw():
        comp = RHO if rng.random() < 1.0 / 3.0 else comps[int(rng.integers(0, len(comps)))]
        # a cell inside the star, within about half its radius of the centre
        cell = tuple(int(v) for v in n // 2 + rng.integers(-n // 5, n // 5 + 1, size=3))
        i, j, k = cell
        return "s", comp, cell, max(abs(S[comp, k, j, i]), 0.1 * rms[comp])

    def jdiff(field, comp, cell, h):
        a, b = final(perturbed(comp, cell, h)), final(perturbed(comp, cell, -h))
        return sum(float((x_ * (p - q)).sum()) for x_, p, q in zip(c["wt"].fabs, a.fabs, b.fabs))

    def grad_of(field, comp, cell):
        i, j, k = cell
        return G[comp, k, j, i]

    # with buoyancy a density entry reaches the whole neighbourhood's MAC velocities, and its
    # central differences carry ~1e-7 of noise at h = 1e-6 x and h / 2 (measured on a 32^3
    # star against the oracle's tangent-linear build: 1e-8 .. 1e-7 for h = 2.5e-7 .. 1e-6 x):
    # the skip threshold sits at 4e-7, still under the 1e-6 bar
    fd = fd_check(grad_of, jdiff, draw, args.sph_fd_entries, 3 * args.sph_fd_entries,
                  skip_tol=4e-7 if gscale else 1e-7)
    fd["grid"] = f"{n}^3 in {len(boxes)} boxes, the same star and steps"
    c["st"].close()
    torch.cuda.empty_cache()
    N = args.sph_adj_n
    return {
        "workload": f"spherical full star, one level {N}^3 in {nboxes} boxes of {min(64, N)}^3, NumSpec 21, "
                    f"ppm_type 2, outflow, exact base state, density and enthalpy perturbed by a smooth 1% field, "
                    "w0 amplitude 1e5 cm/s, the cell velocity held fixed, "
                    + (f"the star's gravity scaled by {gscale:g} (buoyancy: the MAC velocity depends on the density)"
                       if gscale else "no gravity (the MAC velocity independent of the state)")
                    + f", {nsteps} steps, stored states every {ckpt}; J = sum(w rhoX + v rhoh_final), w, v ~ N(0,1)",
        "fwd_ms": ms_fwd, "adj_state_ms": ms_adj, "adj_over_fwd_state": ms_adj / ms_fwd, "device_bytes": nbytes,
        "J": J,
        "fd_check": fd,
    }


def run_spherical(args, barrier, exact=True, n=None):
    """Full-star spherical workload: two levels, level 0 n^3 in uneven
    boxes (edges 16-128), level 1 (ratio 2) 16-64-cell boxes around 3 seeded bubbles, NumSpec
    21, ppm_type 2, exact base state on the fine level's irregular radial grid, polytrope
    star, outflow faces; the level-1 state injected from level 0.  The caller holds no
    edge-state or flux MultiFabs (the library streams the species) unless --sph-edges.
    Graph-replayed stage timed; one step launched per box checked identical.  exact=False:
    the same on uniform radial bins with the reference's default interpolation types (graph
    mode only)."""
    import torch
    from maestroex_gb300 import capi, configs
    from maestroex_gb300.stage import amr_buffers, make_amr_stage
    n = n or args.sph_n
    edges = args.sph_edges
    rng = np.random.default_rng(20261203 + 50)
    l0 = configs.uneven_boxes((n, n, n), [16, 32, 48, 64, 96, 128], rng, p_stop=0.8)
    fine = configs.bubble_boxes((n, n, n), nbubbles=3, cover=args.sph_cover, block_edges=(8, 16, 24, 32),
                                max_edge=32, rng=np.random.default_rng(20261203 + 51))
    cfg = configs.spherical_amr_config(n0=n, nspec=21, ppm_type=2, fine_boxes=fine, level0_boxes=l0, inject=True,
                                       exact=exact)
    st = make_amr_stage(cfg)
    bufs = amr_buffers(cfg, edges=edges)
    names = ("uold", "sold", "gpi")
    # the inputs every repetition starts from, kept in pinned host memory (HBM holds the
    # stage's buffers)
    snap = [{nm: [t.cpu().pin_memory() for t in getattr(b, nm).fabs] for nm in names} for b in bufs]

    def reset():
        for b, sn in zip(bufs, snap):
            for nm, ts in sn.items():
                for dst, src in zip(getattr(b, nm).fabs, ts):
                    dst.copy_(src, non_blocking=True)

    def timed(mode, reps, warm=2):
        for _ in range(warm):
            reset()
            st.stage_forward_levels(bufs, mode=mode)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for _ in range(reps):
            reset()
            torch.cuda.synchronize()
            e0.record()
            st.stage_forward_levels(bufs, mode=mode)
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps, st.launch_count()

    reps = max(1, args.steps // 2)
    ms_graph, l_graph = timed(capi.MODE_GRAPH, reps)
    free, total = torch.cuda.mem_get_info()
    cells = [n ** 3, sum((b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in fine)]
    ncell = sum(cells)
    grid = (f"exact base state ({cfg['nr']} radial bins on the fine grid)" if exact else
            f"uniform radial bins ({cfg['nr']} of dx_fine), w0 linear, s0 quadratic, w0mac / s0mac face averages")
    held = ("edge states and fluxes returned" if edges else
            "no edge-state or flux MultiFabs: the species streamed through the library's slots")
    res = {"workload": f"spherical full star, two levels: level 0 {n}^3 in {len(l0)} uneven boxes (edges 16-128), "
                       f"level 1 (ratio 2) {len(fine)} boxes around 3 bubbles ({cells[1] / 8 / cells[0]:.3f} of "
                       f"the domain), NumSpec 21, ppm_type 2, {grid}, n = 1.5 polytrope (rho_c 2e9, radius "
                       f"0.9 L/2), outflow; level-1 state injected from level 0; {held}",
           "cells_per_level": cells, "unit": UNIT, "device_gb_in_use": (total - free) / 1e9,
           "graph": {"value": ncell / (ms_graph * 1e-3), "ms_per_step": ms_graph, "gpu_launches": l_graph}}
    if exact:
        out_graph = [[f.cpu() for f in b.snew.fabs] for b in bufs]
        ms_box, l_box = timed(capi.MODE_PER_BOX, 1, 1)
        same = all(torch.equal(a, f.cpu()) for og, b in zip(out_graph, bufs) for a, f in zip(og, b.snew.fabs))
        res.update({"per_box": {"value": ncell / (ms_box * 1e-3), "ms_per_step": ms_box, "gpu_launches": l_box},
                    "speedup_graph_vs_per_box": ms_box / ms_graph,
                    "identical_results_graph_vs_per_box": bool(same)})
    st.close()
    del bufs, snap
    torch.cuda.empty_cache()
    return res


def run_velocity(args, barrier):
    """VelocityAdvance + UpdateVel on the bench workload (256^3 in 64 boxes of 64^3, w0 != 0):
    the MAC velocity from AdvancePremac, then madv_velocity_advance timed with CUDA events
    (one launch sequence over all boxes per call; inputs are not modified by the call)."""
    import torch
    from maestroex_gb300 import configs
    from maestroex_gb300.params import RHO
    from maestroex_gb300.stage import MultiFab, StageBuffers, make_stage
    cfg = configs.planar_config(n=(args.n,) * 3, nspec=args.nspec, ppm_type=1, max_grid=args.box,
                                seed=20261203 + 1, w0_amp=1.0e4, cfl=0.7)
    st = make_stage(cfg)
    buf = StageBuffers(cfg).load(cfg)
    boxes = cfg["boxes"]
    umac = [MultiFab(boxes, 1, 1, nodal=d) for d in range(3)]
    st.advance_premac(buf.uold, buf.sold, buf.gpi, umac)
    rh = MultiFab(boxes, 1, 0)
    for t, s in zip(rh.fabs, buf.sold.fabs):
        g = buf.sold.ng
        t.copy_(s[RHO:RHO + 1, g:-g, g:-g, g:-g])
    unew = MultiFab(boxes, 3, buf.sold.ng)
    uedge = [MultiFab(boxes, 3, 0, nodal=d) for d in range(3)]

    def call():
        st.velocity_advance(buf.uold, buf.sold, rh, buf.gpi, umac, unew, uedge)

    for _ in range(3):
        call()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(3, args.steps)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        call()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    launches = st.launch_count()
    st.close()
    ncell = args.n ** 3
    return {"workload": f"VelocityAdvance + UpdateVel, {args.n}^3 in boxes of {args.box}^3, ppm_type 1, w0 != 0, "
                        "x/y periodic, z slipwall / outflow (velocity edge states with the outflow clamp)",
            "value": ncell / (ms * 1e-3), "unit": UNIT, "ms_per_call": ms, "gpu_launches": launches,
            "mode": "batched launches (one per kernel over all boxes)"}


def run_2d(args, barrier):
    """2-D workload: one 256 x 256 box, NumSpec 3, ppm_type 1 (the reference's 2-D build),
    graph-replayed stage."""
    import torch
    from maestroex_gb300 import capi, configs
    from maestroex_gb300.stage import StageBuffers, make_stage
    cfg = configs.workload_2d(n=256)
    st = make_stage(cfg)
    if args.staged_ppm >= 0:
        st.set_option("staged_ppm", args.staged_ppm)
    buf = StageBuffers(cfg).load(cfg)
    snap = {name: [t.clone() for t in getattr(buf, name).fabs] for name in ("uold", "sold", "gpi")}

    def step():
        for name, ts in snap.items():
            for dst, src in zip(getattr(buf, name).fabs, ts):
                dst.copy_(src)
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=capi.MODE_GRAPH)

    for _ in range(3):
        step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tot, reps = 0.0, max(3, args.steps)
    for _ in range(reps):
        for name, ts in snap.items():
            for dst, src in zip(getattr(buf, name).fabs, ts):
                dst.copy_(src)
        torch.cuda.synchronize()
        e0.record()
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=capi.MODE_GRAPH)
        e1.record()
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    ms = tot / reps
    launches = st.launch_count()
    gpu = buf.snew.to_domain(cfg["n"]).cpu().numpy()
    st.close()
    # the oracle on the same inputs: its time on this host (one box: one thread) and the
    # largest relative difference of the updated density, enthalpy and species
    from oracle import pyoracle
    t0 = time.perf_counter()
    ref = pyoracle.run_stage_2d(cfg, nthreads=1)["snew"]
    t_or = time.perf_counter() - t0
    comps = [0, 1] + list(range(4, 4 + cfg["nspec"]))
    err = max(float(np.abs(gpu[c] - ref[c]).max() / np.abs(ref[c]).max()) for c in comps)
    return {"workload": "2-D single level 256 x 256 (one box), NumSpec 3, ppm_type 1, x periodic, "
                        "y slipwall / outflow", "value": 256 * 256 / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
            "gpu_launches": launches, "max_rel_err_vs_oracle": err,
            "cpu_oracle": {"value": 256 * 256 / t_or, "unit": UNIT, "cores": 1, "kind": "port",
                           "sample": "the whole 256 x 256 stage, once"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--box", type=int, default=64)
    ap.add_argument("--nspec", type=int, default=13)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the GPU-vs-oracle parity samples")
    ap.add_argument("--no-per-box", action="store_true")
    ap.add_argument("--amr-n", type=int, default=256, help="level-0 extent of the two-level AMR workload")
    ap.add_argument("--no-amr", action="store_true")
    ap.add_argument("--adj-n", type=int, default=128, help="extent of the multi-step adjoint workload")
    ap.add_argument("--adj-steps", type=int, default=16)
    ap.add_argument("--adj-ckpt", type=int, default=4)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--fd-entries", type=int, default=64, help="central-difference entries of the adjoint leg")
    ap.add_argument("--sph-fd-entries", type=int, default=64,
                    help="central-difference entries of the spherical adjoint leg")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="run one adjoint call (state and velocity gradients) and exit (the command ncu captures)")
    ap.add_argument("--no-2d", action="store_true")
    ap.add_argument("--no-velocity", action="store_true")
    ap.add_argument("--sph-n", type=int, default=384, help="extent of the spherical workload")
    ap.add_argument("--sph-u-n", type=int, default=256, help="extent of the spherical workload on uniform bins")
    ap.add_argument("--sph-cover", type=float, default=0.06,
                    help="bubble radius parameter of the spherical workload's level 1 (0.06: about 11%% of the domain)")
    ap.add_argument("--sph-edges", action="store_true",
                    help="spherical legs: hold edge-state and flux MultiFabs (384^3 then exceeds HBM)")
    ap.add_argument("--no-spherical", action="store_true")
    ap.add_argument("--no-sph-adjoint", action="store_true")
    ap.add_argument("--no-mac", action="store_true")
    ap.add_argument("--sph-adj-n", type=int, default=128, help="extent of the spherical adjoint workload")
    ap.add_argument("--sph-fd-n", type=int, default=64,
                    help="extent of the spherical adjoint's finite-difference check (same star and steps)")
    ap.add_argument("--sph-adj-gravity", type=float, default=1.0e-3,
                    help="spherical adjoint: scale of the star's gravity (0: none)")
    ap.add_argument("--profile-once", action="store_true",
                    help="run one batched stage and exit (the command ncu captures)")
    ap.add_argument("--staged-ppm", type=int, default=-1, choices=[-1, 0, 1],
                    help="PPM form of the headline stage: 1 staged sweeps, 0 three launches, -1 the library default")
    ap.add_argument("--component-streams", type=int, default=-1, choices=[-1, 0, 1],
                    help="headline and AMR stages: 1 MakeEdgeScal components alternate between two streams, "
                         "0 one stream, -1 the library default")
    ap.add_argument("--es-inline", type=int, default=-1, choices=[-1, 0, 1],
                    help="headline and AMR stages: 1 the edge kernels form the predictor's states from Ip / Im, "
                         "0 the predictor stores them, -1 the library default")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    warmup = max(args.warmup, 3)

    if args.impl == "reference":
        if rank != 0:
            return
        # the whole workload: one step of the oracle at 256^3 is about 20 s on 16 cores
        cb = run_cpu_baseline(max(args.steps, 1), 1, nthreads=os.cpu_count() or 1, nspec=args.nspec, n=args.n,
                              box=args.box)
        cfg_desc = {"workload": f"3-D single level {args.n}^3 in {len(cb['cfg']['boxes'])} boxes of {args.box}^3, "
                                f"NumSpec {args.nspec}, ppm_type 1, w0 != 0, x/y periodic, z slipwall/outflow",
                    "implementation": "CPU restatement of the reference stage (the oracle), OpenMP over boxes"}
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": warmup, "ms_per_step": 1e3 * cb["s_per_sample"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": cfg_desc,
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line, default=jsonable))
        return

    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from maestroex_gb300 import build, capi, configs
    from maestroex_gb300.stage import MultiFab, StageBuffers, make_stage
    if rank == 0 or ws == 1:
        build.build_library()
    if ws > 1:
        dist.barrier()

    if args.profile_adjoint:
        run_adjoint(args, lambda: torch.cuda.synchronize())
        return

    t_start = time.perf_counter()
    cfg = configs.planar_config(n=(args.n,) * 3, nspec=args.nspec, ppm_type=1, max_grid=args.box,
                                seed=20261203 + 1, w0_amp=1.0e4, cfl=0.7)
    ncell = args.n ** 3
    st = make_stage(cfg)
    if args.staged_ppm >= 0:
        st.set_option("staged_ppm", args.staged_ppm)
    if args.component_streams >= 0:
        st.set_option("component_streams", args.component_streams)
    if args.es_inline >= 0:
        st.set_option("es_inline", args.es_inline)
    buf = StageBuffers(cfg).load(cfg)
    snap = {name: [t.clone() for t in getattr(buf, name).fabs] for name in ("uold", "sold", "gpi")}

    def reset():
        # the stage mutates sold in place (conversions); restore the inputs on the device
        for name, ts in snap.items():
            for dst, src in zip(getattr(buf, name).fabs, ts):
                dst.copy_(src)

    def step(mode):
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=mode)

    if args.profile_once:
        step(capi.MODE_BATCHED)
        torch.cuda.synchronize()
        print(json.dumps({"profile_once": True, "launches": st.launch_count()}))
        return

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(mode, steps, warm):
        for _ in range(warm):
            reset()
            step(mode)
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(steps):
            reset()  # not timed
            torch.cuda.synchronize()
            ev0.record()
            step(mode)
            ev1.record()
            torch.cuda.synchronize()
            total += ev0.elapsed_time(ev1)
        barrier()
        return max_over_ranks(total / steps, ws)

    sampler = ClockSampler(local)
    sampler.start()
    ms_graph_untuned = timed(capi.MODE_GRAPH, args.steps, warmup)
    # launch-shape autotuner (untimed trials of the batched stage), then the graph again
    tuned = st.autotune(lambda: (reset(), step(capi.MODE_BATCHED)))
    ms_graph = timed(capi.MODE_GRAPH, args.steps, warmup)
    clocks = sampler.stop()
    launches = st.launch_count()
    ms_batched = timed(capi.MODE_BATCHED, max(1, args.steps // 2), 1)
    ms_perbox = None if args.no_per_box else timed(capi.MODE_PER_BOX, max(1, args.steps // 2), 1)

    # end to end through the public API: every step copies its inputs (uold, sold, gpi: the
    # valid cells of every box, which is all the stage reads of them) from pinned host memory
    # and its result (snew's valid cells) back.  Two device buffer sets pipeline the steps:
    # step n+1's inputs travel on one copy stream while step n computes, and step n's result
    # travels back on another while step n+1 computes; each box's valid cells cross the bus
    # as one contiguous block, unpacked into (or packed from) the FAB on the device.
    def valid(mf, b):
        fs, _ = mf._slices(b)
        return mf.fabs[b][(slice(None),) + fs]

    host = {name: [snap[name][b][(slice(None),) + getattr(buf, name)._slices(b)[0]].cpu().contiguous().pin_memory()
                   for b in range(len(cfg["boxes"]))] for name in ("uold", "sold", "gpi")}
    sets = [buf, StageBuffers(cfg).load(cfg)]
    stage_in = {name: [torch.empty_like(t, device="cuda") for t in ts] for name, ts in host.items()}
    nb = len(cfg["boxes"])
    host_out = [[valid(b.snew, q).cpu().contiguous().pin_memory() for q in range(nb)] for b in sets]
    stage_out = [torch.empty_like(t, device="cuda") for t in host_out[0]]
    h2d = sum(t.numel() * 8 for v in host.values() for t in v)
    d2h = sum(t.numel() * 8 for t in host_out[0])
    comp = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in sets]
    ev_done = [torch.cuda.Event() for _ in sets]
    ev_out = [torch.cuda.Event() for _ in sets]

    def copy_in(k):
        bk = sets[k % 2]
        with torch.cuda.stream(s_in):
            s_in.wait_event(ev_out[k % 2])  # this set's previous result has left the device
            for name, hs in host.items():
                mf = getattr(bk, name)
                for q, (tmp, src) in enumerate(zip(stage_in[name], hs)):
                    tmp.copy_(src, non_blocking=True)
                    valid(mf, q).copy_(tmp)
            ev_in[k % 2].record(s_in)

    def compute_and_copy_out(k):
        bk = sets[k % 2]
        comp.wait_event(ev_in[k % 2])
        st.stage_forward(bk.uold, bk.sold, bk.gpi, bk.snew, bk.umac, bk.sedge, bk.sflux, bk.eta,
                         thermal=bk.thermal, mode=capi.MODE_BATCHED, stream=comp)
        ev_done[k % 2].record(comp)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_done[k % 2])
            for q, (dst, tmp) in enumerate(zip(host_out[k % 2], stage_out)):
                tmp.copy_(valid(bk.snew, q))
                dst.copy_(tmp, non_blocking=True)
            ev_out[k % 2].record(s_out)

    def pipeline(n0, n):
        copy_in(n0)
        for k in range(n0, n0 + n):
            if k + 1 < n0 + n:
                copy_in(k + 1)
            compute_and_copy_out(k)
        torch.cuda.synchronize()

    pipeline(0, warmup)
    barrier()
    t0 = time.perf_counter()
    pipeline(warmup, args.steps)
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, ws)
    del sets[1]
    torch.cuda.empty_cache()

    # per-kernel device time of one batched stage (CUDA events around every launch)
    import ctypes as C
    L = capi.lib()
    reset()
    capi.check(L.madv_profile(st.ctx, 1))
    step(capi.MODE_BATCHED)
    rep = C.create_string_buffer(1 << 20)
    capi.check(L.madv_profile_report(st.ctx, rep, len(rep)))
    capi.check(L.madv_profile(st.ctx, 0))
    kern = json.loads(rep.value.decode())
    tf = C.c_double(0.0)
    capi.check(L.madv_probe_fp64_peak(C.byref(tf), C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    # the other workloads run on their own buffers: release this one's first
    st.close()
    del st, buf, snap, sets
    torch.cuda.empty_cache()
    leg_s = {"headline": time.perf_counter() - t_start}

    def leg(name, skip, fn):
        if skip:
            return None
        t0 = time.perf_counter()
        r = fn()
        leg_s[name] = time.perf_counter() - t0
        # progress on stderr (the JSON line on stdout comes at the end)
        print(json.dumps({"leg": name, "seconds": round(leg_s[name], 1), "result": r}, default=jsonable),
              file=sys.stderr, flush=True)
        return r

    amr = leg("amr", args.no_amr, lambda: run_amr(args, ws, max(1, args.steps // 2), warmup, barrier))
    adj = leg("adjoint", args.no_adjoint, lambda: run_adjoint(args, barrier))
    two_d = leg("two_d", args.no_2d, lambda: run_2d(args, barrier))
    vel = leg("velocity_advance", args.no_velocity, lambda: run_velocity(args, barrier))
    sph = leg("spherical", args.no_spherical, lambda: run_spherical(args, barrier))
    sph_u = leg("spherical_uniform_bins", args.no_spherical,
                lambda: run_spherical(args, barrier, exact=False, n=args.sph_u_n))
    sph_adj = leg("spherical_adjoint", args.no_sph_adjoint, lambda: run_spherical_adjoint(args, barrier))
    mac = leg("mac_projection", args.no_mac, lambda: run_mac_projection(args, barrier))

    if rank != 0:
        dist.destroy_process_group()
        return
    peaks, peak_kind = measured_peaks()
    ktot = sum(v[1] for v in kern.values())
    top = sorted(kern.items(), key=lambda kv: -kv[1][1])[:8]
    value = job_value(ncell, ws, ms_graph)
    b_cell = 8 * (2 * args.nspec + 16)
    hbm_gbs = ncell * b_cell / (ms_graph * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": warmup,
        "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"3-D single level {args.n}^3 in {len(cfg['boxes'])} boxes of {args.box}^3, "
                               f"NumSpec {args.nspec}, ppm_type 1, w0 != 0, x/y periodic, z slipwall/outflow",
                   "mode": "batched kernels replayed as one CUDA graph, autotuned threads per block",
                   "l2": "inputs (state 2.4 GB) larger than the 129 MB L2; state reset between steps",
                   "replicas": ws},
        "clocks": clocks,
        "e2e": {"value": ws * ncell / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "mode": "madv_stage_forward (batched) per step; the valid cells of uold, sold, gpi copied in from "
                        "pinned host memory and snew's copied out, each box one contiguous block, pipelined against "
                        "the neighbouring steps' compute on two copy streams"},
        "gpu_launches": launches * args.steps,
        "per_box": {"value": ws * ncell / (ms_perbox * 1e-3) if ms_perbox else None,
                    "ms_per_step": ms_perbox},
        "batched_no_graph": {"value": ws * ncell / (ms_batched * 1e-3), "ms_per_step": ms_batched},
        "autotuner": {"untuned_graph": {"value": ws * ncell / (ms_graph_untuned * 1e-3),
                                        "ms_per_step": ms_graph_untuned},
                      "threads_per_block_chosen": {str(t): sum(1 for k, v in tuned.items()
                                                               if not k.endswith("ppm_form") and v == t)
                                                   for t in sorted({v for k, v in tuned.items()
                                                                    if not k.endswith("ppm_form")})},
                      "ppm_form_chosen": tuned.get("L0 ppm_form"),
                      "speedup": ms_graph_untuned / ms_graph},
        "fp64_peak_tflops_probe": tf.value,
        "kernels_top": {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / ktot, 4)}
                        for k, v in top},
        "roofline": roofline(kern, ncell, ms_graph, tf.value, peaks, peak_kind),
        "stage_hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": peaks.get("hbm_gbs", HBM_PEAK_FALLBACK),
                      "frac": hbm_gbs / peaks.get("hbm_gbs", HBM_PEAK_FALLBACK), "peak_kind": peak_kind,
                      "bytes_per_cell": b_cell},
    }
    if amr is not None:
        line["amr"] = amr
    if adj is not None:
        line["adjoint"] = adj
    if two_d is not None:
        line["two_d"] = two_d
    if vel is not None:
        line["velocity_advance"] = vel
    if sph is not None:
        line["spherical"] = sph
    if sph_u is not None:
        line["spherical_uniform_bins"] = sph_u
    if sph_adj is not None:
        line["spherical_adjoint"] = sph_adj
    if mac is not None:
        line["mac_projection"] = mac
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        cb = run_cpu_baseline(5, 1, nthreads=os.cpu_count() or 1, nspec=args.nspec)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        c1 = run_cpu_baseline(3, 0, nthreads=1, nspec=args.nspec, n=64, box=64)
        line["cpu_baseline_1core"] = {k: c1[k] for k in ("value", "unit", "cores", "kind", "sample")}
        if not args.no_parity:
            line["parity"] = run_parity(cb, args)
            line["max_rel_err_vs_oracle"] = line["parity"]["headline_layout"]["max_rel_err_vs_oracle"]
        leg_s["cpu_baseline_and_parity"] = time.perf_counter() - t0
    line["leg_seconds"] = {k: round(v, 1) for k, v in leg_s.items()}
    print(json.dumps(line, default=jsonable))
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
