#!/usr/bin/env python
"""Benchmark of the RTM hot path: one step = one single-shot migration (forward
propagation with source-wavefield storage + adjoint propagation with imaging) of the
3400 x 700 faulted-model workload (dx 5 m, CPML 50, nt 7500, 3400 receivers).

Metric: Gcell-updates/s, where one migration credits 2 * dimX * dimZ * nt cell-updates
(forward + backward over the padded grid; the source-field reconstruction is not
credited).  `value` times the device-resident plan API (inputs already in HBM); `e2e`
times the reference-shaped host entry point rtm_migrate_shot (host buffers, copies in the
timed region).  `--impl reference` times the CPU implementation of the same path on the
host cores instead.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
Under torchrun (N > 1) every rank runs independent migrations (replicas, no exchange).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
TRAFFIC_SUMMARY = os.path.join(ROOT, "profiles", "k_step_bwd_traffic.txt")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=("gpu", "reference"))
    ap.add_argument("--workload", default="large", choices=("large", "small"))
    ap.add_argument("--storage", default="ring", choices=("ring", "snapshot"))
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of the bounded CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tile-x", type=int, default=0, help="x columns per CTA tile (0: default)")
    ap.add_argument("--nt", type=int, default=0,
                    help="profiling only: shorten the time axis (the reported workload changes)")
    ap.add_argument("--quick", action="store_true",
                    help="profiling only: device-resident timing, no e2e or CPU baseline")
    ap.add_argument("--batch-members", type=int, default=64,
                    help="batched UQ ensemble: velocity realizations (0: skip)")
    ap.add_argument("--batch-nt", type=int, default=7500)
    ap.add_argument("--no-batch-autotune", dest="batch_autotune", action="store_false",
                    help="batched members at the default 32-column tile width")
    ap.add_argument("--plain-sample", type=int, default=6,
                    help="ensemble members also run one at a time through the plain path")
    ap.add_argument("--serve-requests", type=int, default=96,
                    help="serving trace: Poisson-arriving requests (0: skip)")
    ap.add_argument("--serve-load", type=float, default=0.8,
                    help="arrival rate as a fraction of the batched service capacity")
    ap.add_argument("--serve-load-high", type=float, default=1.5,
                    help="second pass of the same trace at this load: a standing queue, the "
                         "server full (0: skip)")
    ap.add_argument("--plain-trace-requests", type=int, default=48,
                    help="serving trace: requests also served one at a time by the plain path")
    ap.add_argument("--plain-trace-seconds", type=float, default=25.0,
                    help="serving trace: wall-time bound of the plain path's run")
    ap.add_argument("--serve-max-members", type=int, default=1024,
                    help="resident migrations the server may hold (at most 1024)")
    ap.add_argument("--serve-capacity", type=float, default=150.0,
                    help="with --only served: the batched capacity (Gcell-updates/s) the arrival "
                         "rate is sized by")
    ap.add_argument("--steps-per-launch", type=int, default=16,
                    help="batched steps per CUDA-graph replay of the server")
    ap.add_argument("--precision-nt", type=int, default=7500,
                    help="reduced-precision storage study: time steps (0: skip)")
    ap.add_argument("--only", default=None, choices=("batched", "served", "precision"),
                    help="profiling only: run one form alone and print its JSON")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def shard(items, rank, world):
    """Round-robin share of independent units (migrations) for one rank: the path shards by
    migration, with no exchange between ranks."""
    return list(items[rank::world])


def reduce_over_ranks(x, op, ws, device):
    """max or sum of a float over the ranks of the default process group (x itself at ws 1)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def workload(args, extend=None):
    """Params and seeded host inputs of the benchmarked workload.  `extend` pads a model
    into the CPML (default: the engine's extend_matrix; the reference arm passes the
    oracle's, so that it never loads the engine library)."""
    from rtmuq2d_gb300 import workloads
    if extend is None:
        import rtmuq2d_gb300 as eng
        extend = eng.extend_matrix
    storage = 1 if args.storage == "ring" else 0
    if args.workload == "large":
        p = workloads.params_large(storage=storage)
        true, mig = workloads.models_large(p, seed=1)
    else:
        p = workloads.params_small(storage=storage)
        true, mig = workloads.models_small(p, seed=0)
    wav = workloads.wavelet_for(p)
    ext_true = extend(p, true)
    ext = extend(p, mig)
    if args.nt:
        p = p.replace(nt=args.nt)
    if args.tile_x:
        p = p.replace(tile_x=args.tile_x)
    return p, ext_true, ext, wav


def workload_name(p):
    return "rtm_single_shot_%dx%d_nt%d" % (p.nx, p.nz, p.nt)


def bench_config(p, args, ws):
    """The `config` of both arms' lines (the same keys and values: the same workload)."""
    return {"workload": workload_name(p), "grid": [p.dim_x, p.dim_z], "nt": p.nt,
            "receivers": p.rec_count, "storage": args.storage, "ring_precision": "fp32",
            "seismogram": "modelled on the true model by the same scheme (trace recording)",
            "parallelism": "replicas" if ws > 1 else "single",
            "l2": "GPU: L2 flushed between timed iterations (256 MB write); CPU: the snapshot "
                  "store of the time axis (4.2 GB at 3500 x 800, nt 7500) streams through memory"}


# the headline metric: Gcell-updates/s (value: the plain single-shot migration; the served
# and batched forms, with p50/p99 latency and their ratio to the plain path, under their keys)
METRIC = "RTM Gcell-updates/s + p50/p99 migration latency: served vs plain, rel-L2\u22641e-3"


def algorithmic_bytes(p):
    """Algorithmic DRAM bytes per launch of each kernel (FP32 fields, ring storage).
    k_step forward : 16 B per cell (u_cur, u_prev, coef read; u_next write)
                     + 16 B per CPML-correction cell (previous psi read, new psi write, xi
                       read + write: the step kernel updates psi itself)
                     + 4 B per ring cell written
    k_step backward: receiver field as forward (16 B/cell + 16 B/CPML cell)
                     + 12 B per reconstruction-region cell (S_cur, S_prev read; S_next write)
                     + 4 B per ring cell read + 4 B per receiver (seismogram row)
                     + imaging every time_slices steps: 32 B per interior cell (FP64
                       image and self image read+write), averaged per launch
    k_bpsi         : 12 B per psi cell (u read, psi read+write): the batched members' psi
                     kernel."""
    dx, dz = p.dim_x, p.dim_z
    cells = dx * dz
    thl, thr, thu, thd = p.th_left, p.th_right, p.th_up, p.th_down
    corr = (thl - 8) * (dz - 8) + (thr - 8) * (dz - 8) + (thu - 8) * dx + (thd - 8) * (dx - 8)
    psi = (thl - 8) * (dz - 8) + (thr - 8) * (dz - 8) + (thu - 8) * (dx - 8) + (thd - 8) * (dx - 8)
    # reconstruction region: [th_left-4, dimX-th_right+4) x z bounds rounded inward to quads
    rz0 = (thu - 4 + 3) // 4 * 4
    rz1 = (dz - thd + 4) // 4 * 4
    ring = 8 * (p.nx + 16) + 8 * (rz1 - rz0)
    region = (p.nx + 8) * (rz1 - rz0)
    interior = p.nx * p.nz
    fwd = 16 * cells + 16 * corr + 4 * ring
    bwd = 16 * cells + 16 * corr + 12 * region + 4 * ring + 4 * p.rec_count + 32 * interior / p.time_slices
    batched_fwd = 16 * cells + 12 * corr + 4 * ring + 12 * psi   # k_mstep + k_bpsi + k_bstrip
    return {"k_step_fwd": fwd, "k_step_bwd": bwd, "k_bpsi": 12 * psi, "batched_fwd_step": batched_fwd}


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_per_launch():
    """DRAM bytes per k_step backward launch from the committed ncu summary, if any."""
    try:
        with open(TRAFFIC_SUMMARY) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch_full_size:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(p, ext, wav, seis, target_s, dtype=np.float32):
    """Times the CPU implementation (oracle port, OpenMP over all host cores) on a bounded
    sample of the workload: the same grid, a shortened time axis."""
    from oracle.oracle import Oracle
    orc = Oracle(fast=True)
    threads = orc.max_threads()
    q = p.as_dict()

    def run(nt):
        qq = dict(q, nt=nt)
        s = np.ascontiguousarray(seis[:, :nt]) if seis is not None else np.zeros((p.rec_count, nt), np.float32)
        t0 = time.perf_counter()
        fwd = orc.forward(qq, ext, wav, snapshots=True)
        orc.adjoint(qq, ext, s, fwd["snapshots"])
        return time.perf_counter() - t0

    nt0 = 40
    t = run(nt0)
    per_step = t / nt0
    nt = int(max(nt0, min(p.nt, target_s / max(per_step, 1e-9))) // p.time_slices * p.time_slices)
    nt = max(nt, p.time_slices)
    t = run(nt)
    cells = 2 * p.dim_x * p.dim_z * nt
    return {"value": cells / t / 1e9, "unit": "Gcell-updates/s", "cores": threads,
            "kind": "port", "seconds": t,
            "sample": "forward+adjoint of the %dx%d padded grid for nt=%d of %d steps "
                      "(oracle/rtm_oracle.c, -O3 OpenMP)" % (p.dim_x, p.dim_z, nt, p.nt)}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b) / den) if den > 0 else None


def cpu_full(p, ext_true, ext, wav, seis, img, slf):
    """The CPU leg at full size: the oracle port (OpenMP over all host cores) models the
    observed seismogram on the true model and migrates the same seismogram the GPU migrated.
    Its migration time is the CPU baseline (the whole workload, not a sample); its outputs are
    the parity reference of the GPU's recorded seismogram and image."""
    from oracle.oracle import Oracle
    orc = Oracle(fast=True)
    q = p.as_dict()
    t0 = time.perf_counter()
    seis_ref = orc.model_seismogram(q, ext_true, wav)
    t_model = time.perf_counter() - t0
    t0 = time.perf_counter()
    img_ref, slf_ref = orc.migrate(q, ext, wav, seis)
    t_mig = time.perf_counter() - t0
    cpu = {"value": p.cell_updates / t_mig / 1e9, "unit": "Gcell-updates/s", "cores": orc.max_threads(),
           "kind": "port",
           "sample": "the whole workload: forward (snapshot storage) + adjoint of the %dx%d padded "
                     "grid, nt=%d, in %.1f s (oracle/rtm_oracle.c, -O3, OpenMP)" % (p.dim_x, p.dim_z, p.nt, t_mig)}
    parity = {"reference": "oracle port (-O3, OpenMP) on the same inputs",
              "seis_rel_l2_vs_oracle": rel_l2(seis, seis_ref), "image_rel_l2_vs_oracle": rel_l2(img, img_ref),
              "self_image_rel_l2_vs_oracle": rel_l2(slf, slf_ref), "oracle_model_seconds": t_model}
    return cpu, parity


def fp64_image(eng, p, ext, wav, seis):
    """The image of an FP64 GPU run of the identical scheme (same storage, FP64 fields)."""
    import torch
    q = p.replace(compute=eng.COMPUTE_FP64, tile_x=0)
    plan = eng.Plan(q)
    plan.forward(torch.from_numpy(ext).cuda(), torch.from_numpy(wav).cuda())
    plan.adjoint(torch.from_numpy(seis).cuda())
    img = torch.empty((p.nx, p.nz), dtype=torch.float64, device="cuda")
    plan.read_image(0, img, as_double=True)
    plan.sync()
    out = img.cpu().numpy()
    plan.close()
    return out


def summary(line):
    """The headline figures of every form in a few hundred bytes (the last key of the line)."""
    def pick(d, *keys):
        return {k: d.get(k) for k in keys} if d else None

    def r3(x):
        return round(x, 4) if isinstance(x, float) else x

    out = {"plain": {"value": r3(line["value"]), "e2e": r3(line["e2e"]["value"]),
                     "e2e_zfp": r3(line["e2e_zfp"]["value"]) if line.get("e2e_zfp") else None,
                     "roofline_frac": r3(line["roofline"]["frac"])}}
    b = line.get("batched")
    if b:
        out["batched"] = {k: r3(v) for k, v in pick(b, "value", "speedup_vs_plain", "members").items()}
        for key, name in (("stencil_kernel_roofline", "k_mstep_frac"), ("forward_step_roofline", "fwd_step_frac")):
            if b.get(key):
                out["batched"][name] = r3(b[key]["frac"])
        if b.get("autotuned_tile_x_by_width_class"):
            out["batched"]["tile_x_by_width_class"] = {k: v["tile_x"] for k, v in
                                                       b["autotuned_tile_x_by_width_class"].items()}
    s = line.get("served")
    if s:
        out["served"] = {k: r3(v) for k, v in pick(s, "requests", "value", "p50_latency_s", "p99_latency_s",
                                                   "hbm_occupancy_mean", "speedup_vs_plain_same_requests").items()}
        if s.get("plain") and s.get("served_same_requests"):
            out["served"]["same_requests"] = s["plain"]["requests"]
            out["served"]["served_p50_p99_s"] = [r3(s["served_same_requests"]["p50_latency_s"]),
                                                 r3(s["served_same_requests"]["p99_latency_s"])]
            out["served"]["plain_p50_p99_s"] = [r3(s["plain"]["p50_latency_s"]), r3(s["plain"]["p99_latency_s"])]
    par = line.get("parity")
    if par:
        out["parity"] = {k: (float("%.3g" % v) if isinstance(v, float) else v) for k, v in par.items()
                         if k.endswith("rel_l2_vs_oracle") or k.endswith("fp64_engine")}
    return out


def _round_floats(v, sig=5):
    if isinstance(v, float):
        return float("%.*g" % (sig, v))
    if isinstance(v, dict):
        return {k: _round_floats(x, sig) for k, x in v.items()}
    if isinstance(v, list):
        return [_round_floats(x, sig) for x in v]
    return v


def compact_line(line):
    """The bench line as printed: the contract's keys, then the summary of every form (early,
    so that a reader keeping only the head of the line still sees batched, served and parity),
    then the details, floats to 5 significant digits."""
    line = dict(line)
    line["summary"] = summary(line)
    head = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
            "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline",
            "cpu_baseline", "clocks", "summary")
    out = {k: line[k] for k in head if k in line}
    out.update({k: v for k, v in line.items() if k not in out})
    return _round_floats(out)


def run_batched(args, eng, rank=0, ws=1):
    """The batched UQ ensemble through the serving engine: every member resident at once,
    advanced together by the batched step kernels.  Timed from the first submit (host
    buffers) to the last image on the host; a sample of the members is also run one at a
    time through the plain path for the served-vs-plain ratio.  With N ranks each runs its
    round-robin share of the members; value = all ranks' cell-updates / the slowest rank's
    time."""
    from rtmuq2d_gb300 import workloads
    members, true, mig = workloads.ensemble(args.batch_members, args.batch_nt)
    members = shard(members, rank, ws)
    wav = workloads.wavelet_for(members[0]["params"])
    inputs = []
    for m in members:
        p = m["params"]
        ext_true, ext = workloads.ensemble_inputs(m, true, mig)
        seis = eng.model_seismogram(p.replace(storage=0), ext_true, wav)
        inputs.append((p, ext, wav, seis))
    cells = sum(p.cell_updates for p, *_ in inputs)
    # plain path, one migration at a time (warm the plan cache with the first member)
    sample = inputs[: max(0, min(args.plain_sample, len(inputs)))]
    plain = None
    plain_images = {}
    if sample:
        eng.migrate_shot(*sample[0])
        t0 = time.perf_counter()
        for i, inp in enumerate(sample):
            plain_images[i] = eng.migrate_shot(*inp)[0]
        dt = time.perf_counter() - t0
        plain = sum(p.cell_updates for p, *_ in sample) / dt / 1e9
    eng.release_cached()
    # batched autotuner: the tile width (32 or 16 columns) per window-width class (nx to the
    # nearest 512 columns), timed on 8 copies of the class's middle member with a 40-step
    # time axis; each member is submitted with its class's width
    tuned, width = {}, [0] * len(inputs)
    if args.batch_autotune:
        classes = {}
        for i, (p, *_) in enumerate(inputs):
            classes.setdefault(int(round(p.nx / 512.0)) * 512, []).append(i)
        for cls, idx in sorted(classes.items()):
            p_rep = inputs[idx[len(idx) // 2]][0]
            tx, ms = eng.autotune_batched(p_rep, members=8, steps=40)
            tuned[str(cls)] = {"tile_x": tx, "tuned_on_nx": p_rep.nx, "members": len(idx),
                               "ms_per_batched_step_of_8": ms}
            for i in idx:
                width[i] = tx
    srv = eng.Server(0, max_members=min(len(inputs), 1024), steps_per_launch=args.steps_per_launch)
    t0 = time.perf_counter()
    ids = [srv.submit(inp[0].replace(tile_x=width[i]), *inp[1:]) for i, inp in enumerate(inputs)]
    # while every member is in its forward pass (they are admitted together), time whole
    # batched steps (k_mstep + k_bpsi + k_bstrip) from the server's CUDA events
    # (and the tile kernel alone on one step per replay, k_mstep, timed by the server)
    fwd_ms, fwd_steps, calls = 0.0, 0, 0
    tile_ms = []
    out = {}
    nt_min = min(p.nt for p, *_ in inputs)
    while True:
        ms0 = srv.stats()["gpu_ms"]
        active, queued = srv.step()
        calls += 1
        if calls >= 2 and (calls + 1) * args.steps_per_launch <= nt_min:
            fwd_ms += srv.stats()["gpu_ms"] - ms0
            fwd_steps += args.steps_per_launch
            tile_ms.append(srv.kernel_ms())
        r = srv.poll()
        while r is not None:
            out[r[0]] = r[1:]
            r = srv.poll()
        if active == 0 and queued == 0 and len(out) == len(ids):
            break
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    step_roof = None
    if fwd_steps:
        step_bytes = sum(algorithmic_bytes(p)["batched_fwd_step"] for p, *_ in inputs)
        achieved = step_bytes / (fwd_ms / fwd_steps * 1e-3) / 1e9
        peak, peak_kind = hbm_peak()
        step_roof = {"bound": "hbm", "what": "whole batched forward step (k_mstep + k_bpsi + k_bstrip)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "algorithmic_bytes_per_step": step_bytes,
                     "ms_per_step": fwd_ms / fwd_steps, "steps_timed": fwd_steps,
                     "note": "CUDA events around graph replays of the server's stream"}
    tile_roof = None
    tile_ms = [t for t in tile_ms if t > 0]
    if tile_ms:
        # k_mstep of one forward step of every member: 16 B per cell (u_cur, u_prev, coef
        # read; u_next write); the CPML, psi and ring work is k_bstrip's and k_bpsi's
        tile_bytes = sum(16 * p.dim_x * p.dim_z for p, *_ in inputs)
        avg = sum(tile_ms) / len(tile_ms)
        achieved = tile_bytes / (avg * 1e-3) / 1e9
        peak, peak_kind = hbm_peak()
        tile_roof = {"bound": "hbm", "what": "k_mstep (batched stencil tiles), one forward step of every member",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": tile_bytes,
                     "ms_per_launch": avg, "launches_timed": len(tile_ms),
                     "working_set_bytes": tile_bytes,
                     "note": "CUDA events around the second step's k_mstep of each graph replay, "
                             "launched without overlap; working set far above L2"}
    agree = max((float(np.linalg.norm(out[ids[i]][0] - img) / max(np.linalg.norm(img), 1e-30))
                 for i, img in plain_images.items()), default=None)
    local_cells = cells
    cells = reduce_over_ranks(local_cells, "sum", ws, "cuda")
    wall = reduce_over_ranks(wall, "max", ws, "cuda")
    widths = [p.nx for p, *_ in inputs]
    value = cells / wall / 1e9
    n_members = int(reduce_over_ranks(len(inputs), "sum", ws, "cuda"))
    return {"workload": "uq_ensemble_%dx_windows%d-%d_nz700_nt%d" % (n_members, min(widths),
                                                                      max(widths), args.batch_nt),
            "members": n_members, "ranks": ws, "value": value, "unit": "Gcell-updates/s",
            "seconds": wall, "gpu_busy_value": local_cells / (st["gpu_ms"] * 1e-3) / 1e9,
            "plain_value_same_members": plain, "plain_sample": len(sample),
            "speedup_vs_plain": value / plain if plain else None,
            "image_agreement_with_plain_rel_l2": agree,
            "steps_per_launch": args.steps_per_launch, "device_bytes": st["bytes_in_use"],
            "autotuned_tile_x_by_width_class": tuned or None,
            "forward_step_roofline": step_roof,
            "stencil_kernel_roofline": tile_roof,
            "gpu_launches": st["launches"],
            "timing": "wall clock from the first submit (host buffers) to the last image on the host"}


def prepare_serving(args, eng):
    """The serving trace's requests: mixed grids, nt and ring precision, each with its own
    velocity realization and its seismogram as a ZFP tol 1e-4 stream."""
    from rtmuq2d_gb300 import synth, workloads
    reqs = workloads.serving_trace(args.serve_requests)
    templates = {}
    for k in sorted({r["grid"] for r in reqs}):
        p, true, mig = workloads.serving_template(k)
        wav = workloads.wavelet_for(p)
        ext_true = eng.extend_matrix(p, true)
        seis = eng.model_seismogram(p.replace(storage=0), ext_true, wav)
        templates[k] = (p, mig, wav, seis)
    # each request carries its seismogram as a ZFP tol 1e-4 stream (decoded by the server's
    # host threads while the GPU steps); one stream per (grid, nt)
    tol = 1e-4
    streams = {}
    prepared = []
    for r in reqs:
        p0, mig, wav, seis = templates[r["grid"]]
        p = p0.replace(nt=r["nt"], precision=r["precision"])
        key = (r["grid"], r["nt"])
        if key not in streams:
            streams[key] = eng.zfp_encode(np.ascontiguousarray(seis[:, : r["nt"]]), tol)
        g = synth.grf_coarse((p.nx, p.nz), p.dx, 200.0, r["seed"])
        ext = eng.extend_matrix(p, (mig.astype(np.float64) * np.exp(0.03 * g)).astype(np.float32))
        prepared.append((p, ext, wav, streams[key]))
    return prepared, streams, tol


def serve_trace(args, eng, prepared, tol, capacity_gcells, load):
    """Poisson arrivals of the prepared requests at `load` x the batched capacity through one
    server; latency = finish - arrival."""
    mean_cells = float(np.mean([p.cell_updates for p, *_ in prepared]))
    rate = load * capacity_gcells * 1e9 / mean_cells          # requests / s
    rng = np.random.default_rng(29)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(prepared)))
    try:
        total_hbm = eng.device_info()["hbm_bytes"]
    except Exception:
        total_hbm = None
    srv = eng.Server(0, max_members=args.serve_max_members, steps_per_launch=args.steps_per_launch)
    done, occ, resident, id_to_req = {}, [], [], {}
    t_start = time.monotonic()
    i = 0
    while len(done) < len(prepared):
        now = time.monotonic() - t_start
        while i < len(prepared) and arrivals[i] <= now:
            p_i, ext_i, wav_i, stream_i = prepared[i]
            id_to_req[srv.submit_zfp(p_i, ext_i, wav_i, stream_i, tol)] = i
            i += 1
        active, queued = srv.step()
        occ.append(srv.stats()["bytes_in_use"])
        resident.append(active)
        r = srv.poll()
        while r is not None:
            done[id_to_req[r[0]]] = r[3][2]
            r = srv.poll()
        if active == 0 and queued == 0 and i < len(prepared):
            time.sleep(max(0.0, min(0.002, arrivals[i] - (time.monotonic() - t_start))))
    wall = time.monotonic() - t_start
    st = srv.stats()
    srv.close()
    lat = np.array([done[k] - (t_start + arrivals[k]) for k in range(len(prepared))])
    cells = sum(p.cell_updates for p, *_ in prepared)
    return {"_latencies": lat, "_arrivals": arrivals, "value": cells / wall / 1e9, "unit": "Gcell-updates/s",
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()), "seconds": wall,
            "arrival_rate_per_s": rate, "offered_load": load,
            "gpu_busy_value": cells / (st["gpu_ms"] * 1e-3) / 1e9,
            "resident_members_mean": float(np.mean(resident)), "resident_members_max": int(np.max(resident)),
            "hbm_occupancy_mean": (float(np.mean(occ)) / total_hbm) if total_hbm else None,
            "hbm_occupancy_max": (float(np.max(occ)) / total_hbm) if total_hbm else None,
            "gpu_launches": st["launches"]}


def plain_on_requests(eng, prepared, tol, n_sample=8):
    """The single-migration path on a sample of the trace's requests (every k-th), one at a
    time from host buffers, each grid's plan warmed by one untimed call first: the plain rate
    on the served workload itself."""
    step = max(1, len(prepared) // n_sample)
    sample = prepared[::step][:n_sample]
    jobs = []
    for p, ext, wav, stream in sample:
        seis = eng.zfp_decode(stream, p.rec_count, p.nt, tol)
        jobs.append((p, ext, wav, seis))
    seen = set()
    for p, ext, wav, seis in jobs:
        key = (p.nx, p.nz, p.nt, p.precision)
        if key not in seen:
            seen.add(key)
            eng.migrate_shot(p, ext, wav, seis)
    t0 = time.perf_counter()
    for job in jobs:
        eng.migrate_shot(*job)
    dt = time.perf_counter() - t0
    eng.release_cached()
    return sum(p.cell_updates for p, *_ in jobs) / dt / 1e9, len(jobs)


def plain_trace(eng, prepared, tol, arrivals, k_max, seconds):
    """The plain path serving the same arrivals: the first requests of the trace (at most
    k_max, stopping after `seconds` of wall time) at their Poisson arrival times, one at a time
    in arrival order through rtm_migrate_shot_zfp (the ZFP seismogram decoded on a host thread
    while the forward pass runs).  Latency = completion - arrival, as for the served requests; the
    service time (decode + migration) of each request is reported beside it.  Each grid's plan
    is warmed by one untimed call first."""
    seen = set()
    for p, ext, wav, stream in prepared[:k_max]:
        key = (p.nx, p.nz, p.nt, p.precision)
        if key not in seen:
            seen.add(key)
            eng.migrate_shot(p, ext, wav, eng.zfp_decode(stream, p.rec_count, p.nt, tol))
    lat, service, cells = [], [], 0
    t_start = time.monotonic()
    for k, (p, ext, wav, stream) in enumerate(prepared[:k_max]):
        now = time.monotonic() - t_start
        if now > seconds:
            break
        if arrivals[k] > now:
            time.sleep(arrivals[k] - now)
        t0 = time.monotonic()
        eng.migrate_shot_zfp(p, ext, wav, stream, tol)
        t1 = time.monotonic()
        lat.append(t1 - (t_start + arrivals[k]))
        service.append(t1 - t0)
        cells += p.cell_updates
    wall = time.monotonic() - t_start
    eng.release_cached()
    lat, service = np.array(lat), np.array(service)
    return {"requests": int(len(lat)), "value": cells / wall / 1e9, "unit": "Gcell-updates/s",
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "service_p50_s": float(np.percentile(service, 50)),
            "service_p99_s": float(np.percentile(service, 99)),
            "note": "the first requests of the same trace at the same arrival times, served one at a "
                    "time (rtm_migrate_shot_zfp each); latency includes the queueing"}


def run_served(args, eng, capacity_gcells):
    """The serving trace at `serve_load` x the batched capacity (the latency view), and the
    same trace at `serve_load_high` (a standing queue: the server's throughput when full);
    beside them the single-migration path on a sample of the same requests."""
    from rtmuq2d_gb300 import workloads
    prepared, streams, tol = prepare_serving(args, eng)
    out = {"workload": "serving_trace_%d_requests" % len(prepared), "requests": len(prepared)}
    served = serve_trace(args, eng, prepared, tol, capacity_gcells, args.serve_load)
    lat, arrivals = served.pop("_latencies"), served.pop("_arrivals")
    out.update(served)
    # the plain path on the same arrivals, and the served latencies of the same requests
    pl = plain_trace(eng, prepared, tol, arrivals, args.plain_trace_requests, args.plain_trace_seconds)
    k = pl["requests"]
    out["plain"] = pl
    out["served_same_requests"] = {"requests": k, "p50_latency_s": float(np.percentile(lat[:k], 50)),
                                   "p99_latency_s": float(np.percentile(lat[:k], 99))}
    out.update({"grids": [list(g) for g in workloads.SERVING_GRIDS], "nt_values": list(workloads.SERVING_NT),
                "seismograms": "ZFP tol 1e-4 streams, decoded on the server's host threads",
                "zfp_bytes_total": int(sum(len(x) for x in streams.values())),
                "ring_precisions": ["fp32", "bf16"]})
    if args.serve_load_high > 0:
        hl = serve_trace(args, eng, prepared, tol, capacity_gcells, args.serve_load_high)
        hl.pop("_latencies")
        hl.pop("_arrivals")
        out["high_load"] = hl
    plain, n = plain_on_requests(eng, prepared, tol)
    out["plain_value_same_requests"] = plain
    out["plain_sample"] = n
    out["speedup_vs_plain_same_requests"] = out["value"] / plain
    if "high_load" in out:
        out["high_load"]["speedup_vs_plain_same_requests"] = out["high_load"]["value"] / plain
    return out


def run_precision(args, eng):
    """Reduced-precision source storage on the 3400 x 700 grid and shot, imaging every 4th
    step: FP32 / BF16 / FP16 boundary rings and imaging-interval snapshots (per-step max-abs
    scales for 16-bit), stencil and CPML in FP32, image accumulated in FP64; relative L2
    error of the image, and of the reconstructed source wavefield at t = 0.5, 1.5, 2.5 s,
    against an FP64 run of the identical scheme."""
    import torch
    from rtmuq2d_gb300 import workloads
    p0 = workloads.params_large(time_slices=4, nt=args.precision_nt)
    true, mig = workloads.models_large(p0, seed=1)
    wav = workloads.wavelet_for(p0)
    ext_true = eng.extend_matrix(p0, true)
    ext = eng.extend_matrix(p0, mig)
    seis = eng.model_seismogram(p0.replace(storage=0), ext_true, wav)
    times = [t for t in (int(round(s / p0.dt)) for s in (0.5, 1.5, 2.5)) if t <= p0.nt - 2]
    d_vel = torch.from_numpy(ext).cuda()
    d_wav = torch.from_numpy(wav).cuda()
    d_seis = torch.from_numpy(seis).cuda()

    def run(p):
        fdt = torch.float64 if p.compute else torch.float32
        plan = eng.Plan(p)
        cap = None
        if p.storage == eng.STORE_RING and times:
            cap = torch.zeros((len(times), p.dim_x, p.dim_z), dtype=fdt, device="cuda")
            plan.capture_source(times, cap)
        t0 = time.perf_counter()
        plan.forward(d_vel, d_wav)
        plan.adjoint(d_seis)
        plan.sync()
        secs = time.perf_counter() - t0
        img = torch.zeros((p.nx, p.nz), dtype=torch.float64, device="cuda")
        plan.read_image(0, img, as_double=True)
        plan.sync()
        out = (img.cpu().numpy(), cap.cpu().numpy().astype(np.float64) if cap is not None else None, secs)
        del plan
        eng.release_cached()
        return out

    inner = (slice(p0.th_left, p0.th_left + p0.nx), slice(p0.th_up, p0.th_up + p0.nz))

    def rel(a, b):
        den = float(np.linalg.norm(b))
        return float(np.linalg.norm(a - b) / den) if den > 0 else None

    ref_img, ref_fields, ref_s = run(p0.replace(storage=eng.STORE_RING, compute=eng.COMPUTE_FP64))
    names = {eng.PREC_FP32: "fp32", eng.PREC_BF16: "bf16", eng.PREC_FP16: "fp16"}
    variants = []
    for storage, sname in ((eng.STORE_RING, "ring"), (eng.STORE_SNAPSHOT, "snapshot")):
        for prec in (eng.PREC_FP32, eng.PREC_BF16, eng.PREC_FP16):
            img, fields, secs = run(p0.replace(storage=storage, precision=prec))
            v = {"storage": sname, "precision": names[prec], "image_rel_l2_vs_fp64": rel(img, ref_img),
                 "seconds": secs,
                 "store_bytes": int(eng.footprint_bytes(p0.replace(storage=storage, precision=prec)))}
            if fields is not None:
                # the reconstruction rebuilds the model interior (not the CPML): compare there
                v["field_rel_l2_vs_fp64"] = {"t=%.1fs" % (t * p0.dt): rel(fields[k][inner], ref_fields[k][inner])
                                             for k, t in enumerate(times)}
            variants.append(v)
    return {"workload": "precision_3400x700_nt%d_imaging_every_4" % p0.nt, "reference": "fp64 run, ring storage",
            "fp64_seconds": ref_s, "variants": variants}


def run_reference(args):
    """The CPU implementation of the path on the host cores (the oracle port: the
    reference's own build cannot travel to this machine).  Nothing here loads the engine
    library: the padding and the observed seismogram come from the oracle too, the
    seismogram modelled on the true model like the GPU arm's."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle.oracle import Oracle
    orc = Oracle(fast=True)
    p, ext_true, ext, wav = workload(args, extend=lambda q, m: orc.extend_matrix(q.as_dict(), m))
    seis = orc.model_seismogram(p.as_dict(), ext_true, wav)
    target = max(2.0, min(20.0, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_sample(p, ext, wav, seis, target / 4)
    vals = []
    last = None
    for _ in range(args.steps):
        last = cpu_sample(p, ext, wav, seis, target)
        vals.append(last["value"])
    v = float(np.mean(vals))
    cells_per_step = 2 * p.dim_x * p.dim_z * p.nt
    line = {"impl": "reference", "metric": METRIC, "value": v,
            "unit": "Gcell-updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": cells_per_step / (v * 1e9) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(p, args, ws),
            "note": "each step times a bounded sample (the same grid, a shortened time axis) of the workload",
            "cpu_baseline": {"value": v, "unit": "Gcell-updates/s", "cores": last["cores"],
                             "kind": last["kind"], "sample": last["sample"]},
            "e2e": {"value": v, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_only(args, eng):
    """One form alone (profiling runs): its JSON, without the single-migration part."""
    if args.only == "batched":
        out = run_batched(args, eng)
    elif args.only == "served":
        out = run_served(args, eng, args.serve_capacity)
    else:
        out = run_precision(args, eng)
    print(json.dumps(out), flush=True)
    return 0


def run_gpu(args):
    import torch
    import rtmuq2d_gb300 as eng

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.only:
        return run_only(args, eng)
    p, ext_true, ext, wav = workload(args)
    # observed data: forward modelling on the true model with trace recording (untimed)
    seis = eng.model_seismogram(p.replace(storage=0), ext_true, wav)
    # step-kernel tile width for this grid shape (plans below use it: tile_x = 0)
    tuned = None
    if not args.tile_x:
        tx, ms = eng.autotune(p, 200)
        tuned = {"tile_x": tx, "ms_per_forward_step": ms}

    stream = torch.cuda.Stream()
    plan = eng.Plan(p)
    plan.set_stream(stream.cuda_stream)
    d_vel = torch.from_numpy(ext).cuda()
    d_wav = torch.from_numpy(wav).cuda()
    d_seis = torch.from_numpy(seis).cuda()
    d_img = torch.empty((p.nx, p.nz), dtype=torch.float32, device="cuda")
    d_slf = torch.empty_like(d_img)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > L2

    def migrate():
        plan.forward(d_vel, d_wav)
        plan.adjoint(d_seis, d_img, d_slf)

    # Sampled kernel timing (of every 16 steps, 8 consecutive k_step launches bracketed by one
    # pair of CUDA events on the plan's stream, so that they keep their programmatic overlap)
    # is switched on before the warm-up, so the time-loop graphs are captured with those
    # events outside the timed region; the timed migrations replay them.
    plan.profile(16)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        migrate()
    torch.cuda.synchronize()
    plan.profile_read()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    launches0 = plan.launches
    times = []
    barrier()
    with sampler:
        for _ in range(args.steps):
            flush.fill_(1.0)                      # L2 flush between timed iterations
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            with torch.cuda.stream(stream):
                migrate()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    barrier()
    prof = plan.profile_read()
    plan.profile(0)
    launches = plan.launches - launches0
    total_ms = reduce_over_ranks(float(sum(times)), "max", ws, "cuda")
    cells = p.cell_updates
    value = ws * args.steps * cells / (total_ms * 1e-3) / 1e9
    if args.quick:
        prof_line = {"quick": True, "value": value, "ms_per_step": total_ms / args.steps,
                     "tile_x": p.tile_x, "nt": p.nt, "storage": args.storage,
                     "fwd_kernel_ms": prof["fwd_ms"] / max(prof["fwd_n"], 1),
                     "bwd_kernel_ms": prof["bwd_ms"] / max(prof["bwd_n"], 1),
                     "gpu_launches": int(launches)}
        if rank == 0:
            print(json.dumps(prof_line), flush=True)
        return 0

    # e2e: the reference-shaped host entry point with host buffers (copies in the timed region)
    e2e_ms = []
    img_h = np.zeros((p.nx, p.nz), np.float32)
    for i in range(1 + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        img_h, slf_h = eng.migrate_shot(p, ext, wav, seis)
        dt = (time.perf_counter() - t0) * 1e3
        if i > 0:
            e2e_ms.append(dt)
    e2e_total = reduce_over_ranks(float(sum(e2e_ms)), "max", ws, "cuda")
    e2e_value = ws * args.steps * cells / (e2e_total * 1e-3) / 1e9
    # the same with the seismogram as the ZFP tol 1e-4 stream the workload specifies: decoded
    # on a host thread while the forward pass runs (rtm_migrate_shot_zfp)
    zfp_tol = 1e-4
    zstream = eng.zfp_encode(seis, zfp_tol)
    zfp_ms = []
    for i in range(1 + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.migrate_shot_zfp(p, ext, wav, zstream, zfp_tol)
        dt = (time.perf_counter() - t0) * 1e3
        if i > 0:
            zfp_ms.append(dt)
    zfp_total = reduce_over_ranks(float(sum(zfp_ms)), "max", ws, "cuda")
    t0 = time.perf_counter()
    eng.zfp_decode(zstream, p.rec_count, p.nt, zfp_tol)
    decode_ms = (time.perf_counter() - t0) * 1e3
    e2e_zfp = {"value": ws * args.steps * cells / (zfp_total * 1e-3) / 1e9, "unit": "Gcell-updates/s",
               "ms_per_step": zfp_total / args.steps, "entry_point": "rtm_migrate_shot_zfp",
               "zfp_tolerance": zfp_tol, "stream_bytes": len(zstream),
               "host_decode_ms": decode_ms,
               "h2d_bytes_per_step": int(ext.nbytes + wav.nbytes + seis.nbytes),
               "d2h_bytes_per_step": int(2 * p.nx * p.nz * 4),
               "note": "the stream in host memory; decode (one host thread, serial: the 0.5.5 stream "
                       "has no block offsets) overlapped with the forward pass; timed per migration"}
    # sanity: the device-resident and host paths produce the same image
    dev_img = d_img.cpu().numpy()
    agree = float(np.linalg.norm(dev_img - img_h) / max(np.linalg.norm(img_h), 1e-30))

    # batched UQ ensemble: every rank runs its share of the members (sharded by migration)
    batched = None
    if args.batch_members > 0:
        barrier()
        with ClockSampler(local) as smp:
            batched = run_batched(args, eng, rank, ws)
        batched["clocks"] = smp.summary()

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    nbytes = algorithmic_bytes(p)
    bwd_avg_ms = prof["bwd_ms"] / max(prof["bwd_n"], 1)
    fwd_avg_ms = prof["fwd_ms"] / max(prof["fwd_n"], 1)
    achieved = nbytes["k_step_bwd"] / (bwd_avg_ms * 1e-3) / 1e9
    peak, peak_kind = hbm_peak()
    roofline = {"bound": "hbm", "kernel": "k_step<float,backward>", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic_per_launch(), "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": nbytes["k_step_bwd"],
                "avg_launch_ms": bwd_avg_ms, "sampled_launches": prof["bwd_n"],
                "fwd_kernel_avg_launch_ms": fwd_avg_ms,
                "fwd_kernel_achieved_gbs": nbytes["k_step_fwd"] / (fwd_avg_ms * 1e-3) / 1e9,
                "timing": "CUDA events on the plan's stream around blocks of 8 consecutive launches "
                          "(of every 16 steps) inside the time-loop graph; avg = block time / launches",
                "note": "the step kernel updates the CPML psi itself (no separate psi kernel); "
                        "traffic: cold-cache ncu reads of one launch"}
    served = None
    if ws == 1 and args.serve_requests > 0:
        cap = batched["value"] if batched else value
        with ClockSampler(local) as smp:
            served = run_served(args, eng, cap)
        served["clocks"] = smp.summary()
        served["plain_value_single_shot_3400x700"] = value
        served["speedup_vs_plain_single_shot"] = served["value"] / value
    precision = None
    if ws == 1 and args.precision_nt > 0:
        precision = run_precision(args, eng)
    cpu, parity = None, None
    if ws == 1 and not args.no_cpu_baseline:
        # parity of this very run: the FP32 image and recorded seismogram against the oracle
        # (full size), and the FP32 image against an FP64 GPU run of the identical scheme
        cpu, parity = cpu_full(p, ext_true, ext, wav, seis, img_h, slf_h)
        parity["image_rel_l2_vs_fp64_engine"] = rel_l2(img_h, fp64_image(eng, p, ext, wav, seis))
    line = {"metric": METRIC, "value": value,
            "unit": "Gcell-updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(p, args, ws), "autotuned": tuned,
            "e2e": {"value": e2e_value, "unit": "Gcell-updates/s", "ms_per_step": e2e_total / args.steps,
                    "h2d_bytes_per_step": int(ext.nbytes + wav.nbytes + seis.nbytes),
                    "d2h_bytes_per_step": int(2 * p.nx * p.nz * 4),
                    "entry_point": "rtm_migrate_shot", "image_agreement_rel_l2": agree},
            "e2e_zfp": e2e_zfp,
            "gpu_launches": int(launches), "roofline": roofline, "cpu_baseline": cpu,
            "clocks": sampler.summary(), "precision": precision, "batched": batched, "served": served,
            "parity": parity}
    print(json.dumps(compact_line(line)), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
