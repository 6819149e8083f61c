"""Run the synthetic UQ ensemble through the serving engine (rtm_server_*).

    python -m rtmuq2d_gb300.ensemble [--members 8] [--nt 200] [--reps 2] [--storage ring]

Builds `members` velocity realizations of the 3400 x 700 faulted model on uneven aperture
windows (rtmuq2d_gb300.workloads.ensemble), submits them all, runs them to completion `reps`
times and prints one JSON line with the throughput of the last repetition.  Observed data is a
seeded random seismogram (the run measures the engine, not the image).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import capi
from . import workloads


def build_inputs(members: int, nt: int, storage: int, precision: int = 0):
    ens, true, mig = workloads.ensemble(members, nt, storage=storage, precision=precision)
    wav = workloads.wavelet_for(ens[0]["params"])
    inputs = []
    for m in ens:
        p = m["params"]
        _, ext = workloads.ensemble_inputs(m, true, mig)
        seis = (np.random.default_rng(m["seed"]).standard_normal((p.rec_count, p.nt)) * 1e-3).astype(np.float32)
        inputs.append((p, ext, wav, seis))
    return inputs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--members", type=int, default=8)
    ap.add_argument("--nt", type=int, default=200)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--storage", default="ring", choices=("ring", "snapshot"))
    ap.add_argument("--steps-per-launch", type=int, default=16)
    a = ap.parse_args(argv)
    storage = capi.STORE_RING if a.storage == "ring" else capi.STORE_SNAPSHOT
    inputs = build_inputs(a.members, a.nt, storage)
    srv = capi.Server(0, max_members=min(a.members, 128), steps_per_launch=a.steps_per_launch)
    cells = sum(p.cell_updates for p, *_ in inputs)
    wall = gpu_ms = 0.0
    for _ in range(a.reps):
        ms0 = srv.stats()["gpu_ms"]
        t0 = time.perf_counter()
        for inp in inputs:
            srv.submit(*inp)
        srv.run_all()
        wall = time.perf_counter() - t0
        gpu_ms = srv.stats()["gpu_ms"] - ms0
    srv.close()
    print(json.dumps({"members": a.members, "nt": a.nt, "storage": a.storage,
                      "widths": [p.nx for p, *_ in inputs], "seconds": wall,
                      "gcell_updates_per_s": cells / wall / 1e9,
                      "gpu_busy_gcell_updates_per_s": cells / (gpu_ms * 1e-3) / 1e9}))


if __name__ == "__main__":
    main()
