"""The RTM workloads as engine parameters plus their seeded inputs.

* ``plain_small``  400 x 200 model, dx 10 m, CPML 40, dt 1 ms, nt 2000, 15 Hz Ricker,
                   shot at (2000 m, 20 m), 400 receivers one per column at 20 m depth
                   (spacingReceiver = 2 puts receiver i at column i, backward_modeling.c:279).
* ``plain_large``  3400 x 700 faulted model, dx 5 m, CPML 50, dt 0.4 ms, nt 7500, 20 Hz
                   Ricker, 3400 receivers at 5 m depth, shot at the surface mid-line.
* ``tiny``         small grids for step-level parity tests.

Each builder returns (params, inputs) where inputs holds the padded migration velocity,
the wavelet, and (when asked) the observed seismogram modelled on the true model.
"""
from __future__ import annotations

import numpy as np

from . import synth
from .capi import RtmParams, STORE_RING


def params_small(**kw) -> RtmParams:
    base = dict(nx=400, nz=200, th_left=40, th_right=40, th_up=40, th_down=40, dx=10.0, dt=1e-3,
                nt=2000, n_wavelet=800, shot_x=200, shot_z=2, rec_first=0, rec_spacing=2,
                rec_count=400, rec_depth=2, time_slices=20, storage=STORE_RING)
    base.update(kw)
    return RtmParams.make(**base)


def params_large(**kw) -> RtmParams:
    base = dict(nx=3400, nz=700, th_left=50, th_right=50, th_up=50, th_down=50, dx=5.0, dt=4e-4,
                nt=7500, n_wavelet=800, shot_x=1700, shot_z=1, rec_first=0, rec_spacing=2,
                rec_count=3400, rec_depth=1, time_slices=20, storage=STORE_RING)
    base.update(kw)
    return RtmParams.make(**base)


def params_tiny(nx=96, nz=64, th=16, nt=240, **kw) -> RtmParams:
    base = dict(nx=nx, nz=nz, th_left=th, th_right=th, th_up=th, th_down=th, dx=10.0, dt=1e-3,
                nt=nt, n_wavelet=min(nt, 120), shot_x=nx // 2, shot_z=2, rec_first=0,
                rec_spacing=2, rec_count=nx, rec_depth=2, time_slices=20, storage=STORE_RING)
    base.update(kw)
    return RtmParams.make(**base)


def extend(p: RtmParams, model: np.ndarray) -> np.ndarray:
    """Host padding with the reference's edge replication (generic_functions.c:5-48)."""
    from .capi import extend_matrix
    return extend_matrix(p, model)


def models_small(p: RtmParams, seed: int = 0):
    true = synth.layered_model(p.nx, p.nz, p.dx, seed)
    mig = synth.smooth(true, 80.0, p.dx)
    return true, mig


def models_large(p: RtmParams, seed: int = 1):
    true = synth.faulted_model(p.nx, p.nz, p.dx, seed)
    mig = synth.smooth(true, 40.0, p.dx)
    return true, mig


def models_tiny(p: RtmParams, seed: int = 0):
    rng = np.random.default_rng(seed)
    z = np.arange(p.nz) * p.dx
    v = np.where(z < p.nz * p.dx * 0.5, 1800.0, 2400.0)
    true = (np.broadcast_to(v, (p.nx, p.nz)) * (1 + 0.02 * rng.standard_normal((p.nx, p.nz)))).astype(np.float32)
    mig = synth.smooth(true, 3 * p.dx, p.dx)
    return true, mig


def wavelet_for(p: RtmParams, f0: float | None = None) -> np.ndarray:
    if f0 is None:
        f0 = 15.0 if p.dt >= 1e-3 else 20.0
    return synth.ricker(f0, p.dt, max(p.n_wavelet, 1))[: max(p.n_wavelet, 1)]


# ---- batched ensemble and serving trace -------------------------------------------------------
def ensemble(n: int = 64, nt: int = 7500, seed: int = 11, storage: int = STORE_RING, precision: int = 0):
    """The batched UQ ensemble: n velocity realizations of the 3400 x 700 faulted model, each
    multiplied by exp(0.03 g_k) (g_k: independent unit Gaussian random field, 200 m
    correlation), paired with one shot on an aperture window of width U[1200, 3400] cells
    (full depth, 700).  The shot sits at the window centre, one receiver per window column.

    Returns (members, true_model) with members a list of dicts: params, offset (first model
    column of the window), seed."""
    base = params_large(storage=storage, precision=precision, nt=nt)
    true, mig = models_large(base, seed=1)
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        w = int(rng.integers(1200, 3401))
        o = int(rng.integers(0, 3400 - w + 1))
        p = base.replace(nx=w, shot_x=w // 2, rec_count=w)
        out.append({"params": p, "offset": o, "seed": seed * 1000 + k})
    return out, true, mig


def ensemble_inputs(member: dict, true: np.ndarray, mig: np.ndarray):
    """Padded true and migration velocities of one ensemble member (the realization
    perturbs the migration model)."""
    p, o = member["params"], member["offset"]
    g = synth.grf_coarse((p.nx, p.nz), p.dx, 200.0, member["seed"])
    vmig = (mig[o:o + p.nx].astype(np.float64) * np.exp(0.03 * g)).astype(np.float32)
    return extend(p, np.ascontiguousarray(true[o:o + p.nx])), extend(p, vmig)


SERVING_GRIDS = ((400, 200), (1200, 400), (2000, 600), (3400, 700))


def serving_template(k: int, nt: int = 7500) -> tuple:
    """Grid template k of the serving trace: (params with nt, true model, migration model).
    The two smaller grids use the layered model at 10 m (dt 1 ms, CPML 40, 15 Hz), the two
    larger the faulted model at 5 m (dt 0.4 ms, CPML 50, 20 Hz); one receiver per column,
    shot at the surface mid-line."""
    nx, nz = SERVING_GRIDS[k]
    if k < 2:
        p = params_small(nx=nx, nz=nz, shot_x=nx // 2, rec_count=nx, nt=nt)
        true, mig = synth.layered_model(nx, nz, p.dx, 100 + k), None
        mig = synth.smooth(true, 80.0, p.dx)
    else:
        p = params_large(nx=nx, nz=nz, shot_x=nx // 2, rec_count=nx, nt=nt)
        true = synth.faulted_model(nx, nz, p.dx, 100 + k)
        mig = synth.smooth(true, 40.0, p.dx)
    return p, true, mig


SERVING_NT = (2000, 3000, 4000, 5000, 6000, 7500)


def serving_trace(n: int, seed: int = 23):
    """Requests of the serving trace: grid template uniform over SERVING_GRIDS, nt uniform
    over SERVING_NT (2000..7500; a few values so that each (grid, nt) seismogram is
    ZFP-compressed once), FP32 or BF16 ring storage, own realization seed."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        reqs.append({"grid": int(rng.integers(0, len(SERVING_GRIDS))),
                     "nt": int(SERVING_NT[int(rng.integers(0, len(SERVING_NT)))]),
                     "precision": int(rng.integers(0, 2)),
                     "seed": seed * 100000 + i})
    return reqs
