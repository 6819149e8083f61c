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
