"""The C-ABI library without a GPU: it loads, exports every entry point declared in
include/*.h, and its host-side logic (parameter checks, footprint, CPML profiles, model
padding) matches the oracle.  No CUDA compute call is made."""
import os
import re

import numpy as np
import pytest

from golden_util import case_params, load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rtm_[a-zA-Z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine):
    lib = engine.lib()
    names = _declared("rtm_gpu.h")
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_params_check_rejects_bad_configurations(engine):
    from rtmuq2d_gb300 import workloads
    from rtmuq2d_gb300.capi import RtmError, params_check
    p = workloads.params_small()
    params_check(p)
    for bad in (dict(th_left=8), dict(nt=2001), dict(time_slices=0), dict(dx=0.0),
                dict(shot_x=10_000), dict(rec_first=-100), dict(rec_depth=10_000),
                dict(storage=7), dict(precision=9), dict(compute=3), dict(tile_x=12),
                dict(compute=1, precision=1)):
        with pytest.raises(RtmError):
            params_check(p.replace(**bad))
    # ring storage needs the shot inside the stencil-only region; snapshots do not
    q = p.replace(shot_z=-38)
    with pytest.raises(RtmError):
        params_check(q)
    params_check(q.replace(storage=0))


def test_entry_points_reject_missing_inputs(engine):
    """Null inputs are refused with RTM_ERR_INVALID before any device work."""
    import ctypes as C
    from rtmuq2d_gb300 import capi, workloads
    p = workloads.params_tiny()
    lib = capi.lib()
    vel = np.ones((p.dim_x, p.dim_z), np.float32)
    wav = np.ones(p.n_wavelet, np.float32)
    seis = np.zeros((p.rec_count, p.nt), np.float32)
    img = np.zeros((p.nx, p.nz), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    inv = capi.RTM_ERR_INVALID
    assert lib.rtm_migrate_shot(C.byref(p), fp(vel), None, fp(seis), fp(img), fp(img)) == inv
    assert lib.rtm_migrate_shot(C.byref(p), fp(vel), fp(wav), None, fp(img), fp(img)) == inv
    assert lib.rtm_migrate_shot(C.byref(p), None, fp(wav), fp(seis), fp(img), fp(img)) == inv
    assert lib.rtm_model_seismogram(C.byref(p), fp(vel), None, fp(seis)) == inv
    rid = C.c_longlong()
    assert lib.rtm_server_submit(None, C.byref(p), fp(vel), fp(wav), fp(seis), C.byref(rid)) == inv
    assert lib.rtm_server_wait(None, 1, None, None, None) == inv


def test_footprint_accounts_for_storage(engine):
    from rtmuq2d_gb300 import workloads
    from rtmuq2d_gb300.capi import footprint_bytes
    p = workloads.params_large()
    ring = footprint_bytes(p)
    snap = footprint_bytes(p.replace(storage=0))
    half = footprint_bytes(p.replace(precision=1))
    ring_cells = 8 * (3400 + 16) + 8 * (700 + 8)
    assert ring > (7500 + 1) * ring_cells * 4
    assert snap > 375 * 3400 * 800 * 4
    assert half < ring
    assert footprint_bytes(p.replace(nt=7)) == -1


@pytest.mark.parametrize("name", ("uneven", "quirks"))
def test_host_setup_matches_reference_fixtures(engine, name):
    from rtmuq2d_gb300.capi import RtmParams, attenuation_profile_cpml, extend_matrix
    d = load()
    p = RtmParams.make(**case_params(d, name))
    assert np.array_equal(extend_matrix(p, d[name + "/model"]), d[name + "/ext"])
    prof = attenuation_profile_cpml(p)
    for k, v in prof.items():
        assert np.allclose(v, d[name + "/prof_" + k], rtol=2e-7, atol=0), k
