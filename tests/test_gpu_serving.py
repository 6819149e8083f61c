"""Serving / batching engine (rtm_server_*): resident migrations advanced together by the
batched step kernels.  Each image matches the reference's (rel-L2 <= 1e-4) and the
single-migration path (<= 1e-5: same scheme, other tiling), and a migration's image is the
same bit for bit whether it runs alone or in a mix of other grids, time axes and storages.
"""
import numpy as np
import pytest

from golden_util import case_params, load, rel_l2

pytestmark = pytest.mark.gpu


def _case(eng, d, name, **kw):
    p = eng.RtmParams.make(**case_params(d, name)).replace(**kw)
    return p, d[name + "/ext"], d[name + "/wavelet"], d[name + "/seis"]


def _shorter(eng, case, nt):
    p, ext, wav, seis = case
    return p.replace(nt=nt), ext, wav, np.ascontiguousarray(seis[:, :nt])


def _mix(eng, d):
    """Different grids, time axes, storages and storage precisions."""
    cases = [_case(eng, d, "uneven", storage=1),
             _case(eng, d, "quirks", storage=0),
             _case(eng, d, "uneven", storage=0, precision=1),
             _case(eng, d, "uneven", storage=1, precision=2)]
    cases.append(_shorter(eng, cases[0], cases[0][0].nt - 60))
    cases.append(_shorter(eng, cases[1], cases[1][0].nt - 80))
    return cases


@pytest.mark.parametrize("name", ("uneven", "quirks"))
@pytest.mark.parametrize("storage", (0, 1))
def test_server_single_request_equals_migrate_shot(engine, name, storage):
    d = load()
    p, ext, wav, seis = _case(engine, d, name, storage=storage)
    try:
        engine.params_check(p)
    except engine.RtmError:
        pytest.skip("shot outside the reconstruction region for this case")
    ref_img, ref_slf = engine.migrate_shot(p, ext, wav, seis)
    img, slf, times = _alone(engine, (p, ext, wav, seis))
    assert rel_l2(img, d[name + "/image"]) <= 1e-4
    assert rel_l2(slf, d[name + "/self"]) <= 1e-4
    assert rel_l2(img, ref_img) <= 1e-5
    assert rel_l2(slf, ref_slf) <= 1e-5
    assert times[0] <= times[1] <= times[2]


def _alone(engine, case):
    srv = engine.Server(0, max_members=4, steps_per_launch=16)
    rid = srv.submit(*case)
    out = srv.run_all()
    srv.close()
    return out[rid]


def test_server_mixed_batch_equals_each_alone(engine):
    d = load()
    cases = _mix(engine, d)
    assert all(_valid(engine, c[0]) for c in cases)
    solo = [_alone(engine, c)[:2] for c in cases]
    # fewer slots than requests: members finish and new ones are admitted mid-run;
    # steps_per_launch not dividing any nt: members finish inside a graph replay
    srv = engine.Server(0, max_members=3, steps_per_launch=7)
    ids = [srv.submit(*c) for c in cases]
    out = srv.run_all()
    st = srv.stats()
    kernel_ms = srv.kernel_ms()
    srv.close()
    for rid, (img, slf) in zip(ids, solo):
        assert np.array_equal(out[rid][0], img), rid
        assert np.array_equal(out[rid][1], slf), rid
    assert st["cell_updates"] == sum(c[0].cell_updates for c in cases)
    assert st["gpu_ms"] > 0 and st["launches"] > 0
    assert 0.0 < kernel_ms < st["gpu_ms"]     # the tile kernel of one step, timed alone


def test_server_wait_returns_the_named_request(engine):
    """rtm_server_wait steps until the named request finishes (out of submission order); the
    others finishing meanwhile stay for rtm_server_poll, and a returned id is refused."""
    d = load()
    cases = _mix(engine, d)[:3]
    solo = [_alone(engine, c)[:2] for c in cases]
    srv = engine.Server(0, max_members=2, steps_per_launch=9)
    ids = [srv.submit(*c) for c in cases]
    img, slf, times = srv.wait(ids[2])
    assert np.array_equal(img, solo[2][0]) and np.array_equal(slf, solo[2][1])
    assert times[0] <= times[1] <= times[2]
    with pytest.raises(engine.RtmError):
        srv.wait(ids[2])
    rest = srv.run_all()
    srv.close()
    assert sorted(rest) == ids[:2]
    for rid, (i, s) in zip(ids[:2], solo[:2]):
        assert np.array_equal(rest[rid][0], i) and np.array_equal(rest[rid][1], s)


def test_server_admission_respects_budget(engine):
    d = load()
    cases = [_case(engine, d, "uneven", storage=1) for _ in range(3)]
    fp = engine.footprint_bytes(cases[0][0])
    srv = engine.Server(int(fp * 1.5), max_members=8, steps_per_launch=32)
    ids = [srv.submit(*c) for c in cases]
    seen = []
    out = {}
    while len(out) < len(ids):
        active, queued = srv.step()
        seen.append(active)
        r = srv.poll()
        while r is not None:
            out[r[0]] = r[1:]
            r = srv.poll()
    assert max(seen) == 1                     # one footprint fits the budget at a time
    assert srv.stats()["bytes_in_use"] <= int(fp * 1.5)
    ref = _alone(engine, cases[0])[0]
    for rid in ids:
        assert np.array_equal(out[rid][0], ref)
    big = cases[0][0].replace(nx=cases[0][0].nx * 4)
    with pytest.raises(engine.RtmError):
        srv.submit(big, np.zeros((big.dim_x, big.dim_z), np.float32), cases[0][2],
                   np.zeros((big.rec_count, big.nt), np.float32))
    with pytest.raises(engine.RtmError):
        srv.submit(cases[0][0].replace(compute=1), *cases[0][1:])
    srv.close()


def test_server_rejects_missing_inputs(engine):
    """A request without its wavelet (n_wavelet > 0) or its seismogram (rec_count > 0) is
    refused at submission, not migrated from whatever the staging buffer holds."""
    import ctypes as C
    from rtmuq2d_gb300 import capi
    d = load()
    p, ext, wav, seis = _case(engine, d, "uneven", storage=1)
    srv = engine.Server(0, max_members=2, steps_per_launch=8)
    lib = capi.lib()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    rid = C.c_longlong()
    ext = np.ascontiguousarray(ext, np.float32)
    wav = np.ascontiguousarray(wav, np.float32)
    seis = np.ascontiguousarray(seis, np.float32)
    assert lib.rtm_server_submit(srv.handle, C.byref(p), fp(ext), None, fp(seis), C.byref(rid)) == \
        capi.RTM_ERR_INVALID
    assert lib.rtm_server_submit(srv.handle, C.byref(p), fp(ext), fp(wav), None, C.byref(rid)) == \
        capi.RTM_ERR_INVALID
    assert lib.rtm_server_submit(srv.handle, C.byref(p), fp(ext), fp(wav), fp(seis), C.byref(rid)) == 0
    srv.params[rid.value] = p                  # what Server.submit records for poll()
    out = srv.run_all()
    srv.close()
    assert list(out) == [rid.value]


def _valid(engine, p):
    try:
        engine.params_check(p)
        return True
    except engine.RtmError:
        return False


def test_server_zfp_submission_equals_decoded_submission(engine):
    """A request carrying the ZFP stream (decoded by the server's host threads while the GPU
    steps) gives the image of the same request carrying the decoded seismogram."""
    d = load()
    p, ext, wav, _ = _case(engine, d, "uneven", storage=1)
    stream = d["zfp/tol1e-4/stream"].tobytes()
    decoded = d["zfp/tol1e-4/decoded"]
    ref = _alone(engine, (p, ext, wav, decoded))[0]
    srv = engine.Server(0, max_members=4, steps_per_launch=16)
    rid = srv.submit_zfp(p, ext, wav, stream, 1e-4)
    rid2 = srv.submit(p, ext, wav, decoded)
    out = srv.run_all()
    srv.close()
    assert np.array_equal(out[rid][0], ref)
    assert np.array_equal(out[rid2][0], ref)


def _phase_cases(engine, oracle):
    """Grids large enough to hold interior tiles (phase 1 of the batched step) beside tiles
    touching a CPML strip (phase 2): the 400 x 200 workload, and a 250 x 258 grid with CPML 30
    whose last z-tile row is shorter than the bottom CPML band."""
    from rtmuq2d_gb300 import workloads
    p = workloads.params_small()
    true, mig = workloads.models_small(p, seed=0)
    wav = workloads.wavelet_for(p)
    ext = engine.extend_matrix(p, mig)
    seis = oracle.model_seismogram(p.as_dict(), engine.extend_matrix(p, true), wav)
    q = workloads.params_small(nx=250, nz=258, th_left=30, th_right=30, th_up=30, th_down=30,
                               nt=1200, shot_x=125, rec_count=125)
    tq, mq = workloads.models_small(q, seed=3)
    wq = workloads.wavelet_for(q)
    extq = engine.extend_matrix(q, mq)
    seisq = oracle.model_seismogram(q.as_dict(), engine.extend_matrix(q, tq), wq)
    return [(p.replace(storage=1), ext, wav, seis),
            (q.replace(storage=1), extq, wq, seisq),
            (p.replace(storage=0), ext, wav, seis),
            (q.replace(storage=0, nt=600), extq, wq, np.ascontiguousarray(seisq[:, :600]))]


def test_server_clear_and_strip_tiles_match_plain_and_oracle(engine, oracle):
    cases = _phase_cases(engine, oracle)
    assert all(_valid(engine, c[0]) for c in cases)
    # two slots for four members of two grids and three time axes: members in different
    # passes share every batched step
    srv = engine.Server(0, max_members=2, steps_per_launch=16)
    ids = [srv.submit(*c) for c in cases]
    out = srv.run_all()
    srv.close()
    for rid, c in zip(ids, cases):
        img, slf = engine.migrate_shot(*c)
        assert rel_l2(out[rid][0], img) <= 1e-5, rid
        assert rel_l2(out[rid][1], slf) <= 1e-5, rid
    for rid, c in zip(ids[:2], cases[:2]):
        ref_img, ref_slf = oracle.migrate(c[0].as_dict(), c[1], c[2], c[3])
        assert rel_l2(out[rid][0], ref_img) <= 1e-4, rid
        assert rel_l2(out[rid][1], ref_slf) <= 1e-4, rid


def test_server_holds_more_than_128_members(engine):
    """More resident members than the old 128-member limit of the batched kernels' tables:
    300 short migrations of a small grid (different shots, so different images) admitted
    together; each image equals the same request migrated alone, bit for bit."""
    d = load()
    p0, ext, wav, seis = _shorter(engine, _case(engine, d, "uneven", storage=1), 40)
    cases = []
    for k in range(300):
        p = p0.replace(shot_x=8 + (k * 7) % max(1, p0.nx - 16))
        if _valid(engine, p):
            cases.append((p, ext, wav, seis))
    assert len(cases) >= 200
    srv = engine.Server(0, max_members=len(cases), steps_per_launch=8)
    ids = [srv.submit(*c) for c in cases]
    out, most = {}, 0
    while True:
        active, queued = srv.step()
        most = max(most, active)
        while True:
            r = srv.poll()
            if r is None:
                break
            out[r[0]] = r[1:]
        if active == 0 and queued == 0 and not srv.params:
            break
    srv.close()
    assert most > 128 and len(out) == len(cases)
    for k in (0, 129, len(cases) - 1):
        img, slf = _alone(engine, cases[k])[:2]
        assert np.array_equal(out[ids[k]][0], img) and np.array_equal(out[ids[k]][1], slf), k


@pytest.mark.parametrize("tile_x", (16, 32))
def test_server_tile_widths_match_plain(engine, tile_x):
    """Both tile widths of the batched kernel (the batched autotuner's choices) give the
    single-migration path's image (rel-L2 <= 1e-5) and the reference's (<= 1e-4)."""
    d = load()
    p, ext, wav, seis = _case(engine, d, "uneven", storage=1)
    ref_img, ref_slf = engine.migrate_shot(p, ext, wav, seis)
    img, slf, _ = _alone(engine, (p.replace(tile_x=tile_x), ext, wav, seis))
    assert rel_l2(img, ref_img) <= 1e-5 and rel_l2(slf, ref_slf) <= 1e-5
    assert rel_l2(img, d["uneven/image"]) <= 1e-4


def test_batched_autotuner_picks_a_width(engine):
    d = load()
    p, ext, wav, seis = _case(engine, d, "uneven", storage=1)
    tx, ms = engine.autotune_batched(p, members=4, steps=24)
    assert tx in (16, 32) and ms > 0
    # later submissions of the shape (tile_x 0) run with it and still match the plain path
    img, slf, _ = _alone(engine, (p.replace(tile_x=0), ext, wav, seis))
    ref_img, _ = engine.migrate_shot(p, ext, wav, seis)
    assert rel_l2(img, ref_img) <= 1e-5
