"""The migration driver on files (rtm_routine, SRC/rtm_iso2d.c:15-177) against the
reference's own rtm_routine run on the same files (tests/golden/make_golden.py): two shots,
ZFP tol 1e-4 seismograms, stacked image and its Laplacian.  Run through the engine's C
entry point and through the reference-named drop-in library."""
import ctypes as C
import os

import numpy as np
import pytest

from golden_util import case_params, load, rel_l2

pytestmark = pytest.mark.gpu


def _setup(engine, tmp_path):
    d = load()
    sim_id, n_shots, first, spacing, depth = (int(v) for v in d["routine/survey"])
    tol = float(d["routine/tol"][0])
    for sub in ("INPUTS", "OUTPUTS"):
        (tmp_path / sub).mkdir()
    d["uneven/model"].astype(np.float32).tofile(tmp_path / "INPUTS" / ("vp_%05d.bin" % sim_id))
    d["uneven/wavelet"].astype(np.float32).tofile(tmp_path / "INPUTS" / "wavelet.bin")
    for k in range(1, n_shots + 1):
        (tmp_path / "INPUTS" / ("seismogram_%05d.zfp" % k)).write_bytes(d["routine/seis_%d" % k].tobytes())
    p = engine.RtmParams.make(**case_params(d, "uneven"))
    s = engine.RtmSurvey.make(str(tmp_path / "INPUTS" / "vp_%05d.bin"), str(tmp_path / "INPUTS" / "wavelet.bin"),
                              str(tmp_path / "INPUTS" / "seismogram_%05d.zfp"),
                              str(tmp_path / "OUTPUTS" / "stackedBrute_%05d.bin"),
                              str(tmp_path / "OUTPUTS" / "stackedLaplacian_%05d.bin"),
                              first_shot=first, shot_depth=depth, shot_spacing=spacing, n_shots=n_shots,
                              zfp_tolerance=tol)
    return d, p, s, sim_id


def _outputs(d, tmp_path, sim_id):
    p = case_params(d, "uneven")
    st = np.fromfile(tmp_path / "OUTPUTS" / ("stackedBrute_%05d.bin" % sim_id), np.float32)
    lp = np.fromfile(tmp_path / "OUTPUTS" / ("stackedLaplacian_%05d.bin" % sim_id), np.float32)
    return st.reshape(p["nx"], p["nz"]), lp.reshape(p["nx"], p["nz"])


@pytest.mark.parametrize("storage", (0, 1))
def test_routine_matches_reference(engine, tmp_path, storage):
    d, p, s, sim_id = _setup(engine, tmp_path)
    engine.routine_run(p.replace(storage=storage), s, sim_id)
    st, lp = _outputs(d, tmp_path, sim_id)
    assert rel_l2(st, d["routine/stacked"]) <= 1e-4
    assert rel_l2(lp, d["routine/laplacian"]) <= 1e-4
    # the shots are stacked on the device: one copy back (stack, Laplacian, status word)
    assert engine.routine_last_transfers() == (1, 2 * p.nx * p.nz * 4 + 4)


def test_device_stack_equals_host_stack(engine, tmp_path):
    """rtm_stack: the shots' images added on the device in shot order equal, bit for bit, the
    host-side sum of the same shots' images from rtm_adjoint_modeling (float32, shot order, as
    rtm_iso2d.c:121-126 sums them), and its Laplacian equals laplacian_filter2D of that sum;
    one device-to-host copy for the whole stack."""
    d, p, s, sim_id = _setup(engine, tmp_path)
    _, n_shots, first, spacing, depth = (int(v) for v in d["routine/survey"])
    tol = float(d["routine/tol"][0])
    ext = engine.extend_matrix(p, d["uneven/model"])
    wav = d["uneven/wavelet"]
    host_img = np.zeros((p.nx, p.nz), np.float32)
    host_slf = np.zeros((p.nx, p.nz), np.float32)
    stack = engine.Stack(p)
    for k in range(n_shots):
        shot = (first + k * spacing, depth)
        seis = engine.zfp_decode(d["routine/seis_%d" % (k + 1)].tobytes(), p.rec_count, p.nt, tol)
        img = np.zeros((p.nx, p.nz), np.float32)
        slf = np.zeros((p.nx, p.nz), np.float32)
        engine.forward_modeling(p, 5, shot, ext, wav)
        engine.adjoint_modeling(p, 5, shot, ext, wav, seis, img, slf)
        host_img = host_img + img
        host_slf = host_slf + slf
        engine.forward_modeling(p, 6, shot, ext, wav)
        stack.adjoint(p.replace(shot_x=shot[0], shot_z=shot[1]), 6, shot, seis)
    out, lap = stack.finish()
    assert stack.transfers() == (1, 2 * p.nx * p.nz * 4 + 4)
    assert np.array_equal(out, host_img)
    assert np.array_equal(lap, engine.laplacian_filter2D(p, host_img))
    raw_img, raw_slf = stack.read_raw()
    assert np.array_equal(raw_img, host_img) and np.array_equal(raw_slf, host_slf)
    norm, _ = stack.finish(normalize_by_self=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        want = np.where(host_slf != 0, host_img / host_slf, np.float32(0)).astype(np.float32)
    assert np.array_equal(norm, want)
    stack.close()


def test_stack_normalization_zero_guard(engine):
    """A pixel whose self-image stack is 0 (no source energy reached it) is 0 in the normalised
    stack, not the 0/0 or x/0 of the reference's commented-out division; every other pixel is
    the float quotient."""
    d = load()
    p = engine.RtmParams.make(**case_params(d, "uneven"))
    rng = np.random.default_rng(4)
    img = rng.standard_normal((p.nx, p.nz)).astype(np.float32)
    slf = np.abs(rng.standard_normal((p.nx, p.nz))).astype(np.float32)
    slf[:, : p.nz // 3] = 0.0                      # a shadow zone
    img[: p.nx // 2, : p.nz // 3] = 0.0           # 0/0 there, x/0 beside it
    stack = engine.Stack(p)
    stack.load(img, slf)
    out, lap = stack.finish(normalize_by_self=True)
    stack.close()
    assert np.isfinite(out).all() and np.isfinite(lap).all()
    assert not np.any(out[:, : p.nz // 3])
    assert np.array_equal(out[:, p.nz // 3:], img[:, p.nz // 3:] / slf[:, p.nz // 3:])


def test_dropin_rtm_routine_matches_reference(engine, tmp_path):
    d, p, s, sim_id = _setup(engine, tmp_path)
    L = engine.dropin_lib()
    L.rtm_dropin_configure.argtypes = [C.POINTER(engine.RtmParams), C.POINTER(engine.RtmSurvey)]
    assert L.rtm_dropin_configure(C.byref(p), C.byref(s)) == 0
    L.rtm_routine(C.c_int(sim_id))
    st, lp = _outputs(d, tmp_path, sim_id)
    assert rel_l2(st, d["routine/stacked"]) <= 1e-4
    assert rel_l2(lp, d["routine/laplacian"]) <= 1e-4


def test_routine_missing_input_is_an_io_error(engine, tmp_path):
    d, p, s, sim_id = _setup(engine, tmp_path)
    os.unlink(tmp_path / "INPUTS" / "seismogram_00002.zfp")
    with pytest.raises(engine.RtmError) as e:
        engine.routine_run(p, s, sim_id)
    assert e.value.status == 6


def test_routine_batch_matches_routine_per_simulation(engine, tmp_path):
    """Two simulations (two velocity files) with their shots through one batched server: each
    simulation's stack equals the single-simulation driver's (<= 1e-5: the batched kernels,
    same scheme), its Laplacian -- a second derivative, which amplifies the stack's last-bit
    differences -- within the image bar 1e-4, and both the reference's (<= 1e-4)."""
    d, p, s, sim_id = _setup(engine, tmp_path)
    other = sim_id + 7
    model = d["uneven/model"].astype(np.float32)
    (model * np.float32(1.03)).tofile(tmp_path / "INPUTS" / ("vp_%05d.bin" % other))
    engine.routine_batch(p, s, [sim_id, other], max_members=3)
    batch = {k: _outputs(d, tmp_path, k) for k in (sim_id, other)}
    for k in (sim_id, other):
        engine.routine_run(p, s, k)
        single = _outputs(d, tmp_path, k)
        assert rel_l2(batch[k][0], single[0]) <= 1e-5, k
        assert rel_l2(batch[k][1], single[1]) <= 1e-4, k
    assert rel_l2(batch[sim_id][0], d["routine/stacked"]) <= 1e-4
    assert rel_l2(batch[sim_id][1], d["routine/laplacian"]) <= 1e-4
    assert rel_l2(batch[other][0], batch[sim_id][0]) > 1e-3     # the second model differs


@pytest.mark.parametrize("batched", (False, True))
def test_routine_stack_normalized_by_self_image(engine, oracle, tmp_path, batched):
    """normalize_by_self: the whole-survey branch the reference leaves commented out
    (rtm_iso2d.c:152), the image stack divided by the self-image stack.  Checked against the
    oracle's per-shot images and self images of the same decoded seismograms, summed in shot
    order: stack * self_stack reproduces the image stack within the image bar (1e-4) wherever
    the quotient is finite."""
    d, p, s, sim_id = _setup(engine, tmp_path)
    s.normalize_by_self = 1
    if batched:
        engine.routine_batch(p, s, [sim_id], max_members=2)
    else:
        engine.routine_run(p, s, sim_id)
    st, lp = _outputs(d, tmp_path, sim_id)
    _, n_shots, first, spacing, depth = (int(v) for v in d["routine/survey"])
    tol = float(d["routine/tol"][0])
    img = np.zeros((p.nx, p.nz), np.float32)
    slf = np.zeros((p.nx, p.nz), np.float32)
    for k in range(n_shots):
        q = p.replace(shot_x=first + k * spacing, shot_z=depth)
        ext = oracle.extend_matrix(q.as_dict(), d["uneven/model"])
        seis = engine.zfp_decode(d["routine/seis_%d" % (k + 1)].tobytes(), q.rec_count, q.nt, tol)
        oi, os_ = oracle.migrate(q.as_dict(), ext, d["uneven/wavelet"], seis)
        img = img + oi
        slf = slf + os_
    ok = np.isfinite(st) & (slf > 0)
    assert ok.mean() > 0.9
    assert rel_l2(st[ok] * slf[ok], img[ok]) <= 1e-4
    assert rel_l2(img, d["routine/stacked"]) <= 1e-4          # the oracle's plain stack, pinned


def test_routine_resumes_from_its_checkpoint(engine, tmp_path):
    """With a checkpoint file, a run that fails at shot 2 (its seismogram missing) keeps the
    stacks of shot 1; the rerun resumes at shot 2 -- shot 1's seismogram is gone by then, so
    it cannot have run it again -- and writes the same files, bit for bit, as an uninterrupted
    run (the same float sums in shot order); the checkpoint is removed afterwards."""
    d, p, s, sim_id = _setup(engine, tmp_path)
    engine.routine_run(p, s, sim_id)
    want = _outputs(d, tmp_path, sim_id)
    for f in (tmp_path / "OUTPUTS").iterdir():
        f.unlink()
    ck = tmp_path / "OUTPUTS" / "stack_%05d.ckpt"
    s2 = engine.RtmSurvey.make(*(getattr(s, k).decode() for k in ("velocity_file", "wavelet_file",
                                                                    "seismogram_file", "stacked_file",
                                                                    "laplacian_file")),
                               first_shot=s.first_shot, shot_depth=s.shot_depth,
                               shot_spacing=s.shot_spacing, n_shots=s.n_shots,
                               zfp_tolerance=s.zfp_tolerance, checkpoint_file=str(ck))
    seis2 = tmp_path / "INPUTS" / "seismogram_00002.zfp"
    hidden = tmp_path / "seismogram_00002.zfp"
    seis2.rename(hidden)
    with pytest.raises(engine.RtmError):
        engine.routine_run(p, s2, sim_id)
    ckpt = tmp_path / "OUTPUTS" / ("stack_%05d.ckpt" % sim_id)
    assert ckpt.exists()
    hidden.rename(seis2)
    (tmp_path / "INPUTS" / "seismogram_00001.zfp").unlink()
    engine.routine_run(p, s2, sim_id)
    got = _outputs(d, tmp_path, sim_id)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    assert not ckpt.exists()
    # with a checkpoint file, the stacks come back after each shot too
    assert engine.routine_last_transfers()[0] == 1 + (s.n_shots - 1)


def test_routine_ignores_a_checkpoint_of_another_survey(engine, tmp_path):
    """A checkpoint left by a survey of the same shape but another shot geometry is not
    resumed: the run starts from zero stacks and writes what an uninterrupted run writes."""
    d, p, s, sim_id = _setup(engine, tmp_path)
    ck = str(tmp_path / "OUTPUTS" / "stack_%05d.ckpt")

    def survey(first_shot):
        return engine.RtmSurvey.make(*(getattr(s, k).decode() for k in ("velocity_file", "wavelet_file",
                                                                          "seismogram_file", "stacked_file",
                                                                          "laplacian_file")),
                                     first_shot=first_shot, shot_depth=s.shot_depth,
                                     shot_spacing=s.shot_spacing, n_shots=s.n_shots,
                                     zfp_tolerance=s.zfp_tolerance, checkpoint_file=ck)

    other = survey(s.first_shot + 2)
    seis2 = tmp_path / "INPUTS" / "seismogram_00002.zfp"
    hidden = tmp_path / "seismogram_00002.zfp"
    seis2.rename(hidden)
    with pytest.raises(engine.RtmError):
        engine.routine_run(p, other, sim_id)       # leaves a checkpoint after its shot 1
    assert os.path.exists(ck % sim_id)
    hidden.rename(seis2)
    engine.routine_run(p, survey(s.first_shot), sim_id)
    got = _outputs(d, tmp_path, sim_id)
    for f in (tmp_path / "OUTPUTS").iterdir():
        f.unlink()
    engine.routine_run(p, s, sim_id)
    want = _outputs(d, tmp_path, sim_id)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
