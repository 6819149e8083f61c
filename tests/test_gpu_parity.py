"""CUDA engine vs the oracle / the reference's own outputs, through the C ABI.

Tolerances (relative L2 over the whole array):
  one step (stencil, CPML)           <= 1e-6   (FMA contraction is the only difference)
  wavefields / seismograms after nt  <= 1e-5
  images, snapshot storage           <= 1e-4   (the stated bar for the FP32 path)
  images, ring reconstruction        <= 1e-4
  FP64 engine vs FP64 oracle         <= 1e-10
"""
import numpy as np
import pytest

from golden_util import case_params, load, rel_l2

pytestmark = pytest.mark.gpu

CASES = ("uneven", "quirks")


def _params(eng, d, name, **kw):
    p = eng.RtmParams.make(**case_params(d, name))
    return p.replace(**kw)


def test_step_stencil_matches_reference_kat(engine):
    d = load()
    p = _params(engine, d, "uneven")
    out = engine.iso_acoustic_wave_equation(p, d["kat/coef"], d["kat/u1"], d["kat/u2"])
    assert rel_l2(out, d["kat/stencil"]) <= 1e-6
    # cells the reference never writes (outer 4-cell frame) are untouched
    assert np.array_equal(out[:4], d["kat/u2"][:4]) and np.array_equal(out[:, -4:], d["kat/u2"][:, -4:])


def test_step_cpml_matches_reference_kat(engine):
    d = load()
    p = _params(engine, d, "uneven")
    psi = {k: d["kat/psi_in_" + k].copy() for k in "lrtb"}
    xi = {k: d["kat/xi_in_" + k].copy() for k in "lrtb"}
    prof = engine.attenuation_profile_cpml(p)
    out = engine.aiso_attenuation_cpml(p, d["kat/u1"], d["kat/u2"], d["kat/coef"], prof, psi, xi)
    assert rel_l2(out, d["kat/cpml"]) <= 1e-6
    for k in "lrtb":
        assert rel_l2(psi[k], d["kat/psi_out_" + k]) <= 1e-6, k
        assert rel_l2(xi[k], d["kat/xi_out_" + k]) <= 1e-6, k


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("storage", (0, 1))
def test_migration_matches_reference(engine, name, storage):
    d = load()
    p = _params(engine, d, name, storage=storage)
    if storage == 1:
        try:
            engine.params_check(p)
        except engine.RtmError:
            pytest.skip("shot outside the reconstruction region for this case")
    img, slf = engine.migrate_shot(p, d[name + "/ext"], d[name + "/wavelet"], d[name + "/seis"])
    assert np.abs(img).max() > 0
    assert rel_l2(img, d[name + "/image"]) <= 1e-4
    assert rel_l2(slf, d[name + "/self"]) <= 1e-4


@pytest.mark.parametrize("name", CASES)
def test_forward_final_fields_and_recording_match_oracle(engine, oracle, name):
    import torch
    d = load()
    p = _params(engine, d, name, storage=0)
    ext, wav = d[name + "/ext"], d[name + "/wavelet"]
    ref = oracle.forward(p.as_dict(), ext, wav, snapshots=False, record=True)
    plan = engine.Plan(p)
    dv = torch.from_numpy(ext).cuda()
    dw = torch.from_numpy(wav).cuda()
    seis = torch.zeros((p.rec_count, p.nt), dtype=torch.float32, device="cuda")
    plan.forward(dv, dw, seis)
    plan.sync()
    last = torch.empty((p.dim_x, p.dim_z), dtype=torch.float32, device="cuda")
    prev = torch.empty_like(last)
    plan.read_field(0, last)
    plan.read_field(1, prev)
    assert rel_l2(last.cpu().numpy(), ref["u_last"]) <= 1e-5
    assert rel_l2(prev.cpu().numpy(), ref["u_prev"]) <= 1e-5
    assert rel_l2(seis.cpu().numpy(), ref["seis"]) <= 1e-5
    plan.close()


def test_model_seismogram_host_entry_point(engine, oracle):
    d = load()
    p = _params(engine, d, "uneven")
    true = d["uneven/ext"] * np.float32(1.04)
    seis = engine.model_seismogram(p, true, d["uneven/wavelet"])
    assert rel_l2(seis, d["uneven/seis"]) <= 1e-5


def test_sim_id_forward_then_adjoint(engine):
    d = load()
    p = _params(engine, d, "uneven", storage=1)
    shot = (p.shot_x, p.shot_z)
    engine.forward_modeling(p, 3, shot, d["uneven/ext"], d["uneven/wavelet"])
    engine.forward_modeling(p, 4, shot, d["uneven/ext"], d["uneven/wavelet"])
    img = np.zeros((p.nx, p.nz), np.float32)
    slf = np.zeros((p.nx, p.nz), np.float32)
    engine.adjoint_modeling(p, 4, shot, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"], img, slf)
    engine.adjoint_modeling(p, 3, shot, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"], img, slf)
    # two identical shots accumulated into the same buffers
    assert rel_l2(img, 2 * d["uneven/image"]) <= 1e-4
    with pytest.raises(engine.RtmError) as e:
        engine.adjoint_modeling(p, 3, shot, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"], img, slf)
    assert e.value.status == 4   # RTM_ERR_STATE: the state of sim 3 was consumed


@pytest.mark.parametrize("storage", (0, 1))
def test_fp64_engine_matches_fp64_oracle(engine, oracle, storage):
    import torch
    d = load()
    name = "uneven"
    p = _params(engine, d, name, storage=storage, compute=1)
    ext, wav, seis = d[name + "/ext"], d[name + "/wavelet"], d[name + "/seis"]
    ref_img, ref_slf = oracle.migrate(p.as_dict(), ext, wav, seis, dtype=np.float64)
    plan = engine.Plan(p)
    plan.forward(torch.from_numpy(ext).cuda(), torch.from_numpy(wav).cuda())
    plan.adjoint(torch.from_numpy(seis).cuda())
    img = torch.empty((p.nx, p.nz), dtype=torch.float64, device="cuda")
    slf = torch.empty_like(img)
    plan.read_image(0, img, as_double=True)
    plan.read_image(1, slf, as_double=True)
    plan.sync()
    tol = 1e-10 if storage == 0 else 1e-8
    assert rel_l2(img.cpu().numpy(), ref_img) <= tol
    assert rel_l2(slf.cpu().numpy(), ref_slf) <= tol
    plan.close()


def test_laplacian_and_xcorr_drop_ins(engine, oracle):
    d = load()
    p = _params(engine, d, "uneven")
    lp = engine.laplacian_filter2D(p, d["kat/lap_in"])
    assert rel_l2(lp, d["kat/lap_out"]) <= 1e-6
    assert np.all(lp[:4] == 0) and np.all(lp[:, -4:] == 0)
    img = np.full((p.nx, p.nz), 0.5, np.float32)
    slf = np.zeros((p.nx, p.nz), np.float32)
    s, r = d["kat/u1"], d["kat/u2"]
    engine.normalized_cross_correlation(p, img, slf, s, r)
    ri, rs = np.full((p.nx, p.nz), 0.5, np.float32), np.zeros((p.nx, p.nz), np.float32)
    oracle.xcorr(p.as_dict(), ri, rs, s, r)
    assert rel_l2(img, ri) <= 1e-6 and rel_l2(slf, rs) <= 1e-6


@pytest.mark.parametrize("tile_x", (8, 16, 32))
def test_tile_widths_agree(engine, tile_x):
    d = load()
    p = _params(engine, d, "uneven", storage=1, tile_x=tile_x)
    img, _ = engine.migrate_shot(p, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"])
    assert rel_l2(img, d["uneven/image"]) <= 1e-4


def test_small_workload_against_oracle(engine, oracle):
    """The 400 x 200, nt = 2000 plain workload: ring and snapshot storage vs the oracle."""
    from rtmuq2d_gb300 import workloads
    p = workloads.params_small()
    true, mig = workloads.models_small(p, seed=0)
    wav = workloads.wavelet_for(p)
    ext_true = engine.extend_matrix(p, true)
    ext = engine.extend_matrix(p, mig)
    seis = oracle.model_seismogram(p.as_dict(), ext_true, wav)
    ref_img, ref_slf = oracle.migrate(p.as_dict(), ext, wav, seis)
    for storage in (0, 1):
        img, slf = engine.migrate_shot(p.replace(storage=storage), ext, wav, seis)
        assert rel_l2(img, ref_img) <= 1e-4, storage
        assert rel_l2(slf, ref_slf) <= 1e-4, storage


@pytest.fixture(scope="module")
def small_workload(engine, oracle):
    """The 400 x 200, nt 2000 workload (CPML 40, 400 receivers) with its observed seismogram
    modelled by the oracle on the true model."""
    from rtmuq2d_gb300 import workloads
    p = workloads.params_small()
    true, mig = workloads.models_small(p, seed=0)
    wav = workloads.wavelet_for(p)
    ext_true = engine.extend_matrix(p, true)
    ext = engine.extend_matrix(p, mig)
    seis = oracle.model_seismogram(p.as_dict(), ext_true, wav)
    return p, ext, wav, seis


def test_small_workload_through_zfp_matches_oracle(engine, oracle, small_workload):
    """The 400 x 200 workload as its configuration states it: the observed seismogram a ZFP
    fixed-accuracy stream at tolerance 1e-4 (written by the codec that is byte-identical to
    the reference's library), decoded on the host by the server and by the file-level path;
    the served and the plain images against the oracle's migration of the decoded data."""
    p, ext, wav, seis = small_workload
    tol = 1e-4
    stream = engine.zfp_encode(seis, tol)
    dec = engine.zfp_decode(stream, p.rec_count, p.nt, tol).reshape(p.rec_count, p.nt)
    assert np.max(np.abs(dec - seis)) <= tol and len(stream) < seis.nbytes
    ref_img, ref_slf = oracle.migrate(p.as_dict(), ext, wav, dec)
    srv = engine.Server(0, max_members=4)
    rid = srv.submit_zfp(p, ext, wav, stream, tol)
    img, slf, _ = srv.wait(rid)
    srv.close()
    assert rel_l2(img, ref_img) <= 1e-4 and rel_l2(slf, ref_slf) <= 1e-4
    img, slf = engine.migrate_shot(p, ext, wav, dec)
    assert rel_l2(img, ref_img) <= 1e-4 and rel_l2(slf, ref_slf) <= 1e-4
    # the host entry point taking the stream itself (decoded on a host thread meanwhile)
    zimg, zslf = engine.migrate_shot_zfp(p, ext, wav, stream, tol)
    assert np.array_equal(zimg, img) and np.array_equal(zslf, slf)
    with pytest.raises(engine.RtmError) as e:
        engine.migrate_shot_zfp(p, ext, wav, stream[: len(stream) // 3], tol)
    assert e.value.status == 7                   # RTM_ERR_DECODE


@pytest.mark.parametrize("storage", (0, 1))
@pytest.mark.parametrize("precision", (1, 2))
def test_16bit_storage_within_1e3_of_fp64_oracle(engine, oracle, small_workload, storage, precision):
    """BF16 / FP16 source-wavefield storage (per-step, per-tile max-abs scales; stencil and
    CPML in FP32, image in FP64) on the 400 x 200, nt 2000 workload: the image within relative
    L2 1e-3 of the FP64 oracle's image of the identical scheme.  The self image squares each
    stored sample, doubling its relative rounding error: BF16 keeps 8 significant bits
    (rounding error up to 2^-9 of a sample), so its self image is held to 3e-3, FP16 (11 bits)
    to 1e-3."""
    p, ext, wav, seis = small_workload
    ref_img, ref_slf = oracle.migrate(p.as_dict(), ext, wav, seis, dtype=np.float64)
    q = p.replace(storage=storage, precision=precision)
    img, slf = engine.migrate_shot(q, ext, wav, seis)
    fp32, _ = engine.migrate_shot(q.replace(precision=0), ext, wav, seis)
    assert not np.array_equal(img, fp32)     # the 16-bit path really ran
    assert rel_l2(img, ref_img) <= 1e-3
    assert rel_l2(slf, ref_slf) <= (3e-3 if precision == 1 else 1e-3)


@pytest.mark.parametrize("storage", (0, 1))
@pytest.mark.parametrize("precision,tol", ((1, 5e-2), (2, 5e-3)))
def test_16bit_storage_close_to_fp32(engine, storage, precision, tol):
    """BF16 / FP16 storage of the source wavefield with per-step, per-tile max-abs scales:
    the image stays close to the FP32-storage image (stencil and CPML stay FP32)."""
    d = load()
    p = _params(engine, d, "uneven", storage=storage)
    ref, _ = engine.migrate_shot(p, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"])
    img, _ = engine.migrate_shot(p.replace(precision=precision), d["uneven/ext"], d["uneven/wavelet"],
                                 d["uneven/seis"])
    err = rel_l2(img, ref)
    assert err <= tol, err
    assert err > 0.0          # the 16-bit path really ran


@pytest.mark.parametrize("compute,tol", ((1, 1e-9), (0, 2e-3)))
def test_reconstructed_source_field_matches_forward(engine, oracle, compute, tol):
    """The boundary-ring reconstruction rebuilds the forward wavefield in reverse time inside
    the reconstruction region (outside it, in the CPML, the field is not rebuilt): the source
    field captured during the adjoint pass at forward times 21 and 101 equals the forward
    field u_t (the oracle's snapshot of step t-1, same precision) over the model interior."""
    import torch
    d = load()
    p = _params(engine, d, "uneven", storage=1, compute=compute)
    dt = torch.float64 if compute else torch.float32
    npd = np.float64 if compute else np.float32
    ext, wav, seis = d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"]
    fwd = oracle.forward(p.as_dict(), ext, wav, snapshots=True, dtype=npd)
    times = [21, 101, p.nt - 1, p.nt]
    plan = engine.Plan(p)
    out = torch.zeros((len(times), p.dim_x, p.dim_z), dtype=dt, device="cuda")
    plan.capture_source(times, out)
    dv = torch.from_numpy(ext).cuda()
    plan.forward(dv, torch.from_numpy(wav).cuda())
    img = torch.zeros((p.nx, p.nz), dtype=dt, device="cuda")
    slf = torch.zeros_like(img)
    plan.adjoint(torch.from_numpy(seis).cuda(), img, slf)
    plan.sync()
    got = out.cpu().numpy()
    inner = (slice(p.th_left, p.th_left + p.nx), slice(p.th_up, p.th_up + p.nz))
    for k, t in enumerate(times[:2]):
        ref = fwd["snapshots"][(t - 1) // p.time_slices]
        err = rel_l2(got[k][inner], ref[inner])
        assert err <= tol, (t, err)
    # u_{nt-1} and u_nt: the forward pass's last two fields, before any reconstruction
    assert rel_l2(got[2], fwd["u_prev"]) <= (1e-12 if compute else 1e-5)
    assert rel_l2(got[3], fwd["u_last"]) <= (1e-12 if compute else 1e-5)


def test_autotune_picks_a_width_and_plans_stay_correct(engine):
    d = load()
    p = _params(engine, d, "uneven", storage=1)
    tx, ms = engine.autotune(p, steps=40)
    assert tx in (8, 16, 32) and ms > 0
    img, _ = engine.migrate_shot(p, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"])
    assert rel_l2(img, d["uneven/image"]) <= 1e-4
