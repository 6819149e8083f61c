"""The oracle (oracle/rtm_oracle.c) pinned to the reference: against the golden fixtures
made by the reference's own code, and -- where the reference tree is present -- against a
live build of it.  CPU only."""
import numpy as np
import pytest

from golden_util import case_params, load, rel_l2

CASES = ("uneven", "quirks")


def _same(a, b, rtol=1e-6):
    """Bit-identical on the machine that made the fixtures; elsewhere libm's powf may differ
    by an ulp in the damping profile, so allow a tight relative bound."""
    if np.array_equal(a, b):
        return True
    return rel_l2(a, b) <= rtol


@pytest.mark.parametrize("name", CASES)
def test_extend_and_profile_match_reference(oracle, name):
    d = load()
    p = case_params(d, name)
    assert np.array_equal(oracle.extend_matrix(p, d[name + "/model"]), d[name + "/ext"])
    prof = oracle.cpml_profile(p)
    for k, v in prof.items():
        assert np.allclose(v, d[name + "/prof_" + k], rtol=2e-7, atol=0), k


@pytest.mark.parametrize("name", CASES)
def test_forward_snapshots_match_reference(oracle, name):
    d = load()
    p = case_params(d, name)
    snaps = oracle.forward(p, d[name + "/ext"], d[name + "/wavelet"])["snapshots"]
    ref = d[name + "/snapshots"]
    assert snaps.shape == ref.shape
    assert _same(snaps, ref)


@pytest.mark.parametrize("name", CASES)
def test_migration_image_matches_reference(oracle, name):
    d = load()
    p = case_params(d, name)
    img, slf = oracle.migrate(p, d[name + "/ext"], d[name + "/wavelet"], d[name + "/seis"])
    assert _same(img, d[name + "/image"])
    assert _same(slf, d[name + "/self"])
    assert np.abs(img).max() > 0


def test_step_kats_match_reference(oracle):
    d = load()
    p = case_params(d, "uneven")
    w = oracle.stencil(p, d["kat/coef"], d["kat/u1"], d["kat/u2"])
    assert np.array_equal(w, d["kat/stencil"])
    psi = {k: d["kat/psi_in_" + k].copy() for k in "lrtb"}
    xi = {k: d["kat/xi_in_" + k].copy() for k in "lrtb"}
    prof = oracle.cpml_profile(p)
    out = oracle.cpml(p, d["kat/u1"], d["kat/u2"], d["kat/coef"], prof, psi, xi)
    assert _same(out, d["kat/cpml"])
    for k in "lrtb":
        assert _same(psi[k], d["kat/psi_out_" + k]), k
        assert _same(xi[k], d["kat/xi_out_" + k]), k
    assert np.array_equal(oracle.laplacian(p, d["kat/lap_in"]), d["kat/lap_out"])


def test_fp64_oracle_close_to_fp32(oracle):
    d = load()
    p = case_params(d, "uneven")
    i32, _ = oracle.migrate(p, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"])
    i64, _ = oracle.migrate(p, d["uneven/ext"], d["uneven/wavelet"], d["uneven/seis"], dtype=np.float64)
    assert rel_l2(i32, i64) < 1e-4


def test_oracle_against_live_reference(oracle):
    from oracle.oracle import Reference
    if not Reference.available():
        pytest.skip("reference tree not present on this machine")
    ref = Reference()
    d = load()
    p = dict(case_params(d, "uneven"))
    p.update(nx=70, nz=50, th_left=13, th_right=15, th_up=16, th_down=12, nt=120, rec_count=35,
             rec_spacing=3, shot_x=40, shot_z=5)
    rng = np.random.default_rng(7)
    model = (1800 + 200 * rng.random((70, 50))).astype(np.float32)
    ext = ref.extend_matrix(p, model)
    assert np.array_equal(ext, oracle.extend_matrix(p, model))
    wav = d["uneven/wavelet"][:80]
    p["n_wavelet"] = 80
    snaps = oracle.forward(p, ext, wav)["snapshots"]
    assert np.array_equal(snaps, ref.forward(p, ext, wav))
    seis = oracle.model_seismogram(p, ext * np.float32(0.97), wav)
    a = oracle.migrate(p, ext, wav, seis)
    b = ref.migrate(p, ext, wav, seis)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
