"""Generate the golden fixtures in tests/golden/ by running the REFERENCE's own C code.

The reference (rtmUq2D) ships no test vectors for its migration path, so these fixtures
are outputs of its own routines -- compiled from its sources by oracle/build_ref.sh --
on small seeded inputs:

  extend_matrix, attenuation_profile_cpml, iso_acoustic_wave_equation,
  aiso_attenuation_cpml, laplacian_filter2D, isotropicAcousticModeling (its snapshot
  file), isotropicAcousticModeling + adjointModeling (image, self image), the ZFP
  round trip through zfp2d_lossyCompression / zfp2d_lossyDecompression, and the whole
  driver rtm_routine on files (two shots, ZFP seismograms, stacked image and Laplacian).

Needs the reference tree (RTM_REFERENCE_ROOT, else a "reference" directory beside the
repository).  Run:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, Reference, dims  # noqa: E402

OUT = os.path.join(HERE, "rtm_golden.npz")

CASES = {
    # uneven CPML (th_up != th_down exercises the extend_matrix bound at :27)
    "uneven": dict(nx=60, nz=40, th_left=16, th_right=18, th_up=14, th_down=20, dx=10.0, dt=1e-3,
                   nt=200, n_wavelet=80, shot_x=30, shot_z=2, rec_first=0, rec_spacing=2,
                   rec_count=60, rec_depth=2, time_slices=20),
    # th_up > th_down; every receiver on one column (spacingReceiver = 1), last one wins
    "quirks": dict(nx=48, nz=36, th_left=12, th_right=13, th_up=17, th_down=12, dx=8.0, dt=8e-4,
                   nt=160, n_wavelet=60, shot_x=20, shot_z=3, rec_first=5, rec_spacing=1,
                   rec_count=7, rec_depth=4, time_slices=20),
}


def ricker(f0, dt, n):
    t = np.arange(n) * dt - 1.2 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def main():
    ref = Reference()
    orc = Oracle()
    out = {}
    for name, p in CASES.items():
        rng = np.random.default_rng(abs(hash(name)) % 2**31 if False else len(name) * 7919)
        model = (2000.0 + 150.0 * rng.standard_normal((p["nx"], p["nz"]))).astype(np.float32)
        model[:, : p["nz"] // 3] = 1600.0
        wav = ricker(18.0, p["dt"], p["n_wavelet"])
        ext = ref.extend_matrix(p, model)
        # observed data: the oracle's recording on a perturbed model (only an input here)
        seis = orc.model_seismogram(p, ext * np.float32(1.04), wav)
        snaps = ref.forward(p, ext, wav)
        img, slf = ref.migrate(p, ext, wav, seis)
        prof = ref.cpml_profile(p)
        out[name + "/model"] = model
        out[name + "/wavelet"] = wav
        out[name + "/ext"] = ext
        out[name + "/seis"] = seis
        out[name + "/snapshots"] = snaps
        out[name + "/image"] = img
        out[name + "/self"] = slf
        for k, v in prof.items():
            out[name + "/prof_" + k] = v
        out[name + "/params"] = np.array([p[k] for k in ("nx", "nz", "th_left", "th_right", "th_up",
                                          "th_down", "nt", "n_wavelet", "shot_x", "shot_z",
                                          "rec_first", "rec_spacing", "rec_count", "rec_depth",
                                          "time_slices")], np.int32)
        out[name + "/fparams"] = np.array([p["dx"], p["dt"]], np.float32)

    # one-step known answers on random fields (uneven geometry)
    p = CASES["uneven"]
    dxx, dzz = dims(p)
    rng = np.random.default_rng(12345)
    u1 = rng.standard_normal((dxx, dzz)).astype(np.float32)
    u2 = rng.standard_normal((dxx, dzz)).astype(np.float32)
    coef = rng.uniform(0.01, 0.07, (dxx, dzz)).astype(np.float32)
    psi, xi = orc.new_strips(p)
    for d in (psi, xi):
        for k in d:
            d[k][...] = rng.standard_normal(d[k].shape).astype(np.float32) * 0.1
    prof = ref.cpml_profile(p)
    step = ref.stencil(p, coef, u1, u2)
    psi_r = {k: v.copy() for k, v in psi.items()}
    xi_r = {k: v.copy() for k, v in xi.items()}
    cp = ref.cpml(p, u1, u2, coef, prof, psi_r, xi_r)
    out["kat/u1"], out["kat/u2"], out["kat/coef"] = u1, u2, coef
    out["kat/stencil"] = step
    out["kat/cpml"] = cp
    for k in psi:
        out["kat/psi_in_" + k] = psi[k]
        out["kat/xi_in_" + k] = xi[k]
        out["kat/psi_out_" + k] = psi_r[k]
        out["kat/xi_out_" + k] = xi_r[k]
    img = rng.standard_normal((p["nx"], p["nz"])).astype(np.float32)
    out["kat/lap_in"] = img
    out["kat/lap_out"] = ref.laplacian(p, img)

    # ZFP round trip through the reference's wrappers (field nx=nrec, ny=nt over [irec][t])
    seis = out["uneven/seis"]
    for tol, tag in ((1e-4, "tol1e-4"), (0.0, "tol0")):
        blob = ref.zfp_compress(seis, seis.shape[0], seis.shape[1], tol)
        with tempfile.NamedTemporaryFile(suffix=".zfp", delete=False) as f:
            f.write(blob)
            path = f.name
        try:
            dec = ref.zfp_decompress(path, seis.shape[0], seis.shape[1], tol)
        finally:
            os.unlink(path)
        out["zfp/" + tag + "/stream"] = np.frombuffer(blob, np.uint8)
        out["zfp/" + tag + "/decoded"] = dec.reshape(seis.shape)
    out["zfp/input"] = seis
    # partial edge blocks in both directions (7 receivers x 158 samples)
    part = np.ascontiguousarray(out["quirks/seis"][:, :158])
    blob = ref.zfp_compress(part, part.shape[0], part.shape[1], 1e-4)
    with tempfile.NamedTemporaryFile(suffix=".zfp", delete=False) as f:
        f.write(blob)
        path = f.name
    try:
        dec = ref.zfp_decompress(path, part.shape[0], part.shape[1], 1e-4)
    finally:
        os.unlink(path)
    out["zfp/partial/input"] = part
    out["zfp/partial/stream"] = np.frombuffer(blob, np.uint8)
    out["zfp/partial/decoded"] = dec.reshape(part.shape)

    # the whole driver: rtm_routine(sim_id) on files (2 shots, ZFP tol 1e-4 seismograms)
    p = dict(CASES["uneven"])
    sim_id, n_shots, first, spacing, tol = 3, 2, 22, 16, 1e-4
    model = out["uneven/model"]
    wav = out["uneven/wavelet"]
    ext_true = ref.extend_matrix(p, model * np.float32(1.04))
    with tempfile.TemporaryDirectory() as tmp:
        for d in ("INPUTS", "OUTPUTS", "TEMPORARY_FILES"):
            os.makedirs(os.path.join(tmp, d))
        model.astype(np.float32).tofile(os.path.join(tmp, "INPUTS", "vp_%05d.bin" % sim_id))
        wav.astype(np.float32).tofile(os.path.join(tmp, "INPUTS", "wavelet.bin"))
        for shot_id in range(1, n_shots + 1):
            q = dict(p, shot_x=first + (shot_id - 1) * spacing)
            seis = orc.model_seismogram(q, ext_true, wav)
            blob = ref.zfp_compress(seis, seis.shape[0], seis.shape[1], tol)
            with open(os.path.join(tmp, "INPUTS", "seismogram_%05d.zfp" % shot_id), "wb") as f:
                f.write(blob)
            out["routine/seis_%d" % shot_id] = np.frombuffer(blob, np.uint8)
        ref.configure(dict(p, shot_x=first), n_shots=n_shots, spacing_shot=spacing, zfp_tolerance=tol)
        ref.set_paths("./INPUTS/vp_%05d.bin", "./INPUTS/wavelet.bin", "./INPUTS/seismogram_%05d.zfp",
                      "./OUTPUTS/stackedBrute_%05d.bin", "./OUTPUTS/stackedLaplacian_%05d.bin")
        ref.rtm_routine(tmp, sim_id)
        out["routine/stacked"] = np.fromfile(os.path.join(tmp, "OUTPUTS", "stackedBrute_%05d.bin" % sim_id),
                                             np.float32).reshape(p["nx"], p["nz"])
        out["routine/laplacian"] = np.fromfile(
            os.path.join(tmp, "OUTPUTS", "stackedLaplacian_%05d.bin" % sim_id), np.float32).reshape(p["nx"], p["nz"])
    out["routine/survey"] = np.array([sim_id, n_shots, first, spacing, p["shot_z"]], np.int32)
    out["routine/tol"] = np.array([tol], np.float32)

    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
