"""The engine's ZFP 0.5.5 fixed-accuracy decoder (host) against the reference's own ZFP
build: the golden streams were written by zfp2d_lossyCompression and decoded by
zfp2d_lossyDecompression (tests/golden/make_golden.py); the decode must be bit-identical."""
import numpy as np
import pytest

from golden_util import load


@pytest.mark.parametrize("tag,tol", (("tol1e-4", 1e-4), ("tol0", 0.0)))
def test_decode_bit_identical_to_reference(engine, tag, tol):
    d = load()
    stream = d["zfp/%s/stream" % tag].tobytes()
    ref = d["zfp/%s/decoded" % tag]
    nrec, nt = ref.shape
    # the reference passes dimension1 = numberOfReceivers (zfp nx), dimension2 = nt (zfp ny)
    out = engine.zfp_decode(stream, nrec, nt, np.float32(tol))
    assert out.dtype == np.float32 and out.shape == ref.shape
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    if tol > 0:
        err = np.abs(out - d["zfp/input"]).max()
        assert 0 < err <= tol


def test_decode_routine_streams_match_tolerance(engine):
    """The driver fixture's seismogram streams decode to fields within the tolerance of each
    other's shot geometry: a sanity check that every stream decodes to its full length."""
    d = load()
    nrec, nt = int(d["uneven/params"][12]), int(d["uneven/params"][6])
    for k in (1, 2):
        out = engine.zfp_decode(d["routine/seis_%d" % k].tobytes(), nrec, nt, d["routine/tol"][0])
        assert np.isfinite(out).all() and np.abs(out).max() > 0


def test_truncated_stream_is_an_error(engine):
    d = load()
    stream = d["zfp/tol0/stream"].tobytes()
    nrec, nt = d["zfp/tol0/decoded"].shape
    with pytest.raises(engine.RtmError) as e:
        engine.zfp_decode(stream[: len(stream) // 2], nrec, nt, 0.0)
    assert e.value.status == 7          # RTM_ERR_DECODE


def test_file_decode_and_missing_file(engine, tmp_path):
    import ctypes as C
    d = load()
    path = tmp_path / "s.zfp"
    path.write_bytes(d["zfp/tol1e-4/stream"].tobytes())
    ref = d["zfp/tol1e-4/decoded"]
    out = np.empty(ref.size, np.float32)
    L = engine.lib()
    st = L.rtm_zfp_decode_file(str(path).encode(), out.ctypes.data_as(C.POINTER(C.c_float)),
                               ref.shape[0], ref.shape[1], C.c_float(1e-4))
    assert st == 0 and np.array_equal(out.reshape(ref.shape), ref)
    st = L.rtm_zfp_decode_file(str(tmp_path / "missing.zfp").encode(),
                               out.ctypes.data_as(C.POINTER(C.c_float)), ref.shape[0], ref.shape[1],
                               C.c_float(1e-4))
    assert st == 6                      # RTM_ERR_IO


def test_dropin_library_exports_reference_names(engine):
    import os
    import re
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "rtm_dropin.h")).read()
    body = hdr.split("#ifdef FIXED_PARAMETERS_H")[0]
    names = set(re.findall(r"^(?:void|int)\s+(\w+)\s*\(", body, re.M))
    assert {"rtm_routine", "isotropicAcousticModeling", "adjointModeling", "zfp2d_lossyDecompression",
            "iso_acoustic_wave_equation", "aiso_attenuation_cpml", "laplacian_filter2D"} <= names
    L = engine.dropin_lib()
    for n in sorted(names):
        assert hasattr(L, n), n


@pytest.mark.parametrize("tag,tol", (("tol1e-4", 1e-4), ("tol0", 0.0)))
def test_encode_byte_identical_to_reference(engine, tag, tol):
    d = load()
    stream = engine.zfp_encode(d["zfp/input"], np.float32(tol))
    assert stream == d["zfp/%s/stream" % tag].tobytes()


def test_partial_blocks_encode_and_decode(engine):
    """7 x 158 field: edge blocks partial in both directions (ZFP's padding rule)."""
    d = load()
    inp, ref_stream, ref_dec = d["zfp/partial/input"], d["zfp/partial/stream"], d["zfp/partial/decoded"]
    assert engine.zfp_encode(inp, np.float32(1e-4)) == ref_stream.tobytes()
    out = engine.zfp_decode(ref_stream.tobytes(), inp.shape[0], inp.shape[1], np.float32(1e-4))
    assert np.array_equal(out.view(np.uint32), ref_dec.view(np.uint32))


def test_encode_decode_round_trip_bound(engine):
    rng = np.random.default_rng(3)
    # magnitudes below 2, so float32 resolves every tolerance tried
    f = (rng.standard_normal((33, 45)) * np.exp(rng.uniform(-20, -1.5, (33, 45)))).astype(np.float32)
    f[3:9, 4:12] = 0.0
    for tol in (1e-2, 1e-4, 1e-6):
        out = engine.zfp_decode(engine.zfp_encode(f, tol), 33, 45, tol)
        assert np.abs(out - f).max() <= tol
    lossless = engine.zfp_decode(engine.zfp_encode(f, 0.0), 33, 45, 0.0)
    assert np.abs(lossless - f).max() <= 1e-6 * np.abs(f).max()


@pytest.mark.parametrize("tag,tol", (("tol1e-4", 1e-4), ("tol0", 0.0)))
def test_dropin_compression_matches_reference_stream(engine, tag, tol):
    """zfp2d_lossyCompression (compression_tools.h:5) through the drop-in library: a malloc'ed
    buffer holding the reference's stream byte for byte, its length returned."""
    import ctypes as C
    d = load()
    inp = np.ascontiguousarray(d["zfp/input"], np.float32)
    L = engine.dropin_lib()
    L.zfp2d_lossyCompression.restype = C.c_int
    L.zfp2d_lossyCompression.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_float), C.c_int, C.c_int,
                                         C.c_float]
    buf = C.c_void_p()
    n = L.zfp2d_lossyCompression(C.byref(buf), inp.ctypes.data_as(C.POINTER(C.c_float)), inp.shape[0],
                                 inp.shape[1], C.c_float(tol))
    ref = d["zfp/%s/stream" % tag].tobytes()
    assert n == len(ref) and buf.value
    assert C.string_at(buf.value, n) == ref
    C.CDLL(None).free(buf)


def _large_field():
    rng = np.random.default_rng(11)
    nrec, nt = 700, 1500                  # 375 block rows: the threaded encoder's chunks
    t = np.arange(nt) * 4e-4
    x = np.arange(nrec)[:, None] * 5.0
    f = np.zeros((nrec, nt), np.float32)
    for t0, v in ((0.2, 1500.0), (0.4, 2200.0)):
        tt = np.sqrt(t0 ** 2 + ((x - 1750.0) / v) ** 2)
        f += (np.exp(-((t[None, :] - tt) * 60.0) ** 2) * np.cos((t[None, :] - tt) * 125.0)).astype(np.float32)
    f += (rng.standard_normal(f.shape) * 1e-3).astype(np.float32)
    f[:, :50] = 0.0                       # empty blocks
    return f


def test_large_field_encode_round_trip(engine):
    """A field large enough for the threaded encoder (block rows in chunks on host threads,
    bit streams concatenated): it decodes within the tolerance."""
    f = _large_field()
    for tol in (1e-4, 1e-6):
        s = engine.zfp_encode(f, tol)
        out = engine.zfp_decode(s, f.shape[0], f.shape[1], tol)
        assert np.abs(out - f).max() <= tol


def test_large_field_encode_matches_reference_library(engine):
    """The threaded encoder writes the reference library's stream byte for byte (ZFP's OpenMP
    mode also concatenates per-chunk streams bit for bit).  Needs the reference's own build
    (oracle/_ref, made from the reference sources where they are present)."""
    import ctypes as C
    import os
    lib = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                       "libref_rtm.so")
    if not os.path.exists(lib):
        pytest.skip("reference build absent")
    ref = C.CDLL(lib)
    ref.zfp2d_lossyCompression.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_float), C.c_int, C.c_int,
                                           C.c_float]
    ref.zfp2d_lossyCompression.restype = C.c_int
    f = np.ascontiguousarray(_large_field())
    for tol in (1e-4, 0.0):
        ptr = C.c_void_p()
        n = ref.zfp2d_lossyCompression(C.byref(ptr), f.ctypes.data_as(C.POINTER(C.c_float)), f.shape[0],
                                       f.shape[1], C.c_float(tol))
        assert n > 0
        assert C.string_at(ptr.value, n) == bytes(engine.zfp_encode(f, tol)), tol


def test_random_and_truncated_streams_never_crash(engine):
    """Random bytes and every truncation of a real stream decode to a status (OK or an
    error), never past the buffer: the bit reader supplies zeros beyond the end and counts
    them, and the decoder reports a stream it over-read."""
    rng = np.random.default_rng(17)
    f = (rng.standard_normal((37, 41)) * 0.3).astype(np.float32)
    s = bytes(engine.zfp_encode(f, 1e-4))
    for cut in range(0, len(s), max(1, len(s) // 97)):
        try:
            engine.zfp_decode(s[:cut], 37, 41, 1e-4)
        except engine.RtmError:
            pass
    for n in (1, 7, 8, 9, 63, 64, 65, 500, 4096):
        junk = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        for tol in (1e-4, 0.0):
            try:
                out = engine.zfp_decode(junk, 37, 41, tol)
                assert out.shape == (37, 41)
            except engine.RtmError:
                pass


def test_codec_in_bounds_under_address_sanitizer(tmp_path):
    """tests/zfp_fuzz.c against csrc/rtm_zfp.c built with AddressSanitizer and UBSan: every
    truncation of a stream, random streams and the threaded encoder stay in bounds."""
    import os
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "zfp_fuzz")
    env = dict(os.environ, TMPDIR=str(tmp_path))
    build = subprocess.run([gcc, "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                            "-fno-omit-frame-pointer", "-std=gnu99", "-I", os.path.join(root, "include"),
                            os.path.join(root, "tests", "zfp_fuzz.c"),
                            os.path.join(root, "rtmuq2d_gb300", "csrc", "rtm_zfp.c"), "-o", exe, "-lm",
                            "-lpthread"], capture_output=True, text=True, env=env)
    if build.returncode != 0:
        pytest.skip("sanitizer build unavailable: " + build.stderr[-200:])
    run = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]


def test_large_field_streams_match_reference_digests(engine):
    """The codec on a field large enough for the threaded encoder (3400 x 750), against the
    digests of the reference library's streams and decodes (tests/golden/zfp_large.json, made
    by tests/golden/make_zfp_large.py with the reference's own ZFP build): byte-identical
    streams and bit-identical decodes at tolerances 1e-4, 1e-6 and 0 -- on any machine, the
    field being rebuilt from integer arithmetic."""
    import hashlib
    import json
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    from make_zfp_large import portable_field
    want = json.load(open(os.path.join(here, "zfp_large.json")))
    f = np.ascontiguousarray(portable_field())
    assert hashlib.sha256(f.tobytes()).hexdigest() == want["field_sha256"]
    for tol_s, d in want["streams"].items():
        tol = float(tol_s)
        s = bytes(engine.zfp_encode(f, tol))
        assert len(s) == d["bytes"] and hashlib.sha256(s).hexdigest() == d["stream_sha256"], tol
        out = np.ascontiguousarray(engine.zfp_decode(s, f.shape[0], f.shape[1], tol), np.float32)
        assert hashlib.sha256(out.tobytes()).hexdigest() == d["decoded_sha256"], tol
