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


_FIXED = r'''
#ifndef FIXED_PARAMETERS_H
#define FIXED_PARAMETERS_H
static char velocityFile[] = "./INPUTS/vp_%05d.bin";
static char waveletFile[] = "./INPUTS/wavelet.bin";
static char seismogramFile[] = "./INPUTS/seismogram_%05d.zfp";
static char stackedFile[] = "./OUTPUTS/stackedBrute_%05d.bin";
static char stackedLaplacianFile[] = "./OUTPUTS/stackedLaplacian_%05d.bin";
static const float zfp_tolerance = 0.0001;
static const float spacingGrid = 10.0;
static const float sampling = 0.001;
static const int numberOfSimulations = 1;
static const int Nx = 37;
static const int Nz = 29;
static const int firstLocationShot = 18;
static const int depthShot = 2;
static const int spacingShot = 4;
static const int numberOfShots = 2;
static const int firstLocationReceiver = 0;
static const int depthReceiver = 2;
static const int spacingReceiver = 2;
static const int numberOfReceivers = 37;
static const int numberOfTimeStep = 200;
static const int sampligWavelet = 60;
static const float cutFrequency = 50.0;
static const int thicknessUp = 14;
static const int thicknessDown = 16;
static const int thicknessLeft = 18;
static const int thicknessRight = 20;
#endif
'''

_MAIN = r'''
#include <stdio.h>
#include <stdlib.h>
#include "fixed_parameters.h"
#define TIME_SLICES 20
#include "rtm_dropin.h"
int main(void)
{
    if (rtm_dropin_configure_from_fixed_parameters() != 0) return 2;
    float *model = (float *)malloc(sizeof(float) * Nx * Nz);
    float *ext = (float *)malloc(sizeof(float) * (Nx + thicknessLeft + thicknessRight) *
                                 (Nz + thicknessUp + thicknessDown));
    if (!model || !ext) return 3;
    for (int i = 0; i < Nx * Nz; ++i) model[i] = (float)i;
    extend_matrix(ext, model);        /* sizes from the configuration, no device work */
    const int dz = Nz + thicknessUp + thicknessDown;
    printf("%g %g %g\n", ext[0], ext[thicknessLeft * dz + thicknessUp],
           ext[(thicknessLeft + Nx - 1) * dz + thicknessUp + Nz - 1]);
    return 0;
}
'''


def test_dropin_header_configures_from_fixed_parameters(engine, tmp_path):
    """A program written against the reference's fixed_parameters.h includes rtm_dropin.h,
    fills the library's configuration from those constants and calls a host entry point
    (extend_matrix) with them: it compiles, links and runs without a GPU."""
    import shutil
    import subprocess
    from rtmuq2d_gb300 import build as B
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    engine.dropin_lib()
    (tmp_path / "fixed_parameters.h").write_text(_FIXED)
    (tmp_path / "main.c").write_text(_MAIN)
    libdir = os.path.dirname(B.DROPIN_LIB)
    exe = tmp_path / "main"
    subprocess.run([gcc, "-std=gnu99", "-I", str(tmp_path), "-I", os.path.join(ROOT, "include"),
                    str(tmp_path / "main.c"), "-o", str(exe), "-L", libdir, "-lrtm_dropin", "-lrtmgpu",
                    "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    # corner of the padding = model[0][0]; interior origin = model[0][0]; last interior cell
    assert [float(v) for v in out] == [0.0, 0.0, float(37 * 29 - 1)]


def test_host_geometry_in_bounds_under_address_sanitizer(tmp_path):
    """tests/host_fuzz.c against csrc/rtm_host.c built with AddressSanitizer and UBSan:
    model padding and CPML profiles for 1 x 1 to 400 x 200 models and thicknesses 12-64."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "host_fuzz")
    env = dict(os.environ, TMPDIR=str(tmp_path))
    build = subprocess.run([gcc, "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                            "-fno-omit-frame-pointer", "-std=gnu99", "-I", os.path.join(ROOT, "include"),
                            os.path.join(ROOT, "tests", "host_fuzz.c"),
                            os.path.join(ROOT, "rtmuq2d_gb300", "csrc", "rtm_host.c"), "-o", exe, "-lm"],
                           capture_output=True, text=True, env=env)
    if build.returncode != 0:
        pytest.skip("sanitizer build unavailable: " + build.stderr[-200:])
    run = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=300)
    assert run.returncode == 0, run.stderr[-2000:]
