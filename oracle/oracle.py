"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

Two CPU implementations of rtmUq2D's migration path are reachable from here:

* ``Oracle``    -- oracle/rtm_oracle.c, the restatement built by oracle/build_oracle.sh.
  It travels with the repository and builds on any host with gcc.
* ``Reference`` -- the reference's own C sources compiled in place by
  oracle/build_ref.sh into oracle/_ref/ (only where the reference tree is present).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module.  The product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
# the reference tree: RTM_REFERENCE_ROOT, else a "reference" directory beside the repository
REFERENCE_ROOT = os.environ.get("RTM_REFERENCE_ROOT",
                                os.path.normpath(os.path.join(HERE, "..", "..", "reference")))

FIELDS_INT = ("nx", "nz", "th_left", "th_right", "th_up", "th_down")
FIELDS_ALL = FIELDS_INT + ("dx", "dt", "nt", "n_wavelet", "shot_x", "shot_z", "rec_first",
                           "rec_spacing", "rec_count", "rec_depth", "time_slices")


class OrcParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("th_left", C.c_int), ("th_right", C.c_int),
                ("th_up", C.c_int), ("th_down", C.c_int), ("dx", C.c_float), ("dt", C.c_float),
                ("nt", C.c_int), ("n_wavelet", C.c_int), ("shot_x", C.c_int), ("shot_z", C.c_int),
                ("rec_first", C.c_int), ("rec_spacing", C.c_int), ("rec_count", C.c_int),
                ("rec_depth", C.c_int), ("time_slices", C.c_int)]


def to_orc(p) -> OrcParams:
    """Build the C struct from any object (or dict) carrying the same field names."""
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    o = OrcParams()
    for name in FIELDS_ALL:
        setattr(o, name, get(name))
    return o


def dims(p):
    o = to_orc(p)
    return o.th_left + o.nx + o.th_right, o.th_up + o.nz + o.th_down


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def build_oracle() -> None:
    subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True,
                   stdout=subprocess.DEVNULL)


def build_reference(root: str = REFERENCE_ROOT) -> bool:
    """Compile the reference sources into oracle/_ref (False if the tree is absent)."""
    if not os.path.isdir(os.path.join(root, "SRC")):
        return False
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), root], check=True,
                   stdout=subprocess.DEVNULL)
    return True


class Oracle:
    """The restatement (oracle/rtm_oracle.c)."""

    def __init__(self, fast: bool = False):
        name = "liboracle_fast.so" if fast else "liboracle.so"
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build_oracle()
        self.lib = C.CDLL(path)
        self.lib.orc_max_threads.restype = C.c_int

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(C.c_int(n))

    def max_threads(self) -> int:
        return int(self.lib.orc_max_threads())

    # -- setup ----------------------------------------------------------------------
    def extend_matrix(self, p, model: np.ndarray) -> np.ndarray:
        dx_, dz_ = dims(p)
        ext = np.zeros((dx_, dz_), np.float32)
        m = _f32(model)
        self.lib.orc_extend_matrix(C.byref(to_orc(p)), _ptr(ext), _ptr(m))
        return ext

    def cpml_profile(self, p) -> dict:
        o = to_orc(p)
        arrs = {k: np.zeros(n, np.float32) for k, n in
                (("a_l", o.th_left), ("a_r", o.th_right), ("a_t", o.th_up), ("a_b", o.th_down),
                 ("b_l", o.th_left), ("b_r", o.th_right), ("b_t", o.th_up), ("b_b", o.th_down))}
        self.lib.orc_cpml_profile(C.byref(o), *[_ptr(arrs[k]) for k in
                                  ("a_l", "a_r", "a_t", "a_b", "b_l", "b_r", "b_t", "b_b")])
        return arrs

    def laplacian(self, p, img: np.ndarray) -> np.ndarray:
        o = to_orc(p)
        src = _f32(img).reshape(o.nx, o.nz)
        out = np.zeros_like(src)
        self.lib.orc_laplacian(C.byref(o), _ptr(out), _ptr(src))
        return out

    # -- per step ---------------------------------------------------------------------
    def coef(self, p, vel_ext, dtype=np.float32):
        dx_, dz_ = dims(p)
        out = np.zeros((dx_, dz_), dtype)
        fn = self.lib.orc_coef_f if dtype == np.float32 else self.lib.orc_coef_d
        fn(C.byref(to_orc(p)), _ptr(out), _ptr(_f32(vel_ext)))
        return out

    def stencil(self, p, coef, u_cur, u_prev):
        dtype = coef.dtype
        w = np.array(u_prev, dtype=dtype, copy=True)
        fn = self.lib.orc_stencil_f if dtype == np.float32 else self.lib.orc_stencil_d
        fn(C.byref(to_orc(p)), _ptr(np.ascontiguousarray(coef)),
           _ptr(np.ascontiguousarray(u_cur, dtype=dtype)), _ptr(w))
        return w

    def cpml(self, p, u_cur, u_next, coef, prof: dict, psi: dict, xi: dict):
        """One CPML update; psi/xi dicts (keys l,r,t,b) are updated in place; returns u_next."""
        dtype = coef.dtype
        w = np.array(u_next, dtype=dtype, copy=True)
        fn = self.lib.orc_cpml_f if dtype == np.float32 else self.lib.orc_cpml_d
        fn(C.byref(to_orc(p)), _ptr(np.ascontiguousarray(u_cur, dtype=dtype)), _ptr(w),
           _ptr(coef), _ptr(prof["a_l"]), _ptr(prof["b_l"]), _ptr(prof["a_r"]), _ptr(prof["b_r"]),
           _ptr(prof["a_t"]), _ptr(prof["b_t"]), _ptr(prof["a_b"]), _ptr(prof["b_b"]),
           _ptr(psi["l"]), _ptr(psi["r"]), _ptr(psi["t"]), _ptr(psi["b"]),
           _ptr(xi["l"]), _ptr(xi["r"]), _ptr(xi["t"]), _ptr(xi["b"]))
        return w

    def xcorr(self, p, img, self_img, src, rcv):
        """normalized_cross_correlation in place on float32 img/self_img (nx x nz)."""
        self.lib.orc_xcorr_f(C.byref(to_orc(p)), _ptr(img), _ptr(self_img), _ptr(_f32(src)),
                             _ptr(_f32(rcv)))

    def new_strips(self, p, dtype=np.float32):
        o = to_orc(p)
        dx_, dz_ = dims(p)
        mk = lambda: {"l": np.zeros((o.th_left, dz_), dtype), "r": np.zeros((o.th_right, dz_), dtype),
                      "t": np.zeros((dx_, o.th_up), dtype), "b": np.zeros((dx_, o.th_down), dtype)}
        return mk(), mk()

    # -- drivers ----------------------------------------------------------------------
    def forward(self, p, vel_ext, wavelet, snapshots=True, record=False, dtype=np.float32):
        o = to_orc(p)
        dx_, dz_ = dims(p)
        nslots = (o.nt + o.time_slices - 1) // o.time_slices
        snaps = np.zeros((nslots, dx_, dz_), dtype) if snapshots else None
        seis = np.zeros((o.rec_count, o.nt), dtype) if record else None
        u_last = np.zeros((dx_, dz_), dtype)
        u_prev = np.zeros((dx_, dz_), dtype)
        fn = self.lib.orc_forward_f if dtype == np.float32 else self.lib.orc_forward_d
        fn(C.byref(o), _ptr(_f32(vel_ext)), _ptr(_f32(wavelet)),
           _ptr(snaps) if snaps is not None else None,
           _ptr(seis) if seis is not None else None, _ptr(u_last), _ptr(u_prev))
        return {"snapshots": snaps, "seis": seis, "u_last": u_last, "u_prev": u_prev}

    def adjoint(self, p, vel_ext, seis, snapshots, dtype=np.float32):
        o = to_orc(p)
        img = np.zeros((o.nx, o.nz), dtype)
        slf = np.zeros((o.nx, o.nz), dtype)
        fn = self.lib.orc_adjoint_f if dtype == np.float32 else self.lib.orc_adjoint_d
        fn(C.byref(o), _ptr(_f32(vel_ext)),
           _ptr(np.ascontiguousarray(seis, dtype=dtype)),
           _ptr(np.ascontiguousarray(snapshots, dtype=dtype)), _ptr(img), _ptr(slf))
        return img, slf

    def migrate(self, p, vel_ext, wavelet, seis, dtype=np.float32):
        fwd = self.forward(p, vel_ext, wavelet, snapshots=True, dtype=dtype)
        return self.adjoint(p, vel_ext, seis, fwd["snapshots"], dtype=dtype)

    def model_seismogram(self, p, vel_ext, wavelet, dtype=np.float32):
        return self.forward(p, vel_ext, wavelet, snapshots=False, record=True, dtype=dtype)["seis"]


class Reference:
    """The reference's own C code, compiled from its sources into oracle/_ref/."""

    def __init__(self):
        path = os.path.join(REF_DIR, "libref_rtm.so")
        if not os.path.exists(path):
            if not build_reference():
                raise FileNotFoundError("reference sources not present; cannot build oracle/_ref")
        self.lib = C.CDLL(path)
        self.lib.adjointModeling.restype = C.c_int
        self.lib.zfp2d_lossyCompression.restype = C.c_int
        self.lib.zfp2d_lossyDecompression.restype = C.c_int

    @staticmethod
    def available() -> bool:
        return (os.path.exists(os.path.join(REF_DIR, "libref_rtm.so"))
                or os.path.isdir(os.path.join(REFERENCE_ROOT, "SRC")))

    def configure(self, p, n_shots=1, spacing_shot=0, zfp_tolerance=0.0, n_sims=1):
        o = to_orc(p)
        if o.time_slices != 20:
            raise ValueError("the reference's TIME_SLICES is the compile-time constant 20")
        iv = (C.c_int * 17)(o.nx, o.nz, o.th_left, o.th_right, o.th_up, o.th_down, o.nt,
                            o.n_wavelet, o.shot_x, o.shot_z, spacing_shot, n_shots,
                            o.rec_first, o.rec_spacing, o.rec_count, o.rec_depth, n_sims)
        fv = (C.c_float * 3)(o.dx, o.dt, zfp_tolerance)
        self.lib.ref_set_params(iv, fv)

    def set_paths(self, vel=None, wav=None, seis=None, stacked=None, laplacian=None):
        enc = lambda s: s.encode() if s is not None else None
        self.lib.ref_set_paths(enc(vel), enc(wav), enc(seis), enc(stacked), enc(laplacian))

    # -- kernels through the reference's own entry points --------------------------------
    def extend_matrix(self, p, model):
        self.configure(p)
        dx_, dz_ = dims(p)
        ext = np.zeros((dx_, dz_), np.float32)
        self.lib.extend_matrix(_ptr(ext), _ptr(_f32(model)))
        return ext

    def cpml_profile(self, p):
        self.configure(p)
        o = to_orc(p)
        a = {k: np.zeros(n, np.float32) for k, n in
             (("a_l", o.th_left), ("a_r", o.th_right), ("a_t", o.th_up), ("a_b", o.th_down),
              ("b_l", o.th_left), ("b_r", o.th_right), ("b_t", o.th_up), ("b_b", o.th_down))}
        self.lib.attenuation_profile_cpml(*[_ptr(a[k]) for k in
                                          ("a_l", "a_r", "a_t", "a_b", "b_l", "b_r", "b_t", "b_b")])
        return a

    def stencil(self, p, coef, u_cur, u_prev):
        self.configure(p)
        w = np.array(u_prev, np.float32, copy=True)
        self.lib.iso_acoustic_wave_equation(_ptr(_f32(coef)), _ptr(_f32(u_cur)), _ptr(w))
        return w

    def cpml(self, p, u_cur, u_next, coef, prof, psi, xi):
        self.configure(p)
        w = np.array(u_next, np.float32, copy=True)
        self.lib.aiso_attenuation_cpml(
            _ptr(_f32(u_cur)), _ptr(w), _ptr(_f32(coef)),
            _ptr(prof["a_l"]), _ptr(prof["b_l"]), _ptr(prof["a_r"]), _ptr(prof["b_r"]),
            _ptr(prof["a_t"]), _ptr(prof["b_t"]), _ptr(prof["a_b"]), _ptr(prof["b_b"]),
            _ptr(psi["l"]), _ptr(psi["r"]), _ptr(psi["t"]), _ptr(psi["b"]),
            _ptr(xi["l"]), _ptr(xi["r"]), _ptr(xi["t"]), _ptr(xi["b"]))
        return w

    def laplacian(self, p, img):
        self.configure(p)
        o = to_orc(p)
        out = np.zeros((o.nx, o.nz), np.float32)
        self.lib.laplacian_filter2D(_ptr(out), _ptr(_f32(img).reshape(o.nx, o.nz)))
        return out

    # -- drivers (run in a scratch working directory: the reference uses ./TEMPORARY_FILES)
    def forward(self, p, vel_ext, wavelet, sim_id=1):
        """isotropicAcousticModeling; returns the snapshot file's content (slots, dimX, dimZ)."""
        self.configure(p)
        o = to_orc(p)
        dx_, dz_ = dims(p)
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.makedirs(os.path.join(tmp, "TEMPORARY_FILES"))
            os.chdir(tmp)
            try:
                shot = (C.c_int * 2)(o.shot_x, o.shot_z)
                self.lib.isotropicAcousticModeling(C.c_int(sim_id), shot, _ptr(_f32(vel_ext)),
                                                   _ptr(_f32(wavelet)))
                raw = np.fromfile(os.path.join(tmp, "TEMPORARY_FILES",
                                               "sourceWavefield_%05d.bin" % sim_id), np.float32)
            finally:
                os.chdir(cwd)
        return raw.reshape(-1, dx_, dz_)

    def migrate(self, p, vel_ext, wavelet, seis, sim_id=1):
        """isotropicAcousticModeling + adjointModeling, as rtm_iso2d.c:85-93 calls them."""
        self.configure(p)
        o = to_orc(p)
        img = np.zeros((o.nx, o.nz), np.float32)
        slf = np.zeros((o.nx, o.nz), np.float32)
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as tmp:
            os.makedirs(os.path.join(tmp, "TEMPORARY_FILES"))
            os.chdir(tmp)
            try:
                shot = (C.c_int * 2)(o.shot_x, o.shot_z)
                v = _f32(vel_ext)
                w = _f32(wavelet)
                self.lib.isotropicAcousticModeling(C.c_int(sim_id), shot, _ptr(v), _ptr(w))
                self.lib.adjointModeling(C.c_int(sim_id), shot, _ptr(v), _ptr(w),
                                         _ptr(_f32(seis)), _ptr(img), _ptr(slf))
            finally:
                os.chdir(cwd)
        return img, slf

    # -- ZFP through the reference's own wrappers (compression_tools.c) -----------------
    def zfp_compress(self, arr: np.ndarray, d1: int, d2: int, tol: float) -> bytes:
        a = _f32(arr)
        buf = C.c_void_p()
        n = self.lib.zfp2d_lossyCompression(C.byref(buf), _ptr(a), C.c_int(d1), C.c_int(d2),
                                            C.c_float(tol))
        data = C.string_at(buf, n)
        C.CDLL(None).free(buf)
        return data

    def zfp_decompress(self, path: str, d1: int, d2: int, tol: float) -> np.ndarray:
        out = np.zeros(d1 * d2, np.float32)
        st = self.lib.zfp2d_lossyDecompression(path.encode(), _ptr(out), C.c_int(d1), C.c_int(d2),
                                               C.c_float(tol))
        if st != 0:
            raise RuntimeError("zfp decode failed")
        return out

    def rtm_routine(self, workdir: str, sim_id: int) -> None:
        """Run rtm_routine(sim_id) with ./INPUTS, ./OUTPUTS, ./TEMPORARY_FILES under workdir."""
        cwd = os.getcwd()
        os.chdir(workdir)
        try:
            self.lib.rtm_routine(C.c_int(sim_id))
        finally:
            os.chdir(cwd)
