"""ctypes binding of librtmgpu (include/rtm_gpu.h).

Host-array entry points take numpy arrays in the reference's layouts; the plan API takes
device pointers (ints, or anything with ``data_ptr()`` such as torch tensors).  Every
call raises ``RtmError`` on a non-zero status.  There is no CPU fallback: if the library
cannot be loaded, importing the engine fails.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

RTM_OK = 0
RTM_ERR_INVALID = 1
RTM_ERR_CUDA = 2
RTM_ERR_NOMEM = 3
RTM_ERR_STATE = 4
RTM_ERR_TIMEOUT = 5
RTM_ERR_IO = 6
RTM_ERR_DECODE = 7
RTM_ERR_BUSY = 8

STORE_SNAPSHOT = 0
STORE_RING = 1
PREC_FP32 = 0
PREC_BF16 = 1
PREC_FP16 = 2
COMPUTE_FP32 = 0
COMPUTE_FP64 = 1


class RtmParams(C.Structure):
    """Run-time form of the reference's SRC/fixed_parameters.h (see include/rtm_gpu.h)."""
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("th_left", C.c_int), ("th_right", C.c_int),
                ("th_up", C.c_int), ("th_down", C.c_int), ("dx", C.c_float), ("dt", C.c_float),
                ("nt", C.c_int), ("n_wavelet", C.c_int), ("shot_x", C.c_int), ("shot_z", C.c_int),
                ("rec_first", C.c_int), ("rec_spacing", C.c_int), ("rec_count", C.c_int),
                ("rec_depth", C.c_int), ("time_slices", C.c_int), ("storage", C.c_int),
                ("precision", C.c_int), ("compute", C.c_int), ("tile_x", C.c_int),
                ("reserved", C.c_int * 3)]

    @classmethod
    def make(cls, **kw) -> "RtmParams":
        p = cls()
        p.storage, p.precision, p.compute, p.tile_x = STORE_RING, PREC_FP32, COMPUTE_FP32, 0
        p.time_slices = 20
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p

    def replace(self, **kw) -> "RtmParams":
        q = RtmParams()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(RtmParams))
        for k, v in kw.items():
            setattr(q, k, v)
        return q

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}

    @property
    def dim_x(self) -> int:
        return self.th_left + self.nx + self.th_right

    @property
    def dim_z(self) -> int:
        return self.th_up + self.nz + self.th_down

    @property
    def cell_updates(self) -> int:
        """Credited work of one migration: 2 * dimX * dimZ * nt (forward + backward)."""
        return 2 * self.dim_x * self.dim_z * self.nt

    def __repr__(self):
        return "RtmParams(%s)" % ", ".join("%s=%r" % kv for kv in self.as_dict().items())


class RtmSurvey(C.Structure):
    """rtm_survey: file patterns and shot layout of the migration driver (rtm_iso2d.c)."""
    _fields_ = [("velocity_file", C.c_char_p), ("wavelet_file", C.c_char_p),
                ("seismogram_file", C.c_char_p), ("stacked_file", C.c_char_p),
                ("laplacian_file", C.c_char_p), ("first_shot", C.c_int), ("shot_depth", C.c_int),
                ("shot_spacing", C.c_int), ("n_shots", C.c_int), ("zfp_tolerance", C.c_float),
                ("normalize_by_self", C.c_int), ("checkpoint_file", C.c_char_p)]

    @classmethod
    def make(cls, velocity_file, wavelet_file, seismogram_file, stacked_file, laplacian_file,
             first_shot, shot_depth, shot_spacing=0, n_shots=1, zfp_tolerance=0.0,
             normalize_by_self=0, checkpoint_file=None) -> "RtmSurvey":
        s = cls()
        s._keep = [x.encode() for x in (velocity_file, wavelet_file, seismogram_file, stacked_file,
                                         laplacian_file)]
        (s.velocity_file, s.wavelet_file, s.seismogram_file, s.stacked_file,
         s.laplacian_file) = s._keep
        s.first_shot, s.shot_depth, s.shot_spacing = first_shot, shot_depth, shot_spacing
        s.n_shots, s.zfp_tolerance = n_shots, zfp_tolerance
        s.normalize_by_self = normalize_by_self
        if checkpoint_file is not None:
            s._keep.append(checkpoint_file.encode())
            s.checkpoint_file = s._keep[-1]
        return s


class RtmError(RuntimeError):
    def __init__(self, status: int, detail: str):
        super().__init__("%s: %s" % (status_string(status), detail))
        self.status = status


_lib = None
_lock = threading.Lock()


def lib():
    """The loaded engine library (built in-tree on first use if absent)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path):
                _build.build()
            L = C.CDLL(path)
            _declare(L)
            _lib = L
    return _lib


def _declare(L):
    P = C.POINTER(RtmParams)
    vp, fp, ip = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int)
    sig = {
        "rtm_params_defaults": (None, [P]),
        "rtm_params_check": (C.c_int, [P]),
        "rtm_footprint_bytes": (C.c_longlong, [P]),
        "rtm_status_string": (C.c_char_p, [C.c_int]),
        "rtm_last_error": (C.c_char_p, []),
        "rtm_device_info": (C.c_int, [C.c_char_p, C.c_int, ip, C.POINTER(C.c_longlong)]),
        "rtm_forward_modeling": (C.c_int, [P, C.c_int, ip, fp, fp]),
        "rtm_adjoint_modeling": (C.c_int, [P, C.c_int, ip, fp, fp, fp, fp, fp]),
        "rtm_migrate_shot": (C.c_int, [P, fp, fp, fp, fp, fp]),
        "rtm_model_seismogram": (C.c_int, [P, fp, fp, fp]),
        "rtm_migrate_shot_zfp": (C.c_int, [P, fp, fp, vp, C.c_size_t, C.c_float, fp, fp]),
        "rtm_iso_acoustic_wave_equation": (C.c_int, [P, fp, fp, fp]),
        "rtm_aiso_attenuation_cpml": (C.c_int, [P, fp, fp, fp] + [fp] * 8 + [fp] * 8),
        "rtm_attenuation_profile_cpml": (None, [P] + [fp] * 8),
        "rtm_extend_matrix": (None, [P, fp, fp]),
        "rtm_laplacian_filter2D": (C.c_int, [P, fp, fp]),
        "rtm_normalized_cross_correlation": (C.c_int, [P, fp, fp, fp, fp]),
        "rtm_autotune": (C.c_int, [P, C.c_int, ip, C.POINTER(C.c_float)]),
        "rtm_plan_create": (C.c_int, [P, C.POINTER(vp)]),
        "rtm_plan_destroy": (C.c_int, [vp]),
        "rtm_plan_set_stream": (C.c_int, [vp, vp]),
        "rtm_plan_forward": (C.c_int, [vp, vp, vp, vp]),
        "rtm_plan_adjoint": (C.c_int, [vp, vp, vp, vp]),
        "rtm_plan_read_field": (C.c_int, [vp, C.c_int, vp]),
        "rtm_plan_read_image": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "rtm_plan_sync": (C.c_int, [vp]),
        "rtm_plan_capture_source": (C.c_int, [vp, C.c_int, ip, vp]),
        "rtm_plan_launch_count": (C.c_longlong, [vp]),
        "rtm_plan_bytes": (C.c_longlong, [vp]),
        "rtm_autotune_batched": (C.c_int, [P, C.c_int, C.c_int, ip, C.POINTER(C.c_float)]),
        "rtm_release_cached": (None, []),
        "rtm_server_create": (C.c_int, [C.c_longlong, C.c_int, C.c_int, C.POINTER(vp)]),
        "rtm_server_destroy": (C.c_int, [vp]),
        "rtm_server_submit": (C.c_int, [vp, P, fp, fp, fp, C.POINTER(C.c_longlong)]),
        "rtm_server_submit_zfp": (C.c_int, [vp, P, fp, fp, vp, C.c_size_t, C.c_float, C.POINTER(C.c_longlong)]),
        "rtm_server_step": (C.c_int, [vp, ip, ip]),
        "rtm_server_poll": (C.c_int, [vp, C.POINTER(C.c_longlong), fp, fp, C.POINTER(C.c_double)]),
        "rtm_server_wait": (C.c_int, [vp, C.c_longlong, fp, fp, C.POINTER(C.c_double)]),
        "rtm_server_stats": (C.c_int, [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                       C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "rtm_server_kernel_ms": (C.c_int, [vp, C.POINTER(C.c_double)]),
        "rtm_migrate_shot_static": (C.c_int, [P, vp, vp, vp, vp, vp, vp]),
        "rtm_zfp_decode_float2d": (C.c_int, [vp, C.c_size_t, C.c_double, C.c_int, C.c_int, fp]),
        "rtm_zfp_decode_file": (C.c_int, [C.c_char_p, fp, C.c_int, C.c_int, C.c_float]),
        "rtm_zfp_encode_bound": (C.c_size_t, [C.c_int, C.c_int]),
        "rtm_zfp_encode_float2d": (C.c_int, [fp, C.c_int, C.c_int, C.c_double, vp, C.c_size_t,
                                             C.POINTER(C.c_size_t)]),
        "rtm_routine_run": (C.c_int, [P, C.POINTER(RtmSurvey), C.c_int]),
        "rtm_routine_batch": (C.c_int, [P, C.POINTER(RtmSurvey), ip, C.c_int, C.c_longlong, C.c_int]),
        "rtm_routine_last_transfers": (C.c_int, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "rtm_stack_create": (C.c_int, [P, C.POINTER(vp)]),
        "rtm_stack_destroy": (C.c_int, [vp]),
        "rtm_stack_load": (C.c_int, [vp, fp, fp]),
        "rtm_adjoint_modeling_stacked": (C.c_int, [P, C.c_int, ip, fp, vp]),
        "rtm_stack_read_raw": (C.c_int, [vp, fp, fp]),
        "rtm_stack_finish": (C.c_int, [vp, C.c_int, fp, fp]),
        "rtm_stack_transfers": (C.c_int, [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "rtm_plan_profile": (C.c_int, [vp, C.c_int]),
        "rtm_plan_profile_read": (C.c_int, [vp, C.POINTER(C.c_double), ip, C.POINTER(C.c_double), ip]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def exported_symbols():
    """Names declared in include/rtm_gpu.h that the binding declares."""
    return ["rtm_params_defaults", "rtm_params_check", "rtm_footprint_bytes", "rtm_status_string",
            "rtm_last_error", "rtm_device_info", "rtm_forward_modeling", "rtm_adjoint_modeling",
            "rtm_migrate_shot", "rtm_migrate_shot_zfp", "rtm_model_seismogram", "rtm_iso_acoustic_wave_equation",
            "rtm_aiso_attenuation_cpml", "rtm_attenuation_profile_cpml", "rtm_extend_matrix",
            "rtm_laplacian_filter2D", "rtm_normalized_cross_correlation", "rtm_autotune", "rtm_plan_create",
            "rtm_plan_destroy", "rtm_plan_set_stream", "rtm_plan_forward", "rtm_plan_adjoint",
            "rtm_plan_read_field", "rtm_plan_read_image", "rtm_plan_sync", "rtm_plan_capture_source",
            "rtm_plan_launch_count",
            "rtm_plan_bytes", "rtm_autotune_batched", "rtm_release_cached", "rtm_plan_profile", "rtm_plan_profile_read",
            "rtm_server_create", "rtm_server_destroy", "rtm_server_submit", "rtm_server_submit_zfp",
            "rtm_server_step",
            "rtm_server_poll", "rtm_server_wait", "rtm_server_stats", "rtm_server_kernel_ms", "rtm_migrate_shot_static",
            "rtm_zfp_decode_float2d", "rtm_zfp_decode_file", "rtm_zfp_encode_bound",
            "rtm_zfp_encode_float2d", "rtm_routine_run", "rtm_routine_batch", "rtm_routine_last_transfers",
            "rtm_stack_create", "rtm_stack_destroy", "rtm_stack_load", "rtm_adjoint_modeling_stacked",
            "rtm_stack_read_raw", "rtm_stack_finish", "rtm_stack_transfers"]


def status_string(st: int) -> str:
    return lib().rtm_status_string(st).decode()


def _check(st: int) -> None:
    if st != RTM_OK:
        raise RtmError(st, lib().rtm_last_error().decode())


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _dev(x):
    if x is None:
        return None
    if isinstance(x, int):
        return C.c_void_p(x)
    return C.c_void_p(x.data_ptr())


# ---- configuration helpers -------------------------------------------------------------------
def params_check(p: RtmParams) -> None:
    _check(lib().rtm_params_check(C.byref(p)))


def footprint_bytes(p: RtmParams) -> int:
    return int(lib().rtm_footprint_bytes(C.byref(p)))


def device_info():
    name = C.create_string_buffer(256)
    sms = C.c_int()
    mem = C.c_longlong()
    _check(lib().rtm_device_info(name, 256, C.byref(sms), C.byref(mem)))
    return {"name": name.value.decode(), "sm_count": sms.value, "hbm_bytes": mem.value}


# ---- host-side set-up (same arithmetic as the reference) ------------------------------------
def attenuation_profile_cpml(p: RtmParams) -> dict:
    a = {k: np.zeros(n, np.float32) for k, n in
         (("a_l", p.th_left), ("a_r", p.th_right), ("a_t", p.th_up), ("a_b", p.th_down),
          ("b_l", p.th_left), ("b_r", p.th_right), ("b_t", p.th_up), ("b_b", p.th_down))}
    lib().rtm_attenuation_profile_cpml(C.byref(p), *[_fp(a[k]) for k in
                                       ("a_l", "a_r", "a_t", "a_b", "b_l", "b_r", "b_t", "b_b")])
    return a


def extend_matrix(p: RtmParams, model: np.ndarray) -> np.ndarray:
    out = np.zeros((p.dim_x, p.dim_z), np.float32)
    lib().rtm_extend_matrix(C.byref(p), _fp(out), _fp(_f32(model)))
    return out


# ---- reference-shaped entry points on host arrays ------------------------------------------
def forward_modeling(p: RtmParams, sim_id: int, shot, velocity, wavelet) -> None:
    """isotropicAcousticModeling: source wavefield stays on the device under sim_id."""
    s = (C.c_int * 2)(*shot) if shot is not None else None
    _check(lib().rtm_forward_modeling(C.byref(p), sim_id, s, _fp(_f32(velocity)), _fp(_f32(wavelet))))


def adjoint_modeling(p: RtmParams, sim_id: int, shot, velocity, wavelet, seismogram,
                     image: np.ndarray, self_image: np.ndarray) -> None:
    """adjointModeling: accumulates into image/self_image (float32, nx x nz, in place)."""
    s = (C.c_int * 2)(*shot) if shot is not None else None
    assert image.dtype == np.float32 and image.flags.c_contiguous
    assert self_image.dtype == np.float32 and self_image.flags.c_contiguous
    _check(lib().rtm_adjoint_modeling(C.byref(p), sim_id, s, _fp(_f32(velocity)), _fp(_f32(wavelet)),
                                      _fp(_f32(seismogram)), _fp(image), _fp(self_image)))


def migrate_shot(p: RtmParams, velocity, wavelet, seismogram):
    img = np.zeros((p.nx, p.nz), np.float32)
    slf = np.zeros((p.nx, p.nz), np.float32)
    _check(lib().rtm_migrate_shot(C.byref(p), _fp(_f32(velocity)), _fp(_f32(wavelet)),
                                  _fp(_f32(seismogram)), _fp(img), _fp(slf)))
    return img, slf


def migrate_shot_zfp(p: RtmParams, velocity, wavelet, stream: bytes, tol: float):
    """migrate_shot with the seismogram as a ZFP fixed-accuracy stream, decoded on a host thread
    while the forward pass runs; returns (image, self image)."""
    img = np.zeros((p.nx, p.nz), np.float32)
    slf = np.zeros((p.nx, p.nz), np.float32)
    buf = np.frombuffer(bytes(stream), np.uint8)
    _check(lib().rtm_migrate_shot_zfp(C.byref(p), _fp(_f32(velocity)), _fp(_f32(wavelet)),
                                      buf.ctypes.data_as(C.c_void_p), buf.size, C.c_float(tol), _fp(img),
                                      _fp(slf)))
    return img, slf


def model_seismogram(p: RtmParams, velocity, wavelet) -> np.ndarray:
    seis = np.zeros((p.rec_count, p.nt), np.float32)
    _check(lib().rtm_model_seismogram(C.byref(p), _fp(_f32(velocity)), _fp(_f32(wavelet)), _fp(seis)))
    return seis


def iso_acoustic_wave_equation(p: RtmParams, pond, wave2, wave3) -> np.ndarray:
    out = np.array(wave3, np.float32, copy=True)
    _check(lib().rtm_iso_acoustic_wave_equation(C.byref(p), _fp(_f32(pond)), _fp(_f32(wave2)), _fp(out)))
    return out


def aiso_attenuation_cpml(p: RtmParams, wave1, wave2, coef, prof: dict, psi: dict, xi: dict):
    out = np.array(wave2, np.float32, copy=True)
    _check(lib().rtm_aiso_attenuation_cpml(
        C.byref(p), _fp(_f32(wave1)), _fp(out), _fp(_f32(coef)),
        _fp(prof["a_l"]), _fp(prof["b_l"]), _fp(prof["a_r"]), _fp(prof["b_r"]),
        _fp(prof["a_t"]), _fp(prof["b_t"]), _fp(prof["a_b"]), _fp(prof["b_b"]),
        _fp(psi["l"]), _fp(psi["r"]), _fp(psi["t"]), _fp(psi["b"]),
        _fp(xi["l"]), _fp(xi["r"]), _fp(xi["t"]), _fp(xi["b"])))
    return out


def normalized_cross_correlation(p: RtmParams, image, self_image, source, receiver) -> None:
    _check(lib().rtm_normalized_cross_correlation(C.byref(p), _fp(image), _fp(self_image),
                                                  _fp(_f32(source)), _fp(_f32(receiver))))


def laplacian_filter2D(p: RtmParams, image) -> np.ndarray:
    out = np.zeros((p.nx, p.nz), np.float32)
    _check(lib().rtm_laplacian_filter2D(C.byref(p), _fp(out), _fp(_f32(image))))
    return out


def zfp_decode(stream: bytes, nx: int, ny: int, tolerance: float) -> np.ndarray:
    """ZFP 0.5.5 fixed-accuracy decode of an nx (fastest) x ny float field; returned as the
    reference's flat buffer viewed (nx, ny) -- (rec_count, nt) for a seismogram."""
    buf = np.frombuffer(bytes(stream), np.uint8)
    out = np.empty(nx * ny, np.float32)
    _check(lib().rtm_zfp_decode_float2d(buf.ctypes.data_as(C.c_void_p), buf.size, float(tolerance),
                                        nx, ny, _fp(out)))
    return out.reshape(nx, ny)


def zfp_encode(field: np.ndarray, tolerance: float) -> bytes:
    """ZFP 0.5.5 fixed-accuracy stream of a (nx, ny) float field in the reference's flat
    layout (zfp nx = field.shape[0] fastest) -- what zfp2d_lossyCompression writes."""
    a = _f32(field)
    nx, ny = a.shape
    cap = lib().rtm_zfp_encode_bound(nx, ny)
    buf = np.empty(cap, np.uint8)
    n = C.c_size_t()
    _check(lib().rtm_zfp_encode_float2d(_fp(a), nx, ny, float(tolerance), buf.ctypes.data_as(C.c_void_p),
                                        cap, C.byref(n)))
    return buf[: n.value].tobytes()


def routine_run(p: RtmParams, survey: RtmSurvey, simulation_id: int) -> None:
    """The migration driver of one simulation on files (rtm_iso2d.c:15-177)."""
    _check(lib().rtm_routine_run(C.byref(p), C.byref(survey), simulation_id))


def routine_batch(p: RtmParams, survey: RtmSurvey, simulation_ids, hbm_budget_bytes: int = 0,
                  max_members: int = 0) -> None:
    """rtm_routine over several simulations through one batched server (the reference's MPI
    fan-out, on one GPU): per simulation the same output files as routine_run."""
    ids = (C.c_int * len(simulation_ids))(*[int(i) for i in simulation_ids])
    _check(lib().rtm_routine_batch(C.byref(p), C.byref(survey), ids, len(simulation_ids),
                                   int(hbm_budget_bytes), int(max_members)))


def routine_last_transfers():
    """(device-to-host copies, bytes) of the last routine_run on this thread."""
    c, b = C.c_longlong(), C.c_longlong()
    _check(lib().rtm_routine_last_transfers(C.byref(c), C.byref(b)))
    return c.value, b.value


class Stack:
    """Shot stack in device memory (include/rtm_gpu.h, rtm_stack_*): shots' images added where
    the adjoint pass leaves them, the final stack and its Laplacian back in one copy."""

    def __init__(self, p: RtmParams):
        self.params = p.replace()
        h = C.c_void_p()
        _check(lib().rtm_stack_create(C.byref(self.params), C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().rtm_stack_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, image_stack=None, self_stack=None):
        a = _f32(image_stack) if image_stack is not None else None
        b = _f32(self_stack) if self_stack is not None else None
        _check(lib().rtm_stack_load(self.handle, _fp(a) if a is not None else None,
                                    _fp(b) if b is not None else None))

    def adjoint(self, p: RtmParams, sim_id: int, shot, seismogram) -> None:
        """rtm_adjoint_modeling of sim_id's forward state, added to this stack."""
        sh = (C.c_int * 2)(*shot)
        s = _f32(seismogram) if seismogram is not None else None
        _check(lib().rtm_adjoint_modeling_stacked(C.byref(p), sim_id, sh, _fp(s) if s is not None else None,
                                                  self.handle))

    def read_raw(self):
        p = self.params
        img = np.empty((p.nx, p.nz), np.float32)
        slf = np.empty((p.nx, p.nz), np.float32)
        _check(lib().rtm_stack_read_raw(self.handle, _fp(img), _fp(slf)))
        return img, slf

    def finish(self, normalize_by_self: bool = False):
        """(stacked image, its Laplacian), nx x nz each."""
        p = self.params
        out = np.empty((p.nx, p.nz), np.float32)
        lap = np.empty((p.nx, p.nz), np.float32)
        _check(lib().rtm_stack_finish(self.handle, int(bool(normalize_by_self)), _fp(out), _fp(lap)))
        return out, lap

    def transfers(self):
        c, b = C.c_longlong(), C.c_longlong()
        _check(lib().rtm_stack_transfers(self.handle, C.byref(c), C.byref(b)))
        return c.value, b.value


def dropin_lib():
    """librtm_dropin.so: the reference's entry-point names over the engine."""
    lib()
    return C.CDLL(_build.DROPIN_LIB)


def autotune_batched(p: RtmParams, members: int = 8, steps: int = 40):
    """Batched tile width (32 or 16) for p's grid shape, used by later server submissions of
    that shape with tile_x = 0; returns (tile_x, ms per batched step of `members` copies)."""
    t = C.c_int()
    ms = C.c_float()
    _check(lib().rtm_autotune_batched(C.byref(p), int(members), int(steps), C.byref(t), C.byref(ms)))
    return t.value, ms.value


def autotune(p: RtmParams, steps: int = 200):
    """Fastest step-kernel tile width for p's grid shape (used by later plans with tile_x = 0);
    returns (tile_x, ms per forward step)."""
    t = C.c_int()
    ms = C.c_float()
    _check(lib().rtm_autotune(C.byref(p), steps, C.byref(t), C.byref(ms)))
    return t.value, ms.value


def release_cached() -> None:
    lib().rtm_release_cached()


# ---- device-resident plan -----------------------------------------------------------------
class Plan:
    """One migration's device state (include/rtm_gpu.h, rtm_plan_*)."""

    def __init__(self, p: RtmParams):
        self.params = p.replace()
        h = C.c_void_p()
        _check(lib().rtm_plan_create(C.byref(self.params), C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().rtm_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int):
        _check(lib().rtm_plan_set_stream(self.handle, C.c_void_p(stream_ptr)))

    def forward(self, d_velocity, d_wavelet, d_seismogram_out=None):
        _check(lib().rtm_plan_forward(self.handle, _dev(d_velocity), _dev(d_wavelet),
                                      _dev(d_seismogram_out)))

    def adjoint(self, d_seismogram, d_image=None, d_self_image=None):
        _check(lib().rtm_plan_adjoint(self.handle, _dev(d_seismogram), _dev(d_image), _dev(d_self_image)))

    def read_field(self, which: int, d_out):
        _check(lib().rtm_plan_read_field(self.handle, which, _dev(d_out)))

    def read_image(self, which: int, d_out, as_double: bool = False):
        _check(lib().rtm_plan_read_image(self.handle, which, int(as_double), _dev(d_out)))

    def sync(self):
        _check(lib().rtm_plan_sync(self.handle))

    def capture_source(self, times, d_out=None):
        """Source wavefield of the next adjoint pass at forward times `times` into d_out
        (len(times) x dimX x dimZ device elements of the compute type); [] clears."""
        t = (C.c_int * max(1, len(times)))(*times)
        _check(lib().rtm_plan_capture_source(self.handle, len(times), t, _dev(d_out)))

    def profile(self, every: int):
        _check(lib().rtm_plan_profile(self.handle, every))

    def profile_read(self):
        fm, bm = C.c_double(), C.c_double()
        fn, bn = C.c_int(), C.c_int()
        _check(lib().rtm_plan_profile_read(self.handle, C.byref(fm), C.byref(fn), C.byref(bm), C.byref(bn)))
        return {"fwd_ms": fm.value, "fwd_n": fn.value, "bwd_ms": bm.value, "bwd_n": bn.value}

    @property
    def launches(self) -> int:
        return int(lib().rtm_plan_launch_count(self.handle))

    @property
    def nbytes(self) -> int:
        return int(lib().rtm_plan_bytes(self.handle))


# ---- serving / batching -------------------------------------------------------------------
class Server:
    """Continuous-batching server of resident migrations (include/rtm_gpu.h, rtm_server_*)."""

    def __init__(self, hbm_budget_bytes: int = 0, max_members: int = 64, steps_per_launch: int = 16):
        h = C.c_void_p()
        _check(lib().rtm_server_create(hbm_budget_bytes, max_members, steps_per_launch, C.byref(h)))
        self.handle = h
        self.params = {}

    def close(self):
        if self.handle:
            lib().rtm_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, p: RtmParams, velocity, wavelet, seismogram) -> int:
        rid = C.c_longlong()
        q = p.replace()
        _check(lib().rtm_server_submit(self.handle, C.byref(q), _fp(_f32(velocity)), _fp(_f32(wavelet)),
                                       _fp(_f32(seismogram)), C.byref(rid)))
        self.params[rid.value] = q
        return rid.value

    def submit_zfp(self, p: RtmParams, velocity, wavelet, stream: bytes, tol: float) -> int:
        """Submit with the seismogram as a ZFP stream; decoded by the server's host threads."""
        rid = C.c_longlong()
        q = p.replace()
        buf = np.frombuffer(bytes(stream), np.uint8)
        _check(lib().rtm_server_submit_zfp(self.handle, C.byref(q), _fp(_f32(velocity)), _fp(_f32(wavelet)),
                                           buf.ctypes.data_as(C.c_void_p), buf.size, C.c_float(tol), C.byref(rid)))
        self.params[rid.value] = q
        return rid.value

    def step(self):
        a, qd = C.c_int(), C.c_int()
        _check(lib().rtm_server_step(self.handle, C.byref(a), C.byref(qd)))
        return a.value, qd.value

    def poll(self):
        """(request_id, image, self_image, (t_submit, t_admit, t_done)) or None."""
        if not self.params:
            return None
        # the finished request's size is unknown until polled: use the largest pending one
        n = max(p.nx * p.nz for p in self.params.values())
        img = np.zeros(n, np.float32)
        slf = np.zeros(n, np.float32)
        rid = C.c_longlong()
        times = (C.c_double * 3)()
        st = lib().rtm_server_poll(self.handle, C.byref(rid), _fp(img), _fp(slf), times)
        if st == RTM_ERR_BUSY:
            return None
        _check(st)
        p = self.params.pop(rid.value)
        m = p.nx * p.nz
        return (rid.value, img[:m].reshape(p.nx, p.nz).copy(), slf[:m].reshape(p.nx, p.nz).copy(),
                tuple(times))

    def wait(self, request_id: int):
        """Steps until request_id has finished: (image, self_image, (t_submit, t_admit, t_done))."""
        p = self.params.get(request_id)       # None: not pending here, the library refuses it
        shape = (p.nx, p.nz) if p is not None else (0,)
        img = np.zeros(shape, np.float32)
        slf = np.zeros(shape, np.float32)
        times = (C.c_double * 3)()
        _check(lib().rtm_server_wait(self.handle, request_id, _fp(img), _fp(slf), times))
        del self.params[request_id]
        return img, slf, tuple(times)

    def stats(self) -> dict:
        cu, ms, ln, by = C.c_longlong(), C.c_double(), C.c_longlong(), C.c_longlong()
        _check(lib().rtm_server_stats(self.handle, C.byref(cu), C.byref(ms), C.byref(ln), C.byref(by)))
        return {"cell_updates": cu.value, "gpu_ms": ms.value, "launches": ln.value, "bytes_in_use": by.value}

    def kernel_ms(self) -> float:
        """CUDA-event time of the tile kernel on the second step of the last step() call's
        graph replay (launched without overlap; 0 if steps_per_launch < 2)."""
        v = C.c_double()
        _check(lib().rtm_server_kernel_ms(self.handle, C.byref(v)))
        return v.value

    def run_all(self):
        """Steps until every submitted migration has finished; returns {id: (img, self, times)}."""
        out = {}
        while True:
            active, queued = self.step()
            while True:
                r = self.poll()
                if r is None:
                    break
                out[r[0]] = r[1:]
            if active == 0 and queued == 0 and not self.params:
                return out
