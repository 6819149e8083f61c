"""rtm_migrate_shot_static: the single-shot migration whose scratch lives in a static device
array inside the library, for callers that cannot call cudaMalloc (device memory owned by
another allocator or held to a fixed budget, or a loop that cannot take an allocation's
implicit device synchronisation).

Called through the C ABI twice in a row -- the second call reuses what the first left in the
shared array -- and compared with the existing plan entry points (rtm_plan_create / _forward /
_adjoint) on the same inputs, within the image tolerance of the parity tests (rel-L2 1e-4).
Before those two calls, a call of another configuration (a smaller grid with BF16 ring
storage) leaves other contents at other offsets of the array.
This file sorts last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IMAGE_TOL = 1e-4


def _rel(a, b):
    a = a.double()
    b = b.double()
    return float((a - b).norm() / b.norm())


def test_static_scratch_migration_matches_plan_entry_points():
    import torch

    import rtmuq2d_gb300 as eng
    from rtmuq2d_gb300 import workloads

    lib = eng.lib()
    fn = lib.rtm_migrate_shot_static
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(eng.RtmParams)] + [C.c_void_p] * 6

    p = workloads.params_small(nt=600)            # 400 x 200 model, ring storage
    assert eng.footprint_bytes(p) <= 64 << 20
    true, mig = workloads.models_small(p, seed=4)
    wav = workloads.wavelet_for(p)
    ext_true = eng.extend_matrix(p, true)
    ext = eng.extend_matrix(p, mig)
    seis = eng.model_seismogram(p, ext_true, wav)
    dv = torch.from_numpy(ext).cuda()
    dw = torch.from_numpy(wav).cuda()
    ds = torch.from_numpy(seis).cuda()

    ref_img = torch.empty((p.nx, p.nz), dtype=torch.float32, device="cuda")
    ref_slf = torch.empty_like(ref_img)
    plan = eng.Plan(p)
    plan.forward(dv, dw)
    plan.adjoint(ds, ref_img, ref_slf)
    plan.sync()
    plan.close()
    assert float(ref_img.abs().max()) > 0

    # another layout first: smaller grid, shorter time axis, 16-bit ring storage
    q = workloads.params_small(nx=240, nz=120, shot_x=120, rec_count=240, nt=400, precision=eng.PREC_BF16)
    qv = torch.from_numpy(eng.extend_matrix(q, mig[:240, :120])).cuda()
    qs = torch.from_numpy(np.ascontiguousarray(seis[:240, :400])).cuda()
    qi = torch.empty((q.nx, q.nz), dtype=torch.float32, device="cuda")
    qsl = torch.empty_like(qi)
    st = fn(C.byref(q), qv.data_ptr(), dw.data_ptr(), qs.data_ptr(), qi.data_ptr(), qsl.data_ptr(), None)
    assert st == 0, lib.rtm_last_error().decode()
    assert bool(torch.isfinite(qi).all())

    for call in range(2):
        img = torch.full((p.nx, p.nz), float("nan"), dtype=torch.float32, device="cuda")
        slf = torch.full_like(img, float("nan"))
        st = fn(C.byref(p), dv.data_ptr(), dw.data_ptr(), ds.data_ptr(), img.data_ptr(),
                slf.data_ptr(), None)
        assert st == 0, lib.rtm_last_error().decode()
        torch.cuda.synchronize()
        assert _rel(img, ref_img) <= IMAGE_TOL, call
        assert _rel(slf, ref_slf) <= IMAGE_TOL, call

    # a migration larger than the static array is refused with a clear error
    big = workloads.params_large()
    st = fn(C.byref(big), dv.data_ptr(), dw.data_ptr(), ds.data_ptr(), img.data_ptr(),
            slf.data_ptr(), None)
    assert st == eng.capi.RTM_ERR_INVALID
    assert b"static array holds" in lib.rtm_last_error()
