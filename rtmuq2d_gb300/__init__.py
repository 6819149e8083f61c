"""GB300-native (sm_103a) engine for rtmUq2D's 2-D isotropic acoustic RTM path.

The compute path is hand-written CUDA in csrc/, exposed through the C ABI of
include/rtm_gpu.h (librtmgpu.so); ``capi`` is its ctypes binding.  There is no CPU
fallback: a missing or unloadable library raises.
"""
from .capi import (COMPUTE_FP32, COMPUTE_FP64, PREC_BF16, PREC_FP16, PREC_FP32, STORE_RING,
                   STORE_SNAPSHOT, Plan, RtmError, RtmParams, RtmSurvey, Server, Stack, adjoint_modeling, autotune, autotune_batched,
                   aiso_attenuation_cpml, attenuation_profile_cpml, device_info, extend_matrix,
                   footprint_bytes, forward_modeling, iso_acoustic_wave_equation,
                   laplacian_filter2D, lib, migrate_shot, migrate_shot_zfp, model_seismogram,
                   normalized_cross_correlation, params_check, release_cached, routine_batch, routine_last_transfers,
                   routine_run,
                   dropin_lib, zfp_decode, zfp_encode)

__all__ = [n for n in dir() if not n.startswith("_")]
