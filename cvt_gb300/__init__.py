"""cvt_gb300 — GB300-native (sm_103a) slanted-plane PatchMatch stereo.

A from-scratch CUDA implementation of the OpenCL path behind CVT's
``PMHuberStereo::depthMap`` (cvt/vision/PMHuberStereo.cpp:64-291), exposed
through the C ABI in include/cvtpm.h (libcvtpm.so) and mirrored here for
torch tensors.
"""
from .params import (CvtpmParams, default_params, PRESET_REFERENCE, PRESET_BASELINE,  # noqa: F401
                     RNG_MWC64X, RNG_PHILOX, ARITH_EXACT, ARITH_FAST)

__all__ = ["CvtpmParams", "default_params", "PRESET_REFERENCE", "PRESET_BASELINE",
           "RNG_MWC64X", "RNG_PHILOX", "ARITH_EXACT", "ARITH_FAST"]


def __getattr__(name):
    if name in ("PMHuberStereo", "CVTException"):
        from . import stereo
        return getattr(stereo, name)
    raise AttributeError(name)
