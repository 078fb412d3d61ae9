"""ctypes mirror of ``cvtpm_params`` (include/cvtpm.h) and its two presets.

REFERENCE holds the constants of the reference's OpenCL path
(cvt/cl/kernel/pmhstereo.cl:27-40, cvt/vision/PMHuberStereo.cpp:70-76,243):
window radius 17, LR thresholds 0.5 px / 10 degrees, theta scale 50, 250 PD
steps, colour weight 26 with the smoothstep spatial ramp, colour share 0.05,
truncations 0.04 / 0.01, MWC64X streams and the reference's exact operation
order.

BASELINE holds the cost constants the benchmark configurations are stated in:
gamma = 10 (a constant colour factor 255/gamma), gradient share alpha = 0.9
(colour share 0.1), tau_col = 10/255, tau_grad = 2/255; Philox streams and the
fast FMA arithmetic.
"""
from __future__ import annotations

import ctypes

RNG_MWC64X, RNG_PHILOX = 0, 1
ARITH_EXACT, ARITH_FAST = 0, 1
SCHEDULE_JACOBI, SCHEDULE_REDBLACK = 0, 1
PROFILE_SMOOTHSTEP, PROFILE_CONSTANT = 0, 1
PRESET_REFERENCE, PRESET_BASELINE = 0, 1

BASELINE_SEED = 0x5EED_0000_CAFE


class CvtpmParams(ctypes.Structure):
    _fields_ = [
        ("patchsize", ctypes.c_int),
        ("depthmax", ctypes.c_float),
        ("iterations", ctypes.c_int),
        ("viewsamples", ctypes.c_int),
        ("dscale", ctypes.c_float),
        ("maxdispdiff", ctypes.c_float),
        ("maxanglediff", ctypes.c_float),
        ("thetascale", ctypes.c_float),
        ("pd_iterations", ctypes.c_int),
        ("color_weight", ctypes.c_float),
        ("color_alpha", ctypes.c_float),
        ("color_maxdiff", ctypes.c_float),
        ("grad_maxdiff", ctypes.c_float),
        ("weight_profile", ctypes.c_int),
        ("rng", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("arith", ctypes.c_int),
        ("schedule", ctypes.c_int),
    ]

    def replace(self, **kw) -> "CvtpmParams":
        p = CvtpmParams()
        ctypes.pointer(p)[0] = self
        for k, v in kw.items():
            if not hasattr(p, k):
                raise AttributeError(k)
            setattr(p, k, v)
        return p

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def default_params(preset: int = PRESET_REFERENCE, **kw) -> CvtpmParams:
    p = CvtpmParams()
    p.patchsize = 17
    p.depthmax = 64.0
    p.iterations = 3
    p.viewsamples = 4
    p.dscale = -1.0
    p.maxdispdiff = 0.5
    p.maxanglediff = 10.0
    p.thetascale = 50.0
    p.pd_iterations = 250
    p.color_weight = 26.0
    p.color_alpha = 0.05
    p.color_maxdiff = 0.04
    p.grad_maxdiff = 0.01
    p.weight_profile = PROFILE_SMOOTHSTEP
    p.rng = RNG_MWC64X
    p.seed = 0
    p.arith = ARITH_EXACT
    p.schedule = SCHEDULE_JACOBI
    if preset == PRESET_BASELINE:
        p.color_weight = 25.5
        p.weight_profile = PROFILE_CONSTANT
        p.color_alpha = 0.1
        p.color_maxdiff = 10.0 / 255.0
        p.grad_maxdiff = 2.0 / 255.0
        p.rng = RNG_PHILOX
        p.seed = BASELINE_SEED
        p.arith = ARITH_FAST
    elif preset != PRESET_REFERENCE:
        raise ValueError(f"unknown preset {preset}")
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p
