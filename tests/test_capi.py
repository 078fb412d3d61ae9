"""The C ABI library (no GPU needed): it loads, exports every function
include/*.h declares, and its presets equal the Python mirror's."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(cvtpm_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def L():
    from cvt_gb300 import _lib
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    names = declared_functions()
    assert len(names) >= 14
    for n in sorted(names):
        assert hasattr(L, n), n


def test_python_binding_covers_header():
    from cvt_gb300 import _lib
    assert declared_functions() == set(_lib.EXPORTS)


def test_presets_match(L):
    from cvt_gb300 import _lib, params
    for preset in (params.PRESET_REFERENCE, params.PRESET_BASELINE):
        assert _lib.c_default_params(preset).as_dict() == params.default_params(preset).as_dict()
    p = params.CvtpmParams()
    assert L.cvtpm_params_default(ctypes.byref(p), 7) != 0


def test_status_strings(L):
    from cvt_gb300 import _lib
    assert _lib.status_string(0) == "ok"
    assert "CUDA" in _lib.status_string(4)
    assert _lib.version().startswith("cvt-gb300")


def test_null_arguments_rejected(L):
    assert L.cvtpm_create(None, 0) != 0
    assert L.cvtpm_destroy(None) != 0
    assert L.cvtpm_set_params(None, None) != 0
    assert L.cvtpm_depthmap(None, None, 0, None, None, 1, 1, 16, 17, 64.0, 1, 4, -1.0, None, 0, None, None) != 0
    us = ctypes.c_float(0.0)
    assert L.cvtpm_tool_pd_time(None, 8, None, ctypes.byref(us)) == 1      # CVTPM_ERR_INVALID_ARGUMENT
    assert L.cvtpm_tool_fp32_peak(0, None, None) == 1


def test_params_struct_layout():
    from cvt_gb300.params import CvtpmParams
    # int, float x7 ... as in include/cvtpm.h; uint64 seed aligned to 8
    assert CvtpmParams.seed.offset % 8 == 0
    assert ctypes.sizeof(CvtpmParams) == 80


def test_noalloc_rejects_misaligned_buffers_before_any_device_call(L):
    """cvtpm_cost_eval_noalloc reads the states as float4 and writes float
    costs: pointers that are not 16- (states) or 4-byte (cost) aligned are
    refused with CVTPM_ERR_INVALID_ARGUMENT before anything touches the
    device, so fake addresses that are never dereferenced suffice here."""
    from cvt_gb300.params import default_params, PRESET_REFERENCE
    p = default_params(PRESET_REFERENCE, patchsize=5)
    img, out = 0x10000, 0x20000                      # aligned, never dereferenced
    W, H = 16, 8

    def call(states, cost):
        return L.cvtpm_cost_eval_noalloc(ctypes.byref(p), img, img, W, H, W * 16, states, cost, None)

    assert call(0x30000 + 4, out) == 1               # states off by 4 bytes
    assert call(0x30000 + 8, out) == 1               # off by 8
    assert call(0x30000, out + 2) == 1               # cost off by 2
    assert call(None, out) == 1
