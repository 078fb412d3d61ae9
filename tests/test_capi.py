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


def test_params_struct_layout():
    from cvt_gb300.params import CvtpmParams
    # int, float x7 ... as in include/cvtpm.h; uint64 seed aligned to 8
    assert CvtpmParams.seed.offset % 8 == 0
    assert ctypes.sizeof(CvtpmParams) == 80
