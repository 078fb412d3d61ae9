"""The C++ facade include/cvt/PMHuberStereo.hpp: it compiles against the C
ABI here, and on a GPU a C++ program using it gives the same disparity map
as the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from bitcmp import bit_diff

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"
CUDA_LIB = "/usr/local/cuda/lib64"


def _gxx():
    g = shutil.which("g++")
    if not g or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or CUDA headers missing")
    return g


def test_facade_compiles(tmp_path):
    g = _gxx()
    src = os.path.join(ROOT, "tests", "cpp", "facade_main.cpp")
    r = subprocess.run([g, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                        "-I", CUDA_INC, src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_matches_oracle(tmp_path, cuda, oracle):
    g = _gxx()
    from cvt_gb300 import scenes
    from cvt_gb300.params import default_params, PRESET_REFERENCE
    from cvt_gb300._lib import LIB_PATH
    exe = str(tmp_path / "facade")
    r = subprocess.run([g, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC,
                        os.path.join(ROOT, "tests", "cpp", "facade_main.cpp"), "-o", exe,
                        LIB_PATH, f"-Wl,-rpath,{os.path.dirname(LIB_PATH)}", "-L", CUDA_LIB, "-lcudart",
                        f"-Wl,-rpath,{CUDA_LIB}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sc = scenes.make_scene(45, 33, 3, 10.0, seed=12)
    sc.left.tofile(tmp_path / "l.raw")
    sc.right.tofile(tmp_path / "r.raw")
    out = tmp_path / "d.raw"
    r = subprocess.run([exe, "45", "33", "5", "10", "2", str(tmp_path / "l.raw"), str(tmp_path / "r.raw"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.float32).reshape(33, 45)
    want, _ = oracle.depthmap(default_params(PRESET_REFERENCE, patchsize=5, depthmax=10.0, iterations=2),
                              sc.left, sc.right)
    assert not bit_diff(got, want).any()


@pytest.mark.gpu
def test_facade_loads_files_and_reads_any_format(tmp_path, cuda, oracle):
    """cvt::Image::load of a CVTRaw RGBA_UINT8 left and a BGRA_UINT8 right,
    depthMap, cvt::Image::save as PFM: the oracle's disparities on the
    read_imagef conversion of both."""
    g = _gxx()
    from cvt_gb300 import scenes, imageio
    from cvt_gb300.params import default_params, PRESET_REFERENCE
    from cvt_gb300._lib import LIB_PATH
    exe = str(tmp_path / "facade")
    r = subprocess.run([g, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC,
                        os.path.join(ROOT, "tests", "cpp", "facade_main.cpp"), "-o", exe,
                        LIB_PATH, f"-Wl,-rpath,{os.path.dirname(LIB_PATH)}", "-L", CUDA_LIB, "-lcudart",
                        f"-Wl,-rpath,{CUDA_LIB}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sc = scenes.make_scene(45, 33, 3, 10.0, seed=13)
    lu8 = np.round(sc.left * 255).astype(np.uint8)
    ru8 = np.ascontiguousarray(np.round(sc.right * 255).astype(np.uint8)[..., [2, 1, 0, 3]])
    imageio.write_raw(tmp_path / "l.raw", lu8, imageio.RGBA_UINT8)
    imageio.write_raw(tmp_path / "r.raw", ru8, imageio.BGRA_UINT8)
    out = tmp_path / "d.pfm"
    r = subprocess.run([exe, "--files", "5", "10", "2", str(tmp_path / "l.raw"), str(tmp_path / "r.raw"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    data = out.read_bytes().split(b"\n", 3)
    assert data[0] == b"Pf" and data[1] == b"45 33"
    got = np.frombuffer(data[3], "<f4").reshape(33, 45)[::-1]
    want, _ = oracle.depthmap(default_params(PRESET_REFERENCE, patchsize=5, depthmax=10.0, iterations=2),
                              oracle.image_to_rgbaf(lu8, imageio.RGBA_UINT8),
                              oracle.image_to_rgbaf(ru8, imageio.BGRA_UINT8))
    assert not bit_diff(got, want).any()


@pytest.mark.gpu
def test_facade_png_pair_and_png_output(tmp_path, cuda, oracle):
    """cvt::Image::load of an 8-bit RGB PNG left (RGBA_UINT8, alpha 255) and a
    16-bit RGBA PNG right (RGBA_UINT16), depthMap, cvt::Image::save as PNG:
    the GRAY_FLOAT map written through the reference's float-to-sRGB
    conversion, against the oracle's disparities on the same inputs."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import pngtool
    from cvt_gb300 import _lib, scenes, imageio
    from cvt_gb300.params import default_params, PRESET_REFERENCE
    from cvt_gb300._lib import LIB_PATH
    g = _gxx()
    exe = str(tmp_path / "facade")
    r = subprocess.run([g, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC,
                        os.path.join(ROOT, "tests", "cpp", "facade_main.cpp"), "-o", exe,
                        LIB_PATH, f"-Wl,-rpath,{os.path.dirname(LIB_PATH)}", "-L", CUDA_LIB, "-lcudart",
                        f"-Wl,-rpath,{CUDA_LIB}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sc = scenes.make_scene(45, 33, 3, 10.0, seed=17)
    l8 = np.round(sc.left[..., :3] * 255).astype(np.int64)
    r16 = np.round(sc.right * 65535).astype(np.int64)
    (tmp_path / "l.png").write_bytes(pngtool.encode(l8, 2, 8, interlace=True))
    (tmp_path / "r.png").write_bytes(pngtool.encode(r16, 6, 16))
    out = tmp_path / "d.png"
    r = subprocess.run([exe, "--files", "5", "10", "2", str(tmp_path / "l.png"), str(tmp_path / "r.png"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got, ct, dp = pngtool.decode(out.read_bytes())
    assert (ct, dp) == (0, 8)
    lu8 = np.concatenate([l8, np.full(l8.shape[:2] + (1,), 255)], -1).astype(np.uint8)
    want, _ = oracle.depthmap(default_params(PRESET_REFERENCE, patchsize=5, depthmax=10.0, iterations=2),
                              oracle.image_to_rgbaf(lu8, imageio.RGBA_UINT8),
                              oracle.image_to_rgbaf(r16.astype(np.uint16), imageio.RGBA_UINT16))
    L = _lib.lib()
    want8 = np.array([L.cvtpm_float_to_srgb_u8(float(v)) for v in want.reshape(-1)]).reshape(want.shape)
    assert np.array_equal(got[..., 0], want8)
