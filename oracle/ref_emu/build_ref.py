"""TEST INFRASTRUCTURE — build recipe of the emulated reference
(oracle/_ref/libpmref.so).  Needs the reference sources (it reads them where
they lie, in the directory named by the CVT_REFERENCE environment variable,
by default /root/reference, and copies none into the repository), so it
runs only where they are present.

  1. translate.py rewrites cvt/cl/kernel/{pmhstereo,RNG,PDHuberWeighted,
     PDHuberWeightedInpaint,fill,Matrix4,TSDFVolume/TSDFVolume}.cl and the
     kernels of cvt::StereoGCVFilter (gradx, prefixsum/*, boxfilter/*,
     guidedfilter/*, stereogcv/*)
     into _build/ref_gen/*.inc (generated, never committed);
  2. one C++ unit per kernel file wraps its .inc in a namespace and registers
     the kernels with clemu;
  3. g++ compiles those, the runtime, the harness and the reference's own
     cvt/vision/PMHuberStereo.cpp (which includes the reference's
     PMHuberStereo.h, PDROF.h and PDROFInpaint.h) against the shims in
     oracle/ref_emu/shim.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
REF = os.environ.get("CVT_REFERENCE", "/root/reference")
GEN = os.path.join(ROOT, "_build", "ref_gen")
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libpmref.so")
KERNEL_FILES = ["RNG", "Matrix4", "pmhstereo", "PDHuberWeighted", "PDHuberWeightedInpaint", "fill",
                "TSDFVolume/TSDFVolume", "gradx", "prefixsum/prefixsum_pblock", "prefixsum/prefixsum_pblock_mul2",
                "prefixsum/prefixsum_pblock_outerrgb", "prefixsum/prefixsum_horiz", "prefixsum/prefixsum_vert",
                "prefixsum/prefixsum_block2", "boxfilter/boxfilter_prefixsum",
                "guidedfilter/guidedfilter_calcab_outerrgb", "guidedfilter/guidedfilter_applyab_gc_outer",
                "stereogcv/costdepthgrad", "stereogcv/costmin", "stereogcv/costdepthconv",
                "stereogcv/occlusioncheck"]
INCLUDE_ONLY = ("RNG", "Matrix4")     # #import-ed by other kernel files, no kernels of their own

sys.path.insert(0, HERE)
import translate  # noqa: E402


def available() -> bool:
    return os.path.isfile(os.path.join(REF, "cvt", "cl", "kernel", "pmhstereo.cl"))


def generate():
    os.makedirs(GEN, exist_ok=True)
    units = []
    for path in KERNEL_FILES:
        name = os.path.basename(path)
        src = open(os.path.join(REF, "cvt", "cl", "kernel", path + ".cl")).read()
        tr = translate.translate(src)
        with open(os.path.join(GEN, name + ".inc"), "w") as f:
            f.write(tr)
        if name in INCLUDE_ONLY:
            continue
        ns = "k_" + name
        lines = ['#include "clemu.h"', "namespace clemu { namespace %s {" % ns, '#include "%s.inc"' % name, "}}",
                 "namespace {", "struct Reg { Reg() {"]
        for k, barrier in translate.kernels(tr):
            lines.append('  clemu::reg_kernel("%s", %s, &clemu::%s::%s);' % (k, "true" if barrier else "false", ns, k))
        lines += ["} } reg_;", "}"]
        if name == "pmhstereo":
            lines += ["float clemu::pmh_patch_eval(Img* c1, Img* g1, Img* c2, Img* g2, float cx, float cy,",
                      "                          const float st[4], int patchsize, int lr) {",
                      "  return clemu::k_pmhstereo::patch_eval_color_grad_weighted(c1, g1, c2, g2, clemu::float2(cx, cy),",
                      "      clemu::float4(st[0], st[1], st[2], st[3]), patchsize, lr);",
                      "}"]
        path = os.path.join(GEN, "unit_%s.cpp" % name)
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
        units.append(path)
    return units


def _arch_flags():
    """fmaf() is exact everywhere; on x86-64 hosts with FMA, -mfma makes it an
    instruction instead of a libm call (results are identical)."""
    import platform
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            if " fma " in open("/proc/cpuinfo").read():
                return ["-mfma"]
        except OSError:
            pass
    return []


def build(force: bool = False, verbose: bool = False) -> str | None:
    if not available():
        return None
    srcs = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".cpp", ".h", ".py"))]
    srcs += [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(HERE, "shim")) for f in fs]
    srcs.append(os.path.join(ROOT, "cvt_gb300", "csrc", "pm_math.h"))
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    units = generate()
    base = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
            "-U_FORTIFY_SOURCE", "-D_FORTIFY_SOURCE=0", "-w", *_arch_flags(),
            "-I", os.path.join(HERE, "shim"), "-I", HERE, "-I", GEN, "-I", os.path.join(ROOT, "cvt_gb300", "csrc"),
            "-I", REF]
    jobs = []
    objs = []
    todo = [(u, []) for u in units]
    todo += [(os.path.join(HERE, "clemu_rt.cpp"), []), (os.path.join(HERE, "ref_harness.cpp"), []),
             (os.path.join(REF, "cvt", "vision", "PMHuberStereo.cpp"),
              ["-include", os.path.join(HERE, "shim", "force_include.h")])]
    for src, extra in todo:
        obj = os.path.join(GEN, os.path.basename(src).replace(".cpp", ".o"))
        cmd = base + extra + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        jobs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    bad = []
    for src, p in jobs:
        out, _ = p.communicate()
        if p.returncode:
            print(out, file=sys.stderr)
            bad.append(src)
    if bad:
        raise RuntimeError(f"emulated reference: compile failed for {bad}")
    # -z now: every symbol bound at load.  Lazy binding would resolve symbols
    # from inside the work-item fibers, on several threads at once, which
    # crashed Python processes intermittently.
    subprocess.run(["g++", "-shared", "-fopenmp", "-Wl,-z,now", "-o", LIB + ".tmp", *objs], check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


RECT_LIB = os.path.join(OUT, "libpmref_rect.so")
RECT_SHIM = os.path.join(HERE, "rect_shim")


def build_rect(force: bool = False, verbose: bool = False) -> str | None:
    """oracle/_ref/libpmref_rect.so: the reference's stereo rectification
    (cvt/vision/StereoCameraCalibration.h with cvt/math) and bilinear warps
    (cvt/util/SIMD.cpp) behind rect_harness.cpp.  SIMD.cpp is compiled with
    hidden visibility and linked with --gc-sections, so SIMD::instance() and
    the SSE variants it would construct (other translation units) drop out;
    the harness calls the generic SIMD methods."""
    if not available():
        return None
    own = [os.path.join(HERE, "rect_harness.cpp"), os.path.join(HERE, "rect_stubs.cpp"), __file__]
    own += [os.path.join(dp, f) for dp, _, fs in os.walk(RECT_SHIM) for f in fs]
    if not force and os.path.exists(RECT_LIB) and all(os.path.getmtime(s) <= os.path.getmtime(RECT_LIB) for s in own):
        return RECT_LIB
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(GEN, exist_ok=True)
    base = ["g++", "-std=c++11", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w", "-fvisibility=hidden",
            "-ffunction-sections", "-fdata-sections", "-include", "cstring", "-I", RECT_SHIM, "-I", REF]
    srcs = [os.path.join(HERE, "rect_harness.cpp"), os.path.join(HERE, "rect_stubs.cpp"),
            os.path.join(REF, "cvt", "util", "SIMD.cpp")]
    objs, jobs = [], []
    for src in srcs:
        obj = os.path.join(GEN, "rect_" + os.path.basename(src).replace(".cpp", ".o"))
        cmd = base + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        jobs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    bad = []
    for src, p in jobs:
        out, _ = p.communicate()
        if p.returncode:
            print(out, file=sys.stderr)
            bad.append(src)
    if bad:
        raise RuntimeError(f"rectification harness: compile failed for {bad}")
    subprocess.run(["g++", "-shared", "-Wl,--gc-sections", "-Wl,-z,now", "-o", RECT_LIB + ".tmp", *objs], check=True)
    os.replace(RECT_LIB + ".tmp", RECT_LIB)
    return RECT_LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv))
    print(build_rect(force=True, verbose="-v" in sys.argv))
