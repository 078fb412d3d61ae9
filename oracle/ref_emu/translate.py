"""TEST INFRASTRUCTURE: mechanical rewrite of the reference's OpenCL C kernel
sources into C++ that compiles against clemu.h.

It changes spelling only, never arithmetic:
  * comments are dropped;
  * `#import "X.cl"` or `#import "../X.cl"` (the reference's textual
    include, util/glcltoheader.cpp) becomes `#include "X.inc"`;
  * vector literals `(float4)( a, b, ... )` become `float4{ a, b, ... }`
    (brace initialisation: components evaluated left to right);
  * swizzles `.xy .xyz .lo .hi` and `.s0` ... `.s7`, `.s01`, `.s0123` ...
    become calls `.xy()` ... (proxy objects or accessors of the vector type);
  * `local T x[..]` declared in a kernel body becomes
    `static thread_local T x[..]`, shared by the work-items of a group
    (clemu runs one group at a time per thread).
It also lists the kernels each file defines and whether they call barrier().
"""
from __future__ import annotations

import re

VEC = r"(?:float[2348]|int[234]|uint[234])"


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def _matching(src: str, i: int, open_ch: str = "(", close_ch: str = ")") -> int:
    depth = 0
    for j in range(i, len(src)):
        if src[j] == open_ch:
            depth += 1
        elif src[j] == close_ch:
            depth -= 1
            if depth == 0:
                return j
    raise ValueError(f"unbalanced {open_ch} at {i}")


def vector_literals(src: str) -> str:
    pat = re.compile(r"\(\s*(" + VEC + r")\s*\)\s*\(")
    while True:
        m = pat.search(src)
        if not m:
            return src
        open_i = m.end() - 1
        close_i = _matching(src, open_i)
        src = src[:m.start()] + m.group(1) + "{" + src[open_i + 1:close_i] + "}" + src[close_i + 1:]


def translate(src: str) -> str:
    src = strip_comments(src)
    src = re.sub(r'#import\s+"(?:\.\./)?(\w+)\.cl"', r'#include "\1.inc"', src)
    src = vector_literals(src)
    src = re.sub(r"\.(xyz|xy|yz|zw|lo|hi)\b(?!\s*\()", r".\1()", src)
    src = re.sub(r"\.(s[0-7]{1,4})\b(?!\s*\()", r".\1()", src)
    src = re.sub(r"(?m)^(\s*)local\s+", r"\1static thread_local ", src)
    return src


def kernels(translated: str):
    """[(name, uses_barrier)] for every kernel the source defines."""
    out = []
    for m in re.finditer(r"(?:__kernel|\bkernel)\s+void\s+(\w+)\s*\(", translated):
        close = _matching(translated, m.end() - 1)
        body_open = translated.index("{", close)
        body_close = _matching(translated, body_open, "{", "}")
        out.append((m.group(1), "barrier(" in translated[body_open:body_close].replace(" ", "")))
    return out
