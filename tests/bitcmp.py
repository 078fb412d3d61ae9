"""Bit-level comparison of float outputs.

Float32 results are compared as their uint32 bit patterns, except that every
NaN counts as one value: the payload and sign of a NaN produced by an
invalid operation are chosen by the hardware (x86, Arm and the GPU each have
their own default NaN), so they carry no result."""
import numpy as np

CANONICAL_NAN = np.uint32(0x7FC00000)


def float_bits(a):
    a = np.ascontiguousarray(a)
    if a.dtype != np.float32:
        return a
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = CANONICAL_NAN
    return b


def bit_diff(got, want):
    """Boolean mask of elements whose bits differ (NaN == NaN)."""
    return float_bits(got) != float_bits(want)
