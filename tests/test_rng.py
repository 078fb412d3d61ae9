"""Random streams: MWC64X as in cvt/cl/kernel/RNG.cl:35-156 and Philox4x32-10."""
import ctypes

import numpy as np

A = 4294883355
M = 18446383549859758079
BASEID = 4077358422479273989


def test_mulmod_matches_bit_serial(oracle):
    rng = np.random.default_rng(3)
    L = oracle.lib()
    for _ in range(2000):
        a, b = (int(v) % M for v in rng.integers(0, 2**63, 2, dtype=np.int64) * 2 + rng.integers(0, 2, 2))
        want = (a * b) % M
        assert L.orc_mwc_mulmod_serial(a, b) == want
        assert L.orc_mwc_mulmod(a, b) == want


def step(x, c):
    xn = (A * x + c) & 0xFFFFFFFF
    carry = 1 if xn < c else 0
    cn = ((A * x) >> 32) + carry
    return xn, cn & 0xFFFFFFFF


def test_skip_ahead_equals_stepping(oracle):
    # RNG_init(linpos, numdraws) = SeedStreams(0,0) then Skip(linpos*numdraws)
    x, c = BASEID // A, BASEID % A
    L = oracle.lib()
    for d in range(0, 300):
        ox, oc = ctypes.c_uint32(), ctypes.c_uint32()
        L.orc_mwc_state(d, ctypes.byref(ox), ctypes.byref(oc))
        assert (ox.value, oc.value) == (x, c), d
        x, c = step(x, c)


def test_mwc_float_stream(oracle):
    out = np.empty(8, np.float32)
    oracle.lib().orc_mwc_stream(45 * 17, 8, out)
    x, c = BASEID // A, BASEID % A
    v = (x * A + c) * pow(A, 45 * 17, M) % M
    x, c = v // A, v % A
    for i in range(8):
        res = x ^ c
        assert out[i] == np.float32(2.3283064365386962890625e-10) * np.float32(res)
        x, c = step(x, c)
    assert ((out >= 0) & (out <= 1)).all()


def test_philox_distinct_streams(oracle):
    a = np.empty(64, np.float32)
    b = np.empty(64, np.float32)
    oracle.lib().orc_philox_stream(1, 10, 0, 0, 64, a)
    oracle.lib().orc_philox_stream(1, 11, 0, 0, 64, b)
    assert not np.array_equal(a, b)
    oracle.lib().orc_philox_stream(1, 10, 0, 0, 64, b)
    assert np.array_equal(a, b)
    big = np.empty(200000, np.float32)
    oracle.lib().orc_philox_stream(7, 3, 1, 0, big.size, big)
    assert abs(big.mean() - 0.5) < 0.005 and ((big >= 0) & (big <= 1)).all()


def test_philox_rounds(oracle):
    # Philox4x32-10 computed from its definition in Python
    def philox(ctr, key):
        c = list(ctr)
        k0, k1 = key
        for _ in range(10):
            p0 = 0xD2511F53 * c[0]
            p1 = 0xCD9E8D57 * c[2]
            c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF,
                 ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF, p0 & 0xFFFFFFFF]
            k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
            k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
        return c
    rng = np.random.default_rng(5)
    for _ in range(50):
        ctr = rng.integers(0, 2**32, 4, dtype=np.uint64).astype(np.uint32)
        key = rng.integers(0, 2**32, 2, dtype=np.uint64).astype(np.uint32)
        out = np.empty(4, np.uint32)
        oracle.lib().orc_philox(ctr, key, out)
        assert list(out) == philox([int(v) for v in ctr], [int(v) for v in key])
