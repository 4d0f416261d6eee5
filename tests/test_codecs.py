"""DDF storage codecs of the oracle: IEEE binary16 conversion (FP16S) against numpy's
round-to-nearest-even float16, and the FP16C format's documented range and precision."""
import numpy as np

import oracle


def _floats(n=200000, seed=0):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    x = x[np.isfinite(x)]
    special = np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e-8, 2.0 ** -24, 2.0 ** -25, 3 * 2.0 ** -26, 6.1e-5,
                        2.0 ** -14, 0.5, 1.0, -1.0, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11], np.float32)
    scaled = (rng.normal(0.0, 1.0, n) * 10.0 ** rng.uniform(-9, 5, n)).astype(np.float32)
    return np.concatenate([x, special, -special, scaled])


def test_fp16s_encode_matches_ieee_rne():
    L = oracle.lib()
    x = _floats()
    ref = (x * np.float32(32768.0)).astype(np.float16).view(np.uint16)
    got = np.array([L.oracle_fp16s_encode(float(v)) for v in x[:20000]], np.uint16)
    assert np.array_equal(got, ref[:20000])


def test_fp16s_decode_exact_for_all_halves():
    L = oracle.lib()
    h = np.arange(0, 65536, dtype=np.uint32).astype(np.uint16)
    finite = np.isfinite(h.view(np.float16))
    ref = h.view(np.float16).astype(np.float32) * np.float32(3.0517578e-5)
    got = np.array([L.oracle_fp16s_decode(int(v)) for v in h], np.float32)
    assert np.array_equal(got[finite], ref[finite])


def test_fp16c_roundtrip_precision_and_range():
    """1-4-11 format: 12 significant bits over +-[6.1e-5, 2) (relative step <= 2^-11), denormals to 3e-8."""
    L = oracle.lib()
    rng = np.random.default_rng(1)
    x = (rng.uniform(-1.99, 1.99, 5000)).astype(np.float32)
    dec = np.array([L.oracle_fp16c_decode(L.oracle_fp16c_encode(float(v))) for v in x], np.float32)
    big = np.abs(x) > 6.2e-5
    assert np.all(np.abs(dec[big] - x[big]) <= np.abs(x[big]) * 2.0 ** -12 * 1.0001)
    # every code decodes to a value that re-encodes to itself (idempotent on the representable set)
    codes = np.arange(0, 65536, dtype=np.uint32)
    vals = np.array([L.oracle_fp16c_decode(int(c)) for c in codes[::7]], np.float32)
    back = np.array([L.oracle_fp16c_decode(L.oracle_fp16c_encode(float(v))) for v in vals], np.float32)
    assert np.array_equal(vals, back)
