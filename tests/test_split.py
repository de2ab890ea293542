"""The FP64 -> BF16-slice split the packing kernels apply before every
tensor-core contraction.

``split_bits`` below emulates, in numpy, the device algorithm step by step
(x taken apart into a truncated FP32 head and a rounded FP32 tail from its bit
pattern, then each FP32 remainder rounded to BF16, nearest even).  The CPU
tests pin its error bounds; the GPU test checks that the device produces the
same bit patterns."""
import ctypes as C

import numpy as np
import pytest


def bf16_rne(f):
    """BF16 bits of float32 values, round to nearest even (finite inputs)."""
    b = np.ascontiguousarray(f, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> np.uint64(16)) & np.uint64(1))) >> np.uint64(16)).astype(np.uint32)


def _f32(bits):
    return np.ascontiguousarray(bits, dtype=np.uint32).view(np.float32)


def split_bits(x, nslices):
    """uint16 array (nslices, n): BF16 bit patterns of the slices of x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    u = x.view(np.uint64)
    sign = (u >> np.uint64(63)).astype(np.uint32)
    E = ((u >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    frac = u & np.uint64(0xFFFFFFFFFFFFF)
    e32 = E - 896
    ok = (e32 > 0) & (e32 < 255)
    hi_bits = (sign << np.uint32(31)) | (np.clip(e32, 0, 255).astype(np.uint32) << np.uint32(23)) | \
        ((u >> np.uint64(29)).astype(np.uint32) & np.uint32(0x7FFFFF))
    hi = _f32(np.where(ok, hi_bits, 0))
    lo_int = np.where(ok, (u & np.uint64(0x1FFFFFFF)).astype(np.uint32), 0).astype(np.uint32)
    es = np.where(ok, E - 948, 1)
    direct = _f32(np.clip(es, 1, 254).astype(np.uint32) << np.uint32(23))
    twostep = _f32(np.clip(es + 64, 1, 254).astype(np.uint32) << np.uint32(23))
    lo = np.where(es >= 1, lo_int.astype(np.float32) * direct,
                  (lo_int.astype(np.float32) * np.float32(2.0 ** -64)) * twostep)
    lo = np.where(sign == 1, -lo, lo).astype(np.float32)
    out = np.zeros((nslices, x.size), dtype=np.uint32)
    b1 = bf16_rne(hi)
    out[0] = b1
    if nslices > 1:
        r = (hi - _f32(b1 << np.uint32(16))) + lo
        b2 = bf16_rne(r)
        out[1] = b2
        if nslices > 2:
            r = r - _f32(b2 << np.uint32(16))
            out[2] = bf16_rne(r)
    out[:, ~ok] = 0
    small = e32 <= 0
    out[0] = np.where(small, sign << np.uint32(15), out[0])
    big = (e32 >= 255) & (E != 0x7FF)
    out[0] = np.where(big, (sign << np.uint32(15)) | 0x7F80, out[0])
    special = E == 0x7FF
    out[0] = np.where(special, (sign << np.uint32(15)) | np.where(frac != 0, 0x7FC0, 0x7F80), out[0])
    return out.astype(np.uint16)


def sign_of(x):
    return (np.ascontiguousarray(x, dtype=np.float64).view(np.uint64) >> np.uint64(63)).astype(np.int64)


def bf16_value(bits):
    return (bits.astype(np.uint32) << np.uint32(16)).view(np.float32).astype(np.float64)


def sample(n=20000, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=n) * 10.0 ** rng.uniform(-30, 30, size=n)
    # exact ties at each slice, carries into the exponent, signs, zeros, range edges
    ties = np.array([1 + 2.0 ** -8, 1 + 3 * 2.0 ** -9, -(1 + 2.0 ** -8), 1 + 2.0 ** -8 + 2.0 ** -17,
                     (2 - 2.0 ** -9), -(2 - 2.0 ** -9), 255.5 / 128, 1 + 2.0 ** -16 + 2.0 ** -25])
    edge = np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -126, 2.0 ** -133, 1e-40, 3e38, 1e-300, 5e-324])
    return np.concatenate([x, ties, ties * 2.0 ** 40, edge])


@pytest.mark.parametrize("nslices,bound", [(1, 2.0 ** -8), (2, 2.0 ** -16), (3, 2.0 ** -24 + 2.0 ** -32)])
def test_split_error_bound(nslices, bound):
    x = sample()
    x = x[(np.abs(x) > 1e-25) & (np.abs(x) < 1e25)]   # slices stay in the BF16 normal range
    b = split_bits(x, nslices)
    approx = sum(bf16_value(b[s]) for s in range(nslices))
    assert np.all(np.abs(x - approx) <= bound * np.abs(x))


def test_split_remainders_are_exact_and_ties_round_to_even():
    x = np.array([1 + 2.0 ** -8, -(1 + 2.0 ** -8), 2 - 2.0 ** -9, 3.0 + 2.0 ** -40, 1 + 3 * 2.0 ** -8])
    b = split_bits(x, 3)
    v = np.stack([bf16_value(b[s]) for s in range(3)])
    assert v[0, 0] == 1.0 and v[1, 0] == 2.0 ** -8                   # tie to even, exact rest
    assert v[0, 1] == -1.0 and v[1, 1] == -(2.0 ** -8)
    assert v[0, 2] == 2.0 and v[1, 2] == -(2.0 ** -9)                 # carry into the exponent
    assert v[0, 3] == 3.0 and v[1, 3] == 2.0 ** -40 and v[2, 3] == 0.0  # the tail below FP32's 24 bits
    assert v[0, 4] == 1 + 2.0 ** -6 and v[1, 4] == -(2.0 ** -8)       # tie to even, upwards
    # three slices keep 24 bits of every value whose slices are all normal
    y = sample(seed=1)
    y = y[(np.abs(y) > 1e-20) & (np.abs(y) < 1e20)]
    bb = split_bits(y, 3)
    assert np.all(np.abs(y - sum(bf16_value(bb[s]) for s in range(3))) <= (2.0 ** -24 + 2.0 ** -32) * np.abs(y))


def test_split_special_values():
    b = split_bits(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-300]), 3)
    assert list(b[0]) == [0x0000, 0x8000, 0x7F80, 0xFF80, 0x7FC0, 0x0000]
    assert not np.any(bf16_value(b[1:]))   # later slices are (signed) zeros


@pytest.mark.gpu
@pytest.mark.parametrize("nslices", [1, 2, 3])
def test_device_split_matches_emulation(gbcc_lib, nslices):
    x = sample(seed=nslices)
    x = np.concatenate([x, [np.inf, -np.inf, np.nan]])
    out = np.zeros(nslices * x.size, dtype=np.uint16)
    st = gbcc_lib.gbcc_testing_split(x.ctypes.data_as(C.c_void_p), x.size, nslices,
                                     out.ctypes.data_as(C.c_void_p))
    assert st == 0
    ref = split_bits(x, nslices)
    got = out.reshape(nslices, x.size)
    bad = np.nonzero(got != ref)
    assert bad[0].size == 0, [(x[i], s, hex(got[s, i]), hex(ref[s, i])) for s, i in zip(*bad)][:5]


def scale_sample(seed=0):
    """Normals of all magnitudes, values at the edges of the normal range,
    subnormals, signed zeros, infinities and NaN."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(4000) * np.exp2(rng.integers(-1070, 1020, 4000))
    edge = [np.finfo(np.float64).tiny, np.finfo(np.float64).tiny * 2, np.finfo(np.float64).max,
            np.finfo(np.float64).max / 2, 5e-324, 1e-310, 2.0 ** -1020, 2.0 ** 1023, 0.0, -0.0,
            np.inf, -np.inf, np.nan, 1.0, -3.0]
    edge = np.array(edge)
    return np.concatenate([x, edge, -edge])


@pytest.mark.gpu
@pytest.mark.parametrize("coef", [1.0, -1.0, 2.0, -2.0, 0.5, -0.5, 4.0, 0.25, 2.0 ** -60, -(2.0 ** 60), 3.0, -0.1])
def test_device_term_scaling_is_the_ieee_product(gbcc_lib, coef):
    """The packing kernels scale a term by +-2^k on the exponent bits (no FP64
    instruction); every value, including those whose product leaves the normal
    range, must come out as the IEEE product."""
    x = scale_sample(seed=int(abs(np.log2(abs(coef)))) + (coef < 0))
    out = np.empty_like(x)
    st = gbcc_lib.gbcc_testing_scale(x.ctypes.data_as(C.c_void_p), x.size, coef, out.ctypes.data_as(C.c_void_p))
    assert st == 0
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        ref = x * coef
    nan = np.isnan(ref)
    bad = np.nonzero((np.isnan(out) != nan) | (~nan & (out.view(np.uint64) != ref.view(np.uint64))))[0]
    assert bad.size == 0, [(hex(x[i:i + 1].view(np.uint64)[0]), hex(out[i:i + 1].view(np.uint64)[0]),
                            hex(ref[i:i + 1].view(np.uint64)[0])) for i in bad[:6]]


def scale_pow2_bits(x, k):
    """Integer transcription of the packing kernels' x * 2^k on the bit
    pattern (fp_bits.cuh: scale_pow2 / scale_pow2_rare): exponent shift for
    normal results, round-to-nearest-even into the subnormals, overflow to
    infinity; zeros, infinities and NaN unchanged."""
    M52 = (1 << 52) - 1
    b = int(np.float64(x).view(np.uint64))
    m, sign = b & ((1 << 63) - 1), b & (1 << 63)
    e = m >> 52
    if m == 0 or e == 0x7FF:
        return np.float64(x)
    if e != 0 and 1 <= e + k <= 0x7FE:
        return np.uint64(b + (k << 52)).view(np.float64)
    s = ((m & M52) | (1 << 52)) if e else m
    q = (e - 1 if e else 0) + k
    lz = (64 - s.bit_length()) - 11
    s <<= lz
    q -= lz
    if q >= 0x7FE:
        r = 0x7FF << 52
    elif q >= 0:
        r = ((q + 1) << 52) | (s & M52)
    else:
        sh = -q
        if sh > 54:
            r = 0
        else:
            lo, rem, half = s >> sh, s & ((1 << sh) - 1), 1 << (sh - 1)
            r = lo + (1 if (rem > half or (rem == half and (lo & 1))) else 0)
    return np.uint64(sign | r).view(np.float64)


@pytest.mark.parametrize("k", [0, 1, -1, 2, -2, 5, -60, 60])
def test_integer_power_of_two_scaling_is_the_ieee_product(k):
    """The algorithm the packing kernels use for power-of-two coefficients
    (checked on the device by test_device_term_scaling_is_the_ieee_product)
    rounds exactly as the IEEE product, across the normal range, into and out
    of the subnormals and up to overflow."""
    x = scale_sample(seed=abs(k) + (k < 0))
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        ref = x * np.float64(2.0) ** k
    got = np.array([scale_pow2_bits(v, k) for v in x])
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint64), ref[~nan].view(np.uint64))
