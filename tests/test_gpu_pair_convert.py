"""FP64 <-> float-float conversions (gfgpu_pairs_from_f64 / gfgpu_pairs_to_f64, the device
functions every pair path uses) against numpy's IEEE casts, bit for bit: h = rn_f32(x),
l = rn_f32(x - h) (x - h exact in FP64) and x' = rn_f64(h + l), on the integer pipe. Exact for zeros
and 2^-74 <= |x| < 2^127 (rounding ties to even, carries into the exponent); below 2^-74 the low
part is 0 and below 2^-126 the pair is +-0. The inputs cover all of these, signed zeros, exact
ties and significands of all ones."""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _inputs():
    rng = np.random.default_rng(7)
    n = 1 << 18
    # log-uniform magnitudes over 2^-140 .. 2^126, random signs
    x = np.exp2(rng.uniform(-140.0, 126.0, n)) * rng.choice([-1.0, 1.0], n)
    # exact ties: a random float significand plus exactly half an FP32 ulp (r = 2^28)
    e = rng.integers(949, 1150, 4096).astype(np.uint64)
    top = rng.integers(0, 1 << 23, 4096).astype(np.uint64)
    bits = (e << np.uint64(52)) | (top << np.uint64(29)) | np.uint64(1 << 28)
    ties = bits.view(np.float64) * rng.choice([-1.0, 1.0], 4096)
    # significand all ones below the FP32 part (rounds up into the next binade)
    ones = ((e << np.uint64(52)) | np.uint64((1 << 52) - 1)).view(np.float64)
    exact = rng.uniform(-1, 1, 4096).astype(np.float32).astype(np.float64)  # l = 0
    special = np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -74, -(2.0 ** -74), 2.0 ** -75, 2.0 ** 126,
                        np.nextafter(2.0 ** 127, 0), 3.0e38, 1e-3, -7.25e-9])
    return np.concatenate([x, ties, ones, exact, special])


def test_pair_conversions_match_ieee_casts():
    from goosefem_gb300 import _dev, _lib

    x = _inputs()
    h = x.astype(np.float32)
    l = (x - h.astype(np.float64)).astype(np.float32)
    xd = torch.as_tensor(x, device="cuda")
    out = torch.empty(2 * x.size, dtype=torch.float32, device="cuda")
    _lib.call("gfgpu_pairs_from_f64", xd.data_ptr(), x.size, out.data_ptr(), _dev.stream())
    got = out.cpu().numpy().reshape(-1, 2)
    ax = np.abs(x)
    exact = (ax == 0) | ((ax >= 2.0 ** -74) & (ax < 2.0 ** 127))
    assert exact.sum() > 0.7 * x.size
    assert np.array_equal(got[exact, 0].view(np.uint32), h[exact].view(np.uint32))
    assert np.array_equal(got[exact, 1].view(np.uint32), l[exact].view(np.uint32))
    # below 2^-74: h = rn(x), l = 0; below 2^-126: h = +-0
    tiny = (ax > 0) & (ax < 2.0 ** -74)
    normal_h = tiny & (ax >= 2.0 ** -126)
    assert np.array_equal(got[normal_h, 0].view(np.uint32), h[normal_h].view(np.uint32))
    assert np.all(got[tiny, 1] == 0)
    sub = tiny & (ax < 2.0 ** -126)
    assert np.all(got[sub, 0] == 0) and np.array_equal(np.signbit(got[sub, 0]), np.signbit(x[sub]))
    # back to FP64: rn(h + l) of the exactly converted parts, bit for bit
    back = torch.empty_like(xd)
    _lib.call("gfgpu_pairs_to_f64", out.data_ptr(), x.size, back.data_ptr(), _dev.stream())
    ref = got[:, 0].astype(np.float64) + got[:, 1].astype(np.float64)
    assert np.array_equal(back.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    # inside the FP32 range the pair holds x to ~2^-48 relative
    m = (ax > 1e-20) & (ax < 1e37)
    assert np.max(np.abs(back.cpu().numpy()[m] - x[m]) / ax[m]) < 2.0 ** -46
