"""FP64 <-> float-float conversions (gfgpu_pairs_from_f64 / gfgpu_pairs_to_f64, the device
functions every pair path uses) against numpy's IEEE casts, bit for bit: h = rn_f32(x),
l = rn_f32(x - h) (x - h exact in FP64) and x' = rn_f64(h + l). The device split runs on the integer
pipe for 2^-74 <= |x| < 2^127 (rounding ties to even, carries into the exponent) and on the
conversion instructions elsewhere; the inputs cover both, signed zeros, exact ties and
significands of all ones."""

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
    assert np.array_equal(got[:, 0].view(np.uint32), h.view(np.uint32))
    assert np.array_equal(got[:, 1].view(np.uint32), l.view(np.uint32))
    back = torch.empty_like(xd)
    _lib.call("gfgpu_pairs_to_f64", out.data_ptr(), x.size, back.data_ptr(), _dev.stream())
    ref = h.astype(np.float64) + l.astype(np.float64)
    assert np.array_equal(back.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    # inside the FP32 range the pair holds x to ~2^-48 relative
    m = (np.abs(x) > 1e-20) & (np.abs(x) < 1e37)
    assert np.max(np.abs(ref[m] - x[m]) / np.abs(x[m])) < 2.0 ** -46
