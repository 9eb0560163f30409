"""Accuracy of the library's own arithmetic (bm_scalar.h) on the GPU.

The substep evaluates its logarithm, exponential, sine, cosine, arctangent,
3x3 SVD and polar decomposition with its own code (the oracle compiles the
same source, which is why the two agree bit for bit).  These tests measure
that code on the device against references that share nothing with it:

* float64 numpy values (glibc's libm) for the elementary functions, in units
  in the last place of the result's type, over dense sweeps;
* CUDA's own functions on the same arguments (bm_math_probe_*), which must
  stay within their documented maximum errors (CUDA C++ Programming Guide,
  mathematical functions appendix: logf 1 ulp, expf 2 ulp, expm1f 1 ulp;
  sin, cos, atan2 in double 2 ulp), so that both are measured with one ruler;
* numpy's float64 SVD for the decompositions, on near-identity, rotated and
  stretched, and moderately ill-conditioned matrices.

The bounds asserted are the ones the library's functions meet, stated in
each test; the reference's Warp builtins (material.py:111,418,515,565,588)
are float32 and promise no tighter bound.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from blademaster_gb300 import _native

    return _native, _native.lib()


def probe_f(kind, x):
    import torch

    native, lib = _lib()
    xs = torch.as_tensor(np.ascontiguousarray(x, np.float32), device="cuda")
    out = torch.empty(2 * len(x), dtype=torch.float32, device="cuda")
    native.check(lib.bm_math_probe_f(kind, ctypes.c_void_p(xs.data_ptr()), len(x), ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    pair = out.cpu().numpy().reshape(-1, 2)
    return pair[:, 0], pair[:, 1]


def probe_d(kind, x, y=None):
    import torch

    native, lib = _lib()
    xs = torch.as_tensor(np.ascontiguousarray(x, np.float64), device="cuda")
    ys = torch.as_tensor(np.ascontiguousarray(y if y is not None else x, np.float64), device="cuda")
    out = torch.empty(2 * len(x), dtype=torch.float64, device="cuda")
    native.check(lib.bm_math_probe_d(kind, ctypes.c_void_p(xs.data_ptr()), ctypes.c_void_p(ys.data_ptr()), len(x),
                                     ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    pair = out.cpu().numpy().reshape(-1, 2)
    return pair[:, 0], pair[:, 1]


def ulps32(value, exact):
    """|value - exact| in units of the last place of float32 at exact."""
    exact32 = np.abs(exact).astype(np.float32)
    unit = np.spacing(exact32).astype(np.float64)
    return np.abs(value.astype(np.float64) - exact) / unit


def ulps64(value, exact):
    return np.abs(value - exact) / np.spacing(np.abs(exact))


def float_sweep(rng, lo_exp, hi_exp, count):
    """Random float32 values with exponents in [lo_exp, hi_exp], plus every 16th float of [0.5, 2)."""
    mant = rng.integers(0, 1 << 23, count, dtype=np.uint32)
    exp = rng.integers(lo_exp + 127, hi_exp + 127 + 1, count).astype(np.uint32)
    random = ((exp << 23) | mant).view(np.float32)
    dense = np.arange(np.float32(0.5).view(np.uint32), np.float32(2.0).view(np.uint32), 16,
                      dtype=np.uint32).view(np.float32)
    return np.concatenate([random, dense])


def test_logf_within_two_and_a_half_ulp():
    rng = np.random.default_rng(1)
    x = float_sweep(rng, -126, 127, 1 << 21)
    ours, cuda = probe_f(0, x)
    exact = np.log(x.astype(np.float64))
    assert ulps32(cuda, exact).max() <= 1.0 + 1e-6  # CUDA's documented bound
    assert ulps32(ours, exact).max() <= 2.5  # atanh series of (m - 1) / (m + 1): 2.48 ulp measured
    special = np.array([0.0, -1.0, np.inf, np.nan, 1.0, 1.0e-45], np.float32)
    ours, _ = probe_f(0, special)
    assert ours[0] == -np.inf and np.isnan(ours[1]) and ours[2] == np.inf and np.isnan(ours[3]) and ours[4] == 0.0
    tiny = float(np.float32(1.0e-45))  # the smallest subnormal, 2^-149
    assert abs(ours[5] - np.log(tiny)) <= 2.5 * float(np.spacing(np.float32(-np.log(tiny))))  # subnormal input


def test_expf_within_two_ulp():
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-87.0, 88.0, 1 << 21), rng.uniform(-1.0, 1.0, 1 << 20)]).astype(np.float32)
    ours, cuda = probe_f(1, x)
    exact = np.exp(x.astype(np.float64))
    assert ulps32(cuda, exact).max() <= 2.0 + 1e-6
    assert ulps32(ours, exact).max() <= 2.0
    ours, _ = probe_f(1, np.array([100.0, -200.0, np.nan, 0.0], np.float32))
    assert ours[0] == np.inf and ours[1] == 0.0 and np.isnan(ours[2]) and ours[3] == 1.0


def test_expm1f_matches_the_reference_rule():
    # material.expm1 (material.py:478-482): a cubic series below |x| = 1e-3, exp(x) - 1 above it,
    # so above the threshold the error is that of exp near 1 (absolute, in ulp of exp(x))
    rng = np.random.default_rng(3)
    small = rng.uniform(-1.0e-3, 1.0e-3, 1 << 20).astype(np.float32)
    large = np.concatenate([rng.uniform(-20.0, 20.0, 1 << 20), rng.uniform(-0.1, 0.1, 1 << 20)]).astype(np.float32)
    large = large[np.abs(large) >= 1.0e-3]
    ours, cuda = probe_f(2, small)
    exact = np.expm1(small.astype(np.float64))
    assert ulps32(cuda, exact).max() <= 1.0 + 1e-6
    assert (np.abs(ours - exact) / np.abs(exact)).max() <= 2.0e-7
    ours, _ = probe_f(2, large)
    exact = np.expm1(large.astype(np.float64))
    unit = np.spacing(np.maximum(np.exp(large), 1.0).astype(np.float32))  # ulp of exp(x), at least of 1
    assert (np.abs(ours - exact) / unit).max() <= 2.5


def test_sin_cos_float64_within_one_and_a_half_ulp():
    # |x| <= 4: relative error, away from the functions' zeros (|f| > 0.1); up to
    # |x| = 1e5: absolute error (the reduction modulo pi/2 keeps it at one ulp of 1)
    rng = np.random.default_rng(4)
    near = rng.uniform(-4.0, 4.0, 1 << 21)
    wide = np.concatenate([rng.uniform(-1.0e5, 1.0e5, 1 << 20), rng.uniform(-1.0e-3, 1.0e-3, 1 << 16)])
    for kind, fn in ((0, np.sin), (1, np.cos)):
        ours, cuda = probe_d(kind, near)
        exact = fn(near)
        away = np.abs(exact) > 0.1
        assert ulps64(cuda[away], exact[away]).max() <= 2.5  # CUDA's 2 ulp plus libm's half ulp
        assert ulps64(ours[away], exact[away]).max() <= 1.5
        ours, cuda = probe_d(kind, wide)
        exact = fn(wide)
        assert np.abs(ours - exact).max() <= 2.3e-16
        assert np.abs(cuda - exact).max() <= 4.5e-16


def test_atan2_float64_within_three_ulp_and_ieee_cases():
    rng = np.random.default_rng(5)
    scale = 10.0 ** rng.uniform(-6, 6, (2, 1 << 20))
    y, x = rng.normal(size=(2, 1 << 20)) * scale
    ours, cuda = probe_d(2, x, y)
    exact = np.arctan2(y, x)
    assert ulps64(cuda, exact).max() <= 3.0
    assert ulps64(ours, exact).max() <= 3.0  # octant reduction and a Taylor series: 3.0 ulp measured
    inf = np.inf
    ys = np.array([0.0, -0.0, 0.0, -0.0, 1.0, -1.0, inf, -inf, inf, 1.0, np.nan])
    xs = np.array([0.0, 0.0, -0.0, -0.0, 0.0, -0.0, inf, -inf, 1.0, -inf, 1.0])
    ours, _ = probe_d(2, xs, ys)
    expected = np.arctan2(ys, xs)
    np.testing.assert_array_equal(ours, expected)
    np.testing.assert_array_equal(np.signbit(ours[:10]), np.signbit(expected[:10]))


def _random_rotations(rng, count):
    q = rng.normal(size=(count, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


@pytest.mark.parametrize("family", ["near_identity", "rotated_stretch", "conditioned_100"])
def test_svd_and_polar_against_float64(family):
    import torch

    native, lib = _lib()
    rng = np.random.default_rng(6)
    count = 1 << 16
    if family == "near_identity":
        A = np.eye(3) + 0.05 * rng.normal(size=(count, 3, 3))
    elif family == "rotated_stretch":
        sigma = rng.uniform(0.5, 2.0, (count, 3))
        A = _random_rotations(rng, count) @ (sigma[:, :, None] * _random_rotations(rng, count))
    else:
        sigma = np.stack([np.ones(count), 10.0 ** rng.uniform(-1, 0, count), np.full(count, 0.01)], 1)
        A = _random_rotations(rng, count) @ (sigma[:, :, None] * _random_rotations(rng, count))
    # five cyclic Jacobi sweeps on A^T A, then a Givens QR: below 1e-6 relative to sigma_max in all
    # three families (8.4e-7 worst measured), a few float32 roundings
    bound = 1.5e-6
    A = A.astype(np.float32)
    dev = {k: torch.empty(count * w, dtype=torch.float32, device="cuda") for k, w in
           (("U", 9), ("s", 3), ("V", 9), ("R", 9))}
    a_dev = torch.as_tensor(A.reshape(-1), device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    native.check(lib.bm_svd_probe(p(a_dev), count, p(dev["U"]), p(dev["s"]), p(dev["V"]), p(dev["R"]),
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    U, s, V, R = (dev[k].cpu().numpy().astype(np.float64) for k in ("U", "s", "V", "R"))
    U, V, R, s = U.reshape(-1, 3, 3), V.reshape(-1, 3, 3), R.reshape(-1, 3, 3), s.reshape(-1, 3)
    A64 = A.astype(np.float64)
    scale = np.linalg.norm(A64, axis=(1, 2))
    eye = np.eye(3)
    # rotations, a faithful factorisation, singular values in decreasing order
    assert np.abs(U @ U.transpose(0, 2, 1) - eye).max() <= bound
    assert np.abs(V @ V.transpose(0, 2, 1) - eye).max() <= bound
    assert np.all(np.linalg.det(U) > 0) and np.all(np.linalg.det(V) > 0)
    rebuilt = U @ (s[:, :, None] * V.transpose(0, 2, 1))
    assert (np.linalg.norm(rebuilt - A64, axis=(1, 2)) / scale).max() <= bound
    exact = np.linalg.svd(A64, compute_uv=False)
    signed = exact * np.where(np.linalg.det(A64) < 0, -1.0, 1.0)[:, None] ** np.array([0, 0, 1])
    assert (np.abs(s - signed).max(axis=1) / exact[:, 0]).max() <= bound
    # polar rotation against U V^T of the float64 SVD (det A > 0 in these families)
    u64, _, vt64 = np.linalg.svd(A64)
    polar = u64 @ vt64
    assert np.all(np.linalg.det(A64) > 0)
    assert np.abs(R - polar).max() <= 2.0e-6
