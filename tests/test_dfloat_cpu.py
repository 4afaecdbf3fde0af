"""The double-float arithmetic of the mixed-precision Davidson subspace
(qdk-chemistry_gb300/csrc/dfloat.cuh), restated step for step in numpy
float32 (IEEE round to nearest, no contraction; an FMA as the float32
rounding of the exact float64 sum), to pin the error bounds the solver
relies on:

* TwoSum returns the exact rounding error of a float32 addition, and the
  FMA TwoProduct the exact error of a float32 product;
* a double-float number built from a double (split) keeps ~48 bits;
* Dot2 accumulation (Ogita, Rump and Oishi 2005) of 2^20 double-float
  products, 4096 lanes of 256 terms each with the lanes summed in FP64 as
  the kernels do, agrees with the exact dot product to 1.1e-15 relative on
  this seed (asserted: 1e-12; a plain FP64 sum is off by 2.2e-16) - far
  below the FP32 sigma's ~1e-7 that enters A V."""
import math

import numpy as np

f32 = np.float32


def fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    e = ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)
    return s, e


def split(x):
    h = x.astype(f32)
    return h, (x - h.astype(np.float64)).astype(f32)


def mac(sx, sy, ax, ay, bx, by):
    p = (ax * bx).astype(f32)
    e = fma(ax, bx, -p)
    e = fma(ax, by, e)
    e = fma(ay, bx, e)
    tx, ty = two_sum(sx, p)
    return tx, (sy + (ty + e).astype(f32)).astype(f32)


def test_error_free_transformations_are_exact():
    rng = np.random.default_rng(5)
    a = (rng.standard_normal(100000) * 10.0 ** rng.integers(-6, 6, 100000)).astype(f32)
    b = (rng.standard_normal(100000) * 10.0 ** rng.integers(-6, 6, 100000)).astype(f32)
    s, e = two_sum(a, b)
    # s + e equals a + b exactly (both sides exact in float64 for float32 inputs)
    assert np.array_equal(s.astype(np.float64) + e.astype(np.float64), a.astype(np.float64) + b.astype(np.float64))
    p = (a * b).astype(f32)
    err = fma(a, b, -p)
    assert np.array_equal(p.astype(np.float64) + err.astype(np.float64), a.astype(np.float64) * b.astype(np.float64))


def test_split_keeps_about_48_bits():
    rng = np.random.default_rng(6)
    x = rng.standard_normal(100000) * 10.0 ** rng.integers(-20, 20, 100000)
    h, lo = split(x)
    rel = np.abs(h.astype(np.float64) + lo.astype(np.float64) - x) / np.abs(x)
    assert rel.max() < 2.0 ** -47


def test_dot2_of_a_davidson_sized_vector():
    rng = np.random.default_rng(7)
    n, lanes = 1 << 20, 4096
    # unit vectors with entries spread over many magnitudes, as CI vectors are
    a = rng.standard_normal(n) * 10.0 ** rng.uniform(-6, 0, n)
    b = a + 1e-3 * rng.standard_normal(n) * np.abs(a)
    a /= np.linalg.norm(a)
    b /= np.linalg.norm(b)
    ax, ay = split(a)
    bx, by = split(b)
    sx = np.zeros(lanes, f32)
    sy = np.zeros(lanes, f32)
    for step in range(n // lanes):
        sl = slice(step * lanes, (step + 1) * lanes)
        sx, sy = mac(sx, sy, ax[sl], ay[sl], bx[sl], by[sl])
    got = float(np.sum(sx.astype(np.float64) + sy.astype(np.float64)))
    # the exact dot of the double-float inputs: every term is a product of two
    # float32 numbers, exact in float64, and fsum rounds their sum correctly
    A = ax.astype(np.float64), ay.astype(np.float64)
    B = bx.astype(np.float64), by.astype(np.float64)
    exact = math.fsum(np.concatenate([A[0] * B[0], A[0] * B[1], A[1] * B[0], A[1] * B[1]]).tolist())
    assert abs(got - exact) <= 1e-12 * abs(exact), (got, exact)
    # and the double-float inputs represent the FP64 vectors to ~48 bits
    assert abs(exact - float(a @ b)) <= 1e-12
