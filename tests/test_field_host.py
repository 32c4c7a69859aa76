"""The device field / curve headers compiled as host code (g++) against the
oracle: Montgomery products, inversion and the XYZZ point formulas incl.
the doubling and opposite-point cases.  No GPU needed."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, REPO, affine_of

BUILD = os.path.join(REPO, "tests", "_build")


@pytest.fixture(scope="module")
def hh():
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "field_host_harness.so")
    src = os.path.join(REPO, "tests", "field_host_harness.cpp")
    hdrs = [os.path.join(PKG, "csrc", f) for f in ("gb_field.cuh", "gb_curve.cuh")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(f) for f in hdrs + [src]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(PKG, "csrc"),
                               "-o", so, src])
    L = ctypes.CDLL(so)
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_fp_fr_mul_inv(hh, orc):
    rng = np.random.default_rng(21)
    P = orc.P_MOD
    for _ in range(200):
        a = int.from_bytes(rng.bytes(48), "little") % P
        b = int.from_bytes(rng.bytes(48), "little") % P
        am, bm = orc.fp_from_int(a), orc.fp_from_int(b)
        out = np.zeros(6, dtype=np.uint64)
        hh.h_fp_mul(_p(out), _p(am), _p(bm))
        assert orc.fp_to_int(out) == a * b % P
        assert (out == orc.fp_from_int(a * b)).all()  # fully reduced, canonical limbs
    a = orc.fp_from_int(123456789)
    out = np.zeros(6, dtype=np.uint64)
    hh.h_fp_inv(_p(out), _p(a))
    assert orc.fp_to_int(out) == pow(123456789, -1, P)
    fa, fb = orc.fr_random(100, rng), orc.fr_random(100, rng)
    for x, y in zip(fa, fb):
        out = np.zeros(4, dtype=np.uint64)
        hh.h_fr_mul(_p(out), _p(x), _p(y))
        assert (out == orc.fr_mul(x, y)).all()
        s, d = np.zeros(4, dtype=np.uint64), np.zeros(4, dtype=np.uint64)
        hh.h_fr_addsub(_p(s), _p(d), _p(x), _p(y))
        xi, yi = orc.fr_to_ints(x)[0], orc.fr_to_ints(y)[0]
        assert orc.fr_to_ints(s)[0] == (xi + yi) % orc.R_MOD
        assert orc.fr_to_ints(d)[0] == (xi - yi) % orc.R_MOD
    # edge values
    rm1 = orc.fr_from_ints([orc.R_MOD - 1])[0]
    out = np.zeros(4, dtype=np.uint64)
    hh.h_fr_mul(_p(out), _p(rm1), _p(rm1))
    assert orc.fr_to_ints(out)[0] == 1


def _sum_check(hh, orc, pts, neg):
    n = len(pts)
    out_a = np.zeros(12, dtype=np.uint64)
    out_j = np.zeros(18, dtype=np.uint64)
    negs = np.ascontiguousarray(neg, dtype=np.uint8)
    hh.h_xyzz_sum(_p(out_a), _p(out_j), _p(np.ascontiguousarray(pts)), _p(negs), n)
    signs = [orc.R_MOD - 1 if x else 1 for x in neg]
    want = affine_of(orc, orc.g1_msm_naive(pts, orc.fr_from_ints(signs)))[0]
    assert (out_a == want).all()
    assert (affine_of(orc, out_j)[0] == want).all()


def test_xyzz_formulas(hh, orc):
    rng = np.random.default_rng(5)
    pts = orc.g1_generator_mul_batch(orc.fr_random(40, rng))
    _sum_check(hh, orc, pts, rng.integers(0, 2, 40))
    # equal points in one accumulator (doubling branch) and opposite points (infinity)
    dup = np.stack([pts[0], pts[1], pts[0], pts[1], pts[0], pts[1]])
    _sum_check(hh, orc, dup, [0, 0, 0, 0, 0, 0])
    _sum_check(hh, orc, dup, [0, 0, 1, 1, 0, 0])
    _sum_check(hh, orc, dup[:4], [0, 0, 1, 1])  # total is infinity
    g = orc.g1_generator()
    for k in (0, 1, 2, 3, 255, 65535, 1 << 20):
        out = np.zeros(12, dtype=np.uint64)
        hh.h_xyzz_mul_small(_p(out), _p(g), k)
        want = affine_of(orc, orc.g1_mul(g, orc.fr_from_ints([k])[0]))[0]
        assert (out == want).all(), k


def test_binary_gcd_inverse(hh, orc):
    """mont_t::inverse_binary (the batch inversion's tile inverse) against
    pow(a, -1) for Fp and Fr, with the edge values 0, 1, 2 and m - 1."""
    rng = np.random.default_rng(22)
    P, R = orc.P_MOD, orc.R_MOD
    for a in [0, 1, 2, P - 1, P - 2, (P + 1) // 2] + [int.from_bytes(rng.bytes(48), "little") % P for _ in range(150)]:
        out = np.zeros(6, dtype=np.uint64)
        hh.h_fp_inv_binary(_p(out), _p(orc.fp_from_int(a)))
        assert orc.fp_to_int(out) == (pow(a, -1, P) if a else 0)
    for a in [0, 1, 2, R - 1, R - 2, (R + 1) // 2] + [int.from_bytes(rng.bytes(32), "little") % R for _ in range(150)]:
        out = np.zeros(4, dtype=np.uint64)
        hh.h_fr_inv_binary(_p(out), _p(orc.fr_from_ints([a])[0]))
        assert orc.fr_to_ints(out)[0] == (pow(a, -1, R) if a else 0)
