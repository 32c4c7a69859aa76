"""Grand products, batch inversion, vector ops and device vectors on the GPU
through the C ABI, bit-exact against the oracle, with the reference's own
test shapes (midnight-sppark-msm/src/lib.rs:4664-4955, 5495-5545)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ln", [0, 1, 2, 17, 1024, 1025, 4099, 32768])
def test_shifted_prefix_product(gb, orc, ln):
    vals = orc.fr_from_ints([(i % 251) + 2 for i in range(ln)])
    seven = orc.fr_from_ints([7])[0]
    got = gb.bls12_381_fr_shifted_prefix_product(vals, seven)
    if ln:
        assert (got == orc.fr_shifted_prefix_product(vals, seven)).all()


def test_shifted_prefix_product_large_random(gb, orc):
    rng = np.random.default_rng(4)
    v = orc.fr_random((1 << 20) + 3, rng)
    init = orc.fr_random(1, rng)[0]
    assert (gb.bls12_381_fr_shifted_prefix_product(v, init) == orc.fr_shifted_prefix_product(v, init)).all()


@pytest.mark.parametrize("ln,cc", [(1024, 5), (1 << 16, 3), (64, 1)])
def test_permutation_products(gb, orc, ln, cc):
    chunk, bf = 2, 4
    sets = (cc + chunk - 1) // chunk
    log_n = ln.bit_length() - 1
    cols = orc.fr_from_ints([(c * 71 + r * 29 + 5) % 65521 for c in range(cc) for r in range(ln)])
    perms = orc.fr_from_ints([(c * 43 + r * 37 + 101) % 65521 for c in range(cc) for r in range(ln)])
    delta = orc.fr_to_ints(orc.fr_const(orc.CONST_DELTA))[0]
    dp = orc.fr_from_ints([pow(delta, c, orc.R_MOD) for c in range(cc)])
    blinds = orc.fr_from_ints([i * 13 + 211 for i in range(sets * bf)])
    beta, gamma = orc.fr_from_ints([17])[0], orc.fr_from_ints([23])[0]
    omega = orc.fr_omega(log_n)
    want = orc.fr_permutation_products(cols, perms, ln, cc, chunk, beta, gamma, omega, dp, blinds, bf)
    dv = gb.bls12_381_fr_permutation_products(cols, perms, ln, cc, chunk, beta, gamma, omega, dp, blinds, bf)
    assert dv.len == sets * ln
    assert (dv.download() == want).all()
    # then to coefficients on the device (lib.rs:4882-4893)
    one = orc.fr_const(orc.CONST_ONE)
    dv.ntt_zeta_batch(log_n, sets, True, one, one, one)
    got = dv.download()
    for s in range(sets):
        assert (got[s * ln:(s + 1) * ln] == orc.fr_ntt(want[s * ln:(s + 1) * ln], log_n, True)).all()


@pytest.mark.parametrize("ln,lc", [(1024, 4), (1 << 16, 1)])
def test_lookup_products(gb, orc, ln, lc):
    bf = 4
    seq = lambda off: orc.fr_from_ints([(i * 29 + off * 43 + 101) % 65521 for i in range(lc * ln)])  # noqa: E731
    ci, ct, pi, pt = seq(1), seq(2), seq(3), seq(4)
    blinds = orc.fr_from_ints([i * 13 + 211 for i in range(lc * bf)])
    beta, gamma = orc.fr_from_ints([17])[0], orc.fr_from_ints([23])[0]
    want = orc.fr_lookup_products(ci, ct, pi, pt, ln, lc, beta, gamma, blinds, bf)
    got = gb.bls12_381_fr_lookup_products(ci, ct, pi, pt, ln, lc, beta, gamma, blinds, bf)
    assert (got.download() == want).all()
    trace = gb.Bls12_381FrDeviceVec.upload(np.concatenate([ci, ct, pi, pt]))
    got2 = gb.bls12_381_fr_lookup_products_device(trace, ln, lc, beta, gamma, blinds, bf)
    assert (got2.download() == want).all()


def test_invert_assign(gb, orc):
    vals = orc.fr_from_ints([0 if i % 257 == 0 else (i % 251) + 2 for i in range(4099)])
    assert (gb.bls12_381_fr_invert_assign(vals) == orc.fr_batch_invert(vals)).all()
    rng = np.random.default_rng(2)
    v = orc.fr_random(100003, rng)
    v[::1000] = 0
    assert (gb.bls12_381_fr_invert_assign(v) == orc.fr_batch_invert(v)).all()


def test_sort_canonical(gb, orc):
    # lib.rs:5527-5545 shape: a squaring sequence plus 0, 1, -1 and duplicates
    R = orc.R_MOD
    cur = 0x12345678
    ints = []
    for i in range(16387):
        cur = (cur * cur + (i * 0x9E3779B9) % (1 << 64)) % R
        ints.append(cur)
    ints += [0, 1, R - 1, ints[17], ints[17]]
    v = orc.fr_from_ints(ints)
    got = gb.bls12_381_fr_sort_canonical(v)
    assert orc.fr_to_ints(got) == sorted(ints)


def test_vector_ops(gb, orc):
    rng = np.random.default_rng(6)
    v = orc.fr_random(5000, rng)
    k = orc.fr_random(1, rng)[0]
    assert (gb.bls12_381_fr_mul_assign(v, k) == orc.fr_mul_assign(v, k)).all()
    z = orc.fr_const(orc.CONST_ZETA)
    z2 = orc.fr_mul(z, z)
    assert (gb.bls12_381_fr_mul_assign_zeta(v, z, z2) == orc.fr_mul_assign_zeta(v, z, z2)).all()
    f = orc.fr_random(7, rng)
    assert (gb.bls12_381_fr_mul_assign_repeating(v, f) == orc.fr_mul_assign_repeating(v, f)).all()
    # lincomb, lib.rs:4684-4711 shape
    pl, pc = 1000, 5
    polys = orc.fr_from_ints([(p * 17 + i * 31 + 5) % 65521 for p in range(pc) for i in range(pl)])
    ks = orc.fr_from_ints([i * 11 + 3 for i in range(pc)])
    want = orc.fr_poly_lincomb(polys, pl, pc, ks)
    assert (gb.bls12_381_fr_poly_lincomb(polys.reshape(pc, pl, 4), ks) == want).all()
    dv = gb.Bls12_381FrDeviceVec.upload(polys)
    assert (gb.bls12_381_fr_device_poly_lincomb(dv, pl, pc, ks).download() == want).all()


def test_quotient_pieces(gb, orc):
    n, pieces = 1024, 3
    rng = np.random.default_rng(8)
    q = orc.fr_random((n - 1) * pieces + 11, rng)
    bl = orc.fr_random(pieces - 1, rng)
    dq = gb.Bls12_381FrDeviceVec.upload(q)
    got = gb.bls12_381_fr_device_quotient_pieces(dq, n, pieces, bl).download()
    assert (got == orc.fr_quotient_pieces(q, n, pieces, bl)).all()


def test_device_vector_ops(gb, orc):
    rng = np.random.default_rng(10)
    a, b = orc.fr_random(300, rng), orc.fr_random(200, rng)
    da = gb.Bls12_381FrDeviceVec.upload(a)
    assert (da.download() == a).all()
    dm = gb.Bls12_381FrDeviceVec.upload_many([a, b])
    assert (dm.download() == np.concatenate([a, b])).all()
    dc = da.concat_host(b)
    assert (dc.download() == np.concatenate([a, b])).all()
    dcm = gb.Bls12_381FrDeviceVec.concat_many_host([da, dm], b[:5])
    assert (dcm.download() == np.concatenate([a, a, b, b[:5]])).all()
    dg = dm.gather_polys(100, [4, 0, 2])
    full = np.concatenate([a, b])
    assert (dg.download() == np.concatenate([full[400:500], full[0:100], full[200:300]])).all()
    idx = np.array([0, 5, 299], dtype=np.uint32)
    vals = orc.fr_random(3, rng)
    da.scatter_host(idx, vals)
    a2 = a.copy()
    a2[idx] = vals
    assert (da.download() == a2).all()
    with pytest.raises(gb.MsmError):
        da.scatter_host(np.array([300], dtype=np.uint32), vals[:1])
