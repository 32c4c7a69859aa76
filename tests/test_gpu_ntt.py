"""Fr NTT / coset LDE on the GPU through the C ABI, bit-exact against the
oracle (reference semantics: natural order, inverse includes 1/n, ZETA
coset with period-3 distribution)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _zeta_pair(orc):
    z = orc.fr_const(orc.CONST_ZETA)
    return z, orc.fr_mul(z, z)


@pytest.mark.parametrize("log_n", [0, 1, 2, 3, 4, 5, 9, 10, 11, 12, 16])
def test_ntt_forward_inverse(gb, orc, log_n):
    n = 1 << log_n
    rng = np.random.default_rng(log_n)
    v = orc.fr_random(n, rng)
    f = gb.bls12_381_fr_ntt(v, inverse=False)
    assert (f == orc.fr_ntt(v, log_n, False)).all()
    i = gb.bls12_381_fr_ntt(v, inverse=True)
    assert (i == orc.fr_ntt(v, log_n, True)).all()
    assert (gb.bls12_381_fr_ntt(f, inverse=True) == v).all()


def test_ntt_reference_sequence(gb, orc):
    # midnight-sppark-msm/src/lib.rs:4714-4740 input (13i + 7) mod 65521
    for ln in (1024, 4096):
        v = orc.fr_from_ints([(i * 13 + 7) % 65521 for i in range(ln)])
        one = orc.fr_const(orc.CONST_ONE)
        host = gb.bls12_381_fr_ntt_zeta(v, False, one, one, one)
        dv = gb.Bls12_381FrDeviceVec.upload(v)
        dv.ntt_zeta(ln.bit_length() - 1, False, one, one, one)
        assert (dv.download() == host).all()
        assert (host == orc.fr_ntt(v, ln.bit_length() - 1, False)).all()


def test_ntt_2p20_against_oracle(gb, orc):
    log_n = 20
    rng = np.random.default_rng(20)
    v = orc.fr_random(1 << log_n, rng)
    f = gb.bls12_381_fr_ntt(v, inverse=False)
    assert (f == orc.fr_ntt(v, log_n, False)).all()
    assert (gb.bls12_381_fr_ntt(f, inverse=True) == v).all()


def test_ntt_zeta_and_divide(gb, orc):
    log_n = 12
    n = 1 << log_n
    rng = np.random.default_rng(3)
    v = orc.fr_random(n, rng)
    z1, z2 = _zeta_pair(orc)
    scale = orc.fr_from_ints([5])[0]
    for inverse in (False, True):
        got = gb.bls12_381_fr_ntt_zeta(v, inverse, scale, z1, z2)
        assert (got == orc.fr_ntt_zeta(v, log_n, inverse, scale, z1, z2)).all()
    t = orc.domain_t_evaluations(4, 10)  # 4 factors, period 4
    got = gb.bls12_381_fr_divide_ntt_zeta(v, t, scale, z2, z1)
    assert (got == orc.fr_divide_ntt_zeta(v, log_n, t, scale, z2, z1)).all()
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.divide_ntt_zeta(log_n, t, scale, z2, z1)
    assert (dv.download() == got).all()


@pytest.mark.parametrize("input_len,count,ext_log_n", [(1024, 1, 12), (1024, 3, 12), (100, 2, 9), (4096, 4, 14)])
def test_coeff_to_extended(gb, orc, input_len, count, ext_log_n):
    # reference test shape lib.rs:4749-4783: (29i + 43c + 11) mod 65521, first 17, second 23
    inp = orc.fr_from_ints([(i * 29 + count * 43 + 11) % 65521 for i in range(input_len * count)])
    first, second = orc.fr_from_ints([17])[0], orc.fr_from_ints([23])[0]
    want = orc.fr_coeff_to_extended_batch(inp, input_len, count, ext_log_n, first, second)
    got = gb.bls12_381_fr_coeff_to_extended_batch(inp.reshape(count, input_len, 4), ext_log_n, first, second)
    assert (got.reshape(-1, 4) == want).all()
    dv = gb.bls12_381_fr_device_coeff_to_extended_batch(inp.reshape(count, input_len, 4), ext_log_n, first, second)
    assert (dv.download() == want).all()


def test_lde_round_trip_with_zeta(gb, orc):
    """coeff -> extended coset -> back (extended_to_coeff semantics)."""
    k, ek = 10, 12
    rng = np.random.default_rng(12)
    coeffs = orc.fr_random(1 << k, rng)
    z1, z2 = _zeta_pair(orc)
    ext = gb.bls12_381_fr_coeff_to_extended_batch(coeffs[None], ek, z1, z2)[0]
    one = orc.fr_const(orc.CONST_ONE)
    back = gb.bls12_381_fr_ntt_zeta(ext, True, one, z2, z1)
    assert (back[: 1 << k] == coeffs).all()
    assert (back[1 << k:] == 0).all()


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5])
def test_ntt_variants(gb, orc, variant):
    """Every pass variant, bit-exact: single transforms at sizes whose pass
    splits differ (one pass, 5+5, 6+5, 8+8, 7+7+7 ...) and a batch of 3 (the
    staged passes pack several sub-blocks, and several transforms, per CTA)."""
    gb.ntt_variant_set(variant)
    try:
        for log_n, count in ((3, 1), (7, 3), (10, 2), (11, 1), (13, 3), (16, 2), (21, 1)):
            rng = np.random.default_rng(100 * variant + log_n)
            v = orc.fr_random(count << log_n, rng)
            one = orc.fr_const(orc.CONST_ONE)
            for inverse in (False, True):
                dv = gb.Bls12_381FrDeviceVec.upload(v)
                dv.ntt_zeta_batch(log_n, count, inverse, one, one, one)
                got = dv.download()
                for p in range(count):
                    seg = v[p << log_n:(p + 1) << log_n]
                    assert (got[p << log_n:(p + 1) << log_n] == orc.fr_ntt(seg, log_n, inverse)).all(), (log_n, p)
        assert gb.ntt_wait_timeouts() == 0
    finally:
        gb.ntt_variant_set(0)


def test_device_vec_batch_ntt(gb, orc):
    log_n, count = 10, 5
    rng = np.random.default_rng(33)
    v = orc.fr_random(count << log_n, rng)
    z1, z2 = _zeta_pair(orc)
    scale = orc.fr_from_ints([3])[0]
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_zeta_batch(log_n, count, True, scale, z1, z2)
    got = dv.download()
    for p in range(count):
        seg = v[p << log_n:(p + 1) << log_n]
        assert (got[p << log_n:(p + 1) << log_n] == orc.fr_ntt_zeta(seg, log_n, True, scale, z1, z2)).all()
