"""The coset forms by the powers of a shift (sppark's coset NTT and LDE,
vendor/sppark-0.1.15/sppark/ntt/ntt.cuh:196-209,283-342, coset generator 7)
on the GPU through the C ABI, bit-exact against the oracle; and the
reporting of an NTT twiddle-copy wait that runs out."""
import numpy as np
import pytest

from conftest import affine_of

pytestmark = pytest.mark.gpu

CUDA_ERROR_LAUNCH_TIMEOUT = 702


def _shift(orc, v):
    return orc.fr_const(orc.CONST_GENERATOR) if v == 7 else orc.fr_from_ints([v])[0]


@pytest.mark.parametrize("input_len,count,ext_log_n", [(1024, 1, 12), (1024, 3, 12), (100, 2, 9), (4096, 4, 14),
                                                       (8, 2, 3), (1 << 11, 1, 11), (5, 1, 6)])
@pytest.mark.parametrize("shift", [7, 123456789])
def test_coeff_to_extended_coset(gb, orc, input_len, count, ext_log_n, shift):
    """coefficients -> evaluations on shift * <w_ext>: host and resident
    entry points, one-pass sizes (prepare kernel) and fused first passes"""
    rng = np.random.default_rng(input_len * 7 + count + ext_log_n)
    inp = orc.fr_random(input_len * count, rng)
    sh = _shift(orc, shift)
    want = orc.fr_coeff_to_extended_coset_batch(inp, input_len, count, ext_log_n, sh)
    got = gb.fr_coeff_to_extended_coset_batch(inp.reshape(count, input_len, 4), ext_log_n, sh)
    assert (got.reshape(-1, 4) == want).all()
    src = gb.Bls12_381FrDeviceVec.upload(inp)
    dv = gb.fr_device_coeff_to_extended_coset_batch(src, input_len, count, ext_log_n, sh)
    assert (dv.download() == want).all()


@pytest.mark.parametrize("variant", [0, 1, 3, 5])
def test_coset_lde_every_variant(gb, orc, variant):
    """the generator coset LDE 2^10 -> 2^12 and 2^12 -> 2^14 under every
    pass variant (4 / 5 fuse the padding and the powers into the first
    pass; 1..3 take the prepare kernel)"""
    gb.ntt_variant_set(variant)
    try:
        g = orc.fr_const(orc.CONST_GENERATOR)
        for k, ek, count in ((10, 12, 2), (12, 14, 1)):
            rng = np.random.default_rng(variant * 100 + k)
            inp = orc.fr_random(count << k, rng)
            want = orc.fr_coeff_to_extended_coset_batch(inp, 1 << k, count, ek, g)
            got = gb.fr_coeff_to_extended_coset_batch(inp.reshape(count, 1 << k, 4), ek, g)
            assert (got.reshape(-1, 4) == want).all(), (k, ek)
    finally:
        gb.ntt_variant_set(0)


@pytest.mark.parametrize("log_n", [0, 1, 3, 9, 10, 11, 16])
def test_ntt_coset_against_oracle(gb, orc, log_n):
    rng = np.random.default_rng(log_n + 500)
    v = orc.fr_random(1 << log_n, rng)
    for shift in (7, 987654321):
        sh = _shift(orc, shift)
        for inverse in (False, True):
            got = gb.fr_ntt_coset(v, inverse, sh)
            assert (got == orc.fr_ntt_coset(v, log_n, inverse, sh)).all(), (shift, inverse)
        assert (gb.fr_ntt_coset(gb.fr_ntt_coset(v, False, sh), True, sh) == v).all()


def test_device_ntt_coset_batch(gb, orc):
    log_n, count = 12, 3
    rng = np.random.default_rng(77)
    v = orc.fr_random(count << log_n, rng)
    g = orc.fr_const(orc.CONST_GENERATOR)
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_coset_batch(log_n, count, False, g)
    fwd = dv.download()
    for p in range(count):
        seg = slice(p << log_n, (p + 1) << log_n)
        assert (fwd[seg] == orc.fr_ntt_coset(v[seg], log_n, False, g)).all()
    dv.ntt_coset_batch(log_n, count, True, g)
    assert (dv.download() == v).all()


@pytest.mark.parametrize("lg,blowup", [(3, 1), (10, 2), (12, 2), (11, 3)])
def test_lde_coset_against_oracle(gb, orc, lg, blowup):
    """sppark NTT::LDE semantics: evaluations -> generator-coset evaluations"""
    v = orc.fr_random(1 << lg, np.random.default_rng(lg * 10 + blowup))
    assert (gb.fr_lde_coset(v, blowup) == orc.fr_lde_coset(v, lg, blowup)).all()


def test_generator_coset_lde_full_size(gb, orc):
    """The NTT + coset LDE configuration's second coset: 16 polynomials of
    2^20 coefficients -> 2^22 evaluations on 7 * <w_ext>, resident, every
    polynomial bit-exact against the oracle; the inverse coset transform
    returns the coefficients followed by zeros."""
    k, ek, count = 20, 22, 16
    rng = np.random.default_rng(2220)
    coeffs = orc.fr_random(count << k, rng)
    g = orc.fr_const(orc.CONST_GENERATOR)
    src = gb.Bls12_381FrDeviceVec.upload(coeffs)
    ext = gb.fr_device_coeff_to_extended_coset_batch(src, 1 << k, count, ek, g)
    got = ext.download()
    for p in range(count):
        want = orc.fr_coeff_to_extended_coset_batch(coeffs[p << k:(p + 1) << k], 1 << k, 1, ek, g)
        assert (got[p << ek:(p + 1) << ek] == want).all(), p
    ext.ntt_coset_batch(ek, count, True, g)
    back = ext.download().reshape(count, 1 << ek, 4)
    assert (back[:, :1 << k].reshape(-1, 4) == coeffs).all()
    assert (back[:, 1 << k:] == 0).all()
    assert gb.ntt_wait_timeouts() == 0


def test_zeta_coeff_to_extended_full_size_fused(gb, orc):
    """The ZETA coset LDE (fused first pass) at 16 x 2^20 -> 2^22 against
    the oracle on two polynomials and by a round trip on all 16."""
    k, ek, count = 20, 22, 16
    rng = np.random.default_rng(2221)
    coeffs = orc.fr_random(count << k, rng)
    z = orc.fr_const(orc.CONST_ZETA)
    z2 = orc.fr_mul(z, z)
    one = orc.fr_const(orc.CONST_ONE)
    dv = gb.bls12_381_fr_device_coeff_to_extended_batch(coeffs.reshape(count, 1 << k, 4), ek, z, z2)
    got = dv.download()
    for p in (0, 15):
        want = orc.fr_coeff_to_extended_batch(coeffs[p << k:(p + 1) << k], 1 << k, 1, ek, z, z2)
        assert (got[p << ek:(p + 1) << ek] == want).all(), p
    dv.ntt_zeta_batch(ek, count, True, one, z2, z)
    back = dv.download().reshape(count, 1 << ek, 4)
    assert (back[:, :1 << k].reshape(-1, 4) == coeffs).all()
    assert (back[:, 1 << k:] == 0).all()


def test_coset_rejects_bad_arguments(gb, orc):
    v = orc.fr_random(64, np.random.default_rng(1))
    with pytest.raises(gb.MsmError):
        gb.fr_coeff_to_extended_coset_batch(v.reshape(1, 64, 4), 5)  # 64 values into 2^5
    with pytest.raises(gb.MsmError):
        gb.fr_ntt_coset(v, False, np.zeros(4, np.uint64))  # zero shift
    src = gb.Bls12_381FrDeviceVec.upload(v)
    with pytest.raises(gb.MsmError):
        gb.fr_device_coeff_to_extended_coset_batch(src, 64, 2, 8)  # source too short


def test_twiddle_wait_timeout_is_reported(gb, orc):
    """A twiddle-copy wait that runs out (the first wait's poll limit set to
    0 by the test hook; the copy still lands in the CTA's second wait) is
    reported as cudaErrorLaunchTimeout by the lane's next synchronising
    call: at once by a host-buffer NTT, and for a resident NTT (which
    returns before its kernels run) by the download of its result.  With
    the default limit again, the next calls are correct."""
    rng = np.random.default_rng(9)
    log_n = 12
    v = orc.fr_random(1 << log_n, rng)
    one = orc.fr_const(orc.CONST_ONE)
    gb.ntt_variant_set(4)
    gb.ntt_wait_timeouts()  # clear
    try:
        gb.ntt_wait_limit_set(0)
        with pytest.raises(gb.MsmError) as e:
            gb.bls12_381_fr_ntt(v)
        assert e.value.code == CUDA_ERROR_LAUNCH_TIMEOUT
        dv = gb.Bls12_381FrDeviceVec.upload(v)
        dv.ntt_zeta(log_n, False, one, one, one)
        with pytest.raises(gb.MsmError) as e:
            dv.download()
        assert e.value.code == CUDA_ERROR_LAUNCH_TIMEOUT
        dv.ntt_ragged([0], [log_n], False, one, one, one)
        assert gb.ntt_wait_timeouts() > 0
    finally:
        gb.ntt_wait_limit_set(None)
        gb.ntt_variant_set(0)
    assert gb.ntt_wait_timeouts() == 0
    assert (gb.bls12_381_fr_ntt(v) == orc.fr_ntt(v, log_n, False)).all()
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_zeta(log_n, False, one, one, one)
    assert (dv.download() == orc.fr_ntt(v, log_n, False)).all()


def test_twiddle_wait_timeout_reported_by_msm_ticket(gb, orc):
    """A resident NTT whose twiddle-copy wait ran out, followed on the same
    lane by an asynchronous context MSM: the ticket's wait is the lane's next
    synchronisation and reports cudaErrorLaunchTimeout instead of points.
    The next ticket, with the default limit again, returns correct points."""
    rng = np.random.default_rng(19)
    log_n = 12
    v = orc.fr_random(1 << log_n, rng)
    one = orc.fr_const(orc.CONST_ONE)
    n = 1000
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    s = orc.fr_random(n, rng)
    ctx = gb.Bls12_381G1MsmContext(b)
    sv = gb.Bls12_381FrDeviceVec.upload(s)
    gb.ntt_variant_set(4)
    gb.ntt_wait_timeouts()  # clear
    try:
        gb.ntt_wait_limit_set(0)
        dv = gb.Bls12_381FrDeviceVec.upload(v)
        dv.ntt_zeta(log_n, False, one, one, one)
        ticket = ctx.device_batch_async(sv, 0, n, 1)
        with pytest.raises(gb.MsmError) as e:
            ticket.wait()
        assert e.value.code == CUDA_ERROR_LAUNCH_TIMEOUT
    finally:
        gb.ntt_wait_limit_set(None)
        gb.ntt_variant_set(0)
    gb.ntt_wait_timeouts()
    got = ctx.device_batch_async(sv, 0, n, 1).wait()
    assert (affine_of(orc, got[0]) == affine_of(orc, orc.g1_msm(b, s))).all()
    ctx.close()
