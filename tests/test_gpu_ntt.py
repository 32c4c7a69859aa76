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


def _ragged_layout(log_ns, rng, gap_max=37):
    """Polynomials at shuffled offsets with gaps between them."""
    order = rng.permutation(len(log_ns))
    offsets = [0] * len(log_ns)
    pos = 0
    for j in order:
        pos += int(rng.integers(0, gap_max))
        offsets[j] = pos
        pos += 1 << log_ns[j]
    return offsets, pos + int(rng.integers(0, gap_max))


@pytest.mark.parametrize("inverse", [False, True])
def test_ntt_ragged_against_oracle(gb, orc, inverse):
    """One persistent launch over transforms of one, two and three passes
    (and 1 to 4 values: a single value stays unchanged as in a single call,
    2 and 4 take the plain path), placed out of order with gaps; every
    transform bit-exact against the oracle, gaps untouched."""
    log_ns = [0, 1, 2, 3, 5, 7, 9, 10, 11, 13, 16, 21, 12, 3, 10]
    rng = np.random.default_rng(71 + inverse)
    offsets, total = _ragged_layout(log_ns, rng)
    v = orc.fr_random(total, rng)
    z1, z2 = _zeta_pair(orc)
    scale = orc.fr_from_ints([9])[0]
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_ragged(offsets, log_ns, inverse, scale, z1, z2)
    got = dv.download()
    covered = np.zeros(total, dtype=bool)
    for off, ln in zip(offsets, log_ns):
        seg = slice(off, off + (1 << ln))
        covered[seg] = True
        assert (got[seg] == orc.fr_ntt_zeta(v[seg], ln, inverse, scale, z1, z2)).all(), ln
    assert (got[~covered] == v[~covered]).all()
    assert gb.ntt_wait_timeouts() == 0


def test_ntt_ragged_batch_shape(gb, orc):
    """64 transforms with the batched configuration's size distribution
    (next powers of two of round(2^U), U uniform in [10, 18]): equal to one
    call per transform, and the inverse restores the input."""
    rng = np.random.default_rng(64)
    log_ns = [max(1, (int(round(2 ** u)) - 1).bit_length()) for u in rng.uniform(10, 18, size=64)]
    offsets, total = _ragged_layout(log_ns, rng, gap_max=3)
    v = orc.fr_random(total, rng)
    one = orc.fr_const(orc.CONST_ONE)
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_ragged(offsets, log_ns, False, one, one, one)
    got = dv.download()
    for j in rng.choice(64, size=8, replace=False):
        off, ln = offsets[j], log_ns[j]
        single = gb.Bls12_381FrDeviceVec.upload(v[off:off + (1 << ln)])
        single.ntt_zeta(ln, False, one, one, one)
        assert (got[off:off + (1 << ln)] == single.download()).all(), ln
    small = [j for j in range(64) if log_ns[j] <= 12][:2]
    for j in small:
        off, ln = offsets[j], log_ns[j]
        assert (got[off:off + (1 << ln)] == orc.fr_ntt(v[off:off + (1 << ln)], ln, False)).all()
    dv.ntt_ragged(offsets, log_ns, True, one, one, one)
    assert (dv.download() == v).all()
    assert gb.ntt_wait_timeouts() == 0


def test_ntt_ragged_full_size(gb, orc):
    """16 x 2^20 and 2 x 2^22 transforms in one launch equal the per-size
    batched path (itself pinned to the oracle at 2^20), and round-trip."""
    rng = np.random.default_rng(2022)
    log_ns = [20] * 16 + [22] * 2
    offsets = list(np.cumsum([0] + [1 << ln for ln in log_ns[:-1]]))
    total = int(offsets[-1]) + (1 << log_ns[-1])
    v = orc.fr_random(total, rng)
    z1, z2 = _zeta_pair(orc)
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_ragged(offsets, log_ns, False, z1, z1, z2)
    got = dv.download()
    a = gb.Bls12_381FrDeviceVec.upload(v[:16 << 20])
    a.ntt_zeta_batch(20, 16, False, z1, z1, z2)
    assert (got[:16 << 20] == a.download()).all()
    b = gb.Bls12_381FrDeviceVec.upload(v[16 << 20:])
    b.ntt_zeta_batch(22, 2, False, z1, z1, z2)
    assert (got[16 << 20:] == b.download()).all()
    del a, b, dv
    # zeta^3 = 1: scaling by zeta forward and zeta^2 inverse restores v
    one = orc.fr_const(orc.CONST_ONE)
    rt = gb.Bls12_381FrDeviceVec.upload(v)
    rt.ntt_ragged(offsets, log_ns, False, z1, one, one)
    rt.ntt_ragged(offsets, log_ns, True, z2, one, one)
    assert (rt.download() == v).all()
    assert gb.ntt_wait_timeouts() == 0


def test_ntt_ragged_rejects_bad_layouts(gb, orc):
    v = orc.fr_random(64, np.random.default_rng(5))
    one = orc.fr_const(orc.CONST_ONE)
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    for offsets, log_ns in (([0, 16], [5, 4]),      # overlap
                            ([40], [5]),             # past the end
                            ([0], [31])):            # above 2^30
        with pytest.raises(gb.MsmError):
            dv.ntt_ragged(offsets, log_ns, False, one, one, one)
    dv.ntt_ragged([], [], False, one, one, one)
    assert (dv.download() == v).all()


def test_device_ntt_single_value(gb, orc):
    """log_n = 0: the single-transform device call leaves the value unscaled
    (bls12_381_g1_msm.cu:3296-3298), the batch call scales it
    (.cu:3360-3375 runs the postprocess for every size)."""
    v = orc.fr_random(3, np.random.default_rng(8))
    z1, z2 = _zeta_pair(orc)
    scale = orc.fr_from_ints([6])[0]
    one = gb.Bls12_381FrDeviceVec.upload(v[:1])
    one.ntt_zeta(0, False, scale, z1, z2)
    assert (one.download() == v[:1]).all()
    batch = gb.Bls12_381FrDeviceVec.upload(v)
    batch.ntt_zeta_batch(0, 3, True, scale, z1, z2)
    assert (batch.download() == np.array([orc.fr_mul(x, scale) for x in v])).all()
