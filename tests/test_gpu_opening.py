"""KZG opening helpers on the GPU through the C ABI, bit-exact against the
oracle's eval_polynomial and kate_division (arithmetic.rs:53-116)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ln,count", [(1, 1), (7, 3), (2048, 2), (8193, 1), (1 << 16, 4)])
def test_eval_polys(gb, orc, ln, count):
    rng = np.random.default_rng(ln + count)
    polys = orc.fr_random(ln * count, rng)
    z = orc.fr_random(1, rng)[0]
    dv = gb.Bls12_381FrDeviceVec.upload(polys)
    got = gb.bls12_381_fr_device_eval_polys(dv, ln, count, z)
    for p in range(count):
        assert (got[p] == orc.fr_eval_poly(polys[p * ln:(p + 1) * ln], z)).all()
    dv.free()


def test_eval_polys_shape_errors(gb, orc):
    dv = gb.Bls12_381FrDeviceVec.upload(orc.fr_random(10, np.random.default_rng(0)))
    z = orc.fr_from_ints([3])[0]
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_device_eval_polys(dv, 3, 3, z)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_device_eval_polys(dv, 0, 1, z)
    dv.free()


@pytest.mark.parametrize("ln,count,zero", [(2, 1, False), (100, 3, False), (4097, 2, False),
                                           (1 << 17, 1, False), (300, 2, True)])
def test_kate_divide(gb, orc, ln, count, zero):
    rng = np.random.default_rng(ln * 3 + count)
    polys = orc.fr_random(ln * count, rng)
    z = orc.fr_from_ints([0])[0] if zero else orc.fr_random(1, rng)[0]
    dv = gb.Bls12_381FrDeviceVec.upload(polys)
    q = gb.fr_device_kate_divide(dv, ln, count, z)
    got = q.download().reshape(count, ln, 4)
    for p in range(count):
        want = orc.fr_kate_division(polys[p * ln:(p + 1) * ln], z)
        assert (got[p, :ln - 1] == want).all()
        assert (got[p, ln - 1] == 0).all()
    q.free()
    dv.free()


@pytest.mark.parametrize("pre_words,n", [(0, 5000), (6, 4096), (8, 1 << 16), (14, 12345)])
def test_device_random_draw_matches_host(gb, pre_words, n):
    """gb_fr_random_chacha20 gives the values fr_random would draw from the
    same rng state, and the host rng ends at the same word."""
    from gb_prover.rng import ChaCha20Rng, fr_random
    a, b = ChaCha20Rng.from_label("draw"), ChaCha20Rng.from_label("draw")
    a._words(pre_words)
    b._words(pre_words)
    want = fr_random(a, n)
    vec, used = gb.fr_random_chacha20(b.seed, b.word_position(), n)
    b.skip_words(used)
    assert (vec.download() == want).all()
    assert a.word_position() == b.word_position()
    vec.free()


def test_eval_many_matches_single_evaluations(gb, orc):
    """gb_fr_device_eval_many over requests of different vectors, counts and
    points equals one evaluation call per request (itself pinned to the
    oracle in this file)."""
    import numpy as np
    rng = np.random.default_rng(91)
    n = 1 << 12
    vecs = [gb.Bls12_381FrDeviceVec.upload(orc.fr_random(c * n, rng)) for c in (3, 1, 5)]
    pts = orc.fr_random(6, rng)
    reqs = [(vecs[0], 3, pts[0]), (vecs[1], 1, pts[1]), (vecs[2], 5, pts[2]), (vecs[0], 3, pts[3]),
            (vecs[2], 5, pts[4]), (vecs[1], 1, orc.fr_from_ints([0])[0])]
    got = gb.fr_device_eval_many(reqs, n)
    for (v, c, p), g in zip(reqs, got):
        assert (g == gb.bls12_381_fr_device_eval_polys(v, n, c, p)).all()
    want0 = orc.fr_eval_poly(vecs[1].download()[:n], pts[1])
    assert (got[1][0] == want0).all()
