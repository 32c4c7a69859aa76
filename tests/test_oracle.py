"""CPU oracle pinned against the reference's literal constants, its real
k=14 SRS fixture and restated known-answer tests.  No GPU needed."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN, affine_of


def test_fr_constants_match_reference_literals(orc):
    # Montgomery limbs copied from vendor/midnight-curves-0.3.1/src/bls12_381/fq.rs
    lit = {
        orc.CONST_GENERATOR: [0x0000000EFFFFFFF1, 0x17E363D300189C0F, 0xFF9C57876F8457B0, 0x351332208FC5A8C4],
        orc.CONST_ROOT: [0xB9B58D8C5F0E466A, 0x5B1B4C801819D7EC, 0x0AF53AE352A31E64, 0x5BF3ADDA19E9B27B],
        orc.CONST_ROOT_INV: [0x4256481ADCF3219A, 0x45F37B7F96B6CAD3, 0xF9C3F1D75F7A3B27, 0x2D2FC049658AFD43],
        orc.CONST_DELTA: [0x70E310D3D146F96A, 0x4B64C08919E299E6, 0x51E114186A8B970D, 0x6185D06627C067CB],
        orc.CONST_ZETA: [0x92D9090B093011D2, 0xFC9CBD719D6AA073, 0xC1F14EF0CD65A1A6, 0x017F6D35E72FCDEB],
        orc.CONST_ONE: [0x00000001FFFFFFFE, 0x5884B7FA00034802, 0x998C4FEFECBC4FF5, 0x1824B159ACC5056F],
    }
    for which, limbs in lit.items():
        assert [int(x) for x in orc.fr_const(which)] == limbs, which


def test_field_mul_matches_python_bigints(orc):
    rng = np.random.default_rng(11)
    a = orc.fr_random(64, rng)
    b = orc.fr_random(64, rng)
    ai, bi = orc.fr_to_ints(a), orc.fr_to_ints(b)
    for k in range(64):
        assert orc.fr_to_ints(orc.fr_mul(a[k], b[k]))[0] == ai[k] * bi[k] % orc.R_MOD
        if ai[k]:
            assert orc.fr_to_ints(orc.fr_inv(a[k]))[0] == pow(ai[k], -1, orc.R_MOD)


def test_generator_and_encodings(orc):
    g = orc.g1_generator()
    assert orc.g1_is_on_curve(g)
    comp = orc.g1_compress(g)
    assert comp.hex().startswith("97f1d3a73197d7942695638c4fa9ac0f")  # zcash encoding of G1
    assert (orc.g1_decompress(comp) == g).all()
    assert (orc.g1_from_uncompressed(orc.g1_to_uncompressed(g)) == g).all()
    inf = np.zeros(12, dtype=np.uint64)
    assert orc.g1_compress(inf)[0] == 0xC0
    assert (orc.g1_decompress(orc.g1_compress(inf)) == inf).all()
    # negative point round-trips through the sort flag
    rng = np.random.default_rng(3)
    pts = orc.g1_generator_mul_batch(orc.fr_random(16, rng))
    for p in pts:
        assert (orc.g1_decompress(orc.g1_compress(p)) == p).all()


def test_srs_fixture_hash():
    lines = open(os.path.join(GOLDEN, "srs_2p14_g1.sha256")).read().split("\n")
    want = [ln.split()[0] for ln in lines if ln.endswith("srs_2p14_g1.bin")][0]
    got = hashlib.sha256(open(os.path.join(GOLDEN, "srs_2p14_g1.bin"), "rb").read()).hexdigest()
    assert got == want


def test_srs_known_answers(orc, srs):
    """Absolute KATs from transient-crypto/static/bls_midnight_2p14:
    g[0] = G; sum_i g_lagrange[i] = G; MSM(g_lagrange, v) = MSM(g, iNTT(v));
    g_lagrange[i] = n^-1 sum_j w^-ij g[j] (params.rs g_to_lagrange)."""
    k, g, gl = srs
    n = 1 << k
    assert (g[0] == orc.g1_generator()).all()
    assert all(orc.g1_is_on_curve(p) for p in g[:64])
    ones = orc.fr_from_ints([1] * n)
    assert (affine_of(orc, orc.g1_msm(gl, ones))[0] == g[0]).all()
    rng = np.random.default_rng(5)
    v = orc.fr_random(n, rng)
    coeffs = orc.fr_ntt(v, k, True)
    assert (affine_of(orc, orc.g1_msm(gl, v)) == affine_of(orc, orc.g1_msm(g, coeffs))).all()
    # a few Lagrange basis points directly
    w = orc.fr_to_ints(orc.fr_omega(k))[0]
    winv = pow(w, -1, orc.R_MOD)
    ninv = pow(n, -1, orc.R_MOD)
    for i in (0, 1, 7, n - 1):
        scal = orc.fr_from_ints([ninv * pow(winv, i * j, orc.R_MOD) % orc.R_MOD for j in range(n)])
        assert (affine_of(orc, orc.g1_msm(g, scal))[0] == gl[i]).all(), i


def test_booth_encoding_kat(orc):
    """msm.rs:570-608: the Booth-decomposed double-and-add equals [s]P for
    window sizes 1..9 (restated with the oracle's group law)."""
    rng = np.random.default_rng(8)
    scalars = orc.fr_random(6, rng)
    pts = orc.g1_generator_mul_batch(orc.fr_random(6, rng))
    for window in range(1, 10):
        for s, p in zip(scalars, pts):
            sv = orc.fr_to_ints(s)[0]
            le = sv.to_bytes(32, "little")
            nwin = 255 // window + 1
            acc = 0
            for i in reversed(range(nwin)):
                acc = acc * (1 << window) + orc.booth_index(i, window, le)
            assert acc % orc.R_MOD == sv, (window, sv)
    # direct group check for one window size
    s, p = scalars[0], pts[0]
    assert (affine_of(orc, orc.g1_mul(p, s)) == affine_of(orc, orc.g1_msm(p[None], s[None], window_bits=5))).all()


def test_msm_naive_matches_pippenger_all_windows(orc):
    rng = np.random.default_rng(2)
    n = 200
    s = orc.fr_random(n, rng)
    s[5] = 0
    s[9] = orc.fr_from_ints([orc.R_MOD - 1])[0]
    b = orc.g1_generator_mul_batch(orc.fr_random(n, rng))
    b[20] = b[21]  # repeated base
    want = affine_of(orc, orc.g1_msm_naive(b, s))
    for c in (1, 2, 4, 7, 11, 16):
        assert (affine_of(orc, orc.g1_msm(b, s, window_bits=c)) == want).all(), c


def _naive_dft(vals, w):
    n = len(vals)
    return [sum(vals[j] * pow(w, j * k, R) for j in range(n)) % R for k in range(n)]


R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


@pytest.mark.parametrize("log_n", [0, 1, 2, 3, 5])
def test_ntt_matches_naive_dft(orc, log_n):
    n = 1 << log_n
    vals = [(13 * i + 7) % 65521 for i in range(n)]
    a = orc.fr_from_ints(vals)
    w = orc.fr_to_ints(orc.fr_omega(log_n))[0]
    assert orc.fr_to_ints(orc.fr_ntt(a, log_n, False)) == _naive_dft(vals, w)
    back = orc.fr_ntt(orc.fr_ntt(a, log_n, False), log_n, True)
    assert (back == a).all()


def test_coeff_to_extended_matches_definition(orc):
    k, ek = 3, 5
    vals = [(29 * i + 11) % 65521 for i in range(1 << k)]
    z = orc.fr_to_ints(orc.fr_const(orc.CONST_ZETA))[0]
    first, second = orc.fr_from_ints([z])[0], orc.fr_from_ints([z * z % R])[0]
    out = orc.fr_to_ints(orc.fr_coeff_to_extended_batch(orc.fr_from_ints(vals), 1 << k, 1, ek, first, second))
    w = orc.fr_to_ints(orc.fr_omega(ek))[0]
    # evaluations of a(X) at zeta * w^i
    for i in (0, 1, 5, 31):
        x = z * pow(w, i, R) % R
        assert out[i] == sum(c * pow(x, j, R) for j, c in enumerate(vals)) % R


def test_sppark_group_gen_is_the_generator(orc):
    # group_gen / group_gen_inverse of vendor/sppark-0.1.15/sppark/ntt/parameters/bls12_381.h:11-12
    # (the coset generator of sppark's coset NTT and LDE) are GENERATOR = 7 and 1/7 (fq.rs:31-33)
    gen = [0x0000000EFFFFFFF1, 0x17E363D300189C0F, 0xFF9C57876F8457B0, 0x351332208FC5A8C4]
    gen_inv = [0xDB6DB6DADB6DB6DC, 0xE6B5824ADB6CC6DA, 0xF8B356E005810DB9, 0x66D0F1E660EC4796]
    assert orc.fr_to_ints(np.array([gen], dtype=np.uint64))[0] == 7
    assert orc.fr_to_ints(np.array([gen_inv], dtype=np.uint64))[0] == pow(7, -1, R)
    assert [int(x) for x in orc.fr_const(orc.CONST_GENERATOR)] == gen


@pytest.mark.parametrize("k,ek", [(3, 5), (4, 4), (2, 6)])
def test_coeff_to_extended_coset_matches_definition(orc, k, ek):
    """a(X) evaluated at shift * w_ext^i, with the generator 7 and another shift"""
    vals = [(31 * i + 5) % 65521 for i in range(1 << k)]
    w = orc.fr_to_ints(orc.fr_omega(ek))[0]
    for shift in (7, 123456789):
        sh = orc.fr_from_ints([shift])[0]
        out = orc.fr_to_ints(orc.fr_coeff_to_extended_coset_batch(orc.fr_from_ints(vals + vals[::-1]), 1 << k,
                                                                  2, ek, sh))
        for p, poly in enumerate((vals, vals[::-1])):
            for i in range(1 << ek):
                x = shift * pow(w, i, R) % R
                assert out[(p << ek) + i] == sum(c * pow(x, j, R) for j, c in enumerate(poly)) % R


def test_ntt_coset_and_lde_definitions(orc):
    log_n = 4
    n = 1 << log_n
    vals = [(17 * i + 3) % 65521 for i in range(n)]
    a = orc.fr_from_ints(vals)
    g = orc.fr_const(orc.CONST_GENERATOR)
    w = orc.fr_to_ints(orc.fr_omega(log_n))[0]
    fwd = orc.fr_to_ints(orc.fr_ntt_coset(a, log_n, False, g))
    # forward coset NTT: evaluations at 7 w^i
    for i in range(n):
        x = 7 * pow(w, i, R) % R
        assert fwd[i] == sum(c * pow(x, j, R) for j, c in enumerate(vals)) % R
    # the inverse undoes it
    assert (orc.fr_ntt_coset(orc.fr_ntt_coset(a, log_n, False, g), log_n, True, g) == a).all()
    # LDE: the evaluations' polynomial on the coset 7 * <w_ext>, blowup 4
    lde = orc.fr_to_ints(orc.fr_lde_coset(a, log_n, 2))
    coeffs = orc.fr_to_ints(orc.fr_ntt(a, log_n, True))
    we = orc.fr_to_ints(orc.fr_omega(log_n + 2))[0]
    for i in (0, 1, 17, 63):
        x = 7 * pow(we, i, R) % R
        assert lde[i] == sum(c * pow(x, j, R) for j, c in enumerate(coeffs)) % R


def test_t_evaluations(orc):
    j, k = 4, 3
    ek = orc.domain_extended_k(j, k)
    assert ek == 5
    t = orc.fr_to_ints(orc.domain_t_evaluations(j, k))
    z = orc.fr_to_ints(orc.fr_const(orc.CONST_ZETA))[0]
    w = orc.fr_to_ints(orc.fr_omega(ek))[0]
    for i in range(1 << (ek - k)):
        x = z * pow(w, i, R) % R
        assert t[i] == pow((pow(x, 1 << k, R) - 1) % R, -1, R)


def test_shifted_prefix_product_kat(orc):
    # midnight-sppark-msm/src/lib.rs:4664-4682 shape
    for ln in (1, 2, 17, 100):
        vals = [(i % 251) + 2 for i in range(ln)]
        got = orc.fr_to_ints(orc.fr_shifted_prefix_product(orc.fr_from_ints(vals), orc.fr_from_ints([7])[0]))
        exp = [7]
        for i in range(1, ln):
            exp.append(exp[-1] * vals[i - 1] % R)
        assert got == exp


def test_permutation_products_kat(orc):
    """lib.rs:4785-4894 restated with Python integers."""
    ln, cc, chunk, bf = 16, 5, 2, 4
    sets = (cc + chunk - 1) // chunk
    beta, gamma = 17, 23
    w = orc.fr_to_ints(orc.fr_omega(4))[0]
    delta = orc.fr_to_ints(orc.fr_const(orc.CONST_DELTA))[0]
    cols = [[(c * 71 + r * 29 + 5) % 65521 for r in range(ln)] for c in range(cc)]
    perms = [[(c * 43 + r * 37 + 101) % 65521 for r in range(ln)] for c in range(cc)]
    dp = [pow(delta, c, R) for c in range(cc)]
    blinds = [i * 13 + 211 for i in range(sets * bf)]
    expected, init = [], 1
    for s in range(sets):
        fr = []
        for r in range(ln):
            num = den = 1
            for c in range(s * chunk, min(cc, s * chunk + chunk)):
                num = num * (cols[c][r] + dp[c] * pow(w, r, R) * beta + gamma) % R
                den = den * (cols[c][r] + beta * perms[c][r] + gamma) % R
            fr.append(num * pow(den, -1, R) % R)
        z = [init]
        for r in range(1, ln):
            z.append(z[-1] * fr[r - 1] % R)
        init = z[ln - bf - 1]
        z[ln - bf:] = blinds[s * bf:(s + 1) * bf]
        expected += z
    got = orc.fr_permutation_products(
        orc.fr_from_ints(sum(cols, [])), orc.fr_from_ints(sum(perms, [])), ln, cc, chunk,
        orc.fr_from_ints([beta])[0], orc.fr_from_ints([gamma])[0], orc.fr_omega(4), orc.fr_from_ints(dp),
        orc.fr_from_ints(blinds), bf)
    assert orc.fr_to_ints(got) == expected


def test_lookup_products_kat(orc):
    ln, lc, bf = 16, 2, 4
    beta, gamma = 17, 23
    seq = lambda off: [(i * 29 + off * 43 + 101) % 65521 for i in range(lc * ln)]  # noqa: E731
    ci, ct, pi, pt = seq(1), seq(2), seq(3), seq(4)
    blinds = [i * 13 + 211 for i in range(lc * bf)]
    expected = []
    for l_ in range(lc):
        o = l_ * ln
        fr = [(ci[o + i] + beta) * (ct[o + i] + gamma) * pow((pi[o + i] + beta) * (pt[o + i] + gamma), -1, R) % R
              for i in range(ln)]
        z = [1]
        for r in range(1, ln):
            z.append(z[-1] * fr[r - 1] % R)
        z[ln - bf:] = blinds[l_ * bf:(l_ + 1) * bf]
        expected += z
    got = orc.fr_lookup_products(orc.fr_from_ints(ci), orc.fr_from_ints(ct), orc.fr_from_ints(pi),
                                 orc.fr_from_ints(pt), ln, lc, orc.fr_from_ints([beta])[0],
                                 orc.fr_from_ints([gamma])[0], orc.fr_from_ints(blinds), bf)
    assert orc.fr_to_ints(got) == expected


def test_quotient_pieces_kat(orc):
    n, pieces = 8, 3
    q = [(i * 7 + 3) % 65521 for i in range((n - 1) * pieces + 5)]
    bl = [1000 + i for i in range(pieces - 1)]
    got = orc.fr_to_ints(orc.fr_quotient_pieces(orc.fr_from_ints(q), n, pieces, orc.fr_from_ints(bl)))
    limbs = [q[p * (n - 1):(p + 1) * (n - 1)] for p in range(pieces)]
    for i in range(1, pieces):  # vanishing/prover.rs:304-318
        limbs[i - 1].append(bl[i - 1])
        limbs[i][0] = (limbs[i][0] - bl[i - 1]) % R
    limbs[-1].append(0)
    assert got == sum(limbs, [])


def test_batch_invert_and_sort(orc):
    vals = [0 if i % 257 == 0 else (i % 251) + 2 for i in range(600)]
    got = orc.fr_to_ints(orc.fr_batch_invert(orc.fr_from_ints(vals)))
    assert got == [pow(v, -1, R) if v else 0 for v in vals]
    rng = np.random.default_rng(4)
    a = orc.fr_random(300, rng)
    assert orc.fr_to_ints(orc.fr_sort_canonical(a)) == sorted(orc.fr_to_ints(a))


def test_eval_and_kate_division(orc):
    """eval_polynomial and kate_division (arithmetic.rs:53-116) against
    integer arithmetic: q (X - z) + a(z) == a, including z = 0 and len 1."""
    rng = np.random.default_rng(11)
    for ln, zv in ((50, None), (33, 0), (1, None), (2, 5)):
        a = orc.fr_random(ln, rng)
        z = orc.fr_random(1, rng)[0] if zv is None else orc.fr_from_ints([zv])[0]
        ai, zi = orc.fr_to_ints(a), orc.fr_to_ints(z[None])[0]
        ev = sum(c * pow(zi, i, R) for i, c in enumerate(ai)) % R
        assert orc.fr_to_ints(orc.fr_eval_poly(a, z)[None])[0] == ev
        q = orc.fr_to_ints(orc.fr_kate_division(a, z))
        assert len(q) == ln - 1
        back = [0] * ln
        for i, c in enumerate(q):
            back[i + 1] = (back[i + 1] + c) % R
            back[i] = (back[i] - c * zi) % R
        back[0] = (back[0] + ev) % R
        assert back == ai


def test_poseidon_oracle_structure():
    """The Poseidon restatement's round structure and witness order: with the
    identity MDS and zero constants the two outer lanes see only the 8 full
    rounds' x^5 and the third lane all 68; a chain's outputs are its
    witness values 253 (the second permutation's final first element), and
    the first permutation's final state sits at 125..127."""
    from oracle import oracle as orc
    R = orc.R_MOD
    ident = [[1 if i == j else 0 for j in range(3)] for i in range(3)]
    zero = [[0, 0, 0] for _ in range(68)]
    x = [5, 7, 11]
    out = orc._poseidon_permute(list(x), ident, zero, None)
    assert out == [pow(5, 5 ** 8, R), pow(7, 5 ** 8, R), pow(11, 5 ** 68, R)]
    rng = np.random.default_rng(3)
    ints = lambda k: [int.from_bytes(rng.bytes(40), "little") % R for _ in range(k)]  # noqa: E731
    mds = [ints(3) for _ in range(3)]
    rc = [ints(3) for _ in range(68)]
    initial, tail0, tail1 = ints(3)
    outs = orc.poseidon_hash_chain(initial, tail0, tail1, 3, mds, rc, 3)
    wit = orc.poseidon_hash_chain(initial, tail0, tail1, 3, mds, rc, 3, witness=True)
    assert len(wit) == 3 * 256
    assert outs == [wit[256 * h + 253] for h in range(3)]
    first = orc._poseidon_permute([initial, tail0, 3], mds, rc, None)
    assert first == wit[125:128]
