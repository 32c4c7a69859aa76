"""KZG SRS and commitments on the GPU: g_to_lagrange reproduces the
reference's real k=14 SRS fixture point for point; the seeded-tau setup and
the commit dispatch agree with the oracle."""
import numpy as np
import pytest

from conftest import affine_of

pytestmark = pytest.mark.gpu


def test_g_to_lagrange_reproduces_real_srs(gb, orc, srs):
    from gb_prover.kzg import g_to_lagrange
    k, g, gl = srs
    got = g_to_lagrange(g, k)
    assert (got == gl).all()


def test_downsize_matches_msm_identity(gb, orc, srs):
    from gb_prover.kzg import ParamsKZG
    k, g, gl = srs
    p12 = ParamsKZG(k, g, gl).downsize(12)
    rng = np.random.default_rng(12)
    v = orc.fr_random(1 << 12, rng)
    lhs = affine_of(orc, orc.g1_msm(p12.g_lagrange, v))
    rhs = affine_of(orc, orc.g1_msm(p12.g, orc.fr_ntt(v, 12, True)))
    assert (lhs == rhs).all()


def test_unsafe_setup_and_commit_dispatch(gb, orc):
    from gb_prover.kzg import ParamsKZG, g_to_lagrange
    rng = np.random.default_rng(3)
    k = 10
    n = 1 << k
    tau = orc.fr_random(1, rng)[0]
    params = ParamsKZG.unsafe_setup(k, tau)
    t = orc.fr_to_ints(tau)[0]
    powers = orc.fr_from_ints([pow(t, i, orc.R_MOD) for i in range(n)])
    assert (params.g == orc.g1_generator_mul_batch(powers)).all()
    assert (params.g_lagrange == g_to_lagrange(params.g, k)).all()
    # commit (coefficients, against g) and commit_lagrange (evaluations, against g_lagrange)
    polys = [orc.fr_random(n, rng) for _ in range(3)] + [orc.fr_random(700, rng)]
    got = params.commit_batch(polys)
    for p, c in zip(polys, got):
        assert (affine_of(orc, c) == affine_of(orc, orc.g1_msm(params.g[:len(p)], p))).all()
    evals = [orc.fr_random(n, rng) for _ in range(2)]
    got = params.commit_lagrange_batch(evals)
    for e, c in zip(evals, got):
        assert (affine_of(orc, c) == affine_of(orc, params.commit(orc.fr_ntt(e, k, True)))).all()
    # KZG trapdoor identity: commit(p) = [p(tau)] G
    p = polys[0]
    pv = sum(c * pow(t, i, orc.R_MOD) for i, c in enumerate(orc.fr_to_ints(p))) % orc.R_MOD
    assert (affine_of(orc, params.commit(p)) == orc.g1_generator_mul_batch(orc.fr_from_ints([pv]))).all()
