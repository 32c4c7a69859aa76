"""Synthetic PLONK/KZG proofs on the GPU backend: byte-identical to the same
driver on the oracle backend under the same seeds, accepted by the
trapdoor verifier. The last test is the full k = 16 configuration."""
import pytest

from plonk_cases import TAU, circuit, config3_circuit

from gb_prover import plonk
from gb_prover.kzg import CircuitTranscript, ParamsKZG
from gb_prover.rng import ChaCha20Rng
from oracle import plonk_cpu, plonk_verify

pytestmark = pytest.mark.gpu

_P = {}


def both_params(k):
    if k not in _P:
        hp = plonk_cpu.setup_params(k, TAU)
        gp = ParamsKZG.unsafe_setup(k, plonk.fr_mont(TAU))
        assert (gp.g == hp.g).all() and (gp.g_lagrange == hp.g_lagrange).all()
        _P[k] = (gp, hp)
    return _P[k]


def prove_both(c, label="prover-rng"):
    fixed, advice, copies = c.synthesize()
    gp, hp = both_params(c.k)
    gbe, hbe = plonk.GpuBackend(gp), plonk_cpu.OracleBackend(hp)
    gpk = plonk.keygen(gp, c, gbe, fixed, copies)
    hpk = plonk.keygen(hp, c, hbe, fixed, copies)
    for a, b in zip(gpk.fixed_commitments + gpk.sigma_commitments, hpk.fixed_commitments + hpk.sigma_commitments):
        assert (a == b).all()
    assert gpk.transcript_repr == hpk.transcript_repr
    gproof = plonk.create_proof(gp, gpk, advice, gbe, CircuitTranscript(), ChaCha20Rng.from_label(label))
    hproof = plonk.create_proof(hp, hpk, advice, hbe, CircuitTranscript(), ChaCha20Rng.from_label(label))
    return hpk, gproof, hproof


@pytest.mark.parametrize("shape", [(7, 3, 3, 0), (8, 3, 3, 1), (8, 4, 5, 2), (9, 8, 4, 2), (10, 5, 3, 1)])
def test_gpu_proof_equals_oracle(gb, shape):
    hpk, gproof, hproof = prove_both(circuit(*shape))
    assert gproof == hproof
    assert plonk_verify.verify(hpk, gproof, TAU)


def test_config3_full_proof(gb):
    """k = 16, 3 advice columns, standard gate, 2^14 copy constraints, one
    2-column lookup into a 2^12-row table, SRS of 2^16 points from a seeded
    tau: identical proof bytes, verified."""
    hpk, gproof, hproof = prove_both(config3_circuit())
    assert gproof == hproof
    assert plonk_verify.verify(hpk, gproof, TAU)


def test_k18_full_proof(gb):
    """k = 18, 3 advice columns, the standard gate, 2^16 copy constraints,
    one 2-column lookup into a 2^14-row table: identical proof bytes,
    verified."""
    c = circuit(18, 3, 3, 1, copies=1 << 16, table_log=14, label="synthetic PLONK/KZG proof, k=18")
    hpk, gproof, hproof = prove_both(c)
    assert gproof == hproof
    assert plonk_verify.verify(hpk, gproof, TAU)


@pytest.mark.parametrize("u,n,tsize,dup", [(250, 256, 32, False), (4090, 4096, 4000, False), (65529, 65536, 4096, True),
                                           (1000, 1024, 1, True)])
def test_device_lookup_permutation_matches_host(gb, orc, u, n, tsize, dup):
    """gb_fr_lookup_permute_device against the host permute_expression_pair
    for two lookups at once: small tables with heavy repetition, a table
    of one value, a full k=16 column."""
    import numpy as np
    from oracle.plonk_cpu import OracleBackend
    rng = np.random.default_rng(u + tsize)
    cols = []
    for _ in range(2):
        table_vals = orc.fr_random(tsize, rng)
        tab = table_vals[rng.integers(0, tsize, size=n)]
        tab[:tsize] = table_vals  # every table value present
        pick = rng.integers(0, min(tsize, 7) if dup else tsize, size=n)
        inp = table_vals[pick]
        cols += [inp, tab]
    comp = np.concatenate(cols)
    nb = n - u
    ib, tb = orc.fr_random(2 * nb, rng), orc.fr_random(2 * nb, rng)
    want = OracleBackend(None).permute_lookups(OracleBackend(None).put(comp), n, u, 2, ib, tb).a
    got = gb.fr_lookup_permute_device(gb.Bls12_381FrDeviceVec.upload(comp), n, u, 2, ib, tb).download()
    assert (got == want).all()


def test_device_lookup_permutation_rejects_missing_input(gb, orc):
    import numpy as np
    rng = np.random.default_rng(3)
    n, u = 256, 250
    tab = orc.fr_random(n, rng)
    inp = tab.copy()
    inp[17] = orc.fr_random(1, rng)[0]
    with pytest.raises(gb.MsmError):
        gb.fr_lookup_permute_device(gb.Bls12_381FrDeviceVec.upload(np.concatenate([inp, tab])), n, u, 1,
                                    orc.fr_random(n - u, rng), orc.fr_random(n - u, rng))


def test_proof_on_the_reference_srs(gb, srs):
    """The reference's own k = 14 SRS (bls_midnight_2p14: g and g_lagrange)
    as the commitment key of both backends: identical proof bytes. Its tau
    is unknown, so this checks parity on real bases, not validity."""
    k, g, gl = srs
    c = circuit(14, 3, 3, 1, copies=1 << 12, table_log=10, label="reference srs circuit")
    fixed, advice, copies = c.synthesize()
    gp = ParamsKZG(k, g, gl)
    hp = plonk_cpu.HostParams(k, g, gl)
    gbe, hbe = plonk.GpuBackend(gp), plonk_cpu.OracleBackend(hp)
    gpk = plonk.keygen(gp, c, gbe, fixed, copies)
    hpk = plonk.keygen(hp, c, hbe, fixed, copies)
    gproof = plonk.create_proof(gp, gpk, advice, gbe, CircuitTranscript(), ChaCha20Rng.from_label("real-srs"))
    hproof = plonk.create_proof(hp, hpk, advice, hbe, CircuitTranscript(), ChaCha20Rng.from_label("real-srs"))
    assert gproof == hproof


def test_native_chacha_blocks_match_restatement(gb):
    """The library's host ChaCha20 blocks (used by ChaCha20Rng once the
    library is loaded) equal the restatement, across the 32-bit counter
    boundary."""
    import numpy as np
    from gb_prover import rng
    key = np.arange(1, 9, dtype=np.uint32) * np.uint32(0x9E3779B9)
    for counter, n in ((0, 1), (7, 3), ((1 << 32) - 2, 4), (1 << 40, 5)):
        got = rng._native_blocks(gb.lib(), key, counter, n)
        want = rng._chacha_blocks(key, counter, n).reshape(-1)
        assert (got == want).all(), counter


def test_device_lookup_permutation_top_limb_ties(gb, orc):
    """Distinct values that share their top 64-bit limb: the sort by the
    top limb alone is then not canonical, and the device permutation must
    fall back to the whole key (equal to the host permutation)."""
    import numpy as np
    from oracle.plonk_cpu import OracleBackend
    rng = np.random.default_rng(1234)
    n, u, tsize = 1024, 1018, 300
    top = 0x1234567890ABCDEF << 192
    ints = sorted({top + int(x) for x in rng.integers(0, 1 << 62, size=tsize)})
    table_vals = orc.fr_from_ints(ints[:tsize])
    tab = table_vals[rng.integers(0, len(table_vals), size=n)]
    tab[:len(table_vals)] = table_vals
    inp = table_vals[rng.integers(0, 40, size=n)]
    comp = np.concatenate([inp, tab])
    nb = n - u
    ib, tb = orc.fr_random(nb, rng), orc.fr_random(nb, rng)
    want = OracleBackend(None).permute_lookups(OracleBackend(None).put(comp), n, u, 1, ib, tb).a
    got = gb.fr_lookup_permute_device(gb.Bls12_381FrDeviceVec.upload(comp), n, u, 1, ib, tb).download()
    assert (got == want).all()
