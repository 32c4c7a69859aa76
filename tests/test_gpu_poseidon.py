"""The reference FFI's Poseidon entry points on the GPU through the C ABI,
bit-exact against the oracle's restatement of the reference kernel
(midnight-sppark-msm/src/bls12_381_g1_msm.cu:2018-2216): hash chains, their
256-value witness per hash, and the witness scattered into the Poseidon
chip's 8 advice columns with the chip's own layout.  The MDS matrix and
round constants are inputs of the entry points; the tests draw them at
random (the permutation's structure, not its constants, is under test)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def chip_layout():
    """poseidon_permutation_witness_layout (midnight-circuits hash/poseidon/
    poseidon_chip.rs:108-128): (column, row) of each of a permutation's 128
    witness values; width 3, 8 full and 60 partial rounds, 5 skips."""
    offset, out = 1, []
    for block in ([(3, 6)] * 4) + ([(3, 8)] * 10) + ([(3, 6)] * 4):
        lo, hi = block
        out += [(c, offset) for c in range(lo, hi)]
        offset += 1
        out += [(c, offset) for c in range(3)]
    assert len(out) == 128
    return out


def _setup(orc, seed):
    rng = np.random.default_rng(seed)
    R = orc.R_MOD
    ints = lambda k: [int.from_bytes(rng.bytes(40), "little") % R for _ in range(k)]  # noqa: E731
    mds, rc = ints(9), ints(68 * 3)
    initial, tail0, tail1 = ints(3)
    return mds, rc, initial, tail0, tail1


def test_poseidon_chain_and_witness(gb, orc):
    mds, rc, initial, tail0, tail1 = _setup(orc, 5)
    M = [mds[3 * i:3 * i + 3] for i in range(3)]
    RC = [rc[3 * r:3 * r + 3] for r in range(68)]
    m = lambda v: orc.fr_from_ints([v])[0]  # noqa: E731
    for length in (1, 3):
        want = orc.poseidon_hash_chain(initial, tail0, tail1, 3, M, RC, length)
        got = gb.bls12_381_fr_poseidon_hash_chain(m(initial), m(tail0), m(tail1), m(3), orc.fr_from_ints(mds),
                                                  orc.fr_from_ints(rc), length)
        assert orc.fr_to_ints(got) == want
        want_w = orc.poseidon_hash_chain(initial, tail0, tail1, 3, M, RC, length, witness=True)
        got_w = gb.bls12_381_fr_poseidon_hash_chain(m(initial), m(tail0), m(tail1), m(3), orc.fr_from_ints(mds),
                                                    orc.fr_from_ints(rc), length, witness=True)
        assert orc.fr_to_ints(got_w) == want_w
        # the witness carries the chain: each hash's output is its value 253
        assert [want_w[256 * h + 253] for h in range(length)] == want
    assert len(gb.bls12_381_fr_poseidon_hash_chain(m(1), m(2), m(3), m(3), orc.fr_from_ints(mds),
                                                   orc.fr_from_ints(rc), 0)) == 0


def test_poseidon_rejects_bad_constants(gb, orc):
    mds, rc, initial, tail0, tail1 = _setup(orc, 6)
    one = orc.fr_from_ints([1])[0]
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_poseidon_hash_chain(one, one, one, one, orc.fr_from_ints(mds[:8]), orc.fr_from_ints(rc), 2)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_poseidon_hash_chain(one, one, one, one, orc.fr_from_ints(mds), orc.fr_from_ints(rc[:-3]),
                                            2, witness=True)


def test_poseidon_advice_from_witness(gb, orc):
    mds, rc, initial, tail0, tail1 = _setup(orc, 7)
    m = lambda v: orc.fr_from_ints([v])[0]  # noqa: E731
    hashes, domain = 3, 256
    wit = gb.bls12_381_fr_poseidon_hash_chain(m(initial), m(tail0), m(tail1), m(3), orc.fr_from_ints(mds),
                                              orc.fr_from_ints(rc), hashes, witness=True)
    rng = np.random.default_rng(8)
    meta = [int.from_bytes(rng.bytes(40), "little") % orc.R_MOD for _ in range(11)]
    layout = chip_layout()
    dv = gb.bls12_381_fr_poseidon_advice_from_witness(wit, hashes, domain, orc.fr_from_ints(meta), layout)
    got = orc.fr_to_ints(dv.download())
    cols = orc.poseidon_advice_from_witness(orc.fr_to_ints(wit), hashes, domain, meta, layout)
    assert got == [v for col in cols for v in col]
    dv.free()
    # the domain must hold the last hash's rows; layout entries must name one of
    # the 8 columns and a row inside the domain
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_poseidon_advice_from_witness(wit, hashes, 2 + 41 * hashes, orc.fr_from_ints(meta), layout)
    bad = list(layout)
    bad[7] = (8, 1)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_poseidon_advice_from_witness(wit, hashes, domain, orc.fr_from_ints(meta), bad)
    bad[7] = (0, 200)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_poseidon_advice_from_witness(wit, hashes, domain, orc.fr_from_ints(meta), bad)
