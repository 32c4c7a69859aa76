"""The synthetic PLONK/KZG prover driver on the oracle backend (CPU):
RNG vectors, graph compilation, permute_expression_pair, proofs that the
trapdoor verifier accepts, and rejection of broken proofs and witnesses."""
import numpy as np
import pytest

from plonk_cases import SHAPES, TAU, circuit

from gb_prover import plonk
from gb_prover.kzg import CircuitTranscript
from gb_prover.rng import ChaCha20Rng, _chacha_blocks, fr_random, mont_to_ints
from oracle import plonk_cpu, plonk_verify

R = plonk.R
_PARAMS = {}


def params(k):
    if k not in _PARAMS:
        _PARAMS[k] = plonk_cpu.setup_params(k, TAU)
    return _PARAMS[k]


def prove(c, fixed, advice, copies, label="prover-rng"):
    p = params(c.k)
    be = plonk_cpu.OracleBackend(p)
    pk = plonk.keygen(p, c, be, fixed, copies)
    proof = plonk.create_proof(p, pk, advice, be, CircuitTranscript(), ChaCha20Rng.from_label(label))
    return pk, proof


def test_chacha20_known_answers():
    # RFC 8439 2.3.2 block function test vector (key 00..1f, counter 1, nonce 0:4a:0 in the IETF layout)
    key = np.frombuffer(bytes(range(32)), dtype="<u4")
    b = _chacha_blocks(key, 1 | (0x09000000 << 32), 1, stream=0x4A000000)
    assert b[0].astype("<u4").tobytes()[:16].hex() == "10f1e7e4d13b5915500fdd1fa32071c4"
    # rand_chacha ChaCha20Rng::from_seed([0; 32]) first words
    r = ChaCha20Rng(bytes(32))
    assert [r.next_u32() for _ in range(4)] == [0xADE0B876, 0x903DF1A0, 0xE56A5D40, 0x28BD8653]


def test_fr_random_rejection_stream():
    a = fr_random(ChaCha20Rng.from_label("s"), 500)
    r2 = ChaCha20Rng.from_label("s")
    b = np.concatenate([fr_random(r2, 1) for _ in range(500)])
    assert (a == b).all()
    assert all(v < R for v in mont_to_ints(a))


def test_fr_random_matches_word_restatement():
    """Fq::random (fq.rs:373-387) restated on next_u64 words: four words,
    the top bit of the last cleared, kept when below r; the draws, in
    Montgomery form, and the stream position after them."""
    for label, n in (("a", 1), ("b", 7), ("c", 300)):
        got = fr_random(ChaCha20Rng.from_label(label), n)
        raw = plonk.fr_random_raw(ChaCha20Rng.from_label(label), n)
        r = ChaCha20Rng.from_label(label)
        want = []
        while len(want) < n:
            w = [r.next_u64() for _ in range(4)]
            v = w[0] | w[1] << 64 | w[2] << 128 | (w[3] & ((1 << 63) - 1)) << 192
            if v < R:
                want.append(v)
        assert mont_to_ints(got) == want
        assert [int(x[0]) | int(x[1]) << 64 | int(x[2]) << 128 | int(x[3]) << 192 for x in raw] == want
        after = ChaCha20Rng.from_label(label)
        fr_random(after, n)
        assert after.word_position() == r.word_position()


def test_rng_word_position_and_skip():
    a = ChaCha20Rng.from_label("skip")
    b = ChaCha20Rng.from_label("skip")
    a.next_u64_array(3)
    for count in (0, 1, 5, 16, 17, 300, 5000):
        want = a._words(count).copy() if count else None
        b.skip_words(0)
        pos = b.word_position()
        b.skip_words(count)
        assert b.word_position() == pos + count
        if count:
            c = ChaCha20Rng.from_label("skip")
            c.skip_words(pos)
            assert (c._words(count) == want).all()
        b = ChaCha20Rng.from_label("skip")
        b.skip_words(a.word_position())
        assert [b.next_u32() for _ in range(3)] == [a.next_u32() for _ in range(3)]


def test_graph_matches_expression(orc):
    """The compiled gate graph, run by the oracle's graph interpreter, equals
    the expression evaluated on the host, row by row."""
    c = circuit(6, 4, 5, 1)
    rng = np.random.default_rng(3)
    n = 64
    fixed = orc.fr_random(c.num_fixed * n, rng)
    adv = orc.fr_random(c.m * n, rng)
    g = plonk.GraphBuilder()
    g.horner((plonk.CONSTANT, 0, 0), [g.add_expression(c.gate)], (plonk.THETA, 0, 0))
    got = orc.fr_to_ints(orc.eval_numerator(n, g.compile(orc.OracleGraph), fixed=fixed, advice=adv,
                                            theta=orc.fr_from_ints([5])[0]))
    fi, ai = orc.fr_to_ints(fixed), orc.fr_to_ints(adv)
    for r in range(n):
        want = c.gate.evaluate(lambda col, rot: fi[col * n + r], lambda col, rot: ai[col * n + r])
        assert got[r] == want


def test_graph_builder_dedup_and_simplify():
    a, b, q = plonk.Expr.advice(0), plonk.Expr.advice(1), plonk.Expr.fixed(0)
    g = plonk.GraphBuilder()
    e = q * a + q * a           # shared subexpressions are stored once
    g.add_expression(e)
    ops = [calc[0] for calc, _ in g.calcs]
    assert ops == [plonk.STORE, plonk.STORE, plonk.MUL, plonk.ADD]
    g2 = plonk.GraphBuilder()
    assert g2.add_expression(a * plonk.Expr.const(1)) == g2.add_expression(a)
    assert g2.add_expression(a * plonk.Expr.const(0)) == (plonk.CONSTANT, 0, 0)
    assert g2.add_expression(b * b)[0] == plonk.INTERMEDIATE and g2.calcs[-1][0][0] == plonk.SQUARE


def test_permute_expression_pair_properties():
    c = circuit(8, 3, 3, 1)
    fixed, advice, copies = c.synthesize()
    p = params(8)
    be = plonk_cpu.OracleBackend(p)
    pk = plonk.keygen(p, c, be, fixed, copies)
    adv = be.put(plonk.ints_to_mont([v for col in advice for v in col]))
    theta = plonk.fr_mont(11)
    comp = be.eval_graphs_lagrange([pk.lookup_input_graphs[0], pk.lookup_table_graphs[0]], pk.fixed_lagrange,
                                   c.num_fixed, adv, c.m, c.n, theta)
    ci, ct = be.to_host(comp, c.n, 0), be.to_host(comp, c.n, 1)
    u = c.usable_rows
    blinds = np.zeros((c.n - u, 4), np.uint64)
    a_p, s_p = plonk._permute_expression_pair(be, ci, ct, u, blinds, blinds)
    A, S = mont_to_ints(a_p[:u]), mont_to_ints(s_p[:u])
    assert A == sorted(mont_to_ints(ci[:u]))
    assert sorted(S) == sorted(mont_to_ints(ct[:u]))
    for i in range(u):
        assert A[i] == S[i] or (i > 0 and A[i] == A[i - 1])
    assert A[0] == S[0]


@pytest.mark.parametrize("shape", SHAPES)
def test_oracle_proof_verifies(shape):
    c = circuit(*shape)
    fixed, advice, copies = c.synthesize()
    assert c.check_witness(fixed, advice)
    pk, proof = prove(c, fixed, advice, copies)
    assert plonk_verify.verify(pk, proof, TAU)


def test_proof_is_deterministic_and_rejects_tampering():
    c = circuit(8, 3, 3, 1)
    fixed, advice, copies = c.synthesize()
    pk, proof = prove(c, fixed, advice, copies)
    _, again = prove(c, fixed, advice, copies)
    assert proof == again
    _, other = prove(c, fixed, advice, copies, label="another-rng")
    assert other != proof and plonk_verify.verify(pk, other, TAU)
    # one bit of the first advice evaluation
    off = 48 * (3 + 2 + 1 + 1 + 1 + 4)
    bad = bytearray(proof)
    bad[off] ^= 1
    assert not plonk_verify.verify(pk, bytes(bad), TAU)
    assert not plonk_verify.verify(pk, proof, TAU + 1)
    assert not plonk_verify.verify(pk, proof[:-1], TAU)


def test_unsatisfied_witnesses_fail():
    c = circuit(8, 3, 3, 1)
    fixed, advice, copies = c.synthesize()
    p = params(8)
    be = plonk_cpu.OracleBackend(p)
    pk = plonk.keygen(p, c, be, fixed, copies)
    # a broken gate row
    bad = [col[:] for col in advice]
    bad[2][5] = (bad[2][5] + 1) % R
    proof = plonk.create_proof(p, pk, bad, be, CircuitTranscript(), ChaCha20Rng.from_label("x"))
    assert not plonk_verify.verify(pk, proof, TAU)
    # a broken copy constraint whose gate row is re-solved
    (_, _), (dc, dr) = copies[0]
    bad = [col[:] for col in advice]
    bad[dc][dr] = (bad[dc][dr] + 7) % R
    m = c.m
    acc = fixed[m + 1][dr] + sum(fixed[j][dr] * bad[j][dr] for j in range(m - 1)) + fixed[m][dr] * bad[0][dr] * bad[1][dr]
    bad[m - 1][dr] = -acc * pow(fixed[m - 1][dr], -1, R) % R
    assert c.check_witness(fixed, bad)
    proof = plonk.create_proof(p, pk, bad, be, CircuitTranscript(), ChaCha20Rng.from_label("x"))
    assert not plonk_verify.verify(pk, proof, TAU)
    # a lookup input outside the table is refused by the prover
    lk_rows = [r for r in range(c.usable_rows) if fixed[c.m + 2][r] == 1]
    bad = [col[:] for col in advice]
    bad[0][lk_rows[0]] = 10 ** 30
    with pytest.raises(ValueError):
        plonk.create_proof(p, pk, bad, be, CircuitTranscript(), ChaCha20Rng.from_label("x"))
