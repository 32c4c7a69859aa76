"""Quotient numerator on the GPU through the C ABI against the oracle, on
seeded random compiled graphs with permutation, lookup and trash terms."""
import numpy as np
import pytest

from numerator_cases import call, random_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("length,seed", [(64, 1), (1024, 2), (1 << 14, 3)])
def test_numerator_matches_oracle(gb, orc, length, seed):
    from gb_prover.graph import Graph
    rng = np.random.default_rng(seed)
    case = random_case(rng, orc.fr_random, length)
    want = call(case, orc.eval_numerator, orc.OracleGraph)
    got = call(case, gb.bls12_381_eval_numerator, Graph)
    assert (got == want).all()
    init = orc.fr_random(length, rng)
    want = call(case, orc.eval_numerator, orc.OracleGraph, run_custom=False, initial_out=init)
    got = call(case, gb.bls12_381_eval_numerator, Graph, run_custom=False, initial_out=init)
    assert (got == want).all()


def test_graph_batch_matches_oracle(gb, orc):
    from gb_prover.graph import Graph
    rng = np.random.default_rng(9)
    n = 2048
    case = random_case(rng, orc.fr_random, n)
    graphs = [case["graphs"]["custom"]] + case["graphs"]["lookups"]
    kw = {k: case[k] for k in ("fixed", "advice", "instance", "challenges", "beta", "gamma", "theta",
                               "trash_challenge", "y", "rot_scale")}
    got = gb.bls12_381_eval_graph_batch(n, [Graph(*g) for g in graphs], **kw)
    for gi, g in enumerate(graphs):
        want = orc.eval_numerator(n, orc.OracleGraph(*g), **{k: case[k] for k in (
            "fixed", "advice", "instance", "challenges", "beta", "gamma", "theta", "trash_challenge", "y",
            "rot_scale")})
        assert (got[gi] == want).all(), gi
