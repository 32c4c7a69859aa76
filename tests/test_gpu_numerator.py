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


def _edge_graphs(rng, fr_random):
    """Graphs at the edges of the interpreter's rules: reads of intermediates
    not yet written and of indices at or above the capacity (zero), a target
    at or above the capacity (not stored), an intermediate written twice
    with reads of both values, a value never read; and a wide graph with 60
    values live at once (more slots than shared memory holds, so the
    local-array interpreter runs)."""
    consts = fr_random(3, rng)
    col = (3, 0, 0)  # advice column 0 at rotation 0
    edge = [
        (2, 0, 0, 0, col, (0, 1, 0)),          # i0 = a * c1
        (0, 1, 0, 0, (1, 0, 0), (1, 5, 0)),    # i1 = i0 + i5 (i5 not yet written: zero)
        (2, 40, 0, 0, (1, 1, 0), col),         # target 40 >= capacity 16: not stored
        (0, 2, 0, 0, (1, 40, 0), (1, 1, 0)),   # i2 = i40 (zero) + i1
        (3, 0, 0, 0, (1, 2, 0), (0, 0, 0)),    # i0 = i2^2 (rewrites i0)
        (6, 3, 0, 2, (1, 0, 0), (1, 1, 0)),    # i3 = Horner(i0; i1; parts i2, i0)
        (4, 7, 0, 0, (1, 3, 0), (0, 0, 0)),    # i7 = 2 i3, never read
        (1, 4, 0, 0, (1, 3, 0), (1, 0, 0)),    # i4 = i3 - i0
        (5, 5, 0, 0, (1, 4, 0), (0, 0, 0)),    # i5 = -i4
        (0, 6, 0, 0, (1, 5, 0), (1, 2, 0)),    # i6 = i5 + i2 (the value)
    ]
    edge_parts = [(1, 2, 0), (1, 0, 0)]
    wide = [(2, i, 0, 0, col, (0, i % 3, 0)) for i in range(60)]
    wide += [(0, 60, 0, 0, (1, 0, 0), (1, 1, 0))]
    wide += [(0, 60, 0, 0, (1, 60, 0), (1, i, 0)) for i in range(2, 60)]
    return [(consts, [0], edge, edge_parts, 10), (consts, [0], wide, [], 61)]


def test_numerator_graph_edge_cases(gb, orc):
    from gb_prover.graph import Graph
    rng = np.random.default_rng(31)
    n = 512
    case = random_case(rng, orc.fr_random, n)
    kw = {k: case[k] for k in ("fixed", "advice", "instance", "challenges", "beta", "gamma", "theta",
                               "trash_challenge", "y", "rot_scale")}
    graphs = _edge_graphs(rng, orc.fr_random)
    got = gb.bls12_381_eval_graph_batch(n, [Graph(*g) for g in graphs], **kw)
    for gi, g in enumerate(graphs):
        want = orc.eval_numerator(n, orc.OracleGraph(*g), **kw)
        assert (got[gi] == want).all(), gi
    # the same graphs as the numerator's custom gate, lookup and trash graphs
    case["graphs"]["custom"] = graphs[0]
    case["graphs"]["lookups"] = [graphs[1]]
    case["graphs"]["trash"] = [graphs[0]]
    want = call(case, orc.eval_numerator, orc.OracleGraph)
    got = call(case, gb.bls12_381_eval_numerator, Graph)
    assert (got == want).all()
