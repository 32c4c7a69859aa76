"""The numerator context through the C ABI (create, eval and the three
trace-context calls) against the oracle, on seeded random graphs and
columns: the context's resident fixed data, one column vector with every
group at its own offset, delta_start = beta * g_coset, and the trace-side
trash, permutation and lookup-permutation outputs."""
import numpy as np
import pytest

from numerator_cases import call, random_case

pytestmark = pytest.mark.gpu

N_FIXED, N_ADVICE, N_INSTANCE = 3, 3, 1
LOOKUPS, TRASH = 2, 2
# in range for the trace domain's columns (kind 0 fixed, 1 advice, 2 instance)
PERM_COLUMNS = [(1, 0), (0, 2), (2, 0), (1, 2), (0, 0)]


def _copy_graph(orc, rng, kind, index):
    """A graph whose value is one column at rotation 0 (sources: kind 2
    fixed, 3 advice, 4 instance; calculation 7 copies its lhs)."""
    return (orc.fr_random(1, rng), [0], [(7, 0, 0, 0, (kind, index, 0), (0, 0, 0))], [], 1)


def _setup(gb, orc, n, n_in, seed):
    from gb_prover.graph import Graph
    rng = np.random.default_rng(seed)
    case = random_case(rng, orc.fr_random, n, n_fixed=N_FIXED, n_advice=N_ADVICE, n_instance=N_INSTANCE, sets=3,
                       chunk=2, lookups=LOOKUPS, trash=TRASH)
    case["permutation_columns"] = list(PERM_COLUMNS)
    ncol = len(PERM_COLUMNS)
    case["permutation_pk_cosets"] = orc.fr_random(ncol * n, rng)
    g_coset = orc.fr_random(1, rng)[0]
    trace_omega = orc.fr_random(1, rng)[0]
    # trace-domain data: fixed columns 1 and 2 are the lookup tables, advice
    # columns 0 and 1 the lookup inputs drawn from them
    fixed_l = orc.fr_random(N_FIXED * n_in, rng).reshape(N_FIXED, n_in, 4)
    advice_l = orc.fr_random(N_ADVICE * n_in, rng).reshape(N_ADVICE, n_in, 4)
    instance_l = orc.fr_random(N_INSTANCE * n_in, rng).reshape(N_INSTANCE, n_in, 4)
    for li in range(LOOKUPS):
        values = orc.fr_random(n_in // 8, rng)
        fixed_l[1 + li] = values[rng.integers(0, len(values), size=n_in)]
        fixed_l[1 + li][:len(values)] = values
        advice_l[li] = values[rng.integers(0, min(len(values), 5), size=n_in)]
    pk_l = orc.fr_random(ncol * n_in, rng)
    G = case["graphs"]
    keep = {
        "custom": Graph(*G["custom"]),
        "lookups": [Graph(*g) for g in G["lookups"]],
        "inputs": [Graph(*_copy_graph(orc, rng, 3, li)) for li in range(LOOKUPS)],
        "tables": [Graph(*_copy_graph(orc, rng, 2, 1 + li)) for li in range(LOOKUPS)],
        "trash": [Graph(*g) for g in G["trash"]],
    }
    ctx = gb.NumeratorContext(
        n, n_in, keep["custom"], fixed=case["fixed"], fixed_lagrange=fixed_l.reshape(-1, 4), fixed_cols=N_FIXED,
        l0=case["l0"], l_last=case["l_last"], l_active=case["l_active"], permutation_columns=PERM_COLUMNS,
        permutation_pk_cosets=case["permutation_pk_cosets"], permutation_pk_lagrange=pk_l, permutation_pk_count=ncol,
        trash_selectors=[d[1] for d in case["trash_data"]], lookup_graphs=keep["lookups"],
        lookup_input_graphs=keep["inputs"], lookup_table_graphs=keep["tables"], trash_graphs=keep["trash"],
        omega=case["omega"], trace_omega=trace_omega, g_coset=g_coset, delta_const=case["delta_const"],
        rot_scale=case["rot_scale"], last_rotation=case["last_rotation"], chunk_len=case["chunk_len"])
    trace = {"fixed": fixed_l, "advice": advice_l, "instance": instance_l, "pk": pk_l, "omega": trace_omega}
    return ctx, case, g_coset, trace, keep, rng


@pytest.mark.parametrize("n,seed", [(256, 1), (1 << 14, 2)])
def test_context_eval_matches_oracle(gb, orc, n, seed):
    ctx, case, g_coset, _, _, rng = _setup(gb, orc, n, n // 4, seed)
    # one column vector: a padding column, instance, advice, permutation
    # products, lookup products / permuted inputs / permuted tables, trash
    lk = case["lookup_data"]
    groups = [orc.fr_random(n, rng), case["instance"], case["advice"], case["permutation_products"],
              np.concatenate([d[0] for d in lk]), np.concatenate([d[1] for d in lk]),
              np.concatenate([d[2] for d in lk]), np.concatenate([d[0] for d in case["trash_data"]])]
    offsets, at = [], 0
    for g in groups:
        offsets.append(at)
        at += len(g) // n
    cols = gb.Bls12_381FrDeviceVec.upload(np.concatenate(groups))
    for _ in range(2):
        case["delta_start"] = orc.fr_mul(case["beta"], g_coset)
        want = call(case, orc.eval_numerator, orc.OracleGraph)
        got = ctx.eval(cols, at, advice_offset=offsets[2], advice_cols=N_ADVICE, instance_offset=offsets[1],
                       instance_cols=N_INSTANCE, challenges=case["challenges"], beta=case["beta"],
                       gamma=case["gamma"], theta=case["theta"], trash_challenge=case["trash_challenge"], y=case["y"],
                       permutation_offset=offsets[3], permutation_sets=case["permutation_sets"],
                       lookup_product_offset=offsets[4], lookup_input_offset=offsets[5],
                       lookup_table_offset=offsets[6], lookup_count=LOOKUPS, trash_offset=offsets[7],
                       trash_count=TRASH).download()
        assert (got == want).all()
        # the context is reused with new challenges
        for k in ("beta", "gamma", "y"):
            case[k] = orc.fr_random(1, rng)[0]
    with pytest.raises(gb.MsmError):
        ctx.eval(cols, at, lookup_count=LOOKUPS - 1, trash_count=TRASH)
    with pytest.raises(gb.MsmError):
        ctx.eval(cols, at, advice_offset=at - 1, advice_cols=2, lookup_count=LOOKUPS, trash_count=TRASH)
    ctx.close()


@pytest.mark.parametrize("n_in,seed", [(256, 3), (4096, 4)])
def test_trace_context_calls_match_oracle(gb, orc, n_in, seed):
    from oracle.plonk_cpu import OracleBackend
    ctx, case, _, trace, keep, rng = _setup(gb, orc, 4 * n_in, n_in, seed)
    advice = gb.Bls12_381FrDeviceVec.upload(trace["advice"].reshape(-1, 4))
    instance = gb.Bls12_381FrDeviceVec.upload(trace["instance"].reshape(-1, 4))
    fixed_flat = trace["fixed"].reshape(-1, 4)
    zero = np.zeros(4, dtype=np.uint64)

    # trash: each compressed expression over the trace, only the trash challenge set
    got = ctx.trace_trash(advice, N_ADVICE, instance, N_INSTANCE, case["challenges"],
                          case["trash_challenge"]).download()
    for ti, g in enumerate(case["graphs"]["trash"]):
        want = orc.eval_numerator(n_in, orc.OracleGraph(*g), fixed=fixed_flat, advice=trace["advice"].reshape(-1, 4),
                                  instance=trace["instance"].reshape(-1, 4), challenges=case["challenges"],
                                  beta=zero, gamma=zero, theta=zero, trash_challenge=case["trash_challenge"], y=zero,
                                  rot_scale=1)
        assert (got[ti * n_in:(ti + 1) * n_in] == want).all(), ti

    # permutation products over the referenced Lagrange columns
    src = {0: trace["fixed"], 1: trace["advice"], 2: trace["instance"]}
    columns = np.concatenate([src[k][i] for k, i in PERM_COLUMNS])
    ncol, chunk, bf = len(PERM_COLUMNS), case["chunk_len"], 3
    sets = (ncol + chunk - 1) // chunk
    beta, gamma = orc.fr_random(2, rng)
    delta = orc.fr_random(ncol, rng)
    blinds = orc.fr_random(sets * bf, rng)
    want = orc.fr_permutation_products(columns, trace["pk"], n_in, ncol, chunk, beta, gamma, trace["omega"], delta,
                                       blinds, bf)
    got = ctx.trace_permutation(advice, N_ADVICE, instance, N_INSTANCE, beta, gamma, delta, blinds, bf).download()
    assert (got == want).all()

    # lookup permutation: [inputs | tables | permuted inputs | permuted tables]
    u = n_in - 6
    nb = n_in - u
    ib, tb = orc.fr_random(LOOKUPS * nb, rng), orc.fr_random(LOOKUPS * nb, rng)
    got = ctx.trace_lookup_permute(advice, N_ADVICE, instance, N_INSTANCE, case["challenges"], case["theta"], u,
                                   ib, tb).download().reshape(4, LOOKUPS, n_in, 4)
    comp = np.concatenate([np.concatenate([trace["advice"][li], trace["fixed"][1 + li]]) for li in range(LOOKUPS)])
    perm = OracleBackend(None).permute_lookups(OracleBackend(None).put(comp), n_in, u, LOOKUPS, ib, tb).a
    perm = perm.reshape(LOOKUPS, 2, n_in, 4)
    for li in range(LOOKUPS):
        assert (got[0, li] == trace["advice"][li]).all()
        assert (got[1, li] == trace["fixed"][1 + li]).all()
        assert (got[2, li] == perm[li, 0]).all()
        assert (got[3, li] == perm[li, 1]).all()
    ctx.close()
