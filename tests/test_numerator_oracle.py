"""The oracle's quotient numerator against an independent Python-integer
restatement of evaluation.rs:3114-3528 on a small random case, and the
custom-gate graph vanishing on rows that satisfy the standard PLONK gate."""
import numpy as np

from numerator_cases import random_case

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def _py_graph(g, cols, n, idx, rot_scale, chal, named, prev, ints):
    consts, rots, calcs, parts, nint = g
    consts = ints(consts)
    inter = [0] * nint

    def val(s):
        k, a, b = s
        if k == 0:
            return consts[a]
        if k == 1:
            return inter[a]
        if k in (2, 3, 4):
            col = cols[k - 2][a]
            return col[(idx + rots[b] * rot_scale) % n]
        if k == 5:
            return chal[a]
        if k == 11:
            return prev
        return named[k]

    last = 0
    for op, tgt, po, pl, lhs, rhs in calcs:
        if op == 0:
            v = (val(lhs) + val(rhs)) % R
        elif op == 1:
            v = (val(lhs) - val(rhs)) % R
        elif op == 2:
            v = val(lhs) * val(rhs) % R
        elif op == 3:
            v = val(lhs) ** 2 % R
        elif op == 4:
            v = 2 * val(lhs) % R
        elif op == 5:
            v = -val(lhs) % R
        elif op == 6:
            f = val(rhs)
            v = val(lhs)
            for k in range(pl):
                v = (v * f + val(parts[po + k])) % R
        else:
            v = val(lhs)
        inter[tgt] = v
        last = v
    return last


def _py_numerator(case, orc):
    ints = orc.fr_to_ints
    n = case["length"]
    split = lambda a: [ints(a[i * n:(i + 1) * n]) for i in range(len(a) // n)]  # noqa: E731
    cols = [split(case["fixed"]), split(case["advice"]), split(case["instance"])]
    chal = ints(case["challenges"])
    s = {k: ints(case[k])[0] for k in ("beta", "gamma", "theta", "trash_challenge", "y", "omega", "delta_start",
                                        "delta_const")}
    named = {6: s["beta"], 7: s["gamma"], 8: s["theta"], 9: s["trash_challenge"], 10: s["y"]}
    l0, ll, la = ints(case["l0"]), ints(case["l_last"]), ints(case["l_active"])
    pp = split(case["permutation_products"])
    pk = split(case["permutation_pk_cosets"])
    rs, y = case["rot_scale"], s["y"]
    out = []
    for idx in range(n):
        v = _py_graph(case["graphs"]["custom"], cols, n, idx, rs, chal, named, 0, ints)
        r_next, r_last = (idx + rs) % n, (idx + case["last_rotation"] * rs) % n
        v = (v * y + (1 - pp[0][idx]) * l0[idx]) % R
        v = (v * y + (pp[-1][idx] ** 2 - pp[-1][idx]) * ll[idx]) % R
        for st in range(1, len(pp)):
            v = (v * y + (pp[st][idx] - pp[st - 1][r_last]) * l0[idx]) % R
        delta = s["delta_start"] * pow(s["omega"], idx, R) % R
        cl, chunk = case["permutation_columns"], case["chunk_len"]
        for st in range(len(pp)):
            left, right = pp[st][r_next], pp[st][idx]
            for j in range(chunk):
                c = st * chunk + j
                if c >= len(cl):
                    break
                kind, ci = cl[c]
                if ci >= len(cols[kind]):
                    continue  # an unknown column contributes nothing (.cu:664-757 behaviour)
                col = cols[kind][ci]
                left = left * (col[idx] + s["beta"] * pk[c][idx] + s["gamma"]) % R
                right = right * (col[idx] + delta + s["gamma"]) % R
                delta = delta * s["delta_const"] % R
            v = (v * y + (left - right) * la[idx]) % R
        for g, (prod, pin, ptab) in zip(case["graphs"]["lookups"], case["lookup_data"]):
            prod, pin, ptab = ints(prod), ints(pin), ints(ptab)
            tv = _py_graph(g, cols, n, idx, rs, chal, named, 0, ints)
            ams = (pin[idx] - ptab[idx]) % R
            rp = (idx - rs) % n
            v = (v * y + (1 - prod[idx]) * l0[idx]) % R
            v = (v * y + (prod[idx] ** 2 - prod[idx]) * ll[idx]) % R
            v = (v * y + (prod[r_next] * (pin[idx] + s["beta"]) * (ptab[idx] + s["gamma"]) - prod[idx] * tv)
                 * la[idx]) % R
            v = (v * y + ams * l0[idx]) % R
            v = (v * y + ams * (pin[idx] - pin[rp]) * la[idx]) % R
        for g, (tc, sel) in zip(case["graphs"]["trash"], case["trash_data"]):
            comp = _py_graph(g, cols, n, idx, rs, chal, named, 0, ints)
            q = cols[0][sel][idx]
            v = (v * y + comp - (1 - q) * ints(tc)[idx]) % R
        out.append(v)
    return out


def test_oracle_numerator_matches_python(orc):
    from numerator_cases import call
    rng = np.random.default_rng(31)
    case = random_case(rng, orc.fr_random, 32)
    got = call(case, orc.eval_numerator, orc.OracleGraph)
    assert orc.fr_to_ints(got) == _py_numerator(case, orc)
    # run_custom = 0 starts from initial_out
    init = orc.fr_random(32, rng)
    got2 = call(case, orc.eval_numerator, orc.OracleGraph, run_custom=False, initial_out=init)
    assert got2.shape == (32, 4)


def test_standard_gate_vanishes_on_satisfied_rows(orc):
    """q_l*a + q_r*b + q_o*c + q_m*a*b + q_c = 0 (the synthetic circuit's gate)
    compiled as a graph evaluates to zero on every satisfying row."""
    rng = np.random.default_rng(5)
    n = 64
    ql, qr, qo, qm, qc, a, b = (orc.fr_to_ints(orc.fr_random(n, rng)) for _ in range(7))
    c = [(-(ql[i] * a[i] + qr[i] * b[i] + qm[i] * a[i] * b[i] + qc[i]) * pow(qo[i], -1, R)) % R for i in range(n)]
    fixed = orc.fr_from_ints(ql + qr + qo + qm + qc)
    advice = orc.fr_from_ints(a + b + c)
    F, A = 2, 3
    calcs = [
        (2, 0, 0, 0, (F, 0, 0), (A, 0, 0)),   # ql*a
        (2, 1, 0, 0, (F, 1, 0), (A, 1, 0)),   # qr*b
        (2, 2, 0, 0, (F, 2, 0), (A, 2, 0)),   # qo*c
        (2, 3, 0, 0, (A, 0, 0), (A, 1, 0)),   # a*b
        (2, 3, 0, 0, (F, 3, 0), (1, 3, 0)),   # qm*a*b
        (0, 4, 0, 0, (1, 0, 0), (1, 1, 0)),
        (0, 4, 0, 0, (1, 4, 0), (1, 2, 0)),
        (0, 4, 0, 0, (1, 4, 0), (1, 3, 0)),
        (0, 4, 0, 0, (1, 4, 0), (F, 4, 0)),
    ]
    g = orc.OracleGraph(np.zeros((0, 4), np.uint64), [0], calcs, [], 5)
    out = orc.eval_numerator(n, g, fixed=fixed, advice=advice)
    assert (out == 0).all()
