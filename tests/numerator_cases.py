"""Seeded synthetic inputs for the quotient-numerator tests: random compiled
gate graphs and random column data, described once and handed both to the
oracle and to the C ABI."""
import numpy as np


def random_graph(rng, fr_random, ncols, nconst=4, nrot=3, ncalc=24, nint=12):
    """A random well-formed graph: sources refer to constants, columns at
    random rotations, challenges, the named scalars and earlier
    intermediates; every op kind including Horner appears."""
    consts = fr_random(nconst, rng)
    rots = [0] + [int(r) for r in rng.integers(-3, 4, size=nrot - 1)]
    calcs, parts = [], []
    written = []

    def src():
        choice = rng.integers(0, 10)
        if choice == 0:
            return (0, int(rng.integers(0, nconst)), 0)
        if choice in (1, 2) and written:
            return (1, int(rng.choice(written)), 0)
        if choice in (3, 4):
            return (2, int(rng.integers(0, ncols[0])), int(rng.integers(0, nrot)))
        if choice in (5, 6):
            return (3, int(rng.integers(0, ncols[1])), int(rng.integers(0, nrot)))
        if choice == 7:
            return (4, int(rng.integers(0, ncols[2])), int(rng.integers(0, nrot)))
        if choice == 8:
            return (5, int(rng.integers(0, 2)), 0)
        return (int(rng.integers(6, 11)), 0, 0)

    for c in range(ncalc):
        op = int(rng.integers(0, 8)) if c else 2
        tgt = int(rng.integers(0, nint))
        if op == 6:
            k = int(rng.integers(1, 4))
            calcs.append((op, tgt, len(parts), k, src(), src()))
            parts += [src() for _ in range(k)]
        else:
            calcs.append((op, tgt, 0, 0, src(), src()))
        written.append(tgt)
    return consts, rots, calcs, parts, nint


def random_case(rng, fr_random, length, n_fixed=3, n_advice=3, n_instance=1, sets=2, chunk=2, lookups=1, trash=1):
    case = {
        "length": length,
        "fixed": fr_random(n_fixed * length, rng),
        "advice": fr_random(n_advice * length, rng),
        "instance": fr_random(n_instance * length, rng),
        "challenges": fr_random(2, rng),
        "rot_scale": 4,
        "last_rotation": -5,
        "chunk_len": chunk,
    }
    for k in ("beta", "gamma", "theta", "trash_challenge", "y", "omega", "delta_start", "delta_const"):
        case[k] = fr_random(1, rng)[0]
    for k in ("l0", "l_last", "l_active"):
        case[k] = fr_random(length, rng)
    ncols = (n_fixed, n_advice, n_instance)
    case["graphs"] = {"custom": random_graph(rng, fr_random, ncols),
                      "lookups": [random_graph(rng, fr_random, ncols, ncalc=8, nint=6) for _ in range(lookups)],
                      "trash": [random_graph(rng, fr_random, ncols, ncalc=6, nint=4) for _ in range(trash)]}
    ncol = sets * chunk - 1
    case["permutation_sets"] = sets
    case["permutation_columns"] = [(int(rng.integers(0, 3)), int(rng.integers(0, 3))) for _ in range(ncol)]
    case["permutation_products"] = fr_random(sets * length, rng)
    case["permutation_pk_cosets"] = fr_random(ncol * length, rng)
    case["lookup_data"] = [tuple(fr_random(length, rng) for _ in range(3)) for _ in range(lookups)]
    case["trash_data"] = [(fr_random(length, rng), int(rng.integers(0, n_fixed))) for _ in range(trash)]
    return case


def call(case, eval_fn, graph_cls, run_custom=True, initial_out=None):
    G = case["graphs"]
    kw = {k: case[k] for k in ("fixed", "advice", "instance", "challenges", "beta", "gamma", "theta",
                               "trash_challenge", "y", "omega", "delta_start", "delta_const", "rot_scale",
                               "last_rotation", "chunk_len", "l0", "l_last", "l_active", "permutation_products",
                               "permutation_sets", "permutation_columns", "permutation_pk_cosets")}
    kw["lookups"] = [(graph_cls(*g),) + d for g, d in zip(G["lookups"], case["lookup_data"])]
    kw["trash"] = [(graph_cls(*g), d[0], d[1]) for g, d in zip(G["trash"], case["trash_data"])]
    kw["initial_out"] = initial_out
    return eval_fn(case["length"], graph_cls(*G["custom"]) if run_custom else None, **kw)
