"""Trapdoor verifier for the synthetic PLONK/KZG proofs.

TEST INFRASTRUCTURE ONLY. The reference verifier needs a pairing
(plonk/verifier.rs, poly/kzg/mod.rs:1806-1976 multi_prepare followed by
the pairing check). The SRS of these tests comes from a known tau, so this
verifier replaces the pairing with the equivalent check in G1:

    (tau - x3) * pi == final_com - v * G

The transcript replay re-derives every challenge from the proof bytes. The
quotient identity at x is rebuilt from the evaluations in the proof:
gates, permutation and lookup terms folded with y
(evaluation.rs:3114-3528 at one point, plonk/verifier.rs). It is then
checked through the opening of h against the combined piece commitments.
"""
import hashlib

import numpy as np

from . import oracle as orc
from gb_prover.kzg import fr_from_uniform_bytes
from gb_prover.plonk import DELTA, R, ZETA, Domain, construct_intermediate_sets, fr_int, fr_mont
from gb_prover.rng import ints_to_mont


class ReadTranscript:
    """CircuitTranscript<Blake2bState> read side (transcript/mod.rs:95-150)."""

    KEY = b"Domain separator for transcript"

    def __init__(self, proof):
        self.state = hashlib.blake2b(digest_size=64, key=self.KEY)
        self.proof = bytes(proof)
        self.pos = 0

    def _absorb(self, b):
        self.state.update(b"\x01")
        self.state.update(b)

    def common_scalar(self, v):
        self._absorb(int(v % R).to_bytes(32, "little"))

    def read_point(self):
        b = self.proof[self.pos:self.pos + 48]
        if len(b) != 48:
            raise ValueError("proof too short")
        self.pos += 48
        self._absorb(b)
        return orc.g1_decompress(b)

    def read_scalar(self):
        b = self.proof[self.pos:self.pos + 32]
        if len(b) != 32:
            raise ValueError("proof too short")
        self.pos += 32
        v = int.from_bytes(b, "little")
        if v >= R:
            raise ValueError("non-canonical scalar")
        self._absorb(b)
        return v

    def squeeze(self):
        self.state.update(b"\x00")
        return fr_int(fr_from_uniform_bytes(self.state.digest()))


def _lin(points, scalars):
    """sum_i [s_i] P_i over affine points and integer scalars -> affine"""
    pts = np.ascontiguousarray(np.stack(points), dtype=np.uint64).reshape(-1, 12)
    jac = orc.g1_msm_naive(pts, ints_to_mont([s % R for s in scalars]))
    return orc.g1_to_affine(jac)[0]


def _lagrange_at(points, evals, z):
    """r(z) for the interpolating polynomial of (points, evals)"""
    acc = 0
    for i, (pi, ei) in enumerate(zip(points, evals)):
        num, den = 1, 1
        for j, pj in enumerate(points):
            if j != i:
                num = num * (z - pj) % R
                den = den * (pi - pj) % R
        acc = (acc + ei * num * pow(den, -1, R)) % R
    return acc


def verify(vk, proof, tau):
    """True when the proof verifies. vk carries the circuit (with its domain),
    fixed and sigma commitments and transcript_repr (a keygen ProvingKey
    works). Malformed proofs (short, bad encodings) verify False."""
    try:
        return _verify(vk, proof, tau)
    except ValueError:
        return False


def _verify(vk, proof, tau):
    c = vk.circuit
    dom = Domain(c.k, c.cs_degree)
    n, m, bf, L = c.n, c.m, c.blinding_factors, c.lookups
    sets = c.permutation_sets
    T = ReadTranscript(proof)
    T.common_scalar(vk.transcript_repr)
    adv_com = [T.read_point() for _ in range(m)]
    theta = T.squeeze()
    perm_com = [(T.read_point(), T.read_point()) for _ in range(L)]
    beta, gamma = T.squeeze(), T.squeeze()
    zp_com = [T.read_point() for _ in range(sets)]
    zl_com = [T.read_point() for _ in range(L)]
    T.squeeze()
    random_com = T.read_point()
    y = T.squeeze()
    pieces = dom.quotient_poly_degree
    h_com = [T.read_point() for _ in range(pieces)]
    x = T.squeeze()
    adv_ev = [T.read_scalar() for _ in c.advice_queries]
    fix_ev = [T.read_scalar() for _ in c.fixed_queries]
    random_eval = T.read_scalar()
    sig_ev = [T.read_scalar() for _ in range(m)]
    zp = []
    for s in range(sets):
        zx, zn = T.read_scalar(), T.read_scalar()
        zl = T.read_scalar() if s + 1 < sets else None
        zp.append((zx, zn, zl))
    lk = [tuple(T.read_scalar() for _ in range(5)) for _ in range(L)]

    # ---- the quotient identity at x
    xn = pow(x, n, R)
    vanish = (xn - 1) % R

    def l_i(i):
        wi = pow(dom.omega, i, R)
        return wi * vanish * pow(n * (x - wi) % R, -1, R) % R

    l0 = l_i(0)
    l_last = l_i(n - bf - 1)
    l_blind = sum(l_i(i) for i in range(n - bf, n)) % R
    l_active = (1 - l_last - l_blind) % R
    adv_map = {q: v for q, v in zip(c.advice_queries, adv_ev)}
    fix_map = {q: v for q, v in zip(c.fixed_queries, fix_ev)}
    fa = lambda col, rot: fix_map[(col, rot)]  # noqa: E731
    aa = lambda col, rot: adv_map[(col, rot)]  # noqa: E731
    acc = c.gate.evaluate(fa, aa)
    # permutation (permutation/verifier.rs expressions)
    acc = (acc * y + l0 * (1 - zp[0][0])) % R
    acc = (acc * y + l_last * (zp[-1][0] * zp[-1][0] - zp[-1][0])) % R
    for s in range(1, sets):
        acc = (acc * y + l0 * (zp[s][0] - zp[s - 1][2])) % R
    cur_delta = beta * x % R
    for s in range(sets):
        cols = c.permutation_columns[s * c.chunk_len:(s + 1) * c.chunk_len]
        left, right = zp[s][1], zp[s][0]
        for j in cols:
            v = adv_map[(j, 0)]
            left = left * (v + beta * sig_ev[j] + gamma) % R
            right = right * (v + cur_delta + gamma) % R
            cur_delta = cur_delta * DELTA % R
        acc = (acc * y + l_active * (left - right)) % R
    # lookups (lookup/verifier.rs expressions)
    for li, (ins, tab, _) in enumerate(c.lookup_args):
        z, zn, a_x, a_prev, s_x = lk[li]
        ci = 0
        for e in ins:
            ci = (ci * theta + e.evaluate(fa, aa)) % R
        ct = 0
        for e in tab:
            ct = (ct * theta + e.evaluate(fa, aa)) % R
        acc = (acc * y + l0 * (1 - z)) % R
        acc = (acc * y + l_last * (z * z - z)) % R
        acc = (acc * y + l_active * (zn * (a_x + beta) * (s_x + gamma) - z * (ci + beta) * (ct + gamma))) % R
        acc = (acc * y + l0 * (a_x - s_x)) % R
        acc = (acc * y + l_active * (a_x - s_x) * (a_x - a_prev)) % R
    h_eval = acc * pow(vanish, -1, R) % R
    split = pow(x, n - 1, R)
    h_combined = _lin(h_com, [pow(split, i, R) for i in range(pieces)])

    # ---- verifier queries, in the prover's order (prover.rs:1993-2063)
    x_next, x_prev, x_last = dom.rotate_omega(x, 1), dom.rotate_omega(x, -1), dom.rotate_omega(x, -(bf + 1))
    Q = []  # (label, commitment, point, eval)
    for (col, rot), v in zip(c.advice_queries, adv_ev):
        Q.append((("adv", col), adv_com[col], dom.rotate_omega(x, rot), v))
    for s in range(sets):
        Q.append((("zp", s), zp_com[s], x, zp[s][0]))
        Q.append((("zp", s), zp_com[s], x_next, zp[s][1]))
    for s in reversed(range(sets - 1)):
        Q.append((("zp", s), zp_com[s], x_last, zp[s][2]))
    for li in range(L):
        z, zn, a_x, a_prev, s_x = lk[li]
        Q += [(("zl", li), zl_com[li], x, z), (("a", li), perm_com[li][0], x, a_x), (("s", li), perm_com[li][1], x, s_x),
              (("a", li), perm_com[li][0], x_prev, a_prev), (("zl", li), zl_com[li], x_next, zn)]
    for (col, rot), v in zip(c.fixed_queries, fix_ev):
        Q.append((("fix", col), vk.fixed_commitments[col], dom.rotate_omega(x, rot), v))
    for i in range(m):
        Q.append((("sig", i), vk.sigma_commitments[i], x, sig_ev[i]))
    Q.append((("h",), h_combined, x, h_eval))
    Q.append((("rand",), random_com, x, random_eval))

    # ---- multi_prepare (poly/kzg/mod.rs:1806-1976) and the trapdoor check
    x1, x2 = T.squeeze(), T.squeeze()
    commits, set_of, point_sets = construct_intermediate_sets([(q[0], q[2]) for q in Q])
    com_pt = {}
    evals = {}
    for label, com, point, v in Q:
        com_pt[label] = com
        evals[(label, point)] = v
    nsets = len(point_sets)
    q_com, q_evals = [], []
    for sid in range(nsets):
        labels = [commits[i] for i, s in enumerate(set_of) if s == sid]
        q_com.append(_lin([com_pt[lb] for lb in labels], [pow(x1, i, R) for i in range(len(labels))]))
        q_evals.append([sum(pow(x1, i, R) * evals[(lb, p)] for i, lb in enumerate(labels)) % R
                        for p in point_sets[sid]])
    order = sorted(range(nsets), key=lambda i: (len(point_sets[i]), i))
    q_com = [q_com[i] for i in order]
    q_evals = [q_evals[i] for i in order]
    point_sets = [point_sets[i] for i in order]
    f_com = T.read_point()
    x3 = T.squeeze()
    q_on_x3 = [T.read_scalar() for _ in range(nsets)]
    f_eval = 0
    for pts, ev, pe in reversed(list(zip(point_sets, q_evals, q_on_x3))):
        r_eval = _lagrange_at(pts, ev, x3)
        den = 1
        for p in pts:
            den = den * (x3 - p) % R
        f_eval = (f_eval * x2 + (pe - r_eval) * pow(den, -1, R)) % R
    x4 = T.squeeze()
    final_com = _lin(q_com + [f_com], [pow(x4, i, R) for i in range(nsets + 1)])
    v = sum(pow(x4, i, R) * e for i, e in enumerate(q_on_x3 + [f_eval])) % R
    pi = T.read_point()
    if T.pos != len(T.proof):
        return False
    lhs = _lin([pi], [(tau - x3) % R])
    g = orc.g1_generator()
    rhs = _lin([final_com, g], [1, (-v) % R])
    return bool((lhs == rhs).all())
