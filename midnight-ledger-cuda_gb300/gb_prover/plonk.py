"""Synthetic PLONK/KZG proofs through the GPU prover path.

This module drives one PLONK proof over the C ABI. It follows
vendor/midnight-proofs-0.8.1/src/plonk/prover.rs:68-1081 (compute_trace +
finalise_proof) for circuits that have advice columns, one custom gate,
copy constraints and lookups, and no instance columns or trash arguments.
Each step issues the same transcript operations in the reference's order:

  * vk hash: common(transcript_repr)                         prover.rs:111-114
  * advice: blind the last bf+1 rows, commit_lagrange, write  prover.rs:1342-1720
  * theta; per lookup: A', S' (permute_expression_pair),
    commit_lagrange both, write                               lookup/prover.rs:688-733,1573-1690
  * beta, gamma; permutation blinds, lookup blinds; the
    permutation products z, then the lookup products z,
    commit_lagrange, write                                    prover.rs:186-341
  * trash challenge; vanishing random poly, commit, write     vanishing/prover.rs:41-97
  * y; the quotient numerator on the extended coset, divide by
    t(X), back to coefficients, split into pieces, blind, commit
    and write                                                 evaluation.rs:3114-3528, vanishing/prover.rs:99-220
  * x; evaluations of advice, fixed, random poly, sigma,
    permutation and lookup polynomials, written in order      prover.rs:1940-1990, permutation/prover.rs:545-670,
                                                              lookup/prover.rs:1341-1520
  * multi_open (x1, x2, f, x3, q evals, x4, pi)              poly/kzg/mod.rs:1978-2600

The driver is written against a backend with polynomial-level operations.
The product backend is `GpuBackend`: device vectors, resident MSM contexts
and CUDA kernels behind the C ABI. The same driver with another backend
gives the same bytes when every operation is exact, and the tests use this
to compare proofs.

Deviations from the reference, each kept deliberately:
  * The random polynomial of the vanishing argument draws its n values from
    the prover rng in order. The reference seeds one ChaCha20 stream per
    rayon thread (vanishing/prover.rs:41-75), so its bytes depend on the
    host's thread count.
  * transcript_repr is the Blake2b-512 ("Halo2-Verify-Key") hash of this
    module's canonical verifying-key bytes, mapped by from_uniform_bytes. It
    has the same role as the reference's hash of the pinned vk debug string.
"""
import hashlib
import struct

import numpy as np

from . import api
from .graph import (ADD, BETA, CONSTANT, DOUBLE, FIXED, ADVICE, INSTANCE, GAMMA, HORNER, INTERMEDIATE, MUL,
                    NEGATE, PREVIOUS, SQUARE, STORE, SUB, THETA, Y, Graph)
from .kzg import CircuitTranscript, ParamsKZG, affine_from_projective_batch, compress, fr_to_repr
from .rng import R2_LIMBS, ChaCha20Rng, fr_random, fr_random_raw, ints_to_mont, mont_to_ints

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
S_TWO_ADICITY = 32
GENERATOR = 7
ROOT_OF_UNITY = pow(GENERATOR, (R - 1) >> 32, R)       # fq.rs:70
DELTA = pow(GENERATOR, 1 << 32, R)                     # fq.rs:481-501
ZETA = pow(GENERATOR, (R - 1) // 3, R)                 # fq.rs:693-702, cube root of unity


def fr_mont(v):
    """one canonical integer -> Montgomery (4,) limbs"""
    return ints_to_mont([v % R])[0]


def fr_int(row):
    return mont_to_ints(np.asarray(row, dtype=np.uint64).reshape(1, 4))[0]


def omega_for(k):
    return pow(ROOT_OF_UNITY, 1 << (S_TWO_ADICITY - k), R)


# ---------------------------------------------------------------- domain

class Domain:
    """EvaluationDomain::new(j, k) (poly/domain.rs:54-159)."""

    def __init__(self, k, j):
        self.k, self.n = k, 1 << k
        self.quotient_poly_degree = j - 1
        ek = k
        while (1 << ek) < self.n * self.quotient_poly_degree:
            ek += 1
        self.extended_k = ek
        self.extended_len = 1 << ek
        self.omega = omega_for(k)
        self.omega_inv = pow(self.omega, -1, R)
        self.extended_omega = omega_for(ek)
        orig = pow(ZETA, self.n, R)
        step = pow(self.extended_omega, self.n, R)
        t, cur = [], orig
        while True:
            t.append(cur)
            cur = cur * step % R
            if cur == orig:
                break
        assert len(t) == 1 << (ek - k)
        self.t_evaluations_inv = [pow((v - 1) % R, -1, R) for v in t]

    def rotate_omega(self, x, rot):
        return x * pow(self.omega if rot >= 0 else self.omega_inv, abs(rot), R) % R


# ---------------------------------------------------------------- expressions

class Expr:
    """plonk/circuit.rs:970-993 Expression (no selectors, no challenges)."""
    __slots__ = ("op", "a", "b")

    def __init__(self, op, a=None, b=None):
        self.op, self.a, self.b = op, a, b

    @staticmethod
    def const(v):
        return Expr("const", v % R)

    @staticmethod
    def fixed(col, rot=0):
        return Expr("fixed", col, rot)

    @staticmethod
    def advice(col, rot=0):
        return Expr("advice", col, rot)

    def __add__(self, o):
        return Expr("sum", self, o)

    def __sub__(self, o):
        return Expr("sum", self, Expr("neg", o))

    def __neg__(self):
        return Expr("neg", self)

    def __mul__(self, o):
        if isinstance(o, Expr):
            return Expr("prod", self, o)
        return Expr("scaled", self, o % R)

    def degree(self):
        if self.op in ("const",):
            return 0
        if self.op in ("fixed", "advice", "instance"):
            return 1
        if self.op in ("neg", "scaled"):
            return self.a.degree()
        if self.op == "sum":
            return max(self.a.degree(), self.b.degree())
        return self.a.degree() + self.b.degree()

    def evaluate(self, fixed, advice):
        """value from query callbacks fixed(col, rot), advice(col, rot)"""
        op = self.op
        if op == "const":
            return self.a
        if op == "fixed":
            return fixed(self.a, self.b)
        if op == "advice":
            return advice(self.a, self.b)
        if op == "neg":
            return -self.a.evaluate(fixed, advice) % R
        if op == "sum":
            return (self.a.evaluate(fixed, advice) + self.b.evaluate(fixed, advice)) % R
        if op == "prod":
            return self.a.evaluate(fixed, advice) * self.b.evaluate(fixed, advice) % R
        return self.a.evaluate(fixed, advice) * self.b % R


class GraphBuilder:
    """GraphEvaluator (evaluation.rs:3531-3790): constants start [0, 1, 2];
    calculations are deduplicated; add_expression simplifies exactly like the
    reference so graphs have the reference's shape. Value sources are
    (kind, a, b) tuples whose tuple order is the derived order of ValueSource."""

    def __init__(self):
        self.constants = [0, 1, 2]
        self.rotations = []
        self.calcs = []          # (calculation, target)
        self.num_intermediates = 0

    def add_rotation(self, rot):
        if rot not in self.rotations:
            self.rotations.append(rot)
        return self.rotations.index(rot)

    def add_constant(self, c):
        c %= R
        if c not in self.constants:
            self.constants.append(c)
        return (CONSTANT, self.constants.index(c), 0)

    def add_calculation(self, calc):
        for existing, target in self.calcs:
            if existing == calc:
                return (INTERMEDIATE, target, 0)
        target = self.num_intermediates
        self.calcs.append((calc, target))
        self.num_intermediates += 1
        return (INTERMEDIATE, target, 0)

    def add_expression(self, e):
        op = e.op
        zero, one, two = (CONSTANT, 0, 0), (CONSTANT, 1, 0), (CONSTANT, 2, 0)
        if op == "const":
            return self.add_constant(e.a)
        if op in ("fixed", "advice", "instance"):
            kind = {"fixed": FIXED, "advice": ADVICE, "instance": INSTANCE}[op]
            return self.add_calculation((STORE, (kind, e.a, self.add_rotation(e.b))))
        if op == "neg":
            if e.a.op == "const":
                return self.add_constant(-e.a.a)
            ra = self.add_expression(e.a)
            return ra if ra == zero else self.add_calculation((NEGATE, ra))
        if op == "sum":
            if e.b.op == "neg":
                ra, rb = self.add_expression(e.a), self.add_expression(e.b.a)
                if ra == zero:
                    return self.add_calculation((NEGATE, rb))
                if rb == zero:
                    return ra
                return self.add_calculation((SUB, ra, rb))
            ra, rb = self.add_expression(e.a), self.add_expression(e.b)
            if ra == zero:
                return rb
            if rb == zero:
                return ra
            return self.add_calculation((ADD, ra, rb) if ra <= rb else (ADD, rb, ra))
        if op == "prod":
            ra, rb = self.add_expression(e.a), self.add_expression(e.b)
            if ra == zero or rb == zero:
                return zero
            if ra == one:
                return rb
            if rb == one:
                return ra
            if ra == two:
                return self.add_calculation((DOUBLE, rb))
            if rb == two:
                return self.add_calculation((DOUBLE, ra))
            if ra == rb:
                return self.add_calculation((SQUARE, ra))
            return self.add_calculation((MUL, ra, rb) if ra <= rb else (MUL, rb, ra))
        # scaled
        if e.b == 0:
            return zero
        if e.b == 1:
            return self.add_expression(e.a)
        cst = self.add_constant(e.b)
        ra = self.add_expression(e.a)
        return self.add_calculation((MUL, ra, cst))

    def horner(self, start, parts, factor):
        return self.add_calculation((HORNER, start, tuple(parts), factor))

    def compile(self, graph_cls=Graph):
        """Flatten into the RawGraph arrays (lib.rs:38-79).  A builder is
        complete once its key is made, so the flattened graph is kept and
        returned again by later calls (proofs reuse their key's graphs)."""
        key = (graph_cls, len(self.calcs), len(self.constants), len(self.rotations), self.num_intermediates)
        cached = getattr(self, "_compiled", None)
        if cached is not None and cached[0] == key:
            return cached[1]
        graph = self._compile(graph_cls)
        self._compiled = (key, graph)
        return graph

    def _compile(self, graph_cls):
        none = (0, 0, 0)
        calcs, parts = [], []
        for calc, target in self.calcs:
            op = calc[0]
            if op == HORNER:
                _, start, ps, factor = calc
                calcs.append((op, target, len(parts), len(ps), start, factor))
                parts.extend(ps)
            elif op in (ADD, SUB, MUL):
                calcs.append((op, target, 0, 0, calc[1], calc[2]))
            else:
                calcs.append((op, target, 0, 0, calc[1], none))
        return graph_cls(ints_to_mont(self.constants), self.rotations, calcs, parts, self.num_intermediates)


# ---------------------------------------------------------------- circuits

class SyntheticCircuit:
    """A seeded synthetic circuit.

    It has m advice columns a_0..a_{m-1}, all in the permutation, and one
    gate of degree d:

        sum_i q_i * a_i + q_m * prod_{j < d-1} a_{j mod (m-1)} + q_c = 0

    The witness is solved for a_{m-1} on every usable row. Each lookup l
    constrains (q_lk_l * a_{2l mod (m-1)}, q_lk_l * a_{(2l+1) mod (m-1)}) to
    lie in the fixed table (t_l0, t_l1) of 2^table_log rows, whose row 0 is
    (0, 0).

    Copy constraints link random earlier cells to free later cells, so they
    hold by construction. With m = 3 and d = 3 the gate is
    q_l*a + q_r*b + q_o*c + q_m*a*b + q_c.

    Fixed columns: q_0..q_{m-1}, q_m, q_c, then (q_lk, t0, t1) per lookup.
    """

    def __init__(self, k, advice=3, degree=3, lookups=1, copies=1 << 14, table_log=12, label="synthetic"):
        if advice < 2 or degree < 2:
            raise ValueError("need at least 2 advice columns and gate degree 2")
        if lookups and advice < 3:
            raise ValueError("lookups need at least 3 advice columns (two inputs and the solved column)")
        self.k, self.n = k, 1 << k
        self.m, self.d, self.lookups, self.copies, self.table_log = advice, degree, lookups, copies, table_log
        self.label = label
        m = advice
        self.num_fixed = m + 2 + 3 * lookups
        q = [Expr.fixed(i) for i in range(m)]
        a = [Expr.advice(i) for i in range(m)]
        qm, qc = Expr.fixed(m), Expr.fixed(m + 1)
        gate = q[0] * a[0]
        for i in range(1, m):
            gate = gate + q[i] * a[i]
        prod = qm
        for j in range(degree - 1):
            prod = prod * a[j % (m - 1)]
        self.gate = gate + prod + qc
        self.lookup_args = []
        for l_ in range(lookups):
            base = m + 2 + 3 * l_
            qlk = Expr.fixed(base)
            c0, c1 = (2 * l_) % (m - 1), (2 * l_ + 1) % (m - 1)
            self.lookup_args.append(([qlk * a[c0], qlk * a[c1]], [Expr.fixed(base + 1), Expr.fixed(base + 2)], (c0, c1)))
        # query lists in registration order (plonk/circuit.rs query_* order)
        self.advice_queries = [(i, 0) for i in range(m)]
        self.fixed_queries = [(i, 0) for i in range(self.num_fixed)]
        self.permutation_columns = list(range(m))
        # ConstraintSystem::degree / blinding_factors (plonk/circuit.rs:2483-2535)
        lookup_deg = max([max(4, 2 + max([1] + [e.degree() for e in ins]) + max([1] + [e.degree() for e in tab]))
                          for ins, tab, _ in self.lookup_args] or [0])
        self.cs_degree = max(3, lookup_deg, self.gate.degree())
        self.blinding_factors = max(3, 1) + 0 + 1 + 1
        self.usable_rows = self.n - (self.blinding_factors + 1)
        self.chunk_len = self.cs_degree - 2
        self.permutation_sets = -(-m // self.chunk_len)
        if (1 << table_log) > self.usable_rows:
            raise ValueError("lookup table does not fit the usable rows")

    def describe(self):
        return "m=%d d=%d lookups=%d copies=%d table=2^%d k=%d" % (self.m, self.d, self.lookups, self.copies,
                                                                     self.table_log, self.k)

    def synthesize(self, seed_label=None):
        """(fixed [num_fixed][n] ints, advice [m][n] ints with zero blinding rows, copies [(src, dst)])."""
        rng = ChaCha20Rng.from_label(seed_label or self.label)
        n, m, u = self.n, self.m, self.usable_rows
        fixed = [[0] * n for _ in range(self.num_fixed)]
        sel = mont_to_ints(fr_random(rng, u * (m + 2)))
        for c in range(m + 2):
            fixed[c][:u] = sel[c * u:(c + 1) * u]
        tsize = 1 << self.table_log
        lookup_row = [-1] * n
        table_pick = [0] * n
        rows = rng.next_u64_array(u * max(self.lookups, 1) + 1)
        for l_ in range(self.lookups):
            base = m + 2 + 3 * l_
            fixed[base + 1][:tsize] = list(range(tsize))
            t1 = mont_to_ints(fr_random(rng, tsize))
            t1[0] = 0
            fixed[base + 2][:tsize] = t1
        # each usable row belongs to at most one lookup; a quarter of the rows per lookup
        for r in range(u):
            v = int(rows[r])
            if self.lookups and (v & 3) == 0:
                l_ = (v >> 2) % self.lookups
                lookup_row[r] = l_
                table_pick[r] = (v >> 8) % tsize
                fixed[m + 2 + 3 * l_][r] = 1
        # free cells: columns 0..m-2 not pinned by the row's lookup
        pinned = set()
        for r in range(u):
            if lookup_row[r] >= 0:
                c0, c1 = self.lookup_args[lookup_row[r]][2]
                pinned.add((c0, r))
                pinned.add((c1, r))
        picks = rng.next_u64_array(3 * self.copies + 16)
        copies, used, pi = [], set(), 0
        while len(copies) < self.copies and pi + 2 < len(picks):
            dr = 1 + int(picks[pi]) % (u - 1)
            dc = int(picks[pi + 1]) % (m - 1)
            src = int(picks[pi + 2]) % (dr * m)
            pi += 3
            if (dc, dr) in pinned or (dc, dr) in used:
                continue
            used.add((dc, dr))
            copies.append(((src % m, src // m), (dc, dr)))
        if len(copies) < self.copies:
            picks = rng.next_u64_array(3 * self.copies)
            pi = 0
            while len(copies) < self.copies:
                dr = 1 + int(picks[pi % len(picks)]) % (u - 1)
                dc = int(picks[(pi + 1) % len(picks)]) % (m - 1)
                src = int(picks[(pi + 2) % len(picks)]) % (dr * m)
                pi += 3
                if (dc, dr) in pinned or (dc, dr) in used:
                    continue
                used.add((dc, dr))
                copies.append(((src % m, src // m), (dc, dr)))
        copy_src = {dst: src for src, dst in copies}
        free_vals = mont_to_ints(fr_random(rng, u * (m - 1)))
        advice = [[0] * n for _ in range(m)]
        tabs = [(fixed[m + 2 + 3 * l_ + 1], fixed[m + 2 + 3 * l_ + 2]) for l_ in range(self.lookups)]
        q_last_inv = _batch_inv(fixed[m - 1][:u])
        for r in range(u):
            for c in range(m - 1):
                advice[c][r] = free_vals[r * (m - 1) + c]
            if lookup_row[r] >= 0:
                l_ = lookup_row[r]
                c0, c1 = self.lookup_args[l_][2]
                advice[c0][r] = tabs[l_][0][table_pick[r]]
                advice[c1][r] = tabs[l_][1][table_pick[r]]
            for c in range(m - 1):
                s = copy_src.get((c, r))
                if s is not None:
                    advice[c][r] = advice[s[0]][s[1]]
            acc = fixed[m + 1][r]
            for c in range(m - 1):
                acc += fixed[c][r] * advice[c][r]
            p = fixed[m][r]
            for j in range(self.d - 1):
                p = p * advice[j % (m - 1)][r] % R
            acc = (acc + p) % R
            advice[m - 1][r] = -acc * q_last_inv[r] % R
        return fixed, advice, copies

    def check_witness(self, fixed, advice):
        """gate and lookup satisfied on every usable row (host check)"""
        for r in range(self.usable_rows):
            v = self.gate.evaluate(lambda c, rot: fixed[c][r], lambda c, rot: advice[c][r])
            if v:
                return False
        for ins, tab, _ in self.lookup_args:
            table = {(tab[0].evaluate(lambda c, rot: fixed[c][r], None), tab[1].evaluate(lambda c, rot: fixed[c][r], None))
                     for r in range(self.usable_rows)}
            for r in range(self.usable_rows):
                key = tuple(e.evaluate(lambda c, rot: fixed[c][r], lambda c, rot: advice[c][r]) for e in ins)
                if key not in table:
                    return False
        return True


def _batch_inv(vals):
    """Montgomery's trick over Python ints (zero maps to zero)"""
    pref, acc = [], 1
    for v in vals:
        pref.append(acc)
        if v:
            acc = acc * v % R
    inv = pow(acc, -1, R)
    out = [0] * len(vals)
    for i in range(len(vals) - 1, -1, -1):
        v = vals[i]
        if v:
            out[i] = inv * pref[i] % R
            inv = inv * v % R
    return out


class PermutationAssembly:
    """permutation::keygen::Assembly (plonk/permutation/keygen.rs:20-110):
    cycles over (column, row) cells, merged smaller into larger."""

    def __init__(self, n, columns):
        self.n, self.cols = n, columns
        self.mapping = [[(i, j) for j in range(n)] for i in range(columns)]
        self.aux = [[(i, j) for j in range(n)] for i in range(columns)]
        self.sizes = [[1] * n for _ in range(columns)]

    def copy(self, lc, lr, rc, rr):
        left, right = self.aux[lc][lr], self.aux[rc][rr]
        if left == right:
            return
        if self.sizes[left[0]][left[1]] < self.sizes[right[0]][right[1]]:
            left, right = right, left
        self.sizes[left[0]][left[1]] += self.sizes[right[0]][right[1]]
        i = right
        while True:
            self.aux[i[0]][i[1]] = left
            i = self.mapping[i[0]][i[1]]
            if i == right:
                break
        self.mapping[lc][lr], self.mapping[rc][rr] = self.mapping[rc][rr], self.mapping[lc][lr]

    def sigma_values(self, omega):
        """build_pk (keygen.rs:138-200): sigma_i[j] = delta^{i'} omega^{j'} of mapping (i', j')"""
        n = self.n
        wp = [1] * n
        for j in range(1, n):
            wp[j] = wp[j - 1] * omega % R
        dp = [pow(DELTA, i, R) for i in range(self.cols)]
        return [[dp[pc] * wp[pr] % R for (pc, pr) in self.mapping[i]] for i in range(self.cols)]


# ---------------------------------------------------------------- keys

class ProvingKey:
    """Fixed and permutation data of a circuit: Lagrange values, coefficient
    forms and extended cosets (backend handles), commitments, and the
    compiled numerator graphs (keygen.rs:307-430)."""

    def device_bytes(self):
        """device memory held by the key's resident vectors"""
        return sum(32 * v.len for v in vars(self).values() if hasattr(v, "len") and hasattr(v, "raw"))


def keygen(params, circuit, backend, fixed=None, copies=None):
    """keygen_vk + keygen_pk for a synthetic circuit (plonk/keygen.rs:240-430)."""
    if fixed is None or copies is None:
        fixed, _, copies = circuit.synthesize()
    n, k = circuit.n, circuit.k
    dom = Domain(k, circuit.cs_degree)
    fixed_vals = ints_to_mont([v for col in fixed for v in col])
    # permutation (permutation/keygen.rs): sigma values from the copy cycles
    asm = PermutationAssembly(n, circuit.m)
    for (sc, sr), (dc, dr) in copies:
        asm.copy(sc, sr, dc, dr)
    sigma = asm.sigma_values(dom.omega)
    return keygen_from_values(params, circuit, backend, fixed_vals, ints_to_mont([v for col in sigma for v in col]))


def keygen_from_values(params, circuit, backend, fixed_vals, sigma_vals, fixed_commitments=None,
                       sigma_commitments=None):
    """The resident proving key from the fixed columns' and the permutation's
    Lagrange values (Montgomery rows, [num_fixed][n] and [m][n]), as
    ProvingKey::read rebuilds it from a key file (plonk/mod.rs:538-590):
    coefficient forms and extended cosets of both, l0 / l_last / l_active,
    the compiled graphs; the commitments are computed unless given (the file's
    verifying key carries them)."""
    n, k = circuit.n, circuit.k
    dom = Domain(k, circuit.cs_degree)
    pk = ProvingKey()
    pk.circuit, pk.domain = circuit, dom
    bf = circuit.blinding_factors
    # fixed: values, coefficients, extended cosets, Lagrange commitments
    pk.fixed_lagrange = backend.put(np.ascontiguousarray(fixed_vals, dtype=np.uint64).reshape(-1, 4))
    pk.fixed_coeffs = backend.lagrange_to_coeff(pk.fixed_lagrange, k, circuit.num_fixed)
    pk.fixed_cosets = backend.coeff_to_extended(pk.fixed_coeffs, k, circuit.num_fixed, dom.extended_k)
    pk.fixed_commitments = (backend.commit_lagrange(pk.fixed_lagrange, n, circuit.num_fixed)
                            if fixed_commitments is None else list(fixed_commitments))
    # permutation
    pk.sigma_lagrange_host = np.ascontiguousarray(sigma_vals, dtype=np.uint64).reshape(-1, 4)
    pk.sigma_lagrange = backend.put(pk.sigma_lagrange_host)
    pk.sigma_coeffs = backend.lagrange_to_coeff(pk.sigma_lagrange, k, circuit.m)
    pk.sigma_cosets = backend.coeff_to_extended(pk.sigma_coeffs, k, circuit.m, dom.extended_k)
    pk.sigma_commitments = (backend.commit_lagrange(pk.sigma_lagrange, n, circuit.m)
                            if sigma_commitments is None else list(sigma_commitments))
    # l0, l_last, l_active (keygen.rs:395-430); l_active is the LDE of its
    # Lagrange values, equal to 1 - (l_last + l_blind) since the LDE is linear
    lag = np.zeros((3, n), dtype=object)
    l_vals = [[0] * n for _ in range(3)]
    l_vals[0][0] = 1
    l_vals[1][n - bf - 1] = 1
    l_vals[2] = [1] * (n - bf - 1) + [0] * (bf + 1)
    del lag
    lh = backend.put(ints_to_mont([v for col in l_vals for v in col]))
    lc = backend.lagrange_to_coeff(lh, k, 3)
    pk.l_cosets = backend.coeff_to_extended(lc, k, 3, dom.extended_k)
    backend.free(lh, lc)
    # compiled graphs (Evaluator::new, evaluation.rs:2723-2820)
    cg = GraphBuilder()
    part = cg.add_expression(circuit.gate)
    cg.horner((PREVIOUS, 0, 0), [part], (Y, 0, 0))
    pk.custom_graph = cg
    pk.lookup_input_graphs, pk.lookup_table_graphs, pk.lookup_graphs = [], [], []
    for ins, tab, _ in circuit.lookup_args:
        gi = GraphBuilder()
        gi.horner((CONSTANT, 0, 0), [gi.add_expression(e) for e in ins], (THETA, 0, 0))
        gt = GraphBuilder()
        gt.horner((CONSTANT, 0, 0), [gt.add_expression(e) for e in tab], (THETA, 0, 0))
        g = GraphBuilder()
        ci = g.horner((CONSTANT, 0, 0), [g.add_expression(e) for e in ins], (THETA, 0, 0))
        ct = g.horner((CONSTANT, 0, 0), [g.add_expression(e) for e in tab], (THETA, 0, 0))
        rg = g.add_calculation((ADD, ct, (GAMMA, 0, 0)))
        lcb = g.add_calculation((ADD, ci, (BETA, 0, 0)))
        g.add_calculation((MUL, lcb, rg))
        pk.lookup_input_graphs.append(gi)
        pk.lookup_table_graphs.append(gt)
        pk.lookup_graphs.append(g)
    pk.transcript_repr = vk_transcript_repr(circuit, pk.fixed_commitments, pk.sigma_commitments)
    return pk


def vk_transcript_repr(circuit, fixed_commitments, sigma_commitments):
    h = hashlib.blake2b(digest_size=64, person=b"Halo2-Verify-Key")
    desc = circuit.describe().encode()
    h.update(struct.pack("<Q", len(desc)))
    h.update(desc)
    h.update(struct.pack("<IIII", circuit.k, circuit.cs_degree, circuit.blinding_factors, circuit.chunk_len))
    for c in list(fixed_commitments) + list(sigma_commitments):
        h.update(compress(c))
    return int.from_bytes(h.digest(), "little") % R


# ---------------------------------------------------------------- prover

def _permute_expression_pair(backend, inp, tab, usable, input_blinds, table_blinds):
    """permute_expression_pair (lookup/prover.rs:1573-1690) on Montgomery
    rows: A' = sorted inputs, S' places one matching table value at the
    first row of each run of equal inputs and the leftover table values,
    in order, into the repeated rows from the bottom up."""
    a_sorted = backend.sort_canonical(inp[:usable])
    t_sorted = backend.sort_canonical(tab[:usable])
    keys_a = a_sorted.view(np.dtype((np.void, 32))).reshape(-1)
    keys_t = t_sorted.view(np.dtype((np.void, 32))).reshape(-1)
    first = np.ones(usable, dtype=bool)
    first[1:] = keys_a[1:] != keys_a[:-1]
    perm_t = np.zeros((usable, 4), dtype=np.uint64)
    perm_t[first] = a_sorted[first]
    unique = set(keys_a[first].tolist())
    removed = np.zeros(usable, dtype=bool)
    seen = set()
    # first occurrence in the sorted table of each unique input value
    for i, kt in enumerate(keys_t.tolist()):
        if kt in unique and kt not in seen:
            seen.add(kt)
            removed[i] = True
    if len(seen) != len(unique):
        raise ValueError("lookup input value missing from the table")
    leftovers = t_sorted[~removed]
    repeated = np.flatnonzero(~first)[::-1]
    if len(leftovers) != len(repeated):
        raise ValueError("lookup table/input multiset mismatch")
    perm_t[repeated] = leftovers
    a_full = np.concatenate([a_sorted, input_blinds])
    t_full = np.concatenate([perm_t, table_blinds])
    return a_full, t_full


class CommitRequest:
    """A proof step's commitment batch: count polynomials of n values in
    device vector (or host array) h, against g_lagrange (lagrange) or g.
    The proof generator yields it and receives a pending object whose
    result() gives the affine points."""

    def __init__(self, h, n, count, lagrange):
        self.h, self.n, self.count, self.lagrange = h, n, count, lagrange


class _Ready:
    """a commitment batch already computed"""

    def __init__(self, points):
        self.points = points

    def result(self):
        return self.points


class _Slice:
    """one proof's share of a fused commitment batch"""

    def __init__(self, fused, start, count):
        self.fused, self.start, self.count = fused, start, count

    def result(self):
        if not hasattr(self.fused, "_points"):
            self.fused._points = self.fused.result()
        return self.fused._points[self.start:self.start + self.count]


def _commit_requests(backend, reqs):
    """pending results of the commitment requests that proofs in lockstep
    yielded at the same step.  With asynchronous commitments, requests of
    one basis and length are fused: their vectors are concatenated on the
    device and committed as one MSM batch, so every stage of the MSM engine
    is one launch for all the proofs; otherwise each runs on its own."""
    commit_async = getattr(backend, "commit_async", None)
    if commit_async is None:
        return [_Ready((backend.commit_lagrange if r.lagrange else backend.commit)(r.h, r.n, r.count))
                for r in reqs]
    out = [None] * len(reqs)
    groups = {}
    for i, r in enumerate(reqs):
        groups.setdefault((r.lagrange, r.n), []).append(i)
    for (lagrange, n), idx in groups.items():
        if len(idx) == 1:
            r = reqs[idx[0]]
            out[idx[0]] = commit_async(r.h, n, r.count, lagrange)
            continue
        parts, counts = [], []
        for i in idx:
            r = reqs[i]
            # each request's polynomials as one vector of count * n values
            parts.append(r.h if r.h.len == r.count * n else r.h.gather_polys(n, list(range(r.count))))
            counts.append(r.count)
        fused = commit_async(backend.cat(parts), n, sum(counts), lagrange)
        at = 0
        for i, cnt in zip(idx, counts):
            out[i] = _Slice(fused, at, cnt)
            at += cnt
    return out


# yielded by a proof generator after it has queued the device work that
# follows a commitment request, before it waits for the points: the driver
# lets every proof of the group queue that work first
WAIT = object()


def _drive(gens, backend):
    """Run proof generators in lockstep: each runs to its next commitment
    request (or WAIT), the requests of a step are committed together, and
    each generator continues with its pending points.  Returns the proofs."""
    proofs = [None] * len(gens)
    sends = [None] * len(gens)
    live = list(range(len(gens)))
    while live:
        asked = []
        for i in live:
            try:
                asked.append((i, gens[i].send(sends[i])))
            except StopIteration as stop:
                proofs[i] = stop.value
        live = [i for i, _ in asked]
        reqs = [(i, r) for i, r in asked if r is not WAIT]
        for i, r in asked:
            if r is WAIT:
                sends[i] = None
        for (i, _), pending in zip(reqs, _commit_requests(backend, [r for _, r in reqs])):
            sends[i] = pending
    return proofs


def create_proof(params, pk, advice_values, backend, transcript, rng):
    """One proof. advice_values: [m][n] canonical ints (usable rows assigned)
    or an (m*n, 4) Montgomery array; rows from usable_rows on are blinded."""
    return _drive([_proof_steps(params, pk, advice_values, backend, transcript, rng)], backend)[0]


def create_proofs(params, pk, advice_list, backend, transcripts, rngs):
    """Several proofs of one circuit in lockstep: at each round every proof's
    commitments join one MSM batch (one launch per MSM stage for all of
    them).  Each proof's bytes equal create_proof's with the same transcript
    and rng: the proofs share launches, not arithmetic."""
    gens = [_proof_steps(params, pk, a, backend, t, r) for a, t, r in zip(advice_list, transcripts, rngs)]
    return _drive(gens, backend)


def _proof_steps(params, pk, advice_values, backend, transcript, rng):
    """The proof as a generator: it yields a CommitRequest at each
    commitment batch and receives its pending points; returns the proof
    bytes."""
    c = pk.circuit
    dom = pk.domain
    n, k, m = c.n, c.k, c.m
    bf, u = c.blinding_factors, c.usable_rows
    ek = dom.extended_k
    w = lambda v: fr_mont(v)  # noqa: E731

    transcript.common_scalar(w(pk.transcript_repr))
    # ---- advice (prover.rs:1342-1720)
    if isinstance(advice_values, np.ndarray):
        adv = np.ascontiguousarray(advice_values, dtype=np.uint64).reshape(m * n, 4)
    else:
        adv = ints_to_mont([v for col in advice_values for v in col]).reshape(m * n, 4)
    blind_rows = np.concatenate([fr_random(rng, n - u) for _ in range(m)])
    blind_idx = (np.arange(m, dtype=np.uint32)[:, None] * n + np.arange(u, n, dtype=np.uint32)[None, :]).reshape(-1)
    put_rows = getattr(backend, "put_with_rows", None)
    if put_rows is not None:
        # the caller's rows go up as they are and the blinding rows are
        # written on the device (no host copy of the witness)
        adv_l = put_rows(adv, blind_idx, blind_rows)
    else:
        adv = adv.copy()
        adv[blind_idx] = blind_rows
        adv_l = backend.put(adv)
    # the commitments are queued first; the transforms that need no
    # challenge run on the device while the host waits for them and writes
    # the transcript
    pending = yield CommitRequest(adv_l, n, m, True)
    adv_c = backend.lagrange_to_coeff(adv_l, k, m)
    adv_e = backend.coeff_to_extended(adv_c, k, m, ek)
    yield WAIT
    for cm in pending.result():
        transcript.write_point(cm)
    theta = fr_int(transcript.squeeze_challenge())

    # ---- lookups: compress, permute, commit A' and S' (lookup/prover.rs:688-733)
    L = c.lookups
    if L:
        comp = backend.eval_graphs_lagrange([g for pair in zip(pk.lookup_input_graphs, pk.lookup_table_graphs)
                                             for g in pair], pk.fixed_lagrange, c.num_fixed, adv_l, m, n,
                                            theta=w(theta))
        blinds = [fr_random(rng, bf + 1) for _ in range(2 * L)]  # per lookup: input, then table
        perm_l = backend.permute_lookups(comp, n, u, L, np.concatenate(blinds[0::2]), np.concatenate(blinds[1::2]))
        pending = yield CommitRequest(perm_l, n, 2 * L, True)
        perm_c = backend.lagrange_to_coeff(perm_l, k, 2 * L)
        perm_e = backend.coeff_to_extended(perm_c, k, 2 * L, ek)
        yield WAIT
        for cm in pending.result():
            transcript.write_point(cm)
    beta = fr_int(transcript.squeeze_challenge())
    gamma = fr_int(transcript.squeeze_challenge())

    # ---- permutation and lookup products (prover.rs:186-341)
    sets = c.permutation_sets
    perm_blinds = fr_random(rng, sets * bf)
    lk_blinds = fr_random(rng, L * bf) if L else np.zeros((0, 4), np.uint64)
    deltas = ints_to_mont([pow(DELTA, j, R) for j in range(m)])
    z_perm = backend.permutation_products(adv_l, pk.sigma_lagrange, n, m, c.chunk_len, w(beta), w(gamma),
                                          w(dom.omega), deltas, perm_blinds, bf)
    if L:
        z_lk = backend.lookup_products(comp, perm_l, n, L, w(beta), w(gamma), lk_blinds, bf)
    # the vanishing argument's random polynomial (vanishing/prover.rs:41-97)
    # comes from the rng alone, so its commitment joins the products' in one
    # batched MSM: committing its Lagrange values against g_lagrange gives the
    # same point as its coefficients against g
    random_poly = backend.random_mont(rng, n)
    parts = [z_perm] + ([z_lk] if L else []) + [backend.coeff_to_lagrange(random_poly, k, 1)]
    pending = yield CommitRequest(backend.cat(parts), n, sets + L + 1, True)
    zp_c = backend.lagrange_to_coeff(z_perm, k, sets)
    zp_e = backend.coeff_to_extended(zp_c, k, sets, ek)
    if L:
        zl_c = backend.lagrange_to_coeff(z_lk, k, L)
        zl_e = backend.coeff_to_extended(zl_c, k, L, ek)
    yield WAIT
    cms = pending.result()
    for cm in cms[:sets + L]:
        transcript.write_point(cm)
    transcript.squeeze_challenge()  # trash challenge (no trash arguments)
    transcript.write_point(cms[sets + L])
    y = fr_int(transcript.squeeze_challenge())

    # ---- quotient (prover.rs:1743-1990, evaluation.rs:3114-3528); the
    # coefficient forms and extended cosets were queued with the commitments
    numer = backend.numerator(
        pk, ek, adv_e, m, w(beta), w(gamma), w(theta), w(y), w(dom.extended_omega), w(beta * ZETA % R),
        w(DELTA), 1 << (ek - k), -(bf + 1), c.chunk_len, zp_e, sets,
        [(g, zl_e, perm_e, li) for li, g in enumerate(pk.lookup_graphs)] if L else [])
    q_coeff = backend.divide_vanishing_to_coeff(numer, ek, ints_to_mont(dom.t_evaluations_inv), w(1),
                                                w(ZETA * ZETA % R), w(ZETA))
    pieces_n = dom.quotient_poly_degree
    h_blinds = fr_random(rng, pieces_n - 1)
    h_pieces = backend.quotient_pieces(q_coeff, n, pieces_n, h_blinds)
    pending = yield CommitRequest(h_pieces, n, pieces_n, False)
    for cm in pending.result():
        transcript.write_point(cm)
    x = fr_int(transcript.squeeze_challenge())

    # ---- evaluations (prover.rs:1940-1990 and the argument evaluate()s)
    x_next = dom.rotate_omega(x, 1)
    x_prev = dom.rotate_omega(x, -1)
    x_last = dom.rotate_omega(x, -(bf + 1))
    # every evaluation at x and its rotations, in one batched call; written
    # to the transcript in the reference's order below
    adv_rots = list(dict.fromkeys(r for _, r in c.advice_queries))
    fix_rots = list(dict.fromkeys(r for _, r in c.fixed_queries))
    reqs = [(adv_c, m, w(dom.rotate_omega(x, rot))) for rot in adv_rots]
    reqs += [(pk.fixed_coeffs, c.num_fixed, w(dom.rotate_omega(x, rot))) for rot in fix_rots]
    reqs += [(random_poly, 1, w(x)), (pk.sigma_coeffs, m, w(x)), (zp_c, sets, w(x)), (zp_c, sets, w(x_next))]
    if sets > 1:
        reqs.append((zp_c, sets, w(x_last)))
    if L:
        reqs += [(zl_c, L, w(x)), (zl_c, L, w(x_next)), (perm_c, 2 * L, w(x)), (perm_c, 2 * L, w(x_prev))]
    vals = [mont_to_ints(arr) for arr in backend.eval_many(reqs, n)]
    adv_at = dict(zip(adv_rots, vals[:len(adv_rots)]))
    fix_at = dict(zip(fix_rots, vals[len(adv_rots):len(adv_rots) + len(fix_rots)]))
    rest = iter(vals[len(adv_rots) + len(fix_rots):])
    for col, rot in c.advice_queries:
        transcript.write_scalar_int(adv_at[rot][col])
    for col, rot in c.fixed_queries:
        transcript.write_scalar_int(fix_at[rot][col])
    # vanishing.evaluate: the combined h polynomial and the random eval (vanishing/prover.rs:321-383)
    split = pow(x, n - 1, R)
    h_poly = backend.lincomb(h_pieces, n, pieces_n, ints_to_mont([pow(split, i, R) for i in range(pieces_n)]))
    random_eval = next(rest)[0]
    transcript.write_scalar_int(random_eval)
    for v in next(rest):
        transcript.write_scalar_int(v)
    zp_x, zp_xn = next(rest), next(rest)
    zp_xl = next(rest) if sets > 1 else []
    for s in range(sets):
        transcript.write_scalar_int(zp_x[s])
        transcript.write_scalar_int(zp_xn[s])
        if s + 1 < sets:
            transcript.write_scalar_int(zp_xl[s])
    if L:
        zl_x, zl_xn, pp_x, pp_xp = next(rest), next(rest), next(rest), next(rest)
        for li in range(L):
            for v in (zl_x[li], zl_xn[li], pp_x[2 * li], pp_xp[2 * li], pp_x[2 * li + 1]):
                transcript.write_scalar_int(v)

    # ---- queries (prover.rs:1993-2063) and multi-open
    P = lambda h, i: (h, i)  # noqa: E731  (polynomial = (handle, index))
    queries = [(P(adv_c, col), dom.rotate_omega(x, rot)) for col, rot in c.advice_queries]
    for s in range(sets):
        queries.append((P(zp_c, s), x))
        queries.append((P(zp_c, s), x_next))
    for s in reversed(range(sets - 1)):
        queries.append((P(zp_c, s), x_last))
    for li in range(L):
        queries += [(P(zl_c, li), x), (P(perm_c, 2 * li), x), (P(perm_c, 2 * li + 1), x),
                    (P(perm_c, 2 * li), x_prev), (P(zl_c, li), x_next)]
    queries += [(P(pk.fixed_coeffs, col), dom.rotate_omega(x, rot)) for col, rot in c.fixed_queries]
    queries += [(P(pk.sigma_coeffs, i), x) for i in range(m)]
    queries += [(P(h_poly, 0), x), (P(random_poly, 0), x)]
    yield from _multi_open_steps(params, backend, n, queries, transcript)
    return transcript.finalize()


def construct_intermediate_sets(queries):
    """construct_intermediate_set_metadata (poly/kzg/utils.rs:48-160):
    commitments in first-query order, point indices in first-seen order,
    point sets numbered by first appearance over commitments, points of a
    set in ascending point index."""
    commits, cpoints = [], []
    point_index = {}
    for poly, point in queries:
        pi = point_index.setdefault(point, len(point_index))
        if poly in commits:
            j = commits.index(poly)
            if pi in cpoints[j]:
                raise ValueError("duplicated query")
            cpoints[j].append(pi)
        else:
            commits.append(poly)
            cpoints.append([pi])
    inverse = {i: p for p, i in point_index.items()}
    set_ids, set_of = {}, []
    for pts in cpoints:
        key = tuple(sorted(set(pts)))
        set_of.append(set_ids.setdefault(key, len(set_ids)))
    point_sets = [None] * len(set_ids)
    for key, sid in set_ids.items():
        point_sets[sid] = [inverse[i] for i in key]
    return commits, set_of, point_sets


def _multi_open_steps(params, backend, n, queries, transcript):
    """KZGCommitmentScheme::multi_open (poly/kzg/mod.rs:1978-2600), as
    proof steps: the f and pi commitments are yielded as CommitRequests."""
    x1 = fr_int(transcript.squeeze_challenge())
    x2 = fr_int(transcript.squeeze_challenge())
    commits, set_of, point_sets = construct_intermediate_sets(queries)
    nsets = len(point_sets)
    # q_j = sum over the set's commitments (in commitment order) of x1^i p_i;
    # the sets are then taken by (number of points, set number)
    members = [[i for i, s in enumerate(set_of) if s == sid] for sid in range(nsets)]
    order = sorted(range(nsets), key=lambda i: (len(point_sets[i]), i))
    members = [members[i] for i in order]
    point_sets = [point_sets[i] for i in order]
    fused = getattr(backend, "multi_open_q_f", None)
    if fused is not None:
        # the q polynomials and f in two device calls (the reference's
        # multi-open entry points)
        qstack, f_poly = fused(commits, members, point_sets, x1, x2, n)
    else:
        gathered = backend.gather(commits, n)
        q_polys = [backend.lincomb_rows(gathered, n, idx, ints_to_mont([pow(x1, i, R) for i in range(len(idx))]))
                   for idx in members]
        # f = sum_j x2^j (q_j / prod_{p in set_j} (X - p)), each division a Kate quotient
        f_parts = []
        for q, pts in zip(q_polys, point_sets):
            cur = q
            for p in pts:
                cur = backend.kate_divide(cur, n, 1, fr_mont(p))
            f_parts.append(cur)
        stack = backend.cat(f_parts)
        f_poly = backend.lincomb(stack, n, nsets, ints_to_mont([pow(x2, j, R) for j in range(nsets)]))
        qstack = backend.cat(q_polys)
    pending = yield CommitRequest(f_poly, n, 1, False)
    transcript.write_point(pending.result()[0])
    x3 = fr_int(transcript.squeeze_challenge())
    for v in backend.eval_polys(qstack, n, nsets, fr_mont(x3)):
        transcript.write_scalar(v)
    x4 = fr_int(transcript.squeeze_challenge())
    scalars = ints_to_mont([pow(x4, j, R) for j in range(nsets + 1)])
    # pi = commit((final - final(x3)) / (X - x3)), final = sum_j x4^j q_j +
    # x4^nsets f; the Kate quotient ignores the constant term
    fused_pi = getattr(backend, "multi_open_pi", None)
    if fused_pi is not None:
        pi_poly, pi_len = fused_pi(qstack, f_poly, n, scalars, fr_mont(x3))
    else:
        allp = backend.cat([qstack, f_poly])
        final = backend.lincomb(allp, n, nsets + 1, scalars)
        pi_poly, pi_len = backend.kate_divide(final, n, 1, fr_mont(x3)), n
    pending = yield CommitRequest(pi_poly, pi_len, 1, False)
    transcript.write_point(pending.result()[0])


# ---------------------------------------------------------------- GPU backend

class _PendingCommit:
    def __init__(self, ticket):
        self.ticket = ticket

    def result(self):
        return list(affine_from_projective_batch(self.ticket.wait()))


class GpuBackend:
    """The product backend: polynomials stay in device vectors, commitments go
    through resident MSM contexts over params' g and g_lagrange, and every
    transform is a CUDA kernel behind the C ABI."""

    def __init__(self, params: ParamsKZG):
        self.params = params

    # storage
    def put(self, arr):
        return api.Bls12_381FrDeviceVec.upload(np.ascontiguousarray(arr, dtype=np.uint64).reshape(-1, 4))

    def get(self, h):
        return h.download()

    def put_with_rows(self, arr, indices, rows):
        """put(arr) with arr[indices] replaced by rows, the rows written on
        the device"""
        v = self.put(arr)
        v.scatter_host(indices, rows)
        return v

    def free(self, *hs):
        for h in hs:
            h.free()

    def cat(self, hs):
        return api.Bls12_381FrDeviceVec.concat_many_host(hs, np.zeros((0, 4), np.uint64))

    def gather(self, polys, n):
        """stack the (handle, index) polynomials into one device vector"""
        parts = []
        for h, i in polys:
            parts.append(h.gather_polys(n, [i]) if h.len != n or i else h)
        return self.cat(parts)

    def lincomb_rows(self, stacked, n, rows, coeffs):
        sub = stacked.gather_polys(n, rows)
        return api.bls12_381_fr_device_poly_lincomb(sub, n, len(rows), coeffs)

    # transforms
    def lagrange_to_coeff(self, h, k, count):
        out = h.gather_polys(1 << k, list(range(count)))
        one = fr_mont(1)
        out.ntt_zeta_batch(k, count, True, one, one, one)
        return out

    def coeff_to_lagrange(self, h, k, count):
        out = h.gather_polys(1 << k, list(range(count)))
        one = fr_mont(1)
        out.ntt_zeta_batch(k, count, False, one, one, one)
        return out

    def coeff_to_extended(self, h, k, count, ek):
        raw = api.ctypes.c_void_p()
        api.check(api.lib().midnight_sppark_bls12_381_fr_device_coeff_to_extended_from_device_batch(
            api.ctypes.byref(raw), h.raw, 1 << k, count, ek, api._fr(fr_mont(ZETA)), api._fr(fr_mont(ZETA * ZETA))))
        return api.Bls12_381FrDeviceVec(raw)

    def divide_vanishing_to_coeff(self, h, ek, t_inv, scale, first, second):
        h.divide_ntt_zeta(ek, t_inv, scale, first, second)
        return h

    def quotient_pieces(self, q, n, pieces, blinds):
        return api.bls12_381_fr_device_quotient_pieces(q, n, pieces, blinds)

    def lincomb(self, h, n, count, scalars):
        return api.bls12_381_fr_device_poly_lincomb(h, n, count, scalars)

    def eval_polys(self, h, n, count, point):
        return api.bls12_381_fr_device_eval_polys(h, n, count, point)

    def eval_many(self, requests, n):
        return api.fr_device_eval_many(requests, n)

    def kate_divide(self, h, n, count, point):
        return api.fr_device_kate_divide(h, n, count, point)

    # commitments
    def _commit(self, h, n, count, lagrange):
        ctx = self.params.context(lagrange)
        res = ctx.device_batch(h, 0, n, count)
        return list(affine_from_projective_batch(res))

    def commit_lagrange(self, h, n, count):
        return self._commit(h, n, count, True)

    def multi_open_q_f(self, commits, members, point_sets, x1, x2, n):
        """the multi-open's q polynomials (one per point set, set order as
        given) as one device vector, and f, through
        ..._fr_multiopen_prepare_device and ..._fr_multiopen_f_poly_device;
        the committed polynomials are read in place when they share one
        device vector, else from one concatenated copy"""
        vecs, base, at = [], {}, 0
        for h, _ in commits:
            if id(h) not in base:
                base[id(h)] = at
                at += h.len // n
                vecs.append(h)
        src = vecs[0] if len(vecs) == 1 else api.Bls12_381FrDeviceVec.concat_many_host(vecs, np.zeros((0, 4), np.uint64))
        refs = [(0, base[id(h)] + i) for h, i in commits]
        q_off, q_idx, q_co = [0], [], []
        for idx in members:
            q_idx += idx
            q_co += [pow(x1, t, R) for t in range(len(idx))]
            q_off.append(len(q_idx))
        pts = ints_to_mont([p for ps in point_sets for p in ps])
        # (one evaluation is asked for, unused: the entry point wants a query)
        _, qvec, _ = api.bls12_381_fr_multiopen_prepare_device((src, src, src), n, refs, q_off, q_idx,
                                                              ints_to_mont(q_co), pts, [0], [0], q_host=False)
        if src is not vecs[0]:
            src.free()
        p_off = [0]
        for ps in point_sets:
            p_off.append(p_off[-1] + len(ps))
        f = api.bls12_381_fr_multiopen_f_poly_device(qvec, n, p_off, pts,
                                                     ints_to_mont([pow(x2, j, R) for j in range(len(point_sets))]))
        return qvec, f

    def multi_open_pi(self, qvec, f, n, scalars, point):
        """(sum_j scalars[j] q_j + scalars[last] f) / (X - point) through
        ..._fr_multiopen_pi_device: n - 1 coefficients"""
        return api.bls12_381_fr_multiopen_pi_device(qvec, f, n, scalars, point), n - 1

    def commit_async(self, h, n, count, lagrange):
        """the commitments of _commit, queued: .result() waits for them"""
        return _PendingCommit(self.params.context(lagrange).device_batch_async(h, 0, n, count))

    def commit(self, h, n, count):
        return self._commit(h, n, count, False)

    # arguments
    def to_mont(self, raw):
        """canonical limb rows -> resident Montgomery values (a product with R^2)"""
        return api.bls12_381_fr_device_poly_lincomb(self.put(raw), len(raw), 1, R2_LIMBS.reshape(1, 4))

    def random_mont(self, rng, n):
        """fr_random(rng, n), resident: large draws run the ChaCha20 stream and
        the rejection sampling on the device, then the host rng skips the
        words they used"""
        if n < 4096:
            return self.put(fr_random(rng, n))
        vec, used = api.fr_random_chacha20(rng.seed, rng.word_position(), n)
        rng.skip_words(used)
        return vec

    def to_host(self, h, n, i):
        return h.gather_polys(n, [i]).download()

    def permute_lookups(self, comp_h, n, u, L, input_blinds, table_blinds):
        return api.fr_lookup_permute_device(comp_h, n, u, L, input_blinds, table_blinds)

    def sort_canonical(self, arr):
        return api.bls12_381_fr_sort_canonical(arr)

    def eval_graphs_lagrange(self, builders, fixed_h, nfixed, adv_h, m, n, theta):
        graphs = [b.compile(Graph) for b in builders]
        return api.eval_graph_batch_device(n, graphs, fixed=fixed_h, fixed_cols=nfixed, advice=adv_h, advice_cols=m,
                                           theta=theta, rot_scale=1)

    def permutation_products(self, adv_h, sigma_h, n, m, chunk, beta, gamma, omega, deltas, blinds, bf):
        return api.fr_permutation_products_device(adv_h, sigma_h, n, m, chunk, beta, gamma, omega, deltas, blinds, bf)

    def lookup_products(self, comp_h, perm_h, n, L, beta, gamma, blinds, bf):
        # trace [compressed inputs | compressed tables | permuted inputs | permuted tables]
        both = self.cat([comp_h, perm_h])
        idx = [2 * i for i in range(L)] + [2 * i + 1 for i in range(L)] + \
              [2 * L + 2 * i for i in range(L)] + [2 * L + 2 * i + 1 for i in range(L)]
        trace = both.gather_polys(n, idx)
        return api.bls12_381_fr_lookup_products_device(trace, n, L, beta, gamma, blinds, bf)

    def numerator(self, pk, ek, adv_e, m, beta, gamma, theta, y, omega, delta_start, delta_const, rot_scale,
                  last_rotation, chunk_len, zp_e, sets, lookups):
        N = 1 << ek
        c = pk.circuit
        zl_e = lookups[0][1] if lookups else None
        perm_e = lookups[0][2] if lookups else None
        return api.eval_numerator_device(
            N, pk.custom_graph.compile(Graph), fixed=pk.fixed_cosets, fixed_cols=c.num_fixed, advice=adv_e,
            advice_cols=m, beta=beta, gamma=gamma, theta=theta, y=y, omega=omega, delta_start=delta_start,
            delta_const=delta_const, rot_scale=rot_scale, last_rotation=last_rotation, chunk_len=chunk_len,
            lagrange=pk.l_cosets, permutation_products=zp_e, permutation_sets=sets,
            permutation_columns=[(1, i) for i in range(m)], permutation_pk_cosets=pk.sigma_cosets,
            permutation_pk_count=m, lookup_products=zl_e, lookup_permuted=perm_e,
            lookup_graphs=[g.compile(Graph) for g, _, _, _ in lookups])
