"""CPU backend for the synthetic PLONK/KZG prover driver.

TEST INFRASTRUCTURE ONLY. This backend runs the prover driver of
gb_prover.plonk on the oracle's C restatements, so that a proof made on the
GPU can be checked byte for byte against one made on the host. Only tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline leg use it.

Each operation restates the reference's CPU step that the GPU backend
replaces:
  * lagrange_to_coeff / coeff_to_extended / extended_to_coeff:
    poly/domain.rs:260-443;
  * commit / commit_lagrange: poly/kzg/mod.rs:1072-1300 (msm_specific over g
    or g_lagrange);
  * products: permutation/prover.rs:327-533, lookup/prover.rs:1075-1240;
  * numerator: evaluation.rs:3114-3528;
  * eval_polynomial / kate_division: utils/arithmetic.rs:53-116.

`setup_params` is ParamsKZG::unsafe_setup with a known tau
(poly/kzg/params.rs:79-129), computed with the oracle's generator
multiplication.
"""
import os
import sys

import numpy as np

from . import oracle as orc

_REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_PKG = os.path.join(_REPO, "midnight-ledger-cuda_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from gb_prover.rng import ints_to_mont, mont_to_ints  # noqa: E402

R = orc.R_MOD


class HostPoly:
    """a stack of polynomials in host memory (identity-compared handle)"""
    __slots__ = ("a",)

    def __init__(self, a):
        self.a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4)

    @property
    def len(self):
        return len(self.a)


class HostParams:
    def __init__(self, k, g, g_lagrange):
        self.k, self.n = k, 1 << k
        self.g, self.g_lagrange = g, g_lagrange


def setup_params(k, tau):
    """g_i = [tau^i] G, g_lagrange_i = [(tau^n - 1)/n * w^i / (tau - w^i)] G
    (params.rs:79-129); tau a canonical integer."""
    n = 1 << k
    w = int(orc.fr_to_ints(orc.fr_omega(k)[None])[0])
    pw = [1] * n
    for i in range(1, n):
        pw[i] = pw[i - 1] * tau % R
    g = orc.g1_generator_mul_batch(ints_to_mont(pw))
    mult = (pow(tau, n, R) - 1) * pow(n, -1, R) % R
    wi, num, den = 1, [], []
    for i in range(n):
        num.append(mult * wi % R)
        den.append((tau - wi) % R)
        wi = wi * w % R
    inv = mont_to_ints(orc.fr_batch_invert(ints_to_mont(den)))
    gl = orc.g1_generator_mul_batch(ints_to_mont([a * b % R for a, b in zip(num, inv)]))
    return HostParams(k, g, gl)


class OracleBackend:
    def __init__(self, params, threads=None):
        self.params = params
        self.threads = threads

    # storage
    def put(self, arr):
        return HostPoly(np.array(arr, dtype=np.uint64, copy=True))

    def get(self, h):
        return h.a

    def free(self, *hs):
        pass

    def cat(self, hs):
        return HostPoly(np.concatenate([h.a for h in hs]))

    def gather(self, polys, n):
        return HostPoly(np.concatenate([h.a[i * n:(i + 1) * n] for h, i in polys]))

    def lincomb_rows(self, stacked, n, rows, coeffs):
        sub = np.concatenate([stacked.a[r * n:(r + 1) * n] for r in rows])
        return HostPoly(orc.fr_poly_lincomb(sub, n, len(rows), coeffs))

    # transforms
    def lagrange_to_coeff(self, h, k, count):
        n = 1 << k
        return HostPoly(np.concatenate([orc.fr_ntt(h.a[i * n:(i + 1) * n], k, True, self.threads)
                                        for i in range(count)]))

    def coeff_to_lagrange(self, h, k, count):
        n = 1 << k
        return HostPoly(np.concatenate([orc.fr_ntt(h.a[i * n:(i + 1) * n], k, False, self.threads)
                                        for i in range(count)]))

    def coeff_to_extended(self, h, k, count, ek):
        from gb_prover.plonk import ZETA
        z1, z2 = ints_to_mont([ZETA, ZETA * ZETA % R])
        return HostPoly(orc.fr_coeff_to_extended_batch(h.a[:count << k], 1 << k, count, ek, z1, z2, self.threads))

    def divide_vanishing_to_coeff(self, h, ek, t_inv, scale, first, second):
        return HostPoly(orc.fr_divide_ntt_zeta(h.a, ek, t_inv, scale, first, second, self.threads))

    def quotient_pieces(self, q, n, pieces, blinds):
        return HostPoly(orc.fr_quotient_pieces(q.a, n, pieces, blinds))

    def lincomb(self, h, n, count, scalars):
        return HostPoly(orc.fr_poly_lincomb(h.a[:n * count], n, count, scalars))

    def eval_polys(self, h, n, count, point):
        return np.stack([orc.fr_eval_poly(h.a[i * n:(i + 1) * n], point) for i in range(count)])

    def eval_many(self, requests, n):
        return [self.eval_polys(h, n, count, point) for h, count, point in requests]

    def kate_divide(self, h, n, count, point):
        out = np.zeros((n * count, 4), dtype=np.uint64)
        for i in range(count):
            out[i * n:i * n + n - 1] = orc.fr_kate_division(h.a[i * n:(i + 1) * n], point)
        return HostPoly(out)

    # commitments
    def _commit(self, h, n, count, bases):
        out = []
        for i in range(count):
            jac = orc.g1_msm(bases[:n], h.a[i * n:(i + 1) * n], self.threads)
            out.append(orc.g1_to_affine(jac)[0])
        return out

    def commit_lagrange(self, h, n, count):
        return self._commit(h, n, count, self.params.g_lagrange)

    def commit(self, h, n, count):
        return self._commit(h, n, count, self.params.g)

    # arguments
    def to_mont(self, raw):
        from gb_prover.rng import R2_LIMBS
        return HostPoly(orc.fr_mul_assign(raw, R2_LIMBS))

    def random_mont(self, rng, n):
        from gb_prover.rng import fr_random
        return HostPoly(fr_random(rng, n))

    def to_host(self, h, n, i):
        return h.a[i * n:(i + 1) * n].copy()

    def permute_lookups(self, comp_h, n, u, L, input_blinds, table_blinds):
        from gb_prover.plonk import _permute_expression_pair
        nb = n - u
        out = []
        for li in range(L):
            out += list(_permute_expression_pair(self, self.to_host(comp_h, n, 2 * li), self.to_host(comp_h, n, 2 * li + 1),
                                                 u, input_blinds[li * nb:(li + 1) * nb],
                                                 table_blinds[li * nb:(li + 1) * nb]))
        return HostPoly(np.concatenate(out))

    def sort_canonical(self, arr):
        return orc.fr_sort_canonical(arr)

    def eval_graphs_lagrange(self, builders, fixed_h, nfixed, adv_h, m, n, theta):
        return HostPoly(np.concatenate([orc.eval_numerator(n, b.compile(orc.OracleGraph), fixed=fixed_h.a,
                                                           advice=adv_h.a, theta=theta, rot_scale=1,
                                                           threads=self.threads) for b in builders]))

    def permutation_products(self, adv_h, sigma_h, n, m, chunk, beta, gamma, omega, deltas, blinds, bf):
        return HostPoly(orc.fr_permutation_products(adv_h.a, sigma_h.a, n, m, chunk, beta, gamma, omega, deltas,
                                                     blinds, bf))

    def lookup_products(self, comp_h, perm_h, n, L, beta, gamma, blinds, bf):
        cols = lambda h, j: h.a[j * n:(j + 1) * n]  # noqa: E731
        stack = lambda h, off: np.concatenate([cols(h, 2 * i + off) for i in range(L)])  # noqa: E731
        return HostPoly(orc.fr_lookup_products(stack(comp_h, 0), stack(comp_h, 1), stack(perm_h, 0), stack(perm_h, 1),
                                               n, L, beta, gamma, blinds, bf))

    def numerator(self, pk, ek, adv_e, m, beta, gamma, theta, y, omega, delta_start, delta_const, rot_scale,
                  last_rotation, chunk_len, zp_e, sets, lookups):
        N = 1 << ek
        lks = []
        for g, zl_e, perm_e, li in lookups:
            pe = perm_e.a
            lks.append((g.compile(orc.OracleGraph), zl_e.a[li * N:(li + 1) * N], pe[2 * li * N:(2 * li + 1) * N],
                        pe[(2 * li + 1) * N:(2 * li + 2) * N]))
        lc = pk.l_cosets.a
        out = orc.eval_numerator(
            N, pk.custom_graph.compile(orc.OracleGraph), fixed=pk.fixed_cosets.a, advice=adv_e.a, beta=beta,
            gamma=gamma, theta=theta, y=y, omega=omega, delta_start=delta_start, delta_const=delta_const,
            rot_scale=rot_scale, last_rotation=last_rotation, chunk_len=chunk_len, l0=lc[:N], l_last=lc[N:2 * N],
            l_active=lc[2 * N:], permutation_products=zp_e.a, permutation_sets=sets,
            permutation_columns=[(1, i) for i in range(m)], permutation_pk_cosets=pk.sigma_cosets.a, lookups=lks,
            threads=self.threads)
        return HostPoly(out)
