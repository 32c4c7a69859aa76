"""ctypes bindings of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg to
check results.  Arrays are numpy uint64 with the reference's memory layout:
Fr (n, 4), G1 affine (n, 12), G1 Jacobian (n, 18), all Montgomery form.
"""
import ctypes
import os

import numpy as np

from . import build as _build

R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
P_MOD = int(
    "1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab",
    16,
)
FR_R = pow(2, 256, R_MOD)
FR_RINV = pow(FR_R, -1, R_MOD)
FP_R = pow(2, 384, P_MOD)
FP_RINV = pow(FP_R, -1, P_MOD)

CONST_ONE, CONST_GENERATOR, CONST_ROOT, CONST_ROOT_INV, CONST_DELTA, CONST_ZETA, CONST_TWO_INV = range(7)

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _declare(_lib)
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _declare(L):
    vp, sz, u32, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int
    sigs = {
        "orc_fr_mul": (None, [vp, vp, vp]),
        "orc_fr_add": (None, [vp, vp, vp]),
        "orc_fr_sub": (None, [vp, vp, vp]),
        "orc_fr_inv": (None, [vp, vp]),
        "orc_fr_constant": (i32, [vp, i32]),
        "orc_fr_from_uniform_bytes": (None, [vp, vp]),
        "orc_fr_cmp_canonical": (i32, [vp, vp]),
        "orc_fp_sqrt": (i32, [vp, vp]),
        "orc_g1_generator": (None, [vp]),
        "orc_g1_is_on_curve": (i32, [vp]),
        "orc_g1_to_affine": (None, [vp, vp]),
        "orc_g1_jac_to_affine_batch": (None, [vp, vp, sz]),
        "orc_g1_from_affine": (None, [vp, vp]),
        "orc_g1_add": (None, [vp, vp, vp]),
        "orc_g1_add_affine": (None, [vp, vp, vp]),
        "orc_g1_double": (None, [vp, vp]),
        "orc_g1_neg": (None, [vp, vp]),
        "orc_g1_mul": (None, [vp, vp, vp]),
        "orc_g1_generator_mul_batch": (None, [vp, vp, sz, i32]),
        "orc_g1_decompress": (i32, [vp, vp]),
        "orc_g1_compress": (None, [vp, vp]),
        "orc_g1_from_uncompressed": (i32, [vp, vp]),
        "orc_g1_to_uncompressed": (None, [vp, vp]),
        "orc_booth_index": (ctypes.c_int32, [sz, sz, vp]),
        "orc_g1_msm_naive": (None, [vp, vp, vp, sz]),
        "orc_g1_msm": (None, [vp, vp, vp, sz, i32, i32]),
        "orc_fr_fft": (None, [vp, u32, vp, i32]),
        "orc_fr_omega": (None, [vp, u32]),
        "orc_fr_ntt": (None, [vp, u32, i32, i32]),
        "orc_fr_mul_assign_zeta": (None, [vp, vp, vp, sz]),
        "orc_fr_mul_assign": (None, [vp, vp, sz]),
        "orc_fr_mul_assign_repeating": (None, [vp, vp, sz, sz]),
        "orc_fr_ntt_zeta": (None, [vp, u32, i32, vp, vp, vp, i32]),
        "orc_fr_divide_ntt_zeta": (None, [vp, u32, vp, sz, vp, vp, vp, i32]),
        "orc_fr_coeff_to_extended_batch": (i32, [vp, vp, sz, sz, u32, vp, vp, i32]),
        "orc_fr_distribute_powers": (None, [vp, sz, vp]),
        "orc_fr_ntt_coset": (None, [vp, u32, i32, vp, i32]),
        "orc_fr_coeff_to_extended_coset_batch": (i32, [vp, vp, sz, sz, u32, vp, i32]),
        "orc_fr_lde_coset": (None, [vp, vp, u32, u32, i32]),
        "orc_domain_extended_k": (u32, [u32, u32]),
        "orc_domain_t_evaluations": (None, [vp, u32, u32]),
        "orc_fr_batch_invert": (None, [vp, sz]),
        "orc_fr_shifted_prefix_product": (None, [vp, vp, sz]),
        "orc_fr_permutation_products": (i32, [vp, vp, vp, sz, sz, sz, vp, vp, vp, vp, vp, sz]),
        "orc_fr_lookup_products": (i32, [vp, vp, vp, vp, vp, sz, sz, vp, vp, vp, sz]),
        "orc_fr_poly_lincomb": (None, [vp, vp, sz, sz, vp]),
        "orc_fr_quotient_pieces": (i32, [vp, vp, sz, sz, sz, vp, sz]),
        "orc_fr_sort_canonical": (None, [vp, sz]),
        "orc_fr_eval_poly": (None, [vp, vp, sz, vp]),
        "orc_fr_kate_division": (None, [vp, vp, sz, vp]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def threads_default():
    return max(1, os.cpu_count() or 1)


# ---------------------------------------------------------------- conversions

def int_to_limbs(v, n):
    return [(v >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(n)]


def limbs_to_int(row):
    return sum(int(x) << (64 * i) for i, x in enumerate(row))


def fr_from_ints(vals):
    """canonical ints -> Montgomery Fr array (n, 4)"""
    out = np.empty((len(vals), 4), dtype=np.uint64)
    for i, v in enumerate(vals):
        out[i] = int_to_limbs((int(v) % R_MOD) * FR_R % R_MOD, 4)
    return out


def fr_to_ints(arr):
    arr = np.asarray(arr, dtype=np.uint64).reshape(-1, 4)
    return [limbs_to_int(r) * FR_RINV % R_MOD for r in arr]


def fp_from_int(v):
    return np.array(int_to_limbs((v % P_MOD) * FP_R % P_MOD, 6), dtype=np.uint64)


def fp_to_int(row):
    return limbs_to_int(row) * FP_RINV % P_MOD


def fr_random(n, rng):
    """Uniform Fr elements (Fq::random-style rejection, fq.rs:373-387),
    returned as Montgomery limbs; a uniform canonical value read as a
    Montgomery representation is itself uniform in Fr."""
    out = np.empty((n, 4), dtype=np.uint64)
    filled = 0
    top = np.uint64(0x7FFFFFFFFFFFFFFF)
    rl = np.array(int_to_limbs(R_MOD, 4), dtype=np.uint64)
    while filled < n:
        k = int((n - filled) * 1.3) + 16
        cand = rng.integers(0, 2**64, size=(k, 4), dtype=np.uint64)
        cand[:, 3] &= top
        # keep cand < r (lexicographic on limbs from the top)
        lt = np.zeros(k, dtype=bool)
        eq = np.ones(k, dtype=bool)
        for i in (3, 2, 1, 0):
            lt |= eq & (cand[:, i] < rl[i])
            eq &= cand[:, i] == rl[i]
        cand = cand[lt]
        take = min(len(cand), n - filled)
        out[filled:filled + take] = cand[:take]
        filled += take
    return out


# ---------------------------------------------------------------- wrappers

def fr_const(which):
    o = np.zeros(4, dtype=np.uint64)
    lib().orc_fr_constant(_p(o), which)
    return o


def fr_mul(a, b):
    o = np.zeros(4, dtype=np.uint64)
    lib().orc_fr_mul(_p(o), _p(np.ascontiguousarray(a, dtype=np.uint64)),
                     _p(np.ascontiguousarray(b, dtype=np.uint64)))
    return o


def fr_inv(a):
    o = np.zeros(4, dtype=np.uint64)
    lib().orc_fr_inv(_p(o), _p(np.ascontiguousarray(a, dtype=np.uint64)))
    return o


def fr_omega(k):
    o = np.zeros(4, dtype=np.uint64)
    lib().orc_fr_omega(_p(o), k)
    return o


def g1_generator():
    o = np.zeros(12, dtype=np.uint64)
    lib().orc_g1_generator(_p(o))
    return o


def g1_generator_mul_batch(scalars, threads=None):
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros((len(s), 12), dtype=np.uint64)
    lib().orc_g1_generator_mul_batch(_p(o), _p(s), len(s), threads or threads_default())
    return o


def g1_to_affine(jac):
    j = np.ascontiguousarray(jac, dtype=np.uint64).reshape(-1, 18)
    o = np.zeros((len(j), 12), dtype=np.uint64)
    lib().orc_g1_jac_to_affine_batch(_p(o), _p(j), len(j))
    return o


def g1_is_on_curve(aff):
    return bool(lib().orc_g1_is_on_curve(_p(np.ascontiguousarray(aff, dtype=np.uint64))))


def g1_msm(bases, scalars, threads=None, window_bits=0):
    b = np.ascontiguousarray(bases, dtype=np.uint64).reshape(-1, 12)
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    assert len(b) == len(s)
    o = np.zeros(18, dtype=np.uint64)
    lib().orc_g1_msm(_p(o), _p(b), _p(s), len(s), threads or threads_default(), window_bits)
    return o


def g1_msm_naive(bases, scalars):
    b = np.ascontiguousarray(bases, dtype=np.uint64).reshape(-1, 12)
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros(18, dtype=np.uint64)
    lib().orc_g1_msm_naive(_p(o), _p(b), _p(s), len(s))
    return o


def g1_add(a, b):
    o = np.zeros(18, dtype=np.uint64)
    lib().orc_g1_add(_p(o), _p(np.ascontiguousarray(a, dtype=np.uint64)),
                     _p(np.ascontiguousarray(b, dtype=np.uint64)))
    return o


def g1_from_affine(a):
    o = np.zeros(18, dtype=np.uint64)
    lib().orc_g1_from_affine(_p(o), _p(np.ascontiguousarray(a, dtype=np.uint64)))
    return o


def g1_mul(p_aff, scalar):
    o = np.zeros(18, dtype=np.uint64)
    lib().orc_g1_mul(_p(o), _p(np.ascontiguousarray(p_aff, dtype=np.uint64)),
                     _p(np.ascontiguousarray(scalar, dtype=np.uint64)))
    return o


def g1_decompress(b48):
    buf = np.frombuffer(bytes(b48), dtype=np.uint8).copy()
    o = np.zeros(12, dtype=np.uint64)
    rc = lib().orc_g1_decompress(_p(o), _p(buf))
    if rc:
        raise ValueError("invalid compressed point (code %d)" % rc)
    return o


def g1_compress(aff):
    o = np.zeros(48, dtype=np.uint8)
    lib().orc_g1_compress(_p(o), _p(np.ascontiguousarray(aff, dtype=np.uint64)))
    return o.tobytes()


def g1_from_uncompressed(b96):
    buf = np.frombuffer(bytes(b96), dtype=np.uint8).copy()
    o = np.zeros(12, dtype=np.uint64)
    rc = lib().orc_g1_from_uncompressed(_p(o), _p(buf))
    if rc:
        raise ValueError("invalid uncompressed point (code %d)" % rc)
    return o


def g1_to_uncompressed(aff):
    o = np.zeros(96, dtype=np.uint8)
    lib().orc_g1_to_uncompressed(_p(o), _p(np.ascontiguousarray(aff, dtype=np.uint64)))
    return o.tobytes()


def booth_index(window_index, window_size, scalar_le32):
    buf = np.frombuffer(bytes(scalar_le32), dtype=np.uint8).copy()
    return lib().orc_booth_index(window_index, window_size, _p(buf))


def fr_fft(a, log_n, omega, threads=None):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_fft(_p(a), log_n, _p(np.ascontiguousarray(omega, dtype=np.uint64)),
                     threads or threads_default())
    return a


def fr_ntt(a, log_n, inverse, threads=None):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_ntt(_p(a), log_n, int(inverse), threads or threads_default())
    return a


def fr_ntt_zeta(a, log_n, inverse, scale, first, second, threads=None):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_ntt_zeta(_p(a), log_n, int(inverse), _p(np.ascontiguousarray(scale, dtype=np.uint64)),
                          _p(np.ascontiguousarray(first, dtype=np.uint64)),
                          _p(np.ascontiguousarray(second, dtype=np.uint64)), threads or threads_default())
    return a


def fr_divide_ntt_zeta(a, log_n, factors, scale, first, second, threads=None):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    f = np.ascontiguousarray(factors, dtype=np.uint64).reshape(-1, 4)
    lib().orc_fr_divide_ntt_zeta(_p(a), log_n, _p(f), len(f),
                                 _p(np.ascontiguousarray(scale, dtype=np.uint64)),
                                 _p(np.ascontiguousarray(first, dtype=np.uint64)),
                                 _p(np.ascontiguousarray(second, dtype=np.uint64)),
                                 threads or threads_default())
    return a


def fr_coeff_to_extended_batch(inputs, input_len, count, ext_log_n, first, second, threads=None):
    i = np.ascontiguousarray(inputs, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros((count << ext_log_n, 4), dtype=np.uint64)
    rc = lib().orc_fr_coeff_to_extended_batch(_p(o), _p(i), input_len, count, ext_log_n,
                                              _p(np.ascontiguousarray(first, dtype=np.uint64)),
                                              _p(np.ascontiguousarray(second, dtype=np.uint64)),
                                              threads or threads_default())
    if rc:
        raise ValueError("coeff_to_extended: input longer than the extended domain")
    return o


def fr_distribute_powers(a, shift):
    """a[i] * shift^i (sppark LDE_distribute_powers, natural index)"""
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_distribute_powers(_p(a), len(a), _p(np.ascontiguousarray(shift, dtype=np.uint64)))
    return a


def fr_ntt_coset(a, log_n, inverse, shift, threads=None):
    """sppark NTT::Base with Type::coset, natural order in and out"""
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_ntt_coset(_p(a), log_n, int(inverse), _p(np.ascontiguousarray(shift, dtype=np.uint64)),
                           threads or threads_default())
    return a


def fr_coeff_to_extended_coset_batch(inputs, input_len, count, ext_log_n, shift, threads=None):
    """coefficients -> evaluations on the coset shift * <w_ext> (powers of shift)"""
    i = np.ascontiguousarray(inputs, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros((count << ext_log_n, 4), dtype=np.uint64)
    rc = lib().orc_fr_coeff_to_extended_coset_batch(_p(o), _p(i), input_len, count, ext_log_n,
                                                    _p(np.ascontiguousarray(shift, dtype=np.uint64)),
                                                    threads or threads_default())
    if rc:
        raise ValueError("coeff_to_extended_coset: input longer than the extended domain")
    return o


def fr_lde_coset(values, lg_dsz, lg_blowup, threads=None):
    """sppark NTT::LDE: evaluations -> evaluations on the generator coset of the
    2^(lg_dsz + lg_blowup) domain"""
    i = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros((1 << (lg_dsz + lg_blowup), 4), dtype=np.uint64)
    lib().orc_fr_lde_coset(_p(o), _p(i), lg_dsz, lg_blowup, threads or threads_default())
    return o


def fr_mul_assign_zeta(a, first, second):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_mul_assign_zeta(_p(a), _p(np.ascontiguousarray(first, dtype=np.uint64)),
                                 _p(np.ascontiguousarray(second, dtype=np.uint64)), len(a))
    return a


def fr_mul_assign(a, s):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_mul_assign(_p(a), _p(np.ascontiguousarray(s, dtype=np.uint64)), len(a))
    return a


def fr_mul_assign_repeating(a, factors):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    f = np.ascontiguousarray(factors, dtype=np.uint64).reshape(-1, 4)
    lib().orc_fr_mul_assign_repeating(_p(a), _p(f), len(f), len(a))
    return a


def domain_extended_k(j, k):
    return lib().orc_domain_extended_k(j, k)


def domain_t_evaluations(j, k):
    ek = domain_extended_k(j, k)
    o = np.zeros((1 << (ek - k), 4), dtype=np.uint64)
    lib().orc_domain_t_evaluations(_p(o), j, k)
    return o


def fr_batch_invert(a):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_batch_invert(_p(a), len(a))
    return a


def fr_shifted_prefix_product(a, initial):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_shifted_prefix_product(_p(a), _p(np.ascontiguousarray(initial, dtype=np.uint64)), len(a))
    return a


def fr_permutation_products(columns, permutations, length, column_count, chunk_len, beta, gamma,
                            omega, delta_powers, blinds, blinding_factors):
    sets = (column_count + chunk_len - 1) // chunk_len
    o = np.zeros((sets * length, 4), dtype=np.uint64)
    c = np.ascontiguousarray(columns, dtype=np.uint64)
    pm = np.ascontiguousarray(permutations, dtype=np.uint64)
    d = np.ascontiguousarray(delta_powers, dtype=np.uint64)
    b = np.ascontiguousarray(blinds if blinds is not None else np.zeros((1, 4)), dtype=np.uint64)
    rc = lib().orc_fr_permutation_products(_p(o), _p(c), _p(pm), length, column_count, chunk_len,
                                           _p(np.ascontiguousarray(beta, dtype=np.uint64)),
                                           _p(np.ascontiguousarray(gamma, dtype=np.uint64)),
                                           _p(np.ascontiguousarray(omega, dtype=np.uint64)),
                                           _p(d), _p(b), blinding_factors)
    if rc:
        raise ValueError("invalid permutation product arguments")
    return o


def fr_lookup_products(ci, ct, pi, pt, length, lookup_count, beta, gamma, blinds, blinding_factors):
    o = np.zeros((lookup_count * length, 4), dtype=np.uint64)
    arrs = [np.ascontiguousarray(x, dtype=np.uint64) for x in (ci, ct, pi, pt)]
    b = np.ascontiguousarray(blinds if blinds is not None else np.zeros((1, 4)), dtype=np.uint64)
    rc = lib().orc_fr_lookup_products(_p(o), *[_p(x) for x in arrs], length, lookup_count,
                                      _p(np.ascontiguousarray(beta, dtype=np.uint64)),
                                      _p(np.ascontiguousarray(gamma, dtype=np.uint64)),
                                      _p(b), blinding_factors)
    if rc:
        raise ValueError("invalid lookup product arguments")
    return o


def fr_poly_lincomb(polys, poly_len, poly_count, scalars):
    o = np.zeros((poly_len, 4), dtype=np.uint64)
    lib().orc_fr_poly_lincomb(_p(o), _p(np.ascontiguousarray(polys, dtype=np.uint64)), poly_len,
                              poly_count, _p(np.ascontiguousarray(scalars, dtype=np.uint64)))
    return o


def fr_quotient_pieces(quotient, poly_len, piece_count, blinds):
    q = np.ascontiguousarray(quotient, dtype=np.uint64).reshape(-1, 4)
    b = np.ascontiguousarray(blinds, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros((poly_len * piece_count, 4), dtype=np.uint64)
    rc = lib().orc_fr_quotient_pieces(_p(o), _p(q), len(q), poly_len, piece_count, _p(b), len(b))
    if rc:
        raise ValueError("invalid quotient piece arguments")
    return o


def fr_sort_canonical(a):
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4).copy()
    lib().orc_fr_sort_canonical(_p(a), len(a))
    return a


def fr_eval_poly(poly, point):
    a = np.ascontiguousarray(poly, dtype=np.uint64).reshape(-1, 4)
    o = np.zeros(4, dtype=np.uint64)
    lib().orc_fr_eval_poly(_p(o), _p(a), len(a), _p(np.ascontiguousarray(point, dtype=np.uint64)))
    return o


def fr_kate_division(poly, point):
    """(a - a(point)) / (X - point): len(a) - 1 coefficients."""
    a = np.ascontiguousarray(poly, dtype=np.uint64).reshape(-1, 4)
    q = np.zeros((max(len(a) - 1, 0), 4), dtype=np.uint64)
    lib().orc_fr_kate_division(_p(q), _p(a), len(a), _p(np.ascontiguousarray(point, dtype=np.uint64)))
    return q


# ---------------------------------------------------------------- quotient numerator

class _VS(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("a", ctypes.c_uint32), ("b", ctypes.c_uint32)]


class _Calc(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint32), ("target", ctypes.c_uint32), ("parts_offset", ctypes.c_uint32),
                ("parts_len", ctypes.c_uint32), ("lhs", _VS), ("rhs", _VS)]


class _Graph(ctypes.Structure):
    _fields_ = [("constants", ctypes.c_void_p), ("constants_len", ctypes.c_size_t),
                ("rotations", ctypes.c_void_p), ("rotations_len", ctypes.c_size_t),
                ("calculations", ctypes.c_void_p), ("calculations_len", ctypes.c_size_t),
                ("horner_parts", ctypes.c_void_p), ("horner_parts_len", ctypes.c_size_t),
                ("num_intermediates", ctypes.c_uint32)]


class _ColRef(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("index", ctypes.c_uint32)]


class OracleGraph:
    """Same description as the product's Graph: (constants, rotations,
    calcs, parts, num_intermediates)."""

    def __init__(self, constants, rotations, calcs, parts, num_intermediates):
        self.constants = np.ascontiguousarray(np.asarray(constants, dtype=np.uint64).reshape(-1, 4))
        self.rotations = np.ascontiguousarray(np.asarray(rotations, dtype=np.int32))
        self.calcs = (_Calc * max(len(calcs), 1))()
        for i, (op, tgt, po, pl, lhs, rhs) in enumerate(calcs):
            self.calcs[i] = _Calc(op, tgt, po, pl, _VS(*lhs), _VS(*rhs))
        self.parts = (_VS * max(len(parts), 1))()
        for i, pt in enumerate(parts):
            self.parts[i] = _VS(*pt)
        self.n = (len(calcs), len(parts))
        self.ni = num_intermediates

    def raw(self):
        def ptr(a):
            return a.ctypes.data_as(ctypes.c_void_p) if a.size else None
        return _Graph(ptr(self.constants), len(self.constants), ptr(self.rotations), len(self.rotations),
                      ctypes.cast(self.calcs, ctypes.c_void_p), self.n[0], ctypes.cast(self.parts, ctypes.c_void_p),
                      self.n[1], self.ni)


def eval_numerator(length, custom_graph, fixed=None, advice=None, instance=None, challenges=None, beta=None,
                   gamma=None, theta=None, trash_challenge=None, y=None, omega=None, delta_start=None,
                   delta_const=None, rot_scale=1, last_rotation=-1, chunk_len=1, l0=None, l_last=None,
                   l_active=None, permutation_products=None, permutation_sets=0, permutation_columns=(),
                   permutation_pk_cosets=None, lookups=(), trash=(), initial_out=None, threads=None):
    """Evaluator::evaluate_numerator (evaluation.rs:3114-3528) restated in C."""
    L = lib()
    f = L.orc_eval_numerator
    vp = ctypes.c_void_p
    f.restype = ctypes.c_int
    z = np.zeros(4, dtype=np.uint64)

    def arr(a):
        return None if a is None else np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4)

    def p(a):
        return None if a is None or not a.size else a.ctypes.data_as(vp)

    def sc(v):
        return np.ascontiguousarray(z if v is None else v, dtype=np.uint64).reshape(4)

    fx, ad, ins, ch = arr(fixed), arr(advice), arr(instance), arr(challenges)
    lag = [arr(x) for x in (l0, l_last, l_active)]
    pp, pk = arr(permutation_products), arr(permutation_pk_cosets)
    pcols = (_ColRef * max(len(permutation_columns), 1))(*[_ColRef(k, i) for k, i in permutation_columns])
    lk = [np.concatenate([arr(l[i]) for l in lookups]) if lookups else None for i in (1, 2, 3)]
    lkg = (_Graph * max(len(lookups), 1))(*[l[0].raw() for l in lookups])
    trc = np.concatenate([arr(t[1]) for t in trash]) if trash else None
    trs = np.array([t[2] for t in trash] or [0], dtype=np.uint32)
    trg = (_Graph * max(len(trash), 1))(*[t[0].raw() for t in trash])
    scal = [sc(v) for v in (beta, gamma, theta, trash_challenge, y, omega, delta_start, delta_const)]
    init = arr(initial_out)
    cg = custom_graph.raw() if custom_graph is not None else _Graph()
    out = np.zeros((length, 4), dtype=np.uint64)
    rc = f(p(out), ctypes.c_size_t(length), p(init), ctypes.c_uint32(1 if custom_graph is not None else 0),
           p(fx), ctypes.c_size_t(0 if fx is None else len(fx) // length), p(ad),
           ctypes.c_size_t(0 if ad is None else len(ad) // length), p(ins),
           ctypes.c_size_t(0 if ins is None else len(ins) // length), p(ch), ctypes.c_size_t(0 if ch is None else len(ch)),
           *[p(s) for s in scal], ctypes.c_int32(rot_scale), ctypes.c_int32(last_rotation), ctypes.c_uint32(chunk_len),
           p(lag[0]), p(lag[1]), p(lag[2]), p(pp), ctypes.c_size_t(permutation_sets), ctypes.cast(pcols, vp),
           ctypes.c_size_t(len(permutation_columns)), p(pk), p(lk[0]), p(lk[1]), p(lk[2]),
           ctypes.c_size_t(len(lookups)), p(trc), trs.ctypes.data_as(vp), ctypes.c_size_t(len(trash)),
           ctypes.byref(cg), ctypes.cast(lkg, vp), ctypes.cast(trg, vp), ctypes.c_int(threads or threads_default()))
    if rc:
        raise ValueError("invalid numerator arguments")
    return out


# ---------------------------------------------------------------- transcript

def blake2b(data, key=b"", outlen=64):
    L = lib()
    out = (ctypes.c_uint8 * outlen)()
    kb = (ctypes.c_uint8 * max(len(key), 1)).from_buffer_copy(key or b"\0")
    db = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
    L.orc_blake2b(out, ctypes.c_size_t(outlen), kb, ctypes.c_size_t(len(key)), db, ctypes.c_size_t(len(data)))
    return bytes(out)


def transcript_replay(ops):
    """ops: list of ("absorb", bytes) or ("squeeze",); returns the challenges (n, 4)."""
    L = lib()
    n = len(ops)
    kinds = (ctypes.c_uint8 * max(n, 1))(*[1 if o[0] == "absorb" else 0 for o in ops])
    bufs = [(ctypes.c_uint8 * max(len(o[1]), 1)).from_buffer_copy(o[1] or b"\0") if o[0] == "absorb" else None
            for o in ops]
    ptrs = (ctypes.c_void_p * max(n, 1))(*[ctypes.cast(b, ctypes.c_void_p) if b is not None else None for b in bufs])
    lens = (ctypes.c_size_t * max(n, 1))(*[len(o[1]) if o[0] == "absorb" else 0 for o in ops])
    nsq = sum(1 for o in ops if o[0] == "squeeze")
    out = np.zeros((max(nsq, 1), 4), dtype=np.uint64)
    L.orc_transcript_replay(kinds, ctypes.c_size_t(n), ptrs, lens, _p(out))
    return out[:nsq]


# ---------------------------------------------------------------- Poseidon (pure Python, small cases)

POSEIDON_WIDTH, POSEIDON_ROUNDS, POSEIDON_FULL_HALF = 3, 68, 4


def _poseidon_permute(state, mds, rc, wit):
    """One width-3 Poseidon permutation over Fr (canonical ints), the round
    structure of midnight-circuits hash/poseidon (4 full, 60 partial, 4 full
    rounds, x^5) as the reference's GPU kernel runs it
    (midnight-sppark-msm/src/bls12_381_g1_msm.cu:2089-2157): the first round
    constants are added first, each round's MDS output gets the next
    round's constants.  wit, when a list, receives the permutation's 128
    witness values in that kernel's order (full round: three cubes, then
    the three new values; per run of six partial rounds: the new third
    value of its first five, then the three new values)."""
    R = R_MOD
    s = [(state[i] + rc[0][i]) % R for i in range(3)]
    for r in range(POSEIDON_ROUNDS):
        full = r < POSEIDON_FULL_HALF or r >= POSEIDON_ROUNDS - POSEIDON_FULL_HALF
        box = list(s)
        cubes = []
        for i in range(3):
            if full or i == 2:
                cube = pow(s[i], 3, R)
                cubes.append(cube)
                box[i] = cube * s[i] * s[i] % R
        nxt = [((rc[r + 1][i] if r + 1 < POSEIDON_ROUNDS else 0) + sum(mds[i][j] * box[j] for j in range(3))) % R
               for i in range(3)]
        if wit is not None:
            if full:
                wit.extend(cubes)
                wit.extend(nxt)
            else:
                p = (r - POSEIDON_FULL_HALF) % 6
                if p < 5:
                    wit.append(nxt[2])
                else:
                    wit.extend(nxt)
        s = nxt
    return s


def poseidon_hash_chain(initial, tail0, tail1, input_len, mds, rc, length, witness=False):
    """bls12_381_g1_msm.cu:2159-2216: canonical ints in, canonical ints out;
    mds 3 x 3, rc 68 x 3.  Returns the chain's outputs, or with witness=True
    its 256 witness values per hash."""
    prev, outs, wit = initial, [], []
    for _ in range(length):
        st = _poseidon_permute([prev, tail0, input_len], mds, rc, wit if witness else None)
        st[0] = (st[0] + tail1) % R_MOD
        st = _poseidon_permute(st, mds, rc, wit if witness else None)
        prev = st[0]
        outs.append(prev)
    return wit if witness else outs


def poseidon_advice_from_witness(witness, hash_count, domain_len, metadata, layout):
    """bls12_381_g1_msm.cu:2018-2075: 8 advice columns x domain_len rows
    (canonical ints, column-major) from a chain's witness (256 per hash),
    layout = 128 (column, row) pairs and 11 metadata values.  The fixed
    cells of each hash are written after the layout's."""
    R = R_MOD
    out = [[0] * domain_len for _ in range(8)]
    for h in range(hash_count):
        for k in range(256):
            col, row = layout[k % 128]
            out[col][2 + 41 * h + 21 * (k // 128) + row] = witness[h * 256 + k]
    for h in range(hash_count):
        r0 = 2 + 41 * h
        w = witness[h * 256:(h + 1) * 256]
        first = [metadata[4] if h == 0 else witness[(h - 1) * 256 + 253], metadata[5], metadata[7]]
        for c in range(3):
            out[c][r0] = first[c]
            out[c][r0 + 1] = (first[c] + metadata[8 + c]) % R
        absorbed = (w[125] + metadata[6]) % R
        out[0][r0 + 20], out[1][r0 + 20], out[2][r0 + 20] = absorbed, w[125], metadata[6]
        second = [absorbed, w[126], w[127]]
        for c in range(3):
            out[c][r0 + 21] = second[c]
            out[c][r0 + 22] = (second[c] + metadata[8 + c]) % R
    out[0][0], out[1][0], out[2][0], out[0][1] = metadata[0], metadata[1], metadata[2], metadata[3]
    return out
