"""Safe wrappers over the C ABI, named after midnight-sppark-msm/src/lib.rs.

Each function validates shapes like its Rust counterpart (lib.rs:1470-4555)
and raises MsmError on a non-zero RustError.  numpy uint64 arrays in the
reference layout are used throughout: Fr (n, 4), affine (n, 12),
projective (n, 18).
"""
import ctypes

import numpy as np

from ._lib import MsmError, RawFr, RawMsmConfig, RawMsmSlice, check, lib

__all__ = [
    "execution_lane_set", "bls12_381_g1_msm", "bls12_381_g1_msm_batch", "Bls12_381G1MsmContext", "MsmTicket",
    "Bls12_381FrDeviceVec", "bls12_381_fr_ntt", "bls12_381_fr_ntt_zeta", "bls12_381_fr_divide_ntt_zeta",
    "bls12_381_fr_coeff_to_extended_batch", "bls12_381_fr_device_coeff_to_extended_batch",
    "bls12_381_fr_mul_assign", "bls12_381_fr_mul_assign_zeta", "bls12_381_fr_mul_assign_repeating",
    "bls12_381_fr_invert_assign", "bls12_381_fr_sort_canonical", "bls12_381_fr_poly_lincomb",
    "bls12_381_fr_shifted_prefix_product", "bls12_381_fr_permutation_products", "bls12_381_fr_lookup_products",
    "bls12_381_fr_lookup_products_device", "bls12_381_fr_device_quotient_pieces",
    "bls12_381_fr_device_poly_lincomb", "g1_generator_mul", "imad_peak", "imad_probe", "ntt_variant_set", "ntt_wait_timeouts", "transfer_counters",
    "transfer_counters_reset", "launch_counter", "lane_stream", "profile_enable", "profile_read", "profile_reset",
    "msm_graphs_enable", "msm_graph_stats",
    "PROFILE_MSM_ACCUMULATE", "PROFILE_MSM_TOTAL", "PROFILE_NTT", "PROFILE_MSM_SORT",
    "PROFILE_MSM_FIXUP", "PROFILE_MSM_REDUCE", "bls12_381_eval_numerator",
    "bls12_381_eval_graph_batch", "bls12_381_fr_device_eval_polys", "fr_device_eval_many", "fr_device_kate_divide",
    "eval_graph_batch_device", "eval_numerator_device", "fr_permutation_products_device", "fr_random_chacha20",
    "fr_lookup_permute_device", "NumeratorContext", "bls12_381_fr_multiopen_prepare",
    "bls12_381_fr_multiopen_prepare_device", "bls12_381_fr_multiopen_f_poly_device",
    "bls12_381_fr_multiopen_pi_device", "bls12_381_fr_lookup_permute_batch", "hook_mask_delay",
    "bls12_381_fr_poseidon_hash_chain", "bls12_381_fr_poseidon_advice_from_witness",
    "hook_delayed_scale", "autotune_set", "autotune_reset", "autotune_report", "ntt_wait_limit_set",
    "FR_GENERATOR", "fr_coeff_to_extended_coset_batch", "fr_device_coeff_to_extended_coset_batch", "fr_ntt_coset",
    "fr_lde_coset", "g1_msm_device",
]

# GENERATOR = 7 (vendor/midnight-curves-0.3.1/src/bls12_381/fq.rs:31-33), Montgomery limbs: the coset
# generator of sppark's coset NTT and LDE (vendor/sppark-0.1.15/sppark/ntt/parameters/bls12_381.h:11)
FR_GENERATOR = np.array([0x0000000EFFFFFFF1, 0x17E363D300189C0F, 0xFF9C57876F8457B0, 0x351332208FC5A8C4],
                        dtype=np.uint64)

PROFILE_MSM_ACCUMULATE, PROFILE_MSM_TOTAL, PROFILE_NTT = 0, 1, 2
# MSM phases: recode + sort, bucket fix-up, bucket reduction + window combination
PROFILE_MSM_SORT, PROFILE_MSM_FIXUP, PROFILE_MSM_REDUCE = 3, 4, 5


def _fr_arr(a):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    return a.reshape(-1, 4)


def _aff_arr(a):
    return np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 12)


def _ptr(a):
    """the address of array a's data, for one foreign call; the caller keeps
    a alive until that call returns (a named array, not a temporary)"""
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def _fr(v):
    return RawFr.from_buffer_copy(np.ascontiguousarray(v, dtype=np.uint64).reshape(4))


def execution_lane_set(lane):
    check(lib().midnight_sppark_execution_lane_set(lane))


# ---------------------------------------------------------------- MSM

def bls12_381_g1_msm(points, scalars):
    """lib.rs bls12_381_g1_msm: sum_i scalars[i] * points[i] (projective)."""
    p, s = _aff_arr(points), _fr_arr(scalars)
    if len(p) != len(s):
        raise MsmError(-1, "point/scalar length mismatch: %d points, %d scalars" % (len(p), len(s)))
    out = np.zeros(18, dtype=np.uint64)
    check(lib().midnight_sppark_bls12_381_g1_msm(_ptr(out), _ptr(p), _ptr(s), len(s)))
    return out


def bls12_381_g1_msm_batch(points, scalars_batch):
    p = _aff_arr(points)
    s = np.ascontiguousarray(scalars_batch, dtype=np.uint64).reshape(-1, len(p), 4)
    out = np.zeros((len(s), 18), dtype=np.uint64)
    check(lib().midnight_sppark_bls12_381_g1_msm_batch(_ptr(out), _ptr(p), _ptr(s), len(p), len(s)))
    return out


class Bls12_381G1MsmContext:
    """lib.rs Bls12_381G1MsmContext: bases uploaded once, reused per call."""

    def __init__(self, points, config=None):
        p = _aff_arr(points)
        self.npoints = len(p)
        cfg = config if config is not None else RawMsmConfig.default(self.npoints)
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_g1_msm_context_create_with_config(ctypes.byref(h), _ptr(p),
                                                                                len(p), cfg))
        self.raw = h

    def device_bytes(self):
        """bytes of device memory the context holds (its precomputed table)"""
        return lib().gb_g1_msm_context_device_bytes(self.raw) if self.raw else 0

    def close(self):
        if self.raw:
            lib().midnight_sppark_bls12_381_g1_msm_context_free(self.raw)
            self.raw = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def batch(self, scalars_batch, npoints=None):
        n = self.npoints if npoints is None else npoints
        s = np.ascontiguousarray(scalars_batch, dtype=np.uint64).reshape(-1, n, 4)
        out = np.zeros((len(s), 18), dtype=np.uint64)
        check(lib().midnight_sppark_bls12_381_g1_msm_context_batch(_ptr(out), self.raw, _ptr(s), n, len(s)))
        return out

    def msm(self, scalars):
        return self.batch(_fr_arr(scalars)[None], npoints=len(_fr_arr(scalars)))[0]

    def device_batch(self, devvec, scalar_offset, npoints, nmsms):
        out = np.zeros((max(nmsms, 1), 18), dtype=np.uint64)
        check(lib().midnight_sppark_bls12_381_g1_msm_context_device_batch(_ptr(out), self.raw, devvec.raw,
                                                                         scalar_offset, npoints, nmsms))
        return out[:nmsms]

    def device_batch_async(self, devvec, scalar_offset, npoints, nmsms):
        """device_batch queued without waiting (gb_g1_msm_context_device_batch_async):
        returns an MsmTicket whose wait() gives the points"""
        h = ctypes.c_void_p()
        check(lib().gb_g1_msm_context_device_batch_async(ctypes.byref(h), self.raw, devvec.raw, scalar_offset,
                                                          npoints, nmsms))
        return MsmTicket(h, nmsms)

    def device_ragged(self, devvec, slices):
        arr = (RawMsmSlice * max(len(slices), 1))()
        for i, (so, po, ln) in enumerate(slices):
            arr[i] = RawMsmSlice(so, po, ln, ln)
        out = np.zeros((max(len(slices), 1), 18), dtype=np.uint64)
        check(lib().midnight_sppark_bls12_381_g1_msm_context_device_ragged(_ptr(out), self.raw, devvec.raw,
                                                                          ctypes.cast(arr, ctypes.c_void_p),
                                                                          len(slices)))
        return out[:len(slices)]

    def device_scrambled_batch(self, devvec, scalar_offset, nmsms, mask_devvec):
        out = np.zeros((max(nmsms, 1), 18), dtype=np.uint64)
        check(lib().midnight_sppark_bls12_381_g1_msm_context_device_scrambled_batch(
            _ptr(out), self.raw, devvec.raw, scalar_offset, self.npoints, nmsms, mask_devvec.raw))
        return out[:nmsms]


# ---------------------------------------------------------------- device vectors

class MsmTicket:
    """An MSM batch in flight; wait() returns its (nmsms, 18) projective
    points once, and releases the library's handle."""

    def __init__(self, raw, nmsms):
        self.raw, self.nmsms = raw, nmsms

    def wait(self):
        if not self.raw:
            raise RuntimeError("MSM ticket already waited for")
        out = np.zeros((max(self.nmsms, 1), 18), dtype=np.uint64)
        raw, self.raw = self.raw, None
        check(lib().gb_msm_ticket_wait(raw, _ptr(out)))
        return out[:self.nmsms]

    def __del__(self):
        if getattr(self, "raw", None):
            try:
                lib().gb_msm_ticket_wait(self.raw, None)
            except Exception:
                pass
            self.raw = None


class Bls12_381FrDeviceVec:
    """lib.rs Bls12_381FrDeviceVec: an opaque resident vector of Fr."""

    def __init__(self, raw):
        self.raw = ctypes.c_void_p(raw) if not isinstance(raw, ctypes.c_void_p) else raw
        self.len = lib().gb_fr_device_vec_len(self.raw)

    @classmethod
    def upload(cls, values):
        v = _fr_arr(values)
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_fr_device_vec_upload(ctypes.byref(h), _ptr(v), len(v)))
        return cls(h)

    @classmethod
    def upload_many(cls, slices):
        arrs = [_fr_arr(s) for s in slices]
        ptrs = (ctypes.c_void_p * max(len(arrs), 1))(*[_ptr(a) for a in arrs])
        lens = (ctypes.c_size_t * max(len(arrs), 1))(*[len(a) for a in arrs])
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_fr_device_vec_upload_many(ctypes.byref(h), ptrs, lens, len(arrs)))
        return cls(h)

    def download(self, length=None):
        n = self.len if length is None else length
        out = np.zeros((n, 4), dtype=np.uint64)
        check(lib().midnight_sppark_bls12_381_fr_device_vec_download(_ptr(out), self.raw, n))
        return out

    def scatter_host(self, indices, values):
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        v = _fr_arr(values)
        check(lib().midnight_sppark_bls12_381_fr_device_vec_scatter_host(self.raw, _ptr(idx), _ptr(v), len(idx)))

    def concat_host(self, suffix):
        v = _fr_arr(suffix)
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_fr_device_vec_concat_host(ctypes.byref(h), self.raw, _ptr(v), len(v)))
        return Bls12_381FrDeviceVec(h)

    @staticmethod
    def concat_many_host(sources, suffix):
        v = _fr_arr(suffix)
        srcs = (ctypes.c_void_p * max(len(sources), 1))(*[s.raw.value for s in sources])
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_fr_device_vec_concat_many_host(ctypes.byref(h), srcs, len(sources),
                                                                             _ptr(v), len(v)))
        return Bls12_381FrDeviceVec(h)

    def gather_polys(self, poly_len, indices):
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_fr_device_vec_gather_polys(ctypes.byref(h), self.raw, poly_len,
                                                                         _ptr(idx), len(idx)))
        return Bls12_381FrDeviceVec(h)

    def download_nonzero_suffixes(self, scalar_offset, poly_len, count):
        """(packed suffixes, starts, nonzero counts): each polynomial from its
        first nonzero coefficient on (lib.rs:2035-2160)."""
        n_out = ctypes.c_size_t()
        starts = np.zeros(count, dtype=np.uint64)
        live = np.zeros(count, dtype=np.uint64)
        f = lib().midnight_sppark_bls12_381_fr_device_vec_download_nonzero_suffixes
        check(f(None, 0, ctypes.byref(n_out), _ptr(starts), _ptr(live), self.raw, scalar_offset, poly_len, count))
        out = np.zeros((max(n_out.value, 1), 4), dtype=np.uint64)
        check(f(_ptr(out), n_out.value, ctypes.byref(n_out), _ptr(starts), _ptr(live), self.raw, scalar_offset,
                poly_len, count))
        return out[:n_out.value], starts, live

    def ntt_zeta(self, log_n, inverse, scale, first, second):
        check(lib().midnight_sppark_bls12_381_fr_device_vec_ntt_zeta(self.raw, log_n, inverse, _fr(scale),
                                                                      _fr(first), _fr(second)))

    def ntt_zeta_batch(self, log_n, count, inverse, scale, first, second):
        check(lib().midnight_sppark_bls12_381_fr_device_vec_ntt_zeta_batch(self.raw, log_n, count, inverse,
                                                                            _fr(scale), _fr(first), _fr(second)))

    def ntt_ragged(self, offsets, log_ns, inverse, scale, first, second):
        """NTTs of polynomials of different sizes in this vector, one
        persistent launch (gb_fr_device_vec_ntt_ragged): polynomial j is the
        2^log_ns[j] values from offsets[j]."""
        off = np.ascontiguousarray(offsets, dtype=np.uintp)
        lg = np.ascontiguousarray(log_ns, dtype=np.uint32)
        if len(off) != len(lg):
            raise ValueError("offsets and log_ns differ in length")
        check(lib().gb_fr_device_vec_ntt_ragged(self.raw, _ptr(off), _ptr(lg), len(off), inverse, _fr(scale),
                                                _fr(first), _fr(second)))

    def ntt_coset_batch(self, log_n, count, inverse, shift=FR_GENERATOR):
        """sppark's coset NTT in place (gb_fr_device_vec_ntt_coset_batch):
        forward NTT(a_i shift^i), inverse iNTT(a)_i shift^-i."""
        check(lib().gb_fr_device_vec_ntt_coset_batch(self.raw, log_n, count, inverse, _fr(shift)))

    def divide_ntt_zeta(self, log_n, factors, scale, first, second):
        f = _fr_arr(factors)
        check(lib().midnight_sppark_bls12_381_fr_device_vec_divide_ntt_zeta(self.raw, log_n, _ptr(f), len(f),
                                                                             _fr(scale), _fr(first), _fr(second)))

    def free(self):
        if self.raw:
            lib().midnight_sppark_bls12_381_fr_device_vec_free(self.raw)
            self.raw = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---------------------------------------------------------------- NTT

def _log2_exact(n):
    if n == 0 or n & (n - 1):
        raise MsmError(-1, "NTT input length must be a power of two, got %d" % n)
    return n.bit_length() - 1


def bls12_381_fr_ntt(values, inverse=False):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_ntt(_ptr(v), _log2_exact(len(v)), inverse))
    return v


def bls12_381_fr_ntt_zeta(values, inverse, scale, first, second):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_ntt_zeta(_ptr(v), _log2_exact(len(v)), inverse, _fr(scale), _fr(first),
                                                      _fr(second)))
    return v


def bls12_381_fr_divide_ntt_zeta(values, factors, scale, first, second):
    v = _fr_arr(values).copy()
    f = _fr_arr(factors)
    check(lib().midnight_sppark_bls12_381_fr_divide_ntt_zeta(_ptr(v), _log2_exact(len(v)), _ptr(f), len(f),
                                                             _fr(scale), _fr(first), _fr(second)))
    return v


def bls12_381_fr_coeff_to_extended_batch(inputs, extended_log_n, first, second):
    a = np.ascontiguousarray(inputs, dtype=np.uint64)
    a = a.reshape(a.shape[0], -1, 4) if a.ndim == 3 else a.reshape(1, -1, 4)
    count, input_len = a.shape[0], a.shape[1]
    out = np.zeros((count, 1 << extended_log_n, 4), dtype=np.uint64)
    check(lib().midnight_sppark_bls12_381_fr_coeff_to_extended_batch(_ptr(out), _ptr(a), input_len, count,
                                                                      extended_log_n, _fr(first), _fr(second)))
    return out


def bls12_381_fr_device_coeff_to_extended_batch(inputs, extended_log_n, first, second):
    a = np.ascontiguousarray(inputs, dtype=np.uint64)
    a = a.reshape(a.shape[0], -1, 4) if a.ndim == 3 else a.reshape(1, -1, 4)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_device_coeff_to_extended_batch(ctypes.byref(h), _ptr(a), a.shape[1],
                                                                            a.shape[0], extended_log_n, _fr(first),
                                                                            _fr(second)))
    return Bls12_381FrDeviceVec(h)


def fr_coeff_to_extended_coset_batch(inputs, extended_log_n, shift=FR_GENERATOR):
    """coefficients (count, input_len, 4) -> evaluations on shift * <w_ext>,
    (count, 2^extended_log_n, 4): the coset LDE by the powers of shift."""
    a = np.ascontiguousarray(inputs, dtype=np.uint64)
    a = a.reshape(a.shape[0], -1, 4) if a.ndim == 3 else a.reshape(1, -1, 4)
    count, input_len = a.shape[0], a.shape[1]
    out = np.zeros((count, 1 << extended_log_n, 4), dtype=np.uint64)
    check(lib().gb_fr_coeff_to_extended_coset_batch(_ptr(out), _ptr(a), input_len, count, extended_log_n,
                                                    _fr(shift)))
    return out


def fr_device_coeff_to_extended_coset_batch(source, input_len, count, extended_log_n, shift=FR_GENERATOR):
    """the same from a resident vector into a new one"""
    h = ctypes.c_void_p()
    check(lib().gb_fr_device_coeff_to_extended_coset_batch(ctypes.byref(h), source.raw, input_len, count,
                                                           extended_log_n, _fr(shift)))
    return Bls12_381FrDeviceVec(h)


def fr_ntt_coset(values, inverse=False, shift=FR_GENERATOR):
    """sppark NTT::Base(..., Type::coset) on one polynomial"""
    v = _fr_arr(values).copy()
    check(lib().gb_fr_ntt_coset(_ptr(v), _log2_exact(len(v)), inverse, _fr(shift)))
    return v


def fr_lde_coset(values, lg_blowup):
    """sppark NTT::LDE: evaluations -> evaluations on the generator coset of
    the domain 2^lg_blowup times larger"""
    v = _fr_arr(values)
    lg = _log2_exact(len(v))
    out = np.zeros((len(v) << lg_blowup, 4), dtype=np.uint64)
    check(lib().gb_fr_lde_coset(_ptr(out), _ptr(v), lg, lg_blowup))
    return out


# ---------------------------------------------------------------- vector ops

def bls12_381_fr_mul_assign(values, scalar):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_mul_assign(_ptr(v), _fr(scalar), len(v)))
    return v


def bls12_381_fr_mul_assign_zeta(values, first, second):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_mul_assign_zeta(_ptr(v), _fr(first), _fr(second), len(v)))
    return v


def bls12_381_fr_mul_assign_repeating(values, factors):
    v = _fr_arr(values).copy()
    f = _fr_arr(factors)
    check(lib().midnight_sppark_bls12_381_fr_mul_assign_repeating(_ptr(v), _ptr(f), len(f), len(v)))
    return v


def bls12_381_fr_invert_assign(values):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_invert_assign(_ptr(v), len(v)))
    return v


def bls12_381_fr_sort_canonical(values):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_sort_canonical(_ptr(v), len(v)))
    return v


def bls12_381_fr_poly_lincomb(polys, scalars):
    p = np.ascontiguousarray(polys, dtype=np.uint64)
    count = p.shape[0]
    p = p.reshape(count, -1, 4)
    k = _fr_arr(scalars)
    out = np.zeros((p.shape[1], 4), dtype=np.uint64)
    check(lib().midnight_sppark_bls12_381_fr_poly_lincomb(_ptr(out), _ptr(p), p.shape[1], count, _ptr(k)))
    return out


def bls12_381_fr_shifted_prefix_product(values, initial):
    v = _fr_arr(values).copy()
    check(lib().midnight_sppark_bls12_381_fr_shifted_prefix_product(_ptr(v), _fr(initial), len(v)))
    return v


# ---------------------------------------------------------------- products

def bls12_381_fr_permutation_products(columns, permutations, length, column_count, chunk_len, beta, gamma, omega,
                                      delta_powers, blind_values, blinding_factors):
    c = _fr_arr(columns)
    p = _fr_arr(permutations)
    d = _fr_arr(delta_powers)
    b = _fr_arr(blind_values) if blind_values is not None and len(blind_values) else None
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_permutation_products(
        ctypes.byref(h), _ptr(c), _ptr(p), length, column_count, chunk_len, _fr(beta), _fr(gamma), _fr(omega),
        _ptr(d), _ptr(b), blinding_factors))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_lookup_products(ci, ct, pi, pt, length, lookup_count, beta, gamma, blind_values, blinding_factors):
    arrs = [_fr_arr(x) for x in (ci, ct, pi, pt)]
    b = _fr_arr(blind_values) if blind_values is not None and len(blind_values) else None
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_lookup_products(ctypes.byref(h), *[_ptr(a) for a in arrs], length,
                                                             lookup_count, _fr(beta), _fr(gamma), _ptr(b),
                                                             blinding_factors))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_lookup_products_device(trace, length, lookup_count, beta, gamma, blind_values, blinding_factors):
    b = _fr_arr(blind_values) if blind_values is not None and len(blind_values) else None
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_lookup_products_device(ctypes.byref(h), trace.raw, length, lookup_count,
                                                                    _fr(beta), _fr(gamma), _ptr(b), blinding_factors))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_device_quotient_pieces(quotient, poly_len, piece_count, blinds):
    b = _fr_arr(blinds)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_device_quotient_pieces(ctypes.byref(h), quotient.raw, poly_len,
                                                                    piece_count, _ptr(b), len(b)))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_device_poly_lincomb(polys, poly_len, poly_count, scalars):
    k = _fr_arr(scalars)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_device_poly_lincomb(ctypes.byref(h), polys.raw, poly_len, poly_count,
                                                                 _ptr(k), len(k)))
    return Bls12_381FrDeviceVec(h)


# ---------------------------------------------------------------- additions

def g1_generator_mul(scalars):
    s = _fr_arr(scalars)
    out = np.zeros((len(s), 12), dtype=np.uint64)
    check(lib().gb_g1_generator_mul(_ptr(out), _ptr(s), len(s)))
    return out


def g1_msm_device(d_points, d_scalars, n):
    """gb_g1_msm_device: one MSM over n affine bases and n scalars at device
    addresses d_points / d_scalars (ints, e.g. torch data_ptr()), no
    precomputed table; the projective result as (18,) uint64."""
    out = np.zeros(18, dtype=np.uint64)
    check(lib().gb_g1_msm_device(_ptr(out), ctypes.c_void_p(d_points), ctypes.c_void_p(d_scalars), n))
    return out


def imad_peak():
    v = ctypes.c_double()
    check(lib().gb_imad_peak(ctypes.byref(v)))
    return v.value


def imad_probe(form):
    """Multiply-adds per second of one probe form (0 = mad.wide chains,
    1..3 = carry-chained rows with 1, 2, 4 accumulator sets per thread)."""
    v = ctypes.c_double()
    check(lib().gb_imad_probe(int(form), ctypes.byref(v)))
    return v.value


def transfer_counters():
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    lib().gb_transfer_counters(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def transfer_counters_reset():
    lib().gb_transfer_counters_reset()


def launch_counter():
    return lib().gb_launch_counter()


def lane_stream():
    """cudaStream_t of the calling thread's lane (as an int)."""
    return lib().gb_lane_stream() or 0


def profile_enable(on=True):
    lib().gb_profile_enable(1 if on else 0)


def profile_read(slot):
    ms, n = ctypes.c_double(), ctypes.c_uint64()
    lib().gb_profile_read(slot, ctypes.byref(ms), ctypes.byref(n))
    return ms.value, n.value


def profile_reset():
    lib().gb_profile_reset()


def msm_graphs_enable(on=True):
    """CUDA-graph replay of repeated context batch shapes (on by default)."""
    check(lib().gb_msm_graphs_enable(1 if on else 0))


def msm_graph_stats():
    """(graphs captured, batches replayed) since the process started."""
    cap, lau = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    check(lib().gb_msm_graph_stats(ctypes.byref(cap), ctypes.byref(lau)))
    return cap.value, lau.value


# ---------------------------------------------------------------- quotient numerator

def _cols(a, length):
    if a is None:
        return None, 0
    a = _fr_arr(a)
    return a, len(a) // length if length else 0


def bls12_381_eval_numerator(length, custom_graph, fixed=None, advice=None, instance=None, challenges=None,
                             beta=None, gamma=None, theta=None, trash_challenge=None, y=None, omega=None,
                             delta_start=None, delta_const=None, rot_scale=1, last_rotation=-1, chunk_len=1,
                             l0=None, l_last=None, l_active=None, permutation_products=None, permutation_sets=0,
                             permutation_columns=(), permutation_pk_cosets=None, lookups=(), trash=(),
                             initial_out=None):
    """midnight_sppark_bls12_381_eval_numerator (evaluation.rs:3114-3528).
    lookups: list of (graph, product_coset, input_coset, table_coset);
    trash: list of (graph, trash_coset, selector_fixed_index)."""
    from .graph import column_refs, graph_array
    z = np.zeros(4, dtype=np.uint64)
    fx, nf = _cols(fixed, length)
    ad, na = _cols(advice, length)
    ins, ni = _cols(instance, length)
    ch = _fr_arr(challenges) if challenges is not None else None
    lag = [None if x is None else _fr_arr(x) for x in (l0, l_last, l_active)]
    pp = None if permutation_products is None else _fr_arr(permutation_products)
    pk = None if permutation_pk_cosets is None else _fr_arr(permutation_pk_cosets)
    pcols = column_refs(list(permutation_columns))
    lk_prod = np.concatenate([_fr_arr(l[1]) for l in lookups]) if lookups else None
    lk_in = np.concatenate([_fr_arr(l[2]) for l in lookups]) if lookups else None
    lk_tab = np.concatenate([_fr_arr(l[3]) for l in lookups]) if lookups else None
    lk_g = graph_array([l[0] for l in lookups])
    tr_c = np.concatenate([_fr_arr(t[1]) for t in trash]) if trash else None
    tr_s = np.array([t[2] for t in trash] or [0], dtype=np.uint32)
    tr_g = graph_array([t[0] for t in trash])
    init = None if initial_out is None else _fr_arr(initial_out)
    out = np.zeros((length, 4), dtype=np.uint64)
    g = custom_graph.raw() if custom_graph is not None else graph_array([])[0]
    f = lambda v: _fr(z if v is None else v)  # noqa: E731
    check(lib().midnight_sppark_bls12_381_eval_numerator(
        _ptr(out), length, _ptr(init), 1 if custom_graph is not None else 0, _ptr(fx), nf, _ptr(ad), na, _ptr(ins),
        ni, _ptr(ch), 0 if ch is None else len(ch), f(beta), f(gamma), f(theta), f(trash_challenge), f(y), f(omega),
        f(delta_start), f(delta_const), rot_scale, last_rotation, chunk_len, _ptr(lag[0]), _ptr(lag[1]),
        _ptr(lag[2]), _ptr(pp), permutation_sets, ctypes.cast(pcols, ctypes.c_void_p), len(permutation_columns),
        _ptr(pk), 0 if pk is None else len(pk) // length, _ptr(lk_prod), _ptr(lk_in), _ptr(lk_tab), len(lookups),
        _ptr(tr_c), _ptr(tr_s), len(trash), g, ctypes.cast(lk_g, ctypes.c_void_p),
        ctypes.cast(tr_g, ctypes.c_void_p)))
    return out


def bls12_381_eval_graph_batch(length, graphs, fixed=None, advice=None, instance=None, challenges=None,
                               beta=None, gamma=None, theta=None, trash_challenge=None, y=None, rot_scale=1):
    from .graph import graph_array
    z = np.zeros(4, dtype=np.uint64)
    fx, nf = _cols(fixed, length)
    ad, na = _cols(advice, length)
    ins, ni = _cols(instance, length)
    ch = _fr_arr(challenges) if challenges is not None else None
    ga = graph_array(list(graphs))
    out = np.zeros((len(graphs), length, 4), dtype=np.uint64)
    f = lambda v: _fr(z if v is None else v)  # noqa: E731
    check(lib().midnight_sppark_bls12_381_eval_graph_batch(
        _ptr(out), length, _ptr(fx), nf, _ptr(ad), na, _ptr(ins), ni, _ptr(ch), 0 if ch is None else len(ch),
        f(beta), f(gamma), f(theta), f(trash_challenge), f(y), rot_scale, ctypes.cast(ga, ctypes.c_void_p),
        len(graphs)))
    return out


# ---------------------------------------------------------------- opening helpers

def bls12_381_fr_device_eval_polys(devvec, poly_len, poly_count, point):
    out = np.zeros((poly_count, 4), dtype=np.uint64)
    check(lib().midnight_sppark_bls12_381_fr_device_eval_polys(_ptr(out), devvec.raw, poly_len, poly_count,
                                                                _fr(point)))
    return out


def fr_device_eval_many(requests, poly_len):
    """Several evaluations in one call (gb_fr_device_eval_many): requests are
    (device vector, polynomial count, point); returns one (count, 4) array
    per request."""
    vecs = (ctypes.c_void_p * len(requests))(*[r[0].raw for r in requests])
    counts = np.array([r[1] for r in requests], dtype=np.uintp)
    points = _fr_arr([r[2] for r in requests])
    out = np.zeros((int(counts.sum()), 4), dtype=np.uint64)
    check(lib().gb_fr_device_eval_many(_ptr(out), ctypes.cast(vecs, ctypes.c_void_p), _ptr(counts), _ptr(points),
                                       len(requests), poly_len))
    res, o = [], 0
    for r in requests:
        res.append(out[o:o + r[1]])
        o += r[1]
    return res


def fr_device_kate_divide(devvec, poly_len, poly_count, point):
    h = ctypes.c_void_p()
    check(lib().gb_fr_device_kate_divide(ctypes.byref(h), devvec.raw, poly_len, poly_count, _fr(point)))
    return Bls12_381FrDeviceVec(h)


# ---------------------------------------------------------------- resident argument / quotient forms

def _raw(v):
    return None if v is None else v.raw


def fr_permutation_products_device(columns, permutations, length, column_count, chunk_len, beta, gamma, omega,
                                   delta_powers, blind_values, blinding_factors):
    d = _fr_arr(delta_powers)
    b = _fr_arr(blind_values) if blind_values is not None and len(blind_values) else None
    h = ctypes.c_void_p()
    check(lib().gb_fr_permutation_products_device(ctypes.byref(h), columns.raw, permutations.raw, length,
                                                  column_count, chunk_len, _fr(beta), _fr(gamma), _fr(omega),
                                                  _ptr(d), _ptr(b), blinding_factors))
    return Bls12_381FrDeviceVec(h)


def eval_graph_batch_device(length, graphs, fixed=None, fixed_cols=0, advice=None, advice_cols=0, instance=None,
                            instance_cols=0, challenges=None, beta=None, gamma=None, theta=None,
                            trash_challenge=None, y=None, rot_scale=1):
    from .graph import graph_array
    z = np.zeros(4, dtype=np.uint64)
    ch = _fr_arr(challenges) if challenges is not None else None
    ga = graph_array(list(graphs))
    f = lambda v: _fr(z if v is None else v)  # noqa: E731
    h = ctypes.c_void_p()
    check(lib().gb_eval_graph_batch_device(
        ctypes.byref(h), length, _raw(fixed), fixed_cols, _raw(advice), advice_cols, _raw(instance), instance_cols,
        _ptr(ch), 0 if ch is None else len(ch), f(beta), f(gamma), f(theta), f(trash_challenge), f(y), rot_scale,
        ctypes.cast(ga, ctypes.c_void_p), len(graphs)))
    return Bls12_381FrDeviceVec(h)


def eval_numerator_device(length, custom_graph, fixed=None, fixed_cols=0, advice=None, advice_cols=0,
                          instance=None, instance_cols=0, challenges=None, beta=None, gamma=None, theta=None,
                          trash_challenge=None, y=None, omega=None, delta_start=None, delta_const=None, rot_scale=1,
                          last_rotation=-1, chunk_len=1, lagrange=None, permutation_products=None,
                          permutation_sets=0, permutation_columns=(), permutation_pk_cosets=None,
                          permutation_pk_count=0, lookup_products=None, lookup_permuted=None, lookup_graphs=(),
                          trash=None, trash_selectors=(), trash_graphs=(), initial=None):
    """gb_eval_numerator_device: every column argument a Bls12_381FrDeviceVec;
    lagrange = l0 | l_last | l_active; lookup_permuted = per lookup its
    permuted input then permuted table coset."""
    from .graph import column_refs, graph_array
    z = np.zeros(4, dtype=np.uint64)
    ch = _fr_arr(challenges) if challenges is not None else None
    pcols = column_refs(list(permutation_columns))
    lk_g = graph_array(list(lookup_graphs))
    tr_g = graph_array(list(trash_graphs))
    tr_s = np.array(list(trash_selectors) or [0], dtype=np.uint32)
    g = custom_graph.raw() if custom_graph is not None else graph_array([])[0]
    f = lambda v: _fr(z if v is None else v)  # noqa: E731
    h = ctypes.c_void_p()
    check(lib().gb_eval_numerator_device(
        ctypes.byref(h), length, _raw(initial), 1 if custom_graph is not None else 0, _raw(fixed), fixed_cols,
        _raw(advice), advice_cols, _raw(instance), instance_cols, _ptr(ch), 0 if ch is None else len(ch), f(beta),
        f(gamma), f(theta), f(trash_challenge), f(y), f(omega), f(delta_start), f(delta_const), rot_scale,
        last_rotation, chunk_len, _raw(lagrange), _raw(permutation_products), permutation_sets,
        ctypes.cast(pcols, ctypes.c_void_p), len(permutation_columns), _raw(permutation_pk_cosets),
        permutation_pk_count, _raw(lookup_products), _raw(lookup_permuted), len(lookup_graphs), _raw(trash),
        _ptr(tr_s), len(trash_graphs), g, ctypes.cast(lk_g, ctypes.c_void_p), ctypes.cast(tr_g, ctypes.c_void_p)))
    return Bls12_381FrDeviceVec(h)


def fr_random_chacha20(key32, word_offset, n):
    """(device vector of n Montgomery values, keystream words consumed)"""
    key = (ctypes.c_uint8 * 32).from_buffer_copy(bytes(key32))
    used = ctypes.c_uint64()
    h = ctypes.c_void_p()
    check(lib().gb_fr_random_chacha20(ctypes.byref(h), key, word_offset, n, ctypes.byref(used)))
    return Bls12_381FrDeviceVec(h), used.value


def fr_lookup_permute_device(compressed, length, usable_rows, lookup_count, input_blinds, table_blinds):
    ib = _fr_arr(input_blinds) if len(input_blinds) else None
    tb = _fr_arr(table_blinds) if len(table_blinds) else None
    h = ctypes.c_void_p()
    check(lib().gb_fr_lookup_permute_device(ctypes.byref(h), compressed.raw, length, usable_rows, lookup_count,
                                            _ptr(ib), _ptr(tb)))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_lookup_permute_batch(compressed_inputs, compressed_tables, length, lookup_count, usable_rows,
                                      input_blinds, table_blinds):
    """midnight_sppark_bls12_381_fr_lookup_permute_batch: a device vector
    [inputs | tables | permuted inputs | permuted tables]."""
    ci, ct = _fr_arr(compressed_inputs), _fr_arr(compressed_tables)
    nb = length - usable_rows
    ib = _fr_arr(input_blinds) if nb else np.zeros((1, 4), dtype=np.uint64)
    tb = _fr_arr(table_blinds) if nb else np.zeros((1, 4), dtype=np.uint64)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_lookup_permute_batch(
        ctypes.byref(h), _ptr(ci), _ptr(ct), length, lookup_count, usable_rows, ib.ctypes.data_as(ctypes.c_void_p),
        tb.ctypes.data_as(ctypes.c_void_p), nb))
    return Bls12_381FrDeviceVec(h)


def hook_mask_delay(delay_ms):
    """test hook: delay the next scrambled batches' mask producer"""
    lib().midnight_sppark_test_mask_delay(int(delay_ms))


def hook_delayed_scale(vec, scale, delay_ms):
    """test hook: vec *= scale on this lane after holding it back delay_ms"""
    check(lib().midnight_sppark_test_delayed_scale(vec.raw, _fr(scale), int(delay_ms)))


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def bls12_381_fr_multiopen_prepare(polys, poly_len, q_offsets, q_poly_indices, q_coefficients, points,
                                   query_poly_indices, query_point_indices):
    """midnight_sppark_bls12_381_fr_multiopen_prepare: host polynomials
    [poly_count][poly_len]; returns (q [q_count * poly_len], evaluations
    [query_count])."""
    p = _fr_arr(polys)
    qo, qi, qc = _u32(q_offsets), _u32(q_poly_indices), _fr_arr(q_coefficients)
    pts, rp, rq = _fr_arr(points), _u32(query_poly_indices), _u32(query_point_indices)
    q = np.zeros(((len(qo) - 1) * poly_len, 4), dtype=np.uint64)
    ev = np.zeros((max(len(rp), 1), 4), dtype=np.uint64)
    check(lib().midnight_sppark_bls12_381_fr_multiopen_prepare(
        _ptr(q), _ptr(ev), _ptr(p), poly_len, len(p) // poly_len, _ptr(qo), len(qo), _ptr(qi), _ptr(qc), len(qi),
        _ptr(pts), len(pts), _ptr(rp), _ptr(rq), len(rp)))
    return q, ev[:len(rp)]


def bls12_381_fr_multiopen_prepare_device(sources, poly_len, poly_refs, q_offsets, q_poly_indices, q_coefficients,
                                          points, query_poly_indices, query_point_indices, q_host=True):
    """..._multiopen_prepare_device: sources = (dynamic, fixed, extra)
    Bls12_381FrDeviceVec, poly_refs = [(source, index)]; returns (q on the
    host or None, q as a new device vector, evaluations)."""
    from ._lib import RawDevicePolyRef
    refs = (RawDevicePolyRef * max(len(poly_refs), 1))()
    for i, (src, idx) in enumerate(poly_refs):
        refs[i] = RawDevicePolyRef(src, idx)
    qo, qi, qc = _u32(q_offsets), _u32(q_poly_indices), _fr_arr(q_coefficients)
    pts, rp, rq = _fr_arr(points), _u32(query_poly_indices), _u32(query_point_indices)
    q = np.zeros(((len(qo) - 1) * poly_len, 4), dtype=np.uint64) if q_host else None
    ev = np.zeros((max(len(rp), 1), 4), dtype=np.uint64)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_multiopen_prepare_device(
        _ptr(q), ctypes.byref(h), _ptr(ev), sources[0].raw, sources[1].raw, sources[2].raw, poly_len,
        ctypes.cast(refs, ctypes.c_void_p), len(poly_refs), _ptr(qo), len(qo), _ptr(qi), _ptr(qc), len(qi),
        _ptr(pts), len(pts), _ptr(rp), _ptr(rq), len(rp)))
    return q, Bls12_381FrDeviceVec(h), ev[:len(rp)]


def bls12_381_fr_multiopen_f_poly_device(q_vec, poly_len, point_offsets, points, combination_scalars):
    po, pts, sc = _u32(point_offsets), _fr_arr(points), _fr_arr(combination_scalars)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_multiopen_f_poly_device(
        ctypes.byref(h), q_vec.raw, poly_len, _ptr(po), len(po), _ptr(pts), len(pts), _ptr(sc), len(sc)))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_multiopen_pi_device(q_vec, f_vec, poly_len, combination_scalars, point):
    sc = _fr_arr(combination_scalars)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_multiopen_pi_device(
        ctypes.byref(h), q_vec.raw, f_vec.raw, poly_len, _ptr(sc), len(sc), _fr(point)))
    return Bls12_381FrDeviceVec(h)


def bls12_381_fr_poseidon_hash_chain(initial, tail0, tail1, input_len, mds, round_constants, length,
                                     witness=False):
    """lib.rs bls12_381_fr_poseidon_hash_chain[_witness]: the chain's length
    outputs, or its 256-value witness per hash (witness=True)."""
    m, rc = _fr_arr(mds), _fr_arr(round_constants)
    if length == 0:
        return np.zeros((0, 4), dtype=np.uint64)
    out = np.zeros((length * (256 if witness else 1), 4), dtype=np.uint64)
    f = (lib().midnight_sppark_bls12_381_fr_poseidon_hash_chain_witness if witness
         else lib().midnight_sppark_bls12_381_fr_poseidon_hash_chain)
    check(f(_ptr(out), length, _fr(initial), _fr(tail0), _fr(tail1), _fr(input_len), _ptr(m), len(m), _ptr(rc),
            len(rc)))
    return out


def bls12_381_fr_poseidon_advice_from_witness(witness, hash_count, domain_len, metadata, layout):
    """lib.rs poseidon_advice_from_witness: a Bls12_381FrDeviceVec of 8
    advice columns x domain_len rows; layout = 128 (column, row) pairs"""
    w, meta = _fr_arr(witness), _fr_arr(metadata)
    lay = np.array([(c << 8) | r for c, r in layout], dtype=np.uint16)
    h = ctypes.c_void_p()
    check(lib().midnight_sppark_bls12_381_fr_poseidon_advice_from_witness(
        ctypes.byref(h), _ptr(w), hash_count, domain_len, _ptr(meta), len(meta), _ptr(lay), len(lay)))
    return Bls12_381FrDeviceVec(h)


class NumeratorContext:
    """midnight_sppark_bls12_381_numerator_context_{create,eval,free} and the
    trace-context calls on it (bls12_381_g1_msm.cu:5517-6162).  Host arrays
    are Montgomery Fr rows ([rows][4] uint64), column groups laid out
    [column][rows]: extended-coset data has `length` rows, Lagrange-basis
    (trace) data `input_len` rows.  The graphs are copied into device memory
    at creation."""

    def __init__(self, length, input_len, custom_graph, fixed=None, fixed_lagrange=None, fixed_cols=0, l0=None,
                 l_last=None, l_active=None, permutation_columns=(), permutation_pk_cosets=None,
                 permutation_pk_lagrange=None, permutation_pk_count=0, trash_selectors=(), lookup_graphs=(),
                 lookup_input_graphs=(), lookup_table_graphs=(), trash_graphs=(), omega=None, trace_omega=None,
                 g_coset=None, delta_const=None, rot_scale=1, last_rotation=-1, chunk_len=1):
        from .graph import column_refs, graph_array
        z = np.zeros(4, dtype=np.uint64)
        arr = lambda v: None if v is None else _fr_arr(v)  # noqa: E731
        f = lambda v: _fr(z if v is None else v)  # noqa: E731
        fx, fl, pk, pl = arr(fixed), arr(fixed_lagrange), arr(permutation_pk_cosets), arr(permutation_pk_lagrange)
        lag = [arr(x) for x in (l0, l_last, l_active)]
        pcols = column_refs(list(permutation_columns))
        tr_s = np.array(list(trash_selectors) or [0], dtype=np.uint32)
        lk, lki, lkt, tr = (graph_array(list(g)) for g in (lookup_graphs, lookup_input_graphs, lookup_table_graphs,
                                                            trash_graphs))
        self.length, self.input_len = length, input_len
        self._h = ctypes.c_void_p()
        vp = lambda a: ctypes.cast(a, ctypes.c_void_p)  # noqa: E731
        check(lib().midnight_sppark_bls12_381_numerator_context_create(
            ctypes.byref(self._h), length, input_len, _ptr(fx), _ptr(fl), fixed_cols, _ptr(lag[0]), _ptr(lag[1]),
            _ptr(lag[2]), vp(pcols), len(permutation_columns), _ptr(pk), _ptr(pl), permutation_pk_count,
            _ptr(tr_s) if len(trash_selectors) else None, len(trash_selectors), custom_graph.raw(), vp(lk), vp(lki),
            vp(lkt), len(lookup_graphs), vp(tr), f(omega), f(trace_omega), f(g_coset), f(delta_const), rot_scale,
            last_rotation, chunk_len))

    def eval(self, columns, total_columns, advice_offset=0, advice_cols=0, instance_offset=0, instance_cols=0,
             challenges=None, beta=None, gamma=None, theta=None, trash_challenge=None, y=None, permutation_offset=0,
             permutation_sets=0, lookup_product_offset=0, lookup_input_offset=0, lookup_table_offset=0,
             lookup_count=0, trash_offset=0, trash_count=0):
        """The numerator over one Bls12_381FrDeviceVec of total_columns x length
        values; a new device vector of length rows."""
        z = np.zeros(4, dtype=np.uint64)
        f = lambda v: _fr(z if v is None else v)  # noqa: E731
        ch = None if challenges is None else _fr_arr(challenges)
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_numerator_context_eval(
            ctypes.byref(h), self._h, columns.raw, total_columns, advice_offset, advice_cols, instance_offset,
            instance_cols, _ptr(ch), 0 if ch is None else len(ch), f(beta), f(gamma), f(theta), f(trash_challenge),
            f(y), permutation_offset, permutation_sets, lookup_product_offset, lookup_input_offset,
            lookup_table_offset, lookup_count, trash_offset, trash_count))
        return Bls12_381FrDeviceVec(h)

    def trace_trash(self, advice, advice_cols, instance, instance_cols, challenges, trash_challenge):
        ch = None if challenges is None else _fr_arr(challenges)
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_trace_context_trash(
            ctypes.byref(h), self._h, _raw(advice), advice_cols, _raw(instance), instance_cols, _ptr(ch),
            0 if ch is None else len(ch), _fr(trash_challenge)))
        return Bls12_381FrDeviceVec(h)

    def trace_permutation(self, advice, advice_cols, instance, instance_cols, beta, gamma, delta_powers,
                          blind_values, blinding_factors):
        d = _fr_arr(delta_powers)
        b = _fr_arr(blind_values) if blind_values is not None and len(blind_values) else None
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_trace_context_permutation(
            ctypes.byref(h), self._h, _raw(advice), advice_cols, _raw(instance), instance_cols, _fr(beta),
            _fr(gamma), _ptr(d), len(d), _ptr(b), 0 if b is None else len(b), blinding_factors))
        return Bls12_381FrDeviceVec(h)

    def trace_lookup_permute(self, advice, advice_cols, instance, instance_cols, challenges, theta, usable_rows,
                             input_blinds, table_blinds):
        ch = None if challenges is None else _fr_arr(challenges)
        nb = self.input_len - usable_rows
        ib = _fr_arr(input_blinds) if nb else None
        tb = _fr_arr(table_blinds) if nb else None
        h = ctypes.c_void_p()
        check(lib().midnight_sppark_bls12_381_trace_context_lookup_permute(
            ctypes.byref(h), self._h, _raw(advice), advice_cols, _raw(instance), instance_cols, _ptr(ch),
            0 if ch is None else len(ch), _fr(theta), usable_rows, _ptr(ib), _ptr(tb), nb))
        return Bls12_381FrDeviceVec(h)

    def close(self):
        if self._h:
            lib().midnight_sppark_bls12_381_numerator_context_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- autotuner

def ntt_variant_set(variant):
    """Force the NTT pass variant (1..5, see gb_ntt_variant_set); 0 = default."""
    lib().gb_ntt_variant_set(int(variant))


def ntt_wait_limit_set(spins):
    """test hook (gb_ntt_wait_limit_set): poll limit of the first twiddle-copy
    wait; None or negative restores the default"""
    lib().gb_ntt_wait_limit_set(-1 if spins is None else int(spins))


def ntt_wait_timeouts():
    """Staged NTT passes whose twiddle copy timed out since the last call."""
    v = ctypes.c_uint32()
    check(lib().gb_ntt_wait_timeouts(ctypes.byref(v)))
    return v.value


def autotune_set(enabled=True):
    lib().gb_autotune_set(1 if enabled else 0)


def autotune_reset():
    lib().gb_autotune_reset()


def autotune_report():
    """{key: chosen value} of every tuned key"""
    n = lib().gb_autotune_report(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    lib().gb_autotune_report(buf, n + 1)
    out = {}
    for item in buf.value.decode().split(";"):
        if "=" in item:
            k, v = item.split("=")
            out[k] = int(v)
    return out
