"""ctypes loader for libgbprover.so and the C ABI declarations."""
import ctypes
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
REPO_ROOT = os.path.dirname(PKG_ROOT)
HEADER = os.path.join(REPO_ROOT, "include", "gb_prover.h")

if PKG_ROOT not in sys.path:
    sys.path.insert(0, PKG_ROOT)

import build_lib as _build_lib  # noqa: E402


class MsmError(RuntimeError):
    """Error returned by the library (mirrors lib.rs MsmError::Sppark)."""

    def __init__(self, code, message):
        super().__init__("gb prover call failed (code %d): %s" % (code, message))
        self.code = code
        self.message = message


class RustError(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("message", ctypes.c_void_p)]


class RawMsmConfig(ctypes.Structure):
    """bls12_381_g1_msm.cu:50-61 / lib.rs Bls12_381MsmConfig"""
    _fields_ = [(name, ctypes.c_uint32) for name in (
        "domain_k", "min_msm_scalars", "unfiltered_min_scalars", "window_bits", "sort_grid_divisor",
        "sort_window_lanes", "integration_blocks", "batch_lanes", "reuse_event", "device_reduce")]

    @classmethod
    def default(cls, npoints, window_bits=0):
        k = max(0, (max(npoints, 1) - 1).bit_length())
        return cls(k, 100000, 32768, window_bits, 3, 2, 1, 4, 0, 3)


class RawMsmSlice(ctypes.Structure):
    _fields_ = [("scalar_offset", ctypes.c_size_t), ("point_offset", ctypes.c_size_t),
                ("len", ctypes.c_size_t), ("nonzero_len", ctypes.c_size_t)]


class RawFr(ctypes.Structure):
    _fields_ = [("limbs", ctypes.c_uint64 * 4)]


class RawDevicePolyRef(ctypes.Structure):
    """source 0 dynamic, 1 fixed, 2 extra device vector; index-th polynomial"""
    _fields_ = [("source", ctypes.c_uint32), ("index", ctypes.c_uint32)]


_lib = None
_libc = ctypes.CDLL(None)
_libc.free.argtypes = [ctypes.c_void_p]


def library_path():
    return _build_lib.LIB


def build(force=False, verbose=False):
    return _build_lib.build(force=force, verbose=verbose)


def _declare(L):
    from .graph import RawGraph
    vp, sz, u32, b = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_bool
    i32 = ctypes.c_int32
    fr = RawFr
    E = RustError
    sigs = {
        "midnight_sppark_execution_lane_set": (E, [u32]),
        "midnight_sppark_bls12_381_g1_msm": (E, [vp, vp, vp, sz]),
        "midnight_sppark_bls12_381_g1_msm_batch": (E, [vp, vp, vp, sz, sz]),
        "midnight_sppark_bls12_381_g1_msm_context_create": (E, [vp, vp, sz]),
        "midnight_sppark_bls12_381_g1_msm_context_create_with_config": (E, [vp, vp, sz, RawMsmConfig]),
        "midnight_sppark_bls12_381_g1_msm_context_free": (None, [vp]),
        "midnight_sppark_bls12_381_g1_msm_context_batch": (E, [vp, vp, vp, sz, sz]),
        "midnight_sppark_bls12_381_g1_msm_context_device_batch": (E, [vp, vp, vp, sz, sz, sz]),
        "midnight_sppark_bls12_381_g1_msm_context_device_ragged": (E, [vp, vp, vp, vp, sz]),
        "midnight_sppark_bls12_381_g1_msm_context_device_scrambled_batch": (E, [vp, vp, vp, sz, sz, sz, vp]),
        "midnight_sppark_bls12_381_fr_ntt": (E, [vp, u32, b]),
        "midnight_sppark_bls12_381_fr_ntt_zeta": (E, [vp, u32, b, fr, fr, fr]),
        "midnight_sppark_bls12_381_fr_divide_ntt_zeta": (E, [vp, u32, vp, sz, fr, fr, fr]),
        "midnight_sppark_bls12_381_fr_coeff_to_extended_batch": (E, [vp, vp, sz, sz, u32, fr, fr]),
        "midnight_sppark_bls12_381_fr_device_coeff_to_extended_batch": (E, [vp, vp, sz, sz, u32, fr, fr]),
        "midnight_sppark_bls12_381_fr_device_coeff_to_extended_from_device_batch": (E, [vp, vp, sz, sz, u32, fr, fr]),
        "midnight_sppark_bls12_381_fr_device_vec_ntt_zeta": (E, [vp, u32, b, fr, fr, fr]),
        "midnight_sppark_bls12_381_fr_device_vec_ntt_zeta_batch": (E, [vp, u32, sz, b, fr, fr, fr]),
        "midnight_sppark_bls12_381_fr_device_vec_divide_ntt_zeta": (E, [vp, u32, vp, sz, fr, fr, fr]),
        "midnight_sppark_bls12_381_fr_mul_assign": (E, [vp, fr, sz]),
        "midnight_sppark_bls12_381_fr_mul_assign_zeta": (E, [vp, fr, fr, sz]),
        "midnight_sppark_bls12_381_fr_mul_assign_repeating": (E, [vp, vp, sz, sz]),
        "midnight_sppark_bls12_381_fr_invert_assign": (E, [vp, sz]),
        "midnight_sppark_bls12_381_fr_sort_canonical": (E, [vp, sz]),
        "midnight_sppark_bls12_381_fr_poly_lincomb": (E, [vp, vp, sz, sz, vp]),
        "midnight_sppark_bls12_381_fr_shifted_prefix_product": (E, [vp, fr, sz]),
        "midnight_sppark_bls12_381_fr_permutation_products": (E, [vp, vp, vp, sz, sz, sz, fr, fr, fr, vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_lookup_products": (E, [vp, vp, vp, vp, vp, sz, sz, fr, fr, vp, sz]),
        "midnight_sppark_bls12_381_fr_lookup_products_device": (E, [vp, vp, sz, sz, fr, fr, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_quotient_pieces": (E, [vp, vp, sz, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_poly_lincomb": (E, [vp, vp, sz, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_upload": (E, [vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_upload_many": (E, [vp, vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_download": (E, [vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_scatter_host": (E, [vp, vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_concat_host": (E, [vp, vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_concat_many_host": (E, [vp, vp, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_gather_polys": (E, [vp, vp, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_free": (None, [vp]),
        "gb_fr_device_vec_len": (sz, [vp]),
        "gb_g1_generator_mul": (E, [vp, vp, sz]),
        "gb_g1_generator_mul_device": (E, [vp, vp, sz]),
        "gb_imad_peak": (E, [ctypes.POINTER(ctypes.c_double)]),
        "gb_imad_probe": (E, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
        "gb_g1_to_lagrange": (E, [vp, vp, u32]),
        "gb_g1_jacobian_to_affine_batch": (E, [vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_eval_polys": (E, [vp, vp, sz, sz, fr]),
        "gb_fr_device_kate_divide": (E, [vp, vp, sz, sz, fr]),
        "gb_fr_device_eval_many": (E, [vp, vp, vp, vp, sz, sz]),
        "gb_kzg_setup": (E, [vp, vp, fr, u32]),
        "gb_transfer_counters": (None, [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
        "gb_transfer_counters_reset": (None, []),
        "gb_error_free": (None, [vp]),
        "gb_launch_counter": (ctypes.c_uint64, []),
        "gb_lane_stream": (vp, []),
        "gb_profile_enable": (None, [ctypes.c_int]),
        "gb_profile_read": (None, [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]),
        "gb_profile_reset": (None, []),
        "gb_fr_shifted_prefix_product_noalloc": (E, [vp, fr, sz, vp]),
        "midnight_sppark_bls12_381_eval_numerator": (E, [
            vp, sz, vp, u32, vp, sz, vp, sz, vp, sz, vp, sz, fr, fr, fr, fr, fr, fr, fr, fr, i32, i32, u32,
            vp, vp, vp, vp, sz, vp, sz, vp, sz, vp, vp, vp, sz, vp, vp, sz, RawGraph, vp, vp]),
        "midnight_sppark_bls12_381_eval_graph_batch": (E, [
            vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, fr, fr, fr, fr, fr, i32, vp, sz]),
        "gb_eval_graph_batch_device": (E, [
            vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, fr, fr, fr, fr, fr, i32, vp, sz]),
        "gb_eval_numerator_device": (E, [
            vp, sz, vp, u32, vp, sz, vp, sz, vp, sz, vp, sz, fr, fr, fr, fr, fr, fr, fr, fr, i32, i32, u32,
            vp, vp, sz, vp, sz, vp, sz, vp, vp, sz, vp, vp, sz, RawGraph, vp, vp]),
        "gb_fr_permutation_products_device": (E, [vp, vp, vp, sz, sz, sz, fr, fr, fr, vp, vp, sz]),
        "gb_fr_random_chacha20": (E, [vp, vp, ctypes.c_uint64, sz, vp]),
        "gb_chacha20_blocks": (E, [vp, ctypes.c_uint64, ctypes.c_uint64, sz, vp]),
        "gb_fr_lookup_permute_device": (E, [vp, vp, sz, sz, sz, vp, vp]),
        "midnight_sppark_bls12_381_numerator_context_create": (E, [
            vp, sz, sz, vp, vp, sz, vp, vp, vp, vp, sz, vp, vp, sz, vp, sz, RawGraph, vp, vp, vp, sz, vp,
            fr, fr, fr, fr, i32, i32, u32]),
        "midnight_sppark_bls12_381_numerator_context_free": (None, [vp]),
        "midnight_sppark_bls12_381_fr_multiopen_prepare": (E, [
            vp, vp, vp, sz, sz, vp, sz, vp, vp, sz, vp, sz, vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_multiopen_prepare_device": (E, [
            vp, vp, vp, vp, vp, vp, sz, vp, sz, vp, sz, vp, vp, sz, vp, sz, vp, vp, sz]),
        "midnight_sppark_bls12_381_fr_multiopen_f_poly_device": (E, [vp, vp, sz, vp, sz, vp, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_multiopen_pi_device": (E, [vp, vp, vp, sz, vp, sz, fr]),
        "midnight_sppark_bls12_381_fr_poseidon_hash_chain": (E, [vp, sz, fr, fr, fr, fr, vp, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_poseidon_hash_chain_witness": (E, [vp, sz, fr, fr, fr, fr, vp, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_poseidon_advice_from_witness": (E, [vp, vp, sz, sz, vp, sz, vp, sz]),
        "midnight_sppark_bls12_381_fr_device_vec_download_nonzero_suffixes": (E, [
            vp, sz, vp, vp, vp, vp, sz, sz, sz]),
        "midnight_sppark_bls12_381_fr_lookup_permute_batch": (E, [vp, vp, vp, sz, sz, sz, vp, vp, sz]),
        "midnight_sppark_test_mask_delay": (None, [u32]),
        "midnight_sppark_test_delayed_scale": (E, [vp, fr, u32]),
        "midnight_sppark_bls12_381_numerator_context_eval": (E, [
            vp, vp, vp, sz, sz, sz, sz, sz, vp, sz, fr, fr, fr, fr, fr, sz, sz, sz, sz, sz, sz, sz, sz]),
        "midnight_sppark_bls12_381_trace_context_trash": (E, [vp, vp, vp, sz, vp, sz, vp, sz, fr]),
        "midnight_sppark_bls12_381_trace_context_permutation": (E, [
            vp, vp, vp, sz, vp, sz, fr, fr, vp, sz, vp, sz, sz]),
        "midnight_sppark_bls12_381_trace_context_lookup_permute": (E, [
            vp, vp, vp, sz, vp, sz, vp, sz, fr, sz, vp, vp, sz]),
        "gb_autotune_set": (None, [ctypes.c_int]),
        "gb_ntt_variant_set": (None, [ctypes.c_int]),
        "gb_ntt_wait_timeouts": (E, [ctypes.POINTER(ctypes.c_uint32)]),
        "gb_fr_device_vec_ntt_ragged": (E, [vp, vp, vp, sz, b, fr, fr, fr]),
        "gb_ntt_wait_limit_set": (None, [ctypes.c_int64]),
        "gb_g1_msm_device": (E, [vp, vp, vp, sz]),
        "gb_g1_msm_context_device_batch_async": (E, [vp, vp, vp, sz, sz, sz]),
        "gb_msm_ticket_wait": (E, [vp, vp]),
        "gb_msm_graphs_enable": (E, [ctypes.c_int]),
        "gb_msm_graph_stats": (E, [vp, vp]),
        "gb_g1_msm_context_device_bytes": (sz, [vp]),
        "gb_fr_coeff_to_extended_coset_batch": (E, [vp, vp, sz, sz, u32, fr]),
        "gb_fr_device_coeff_to_extended_coset_batch": (E, [vp, vp, sz, sz, u32, fr]),
        "gb_fr_device_vec_ntt_coset_batch": (E, [vp, u32, sz, b, fr]),
        "gb_fr_ntt_coset": (E, [vp, u32, b, fr]),
        "gb_fr_lde_coset": (E, [vp, vp, u32, u32]),
        "gb_autotune_reset": (None, []),
        "gb_autotune_report": (sz, [vp, sz]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return sigs


def header_symbols():
    """Every function name declared GB_API in include/gb_prover.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GB_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def lib(build_if_stale=False):
    """Load libgbprover.so (rebuilding it first if asked and out of date);
    raise MsmError if it is absent -- there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_stale:
        build()
    if not os.path.exists(path):
        raise MsmError(-1, "libgbprover.so not built at %s (run __graft_entry__.build())" % path)
    L = ctypes.CDLL(path)
    _declare(L)
    _lib = L
    return L


def check(err):
    """Turn a RustError into MsmError, freeing its message (lib.rs From<Error>)."""
    if err.code == 0:
        if err.message:
            _libc.free(err.message)
        return
    msg = ""
    if err.message:
        msg = ctypes.string_at(err.message).decode("utf-8", "replace")
        _libc.free(err.message)
    raise MsmError(err.code, msg or ("sppark::Error #%d" % err.code))
