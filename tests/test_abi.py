"""The C ABI library loads and exports every symbol include/gb_prover.h
declares; without a GPU its compute calls fail loudly with an error code
(no CPU fallback).  Runs on CPU."""
import ctypes
import subprocess

import numpy as np
import pytest


def test_header_symbols_exported(gb):
    import gb_prover._lib as L
    declared = L.header_symbols()
    assert len(declared) >= 45
    out = subprocess.run(["nm", "-D", "--defined-only", L.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    lib = gb.lib()
    for s in declared:
        assert hasattr(lib, s), s


def test_reference_ffi_names_covered(gb):
    """Every midnight_sppark_* function this library declares is one the
    reference's Rust crate binds (midnight-sppark-msm/src/lib.rs:763-1362)."""
    import gb_prover._lib as L
    ours = [s for s in L.header_symbols() if s.startswith("midnight_sppark_")]
    assert "midnight_sppark_bls12_381_g1_msm" in ours
    assert "midnight_sppark_bls12_381_fr_ntt" in ours
    assert "midnight_sppark_bls12_381_fr_permutation_products" in ours


def test_no_gpu_fails_loudly(gb):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; the no-GPU error path is not reachable")
    vals = np.zeros((4, 4), dtype=np.uint64)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_ntt(vals, False)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_g1_msm(np.zeros((1, 12), dtype=np.uint64), np.zeros((1, 4), dtype=np.uint64))


def test_argument_validation_without_gpu(gb):
    """Argument errors are reported before any device work
    (bls12_381_g1_msm.cu:6318-6331 behaviour: cudaErrorInvalidValue)."""
    lib = gb.lib()
    h = ctypes.c_void_p()
    err = lib.midnight_sppark_bls12_381_fr_permutation_products(ctypes.byref(h), None, None, 0, 0, 0, gb.api._fr(
        np.zeros(4, dtype=np.uint64)), gb.api._fr(np.zeros(4, dtype=np.uint64)), gb.api._fr(
        np.zeros(4, dtype=np.uint64)), None, None, 0)
    assert err.code == 1
    with pytest.raises(gb.MsmError) as e:
        gb.api.check(err)
    assert "invalid permutation product arguments" in str(e.value)
    err = lib.midnight_sppark_execution_lane_set(99)
    assert err.code == 1
    gb.api.check(lib.midnight_sppark_execution_lane_set(0))


def test_context_and_multiopen_validation_without_gpu(gb):
    """The numerator context, multi-open and lookup batch entry points check
    their arguments before any device work, with the reference's messages
    (bls12_381_g1_msm.cu:3617-3642, 5548-5561, 5150-5155)."""
    lib = gb.lib()
    z = gb.api._fr(np.zeros(4, dtype=np.uint64))
    h = ctypes.c_void_p()
    # create without l0 / l_last / l_active
    err = lib.midnight_sppark_bls12_381_numerator_context_create(
        ctypes.byref(h), 16, 4, None, None, 0, None, None, None, None, 0, None, None, 0, None, 0,
        gb.graph.RawGraph(), None, None, None, 0, None, z, z, z, z, 1, -1, 1)
    with pytest.raises(gb.MsmError, match="invalid numerator context arguments"):
        gb.api.check(err)
    # non-monotonic q offsets
    polys = np.zeros((8, 4), dtype=np.uint64)
    with pytest.raises(gb.MsmError, match="non-monotonic multi-open q offsets"):
        gb.bls12_381_fr_multiopen_prepare(polys, 4, [0, 2, 1, 3], [0, 1, 1], np.zeros((3, 4), np.uint64),
                                          np.zeros((1, 4), np.uint64), [0], [0])
    # a query point out of range
    with pytest.raises(gb.MsmError, match="multi-open query index out of range"):
        gb.bls12_381_fr_multiopen_prepare(polys, 4, [0, 1], [0], np.zeros((1, 4), np.uint64),
                                          np.zeros((1, 4), np.uint64), [0], [1])
    # blind count that does not match len - usable_rows
    err = lib.midnight_sppark_bls12_381_fr_lookup_permute_batch(
        ctypes.byref(h), gb.api._ptr(polys), gb.api._ptr(polys), 8, 1, 6, gb.api._ptr(polys), gb.api._ptr(polys), 1)
    with pytest.raises(gb.MsmError, match="invalid resident lookup permutation arguments"):
        gb.api.check(err)


def test_host_affine_conversion_matches_oracle(gb, orc):
    """gb_g1_jacobian_to_affine_batch (host only, no GPU needed) against the
    oracle's conversion: real points in Jacobian form with random Z, the
    point at infinity among them, batches of 0..9 points."""
    from gb_prover import kzg
    P = kzg.P_MOD
    rng = np.random.default_rng(11)
    g_aff = orc.g1_generator_mul_batch(orc.fr_from_ints([3, 5, 7, 11, 13, 17, 19, 23]))
    gb.lib()
    for trial in range(60):
        m = int(rng.integers(0, 10))
        rows = []
        for i in range(m):
            a = g_aff[int(rng.integers(0, len(g_aff)))]
            if rng.random() < 0.2:
                rows.append(np.zeros(18, dtype=np.uint64))
                continue
            # (x, y) -> (x z^2, y z^3, z) in Montgomery form for a random z
            x = kzg._int(a[0:6]) * kzg._FP_RINV % P
            y = kzg._int(a[6:12]) * kzg._FP_RINV % P
            z = int.from_bytes(rng.bytes(48), "little") % P or 1
            vals = [x * z * z % P, y * z * z * z % P, z]
            rows.append(np.array([limb for v in vals for limb in kzg._limbs(v * kzg._FP_R % P, 6)],
                                 dtype=np.uint64))
        jac = np.array(rows, dtype=np.uint64).reshape(m, 18)
        got = kzg.affine_from_projective_batch(jac)
        want = orc.g1_to_affine(jac) if m else np.zeros((0, 12), np.uint64)
        assert got.shape == (m, 12)
        assert (got == want).all(), trial
        # the Python-integer form (processes without the library) agrees
        assert (kzg._affine_from_projective_batch_py(jac) == want).all(), trial
    with pytest.raises(gb.MsmError):
        gb.api.check(gb.lib().gb_g1_jacobian_to_affine_batch(None, None, 1))
