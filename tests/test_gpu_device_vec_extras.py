"""Device-vector downloads of nonzero suffixes, the host-buffer lookup
permutation batch, and the two test hooks (a delayed producer on another
lane; a delayed scramble mask) through the C ABI, against the oracle."""
import numpy as np
import pytest

from conftest import affine_of

pytestmark = pytest.mark.gpu


def test_download_nonzero_suffixes(gb, orc):
    rng = np.random.default_rng(21)
    n, offset = 20000, 5  # more than one 8192-value slice per polynomial
    polys = [orc.fr_random(n, rng) for _ in range(5)]
    polys[1][:9000] = 0
    polys[1][12000:12100] = 0
    polys[2][:] = 0
    polys[3][:-1] = 0
    polys[4][:8192] = 0
    data = np.concatenate([orc.fr_random(offset, rng)] + polys + [orc.fr_random(3, rng)])
    v = gb.Bls12_381FrDeviceVec.upload(data)
    out, starts, live = v.download_nonzero_suffixes(offset, n, len(polys))
    want_starts, want_live, want_out = [], [], []
    for p in polys:
        nz = np.flatnonzero(p.any(axis=1))
        s = int(nz[0]) if len(nz) else n
        want_starts.append(s)
        want_live.append(len(nz))
        want_out.append(p[s:])
    assert list(starts) == want_starts
    assert list(live) == want_live
    assert (out == np.concatenate(want_out)).all()
    f = gb.lib().midnight_sppark_bls12_381_fr_device_vec_download_nonzero_suffixes
    import ctypes
    n_out = ctypes.c_size_t()
    st = np.zeros(len(polys), dtype=np.uint64)
    small = np.zeros((10, 4), dtype=np.uint64)
    with pytest.raises(gb.MsmError):  # output too small
        gb.api.check(f(gb.api._ptr(small), 10, ctypes.byref(n_out), gb.api._ptr(st), None, v.raw, offset, n,
                       len(polys)))
    with pytest.raises(gb.MsmError):  # range past the vector
        v.download_nonzero_suffixes(offset + 10, n, len(polys))


def test_lookup_permute_batch_matches_oracle(gb, orc):
    from oracle.plonk_cpu import OracleBackend
    rng = np.random.default_rng(22)
    n, u, lookups = 4096, 4090, 2
    inputs, tables = [], []
    for _ in range(lookups):
        values = orc.fr_random(300, rng)
        tab = values[rng.integers(0, 300, size=n)]
        tab[:300] = values
        inputs.append(values[rng.integers(0, 40, size=n)])
        tables.append(tab)
    nb = n - u
    ib, tb = orc.fr_random(lookups * nb, rng), orc.fr_random(lookups * nb, rng)
    got = gb.bls12_381_fr_lookup_permute_batch(np.concatenate(inputs), np.concatenate(tables), n, lookups, u, ib,
                                               tb).download().reshape(4, lookups, n, 4)
    comp = np.concatenate([np.concatenate([inputs[i], tables[i]]) for i in range(lookups)])
    want = OracleBackend(None).permute_lookups(OracleBackend(None).put(comp), n, u, lookups, ib, tb).a
    want = want.reshape(lookups, 2, n, 4)
    for i in range(lookups):
        assert (got[0, i] == inputs[i]).all()
        assert (got[1, i] == tables[i]).all()
        assert (got[2, i] == want[i, 0]).all()
        assert (got[3, i] == want[i, 1]).all()
    bad = [x.copy() for x in inputs]
    bad[1][17] = orc.fr_random(1, rng)[0]
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_lookup_permute_batch(np.concatenate(bad), np.concatenate(tables), n, lookups, u, ib, tb)


def test_delayed_producer_on_another_lane(gb, orc):
    """A vector scaled on lane 1 behind a 300 ms hold is read on lane 2: the
    reader must wait for the scaling (the reference's cross-lane readiness
    regression)."""
    rng = np.random.default_rng(23)
    values = orc.fr_random(1 << 16, rng)
    k = orc.fr_random(1, rng)[0]
    try:
        gb.execution_lane_set(0)
        v = gb.Bls12_381FrDeviceVec.upload(values)
        gb.execution_lane_set(1)
        gb.hook_delayed_scale(v, k, 300)
        gb.execution_lane_set(2)
        got = v.download()
    finally:
        gb.execution_lane_set(0)
    assert (got == orc.fr_mul_assign(values, k)).all()


def test_scrambled_batch_with_delayed_mask(gb, orc):
    rng = np.random.default_rng(24)
    n = 3000
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    s = np.stack([orc.fr_random(n, rng) for _ in range(2)])
    mask = orc.fr_random(n, rng)
    ctx = gb.Bls12_381G1MsmContext(b)
    dv = gb.Bls12_381FrDeviceVec.upload(s.reshape(-1, 4))
    mv = gb.Bls12_381FrDeviceVec.upload(mask)
    try:
        gb.hook_mask_delay(200)
        got = ctx.device_scrambled_batch(dv, 0, 2, mv)
    finally:
        gb.hook_mask_delay(0)
    R = orc.R_MOD
    mi = orc.fr_to_ints(mask)
    for i in range(2):
        masked = orc.fr_from_ints([(x + y) % R for x, y in zip(orc.fr_to_ints(s[i]), mi)])
        assert (affine_of(orc, got[i]) == affine_of(orc, orc.g1_msm(b, masked))).all()
    ctx.close()
