"""The batched MSM/NTT configuration at its own sizes: the 64 MSMs (sizes
round(2^U), U uniform in [10, 18], scalars 70% uniform Fr, 20% below 2^64,
10% zero) that the benchmark times, in one ragged batch over a resident
2^18 base set, every MSM against the oracle's Pippenger; and the 64 NTTs of
the matching power-of-two sizes in one work-queue launch, every transform
against the oracle."""
import numpy as np
import pytest

from conftest import affine_of

pytestmark = pytest.mark.gpu


def test_config4_msm_batch_against_oracle(gb, orc):
    import bench
    sizes, scal, base_scalars, _ = bench.config4_inputs()
    assert len(sizes) == 64 and min(sizes) >= 1 << 10 and max(sizes) <= 1 << 18
    bases = gb.g1_generator_mul(base_scalars)
    ctx = gb.Bls12_381G1MsmContext(bases)
    flat = np.concatenate(scal)
    dv = gb.Bls12_381FrDeviceVec.upload(flat)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int)
    got = ctx.device_ragged(dv, [(int(o), 0, n) for o, n in zip(offs, sizes)])
    for j, n in enumerate(sizes):
        want = orc.g1_msm(bases[:n], scal[j])
        assert (affine_of(orc, got[j]) == affine_of(orc, want)).all(), (j, n)
    # the autotuned engine gives the same points
    gb.autotune_reset()
    gb.autotune_set(True)
    try:
        tuned = ctx.device_ragged(dv, [(int(o), 0, n) for o, n in zip(offs, sizes)])
    finally:
        gb.autotune_set(False)
        gb.autotune_reset()
    for j in range(64):
        assert (affine_of(orc, tuned[j]) == affine_of(orc, got[j])).all(), j
    ctx.close()


def test_config4_ntt_queue_against_oracle(gb, orc):
    import bench
    _, _, _, logs = bench.config4_inputs()
    rng = np.random.default_rng(4005)
    offs = np.concatenate([[0], np.cumsum([1 << lg for lg in logs])[:-1]]).astype(np.uint64)
    v = orc.fr_random(int(sum(1 << lg for lg in logs)), rng)
    one = orc.fr_const(orc.CONST_ONE)
    dv = gb.Bls12_381FrDeviceVec.upload(v)
    dv.ntt_ragged(offs, logs, False, one, one, one)
    got = dv.download()
    for off, lg in zip(offs, logs):
        seg = slice(int(off), int(off) + (1 << lg))
        assert (got[seg] == orc.fr_ntt(v[seg], lg, False)).all(), lg
    dv.ntt_ragged(offs, logs, True, one, one, one)
    assert (dv.download() == v).all()
    assert gb.ntt_wait_timeouts() == 0
