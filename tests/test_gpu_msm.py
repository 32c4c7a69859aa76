"""G1 multiexp on the GPU through the C ABI, bit-exact (affine) against the
oracle: the reference's own test shapes, edge cases, every context entry
point and the real-SRS known answers."""
import numpy as np
import pytest

from conftest import affine_of

pytestmark = pytest.mark.gpu


def _ref_batch_scalars(orc, n, batch):
    # midnight-sppark-msm/src/lib.rs:5033-5079: 1 / ((29i + 43b + 11) mod 65521 + 1)
    R = orc.R_MOD
    return orc.fr_from_ints([pow((i * 29 + batch * 43 + 11) % 65521 + 1, -1, R) for i in range(n)])


def _check(orc, got_jac, bases, scalars):
    want = affine_of(orc, orc.g1_msm(bases, scalars))
    assert (affine_of(orc, got_jac) == want).all()


def test_generator_mul_matches_oracle(gb, orc):
    rng = np.random.default_rng(1)
    s = orc.fr_random(1000, rng)
    s[0] = 0
    s[1] = orc.fr_from_ints([1])[0]
    s[2] = orc.fr_from_ints([orc.R_MOD - 1])[0]
    got = gb.g1_generator_mul(s)
    assert (got == orc.g1_generator_mul_batch(s)).all()


def test_msm_reference_shape_4096(gb, orc):
    n = 4096
    bases = orc.g1_generator_mul_batch(orc.fr_from_ints(list(range(1, n + 1))))
    for b in range(2):
        s = _ref_batch_scalars(orc, n, b)
        _check(orc, gb.bls12_381_g1_msm(bases, s), bases, s)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 255, 1000, 1 << 12])
def test_msm_random_sizes(gb, orc, n):
    rng = np.random.default_rng(n)
    s = orc.fr_random(n, rng)
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    _check(orc, gb.bls12_381_g1_msm(b, s), b, s)


def test_msm_edge_cases(gb, orc):
    rng = np.random.default_rng(7)
    n = 3000
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    # all-zero scalars -> infinity
    z = np.zeros((n, 4), dtype=np.uint64)
    out = gb.bls12_381_g1_msm(b, z)
    assert (out[12:18] == 0).all()
    # empty input -> infinity
    out = gb.bls12_381_g1_msm(np.zeros((0, 12), np.uint64), np.zeros((0, 4), np.uint64))
    assert (out[12:18] == 0).all()
    # max scalars, small scalars, repeated bases (bucket collisions: doubling
    # and cancellation inside buckets), P and -P style cancellations
    s = orc.fr_random(n, rng)
    s[:100] = orc.fr_from_ints([orc.R_MOD - 1] * 100)
    s[100:200] = orc.fr_from_ints([1] * 100)
    s[200:300] = 0
    b2 = b.copy()
    b2[300:700] = b[0]
    s[300:700] = orc.fr_from_ints([5] * 400)
    s[700:800] = orc.fr_from_ints([orc.R_MOD - 5] * 100)
    b2[700:800] = b[0]
    _check(orc, gb.bls12_381_g1_msm(b2, s), b2, s)
    # infinity among the bases
    b3 = b.copy()
    b3[10] = 0
    _check(orc, gb.bls12_381_g1_msm(b3, s), b3, s)
    # a sum that cancels to infinity exactly: s*P + (r-s)*P
    pair_b = np.stack([b[1], b[1]])
    pair_s = orc.fr_from_ints([12345, orc.R_MOD - 12345])
    out = gb.bls12_381_g1_msm(pair_b, pair_s)
    assert (out[12:18] == 0).all()


def test_msm_batch_and_contexts(gb, orc):
    rng = np.random.default_rng(9)
    n = 5000
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    sb = np.stack([orc.fr_random(n, rng) for _ in range(3)])
    want = [affine_of(orc, orc.g1_msm(b, sb[i])) for i in range(3)]
    got = gb.bls12_381_g1_msm_batch(b, sb)
    for i in range(3):
        assert (affine_of(orc, got[i]) == want[i]).all()
    for window in (0, 9, 13, 16):
        ctx = gb.Bls12_381G1MsmContext(b, gb.RawMsmConfig.default(n, window))
        got = ctx.batch(sb)
        for i in range(3):
            assert (affine_of(orc, got[i]) == want[i]).all(), window
        ctx.close()
    ctx = gb.Bls12_381G1MsmContext(b)
    dv = gb.Bls12_381FrDeviceVec.upload(np.concatenate([np.zeros((7, 4), np.uint64), sb.reshape(-1, 4)]))
    got = ctx.device_batch(dv, 7, n, 3)
    for i in range(3):
        assert (affine_of(orc, got[i]) == want[i]).all()
    # ragged slices: a prefix of the bases and a full-length slice
    got = ctx.device_ragged(dv, [(7, 0, n), (7 + n, 0, 1000), (7 + 2 * n + 10, 10, 3000)])
    assert (affine_of(orc, got[0]) == want[0]).all()
    assert (affine_of(orc, got[1]) == affine_of(orc, orc.g1_msm(b[:1000], sb[1][:1000]))).all()
    assert (affine_of(orc, got[2]) == affine_of(orc, orc.g1_msm(b[10:3010], sb[2][10:3010]))).all()
    # scrambled: MSM(s + mask)
    mask = orc.fr_random(n, rng)
    mv = gb.Bls12_381FrDeviceVec.upload(mask)
    got = ctx.device_scrambled_batch(dv, 7, 3, mv)
    R = orc.R_MOD
    mi = orc.fr_to_ints(mask)
    for i in range(3):
        si = orc.fr_to_ints(sb[i])
        masked = orc.fr_from_ints([(x + y) % R for x, y in zip(si, mi)])
        assert (affine_of(orc, got[i]) == affine_of(orc, orc.g1_msm(b, masked))).all()
    ctx.close()


def test_msm_2p16(gb, orc):
    """The 2^16 configuration: uniform scalars, bases [r_i]G."""
    rng = np.random.default_rng(16)
    n = 1 << 16
    s = orc.fr_random(n, rng)
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    want = affine_of(orc, orc.g1_msm(b, s))
    assert (affine_of(orc, gb.bls12_381_g1_msm(b, s)) == want).all()
    ctx = gb.Bls12_381G1MsmContext(b)
    assert (affine_of(orc, ctx.msm(s)) == want).all()
    ctx.close()


def test_msm_real_srs_known_answers(gb, orc, srs):
    """Real bases from the reference's k=14 SRS: MSM(g_lagrange, 1) = G and
    MSM(g_lagrange, v) = MSM(g, iNTT(v)) with the NTT also on the GPU."""
    k, g, gl = srs
    n = 1 << k
    ones = orc.fr_from_ints([1] * n)
    assert (affine_of(orc, gb.bls12_381_g1_msm(gl, ones))[0] == g[0]).all()
    rng = np.random.default_rng(14)
    v = orc.fr_random(n, rng)
    coeffs = gb.bls12_381_fr_ntt(v, inverse=True)
    assert (coeffs == orc.fr_ntt(v, k, True)).all()
    ctx_g = gb.Bls12_381G1MsmContext(g)
    ctx_l = gb.Bls12_381G1MsmContext(gl)
    a = affine_of(orc, ctx_l.msm(v))
    b = affine_of(orc, ctx_g.msm(coeffs))
    assert (a == b).all()
    assert (a == affine_of(orc, orc.g1_msm(gl, v))).all()
    ctx_g.close()
    ctx_l.close()


def test_msm_2p20_linearity(gb, orc):
    """Full-size property: MSM(s + t) = MSM(s) + MSM(t) at n = 2^20 on the
    GPU (both context and plain paths), one oracle check of MSM(s)."""
    rng = np.random.default_rng(20)
    n = 1 << 20
    s = orc.fr_random(n, rng)
    t = orc.fr_random(n, rng)
    R = orc.R_MOD
    st = orc.fr_from_ints([(x + y) % R for x, y in zip(orc.fr_to_ints(s), orc.fr_to_ints(t))])
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    ctx = gb.Bls12_381G1MsmContext(b)
    res = ctx.batch(np.stack([s, t, st]))
    lhs = affine_of(orc, res[2])
    rhs = affine_of(orc, orc.g1_add(res[0], res[1]))
    assert (lhs == rhs).all()
    assert (affine_of(orc, res[0]) == affine_of(orc, orc.g1_msm(b, s))).all()
    plain = gb.bls12_381_g1_msm(b, t)
    assert (affine_of(orc, plain) == affine_of(orc, res[1])).all()
    ctx.close()


def _mixed_scalars(orc, n, rng):
    """70% uniform Fr, 20% uniform below 2^64, 10% zero (the batched configuration's mix)."""
    s = orc.fr_random(n, rng)
    u = rng.random(n)
    small = (u >= 0.7) & (u < 0.9)
    s[small] = orc.fr_from_ints([int(x) for x in rng.integers(0, 2**63, size=int(small.sum()), dtype=np.int64)])
    s[u >= 0.9] = 0
    return s


def test_ragged_batch_uneven_sizes(gb, orc):
    """One batched call over MSMs of uneven sizes, offsets and an empty slice,
    each equal to its own oracle MSM."""
    rng = np.random.default_rng(44)
    N = 1 << 14
    b = gb.g1_generator_mul(orc.fr_random(N, rng))
    sizes = [1 << 10, 3000, 0, 1, 1 << 13, 777, N]
    offs = [0, 100, 5, 9, 0, 2000, 0]
    scal = [_mixed_scalars(orc, n, rng) for n in sizes]
    flat = np.concatenate([x for x in scal if len(x)] + [np.zeros((1, 4), np.uint64)])
    so, slices = 0, []
    for n, po in zip(sizes, offs):
        slices.append((so, po, n))
        so += n
    ctx = gb.Bls12_381G1MsmContext(b)
    dv = gb.Bls12_381FrDeviceVec.upload(flat)
    got = ctx.device_ragged(dv, slices)
    for i, (n, po) in enumerate(zip(sizes, offs)):
        want = affine_of(orc, orc.g1_msm(b[po:po + n], scal[i])) if n else np.zeros((1, 12), np.uint64)
        assert (affine_of(orc, got[i]) == want).all(), i
    ctx.close()


def test_batch_plain_matches_single_calls(gb, orc):
    rng = np.random.default_rng(45)
    n = 2500
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    sb = np.stack([_mixed_scalars(orc, n, rng) for _ in range(5)])
    got = gb.bls12_381_g1_msm_batch(b, sb)
    for i in range(5):
        assert (affine_of(orc, got[i]) == affine_of(orc, gb.bls12_381_g1_msm(b, sb[i]))).all()
        assert (affine_of(orc, got[i]) == affine_of(orc, orc.g1_msm(b, sb[i]))).all()


@pytest.mark.parametrize("kind", ["ones", "two_values", "sparse_small"])
def test_skewed_buckets(gb, orc, kind):
    """Digit distributions that pile most points into a few buckets (every
    scalar 1, two values, small values): long buckets are summed in
    parallel and the result equals the oracle's, for the plain path and the
    precomputed context path."""
    rng = np.random.default_rng(31)
    n = 1 << 16
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    if kind == "ones":
        s = orc.fr_from_ints([1] * n)
    elif kind == "two_values":
        s = orc.fr_from_ints([int(v) for v in rng.choice([3, 5], size=n)])
    else:
        s = orc.fr_from_ints([int(v) for v in rng.integers(0, 16, size=n)])
    want = affine_of(orc, orc.g1_msm(b, s))
    assert (affine_of(orc, gb.bls12_381_g1_msm(b, s)) == want).all()
    ctx = gb.Bls12_381G1MsmContext(b)
    assert (affine_of(orc, ctx.msm(s)) == want).all()
    ctx.close()


def test_sparse_top_window_config(gb, orc):
    """window_bits 15: the 18th window holds only the carry out of bit 254,
    so about half the points share one bucket of the top window."""
    rng = np.random.default_rng(15)
    n = 1 << 15
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    s = orc.fr_random(n, rng)
    ctx = gb.Bls12_381G1MsmContext(b, gb.RawMsmConfig.default(n, 15))
    assert (affine_of(orc, ctx.msm(s)) == affine_of(orc, orc.g1_msm(b, s))).all()
    ctx.close()


def test_autotuned_paths_match_oracle(gb, orc):
    """With the autotuner on, the window and NTT variant it picks change
    nothing in the results: plain batch, small ragged items, NTTs."""
    rng = np.random.default_rng(77)
    gb.autotune_reset()
    gb.autotune_set(True)
    try:
        n = 3000
        b = gb.g1_generator_mul(orc.fr_random(n, rng))
        sb = np.stack([_mixed_scalars(orc, n, rng) for _ in range(3)])
        got = gb.bls12_381_g1_msm_batch(b, sb)
        for i in range(3):
            assert (affine_of(orc, got[i]) == affine_of(orc, orc.g1_msm(b, sb[i]))).all()
        big = gb.g1_generator_mul(orc.fr_random(1 << 14, rng))
        ctx = gb.Bls12_381G1MsmContext(big)
        flat = np.concatenate([_mixed_scalars(orc, 700, rng), _mixed_scalars(orc, 500, rng)])
        dv = gb.Bls12_381FrDeviceVec.upload(flat)
        got = ctx.device_ragged(dv, [(0, 0, 700), (700, 100, 500)])
        assert (affine_of(orc, got[0]) == affine_of(orc, orc.g1_msm(big[:700], flat[:700]))).all()
        assert (affine_of(orc, got[1]) == affine_of(orc, orc.g1_msm(big[100:600], flat[700:]))).all()
        ctx.close()
        for log_n in (12, 18):
            v = orc.fr_random(1 << log_n, rng)
            assert (gb.bls12_381_fr_ntt(v, inverse=False) == orc.fr_ntt(v, log_n, False)).all()
        rep = gb.autotune_report()
        assert any(k.startswith("msm:") for k in rep) and any(k.startswith("ntt:") for k in rep)
    finally:
        gb.autotune_set(False)


def test_context_batch_pinned_host_scalars(gb, orc):
    """Page-locked host scalars are read in place by the device (no staging
    copy): the results equal the pageable path's and the oracle's."""
    import torch
    rng = np.random.default_rng(77)
    n, m = 1 << 12, 3
    bases = gb.g1_generator_mul(orc.fr_random(n, rng))
    scalars = orc.fr_random(n * m, rng).reshape(m, n, 4)
    ctx = gb.Bls12_381G1MsmContext(bases)
    pinned = torch.empty((m, n, 4), dtype=torch.int64, pin_memory=True)
    view = pinned.numpy().view(np.uint64)
    view[:] = scalars
    got = ctx.batch(view)
    want = ctx.batch(np.array(scalars))
    assert (affine_of(orc, got) == affine_of(orc, want)).all()
    assert (affine_of(orc, got[1:2]) == affine_of(orc, orc.g1_msm(bases, scalars[1])[None])).all()


@pytest.mark.parametrize("log_n", [0, 5, 12, 16])
def test_msm_device_pointers_no_table(gb, orc, log_n):
    """gb_g1_msm_device on torch-owned device memory equals the oracle."""
    import torch
    torch.cuda.set_device(0)
    rng = np.random.default_rng(900 + log_n)
    n = 1 << log_n if log_n else 0
    b = gb.g1_generator_mul(orc.fr_random(max(n, 1), rng))[:n]
    s = orc.fr_random(n, rng)
    db = torch.from_numpy(b.view(np.int64).copy()).cuda()
    ds = torch.from_numpy(s.view(np.int64).copy()).cuda()
    torch.cuda.synchronize()
    got = gb.g1_msm_device(db.data_ptr(), ds.data_ptr(), n)
    if n == 0:
        assert (affine_of(orc, got) == 0).all()
    else:
        assert (affine_of(orc, got) == affine_of(orc, orc.g1_msm(b, s))).all()


def test_context_device_batch_async(gb, orc):
    """gb_g1_msm_context_device_batch_async: several batches in flight at
    once, with NTT work queued behind them on the same lane, waited for out
    of order; each equals the oracle.  A ticket dropped without a wait is
    released, and an empty batch completes."""
    rng = np.random.default_rng(31)
    n = 3000
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    sb = np.stack([orc.fr_random(n, rng) for _ in range(4)])
    want = [affine_of(orc, orc.g1_msm(b, sb[i])) for i in range(4)]
    ctx = gb.Bls12_381G1MsmContext(b)
    dv = gb.Bls12_381FrDeviceVec.upload(sb.reshape(-1, 4))
    t1 = ctx.device_batch_async(dv, 0, n, 2)
    other = gb.Bls12_381FrDeviceVec.upload(orc.fr_random(1 << 12, rng))
    one = orc.fr_from_ints([1])[0]
    other.ntt_zeta_batch(12, 1, False, one, one, one)
    t2 = ctx.device_batch_async(dv, 2 * n, n, 2)
    dropped = ctx.device_batch_async(dv, 0, n, 1)
    empty = ctx.device_batch_async(dv, 0, n, 0)
    got2 = t2.wait()
    got1 = t1.wait()
    del dropped
    assert len(empty.wait()) == 0
    for i in range(2):
        assert (affine_of(orc, got1[i]) == want[i]).all()
        assert (affine_of(orc, got2[i]) == want[2 + i]).all()
    with pytest.raises(RuntimeError):
        t1.wait()
    # the same points as the synchronous call
    sync = ctx.device_batch(dv, 0, n, 4)
    for i in range(4):
        assert (affine_of(orc, sync[i]) == want[i]).all()
    with pytest.raises(Exception):
        ctx.device_batch_async(dv, 0, n, 5)  # past the end of the vector
    ctx.close()


def test_ticket_waited_on_another_thread(gb, orc):
    """A ticket queued on one thread's lane and waited for by another thread
    (on another lane): the wait checks the queuing lane's status and returns
    the points."""
    import threading
    rng = np.random.default_rng(41)
    n = 2000
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    s = orc.fr_random(n, rng)
    ctx = gb.Bls12_381G1MsmContext(b)
    dv = gb.Bls12_381FrDeviceVec.upload(s)
    box = {}

    def producer():
        gb.execution_lane_set(3)
        box["t"] = ctx.device_batch_async(dv, 0, n, 1)
        gb.execution_lane_set(0)

    def consumer():
        gb.execution_lane_set(5)
        box["p"] = box["t"].wait()
        gb.execution_lane_set(0)

    for f in (producer, consumer):
        th = threading.Thread(target=f)
        th.start()
        th.join()
    assert (affine_of(orc, box["p"][0]) == affine_of(orc, orc.g1_msm(b, s))).all()
    ctx.close()


def test_context_batches_replay_graphs(gb, orc):
    """A context batch shape seen before replays its captured CUDA graph
    (captured the second time the shape comes) with fresh descriptors: new
    scalars, the same points as the oracle and as the launch-by-launch
    path, synchronous and asynchronous calls, a plain-window batch of small
    items beside the table batch."""
    rng = np.random.default_rng(41)
    n = 2500
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    ctx = gb.Bls12_381G1MsmContext(b)
    gb.msm_graphs_enable(True)
    try:
        cap0, lau0 = gb.msm_graph_stats()
        # synchronous calls, then queued ones
        for asynchronous in (False, True):
            for rep in range(3):
                sb = np.stack([orc.fr_random(n, rng) for _ in range(3)])
                dv = gb.Bls12_381FrDeviceVec.upload(sb.reshape(-1, 4))
                got = ctx.device_batch_async(dv, 0, n, 3).wait() if asynchronous else ctx.device_batch(dv, 0, n, 3)
                for i in range(3):
                    assert (affine_of(orc, got[i]) == affine_of(orc, orc.g1_msm(b, sb[i]))).all(), (rep, i)
                dv.free()
            # captured the second time the shape comes (the first, if an
            # earlier context at the same address had this shape), replayed
            # after that
            cap1, lau1 = gb.msm_graph_stats()
            assert cap1 - cap0 <= 1 and lau1 - lau0 >= 2, asynchronous
            cap0, lau0 = cap1, lau1
        # small items (plain windows over the context's bases) beside a big
        # one: two batches, each through its own graph
        sizes, offs = [n, 40, 7], [0, 300, 2000]
        for rep in range(2):
            sc = [orc.fr_random(m, rng) for m in sizes]
            dv = gb.Bls12_381FrDeviceVec.upload(np.concatenate(sc))
            slices, so = [], 0
            for m, po in zip(sizes, offs):
                slices.append((so, po, m))
                so += m
            got = ctx.device_ragged(dv, slices)
            for i, (m, po) in enumerate(zip(sizes, offs)):
                assert (affine_of(orc, got[i]) == affine_of(orc, orc.g1_msm(b[po:po + m], sc[i]))).all(), (rep, i)
            dv.free()
        cap2, lau2 = gb.msm_graph_stats()
        assert cap2 - cap1 <= 2 and lau2 - lau1 >= 2
        lau1 = lau2
        gb.msm_graphs_enable(False)
        sb = np.stack([orc.fr_random(n, rng) for _ in range(3)])
        dv = gb.Bls12_381FrDeviceVec.upload(sb.reshape(-1, 4))
        direct = ctx.device_batch(dv, 0, n, 3)
        gb.msm_graphs_enable(True)
        replay = ctx.device_batch(dv, 0, n, 3)
        assert gb.msm_graph_stats()[1] > lau1
        for i in range(3):
            assert (affine_of(orc, direct[i]) == affine_of(orc, replay[i])).all()
        dv.free()
    finally:
        gb.msm_graphs_enable(True)
        ctx.close()


def test_async_batch_reads_scalars_as_queued(gb, orc):
    """A queued batch is ordered before the lane's later work: that work may
    transform the vector in place or free it before the ticket is waited
    for, and the points are those of the scalars at the call."""
    rng = np.random.default_rng(47)
    log_n = 12
    n = 1 << log_n
    b = gb.g1_generator_mul(orc.fr_random(n, rng))
    sb = np.stack([orc.fr_random(n, rng) for _ in range(3)])
    want = [affine_of(orc, orc.g1_msm(b, sb[i])) for i in range(3)]
    ctx = gb.Bls12_381G1MsmContext(b)
    one = orc.fr_from_ints([1])[0]
    for rep in range(3):  # the third call replays the shape's graph
        dv = gb.Bls12_381FrDeviceVec.upload(sb.reshape(-1, 4))
        ticket = ctx.device_batch_async(dv, 0, n, 3)
        dv.ntt_zeta_batch(log_n, 3, False, one, one, one)
        dv.free()
        got = ticket.wait()
        for i in range(3):
            assert (affine_of(orc, got[i]) == want[i]).all(), (rep, i)
    ctx.close()
