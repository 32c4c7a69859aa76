"""The reference's multi-open entry points (prepare, prepare_device, f_poly,
pi) through the C ABI against the oracle's polynomial evaluation, linear
combination and Kate division, on seeded random polynomials."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _q_layout(rng, poly_count, q_count):
    """q k = a random non-empty set of (polynomial, coefficient) items"""
    offsets, items = [0], []
    for _ in range(q_count):
        k = int(rng.integers(1, 4))
        items += [int(i) for i in rng.integers(0, poly_count, size=k)]
        offsets.append(len(items))
    return offsets, items


def _want_q(orc, polys, n, offsets, items, coeffs):
    out = []
    for k in range(len(offsets) - 1):
        sel = items[offsets[k]:offsets[k + 1]]
        stack = np.concatenate([polys[i * n:(i + 1) * n] for i in sel])
        out.append(orc.fr_poly_lincomb(stack, n, len(sel), coeffs[offsets[k]:offsets[k + 1]]))
    return np.concatenate(out)


def _floor_divide(orc, poly, pts):
    """floor(poly / prod (X - p)) at the same length (top coefficients zero)"""
    cur = poly
    for p in pts:
        q = orc.fr_kate_division(cur, p)
        cur = np.concatenate([q, np.zeros((1, 4), dtype=np.uint64)])
    return cur


@pytest.mark.parametrize("n,seed", [(257, 1), (1 << 14, 2)])
def test_multiopen_prepare_matches_oracle(gb, orc, n, seed):
    rng = np.random.default_rng(seed)
    poly_count, q_count, npts = 6, 4, 3
    polys = orc.fr_random(poly_count * n, rng)
    offsets, items = _q_layout(rng, poly_count, q_count)
    coeffs = orc.fr_random(len(items), rng)
    points = orc.fr_random(npts, rng)
    qp = [int(i) for i in rng.integers(0, poly_count, size=9)]
    qx = [int(i) for i in rng.integers(0, npts, size=9)]
    q, ev = gb.bls12_381_fr_multiopen_prepare(polys, n, offsets, items, coeffs, points, qp, qx)
    assert (q == _want_q(orc, polys, n, offsets, items, coeffs)).all()
    want = np.array([orc.fr_eval_poly(polys[p * n:(p + 1) * n], points[x]) for p, x in zip(qp, qx)])
    assert (ev == want).all()
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_multiopen_prepare(polys, n, [0, 2, 1, len(items)], items, coeffs, points, qp, qx)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_multiopen_prepare(polys, n, offsets, items, coeffs, points, qp, [npts] + qx[1:])


def test_multiopen_prepare_device_matches_host(gb, orc):
    rng = np.random.default_rng(5)
    n = 1024
    counts = (3, 2, 4)  # dynamic, fixed, extra
    data = [orc.fr_random(c * n, rng) for c in counts]
    sources = [gb.Bls12_381FrDeviceVec.upload(d) for d in data]
    refs = [(s, i) for s, c in enumerate(counts) for i in range(c)]
    rng.shuffle(refs)
    refs = [(int(s), int(i)) for s, i in refs]
    flat = np.concatenate([data[s][i * n:(i + 1) * n] for s, i in refs])
    offsets, items = _q_layout(rng, len(refs), 5)
    coeffs = orc.fr_random(len(items), rng)
    points = orc.fr_random(2, rng)
    qp = [int(i) for i in rng.integers(0, len(refs), size=6)]
    qx = [int(i) for i in rng.integers(0, 2, size=6)]
    q_host, q_dev, ev = gb.bls12_381_fr_multiopen_prepare_device(sources, n, refs, offsets, items, coeffs, points,
                                                                 qp, qx)
    want_q, want_ev = gb.bls12_381_fr_multiopen_prepare(flat, n, offsets, items, coeffs, points, qp, qx)
    assert (q_host == want_q).all()
    assert (q_dev.download() == want_q).all()
    assert (ev == want_ev).all()
    _, q_dev2, _ = gb.bls12_381_fr_multiopen_prepare_device(sources, n, refs, offsets, items, coeffs, points, qp, qx,
                                                            q_host=False)
    assert (q_dev2.download() == want_q).all()
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_multiopen_prepare_device(sources, n, refs[:-1] + [(1, counts[1])], offsets, items, coeffs,
                                                 points, qp, qx)


@pytest.mark.parametrize("n,seed", [(130, 3), (1 << 13, 4)])
def test_multiopen_f_and_pi_match_oracle(gb, orc, n, seed):
    rng = np.random.default_rng(seed)
    # q 1 has no points; q 3 three
    point_offsets = [0, 1, 1, 3, 6]
    q_count = len(point_offsets) - 1
    points = orc.fr_random(point_offsets[-1], rng)
    qs = orc.fr_random(q_count * n, rng)
    scalars = orc.fr_random(q_count, rng)
    q_vec = gb.Bls12_381FrDeviceVec.upload(qs)
    f_vec = gb.bls12_381_fr_multiopen_f_poly_device(q_vec, n, point_offsets, points, scalars)
    divided = np.concatenate([_floor_divide(orc, qs[k * n:(k + 1) * n],
                                            points[point_offsets[k]:point_offsets[k + 1]]) for k in range(q_count)])
    want_f = orc.fr_poly_lincomb(divided, n, q_count, scalars)
    f = f_vec.download()
    assert (f == want_f).all()

    pi_scalars = orc.fr_random(q_count + 1, rng)
    x = orc.fr_random(1, rng)[0]
    pi = gb.bls12_381_fr_multiopen_pi_device(q_vec, f_vec, n, pi_scalars, x).download()
    combined = orc.fr_poly_lincomb(np.concatenate([qs, want_f]), n, q_count + 1, pi_scalars)
    want_pi = orc.fr_kate_division(combined, x)
    assert pi.shape == (n - 1, 4)
    assert (pi == want_pi).all()
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_multiopen_f_poly_device(q_vec, n, [0, 2, 1, 3, 6], points, scalars)
    with pytest.raises(gb.MsmError):
        gb.bls12_381_fr_multiopen_pi_device(q_vec, f_vec, n, pi_scalars[:-1], x)
