"""Proof serving with continuous batching, on the oracle backend (CPU):
proofs in the mix equal the proofs made alone, the HBM budget bounds what
is in flight, a failing request does not stop the server."""
import numpy as np

from plonk_cases import TAU, circuit

from gb_prover import plonk, serve
from gb_prover.kzg import CircuitTranscript
from gb_prover.rng import ChaCha20Rng, ints_to_mont
from oracle import plonk_cpu


def _entries():
    out, wit = {}, {}
    for cid, shape in enumerate([(7, 3, 3, 0), (8, 3, 3, 1), (8, 4, 5, 2)]):
        c = circuit(*shape)
        fixed, advice, copies = c.synthesize()
        p = plonk_cpu.setup_params(c.k, TAU)
        pk = plonk.keygen(p, c, plonk_cpu.OracleBackend(p), fixed, copies)
        out[cid] = (p, pk)
        wit[cid] = ints_to_mont([v for col in advice for v in col])
    return out, wit


def _alone(entries, cid, witness, seed):
    p, pk = entries[cid]
    return plonk.create_proof(p, pk, witness, plonk_cpu.OracleBackend(p), CircuitTranscript(),
                              ChaCha20Rng.from_label(seed))


def test_mix_equals_alone_and_budget_holds():
    entries, wit = _entries()
    sizes = {cid: serve.proof_footprint_bytes(pk.circuit) for cid, (_, pk) in entries.items()}
    budget = max(sizes.values()) + min(sizes.values())
    srv = serve.ProofServer(entries, slots=3, hbm_budget=budget, backend_factory=plonk_cpu.OracleBackend,
                            set_lane=None)
    rng = np.random.default_rng(5)
    reqs = [(int(c), wit[int(c)], "req-%d" % i) for i, c in enumerate(rng.integers(0, 3, size=12))]
    done, t0 = serve.run_stream(srv, reqs, serve.poisson_arrivals(rng, 200.0, len(reqs)))
    srv.close()
    assert srv.peak_in_use <= budget
    for (cid, w, seed), r in zip(reqs, done):
        assert r.future.result() == _alone(entries, cid, w, seed)
    s = serve.latency_summary(done, t0)
    assert s["proofs"] == 12 and s["p99_ms"] >= s["p50_ms"] > 0


def test_failed_request_isolated():
    entries, wit = _entries()
    srv = serve.ProofServer(entries, slots=2, backend_factory=plonk_cpu.OracleBackend, set_lane=None)
    bad = srv.submit(1, wit[1][: len(wit[1]) // 2], "bad")  # truncated witness
    good = srv.submit(0, wit[0], "good")
    srv.drain()
    srv.close()
    assert bad.future.exception() is not None
    assert good.future.result() == _alone(entries, 0, wit[0], "good")


def test_lockstep_proofs_equal_alone():
    """plonk.create_proofs runs several proofs of one circuit in lockstep
    (their commitments requested together at every round): each proof's
    bytes equal the proof made alone.  The server's lockstep groups give the
    same bytes as well."""
    entries, wit = _entries()
    p, pk = entries[2]
    seeds = ["lock-%d" % i for i in range(3)]
    together = plonk.create_proofs(p, pk, [wit[2]] * 3, plonk_cpu.OracleBackend(p),
                                   [CircuitTranscript() for _ in seeds], [ChaCha20Rng.from_label(s) for s in seeds])
    assert together == [_alone(entries, 2, wit[2], s) for s in seeds]
    srv = serve.ProofServer(entries, slots=2, backend_factory=plonk_cpu.OracleBackend, set_lane=None, lockstep=3)
    reqs = [srv.submit(cid, wit[cid], "g-%d" % i) for i, cid in enumerate([2, 2, 1, 2, 0, 2])]
    srv.drain()
    for i, (r, cid) in enumerate(zip(reqs, [2, 2, 1, 2, 0, 2])):
        assert r.future.result() == _alone(entries, cid, wit[cid], "g-%d" % i)
    srv.close()
