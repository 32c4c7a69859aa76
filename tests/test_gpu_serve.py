"""Proof serving on the GPU: proofs made by the continuous-batching server
(several lanes in flight) are byte-identical to the same requests proved
alone, and the HBM budget bounds the proofs in flight."""
import numpy as np
import pytest

from plonk_cases import TAU, circuit

from gb_prover import plonk, serve
from gb_prover.kzg import CircuitTranscript, ParamsKZG
from gb_prover.rng import ChaCha20Rng, ints_to_mont

pytestmark = pytest.mark.gpu


def test_gpu_serving_mix_equals_alone(gb):
    srs = ParamsKZG.unsafe_setup(10, plonk.fr_mont(TAU))
    entries, wit = {}, {}
    for cid, shape in enumerate([(8, 3, 3, 0), (9, 3, 3, 1), (10, 4, 5, 2)]):
        c = circuit(*shape)
        fixed, advice, copies = c.synthesize()
        p = srs.downsize(c.k)
        entries[cid] = (p, plonk.keygen(p, c, plonk.GpuBackend(p), fixed, copies))
        wit[cid] = ints_to_mont([v for col in advice for v in col])
    sizes = [serve.proof_footprint_bytes(pk.circuit) for _, pk in entries.values()]
    budget = 2 * max(sizes)
    rng = np.random.default_rng(9)
    reqs = [(int(c), wit[int(c)], "r%d" % i) for i, c in enumerate(rng.integers(0, 3, size=24))]
    srv = serve.ProofServer(entries, slots=4, hbm_budget=budget)
    done, _ = serve.run_stream(srv, reqs, serve.poisson_arrivals(rng, 500.0, len(reqs)))
    srv.close()
    assert srv.peak_in_use <= budget
    for (cid, w, seed), r in zip(reqs, done):
        p, pk = entries[cid]
        alone = plonk.create_proof(p, pk, w, plonk.GpuBackend(p), CircuitTranscript(), ChaCha20Rng.from_label(seed))
        assert r.future.result() == alone


def test_gpu_fused_commitments_equal_alone(gb):
    """The server with the proofs' commitments fused into shared ragged MSM
    batches (CommitBatcher): same proof bytes as each request alone, with
    batches that really held several proofs' commitments."""
    srs = ParamsKZG.unsafe_setup(10, plonk.fr_mont(TAU))
    entries, wit = {}, {}
    for cid, shape in enumerate([(9, 3, 3, 1), (10, 4, 4, 1)]):
        c = circuit(*shape)
        fixed, advice, copies = c.synthesize()
        p = srs.downsize(c.k)
        entries[cid] = (p, plonk.keygen(p, c, plonk.GpuBackend(p), fixed, copies))
        wit[cid] = ints_to_mont([v for col in advice for v in col])
    rng = np.random.default_rng(17)
    reqs = [(int(c), wit[int(c)], "f%d" % i) for i, c in enumerate(rng.integers(0, 2, size=16))]
    srv = serve.ProofServer(entries, slots=4, fuse_commits=True)
    done, _ = serve.run_stream(srv, reqs, [0.0] * len(reqs))
    srv.close()
    assert srv.batcher.fused_requests > srv.batcher.batches  # some batches held several requests
    for (cid, w, seed), r in zip(reqs, done):
        p, pk = entries[cid]
        alone = plonk.create_proof(p, pk, w, plonk.GpuBackend(p), CircuitTranscript(), ChaCha20Rng.from_label(seed))
        assert r.future.result() == alone


def test_gpu_lockstep_proofs_equal_alone(gb):
    """plonk.create_proofs on the GPU: four proofs of one circuit in
    lockstep, every round's commitments fused into one MSM batch through the
    asynchronous context entry point, give each proof's bytes as made
    alone; and the server's lockstep groups (3 per lane) do too."""
    from oracle import plonk_cpu, plonk_verify
    c = circuit(9, 3, 4, 1)
    fixed, advice, copies = c.synthesize()
    p = ParamsKZG.unsafe_setup(9, plonk.fr_mont(TAU))
    be = plonk.GpuBackend(p)
    pk = plonk.keygen(p, c, be, fixed, copies)
    w = ints_to_mont([v for col in advice for v in col])
    seeds = ["ls%d" % i for i in range(4)]
    together = plonk.create_proofs(p, pk, [w] * 4, be, [CircuitTranscript() for _ in seeds],
                                   [ChaCha20Rng.from_label(s) for s in seeds])
    alone = [plonk.create_proof(p, pk, w, be, CircuitTranscript(), ChaCha20Rng.from_label(s)) for s in seeds]
    assert together == alone
    hp = plonk_cpu.setup_params(9, TAU)
    hpk = plonk.keygen(hp, c, plonk_cpu.OracleBackend(hp), fixed, copies)
    oracle_proof = plonk.create_proof(hp, hpk, w, plonk_cpu.OracleBackend(hp), CircuitTranscript(),
                                      ChaCha20Rng.from_label(seeds[0]))
    assert together[0] == oracle_proof
    assert plonk_verify.verify(hpk, together[0], TAU)
    srv = serve.ProofServer({0: (p, pk)}, slots=2, lockstep=3)
    reqs = [srv.submit(0, w, "sg%d" % i) for i in range(7)]
    srv.drain()
    srv.close()
    for i, r in enumerate(reqs):
        assert r.future.result() == plonk.create_proof(p, pk, w, be, CircuitTranscript(),
                                                       ChaCha20Rng.from_label("sg%d" % i))
