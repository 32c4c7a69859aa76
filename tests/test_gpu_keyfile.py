"""Proving-key files on the GPU: a key written from the device and read
back into resident state proves the same bytes as the key it came from and
as the oracle backend; a /prove request carrying the key file is served
through the key store (SRS downsized to the key's size)."""
import hashlib

import pytest

from plonk_cases import TAU, circuit

pytestmark = pytest.mark.gpu


def test_gpu_key_file_round_trip_proves_same_bytes(gb, orc):
    from gb_prover import keyfile, plonk
    from gb_prover.kzg import CircuitTranscript, ParamsKZG
    from gb_prover.rng import ChaCha20Rng, ints_to_mont
    from oracle import plonk_cpu
    c = circuit(10, 4, 4, 1)
    fixed, advice, copies = c.synthesize()
    params = ParamsKZG.unsafe_setup(c.k, plonk.fr_mont(TAU))
    be = plonk.GpuBackend(params)
    pk = plonk.keygen(params, c, be, fixed, copies)
    data = keyfile.write_pk(pk, be)
    pk2 = keyfile.read_pk(data, params, be)
    assert keyfile.write_pk(pk2, be) == data
    wit = ints_to_mont([v for col in advice for v in col])
    p1 = plonk.create_proof(params, pk, wit, be, CircuitTranscript(), ChaCha20Rng.from_label("gpu-kf"))
    p2 = plonk.create_proof(params, pk2, wit, be, CircuitTranscript(), ChaCha20Rng.from_label("gpu-kf"))
    assert p1 == p2
    # the same key file read on the oracle backend proves the same bytes
    hp = plonk_cpu.setup_params(c.k, TAU)
    ob = plonk_cpu.OracleBackend(hp)
    pk3 = keyfile.read_pk(data, hp, ob)
    assert plonk.create_proof(hp, pk3, wit, ob, CircuitTranscript(), ChaCha20Rng.from_label("gpu-kf")) == p1


def test_gpu_prove_request_with_key_material(gb, orc):
    from gb_prover import keyfile, plonk, serve, wire
    from gb_prover.kzg import CircuitTranscript, ParamsKZG
    from gb_prover.rng import ChaCha20Rng, ints_to_mont
    srs = ParamsKZG.unsafe_setup(11, plonk.fr_mont(TAU))
    c = circuit(9, 3, 3, 1)
    fixed, advice, copies = c.synthesize()
    params = srs.downsize(c.k)
    be = plonk.GpuBackend(params)
    pk = plonk.keygen(params, c, be, fixed, copies)
    data = keyfile.write_pk(pk, be)
    wit = ints_to_mont([v for col in advice for v in col])
    want = plonk.create_proof(params, pk, wit, be, CircuitTranscript(), ChaCha20Rng.from_label("req"))
    store = serve.KeyStore.from_srs(srs)
    srv = serve.ProofServer({}, slots=2, keystore=store)
    try:
        resp = srv.handle(wire.encode_request(wit, "req", key_bytes=data))
        assert wire.decode_response(resp) == want
        resp = srv.handle(wire.encode_request(wit, "req", key_id=hashlib.sha256(data).digest()))
        assert wire.decode_response(resp) == want
    finally:
        srv.close()
