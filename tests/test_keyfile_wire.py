"""Proving-key files and the /prove wire format on the CPU (oracle backend).

The serialize crate's encoding is pinned to the reference's own test
vectors (serialize/tests/serialize.rs:141-174); the key file round-trips
byte for byte, and a key read back proves the same bytes as the key it was
written from; a /prove request through the server's request loop answers
with the proof the key gives alone."""
import gzip
import hashlib
import io
import struct

import numpy as np
import pytest

from plonk_cases import TAU, circuit

from gb_prover import keyfile, plonk, serve, wire
from gb_prover.kzg import CircuitTranscript
from gb_prover.rng import ChaCha20Rng, ints_to_mont
from oracle import plonk_cpu


def _ser_compact(v):
    out = io.BytesIO()
    wire.write_compact(out, v)
    b = out.getvalue()
    assert wire.read_compact(io.BytesIO(b)) == v
    return list(b)


def test_scale_compact_reference_vectors():
    # serialize/tests/serialize.rs:150-160 (u128 values)
    assert _ser_compact(0) == [0x00]
    assert _ser_compact(1) == [0x04]
    assert _ser_compact(42) == [0xA8]
    assert _ser_compact(69) == [0x15, 0x01]
    assert _ser_compact(65535) == [0xFE, 0xFF, 0x03, 0x00]
    assert _ser_compact(100000000000000) == [0x0B, 0x00, 0x40, 0x7A, 0x10, 0xF3, 0x5A]
    # the size boundaries of the four forms
    for v in (63, 64, (1 << 14) - 1, 1 << 14, (1 << 30) - 1, 1 << 30, (1 << 32) - 1, 1 << 40):
        _ser_compact(v)


def test_scale_vec_reference_vector():
    # serialize/tests/serialize.rs:163-174: Vec<u16> [4, 8, 15, 16, 23, 42]
    out = io.BytesIO()
    vals = [4, 8, 15, 16, 23, 42]
    wire.write_u32(out, len(vals))
    for v in vals:
        out.write(struct.pack("<H", v))
    assert list(out.getvalue()) == [0x18, 0x04, 0x00, 0x08, 0x00, 0x0F, 0x00, 0x10, 0x00, 0x17, 0x00, 0x2A, 0x00]


def test_scale_rejects_non_canonical():
    for bad in ([0x01, 0x00], [0x02, 0x05, 0x00, 0x00], [0x03, 0x01, 0x02, 0x03, 0x00]):
        with pytest.raises(ValueError):
            wire.read_compact(io.BytesIO(bytes(bad)))
    with pytest.raises(ValueError):
        wire.untag(b"midnight:other:xyz", wire.REQUEST_TAG)


def _key(shape=(7, 3, 3, 1)):
    c = circuit(*shape)
    fixed, advice, copies = c.synthesize()
    params = plonk_cpu.setup_params(c.k, TAU)
    be = plonk_cpu.OracleBackend(params)
    pk = plonk.keygen(params, c, be, fixed, copies)
    return params, be, pk, ints_to_mont([v for col in advice for v in col])


def test_key_file_round_trip_and_prove():
    params, be, pk, wit = _key()
    data = keyfile.write_pk(pk, be)
    raw = gzip.decompress(data)
    # MidnightPK: k, relation, then the verifying key's version byte and k
    assert raw[0] == pk.circuit.k
    rel = keyfile.write_relation(pk.circuit)
    assert raw[1:1 + len(rel)] == rel
    assert raw[1 + len(rel):3 + len(rel)] == bytes([keyfile.VK_VERSION, pk.circuit.k])
    c2, fc, sc, fixed, sigma = keyfile.parse_pk(data)
    assert c2.describe() == pk.circuit.describe()
    assert all((a == b).all() for a, b in zip(fc, pk.fixed_commitments))
    assert all((a == b).all() for a, b in zip(sc, pk.sigma_commitments))
    assert (fixed == be.get(pk.fixed_lagrange)).all() and (sigma == pk.sigma_lagrange_host).all()
    pk2 = keyfile.read_pk(data, params, be)
    assert keyfile.write_pk(pk2, be) == data
    assert pk2.transcript_repr == pk.transcript_repr
    p1 = plonk.create_proof(params, pk, wit, be, CircuitTranscript(), ChaCha20Rng.from_label("kf"))
    p2 = plonk.create_proof(params, pk2, wit, be, CircuitTranscript(), ChaCha20Rng.from_label("kf"))
    assert p1 == p2


def test_key_file_rejects_damage():
    params, be, pk, _ = _key((7, 3, 3, 0))
    raw = bytearray(gzip.decompress(keyfile.write_pk(pk, be)))
    rel_len = len(keyfile.write_relation(pk.circuit))
    off = 1 + rel_len
    cases = []
    bad = bytearray(raw)
    bad[off] = 0x02  # version byte
    cases.append(bad)
    bad = bytearray(raw)
    bad[off + 7] ^= 0x01  # a coordinate byte of the first fixed commitment: off the curve
    cases.append(bad)
    cases.append(raw[:-5])  # truncated
    cases.append(raw + b"\x00")  # trailing byte
    for b in cases:
        with pytest.raises(ValueError):
            keyfile.parse_pk(gzip.compress(bytes(b)))


def test_prove_request_through_the_server():
    params, be, pk, wit = _key((7, 3, 3, 1))
    data = keyfile.write_pk(pk, be)
    kid = hashlib.sha256(data).digest()
    store = serve.KeyStore(lambda k: params, capacity=2, backend_factory=plonk_cpu.OracleBackend)
    srv = serve.ProofServer({}, slots=2, backend_factory=plonk_cpu.OracleBackend, set_lane=None, keystore=store)
    try:
        req = wire.encode_request(wit, "wire-1", key_bytes=data)
        assert req.startswith(b"midnight:" + wire.REQUEST_TAG.encode() + b":")
        k2, kid2, w2, seed = wire.decode_request(req)
        assert k2 == data and kid2 == kid and (w2 == wit).all() and seed == "wire-1"
        resp = srv.handle(req)
        proof = wire.decode_response(resp)
        want = plonk.create_proof(params, pk, wit, be, CircuitTranscript(), ChaCha20Rng.from_label("wire-1"))
        assert proof == want
        # the key is held now: a request naming it by id alone is served
        resp2 = srv.handle(wire.encode_request(wit, "wire-1", key_id=kid))
        assert wire.decode_response(resp2) == want
        assert len(store) == 1
        # an unknown key without key material is refused
        with pytest.raises(KeyError):
            srv.handle(wire.encode_request(wit, "x", key_id=bytes(32)))
    finally:
        srv.close()
