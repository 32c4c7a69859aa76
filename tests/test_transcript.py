"""Fiat-Shamir transcript (transcript/implementors.rs:13-33, mod.rs:95-150):
the oracle's RFC 7693 BLAKE2b against the RFC's test vector and Python's
hashlib, and the host mirror's CircuitTranscript against an oracle replay."""
import hashlib

import numpy as np


def test_blake2b_rfc7693_vector(orc):
    want = bytes.fromhex(
        "ba80a53f981c4d0d6a2797b69f12f6e94c212f14685ac4b74b12bb6fdbffa2d1"
        "7d87c5392aab792dc252d5de4533cc9518d38aa8dbf1925ab92386edd4009923")
    assert orc.blake2b(b"abc") == want


def test_blake2b_keyed_matches_hashlib(orc):
    rng = np.random.default_rng(1)
    for ln in (0, 1, 127, 128, 129, 1000):
        data = rng.bytes(ln)
        key = b"Domain separator for transcript"
        assert orc.blake2b(data, key) == hashlib.blake2b(data, digest_size=64, key=key).digest(), ln


def test_transcript_matches_oracle_replay(gb, orc):
    from gb_prover.kzg import CircuitTranscript, compress, fr_to_repr
    rng = np.random.default_rng(7)
    pts = orc.g1_generator_mul_batch(orc.fr_random(3, rng))
    scal = orc.fr_random(3, rng)
    t = CircuitTranscript()
    ops = []
    got = []
    for i in range(3):
        t.write_point(pts[i])
        ops.append(("absorb", orc.g1_compress(pts[i])))
        t.write_scalar(scal[i])
        ops.append(("absorb", orc.fr_to_ints(scal[i])[0].to_bytes(32, "little")))
        got.append(t.squeeze_challenge())
        ops.append(("squeeze",))
    want = orc.transcript_replay(ops)
    assert (np.array(got) == want).all()
    # the proof bytes are the written encodings in order
    assert t.finalize() == b"".join(compress(pts[i]) + fr_to_repr(scal[i]) for i in range(3))
    assert compress(pts[0]) == orc.g1_compress(pts[0])
