"""Wire format of the proof server: the reference's `serialize` crate
encoding and the /prove request and response built on it.

Encoding (serialize/src/util.rs:118-300, serializable.rs:20-130):
  * u8, u16, i8 .. i128: little-endian bytes;
  * u32, u64, u128: the SCALE compact form (ScaleBigInt): below 2^6 one byte
    v << 2; below 2^14 two bytes (v << 2 | 1) LE; below 2^30 four bytes
    (v << 2 | 2) LE; else a byte ((n - 4) << 2 | 3) and the n significant
    bytes LE.  Decoding rejects the non-canonical forms the reference
    rejects (a zero second byte, zero third and fourth bytes, a zero last
    byte);
  * Vec<T>: the length as a compact u32, then the elements; Option<T>: a
    byte 0, or 1 then the value; str: the length as a compact u64, then the
    UTF-8 bytes; [u8; N]: the bytes;
  * tagged_serialize: the ASCII prefix "midnight:" + tag + ":" then the value
    (serializable.rs:24-33).

The reference's /prove (proof-server/src/endpoints.rs:246-343) decodes a
tagged (ProofPreimageVersioned, Option<ProvingKeyMaterial>, Option<Fr>),
resolves the key (cached by the hash of its bytes, transient-crypto/src/
proofs.rs:405-470: an LRU of 5 keys), proves on a worker and answers with
the tagged proof.  A ProofPreimage is the ZKIR transcript of a Midnight
contract call, which needs the Rust ZKIR front end; here the request
carries the synthetic circuit's witness instead:

  ProveRequest, tag "gb-prove-request[v1]":
      key: Option<Vec<u8>>    proving-key file bytes (keyfile.py); None to use
                              a key the server already holds
      key_id: [u8; 32]        SHA-256 of the key file bytes
      witness: Vec<[u8; 32]>  advice values, column by column, 32-byte
                              little-endian canonical field elements
      seed: str               the prover rng's label (blinding factors)
  ProofResponse, tag "gb-proof[v1]": proof: Vec<u8>
"""
import hashlib
import io

import numpy as np

GLOBAL_TAG = b"midnight:"
REQUEST_TAG = "gb-prove-request[v1]"
RESPONSE_TAG = "gb-proof[v1]"


# ---------------------------------------------------------------- primitives

def write_compact(out, v):
    if v < 0:
        raise ValueError("compact integers are unsigned")
    if v < 1 << 6:
        out.write(bytes([v << 2]))
    elif v < 1 << 14:
        out.write(((v << 2) | 1).to_bytes(2, "little"))
    elif v < 1 << 30:
        out.write(((v << 2) | 2).to_bytes(4, "little"))
    else:
        n = (v.bit_length() + 7) // 8
        if n > 67:
            raise ValueError("compact integer too large")
        out.write(bytes([((n - 4) << 2) | 3]))
        out.write(v.to_bytes(n, "little"))


def _exact(inp, n):
    b = inp.read(n)
    if len(b) != n:
        raise ValueError("unexpected end of input")
    return b


def read_compact(inp):
    first = _exact(inp, 1)[0]
    mode = first & 3
    if mode == 0:
        return first >> 2
    if mode == 1:
        second = _exact(inp, 1)[0]
        if second == 0:
            raise ValueError("non-canonical compact encoding")
        return int.from_bytes(bytes([first, second]), "little") >> 2
    if mode == 2:
        rest = _exact(inp, 3)
        if rest[1] == 0 and rest[2] == 0:
            raise ValueError("non-canonical compact encoding")
        return int.from_bytes(bytes([first]) + rest, "little") >> 2
    n = (first >> 2) + 4
    b = _exact(inp, n)
    v = int.from_bytes(b, "little")
    if b[-1] == 0:
        raise ValueError("non-canonical compact encoding")
    return v


def write_u32(out, v):
    if not 0 <= v < 1 << 32:
        raise ValueError("u32 out of range")
    write_compact(out, v)


def read_u32(inp):
    v = read_compact(inp)
    if v >= 1 << 32:
        raise ValueError("out of range for u32")
    return v


def write_u64(out, v):
    if not 0 <= v < 1 << 64:
        raise ValueError("u64 out of range")
    write_compact(out, v)


def read_u64(inp):
    v = read_compact(inp)
    if v >= 1 << 64:
        raise ValueError("out of range for u64")
    return v


def write_str(out, s):
    b = s.encode("utf-8")
    write_u64(out, len(b))
    out.write(b)


def read_str(inp):
    return _exact(inp, read_u64(inp)).decode("utf-8")


def write_bytes_vec(out, b):
    write_u32(out, len(b))
    out.write(b)


def read_bytes_vec(inp):
    return _exact(inp, read_u32(inp))


def tagged(tag, body):
    return GLOBAL_TAG + tag.encode("ascii") + b":" + body


def untag(data, tag):
    prefix = GLOBAL_TAG + tag.encode("ascii") + b":"
    if not data.startswith(prefix):
        raise ValueError("expected a value tagged %r" % tag)
    return io.BytesIO(data[len(prefix):])


def _finish(inp):
    if inp.read(1):
        raise ValueError("trailing bytes")


# ---------------------------------------------------------------- /prove

R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
_R = pow(2, 256, R_MOD)
_RINV = pow(_R, -1, R_MOD)


def encode_request(witness_mont, seed, key_bytes=None, key_id=None):
    """witness_mont: (m*n, 4) Montgomery rows, column by column"""
    if key_id is None:
        if key_bytes is None:
            raise ValueError("a request names its key by id or carries it")
        key_id = hashlib.sha256(key_bytes).digest()
    out = io.BytesIO()
    if key_bytes is None:
        out.write(b"\x00")
    else:
        out.write(b"\x01")
        write_bytes_vec(out, key_bytes)
    if len(key_id) != 32:
        raise ValueError("key id is 32 bytes")
    out.write(key_id)
    w = np.ascontiguousarray(witness_mont, dtype=np.uint64).reshape(-1, 4)
    write_u32(out, len(w))
    for row in w:
        v = sum(int(x) << (64 * i) for i, x in enumerate(row)) * _RINV % R_MOD
        out.write(v.to_bytes(32, "little"))
    write_str(out, seed)
    return tagged(REQUEST_TAG, out.getvalue())


def decode_request(data):
    """(key bytes or None, key id, witness (m*n, 4) Montgomery rows, seed)"""
    inp = untag(data, REQUEST_TAG)
    flag = _exact(inp, 1)[0]
    if flag not in (0, 1):
        raise ValueError("bad option flag")
    key = read_bytes_vec(inp) if flag else None
    key_id = _exact(inp, 32)
    if key is not None and hashlib.sha256(key).digest() != key_id:
        raise ValueError("key id does not match the key bytes")
    n = read_u32(inp)
    raw = _exact(inp, 32 * n)
    w = np.zeros((n, 4), dtype=np.uint64)
    for i in range(n):
        v = int.from_bytes(raw[32 * i:32 * i + 32], "little")
        if v >= R_MOD:
            raise ValueError("witness value not below the modulus")
        m = v * _R % R_MOD
        w[i] = [(m >> (64 * j)) & 0xFFFFFFFFFFFFFFFF for j in range(4)]
    seed = read_str(inp)
    _finish(inp)
    return key, key_id, w, seed


def encode_response(proof):
    out = io.BytesIO()
    write_bytes_vec(out, proof)
    return tagged(RESPONSE_TAG, out.getvalue())


def decode_response(data):
    inp = untag(data, RESPONSE_TAG)
    proof = read_bytes_vec(inp)
    _finish(inp)
    return proof
