"""Proving-key files: the byte layout a Midnight proof server stores and
loads keys in, and the resident key rebuilt from one.

The layout follows the reference's key path:

  * zkir's `read_raw_pk` / `write_raw_pk` (zkir/src/ir.rs:186-199) wrap the
    key in a gzip stream (flate2 GzEncoder / GzDecoder);
  * inside it, `MidnightPK::write` (vendor/midnight-zk-stdlib-2.3.1/src/
    lib.rs:1689-1722): one byte k, the relation, then the proving key;
  * `ProvingKey::write` (vendor/midnight-proofs-0.8.1/src/plonk/mod.rs:
    516-521): the verifying key, the fixed columns' Lagrange values, the
    permutation's sigma values;
  * `VerifyingKey::write` (plonk/mod.rs:220-231): version byte 0x03, k, a
    u32 little-endian count of fixed commitments, each commitment, then
    the permutation verifying key (one commitment per permutation column,
    permutation.rs:105-113);
  * commitments in SerdeFormat::RawBytes: the 96-byte uncompressed zcash
    encoding (`write_raw` = `to_uncompressed`, g1.rs:483-485);
  * polynomial lists (utils/helpers.rs:132-155, poly/mod.rs:264-285): a u32
    big-endian count, then per polynomial a u32 big-endian length and the
    values as 32-byte raw Montgomery limbs (`write_raw`, fq.rs:903-908).

Reading rebuilds what `ProvingKey::read` (plonk/mod.rs:538-590) derives
from the stored values: coefficient forms and extended cosets of the fixed
and sigma columns, l0 / l_last / l_active and the compiled constraint
graphs, all resident on the device; the commitments come from the file.

The relation section is the reference's ZKIR circuit, which only the Rust
toolchain can compile; here it holds the parameters of the synthetic
circuits this prover builds (k, advice columns, gate degree, lookups, copy
constraints, table size, label), in the serialize crate's encoding
(wire.py), so a key file determines its circuit as in the reference.
"""
import gzip
import io
import struct

import numpy as np

from . import wire
from .kzg import P_MOD, R_MOD, _FP_R, _FP_RINV, _int, _limbs, from_uncompressed
from .plonk import SyntheticCircuit, keygen_from_values

VK_VERSION = 0x03
RELATION_TAG = "gb-synthetic-relation[v1]"
PK_COMPRESSION_LEVEL = 6


def to_uncompressed(affine):
    """zcash 96-byte uncompressed encoding of an affine point (g1.rs to_uncompressed)."""
    a = np.asarray(affine, dtype=np.uint64).reshape(12)
    if not a.any():
        return bytes([0x40]) + bytes(95)
    x = _int(a[0:6]) * _FP_RINV % P_MOD
    y = _int(a[6:12]) * _FP_RINV % P_MOD
    return x.to_bytes(48, "big") + y.to_bytes(48, "big")


def _write_polys(out, rows, count, n):
    """a polynomial list: u32 BE count, per polynomial u32 BE length + raw limbs"""
    rows = np.ascontiguousarray(rows, dtype="<u8").reshape(count, n, 4)
    out.write(struct.pack(">I", count))
    for p in range(count):
        out.write(struct.pack(">I", n))
        out.write(rows[p].tobytes())


def _read_polys(inp, checked):
    (count,) = struct.unpack(">I", _exact(inp, 4))
    polys = []
    for _ in range(count):
        (n,) = struct.unpack(">I", _exact(inp, 4))
        a = np.frombuffer(_exact(inp, 32 * n), dtype="<u8").reshape(n, 4).astype(np.uint64)
        if checked and not _all_below_r(a):
            raise ValueError("field element not below the modulus")
        polys.append(a)
    return polys


def _all_below_r(a):
    r = np.array(_limbs(R_MOD, 4), dtype=np.uint64)
    lt = np.zeros(len(a), dtype=bool)
    eq = np.ones(len(a), dtype=bool)
    for i in (3, 2, 1, 0):
        lt |= eq & (a[:, i] < r[i])
        eq &= a[:, i] == r[i]
    return bool(lt.all())


def _exact(inp, n):
    b = inp.read(n)
    if len(b) != n:
        raise ValueError("key file truncated")
    return b


def write_relation(circuit):
    """the synthetic circuit's parameters in the serialize crate's encoding"""
    out = io.BytesIO()
    for v in (circuit.k, circuit.m, circuit.d, circuit.lookups, circuit.copies, circuit.table_log):
        wire.write_u32(out, v)
    wire.write_str(out, circuit.label)
    return out.getvalue()


def read_relation(inp):
    k, m, d, lookups, copies, table_log = (wire.read_u32(inp) for _ in range(6))
    label = wire.read_str(inp)
    return SyntheticCircuit(k, advice=m, degree=d, lookups=lookups, copies=copies, table_log=table_log,
                            label=label)


def write_pk(pk, backend, compress_level=PK_COMPRESSION_LEVEL):
    """MidnightPK bytes of a resident proving key, gzip-wrapped as zkir's
    write_raw_pk does"""
    c = pk.circuit
    raw = io.BytesIO()
    raw.write(bytes([c.k]))
    raw.write(write_relation(c))
    # verifying key
    raw.write(bytes([VK_VERSION, c.k]))
    raw.write(struct.pack("<I", len(pk.fixed_commitments)))
    for p in pk.fixed_commitments:
        raw.write(to_uncompressed(p))
    for p in pk.sigma_commitments:
        raw.write(to_uncompressed(p))
    # fixed values, then the permutation's sigma values
    _write_polys(raw, backend.get(pk.fixed_lagrange), c.num_fixed, c.n)
    _write_polys(raw, pk.sigma_lagrange_host, c.m, c.n)
    return gzip.compress(raw.getvalue(), compresslevel=compress_level, mtime=0)


def parse_pk(data, checked=True):
    """(circuit, fixed commitments, sigma commitments, fixed values, sigma
    values) from key-file bytes; `checked` verifies every point is on the
    curve and every field element below the modulus (RawBytes), else the
    values are taken as they are (RawBytesUnchecked)"""
    inp = io.BytesIO(gzip.decompress(data))
    k = _exact(inp, 1)[0]
    circuit = read_relation(inp)
    if circuit.k != k:
        raise ValueError("key file k does not match its relation")
    version, vk_k = _exact(inp, 2)
    if version != VK_VERSION:
        raise ValueError("unexpected verifying-key version byte")
    if vk_k != k:
        raise ValueError("verifying key k does not match")
    (nfixed,) = struct.unpack("<I", _exact(inp, 4))
    if nfixed != circuit.num_fixed:
        raise ValueError("fixed column count does not match the relation")

    def point():
        b = _exact(inp, 96)
        if checked:
            return from_uncompressed(b)
        if b[0] & 0x40:
            return np.zeros(12, dtype=np.uint64)
        x = int.from_bytes(bytes([b[0] & 0x1F]) + b[1:48], "big")
        y = int.from_bytes(b[48:96], "big")
        return np.array(_limbs(x * _FP_R % P_MOD, 6) + _limbs(y * _FP_R % P_MOD, 6), dtype=np.uint64)

    fixed_c = [point() for _ in range(nfixed)]
    sigma_c = [point() for _ in range(circuit.m)]
    fixed = _read_polys(inp, checked)
    sigma = _read_polys(inp, checked)
    if len(fixed) != nfixed or len(sigma) != circuit.m or any(len(p) != circuit.n for p in fixed + sigma):
        raise ValueError("polynomial count or length does not match the relation")
    if inp.read(1):
        raise ValueError("trailing bytes after the proving key")
    return circuit, fixed_c, sigma_c, np.concatenate(fixed), np.concatenate(sigma)


def read_pk(data, params, backend, checked=True):
    """the resident proving key of a key file (ProvingKey::read): the stored
    values go to the device and the derived forms are computed there"""
    circuit, fixed_c, sigma_c, fixed, sigma = parse_pk(data, checked)
    if params.k != circuit.k:
        raise ValueError("SRS size does not match the key")
    return keygen_from_values(params, circuit, backend, fixed, sigma, fixed_c, sigma_c)
