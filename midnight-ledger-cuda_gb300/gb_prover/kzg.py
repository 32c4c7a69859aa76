"""KZG commitment layer and Fiat-Shamir transcript over the C ABI.

ParamsKZG mirrors vendor/midnight-proofs-0.8.1/src/poly/kzg/params.rs:38-260
(g, g_lagrange; seeded-tau setup; downsize via g_to_lagrange; the RawBytes
file format).  The commit functions mirror KZGCommitmentScheme::{commit,
commit_batch, commit_lagrange, commit_lagrange_batch} (poly/kzg/mod.rs:
1072-1430): coefficient-form polynomials commit against g, Lagrange-form
against g_lagrange, every batch through one resident MSM context per basis
(the reference's context cache, g1.rs:744-786).  CircuitTranscript mirrors
CircuitTranscript<Blake2bState> (transcript/mod.rs:95-150,
implementors.rs:13-33,140-170).
"""
import ctypes
import hashlib
import struct

import numpy as np

from ._lib import MsmError, check, lib
from .api import Bls12_381G1MsmContext, _fr, _ptr

P_MOD = int("1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab", 16)
R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
_FP_R = pow(2, 384, P_MOD)
_FP_RINV = pow(_FP_R, -1, P_MOD)
_FR_R = pow(2, 256, R_MOD)
_FR_RINV = pow(_FR_R, -1, R_MOD)


def _limbs(v, n):
    return [(v >> (64 * i)) & 0xFFFFFFFFFFFFFFFF for i in range(n)]


def _int(row):
    """little-endian u64 limbs -> integer"""
    return int.from_bytes(np.ascontiguousarray(row, dtype="<u8").tobytes(), "little")


# Montgomery factors of the affine conversion: with X = x R, Y = y R and
# Z = z R (mod p), the affine point's Montgomery coordinates are
# X R^2 / Z^2 and Y R^3 / Z^3
_FP_R2 = _FP_R * _FP_R % P_MOD
_FP_R3 = _FP_R2 * _FP_R % P_MOD


# ---------------------------------------------------------------- point encodings (host side)

def affine_from_projective(jac):
    """Jacobian (18 u64, Montgomery) -> affine (12 u64); infinity -> zeros."""
    return affine_from_projective_batch(np.asarray(jac, dtype=np.uint64).reshape(1, 18))[0]


def affine_from_projective_batch(jacs):
    """affine_from_projective over a batch with one field inversion
    (Montgomery's trick): (m, 18) Jacobian rows -> (m, 12) affine rows.
    Through the library's host-side gb_g1_jacobian_to_affine_batch once
    this process has loaded it, else in Python integers."""
    from . import _lib as _l
    if _l._lib is not None:
        src = np.ascontiguousarray(jacs, dtype=np.uint64).reshape(-1, 18)
        out = np.empty((len(src), 12), dtype=np.uint64)
        check(_l._lib.gb_g1_jacobian_to_affine_batch(_ptr(out), _ptr(src), len(src)))
        return out
    return _affine_from_projective_batch_py(jacs)


def _affine_from_projective_batch_py(jacs):
    raw = np.ascontiguousarray(jacs, dtype="<u8").reshape(-1, 18).tobytes()
    m = len(raw) // 144
    frm = int.from_bytes
    zs = [frm(raw[144 * i + 96:144 * i + 144], "little") % P_MOD for i in range(m)]
    prefix, acc = [], 1
    for z in zs:
        prefix.append(acc)
        if z:
            acc = acc * z % P_MOD
    inv = pow(acc, -1, P_MOD)
    rows = [bytes(96)] * m
    for i in range(m - 1, -1, -1):
        z = zs[i]
        if z == 0:
            continue
        zi = inv * prefix[i] % P_MOD
        inv = inv * z % P_MOD
        zi2 = zi * zi % P_MOD
        ax = frm(raw[144 * i:144 * i + 48], "little") * zi2 % P_MOD * _FP_R2 % P_MOD
        ay = frm(raw[144 * i + 48:144 * i + 96], "little") * zi2 % P_MOD * zi % P_MOD * _FP_R3 % P_MOD
        rows[i] = ax.to_bytes(48, "little") + ay.to_bytes(48, "little")
    return np.frombuffer(bytearray(b"".join(rows)), dtype="<u8").reshape(m, 12)


def compress(affine):
    """zcash 48-byte compressed encoding of an affine point (g1.rs:1179-1211)."""
    b = np.ascontiguousarray(affine, dtype="<u8").reshape(12).tobytes()
    xm, ym = int.from_bytes(b[:48], "little"), int.from_bytes(b[48:], "little")
    if not xm and not ym:
        return bytes([0xC0]) + bytes(47)
    x = xm * _FP_RINV % P_MOD
    y = ym * _FP_RINV % P_MOD
    out = bytearray(x.to_bytes(48, "big"))
    out[0] |= 0x80
    if y > P_MOD - y:
        out[0] |= 0x20
    return bytes(out)


def from_uncompressed(b96):
    """zcash 96-byte uncompressed encoding -> affine Montgomery limbs."""
    flags = b96[0]
    if flags & 0x80:
        raise ValueError("compressed flag set in an uncompressed encoding")
    if flags & 0x40:
        return np.zeros(12, dtype=np.uint64)
    x = int.from_bytes(bytes([flags & 0x1F]) + b96[1:48], "big")
    y = int.from_bytes(b96[48:96], "big")
    if x >= P_MOD or y >= P_MOD or (y * y - x * x * x - 4) % P_MOD:
        raise ValueError("point not on the curve")
    return np.array(_limbs(x * _FP_R % P_MOD, 6) + _limbs(y * _FP_R % P_MOD, 6), dtype=np.uint64)


def fr_to_repr(fr):
    """Fr (Montgomery limbs) -> 32-byte little-endian canonical repr."""
    return (_int(np.asarray(fr).reshape(4)) * _FR_RINV % R_MOD).to_bytes(32, "little")


def fr_from_uniform_bytes(b64):
    """fq.rs:704-725: the 512-bit little-endian value of the bytes, mod r."""
    v = int.from_bytes(b64, "little") % R_MOD
    return np.frombuffer(bytearray((v * _FR_R % R_MOD).to_bytes(32, "little")), dtype="<u8")


# ---------------------------------------------------------------- SRS

class ParamsKZG:
    def __init__(self, k, g, g_lagrange):
        self.k = k
        self.n = 1 << k
        self.g = np.ascontiguousarray(g, dtype=np.uint64).reshape(self.n, 12)
        self.g_lagrange = np.ascontiguousarray(g_lagrange, dtype=np.uint64).reshape(self.n, 12)
        self._ctx = {}

    @classmethod
    def unsafe_setup(cls, k, tau):
        """params.rs:79-129 with a given tau (Montgomery Fr)."""
        n = 1 << k
        g = np.zeros((n, 12), dtype=np.uint64)
        gl = np.zeros((n, 12), dtype=np.uint64)
        check(lib().gb_kzg_setup(_ptr(g), _ptr(gl), _fr(tau), k))
        return cls(k, g, gl)

    @classmethod
    def read_raw_bytes(cls, data):
        """params.rs:188-260 SerdeFormat::RawBytes: u32 k, 2^k g, 2^k
        g_lagrange (96-byte uncompressed each), then the G2 elements."""
        k = struct.unpack("<I", data[:4])[0]
        n = 1 << k
        pts = [from_uncompressed(data[4 + 96 * i:4 + 96 * (i + 1)]) for i in range(2 * n)]
        return cls(k, np.array(pts[:n]), np.array(pts[n:]))

    def downsize(self, new_k):
        """params.rs:60-77: truncate g, recompute g_lagrange = iFFT(g)/n."""
        if new_k == self.k:
            return self
        n = 1 << new_k
        g = self.g[:n].copy()
        gl = g_to_lagrange(g, new_k)
        return ParamsKZG(new_k, g, gl)

    def device_bytes(self):
        """device memory held by this SRS's resident MSM contexts (their
        precomputed tables)"""
        return sum(c.device_bytes() for c in self._ctx.values())

    def context(self, lagrange):
        key = bool(lagrange)
        if key not in self._ctx:
            self._ctx[key] = Bls12_381G1MsmContext(self.g_lagrange if lagrange else self.g)
        return self._ctx[key]

    # KZGCommitmentScheme (poly/kzg/mod.rs:1072-1430)
    def commit(self, poly):
        return self.commit_batch([poly])[0]

    def commit_lagrange(self, evals):
        return self.commit_lagrange_batch([evals])[0]

    def commit_batch(self, polys):
        return self._commit(polys, lagrange=False)

    def commit_lagrange_batch(self, polys):
        return self._commit(polys, lagrange=True)

    def _commit(self, polys, lagrange):
        polys = [np.ascontiguousarray(p, dtype=np.uint64).reshape(-1, 4) for p in polys]
        if not polys:
            return []
        ctx = self.context(lagrange)
        out = []
        # same-length polynomials go through one batch call
        by_len = {}
        for i, p in enumerate(polys):
            if len(p) > self.n:
                raise MsmError(-1, "polynomial longer than the SRS")
            by_len.setdefault(len(p), []).append(i)
        res = [None] * len(polys)
        for ln, idxs in by_len.items():
            batch = np.stack([polys[i] for i in idxs])
            r = ctx.batch(batch, npoints=ln)
            for j, i in enumerate(idxs):
                res[i] = r[j]
        return res


def g_to_lagrange(g, k):
    g = np.ascontiguousarray(g, dtype=np.uint64).reshape(1 << k, 12)
    out = np.zeros_like(g)
    check(lib().gb_g1_to_lagrange(_ptr(out), _ptr(g), k))
    return out


# ---------------------------------------------------------------- transcript

class CircuitTranscript:
    """Blake2b-512 keyed with "Domain separator for transcript"; absorb =
    0x01 || bytes, squeeze = 0x00 then the running digest mapped to Fr by
    from_uniform_bytes; points are written compressed, scalars as 32-byte
    little-endian canonical values (transcript/implementors.rs:13-33,140-170)."""

    KEY = b"Domain separator for transcript"

    def __init__(self, proof=b""):
        self.state = hashlib.blake2b(digest_size=64, key=self.KEY)
        self.buffer = bytearray()
        self.read_buf = memoryview(bytes(proof))
        self.pos = 0

    def _absorb(self, b):
        self.state.update(b"\x01")
        self.state.update(b)

    def common_point(self, affine):
        self._absorb(compress(affine))

    def common_scalar(self, fr):
        self._absorb(fr_to_repr(fr))

    def write_point(self, affine):
        b = compress(affine)
        self._absorb(b)
        self.buffer += b

    def write_scalar(self, fr):
        b = fr_to_repr(fr)
        self._absorb(b)
        self.buffer += b

    def write_scalar_int(self, v):
        """write_scalar of the field element with canonical value v mod r"""
        b = (v % R_MOD).to_bytes(32, "little")
        self._absorb(b)
        self.buffer += b

    def squeeze_challenge(self):
        self.state.update(b"\x00")
        return fr_from_uniform_bytes(self.state.digest())

    def finalize(self):
        return bytes(self.buffer)
