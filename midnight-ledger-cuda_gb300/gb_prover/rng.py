"""Seeded randomness for the prover's blinding values and synthetic circuits.

`ChaCha20Rng` restates rand_chacha's ChaCha20Rng (rand_chacha 0.3.1, the
`ChaCha20Rng` of vendor/midnight-proofs-0.8.1/src/plonk/vanishing/prover.rs:41-75
and the `StdRng` family): the 20-round ChaCha block function of RFC 8439
with a 64-bit block counter in words 12-13 and a 64-bit stream id (0) in
words 14-15, output words consumed in order, `next_u64` = low word | high
word << 32.  `seed_from_u64` is rand_core 0.6's PCG32 seed expansion.

`fr_random` is `Fq::random` (vendor/midnight-curves-0.3.1/src/bls12_381/fq.rs:373-387):
four u64 draws, the top bit masked, rejected when >= r, stored in
Montgomery form.
"""
import hashlib

import numpy as np

R_MOD = 0x73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001
_MASK64 = (1 << 64) - 1
_SIGMA = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)


def _rotl(x, n):
    return (x << np.uint32(n)) | (x >> np.uint32(32 - n))


def _chacha_blocks(key_words, counter0, nblocks, stream=0):
    """nblocks consecutive 64-byte ChaCha20 blocks as an (nblocks, 16) u32 array."""
    ctr = np.arange(counter0, counter0 + nblocks, dtype=np.uint64)
    st = np.empty((16, nblocks), dtype=np.uint32)
    st[0:4] = _SIGMA[:, None]
    st[4:12] = np.asarray(key_words, dtype=np.uint32)[:, None]
    st[12] = (ctr & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    st[13] = (ctr >> np.uint64(32)).astype(np.uint32)
    st[14] = np.uint32(stream & 0xFFFFFFFF)
    st[15] = np.uint32(stream >> 32)
    x = [st[i].copy() for i in range(16)]

    def qr(a, b, c, d):
        x[a] += x[b]; x[d] ^= x[a]; x[d] = _rotl(x[d], 16)
        x[c] += x[d]; x[b] ^= x[c]; x[b] = _rotl(x[b], 12)
        x[a] += x[b]; x[d] ^= x[a]; x[d] = _rotl(x[d], 8)
        x[c] += x[d]; x[b] ^= x[c]; x[b] = _rotl(x[b], 7)

    with np.errstate(over="ignore"):
        for _ in range(10):
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
        out = np.stack([x[i] + st[i] for i in range(16)], axis=1)
    return out


def _chacha_block_int(key_words, counter, stream=0):
    """One block with Python integers: far cheaper than the array form for
    the few blocks a proof's host-side draws need."""
    M = 0xFFFFFFFF
    st = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574] + [int(k) for k in key_words] + [
        counter & M, (counter >> 32) & M, stream & M, (stream >> 32) & M]
    x = list(st)
    for _ in range(10):
        for a, b, c, d in ((0, 4, 8, 12), (1, 5, 9, 13), (2, 6, 10, 14), (3, 7, 11, 15),
                           (0, 5, 10, 15), (1, 6, 11, 12), (2, 7, 8, 13), (3, 4, 9, 14)):
            xa, xb, xc, xd = x[a], x[b], x[c], x[d]
            xa = (xa + xb) & M; xd ^= xa; xd = ((xd << 16) | (xd >> 16)) & M
            xc = (xc + xd) & M; xb ^= xc; xb = ((xb << 12) | (xb >> 20)) & M
            xa = (xa + xb) & M; xd ^= xa; xd = ((xd << 8) | (xd >> 24)) & M
            xc = (xc + xd) & M; xb ^= xc; xb = ((xb << 7) | (xb >> 25)) & M
            x[a], x[b], x[c], x[d] = xa, xb, xc, xd
    return np.array([(x[i] + st[i]) & M for i in range(16)], dtype=np.uint32)


def _native_lib():
    """The CUDA library once this process has loaded it (its host-side
    gb_chacha20_blocks computes blocks in C), else None: the oracle-only
    paths keep the restatements above."""
    from . import _lib
    return _lib._lib


def _native_blocks(L, key_words, counter0, nblocks):
    import ctypes
    from ._lib import check
    key = np.ascontiguousarray(key_words, dtype=np.uint32)
    out = np.empty(16 * nblocks, dtype=np.uint32)
    check(L.gb_chacha20_blocks(key.ctypes.data_as(ctypes.c_void_p), counter0, 0, nblocks,
                               out.ctypes.data_as(ctypes.c_void_p)))
    return out


class ChaCha20Rng:
    def __init__(self, seed: bytes):
        if len(seed) != 32:
            raise ValueError("ChaCha20Rng seed must be 32 bytes")
        self._key = np.frombuffer(seed, dtype="<u4").astype(np.uint32)
        self._block = 0
        self._buf = np.zeros(0, dtype=np.uint32)
        self._pos = 0

    @classmethod
    def seed_from_u64(cls, state: int):
        """rand_core SeedableRng::seed_from_u64: PCG32 fills the 32-byte seed."""
        mul, inc = 6364136223846793005, 11634580027462260723
        out = bytearray()
        state &= _MASK64
        for _ in range(8):
            state = (state * mul + inc) & _MASK64
            xorshifted = (((state >> 18) ^ state) >> 27) & 0xFFFFFFFF
            rot = state >> 59
            v = ((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & 0xFFFFFFFF
            out += v.to_bytes(4, "little")
        return cls(bytes(out))

    @classmethod
    def from_label(cls, label: str):
        """Seed = SHA-256 of a workload label."""
        return cls(hashlib.sha256(label.encode()).digest())

    def _words(self, count):
        """The next `count` keystream words, in order."""
        have = len(self._buf) - self._pos
        if have < count:
            need = count - have
            nblocks = (need + 15) // 16
            L = _native_lib()
            if L is not None:
                nblocks = max(nblocks, 16)
                fresh = _native_blocks(L, self._key, self._block, nblocks)
            elif nblocks <= 4:
                # a few words (blinding values): scalar blocks
                fresh = np.concatenate([_chacha_block_int(self._key, self._block + b) for b in range(nblocks)])
            else:
                nblocks = max(nblocks, 256)
                fresh = _chacha_blocks(self._key, self._block, nblocks).reshape(-1)
            self._block += nblocks
            self._buf = np.concatenate([self._buf[self._pos:], fresh])
            self._pos = 0
        w = self._buf[self._pos:self._pos + count]
        self._pos += count
        return w

    @property
    def seed(self):
        return self._key.astype("<u4").tobytes()

    def word_position(self):
        """absolute index of the next keystream word"""
        return self._block * 16 - (len(self._buf) - self._pos)

    def skip_words(self, count):
        """advance the stream by `count` words"""
        have = len(self._buf) - self._pos
        if count <= have:
            self._pos += count
            return
        target = self.word_position() + count
        self._block = target // 16
        self._buf = np.zeros(0, dtype=np.uint32)
        self._pos = 0
        if target % 16:
            self._words(16)  # refill with the block holding the target
            self._pos = target % 16

    def next_u32(self):
        return int(self._words(1)[0])

    def next_u64_array(self, count):
        w = self._words(2 * count).astype(np.uint64).reshape(-1, 2)
        return w[:, 0] | (w[:, 1] << np.uint64(32))

    def next_u64(self):
        return int(self.next_u64_array(1)[0])

    def fill_bytes(self, n):
        nw = (n + 3) // 4
        return self._words(nw).astype("<u4").tobytes()[:n]


_R2 = pow(2, 512, R_MOD)


def ints_to_mont(vals):
    """canonical integers -> (n, 4) u64 Montgomery limbs (R = 2^256)"""
    b = b"".join(((int(v) << 256) % R_MOD).to_bytes(32, "little") for v in vals)
    return np.frombuffer(bytearray(b), dtype="<u8").reshape(-1, 4)


_RINV = pow(1 << 256, -1, R_MOD)


def _row_ints(arr):
    """(n, 4) u64 limb rows -> their integer values"""
    b = np.ascontiguousarray(arr, dtype="<u8").reshape(-1, 4).tobytes()
    frm = int.from_bytes
    return [frm(b[i:i + 32], "little") for i in range(0, len(b), 32)]


def mont_to_ints(arr):
    """(n, 4) u64 Montgomery limbs -> canonical integers"""
    rinv = _RINV
    return [v * rinv % R_MOD for v in _row_ints(arr)]


def raw_to_mont(raw):
    """canonical limb rows (< r) -> Montgomery rows"""
    return ints_to_mont(_row_ints(raw))


def fr_random(rng: ChaCha20Rng, n):
    """n field elements by Fq::random's rejection rule, Montgomery form (n, 4)."""
    return ints_to_mont(_fr_random_ints(rng, n))


# R^2 mod r as limbs: a Montgomery product with it maps a canonical value
# to its Montgomery form
R2_LIMBS = np.array([(_R2 >> (64 * i)) & _MASK64 for i in range(4)], dtype=np.uint64)


_TOP_MASK = (1 << 255) - 1


def _fr_random_ints(rng: ChaCha20Rng, n):
    """The canonical values of n draws of fr_random: each candidate is four
    next_u64 words (eight keystream words, one little-endian 256-bit value)
    with bit 255 cleared, kept when below r."""
    got = []
    frm = int.from_bytes
    while len(got) < n:
        want = n - len(got)
        draw = want + want // 8 + 8
        b = np.ascontiguousarray(rng._words(8 * draw), dtype="<u4").tobytes()
        used = draw
        for i in range(draw):
            v = frm(b[32 * i:32 * i + 32], "little") & _TOP_MASK
            if v < R_MOD:
                got.append(v)
                if len(got) == n:
                    used = i + 1
                    break
        # the draws after the last one taken go back, so the stream matches
        # one-at-a-time sampling
        rng._pos -= (draw - used) * 8
    return got


def fr_random_raw(rng: ChaCha20Rng, n):
    """The draws of fr_random as canonical limb rows (n, 4), before the
    Montgomery conversion."""
    b = b"".join(v.to_bytes(32, "little") for v in _fr_random_ints(rng, n))
    return np.frombuffer(bytearray(b), dtype="<u8").reshape(-1, 4)
