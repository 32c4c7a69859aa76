"""Generate the committed golden fixtures from the reference tree.

Reads the reference's real k=14 SRS file
(transient-crypto/static/bls_midnight_2p14, format of
vendor/midnight-proofs-0.8.1/src/poly/kzg/params.rs:170-260 RawBytes:
u32-LE k, 2^k G1 `g` points, 2^k G1 `g_lagrange` points, each in the
96-byte zcash uncompressed encoding, then g2 and s_g2) and re-encodes the
G1 points in the 48-byte zcash compressed encoding to halve the size:

  srs_2p14_g1.bin : b"GBSRS1\\0\\0", u32-LE k, 2^k compressed g,
                    2^k compressed g_lagrange
  srs_2p14_g1.sha256 : sha256 of the source file and of srs_2p14_g1.bin

Run where the reference tree is checked out, giving its root:
    python tests/golden/make_fixtures.py <reference-root>
"""
import hashlib
import os
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402


def main(ref_root):
    src = os.path.join(ref_root, "transient-crypto", "static", "bls_midnight_2p14")
    data = open(src, "rb").read()
    k = struct.unpack("<I", data[:4])[0]
    n = 1 << k
    off = 4
    out = bytearray(b"GBSRS1\0\0" + struct.pack("<I", k))
    for _ in range(2 * n):
        aff = orc.g1_from_uncompressed(data[off:off + 96])
        off += 96
        out += orc.g1_compress(aff)
    assert off + 2 * 192 == len(data), "unexpected SRS trailer length"
    dst = os.path.join(HERE, "srs_2p14_g1.bin")
    open(dst, "wb").write(bytes(out))
    with open(os.path.join(HERE, "srs_2p14_g1.sha256"), "w") as f:
        f.write("%s  bls_midnight_2p14\n" % hashlib.sha256(data).hexdigest())
        f.write("%s  srs_2p14_g1.bin\n" % hashlib.sha256(bytes(out)).hexdigest())
    print("wrote", dst, len(out), "bytes, k =", k)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py <reference-root>")
    main(sys.argv[1])
