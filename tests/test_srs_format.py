"""The SRS RawBytes file format (params.rs:188-260) parsed by the host
mirror, on the real k=14 fixture re-encoded uncompressed by the oracle."""
import struct

import numpy as np


def test_read_raw_bytes_round_trip(orc, srs):
    from gb_prover.kzg import ParamsKZG, compress
    k, g, gl = srs
    n = 1 << k
    sel = slice(0, 1 << 6)  # a 2^6 prefix keeps the CPU test fast
    kk = 6
    blob = struct.pack("<I", kk) + b"".join(orc.g1_to_uncompressed(p) for p in g[sel]) + \
        b"".join(orc.g1_to_uncompressed(p) for p in gl[sel]) + bytes(384)
    params = ParamsKZG.read_raw_bytes(blob)
    assert params.k == kk and (params.g == g[sel]).all() and (params.g_lagrange == gl[sel]).all()
    assert compress(g[0]) == orc.g1_compress(g[0])
    assert n == 16384
