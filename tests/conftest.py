import os
import struct
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "midnight-ledger-cuda_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device and the built libgbprover.so")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gb():
    import gb_prover
    gb_prover.lib(build_if_stale=True)
    return gb_prover


_SRS_CACHE = {}


def load_srs():
    """The reference's real k=14 SRS (g and g_lagrange) from the committed
    compressed fixture, decoded by the oracle: (k, g[2^k,12], g_lagrange[2^k,12])."""
    if "srs" in _SRS_CACHE:
        return _SRS_CACHE["srs"]
    from oracle import oracle
    data = open(os.path.join(GOLDEN, "srs_2p14_g1.bin"), "rb").read()
    assert data[:8] == b"GBSRS1\0\0"
    k = struct.unpack("<I", data[8:12])[0]
    n = 1 << k
    pts = np.zeros((2 * n, 12), dtype=np.uint64)
    off = 12
    for i in range(2 * n):
        pts[i] = oracle.g1_decompress(data[off:off + 48])
        off += 48
    _SRS_CACHE["srs"] = (k, pts[:n].copy(), pts[n:].copy())
    return _SRS_CACHE["srs"]


@pytest.fixture(scope="session")
def srs():
    return load_srs()


def affine_of(orc, jac):
    """Jacobian (18 u64) -> affine (12 u64), via the oracle."""
    return orc.g1_to_affine(np.asarray(jac, dtype=np.uint64).reshape(-1, 18))
