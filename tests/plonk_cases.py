"""Seeded synthetic circuits for the prover tests, shared by the CPU and GPU
suites: (k, advice columns, gate degree, lookups)."""
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "midnight-ledger-cuda_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from gb_prover import plonk  # noqa: E402

TAU = 0x5EED_0F_7A0  # the trapdoor of the seeded test SRS

SHAPES = [(7, 3, 3, 0), (8, 3, 3, 1), (8, 5, 3, 1), (8, 4, 5, 2), (9, 8, 4, 2), (8, 3, 4, 0), (7, 2, 2, 0)]


def circuit(k, m, d, L, copies=None, table_log=None, label=None):
    return plonk.SyntheticCircuit(k, advice=m, degree=d, lookups=L,
                                  copies=copies if copies is not None else 1 << (k - 3),
                                  table_log=table_log if table_log is not None else k - 3,
                                  label=label or "circuit-%d-%d-%d-%d" % (k, m, d, L))


def config3_circuit():
    """k = 16, 3 advice columns, the standard gate, 2^14 copy constraints,
    one 2-column lookup into a 2^12-row table."""
    return plonk.SyntheticCircuit(16, advice=3, degree=3, lookups=1, copies=1 << 14, table_log=12,
                                  label="full synthetic PLONK/KZG proof, k=16")
