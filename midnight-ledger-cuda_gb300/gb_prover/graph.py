"""Compiled gate graphs for the numerator entry points.

`Graph` packs the flattened GraphEvaluator form (evaluation.rs:47-241,
lib.rs:38-79) -- constants, rotations, calculations and Horner parts -- into
the ctypes RawGraph struct of include/gb_prover.h, keeping the arrays alive.
"""
import ctypes

import numpy as np

# ValueSource kinds (include/gb_prover.h)
CONSTANT, INTERMEDIATE, FIXED, ADVICE, INSTANCE, CHALLENGE, BETA, GAMMA, THETA, TRASH, Y, PREVIOUS = range(12)
# Calculation ops
ADD, SUB, MUL, SQUARE, DOUBLE, NEGATE, HORNER, STORE = range(8)


class RawValueSource(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("a", ctypes.c_uint32), ("b", ctypes.c_uint32)]


class RawCalculation(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint32), ("target", ctypes.c_uint32), ("parts_offset", ctypes.c_uint32),
                ("parts_len", ctypes.c_uint32), ("lhs", RawValueSource), ("rhs", RawValueSource)]


class RawGraph(ctypes.Structure):
    _fields_ = [("constants", ctypes.c_void_p), ("constants_len", ctypes.c_size_t),
                ("rotations", ctypes.c_void_p), ("rotations_len", ctypes.c_size_t),
                ("calculations", ctypes.c_void_p), ("calculations_len", ctypes.c_size_t),
                ("horner_parts", ctypes.c_void_p), ("horner_parts_len", ctypes.c_size_t),
                ("num_intermediates", ctypes.c_uint32)]


class RawColumnRef(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("index", ctypes.c_uint32)]


class Graph:
    """constants: (k, 4) Montgomery Fr; rotations: ints; calcs: list of
    (op, target, parts_offset, parts_len, (kind, a, b), (kind, a, b));
    parts: list of (kind, a, b)."""

    def __init__(self, constants, rotations, calcs, parts, num_intermediates):
        self.constants = np.ascontiguousarray(np.asarray(constants, dtype=np.uint64).reshape(-1, 4))
        self.rotations = np.ascontiguousarray(np.asarray(rotations, dtype=np.int32))
        self.calcs = (RawCalculation * max(len(calcs), 1))()
        for i, (op, tgt, po, pl, lhs, rhs) in enumerate(calcs):
            self.calcs[i] = RawCalculation(op, tgt, po, pl, RawValueSource(*lhs), RawValueSource(*rhs))
        self.parts = (RawValueSource * max(len(parts), 1))()
        for i, pt in enumerate(parts):
            self.parts[i] = RawValueSource(*pt)
        self.ncalcs, self.nparts = len(calcs), len(parts)
        self.num_intermediates = num_intermediates

    def raw(self):
        def ptr(a):
            return a.ctypes.data_as(ctypes.c_void_p) if a.size else None
        return RawGraph(ptr(self.constants), len(self.constants), ptr(self.rotations), len(self.rotations),
                        ctypes.cast(self.calcs, ctypes.c_void_p), self.ncalcs,
                        ctypes.cast(self.parts, ctypes.c_void_p), self.nparts, self.num_intermediates)


def column_refs(refs):
    arr = (RawColumnRef * max(len(refs), 1))()
    for i, (k, idx) in enumerate(refs):
        arr[i] = RawColumnRef(k, idx)
    return arr


def graph_array(graphs):
    arr = (RawGraph * max(len(graphs), 1))()
    for i, g in enumerate(graphs):
        arr[i] = g.raw()
    return arr
