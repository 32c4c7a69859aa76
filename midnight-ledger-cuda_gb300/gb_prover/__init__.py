"""Host-side mirror of the reference's Rust wrappers over the prover FFI.

The reference's safe wrappers live in midnight-sppark-msm/src/lib.rs:1470-4555
(`bls12_381_g1_msm`, `Bls12_381G1MsmContext`, `Bls12_381FrDeviceVec`,
`bls12_381_fr_ntt`, the product and quotient helpers).  This package exposes
the same operations with the same names, argument meaning and error
behaviour over ctypes, calling libgbprover.so through the C ABI declared in
include/gb_prover.h.  Arrays are numpy uint64 in the reference's memory
layout: Fr (n, 4), G1 affine (n, 12), G1 projective (n, 18), Montgomery form.

There is no CPU fallback: importing works anywhere, but every call raises
`MsmError` if the CUDA library cannot be loaded or reports an error.
"""
from ._lib import (  # noqa: F401
    MsmError,
    RawMsmConfig,
    RawMsmSlice,
    lib,
    library_path,
    build,
)
from .api import *  # noqa: F401,F403
