"""The allocation-free shifted prefix product, called through the C ABI.

Some callers cannot allocate device memory when they need a grand product
(for example a server that reserved its whole HBM budget up front, or a
prover lane that must not stall other lanes with cudaMalloc/cudaFree).
gb_fr_shifted_prefix_product_noalloc serves them: it works in place on the
caller's device buffer and keeps its temporaries in a fixed 64 KiB device
array.  This test checks it against the allocating entry point
midnight_sppark_bls12_381_fr_shifted_prefix_product, bit for bit, on two
calls in a row (the second reuses the scratch the first left behind), plus
its size limit.  The file sorts last so a stop-at-first-failure run has
already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_LEN = 1 << 22


def _noalloc(gb, d_tensor, initial, length, stream):
    f = gb.lib().gb_fr_shifted_prefix_product_noalloc
    return f(ctypes.c_void_p(d_tensor.data_ptr()), gb.api._fr(initial), length, ctypes.c_void_p(stream))


def _cudart():
    """The CUDA runtime that libgbprover.so loaded (found in this process's maps)."""
    for line in open("/proc/self/maps"):
        path = line.split()[-1]
        if "libcudart.so" in path:
            return ctypes.CDLL(path)
    pytest.skip("libcudart not mapped")


def _pool_bytes(rt, device):
    """(used, reserved) bytes of the device's default memory pool, the pool
    the library's stream-ordered allocations come from"""
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), device) == 0
    out = []
    for attr in (0x7, 0x5):  # cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrReservedMemCurrent
        v = ctypes.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, attr, ctypes.byref(v)) == 0
        out.append(v.value)
    return tuple(out)


def test_noalloc_matches_allocating_entry_point_twice(gb, orc):
    import torch

    torch.cuda.set_device(0)
    rng = np.random.default_rng(2222)
    stream = torch.cuda.current_stream().cuda_stream
    for length in (MAX_LEN, 100003):
        values = orc.fr_random(length, rng)
        initial = orc.fr_random(1, rng)[0]
        want = gb.bls12_381_fr_shifted_prefix_product(values, initial)
        dev = torch.from_numpy(values.view(np.int64).copy()).cuda()
        torch.cuda.synchronize()
        gb.api.check(_noalloc(gb, dev, initial, length, stream))
        torch.cuda.synchronize()
        got = dev.cpu().numpy().view(np.uint64).reshape(-1, 4)
        assert (got == want).all(), length


def test_noalloc_rejects_oversize_and_host_memory(gb, orc):
    import torch

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    one = orc.fr_const(orc.CONST_ONE)
    dev = torch.zeros(8, dtype=torch.int64, device="cuda")
    err = _noalloc(gb, dev, one, MAX_LEN + 1, stream)
    assert err.code == 1
    with pytest.raises(gb.MsmError, match="maximum"):
        gb.api.check(err)
    host = torch.zeros(8, dtype=torch.int64)
    err = _noalloc(gb, host, one, 2, stream)
    assert err.code == 1
    with pytest.raises(gb.MsmError, match="device memory"):
        gb.api.check(err)


def test_noalloc_allocates_nothing(gb, orc):
    """After a first call (which looks up the scratch array's address), a call
    changes neither the device pool the library allocates from nor torch's
    allocator: nothing is allocated or freed."""
    import torch

    torch.cuda.set_device(0)
    rng = np.random.default_rng(2223)
    stream = torch.cuda.current_stream().cuda_stream
    length = 1 << 20
    values = orc.fr_random(length, rng)
    initial = orc.fr_random(1, rng)[0]
    want = gb.bls12_381_fr_shifted_prefix_product(values, initial)
    dev = torch.from_numpy(values.view(np.int64).copy()).cuda()
    warm = dev.clone()
    gb.api.check(_noalloc(gb, warm, initial, length, stream))
    torch.cuda.synchronize()
    rt = _cudart()
    before = _pool_bytes(rt, 0)
    torch_before = torch.cuda.memory_allocated()
    gb.api.check(_noalloc(gb, dev, initial, length, stream))
    torch.cuda.synchronize()
    assert _pool_bytes(rt, 0) == before
    assert torch.cuda.memory_allocated() == torch_before
    got = dev.cpu().numpy().view(np.uint64).reshape(-1, 4)
    assert (got == want).all()
