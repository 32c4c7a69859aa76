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
