"""csem_cdot_dev_noalloc against csem_cdot_dev, through the C ABI.

The allocation-free variant keeps its partial sums in a fixed array in the library's
device image. It must give the same bits as the allocating entry point, twice in a row
(the second call reuses the array the first one wrote), leave device free memory
unchanged across those calls, and refuse batches larger than its fixed scratch.
"""
import ctypes as C

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs

pytestmark = pytest.mark.gpu

_ARGS = [C.c_int, C.c_long, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]


def _bind(name):
    f = getattr(cs.lib(), name)
    f.restype = C.c_int
    f.argtypes = _ARGS
    return f


@pytest.mark.parametrize("prec", [64, 32])
def test_noalloc_dot_equals_allocating_dot(gpu, prec):
    import torch
    noalloc, alloc = _bind("csem_cdot_dev_noalloc"), _bind("csem_cdot_dev")
    dt = torch.complex128 if prec == 64 else torch.complex64
    gen = torch.Generator(device="cuda").manual_seed(11 + prec)
    for n, nsys in ((1, 1), (1000, 3), (300001, 5), (2_100_000, 64)):  # the last one uses all 1024 blocks
        a = torch.randn(nsys, n, dtype=dt, device="cuda", generator=gen)
        b = torch.randn(nsys, n, dtype=dt, device="cuda", generator=gen)
        ref, out1, out2 = (torch.full((nsys, 2), float("nan"), dtype=torch.float64, device="cuda") for _ in range(3))
        torch.cuda.synchronize()
        assert alloc(prec, n, nsys, a.data_ptr(), b.data_ptr(), ref.data_ptr(), None) == 0
        assert noalloc(prec, n, nsys, a.data_ptr(), b.data_ptr(), out1.data_ptr(), None) == 0  # first use
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        assert noalloc(prec, n, nsys, a.data_ptr(), b.data_ptr(), out1.data_ptr(), None) == 0
        assert noalloc(prec, n, nsys, a.data_ptr(), b.data_ptr(), out2.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert torch.equal(out1, ref) and torch.equal(out2, ref), (n, nsys)
        exact = (a.to(torch.complex128) * b.to(torch.complex128).conj()).sum(dim=1)
        got = torch.complex(ref[:, 0], ref[:, 1])
        scale = (a.abs().double() * b.abs().double()).sum(dim=1)
        assert bool(((got - exact).abs() <= 1e-12 * scale + 1e-300).all())


def test_noalloc_dot_rejects_oversized_batch(gpu):
    import torch
    noalloc = _bind("csem_cdot_dev_noalloc")
    a = torch.zeros(65, 8, dtype=torch.complex128, device="cuda")
    out = torch.zeros(65, 2, dtype=torch.float64, device="cuda")
    rc = noalloc(64, 8, 65, a.data_ptr(), a.data_ptr(), out.data_ptr(), None)
    assert rc == -7  # CSEM_ETOOBIG
    assert b"64 systems" in cs.lib().csem_last_error()
    assert noalloc(16, 8, 1, a.data_ptr(), a.data_ptr(), out.data_ptr(), None) < 0
