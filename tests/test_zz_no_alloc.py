"""pfs_residual_norms_static: the residual norms for callers that must not
allocate device memory (a host whose device memory is owned entirely by
another allocator, or a latency-critical caller that cannot let cudaMalloc
synchronize the device). Its reduction scratch is a fixed array inside the
library instead of an allocation. Two calls in a row, through the C ABI,
must give what the allocating pfs_residual_norms gives on the same fields.

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

REL = 1e-12  # the tolerance the residual tests use


def _fields(w, h, seed):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    ld = (w + 31) // 32 * 32
    p = torch.randn(h, ld, generator=g).cuda()
    b = torch.randn(h, ld, generator=g).cuda()
    return p, b


def _call(fn, p, b, w):
    lib_fn = fn
    h, ld = p.shape
    rr, bb = C.c_double(), C.c_double()
    st = lib_fn(C.c_void_p(p.data_ptr()), C.c_void_p(b.data_ptr()), w, h, ld, C.byref(rr), C.byref(bb), None)
    return st, rr.value, bb.value


@pytest.mark.gpu
@pytest.mark.parametrize("w,h", [(2048, 2048), (260, 132), (37, 29)])
def test_static_norms_match_allocating_entry_point(cuda_device, pfs_lib, w, h):
    lib = pfs_lib.lib()
    for call in range(2):  # two calls in a row share the library's scratch
        p, b = _fields(w, h, seed=100 * call + w)
        st, rr_s, bb_s = _call(lib.pfs_residual_norms_static, p, b, w)
        assert st == 0, lib.pfs_last_error()
        st, rr_a, bb_a = _call(lib.pfs_residual_norms, p, b, w)
        assert st == 0, lib.pfs_last_error()
        assert rr_s == pytest.approx(rr_a, rel=REL) and bb_s == pytest.approx(bb_a, rel=REL), (call, w, h)
        assert rr_s > 0 and bb_s > 0


@pytest.mark.gpu
def test_static_norms_reject_oversized_grid(cuda_device, pfs_lib):
    lib = pfs_lib.lib()
    p, b = _fields(64, 64, seed=1)
    rr, bb = C.c_double(), C.c_double()
    st = lib.pfs_residual_norms_static(C.c_void_p(p.data_ptr()), C.c_void_p(b.data_ptr()), 65536, 32768, 65536,
                                       C.byref(rr), C.byref(bb), None)
    assert st == 1 and b"exceeds" in lib.pfs_last_error()


@pytest.mark.gpu
def test_static_norms_allocate_no_device_memory(cuda_device, pfs_lib):
    # The entry point's whole contract: no device allocation. Warm up first on
    # other grid sizes (the first launch of each kernel path loads the
    # library's kernels, which the driver may place in device memory), then
    # call it repeatedly at new sizes and compare the device's free memory.
    import torch
    lib = pfs_lib.lib()
    for w, h in ((260, 36), (37, 29)):  # vector-load and scalar kernel paths
        p, b = _fields(w, h, seed=7)
        assert _call(lib.pfs_residual_norms_static, p, b, w)[0] == 0, lib.pfs_last_error()
    fields = [(_fields(w, h, seed=w), w) for w, h in ((1024, 768), (93, 61))]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for (p, b), w in fields:
        for _ in range(3):
            assert _call(lib.pfs_residual_norms_static, p, b, w)[0] == 0, lib.pfs_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
