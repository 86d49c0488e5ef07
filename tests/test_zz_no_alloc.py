"""The allocation-free dot product, gb_ddotv_noalloc_dev, through the C ABI.

It exists for callers that must not call cudaMalloc/cudaFree (those calls can
synchronize the device, and some host applications own all device memory
themselves); its partial sums live in a fixed file-scope device array instead
of the library's pool.  Two calls in a row must match the allocating entry
point, gb_ddotv_dev, within the dot-product tolerance used by the other tests
-- the second call also shows that the previous call's leftovers in the shared
array do not leak into the result.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import _lib

pytestmark = pytest.mark.gpu


def _dot_tol(x, y):
    n = x.numel()
    return 2 * n * np.finfo(np.float64).eps * float((x.double() * y.double()).abs().sum())


def test_noalloc_dotv_matches_allocating_entry_point_twice(gblib):
    """Both entry points partition the vectors the same way (the SM count of the current
    device) and reduce the partial sums in the same order, so their results are the same
    bits; the torch sum is a third opinion within the dot-product tolerance."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    L.gb_ddotv_noalloc_dev.restype = C.c_int
    L.gb_ddotv_noalloc_dev.argtypes = [C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                       C.c_void_p, C.c_void_p]
    torch.cuda.set_device(0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream or 1)
    g = torch.Generator(device="cpu").manual_seed(11)
    # different partitions, a strided one, a zero increment (every element is x[0], y[0]), and
    # an empty product (rho = 0, whatever the shared array holds from the calls before)
    cases = [(1_000_003, 1), (300_001, 2), (5_000, 0), (0, 1)]
    for n, inc in cases:
        size = max(1, n * inc)
        x = (torch.rand(size, generator=g, dtype=torch.float64) * 2 - 1).cuda()
        y = (torch.rand(size, generator=g, dtype=torch.float64) * 2 - 1).cuda()
        rho_new = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        rho_old = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        rc = L.gb_ddotv_noalloc_dev(n, x.data_ptr(), inc, y.data_ptr(), inc, rho_new.data_ptr(), stream)
        assert rc == 0, _lib.last_error()
        rc = L.gb_ddotv_dev(n, x.data_ptr(), inc, y.data_ptr(), inc, rho_old.data_ptr(), stream)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        a, b = float(rho_new.item()), float(rho_old.item())
        if n == 0:
            assert a == 0.0 and b == 0.0
            continue
        assert np.float64(a).tobytes() == np.float64(b).tobytes(), (n, inc, a, b)
        xs = x[0].expand(n) if inc == 0 else x[::inc][:n]
        ys = y[0].expand(n) if inc == 0 else y[::inc][:n]
        tol = _dot_tol(xs, ys)
        ref = float((xs * ys).sum())
        assert abs(a - ref) <= tol
