"""The small/skinny (gemmsup) engine and the config-explicit GEMM entry point
against the CPU oracle; split-K partial sums fold in a fixed order, so every
config is deterministic run to run."""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import _lib
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _cfg(L, dtype, config, ta, tb, alpha, a, b, beta, c):
    torch = pytest.importorskip("torch")
    m, n = c.shape
    k = a.shape[0] if ta else a.shape[1]
    tdt = torch.float64 if dtype == 0 else torch.float32
    A = torch.from_numpy(np.asfortranarray(a).T.copy()).cuda().t()
    B = torch.from_numpy(np.asfortranarray(b).T.copy()).cuda().t()
    Cd = torch.from_numpy(np.asfortranarray(c).T.copy()).cuda().t()
    assert A.dtype == tdt
    L.gb_gemm_config_dev.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int64,
                                     C.c_double, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int64,
                                     C.c_int64, C.c_double, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
    rc = L.gb_gemm_config_dev(dtype, config, 8 if ta else 0, 8 if tb else 0, m, n, k, alpha, A.data_ptr(),
                              A.stride(0), A.stride(1), B.data_ptr(), B.stride(0), B.stride(1), beta,
                              Cd.data_ptr(), Cd.stride(0), Cd.stride(1), None)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return Cd.cpu().numpy()


@pytest.mark.parametrize("config", range(6))
@pytest.mark.parametrize("dtype", [0, 1])
@pytest.mark.parametrize("m,n,k", [(6, 800, 800), (300, 5, 1000), (129, 65, 4000), (64, 64, 16), (1, 1, 3)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, True)])
def test_config_engines_vs_oracle(gblib, config, dtype, m, n, k, ta, tb):
    dt = np.float64 if dtype == 0 else np.float32
    a = H.normalize(po.uniform((k, m) if ta else (m, k), 1, dtype=dt)).astype(dt)
    b = H.normalize(po.uniform((n, k) if tb else (k, n), 2, dtype=dt)).astype(dt)
    c0 = H.normalize(po.uniform((m, n), 3, dtype=dt)).astype(dt)
    got = _cfg(gblib, dtype, config, ta, tb, 2.0, a, b, 1.2, c0)
    r = H.gemm_residual(2.0, H.op(a, 8 if ta else 0).astype(np.float64), H.op(b, 8 if tb else 0).astype(np.float64),
                        1.2, c0.astype(np.float64), got.astype(np.float64))
    assert r < (1e-14 if dtype == 0 else 1e-5)


@pytest.mark.parametrize("config", [3, 5])
def test_split_k_deterministic_and_beta0_nan(gblib, config):
    m, n, k = 200, 90, 3000
    a = po.uniform((m, k), 4)
    b = po.uniform((k, n), 5)
    c = np.full((m, n), np.nan, order="F")
    r1 = _cfg(gblib, 0, config, False, False, 1.0, a, b, 0.0, c)
    r2 = _cfg(gblib, 0, config, False, False, 1.0, a, b, 0.0, c)
    assert np.isfinite(r1).all()
    assert np.array_equal(r1, r2)
    hi, lo = po.dd_gemm_full(0, 0, 1.0, a, b, 0.0, np.zeros((m, n), order="F"))
    assert np.all(np.abs(r1 - hi - lo) <= 2 * k * H.EPS * (np.abs(a) @ np.abs(b)))


def test_config_rejects_unknown(gblib):
    torch = pytest.importorskip("torch")
    x = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
    L = gblib
    rc = L.gb_gemm_config_dev(0, 99, 0, 0, 4, 4, 4, 1.0, x.data_ptr(), 1, 4, x.data_ptr(), 1, 4, 0.0,
                              x.data_ptr(), 1, 4, None)
    assert rc != 0
    L.gb_clear_last_error()
