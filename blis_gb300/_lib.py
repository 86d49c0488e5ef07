"""Loader for libblis_gb300.so with ctypes signatures for every exported entry.

The shared library is the product; this module only binds it.  It raises
immediately when the library is missing: there is no fallback path.
"""
import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libblis_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "blis_gb300.h")

_lib = None

_i32 = C.c_int32
_i64 = C.c_int64
_d = C.c_double
_f = C.c_float
_vp = C.c_void_p
_ip = C.POINTER(C.c_int32)
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_cp = C.c_char_p


class DComplex(C.Structure):
    """gb_dcomplex (BLIS dcomplex): real, imag."""
    _fields_ = [("real", C.c_double), ("imag", C.c_double)]


class SComplex(C.Structure):
    """gb_scomplex (BLIS scomplex): real, imag."""
    _fields_ = [("real", C.c_float), ("imag", C.c_float)]


def _sig(L, name, res, args):
    fn = getattr(L, name)
    fn.restype = res
    fn.argtypes = args


def declared_functions():
    """Names of the functions declared in include/blis_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\**\s+\**([a-z][A-Za-z0-9_]*)\s*\(",
                                 text, flags=re.M)))


def load(path=None):
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libblis_gb300.so is not built (%s); run __graft_entry__.build()" % path)
    L = C.CDLL(path, mode=C.RTLD_GLOBAL)
    gemm_blas = [_cp, _cp, _ip, _ip, _ip, _vp, _vp, _ip, _vp, _ip, _vp, _vp, _ip]
    _sig(L, "dgemm_", None, gemm_blas)
    _sig(L, "sgemm_", None, gemm_blas)
    _sig(L, "dtrsm_", None, [_cp, _cp, _cp, _cp, _ip, _ip, _dp, _vp, _ip, _vp, _ip])
    _sig(L, "dgemv_", None, [_cp, _ip, _ip, _dp, _vp, _ip, _vp, _ip, _dp, _vp, _ip])
    _sig(L, "daxpy_", None, [_ip, _dp, _vp, _ip, _vp, _ip])
    _sig(L, "ddot_", _d, [_ip, _vp, _ip, _vp, _ip])
    batch = [_cp, _cp, _ip, _ip, _ip, _vp, _vp, _ip, _vp, _ip, _vp, _vp, _ip, _ip, _ip]
    _sig(L, "dgemm_batch_", None, batch)
    _sig(L, "sgemm_batch_", None, batch)
    _sig(L, "xerbla_", C.c_int, [_cp, _ip, C.c_long])
    _sig(L, "zgemm_", None, [_cp, _cp, _ip, _ip, _ip, _vp, _vp, _ip, _vp, _ip, _vp, _vp, _ip])
    _sig(L, "cgemm_", None, [_cp, _cp, _ip, _ip, _ip, _vp, _vp, _ip, _vp, _ip, _vp, _vp, _ip])
    cz = [C.c_int, C.c_int, _i64, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64]
    _sig(L, "ztrsm_", None, [_cp, _cp, _cp, _cp, _ip, _ip, _vp, _vp, _ip, _vp, _ip])
    _sig(L, "bli_ztrsm", None, [C.c_int] * 4 + [_i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64])
    _sig(L, "gb_ztrsm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64, _i64,
                                                      _vp])
    _sig(L, "gb_zgemm", None, cz)
    _sig(L, "gb_cgemm", None, cz)
    _sig(L, "gb_dgemm_ozaki", None, [C.c_int, C.c_int, _i64, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64,
                                     _vp, _vp, _i64, _i64, C.c_int])
    _sig(L, "bli_zgemm", None, cz)
    _sig(L, "bli_cgemm", None, cz)
    _sig(L, "gb_zgemm_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64,
                                      _i64, DComplex, _vp, _i64, _i64, _vp])
    _sig(L, "gb_cgemm_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _i64, SComplex, _vp, _i64, _i64, _vp, _i64,
                                      _i64, SComplex, _vp, _i64, _i64, _vp])
    _sig(L, "zherk_", None, [_cp, _cp, _ip, _ip, _vp, _vp, _ip, _vp, _vp, _ip])
    _sig(L, "cherk_", None, [_cp, _cp, _ip, _ip, _vp, _vp, _ip, _vp, _vp, _ip])
    her2k_blas = [_cp, _cp, _ip, _ip, _vp, _vp, _ip, _vp, _ip, _vp, _vp, _ip]
    _sig(L, "zher2k_", None, her2k_blas)
    _sig(L, "cher2k_", None, her2k_blas)
    hemm_blas = [_cp, _cp, _ip, _ip, _vp, _vp, _ip, _vp, _ip, _vp, _vp, _ip]
    for name in ("zhemm_", "chemm_", "zsymm_", "csymm_"):
        _sig(L, name, None, hemm_blas)
    _sig(L, "dsyr2k_", None, [_cp, _cp, _ip, _ip, _dp, _vp, _ip, _vp, _ip, _dp, _vp, _ip])
    herk_t = [C.c_int, C.c_int, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _vp, _i64, _i64]
    _sig(L, "bli_zherk", None, herk_t)
    _sig(L, "bli_cherk", None, herk_t)
    her2k_t = [C.c_int, C.c_int, C.c_int, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64]
    _sig(L, "bli_zher2k", None, her2k_t)
    _sig(L, "bli_cher2k", None, her2k_t)
    _sig(L, "bli_dsyr2k", None, her2k_t)
    hemm_t = [C.c_int] * 4 + [_i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64]
    for name in ("bli_zhemm", "bli_chemm", "bli_zsymm", "bli_csymm"):
        _sig(L, name, None, hemm_t)
    _sig(L, "gb_zherk_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _d, _vp, _i64, _i64, _d, _vp, _i64, _i64, _vp])
    _sig(L, "gb_zher2k_dev", C.c_int, [C.c_int, C.c_int, C.c_int, _i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64,
                                       _i64, _d, _vp, _i64, _i64, _vp])
    zhemm_d = [C.c_int] * 4 + [_i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64, _i64, DComplex, _vp, _i64, _i64,
                               _vp]
    _sig(L, "gb_zhemm_dev", C.c_int, zhemm_d)
    _sig(L, "gb_zsymm_dev", C.c_int, zhemm_d)
    _sig(L, "bli_dtrmm3", None, [C.c_int] * 5 + [_i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64,
                                                  _i64])
    _sig(L, "gb_dtrmm3_dev", C.c_int, [C.c_int] * 5 + [_i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64, _d, _vp,
                                                         _i64, _i64, _vp])
    _sig(L, "gb_dsyr2k_dev", C.c_int, [C.c_int, C.c_int, C.c_int, _i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64,
                                       _d, _vp, _i64, _i64, _vp])
    _sig(L, "dscal_", None, [_ip, _dp, _vp, _ip])
    _sig(L, "dcopy_", None, [_ip, _vp, _ip, _vp, _ip])
    _sig(L, "idamax_", _i32, [_ip, _vp, _ip])
    _sig(L, "dger_", None, [_ip, _ip, _dp, _vp, _ip, _vp, _ip, _vp, _ip])
    _sig(L, "dtrsv_", None, [_cp, _cp, _cp, _ip, _vp, _ip, _vp, _ip])
    _sig(L, "dtrmm_", None, [_cp, _cp, _cp, _cp, _ip, _ip, _dp, _vp, _ip, _vp, _ip])
    _sig(L, "dsymm_", None, [_cp, _cp, _ip, _ip, _dp, _vp, _ip, _vp, _ip, _dp, _vp, _ip])
    _sig(L, "dsyrk_", None, [_cp, _cp, _ip, _ip, _dp, _vp, _ip, _dp, _vp, _ip])
    _sig(L, "dgemmt_", None, [_cp, _cp, _cp, _ip, _ip, _dp, _vp, _ip, _vp, _ip, _dp, _vp, _ip])
    _sig(L, "cblas_dgemm", None, [C.c_int] * 3 + [_i32] * 3 + [_d, _vp, _i32, _vp, _i32, _d, _vp, _i32])
    _sig(L, "cblas_sgemm", None, [C.c_int] * 3 + [_i32] * 3 + [_f, _vp, _i32, _vp, _i32, _f, _vp, _i32])
    _sig(L, "cblas_dtrsm", None, [C.c_int] * 5 + [_i32, _i32, _d, _vp, _i32, _vp, _i32])
    _sig(L, "cblas_dgemv", None, [C.c_int, C.c_int, _i32, _i32, _d, _vp, _i32, _vp, _i32, _d, _vp, _i32])
    _sig(L, "cblas_daxpy", None, [_i32, _d, _vp, _i32, _vp, _i32])
    _sig(L, "cblas_ddot", _d, [_i32, _vp, _i32, _vp, _i32])
    _sig(L, "cblas_dgemm_batch", None, [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                        _vp, _vp, _vp, _i32, _vp])
    tg = [C.c_int, C.c_int, _i64, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp, _i64, _i64]
    _sig(L, "bli_dgemm", None, tg)
    _sig(L, "bli_sgemm", None, tg)
    _sig(L, "bli_dgemm_ex", None, tg + [_vp, _vp])
    tt = [C.c_int] * 4 + [_i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64]
    _sig(L, "bli_dtrsm", None, tt)
    _sig(L, "bli_dtrsm_ex", None, tt + [_vp, _vp])
    _sig(L, "bli_dscalv", None, [C.c_int, _i64, _vp, _vp, _i64])
    _sig(L, "bli_dcopyv", None, [C.c_int, _i64, _vp, _i64, _vp, _i64])
    _sig(L, "bli_damaxv", None, [_i64, _vp, _i64, _vp])
    _sig(L, "bli_dger", None, [C.c_int, C.c_int, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _i64])
    _sig(L, "bli_dtrsv", None, [C.c_int] * 3 + [_i64, _vp, _vp, _i64, _i64, _vp, _i64])
    _sig(L, "bli_dtrmm", None, tt)
    _sig(L, "bli_dsymm", None, [C.c_int] * 4 + [_i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp,
                                                 _i64, _i64])
    _sig(L, "bli_dsyrk", None, [C.c_int, C.c_int, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _vp, _i64, _i64])
    _sig(L, "bli_dgemmt", None, [C.c_int] * 3 + [_i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _i64, _vp, _vp,
                                                  _i64, _i64])
    tv = [C.c_int, C.c_int, _i64, _i64, _vp, _vp, _i64, _i64, _vp, _i64, _vp, _vp, _i64]
    _sig(L, "bli_dgemv", None, tv)
    _sig(L, "bli_dgemv_ex", None, tv + [_vp, _vp])
    _sig(L, "bli_daxpyv", None, [C.c_int, _i64, _vp, _vp, _i64, _vp, _i64])
    _sig(L, "bli_daxpyv_ex", None, [C.c_int, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp])
    _sig(L, "bli_ddotv", None, [C.c_int, C.c_int, _i64, _vp, _i64, _vp, _i64, _vp])
    _sig(L, "bli_ddotv_ex", None, [C.c_int, C.c_int, _i64, _vp, _i64, _vp, _i64, _vp, _vp, _vp])
    dg = [C.c_int, C.c_int, _i64, _i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64, _d, _vp, _i64, _i64]
    _sig(L, "gb_dgemm_dev", C.c_int, dg + [_vp])
    _sig(L, "gb_dgemm_ozaki_dev", C.c_int, dg + [C.c_int, _vp])
    _sig(L, "gb_dgemm_ozaki_crt_dev", C.c_int, dg + [C.c_int, _vp])
    sg = [C.c_int, C.c_int, _i64, _i64, _i64, _f, _vp, _i64, _i64, _vp, _i64, _i64, _f, _vp, _i64, _i64]
    _sig(L, "gb_sgemm_dev", C.c_int, sg + [_vp])
    _sig(L, "gb_dtrsm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64, _vp])
    _sig(L, "gb_strsm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, _f, _vp, _i64, _i64, _vp, _i64, _i64, _vp])
    _sig(L, "gb_zgemv_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64, DComplex,
                                      _vp, _i64, _vp])
    _sig(L, "gb_cgemv_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, SComplex, _vp, _i64, _i64, _vp, _i64, SComplex,
                                      _vp, _i64, _vp])
    _sig(L, "gb_ztrmm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64, _i64,
                                                      _vp])
    _sig(L, "gb_ctrmm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, SComplex, _vp, _i64, _i64, _vp, _i64, _i64,
                                                      _vp])
    _sig(L, "gb_zsyrk_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, DComplex, _vp, _i64, _i64, DComplex, _vp, _i64,
                                      _i64, _vp])
    _sig(L, "gb_csyrk_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, SComplex, _vp, _i64, _i64, SComplex, _vp, _i64,
                                      _i64, _vp])
    _sig(L, "gb_zsyr2k_dev", C.c_int, [C.c_int, C.c_int, C.c_int, _i64, _i64, DComplex, _vp, _i64, _i64, _vp, _i64,
                                       _i64, DComplex, _vp, _i64, _i64, _vp])
    _sig(L, "gb_csyr2k_dev", C.c_int, [C.c_int, C.c_int, C.c_int, _i64, _i64, SComplex, _vp, _i64, _i64, _vp, _i64,
                                       _i64, SComplex, _vp, _i64, _i64, _vp])
    _sig(L, "gb_ctrsm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, SComplex, _vp, _i64, _i64, _vp, _i64, _i64,
                                                      _vp])
    _sig(L, "gb_dscalv_dev", C.c_int, [_i64, _d, _vp, _i64, _vp])
    _sig(L, "gb_dcopyv_dev", C.c_int, [_i64, _vp, _i64, _vp, _i64, _vp])
    _sig(L, "gb_damaxv_dev", C.c_int, [_i64, _vp, _i64, _vp, _vp])
    _sig(L, "gb_dger_dev", C.c_int, [_i64, _i64, _d, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp])
    _sig(L, "gb_dtrsv_dev", C.c_int, [C.c_int] * 3 + [_i64, _d, _vp, _i64, _i64, _vp, _i64, _vp])
    _sig(L, "gb_dtrmm_dev", C.c_int, [C.c_int] * 4 + [_i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64, _vp])
    _sig(L, "gb_dsymm_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64, _d,
                                      _vp, _i64, _i64, _vp])
    _sig(L, "gb_dgemmt_dev", C.c_int, [C.c_int] * 3 + [_i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64, _d,
                                                        _vp, _i64, _i64, _vp])
    _sig(L, "gb_dsyrk_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _d, _vp, _i64, _i64, _d, _vp, _i64, _i64,
                                      _vp])
    _sig(L, "gb_daxpyv_dev", C.c_int, [_i64, _d, _vp, _i64, _vp, _i64, _vp])
    _sig(L, "gb_ddotv_dev", C.c_int, [_i64, _vp, _i64, _vp, _i64, _vp, _vp])
    _sig(L, "gb_dgemv_dev", C.c_int, [C.c_int, _i64, _i64, _d, _vp, _i64, _i64, _vp, _i64, _d, _vp, _i64, _vp])
    _sig(L, "gb_bgemm_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _i64, _f, _vp, _i64, _i64, _vp, _i64, _i64,
                                        _f, _vp, _i64, _i64, _vp])
    _sig(L, "gb_gemm_config_dev", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _i64, _i64, _i64, _d, _vp, _i64,
                                            _i64, _vp, _i64, _i64, _d, _vp, _i64, _i64, _vp])
    _sig(L, "gb_gemm_batch_dev", C.c_int, [_vp, _i64, C.c_int, C.c_int, _vp])
    _sig(L, "gb_batch_plan_create", C.c_int, [_vp, _i64, C.c_int, C.POINTER(C.c_void_p)])
    _sig(L, "gb_batch_plan_run", C.c_int, [_vp, C.c_int, _vp])
    _sig(L, "gb_batch_plan_destroy", C.c_int, [_vp])
    _sig(L, "gb_batch_plan_create_ex", C.c_int, [_vp, _i64, C.c_int, C.c_int, C.POINTER(C.c_void_p)])
    _sig(L, "gb_batch_plan_policy", C.c_int, [_vp])
    _sig(L, "gb_randm_dev", C.c_int, [C.c_int, C.c_int, _vp, _i64, _i64, _i64, _i64, C.c_uint64, _d, _d, _vp])
    _sig(L, "gb_dd_gemm_entries_dev", C.c_int, [C.c_int, C.c_int, _i64, _d, _vp, _i64, _i64, _vp, _i64, _i64,
                                                 _d, _vp, _i64, _i64, _i64, _vp, _vp, _vp, _vp, _vp])
    _sig(L, "gb_set_ozaki_ctas", C.c_int, [C.c_int])
    _sig(L, "gb_set_sgemm_mode", C.c_int, [C.c_int])
    _sig(L, "gb_selector_load", C.c_int, [_vp, C.c_int])
    _sig(L, "gb_selector_load_file", C.c_int, [_cp])
    _sig(L, "gb_selector_unload", C.c_int, [])
    _sig(L, "gb_set_gemm_autoselect", C.c_int, [C.c_int])
    _sig(L, "gb_selector_choose", C.c_int, [C.c_int, _i64, _i64, _i64, C.c_int, C.c_int, C.c_int, _d, _d,
                                            C.POINTER(C.c_int), C.POINTER(C.c_int)])
    _sig(L, "gb_ozaki_verify_slices_dev", C.c_int, [C.c_int, C.c_int, _i64, _i64, _i64, _vp, _i64, _i64, _vp,
                                                    _i64, _i64, C.c_int, C.c_int, C.POINTER(C.c_int), _vp])
    _sig(L, "gb_init", C.c_int, [C.c_int])
    _sig(L, "gb_set_dgemm_mode", C.c_int, [C.c_int, C.c_int])
    _sig(L, "gb_get_last_error", C.c_int, [C.c_char_p, C.c_size_t])
    _sig(L, "gb_clear_last_error", None, [])
    _sig(L, "gb_launch_count", _i64, [])
    _sig(L, "gb_set_kernel_timing", C.c_int, [C.c_int])
    _sig(L, "gb_kernel_time_ms", _d, [_cp, C.POINTER(_i64)])
    _sig(L, "gb_kernel_trace", _i64, [C.c_void_p, _i64])
    _sig(L, "gb_synchronize", C.c_int, [])
    _lib = L
    return L


def last_error():
    buf = C.create_string_buffer(512)
    code = load().gb_get_last_error(buf, 512)
    return code, buf.value.decode(errors="replace")


def check(rc, what="call"):
    if rc != 0:
        code, msg = last_error()
        raise RuntimeError("%s failed (%d): %s" % (what, rc, msg))
    return rc
