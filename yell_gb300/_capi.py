"""ctypes binding of the C ABI in include/yell_gb300.h.

The library must have been built (``yell_gb300.build.build()``); there is no
CPU fallback, and loading fails loudly when the shared object is missing.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libyell_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "yell_gb300.h")

YELL_OK = 0
YELL_ERR_INVALID_ARGUMENT = 1
YELL_ERR_UNSUPPORTED_DEGREE = 2
YELL_ERR_INVALID_MODULUS = 3
YELL_ERR_CUDA = 4
YELL_ERR_OUT_OF_MEMORY = 5
YELL_ERR_BUDGET = 6
YELL_ERR_TIMEOUT = 7
YELL_ERR_CANCELLED = 8
YELL_ERR_NOT_FOUND = 9
YELL_ERR_NO_DEVICE = 10

YELL_FORWARD, YELL_FORWARD_LAZY, YELL_BACKWARD = 0, 1, 2
YELL_OP_MULMOD, YELL_OP_ADDMOD, YELL_OP_SUBMOD, YELL_OP_MULADD, YELL_OP_NEGATE = 0, 1, 2, 3, 4


class PolymulDesc(ctypes.Structure):
    """struct yell_polymul_desc"""
    _fields_ = [("c", ctypes.c_void_p), ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("log_n", ctypes.c_uint32), ("L", ctypes.c_uint32), ("cm0", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class YellError(RuntimeError):
    def __init__(self, status: int, fn: str, detail: str):
        self.status = status
        super().__init__(f"{fn} failed with status {status}: {detail}")


_u8p = ctypes.c_void_p
_u32, _u64, _sz, _int = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int
_vp = ctypes.c_void_p

# name -> (restype, argtypes); pointers are passed as c_void_p (addresses).
SIGNATURES = {
    "yell_abi_version": (_int, []),
    "yell_status_string": (ctypes.c_char_p, [_int]),
    "yell_last_error": (ctypes.c_char_p, []),
    "yell_kernel_launches": (_u64, []),
    "yell_allocations": (_u64, []),
    "yell_max_moduli": (_u32, []),
    "yell_min_log_degree": (_u32, []),
    "yell_max_log_degree": (_u32, []),
    "yell_prime": (_u64, [_u32]),
    "yell_prime_pn": (_u64, [_u32]),
    "yell_primitive_root": (_u64, [_u32]),
    "yell_init_table": (_int, [_u32, _u32]),
    "yell_init_ntt_tables": (_int, [_u32, _u32]),
    "yell_init_ntt_tables_range": (_int, [_u32, _u32, _u32]),
    "yell_ntt_tables": (_int, [_u32, _u32, _vp, _vp]),
    "yell_ntt_forward": (_int, [_vp, _u32, _u32]),
    "yell_ntt_forward_lazy": (_int, [_vp, _u32, _u32]),
    "yell_ntt_backward": (_int, [_vp, _u32, _u32]),
    "yell_poly_forward": (_int, [_vp, _u32, _u32]),
    "yell_poly_forward_lazy": (_int, [_vp, _u32, _u32]),
    "yell_poly_backward": (_int, [_vp, _u32, _u32]),
    "yell_poly_mulmod": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell_poly_addmod": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell_poly_submod": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell_poly_add_product_of": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell_poly_negate": (_int, [_vp, _u32, _u32]),
    "yell_polymul_host": (_int, [_vp, _vp, _vp, _u32, _u32, _u32, _u32]),
    "yell_host_alloc": (_vp, [_sz]),
    "yell_host_free": (None, [_vp]),
    "yell_set_host_access": (_int, [_int]),
    "yell_host_access": (_int, [_vp]),
    "yell_dev_ntt": (_int, [_vp, _u32, _u32, _u32, _u32, _int, _vp]),
    "yell_dev_ntt_limbs": (_int, [_vp, _vp, _u32, _u32, _int, _vp]),
    "yell_dev_elementwise": (_int, [_int, _vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp]),
    "yell_polymul_scratch_words": (_sz, [_u32, _u32, _u32]),
    "yell_dev_polymul": (_int, [_vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp, _sz, _vp]),
    "yell_synchronize": (_int, []),
    "yell_profile_start": (_int, []),
    "yell_profile_stop": (_int, []),
    "yell_profile_count": (_int, []),
    "yell_profile_get": (_int, [_int, ctypes.c_char_p, _sz, _vp, _vp]),
    "yell_dev_polymul_noalloc": (_int, [_vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp]),
    "yell_dev_polymul_batch": (_int, [_vp, _u32, _vp]),
    "yell_calibrate_butterflies": (_int, [_vp, _vp]),
    "yell32_calibrate_butterflies": (_int, [_vp, _vp]),
    "yell_negacyclic_forward_lazy": (_int, [_vp, _u64, _vp, _vp, _u64]),
    "yell_negacyclic_backward_lazy": (_int, [_vp, _u64, _vp, _vp, _u64]),
    "yell32_max_moduli": (_u32, []),
    "yell32_max_log_degree": (_u32, []),
    "yell32_prime": (_u32, [_u32]),
    "yell32_prime_pn": (_u32, [_u32]),
    "yell32_primitive_root": (_u32, [_u32]),
    "yell32_ntt_tables": (_int, [_u32, _u32, _vp, _vp]),
    "yell32_init_ntt_tables": (_int, [_u32, _u32, _u32]),
    "yell32_ntt_forward": (_int, [_vp, _u32, _u32]),
    "yell32_ntt_forward_lazy": (_int, [_vp, _u32, _u32]),
    "yell32_ntt_backward": (_int, [_vp, _u32, _u32]),
    "yell32_dev_ntt": (_int, [_vp, _u32, _u32, _u32, _u32, _int, _vp]),
    "yell32_dev_polymul": (_int, [_vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp]),
    "yell32_wait_status": (_int, [_vp]),
    "yell32_wait_check": (_int, [_u64, _vp]),
    "yell32_dev_elementwise": (_int, [_int, _vp, _vp, _vp, _u32, _u32, _u32, _u32, _vp]),
    "yell32_poly_forward": (_int, [_vp, _u32, _u32]),
    "yell32_poly_forward_lazy": (_int, [_vp, _u32, _u32]),
    "yell32_poly_backward": (_int, [_vp, _u32, _u32]),
    "yell32_poly_mulmod": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell32_poly_addmod": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell32_poly_submod": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell32_poly_add_product_of": (_int, [_vp, _vp, _vp, _u32, _u32]),
    "yell32_poly_negate": (_int, [_vp, _u32, _u32]),
    "yell_dev_polymul_batch_queue": (_int, [_vp, _u32, _vp]),
    "yell_dev_polymul_batch_phased": (_int, [_vp, _u32, _vp]),
    "yell_batch_queue_status": (_int, [_vp]),
    "yell_batch_queue_wait_check": (_int, [_u64, _vp]),
    "yell_dev_poly_alloc": (_int, [_u32, _u32, _u32, _vp]),
    "yell_dev_poly_free": (_int, [_vp]),
    "yell_dev_poly_info": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "yell_dev_poly_upload": (_int, [_vp, _vp]),
    "yell_dev_poly_download": (_int, [_vp, _vp]),
    "yell_dev_poly_ntt": (_int, [_vp, ctypes.c_int]),
    "yell_dev_poly_op": (_int, [ctypes.c_int, _vp, _vp, _vp]),
    "yell_dev_poly_mul": (_int, [_vp, _vp, _vp]),
    "yell_batch_submit": (_int, [_vp, _vp, _vp, _u32, _vp]),
    "yell_batch_wait": (_int, [_vp, ctypes.c_double]),
    "yell_batch_release": (_int, [_vp]),
    "yell_crt_words": (_int, [_u32, _u32, _vp]),
    "yell_dev_crt_lift": (_int, [_vp, _vp, _u32, _u32, _u32, _u32, _vp]),
    "yell_poly_to_bigint": (_int, [_vp, _vp, _u32, _u32]),
    "yell_dev_sample_uniform": (_int, [_vp, _u32, _u32, _u32, _u32, _u64, _vp]),
    "yell_dev_sample_zo": (_int, [_vp, _u32, _u32, _u32, _u32, _u32, _u64, _vp]),
    "yell_dev_sample_hwt": (_int, [_vp, _u32, _u32, _u32, _u32, _u32, _u64, _vp]),
    "yell_dev_sample_gaussian": (_int, [_vp, _u32, _u32, _u32, _u32, ctypes.c_double, _u32, _u64, _u64, _vp]),
    "yell_gaussian_table": (_int, [ctypes.c_double, _u32, _vp, _u32]),
    "yell_variant_count": (_int, [_u32, _vp]),
    "yell_variant_name": (_int, [_u32, _u32, ctypes.c_char_p, _sz]),
    "yell_set_variant": (_int, [_u32, _u32]),
    "yell_get_variant": (_int, [_u32, _vp]),
    "yell_autotune": (_int, [_u32, _u32, _u32, _vp, _vp]),
    "yell_server_create": (_int, [_vp, _vp]),
    "yell_server_destroy": (_int, [_vp]),
    "yell_server_submit": (_int, [_vp, _vp, _vp]),
    "yell_server_wait": (_int, [_vp, _u64, ctypes.c_double, _vp]),
    "yell_server_cancel": (_int, [_vp, _u64]),
    "yell_server_pause": (_int, [_vp, _int]),
    "yell_server_get_stats": (_int, [_vp, _int, _vp]),
    "yell_server_load_test": (_int, [_vp, _vp, _u32, ctypes.c_double, ctypes.c_double, _u64, _vp]),
}

_lib = None


def header_symbols(path: str = HEADER) -> list[str]:
    """Function names declared in the C header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(yell_[a-z0-9_]+)\s*\(", text)))


def load(path: str = LIB_PATH):
    """Loads the library once; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, fn: str) -> None:
    if status != YELL_OK:
        detail = load().yell_last_error().decode(errors="replace")
        raise YellError(status, fn, detail)


def call(name: str, *args):
    """Calls an int-returning entry point and raises YellError on failure."""
    st = getattr(load(), name)(*args)
    check(st, name)
    return st
