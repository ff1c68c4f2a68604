"""ctypes binding of libminifem_gb300.so (include/mfem_gpu.h).

There is no fallback: if the library is missing or fails to load, importing
this module raises, and every operator of this package needs it.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libminifem_gb300.so")

MFEM_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "no CUDA device", -4: "call out of order",
          -5: "CSR pattern mismatch", -6: "Not enough colors", -7: "capacity exceeded",
          -8: "device wait timed out"}
OP_LAP, OP_ELA = 0, 1
FP64, FP32 = 0, 1
AUTO, GATHER, SCATTER, ATOMIC = -1, 0, 1, 2
ORDER_SORTED, ORDER_REFERENCE = 0, 1
LOCALITY_MORTON, LOCALITY_BISECTION = 1, 2

_vp, _ip, _dp, _fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_float)

_SIGS = {
    "mfem_abi_version": ([], C.c_int),
    "mfem_status_string": ([C.c_int], C.c_char_p),
    "mfem_last_error": ([_vp], C.c_char_p),
    "mfem_create": ([C.POINTER(_vp), C.c_int], C.c_int),
    "mfem_destroy": ([_vp], C.c_int),
    "mfem_get_stream": ([_vp, C.POINTER(_vp)], C.c_int),
    "mfem_set_mesh": ([_vp, _vp, _vp, C.c_int, C.c_int], C.c_int),
    "mfem_update_coords": ([_vp, _vp], C.c_int),
    "mfem_create_nodeToNode": ([_vp, C.c_int, _vp, _vp, C.c_int, _ip], C.c_int),
    "mfem_create_nodeToNode_incidence": ([_vp, _vp, _vp, _vp, _vp, C.c_int, _ip], C.c_int),
    "mfem_create_elemToEdge": ([_vp, _vp], C.c_int),
    "mfem_set_pattern": ([_vp, _vp, _vp, C.c_int], C.c_int),
    "mfem_coloring_creation": ([_vp, C.c_ulonglong, _vp, _vp, C.c_int, _ip], C.c_int),
    "mfem_rcm_permutation": ([_vp, _vp], C.c_int),
    "mfem_locality_permutation": ([_vp, C.c_int, _vp], C.c_int),
    "mfem_set_coefficients": ([_vp, C.c_int, _vp], C.c_int),
    "mfem_assemble": ([_vp, C.c_int, C.c_int, C.c_int], C.c_int),
    "mfem_assemble_prec": ([_vp, C.c_int, C.c_int, C.c_int], C.c_int),
    "mfem_set_check_bounds": ([_vp, _vp], C.c_int),
    "mfem_set_interfaces": ([_vp, C.c_int, _vp, _vp], C.c_int),
    "mfem_halo_pack": ([_vp, _vp], C.c_int),
    "mfem_halo_add": ([_vp, _vp], C.c_int),
    "mfem_prec_init": ([_vp], C.c_int),
    "mfem_prec_inversion": ([_vp, _ip], C.c_int),
    "mfem_set_sliver_threshold": ([_vp, C.c_double], C.c_int),
    "mfem_set_option": ([_vp, C.c_char_p, C.c_double], C.c_int),
    "mfem_tile_info": ([_vp, _ip, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                        C.POINTER(C.c_longlong), _ip], C.c_int),
    "mfem_get_flagged": ([_vp, _ip], C.c_int),
    "mfem_get_values": ([_vp, _vp], C.c_int),
    "mfem_get_values_f32": ([_vp, _vp], C.c_int),
    "mfem_get_prec": ([_vp, _vp], C.c_int),
    "mfem_values_device": ([_vp, C.POINTER(_vp), _ip], C.c_int),
    "mfem_prec_device": ([_vp, C.POINTER(_vp)], C.c_int),
    "mfem_synchronize": ([_vp], C.c_int),
    "mfem_step_async": ([_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp,
                         C.POINTER(C.c_longlong)], C.c_int),
    "mfem_wait": ([_vp, C.c_longlong], C.c_int),
    "mfem_spmv": ([_vp, _vp, _vp, C.c_int], C.c_int),
    "mfem_prec_apply": ([_vp, _vp, _vp], C.c_int),
    "mfem_pcg": ([_vp, _vp, _vp, C.c_double, C.c_int, C.c_int, _ip, C.POINTER(C.c_double)], C.c_int),
    "mfem_profile": ([_vp, C.c_int], C.c_int),
    "mfem_profile_read": ([_vp, C.c_char_p, C.c_int, _fp, C.c_int, _ip], C.c_int),
    "mfem_get_sizes": ([_vp, _ip, _ip, _ip, _ip], C.c_int),
    "mfem_assemble_noalloc": ([_vp, C.c_int, _vp, _vp, _vp, _vp], C.c_int),
    "mfem_fp64_rate": ([_vp, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "mfem_selftest_dmul": ([_vp, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong),
                            C.POINTER(C.c_ulonglong)], C.c_int),
    "mfem_batch_create": ([C.POINTER(_vp), C.c_int], C.c_int),
    "mfem_batch_destroy": ([_vp], C.c_int),
    "mfem_batch_last_error": ([_vp], C.c_char_p),
    "mfem_batch_get_stream": ([_vp, C.POINTER(_vp)], C.c_int),
    "mfem_batch_add": ([_vp, _vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfem_batch_set_coefficients": ([_vp, C.c_int, _vp], C.c_int),
    "mfem_batch_assemble": ([_vp, C.c_int, C.c_int], C.c_int),
    "mfem_batch_synchronize": ([_vp], C.c_int),
    "mfem_batch_get_values": ([_vp, C.c_int, C.c_int, C.c_int, _vp], C.c_int),
    "mfem_batch_get_prec": ([_vp, C.c_int, C.c_int, _vp], C.c_int),
    "mfem_batch_info": ([_vp, _ip, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), _ip, _ip],
                        C.c_int),
    "mfem_assembly": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int],
                      C.c_int),
    "mfem_prec_init_host": ([_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int], C.c_int),
    "mfem_prec_inversion_host": ([_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int], C.c_int),
}


class MfemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built: run python mini-fem_gb300/build.py "
                          "(the package has no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = _load()


def exported_symbols() -> list[str]:
    return sorted(_SIGS)
