"""ctypes binding of libmsod.so, the library's C ABI (include/msod.h).

The library is built in-tree by ``minisod2d_gb300.build`` (``__graft_entry__.build()``
calls it).  Loading never falls back to anything else: if the shared object is
missing the import of a kernel fails with ``MsodLibraryMissing``.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmsod.so")

MSOD_OK = 0
MSOD_ERR_INVALID_ARG = 1
MSOD_ERR_PORDER = 2
MSOD_ERR_CUDA = 3
MSOD_ERR_BAD_TABLES = 4
MSOD_ERR_NO_DEVICE = 5
MSOD_ERR_INTERNAL = 6
MSOD_ERR_UNSUPPORTED = 7
MSOD_ERR_BAD_MODEL = 8
MSOD_MAX_PORDER = 8
MSOD_FIELDS_SMOOTH = 0
MSOD_FIELDS_SHOCK = 1
MSOD_PREC_FP16 = 0
MSOD_PREC_BF16 = 1
MSOD_PREC_FP32 = 2
MSOD_MU_E_GIVEN = 0
MSOD_MU_E_PLAIN = 1
MSOD_MU_E_LEARNED = 2

_i, _u64, _i64, _f, _d, _p, _sz = C.c_int, C.c_uint64, C.c_int64, C.c_float, C.c_double, C.c_void_p, C.c_size_t

# Symbol -> argument types.  Every symbol declared in include/msod.h appears here.
_GEOM = [_i, _i, _i, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]  # porder..gmshAtoK (with Ngp, dNgp, xgp)
_GEOM64 = [_i, _i, _i, _p, _p, _p, _p, _p, _p, _p, _p]            # porder, nelem, npoin, connec, He, gpvol, dlx, inv, AtoI/J/K
SIGNATURES = {
    "msod_init": [_i],
    "msod_finalize": [],
    "msod_last_error_string": [],
    "msod_version": [],
    "msod_set_checked": [_i],
    "msod_malloc": [C.POINTER(_p), _sz],
    "msod_free": [_p],
    "msod_h2d": [_p, _p, _sz, _p],
    "msod_lumped_mass": [_i, _i, _i, _p, _p, _p, _p],
    "msod_rk4_workspace_bytes": [_i, C.POINTER(_sz)],
    "msod_rk4_step": _GEOM64 + [_f, _f, _f, _f] + [_p] * 4 + [_f] + [_p] * 4 + [_sz, _p],
    "msod_d2h": [_p, _p, _sz, _p],
    "msod_memset": [_p, _i, _sz, _p],
    "msod_stream_synchronize": [_p],
    "msod_convec_ijk": _GEOM + [_p] * 8 + [_p],
    "msod_convec_ijk_split": _GEOM + [_p] * 8 + [_p],
    "msod_diffusion_ijk": _GEOM + [_f, _f] + [_p] * 9 + [_p],
    "msod_convec_diffusion_ijk": _GEOM + [_f, _f] + [_p] * 9 + [_p] * 6 + [_p],
    "msod_convec_ijk_f64": _GEOM64 + [_p] * 8 + [_p],
    "msod_convec_ijk_mixed": [_i] + _GEOM64 + [_p] * 8 + [_p],
    "msod_diffusion_ijk_mixed": [_i] + _GEOM64 + [_f, _f] + [_p] * 9 + [_p],
    "msod_diffusion_ijk_mixed_nu": [_i] + _GEOM64 + [_f, _f] + [_p] * 9 + [_p],
    "msod_diffusion_ijk_f64": _GEOM64 + [_d, _d] + [_p] * 9 + [_p],
    "msod_check_element_tables": [_i, _i, _i, _p, _p, _p, _p, _p, _p, _p],
    "msod_check_element_tables_noalloc": [_i, _i, _i, _p, _p, _p, _p, _p, _p, _p],
    "msod_fem_convec": [_i, _i] + [_p] * 13 + [_p],
    "msod_fem_convec_f64": [_i, _i] + [_p] * 13 + [_p],
    "msod_fem_diffu": [_i, _i] + [_p] * 5 + [_f, _f] + [_p] * 9 + [_p],
    "msod_fem_diffu_f64": [_i, _i] + [_p] * 5 + [_d, _d] + [_p] * 9 + [_p],
    "msod_tet_jacobian": [_i, _i] + [_p] * 6 + [_p],
    "msod_tet_jacobian_f64": [_i, _i] + [_p] * 6 + [_p],
    "msod_tet_element_tables": [_p] * 4,
    "msod_tet_element_tables_f64": [_p] * 4,
    "msod_tet_mesh_disconnected": [_i, _p, _p, _p],
    "msod_elem_jacobian": [_i, _i, _i, _p, _p, _p, _p, _p, _p, _p],
    "msod_elem_jacobian_f64": [_i, _i, _i, _p, _p, _p, _p, _p, _p, _p],
    "msod_fem_element_tables": [_i] + [_p] * 10,
    "msod_fem_element_tables_f64": [_i] + [_p] * 10,
    "msod_mesh_structured": [_i, _i, _i, _i, _p, _p, _p, _d, _u64, _p, _p],
    "msod_fields_recipe": [_i, _i, _u64, _i64, _p, _p, _p, _p, _p, _p, _p, _p],
    "msod_mesh_disconnected": [_i, _i, _p, _p, _p],
    "msod_reference_ic": [_i, _i, _i64] + [_p] * 10,
    "msod_entropy_viscosity": [_i, _i, _i] + [_p] * 8 + [_p, _p, _p, _f, _f, _f, _i, _p, _p, _p, _p],
    "msod_mlp_features": [_i, _i, _i] + [_p] * 8 + [_p, _p, _p, _f, _f, _f, _p, _p, _p],
    "msod_mlp_create": [C.POINTER(_p), _u64],
    "msod_mlp_destroy": [_p],
    "msod_mlp_train": [_p, _p, _p, _p, _i, _i, _i, _f, _u64, _p, _p],
    "msod_mlp_gradient": [_p, _p, _p, _p, _p, _i, _p, _p],
    "msod_mlp_get_params": [_p, _p, _p],
    "msod_mlp_set_params": [_p, _p, _p],
    "msod_mlp_predict": [_p, _p, _p, _i, _p, _p, _p, _p],
    "msod_mlp_save": [_p, C.c_char_p],
    "msod_mlp_load": [_p, C.c_char_p],
    "msod_learned_viscosity": [_p, _i, _i, _i] + [_p] * 8 + [_p, _p, _p, _f, _f, _f, _f, _p, _p, _p],
    "msod_diffusion_ijk_nu": [_i, _i, _i] + [_p] * 8 + [_f, _f] + [_p] * 9 + [_p],
    "msod_set_mode": [_i, _i, _p],
    "msod_get_mode": [_p, _p],
    "msod_diffusion_ijk_learned": [_p, _i, _i, _i] + [_p] * 8 + [_f, _f] + [_p] * 6 + [_f] * 4 + [_p] * 6,
}


class MsodError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("msod error %d: %s" % (code, msg))
        self.code = code


class MsodLibraryMissing(ImportError):
    pass


_lib = None
_lock = threading.Lock()


def lib():
    """The loaded libmsod.so (raises MsodLibraryMissing if it was not built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise MsodLibraryMissing(
                        "libmsod.so is not built; run `python -c \"import __graft_entry__ as g; g.build()\"`")
                L = C.CDLL(LIB_PATH)
                for name, argt in SIGNATURES.items():
                    fn = getattr(L, name)
                    fn.argtypes = argt
                    fn.restype = C.c_char_p if name == "msod_last_error_string" else C.c_int
                _lib = L
    return _lib


def check(rc):
    if rc != MSOD_OK:
        msg = lib().msod_last_error_string()
        raise MsodError(rc, msg.decode() if msg else "")
    return rc


def call(name, *args):
    return check(getattr(lib(), name)(*args))
