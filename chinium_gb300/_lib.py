"""ctypes binding of the C ABI in include/chinium_xc.h.

The library is built in-tree (``chinium_gb300/_build/libchinium_xc.so``).  A
missing or unloadable library is an error: there is no fallback path.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libchinium_xc.so")
DATA_PATH = os.path.join(HERE, "data")

XC_OK = 0
STATUS = {
    -1: "XC_ERR_ARG", -2: "XC_ERR_IO", -3: "XC_ERR_CUDA", -4: "XC_ERR_STATE", -5: "XC_ERR_NOMEM",
    -6: "XC_ERR_UNSUPPORTED", -7: "XC_ERR_NUMERIC", -8: "XC_ERR_TIMEOUT", -9: "XC_ERR_INTERNAL",
}
PRECISION_FP64 = 0
PRECISION_MIXED = 1


class XCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class GridInfo(ctypes.Structure):
    _fields_ = [("npoints", ctypes.c_long), ("npoints_padded", ctypes.c_long), ("nblocks", ctypes.c_int),
                ("nbasis", ctypes.c_int), ("nspin", ctypes.c_int), ("type", ctypes.c_int),
                ("ao_elements", ctypes.c_long), ("screened_pairs", ctypes.c_long),
                ("mixed_tiles", ctypes.c_int), ("mixed_pairs", ctypes.c_long), ("mixed_rows", ctypes.c_long),
                ("mixed_store_bytes", ctypes.c_long), ("mixed_launches", ctypes.c_int),
                ("mixed_units_full", ctypes.c_long), ("mixed_units_sym", ctypes.c_long),
                ("mixed_fock_jobs", ctypes.c_long), ("mixed_fock_tau_jobs", ctypes.c_long),
                ("mixed_presplit", ctypes.c_long), ("mixed_presplit_bytes", ctypes.c_long),
                ("mixed_fock_items", ctypes.c_long), ("mixed_empty_tiles", ctypes.c_long)]


class MixedConfig(ctypes.Structure):
    _fields_ = [("screen", ctypes.c_double), ("fock_tiles", ctypes.c_int), ("spatial", ctypes.c_int),
                ("func_float_above", ctypes.c_double), ("v_operands", ctypes.c_int), ("reserved", ctypes.c_int)]


class TuneCandidate(ctypes.Structure):
    _fields_ = [("cfg", MixedConfig), ("ms", ctypes.c_double), ("max_de", ctypes.c_double),
                ("max_dv", ctypes.c_double), ("kept_pairs", ctypes.c_long), ("accepted", ctypes.c_int)]


class TuneReport(ctypes.Structure):
    _fields_ = [("best", MixedConfig), ("ms_best", ctypes.c_double), ("ms_reference", ctypes.c_double),
                ("ncand", ctypes.c_int), ("cand", TuneCandidate * 32)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_L = ctypes.c_long
_S = ctypes.c_char_p
_PP = ctypes.POINTER(ctypes.c_void_p)

SIGNATURES = {
    "xc_last_error": [_P, ctypes.c_size_t],
    "xc_set_data_path": [_S],
    "xc_basis_create": [_I, _P, _P, _S, _PP],
    "xc_basis_create_shells": [_I, _P, _P, _I, _P, _P, _P, _P, _P, _I, _PP],
    "xc_basis_nbasis": [_P, _P],
    "xc_basis_nshells": [_P, _P],
    "xc_basis_shells": [_P, _P, _P, _P, _P],
    "xc_basis_primitives": [_P, _P, _P],
    "xc_basis_destroy": [_P],
    "xc_grid_create": [_P, _S, _I, _D, _PP],
    "xc_grid_destroy": [_P],
    "xc_grid_set_stream": [_P, _P],
    "xc_grid_set_type": [_P, _I],
    "xc_grid_get_ao": [_P, _I],
    "xc_grid_num_electrons": [_P, _P],
    "xc_grid_get_density": [_P, _P, _I],
    "xc_grid_get_energy": [_P, _P],
    "xc_grid_get_fock": [_P, _P],
    "xc_grid_info_get": [_P, _P],
    "xc_grid_points": [_P, _P, _P, _P, _P, _P, _P, _P, _P],
    "xc_grid_density_values": [_P, _P, _P, _P, _P],
    "xc_grid_potential_values": [_P, _P, _P, _P, _P],
    "xc_grid_block_ao": [_P, _I, _P, _P, _P],
    "xc_functional_read": [_S, _I, _PP],
    "xc_functional_create": [_P, _I, _I, _PP],
    "xc_functional_destroy": [_P],
    "xc_functional_exx": [_P, _P],
    "xc_functional_family": [_P, _P],
    "xc_evaluate": [_P, _P, _S],
    "xc_functional_eval_points": [_P, _L, _P, _P, _P, _P, _P, _P, _P],
    "xc_build": [_P, _P, _P, _I, _I, _P, _P],
    "xc_build_device": [_P, _P, _P, _I, _I, _P, _P],
    "xc_sap_fock": [_P, _P],
    "xc_sap_fock_tc": [_P, _P],
    "xc_grid_energy_grad": [_P, _P, _P, _I, _P],
    "xc_grid_fock_skeleton": [_P, _P, _P, _I, _P, _P],
    "xc_functional_fxc_points": [_P, _L, _P, _P, _P, _P, _P],
    "xc_grid_get_density_u": [_P, _P, _I, _I],
    "xc_grid_get_fock_u": [_P, _P],
    "xc_grid_set_response_precision": [_P, _I],
    "xc_build_response": [_P, _P, _P, _I, _I, _I, _P, _P],
    "xc_functional_energy_static": [_P, _L, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "xc_build_incremental": [_P, _P, _P, _I, _I, _P, _P],
    "xc_mlp_create": [_I, _I, _I, _I, _PP],
    "xc_mlp_destroy": [_P],
    "xc_mlp_nparams": [_P, _P],
    "xc_mlp_set_params": [_P, _P],
    "xc_mlp_get_params": [_P, _P],
    "xc_mlp_forward": [_P, _I, _P, _P, _I],
    "xc_mlp_backward": [_P, _I, _P, _P, _P],
    "xc_mlp_train_step": [_P, _I, _P, _P, _P, ctypes.c_float, _P],
    "xc_int1e": [_P, _P, _P, _P],
    "xc_dipole": [_P, _P, _P],
    "xc_eri": [_P, _P, _D],
    "xc_jk_create": [_P, _D, _D, _PP],
    "xc_jk_destroy": [_P],
    "xc_jk_info": [_P, _P, _P, _P],
    "xc_jk_set_stream": [_P, _P],
    "xc_jk_build": [_P, _I, _P, _P, _P],
    "xc_jk_build_device": [_P, _I, _P, _P, _P],
    "xc_grid_profile": [_P, _I],
    "xc_grid_stage_ms": [_P, _P],
    "xc_grid_kernel_ms": [_P, _P],
    "xc_grid_create_batch": [_I, _P, _S, _I, _PP],
    "xc_grid_molecules": [_P, _P, _P, _P, _P],
    "xc_grid_set_mixed_config": [_P, _P],
    "xc_grid_get_mixed_config": [_P, _P],
    "xc_grid_wait_probe": [_P, _D],
    "xc_grid_tune": [_P, _P, _P, _I, _D, _D, _I, _P],
}

_lib = None


def header_symbols():
    """Function names declared in include/*.h."""
    import glob
    import re
    names = set()
    for path in glob.glob(os.path.join(os.path.dirname(HERE), "include", "*.h")):
        with open(path) as f:
            names |= set(re.findall(r"^int\s+(xc_\w+)\s*\(", f.read(), flags=re.M))
    return sorted(names)


def lib():
    """Load the library (building it first if absent).  Raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.xc_set_data_path(DATA_PATH.encode())
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().xc_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status):
    if status != XC_OK:
        raise XCError(status, last_error())
    return status
