"""ctypes binding of the C ABI in include/mdft_gb300.h.

The shared library is built in-tree (``mini_mdft_gb300/lib``).  Loading fails
loudly when it is missing: there is no CPU fallback for the hot path.
"""
import ctypes as C
import os
import re

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libmdft_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_PKG), "include", "mdft_gb300.h")

MDFT_OK = 0
MDFT_ERR_TIMEOUT = 6
MDFT_F64 = 0
MDFT_F32 = 1
MDFT_F64_DF = 2

_lib = None

vp = C.c_void_p
dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
i32 = C.c_int
f64 = C.c_double
sz = C.c_size_t

SIGNATURES = {
    "mdft_abi_version": (i32, []),
    "mdft_last_error": (C.c_char_p, []),
    "mdft_grid_create": (i32, [C.POINTER(vp), i32, i32, i32, f64, f64, f64, i32, i32]),
    "mdft_grid_destroy": (i32, [vp]),
    "mdft_grid_info": (i32, [vp, ip]),
    "mdft_grid_kvectors": (i32, [vp, dp, dp, dp]),
    "mdft_grid_angular": (i32, [vp, dp, dp, dp]),
    "mdft_grid_opmap": (i32, [vp, ip, ip, ip, ip, ip, dp]),
    "mdft_grid_ang_matrices": (i32, [vp, dp, dp]),
    "mdft_opt_create": (i32, [C.POINTER(vp), vp, i32]),
    "mdft_opt_create_batched": (i32, [C.POINTER(vp), vp, i32, i32]),
    "mdft_opt_destroy": (i32, [vp]),
    "mdft_opt_angl2proj": (i32, [vp, vp, vp, vp]),
    "mdft_opt_proj2angl": (i32, [vp, vp, vp, vp]),
    "mdft_opt_angl2proj_from_xi": (i32, [vp, vp, f64, vp, vp]),
    "mdft_conv_create": (i32, [C.POINTER(vp), vp, ip, dp, i32, i32, f64, i32]),
    "mdft_conv_create_batched": (i32, [C.POINTER(vp), vp, ip, dp, i32, i32, f64, i32, i32]),
    "mdft_conv_create_from_file": (i32, [C.POINTER(vp), vp, C.c_char_p, i32, i32]),
    "mdft_conv_destroy": (i32, [vp]),
    "mdft_conv_execute": (i32, [vp, vp, vp]),
    "mdft_conv_execute_timed": (i32, [vp, vp, vp, C.POINTER(vp)]),
    "mdft_conv_execute_timed_passes": (i32, [vp, vp, vp, C.POINTER(vp)]),
    "mdft_conv_fft": (i32, [vp, vp, i32, vp]),
    "mdft_conv_kspace": (i32, [vp, vp, vp]),
    "mdft_conv_info": (i32, [vp, ip, dp]),
    "mdft_conv_gamma_p_map": (i32, [vp, ip]),
    "mdft_conv_mnmunukhi_q": (i32, [vp, dp]),
    "mdft_luc_read": (i32, [C.c_char_p, i32, f64, ip, dp, ip, dp]),
    "mdft_luc_write": (i32, [C.c_char_p, ip, dp, i32, i32, f64, C.c_char_p]),
    "mdft_get_delta_rho": (i32, [vp, vp, sz, f64, i32, vp]),
    "mdft_get_delta_f": (i32, [vp, vp, vp, vp, vp, sz, i32, f64, f64, i32, vp]),
    "mdft_get_delta_f_noalloc": (i32, [vp, vp, vp, vp, vp, sz, i32, f64, f64, i32, vp]),
    "mdft_scratch_pool": (i32, [C.POINTER(vp)]),
    "mdft_wait_timeouts": (i32, [ip]),
    "mdft_wait_selftest": (i32, [i32, vp]),
    "mdft_grid_barrier_selftest": (i32, [i32, vp]),
    "mdft_server_create": (i32, [C.POINTER(vp), i32, i32, sz]),
    "mdft_server_destroy": (i32, [vp]),
    "mdft_server_add_solvent": (i32, [vp, i32, i32, ip, dp, i32, i32, f64, f64, f64, ip]),
    "mdft_server_submit": (i32, [vp, i32, i32, i32, i32, f64, f64, f64, vp, i32, f64,
                                 C.POINTER(C.c_longlong)]),
    "mdft_server_wait": (i32, [vp, C.c_longlong, vp, dp, dp]),
    "mdft_server_stats": (i32, [vp, dp]),
    "mdft_server_set_solvent_model": (i32, [vp, i32, dp, i32, f64, f64]),
    "mdft_server_submit_solute": (i32, [vp, i32, i32, i32, i32, f64, f64, f64, dp, i32, dp, i32, f64,
                                        C.POINTER(C.c_longlong)]),
    "mdft_server_wait_solute": (i32, [vp, C.c_longlong, dp, dp, ip, ip, dp]),
    "mdft_vext_lj_coulomb": (i32, [vp, dp, i32, dp, i32, f64, vp, vp]),
    "mdft_solver_create": (i32, [C.POINTER(vp), vp, vp, vp, f64, f64, f64, i32]),
    "mdft_solver_energy": (i32, [vp, vp, vp, dp, vp]),
    "mdft_solver_minimize": (i32, [vp, vp, i32, f64, f64, dp, ip, vp]),
    "mdft_solver_status": (i32, [vp, ip]),
    "mdft_solver_destroy": (i32, [vp]),
}


def header_symbols():
    """Function names declared in include/mdft_gb300.h."""
    txt = open(HEADER_PATH).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mdft_[a-z0-9_]+)\s*\(", txt)))


class MdftError(RuntimeError):
    """Raised for a non-zero mdft_status (the reference raises
    std::runtime_error from Throw_If)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libmdft_gb300.so is not built; run __graft_entry__.build() "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != MDFT_OK:
        msg = lib().mdft_last_error()
        raise MdftError(rc, msg.decode() if msg else "error %d" % rc)
    return rc
