"""ctypes mirror of include/mge_gpu.h (the C-ABI of the GB300 cycle).

The structs here are byte-for-byte the C structs of the header; the loader
binds every exported entry point with its argument types so a wrong call
fails in Python instead of corrupting memory.
"""
import ctypes as C
import os

MGE_OK = 0
MGE_ENAN = -1
MGE_ENEGPRESS = -2
MGE_EZERORHO = -3
MGE_EBADCFG = -4
MGE_ENOMEM = -5
MGE_ETIMEOUT = -6
MGE_ECUDA = -7
MGE_ENOTFOUND = -8

ERROR_NAMES = {
    MGE_ENAN: "MGE_ENAN",
    MGE_ENEGPRESS: "MGE_ENEGPRESS",
    MGE_EZERORHO: "MGE_EZERORHO",
    MGE_EBADCFG: "MGE_EBADCFG",
    MGE_ENOMEM: "MGE_ENOMEM",
    MGE_ETIMEOUT: "MGE_ETIMEOUT",
    MGE_ECUDA: "MGE_ECUDA",
    MGE_ENOTFOUND: "MGE_ENOTFOUND",
}

MGE_EQN_EULER, MGE_EQN_NS = 0, 1
MGE_DIS_CENTRAL, MGE_DIS_ROE1, MGE_DIS_ROE2 = 0, 1, 2
MGE_DISSIP_SCALAR, MGE_DISSIP_MATRIX = 0, 1
MGE_PREC_FP64, MGE_PREC_MIXED, MGE_PREC_REFINED = 0, 1, 2
MGE_MAX_STAGE = 8
MGE_MAX_LEVEL = 16
MGE_MAX_CLOUD = 8

_d = C.c_double
_i = C.c_int


class MgeParams(C.Structure):
    _fields_ = [
        ("mstage", _i),
        ("cstp", _d * MGE_MAX_STAGE),
        ("cdis", _d * MGE_MAX_STAGE),
        ("cfl", _d),
        ("vt", _i),
        ("vis2", _d),
        ("vis4", _d),
        ("smoo", _d),
        ("mgtype", _i),
        ("eqntype", _i),
        ("distype", _i),
        ("dissip", _i),
        ("gamma", _d),
        ("rm", _d),
        ("alpha", _d),
        ("beta", _d),
        ("rho0", _d),
        ("p0", _d),
        ("c0", _d),
        ("ei0", _d),
        ("u0", _d),
        ("v0", _d),
        ("w0", _d),
        ("h0", _d),
        ("viscl", _d),
        ("prlmean", _d),
        ("gas_const", _d),
        ("limfac", _d),
        ("epsentr", _d),
        ("wall_adiabatic", _i),
        ("irs_variant", _i),
        ("precision", _i),
        ("nlevel", _i),
        ("mcyc", _i * MGE_MAX_LEVEL),
        ("conv_drop", _d),
        ("execmode", _i),
        ("dtstep", _d),
    ]


_pi32 = C.POINTER(C.c_int32)
_pd = C.POINTER(C.c_double)


# MGE_ABI_VERSION of include/mge_gpu.h: the layout of the structs below
MGE_ABI_VERSION = 2


class MgeBlockDesc(C.Structure):
    _fields_ = [
        ("nx", _i),
        ("ny", _i),
        ("nz", _i),
        ("h", _d * 3),
        ("origin", _d * 3),
        ("cellvolume", _d),
        ("si", _d * 3),
        ("sj", _d * 3),
        ("sk", _d * 3),
        ("bctype", _i * 6),
        ("facenvec", (_d * 3) * 6),
        ("blank", _pi32),
        ("nmir", _i),
        ("ccid", _pi32),
        ("scid", _pi32),
        ("faceid", _pi32),
        ("zz", _pi32),
        ("npoint", _pi32),
        ("ijkdex", _pi32),
        ("coef", _pd),
        ("nvec", _pd),
        ("qb", _pd),
        ("area", _pd),
        ("parent", _i),
        ("ratio", _i * 3),
        ("offset", _i * 3),
        ("psurf", _pd),
    ]


class MgeForces(C.Structure):
    _fields_ = [("force", _d * 3), ("moment", _d * 3), ("cl", _d), ("cd", _d)]


class MgeSolveOpts(C.Structure):
    _fields_ = [
        ("max_cycles_total", _i),
        ("ref_area", _d),
        ("moment_center", _d * 3),
        ("use_graph", _i),
        ("refine_drop", _d),
    ]


# (name, restype, argtypes) shared by the product library (prefix mge_) and
# the oracle (prefix mgeo_); the context pointer is an opaque c_void_p.
_vp = C.c_void_p
_ppv = C.POINTER(C.c_void_p)
SIGNATURES = [
    ("destroy", None, [_vp]),
    ("last_error", C.c_char_p, [_vp]),
    ("add_block", _i, [_vp, C.POINTER(MgeBlockDesc), _i, _i]),
    ("commit", _i, [_vp]),
    ("init_flow", _i, [_vp]),
    ("upload_state", _i, [_vp, _i, _i, _pd]),
    ("download_field", _i, [_vp, _i, _i, C.c_char_p, _pd, C.c_size_t]),
    ("timestep", _i, [_vp, _i, _i]),
    ("euler", _i, [_vp, _i, _i, _i, _i, _i, _i, _i, _i]),
    ("euler_partial", _i, [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _i]),
    ("movco", _i, [_vp, _i]),
    ("movfin", _i, [_vp, _i, _i]),
    ("bc_overlap", _i, [_vp, _i]),
    ("get_rtrms", _i, [_vp, _i, _i, _i, _pd]),
    ("solve", _i, [_vp, C.POINTER(MgeSolveOpts), _pd, _i, C.POINTER(_i), C.POINTER(MgeForces)]),
    ("forces_compute", _i, [_vp, _i, C.POINTER(MgeSolveOpts), C.POINTER(MgeForces)]),
    ("upload_solut", _i, [_vp, _i, _i, _d, _pd, C.c_size_t, C.POINTER(_i)]),
    ("time_advance", _i, [_vp, C.POINTER(_i)]),
    ("move_surface", _i, [_vp, _i, _i, _pd, _pd, _pd, _d]),
    ("get_surface", _i, [_vp, _i, _i, _pd]),
]

# entry points only the product library has (mge_init also takes the device)
ORACLE_INIT = ("init", _i, [C.POINTER(MgeParams), _ppv])
PRODUCT_ONLY = [
    ("init", _i, [C.POINTER(MgeParams), _i, _ppv]),
    ("abi_version", _i, []),
    ("build_info", C.c_char_p, []),
    ("params_default", None, [C.POINTER(MgeParams), _d, _d, _d, _d]),
    ("download_state", _i, [_vp, _i, _i, _pd, _pd]),
    ("device_bytes", C.c_size_t, [_vp]),
    ("sync", _i, [_vp]),
    ("cycle", _i, [_vp, _i, _i, _pd]),
    ("last_cycle_ms", _d, [_vp]),
    ("launch_count", C.c_longlong, [_vp]),
    ("kernel_times", _i, [_vp, _i, _i, _pd, _i]),
    ("coop_trace", _i, [_vp, _i, _pd, _i]),
    ("cycle_async", _i, [_vp, _i]),
    ("cycle_poll", _i, [_vp, _i, _pd]),
    ("group_cycle_async", _i, [_vp, _i, _i]),
    ("group_cycle_poll", _i, [_vp, _i, _i, _pd, C.POINTER(C.c_int)]),
    ("prolong_async", _i, [_vp, _i]),
    ("set_coop_ctas", _i, [_vp, _i]),
    ("tuned", _i, [_vp, _i, _i, C.POINTER(_i), C.POINTER(_i)]),
    ("set_precision", _i, [_vp, _i]),
    ("device_mem", _i, [_i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("residual_norm_noalloc", _i, [_vp, _vp, _vp, _i, _i, _i, _d, _i, _d, _vp, _vp]),
    ("write_restart", _i, [_vp, C.c_char_p, C.POINTER(_i), _i]),
    ("read_restart", _i, [_vp, C.c_char_p, C.POINTER(_i), _i]),
    ("restart_format", C.c_longlong, [_i, _i, _i, _i, _pd, C.c_char_p, C.c_longlong]),
    ("restart_parse", C.c_longlong, [C.c_char_p, C.c_longlong, _i, _i, _i, _i, _pd]),
]
KERNEL_KINDS = ["timestep", "prep", "face", "rec", "combine", "irs_i", "irs_j", "irs_k_update", "cutcell", "bcond",
                "rtrms"]

# the entry points declared in include/mge_gpu.h, in declaration order
HEADER_SYMBOLS = [
    "mge_abi_version", "mge_build_info", "mge_params_default", "mge_init", "mge_destroy",
    "mge_last_error", "mge_add_block", "mge_commit", "mge_init_flow", "mge_upload_state",
    "mge_download_state", "mge_download_field", "mge_timestep", "mge_euler", "mge_movco",
    "mge_movfin", "mge_bc_overlap", "mge_get_rtrms", "mge_solve", "mge_forces_compute",
    "mge_cycle", "mge_cycle_async", "mge_cycle_poll", "mge_group_cycle_async", "mge_group_cycle_poll", "mge_prolong_async", "mge_set_coop_ctas", "mge_device_mem", "mge_tuned", "mge_set_precision",
    "mge_coop_trace", "mge_last_cycle_ms", "mge_launch_count", "mge_kernel_times", "mge_residual_norm_noalloc", "mge_euler_partial", "mge_device_bytes", "mge_sync",
    "mge_upload_solut", "mge_write_restart", "mge_read_restart", "mge_restart_format", "mge_restart_parse",
    "mge_time_advance", "mge_move_surface", "mge_get_surface",
]


def bind(lib, prefix, table):
    for name, res, args in table:
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
    return lib


def error_name(code):
    return ERROR_NAMES.get(code, str(code))


PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
