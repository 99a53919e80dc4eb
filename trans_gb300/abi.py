"""ctypes mirror of include/trans_gpu.h (the C ABI of the hot path).

The structures are shared by every caller of the ABI: the Python driver in this package and
any test harness that feeds the same inputs to another implementation of the same ABI.
"""
import ctypes as C

TRANS_OK = 0
TRANS_E_ARG = -1
TRANS_E_CUDA = -2
TRANS_E_NAN = -3
TRANS_E_TIMEOUT = -4
TRANS_E_MEMORY = -5

TRANS_FP64 = 0
TRANS_MIXED = 1

ERRORS = {
    TRANS_E_ARG: "invalid argument",
    TRANS_E_CUDA: "CUDA error",
    TRANS_E_NAN: "NaN in density increment",
    TRANS_E_TIMEOUT: "device wait timed out",
    TRANS_E_MEMORY: "device memory budget exhausted",
}

_PARAM_DOUBLES = [
    "XM", "RXM2", "PPF", "Csthlnd", "Csth1", "Ref", "Tiny",
    "VxF", "VyF", "VzF",
]
_PARAM_DOUBLES2 = [
    "P0in", "T0in", "Pouthub",
    "VisRatio", "FSTI", "Rkf", "Rof", "Rmiuf",
    "A1", "Beta_star", "Sigk1", "Sigo1", "Beta1", "Gama1", "Sigk2", "Sigo2", "Beta2", "Gama2",
    "Prod_Lmt",
    "F_limiter1", "F_limiter2", "gama_max", "gama_min",
    "DT_LUSGS_Main", "DT_LUSGS_Sub", "CFL_Main", "CFL_Sub_start", "CFL_Sub_end",
    "Trans_location", "Alscale",
]
_PARAM_INTS = [
    "CFL_Sub_step", "IF_Local_Main", "IF_Local_Sub",
    "Kind_Spatial", "Kind_Roe", "Kind_Model", "Kind_Hybrid", "Kind_SubHY",
    "Kind_Dual", "Kchld", "IF_RK",
    "IF_Euler", "IF_Turb_org", "KItm", "IF_Comppress", "IF_Precondition", "Kind_RotMod",
    "If_fix_Transition", "KI_ini",
    "precision", "pad_",
]


class TransParams(C.Structure):
    _fields_ = ([(n, C.c_double) for n in _PARAM_DOUBLES]
                + [("omega", C.c_double * 3)]
                + [(n, C.c_double) for n in _PARAM_DOUBLES2]
                + [(n, C.c_int) for n in _PARAM_INTS])


I3 = C.c_int * 3


class TransConn(C.Structure):
    _fields_ = [
        ("BCType", C.c_int), ("SubBCType", C.c_int), ("PerType", C.c_int), ("lcross", C.c_int),
        ("pointStart", I3), ("pointEnd", I3),
        ("IJKDirect", C.c_int), ("LeftOrRight", C.c_int),
        ("IJKAdd", I3), ("CIJKAdd", I3), ("CIJKAdd1", I3), ("CIJKAdd2", I3),
        ("CEIJKAdd", I3), ("CEIJKAdd1", I3), ("CEIJKAdd2", I3),
        ("Transform", I3), ("TransformT", I3), ("revMatrix", I3),
        ("TargetBlock", C.c_int), ("TargetConn", C.c_int),
        ("rotateAngle", C.c_double),
    ]


class TransBlock(C.Structure):
    _fields_ = [
        ("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("id", C.c_int),
        ("nconn", C.c_int), ("pad_", C.c_int),
        ("conn", C.POINTER(TransConn)),
        ("markwall", C.POINTER(C.c_int) * 6),
    ]


class TransNorms(C.Structure):
    _fields_ = [
        ("DRSa", C.c_double), ("DUa", C.c_double), ("DRSk", C.c_double), ("DUk", C.c_double),
        ("DRSo", C.c_double), ("DUo", C.c_double),
        ("Ima", C.c_int), ("Jma", C.c_int), ("Kma", C.c_int), ("nan_flag", C.c_int),
    ]


class TransIntegrals(C.Structure):
    _fields_ = [
        ("mass_in", C.c_double), ("p0_in", C.c_double), ("p_in", C.c_double),
        ("mass_out", C.c_double), ("p0_out", C.c_double), ("p_out", C.c_double),
        ("loss", C.c_double), ("force_p", C.c_double * 3), ("force_v", C.c_double * 3),
    ]

    def as_dict(self):
        return {"mass_in": self.mass_in, "p0_in": self.p0_in, "p_in": self.p_in,
                "mass_out": self.mass_out, "p0_out": self.p0_out, "p_out": self.p_out,
                "loss": self.loss, "force_p": list(self.force_p), "force_v": list(self.force_v)}


# field ids (enum trans_field)
FIELDS = ["V", "PP", "T", "RMIU", "WT0", "WT1", "SD", "GRAD", "VOL", "ALAGM", "DST", "ALENG",
          "ASENG", "XC", "YC", "ZC", "RAD", "THTC", "D", "RDS", "DTM", "DQDXYZ", "SHOCK", "WT2"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}

# Fortran allocation of each field: (leading components, lower bound, upper-bound offset from
# the node count N, i.e. ub = N + 2 for every field).
FIELD_LAYOUT = {
    "V": ((7,), -2), "PP": ((), -2), "T": ((), -2), "RMIU": ((), -2),
    "WT0": ((7,), 1), "WT1": ((7,), 1),
    "SD": ((3, 3), -2), "GRAD": ((3,), -2), "VOL": ((), -2), "ALAGM": ((3,), -2),
    "DST": ((), -2), "ALENG": ((), -2), "ASENG": ((), 1),
    "XC": ((), 0), "YC": ((), 0), "ZC": ((), 0), "RAD": ((), -2), "THTC": ((), -2),
    "D": ((7,), 0), "RDS": ((3,), 0), "DTM": ((), 1), "DQDXYZ": ((18,), -1), "SHOCK": ((), -2),
    "WT2": ((7,), 1),
}

STAGES = ["SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS", "UPDATE", "UPDATE_U"]
STAGE_ID = {n: i for i, n in enumerate(STAGES)}


def field_shape(name, ni, nj, nk):
    """numpy shape (Fortran order) of field `name` for a block with node counts ni,nj,nk."""
    comps, lb = FIELD_LAYOUT[name]
    ext = tuple(n + 2 - lb + 1 for n in (ni, nj, nk))
    return comps + ext


def bind_common(lib):
    """Declare argument types of the ABI functions on a loaded library."""
    vp = C.c_void_p
    lib.trans_create.argtypes = [C.POINTER(TransParams), C.c_int, C.POINTER(TransBlock), C.POINTER(vp)]
    lib.trans_destroy.argtypes = [vp]
    lib.trans_set_field.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_get_field.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_iterate.argtypes = [vp, C.c_int, C.POINTER(TransNorms)]
    lib.trans_run_stage.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    lib.trans_get_norms.argtypes = [vp, C.POINTER(TransNorms)]
    lib.trans_sync.argtypes = [vp]
    lib.trans_device_bytes.argtypes = [vp]
    lib.trans_device_bytes.restype = C.c_longlong
    lib.trans_kernel_launches.argtypes = [vp]
    lib.trans_kernel_launches.restype = C.c_longlong
    lib.trans_stage_times.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
    lib.trans_probe_fma_gflops.argtypes = [C.c_int]
    lib.trans_probe_fma_gflops.restype = C.c_double
    lib.trans_probe_chain_us.argtypes = [C.c_int, C.c_int]
    lib.trans_probe_chain_us.restype = C.c_double
    lib.trans_time_iterations.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(TransNorms)]
    lib.trans_update_static_scratch.argtypes = [vp, C.c_int, C.POINTER(TransNorms)]
    lib.trans_kernel_times.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int]
    lib.trans_kernel_class.argtypes = [C.c_int]
    lib.trans_kernel_class.restype = C.c_char_p
    lib.trans_batch_create.argtypes = [C.c_int, C.c_longlong, C.POINTER(vp)]
    lib.trans_batch_case_bytes.argtypes = [C.POINTER(TransParams), C.c_int, C.POINTER(TransBlock)]
    lib.trans_batch_case_bytes.restype = C.c_longlong
    lib.trans_batch_add.argtypes = [vp, C.POINTER(TransParams), C.c_int, C.POINTER(TransBlock), C.POINTER(C.c_int)]
    lib.trans_batch_remove.argtypes = [vp, C.c_int]
    lib.trans_batch_set_field.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_batch_get_field.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_batch_iterate.argtypes = [vp, C.c_int]
    lib.trans_batch_case_norms.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(TransNorms), C.POINTER(TransNorms)]
    lib.trans_batch_bytes_in_use.argtypes = [vp]
    lib.trans_batch_bytes_in_use.restype = C.c_longlong
    lib.trans_batch_cases.argtypes = [vp, C.POINTER(C.c_int), C.c_int]
    lib.trans_prepare.argtypes = [vp, C.c_int]
    lib.trans_batch_time_iterations.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
    lib.trans_get_integrals.argtypes = [vp, C.POINTER(TransIntegrals)]
    lib.trans_get_wall_cp.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_get_wall_forces.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_halo_pack.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_halo_unpack.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(TransConn), C.POINTER(C.c_double)]
    lib.trans_batch_get_integrals.argtypes = [vp, C.c_int, C.POINTER(TransIntegrals)]
    lib.trans_batch_integrals.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(TransIntegrals), C.c_int]
    lib.trans_batch_get_wall_cp.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.trans_block_metrics.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int),
                                        C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double)]
    lib.trans_wall_distance.argtypes = [C.c_longlong, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int),
                                        C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double)]
    PP = C.POINTER(C.POINTER(C.c_double))
    IP = C.POINTER(C.c_int)
    lib.trans_set_fields.argtypes = [vp, C.c_int, IP, IP, PP]
    lib.trans_get_fields.argtypes = [vp, C.c_int, IP, IP, PP]
    lib.trans_batch_set_fields.argtypes = [vp, C.c_int, C.c_int, IP, IP, PP]
    lib.trans_batch_get_fields.argtypes = [vp, C.c_int, C.c_int, IP, IP, PP]
    lib.trans_check_conversions.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]
    lib.trans_tuning.argtypes = [vp]
    lib.trans_tuning.restype = C.c_char_p
    lib.trans_last_error.argtypes = [vp]
    lib.trans_last_error.restype = C.c_char_p
    return lib


EXPORTED = ["trans_create", "trans_destroy", "trans_set_field", "trans_get_field", "trans_iterate",
            "trans_run_stage", "trans_get_norms", "trans_sync", "trans_device_bytes",
            "trans_kernel_launches", "trans_last_error", "trans_stage_times", "trans_probe_fma_gflops", "trans_probe_chain_us",
            "trans_time_iterations", "trans_update_static_scratch", "trans_tuning", "trans_kernel_times",
            "trans_kernel_class", "trans_batch_create", "trans_batch_case_bytes", "trans_batch_add",
            "trans_batch_remove", "trans_batch_set_field", "trans_batch_get_field", "trans_batch_iterate",
            "trans_batch_case_norms", "trans_batch_bytes_in_use", "trans_batch_cases", "trans_prepare",
            "trans_batch_time_iterations", "trans_get_integrals", "trans_get_wall_cp", "trans_get_wall_forces", "trans_halo_pack", "trans_halo_unpack",
            "trans_batch_get_integrals", "trans_batch_integrals", "trans_batch_get_wall_cp", "trans_wall_distance",
            "trans_set_fields", "trans_get_fields", "trans_batch_set_fields", "trans_batch_get_fields",
            "trans_block_metrics", "trans_check_conversions"]
TRANS_NKCLASS = 17
