"""ctypes mirror of include/sphmp.h (structs, enums, the exported symbol list).

Pure data definitions: importing this module loads nothing and needs no GPU.
"""
import ctypes as C

MAX_PHASES = 3
GRID_UNDEF = 0xFFFFFFFF
TYPE_FLUID = 0
TYPE_BOUNDARY = 1

# sphmp_status
OK = 0
ERR_INVALID_ARG = 1
ERR_CAPACITY = 2
ERR_CUDA = 3
ERR_UNSUPPORTED_TYPE = 4
ERR_NOT_FINITE = 5
ERR_CELL_OVERFLOW = 6
ERR_STATE = 7
ERR_NO_DEVICE = 8
ERR_BAD_MASS = 9
ERR_GRID = 10
ERR_TIMEOUT = 11
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "CAPACITY", 3: "CUDA", 4: "UNSUPPORTED_TYPE", 5: "NOT_FINITE",
    6: "CELL_OVERFLOW", 7: "STATE", 8: "NO_DEVICE", 9: "BAD_MASS", 10: "GRID", 11: "TIMEOUT",
}

# sphmp_eos / sphmp_schedule
EOS_TAIT = 0
EOS_LINEAR = 1
SCHEDULE_REFERENCE = 0
SCHEDULE_FUSED = 1
SCHEDULE_PROJECTU = 2
CELL_ORDER_LINEAR = 0
CELL_ORDER_MORTON = 1

# sphmp_field
F_POS, F_VEL, F_VELEVAL, F_PRESSURE, F_DENS, F_RESTDENS, F_VISC, F_ACCEL = range(8)
F_ALPHA, F_ALPHA_PRE, F_DRIFT, F_APREV, F_PMOD, F_TYPE, F_MASS, F_BORNID = range(8, 16)
F_MGCELL, F_MIDSORT, F_MGNDX, F_MGRIDOFF, F_MGRIDCNT = range(16, 21)
F_VELXCOR = 21
F_COUNT = 22

# the learned large-step corrector (include/sphmp_learned.h)
LC_FEATURES = 48
LC_HIDDEN = 128
LC_OUTPUTS = 4
LC_PARAMS = 39812

_f3 = C.c_float * 3


class Params(C.Structure):
    """sphmp_params: the reference ParamCarrier (464 bytes) followed by extensions."""

    _fields_ = [
        ("acclimit", C.c_float), ("vlimit", C.c_float), ("gravity", _f3), ("volmin", _f3),
        ("volmax", _f3), ("softminx", _f3), ("softmaxx", _f3),
        ("num", C.c_int32), ("maxNum", C.c_int32), ("dt", C.c_float), ("simscale", C.c_float),
        ("viscosity", C.c_float), ("restdensity", C.c_float), ("mass", C.c_float), ("radius", C.c_float),
        ("smoothradius", C.c_float), ("scalep", C.c_float),
        ("massArr", _f3), ("densArr", _f3), ("viscArr", _f3), ("boundstiff", C.c_float),
        ("kpoly6", C.c_float), ("kspiky", C.c_float), ("kspikydiff", C.c_float),
        ("klaplacian", C.c_float), ("kspline", C.c_float),
        ("bmass", C.c_float), ("bRestdensity", C.c_float), ("bvisc", C.c_float),
        ("cellsize", C.c_float), ("searchnum", C.c_int32), ("neighbornum", C.c_int32),
        ("neighborid", C.c_int32 * 27),
        ("gridmin", _f3), ("gridmax", _f3), ("gridsize", _f3), ("gridIdfac", _f3),
        ("gridres", C.c_int32 * 3), ("gridtotal", C.c_int32),
        ("mpmcellsize", C.c_float), ("mpmXmin", _f3), ("mpmXmax", _f3), ("mpmRes", C.c_int32 * 3),
        ("mpmNodeNum", C.c_int32), ("solidK", C.c_float), ("solidG", C.c_float),
        ("a_phi", C.c_float), ("a_psi", C.c_float), ("k_c", C.c_float), ("w_deltax", C.c_float),
        ("fijn", C.c_float), ("SFlipControl", C.c_float), ("LFlipControl", C.c_float),
        ("mpmSplitNum", C.c_int32), ("collisionStiff", C.c_float), ("surfaceTensionK", C.c_float),
        ("surfaceTensionFluidC", C.c_float), ("fBlending", C.c_float),
        # extensions
        ("nphase", C.c_int32), ("multiphase", C.c_int32), ("surface_tension", C.c_int32),
        ("eos", C.c_int32), ("eos_stiffness", C.c_float), ("mf_relax", C.c_float),
        ("mf_diffusion", C.c_float), ("mf_cont", C.c_float), ("mf_cont1", C.c_float),
        ("mf_cont2", C.c_float), ("mf_pintstiff", C.c_float), ("mf_omega", C.c_float),
        ("mf_visc_factor", C.c_float), ("cell_order", C.c_int32), ("bucket_window", C.c_int32),
        ("heavy_list", C.c_int32),
    ]

    def copy(self):
        other = Params()
        C.memmove(C.byref(other), C.byref(self), C.sizeof(Params))
        return other

    def as_dict(self):
        out = {}
        for name, typ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out

    @classmethod
    def from_dict(cls, d):
        p = cls()
        for name, typ in cls._fields_:
            if name not in d:
                continue
            v = d[name]
            if hasattr(getattr(p, name), "__len__"):
                arr = getattr(p, name)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(p, name, v)
        return p


assert C.sizeof(Params) == 464 + 64, C.sizeof(Params)
assert Params.fBlending.offset == 460


class DisplayPack(C.Structure):
    _fields_ = [("pos", _f3), ("color", C.c_float * 4), ("type", C.c_int32)]


class CalcPack(C.Structure):
    _fields_ = [
        ("vel", _f3), ("veleval", _f3), ("pressure", C.c_float), ("dens", C.c_float),
        ("restdens", C.c_float), ("mass", C.c_float), ("visc", C.c_float), ("bornid", C.c_int32),
        ("accel", _f3), ("deformGrad", C.c_float * 9), ("stress", C.c_float * 9), ("B", C.c_float * 9),
        ("solidG", C.c_float), ("solidK", C.c_float), ("X", _f3), ("invA", C.c_float * 9),
    ]


assert C.sizeof(DisplayPack) == 32
assert C.sizeof(CalcPack) == 224

# numpy structured dtypes with the same byte layout (for bulk AoS transfers)
def display_dtype():
    import numpy as np
    return np.dtype([("pos", "<f4", 3), ("color", "<f4", 4), ("type", "<i4")])


def calc_dtype():
    import numpy as np
    return np.dtype([
        ("vel", "<f4", 3), ("veleval", "<f4", 3), ("pressure", "<f4"), ("dens", "<f4"),
        ("restdens", "<f4"), ("mass", "<f4"), ("visc", "<f4"), ("bornid", "<i4"), ("accel", "<f4", 3),
        ("deformGrad", "<f4", 9), ("stress", "<f4", 9), ("B", "<f4", 9), ("solidG", "<f4"),
        ("solidK", "<f4"), ("X", "<f4", 3), ("invA", "<f4", 9),
    ])


# every symbol declared in include/sphmp.h, include/sphmp_learned.h and include/sphmp_legacy.h
EXPORTED_SYMBOLS = [
    "sphmp_params_default", "sphmp_setup_constants", "sphmp_setup_grid", "sphmp_add_fluid_volume",
    "sphmp_add_wall", "sphmp_add_open_box", "sphmp_boundary_spacing",
    "sphmp_create", "sphmp_destroy", "sphmp_set_params", "sphmp_get_params", "sphmp_set_stream",
    "sphmp_sync", "sphmp_num_particles", "sphmp_step_profile", "sphmp_upload_aos", "sphmp_download_aos", "sphmp_emit_aos",
    "sphmp_upload_field", "sphmp_download_field", "sphmp_get_particle_index", "sphmp_get_grid_list",
    "sphmp_rearrange_data", "sphmp_compute_boundary_density", "sphmp_compute_pressure",
    "sphmp_compute_drift_vel", "sphmp_compute_alpha_advance", "sphmp_compute_correction",
    "sphmp_compute_force", "sphmp_compute_force_projectu", "sphmp_advance", "sphmp_step", "sphmp_conservation",
    "sphmp_iisph_density", "sphmp_iisph_predict_advection", "sphmp_iisph_pressure_iteration",
    "sphmp_iisph_pressure_solve", "sphmp_iisph_integrate", "sphmp_step_iisph", "sphmp_autotune",
    "sphmp_device_errors", "sphmp_last_error", "sphmp_version", "sphmp_sort_cells_noalloc",
    "sphmp_write_frame_text", "sphmp_read_bi2", "sphmp_add_bi2_shape", "sphmp_save_state", "sphmp_load_state",
    "sphmp_download_display_async", "sphmp_download_wait", "sphmp_emit_disk", "sphmp_set_device_emitter",
    # the learned large-step corrector (include/sphmp_learned.h)
    "sphmp_corrector_create", "sphmp_corrector_destroy", "sphmp_corrector_set_params", "sphmp_corrector_get_params",
    "sphmp_corrector_set_normalisation", "sphmp_corrector_forward", "sphmp_corrector_gradients",
    "sphmp_corrector_train_step", "sphmp_corrector_sync", "sphmp_gemm_bf16_tn", "sphmp_step_large",
    "sphmp_learned_features", "sphmp_copy_state", "sphmp_compare_states", "sphmp_rollout",
    # reference entry-point names (include/sphmp_legacy.h)
    "cudaInit", "cudaExit", "FluidClearCUDA", "FluidSetupCUDA", "GetParticleIndexCUDA",
    "GetGridListCUDA", "RearrageDataCUDA", "InitialSortCUDA", "SortGridCUDA", "CountingSortFullCUDA_", "MfComputePressureCUDA", "MfComputeDriftVelCUDA",
    "MfComputeAlphaAdvanceCUDA", "MfComputeCorrectionCUDA", "MfComputeForceCUDA", "ComputeForceCUDA_ProjectU",
    "MfAdvanceCUDA", "ComputeDensityIISPH_CUDA", "PredictAdvection", "PressureSolve", "Integration",
    "ComputeBoundaryDensity", "computeNumBlocks", "sphmp_legacy_context", "TransferToCUDA",
    "TransferFromCUDA", "EmitUpdateCUDA",
]


class Bi2Info(C.Structure):
    """sphmp_bi2_info: header of a BINX-020 (.bi2) particle file."""
    _fields_ = [("fmt", C.c_int32), ("bitorder", C.c_int32), ("full", C.c_int32), ("data2d", C.c_int32),
                ("dp", C.c_float), ("h", C.c_float), ("b", C.c_float), ("rhop0", C.c_float), ("gamma", C.c_float),
                ("massbound", C.c_float), ("massfluid", C.c_float), ("time", C.c_float),
                ("np", C.c_int32), ("nfixed", C.c_int32), ("nmoving", C.c_int32), ("nfloat", C.c_int32),
                ("nfluidout", C.c_int32), ("nbound", C.c_int32), ("nfluid", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    """sphmp_tuning (include/sphmp.h): the autotuner's choice and its step times."""
    _fields_ = [("cell_order", C.c_int32), ("bucket_window", C.c_int32), ("heavy_list", C.c_int32),
                ("trials", C.c_int32), ("ms_per_step", C.c_float), ("ms_before", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RolloutStats(C.Structure):
    """sphmp_rollout_stats (include/sphmp_learned.h)."""
    _fields_ = [("large_steps", C.c_int32), ("plain_steps", C.c_int32), ("audits", C.c_int32),
                ("fallbacks", C.c_int32), ("density_err_max", C.c_double), ("alpha_err_max", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Emitter(C.Structure):
    """sphmp_emitter: a disk emitter (position, unit direction, speed, radius, lattice spacing)."""
    _fields_ = [("position", C.c_float * 3), ("dir", C.c_float * 3), ("vel", C.c_float), ("radius", C.c_float),
                ("spacing", C.c_float)]
