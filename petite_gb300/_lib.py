"""ctypes binding of include/petite_gpu.h.

The engine has no CPU fallback: if the library is missing or a CUDA device
is absent, the calls that need it raise.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

N_PROC = 8
N_NS = 8

STATUS_NAMES = {0: "PT_OK", 1: "PT_NO_SAMPLE", 2: "PT_TIMEOUT", 3: "PT_BAD_TABLE", 4: "PT_OOM",
                5: "PT_CUDA_ERR", 6: "PT_BAD_ARG"}
PT_OK, PT_NO_SAMPLE, PT_TIMEOUT, PT_BAD_TABLE, PT_OOM, PT_CUDA_ERR, PT_BAD_ARG = range(7)

EXPORTS = ("pt_create", "pt_destroy", "pt_strerror", "pt_last_error_info", "pt_last_run_stats",
           "pt_last_kernel_times", "pt_alu_peaks", "pt_set_batch_tuning", "pt_run_sm", "pt_run_sm_noalloc", "pt_run_batch",
           "pt_sample_only", "pt_dsigma", "pt_moliere_inverse_cdf",
           "pt_vegas_accumulate", "pt_vegas_adapt", "pt_find_maxes",
           "pt_dark_create", "pt_dark_destroy", "pt_dark_dsigma", "pt_dark_sample_only", "pt_run_dark",
           "pt_run_batch_dark", "pt_dark_screen32",
           "pt_dark_yield", "pt_dark_yield_adjoint", "pt_detector_cut")

# pt_run_sm_noalloc: largest particle-store capacity (its static scratch)
NOALLOC_MAX_ROWS = 1 << 19


class PtTables(C.Structure):
    _fields_ = [
        ("map_base", C.c_int32 * N_PROC), ("map_rows", C.c_int32 * N_PROC), ("n_rows", C.c_int32),
        ("map_energy", C.c_void_p), ("map_maxF", C.c_void_p), ("map_neval", C.c_void_p),
        ("grid_offset", C.c_void_p), ("grid_ninc", C.c_void_p), ("grid_nodes", C.c_void_p),
        ("grid_f32x4", C.c_void_p), ("n_nodes", C.c_int64),
        ("ns_base", C.c_int32 * N_NS), ("ns_len", C.c_int32 * N_NS), ("ns_x", C.c_void_p), ("ns_y", C.c_void_p),
        ("ns_x32", C.c_void_p), ("ns_y32", C.c_void_p), ("ns_s32", C.c_void_p),
        ("ns_lnx0", C.c_float * N_NS), ("ns_invdlog", C.c_float * N_NS),
        ("map_energy32", C.c_void_p), ("map_cnorm32", C.c_void_p),
        ("map_lnE0", C.c_float * N_PROC), ("map_invdlog", C.c_float * N_PROC),
        ("Z", C.c_double), ("A", C.c_double), ("rho", C.c_double), ("dEdx_GeV_per_m", C.c_double),
        ("Eg_min", C.c_double), ("Ee_min", C.c_double),
        ("min_calc_electron", C.c_double), ("min_calc_positron", C.c_double),
        ("min_calc_muon", C.c_double), ("min_calc_photon", C.c_double),
        ("a0sq", C.c_double), ("Z2a04", C.c_double), ("Z23", C.c_double), ("Z13", C.c_double),
    ]


class PtParticles(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("p0", "r0", "pf", "rf", "weight", "mass", "pid", "gen", "proc",
                                          "bit", "primary", "draws", "parent", "pkey")] + [("capacity", C.c_int64)]


HIST_BINS = 100
N_COUNTS = 16
N_ESUM = 8


class PtTally(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("energy", C.c_void_p), ("hist", C.c_void_p),
                ("primary_count", C.c_void_p), ("primary_edep", C.c_void_p), ("z_max", C.c_double)]


class PtOpts(C.Structure):
    _fields_ = [("min_energy", C.c_double), ("max_n_integrators", C.c_int64), ("rescale_MCS", C.c_double),
                ("multiple_scattering", C.c_int32), ("precision", C.c_int32), ("seed", C.c_uint64),
                ("primary_offset", C.c_int64), ("mcs_mode", C.c_int32), ("loop_limit", C.c_int32)]


N_DARK = 4
DARK_MAX_MASSES = 8
DARK_BOUND = 4
TWOBODY = 4            # TwoBody_BSMDecay: active bit and yield slot
TWOBODY_CODE = 8       # its vectors' process code


class PtDarkMaps(C.Structure):
    _fields_ = [("n_masses", C.c_int32), ("mass", C.c_double * DARK_MAX_MASSES),
                ("map_base", C.c_int32 * (DARK_MAX_MASSES * N_DARK)), ("map_rows", C.c_int32 * (DARK_MAX_MASSES * N_DARK)),
                ("n_rows", C.c_int32), ("map_energy", C.c_void_p), ("map_maxF", C.c_void_p), ("map_neval", C.c_void_p),
                ("grid_offset", C.c_void_p), ("grid_ninc", C.c_void_p), ("grid_nodes", C.c_void_p),
                ("n_nodes", C.c_int64), ("Z", C.c_double), ("A", C.c_double), ("grid_f32x2", C.c_void_p)]


class PtDarkParams(C.Structure):
    _fields_ = [("mass_index", C.c_int32), ("bound_electron", C.c_int32), ("active", C.c_int32),
                ("mV", C.c_double), ("coupling", C.c_double), ("Zeff", C.c_double),
                ("E_res", C.c_double), ("E_compth", C.c_double), ("min_dark", C.c_double * 5),
                ("min_calc_photon", C.c_double),
                ("w_x", C.c_void_p * 4), ("w_y", C.c_void_p * 4), ("w_n", C.c_int32 * 4),
                ("dr_Ei", C.c_void_p * 4), ("dr_bins", C.c_void_p * 4), ("dr_nbins", C.c_void_p * 4),
                ("dr_n", C.c_int32 * 4), ("dr_nbmax", C.c_int32 * 4),
                ("nsc_lx", C.c_void_p), ("nsc_ly", C.c_void_p), ("nsc_n", C.c_int32),
                ("kinetic_mixing", C.c_double), ("ann_E0", C.c_double), ("ann_K", C.c_double),
                ("ii_x", C.c_void_p * 3), ("ii_y", C.c_void_p * 3), ("ii_n", C.c_int32 * 3), ("precision", C.c_int32)]


class PtDarkHist(C.Structure):
    _fields_ = [("counts", C.c_void_p), ("bins", C.c_int32), ("reserved0", C.c_int32), ("log10_lo", C.c_double),
                ("log10_hi", C.c_double)]


class PtDarkOut(C.Structure):
    _fields_ = [("p4", C.c_void_p), ("r", C.c_void_p), ("weight", C.c_void_p), ("parent", C.c_void_p),
                ("process", C.c_void_p), ("draws", C.c_void_p), ("capacity", C.c_int64),
                ("yield_", C.c_void_p), ("yield_E", C.c_void_p), ("hist", PtDarkHist)]


class PtTrainTarget(C.Structure):
    _fields_ = [("Eg_min", C.c_double), ("Ee_min", C.c_double), ("a0sq", C.c_double), ("Z2a04", C.c_double),
                ("mV", C.c_double), ("MT", C.c_double), ("Z", C.c_double), ("A", C.c_double)]


TRAIN_DARK = 16


class PtBatchTuning(C.Structure):
    _fields_ = [("refill_min", C.c_int32 * 2), ("chunk", C.c_int32 * 2), ("loop", C.c_int32), ("staging", C.c_int32),
                ("threads", C.c_int32), ("barrier_ns", C.c_int32), ("lanes", C.c_int32)]


class PetiteGPUError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_LIB = None


def library_path() -> str:
    return os.path.join(_build.LIBDIR, _build.LIBNAME)


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads (building first if needed) the CUDA library; raises if impossible."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build_if_missing and not _build.up_to_date(path):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"petite_gb300 CUDA library not built: {path}")
    lib = C.CDLL(path)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    lib.pt_create.argtypes = [C.POINTER(PtTables), C.POINTER(vp)]
    lib.pt_create.restype = C.c_int
    lib.pt_destroy.argtypes = [vp]
    lib.pt_destroy.restype = None
    lib.pt_strerror.argtypes = [C.c_int]
    lib.pt_strerror.restype = C.c_char_p
    lib.pt_last_error_info.argtypes = [vp, C.POINTER(i32), C.POINTER(C.c_double), C.POINTER(i32)]
    lib.pt_last_error_info.restype = C.c_int
    lib.pt_last_run_stats.argtypes = [vp, C.POINTER(i64), C.POINTER(i64)]
    lib.pt_last_run_stats.restype = C.c_int
    lib.pt_last_kernel_times.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.pt_last_kernel_times.restype = C.c_int
    lib.pt_alu_peaks.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), vp]
    lib.pt_alu_peaks.restype = C.c_int
    lib.pt_set_batch_tuning.argtypes = [vp, C.POINTER(PtBatchTuning)]
    lib.pt_set_batch_tuning.restype = C.c_int
    lib.pt_run_sm.argtypes = [vp, C.POINTER(PtParticles), i64, C.POINTER(PtOpts), C.POINTER(i64), vp]
    lib.pt_run_sm.restype = C.c_int
    lib.pt_run_sm_noalloc.argtypes = [vp, C.POINTER(PtParticles), i64, C.POINTER(PtOpts), C.POINTER(i64), vp]
    lib.pt_run_sm_noalloc.restype = C.c_int
    lib.pt_dark_create.argtypes = [vp, C.POINTER(PtDarkMaps), C.POINTER(vp)]
    lib.pt_dark_destroy.argtypes = [vp]
    lib.pt_dark_destroy.restype = None
    lib.pt_dark_dsigma.argtypes = [vp, i32, vp, vp, i64, C.c_double, vp, vp]
    lib.pt_dark_sample_only.argtypes = [vp, C.POINTER(PtDarkParams), i32, vp, vp, i64, C.POINTER(PtOpts), vp, vp, vp,
                                        vp]
    lib.pt_run_dark.argtypes = [vp, C.POINTER(PtDarkParams), C.POINTER(PtParticles), i64, C.POINTER(PtOpts),
                                C.POINTER(PtDarkOut), C.POINTER(i64), vp]
    lib.pt_dark_yield.argtypes = [vp, i32, vp, vp, vp, vp, i64, i64, C.c_uint64, vp, vp, vp]
    lib.pt_dark_yield_adjoint.argtypes = [vp, i32, vp, vp, vp, i64, i64, C.c_uint64, vp, vp, vp, vp]
    for f in ("pt_dark_create", "pt_dark_dsigma", "pt_dark_sample_only", "pt_run_dark", "pt_dark_yield",
              "pt_dark_yield_adjoint"):
        getattr(lib, f).restype = C.c_int
    lib.pt_run_batch.argtypes = [vp, vp, vp, vp, vp, i64, C.POINTER(PtOpts), C.POINTER(PtTally), i64, vp]
    lib.pt_run_batch.restype = C.c_int
    lib.pt_dark_screen32.argtypes = [vp, C.c_int32, vp, vp, i64, C.c_double, vp, vp, vp]
    lib.pt_dark_screen32.restype = C.c_int
    lib.pt_run_batch_dark.argtypes = [vp, vp, C.POINTER(PtDarkParams), C.c_int32, vp, vp, vp, vp, i64,
                                      C.POINTER(PtOpts), C.POINTER(PtTally), i64, vp, vp, C.POINTER(PtDarkHist),
                                      C.POINTER(i64), vp]
    lib.pt_run_batch_dark.restype = C.c_int
    lib.pt_sample_only.argtypes = [vp, i32, vp, vp, i64, C.POINTER(PtOpts), vp, vp, vp, vp]
    lib.pt_sample_only.restype = C.c_int
    lib.pt_dsigma.argtypes = [vp, i32, vp, vp, i64, i32, vp, vp]
    lib.pt_dsigma.restype = C.c_int
    lib.pt_detector_cut.argtypes = [vp, i64, vp, i64, vp, i64, vp, i32, C.c_double, C.c_double, i32, C.c_double,
                                    C.c_double, vp, vp, vp]
    lib.pt_detector_cut.restype = C.c_int
    lib.pt_moliere_inverse_cdf.argtypes = [vp, vp, i64, i32, vp, vp]
    lib.pt_moliere_inverse_cdf.restype = C.c_int
    i32p = C.POINTER(i32)                    # host arrays of increments per dimension
    lib.pt_vegas_accumulate.argtypes = [i32, C.POINTER(PtTrainTarget), vp, i32, i32, i32p, vp, i32, i64, C.c_uint64,
                                        i32, vp, vp, vp, vp]
    lib.pt_vegas_adapt.argtypes = [i32, i32, i32p, vp, i32, vp, vp, C.c_double, vp]
    lib.pt_find_maxes.argtypes = [i32, C.POINTER(PtTrainTarget), i32, vp, i32, i32, i32p, vp, i32, i32, i32,
                                  C.c_uint64, vp, vp, vp]
    for f in ("pt_vegas_accumulate", "pt_vegas_adapt", "pt_find_maxes"):
        getattr(lib, f).restype = C.c_int
    _LIB = lib
    return lib


def check(status: int, what: str = ""):
    if status != PT_OK:
        msg = load().pt_strerror(status).decode()
        raise PetiteGPUError(status, f"{what}: {msg}" if what else msg)
