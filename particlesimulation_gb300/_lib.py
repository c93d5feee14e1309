"""ctypes binding of ``libpmgb.so`` (include/pmgb.h).

There is no fallback: if the CUDA library is missing the import of a method fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libpmgb.so")

PMGB_OK, PMGB_EINVAL, PMGB_ECUDA, PMGB_EESCAPED, PMGB_ETIMEOUT, PMGB_ENOMEM = range(6)
UNITS_CODE, UNITS_ORIGINAL = 0, 1
DIAG_WIDTH = 12  # PMGB_DIAG_WIDTH

# Every symbol declared in include/pmgb.h (checked by tests/test_abi.py).
EXPORTS = [
    "pmgb_pm_create", "pmgb_pm_destroy", "pmgb_pm_init_greens_function", "pmgb_pm_method_step",
    "pmgb_pm_run", "pmgb_pm_advance", "pmgb_pm_get_particles", "pmgb_pm_set_particles", "pmgb_pm_escaped",
    "pmgb_pm_get_density", "pmgb_pm_get_potential", "pmgb_pm_get_greens_function",
    "pmgb_pm_stage_times", "pmgb_pm_size", "pmgb_pm_set_diagnostics", "pmgb_pm_get_diagnostics",
    "pmgb_recorder_create", "pmgb_recorder_destroy", "pmgb_recorder_flush",
    "pmgb_recorder_frames_written", "pmgb_pm_run_recorded", "pmgb_sample_plummer",
    "pmgb_sample_disk_linear",
    "pmgb_p3m_create", "pmgb_p3m_destroy",
    "pmgb_p3m_force", "pmgb_p3m_run", "pmgb_p3m_get_cell_lists", "pmgb_p3m_get_sr_table",
    "pmgb_p3m_pair_count", "pmgb_fp32_peak_probe", "pmgb_kernel_launches",
    "pmgb_chaining_mesh_fill_noalloc", "pmgb_p3m_set_pair_counting", "pmgb_p3m_set_symmetric",
    "pmgb_p3m_get_symmetric", "pmgb_p3m_get_subcolumns",
    "pmgb_closure_create", "pmgb_closure_destroy", "pmgb_closure_set_mode", "pmgb_closure_get_mode",
    "pmgb_closure_collect", "pmgb_closure_train", "pmgb_closure_param_count",
    "pmgb_closure_get_params", "pmgb_closure_set_params", "pmgb_closure_judge", "pmgb_closure_run",
    "pmgb_closure_features", "pmgb_closure_scales", "pmgb_mlp_eval", "pmgb_mlp_gradients",
    "pmgb_tc_wait_probe",
    "pmgb_ensemble_create", "pmgb_ensemble_destroy", "pmgb_ensemble_run", "pmgb_ensemble_advance",
    "pmgb_ensemble_get_particles", "pmgb_ensemble_tuning", "pmgb_ensemble_size",
    "pmgb_pm_get_stream", "pmgb_direct_sum_fp64", "pmgb_fft3d",
    "pmgb_leapfrog", "pmgb_pm_leapfrog", "pmgb_pm_get_integer_step_velocities",
    "pmgb_pm_total_external_force",
    "pmgb_last_error", "pmgb_version",
]


class ExternalField(C.Structure):
    _fields_ = [("kind", C.c_int), ("center", C.c_float * 3), ("R", C.c_float), ("M", C.c_float),
                ("G", C.c_float)]


class PMConfigC(C.Structure):
    _fields_ = [
        ("grid", C.c_int * 3), ("box", C.c_float * 3), ("H", C.c_float), ("DT", C.c_float),
        ("G", C.c_float), ("interpolation", C.c_int), ("finite_diff", C.c_int),
        ("greens", C.c_int), ("particle_diameter", C.c_float), ("ext", ExternalField),
        ("sort_interval", C.c_int), ("periodic", C.c_int),
    ]


class P3MConfigC(C.Structure):
    _fields_ = [
        ("comp_box", C.c_float * 3), ("cutoff", C.c_float), ("particle_diameter", C.c_float),
        ("softening", C.c_float), ("cloud_shape", C.c_int), ("use_table", C.c_int),
        ("y_sorting", C.c_int),
    ]


_lib = None


def lib() -> C.CDLL:
    """The loaded CUDA library; raises if it was not built (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int)
        L.pmgb_pm_create.argtypes = [C.POINTER(PMConfigC), C.c_int, fp, fp, C.POINTER(vp)]
        L.pmgb_pm_destroy.argtypes = [vp]
        L.pmgb_pm_init_greens_function.argtypes = [vp]
        L.pmgb_pm_method_step.argtypes = [vp]
        L.pmgb_pm_run.argtypes = [vp, C.c_int, ip]
        L.pmgb_pm_advance.argtypes = [vp, C.c_int, ip, fp]
        L.pmgb_pm_get_particles.argtypes = [vp, fp, fp, fp, C.c_int]
        L.pmgb_pm_set_particles.argtypes = [vp, fp, fp, C.c_int]
        L.pmgb_pm_escaped.argtypes = [vp, ip]
        L.pmgb_pm_get_density.argtypes = [vp, fp]
        L.pmgb_pm_get_potential.argtypes = [vp, fp]
        L.pmgb_pm_get_greens_function.argtypes = [vp, fp]
        L.pmgb_pm_stage_times.argtypes = [vp, fp]
        L.pmgb_pm_size.argtypes = [vp, ip, ip]
        L.pmgb_pm_set_diagnostics.argtypes = [vp, C.c_int]
        L.pmgb_pm_get_diagnostics.argtypes = [vp, C.POINTER(C.c_double), C.c_int, ip]
        L.pmgb_recorder_create.argtypes = [C.c_int, C.c_int, C.c_char_p, C.POINTER(C.c_char_p),
                                           C.c_int, C.POINTER(vp)]
        L.pmgb_recorder_destroy.argtypes = [vp]
        L.pmgb_recorder_flush.argtypes = [vp, C.c_char_p, C.c_int]
        L.pmgb_recorder_frames_written.argtypes = [vp, C.POINTER(C.c_longlong)]
        L.pmgb_pm_run_recorded.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, ip]
        L.pmgb_sample_plummer.argtypes = [C.c_uint, C.c_ulonglong, fp, C.c_float, C.c_float, C.c_float,
                                          C.c_float, C.c_int, fp]
        L.pmgb_sample_disk_linear.argtypes = [C.c_uint, C.c_ulonglong, fp, C.c_float, C.c_float, C.c_float,
                                              C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, fp]
        L.pmgb_p3m_create.argtypes = [vp, C.POINTER(P3MConfigC), C.POINTER(vp)]
        L.pmgb_p3m_destroy.argtypes = [vp]
        L.pmgb_p3m_force.argtypes = [vp]
        L.pmgb_p3m_run.argtypes = [vp, C.c_int, ip]
        L.pmgb_p3m_get_cell_lists.argtypes = [vp, ip, ip, ip]
        L.pmgb_p3m_get_sr_table.argtypes = [vp, fp, fp]
        L.pmgb_p3m_pair_count.argtypes = [vp, C.POINTER(C.c_ulonglong)]
        L.pmgb_fp32_peak_probe.argtypes = [fp]
        L.pmgb_kernel_launches.argtypes = [C.POINTER(C.c_longlong)]
        L.pmgb_chaining_mesh_fill_noalloc.argtypes = [vp, C.c_int, C.POINTER(P3MConfigC), C.c_float,
                                                      vp, vp, ip, vp]
        L.pmgb_p3m_set_pair_counting.argtypes = [vp, C.c_int]
        L.pmgb_p3m_set_symmetric.argtypes = [vp, C.c_int]
        L.pmgb_p3m_get_symmetric.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_uint)]
        L.pmgb_p3m_get_subcolumns.argtypes = [vp, C.POINTER(C.c_int)]
        L.pmgb_closure_create.argtypes = [vp, C.POINTER(P3MConfigC), C.c_float, C.c_int,
                                          C.c_ulonglong, C.POINTER(vp)]
        L.pmgb_closure_destroy.argtypes = [vp]
        L.pmgb_closure_set_mode.argtypes = [vp, C.c_int]
        L.pmgb_closure_get_mode.argtypes = [vp, ip]
        L.pmgb_closure_collect.argtypes = [vp, C.c_int, ip]
        L.pmgb_closure_train.argtypes = [vp, C.c_int, C.c_int, C.c_float, fp]
        L.pmgb_closure_get_params.argtypes = [vp, fp, C.c_int]
        L.pmgb_closure_set_params.argtypes = [vp, fp, C.c_int]
        L.pmgb_closure_judge.argtypes = [vp, C.c_int, fp]
        L.pmgb_closure_run.argtypes = [vp, C.c_int, C.c_float, C.c_int, C.c_int, ip, ip, fp]
        L.pmgb_closure_features.argtypes = [vp, fp, fp]
        L.pmgb_closure_scales.argtypes = [vp, fp, ip]
        L.pmgb_mlp_eval.argtypes = [fp, C.c_int, fp, fp]
        L.pmgb_mlp_gradients.argtypes = [fp, C.c_int, fp, fp, fp, fp]
        L.pmgb_tc_wait_probe.argtypes = [C.c_int, C.c_int]
        L.pmgb_ensemble_create.argtypes = [C.c_int, C.POINTER(PMConfigC), ip, C.POINTER(fp),
                                           C.POINTER(fp), C.POINTER(vp)]
        L.pmgb_ensemble_destroy.argtypes = [vp]
        L.pmgb_ensemble_run.argtypes = [vp, C.c_int, ip, fp]
        L.pmgb_ensemble_advance.argtypes = [vp, C.c_int, fp]
        L.pmgb_ensemble_get_particles.argtypes = [vp, C.c_int, fp, fp, fp, C.c_int]
        L.pmgb_ensemble_tuning.argtypes = [vp, ip, ip, fp]
        L.pmgb_ensemble_size.argtypes = [vp, ip, C.POINTER(C.c_longlong)]
        L.pmgb_pm_get_stream.argtypes = [vp, C.POINTER(vp)]
        dp = C.POINTER(C.c_double)
        L.pmgb_direct_sum_fp64.argtypes = [C.c_int, fp, fp, C.c_double, C.c_double, C.c_int, ip,
                                           C.c_double, dp]
        L.pmgb_fft3d.argtypes = [C.c_int, C.c_int, C.c_int, fp, fp, C.c_int]
        L.pmgb_leapfrog.argtypes = [C.c_int, C.c_int, fp, fp, fp, fp, C.c_float]
        L.pmgb_pm_leapfrog.argtypes = [vp, C.c_int, C.c_float]
        L.pmgb_pm_get_integer_step_velocities.argtypes = [vp, fp, C.c_int]
        L.pmgb_pm_total_external_force.argtypes = [vp, fp]
        L.pmgb_last_error.restype = C.c_char_p
        L.pmgb_version.restype = C.c_char_p
        _lib = L
    return _lib


class PMGBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pmgb error {code}: {msg}")
        self.code = code


def check(rc: int) -> int:
    """Raise like the reference: bad arguments -> ValueError (std::invalid_argument), CUDA
    failures -> PMGBError.  PMGB_EESCAPED is not an error (the reference prints and stops)."""
    if rc in (PMGB_OK, PMGB_EESCAPED):
        return rc
    msg = lib().pmgb_last_error().decode(errors="replace")
    if rc == PMGB_EINVAL:
        raise ValueError(msg)
    raise PMGBError(rc, msg)
