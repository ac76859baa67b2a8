"""ctypes mirror of the C-ABI (include/tsr_capi.h) and of the reference's
hot-path structs (include/tsr_types.h, field for field the reference's
include/macro_mesh.h, micro_mesh.h, Keff.h, soil.h, user_data.h,
exprem_options.h and exprem_stats.h).

The library is loaded from the package directory (built in tree by
``twoscalerich_gb300.build``).  There is no fallback: if the shared library
is missing, importing the GPU entry points raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtsr_gb300.so")

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
fp = C.POINTER(C.c_float)


class MacroMesh(C.Structure):
    _fields_ = [
        ("no_verts", C.c_int), ("no_nodes", C.c_int), ("no_elements", C.c_int),
        ("elements", ip), ("nodes", dp), ("shape_funcs", dp), ("normals", dp),
        ("boundary_edge_midpts", dp), ("boundary_edge_normals", dp),
        ("boundary_edge_lens", dp), ("boundary_condition_edges", ip),
        ("CV_area", dp), ("SCV_area", dp), ("midx", dp), ("midy", dp),
        ("centroid_elements", dp),
    ]


class MicroMesh(C.Structure):
    _fields_ = [
        ("no_nodes", C.c_int), ("no_elements", C.c_int), ("elements", ip),
        ("boundary_nodes", ip), ("nodes", dp), ("shape_funcs", dp), ("normals", dp),
        ("boundary_edges", ip), ("boundary_edge_midpts", dp),
        ("boundary_edge_normals", dp), ("boundary_edge_lens", dp),
        ("centroid_elements", dp), ("CV_area", dp), ("midx", dp), ("midy", dp),
        ("cell_area", C.c_double), ("vectors", dp), ("no_verts", C.c_int),
        ("element_area", dp),
    ]


class Keff(C.Structure):
    _fields_ = [
        ("epsilonA", C.c_double), ("no_hvalues", C.c_int), ("logr", C.c_double),
        ("logh_first", C.c_double), ("logh_values", dp), ("Keff_values", dp),
    ]


class Soil(C.Structure):
    _fields_ = [("Ksat", C.c_double), ("thetar", C.c_double), ("thetas", C.c_double),
                ("alpha", C.c_double), ("n", C.c_double), ("m", C.c_double)]


class UserData(C.Structure):
    _fields_ = [
        ("macro_mesh", MacroMesh), ("micro_mesh", MicroMesh),
        ("effective_conductivity", Keff), ("soilA", Soil), ("soilB", Soil),
        ("boundary_flux", C.c_double), ("N", C.c_int), ("model_type", C.c_int),
        ("NUM_THREADS", C.c_uint),
    ]


class ExpremOptions(C.Structure):
    _fields_ = [
        ("AbsTol", C.c_double), ("RelTol", C.c_double), ("MinKrylov", C.c_int),
        ("MaxKrylov", C.c_int), ("MinStep", C.c_double), ("MaxStep", C.c_double),
        ("MaxNumSteps", C.c_int), ("SafetyFac", C.c_double), ("MinStepDecFac", C.c_double),
        ("MaxStepIncFac", C.c_double), ("InitStep", C.c_double),
    ]


class ExpremStats(C.Structure):
    _fields_ = [
        ("CurrentStep", C.c_double), ("CurrentTime", C.c_double), ("CurrentKryDim", C.c_int),
        ("CurrentSoln", dp), ("NumSteps", C.c_int), ("FuncEvals", C.c_int),
    ]


class ModelExt(C.Structure):
    _fields_ = [
        ("dirichlet_h", C.c_double), ("specific_storage", C.c_double),
        ("kface_mode", C.c_int), ("n_templates", C.c_int), ("cell_scale", dp),
        ("templates", C.POINTER(MicroMesh)), ("cell_template", ip),
        ("cell_soilB", C.POINTER(Soil)), ("scenarios", C.c_int), ("reserved2", C.c_int),
        ("scen_soilA", C.POINTER(Soil)), ("scen_keff_scale", dp),
        ("cell_learned", ip), ("closure_coef", dp),
    ]


# status codes (include/tsr_capi.h)
TSR_OK = 0
STATUS_NAMES = {0: "OK", 1: "CUDA", 2: "NAN", 3: "BOUNDS", 4: "TIMEOUT", 5: "ARG", 6: "ALLOC",
                7: "SINGULAR", 8: "MINSTEP", 9: "MAXSTEPS", 10: "GFUNC", 11: "IO"}

# every symbol include/tsr_capi.h declares, with its ctypes signature
_SIGNATURES = {
    "tsr_version": (C.c_int, []),
    "tsr_last_error_message": (C.c_char_p, []),
    "tsr_macro_mesh_properties": (C.c_int, [C.c_char_p, C.POINTER(MacroMesh), ip]),
    "tsr_macro_mesh_build": (C.c_int, [C.c_int, C.c_int, dp, C.c_int, ip, C.c_int, ip, ip,
                                       C.POINTER(MacroMesh)]),
    "tsr_macro_mesh_build_device": (C.c_int, [C.c_int, C.c_int, dp, C.c_int, ip, C.c_int, ip, ip,
                                       C.POINTER(MacroMesh)]),
    "tsr_micro_mesh_properties": (C.c_int, [C.c_char_p, C.POINTER(MicroMesh)]),
    "tsr_micro_mesh_build": (C.c_int, [C.c_double, C.c_double, C.c_int, C.c_int, dp, C.c_int,
                                       ip, C.c_int, ip, C.POINTER(MicroMesh)]),
    "tsr_read_effective_conductivity": (C.c_int, [C.c_char_p, C.POINTER(Keff)]),
    "tsr_set_exprem_options": (C.c_int, [C.POINTER(ExpremOptions)]),
    "tsr_macro_mesh_free": (None, [C.POINTER(MacroMesh)]),
    "tsr_micro_mesh_free": (None, [C.POINTER(MicroMesh)]),
    "tsr_keff_free": (None, [C.POINTER(Keff)]),
    "tsr_phipade": (C.c_int, [dp, dp, C.c_double, C.c_int, C.c_int]),
    "tsr_calibrate_micro_boundary": (C.c_int, [C.POINTER(UserData), C.POINTER(ModelExt), dp]),
    "tsr_init": (C.c_void_p, [C.POINTER(UserData), C.POINTER(ModelExt), C.c_void_p, C.c_int]),
    "tsr_free": (None, [C.c_void_p]),
    "tsr_stream": (C.c_void_p, [C.c_void_p]),
    "tsr_num_unknowns": (C.c_int, [C.c_void_p]),
    "tsr_g_eval": (C.c_int, [C.c_void_p, dp, dp]),
    "tsr_g_eval_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "tsr_jv": (C.c_int, [C.c_void_p, dp, dp, dp, C.c_double, dp]),
    "tsr_jv_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                C.c_void_p]),
    "tsr_water_content": (C.c_int, [C.c_void_p, dp, dp]),
    "tsr_dot": (C.c_int, [C.c_void_p, dp, dp, C.c_int, dp]),
    "tsr_exprem_step": (C.c_int, [C.c_void_p, dp, C.c_double, dp, dp, dp,
                                  C.POINTER(ExpremOptions), C.POINTER(ExpremStats)]),
    "tsr_exprem_load": (C.c_int, [C.c_void_p, dp, C.c_double]),
    "tsr_exprem_advance": (C.c_int, [C.c_void_p, C.c_double, dp, dp, C.POINTER(ExpremOptions),
                                     C.POINTER(ExpremStats), dp]),
    "tsr_exprem_store": (C.c_int, [C.c_void_p, dp]),
    "tsr_checkpoint_save": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(ExpremStats)]),
    "tsr_checkpoint_load": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(ExpremStats)]),
    "tsr_num_scenarios": (C.c_int, [C.c_void_p]),
    "tsr_scenario_range": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_longlong)]),
    "tsr_ensemble_advance": (C.c_int, [C.c_void_p, C.c_double, dp, C.POINTER(dp),
                                       C.POINTER(ExpremOptions), C.POINTER(ExpremStats), dp,
                                       C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "tsr_ensemble_water": (C.c_int, [C.c_void_p, dp, dp]),
    "tsr_ensemble_load": (C.c_int, [C.c_void_p, dp, dp]),
    "tsr_gfunc_gpu": (C.c_int, [dp, dp, C.POINTER(UserData)]),
    "tsr_set_default_ext": (C.c_int, [C.POINTER(ModelExt), C.c_int]),
    "tsr_release_all": (None, []),
    "tsr_autotune": (C.c_int, [C.c_void_p, dp, C.c_int, dp, ip, ip]),
    "tsr_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "tsr_profile_read": (C.c_int, [C.c_void_p, C.c_int, dp, C.POINTER(C.c_longlong), dp]),
    "tsr_kernel_launches": (C.c_ulonglong, []),
    "tsr_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "tsr_set_fused_gs": (C.c_int, [C.c_void_p, C.c_int]),
    "tsr_set_gram_schmidt": (C.c_int, [C.c_void_p, C.c_int]),
    "tsr_set_calibrated_output": (C.c_int, [C.c_void_p, C.c_int]),
    "tsr_step_diagnostics": (C.c_int, [C.c_void_p, C.c_int, dp]),
    "tsr_cell_plan": (C.c_int, [C.c_void_p, ip]),
    "tsr_set_cell_plan": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "tsr_keff_homogenize": (C.c_int, [C.POINTER(MicroMesh), C.c_double, C.c_double, C.c_int, C.c_double,
                                      C.POINTER(Soil), C.c_double, C.c_double, C.c_double, C.c_int,
                                      dp, dp, dp]),
    "tsr_calibrate_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "tsr_save_solution": (C.c_int, [C.c_char_p, dp, dp, C.c_int, C.POINTER(UserData)]),
    "tsr_wait_probe": (C.c_int, [C.c_int]),
    "tsr_fp64_peak": (C.c_int, [dp]),
    "tsr_mark": (C.c_int, [C.c_void_p, C.c_int]),
    "tsr_elapsed_ms": (C.c_int, [C.c_void_p, C.c_int, C.c_int, dp]),
    "tsr_sync": (C.c_int, [C.c_void_p]),
    "tsr_pinned_alloc": (C.c_void_p, [C.c_size_t]),
    "tsr_pinned_free": (None, [C.c_void_p]),
    "tsr_mlp_num_params": (C.c_int, []),
    "tsr_mlp_create": (C.c_void_p, []),
    "tsr_mlp_free": (None, [C.c_void_p]),
    "tsr_mlp_set_params": (C.c_int, [C.c_void_p, fp]),
    "tsr_mlp_get_params": (C.c_int, [C.c_void_p, fp]),
    "tsr_mlp_forward": (C.c_int, [C.c_void_p, fp, C.c_int, fp, C.c_int]),
    "tsr_mlp_grad": (C.c_int, [C.c_void_p, fp, fp, C.c_int, fp, fp]),
    "tsr_mlp_set_data": (C.c_int, [C.c_void_p, fp, fp, C.c_longlong]),
    "tsr_mlp_train": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_ulonglong, fp]),
    "tsr_mlp_adamw_step": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "tsr_closure_set_learned": (C.c_int, [C.c_void_p, ip]),
    "tsr_closure_set_coef": (C.c_int, [C.c_void_p, dp]),
    "tsr_closure_read": (C.c_int, [C.c_void_p, ip, dp, ip]),
    "tsr_closure_attach": (C.c_int, [C.c_void_p, C.c_void_p, dp, fp, C.c_double, C.c_double, C.c_int]),
    "tsr_closure_attach_ensemble": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double]),
    "tsr_closure_update": (C.c_int, [C.c_void_p, ip]),
    "tsr_closure_advance": (C.c_int, [C.c_void_p, C.c_double, dp, dp, C.POINTER(ExpremOptions),
                                      C.POINTER(ExpremStats), dp, ip]),
    "tsr_cell_summary": (C.c_int, [C.c_void_p, dp, dp]),
    "tsr_dot_device_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_void_p]),
}

_lib = None


def load():
    """Load libtsr_gb300.so (raises OSError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libtsr_gb300.so is not built; run twoscalerich_gb300.build.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def declared_symbols():
    return sorted(_SIGNATURES)


def ptr(a):
    """double* / int* of a contiguous numpy array (or NULL for None)."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array passed to the C-ABI must be C-contiguous")
    if a.dtype == np.float64:
        return a.ctypes.data_as(dp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(ip)
    raise TypeError("unsupported dtype %s" % a.dtype)


def last_error():
    return load().tsr_last_error_message().decode()


class TsrError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        super().__init__("%s failed: %s (%s)" % (where, STATUS_NAMES.get(code, code), last_error()))


def check(code, where):
    if code != TSR_OK:
        raise TsrError(code, where)
    return code


def as_array(p, n, dtype=np.float64):
    """Copy n items behind a ctypes pointer into a numpy array."""
    if n == 0:
        return np.zeros(0, dtype)
    ct = C.c_double if dtype == np.float64 else C.c_int
    buf = C.cast(p, C.POINTER(ct * n)).contents
    return np.frombuffer(buf, dtype=dtype, count=n).copy()


class PinnedArray:
    """A float64 numpy view of page-locked host memory (cudaMallocHost)."""

    def __init__(self, n):
        lib = load()
        self._p = lib.tsr_pinned_alloc(8 * n)
        if not self._p:
            raise MemoryError("tsr_pinned_alloc(%d) failed: %s" % (8 * n, last_error()))
        buf = (C.c_double * n).from_address(self._p)
        self.a = np.frombuffer(buf, dtype=np.float64, count=n)

    def free(self):
        if self._p:
            self.a = None
            load().tsr_pinned_free(self._p)
            self._p = None
