"""CPU oracle of the two-scale hot path -- TEST INFRASTRUCTURE ONLY.

Loaded by the tests, by the smoke check and by the CPU-baseline leg of the
benchmark; never by the library.  ``load()`` returns the oracle built from
tsr_oracle.c; ``load_ref()`` the reference's own sources compiled by
``make -C oracle ref`` (present only where the reference tree is).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "libtsr_oracle.so")
# same source built with the C library's log/exp (used to time the CPU baseline)
ORACLE_LIBM_LIB = os.path.join(HERE, "libtsr_oracle_libm.so")
REF_LIB = os.path.join(HERE, "_ref", "libtsr_ref.so")

_o = None
_om = None
_r = None


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args


def load(libm=False):
    """The bitwise oracle, or (libm=True) its C-library-math build."""
    global _o, _om
    if (_om if libm else _o) is None:
        from twoscalerich_gb300 import capi
        path = ORACLE_LIBM_LIB if libm else ORACLE_LIB
        if not os.path.exists(path):
            raise OSError("oracle not built (make -C oracle oracle)")
        lib = C.CDLL(path)
        dp, vp = capi.dp, C.c_void_p
        _sig(lib, "oracle_create", vp, [C.POINTER(capi.UserData), C.POINTER(capi.ModelExt)])
        _sig(lib, "oracle_destroy", None, [vp])
        _sig(lib, "oracle_num_unknowns", C.c_long, [vp])
        _sig(lib, "oracle_g", C.c_int, [vp, dp, dp, C.c_int])
        _sig(lib, "oracle_jv", C.c_int, [vp, dp, dp, dp, C.c_double, dp, C.c_int])
        _sig(lib, "oracle_water", C.c_int, [vp, dp, dp])
        _sig(lib, "oracle_water_scenarios", C.c_int, [vp, dp, dp])
        _sig(lib, "oracle_cell_summary", C.c_int, [vp, dp, dp, dp])
        _sig(lib, "oracle_vg_head", C.c_double, [C.POINTER(capi.Soil), C.c_double])
        _sig(lib, "oracle_dot", C.c_double, [dp, dp, C.c_long])
        _sig(lib, "oracle_vsum", C.c_double, [dp, C.c_long])
        _sig(lib, "oracle_wsq", C.c_double, [dp, dp, C.c_long])
        _sig(lib, "oracle_phipade", C.c_int, [dp, dp, C.c_double, C.c_int, C.c_int, C.c_int])
        _sig(lib, "oracle_exprem_step", C.c_int, [vp, dp, C.c_double, dp, dp, dp,
                                                  C.POINTER(capi.ExpremOptions),
                                                  C.POINTER(capi.ExpremStats), C.c_int])
        _sig(lib, "oracle_set_gram_schmidt", C.c_int, [vp, C.c_int])
        for f in ("log", "exp", "expm1", "log1p"):
            _sig(lib, "oracle_math_" + f, C.c_double, [C.c_double])
        _sig(lib, "oracle_math_log1p_unit", C.c_double, [C.c_double, dp])
        ip = capi.ip
        _sig(lib, "oracle_macro_mesh_build", C.c_int,
             [C.c_int, C.c_int, dp, C.c_int, ip, C.c_int, ip, ip, C.POINTER(capi.MacroMesh)])
        _sig(lib, "oracle_micro_mesh_build", C.c_int,
             [C.c_double, C.c_double, C.c_int, C.c_int, dp, C.c_int, ip, C.c_int, ip,
              C.POINTER(capi.MicroMesh)])
        _sig(lib, "oracle_macro_mesh_free", None, [C.POINTER(capi.MacroMesh)])
        _sig(lib, "oracle_micro_mesh_free", None, [C.POINTER(capi.MicroMesh)])
        _sig(lib, "oracle_set_exprem_options", C.c_int, [C.POINTER(capi.ExpremOptions)])
        _sig(lib, "oracle_math_div_many", None, [dp, dp, dp, C.c_long])
        _sig(lib, "oracle_vg", None, [C.POINTER(capi.Soil), C.c_double, C.c_double, dp])
        _sig(lib, "oracle_keff", None, [C.POINTER(capi.Keff), C.c_double, dp])
        _sig(lib, "oracle_dirichlet_mask", C.c_int, [vp, C.POINTER(C.c_ubyte)])
        if libm:
            _om = lib
        else:
            _o = lib
    return _om if libm else _o


class MeshLib:
    """The oracle's mesh preprocessing and solver defaults under the names
    the problem builder calls (twoscalerich_gb300.problem, argument `lib`):
    problems built with it load nothing of the GB300 library."""

    def __init__(self, libm=False):
        lib = load(libm)
        self.tsr_macro_mesh_build = lib.oracle_macro_mesh_build
        self.tsr_micro_mesh_build = lib.oracle_micro_mesh_build
        self.tsr_macro_mesh_free = lib.oracle_macro_mesh_free
        self.tsr_micro_mesh_free = lib.oracle_micro_mesh_free
        self.tsr_set_exprem_options = lib.oracle_set_exprem_options

    @staticmethod
    def tsr_keff_free(keff):
        raise RuntimeError("the oracle builds no Keff table from files")


def load_ref():
    """The reference's own phipade / mesh / Keff / options / writer, or None."""
    global _r
    if _r is None:
        if not os.path.exists(REF_LIB):
            return None
        from twoscalerich_gb300 import capi
        lib = C.CDLL(REF_LIB)
        dp = capi.dp
        _sig(lib, "ref_macro_mesh_properties", C.c_int, [C.c_char_p, C.POINTER(capi.MacroMesh), capi.ip])
        _sig(lib, "ref_micro_mesh_properties", C.c_int, [C.c_char_p, C.POINTER(capi.MicroMesh)])
        _sig(lib, "ref_read_effective_conductivity", C.c_int, [C.c_char_p, C.POINTER(capi.Keff)])
        _sig(lib, "ref_set_exprem_options", C.c_int, [C.POINTER(capi.ExpremOptions)])
        _sig(lib, "ref_phipade", C.c_int, [dp, dp, C.c_double, C.c_int, C.c_int])
        _sig(lib, "ref_save_solution", None, [C.c_char_p, dp, dp, C.c_int, C.POINTER(capi.UserData)])
        _r = lib
    return _r


class Oracle:
    """The oracle bound to one problem (twoscalerich_gb300.problem.Problem)."""

    def __init__(self, problem, nthreads=1, libm=False, gram_schmidt=0):
        """gram_schmidt: 0 modified Gram-Schmidt, 1 classical twice (CGS2)."""
        self.lib = load(libm)
        self.p = problem
        self.h = self.lib.oracle_create(C.byref(problem.ud), C.byref(problem.ext))
        if not self.h:
            raise RuntimeError("oracle_create failed")
        if self.lib.oracle_set_gram_schmidt(self.h, gram_schmidt) != 0:
            raise ValueError("unknown Gram-Schmidt variant %r" % gram_schmidt)
        self.N = problem.N
        self.nthreads = nthreads

    def _p(self, a):
        from twoscalerich_gb300.capi import ptr
        return ptr(a)

    def g(self, u):
        out = np.empty(self.N)
        self.flag = self.lib.oracle_g(self.h, self._p(u), self._p(out), self.nthreads)
        return out

    def jv(self, u, g0, v, eps):
        out = np.empty(self.N)
        self.lib.oracle_jv(self.h, self._p(u), self._p(g0), self._p(v), eps, self._p(out),
                           self.nthreads)
        return out

    def water(self, u):
        w = C.c_double()
        self.lib.oracle_water(self.h, self._p(u), C.byref(w))
        return w.value

    def water_scenarios(self, u):
        w = np.empty(self.p.S)
        self.lib.oracle_water_scenarios(self.h, self._p(u), self._p(w))
        return w

    def cell_summary(self, u, g):
        out = np.empty(5 * self.p.Ne)
        self.lib.oracle_cell_summary(self.h, self._p(u), self._p(g), self._p(out))
        return out.reshape(self.p.Ne, 5)

    def dot(self, x, y):
        return self.lib.oracle_dot(self._p(x), self._p(y), x.size)

    def exprem_step(self, t, u, tspan, solns, opts, stats):
        tt = C.c_double(t)
        rc = self.lib.oracle_exprem_step(self.h, C.byref(tt), self.p.tend, self._p(tspan),
                                         self._p(solns), self._p(u), C.byref(opts),
                                         C.byref(stats), self.nthreads)
        if rc != 0:
            raise RuntimeError("oracle_exprem_step failed with %d" % rc)
        return tt.value

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
