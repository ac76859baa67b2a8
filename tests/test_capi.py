"""The C-ABI library: it loads, exports every entry point its headers
declare, and its host-side entry points work without a GPU."""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from tests.helpers import ROOT, reference_root
from twoscalerich_gb300 import capi


def declared_c_symbols():
    text = open(os.path.join(ROOT, "include", "tsr_capi.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tsr_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = capi.load()
    names = declared_c_symbols()
    assert len(names) > 30
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes binding covers exactly the declared set
    assert sorted(capi.declared_symbols()) == names


@pytest.mark.skipif(shutil.which("nm") is None, reason="nm not available")
def test_cpp_dropins_exported_with_reference_signatures():
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", capi.LIB_PATH], capture_output=True,
                         text=True).stdout
    assert "Gfunc_gpu(double*, double*, user_data_struct)" in out
    assert ("exprem_gpu(int (*)(double*, double*, user_data_struct), int, double&, double, double*, "
            "double*, double*, user_data_struct, exprem_options_struct, exprem_stats_struct&)") in out


STRUCTS = [("macro_mesh_struct", capi.MacroMesh), ("micro_mesh_struct", capi.MicroMesh),
           ("Keff_struct", capi.Keff), ("soil_struct", capi.Soil),
           ("user_data_struct", capi.UserData), ("exprem_options_struct", capi.ExpremOptions),
           ("exprem_stats_struct", capi.ExpremStats)]


def _layout_probe(includes, tmp_path):
    """sizeof and every field offset of the structs, as a C++ compiler sees them."""
    src = ["#include <cstdio>", "#include <cstddef>"] + ['#include "%s"' % i for i in includes]
    src.append("int main() {")
    for cname, cls in STRUCTS:
        src.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            src.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    src.append("return 0; }")
    cpp = tmp_path / "probe.cpp"
    cpp.write_text("\n".join(src) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["g++", "-o", str(exe), str(cpp)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return dict(line.rsplit(" ", 1) for line in out.split("\n") if line)


def _ctypes_layout():
    d = {}
    for cname, cls in STRUCTS:
        d[cname] = str(C.sizeof(cls))
        for f, _ in cls._fields_:
            d["%s.%s" % (cname, f)] = str(getattr(cls, f).offset)
    return d


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_structs_layout_matches_header(tmp_path):
    assert _layout_probe([os.path.join(ROOT, "include", "tsr_types.h")], tmp_path) == _ctypes_layout()


@pytest.mark.skipif(shutil.which("g++") is None or reference_root() is None,
                    reason="reference headers not present")
def test_structs_layout_matches_reference_headers(tmp_path):
    ref = os.path.join(reference_root(), "include") + os.sep
    heads = [ref + h for h in ("macro_mesh.h", "micro_mesh.h", "Keff.h", "soil.h", "user_data.h",
                               "exprem_options.h", "exprem_stats.h")]
    assert _layout_probe(heads, tmp_path) == _ctypes_layout()


def test_init_without_gpu_fails_cleanly():
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from twoscalerich_gb300 import problem as P
    p = P.config1()
    lib = capi.load()
    h = lib.tsr_init(C.byref(p.ud), C.byref(p.ext), None, 0)
    assert not h
    assert "CUDA" in capi.last_error() or "device" in capi.last_error()


def test_phipade_argument_errors():
    lib = capi.load()
    phi = np.zeros(4)
    H = np.zeros(6)
    assert lib.tsr_phipade(capi.ptr(phi), capi.ptr(H), 1.0, 0, 2) == 5
    assert lib.tsr_phipade(capi.ptr(phi), capi.ptr(H), 1.0, 3, 2) == 5
