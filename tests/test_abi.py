"""The C-ABI library loads and exports every entry point the header
declares (no GPU work)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "picpp_gb300.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pic_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib_path():
    from picpp_gb300 import build
    return build.build()


def test_header_declares_the_reference_call_surface():
    names = declared()
    for must in ("pic_create", "pic_tristan_evaluate_b_half_step", "pic_move_particles", "pic_tristan_update_flux",
                 "pic_tristan_evaluate_e", "pic_update_electromagnetic_parameters", "pic_evaluate_electric_field",
                 "pic_evaluate_magnetic_field", "pic_update_fields", "pic_energy", "pic_sort_particles"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in declared():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pic_\w+)", out))
    assert set(declared()) <= exported


def test_python_wrapper_binds_every_export(lib_path):
    import picpp_gb300 as P
    assert set(P.EXPORTS) == set(declared())
    P.load_library(lib_path)


def test_cpp_mirror_compiles_against_the_header(tmp_path):
    """The C++ Simulation mirror (include/picpp_gb300_simulation.hpp) is
    valid C++17 against the C header."""
    src = tmp_path / "use.cpp"
    src.write_text('#include "picpp_gb300_simulation.hpp"\n'
                   'void f(const pic_config& c) { picpp::GpuSimulation s(c); s.tristanEvaluateBhalfStep();'
                   ' s.moveParticles(); s.tristanUpdateFlux(); s.tristanEvaluateE(); s.updateEnergy(); }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_null_arguments_fail_without_a_device(lib_path):
    lib = ctypes.CDLL(lib_path)
    lib.pic_create.restype = ctypes.c_int
    assert lib.pic_create(None, None) == 1
    lib.pic_last_error.restype = ctypes.c_char_p
    assert lib.pic_last_error(None) == b"null context"
