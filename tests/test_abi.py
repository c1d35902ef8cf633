"""The C-ABI library: it builds, loads and exports every symbol include/ma.h declares."""
import os
import re

import pytest

from conftest import ROOT, has_gpu


def _declared():
    with open(os.path.join(ROOT, "include", "ma.h")) as fh:
        src = fh.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ma_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported():
    from mongeampere_gb300 import _lib
    lib = _lib.load()
    declared = _declared()
    assert declared, "no declarations found"
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes table covers the whole header
    assert set(declared) == set(_lib.SIGNATURES)


def test_no_device_is_reported():
    if has_gpu():
        pytest.skip("a GPU is present")
    import ctypes
    from mongeampere_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ma_ctx_create(0, ctypes.byref(h)) == _lib.MA_ERR_NO_DEVICE
    assert lib.ma_status_string(_lib.MA_EMPTY_CELL).decode() == "a Laguerre cell is empty"


def test_python_api_fails_loudly_without_device():
    if has_gpu():
        pytest.skip("a GPU is present")
    from mongeampere_gb300 import _lib, api
    with pytest.raises(_lib.MaError):
        api.Context(0)


def _build_wrapper_example(tmp_path, name="wrapper_example"):
    import shutil
    import subprocess
    from mongeampere_gb300 import build as B
    lib = B.build()
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path / name)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-Wall", "-I", os.path.join(root, "include"),
                           os.path.join(root, "tests", "cpp", name + ".cpp"), "-o", exe,
                           "-L", os.path.dirname(lib), "-lma_gb300", "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def test_cpp_wrapper_builds_and_reports_missing_device(tmp_path):
    # the reference-shaped C++ API links against the library; without a GPU the
    # error surfaces as MA::Error (exit status 3)
    import subprocess
    exe = _build_wrapper_example(tmp_path)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered by the GPU test")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 3 and "no usable CUDA device" in r.stdout


@pytest.mark.gpu
def test_cpp_wrapper_runs(tmp_path):
    import subprocess
    exe = _build_wrapper_example(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_image_and_drawing_wrappers_build(tmp_path):
    # MA::Density::image and MA::draw_laguerre_diagram link against the library;
    # without a GPU the error surfaces as MA::Error (exit status 3)
    import subprocess
    exe = _build_wrapper_example(tmp_path, "wrapper_image_raster")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 3 and "no usable CUDA device" in r.stdout


def test_static_solve_checks_arguments_before_the_device():
    # ma_laplacian_solve_static (the Newton solve that allocates nothing) rejects a
    # system beyond its fixed scratch and null pointers on the host, before any CUDA
    # call; with valid arguments and no GPU it reports the missing device
    if has_gpu():
        pytest.skip("a GPU is present: covered by the GPU test")
    import ctypes
    from mongeampere_gb300 import _lib
    lib = _lib.load()
    buf = (ctypes.c_double * 4)()
    ibuf = (ctypes.c_int32 * 4)()
    it = ctypes.c_int64(0)
    args = (ibuf, ibuf, buf, buf, buf, 1e-10, 0, ctypes.byref(it), None)
    assert lib.ma_laplacian_solve_static((1 << 18) + 1, *args) == _lib.MA_ERR_BUFFER_TOO_SMALL
    assert lib.ma_laplacian_solve_static(0, *args) == _lib.MA_ERR_INVALID_ARGUMENT
    assert lib.ma_laplacian_solve_static(3, None, ibuf, buf, buf, buf, 1e-10, 0, ctypes.byref(it),
                                         None) == _lib.MA_ERR_INVALID_ARGUMENT
    assert lib.ma_laplacian_solve_static(3, *args) == _lib.MA_ERR_NO_DEVICE


def test_solve_defaults_are_the_references():
    # MA::ot_solve(..., double eps_g = 1e-7, size_t maxiter = 100, ...)
    # (optimal_transport.hpp:89-99) with its stop rule |m - nu|_2 < eps_g (:150), FP64
    # and the caller's initial weights; host-only, no device needed
    from mongeampere_gb300 import _lib
    lib = _lib.load()
    o = _lib.MaSolveOpts()
    lib.ma_solve_opts_default(o)
    assert o.eps_g == 1e-7 and o.maxiter == 100
    assert o.stop_rule == 0 and o.precision == 0 and o.init == 0 and o.verbose == 0
    # every status has a message
    for s in range(_lib.MA_CG_NOCONV + 1):
        assert lib.ma_status_string(s).decode() != "unknown status"


def test_header_is_plain_c(tmp_path):
    # include/ma.h is a C ABI: a C11 caller compiles against it with -pedantic, links
    # the library and calls a host-only entry point
    import shutil
    import subprocess
    from mongeampere_gb300 import build as B
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no gcc")
    lib = B.build()
    src = tmp_path / "caller.c"
    src.write_text('#include "ma.h"\n'
                   "int main(void)\n{\n    ma_solve_opts o;\n    ma_solve_opts_default(&o);\n"
                   "    return o.maxiter == 100 && o.eps_g == 1e-7 ? 0 : 1;\n}\n")
    exe = str(tmp_path / "caller")
    subprocess.check_call([gcc, "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                           os.path.join(ROOT, "include"), str(src), "-o", exe, "-L", os.path.dirname(lib),
                           "-lma_gb300", "-Wl,-rpath," + os.path.dirname(lib)])
    assert subprocess.run([exe]).returncode == 0
