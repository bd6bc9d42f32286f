"""The drop-in boundary compiles and links on the host (no GPU calls).

* The reference's own src/src-mpi/main1.C, unchanged, compiles against the
  drop-in classes of include/amcafe/ (with a single-rank MPI header, the
  test-only shim in oracle/ref_shims/) and links against libcafe_gpu.so
  (skipped where the reference checkout is absent).
* tests/native/dropin_loop.cpp (a loop over the drop-in classes) and
  tests/native/capi_loop.c (a C program over include/cafe_gpu.h) compile
  warning-free and link; the GPU tests run them (test_gpu_dropin.py).
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


def _lib():
    from amcafe_gb300 import _native
    from amcafe_gb300 import build as b

    if not os.path.exists(_native.LIB_PATH):
        b.build_engine()
    return os.path.dirname(_native.LIB_PATH)


def _link_flags():
    d = _lib()
    return ["-L" + d, "-lcafe_gpu", "-Wl,-rpath," + d]


def test_reference_main_compiles_against_dropin_classes(tmp_path):
    from amcafe_gb300 import build as b

    main = os.path.join(b.REF_SRC, "main1.C")
    if not os.path.exists(main):
        pytest.skip("reference checkout not present")
    # compiled from a scratch copy: a quoted #include searches the including
    # file's own folder first, which beside the original holds the
    # reference's headers
    src = tmp_path / "main1.C"
    src.write_bytes(open(main, "rb").read())
    exe = str(tmp_path / "cafe_main_gpu")
    cmd = ["g++", "-std=c++11", "-O1", "-Wall", "-Wno-unused-variable", "-Wno-unused-but-set-variable",
           "-I" + os.path.join(ROOT, "include", "amcafe"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle", "ref_shims"), str(src), "-o", exe] + _link_flags()
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert os.path.exists(exe)


def test_native_drivers_compile_and_link(tmp_path):
    r = subprocess.run(["g++", "-std=c++11", "-O1", "-Wall", "-Wextra", "-Werror",
                        "-I" + os.path.join(ROOT, "include", "amcafe"), "-I" + os.path.join(ROOT, "include"),
                        os.path.join(HERE, "native", "dropin_loop.cpp"), "-o", str(tmp_path / "dropin_loop")]
                       + _link_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "native", "capi_loop.c"),
                        "-o", str(tmp_path / "capi_loop")] + _link_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
