"""The C++ host side: GB300Simulator<CELL> (the CUDASimulator drop-in) with
unchanged Initializer / Writer / Steerer plugins, and user cells that run
their own update() on the device (gb300cell.cuh).

Not-GPU: the drop-in header compiles and links both against this package's
declarations and - where the reference's headers are present - against the
reference's own Simulator / plugin classes; the user-cell program compiles
with nvcc the same two ways, the second with the reference's own TestCell
and TestInitializer.  GPU: both programs (tests/cpp/gb300simulator_test.cpp,
tests/cpp/gb300_cell_test.cu) run and report OK.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "gb300simulator_test.cpp")
REF = os.environ.get("LGD_REFERENCE_ROOT", "/root/reference")
CELL_SRC = os.path.join(ROOT, "tests", "cpp", "gb300_cell_test.cu")


def compile_test(out, with_reference=False):
    import __graft_entry__
    __graft_entry__.build()
    libdir = os.path.join(ROOT, "libgeodecomp_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(libdir, "include"), SRC, "-L", libdir, "-llgd_gb300",
           "-Wl,-rpath," + libdir, "-o", out]
    if with_reference:
        cmd[3:3] = ["-DLGD_GB300_WITH_REFERENCE", "-I", os.path.join(ROOT, "oracle", "ref_config"),
                    "-I", os.path.join(REF, "src"), "-I", os.path.join(REF, "lib", "libflatarray", "include")]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_dropin_builds_with_package_declarations(tmp_path):
    exe = compile_test(str(tmp_path / "t"))
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode in (0, 2), res.stdout + res.stderr   # 2: no GPU here


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "libgeodecomp")),
                    reason="reference headers not present on this machine")
def test_dropin_builds_against_reference_plugins(tmp_path):
    exe = compile_test(str(tmp_path / "t"), with_reference=True)
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode in (0, 2), res.stdout + res.stderr


def compile_cell_test(out, with_reference=False):
    """The user-cell program, compiled by nvcc for sm_103a."""
    import __graft_entry__
    from libgeodecomp_gb300 import build
    __graft_entry__.build()
    libdir = os.path.join(ROOT, "libgeodecomp_gb300")
    cmd = [build.nvcc(), *build.ARCH, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(libdir, "include"), CELL_SRC, "-L", libdir, "-llgd_gb300",
           "-Xlinker", "-rpath=" + libdir, "-o", out]
    if with_reference:
        cmd[1:1] = ["-DLGD_GB300_WITH_REFERENCE", "-I", os.path.join(ROOT, "oracle", "ref_config_cuda"),
                    "-I", os.path.join(REF, "src"), "-I", os.path.join(REF, "lib", "libflatarray", "include")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-3000:] + res.stderr[-3000:]
    if not with_reference:      # the reference's own headers warn under nvcc
        assert "warning" not in res.stderr, res.stderr[-3000:]
    return out


def test_user_cell_program_builds(tmp_path):
    exe = compile_cell_test(str(tmp_path / "c"))
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode in (0, 2), res.stdout + res.stderr   # 2: no GPU here


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "libgeodecomp")),
                    reason="reference headers not present on this machine")
def test_user_cell_program_builds_with_reference_testcell(tmp_path):
    """The reference's own TestCell and TestInitializer, unchanged, compile
    through the device path (their update() becomes the kernel's body)."""
    exe = compile_cell_test(str(tmp_path / "c"), with_reference=True)
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode in (0, 2), res.stdout + res.stderr


@pytest.mark.gpu
def test_user_cells_on_gpu(tmp_path):
    exe = compile_cell_test(str(tmp_path / "c"))
    res = subprocess.run([exe], capture_output=True, text=True, timeout=600, cwd=str(tmp_path))
    assert res.returncode == 0 and "OK" in res.stdout, res.stdout + res.stderr


@pytest.mark.gpu
def test_dropin_conformance_on_gpu(tmp_path):
    exe = compile_test(str(tmp_path / "t"))
    res = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and "OK" in res.stdout, res.stdout + res.stderr
