"""The C++ host side (include/wg_gpu.hpp) compiles with g++ and links against the
library; its non-GPU calls behave (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cpp_shim_compiles_links_and_runs(tmp_path):
    from watergap2_gb300 import build, gpu
    if not os.path.exists(gpu.LIB_PATH):
        build.build()
    exe = tmp_path / "shim"
    libdir = os.path.dirname(gpu.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_compile.cpp"), "-L", libdir, "-lwg_gpu",
           f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True)
    assert out.stdout.strip() == "ok"


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_dropin_shims_compile_with_the_reference_classes():
    """include/wg_gpu.hpp's stand-ins instantiated with the reference's own
    WghmStateFile, AdditionalOutputInputFile, SnowInElevationFile and
    calibParamClass (their headers, where the reference sources were built)."""
    from oracle import ref_case
    src = ref_case.source_dir()
    if src is None:
        pytest.skip("the reference's sources are not on this machine")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-I", os.path.join(ROOT, "include"), "-I", src,
           os.path.join(ROOT, "tests", "cpp", "shim_reference_types.cpp")]
    subprocess.run(cmd, check=True)
