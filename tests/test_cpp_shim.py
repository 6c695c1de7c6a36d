"""The C++ shim with the reference's method names (include/RGBDOdometryGB.hpp)
compiles against the C ABI and links against libslam_gb300.so; a program
using it runs its argument checks without a GPU."""
import os
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include "RGBDOdometryGB.hpp"
#include <cstdio>
int main() {
    try {
        RGBDOdometryGB odo(0, 480, 319.5f, 239.5f, 525.f, 525.f);  // invalid width
        return 2;
    } catch (const RGBDOdometryGB::Error &e) {
        std::printf("%d\n", e.status);
        return e.status == ODO_ERR_ARG ? 0 : 3;
    }
}
'''


def test_shim_compiles_links_and_reports_errors(built, tmp_path):
    from slam_gb300 import _build
    src = tmp_path / "use_shim.cpp"
    src.write_text(SRC)
    exe = tmp_path / "use_shim"
    libdir = os.path.dirname(_build.LIB)
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src),
                           "-L" + libdir, "-lslam_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "1"
