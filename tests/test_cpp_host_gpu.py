"""A setup written in C++ against the reference's LBM interface (fluidx3d_gb300/host/lbm.hpp),
compiled and run on the GPU: its 64^3 Taylor-Green result equals the reference's bit for bit."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

import lbm_cases as LC

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_taylor_green_setup_matches_reference(gpu, solver_lib, tmp_path, golden_dir):
    from fluidx3d_gb300 import build
    exe = tmp_path / "tgv_setup"
    libdir = os.path.dirname(build.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "fluidx3d_gb300", "host"),
                    os.path.join(ROOT, "tests", "cpp", "taylor_green_setup.cpp"), "-L", libdir, "-lfluidx3d_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    f = LC.TGV64.fields()
    state = tmp_path / "state.bin"
    with open(state, "wb") as fh:
        fh.write(f["rho"].tobytes())
        fh.write(f["u"].tobytes())
    out = subprocess.run([str(exe), str(state)], check=True, capture_output=True, text=True).stdout
    assert "t 1000" in out
    N = 64 ** 3
    data = np.fromfile(state, dtype=np.float32)
    rho, u = data[:N], data[N:]
    g = np.load(os.path.join(golden_dir, "tgv64.npz"))
    assert hashlib.sha256(rho.tobytes()).hexdigest() == str(g["rho_sha256"])
    assert hashlib.sha256(u.tobytes()).hexdigest() == str(g["u_sha256"])
    assert np.float32(float(out.split()[1])) == g["ux_center"]
