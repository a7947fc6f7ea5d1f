"""The C++ drop-in operator header compiles against the C ABI (CPU), and on a
GPU drives one step through std::vector<Particle> like the reference's
ParticleGroup does, agreeing with the Python host path."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "pclop_demo.cpp")


def compile_demo(tmp_path):
    from vortegrid_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "pclop_demo")
    subprocess.check_call(["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                           lib, "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def test_header_compiles(tmp_path):
    assert os.path.exists(compile_demo(tmp_path))


@pytest.mark.gpu
def test_cpp_operator_matches_python(tmp_path):
    import vortegrid_gb300 as vg
    from vortegrid_gb300 import workloads
    exe = compile_demo(tmp_path)
    pos, w, s = workloads.ring(2000, seed=9)
    recs = vg.make_particles(pos, w, s)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    recs.tofile(inp)
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=vg.PARTICLE_DTYPE)
    op = vg.PclOpVortonSim(0.01)
    op.mMinCorner = np.array([-1.5, -1.5, -1.0], np.float32)
    op.mMaxCorner = np.array([1.5, 1.5, 1.0], np.float32)
    mine = recs.copy()
    op.Operate(mine, np.float32(1.0 / 30.0), 0)
    assert np.array_equal(got["velocity"], mine["velocity"])
    assert np.array_equal(got["angular_velocity"], mine["angular_velocity"])
