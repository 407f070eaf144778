"""The C++ host classes (nlmech_gb300/host/nlm_fdmodel.hpp) build against the
C ABI, and on a GPU reproduce the Python binding's run of the same deck."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "nlmech_gb300", "host")


def build_example(tmp_path):
    from nlmech_gb300 import build
    build.build()
    exe = str(tmp_path / "fd_example")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall",
                           os.path.join(HOST, "fd_example.cpp"), "-o", exe,
                           "-L", os.path.join(ROOT, "nlmech_gb300"), "-lnlmgpu",
                           "-Wl,-rpath," + os.path.join(ROOT, "nlmech_gb300")])
    return exe


def test_host_classes_compile_and_link(tmp_path):
    assert os.path.exists(build_example(tmp_path))


@pytest.mark.gpu
def test_host_example_matches_python_binding(tmp_path, gpu):
    from nlmech_gb300 import abi, configs
    out = subprocess.check_output([build_example(tmp_path)]).decode()
    m = re.match(r"step (\d+) time (\S+) umax (\S+) broken (\d+)", out)
    assert m, out
    p = configs.rnp_plate(40, 1e-3, 3, 0.2 * 0.04, 0.1, 2e-8, 200, jitter=0.0)
    model = gpu.FDModel(p, precision=abi.FP64)
    model.run(200)
    u = model.state()[0]
    assert int(m.group(1)) == 200
    assert float(m.group(3)) == pytest.approx(np.linalg.norm(u, axis=1).max(), rel=1e-12)
    assert int(m.group(4)) == int(model.bond_state().sum())
