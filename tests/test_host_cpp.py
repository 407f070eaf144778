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
    m = re.match(r"step (\d+) time (\S+) umax (\S+) broken (\d+) strain (\S+) kinetic (\S+)",
                 out)
    assert m, out
    p = configs.rnp_plate(40, 1e-3, 3, 0.2 * 0.04, 0.1, 2e-8, 200, jitter=0.0)
    model = gpu.FDModel(p, precision=abi.FP64)
    model.run(200)
    u = model.state()[0]
    assert int(m.group(1)) == 200
    assert float(m.group(3)) == pytest.approx(np.linalg.norm(u, axis=1).max(), rel=1e-12)
    assert int(m.group(4)) == int(model.bond_state().sum())
    _, tot = model.energies()
    assert float(m.group(5)) == pytest.approx(tot[0], rel=1e-6)
    assert float(m.group(6)) == pytest.approx(tot[2], rel=1e-6)


@pytest.mark.gpu
def test_host_quasi_static_matches_python_binding(tmp_path, gpu):
    """QuasiStaticModel<ElasticState> through the C++ class and through the
    Python binding: same plate, loads and Solver block, three load steps."""
    from nlmech_gb300 import configs
    from nlmech_gb300.decks import BC, MaterialDeck, Problem
    out = subprocess.check_output([build_example(tmp_path), "qs"]).decode()
    m = re.match(r"qs newton (\d+) residual (\S+) umax (\S+)", out)
    assert m, out
    x, vol = configs.grid2d(14, 10, 0.1, jitter=0.0)
    mat = MaterialDeck(kind="ElasticState", density=1200.0, K=4000.0, G=1500.0)
    edge = dict(y1=-0.01, y2=1.01, spatial_fn="constant")
    ubc = [BC(region="rectangle", x1=-0.01, x2=0.12, direction=[1, 2], time_fn="constant",
              time_params=[0.0], spatial_params=[1.0], **edge),
           BC(region="rectangle", x1=1.28, x2=1.41, direction=[2], time_fn="linear",
              time_params=[0.01], spatial_params=[1.0], **edge)]
    fbc = [BC(region="rectangle", x1=1.28, x2=1.41, direction=[1], time_fn="linear",
              time_params=[1.0], spatial_params=[-50.0], **edge)]
    p = Problem(dim=2, x=x, volume=vol, horizon=0.3, mesh_size=0.1, material=mat,
                ubc=ubc, fbc=fbc)
    q = gpu.ESQSModel(p, gpu.esqs_params(max_iters=50, tol=1e-9, jacobian=1, dt=0.25))
    iters, _, res = q.solve(3)
    u, _ = q.get()
    assert float(m.group(2)) < 1e-9
    assert int(m.group(1)) == int(iters[-1])
    assert float(m.group(3)) == pytest.approx(np.linalg.norm(u, axis=1).max(), rel=1e-9)
