"""Build the golden fixtures of the quasi-static ElasticState examples.

Run in a checkout that has the NLMech reference tree (NLMECH_REFERENCE, or
the refshim recipe's default location); writes qs_1d.npz and qs_2d.npz beside this script.  The
fixtures are the reference's own stored results:

  examples/qsModel/1D/output_res.vtu  (33 nodes, deck examples/qsModel/1D/input.yaml)
  examples/qsModel/2D/output_res.vtu  (289 nodes, deck examples/qsModel/2D/input.yaml)

VTU files are "appended, base64, zlib" VTK XML (header_type UInt32); the
decoder below follows the VTK XML file-format documentation.

Reference coordinates: the 1-D mesh is examples/qsModel/1D/mesh.vtu.  The 2-D
mesh is not stored; the reference test generates it with tools/mesh
(uniformSquare, tools/mesh/src/2d/fe2D.cpp:115-160: x = x0 + i*h, volumes
halved on edges) and writes Points as Float32, so the coordinates the solver
read are float32(i*h).  The script rebuilds them that way and checks them
against Points - Displacement of the stored result.
"""
import base64
import json
import os
import re
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.oracle import REF_TREE as REF  # noqa: E402


def read_vtu(path):
    txt = open(path, "rb").read().decode("latin1")
    arrays = re.findall(r"<DataArray([^>]*)>", txt)
    app = txt[txt.index("<AppendedData"):]
    app = app[app.index("_") + 1:]
    app = app[: app.index("</AppendedData>")].strip()
    out = {}
    for a in arrays:
        name = re.search(r'Name="([^"]*)"', a).group(1)
        typ = re.search(r'type="([^"]*)"', a).group(1)
        off = int(re.search(r'offset="\s*(\d+)', a).group(1))
        nc = re.search(r'NumberOfComponents="(\d+)"', a)
        nc = int(nc.group(1)) if nc else 1
        nb = struct.unpack("<3I", base64.b64decode(app[off:off + 16])[:12])[0]
        hlen = 4 * (3 + nb)
        hchars = ((hlen + 2) // 3) * 4
        hdr = base64.b64decode(app[off:off + hchars])
        sizes = struct.unpack("<%dI" % (3 + nb), hdr[:hlen])[3:]
        dchars = ((sum(sizes) + 2) // 3) * 4
        data = base64.b64decode(app[off + hchars:off + hchars + dchars])
        raw, p = b"", 0
        for s in sizes:
            raw += zlib.decompress(data[p:p + s])
            p += s
        dt = {"Float64": "<f8", "Float32": "<f4", "Int64": "<i8", "UInt8": "u1"}[typ]
        arr = np.frombuffer(raw, dtype=dt)
        out[name] = arr.reshape(-1, nc) if nc > 1 else arr
    return out


def main():
    # ---- 1-D: examples/qsModel/1D ----
    d1 = os.path.join(REF, "examples/qsModel/1D")
    mesh = read_vtu(os.path.join(d1, "mesh.vtu"))
    res = read_vtu(os.path.join(d1, "output_res.vtu"))
    x = mesh["Points"].astype(np.float64)
    deck1 = {
        # input.yaml: Dimension 1, Horizon 1, Horizon_h_Ratio 3, ElasticState,
        # E 4000, Density 1; Displacement_BC Line [-0.1,0.3] dir [1] constant 0
        # (spatial constant 1); Force_BC Line [15.8,16.5] dir [1] linear [1],
        # spatial constant [160]; Solver CG, 100 iterations, tol 1e-9,
        # perturbation 1e-7; Final_Time 1, Time_Steps 1.
        "dim": 1, "horizon": 1.0, "h_ratio": 3, "E": 4000.0, "density": 1.0,
        "ubc": [{"region": "line", "x1": -0.1, "x2": 0.3, "dir": [1],
                 "time_fn": "constant", "time_params": [0.0],
                 "spatial_fn": "constant", "spatial_params": [1.0]}],
        "fbc": [{"region": "line", "x1": 15.8, "x2": 16.5, "dir": [1],
                 "time_fn": "linear", "time_params": [1.0],
                 "spatial_fn": "constant", "spatial_params": [160.0]}],
        "solver": "ConjugateGradient", "max_iters": 100, "tol": 1e-9,
        "perturbation": 1e-7, "final_time": 1.0, "time_steps": 1,
        "compare_tol": 1e-7,  # input_compare.yaml
    }
    np.savez_compressed(
        os.path.join(HERE, "qs_1d.npz"), x=x, volume=mesh["Node_Volume"],
        displacement=res["Displacement"], force=res["Force"],
        neighbors=res["Neighbors"], fixity=res["Fixity"],
        strain_energy=res["Strain_Energy"], deck=json.dumps(deck1))

    # ---- 2-D: examples/qsModel/2D ----
    d2 = os.path.join(REF, "examples/qsModel/2D")
    res = read_vtu(os.path.join(d2, "output_res.vtu"))
    h = 0.5 / 5  # input_mesh.yaml: Horizon 0.5, Horizon_h_Ratio 5
    nx = ny = int(1.6 / h)  # size_t((1.6 - 0) / h) as in fe2D.cpp:138-139
    xs = np.zeros((nx + 1) * (ny + 1) * 3)
    vol = np.full((nx + 1) * (ny + 1), h * h)
    for j in range(ny + 1):
        for i in range(nx + 1):
            n = j * (nx + 1) + i
            xs[3 * n] = np.float32(0.0 + float(i) * h)
            xs[3 * n + 1] = np.float32(0.0 + float(j) * h)
            if i == 0 or i == nx:
                vol[n] *= 0.5
            if j == 0 or j == ny:
                vol[n] *= 0.5
    x2 = xs.reshape(-1, 3)
    back = res["Points"].astype(np.float64) - res["Displacement"]
    err = np.abs(back - x2).max()
    assert err < 1e-6, err
    assert np.array_equal(vol, res["Node_Volume"])
    deck2 = {
        # input.yaml: Dimension 2, Horizon 0.5, Horizon_h_Ratio 5,
        # ElasticState K 4000, G 1500, Density 1200, plane stress;
        # Displacement_BC two sets Line [1.55,1.65] dir [1] and dir [2],
        # constant 0; Force_BC Line [-0.1,0.05] dir [1] linear [1],
        # spatial constant [-250]; Solver BiCGSTAB, 200 iterations,
        # tol 1e-6, perturbation 1e-7; Final_Time 1, Time_Steps 1.
        "dim": 2, "horizon": 0.5, "h_ratio": 5, "K": 4000.0, "G": 1500.0,
        "density": 1200.0, "plane_strain": False,
        "ubc": [{"region": "line", "x1": 1.55, "x2": 1.65, "dir": [1],
                 "time_fn": "constant", "time_params": [0.0],
                 "spatial_fn": "constant", "spatial_params": [1.0]},
                {"region": "line", "x1": 1.55, "x2": 1.65, "dir": [2],
                 "time_fn": "constant", "time_params": [0.0],
                 "spatial_fn": "constant", "spatial_params": [1.0]}],
        "fbc": [{"region": "line", "x1": -0.1, "x2": 0.05, "dir": [1],
                 "time_fn": "linear", "time_params": [1.0],
                 "spatial_fn": "constant", "spatial_params": [-250.0]}],
        "solver": "BiCGSTAB", "max_iters": 200, "tol": 1e-6,
        "perturbation": 1e-7, "final_time": 1.0, "time_steps": 1,
        "compare_tol": 1e-7,
    }
    np.savez_compressed(
        os.path.join(HERE, "qs_2d.npz"), x=x2, volume=vol,
        displacement=res["Displacement"], force=res["Force"],
        neighbors=res["Neighbors"], fixity=res["Fixity"],
        strain_energy=res["Strain_Energy"], deck=json.dumps(deck2))
    print("wrote qs_1d.npz, qs_2d.npz; 2-D coordinate check max err", err)


if __name__ == "__main__":
    sys.exit(main())
