"""Reading the reference's decks and mesh files (nlmech_gb300/deckfile.py,
meshfile.py): the YAML subset, every field inp::Input reads for the models
here, the CSV / Gmsh / VTU mesh readers and nodal volumes.  A deck read from
a file gives the same oracle run, bit for bit, as the same problem built in
code; the reference's own example decks parse, and the 1-D quasi-static one
yields the nodes and volumes of its stored result."""
import os

import numpy as np
import pytest

from nlmech_gb300 import abi, configs, deckfile, meshfile, vtu
from nlmech_gb300.decks import BC, Crack
from oracle import oracle as orc

REF = orc.REF_TREE
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "examples")),
                               reason="reference tree not present")


def test_yaml_subset():
    txt = """
Model:            # comment
  Dimension: 2
  Discretization_Type:
    Spatial: finite_difference
    Time: velocity_verlet
  Final_Time: 2.0e-5
Output:
  Tags:
    - Displacement
    - Damage_Z   # trailing comment
  Flags: [1,2, 3]
  Flag: True
  Name: "a: b"
Time_Function:
  Parameters:
    - -5.0
  Parameters: [1]
List:
- k: 1
  j: [0.5]
- 7
"""
    d = deckfile.parse_yaml(txt)
    assert d["Model"]["Dimension"] == 2 and d["Model"]["Final_Time"] == 2.0e-5
    assert d["Model"]["Discretization_Type"] == {"Spatial": "finite_difference",
                                                 "Time": "velocity_verlet"}
    assert d["Output"]["Tags"] == ["Displacement", "Damage_Z"]
    assert d["Output"]["Flags"] == [1, 2, 3] and d["Output"]["Flag"] is True
    assert d["Output"]["Name"] == "a: b"
    assert d["Time_Function"]["Parameters"] == [-5.0]  # the first of a repeated key
    assert d["List"] == [{"k": 1, "j": [0.5]}, 7]


DECK = """
Model:
  Dimension: 2
  Discretization_Type:
    Spatial: finite_difference
    Time: central_difference
  Final_Time: 4.0e-6
  Time_Steps: 200
  Horizon: 0.003
  Horizon_h_Ratio: 3
Policy:
  Enable_PostProcessing: true
Mesh:
  File: mesh.csv
Material:
  Type: PDBond
  Density: 2440.0
  Compute_From_Classical: true
  E: 72.0e9
  Gc: 3.8
  Bond_Potential:
    Type: 1
    Check_Sc_Factor: 1.0
    Irreversible_Bond_Fracture: true
  Influence_Function:
    Type: 1
Fracture:
  Cracks:
    Sets: 2
    Set_1:
      Orientation: 1
      Line: [0.015, 0.02, 0.025, 0.02]
    Set_2:
      Orientation: -1
      Line: [0.03, 0.005, 0.03, 0.015]
      Activation_Time: 1.0e-6
No_Fail_Region:
  Factor: 0.5
  Compute_And_Not_Store: false
  Num_Regions: 1
  Region_1:
    Type: Circle
    Parameters: [0.01, 0.01, 0.0, 0.003]
Displacement_BC:
  Sets: 2
  Set_1:
    Location:
      Rectangle: [-0.001, -0.001, 0.041, 0.003]
    Direction: [2]
    Time_Function:
      Type: linear
      Parameters:
        - -0.2
    Spatial_Function:
      Type: constant
  Set_2:
    Location:
      Rectangle: [-0.001, 0.037, 0.041, 0.041]
    Direction: [2]
    Time_Function:
      Type: linear
      Parameters:
        - 0.2
    Spatial_Function:
      Type: constant
Force_BC:
  Sets: 1
  Set_1:
    Location:
      Angled_Rectangle: [0.002, 0.015, 0.008, 0.025]
      Angle: 0.3
    Direction: [1]
    Time_Function:
      Type: sin
      Parameters: [1.0e13, 2.0e4]
    Spatial_Function:
      Type: constant
      Parameters: [1.0]
Initial_Condition:
  Velocity:
    Type: gaussian
    Parameters: [0.02, 0.02, 1.0, 0.5, 1.0e-4, 0.3]
Output:
  Path: ./out/
  Tags:
    - Displacement
    - Damage_Z
  Output_Interval: 50
  Output_Criteria:
    Type: max_Z
    New_Interval: 10
    Parameters: [0.9]
"""


def _write_deck(tmp_path):
    x, vol = configs.grid2d(40, 40, 1e-3, seed=21)
    with open(tmp_path / "mesh.csv", "w") as fh:
        fh.write("id,x,y,volume\n")
        for i in range(x.shape[0]):
            fh.write("%d,%.17g,%.17g,%.17g\n" % (i, x[i, 0], x[i, 1], vol[i]))
    (tmp_path / "input.yaml").write_text(DECK)
    return x, vol


def _same_problem_in_code(x, vol):
    p = configs.rnp_plate(40, 1e-3, 3, 0.0, 0.2, 2e-8, 200, seed=21)
    p.x, p.volume = x, vol
    p.dt = 4.0e-6 / 200  # Final_Time / Time_Steps, as inp::Input forms it
    p.horizon, p.mesh_size = 0.003, 0.003 / 3  # h = Horizon / Horizon_h_Ratio
    p.scheme = abi.CENTRAL_DIFFERENCE
    p.material.influence_type = 1
    p.material.influence_params = []
    p.ubc = [BC(region="rectangle", x1=-0.001, y1=-0.001, x2=0.041, y2=0.003, direction=[2],
                time_fn="linear", time_params=[-0.2]),
             BC(region="rectangle", x1=-0.001, y1=0.037, x2=0.041, y2=0.041, direction=[2],
                time_fn="linear", time_params=[0.2])]
    p.fbc = [BC(region="angled_rectangle", x1=0.002, y1=0.015, x2=0.008, y2=0.025, theta=0.3,
                direction=[1], time_fn="sin", time_params=[1.0e13, 2.0e4])]
    p.cracks = [Crack(kind="edge", orientation=1, pb=(0.015, 0.02), pt=(0.025, 0.02)),
                Crack(kind="edge", orientation=-1, pb=(0.03, 0.005), pt=(0.03, 0.015),
                      activation_time=1.0e-6)]
    p.no_fail, p.no_fail_tol = abi.NOFAIL_DATA, 0.5 * 0.003
    p.nofail_regions = [("Circle", [0.01, 0.01, 0.0, 0.003])]
    r = np.sqrt((x[:, 0] - 0.02) ** 2 + (x[:, 1] - 0.02) ** 2 + x[:, 2] ** 2)
    g = 0.3 * np.exp(-(r * r) / 1.0e-4)
    p.v0 = np.stack([g * 1.0, g * 0.5, 0 * g], axis=1)
    return p


def test_deck_fields(tmp_path):
    x, vol = _write_deck(tmp_path)
    d = deckfile.read_deck(str(tmp_path / "input.yaml"))
    p = d.problem
    assert p.dim == 2 and p.horizon == 0.003 and p.mesh_size == 0.003 / 3
    assert p.dt == 4.0e-6 / 200 and p.steps == 200 and p.scheme == abi.CENTRAL_DIFFERENCE
    assert np.array_equal(p.x, x) and np.array_equal(p.volume, vol)
    assert p.material.kind == "RNPBond" and p.material.E == 72.0e9 and p.material.Gc == 3.8
    assert p.material.influence_type == 1 and p.material.irreversible
    assert [c.activation_time for c in p.cracks] == [-1.0, 1.0e-6]
    assert p.no_fail == abi.NOFAIL_DATA and p.no_fail_tol == 0.003 * 0.5
    assert p.nofail_regions == [("Circle", [0.01, 0.01, 0.0, 0.003])]
    assert [b.region for b in p.ubc] == ["rectangle", "rectangle"]
    assert p.ubc[0].x2 == 0.041 and p.ubc[0].y2 == 0.003 and p.ubc[0].time_params == [-0.2]
    assert p.fbc[0].region == "angled_rectangle" and p.fbc[0].theta == 0.3
    assert p.u0 is None and p.v0 is not None
    o = d.output
    assert o.tags == ["Displacement", "Damage_Z"] and o.dt_out == 50
    assert o.criteria == "max_Z" and o.dt_out_criteria == 10 and o.criteria_params == [0.9]
    assert o.path == os.path.join(str(tmp_path), "./out/")


def test_deck_runs_like_the_problem_built_in_code(tmp_path):
    x, vol = _write_deck(tmp_path)
    a = orc.OracleFD(deckfile.read_deck(str(tmp_path / "input.yaml")).problem)
    b = orc.OracleFD(_same_problem_in_code(x, vol))
    a.run(120)
    b.run(120)
    for ua, ub in zip(a.state(), b.state()):
        assert np.array_equal(ua, ub)
    assert np.array_equal(a.bond_state(), b.bond_state())
    assert np.array_equal(a.fixity(), b.fixity())


def test_refused_decks(tmp_path):
    _write_deck(tmp_path)
    bad = {
        "  Dimension: 2\n": "",                                   # no dimension
        "  Density: 2440.0\n": "",                                # no density
        "    Type: max_Z\n": "    Type: max_Z\n  File_Format: msh\n",
        "      Type: sin\n": "      Type: cubic\n",               # unknown function
    }
    for old, new in bad.items():
        (tmp_path / "bad.yaml").write_text(DECK.replace(old, new, 1))
        with pytest.raises(deckfile.DeckError):
            deckfile.read_deck(str(tmp_path / "bad.yaml"))


def test_mesh_volumes_and_size(tmp_path):
    # triangles: a unit square split into 2 n^2 triangles; every node gets a
    # third of its triangles' areas and the total is the square's area
    n = 6
    g = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(g, g, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), 0 * X.ravel()], axis=1)
    idx = np.arange((n + 1) ** 2).reshape(n + 1, n + 1)
    tris, quads = [], []
    for i in range(n):
        for j in range(n):
            a, b, c, d = idx[i, j], idx[i + 1, j], idx[i + 1, j + 1], idx[i, j + 1]
            tris += [[a, b, c], [a, c, d]]
            quads.append([a, b, c, d])
    h = 1.0 / n
    for etype, E in ((meshfile.VTK_TRIANGLE, tris), (meshfile.VTK_QUAD, quads)):
        m = meshfile.Mesh(nodes=nodes, volumes=None, element_type=etype,
                          elements=np.array(E, dtype=np.int64))
        v = meshfile.compute_volumes(m)
        assert abs(v.sum() - 1.0) < 1e-12
        assert abs(v[idx[3, 3]] - h * h) < 1e-12              # interior node
        assert abs(v[idx[0, 3]] - 0.5 * h * h) < 1e-12        # edge node
        c = meshfile.nodes_at_centroid(m)
        assert abs(c.volumes.sum() - 1.0) < 1e-12
    assert meshfile.mesh_size(nodes) == pytest.approx(h, rel=1e-12)
    # Gmsh 2.2 file of the same quads, elements in two entities
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(len(nodes))]
    lines += ["%d %.17g %.17g 0" % (k + 1, p[0], p[1]) for k, p in enumerate(nodes)]
    lines += ["$EndNodes", "$Elements", str(len(quads) + 1), "1 15 2 0 1 1"]
    for k, q in enumerate(quads):
        ent = 2 if k % 2 else 1
        lines.append("%d 3 2 0 %d %s" % (k + 2, ent, " ".join(str(v + 1) for v in q)))
    lines.append("$EndElements")
    (tmp_path / "q.msh").write_text("\n".join(lines) + "\n")
    m = meshfile.read_mesh(str(tmp_path / "q.msh"), 2)
    assert m.element_type == meshfile.VTK_QUAD and np.allclose(m.nodes, nodes)
    want = [q for k, q in enumerate(quads) if k % 2 == 0] + [q for k, q in enumerate(quads) if k % 2]
    assert np.array_equal(m.elements, np.array(want))
    assert abs(m.volumes.sum() - 1.0) < 1e-12
    # VTU with a stored volume
    vtu.write_points(str(tmp_path / "m.vtu"), nodes, [("Node_Volume", m.volumes)])
    mv = meshfile.read_mesh(str(tmp_path / "m.vtu"), 2)
    assert np.array_equal(mv.volumes, m.volumes) and np.array_equal(mv.nodes, nodes)


@needs_ref
def test_reference_example_decks_parse():
    n = 0
    for root, _, files in os.walk(os.path.join(REF, "examples")):
        for f in files:
            if f.endswith(".yaml"):
                with open(os.path.join(root, f)) as fh:
                    d = deckfile.parse_yaml(fh.read())
                assert isinstance(d, dict) and d, f
                n += 1
    assert n >= 15


@needs_ref
def test_reference_qs_1d_deck_reads_its_mesh():
    z = np.load(os.path.join(GOLD, "qs_1d.npz"))
    d = deckfile.read_deck(os.path.join(REF, "examples/qsModel/1D/input.yaml"))
    assert d.quasi_static and d.problem.dim == 1
    assert np.array_equal(d.problem.x, z["x"]) and np.array_equal(d.problem.volume, z["volume"])
    assert d.problem.material.kind == "ElasticState"
    assert float(d.solver["Tolerance"]) > 0


@needs_ref
def test_reference_gmsh_deck_reads_its_mesh():
    d = deckfile.read_deck(os.path.join(REF, "examples/fdModel/logo/input.yaml"))
    p = d.problem
    assert p.n == 5107 and p.horizon == 0.1 and p.mesh_size == 0.1 / 4
    # nodal volumes from the triangles add up to the meshed area
    m = meshfile.read_mesh(os.path.join(REF, "examples/fdModel/logo/mesh.msh"), 2)
    x = m.nodes
    E = m.elements
    area = 0.5 * np.abs((x[E[:, 1], 0] - x[E[:, 0], 0]) * (x[E[:, 2], 1] - x[E[:, 0], 1]) -
                        (x[E[:, 2], 0] - x[E[:, 0], 0]) * (x[E[:, 1], 1] - x[E[:, 0], 1]))
    assert abs(p.volume.sum() - area.sum()) < 1e-12 * area.sum()
    assert p.fbc[0].spatial_fn == "sin_x" and p.fbc[0].time_params == [1.5e9]


@pytest.mark.skipif(not orc.refshim_available(), reason="reference source tree not present")
def test_nodal_volumes_match_reference_computevol():
    """meshfile.compute_volumes against the reference's fe::Mesh::computeVol
    (its own quadrature, run through the refshim) on jittered triangle and
    quadrangle meshes and, with the reference tree, its Gmsh example."""
    rng = np.random.default_rng(3)
    n = 9
    g = np.linspace(0.0, 2.0, n + 1)
    X, Y = np.meshgrid(g, g, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), 0 * X.ravel()], axis=1)
    nodes[:, :2] += rng.uniform(-0.04, 0.04, size=(nodes.shape[0], 2))
    idx = np.arange((n + 1) ** 2).reshape(n + 1, n + 1)
    tris, quads = [], []
    for i in range(n):
        for j in range(n):
            a, b, c, d = idx[i, j], idx[i + 1, j], idx[i + 1, j + 1], idx[i, j + 1]
            tris += [[a, b, c], [a, c, d]]
            quads.append([a, b, c, d])
    cases = [(meshfile.VTK_TRIANGLE, np.array(tris)), (meshfile.VTK_QUAD, np.array(quads))]
    logo = os.path.join(REF, "examples/fdModel/logo/mesh.msh")
    meshes = [meshfile.Mesh(nodes=nodes, volumes=None, element_type=t, elements=E) for t, E in cases]
    if os.path.exists(logo):
        meshes.append(meshfile.read_msh(logo, 2))
    for m in meshes:
        ours = meshfile.compute_volumes(m)
        ref = orc.ref_mesh_volumes(2, m.nodes, m.element_type, m.elements)
        assert np.abs(ours - ref).max() <= 1e-13 * np.abs(ref).max(), m.element_type
