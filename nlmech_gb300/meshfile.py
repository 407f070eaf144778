"""Mesh files of the reference's decks: fe::Mesh::createData
(src/fe/mesh.cpp:102-229) with the CSV, Gmsh (.msh) and VTU readers of
src/rw/reader.cpp, nodal volumes from the elements (fe::Mesh::computeVol,
mesh.cpp:231-309) and the mesh size guess (computeMeshSize, :326-350).

    mesh = read_mesh("mesh.vtu", dim=2)
    mesh.nodes, mesh.volumes, mesh.element_type, mesh.elements
"""
import csv
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import vtu

VTK_VERTEX, VTK_LINE, VTK_TRIANGLE, VTK_QUAD, VTK_TETRA = 1, 3, 5, 9, 10
_VERTS = {VTK_VERTEX: 1, VTK_LINE: 2, VTK_TRIANGLE: 3, VTK_QUAD: 4, VTK_TETRA: 4}


@dataclass
class Mesh:
    nodes: np.ndarray                      # (n, 3) float64
    volumes: Optional[np.ndarray]          # (n,) float64, None until computed
    element_type: int = VTK_VERTEX         # VTK cell type
    elements: Optional[np.ndarray] = None  # (n_elem, vertices) int64


def read_csv(path, dim):
    """rw::reader::readCsvFile (reader.cpp:15-56): columns named id, x[, y[,
    z]], volume in any order, other columns ignored."""
    names = ["x", "y", "z"][:dim] + ["volume"]
    with open(path, newline="") as fh:
        rows = list(csv.reader(fh))
    head = [h.strip() for h in rows[0]]
    missing = [c for c in ["id"] + names if c not in head]
    if missing:
        raise ValueError("%s: missing CSV columns %s" % (path, missing))
    col = {c: head.index(c) for c in names}
    data = [r for r in rows[1:] if any(v.strip() for v in r)]
    nodes = np.zeros((len(data), 3))
    vol = np.zeros(len(data))
    for k, r in enumerate(data):
        for d, c in enumerate(["x", "y", "z"][:dim]):
            nodes[k, d] = float(r[col[c]])
        vol[k] = float(r[col["volume"]])
    return Mesh(nodes=nodes, volumes=vol)


def read_msh(path, dim):
    """Gmsh ASCII 2.2 meshes as MshReader::readMesh (mshReader.cpp:13-117)
    reads them through the Gmsh API: node tag t is node t - 1; the elements
    are the 3-node triangles if there are any, else the 4-node quadrangles,
    grouped by elementary entity in ascending tag order."""
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    try:
        k = lines.index("$MeshFormat")
    except ValueError:
        raise ValueError("%s: not a Gmsh file" % path)
    version = lines[k + 1].split()
    if not version[0].startswith("2") or version[1] != "0":
        raise ValueError("%s: only Gmsh ASCII 2.x meshes are read (found %s)"
                         % (path, " ".join(version)))
    k = lines.index("$Nodes")
    nn = int(lines[k + 1])
    tags = np.zeros(nn, dtype=np.int64)
    xyz = np.zeros((nn, 3))
    for q in range(nn):
        f = lines[k + 2 + q].split()
        tags[q] = int(f[0])
        xyz[q] = [float(v) for v in f[1:4]]
    nodes = np.zeros((int(tags.max()), 3))
    nodes[tags - 1] = xyz
    k = lines.index("$Elements")
    ne = int(lines[k + 1])
    by_type = {2: [], 3: []}
    for q in range(ne):
        f = [int(v) for v in lines[k + 2 + q].split()]
        etype, ntags = f[1], f[2]
        if etype in by_type:
            entity = f[4] if ntags >= 2 else 0
            by_type[etype].append((entity, q, f[3 + ntags:]))
    if by_type[2]:
        etype, vt, chosen = VTK_TRIANGLE, 3, by_type[2]
    elif by_type[3]:
        etype, vt, chosen = VTK_QUAD, 4, by_type[3]
    else:
        raise ValueError("%s: only 3-node triangle or 4-node quadrangle meshes are read" % path)
    chosen.sort(key=lambda e: (e[0], e[1]))
    elems = np.array([e[2][:vt] for e in chosen], dtype=np.int64) - 1
    return Mesh(nodes=nodes, volumes=None, element_type=etype, elements=elems)


def read_vtu_mesh(path, dim, finite_difference=True):
    """readVtuFileNodes / readVtuFilePointData / readVtuFileCells: points,
    then "Node_Volume" (or "Volume") for a finite-difference model, and the
    cells when no volume is stored."""
    d = vtu.read_vtu(path)
    pts = np.asarray(d["Points"], dtype=np.float64).reshape(-1, 3)
    vol = None
    if finite_difference:
        for name in ("Node_Volume", "Volume"):
            if name in d:
                vol = np.asarray(d[name], dtype=np.float64).reshape(-1)
                break
    mesh = Mesh(nodes=pts.copy(), volumes=vol)
    if vol is None and "connectivity" in d and "types" in d and len(d["types"]):
        conn = np.asarray(d["connectivity"], dtype=np.int64)
        offs = np.asarray(d["offsets"], dtype=np.int64)
        etype = int(d["types"][0])
        nv = _VERTS.get(etype)
        if nv is None:
            raise ValueError("%s: VTK cell type %d is not read" % (path, etype))
        starts = np.concatenate([[0], offs[:-1]])
        mesh.element_type = etype
        mesh.elements = np.stack([conn[starts + q] for q in range(nv)], axis=1)
    return mesh


def _gauss2():
    g = 1.0 / np.sqrt(3.0)
    return [(-g, -g), (g, -g), (g, g), (-g, g)]


def compute_volumes(mesh):
    """Nodal volume V_i = sum over the elements of node i of the integral of
    its shape function (fe::Mesh::computeVol, mesh.cpp:231-309, with the
    absolute element size): a third of a triangle's area, a quarter of a
    tetrahedron's volume, and 2 x 2 Gauss points for a bilinear quadrangle."""
    n = mesh.nodes.shape[0]
    vol = np.zeros(n)
    x = mesh.nodes
    E = mesh.elements
    if E is None or len(E) == 0:
        raise ValueError("no elements to compute nodal volumes from")
    if mesh.element_type == VTK_TRIANGLE:
        a, b, c = x[E[:, 0]], x[E[:, 1]], x[E[:, 2]]
        area = 0.5 * np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) -
                            (c[:, 0] - a[:, 0]) * (b[:, 1] - a[:, 1]))
        for q in range(3):
            np.add.at(vol, E[:, q], area / 3.0)
    elif mesh.element_type == VTK_TETRA:
        a, b, c, d = (x[E[:, q]] for q in range(4))
        v6 = np.abs(np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a)))
        for q in range(4):
            np.add.at(vol, E[:, q], v6 / 24.0)
    elif mesh.element_type == VTK_QUAD:
        xe = x[E][:, :, :2]                              # (ne, 4, 2)
        sgn = np.array([(-1, -1), (1, -1), (1, 1), (-1, 1)], dtype=np.float64)
        for xi, eta in _gauss2():
            N = 0.25 * (1 + sgn[:, 0] * xi) * (1 + sgn[:, 1] * eta)
            dN_dxi = 0.25 * sgn[:, 0] * (1 + sgn[:, 1] * eta)
            dN_deta = 0.25 * sgn[:, 1] * (1 + sgn[:, 0] * xi)
            J00 = xe[:, :, 0] @ dN_dxi
            J01 = xe[:, :, 0] @ dN_deta
            J10 = xe[:, :, 1] @ dN_dxi
            J11 = xe[:, :, 1] @ dN_deta
            detJ = np.abs(J00 * J11 - J01 * J10)
            for q in range(4):
                np.add.at(vol, E[:, q], N[q] * detJ)
    else:
        raise ValueError("nodal volumes are computed for triangles, quadrangles and tetrahedra")
    return vol


def nodes_at_centroid(mesh):
    """fe::Mesh::nodesAtCentroid (mesh.cpp:448-470) with
    util::geometry::getCenterAndVol (utilGeom.cpp:214-279): one node per
    element; triangle and tetrahedron: vertex mean and |size|; quadrangle: the
    one-point Gauss rule, i.e. the vertex mean and 4 |det J(0, 0)|."""
    x = mesh.nodes
    E = mesh.elements
    if mesh.element_type == VTK_TRIANGLE:
        a, b, c = x[E[:, 0]], x[E[:, 1]], x[E[:, 2]]
        vol = 0.5 * np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) -
                           (c[:, 0] - a[:, 0]) * (b[:, 1] - a[:, 1]))
        cen = a / 3. + b / 3. + c / 3.
    elif mesh.element_type == VTK_QUAD:
        q = x[E]
        cen = 0.25 * (q[:, 0] + q[:, 1] + q[:, 2] + q[:, 3])
        # d x / d xi and d x / d eta of the bilinear map at the centre
        dxi = 0.25 * (-q[:, 0] + q[:, 1] + q[:, 2] - q[:, 3])
        deta = 0.25 * (-q[:, 0] - q[:, 1] + q[:, 2] + q[:, 3])
        vol = 4.0 * np.abs(dxi[:, 0] * deta[:, 1] - dxi[:, 1] * deta[:, 0])
    elif mesh.element_type == VTK_TETRA:
        a, b, c, d = (x[E[:, q]] for q in range(4))
        vol = np.abs(np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a))) / 6.0
        cen = a / 4. + b / 4. + c / 4. + d / 4.
    else:
        raise ValueError("centroid nodes are built from triangles, quadrangles or tetrahedra")
    return Mesh(nodes=cen, volumes=vol)


def mesh_size(nodes):
    """fe::Mesh::computeMeshSize (mesh.cpp:326-350): start from |x_0 - x_1| and
    take every pair distance that is definitelyLessThan the current guess, in
    row order."""
    x = np.asarray(nodes, dtype=np.float64).reshape(-1, 3)
    n = x.shape[0]
    if n < 2:
        return 0.0
    d01 = x[0] - x[1]
    guess = float(np.sqrt(d01[0] * d01[0] + d01[1] * d01[1] + d01[2] * d01[2]))
    for i in range(n):
        dd = x[i] - x
        val = np.sqrt(dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1] + dd[:, 2] * dd[:, 2])
        val[i] = np.inf
        while True:
            less = (guess - val) > np.maximum(np.abs(val), abs(guess)) * 1e-5
            if not less.any():
                break
            j = int(np.argmax(less))
            guess = float(val[j])
            val[:j + 1] = np.inf
    return guess


def read_mesh(path, dim, finite_difference=True, centroid_based=False):
    """fe::Mesh::createData: the reader by extension, then nodal volumes for
    a finite-difference model when the file holds none."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".csv":
        if not finite_difference:
            raise ValueError("a .csv mesh is for finite-difference models")
        mesh = read_csv(path, dim)
    elif ext == ".msh":
        mesh = read_msh(path, dim)
    elif ext == ".vtu":
        mesh = read_vtu_mesh(path, dim, finite_difference)
    else:
        raise ValueError("mesh file %s: expected .csv, .msh or .vtu" % path)
    if centroid_based and mesh.elements is not None and finite_difference:
        return nodes_at_centroid(mesh)
    if finite_difference and mesh.volumes is None:
        mesh.volumes = compute_volumes(mesh)
    return mesh
