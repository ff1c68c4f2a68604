"""Mesh import (Gmsh 2.2 / 4.1 ASCII, legacy VTK) into the reference's input
layout: the imported mesh equals the generated one it was written from,
boundary codes from tagged faces included."""
import os

import numpy as np
import pytest

from minifem import meshio
from minifem.meshgen import cube_mesh, read_reference_input

# face tags of the unit cube's sides, in the order the generator applies codes
TAG_Z0, TAG_Y0, TAG_X0, TAG_OUT = 3, 2, 1, 4
CODES = {TAG_Z0: 54, TAG_Y0: 53, TAG_X0: 52, TAG_OUT: 10}


def _boundary_faces(m):
    """Boundary triangles (faces of one tetrahedron only) with the tag of the
    cube side they lie on."""
    e = m.elemToNode
    faces = np.concatenate([e[:, [0, 1, 2]], e[:, [0, 1, 3]], e[:, [0, 2, 3]], e[:, [1, 2, 3]]])
    key = np.sort(faces, axis=1)
    _, idx, cnt = np.unique(key, axis=0, return_index=True, return_counts=True)
    bf = faces[idx[cnt == 1]]
    x = m.coord[bf - 1]                                   # (F, 3, 3)
    tags = np.full(len(bf), TAG_OUT)
    for d, t in ((0, TAG_X0), (1, TAG_Y0), (2, TAG_Z0)):
        tags[np.all(x[:, :, d] == 0.0, axis=1)] = t
    return bf, tags


def _write_msh22(path, m, node_tags):
    bf, ft = _boundary_faces(m)
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % m.nbNodes)
        for t, (x, y, z) in zip(node_tags, m.coord):
            f.write(f"{t} {float(x)!r} {float(y)!r} {float(z)!r}\n")
        f.write("$EndNodes\n$Elements\n%d\n" % (len(bf) + m.nbElem))
        k = 1
        for face, tag in zip(bf, ft):
            n = node_tags[face - 1]
            f.write(f"{k} 2 2 {tag} {tag} {n[0]} {n[1]} {n[2]}\n")
            k += 1
        for el in m.elemToNode:
            n = node_tags[el - 1]
            f.write(f"{k} 4 2 9 9 {n[0]} {n[1]} {n[2]} {n[3]}\n")
            k += 1
        f.write("$EndElements\n")


def _write_msh41(path, m):
    bf, ft = _boundary_faces(m)
    with open(path, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n$Entities\n0 0 4 1\n")
        for s in (1, 2, 3, 4):       # surface entity s carries physical tag s
            f.write(f"{s} 0 0 0 1 1 1 1 {s} 0\n")
        f.write("1 0 0 0 1 1 1 1 9 0\n$EndEntities\n")
        f.write(f"$Nodes\n1 {m.nbNodes} 1 {m.nbNodes}\n3 1 0 {m.nbNodes}\n")
        for i in range(m.nbNodes):
            f.write(f"{i + 1}\n")
        for x, y, z in m.coord:
            f.write(f"{float(x)!r} {float(y)!r} {float(z)!r}\n")
        f.write("$EndNodes\n$Elements\n5 %d 1 %d\n" % (len(bf) + m.nbElem, len(bf) + m.nbElem))
        k = 1
        for s in (1, 2, 3, 4):
            sel = bf[ft == s]
            f.write(f"2 {s} 2 {len(sel)}\n")
            for face in sel:
                f.write(f"{k} {face[0]} {face[1]} {face[2]}\n")
                k += 1
        f.write(f"3 1 4 {m.nbElem}\n")
        for el in m.elemToNode:
            f.write(f"{k} {el[0]} {el[1]} {el[2]} {el[3]}\n")
            k += 1
        f.write("$EndElements\n")


def _write_vtk(path, m):
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\nmesh\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {m.nbNodes} double\n")
        for x, y, z in m.coord:
            f.write(f"{float(x)!r} {float(y)!r} {float(z)!r}\n")
        f.write(f"CELLS {m.nbElem} {5 * m.nbElem}\n")
        for el in m.elemToNode - 1:
            f.write(f"4 {el[0]} {el[1]} {el[2]} {el[3]}\n")
        f.write(f"CELL_TYPES {m.nbElem}\n" + "10\n" * m.nbElem)
        f.write(f"POINT_DATA {m.nbNodes}\nSCALARS boundNodesCode int 1\nLOOKUP_TABLE default\n")
        f.write("\n".join(str(int(c)) for c in m.boundNodesCode) + "\n")


def _same(a, b):
    assert np.array_equal(a.coord, b.coord)
    assert np.array_equal(a.elemToNode, b.elemToNode)
    assert np.array_equal(a.boundNodesCode, b.boundNodesCode)
    assert a.nbEdges == b.nbEdges


@pytest.fixture(scope="module")
def mesh():
    return cube_mesh(4, seed=1, op="ela")


def test_count_nnz_matches_the_pattern_size(mesh):
    assert meshio.count_nnz(mesh.elemToNode, mesh.nbNodes) == mesh.nbEdges


def test_gmsh22_roundtrip(tmp_path, mesh):
    p = str(tmp_path / "cube.msh")
    _write_msh22(p, mesh, np.arange(1, mesh.nbNodes + 1))
    _same(meshio.read_gmsh(p, CODES), mesh)


def test_gmsh22_node_tags_are_renumbered(tmp_path, mesh):
    """Node tags need not be 1..N: they are renumbered in ascending tag order."""
    tags = 1000 + 7 * np.random.default_rng(3).permutation(mesh.nbNodes)
    p = str(tmp_path / "cube.msh")
    _write_msh22(p, mesh, tags)
    got = meshio.read_gmsh(p, CODES)
    new = np.argsort(np.argsort(tags)) + 1                # new number of old node i
    assert np.array_equal(got.elemToNode, new[mesh.elemToNode - 1])
    coord = np.empty_like(mesh.coord)
    coord[new - 1] = mesh.coord
    assert np.array_equal(got.coord, coord)
    code = np.empty_like(mesh.boundNodesCode)
    code[new - 1] = mesh.boundNodesCode
    assert np.array_equal(got.boundNodesCode, code)


def test_gmsh41_roundtrip(tmp_path, mesh):
    p = str(tmp_path / "cube41.msh")
    _write_msh41(p, mesh)
    _same(meshio.read_gmsh(p, CODES), mesh)


def test_vtk_roundtrip(tmp_path, mesh):
    p = str(tmp_path / "cube.vtk")
    _write_vtk(p, mesh)
    _same(meshio.read_vtk(p), mesh)


def test_cli_writes_the_reference_tree(tmp_path, mesh):
    p = str(tmp_path / "cube.msh")
    _write_msh22(p, mesh, np.arange(1, mesh.nbNodes + 1))
    root = str(tmp_path / "data")
    meshio.main([p, root, "CUBE", "ela"] + [f"--code={t}={c}" for t, c in CODES.items()])
    got = read_reference_input(os.path.join(root, "CUBE", "inputs", "ela_1_0"))
    _same(got, mesh)


def test_rejects_files_without_tetrahedra(tmp_path):
    p = str(tmp_path / "empty.msh")
    with open(p, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n"
                "$Elements\n0\n$EndElements\n")
    with pytest.raises(ValueError):
        meshio.read_gmsh(p)
