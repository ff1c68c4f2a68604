"""Mesh import for the drop-in driver.

Reads tetrahedral meshes from Gmsh files (ASCII, format 2.2 or 4.1) and legacy
VTK unstructured grids (ASCII) and writes them in the reference's input layout
(src/IO.cc:61-96, the tree of src/IO.cc:66-68) -- the job of the mesh writer
the reference relies on (DefMesh's `store_input_data_`, src/IO.cc:99-127), which
is not part of the reference tree.

Boundary codes (src/Fortran/qdmrd4.f: 52 fixes x, 53 y, 54 z, any other
non-zero code all three) come from tagged boundary triangles: `codes` maps a
Gmsh physical tag to a code, applied in the mapping's order (a node on faces
of several tags keeps the code of the last one); a VTK file may carry them as
the point scalars `boundNodesCode`.

    python -m minifem.meshio in.msh <root> <mesh_name> <lap|ela> [--code TAG=CODE ...]
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from .meshgen import Mesh, write_reference_tree

TET, TRI = 4, 2                     # Gmsh element types
VTK_TET = 10


def count_nnz(elemToNode: np.ndarray, nbNodes: int) -> int:
    """Entries of the CSR pattern (node pairs sharing an element, diagonal
    included): the nbEdges the reference reads from the mesh file and that must
    equal the pattern's size (src/main.cc:246)."""
    e = np.asarray(elemToNode, dtype=np.int64) - 1
    a = np.repeat(e, 4, axis=1).reshape(-1)
    b = np.tile(e, (1, 4)).reshape(-1)
    return int(np.unique(a * nbNodes + b).size)


def _codes_from_faces(nbNodes, faces, face_tags, codes):
    out = np.zeros(nbNodes, np.int32)
    if not codes or faces is None or len(faces) == 0:
        return out
    for tag, code in codes.items():
        sel = faces[face_tags == tag]
        if len(sel):
            out[np.unique(sel.reshape(-1)) - 1] = code
    return out


def _mesh(coord, tets, code, op):
    coord = np.ascontiguousarray(coord, np.float64)
    tets = np.ascontiguousarray(tets, np.int32)
    return Mesh(coord=coord, elemToNode=tets, boundNodesCode=np.ascontiguousarray(code, np.int32),
                nbEdges=count_nnz(tets, len(coord)), coef=None, op=op,
                meta={"imported": True})


def _renumber(tags, tets, faces):
    """Node tags (any positive integers) -> 1..N in ascending tag order."""
    order = np.argsort(tags, kind="stable")
    lut = np.zeros(int(tags.max()) + 1, np.int64)
    lut[tags[order]] = np.arange(1, len(tags) + 1)
    t = lut[tets]
    f = lut[faces] if faces is not None and len(faces) else faces
    if (t == 0).any():
        raise ValueError("an element references a node that is not defined")
    return order, t, f


def _sections(lines):
    out, i = {}, 0
    while i < len(lines):
        ln = lines[i].strip()
        if ln.startswith("$") and not ln.startswith("$End"):
            name = ln[1:]
            j = i + 1
            while j < len(lines) and lines[j].strip() != "$End" + name:
                j += 1
            out[name] = lines[i + 1:j]
            i = j
        i += 1
    return out


def read_gmsh(path: str, codes: dict | None = None, op: str = "ela") -> Mesh:
    """Tetrahedra (type 4) of a Gmsh ASCII file, format 2.2 or 4.1; boundary codes
    from triangles (type 2) by physical tag."""
    with open(path) as f:
        sec = _sections(f.read().splitlines())
    if "MeshFormat" not in sec:
        raise ValueError(f"{path}: not a Gmsh file")
    version = sec["MeshFormat"][0].split()
    if version[1] != "0":
        raise ValueError(f"{path}: binary Gmsh files are not supported")
    major = int(float(version[0]))
    if major == 2:
        nl = sec["Nodes"]
        n = int(nl[0])
        arr = np.array([ln.split() for ln in nl[1:1 + n]], dtype=np.float64)
        tags, coord = arr[:, 0].astype(np.int64), arr[:, 1:4]
        el = sec["Elements"]
        m = int(el[0])
        tets, faces, ftags = [], [], []
        for ln in el[1:1 + m]:
            v = [int(x) for x in ln.split()]
            typ, ntag = v[1], v[2]
            nodes = v[3 + ntag:]
            if typ == TET:
                tets.append(nodes[:4])
            elif typ == TRI:
                faces.append(nodes[:3])
                ftags.append(v[3] if ntag > 0 else 0)
    elif major == 4:
        phys = {}
        if "Entities" in sec:
            ent = sec["Entities"]
            counts = [int(x) for x in ent[0].split()]
            k = 1
            for dim, cnt in enumerate(counts):
                for _ in range(cnt):
                    v = ent[k].split()
                    k += 1
                    tag = int(v[0])
                    p = 4 if dim == 0 else 7          # after the point or the bounding box
                    nphys = int(v[p])
                    phys[(dim, tag)] = [int(x) for x in v[p + 1:p + 1 + nphys]]
        nl = sec["Nodes"]
        nblocks = int(nl[0].split()[0])
        k, tags, coord = 1, [], []
        for _ in range(nblocks):
            _, _, param, cnt = (int(x) for x in nl[k].split())
            k += 1
            tags.extend(int(nl[k + i]) for i in range(cnt))
            k += cnt
            for i in range(cnt):
                coord.append([float(x) for x in nl[k + i].split()[:3]])
            k += cnt
        tags, coord = np.array(tags, np.int64), np.array(coord, np.float64)
        el = sec["Elements"]
        nblocks = int(el[0].split()[0])
        k, tets, faces, ftags = 1, [], [], []
        for _ in range(nblocks):
            dim, etag, typ, cnt = (int(x) for x in el[k].split())
            k += 1
            for i in range(cnt):
                v = [int(x) for x in el[k + i].split()]
                if typ == TET:
                    tets.append(v[1:5])
                elif typ == TRI:
                    faces.append(v[1:4])
                    pt = phys.get((dim, etag), [])
                    ftags.append(pt[0] if pt else 0)
            k += cnt
    else:
        raise ValueError(f"{path}: Gmsh format {version[0]} is not supported")
    if not tets:
        raise ValueError(f"{path}: no tetrahedra")
    faces_a = np.array(faces, np.int64) if faces else None
    order, t, f = _renumber(tags, np.array(tets, np.int64), faces_a)
    code = _codes_from_faces(len(tags), f, np.array(ftags, np.int64), codes)
    return _mesh(coord[order], t, code, op)


def read_vtk(path: str, op: str = "ela") -> Mesh:
    """Tetrahedra (cell type 10) of a legacy ASCII VTK unstructured grid; point
    scalars named boundNodesCode, if present, are the boundary codes."""
    with open(path) as f:
        tok = f.read().split()
    up = [t.upper() for t in tok]
    if "UNSTRUCTURED_GRID" not in up or "ASCII" not in up:
        raise ValueError(f"{path}: not an ASCII unstructured-grid VTK file")
    i = up.index("POINTS")
    n = int(tok[i + 1])
    coord = np.array(tok[i + 3:i + 3 + 3 * n], dtype=np.float64).reshape(n, 3)
    i = up.index("CELLS")
    m, size = int(tok[i + 1]), int(tok[i + 2])
    cells = np.array(tok[i + 3:i + 3 + size], dtype=np.int64)
    i = up.index("CELL_TYPES")
    types = np.array(tok[i + 2:i + 2 + m], dtype=np.int64)
    tets, k = [], 0
    for c in range(m):
        cnt = int(cells[k])
        if types[c] == VTK_TET:
            tets.append(cells[k + 1:k + 1 + cnt])
        k += cnt + 1
    if not tets:
        raise ValueError(f"{path}: no tetrahedra")
    code = np.zeros(n, np.int32)
    for j in range(len(tok) - 1):
        if up[j] == "SCALARS" and tok[j + 1] == "boundNodesCode":
            s = j + 2
            while up[s] != "LOOKUP_TABLE":
                s += 1
            code = np.array(tok[s + 2:s + 2 + n], dtype=np.float64).astype(np.int32)
    return _mesh(coord, np.array(tets, np.int64) + 1, code, op)


def read_mesh(path: str, codes: dict | None = None, op: str = "ela") -> Mesh:
    ext = os.path.splitext(path)[1].lower()
    if ext == ".msh":
        return read_gmsh(path, codes, op)
    if ext == ".vtk":
        return read_vtk(path, op)
    raise ValueError(f"{path}: unknown mesh format (.msh or .vtk)")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("input")
    ap.add_argument("root")
    ap.add_argument("mesh_name")
    ap.add_argument("op", choices=["lap", "ela"])
    ap.add_argument("--code", action="append", default=[],
                    help="TAG=CODE: boundary code of the triangles of a Gmsh physical tag")
    a = ap.parse_args(argv)
    codes = {}
    for c in a.code:
        t, v = c.split("=")
        codes[int(t)] = int(v)
    mesh = read_mesh(a.input, codes, a.op)
    path = write_reference_tree(mesh, a.root, a.mesh_name, a.op)
    print(f"{path}: {mesh.nbElem} elements, {mesh.nbNodes} nodes, {mesh.nbEdges} CSR entries")


if __name__ == "__main__":
    main()
