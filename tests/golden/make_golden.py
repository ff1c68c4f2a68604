"""Generate the committed golden fixtures from the reference's own operators.

Run in a checkout that has the reference tree (its root: --ref-root, else
$MINIFEM_REF_ROOT, else the REF_ROOT default of oracle/Makefile):

    python tests/golden/make_golden.py [--ref-root <reference root>]

It compiles the reference sources with the stand-ins of oracle/shim (make -C
oracle ref), runs the reference's create_nodeToNode / create_elemToEdge /
assembly / prec_init / prec_inversion (REF build) and coloring_creation +
colour-ordered assembly (COLORING build) on small meshes, and stores inputs and
outputs as .npz files beside this script.  The GPU tests compare against these
files on machines where the reference tree is absent.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "mini-fem_gb300"))

import pyoracle as O  # noqa: E402
from minifem.meshgen import Mesh, cube_mesh  # noqa: E402


def single_tet(op: str) -> Mesh:
    """The right-angle unit tetrahedron; its gradients are known in closed form
    (g0 = -(1,1,1)-ish permuted by the reference's b/c ordering)."""
    coord = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    e2n = np.array([[1, 2, 3, 4]], dtype=np.int32)
    code = np.array([0, 52, 53, 10], dtype=np.int32)
    return Mesh(coord=coord, elemToNode=e2n, boundNodesCode=code, nbEdges=16, op=op)


CASES = {
    "tet_lap": lambda: single_tet("lap"),
    "tet_ela": lambda: single_tet("ela"),
    "cube2_lap": lambda: cube_mesh(2, seed=0, op="lap", jitter=0.0, permute=False,
                                   coefficients=False),
    "cube2_ela": lambda: cube_mesh(2, seed=0, op="ela", jitter=0.0, permute=False,
                                   coefficients=False),
    "n4_lap": lambda: cube_mesh(4, seed=11, op="lap", coefficients=False),
    "n4_ela": lambda: cube_mesh(4, seed=12, op="ela", coefficients=False),
    "n5_stress_ela": lambda: cube_mesh(5, seed=13, op="ela", jitter=0.45,
                                       coefficients=False, sliver_fraction=0.05),
}


def make(name: str, mesh: Mesh) -> dict:
    op = mesh.op
    R, RC = O.Ref("ref"), O.Ref("coloring")
    N, E = mesh.nbNodes, mesh.nbElem
    row, col = R.pattern(mesh.elemToNode, N, mesh.nbEdges)
    e2e = R.elem_to_edge(row, col, mesh.elemToNode)
    vals = R.assembly(mesh.coord, row, col, mesh.elemToNode, mesh.nbEdges, op)
    markf = O.checkbounds(mesh.boundNodesCode)
    prec = R.prec(vals, row, col, markf, N, op)
    # COLORING build: colour, permute the elements, rebuild the CSR, assemble
    e2n_c, perm, cidx = RC.coloring(mesh.elemToNode, N)
    row_c, col_c = RC.pattern(e2n_c, N, mesh.nbEdges)
    vals_c = RC.assembly(mesh.coord, row_c, col_c, e2n_c, mesh.nbEdges, op)
    return {
        "op": np.array(op), "coord": mesh.coord, "elemToNode": mesh.elemToNode,
        "boundNodesCode": mesh.boundNodesCode, "nbEdges": np.array(mesh.nbEdges),
        "row": row, "col": col, "elemToEdge": e2e, "values": vals, "prec": prec,
        "checkBounds": markf,
        "matrix_norm": np.array(O.norm(vals)), "prec_norm": np.array(O.norm(prec)),
        "color_perm": perm, "color_index": cidx, "color_elemToNode": e2n_c,
        "color_row": row_c, "color_col": col_c, "color_values": vals_c,
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=None)
    args = ap.parse_args()
    if not O.build_ref(args.ref_root):
        sys.exit(f"cannot build the reference operators from {args.ref_root or O.ref_root()}")
    O.build_port()
    for name, fn in CASES.items():
        out = make(name, fn())
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: E={out['elemToNode'].shape[0]} N={out['coord'].shape[0]} "
              f"nnz={int(out['nbEdges'])} colours={len(out['color_index']) - 1}")


if __name__ == "__main__":
    main()
