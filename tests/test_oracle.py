"""The oracle (CPU restatement) against the reference: committed golden vectors
everywhere, and the reference's own code compiled here when its tree exists."""
import os

import numpy as np
import pytest

import pyoracle as O
from conftest import golden_cases, load_golden
from minifem.meshgen import cube_mesh, cube_sizes


@pytest.mark.parametrize("name", golden_cases())
def test_port_matches_golden(name):
    g = load_golden(name)
    op = str(g["op"])
    N = g["coord"].shape[0]
    row, col = O.pattern(g["elemToNode"], N)
    assert np.array_equal(row, g["row"]) and np.array_equal(col, g["col"])
    assert np.array_equal(O.elem_to_edge(row, col, g["elemToNode"]), g["elemToEdge"])
    vals = O.assembly(g["coord"], row, col, g["elemToNode"], int(g["nbEdges"]), op)
    assert vals.tobytes() == g["values"].tobytes()
    markf = O.checkbounds(g["boundNodesCode"])
    assert np.array_equal(markf, g["checkBounds"])
    prec, _ = O.prec(vals, row, col, markf, N, op)
    assert prec.tobytes() == g["prec"].tobytes()
    assert O.norm(vals) == float(g["matrix_norm"])


@pytest.mark.parametrize("name", golden_cases())
def test_port_colouring_matches_golden(name):
    g = load_golden(name)
    op = str(g["op"])
    N = g["coord"].shape[0]
    part, index = O.coloring(g["elemToNode"], N)
    assert np.array_equal(index, g["color_index"])
    # stable colour order, then the COLORING build's values
    order = np.argsort(part, kind="stable")
    assert np.array_equal(np.asarray(g["color_perm"])[order], np.arange(len(order)))
    e2n_c = g["elemToNode"][order]
    assert np.array_equal(e2n_c, g["color_elemToNode"])
    row, col = O.pattern(e2n_c, N)
    vals = O.assembly(g["coord"], row, col, e2n_c, int(g["nbEdges"]), op)
    assert vals.tobytes() == g["color_values"].tobytes()


def test_single_tet_closed_form():
    """Right-angle tet (0,0,0),(1,0,0),(0,1,0),(0,0,1): with the reference's
    b/c order the signed 6V is -1 and the gradients are +-unit vectors."""
    g = load_golden("tet_lap")
    vals = g["values"].reshape(4, 4)
    # barycentric gradients: n0 -> (-1,-1,-1), n1 -> e_x, n2 -> e_y, n3 -> e_z
    G = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    # the reference's rows are g0 = b x c / vol etc.; the Laplacian block is G G^T up to
    # the row order the reference's elemCoef produces
    gram = G @ G.T
    assert sorted(np.diag(vals)) == sorted(np.diag(gram))
    assert np.isclose(vals.sum(), 0.0)


def test_norm_is_reference_formula():
    x = np.array([3.0, 4.0])
    assert O.norm(x) == 5.0


REF = O.ref_available()


@pytest.mark.skipif(not (REF and O.build_ref()), reason="reference tree not present")
@pytest.mark.parametrize("n,op,seed,jit", [(7, "lap", 1, 0.2), (7, "ela", 2, 0.2),
                                           (9, "ela", 3, 0.45), (12, "ela", 4, 0.2)])
def test_port_matches_reference_build(n, op, seed, jit):
    m = cube_mesh(n, seed=seed, op=op, jitter=jit, coefficients=False)
    R = O.Ref("ref")
    E, N, nnz = cube_sizes(n)
    row, col = R.pattern(m.elemToNode, N, nnz)
    prow, pcol = O.pattern(m.elemToNode, N)
    assert np.array_equal(row, prow) and np.array_equal(col, pcol)
    v = R.assembly(m.coord, row, col, m.elemToNode, nnz, op)
    assert v.tobytes() == O.assembly(m.coord, row, col, m.elemToNode, nnz, op).tobytes()
    mk = O.checkbounds(m.boundNodesCode)
    assert R.prec(v, row, col, mk, N, op).tobytes() == O.prec(v, row, col, mk, N, op)[0].tobytes()


@pytest.mark.skipif(not (REF and O.build_ref()), reason="reference tree not present")
def test_reference_driver_end_to_end(tmp_path):
    """The reference's own main.cc/FEM.cc loop on a generated mesh tree: its
    numerical check (src/FEM.cc:59-98) against the oracle's norms."""
    import subprocess
    m = cube_mesh(6, seed=9, op="ela", coefficients=False)
    r = O.full(m, coef=None)
    from minifem.meshgen import write_reference_tree
    write_reference_tree(m, str(tmp_path), "LM6", "ela", O.norm(r["values"]), O.norm(r["prec"]))
    exe = os.path.join(O.REF_DIR, "miniFEM_ref")
    out = subprocess.run([exe, "LM6", "ela", "3"], cwd=tmp_path, capture_output=True, text=True,
                         env={**os.environ, "MINIFEM_DATA_PATH": str(tmp_path)}, timeout=60)
    assert out.returncode == 0, out.stderr
    diffs = [float(l.split(":")[1]) for l in out.stdout.splitlines() if "difference" in l]
    assert diffs == [0.0, 0.0], out.stdout
