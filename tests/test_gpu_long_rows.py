"""Rows far longer than a cube's: the fan mesh, whose centre node touches every
element and whose CSR row holds every node.  The pattern builder takes rows of
more than 128 entries to one CTA each; the FP32 path falls back from the row
tiles to the per-element kernel when a node touches more elements than a tile
holds.  The pattern (both column orders) and the FP64 gather are bit-exact with
the oracle, FP32 within its tolerance."""
import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import fan_mesh
from test_gpu_parity import TOL_FP32, contribution_scale, gpu_full, keyed

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("subdivisions", [2, 3])
@pytest.mark.parametrize("op", ["lap", "ela"])
@pytest.mark.parametrize("order", ["reference", "sorted"])
def test_fan_mesh_fp64_bit_exact(gpu, subdivisions, op, order):
    m = fan_mesh(subdivisions, seed=5 + subdivisions, op=op)
    row, col, vals, prec = gpu_full(gpu, m, op, m.coef, order)
    ref = O.full(m, op=op, coef=m.coef)
    assert int(row[-1]) == m.nbEdges and np.diff(row).max() == m.nbNodes
    if order == "reference":
        assert np.array_equal(row, ref["row"]) and np.array_equal(col, ref["col"])
        assert vals.tobytes() == ref["values"].tobytes()
    else:
        d = O.op_dim(op)
        r1, c1, v1 = keyed(row, col, vals, d)
        r2, c2, v2 = keyed(ref["row"], ref["col"], ref["values"], d)
        assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
        assert v1.tobytes() == v2.tobytes()
        # columns ascend within every row
        rr = np.repeat(np.arange(len(row) - 1), np.diff(row))
        assert np.all((np.diff(col) > 0) | (np.diff(rr) != 0))
    assert prec.tobytes() == ref["prec"].tobytes()


def test_fan_mesh_elem_to_edge(gpu):
    m = fan_mesh(3, seed=2)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("reference")
    assert np.array_equal(a.create_elemToEdge(), O.elem_to_edge(row, col, m.elemToNode))


def uv_fan(nlon, nlat, seed, op):
    """Fan over a latitude-longitude sphere: nlon * (nlat - 1) + 2 surface nodes,
    twice as many triangles less four.  At (18, 8) the centre row has 129 entries
    (past the 128 of the per-thread pattern pass) and the centre's diagonal 252
    contributions (within the row tiles' 255)."""
    from minifem.meshgen import Mesh, coefficient_set
    th = np.pi * np.arange(1, nlat) / nlat
    ph = 2 * np.pi * np.arange(nlon) / nlon
    ring = np.stack([np.outer(np.sin(th), np.cos(ph)), np.outer(np.sin(th), np.sin(ph)),
                     np.outer(np.cos(th), np.ones(nlon))], axis=2).reshape(-1, 3)
    sv = np.vstack([[0, 0, 1], ring, [0, 0, -1]])
    idx = lambda i, j: 1 + i * nlon + (j % nlon)
    tri = []
    for j in range(nlon):
        tri.append((0, idx(0, j), idx(0, j + 1)))
        tri.append((len(sv) - 1, idx(nlat - 2, j + 1), idx(nlat - 2, j)))
        for i in range(nlat - 2):
            tri.append((idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)))
            tri.append((idx(i, j), idx(i + 1, j + 1), idx(i, j + 1)))
    tri = np.array(tri) + 1
    coord = np.vstack([np.zeros((1, 3)), sv])
    e2n = np.concatenate([np.zeros((len(tri), 1), np.int64), tri], axis=1)
    X = coord[e2n]
    vol = np.einsum("ij,ij->i", X[:, 0] - X[:, 3], np.cross(X[:, 2] - X[:, 3], X[:, 1] - X[:, 3]))
    e2n[vol < 0] = e2n[vol < 0][:, [0, 2, 1, 3]]
    perm = np.random.default_rng(seed).permutation(len(coord))
    code = np.where(coord[:, 2] < 0, 10, 0).astype(np.int32)
    newOfOld = np.empty_like(perm)
    newOfOld[perm] = np.arange(len(perm))
    return Mesh(coord=np.ascontiguousarray(coord[perm]),
                elemToNode=np.ascontiguousarray(newOfOld[e2n] + 1, dtype=np.int32),
                boundNodesCode=code[perm], nbEdges=0, coef=coefficient_set(op, len(tri), seed),
                op=op)


@pytest.mark.parametrize("mesh,tile,fits", [("uv", None, True), ("ico2", None, False),
                                             ("ico3", None, False), ("uv", (8, 128), False)])
@pytest.mark.parametrize("op", ["lap", "ela"])
def test_fan_mesh_fp32_within_tolerance(gpu, mesh, tile, fits, op):
    """The latitude-longitude fan fits the default row tiles; the icosphere fans
    (320 and 1280 contributions to the centre's diagonal) and 128-element tiles
    do not, and the per-element kernel assembles."""
    m = uv_fan(18, 8, 9, op) if mesh == "uv" else fan_mesh(int(mesh[3:]), seed=9, op=op)
    a = gpu(0)
    a.set_option("fp32_kernel", 1)
    if tile:
        a.set_option("tile_rows", tile[0])
        a.set_option("tile_elems", tile[1])
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("reference")
    assert np.diff(row).max() == m.nbNodes > 128
    a.set_coefficients(op, m.coef)
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.assembly(op, "fp32", "gather", prec=True)
    if fits:
        assert a.tile_info()["tiles"] > 0
    else:
        with pytest.raises(Exception, match="does not fit"):
            a.tile_info()
    v32 = a.values_f32().astype(np.float64)
    ref = O.full(m, op=op, coef=m.coef)
    d = O.op_dim(op)
    S = contribution_scale(m, ref["row"], ref["col"], op, m.coef)
    err = np.abs(v32.reshape(-1, d) - ref["values"].reshape(-1, d)) / S[:, None]
    assert err.max() < TOL_FP32, err.max()
    p = a.prec()
    rel = np.abs(p - ref["prec"]) / (np.abs(ref["prec"]).reshape(-1, d).max(axis=1).repeat(d) + 1e-300)
    assert rel.max() < 1e-4


def test_uv_fan_fp64_bit_exact(gpu):
    m = uv_fan(18, 8, 3, "ela")
    row, col, vals, prec = gpu_full(gpu, m, "ela", m.coef, "reference")
    ref = O.full(m, op="ela", coef=m.coef)
    assert np.array_equal(row, ref["row"]) and np.array_equal(col, ref["col"])
    assert vals.tobytes() == ref["values"].tobytes()
    assert prec.tobytes() == ref["prec"].tobytes()


def test_fan_mesh_unfit_for_batch_is_reported(gpu):
    import minifem
    m = fan_mesh(3, seed=1, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    b = minifem.Batch(0)
    with pytest.raises(Exception):
        b.add(a, "ela", m.coef[None])
        b.assemble("fp32", prec=True)
        b.synchronize()
    # the context stays usable
    a.set_coefficients("ela", m.coef)
    a.assembly("ela", "fp64", "gather", prec=True)
    assert np.all(np.isfinite(a.values()))


def test_node_beyond_the_long_row_limit_is_reported(gpu):
    """A node touching 5120 elements (4 subdivisions) is past the pattern
    builder's 4096: the call fails with an error before the long-row pass is launched."""
    m = fan_mesh(4, seed=1, op="lap")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    with pytest.raises(Exception):
        a.create_nodeToNode("reference")


def test_fan_mesh_needs_more_colours_than_the_reference_allows(gpu):
    """Every element of the fan mesh touches the centre, so each needs its own
    colour: past 128 colours the colouring fails as the reference's does
    (coloring.cc:66-69), and the context stays usable."""
    m = fan_mesh(3, seed=4, op="lap")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("reference")
    with pytest.raises(Exception, match="colors"):
        a.coloring_creation(seed=1)
    a.set_coefficients("lap", m.coef)
    a.assembly("lap", "fp64", "gather")
    ref = O.full(m, op="lap", coef=m.coef)
    assert a.values().tobytes() == ref["values"].tobytes()
