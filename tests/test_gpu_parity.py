"""GPU path against the oracle: bit-exact for the FP64 gather (the reference's
summation order, -fmad=false), the pattern, positions and the preconditioner;
within stated tolerances for the colour scatter, the atomic strategy and FP32."""
import numpy as np
import pytest

import pyoracle as O
from conftest import golden_cases, load_golden
from minifem.meshgen import cube_mesh

pytestmark = pytest.mark.gpu

# FP64 strategies other than the ordered gather: error per entry relative to
# the sum of magnitudes of that entry's contributions (hard cancellation makes a
# plain relative error meaningless for near-zero entries).
TOL_FP64_REORDERED = 1e-13
# FP32 (compensated sums, FP64 slivers): error relative to the block scale
# sum_e |g_j| |g_k| max(A, B, mu) of the entry's contributions.
TOL_FP32 = 1e-6


def keyed(row, col, vals, dim):
    """{(r, c): block} dictionary-free form: sort entries by (row, col)."""
    N = len(row) - 1
    r = np.repeat(np.arange(N), np.diff(row))
    order = np.lexsort((col, r))
    return r[order], col[order], vals.reshape(-1, dim)[order]


def contribution_scale(mesh, row, col, op, coef):
    """Per-entry sum of |contribution| magnitudes (FP64), keyed like `keyed`."""
    e2e = O.elem_to_edge(row, col, mesh.elemToNode).reshape(-1, 16)
    X = mesh.coord[mesh.elemToNode - 1]
    a, b, c = X[:, 0] - X[:, 3], X[:, 2] - X[:, 3], X[:, 1] - X[:, 3]
    G = np.empty((len(a), 4, 3))
    # rows as assembly.cc:106-114 forms them: g0 = b x c, g1 = a x b, g2 = c x a
    G[:, 0] = np.cross(b, c); G[:, 1] = np.cross(a, b); G[:, 2] = np.cross(c, a)
    G[:, 3] = -(G[:, 0] + G[:, 1] + G[:, 2])
    vol = np.einsum("ij,ij->i", a, G[:, 0])
    G /= vol[:, None, None]
    gn = np.linalg.norm(G, axis=2)
    if coef is None:
        w = np.full(len(a), 2.25 if op == "ela" else 1.0)
    elif op == "lap":
        w = coef
    else:
        E, nu = coef[:, 0], coef[:, 1]
        lam = E * nu / ((1 + nu) * (1 - 2 * nu)); mu = E / (2 * (1 + nu))
        w = lam + 2 * mu
    sc = (gn[:, :, None] * gn[:, None, :] * w[:, None, None]).reshape(-1)
    S = np.zeros(len(col)); np.add.at(S, e2e.reshape(-1), sc)
    return S


def gpu_full(Asm, mesh, op, coef, order="reference", precision="fp64", strategy="gather",
             fused=False):
    a = Asm(0)
    a.set_mesh(mesh.coord, mesh.elemToNode)
    row, col = a.create_nodeToNode(order)
    a.set_coefficients(op, coef)
    a.set_check_bounds(O.checkbounds(mesh.boundNodesCode))
    if strategy == "scatter":
        a.coloring_creation(seed=1)
    if fused:
        a.assembly(op, precision, strategy, prec=True)
    else:
        a.assembly(op, precision, strategy)
        a.prec_init()
        a.prec_inversion()
    vals = a.values()
    prec = a.prec()
    a.close()
    return row, col, vals, prec


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("fused", [False, True])
def test_gather_fp64_bit_exact_vs_golden(gpu, name, fused):
    g = load_golden(name)
    op = str(g["op"])

    class M:  # golden fixture as a mesh
        coord, elemToNode, boundNodesCode = g["coord"], g["elemToNode"], g["boundNodesCode"]
    row, col, vals, prec = gpu_full(gpu, M, op, None, "reference", fused=fused)
    assert np.array_equal(row, g["row"]) and np.array_equal(col, g["col"])
    assert vals.tobytes() == g["values"].tobytes()
    assert prec.tobytes() == g["prec"].tobytes()


@pytest.mark.parametrize("name", golden_cases())
def test_colour_ordered_golden_bit_exact(gpu, name):
    """The COLORING build's result (colour-permuted elements) is reproduced bit for
    bit by the gather on the permuted mesh: ascending element order is exactly
    its visiting order."""
    g = load_golden(name)
    op = str(g["op"])
    a = gpu(0)
    a.set_mesh(g["coord"], g["color_elemToNode"])
    row, col = a.create_nodeToNode("reference")
    assert np.array_equal(col, g["color_col"])
    a.assembly(op)
    assert a.values().tobytes() == g["color_values"].tobytes()


@pytest.mark.parametrize("n,op,seed,coef,jit", [
    (6, "lap", 1, False, 0.2), (6, "ela", 2, False, 0.2), (9, "lap", 3, True, 0.2),
    (9, "ela", 4, True, 0.2), (11, "ela", 5, True, 0.45), (14, "lap", 6, True, 0.2),
    (14, "ela", 7, True, 0.2)])
@pytest.mark.parametrize("order", ["sorted", "reference"])
def test_gather_fp64_bit_exact_vs_oracle(gpu, n, op, seed, coef, jit, order):
    m = cube_mesh(n, seed=seed, op=op, jitter=jit)
    c = m.coef if coef else None
    row, col, vals, prec = gpu_full(gpu, m, op, c, order)
    ref = O.full(m, op=op, coef=c)
    if order == "reference":
        assert np.array_equal(row, ref["row"]) and np.array_equal(col, ref["col"])
        assert vals.tobytes() == ref["values"].tobytes()
    else:
        # same entries, ascending columns
        d = O.op_dim(op)
        r1, c1, v1 = keyed(row, col, vals, d)
        r2, c2, v2 = keyed(ref["row"], ref["col"], ref["values"], d)
        assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
        assert v1.tobytes() == v2.tobytes()
    assert prec.tobytes() == ref["prec"].tobytes()


@pytest.mark.parametrize("op", ["lap", "ela"])
def test_fp64_gather_same_bits_concurrent_and_serial(gpu, op):
    """The diagonal and off-diagonal unit kernels run concurrently on two
    streams; with per-kernel profiling on they run one after the other.  Both
    give the oracle's bits (values and preconditioner)."""
    m = cube_mesh(12, seed=21, op=op)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("reference")
    a.set_coefficients(op, m.coef)
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.assembly(op, "fp64", "gather", prec=True)
    v1, p1 = a.values(), a.prec()
    a.profile(True)
    a.assembly(op, "fp64", "gather", prec=True)
    v2, p2 = a.values(), a.prec()
    a.profile(False)
    assert v1.tobytes() == v2.tobytes() and p1.tobytes() == p2.tobytes()
    ref = O.full(m, op=op, coef=m.coef)
    assert v1.tobytes() == ref["values"].tobytes() and p1.tobytes() == ref["prec"].tobytes()


def test_elem_to_edge_matches_reference(gpu):
    m = cube_mesh(8, seed=3)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("reference")
    assert np.array_equal(a.create_elemToEdge(), O.elem_to_edge(row, col, m.elemToNode))


@pytest.mark.parametrize("strategy", ["scatter", "atomic"])
@pytest.mark.parametrize("op,n", [("lap", 12), ("ela", 12), ("ela", 30)])
def test_reordered_fp64_strategies(gpu, strategy, op, n):
    m = cube_mesh(n, seed=8, op=op)
    row, col, vals, prec = gpu_full(gpu, m, op, m.coef, "reference", strategy=strategy)
    ref = O.full(m, op=op)
    d = O.op_dim(op)
    S = contribution_scale(m, ref["row"], ref["col"], op, m.coef)
    err = np.abs(vals.reshape(-1, d) - ref["values"].reshape(-1, d)) / S[:, None]
    assert err.max() < TOL_FP64_REORDERED


def test_colouring_is_valid(gpu):
    m = cube_mesh(10, seed=2)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    perm, index = a.coloring_creation(seed=5)
    E = m.nbElem
    assert sorted(perm) == list(range(E))
    assert index[0] == 0 and index[-1] == E and len(index) - 1 <= 128
    colour = np.searchsorted(index, perm, side="right") - 1
    # no two elements sharing a node carry the same colour
    for k in range(4):
        for l in range(k + 1, 4):
            pass
    node_col = {}
    for e in range(E):
        for nd in m.elemToNode[e]:
            key = (int(nd), int(colour[e]))
            assert key not in node_col, "colour conflict"
            node_col[key] = e
    # stable within a colour
    for c in range(len(index) - 1):
        members = np.nonzero(colour == c)[0]
        assert np.all(np.diff(perm[members]) == 1)


@pytest.mark.parametrize("kernel,tile", [(0, None), (1, None), (1, (8, 128))])
@pytest.mark.parametrize("op,n,jit,sliver", [("lap", 14, 0.2, 0.0), ("ela", 14, 0.2, 0.0),
                                              ("ela", 12, 0.45, 0.05)])
def test_fp32_within_tolerance(gpu, op, n, jit, sliver, kernel, tile):
    m = cube_mesh(n, seed=11, op=op, jitter=jit, sliver_fraction=sliver,
                  jump=1e6 if sliver else 1.0, nu_max=0.45 if sliver else 0.35)
    a = gpu(0)
    a.set_option("fp32_kernel", kernel)
    if tile:
        a.set_option("tile_rows", tile[0])
        a.set_option("tile_elems", tile[1])
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("reference")
    a.set_coefficients(op, m.coef)
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.assembly(op, "fp32", "gather", prec=True)
    v32 = a.values_f32().astype(np.float64)
    ref = O.full(m, op=op)
    d = O.op_dim(op)
    S = contribution_scale(m, ref["row"], ref["col"], op, m.coef)
    err = np.abs(v32.reshape(-1, d) - ref["values"].reshape(-1, d)) / S[:, None]
    assert err.max() < TOL_FP32, err.max()
    if sliver:
        assert a.flagged() > 0
    # the preconditioner: FP64 inverse of the compensated diagonal blocks
    p = a.prec()
    assert np.all(np.isfinite(p))
    rel = np.abs(p - ref["prec"]) / (np.abs(ref["prec"]).reshape(-1, d).max(axis=1).repeat(d) + 1e-300)
    assert rel.max() < 1e-4
    # deterministic: a second assembly gives the same bits
    a.assembly(op, "fp32", "gather", prec=True)
    assert a.values_f32().tobytes() == v32.astype(np.float32).tobytes()


def test_reference_shaped_calls_bit_exact(gpu):
    """assembly / prec_init / prec_inversion with the reference's arguments."""
    import minifem
    m = cube_mesh(8, seed=4, op="ela")
    ref = O.full(m, op="ela", coef=None)
    row, col = ref["row"], ref["col"]
    nnz = int(row[-1])
    a = gpu(0)
    vals = np.zeros(nnz * 9)
    e2n = np.ascontiguousarray(m.elemToNode.reshape(-1))
    for _ in range(2):   # second call reuses the cached pattern
        minifem.assembly(m.coord, vals, row, col, e2n, None, m.nbElem, nnz, 9, 1, ctx=a)
        assert vals.tobytes() == ref["values"].tobytes()
        prec = np.zeros(m.nbNodes * 9)
        minifem.prec_init(prec, vals, row, col, m.nbNodes, 9, ctx=a)
        minifem.prec_inversion(prec, row, col, ref["checkBounds"], m.nbNodes, 1, ctx=a)
        assert prec.tobytes() == ref["prec"].tobytes()


def test_errors_are_reported_not_faulted(gpu):
    import minifem
    m = cube_mesh(4, seed=1)
    a = gpu(0)
    with pytest.raises(minifem.MfemError):          # assembly before any mesh
        a.assembly("ela")
    bad = m.elemToNode.copy()
    bad[0, 0] = m.nbNodes + 5
    with pytest.raises(minifem.MfemError):          # node index out of range
        a.set_mesh(m.coord, bad)
    a.set_mesh(m.coord, m.elemToNode)
    with pytest.raises(minifem.MfemError):          # pattern missing
        a.assembly("ela")
    row, col = a.create_nodeToNode()
    # a pattern that misses an element pair is rejected
    r2, c2 = row.copy(), col.copy()
    c2[1] = c2[0]
    with pytest.raises(minifem.MfemError):
        a.set_pattern(r2, c2)
    with pytest.raises(minifem.MfemError):          # scatter without colouring
        b = gpu(0)
        b.set_mesh(m.coord, m.elemToNode)
        b.create_nodeToNode()
        b.assembly("ela", "fp64", "scatter")


def test_isolated_node_and_singular_block(gpu):
    """A node no element touches: prec_init leaves zeros, the lap inverse is inf
    and the ela block (no diagonal entry) is left as masked (elasclpr.f:29-32)."""
    m = cube_mesh(3, seed=1, op="lap", coefficients=False)
    coord = np.vstack([m.coord, [[5.0, 5.0, 5.0]]])
    code = np.concatenate([m.boundNodesCode, [0]]).astype(np.int32)

    class M:
        pass
    M.coord, M.elemToNode, M.boundNodesCode = coord, m.elemToNode, code
    M.nbNodes, M.nbElem = coord.shape[0], m.nbElem
    for op in ("lap", "ela"):
        row, col, vals, prec = gpu_full(gpu, M, op, None, "reference")
        ref = O.full(M, op=op, coef=None)
        assert vals.tobytes() == ref["values"].tobytes()
        assert prec.tobytes() == ref["prec"].tobytes()
        # the FP32 tile path: the isolated node is an empty row of the device
        # tile plan; values within the FP32 tolerance, the preconditioner
        # non-finite exactly where the reference's is and close elsewhere
        a = gpu(0)
        a.set_option("fp32_kernel", 1)
        a.set_mesh(M.coord, M.elemToNode)
        a.create_nodeToNode("reference")
        a.set_coefficients(op, None)
        a.set_check_bounds(O.checkbounds(M.boundNodesCode))
        a.assembly(op, "fp32", "gather", prec=True)
        v = a.values_f32().astype(np.float64)
        assert np.abs(v - ref["values"]).max() <= TOL_FP32 * np.abs(ref["values"]).max()
        p = a.prec()
        fin = np.isfinite(ref["prec"])
        assert np.array_equal(np.isfinite(p), fin)
        assert np.abs(p[fin] - ref["prec"][fin]).max() <= 1e-4 * np.abs(ref["prec"][fin]).max()


def test_empty_mesh_is_rejected(gpu):
    import minifem
    a = gpu(0)
    with pytest.raises(minifem.MfemError):
        a.set_mesh(np.zeros((4, 3)), np.zeros((0, 4), np.int32))


def test_degenerate_element_matches_the_reference(gpu):
    """Elements of zero volume (two nodes made to coincide): the reference's
    1/vol makes their gradients infinite and entries NaN or infinite; the FP64
    gather reproduces every finite entry bit for bit and NaN where the oracle
    has NaN (NaN payloads are the hardware's), and the FP32 path is non-finite
    exactly where the FP64 one is."""
    m = cube_mesh(4, seed=2, op="ela", jitter=0.0, permute=False)
    e = m.elemToNode[10] - 1
    coord = m.coord.copy()
    coord[e[3]] = coord[e[0]]

    class M:
        pass
    M.coord, M.elemToNode, M.boundNodesCode = coord, m.elemToNode, m.boundNodesCode
    M.nbNodes, M.nbElem, M.coef = coord.shape[0], m.nbElem, m.coef
    row, col, vals, prec = gpu_full(gpu, M, "ela", m.coef, "reference")
    ref = O.full(M, op="ela")
    nan = np.isnan(ref["values"])
    assert nan.any()
    assert np.array_equal(np.isnan(vals), nan)
    assert vals[~nan].tobytes() == ref["values"][~nan].tobytes()
    a = gpu(0)
    a.set_mesh(coord, m.elemToNode)
    a.create_nodeToNode("reference")
    a.set_coefficients("ela", m.coef)
    a.assembly("ela", "fp32", "gather", prec=False)
    assert np.array_equal(np.isfinite(a.values_f32()), np.isfinite(ref["values"]))
    fin = np.isfinite(ref["prec"])
    assert np.array_equal(np.isfinite(prec), fin)
    assert prec[fin].tobytes() == ref["prec"][fin].tobytes()


def test_rcm_renumbering_is_a_permutation_and_exact(gpu):
    """RCM shrinks the bandwidth of the randomly numbered cube, and assembling the
    renumbered mesh gives the permuted matrix bit for bit (same elements, same
    order, same sums)."""
    from minifem.meshgen import bandwidth, renumber_nodes
    m = cube_mesh(10, seed=6, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("sorted")
    perm = a.rcm_permutation()
    assert sorted(perm) == list(range(m.nbNodes))
    r = renumber_nodes(m, perm)
    assert bandwidth(r.elemToNode) < bandwidth(m.elemToNode) / 4
    a.set_coefficients("ela", m.coef)
    a.assembly("ela")
    v = a.values().reshape(-1, 9)
    b = gpu(0)
    b.set_mesh(r.coord, r.elemToNode)
    row2, col2 = b.create_nodeToNode("sorted")
    b.set_coefficients("ela", m.coef)
    b.assembly("ela")
    v2 = b.values().reshape(-1, 9)
    rr = np.repeat(np.arange(m.nbNodes), np.diff(row))
    key_old = perm[rr].astype(np.int64) * m.nbNodes + perm[col - 1]
    rr2 = np.repeat(np.arange(m.nbNodes), np.diff(row2))
    key_new = rr2.astype(np.int64) * m.nbNodes + (col2 - 1)
    o1, o2 = np.argsort(key_old), np.argsort(key_new)
    assert np.array_equal(key_old[o1], key_new[o2])
    assert v[o1].tobytes() == v2[o2].tobytes()


@pytest.mark.parametrize("kind", ["morton", "bisection"])
def test_locality_renumbering_is_a_permutation_and_exact(gpu, kind):
    """Morton and recursive-bisection orderings: permutations that shrink the mean
    index spread of the elements of the randomly numbered cube (space-filling
    orders keep a few long jumps, so not the maximum bandwidth); the renumbered
    mesh assembles to the permuted matrix bit for bit."""
    from minifem.meshgen import renumber_nodes
    m = cube_mesh(10, seed=6, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("sorted")
    perm = a.locality_permutation(kind)
    assert sorted(perm) == list(range(m.nbNodes))
    r = renumber_nodes(m, perm)

    def spread(e2n):
        return float(np.mean(e2n.max(axis=1) - e2n.min(axis=1)))
    assert spread(r.elemToNode) < spread(m.elemToNode) / 4
    a.set_coefficients("ela", m.coef)
    a.assembly("ela")
    v = a.values().reshape(-1, 9)
    b = gpu(0)
    b.set_mesh(r.coord, r.elemToNode)
    row2, col2 = b.create_nodeToNode("sorted")
    b.set_coefficients("ela", m.coef)
    b.assembly("ela")
    v2 = b.values().reshape(-1, 9)
    rr = np.repeat(np.arange(m.nbNodes), np.diff(row))
    key_old = perm[rr].astype(np.int64) * m.nbNodes + perm[col - 1]
    rr2 = np.repeat(np.arange(m.nbNodes), np.diff(row2))
    key_new = rr2.astype(np.int64) * m.nbNodes + (col2 - 1)
    o1, o2 = np.argsort(key_old), np.argsort(key_new)
    assert np.array_equal(key_old[o1], key_new[o2])
    assert v[o1].tobytes() == v2[o2].tobytes()


def test_renumbering_tuner(gpu):
    from minifem import autotune
    m = cube_mesh(12, seed=8, op="ela")
    r = autotune.tune_renumbering(m, "ela", "fp32", repeats=2)
    assert r["choice"] in autotune.RENUMBERINGS
    assert [t[0] for t in r["timings"]] == list(autotune.RENUMBERINGS)
    if r["choice"] != "identity":
        assert sorted(r["newOfOld"]) == list(range(m.nbNodes))


def test_autotuner_picks_a_valid_variant(gpu, tmp_path):
    from minifem import autotune
    m = cube_mesh(12, seed=3, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_coefficients("ela", m.coef)
    cache = str(tmp_path / "tune.json")
    r = autotune.tune(a, "ela", "fp32", repeats=2, cache=cache)
    assert r["choice"]["strategy"] == "gather" and len(r["timings"]) >= 2
    r2 = autotune.tune(a, "ela", "fp32", cache=cache)      # cached: no timing
    assert r2["choice"] == r["choice"]
    f = autotune.tune(a, "ela", "fp64", repeats=2)
    assert f["choice"]["strategy"] in ("gather", "atomic", "scatter")


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_equals_single_mesh_entry_points(gpu, precision):
    """Meshes of uneven size, lap and ela, several coefficient sets each: every
    (mesh, set) of one batched iteration equals the single-mesh entry point bit
    for bit (same plans, same arithmetic)."""
    import minifem
    specs = [(5, "lap", 2), (9, "ela", 3), (7, "ela", 1), (11, "lap", 2)]
    b = minifem.Batch(0)
    asms, sets = [], []
    for n, op, k in specs:
        meshes = [cube_mesh(n, seed=100 * n + s, op=op) for s in range(k)]
        m = meshes[0]
        a = gpu(0)
        a.set_mesh(m.coord, m.elemToNode)
        a.create_nodeToNode("sorted")
        a.set_check_bounds(O.checkbounds(m.boundNodesCode))
        cs = np.stack([mm.coef for mm in meshes])
        b.add(a, op, cs)
        asms.append((a, op))
        sets.append(cs)
    info = b.info()
    assert info["items"] == len(specs)
    for it in range(2):                      # graph replays
        b.assemble(precision, prec=True)
        b.synchronize()
    for i, ((a, op), cs) in enumerate(zip(asms, sets)):
        for s in range(cs.shape[0]):
            a.set_coefficients(op, cs[s])
            a.assembly(op, precision, "gather", prec=True)
            ref_v = a.values_f32() if precision == "fp32" else a.values()
            got = b.values(i, s, precision)
            assert got.tobytes() == ref_v.tobytes(), (i, s)
            assert b.prec(i, s).tobytes() == a.prec().tobytes(), (i, s)


def test_bounded_wait_reports_timeout_and_context_stays_usable(gpu):
    """The tile kernel's wait for its staged copies is bounded: when the barrier
    expects bytes that never arrive (a testing option), the wait gives up after
    `wait_limit` polls, the next read reports MFEM_ERR_TIMEOUT, and the context
    assembles correctly afterwards.  No fault, no trap, no hang."""
    import minifem
    m = cube_mesh(4, seed=2, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("reference")
    a.set_coefficients("ela", m.coef)
    a.set_option("wait_limit", 200)
    a.set_option("test_missing_bytes", 16)
    a.assembly("ela", "fp32", "gather", prec=True)
    with pytest.raises(minifem.MfemError) as ei:
        a.values_f32()
    assert ei.value.code == -8
    a.set_option("test_missing_bytes", 0)
    a.set_option("wait_limit", 1 << 22)
    a.assembly("ela", "fp32", "gather", prec=True)
    v = a.values_f32().astype(np.float64)
    ref = O.full(m, op="ela")
    assert np.abs(v - ref["values"]).max() / np.abs(ref["values"]).max() < 1e-6
