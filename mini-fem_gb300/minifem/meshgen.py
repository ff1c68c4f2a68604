"""Synthetic P1 tetrahedral meshes in Mini-FEM's input format.

The reference reads its meshes (LM6, EIB) from binary files written by the
DefMesh tool (src/IO.cc:61-96 reads them, src/IO.cc:99-127 ``store_input_data_``
writes them).  Neither the meshes nor DefMesh ship with the reference, so this
module generates stand-ins of the same sizes:

* an n x n x n node grid on the unit cube, h = 1/(n-1), every hexahedron split
  into the 6 Kuhn tetrahedra around its main diagonal (one consistent diagonal
  direction, so the mesh is conforming): E = 6 (n-1)^3 elements;
* node coordinates jittered uniformly by +-jitter*h per axis, except along the
  normal of a boundary face (boundary nodes stay on their face);
* optionally a random permutation of the node numbering;
* boundary codes (src/Fortran/DefMesh_jlog.h): x=0 -> 52, y=0 -> 53, z=0 -> 54
  (symmetry planes: one constrained DOF), the other three faces -> 10 (all DOFs
  constrained), interior -> 0, so both branches of src/Fortran/elasclpr.f:19-27
  are exercised;
* per-element coefficients: kappa ~ U[0.5, 2] (lap) or Young's modulus E
  log-uniform in [1e9, 2e11] and Poisson ratio nu ~ U[0.2, 0.35] (ela);
* a stress variant: a fraction of tetrahedra flattened toward slivers (aspect up
  to 1e4) and a 1e6 jump of E across a random half-space.

Random numbers come from a counter-based splitmix64 stream, so every array is a
pure function of (n, seed, options) on any machine.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

# Kuhn split: path 000 -> e_a -> e_a + e_b -> 111 for each axis order (a, b, c)
_KUHN = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))

JL_OUT, JL_SYMX, JL_SYMY, JL_SYMZ = 10, 52, 53, 54


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        z += _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def rng_u64(seed: int, stream: int, count: int) -> np.ndarray:
    """count 64-bit draws of stream `stream` under `seed` (splitmix64 counters)."""
    base = _mix(np.array([(seed * 0x100000001B3 + stream * 0x9E37) & 0xFFFFFFFFFFFFFFFF],
                         dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        ctr = base + np.arange(count, dtype=np.uint64) * _GOLDEN
    return _mix(ctr)


def rng_uniform(seed: int, stream: int, count: int) -> np.ndarray:
    """count doubles uniform in [0, 1)."""
    return (rng_u64(seed, stream, count) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def cube_sizes(n: int) -> tuple[int, int, int]:
    """(nbElem, nbNodes, nnz) of the Kuhn cube with n nodes per side."""
    m = n - 1
    nodes = n ** 3
    edges = 3 * n * n * m + 3 * n * m * m + m ** 3
    return 6 * m ** 3, nodes, nodes + 2 * edges


@dataclass
class Mesh:
    """A mesh in the reference's conventions (1-based elemToNode)."""
    coord: np.ndarray            # float64 [N, 3]
    elemToNode: np.ndarray       # int32   [E, 4], 1-based
    boundNodesCode: np.ndarray   # int32   [N]
    nbEdges: int                 # CSR entries including the diagonal
    coef: np.ndarray | None = None   # float64 [E] (kappa) or [E, 2] (E, nu)
    op: str = "ela"
    meta: dict = field(default_factory=dict)

    @property
    def nbElem(self) -> int:
        return int(self.elemToNode.shape[0])

    @property
    def nbNodes(self) -> int:
        return int(self.coord.shape[0])

    @property
    def nbBoundNodes(self) -> int:
        return int(np.count_nonzero(self.boundNodesCode))


def _grid_nodes(n: int):
    i = np.arange(n ** 3, dtype=np.int64)
    return i % n, (i // n) % n, i // (n * n)


def cube_mesh(n: int, seed: int = 0, *, op: str = "ela", jitter: float = 0.2,
              permute: bool = True, coefficients: bool = True,
              sliver_fraction: float = 0.0, sliver_max_aspect: float = 1e4,
              jump: float = 1.0, nu_max: float = 0.35) -> Mesh:
    """Jittered, optionally node-permuted Kuhn cube with n nodes per side."""
    if n < 2:
        raise ValueError("n must be >= 2")
    h = 1.0 / (n - 1)
    N = n ** 3
    gi, gj, gk = _grid_nodes(n)
    g = np.stack([gi, gj, gk], axis=1)
    coord = g.astype(np.float64) * h
    u = rng_uniform(seed, 1, 3 * N).reshape(N, 3)
    d = (2.0 * u - 1.0) * (jitter * h)
    d[(g == 0) | (g == n - 1)] = 0.0
    coord += d

    # elements: hex (i, j, k) -> 6 tets, element id = 6 * hex + t
    m = n - 1
    hx = np.arange(m ** 3, dtype=np.int64)
    hi, hj, hk = hx % m, (hx // m) % m, hx // (m * m)
    base = hi + n * hj + n * n * hk
    step = np.array([1, n, n * n], dtype=np.int64)
    e2n = np.empty((m ** 3, 6, 4), dtype=np.int64)
    for t, (a, b, _) in enumerate(_KUHN):
        e2n[:, t, 0] = base
        e2n[:, t, 1] = base + step[a]
        e2n[:, t, 2] = base + step[a] + step[b]
        e2n[:, t, 3] = base + step.sum()
    e2n = e2n.reshape(-1, 4)
    E = e2n.shape[0]

    code = np.zeros(N, dtype=np.int32)
    code[gk == 0] = JL_SYMZ
    code[gj == 0] = JL_SYMY
    code[gi == 0] = JL_SYMX
    code[(gi == n - 1) | (gj == n - 1) | (gk == n - 1)] = JL_OUT

    meta = {"n": n, "seed": seed, "jitter": jitter, "permute": permute, "h": h}
    if sliver_fraction > 0.0:
        meta["slivers_made"] = _make_slivers(coord, e2n, g, n, seed, sliver_fraction,
                                             sliver_max_aspect)

    coef = None
    if coefficients:
        if op == "lap":
            coef = 0.5 + 1.5 * rng_uniform(seed, 3, E)
        else:
            ue = rng_uniform(seed, 4, E)
            un = rng_uniform(seed, 5, E)
            young = np.exp(np.log(1e9) + ue * (np.log(2e11) - np.log(1e9)))
            nu = 0.2 + un * (nu_max - 0.2)
            if jump != 1.0:
                cen = coord[e2n].mean(axis=1)
                w = rng_uniform(seed, 6, 6)
                normal = w[:3] - 0.5
                normal /= np.linalg.norm(normal)
                point = 0.25 + 0.5 * w[3:]
                young = np.where((cen - point) @ normal > 0.0, young * jump, young)
            coef = np.stack([young, nu], axis=1)

    if permute:
        keys = rng_u64(seed, 2, N)
        order = np.argsort(keys, kind="stable")
        new_of_old = np.empty(N, dtype=np.int64)
        new_of_old[order] = np.arange(N, dtype=np.int64)
        coord = coord[order]
        code = code[order]
        e2n = new_of_old[e2n]

    _, _, nnz = cube_sizes(n)
    return Mesh(coord=np.ascontiguousarray(coord),
                elemToNode=np.ascontiguousarray((e2n + 1).astype(np.int32)),
                boundNodesCode=code, nbEdges=nnz, coef=coef, op=op, meta=meta)


def _make_slivers(coord, e2n, g, n, seed, fraction, max_aspect):
    """Flatten about `fraction` of the tets: for each chosen tet whose nodes are
    all interior and untouched so far, move its first node toward the plane of
    the opposite face so that its height shrinks by a factor 10^-U(0, log10
    max_aspect).  Returns the number of tets flattened."""
    E = e2n.shape[0]
    want = int(round(fraction * E))
    if want <= 0:
        return 0
    pick = np.argsort(rng_u64(seed, 7, E), kind="stable")
    shrink = 10.0 ** (-rng_uniform(seed, 8, E) * np.log10(max_aspect))
    interior = np.all((g > 0) & (g < n - 1), axis=1)
    moved = np.zeros(coord.shape[0], dtype=bool)
    made = 0
    for e in pick:
        if made >= want:
            break
        nodes = e2n[e]
        if not interior[nodes].all() or moved[nodes].any():
            continue
        p = coord[nodes[0]]
        a, b, c = coord[nodes[1]], coord[nodes[2]], coord[nodes[3]]
        nrm = np.cross(b - a, c - a)
        nn = np.linalg.norm(nrm)
        if nn == 0.0:
            continue
        nrm /= nn
        dist = np.dot(p - a, nrm)
        coord[nodes[0]] = p - (1.0 - shrink[e]) * dist * nrm
        moved[nodes] = True
        made += 1
    return made


def _icosphere(subdivisions: int):
    """Unit icosphere: vertices [V, 3] and outward-oriented triangles [F, 3]
    (each subdivision splits a triangle into four at its edge midpoints)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
         (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9),
             (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2),
             (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]
        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int64)


def fan_mesh(subdivisions: int, seed: int = 0, *, op: str = "ela",
             permute: bool = True) -> Mesh:
    """A ball of tetrahedra that all share its centre node: one tetrahedron per
    triangle of an icosphere (20 * 4**subdivisions of them), so the centre's CSR
    row holds every node of the mesh.  A worst case for row lengths and for
    elements per node (1280 at 3 subdivisions), where the cube has at most 24.
    Surface nodes in the lower half (z < 0) are fixed in all directions."""
    sv, tri = _icosphere(subdivisions)
    N = len(sv) + 1
    coord = np.vstack([np.zeros((1, 3)), sv])
    e2n = np.concatenate([np.zeros((len(tri), 1), np.int64), tri + 1], axis=1)
    code = np.zeros(N, dtype=np.int32)
    code[1:][sv[:, 2] < 0.0] = JL_OUT
    if permute:
        keys = rng_u64(seed, 2, N)
        order = np.argsort(keys, kind="stable")
        new_of_old = np.empty(N, dtype=np.int64)
        new_of_old[order] = np.arange(N, dtype=np.int64)
        coord, code, e2n = coord[order], code[order], new_of_old[e2n]
        e2n = e2n[np.argsort(rng_u64(seed, 7, len(e2n)), kind="stable")]
    F = len(tri)
    nnz = N + 2 * (3 * F // 2 + (N - 1))      # diagonal + both directions of every edge
    return Mesh(coord=np.ascontiguousarray(coord),
                elemToNode=np.ascontiguousarray((e2n + 1).astype(np.int32)),
                boundNodesCode=code, nbEdges=nnz,
                coef=coefficient_set(op, F, seed), op=op,
                meta={"subdivisions": subdivisions, "seed": seed, "centre_elements": F})


def coefficient_set(op: str, nbElem: int, seed: int, nu_max: float = 0.35) -> np.ndarray:
    """One more per-element coefficient set with the generator's distributions:
    kappa ~ U[0.5, 2] (lap, [E]) or (E log-uniform in [1e9, 2e11], nu ~ U[0.2,
    nu_max]) (ela, [E, 2])."""
    if op == "lap":
        return 0.5 + 1.5 * rng_uniform(seed, 3, nbElem)
    ue = rng_uniform(seed, 4, nbElem)
    un = rng_uniform(seed, 5, nbElem)
    young = np.exp(np.log(1e9) + ue * (np.log(2e11) - np.log(1e9)))
    return np.stack([young, 0.2 + un * (nu_max - 0.2)], axis=1)


def renumber_nodes(mesh: Mesh, newOfOld: np.ndarray) -> Mesh:
    """The same mesh with node i renamed newOfOld[i] (elements keep their order)."""
    newOfOld = np.asarray(newOfOld, dtype=np.int64)
    coord = np.empty_like(mesh.coord)
    coord[newOfOld] = mesh.coord
    code = np.empty_like(mesh.boundNodesCode)
    code[newOfOld] = mesh.boundNodesCode
    e2n = (newOfOld[mesh.elemToNode - 1] + 1).astype(np.int32)
    return Mesh(coord=coord, elemToNode=e2n, boundNodesCode=code, nbEdges=mesh.nbEdges,
                coef=mesh.coef, op=mesh.op, meta=dict(mesh.meta, renumbered=True))


def bandwidth(elemToNode: np.ndarray) -> int:
    """max |i - j| over node pairs sharing an element."""
    e = elemToNode.astype(np.int64)
    return int((e.max(axis=1) - e.min(axis=1)).max())


def _count_nnz(e2n: np.ndarray, nbNodes: int) -> int:
    e = np.asarray(e2n, dtype=np.int64) - 1
    a = np.repeat(e, 4, axis=1).reshape(-1)
    b = np.tile(e, (1, 4)).reshape(-1)
    return int(np.unique(a * nbNodes + b).size)


@dataclass
class Domain:
    """One rank's sub-domain in the reference's per-rank input convention
    (src/IO.cc:61-96, file <op>_<nbBlocks>_<rank>): a mesh with local 1-based
    ids, and the interfaces with its neighbours -- interface i lists the local
    nodes shared with rank neighborsList[i] - 1 (src/halo.cc:53-56), in ascending
    global node order, so both sides list the same nodes in the same order."""
    mesh: Mesh
    rank: int
    nbBlocks: int
    neighborsList: np.ndarray    # int32 [max(nbIntf, 1) * 3]; first nbIntf: neighbour rank + 1
    intfIndex: np.ndarray        # int32 [nbIntf + 1]
    intfNodes: np.ndarray        # int32 [nbIntfNodes], 1-based local nodes
    globalNode: np.ndarray       # int64 [local nodes]: 0-based global node
    globalElem: np.ndarray       # int64 [local elements]: global element (ascending)

    @property
    def nbIntf(self) -> int:
        return int(self.intfIndex.size - 1)

    @property
    def neighbors(self) -> np.ndarray:
        """0-based neighbour rank of each interface."""
        return self.neighborsList[: self.nbIntf].astype(np.int64) - 1


def _bisect(cen: np.ndarray, ids: np.ndarray, parts: int, first: int, part: np.ndarray) -> None:
    """Recursive coordinate bisection: `parts` blocks numbered from `first`,
    each cut across the longest extent of the element centroids, the element
    counts split in proportion to the blocks on each side."""
    if parts == 1:
        part[ids] = first
        return
    c = cen[ids]
    axis = int(np.argmax(c.max(axis=0) - c.min(axis=0)))
    order = ids[np.argsort(c[:, axis], kind="stable")]
    left = parts // 2
    cut = (order.size * left) // parts
    _bisect(cen, order[:cut], left, first, part)
    _bisect(cen, order[cut:], parts - left, first + left, part)


def split_domains(mesh: Mesh, nbBlocks: int) -> list[Domain]:
    """Element-wise domain decomposition into nbBlocks parts of (nearly) equal
    element counts by recursive coordinate bisection of the element centroids,
    as a mesh partitioner would produce the reference's per-rank inputs (four
    or more parts meet along lines, so some nodes lie on several interfaces).
    Each rank keeps its elements in ascending global order and its nodes in
    ascending global order, so a node interior to a rank sums the same
    contributions in the same order as the undivided mesh."""
    E, N = mesh.nbElem, mesh.nbNodes
    e2n0 = np.asarray(mesh.elemToNode, np.int64) - 1
    cen = mesh.coord[e2n0].mean(axis=1)
    part = np.empty(E, np.int64)
    _bisect(cen, np.arange(E), nbBlocks, 0, part)
    # ranks touching each node (as a bit set, nbBlocks <= 63)
    if nbBlocks > 63:
        raise ValueError("at most 63 blocks")
    touch = np.zeros(N, np.uint64)
    np.bitwise_or.at(touch, e2n0.reshape(-1), (np.uint64(1) << part.astype(np.uint64)).repeat(4))
    out = []
    for p in range(nbBlocks):
        ge = np.nonzero(part == p)[0]
        gn = np.unique(e2n0[ge].reshape(-1))
        local = np.full(N, -1, np.int64)
        local[gn] = np.arange(gn.size)
        e2n = (local[e2n0[ge]] + 1).astype(np.int32)
        neigh, index, nodes = [], [0], []
        for q in range(nbBlocks):
            if q == p:
                continue
            shared = gn[(touch[gn] >> np.uint64(q)) & np.uint64(1) == 1]
            if shared.size == 0:
                continue
            neigh.append(q + 1)
            nodes.append(local[shared] + 1)
            index.append(index[-1] + shared.size)
        nbIntf = len(neigh)
        nl = np.zeros(max(nbIntf, 1) * 3, np.int32)
        nl[:nbIntf] = neigh
        sub_mesh = Mesh(coord=np.ascontiguousarray(mesh.coord[gn]), elemToNode=e2n,
                        boundNodesCode=np.ascontiguousarray(mesh.boundNodesCode[gn]),
                        nbEdges=_count_nnz(e2n, gn.size),
                        coef=None if mesh.coef is None else np.ascontiguousarray(mesh.coef[ge]),
                        op=mesh.op, meta=dict(mesh.meta, rank=p, nbBlocks=nbBlocks))
        out.append(Domain(mesh=sub_mesh, rank=p, nbBlocks=nbBlocks, neighborsList=nl,
                          intfIndex=np.asarray(index, np.int32),
                          intfNodes=(np.concatenate(nodes) if nodes else np.zeros(0, np.int64))
                          .astype(np.int32),
                          globalNode=gn, globalElem=ge))
    return out


def write_reference_input(mesh: Mesh, path: str, domain: Domain | None = None) -> None:
    """Write `mesh` in the binary layout that src/IO.cc:61-96 reads; with a
    domain, its interfaces (neighborsList, intfIndex, intfNodes), else one rank
    with no interfaces."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    if domain is None:
        nl, idx, nodes = np.zeros(3, np.int32), np.zeros(1, np.int32), np.zeros(0, np.int32)
    else:
        nl, idx, nodes = domain.neighborsList, domain.intfIndex, domain.intfNodes
    nbIntf = int(idx.size - 1)
    hdr = np.array([mesh.nbElem, mesh.nbNodes, mesh.nbEdges, nbIntf, int(nodes.size),
                    mesh.nbBoundNodes], dtype=np.int32)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(mesh.coord, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(mesh.elemToNode, dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(nl, dtype=np.int32).tobytes())      # neighborsList[max(nbIntf,1)*3]
        f.write(np.ascontiguousarray(idx, dtype=np.int32).tobytes())     # intfIndex[nbIntf+1]
        f.write(np.ascontiguousarray(nodes, dtype=np.int32).tobytes())   # intfNodes[nbIntfNodes]
        f.write(np.ascontiguousarray(mesh.boundNodesCode, dtype=np.int32).tobytes())


def read_reference_input(path: str) -> Mesh:
    """Read a file in the layout of src/IO.cc:61-96."""
    with open(path, "rb") as f:
        raw = f.read()
    hdr = np.frombuffer(raw, dtype=np.int32, count=6)
    E, N, nnz, nbIntf, nbIntfNodes, _ = (int(x) for x in hdr)
    off = 24
    need = off + N * 24 + E * 16 + max(nbIntf, 1) * 12 + (nbIntf + 1) * 4 + nbIntfNodes * 4 + N * 4
    if len(raw) < need:
        raise ValueError(f"{path}: truncated mesh file ({len(raw)} < {need} bytes)")
    coord = np.frombuffer(raw, dtype=np.float64, count=3 * N, offset=off).reshape(N, 3)
    off += 24 * N
    e2n = np.frombuffer(raw, dtype=np.int32, count=4 * E, offset=off).reshape(E, 4)
    off += 16 * E
    nl = np.frombuffer(raw, dtype=np.int32, count=max(nbIntf, 1) * 3, offset=off)
    off += max(nbIntf, 1) * 12
    idx = np.frombuffer(raw, dtype=np.int32, count=nbIntf + 1, offset=off)
    off += (nbIntf + 1) * 4
    nodes = np.frombuffer(raw, dtype=np.int32, count=nbIntfNodes, offset=off)
    off += nbIntfNodes * 4
    code = np.frombuffer(raw, dtype=np.int32, count=N, offset=off)
    return Mesh(coord=coord.copy(), elemToNode=e2n.copy(), boundNodesCode=code.copy(),
                nbEdges=nnz, meta={"neighborsList": nl.copy(), "intfIndex": idx.copy(),
                                   "intfNodes": nodes.copy()})


def write_reference_tree(mesh: Mesh, root: str, mesh_name: str, op: str,
                         matrix_norm: float | None = None,
                         prec_norm: float | None = None, domain: Domain | None = None) -> str:
    """Lay out <root>/<mesh_name>/inputs/<op>_<nbBlocks>_<rank> (and
    checkings/<op>_<nbBlocks>_<rank> when the reference norms are given), the
    tree the driver reads (src/IO.cc:29-31, :66-68); one rank (_1_0) without a
    domain.  Returns the input file path."""
    tag = f"{op}_1_0" if domain is None else f"{op}_{domain.nbBlocks}_{domain.rank}"
    path = os.path.join(root, mesh_name, "inputs", tag)
    write_reference_input(mesh, path, domain)
    if matrix_norm is not None:
        chk = os.path.join(root, mesh_name, "checkings", tag)
        os.makedirs(os.path.dirname(chk), exist_ok=True)
        with open(chk, "w") as f:
            f.write(f"{matrix_norm:.17g}\n{prec_norm:.17g}\n")
    return path
