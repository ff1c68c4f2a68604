"""Oracle (test infrastructure only): ctypes access to the CPU restatement
(`_build/liboracle.so`, from oracle.c) and, where it was built, to the
reference's own operators (`_ref/libminifem_ref.so`, `_ref/libminifem_coloring.so`).

Only tests, the smoke check and the benchmark's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build_port() -> str:
    """Compile oracle.c (make port).  Cheap; safe on any host."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def ref_root() -> str:
    """Root of the reference tree: $MINIFEM_REF_ROOT, else the default that the
    oracle's Makefile names (REF_ROOT), the one place where it is written."""
    env = os.environ.get("MINIFEM_REF_ROOT")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref-root"], capture_output=True,
                       text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def ref_available() -> bool:
    """True where the reference sources exist (never on a host without them)."""
    root = ref_root()
    return bool(root) and os.path.isdir(os.path.join(root, "src"))


def build_ref(root: str | None = None) -> bool:
    """Compile the reference operators where the reference tree exists."""
    root = root or ref_root()
    if not root or not os.path.isdir(os.path.join(root, "src")):
        return False
    r = subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={root}", "-j4"],
                       capture_output=True, text=True)
    return r.returncode == 0


_port = None


def port() -> C.CDLL:
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build_port()
        lib = C.CDLL(PORT_SO)
        lib.orc_node_to_elem.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p]
        lib.orc_create_nodeToNode.argtypes = [_i32p, _i32p, _i32p, _i32p, _i32p, C.c_int]
        lib.orc_create_elemToEdge.argtypes = [_i32p, _i32p, _i32p, _i32p, C.c_int]
        lib.orc_assembly.argtypes = [_f64p, _f64p, _i32p, _i32p, _i32p, C.c_int, C.c_int,
                                     C.c_int, C.c_int, C.c_void_p]
        lib.orc_assembly_positions.argtypes = [_f64p, _f64p, _i32p, _i32p, C.c_int,
                                               C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.orc_assembly_ordered.argtypes = [_f64p, _f64p, _i32p, _i32p, _i32p, _i32p,
                                             C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.orc_prec_init.argtypes = [_f64p, _f64p, _i32p, _i32p, C.c_int, C.c_int]
        lib.orc_prec_inversion.argtypes = [_f64p, _i32p, _i32p, _i32p, C.c_int, C.c_int]
        lib.orc_prec_inversion.restype = C.c_int
        lib.orc_threads.argtypes = []
        lib.orc_threads.restype = C.c_int
        lib.orc_set_threads.argtypes = [C.c_int]
        lib.orc_set_threads.restype = None
        lib.orc_halo_pack.argtypes = [_f64p, _i32p, _i32p, C.c_int, C.c_int, _f64p]
        lib.orc_halo_pack.restype = None
        lib.orc_halo_add.argtypes = [_f64p, _i32p, _i32p, C.c_int, C.c_int, _f64p]
        lib.orc_halo_add.restype = None
        lib.orc_dqmrd4.argtypes = [C.c_int, _i32p, C.POINTER(C.c_int), _i32p,
                                   C.POINTER(C.c_int)]
        lib.orc_e_essbcm.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _i32p, _i32p]
        lib.orc_coloring.argtypes = [_i32p, C.c_int, C.c_int, _i32p, _i32p]
        lib.orc_coloring.restype = C.c_int
        lib.orc_norm.argtypes = [_f64p, C.c_long]
        lib.orc_norm.restype = C.c_double
        lib.orc_getrf_getri3.argtypes = [_f64p]
        lib.orc_getrf_getri3.restype = C.c_int
        _port = lib
    return _port


def threads() -> int:
    """Threads of the port's OpenMP loops (matrix reset, prec_init, prec_inversion)."""
    return int(port().orc_threads())


def set_threads(n: int) -> None:
    """1: the reference's REF build (every loop serial); the host's cores: its
    OMP/COLORING builds (reset and preconditioner loops in parallel)."""
    port().orc_set_threads(int(n))


def _coef_ptr(coef):
    if coef is None:
        return None
    return np.ascontiguousarray(coef, dtype=np.float64).ctypes.data_as(C.c_void_p)


def op_dim(op: str) -> int:
    return 1 if op == "lap" else 9


def op_id(op: str) -> int:
    return 0 if op == "lap" else 1


def pattern(e2n: np.ndarray, nbNodes: int):
    """(row, col) as src/main.cc:243-250 builds them (first-occurrence columns)."""
    lib = port()
    e2n = np.ascontiguousarray(e2n, dtype=np.int32)
    E = e2n.shape[0]
    idx = np.zeros(nbNodes + 1, np.int32)
    val = np.zeros(4 * E, np.int32)
    lib.orc_node_to_elem(nbNodes, E, e2n, idx, val)
    # an upper bound on the row lengths: 4 * (elements per node)
    cap = int(np.minimum(np.diff(idx) * 4, nbNodes).sum())
    row = np.zeros(nbNodes + 1, np.int32)
    col = np.zeros(max(cap, 1), np.int32)
    lib.orc_create_nodeToNode(row, col, idx, val, e2n, nbNodes)
    return row, col[: row[-1]].copy()


def node_to_elem(e2n, nbNodes):
    """(index, value) as DC_create_nodeToElem lists them: ascending element id
    per node, 0-based element ids (src/main.cc:243-247)."""
    e2n = np.ascontiguousarray(e2n, dtype=np.int32)
    idx = np.zeros(nbNodes + 1, np.int32)
    val = np.zeros(4 * e2n.shape[0], np.int32)
    port().orc_node_to_elem(nbNodes, e2n.shape[0], e2n, idx, val)
    return idx, val


def pattern_from_incidence(idx, val, e2n, nbNodes):
    """create_nodeToNode (src/matrix.cc:55-91) over the given node -> element
    lists, in their order."""
    lib = port()
    e2n = np.ascontiguousarray(e2n, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.int32)
    cap = int(np.minimum(np.diff(idx) * 4, nbNodes).sum())
    row = np.zeros(nbNodes + 1, np.int32)
    col = np.zeros(max(cap, 1), np.int32)
    lib.orc_create_nodeToNode(row, col, idx, val, e2n, nbNodes)
    return row, col[: row[-1]].copy()


def elem_to_edge(row, col, e2n):
    lib = port()
    e2n = np.ascontiguousarray(e2n, dtype=np.int32)
    out = np.zeros(e2n.shape[0] * 16, np.int32)
    lib.orc_create_elemToEdge(row, col, e2n, out, e2n.shape[0])
    return out


def checkbounds(code: np.ndarray) -> np.ndarray:
    """Dirichlet mask as src/main.cc:340-346 builds it (dqmrd4_ + e_essbcm_)."""
    lib = port()
    code = np.ascontiguousarray(code, dtype=np.int32)
    N = code.shape[0]
    nnd = C.c_int(int(np.count_nonzero(code)))
    ier = C.c_int(0)
    nlim = np.zeros(max(nnd.value, 1), np.int32)
    lib.orc_dqmrd4(N, code, C.byref(nnd), nlim, C.byref(ier))
    if ier.value != 0:
        raise RuntimeError("dqmrd4: boundary list overflow")
    markf = np.zeros(3 * N, np.int32)
    lib.orc_e_essbcm(3, N, nnd.value, nlim, code, markf)
    return markf


def assembly(coord, row, col, e2n, nbEdges, op, coef=None):
    lib = port()
    d = op_dim(op)
    vals = np.zeros(nbEdges * d, np.float64)
    lib.orc_assembly(np.ascontiguousarray(coord, np.float64).reshape(-1), vals, row, col,
                     np.ascontiguousarray(e2n, np.int32).reshape(-1), e2n.shape[0],
                     nbEdges, d, op_id(op), _coef_ptr(coef))
    return vals


def assembly_ordered(coord, row, col, e2n, order, nbEdges, op, coef=None):
    lib = port()
    d = op_dim(op)
    vals = np.zeros(nbEdges * d, np.float64)
    lib.orc_assembly_ordered(np.ascontiguousarray(coord, np.float64).reshape(-1), vals,
                             row, col, np.ascontiguousarray(e2n, np.int32).reshape(-1),
                             np.ascontiguousarray(order, np.int32), e2n.shape[0], nbEdges,
                             d, op_id(op), _coef_ptr(coef))
    return vals


def prec(values, row, col, markf, nbNodes, op):
    lib = port()
    d = op_dim(op)
    p = np.zeros(nbNodes * d, np.float64)
    lib.orc_prec_init(p, values, row, col, nbNodes, d)
    nbad = lib.orc_prec_inversion(p, row, col, markf, nbNodes, op_id(op))
    return p, nbad


def prec_blocks(values, row, col, nbNodes, op):
    """prec_init alone (src/preconditioner.cc:52-87): the diagonal blocks."""
    d = op_dim(op)
    p = np.zeros(nbNodes * d, np.float64)
    port().orc_prec_init(p, values, row, col, nbNodes, d)
    return p


def prec_invert(p, row, col, markf, nbNodes, op):
    """prec_inversion alone (src/preconditioner.cc:25-49), in place; returns the
    number of singular blocks."""
    return port().orc_prec_inversion(p, row, col, np.ascontiguousarray(markf, np.int32), nbNodes,
                                     op_id(op))


def halo_pack(p, intfIndex, intfNodes, op):
    """The send buffer of MPI_halo_exchange (src/halo.cc:66-77)."""
    d = op_dim(op)
    intfIndex = np.ascontiguousarray(intfIndex, np.int32)
    intfNodes = np.ascontiguousarray(intfNodes, np.int32)
    nb = len(intfIndex) - 1
    send = np.zeros(max(int(intfIndex[-1]) * d, 1) if nb > 0 else 1, np.float64)
    if nb > 0:
        port().orc_halo_pack(p, intfIndex, intfNodes, nb, d, send)
    return send[: int(intfIndex[-1]) * d] if nb > 0 else send[:0]


def halo_add(p, intfIndex, intfNodes, recv, op):
    """The additions of MPI_halo_exchange (src/halo.cc:96-112), in place."""
    intfIndex = np.ascontiguousarray(intfIndex, np.int32)
    nb = len(intfIndex) - 1
    if nb > 0:
        port().orc_halo_add(p, intfIndex, np.ascontiguousarray(intfNodes, np.int32), nb, op_dim(op),
                            np.ascontiguousarray(recv, np.float64))


def getrf_getri3(a_colmajor: np.ndarray):
    a = np.ascontiguousarray(a_colmajor, dtype=np.float64).copy()
    info = port().orc_getrf_getri3(a)
    return a, info


def coloring(e2n, nbNodes):
    lib = port()
    e2n = np.ascontiguousarray(e2n, dtype=np.int32)
    part = np.zeros(e2n.shape[0], np.int32)
    index = np.zeros(130, np.int32)
    nc = lib.orc_coloring(e2n, e2n.shape[0], nbNodes, part, index)
    if nc < 0:
        raise RuntimeError("Not enough colors")
    return part, index[: nc + 1].copy()


def norm(x) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    return port().orc_norm(x, x.size)


def full(mesh, op=None, coef="mesh"):
    """Run the whole path on the CPU: pattern, assembly, prec.  Returns a dict."""
    op = op or mesh.op
    c = mesh.coef if isinstance(coef, str) else coef
    row, col = pattern(mesh.elemToNode, mesh.nbNodes)
    vals = assembly(mesh.coord, row, col, mesh.elemToNode, int(row[-1]), op, c)
    markf = checkbounds(mesh.boundNodesCode)
    p, nbad = prec(vals, row, col, markf, mesh.nbNodes, op)
    return {"row": row, "col": col, "values": vals, "prec": p, "checkBounds": markf,
            "singular_blocks": nbad}


# ---------------------------------------------------------------- reference build

class Ref:
    """The reference's own operators (REF or COLORING build), when compiled."""

    def __init__(self, flavour: str = "ref"):
        so = os.path.join(REF_DIR, f"libminifem_{flavour}.so")
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        lib = C.CDLL(so)
        lib.ref_create_pattern.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p]
        lib.ref_create_pattern.restype = C.c_int
        lib.ref_create_elemToEdge.argtypes = [_i32p, _i32p, _i32p, _i32p, C.c_int]
        lib.ref_assembly.argtypes = [_f64p, _f64p, _i32p, _i32p, _i32p, C.c_int, C.c_int,
                                     C.c_int, C.c_int]
        lib.ref_prec_init.argtypes = [_f64p, _f64p, _i32p, _i32p, C.c_int, C.c_int]
        lib.ref_prec_inversion.argtypes = [_f64p, _i32p, _i32p, _i32p, C.c_int, C.c_int]
        lib.ref_coloring.argtypes = [_i32p, C.c_int, C.c_int, _i32p, _i32p]
        lib.ref_coloring.restype = C.c_int
        self.lib = lib

    @staticmethod
    def available(flavour: str = "ref") -> bool:
        return os.path.exists(os.path.join(REF_DIR, f"libminifem_{flavour}.so"))

    def pattern(self, e2n, nbNodes, nbEdges):
        e2n = np.ascontiguousarray(e2n, np.int32).reshape(-1).copy()
        row = np.zeros(nbNodes + 1, np.int32)
        col = np.zeros(nbEdges, np.int32)
        nnz = self.lib.ref_create_pattern(nbNodes, e2n.size // 4, e2n, row, col)
        if nnz != nbEdges:
            raise RuntimeError(f"nnz {nnz} != nbEdges {nbEdges}")
        return row, col

    def elem_to_edge(self, row, col, e2n):
        e2n = np.ascontiguousarray(e2n, np.int32).reshape(-1).copy()
        out = np.zeros(e2n.size * 4, np.int32)
        self.lib.ref_create_elemToEdge(row, col, e2n, out, e2n.size // 4)
        return out

    def assembly(self, coord, row, col, e2n, nbEdges, op):
        d = op_dim(op)
        vals = np.zeros(nbEdges * d, np.float64)
        e2n = np.ascontiguousarray(e2n, np.int32).reshape(-1).copy()
        self.lib.ref_assembly(np.ascontiguousarray(coord, np.float64).reshape(-1).copy(),
                              vals, row, col, e2n, e2n.size // 4, nbEdges, d, op_id(op))
        return vals

    def prec(self, values, row, col, markf, nbNodes, op):
        d = op_dim(op)
        p = np.zeros(nbNodes * d, np.float64)
        self.lib.ref_prec_init(p, values, row, col, nbNodes, d)
        self.lib.ref_prec_inversion(p, row, col, np.ascontiguousarray(markf, np.int32),
                                    nbNodes, op_id(op))
        return p

    def coloring(self, e2n, nbNodes):
        """Returns (permuted elemToNode, colorPerm, colorIndex)."""
        e2n = np.ascontiguousarray(e2n, np.int32).reshape(-1).copy()
        E = e2n.size // 4
        perm = np.zeros(E, np.int32)
        index = np.zeros(130, np.int32)
        nc = self.lib.ref_coloring(e2n, E, nbNodes, perm, index)
        return e2n.reshape(E, 4), perm, index[: nc + 1].copy()
