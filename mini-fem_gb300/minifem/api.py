"""Python mirror of the reference's operator interface, on the GPU.

`Assembler` holds one device context (one mesh).  Its methods carry the names of
the reference functions they replace:

    create_nodeToNode   src/matrix.cc:55-91      (CSR pattern)
    create_elemToEdge   src/matrix.cc:25-52      (16 CSR positions per element)
    coloring_creation   src/coloring.cc:84-109   (element colouring)
    assembly            src/assembly.cc:615-720  (values, on the device)
    prec_init           src/preconditioner.cc:52-87
    prec_inversion      src/preconditioner.cc:25-49 + src/Fortran/elasclpr.f

The module-level functions `assembly`, `prec_init` and `prec_inversion` take
exactly the reference's arguments (host arrays in, host arrays out).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

_STRATEGIES = {"auto": N.AUTO, "gather": N.GATHER, "scatter": N.SCATTER, "atomic": N.ATOMIC}
_PRECISIONS = {"fp64": N.FP64, "fp32": N.FP32}
_ORDERS = {"sorted": N.ORDER_SORTED, "reference": N.ORDER_REFERENCE}


def op_id(op) -> int:
    if op in (0, 1):
        return int(op)
    if op == "lap":
        return N.OP_LAP
    if op == "ela":
        return N.OP_ELA
    raise ValueError(f"unknown operator {op!r}")


def op_dim(op) -> int:
    return 1 if op_id(op) == N.OP_LAP else 9


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Assembler:
    """Device-resident assembly of one mesh (one CUDA context on `device`)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = N.lib.mfem_create(C.byref(h), device)
        if rc != N.MFEM_OK:
            raise N.MfemError(rc, N.lib.mfem_status_string(rc).decode())
        self._h = h
        self.device = device
        self._keep = {}
        self.nbElem = self.nbNodes = self.nbEdges = 0
        self.op = None
        self.precision = None

    # -- plumbing
    def _check(self, rc: int):
        if rc != N.MFEM_OK:
            raise N.MfemError(rc, N.lib.mfem_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            N.lib.mfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        self._check(N.lib.mfem_get_stream(self._h, C.byref(s)))
        return s.value or 0

    # -- mesh and structures
    def set_mesh(self, coord, elemToNode):
        coord, e2n = _f64(coord), _i32(elemToNode)
        self._keep["coord"], self._keep["e2n"] = coord, e2n
        self.nbNodes, self.nbElem = coord.reshape(-1, 3).shape[0], e2n.reshape(-1, 4).shape[0]
        self._check(N.lib.mfem_set_mesh(self._h, _ptr(coord), _ptr(e2n), self.nbElem, self.nbNodes))

    def update_coords(self, coord):
        coord = _f64(coord)
        self._keep["coord"] = coord
        self._check(N.lib.mfem_update_coords(self._h, _ptr(coord)))

    def create_nodeToNode(self, order: str = "sorted"):
        """(row[N+1] 0-based, col[nnz] 1-based), built on the device."""
        nnz = C.c_int()
        self._check(N.lib.mfem_create_nodeToNode(self._h, _ORDERS[order], None, None, 0,
                                                 C.byref(nnz)))
        row = np.empty(self.nbNodes + 1, np.int32)
        col = np.empty(nnz.value, np.int32)
        self._check(N.lib.mfem_create_nodeToNode(self._h, _ORDERS[order], _ptr(row), _ptr(col),
                                                 col.size, C.byref(nnz)))
        self.nbEdges = nnz.value
        self._keep["row"], self._keep["col"] = row, col
        return row, col

    def set_pattern(self, row, col):
        row, col = _i32(row), _i32(col)
        self._keep["row"], self._keep["col"] = row, col
        self._check(N.lib.mfem_set_pattern(self._h, _ptr(row), _ptr(col), col.size))
        self.nbEdges = col.size

    def rcm_permutation(self):
        """newOfOld[N]: reverse Cuthill-McKee renumbering of the current pattern."""
        out = np.empty(self.nbNodes, np.int32)
        self._check(N.lib.mfem_rcm_permutation(self._h, _ptr(out)))
        return out

    def locality_permutation(self, kind: str = "bisection"):
        """newOfOld[N]: Morton ("morton") or recursive-coordinate-bisection
        ("bisection") renumbering of the nodes from their coordinates."""
        k = {"morton": N.LOCALITY_MORTON, "bisection": N.LOCALITY_BISECTION}[kind]
        out = np.empty(self.nbNodes, np.int32)
        self._check(N.lib.mfem_locality_permutation(self._h, k, _ptr(out)))
        return out

    def create_elemToEdge(self):
        out = np.empty(self.nbElem * 16, np.int32)
        self._check(N.lib.mfem_create_elemToEdge(self._h, _ptr(out)))
        return out

    def coloring_creation(self, seed: int = 0):
        """(colorPerm[E], colorIndex[nbColors+1]); colorPerm[old] = new position."""
        perm = np.empty(self.nbElem, np.int32)
        index = np.empty(129, np.int32)
        nc = C.c_int()
        self._check(N.lib.mfem_coloring_creation(self._h, seed, _ptr(perm), _ptr(index), 129,
                                                 C.byref(nc)))
        return perm, index[: nc.value + 1].copy()

    # -- assembly
    def set_coefficients(self, op, coef=None):
        c = None if coef is None else _f64(coef)
        self._keep["coef"] = c
        self._check(N.lib.mfem_set_coefficients(self._h, op_id(op), _ptr(c)))

    def set_check_bounds(self, checkBounds):
        cb = None if checkBounds is None else _i32(checkBounds)
        self._keep["cb"] = cb
        self._check(N.lib.mfem_set_check_bounds(self._h, _ptr(cb)))

    def set_sliver_threshold(self, q: float):
        self._check(N.lib.mfem_set_sliver_threshold(self._h, float(q)))

    def set_option(self, name: str, value: float):
        self._check(N.lib.mfem_set_option(self._h, name.encode(), float(value)))

    def tile_info(self) -> dict:
        t, s = C.c_int(), C.c_int()
        e, u, k = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self._check(N.lib.mfem_tile_info(self._h, C.byref(t), C.byref(e), C.byref(u), C.byref(k),
                                         C.byref(s)))
        return {"tiles": t.value, "tile_elems": e.value, "units": u.value,
                "contributions": k.value, "smem_bytes": s.value}

    def selftest_dmul(self, n: int, seed: int = 1) -> tuple[int, int]:
        """(pairs on the fast path, mismatches) of the integer-pipe double
        multiplication against the FP64 unit over n seeded operand pairs."""
        f, m = C.c_ulonglong(), C.c_ulonglong()
        self._check(N.lib.mfem_selftest_dmul(self._h, n, seed, C.byref(f), C.byref(m)))
        return f.value, m.value

    def fp64_rate(self, kind: str = "add") -> float:
        """Measured FP64 pipe rate of this context's device, operations per
        second (kind "add" or "fma")."""
        r = C.c_double()
        self._check(N.lib.mfem_fp64_rate(self._h, 0 if kind == "add" else 1, C.byref(r)))
        return r.value

    def flagged(self) -> int:
        n = C.c_int()
        self._check(N.lib.mfem_get_flagged(self._h, C.byref(n)))
        return n.value

    def assembly(self, op, precision: str = "fp64", strategy: str = "gather", prec: bool = False):
        fn = N.lib.mfem_assemble_prec if prec else N.lib.mfem_assemble
        self._check(fn(self._h, op_id(op), _PRECISIONS[precision], _STRATEGIES[strategy]))
        self.op, self.precision = op_id(op), precision

    def step_async(self, op, precision, values, prec=None, coord=None, coef=None,
                   strategy: str = "gather") -> int:
        """One pipelined FEM-loop step (mfem_step_async): host inputs in, host
        results out on a second stream, no wait.  `values` (float32 for fp32,
        float64 for fp64) and `prec` (float64 or None) must stay alive and
        untouched until wait(ticket); pinned arrays make the copies asynchronous."""
        want = np.float32 if precision == "fp32" else np.float64
        if values.dtype != want or not values.flags.c_contiguous:
            raise ValueError(f"values must be a contiguous {np.dtype(want).name} array")
        if values.size != self.nbEdges * op_dim(op):
            raise ValueError("values has the wrong size")
        if prec is not None and (prec.dtype != np.float64 or prec.size != self.nbNodes * op_dim(op)
                                 or not prec.flags.c_contiguous):
            raise ValueError("prec must be a contiguous float64 array of nbNodes*opDim")
        for a in (coord, coef):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError("coord and coef must be contiguous float64 arrays")
        t = C.c_longlong()
        self._check(N.lib.mfem_step_async(
            self._h, op_id(op), _PRECISIONS[precision], _STRATEGIES[strategy],
            None if coord is None else _ptr(coord), None if coef is None else _ptr(coef),
            _ptr(values), None if prec is None else _ptr(prec), C.byref(t)))
        self.op, self.precision = op_id(op), precision
        return t.value

    def wait(self, ticket: int):
        self._check(N.lib.mfem_wait(self._h, ticket))

    # -- consumer of the assembled system
    def spmv(self, x_dev: int, y_dev: int, constrained: bool = False):
        """y = A x on device pointers (nbNodes*opDim doubles each)."""
        self._check(N.lib.mfem_spmv(self._h, C.c_void_p(x_dev), C.c_void_p(y_dev), int(constrained)))

    def prec_apply(self, r_dev: int, z_dev: int):
        self._check(N.lib.mfem_prec_apply(self._h, C.c_void_p(r_dev), C.c_void_p(z_dev)))

    def pcg(self, b, x0=None, rtol: float = 1e-8, max_iter: int = 1000,
            constrained: bool = True):
        """Block-Jacobi preconditioned CG on the latest assembly (host arrays);
        returns (x, iterations, relative residual)."""
        b = _f64(b)
        x = np.zeros_like(b) if x0 is None else _f64(x0).copy()
        it, rel = C.c_int(), C.c_double()
        self._check(N.lib.mfem_pcg(self._h, _ptr(b), _ptr(x), rtol, max_iter, int(constrained),
                                   C.byref(it), C.byref(rel)))
        return x, it.value, rel.value

    def prec_init(self):
        self._check(N.lib.mfem_prec_init(self._h))

    def prec_inversion(self) -> int:
        n = C.c_int()
        self._check(N.lib.mfem_prec_inversion(self._h, C.byref(n)))
        return n.value

    def synchronize(self):
        self._check(N.lib.mfem_synchronize(self._h))

    # -- results
    def values(self):
        out = np.empty(self.nbEdges * op_dim(self.op), np.float64)
        self._check(N.lib.mfem_get_values(self._h, _ptr(out)))
        return out

    def values_f32(self):
        out = np.empty(self.nbEdges * op_dim(self.op), np.float32)
        self._check(N.lib.mfem_get_values_f32(self._h, _ptr(out)))
        return out

    def prec(self):
        out = np.empty(self.nbNodes * op_dim(self.op), np.float64)
        self._check(N.lib.mfem_get_prec(self._h, _ptr(out)))
        return out

    def profile(self, enable: bool = True):
        self._check(N.lib.mfem_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        """[(region name, ms)] recorded since the last read."""
        names = C.create_string_buffer(1 << 16)
        ms = (C.c_float * 4096)()
        cnt = C.c_int()
        self._check(N.lib.mfem_profile_read(self._h, names, len(names), ms, 4096, C.byref(cnt)))
        nm = names.value.decode().split(";")[: cnt.value]
        return list(zip(nm, [ms[i] for i in range(cnt.value)]))

    def device_values(self):
        p, prec = C.c_void_p(), C.c_int()
        self._check(N.lib.mfem_values_device(self._h, C.byref(p), C.byref(prec)))
        return p.value, prec.value


class Batch:
    """Several meshes (Assemblers) x coefficient sets assembled per iteration by one
    CUDA-graph replay (FP32: one persistent launch over all tiles)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = N.lib.mfem_batch_create(C.byref(h), device)
        if rc != N.MFEM_OK:
            raise N.MfemError(rc, N.lib.mfem_status_string(rc).decode())
        self._h = h
        self.items = []
        self._keep = []

    def _check(self, rc):
        if rc != N.MFEM_OK:
            raise N.MfemError(rc, N.lib.mfem_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            N.lib.mfem_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        self._check(N.lib.mfem_batch_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def add(self, asm: Assembler, op, coef_sets=None):
        """coef_sets: array [nSets, ...per-element coefficients...] or None."""
        if coef_sets is None:
            n, ptr = 1, None
        else:
            cs = _f64(coef_sets)
            n = cs.shape[0]
            self._keep.append(cs)
            ptr = _ptr(cs)
        self._check(N.lib.mfem_batch_add(self._h, asm._h, op_id(op), n, ptr))
        self.items.append((asm, op_id(op), n))
        return len(self.items) - 1

    def set_coefficients(self, item: int, coef_sets):
        cs = _f64(coef_sets)
        self._keep.append(cs)
        self._check(N.lib.mfem_batch_set_coefficients(self._h, item, _ptr(cs)))

    def assemble(self, precision: str = "fp32", prec: bool = True):
        self._check(N.lib.mfem_batch_assemble(self._h, _PRECISIONS[precision], 1 if prec else 0))

    def synchronize(self):
        self._check(N.lib.mfem_batch_synchronize(self._h))

    def values(self, item: int, set_: int, precision: str = "fp32"):
        asm, op, _ = self.items[item]
        out = np.empty(asm.nbEdges * op_dim(op), np.float32 if precision == "fp32" else np.float64)
        self._check(N.lib.mfem_batch_get_values(self._h, item, set_, _PRECISIONS[precision],
                                                _ptr(out)))
        return out

    def prec(self, item: int, set_: int):
        asm, op, _ = self.items[item]
        out = np.empty(asm.nbNodes * op_dim(op), np.float64)
        self._check(N.lib.mfem_batch_get_prec(self._h, item, set_, _ptr(out)))
        return out

    def info(self):
        ni, e, asmb, w, g = C.c_int(), C.c_longlong(), C.c_longlong(), C.c_int(), C.c_int()
        self._check(N.lib.mfem_batch_info(self._h, C.byref(ni), C.byref(e), C.byref(asmb),
                                          C.byref(w), C.byref(g)))
        return {"items": ni.value, "elements": e.value, "assemblies": asmb.value,
                "work": w.value, "grid": g.value}


# ---- reference-shaped calls on a shared default context ---------------------------

_default: Assembler | None = None


def _ctx() -> Assembler:
    global _default
    if _default is None:
        _default = Assembler(0)
    return _default


def assembly(coord, nodeToNodeValue, nodeToNodeRow, nodeToNodeColumn, elemToNode,
             elemToEdge, nbElem, nbEdges, operatorDim, operatorID, ctx: Assembler | None = None):
    """assembly() of src/headers/assembly.h:61-63: fills nodeToNodeValue in place."""
    a = ctx or _ctx()
    a._check(N.lib.mfem_assembly(a._h, _ptr(coord), _ptr(nodeToNodeValue), _ptr(nodeToNodeRow),
                                 _ptr(nodeToNodeColumn), _ptr(elemToNode),
                                 None if elemToEdge is None else _ptr(elemToEdge), nbElem,
                                 nbEdges, operatorDim, operatorID))


def prec_init(prec, nodeToNodeValue, nodeToNodeRow, nodeToNodeColumn, nbNodes, operatorDim,
              ctx: Assembler | None = None):
    """prec_init() of src/headers/preconditioner.h:31-32: fills prec in place."""
    a = ctx or _ctx()
    a._check(N.lib.mfem_prec_init_host(a._h, _ptr(prec), _ptr(nodeToNodeValue),
                                       _ptr(nodeToNodeRow), _ptr(nodeToNodeColumn), nbNodes,
                                       operatorDim))


def prec_inversion(prec, nodeToNodeRow, nodeToNodeColumn, checkBounds, nbNodes, operatorID,
                   ctx: Assembler | None = None):
    """prec_inversion() of src/headers/preconditioner.h:27-28: inverts prec in place."""
    a = ctx or _ctx()
    a._check(N.lib.mfem_prec_inversion_host(a._h, _ptr(prec), _ptr(nodeToNodeRow),
                                            _ptr(nodeToNodeColumn), _ptr(checkBounds), nbNodes,
                                            operatorID))
