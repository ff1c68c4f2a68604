"""The reference driver's call sequence (src/main.cc:209-250, 319-333; src/FEM.cc:177-234)
through the drop-in C ABI, on the GPU:

* create_nodeToNode follows the caller's node -> element lists, in the caller's
  order (src/matrix.cc:66-85), also when they are not ascending;
* the element rows permuted in place between calls (DC_permute_int_2d_array,
  src/main.cc:229) under the same pointer are seen by the next assembly call;
* the OPTIMIZED build's create_elemToEdge positions equal the oracle's.
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import cube_mesh

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _ctx():
    from minifem import _native as N
    h = C.c_void_p()
    assert N.lib.mfem_create(C.byref(h), 0) == 0
    return N, h


def _check(N, h, rc):
    assert rc == 0, N.lib.mfem_last_error(h).decode()


@pytest.mark.parametrize("shuffle", [False, True])
def test_create_nodeToNode_follows_caller_incidence(shuffle):
    m = cube_mesh(9, seed=5, op="ela", coefficients=False)
    N_, E = m.nbNodes, m.nbElem
    e2n = np.ascontiguousarray(m.elemToNode, np.int32)
    idx, val = O.node_to_elem(e2n, N_)
    if shuffle:
        rng = np.random.default_rng(7)
        for i in range(N_):
            seg = val[idx[i]:idx[i + 1]]
            val[idx[i]:idx[i + 1]] = seg[rng.permutation(seg.size)]
    row_ref, col_ref = O.pattern_from_incidence(idx, val, e2n, N_)
    N, h = _ctx()
    try:
        _check(N, h, N.lib.mfem_set_mesh(h, None, _p(e2n), E, N_))
        row = np.zeros(N_ + 1, np.int32)
        col = np.zeros(col_ref.size, np.int32)
        nnz = C.c_int()
        _check(N, h, N.lib.mfem_create_nodeToNode_incidence(h, _p(idx), _p(val), _p(row), _p(col),
                                                             col.size, C.byref(nnz)))
        assert nnz.value == col_ref.size
        assert np.array_equal(row, row_ref) and np.array_equal(col, col_ref)
        # an element id outside the mesh is refused
        bad = val.copy()
        bad[3] = E
        rc = N.lib.mfem_create_nodeToNode_incidence(h, _p(idx), _p(bad), _p(row), _p(col),
                                                    col.size, C.byref(nnz))
        assert rc == -1 and "nodeToElem" in N.lib.mfem_last_error(h).decode()
    finally:
        N.lib.mfem_destroy(h)


@pytest.mark.parametrize("op", ["lap", "ela"])
def test_in_place_permutation_between_assembly_calls(op):
    """src/main.cc order: coloring_creation, the element rows permuted in place,
    create_nodeToNode, then the FEM loop; here the rows are permuted in place once
    more between two assembly calls with the same arrays: the second call must
    assemble the permuted mesh (bit-exact against the oracle in its new order)."""
    m = cube_mesh(8, seed=11, op=op, coefficients=False)
    N_, E = m.nbNodes, m.nbElem
    d = O.op_dim(op)
    coord = np.ascontiguousarray(m.coord, np.float64)
    e2n = np.ascontiguousarray(m.elemToNode, np.int32).copy()
    N, h = _ctx()
    try:
        # coloring_creation + in-place permutation (src/main.cc:212-232)
        perm = np.zeros(E, np.int32)
        index = np.zeros(129, np.int32)
        nc = C.c_int()
        _check(N, h, N.lib.mfem_set_mesh(h, None, _p(e2n), E, N_))
        _check(N, h, N.lib.mfem_coloring_creation(h, 0, _p(perm), _p(index), 129, C.byref(nc)))
        permuted = np.empty_like(e2n)
        permuted[perm] = e2n
        e2n[:] = permuted                       # same array, new contents
        # create_nodeToNode from DC-lib-style lists (src/main.cc:238-250)
        idx, val = O.node_to_elem(e2n, N_)
        _check(N, h, N.lib.mfem_set_mesh(h, None, _p(e2n), E, N_))
        nnz = C.c_int()
        _check(N, h, N.lib.mfem_create_nodeToNode_incidence(h, _p(idx), _p(val), None, None, 0,
                                                             C.byref(nnz)))
        row = np.zeros(N_ + 1, np.int32)
        col = np.zeros(nnz.value, np.int32)
        _check(N, h, N.lib.mfem_create_nodeToNode_incidence(h, _p(idx), _p(val), _p(row), _p(col),
                                                             col.size, C.byref(nnz)))
        vals = np.zeros(nnz.value * d, np.float64)
        for step in range(2):
            _check(N, h, N.lib.mfem_assembly(h, _p(coord), _p(vals), _p(row), _p(col), _p(e2n),
                                             None, E, nnz.value, d, O.op_id(op)))
            ref = O.assembly(coord, row, col, e2n, nnz.value, op)
            assert vals.tobytes() == ref.tobytes(), f"step {step}"
            # DC_permute_int_2d_array-style in-place reversal of the element rows
            e2n[:] = e2n[::-1].copy()
    finally:
        N.lib.mfem_destroy(h)


def test_optimized_elemToEdge_matches_oracle():
    m = cube_mesh(7, seed=2, op="ela", coefficients=False)
    N_, E = m.nbNodes, m.nbElem
    e2n = np.ascontiguousarray(m.elemToNode, np.int32)
    idx, val = O.node_to_elem(e2n, N_)
    row_ref, col_ref = O.pattern_from_incidence(idx, val, e2n, N_)
    N, h = _ctx()
    try:
        _check(N, h, N.lib.mfem_set_mesh(h, None, _p(e2n), E, N_))
        row = np.zeros(N_ + 1, np.int32)
        col = np.zeros(col_ref.size, np.int32)
        nnz = C.c_int()
        _check(N, h, N.lib.mfem_create_nodeToNode_incidence(h, _p(idx), _p(val), _p(row), _p(col),
                                                             col.size, C.byref(nnz)))
        pos = np.zeros(16 * E, np.int32)
        _check(N, h, N.lib.mfem_create_elemToEdge(h, _p(pos)))
        assert np.array_equal(pos, O.elem_to_edge(row_ref, col_ref, e2n))
    finally:
        N.lib.mfem_destroy(h)
