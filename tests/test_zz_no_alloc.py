"""mfem_assemble_noalloc: the allocation-free FP64 gather for callers that cannot
allocate device memory while they assemble (solvers that own all device memory
through their own pool, loops that cannot afford cudaFree's implicit device
synchronisation, real-time loops).  Its result
must equal the allocating entry point's (mfem_assemble, FP64 gather) -- bit for bit,
the tolerance of the FP64 gather tests -- on two calls in a row.  This file is
collected last so that a run stopping at the first failure has run everything else."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ELEM = 131072


def _setup(op, coef, n=20, seed=3):
    import minifem
    from minifem.meshgen import cube_mesh
    m = cube_mesh(n, seed=seed, op=op)
    a = minifem.Assembler(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    c = m.coef if coef else None
    a.set_coefficients(op, c)
    a.assembly(op, "fp64", "gather")          # the existing, allocating entry point
    return m, a, c, a.values()


@pytest.mark.parametrize("op,coef", [("ela", True), ("ela", False), ("lap", True)])
def test_no_alloc_matches_allocating_entry_point(op, coef):
    import torch
    from minifem import _native as N
    m, a, c, expected = _setup(op, coef)
    assert m.nbElem <= MAX_ELEM
    dev = torch.device("cuda", 0)
    d_coord = torch.from_numpy(np.ascontiguousarray(m.coord)).to(dev)
    d_coef = torch.from_numpy(np.ascontiguousarray(c)).to(dev) if c is not None else None
    d_vals = torch.empty(expected.size, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    free_before = None
    for call in range(2):
        d_vals.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        if call == 1:
            free_before = torch.cuda.mem_get_info(dev)[0]
        rc = N.lib.mfem_assemble_noalloc(a._h, 0 if op == "lap" else 1,
                                         C.c_void_p(d_coord.data_ptr()),
                                         C.c_void_p(d_coef.data_ptr()) if d_coef is not None else None,
                                         C.c_void_p(d_vals.data_ptr()),
                                         C.c_void_p(stream.cuda_stream))
        assert rc == 0, N.lib.mfem_last_error(a._h).decode()
        torch.cuda.synchronize(dev)
        if call == 1:
            # nothing was allocated on the device by the second call
            assert torch.cuda.mem_get_info(dev)[0] == free_before
        got = d_vals.cpu().numpy()
        assert got.tobytes() == expected.tobytes(), f"call {call} differs"
    a.close()


def test_no_alloc_rejects_meshes_beyond_its_limit():
    import torch
    from minifem import _native as N
    import minifem
    from minifem.meshgen import cube_mesh
    m = cube_mesh(29, seed=1, op="lap", coefficients=False)   # 131,712 elements
    assert m.nbElem > MAX_ELEM
    a = minifem.Assembler(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.assembly("lap", "fp64", "gather")
    dev = torch.device("cuda", 0)
    d_coord = torch.from_numpy(np.ascontiguousarray(m.coord)).to(dev)
    d_vals = torch.zeros(a.nbEdges, dtype=torch.float64, device=dev)
    rc = N.lib.mfem_assemble_noalloc(a._h, 0, C.c_void_p(d_coord.data_ptr()), None,
                                     C.c_void_p(d_vals.data_ptr()), None)
    assert rc == -7   # MFEM_ERR_CAPACITY
    assert "131072" in N.lib.mfem_last_error(a._h).decode()
    a.close()
