"""Consumer of the assembled system: block-CSR SpMV, block-Jacobi apply and
block-Jacobi preconditioned CG, against scipy on the same assembled matrix."""
import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import cube_mesh

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
sp = pytest.importorskip("scipy.sparse")
spla = pytest.importorskip("scipy.sparse.linalg")


def _assembled(gpu, op, n=8, precision="fp64", seed=3):
    m = cube_mesh(n, seed=seed, op=op)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    row, col = a.create_nodeToNode("sorted")
    a.set_coefficients(op, m.coef)
    markf = O.checkbounds(m.boundNodesCode)
    a.set_check_bounds(markf)
    a.assembly(op, precision, "gather", prec=True)
    vals = a.values_f32().astype(np.float64) if precision == "fp32" else a.values()
    return m, a, np.asarray(row), np.asarray(col), vals, a.prec(), markf


def _matrix(row, col, vals, dim):
    N = len(row) - 1
    if dim == 1:
        return sp.csr_matrix((vals, col - 1, row), shape=(N, N))
    return sp.bsr_matrix((vals.reshape(-1, 3, 3), col - 1, row), shape=(3 * N, 3 * N)).tocsr()


def _free_mask(markf, N, dim):
    """1 for free DOFs, 0 for constrained ones (markf: Fortran markf(N,3))."""
    mk = np.asarray(markf).reshape(3, N).T != 0        # (N, 3)
    if dim == 1:
        return (~mk.any(axis=1)).astype(np.float64)
    return (~mk).reshape(-1).astype(np.float64)


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("op,precision", [("ela", "fp64"), ("ela", "fp32"), ("lap", "fp64")])
@pytest.mark.parametrize("constrained", [False, True])
def test_spmv_matches_scipy(gpu, op, precision, constrained):
    m, a, row, col, vals, prec, markf = _assembled(gpu, op, precision=precision)
    dim = 1 if op == "lap" else 3
    N = len(row) - 1
    A = _matrix(row, col, vals, dim)
    x = np.random.default_rng(1).standard_normal(N * dim)
    xd, yd = _dev(x), torch.empty(N * dim, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()       # the library runs on its own stream
    a.spmv(xd.data_ptr(), yd.data_ptr(), constrained)
    a.synchronize()
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    if constrained:
        f = _free_mask(markf, N, dim)
        ref = f * (A @ (f * x)) + (1 - f) * x
    else:
        ref = A @ x
    # summation order differs from scipy's: relative to the row's magnitude sum
    scale = abs(A) @ abs(x) + abs(x)
    assert np.max(np.abs(y - ref) / scale) < 1e-13


def test_prec_apply_matches_blocks(gpu):
    m, a, row, col, vals, prec, markf = _assembled(gpu, "ela")
    N = len(row) - 1
    r = np.random.default_rng(2).standard_normal(N * 3)
    rd, zd = _dev(r), torch.empty(N * 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    a.prec_apply(rd.data_ptr(), zd.data_ptr())
    a.synchronize()
    torch.cuda.synchronize()
    P = prec.reshape(N, 3, 3)
    ref = np.einsum("nij,nj->ni", P, r.reshape(N, 3)).reshape(-1)
    scale = np.einsum("nij,nj->ni", np.abs(P), np.abs(r.reshape(N, 3))).reshape(-1)
    assert np.max(np.abs(zd.cpu().numpy() - ref) / scale) < 1e-15 * 4


@pytest.mark.parametrize("op,precision", [("ela", "fp64"), ("ela", "fp32"), ("lap", "fp64")])
def test_pcg_solves_constrained_system(gpu, op, precision):
    m, a, row, col, vals, prec, markf = _assembled(gpu, op, n=9, precision=precision)
    dim = 1 if op == "lap" else 3
    N = len(row) - 1
    A = _matrix(row, col, vals, dim)
    f = _free_mask(markf, N, dim)
    F = sp.diags(f)
    Ared = (F @ A @ F + sp.diags(1 - f)).tocsc()
    b = np.random.default_rng(5).standard_normal(N * dim)
    x, it, rel = a.pcg(b, rtol=1e-10, max_iter=2000)
    assert rel <= 1e-10 and 0 < it < 2000
    xs = spla.spsolve(Ared, b)
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-6
    # true residual of the returned solution
    assert np.linalg.norm(Ared @ x - b) / np.linalg.norm(b) < 1e-8
    # deterministic reductions: a second solve gives the same bits
    x2, it2, _ = a.pcg(b, rtol=1e-10, max_iter=2000)
    assert it2 == it and x2.tobytes() == x.tobytes()


def test_solver_needs_an_assembly(gpu):
    m = cube_mesh(5, seed=1, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    with pytest.raises(Exception):
        a.pcg(np.ones(a.nbNodes * 3))
