"""Consumer of the assembled system: block-CSR SpMV against the correctly
rounded product (exact parts, math.fsum) within stated bounds and against
scipy, block-Jacobi apply and block-Jacobi preconditioned CG, on the same
assembled matrix."""
import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import cube_mesh
from spmv_exact import BOUND, exact_apply as _exact_apply

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


@pytest.mark.parametrize("op,precision", [("ela", "fp64"), ("ela", "fp32"), ("lap", "fp64"), ("lap", "fp32")])
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
    f = _free_mask(markf, N, dim) if constrained else np.ones(N * dim)
    ref, scale = _exact_apply(row, col, vals, dim, f * x)
    free = f != 0
    assert np.array_equal(y[~free], x[~free])          # constrained rows: the identity
    live = free & (scale > 0)
    assert np.all(y[free & ~live] == 0.0)
    assert np.max(np.abs(y[live] - ref[live]) / scale[live]) < BOUND[precision]
    # and scipy's product agrees to its own rounding
    sref = f * (A @ (f * x)) + (1 - f) * x
    assert np.max(np.abs(y - sref) / (abs(A) @ abs(f * x) + abs(x))) < 1e-13


def _spmv(a, x):
    xd = _dev(x)
    yd = torch.empty(len(x), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    a.spmv(xd.data_ptr(), yd.data_ptr(), False)
    a.synchronize()
    torch.cuda.synchronize()
    return yd.cpu().numpy()


@pytest.mark.parametrize("op", ["ela", "lap"])
def test_spmv_fp32_values_any_scale(gpu, op):
    """FP32 values: x is scaled by a power of two and split into FP32 parts;
    rows the split cannot serve (entries far below the largest, all-zero rows)
    take the FP64 chain.  Every case within the FP32 bound of the row's
    magnitude sum, exact zeros where every product is zero."""
    m, a, row, col, vals, prec, markf = _assembled(gpu, op, precision="fp32")
    dim = 1 if op == "lap" else 3
    N = len(row) - 1
    A = _matrix(row, col, vals, dim)
    n = N * dim
    rng = np.random.default_rng(7)
    cases = {
        "tiny": rng.standard_normal(n) * 1e-200,
        "huge": rng.standard_normal(n) * 1e200,
        "spread": rng.standard_normal(n) * 10.0 ** rng.uniform(-40, 40, n),
        "sparse": np.where(rng.random(n) < 0.05, rng.standard_normal(n), 0.0),
        "zero": np.zeros(n),
    }
    for name, x in cases.items():
        y = _spmv(a, x)
        ref, scale = _exact_apply(row, col, vals, dim, x)
        live = scale > 0
        assert np.all(y[~live] == 0.0), name
        assert np.max(np.abs(y[live] - ref[live]) / scale[live], initial=0.0) < BOUND["fp32"], name


def test_spmv_fp32_values_non_finite(gpu):
    """A NaN or infinite x entry: the rows whose pattern holds its node come out
    NaN or infinite as with FP64 values; every other row is unaffected."""
    m, a, row, col, vals, prec, markf = _assembled(gpu, "ela", precision="fp32")
    N = len(row) - 1
    A = _matrix(row, col, vals, 3)
    rng = np.random.default_rng(8)
    for bad in (np.nan, np.inf):
        x = rng.standard_normal(3 * N)
        node = N // 2
        x[3 * node + 1] = bad
        y = _spmv(a, x)
        rows = np.repeat(np.arange(N), np.diff(row))
        hit = np.zeros(N, bool)
        hit[rows[col - 1 == node]] = True
        hit3 = np.repeat(hit, 3)
        assert not np.isfinite(y[hit3]).any()
        xf = np.where(np.isfinite(x), x, 0.0)
        ref, scale = _exact_apply(row, col, vals, 3, xf)
        ok = ~hit3
        assert np.isfinite(y[ok]).all()
        assert np.max(np.abs(y[ok] - ref[ok]) / scale[ok]) < BOUND["fp32"]


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


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pcg_scale_equivariant(gpu, precision):
    """b times a power of two gives the same iterations and exactly the solution
    times that power: every reduction, alpha and beta is scale-free in FP64,
    and the FP32-valued operator's split follows the scale of p (the FP32
    arithmetic then sees the same significands), over 600 binary orders."""
    m, a, row, col, vals, prec, markf = _assembled(gpu, "ela", n=9, precision=precision)
    N = len(row) - 1
    b = np.random.default_rng(11).standard_normal(3 * N)
    x0, it0, rel0 = a.pcg(b, rtol=1e-10, max_iter=2000)
    for k in (-300, 300):
        x1, it1, rel1 = a.pcg(np.ldexp(b, k), rtol=1e-10, max_iter=2000)
        assert it1 == it0 and rel1 == rel0
        assert x1.tobytes() == np.ldexp(x0, k).tobytes()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pcg_stops_at_the_iteration_limit(gpu, precision):
    """maxIter below what the tolerance needs: exactly maxIter iterations (also
    when maxIter is not a multiple of the iterations enqueued per look at the
    stop flag: the flag freezes the iterate), and the same bits when repeated."""
    m, a, row, col, vals, prec, markf = _assembled(gpu, "ela", n=9, precision=precision)
    N = len(row) - 1
    b = np.random.default_rng(13).standard_normal(3 * N)
    x5, it5, rel5 = a.pcg(b, rtol=1e-14, max_iter=5)
    assert it5 == 5 and rel5 > 1e-14
    x13, it13, rel13 = a.pcg(b, rtol=1e-14, max_iter=13)   # not a multiple of the batch
    assert it13 == 13 and np.isfinite(rel13)
    # a repeated limited solve gives the same iterate
    x5b, it5b, rel5b = a.pcg(b, rtol=1e-14, max_iter=5)
    assert it5b == 5 and rel5b == rel5 and x5b.tobytes() == x5.tobytes()


def test_solver_needs_an_assembly(gpu):
    m = cube_mesh(5, seed=1, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    with pytest.raises(Exception):
        a.pcg(np.ones(a.nbNodes * 3))
