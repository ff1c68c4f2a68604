import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import (cube_mesh, cube_sizes, fan_mesh, read_reference_input,
                             write_reference_input)


@pytest.mark.parametrize("n,expect", [(30, (146334, 27000, 383758)),
                                      (60, (1232274, 216000, 3154318)),
                                      (100, (5821794, 1000000, 14761198))])
def test_sizes_match_the_benchmark_configs(n, expect):
    assert cube_sizes(n) == expect


def test_deterministic_and_seeded():
    a = cube_mesh(6, seed=3)
    b = cube_mesh(6, seed=3)
    c = cube_mesh(6, seed=4)
    assert np.array_equal(a.coord, b.coord) and np.array_equal(a.elemToNode, b.elemToNode)
    assert not np.array_equal(a.coord, c.coord)


def test_permutation_and_boundary_codes():
    m = cube_mesh(5, seed=1)
    assert sorted(np.unique(m.elemToNode)) == list(range(1, m.nbNodes + 1))
    codes, counts = np.unique(m.boundNodesCode, return_counts=True)
    assert set(codes) == {0, 10, 52, 53, 54}
    assert counts[list(codes).index(0)] == 27   # interior of a 5^3 grid
    # boundary nodes stay on their face
    on_x0 = m.boundNodesCode == 52
    assert np.all(m.coord[on_x0, 0] == 0.0)


def test_coefficient_ranges():
    m = cube_mesh(8, seed=2, op="ela")
    E, nu = m.coef[:, 0], m.coef[:, 1]
    assert E.min() >= 1e9 and E.max() <= 2e11
    assert nu.min() >= 0.2 and nu.max() <= 0.35
    lap = cube_mesh(8, seed=2, op="lap")
    assert lap.coef.min() >= 0.5 and lap.coef.max() <= 2.0


def test_stress_variant_makes_slivers_and_jump():
    m = cube_mesh(12, seed=5, op="ela", jitter=0.45, sliver_fraction=0.05, jump=1e6, nu_max=0.45)
    assert m.meta["slivers_made"] > 0
    E = m.coef[:, 0]
    assert E.max() / E.min() > 1e6


def test_reference_file_round_trip(tmp_path):
    m = cube_mesh(4, seed=7)
    p = tmp_path / "ela_1_0"
    write_reference_input(m, str(p))
    r = read_reference_input(str(p))
    assert np.array_equal(r.coord, m.coord) and np.array_equal(r.elemToNode, m.elemToNode)
    assert np.array_equal(r.boundNodesCode, m.boundNodesCode) and r.nbEdges == m.nbEdges


def test_truncated_file_is_rejected(tmp_path):
    m = cube_mesh(4, seed=7)
    p = tmp_path / "ela_1_0"
    write_reference_input(m, str(p))
    data = p.read_bytes()
    p.write_bytes(data[: len(data) // 2])
    with pytest.raises(ValueError):
        read_reference_input(str(p))


@pytest.mark.parametrize("subdivisions", [1, 2, 3])
def test_fan_mesh_centre_row_holds_every_node(subdivisions):
    """Every tetrahedron of the fan mesh touches the centre node: its row holds
    all nodes, the element volumes are positive in the reference's orientation,
    and the stated CSR size is the pattern's."""
    m = fan_mesh(subdivisions, seed=3)
    F = 20 * 4 ** subdivisions
    assert m.nbElem == F and m.nbNodes == 10 * 4 ** subdivisions + 3
    row, col = O.pattern(m.elemToNode, m.nbNodes)
    assert int(row[-1]) == m.nbEdges
    assert np.diff(row).max() == m.nbNodes
    X = m.coord[m.elemToNode - 1]
    a, b, c = X[:, 0] - X[:, 3], X[:, 2] - X[:, 3], X[:, 1] - X[:, 3]
    assert np.einsum("ij,ij->i", a, np.cross(b, c)).min() > 0.0
