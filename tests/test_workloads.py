"""Synthetic workload generators (host only): FCC lattices, the periodic box's
cell grid, including grids of larger cells (cell_factor) for dense cells."""
import numpy as np
import pytest

from exanbody_gb300 import workloads


@pytest.mark.parametrize("n,factor", [(20, 1.0), (20, 1.9), (20, 2.0), (20, 2.5), (100, 1.0), (100, 2.0)])
def test_cell_grid_covers_the_box_with_cells_of_at_least_the_factor(n, factor):
    w = workloads.lj_fcc_system(n, 0.8442, 1.44, 1, cell_factor=factor)
    g = w["geom"]
    nbh = 2.5 + 0.3
    assert g["cell_size"] >= factor * nbh * (1 - 1e-12)
    L = n * w["a"]
    for d, e in zip(g["dims"], g["extent"]):
        assert d >= 2
        assert abs(d * g["cell_size"] - e) <= 1e-9 * e
        assert abs(e - L) <= 1e-9 * L  # a cube of whole cells: the lattice period
    r = w["r"]
    assert r.min() >= 0.0 and r.max() < L and len(r) == 4 * n ** 3


def test_slab_is_elongated_with_matching_cells():
    w = workloads.lj_slab_system(12, cell_factor=2.0)
    g = w["geom"]
    assert g["dims"][2] == 2 * g["dims"][0] and g["cell_size"] >= 2.0 * 2.8
    z = w["r"][:, 2]
    assert z.min() > 0.2 * g["extent"][2] and z.max() < 0.8 * g["extent"][2]


def test_fcc_lattice_elongated_block():
    r, a = workloads.fcc_lattice(5, 0.8442, nz=7)
    assert r.shape == (4 * 5 * 5 * 7, 3)
    assert np.isclose(a, (4 / 0.8442) ** (1 / 3))
    assert r[:, 2].max() < 7 * a and r[:, 0].max() < 5 * a
