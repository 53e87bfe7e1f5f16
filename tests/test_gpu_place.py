"""Placement of a flat particle array into cell order on the device (xnb_system_add
without cell counts): the cell of domain_periodic_location with positions wrapped
by whole cells, input order kept inside each cell, mirrors and cell table set.
Checked against a numpy restatement of the same bucketing, bit for bit."""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import ncells, new_batch

pytestmark = pytest.mark.gpu


def bucket(r, geom):
    """numpy form of the placement: (order of input rows, wrapped positions, cell)."""
    o = np.asarray(geom["origin"], np.float64)
    cs = float(geom["cell_size"])
    dims = np.asarray(geom["dims"], np.int64)
    r = r.copy()
    loc = np.empty_like(r, dtype=np.int64)
    for ax in range(3):
        l = np.floor((r[:, ax] - o[ax]) / cs).astype(np.int64)
        w = np.mod(l, dims[ax])
        moved = w != l
        r[moved, ax] = r[moved, ax] + (w[moved] - l[moved]).astype(np.float64) * cs
        loc[:, ax] = w
    cell = (loc[:, 2] * dims[1] + loc[:, 1]) * dims[0] + loc[:, 0]
    order = np.argsort(cell, kind="stable")
    return order, r, cell


def check(w, r_in):
    b = new_batch([len(r_in)], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), r_in, w["v"], w["id"])
    P = b.download(s)
    order, rw, cell = bucket(r_in, w["geom"])
    assert np.array_equal(P["id"], w["id"][order])
    assert np.array_equal(P["cell"], cell[order].astype(np.int32))
    for ax, k in enumerate(("rx", "ry", "rz")):
        assert np.array_equal(P[k], rw[order, ax])
    for ax, k in enumerate(("vx", "vy", "vz")):
        assert np.array_equal(P[k], w["v"][order, ax])


def test_flat_placement_matches_stable_bucketing():
    w = workloads.lj_fcc_system(16, 0.8442, 1.44, 31)
    r = w["r"].copy()
    rng = np.random.default_rng(4)
    L = np.asarray(w["geom"]["extent"]) - np.asarray(w["geom"]["origin"])
    shift = rng.integers(-1, 2, size=r.shape) * L  # a third of the coordinates one period out
    check(w, r + shift)


def test_dense_cells_fall_back_to_host_placement():
    # 2 x 2 x 2 cells for 32,000 atoms: 4,000 per cell on average, some above
    # the device pass's 4,096 limit
    w = dict(workloads.lj_fcc_system(20, 0.8442, 1.44, 8))
    L = w["geom"]["extent"][0] - w["geom"]["origin"][0]
    w["geom"] = dict(w["geom"], dims=[2, 2, 2], cell_size=L / 2)
    rng = np.random.default_rng(9)
    r = w["r"].copy()
    r[:, 0] = np.where(rng.random(len(r)) < 0.6, r[:, 0] * 0.5, r[:, 0])  # crowd the low-x cells
    check(w, r)
