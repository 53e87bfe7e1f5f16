"""Host-side checks of two bounds the kernels rely on.

1. Sub-cell pair pruning (csrc/xnb_build_sub.cu): the integer box-gap test,
   widened by 1e-5, keeps every sub-cell pair that the reference's FP64 box test
   keeps (max_distance_sub_cell_pairs, amr/lib/amr_grid_algorithm.cpp:102-218:
   min distance between the boxes <= max_dist), and every particle pair within
   nbh_dist whose particles lie in those boxes.
2. Packed position residuals (csrc/xnb_internal.cuh, lo_code / lo_field): the
   residual lo = fl32((x - o) - fl32(x - o)) is packed as a signed 10-bit
   multiple of lo_step = ulp32(X) / 1024 and decoded within lo_step of lo for
   every |x - o| <= X; the compensated FP32 displacement built from packed
   residuals stays within 2u|d| + 2 lo_step of the FP64 one per axis, so the
   mixed path's cutoff margin (xnb_api.cu, make_desc) covers its r^2 error.
"""
import math

import numpy as np
import pytest

F32 = np.float32


# ---------------------------------------------------------------- sub-cells
def gap(ia, sa, d, ib, sb):
    """the kernel's box_gap: units of cell / (sa sb)"""
    alo, ahi = ia * sb, ia * sb + sb
    blo = d * sa * sb + ib * sa
    bhi = blo + sa
    return max(0, blo - ahi, alo - bhi)


def kept_integer(ia, ja, ka, sa, off, ib, jb, kb, sb, reach_f):
    g = [gap(ia, sa, off[0], ib, sb), gap(ja, sa, off[1], jb, sb), gap(ka, sa, off[2], kb, sb)]
    lim = F32(reach_f) * F32(sa * sb)
    return F32(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) <= lim * lim


def min_dist2_fp64(cs, sa, a, sb, off, b):
    """the reference's AABB test: boxes in FP64 relative to cell a's corner"""
    ha, hb = cs / sa, cs / sb
    d2 = 0.0
    for ax in range(3):
        alo, ahi = a[ax] * ha, (a[ax] + 1) * ha
        blo, bhi = off[ax] * cs + b[ax] * hb, off[ax] * cs + (b[ax] + 1) * hb
        g = max(0.0, blo - ahi, alo - bhi)
        d2 += g * g
    return d2


def reach(nbh, cs):
    return np.nextafter(F32(nbh / cs * (1.0 + 1e-5)), F32(2.0))


@pytest.mark.parametrize("cs", [2.8, 2.85, 4.0, 5.418, 5.6, 5.792, 6.718, 8.4])
def test_integer_reach_keeps_every_reference_subcell_pair(cs):
    nbh = 2.8
    r = reach(nbh, cs)
    offsets = [(di, dj, dk) for dk in (-1, 0, 1) for dj in (-1, 0, 1) for di in (-1, 0, 1)]
    for sa in (1, 2, 3):
        for sb in (1, 2, 3):
            for off in offsets:
                for ka in range(sa):
                    for ja in range(sa):
                        for ia in range(sa):
                            for kb in range(sb):
                                for jb in range(sb):
                                    for ib in range(sb):
                                        ref = min_dist2_fp64(cs, sa, (ia, ja, ka), sb, off, (ib, jb, kb)) <= nbh * nbh
                                        ours = kept_integer(ia, ja, ka, sa, off, ib, jb, kb, sb, r)
                                        assert ours or not ref, (cs, sa, sb, off, (ia, ja, ka), (ib, jb, kb))


def test_pruned_subcells_hold_no_neighbour_pairs():
    """Random particles in random sub-cells of neighbouring cells: a pair within
    nbh always lies in a kept sub-cell pair (keys as the rebin computes them)."""
    rng = np.random.default_rng(3)
    nbh = 2.8
    for cs in (5.6, 6.718, 4.0):
        r = reach(nbh, cs)
        for sa in (2, 3):
            for sb in (1, 2, 3):
                for _ in range(4000):
                    off = rng.integers(-1, 2, size=3)
                    pa = rng.random(3) * cs
                    pb = off * cs + rng.random(3) * cs
                    if np.sum((pa - pb) ** 2) > nbh * nbh:
                        continue
                    ka = np.minimum((pa / cs * sa).astype(int), sa - 1)
                    kb = np.minimum(((pb - off * cs) / cs * sb).astype(int), sb - 1)
                    assert kept_integer(ka[0], ka[1], ka[2], sa, off, kb[0], kb[1], kb[2], sb, r)


# ---------------------------------------------------------------- residuals
def lo_step_of(X):
    e = math.frexp(X)[1]
    return F32(math.ldexp(1.0, e - 34)), F32(math.ldexp(1.0, 34 - e))


def lo_code(lo, inv):
    t = F32(lo) * F32(inv)  # exact: inv is a power of two
    q = int(np.rint(np.float64(t)))  # fmaf(lo, inv, 1.5 2^23) rounds to nearest even
    return max(-511, min(511, q))


@pytest.mark.parametrize("X", [36.4, 170.8, 700.0, 1023.0])
def test_packed_residual_within_one_quantum(X):
    step, inv = lo_step_of(X)
    rng = np.random.default_rng(7)
    x = rng.uniform(-0.02 * X, X, 20000)
    hi = x.astype(F32)
    lo = (x - hi.astype(np.float64)).astype(F32)
    q = np.array([lo_code(v, inv) for v in lo])
    dec = q.astype(np.float64) * np.float64(step)
    assert np.abs(dec - lo.astype(np.float64)).max() <= float(step)
    # hi + decoded residual within the residual's own rounding plus one quantum of x
    assert np.abs(hi.astype(np.float64) + dec - x).max() <= float(step) + 2.0 ** -48 * X * 2


@pytest.mark.parametrize("X", [36.4, 170.8, 700.0])
def test_compensated_displacement_and_cutoff_margin(X):
    """dx = fma(qb - qa, step, hb - ha) in FP32 is within 2u|d| + 2 step of the
    FP64 displacement, and |r2_f32 - d2| stays below the cutoff margin of
    make_desc at rc = 2.5 (4 (6u (rc^2 + 1) + 2 sqrt(3) rc delta + 3 delta^2))."""
    u = 2.0 ** -24
    step, inv = lo_step_of(X)
    delta = 2.0 * float(step)
    rc = 2.5
    margin = 4.0 * (6.0 * u * (rc * rc + 1.0) + 2.0 * math.sqrt(3.0) * rc * delta + 3.0 * delta * delta)
    rng = np.random.default_rng(11)
    n = 20000
    xa = rng.uniform(0.0, X - 3.0, (n, 3))
    dvec = rng.normal(size=(n, 3))
    dvec *= (rng.uniform(0.8, 2.6, n) / np.linalg.norm(dvec, axis=1))[:, None]
    xb = xa + dvec
    ha, hb = xa.astype(F32), xb.astype(F32)
    la = (xa - ha.astype(np.float64)).astype(F32)
    lb = (xb - hb.astype(np.float64)).astype(F32)
    qa = np.vectorize(lambda v: lo_code(v, inv))(la)
    qb = np.vectorize(lambda v: lo_code(v, inv))(lb)
    dh = (hb - ha).astype(F32)
    dq = (qb - qa).astype(F32)
    dx = (dq.astype(np.float64) * float(step) + dh.astype(np.float64)).astype(F32)  # one rounding, as fmaf
    d64 = xb - xa
    d = np.linalg.norm(d64, axis=1)
    err = np.abs(dx.astype(np.float64) - d64)
    # (+ the FP32 rounding of each residual, at most 2^-48 X)
    assert np.all(err <= 2 * u * np.abs(d64) + delta + 2.0 ** -46 * X)
    r2 = (dx[:, 0] * dx[:, 0] + dx[:, 1] * dx[:, 1] + dx[:, 2] * dx[:, 2]).astype(F32)
    assert np.abs(r2.astype(np.float64) - d * d)[d <= rc + 0.1].max() <= margin / 4 * 1.5
