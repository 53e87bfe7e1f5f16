"""Reference-format chunk-neighbour streams built on the GPU (xnb_chunk_neighbors_stream)
against the oracle's own stream encoder, and the GPU verify_chunk_neighbors.

The oracle restates chunk_neighbors_execute.h's encoder; the GPU streams must equal
its streams word for word (offset table, group counts, encoded cells, particle
indices, ghost-cell indices) at init and after rebuilds, and the GPU checker must
find nothing wrong with them."""
import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import ncells, new_batch, oracle_from

pytestmark = pytest.mark.gpu


def gpu_system(w, list_factor=1.3):
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=list_factor)
    return b, s


def host_streams(b, s, T):
    buf, off = b.chunk_neighbors_stream(s, T)
    return buf.cpu().numpy().view(np.uint16), off.cpu().numpy().astype(np.int64)


def dual_counts(stream, na):
    """Second offset table from a one-table stream: per particle, neighbours in
    cells that precede the cell in grid order or earlier in the same cell."""
    body = stream[(na + 1) * 2:]
    out = []
    for pa in range(na):
        o = int(stream[pa * 2]) | (int(stream[pa * 2 + 1]) << 16)
        p = o - 1
        groups = int(body[p]); p += 1
        lower = 0
        for _ in range(groups):
            enc, cnt = int(body[p]), int(body[p + 1]); p += 2
            di, dj, dk = (enc & 31) - 16, ((enc >> 5) & 31) - 16, ((enc >> 10) & 31) - 16
            rel = dk * 9 + dj * 3 + di
            for q in range(cnt):
                pb = int(body[p + q])
                lower += rel < 0 or (rel == 0 and pb < pa)
            p += cnt
        out.append(lower)
    return out


def compare_with_oracle(b, s, o, w):
    st, off = host_streams(b, s, 1)
    nc = ncells(w["geom"])
    assert len(off) == nc + 1 and off[0] == 0 and off[-1] == len(st)
    for c in range(nc):
        want = o.cell_stream(c)
        got = st[off[c]:off[c + 1]]
        assert np.array_equal(got, want), "cell %d stream differs" % c
    return st, off


def test_streams_equal_oracle_at_init_and_after_rebuilds():
    w = workloads.lj_fcc_system(20, 0.8442, 1.44, 12345)  # 32,000 atoms
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    o = oracle_from(w)
    o.init()
    compare_with_oracle(b, s, o, w)
    checked = 0
    for _ in range(40):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        o.step()
        if b.info(s).rebuilds != r0:
            # the rebuild ran after this step's position push: lists match positions
            compare_with_oracle(b, s, o, w)
            checked += 1
    assert checked >= 3


def test_offset_table_variants_and_checker():
    w = workloads.lj_fcc_system(14, 0.8442, 1.44, 3)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_MIXED)
    b.step(30, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    b.chunk_neighbors(s)  # fresh lists for the current positions
    s1, o1 = host_streams(b, s, 1)
    s0, o0 = host_streams(b, s, 0)
    s2, o2 = host_streams(b, s, 2)
    counts = b.download(s)["cell"]
    na = np.bincount(counts, minlength=ncells(w["geom"]))
    for c in range(ncells(w["geom"])):
        a1, a0, a2 = s1[o1[c]:o1[c + 1]], s0[o0[c]:o0[c + 1]], s2[o2[c]:o2[c + 1]]
        n = int(na[c])
        if n == 0:
            assert len(a1) == len(a0) == len(a2) == 0
            continue
        body1 = a1[(n + 1) * 2:]
        assert np.array_equal(a0, body1), "no-table stream is the one-table body"
        t2 = (2 * n + 1) * 2
        assert np.array_equal(a2[t2:], body1)
        dual = [int(a2[(n + 1 + p) * 2]) | (int(a2[(n + 1 + p) * 2 + 1]) << 16) for p in range(n)]
        assert dual == dual_counts(a1, n)
    for T in (0, 1, 2):
        buf, off = b.chunk_neighbors_stream(s, T)
        res = b.verify_chunk_neighbors(s, buf, off, T)
        assert all(v == 0 for v in res.values()), (T, res)


def test_checker_clean_on_slab_and_dense_cells():
    slab = workloads.lj_slab_system(10, 0.8442, 0.8, 7)
    b, s = gpu_system(slab)
    b.init_particles(s, xnb.PREC_MIXED)
    b.step(20, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
    b.chunk_neighbors(s)
    buf, off = b.chunk_neighbors_stream(s, 1)
    assert all(v == 0 for v in b.verify_chunk_neighbors(s, buf, off, 1).values())
    # 3 cells per side of a 1372-atom box: ~51 particles per cell (more than a
    # warp of them, and dense enough for the in-cell sub-grid sort)
    dense = dict(workloads.lj_fcc_system(7, 0.8442, 1.44, 9))
    L = dense["geom"]["extent"][0] - dense["geom"]["origin"][0]
    dense["geom"] = dict(dense["geom"], dims=[3, 3, 3], cell_size=L / 3)
    b2, s2 = gpu_system(dense)
    b2.init_particles(s2, xnb.PREC_FP64_EXACT)
    buf, off = b2.chunk_neighbors_stream(s2, 2)
    assert all(v == 0 for v in b2.verify_chunk_neighbors(s2, buf, off, 2).values())


def test_stale_lists_are_refused():
    w = workloads.lj_fcc_system(8, 0.8442, 1.44, 5)
    b, s = gpu_system(w)
    b.init_particles(s, xnb.PREC_MIXED)
    b.push_f_v_r(1.0, s)
    with pytest.raises(xnb.XnbError):
        b.chunk_neighbors_stream(s, 1)
    b.chunk_neighbors(s)
    buf, off = b.chunk_neighbors_stream(s, 1)
    assert len(buf) > 0


def test_full_size_lists_are_the_fp64_neighbour_sets():
    """The 4,000,000-atom benchmark system on the mixed path: at init and after
    each rebuild of 40 steps, every list equals the exhaustive FP64 search of the
    27-cell block (no missing or extra pair, no self, order and format kept)."""
    w = workloads.lj_fcc_system(100, 0.8442, 1.44, 12345)
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])], list_per_atom=160.0)
    s = b.add_system(xnb.lj_params(w["geom"]), w["r"], w["v"], w["id"], list_factor=1.2)
    b.init_particles(s, xnb.PREC_MIXED)
    checked = 0

    def check():
        buf, off = b.chunk_neighbors_stream(s, 2)
        res = b.verify_chunk_neighbors(s, buf, off, 2)
        assert all(v == 0 for v in res.values()), res

    check()
    for _ in range(40):
        r0 = b.info(s).rebuilds
        b.step(1, xnb.PREC_MIXED, xnb.STEP_HOST_SYNC)
        if b.info(s).rebuilds != r0:
            check()
            checked += 1
    assert checked >= 4
