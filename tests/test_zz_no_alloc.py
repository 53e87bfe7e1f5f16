"""The allocation-free neighbour build (xnb_chunk_neighbors_noalloc).

Callers that cannot allocate device memory at the point where they need
neighbour lists -- a host framework that owns all device memory through its
own pools, or a step loop that must not stall on the device-wide
synchronisation cudaFree can impose -- use this entry point with their own
input and output buffers; its scratch is a static device array inside the
library.

The lists it returns must equal the ones the batch entry points build for the
same positions (integer work: exact equality), on consecutive calls that share
the scratch array, including cells whose candidates exceed one staging round.
Its limits (particles, cells, 32-bit entry positions) and the capacity error
are checked too. This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from exanbody_gb300 import workloads, xnb
from helpers import ncells, new_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def batch_lists(w, steps):
    """Reference lists from the existing entry points (batch, init, steps)."""
    b = new_batch([w["n_atoms"]], [ncells(w["geom"])])
    params = xnb.lj_params(w["geom"])
    s = b.add_system(params, w["r"], w["v"], w["id"])
    b.init_particles(s, xnb.PREC_FP64_EXACT)
    if steps:
        b.step(steps, xnb.PREC_FP64_EXACT, xnb.STEP_HOST_SYNC)
        b.update_particles_full(s)  # lists built from the current positions
    P = b.download(s)
    ida, idb, cnt = b.pairs(s)
    b.close()
    return params, P, ida, idb, cnt


def noalloc_buffers(P, nc, cap):
    n = len(P["id"])
    dev = torch.device("cuda", 0)
    counts = np.bincount(P["cell"], minlength=nc).astype(np.uint32)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32)
    t = {k: torch.from_numpy(np.ascontiguousarray(P[k])).to(dev) for k in ("rx", "ry", "rz")}
    t["cs"] = torch.from_numpy(starts.view(np.int32)).to(dev)
    t["cc"] = torch.from_numpy(counts.view(np.int32)).to(dev)
    t["nbr"] = torch.full((max(cap, 1),), -7, dtype=torch.int32, device=dev)
    t["nst"] = torch.full((n,), -7, dtype=torch.int32, device=dev)
    t["ncn"] = torch.full((n,), -7, dtype=torch.int32, device=dev)
    return t


def call_noalloc(params, n, t, cap):
    stream = torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream
    return xnb.chunk_neighbors_noalloc(params, n, t["rx"].data_ptr(), t["ry"].data_ptr(), t["rz"].data_ptr(),
                                       t["cs"].data_ptr(), t["cc"].data_ptr(), t["nbr"].data_ptr(), cap,
                                       t["nst"].data_ptr(), t["ncn"].data_ptr(), stream=stream)


def noalloc_lists(params, P, nc):
    n = len(P["id"])
    cap = n * 100 + 64
    t = noalloc_buffers(P, nc, cap)
    total = call_noalloc(params, n, t, cap)
    torch.cuda.synchronize()
    ent = t["nbr"][:total].cpu().numpy().view(np.uint32)
    st = t["nst"].cpu().numpy().view(np.uint32)
    cn = t["ncn"].cpu().numpy().view(np.uint32)
    ids = P["id"]
    ida = np.repeat(ids, cn)
    idb = np.empty(total, np.uint64)
    k = 0
    for q in range(n):
        idb[k:k + cn[q]] = ids[ent[st[q]:st[q] + cn[q]] >> 5]
        k += cn[q]
    return ida, idb, cn.astype(np.int32)


def test_noalloc_matches_batch_build_on_consecutive_calls():
    cases = [
        (workloads.lj_fcc_system(20, 0.8442, 1.44, 12345), 25),  # 32,000 atoms, 11^3 cells, after moves
        (workloads.lj_fcc_system(5, 1.0, 1.2, 8), 10),           # 500 atoms, 2^3 dense cells (AMR order)
    ]
    for w, steps in cases + cases[:1]:  # three calls in a row on the shared scratch
        params, P, ida, idb, cnt = batch_lists(w, steps)
        ga, gb, gc = noalloc_lists(params, P, ncells(w["geom"]))
        assert np.array_equal(gc, cnt)
        assert np.array_equal(ga, ida) and np.array_equal(gb, idb)


def test_noalloc_rejects_sizes_above_its_scratch():
    w = workloads.lj_fcc_system(4, 0.8442, 1.44, 1)
    params = xnb.lj_params(w["geom"])
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    ib = torch.zeros(16, dtype=torch.int32, device=dev)
    with pytest.raises(xnb.XnbError) as e:
        xnb.chunk_neighbors_noalloc(params, (1 << 20) + 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                    ib.data_ptr(), ib.data_ptr(), ib.data_ptr(), 16, ib.data_ptr(), ib.data_ptr())
    assert e.value.code == -1 and "1048576 particles" in str(e.value)


def test_noalloc_stages_dense_cells_in_rounds():
    """62 atoms per cell: each cell has ~1,700 candidates, more than one staging
    round of the kernel (640), so lists are carried across rounds."""
    w = workloads.lj_fcc_system(4, 1.0, 0.9, 7)
    params, P, ida, idb, cnt = batch_lists(w, 10)
    nc = ncells(w["geom"])
    per_cell = np.bincount(P["cell"], minlength=nc)
    assert per_cell.max() * 27 > 640
    ga, gb, gc = noalloc_lists(params, P, nc)
    assert np.array_equal(gc, cnt)
    assert np.array_equal(ga, ida) and np.array_equal(gb, idb)


def test_noalloc_capacity_error_reports_the_total_and_writes_no_list():
    w = workloads.lj_fcc_system(6, 0.8442, 1.44, 3)
    params, P, ida, idb, cnt = batch_lists(w, 0)
    nc = ncells(w["geom"])
    n = len(P["id"])
    total = int(cnt.sum())
    t = noalloc_buffers(P, nc, total - 1)
    with pytest.raises(xnb.XnbError) as e:
        call_noalloc(params, n, t, total - 1)
    assert e.value.code == xnb.ERR_CAPACITY
    assert e.value.total == total
    torch.cuda.synchronize()
    # the fill pass did not run: entries and starts keep their sentinel
    assert bool((t["nbr"] == -7).all()) and bool((t["nst"] == -7).all())
    # the count pass ran: counts are the batch build's
    assert np.array_equal(t["ncn"].cpu().numpy(), cnt)
    # the same buffers with the exact capacity then succeed
    assert call_noalloc(params, n, t, total) == total


@pytest.mark.parametrize("dims", [(64, 64, 33), (65536, 65536, 2)])
def test_noalloc_rejects_cell_counts_above_its_scratch(dims):
    """(64, 64, 33) is 135,168 cells; (65536, 65536, 2) is 2^33, which a 32-bit
    product would wrap to 0: both are rejected before any launch."""
    geom = {"origin": (0.0, 0.0, 0.0), "extent": tuple(2.9 * d for d in dims), "dims": dims, "cell_size": 2.9}
    params = xnb.lj_params(geom)
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    ib = torch.zeros(16, dtype=torch.int32, device=dev)
    with pytest.raises(xnb.XnbError) as e:
        xnb.chunk_neighbors_noalloc(params, 4, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), ib.data_ptr(),
                                    ib.data_ptr(), ib.data_ptr(), 16, ib.data_ptr(), ib.data_ptr())
    assert e.value.code == -1 and "131072 cells" in str(e.value)
