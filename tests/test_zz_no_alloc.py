"""The allocation-free neighbour build (xnb_chunk_neighbors_noalloc).

Callers that cannot allocate device memory at the point where they need
neighbour lists -- a host framework that owns all device memory through its
own pools, or code running inside CUDA stream capture, where allocation calls
are not permitted -- use this entry point with their own input and output
buffers; its scratch is a static device array inside the library.

The lists it returns must equal the ones the batch entry points build for the
same positions (integer work: exact equality), on consecutive calls that share
the scratch array. This file is collected last.
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


def noalloc_lists(params, P, nc):
    n = len(P["id"])
    dev = torch.device("cuda", 0)
    counts = np.bincount(P["cell"], minlength=nc).astype(np.uint32)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32)
    t = {k: torch.from_numpy(np.ascontiguousarray(P[k])).to(dev) for k in ("rx", "ry", "rz")}
    cs = torch.from_numpy(starts.view(np.int32)).to(dev)
    cc = torch.from_numpy(counts.view(np.int32)).to(dev)
    cap = n * 100 + 64
    nbr = torch.empty(cap, dtype=torch.int32, device=dev)
    nst = torch.empty(n, dtype=torch.int32, device=dev)
    ncn = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    total = xnb.chunk_neighbors_noalloc(params, n, t["rx"].data_ptr(), t["ry"].data_ptr(), t["rz"].data_ptr(),
                                        cs.data_ptr(), cc.data_ptr(), nbr.data_ptr(), cap, nst.data_ptr(),
                                        ncn.data_ptr(), stream=stream)
    torch.cuda.synchronize()
    ent = nbr[:total].cpu().numpy().view(np.uint32)
    st = nst.cpu().numpy().view(np.uint32)
    cn = ncn.cpu().numpy().view(np.uint32)
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
