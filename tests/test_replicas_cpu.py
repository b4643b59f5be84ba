"""Multi-rank coupling of the walker population with world_size 2 (gloo, CPU).

Each rank holds its own walkers; the population shift, the measurement sum
and the comb must equal those of one process holding the concatenated
population (the reference's MPI semantics, DQMC/MixedEstimator.cpp:472-475,
:535-538, :559-635).
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from vmc_gb300 import ranks
        rng = np.random.default_rng(100 + rank)
        nwalk, L = 16, 6
        dets = rng.standard_normal((nwalk, L)) + 1j * rng.standard_normal((nwalk, L))
        ovl = rng.standard_normal(nwalk) + 1j * rng.standard_normal(nwalk)
        w = rng.random(nwalk) * 2
        w[3] = 0.0
        es, tot = ranks.population_shift(w, -10.0, nwalk, 0.005, dist)
        nd, no, nw = ranks.distributed_comb(dets, ovl, w, 0.37 if rank == 0 else 0.99, dist)
        q.put((rank, dets, ovl, w, es, tot, nd, no, nw))
    finally:
        dist.destroy_process_group()


def test_two_ranks_match_single_process():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in range(2)], key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from vmc_gb300 import ranks
    dets = np.concatenate([r[1] for r in res])
    ovl = np.concatenate([r[2] for r in res])
    w = np.concatenate([r[3] for r in res])
    nwalk = len(res[0][3])
    tot = w.sum()
    es = -10.0 - 0.1 * np.log(tot / (nwalk * 2)) / 0.005
    for r in res:
        assert abs(r[4] - es) < 1e-12 and abs(r[5] - tot) < 1e-12
    idx, ctot = ranks.comb_indices(w, 0.37, nwalk, 2)  # zeta of rank 0
    for r in res:
        mine = idx[r[0] * nwalk:(r[0] + 1) * nwalk]
        assert np.array_equal(r[6], dets[mine])
        assert np.array_equal(r[7], ovl[mine])
        assert np.allclose(r[8], ctot / 2 / nwalk)
    # a zero-weight walker is never selected
    assert 3 not in idx
    # the moves: each rank receives exactly the foreign sources of its new
    # walkers, once each, and sends what the other rank receives from it
    s0, r0 = ranks.comb_moves(idx, nwalk, 2, 0)
    s1, r1 = ranks.comb_moves(idx, nwalk, 2, 1)
    assert np.array_equal(s0.get(1, []), r1.get(0, np.array([], int)) - 0 * nwalk)
    assert np.array_equal(s1.get(0, []), r0.get(1, np.array([], int)) - nwalk)
    assert sum(len(v) for v in r0.values()) == len(np.unique(idx[:nwalk][idx[:nwalk] >= nwalk]))
