"""Multi-rank population control and comb over torch.distributed (host side).

The reference couples its MPI ranks three ways (DQMC/MixedEstimator.cpp):
the sum of weights for the population-control shift (:472-475,
MPI_Allreduce), the weighted energy sum at measurement (:535-538) and the comb
reconfiguration (:559-635: MPI_Gather of weights, overlaps and dets to rank 0,
systematic resampling with one uniform zeta from rank 0's generator,
MPI_Scatter back, MPI_Bcast of the total weight).  These helpers give every
rank the walkers the single-process comb over the concatenated population
would give it, with torch.distributed (NCCL between GPUs, gloo on CPU), one
rank per GPU: the weights are all-gathered, every rank computes the same
resampling, and only the walkers that change rank move, point to point.  Walker data stay in the reference's
serial layout (``DQMCWalkers.get_det``/``set_det``).
"""
import numpy as np


def global_sum(x, dist):
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t)
    return float(t.item())


def population_shift(local_weights, e_estimate, nwalk, dt, dist):
    """eshift = eEstimate - 0.1 ln(sum_w / (nwalk P)) / dt over all ranks (MixedEstimator.cpp:472-475)."""
    P = dist.get_world_size()
    total = global_sum(np.sum(local_weights), dist)
    return e_estimate - 0.1 * np.log(total / (nwalk * P)) / dt, total


def comb_indices(weights_all, zeta, nwalk, nprocs):
    """Source walker of every slot of the new population (MixedEstimator.cpp:595-608)."""
    cum = np.cumsum(weights_all)
    tot = cum[-1]
    z = (np.arange(nprocs * nwalk) + zeta) / nwalk / nprocs
    idx = np.searchsorted(cum, z * tot, side="left")
    return np.minimum(idx, len(weights_all) - 1), tot


def comb_moves(idx, nwalk, nprocs, rank):
    """The walker moves of one rank for the comb with source indices idx (every
    rank computes the same idx from the gathered weights, so the moves need no
    negotiation).  Returns (sends, recvs): sends[q] = this rank's local walker
    indices that rank q's new walkers copy (each once), recvs[q] = the global
    indices this rank copies from rank q (each once), both sorted."""
    sends, recvs = {}, {}
    mine = idx[rank * nwalk:(rank + 1) * nwalk]
    for q in range(nprocs):
        if q == rank:
            continue
        theirs = np.unique(idx[q * nwalk:(q + 1) * nwalk])
        s = theirs[theirs // nwalk == rank] - rank * nwalk
        if len(s):
            sends[q] = s
        rv = np.unique(mine[mine // nwalk == q])
        if len(rv):
            recvs[q] = rv
    return sends, recvs


def distributed_comb(dets, overlaps, weights, zeta, dist):
    """Comb over all ranks; returns this rank's new (dets, overlaps, weights).

    dets: (nwalk, L) complex (serial layout), overlaps (nwalk,) complex,
    weights (nwalk,); zeta is used from rank 0 (broadcast).  Only the weights
    are gathered (nwalk P doubles); each walker chosen by another rank then
    travels once, point to point, as one packed message per peer (its dets
    and overlap), instead of every rank gathering every walker."""
    import torch
    P, r = dist.get_world_size(), dist.get_rank()
    nwalk = len(weights)
    z = torch.tensor([float(zeta)], dtype=torch.float64)
    dist.broadcast(z, src=0)
    w_all = [torch.zeros(nwalk, dtype=torch.float64) for _ in range(P)]
    dist.all_gather(w_all, torch.as_tensor(np.asarray(weights, np.float64)))
    w_all = torch.cat(w_all).numpy()
    idx, tot = comb_indices(w_all, float(z.item()), nwalk, P)
    d = np.ascontiguousarray(dets, np.complex128)
    o = np.ascontiguousarray(overlaps, np.complex128)
    L = d.shape[1]
    sends, recvs = comb_moves(idx, nwalk, P, r)

    def pack(rows):  # (n, 2 L + 2) doubles: the walker's dets, then its overlap
        return np.concatenate([d[rows].view(np.float64), o[rows].view(np.float64).reshape(-1, 2)], axis=1)

    reqs, bufs = [], {}
    for q, rows in sends.items():
        t = torch.from_numpy(np.ascontiguousarray(pack(rows)))
        bufs[("s", q)] = t
        reqs.append(dist.isend(t, dst=q))
    for q, src in recvs.items():
        t = torch.zeros((len(src), 2 * L + 2), dtype=torch.float64)
        bufs[("r", q)] = t
        reqs.append(dist.irecv(t, src=q))
    for q in reqs:
        q.wait()
    mine = idx[r * nwalk:(r + 1) * nwalk]
    new_d = np.empty_like(d)
    new_o = np.empty_like(o)
    for k, s in enumerate(mine):
        q = s // nwalk
        if q == r:
            new_d[k] = d[s - r * nwalk]
            new_o[k] = o[s - r * nwalk]
        else:
            row = bufs[("r", q)].numpy()[np.searchsorted(recvs[q], s)]
            new_d[k] = row[:2 * L].view(np.complex128)
            new_o[k] = row[2 * L:].view(np.complex128)[0]
    new_w = np.full(nwalk, tot / P / nwalk)
    return new_d, new_o, new_w
