"""Multi-rank population control and comb over torch.distributed (host side).

The reference couples its MPI ranks three ways (DQMC/MixedEstimator.cpp):
the sum of weights for the population-control shift (:472-475,
MPI_Allreduce), the weighted energy sum at measurement (:535-538) and the comb
reconfiguration (:559-635: MPI_Gather of weights, overlaps and dets to rank 0,
systematic resampling with one uniform zeta from rank 0's generator,
MPI_Scatter back, MPI_Bcast of the total weight).  These helpers do the same
with torch.distributed collectives (NCCL between GPUs, gloo on CPU), one rank
per GPU; every rank ends with the walkers the single-process comb over the
concatenated population would give it.  Walker data stay in the reference's
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


def distributed_comb(dets, overlaps, weights, zeta, dist):
    """Comb over all ranks; returns this rank's new (dets, overlaps, weights).

    dets: (nwalk, L) complex (serial layout), overlaps (nwalk,) complex,
    weights (nwalk,); zeta is used from rank 0 (broadcast)."""
    import torch
    P, r = dist.get_world_size(), dist.get_rank()
    nwalk = len(weights)
    z = torch.tensor([float(zeta)], dtype=torch.float64)
    dist.broadcast(z, src=0)
    w_all = [torch.zeros(nwalk, dtype=torch.float64) for _ in range(P)]
    dist.all_gather(w_all, torch.as_tensor(np.asarray(weights, np.float64)))
    w_all = torch.cat(w_all).numpy()
    idx, tot = comb_indices(w_all, float(z.item()), nwalk, P)
    # every rank contributes its walkers; the receivers pick their sources
    d = torch.view_as_real(torch.as_tensor(np.ascontiguousarray(dets, np.complex128)))
    o = torch.view_as_real(torch.as_tensor(np.ascontiguousarray(overlaps, np.complex128)))
    d_all = [torch.zeros_like(d) for _ in range(P)]
    o_all = [torch.zeros_like(o) for _ in range(P)]
    dist.all_gather(d_all, d)
    dist.all_gather(o_all, o)
    d_all = torch.view_as_complex(torch.cat(d_all)).numpy()
    o_all = torch.view_as_complex(torch.cat(o_all)).numpy()
    mine = idx[r * nwalk:(r + 1) * nwalk]
    new_w = np.full(nwalk, tot / P / nwalk)
    return d_all[mine], o_all[mine], new_w
