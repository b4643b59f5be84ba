"""The reference's DQMC input and output files, for callers moving a run over.

A reference run directory holds ``afqmc.json`` (the settings), ``FCIDUMP_chol``
(the integrals, HDF5; read by :mod:`vmc_gb300.hdf5`) and the trial orbitals
``rhf.txt`` (N x N) and / or ``uhf.txt`` (N x 2N: alpha orbitals, then beta),
as executables/DQMC.cpp:74-153 and utils/input.cpp:376-384 read them, and
optionally ``spinRDM.0.0.txt`` (a spin-orbital 2-RDM from Dice whose 1-RDM
replaces the mean-field Green's function of the background subtraction,
DQMC/DQMCWalker.cpp:39-58, utils/input.cpp:1043-1091); the run writes
``samples.dat`` (DQMC/MixedEstimator.cpp:680-682: total weight and energy per
block), ``afqmc.dat`` (a header and one row per block, :351-352, :369-375,
:423-425, :530-544, :664-671) and ``blocking.tmp`` (:15-50, :684).

    wk, run = load_case("path/to/run")
    tw, te, stats = wk.run(**run)
    write_samples("samples.dat", tw, te)
"""
import json
import os

import numpy as np

from .hdf5 import read_fcidump_chol


def read_trials(directory, norb, nalpha, nbeta):
    """{"rhf": ("rhf", phi)} and / or {"uhf": ("uhf", phi_a, phi_b)} from the
    trial files present: the first nalpha columns of rhf.txt; columns [0, nalpha)
    and [N, N + nbeta) of uhf.txt."""
    out = {}
    p = os.path.join(directory, "rhf.txt")
    if os.path.exists(p):
        m = np.loadtxt(p).reshape(norb, norb)
        out["rhf"] = ("rhf", np.ascontiguousarray(m[:, :nalpha]))
    p = os.path.join(directory, "uhf.txt")
    if os.path.exists(p):
        m = np.loadtxt(p).reshape(norb, 2 * norb)
        out["uhf"] = ("uhf", np.ascontiguousarray(m[:, :nalpha]), np.ascontiguousarray(m[:, norb:norb + nbeta]))
    return out


def read_spin_rdm(path, norb, nalpha, nbeta):
    """Mean-field Green's function [2][norb][norb] from a spinRDM.0.0.txt file.

    Each line is ``a b c d value``: an element of the spin-orbital 2-RDM
    (spin orbital 2i is alpha orbital i, 2i + 1 beta).  The 1-RDM is its
    contraction, each line adding +value to (a, c) if b == d, -value to (a, d)
    if b == c, -value to (b, c) if a == d and +value to (b, d) if a == c, then
    divided by nalpha + nbeta - 1 (utils/input.cpp:1043-1091); the alpha and
    beta blocks are the even-even and odd-odd entries (DQMCWalker.cpp:50-57)."""
    ns = 2 * norb
    one = np.zeros((ns, ns))
    with open(path) as f:
        for line in f:
            w = line.split()
            if len(w) < 5:
                continue
            a, b, c, d = (int(x) for x in w[:4])
            v = float(w[4])
            if b == d:
                one[a, c] += v
            if b == c:
                one[a, d] -= v
            if a == d:
                one[b, c] -= v
            if a == c:
                one[b, d] += v
    one /= (nalpha + nbeta - 1)
    return np.stack([one[0::2, 0::2], one[1::2, 1::2]])


def ham_arrays(ints):
    """The integral dict of :func:`vmc_gb300.hdf5.read_fcidump_chol` in the form
    ``from_reference_inputs`` takes (restricted h1 / h1mod / chol, or the
    ``_up`` / ``_dn`` pairs as h1u / h1umod / cholu)."""
    d = {k: ints[k] for k in ("norb", "nalpha", "nbeta", "ecore")}
    for k in ("h1", "h1mod", "chol", "h1u", "h1umod", "cholu"):
        if k in ints:
            d[k] = ints[k]
    return d


def run_options(cfg, nprocs=1):
    """Keyword arguments of ``DQMCWalkers.run`` from the ``sampling`` block of
    afqmc.json, with the reference's defaults where a key is absent
    (utils/input.cpp:123-192; its default seed is the clock, here 0)."""
    s = cfg.get("sampling", {})
    return dict(nsteps=int(s.get("nsteps", 10)), nsweeps=int(s.get("stochasticIter", 10000)),
                ortho_steps=int(s.get("orthoSteps", 50)), seed=int(s.get("seed", 0)), nprocs=int(nprocs),
                burn_iter=int(s.get("burnIter", 0)), cholesky_threshold=float(s.get("choleskyThreshold", 0.005)))


def load_case(directory, nprocs=1, precision="ref32", device=0):
    """Walkers set up from a reference run directory, and the ``run`` options.

    nprocs: emulated MPI ranks (the handle holds nprocs x nwalk walkers).
    precision: "ref32" reproduces the reference's arithmetic (FP32 VHS), "fp64"
    and "mixed" are this library's forms."""
    from .afqmc import from_reference_inputs
    cfg = json.load(open(os.path.join(directory, "afqmc.json")))
    ints = read_fcidump_chol(os.path.join(directory, "FCIDUMP_chol"))
    trials = read_trials(directory, ints["norb"], ints["nalpha"], ints["nbeta"])
    green = None
    p = os.path.join(directory, "spinRDM.0.0.txt")
    if os.path.exists(p):  # the reference uses it whenever the file is there
        green = read_spin_rdm(p, ints["norb"], ints["nalpha"], ints["nbeta"])
    wk = from_reference_inputs(ham_arrays(ints), trials, cfg, nprocs=nprocs, precision=precision, device=device,
                               green=green)
    return wk, run_options(cfg, nprocs)


def write_samples(path, total_weights, total_energies):
    """samples.dat as the reference writes it: one "%.7e      %.10e " line per block."""
    with open(path, "w") as f:
        for w, e in zip(total_weights, total_energies):
            f.write("%.7e      %.10e \n" % (w, e))


BLOCK_SIZES = (1, 2, 5, 10, 20, 50, 70, 100, 200, 500)


def blocking(weights, energies):
    """Blocking analysis of weighted block energies (MixedEstimator.cpp:15-50).

    For each block size k <= n / 2 the series is cut into n // k groups; a
    group's energy is its weighted mean, and the error of the weighted mean of
    the groups is sqrt(sum_j W_j (E_j - mean)^2 / (V1 - V2 / V1) / (n_groups - 1))
    with V1 = sum W_j, V2 = sum W_j^2.  The stochastic error estimate is the
    first plateau: the larger of two consecutive errors once the second is
    within 5% of the first (-1 if none).  Returns (mean, error, rows) with rows
    (k, n_groups, mean, error)."""
    w = np.asarray(weights, dtype=np.float64)
    e = np.asarray(energies, dtype=np.float64)
    n = len(w)
    we = w * e
    mean_all = we.sum() / w.sum()
    rows, prev, plateau = [], 0.0, -1.0
    for k in BLOCK_SIZES:
        if k > n / 2.0:
            break
        nb = n // k
        bw = w[:nb * k].reshape(nb, k).sum(1)
        be = we[:nb * k].reshape(nb, k).sum(1) / bw
        v1, v2 = bw.sum(), (bw ** 2).sum()
        m = (bw * be).sum() / v1
        err = np.sqrt((bw * (be - m) ** 2).sum() / (v1 - v2 / v1) / (nb - 1))
        rows.append((k, nb, m, err))
        if err < 1.05 * prev and plateau < 0.0:
            plateau = max(err, prev)
        prev = err
    return mean_all, plateau, rows


def blocking_samples(total_weights, total_energies, burn_iter=0):
    """The part of a run's series that the reference analyses: the measured
    blocks after the first max(40, burnIter) (MixedEstimator.cpp:660-664, :684);
    None when the run has 40 blocks or fewer (it writes no blocking.tmp then)."""
    n = len(total_weights)
    skip = max(40, int(burn_iter))
    if n <= 40 or skip >= n:
        return None
    return np.asarray(total_weights)[skip:], np.asarray(total_energies)[skip:]


def write_blocking(path, total_weights, total_energies, burn_iter=0):
    """blocking.tmp in the reference's format; returns (mean, error) or None."""
    s = blocking_samples(total_weights, total_energies, burn_iter)
    if s is None:
        return None
    mean, err, rows = blocking(*s)
    with open(path, "w") as f:
        f.write("Number of samples: %d\n" % len(s[0]))
        f.write("Mean energy: %.8e\n" % mean)
        f.write("Block size    # of blocks        Mean                Error\n")
        for k, nb, m, e in rows:
            f.write("  %4d           %4d       %.8e       %.6e\n" % (k, nb, m, e))
        if err > 0.0:
            f.write("Stochastic error estimate: %g\n" % err)
    return mean, err


def afqmc_dat_rows(total_weights, total_energies, eshifts, walltimes, dt, nsteps, burn_iter=0):
    """The per-block rows of afqmc.dat (MixedEstimator.cpp:423-425, :530-544):
    block, imaginary time, eshift, total weight, block energy, the running
    weighted average of the blocks after equilibration ("-" during it: step dt
    < 10 or step < burnIter nsteps), wall time."""
    rows, num, den = [], 0.0, 0.0
    for b in range(len(total_weights)):
        step = b * nsteps
        tw, te = float(total_weights[b]), float(total_energies[b])
        if b == 0:
            rows.append(" %5d     %.3e       %.5e     %.5e      %.9e       %9s                %.2e \n"
                        % (0, 0.0, te, tw, te, "-", walltimes[0]))
        elif step * dt < 10.0 or step < burn_iter * nsteps:
            rows.append(" %5d     %.3e       %.5e     %.5e      %.9e         %7s                %.2e \n"
                        % (b, dt * step, eshifts[b], tw, te, "-", walltimes[b]))
        else:
            num += te * tw
            den += tw
            rows.append(" %5d     %.3e       %.5e     %.5e      %.9e        %.9e        %.2e \n"
                        % (b, dt * step, eshifts[b], tw, te, num / den, walltimes[b]))
    return rows


def write_afqmc_dat(path, total_weights, total_energies, stats, dt, nsteps, nchol, burn_iter=0, stage_s=None):
    """afqmc.dat of a run (``DQMCWalkers.run(..., block_info=True)``): the
    header (initial-state energy, Cholesky truncation), the block rows and the
    closing summary (MixedEstimator.cpp:351-352, :369-375, :423-425, :664-671).
    stage_s: optional seconds of "vhs", "prop", "fb", "energy" and "total"
    (the handle's stage timers); without it those lines carry the run's wall
    time only."""
    e_ref, delta, n_ene = stats["e_ref"], stats["delta"], stats["nchol_ene"]
    with open(path, "a") as f:
        f.write("# Initial state energy:  %.6g\n" % e_ref)
        f.write("# Number of Cholesky vectors: %d\n" % nchol)
        if n_ene < nchol:
            f.write("# Using truncated Cholesky with %d vectors for energy calculations\n" % n_ene)
            f.write("# Initial state energy with truncated Cholesky:  (%.6g,0)\n" % (e_ref - delta))
        f.write("#\n")
        f.write("# block     propTime           eshift          weight             energy          "
                "cumulative_energy          walltime\n")
        for r in afqmc_dat_rows(total_weights, total_energies, stats["eshift"], stats["walltime"], dt, nsteps,
                                burn_iter):
            f.write(r)
        st = stage_s or {}
        total = st.get("total", float(stats["walltime"][-1]))
        f.write("#\n# Total propagation time:  %g s\n" % total)
        f.write("#    VHS Time: %g s\n" % st.get("vhs", 0.0))
        f.write("#    Matmul Time: %g s\n" % st.get("prop", 0.0))
        f.write("#    Force bias Time: %g s\n" % st.get("fb", 0.0))
        f.write("# Energy evaluation time:  %g s\n#\n" % st.get("energy", 0.0))
        f.write("# Number of large deviations:  %d\n" % stats["n_large_deviations"])


def write_one_rdm(directory, rdm, cumulative_weight, rank=0):
    """The 1-RDM files of MixedEstimator.cpp:52-110: ``rdm_<rank>.dat`` for a
    spin-summed matrix (rdm of shape (1, N, N) or (N, N)), ``rdm_up_<rank>.dat``
    and ``rdm_dn_<rank>.dat`` for an up / down pair; the cumulative weight on
    the first line, then one row per line, entries separated by two spaces."""
    r = np.asarray(rdm, dtype=np.float64)
    if r.ndim == 2:
        r = r[None]
    names = ["rdm_%d.dat" % rank] if len(r) == 1 else ["rdm_up_%d.dat" % rank, "rdm_dn_%d.dat" % rank]
    paths = []
    for name, m in zip(names, r):
        p = os.path.join(directory, name)
        with open(p, "w") as f:
            f.write("%g\n" % cumulative_weight)
            for row in m:
                f.write("".join("%g  " % v for v in row) + "\n")
        paths.append(p)
    return paths
