"""The reference's DQMC input and output files, for callers moving a run over.

A reference run directory holds ``afqmc.json`` (the settings), ``FCIDUMP_chol``
(the integrals, HDF5; read by :mod:`vmc_gb300.hdf5`) and the trial orbitals
``rhf.txt`` (N x N) and / or ``uhf.txt`` (N x 2N: alpha orbitals, then beta),
as executables/DQMC.cpp:74-153 and utils/input.cpp:376-384 read them; the run
writes ``samples.dat`` (DQMC/MixedEstimator.cpp:680-682: total weight and
energy per block).

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
    wk = from_reference_inputs(ham_arrays(ints), trials, cfg, nprocs=nprocs, precision=precision, device=device)
    return wk, run_options(cfg, nprocs)


def write_samples(path, total_weights, total_energies):
    """samples.dat as the reference writes it: one "%.7e      %.10e " line per block."""
    with open(path, "w") as f:
        for w, e in zip(total_weights, total_energies):
            f.write("%.7e      %.10e \n" % (w, e))
