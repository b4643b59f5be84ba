"""Seeded synthetic Hamiltonians and mean-field trials for the AFQMC workloads.

The reference's own inputs come from pyscf (scripts/QMCUtils.py); there is no
pyscf here and the benchmark shapes (norb 20...400) have no reference data, so
these generators stand in for them with the value distributions the workload
definitions give:

* Cholesky vectors L_g: real symmetric N x N, upper-triangle entries
  N(0, sigma_g^2 / N) mirrored, sigma_g = 0.5 exp(-g/20).  The 1/N in the
  variance keeps sum_g ||L_g||_2^2 near 10 at every N, the value of the
  reference's H2O fixture (tests/DQMC/rhf_rhf: 10.4); without it the two-body
  operator grows with N (x18 at N=20, x370 at N=400) and every walker's
  importance weight leaves [1e-3, 100] in the first step, killing the population;
* h1: symmetric, off-diagonal N(0, 0.1^2), diagonal -2 + 0.2 i + N(0, 0.1^2);
* h1Mod = h1 - 1/2 sum_g L_g L_g (scripts/QMCUtils.py:537-538), ecore = 0;
* trial: lowest-n eigenvectors of the self-consistent Fock matrix
  F_s = h1 + sum_g [tr(P L_g) L_g - L_g P_s L_g] (RHF: P = 2 P_a), iterated from
  the h1 guess; the UHF trial is one spin-broken diagonalisation of that Fock
  matrix plus / minus a seeded symmetric perturbation.

All randomness comes from numpy's ``MT19937`` bit generator seeded with
``20261203 + index`` for the numbered workloads.
"""
import numpy as np

WORKLOADS = {
    # name: (norb, nocc, nchol, walkers, trial)
    "cfg1": dict(norb=20, nocc=5, nchol=80, walkers=64, trial="rhf", index=1),
    "cfg2": dict(norb=120, nocc=20, nchol=600, walkers=2048, trial="uhf", index=2),
    "cfg4": dict(norb=200, nocc=30, nchol=1000, walkers=4096, trial="uhf", index=4),
    "cfg5": dict(norb=400, nocc=60, nchol=2400, walkers=1024, trial="uhf", index=5),
}


def _rng(seed):
    return np.random.Generator(np.random.MT19937(seed))


def make_integrals(norb, nchol, seed):
    """(h1, h1mod, chol[g, p, q], ecore) with the distributions above."""
    rng = _rng(seed)
    N, G = norb, nchol
    sig = 0.5 * np.exp(-np.arange(G) / 20.0) / np.sqrt(N)
    iu = np.triu_indices(N)
    chol = np.zeros((G, N, N))
    vals = rng.standard_normal((G, len(iu[0]))) * sig[:, None]
    chol[:, iu[0], iu[1]] = vals
    chol[:, iu[1], iu[0]] = vals
    h1 = np.zeros((N, N))
    off = rng.standard_normal(len(iu[0])) * 0.1
    h1[iu] = off
    h1[iu[1], iu[0]] = off
    h1[np.diag_indices(N)] = -2.0 + 0.2 * np.arange(N) + rng.standard_normal(N) * 0.1
    lt = chol.transpose(1, 0, 2).reshape(N, G * N)    # [p, (g, r)]
    h1mod = h1 - 0.5 * (lt @ chol.reshape(G * N, N))
    return h1, h1mod, chol, 0.0


def _fock(h1, chol, c_tot, c_s):
    """F_s = h1 + sum_g [tr(P L_g) L_g - L_g P_s L_g] with P_s = c_s c_s^T.

    c_tot lists the occupied blocks whose densities add up to P.  Written as two
    GEMMs over (g, orbital) so it stays fast for nchol in the thousands."""
    G, N, _ = chol.shape
    lf = chol.reshape(G, N * N)
    ptot = sum(c @ c.T for c in c_tot)
    j = lf @ ptot.ravel()
    fock = h1 + (j @ lf).reshape(N, N)
    lc = chol @ c_s                                   # (G, N, n)
    lc2 = lc.transpose(1, 0, 2).reshape(N, -1)        # (N, G n)
    return fock - lc2 @ lc2.T


def scf(h1, chol, nalpha, nbeta, uhf=False, seed=0, iters=30, damp=0.5):
    """Mean-field trial orbitals: returns (phi_a, phi_b).

    Closed-shell Roothaan iterations with Fock damping from the h1 guess.  For
    the UHF trial, one final spin-broken Fock diagonalisation: F + x for alpha
    and F - x for beta, x a seeded symmetric perturbation of scale 0.05."""
    c = np.linalg.eigh(h1)[1][:, :nalpha]
    f_old = None
    for _ in range(iters):
        f = _fock(h1, chol, [c, c], c)
        if f_old is not None:
            f = damp * f_old + (1 - damp) * f
        f_old = f
        c = np.linalg.eigh(f)[1][:, :nalpha]
    if not uhf:
        return c, c[:, :nbeta]
    N = h1.shape[0]
    rng = _rng(seed + 7919)
    x = rng.standard_normal((N, N)) * 0.05
    x = (x + x.T) / 2
    ca = np.linalg.eigh(f + x)[1][:, :nalpha]
    cb = np.linalg.eigh(f - x)[1][:, :nbeta]
    return ca, cb


def make_system(norb, nocc, nchol, seed, trial="uhf"):
    """A synthetic system: dict with the Hamiltonian arrays and trial orbitals."""
    h1, h1mod, chol, ecore = make_integrals(norb, nchol, seed)
    pa, pb = scf(h1, chol, nocc, nocc, uhf=(trial == "uhf"), seed=seed)
    return dict(norb=norb, nalpha=nocc, nbeta=nocc, nchol=nchol, ecore=ecore,
                h1=h1, h1mod=h1mod, chol=chol, phi_a=pa, phi_b=pb, trial=trial)


def workload(name):
    """System of one of the numbered workloads (see WORKLOADS)."""
    w = WORKLOADS[name]
    sysd = make_system(w["norb"], w["nocc"], w["nchol"], 20261203 + w["index"], w["trial"])
    sysd["walkers"] = w["walkers"]
    return sysd


def multi_system_batch(nsys=16, walkers=256, seed=20261203 + 3, nmin=40, nmax=200):
    """Uneven multi-system batch: norb ~ U[nmin, nmax], nocc = round(norb/6), nchol = 5 norb."""
    rng = _rng(seed)
    norbs = rng.integers(nmin, nmax + 1, size=nsys)
    out = []
    for i, n in enumerate(norbs):
        n = int(n)
        s = make_system(n, int(round(n / 6)), 5 * n, seed + 1000 * (i + 1), "uhf")
        s["walkers"] = walkers
        out.append(s)
    return out
