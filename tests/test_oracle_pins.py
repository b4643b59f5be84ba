"""Pins of the CPU oracle against the reference's own regression fixtures.

The reference's DQMC tests (tests/runDQMC.sh, tests/testEnergy.py:108-121) run
4 MPI ranks x 20 walkers for 50 blocks of 50 steps and compare samples.ref.
The oracle emulates the 4 ranks (mt19937(seed + rank), per-walker normal
streams, rank-0 comb) in the reference's own mixed precision (mode "ref") and
must reproduce every line of samples.ref to its printed precision.
"""
import os

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests import refcases

# the reference checkout, when one is at hand (the golden fixtures stand in for it otherwise)
REF_ROOT = os.environ.get("VMC_REFERENCE_ROOT", "")


@pytest.mark.parametrize("name", refcases.FIXTURES)
def test_trial_energy_kat(name):
    """E_L at the reference determinant = samples.ref line 1 (t = 0 block)."""
    c = refcases.load(name)
    e = O.hf_energy(c["trial"], c["ham"], c["ref_phi"], c["rhf_walker"])
    assert abs(e.imag) < 1e-10
    assert abs(e.real - c["samples"][0, 1]) < 1e-9


@pytest.mark.parametrize("name", refcases.FIXTURES)
def test_samples_series(name):
    """All 50 (weight, energy) blocks of samples.ref, 4 emulated ranks."""
    c = refcases.load(name)
    s = c["cfg"]["sampling"]
    tw, te, info = O.run(c["ham"], c["trial"], c["ref_phi"], c["rhf_walker"], int(s["seed"]), nprocs=4,
                         nwalk=int(s["nwalk"]), dt=float(s["dt"]), nsteps=int(s["nsteps"]),
                         nsweeps=int(s["stochasticIter"]), ortho_steps=int(s["orthoSteps"]),
                         cholesky_threshold=float(s["choleskyThreshold"]), mode="ref",
                         right_phi=c["right_phi"])
    ref = c["samples"]
    # samples.dat prints "%.7e %.10e": half a unit in the last printed digit
    assert np.abs(tw - ref[:, 0]).max() <= 0.5e-7 * 10 ** np.floor(np.log10(ref[:, 0].max())) + 1e-12
    assert np.abs(te - ref[:, 1]).max() <= 0.5e-10 * 10 ** np.floor(np.log10(np.abs(ref[:, 1]).max())) + 1e-11


def test_householder_convention():
    """Eigen's Householder QR convention: real R diagonal, beta = -sign(Re c0) ||x||."""
    rng = np.random.default_rng(0)
    a = rng.standard_normal((12, 5)) + 1j * rng.standard_normal((12, 5))
    q, rd = O.householder_qr(a)
    assert np.allclose(q.conj().T @ q, np.eye(5), atol=1e-13)
    r = q.conj().T @ a
    assert np.allclose(np.tril(r, -1), 0, atol=1e-12)
    assert np.allclose(np.diag(r), rd, atol=1e-12)
    assert np.all(np.abs(rd.imag) < 1e-14)
    assert np.sign(rd[0].real) == -np.sign(a[0, 0].real)


@pytest.mark.skipif(not REF_ROOT or not os.path.isdir(REF_ROOT), reason="VMC_REFERENCE_ROOT not set to a reference checkout")
@pytest.mark.parametrize("name", refcases.FIXTURES)
def test_fixture_npz_matches_reference(name):
    """The committed npz equals a fresh conversion of the reference's files."""
    from vmc_gb300.hdf5 import read_fcidump_chol
    d = os.path.join(REF_ROOT, "tests", "DQMC", name)
    ints = read_fcidump_chol(os.path.join(d, "FCIDUMP_chol"))
    c = refcases.load(name)
    for k in ("h1", "h1mod", "chol", "h1u", "h1umod", "cholu"):
        if k in ints:
            assert np.array_equal(ints[k], c["raw"][k])
    assert np.array_equal(np.loadtxt(os.path.join(d, "samples.ref")), c["samples"])
