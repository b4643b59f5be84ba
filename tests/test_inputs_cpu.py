"""Reference input and output files (vmc_gb300/inputs.py, vmc_gb300/hdf5.py) on CPU.

* The trial readers take the columns the reference takes (rhf.txt: the first
  nalpha; uhf.txt: [0, nalpha) and [N, N + nbeta)), checked on written files.
* run_options maps afqmc.json's sampling block, with the reference's defaults.
* write_samples writes the reference's samples.dat line format, which reads
  back as the two columns.
* The HDF5 reader reproduces the arrays of the committed reference fixtures
  from the reference's own FCIDUMP_chol files (skipped where those files are
  not present).
"""
import json
import os

import numpy as np
import pytest

from vmc_gb300 import inputs

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout, when one is at hand (VMC_REFERENCE_ROOT); the tests that read it skip otherwise
REF = os.environ.get("VMC_REFERENCE_ROOT", "")


def test_trial_readers(tmp_path):
    N, na, nb = 6, 3, 2
    rng = np.random.default_rng(0)
    r = rng.standard_normal((N, N))
    u = rng.standard_normal((N, 2 * N))
    np.savetxt(tmp_path / "rhf.txt", r)
    np.savetxt(tmp_path / "uhf.txt", u)
    t = inputs.read_trials(str(tmp_path), N, na, nb)
    assert np.allclose(t["rhf"][1], r[:, :na])
    assert np.allclose(t["uhf"][1], u[:, :na]) and np.allclose(t["uhf"][2], u[:, N:N + nb])


def test_run_options_and_samples(tmp_path):
    cfg = {"sampling": {"nsteps": 5, "stochasticIter": 7, "orthoSteps": 5, "seed": 42, "choleskyThreshold": 1e-4}}
    o = inputs.run_options(cfg, nprocs=4)
    assert o == dict(nsteps=5, nsweeps=7, ortho_steps=5, seed=42, nprocs=4, burn_iter=0, cholesky_threshold=1e-4)
    d = inputs.run_options({})
    assert (d["nsteps"], d["nsweeps"], d["ortho_steps"], d["cholesky_threshold"]) == (10, 10000, 50, 0.005)
    tw, te = np.array([80.0, 80.3205]), np.array([-75.983984246, -76.077962434])
    p = tmp_path / "samples.dat"
    inputs.write_samples(str(p), tw, te)
    assert open(p).readline() == "8.0000000e+01      -7.5983984246e+01 \n"
    back = np.loadtxt(p)
    assert np.allclose(back[:, 0], tw, rtol=1e-7) and np.allclose(back[:, 1], te, rtol=1e-10)


@pytest.mark.parametrize("name", ["rhf_rhf", "uhf_uhf_ui"])
def test_hdf5_reader_matches_fixtures(name):
    if not REF:
        pytest.skip("VMC_REFERENCE_ROOT not set")
    d = os.path.join(REF, "tests", "DQMC", name)
    if not os.path.exists(os.path.join(d, "FCIDUMP_chol")):
        pytest.skip("reference run directory not present")
    ints = inputs.read_fcidump_chol(os.path.join(d, "FCIDUMP_chol"))
    z = np.load(os.path.join(HERE, "golden", "ref_%s.npz" % name))
    for k in ("h1", "h1mod", "chol", "h1u", "h1umod", "cholu"):
        if k in z.files:
            assert np.array_equal(ints[k], z[k]), k
    cfg = json.load(open(os.path.join(d, "afqmc.json")))
    t = inputs.read_trials(d, ints["norb"], ints["nalpha"], ints["nbeta"])
    assert set(t) == {k.replace("_txt", "") for k in z.files if k.endswith("_txt")}
    assert inputs.run_options(cfg)["nsteps"] == int(cfg["sampling"]["nsteps"])
