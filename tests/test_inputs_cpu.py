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


def _slater_spin_rdm_file(path, N, na, nb, seed):
    """spinRDM.0.0.txt of a Slater determinant: Gamma_abcd = g_ac g_bd - g_ad g_bc
    over spin orbitals (2i alpha, 2i + 1 beta), one line per a < b, c < d."""
    rng = np.random.default_rng(seed)
    ca = np.linalg.qr(rng.standard_normal((N, N)))[0][:, :na]
    cb = np.linalg.qr(rng.standard_normal((N, N)))[0][:, :nb]
    g = np.zeros((2 * N, 2 * N))
    g[0::2, 0::2] = ca @ ca.T
    g[1::2, 1::2] = cb @ cb.T
    with open(path, "w") as f:
        for a in range(2 * N):
            for b in range(a + 1, 2 * N):
                for c in range(2 * N):
                    for d in range(c + 1, 2 * N):
                        v = g[a, c] * g[b, d] - g[a, d] * g[b, c]
                        if abs(v) > 1e-14:
                            f.write("%d %d %d %d %.17e\n" % (a, b, c, d, v))
    return ca @ ca.T, cb @ cb.T


def test_spin_rdm_reader(tmp_path):
    """The 1-RDM contracted from a determinant's 2-RDM is its density matrix."""
    N, na, nb = 5, 3, 2
    p = tmp_path / "spinRDM.0.0.txt"
    ga, gb = _slater_spin_rdm_file(str(p), N, na, nb, 3)
    green = inputs.read_spin_rdm(str(p), N, na, nb)
    assert green.shape == (2, N, N)
    assert np.allclose(green[0], ga, atol=1e-12) and np.allclose(green[1], gb, atol=1e-12)


def test_blocking_and_afqmc_dat(tmp_path):
    """blocking.tmp: the weighted mean, the block-size-1 error equals the
    weighted standard error written out directly, the plateau rule; afqmc.dat:
    header, one row per block, '-' in the cumulative column during
    equilibration (step dt < 10), the running weighted average after it."""
    rng = np.random.default_rng(5)
    n = 140
    tw = 80 + rng.random(n)
    te = -76.0 + 0.01 * rng.standard_normal(n)
    res = inputs.write_blocking(str(tmp_path / "blocking.tmp"), tw, te, burn_iter=0)
    assert res is not None
    w, e = tw[40:], te[40:]
    mean, err, rows = inputs.blocking(w, e)
    assert abs(mean - (w * e).sum() / w.sum()) < 1e-12
    v1, v2 = w.sum(), (w ** 2).sum()
    m1 = (w * e).sum() / v1
    se1 = np.sqrt((w * (e - m1) ** 2).sum() / (v1 - v2 / v1) / (len(w) - 1))
    assert rows[0][:2] == (1, 100) and abs(rows[0][3] - se1) < 1e-15
    assert [r[0] for r in rows] == [1, 2, 5, 10, 20, 50]
    txt = open(tmp_path / "blocking.tmp").read().splitlines()
    assert txt[0] == "Number of samples: 100" and txt[1].startswith("Mean energy: -7.")
    assert inputs.write_blocking(str(tmp_path / "none.tmp"), tw[:40], te[:40]) is None
    stats = dict(e_ref=-75.98, delta=1e-4, nchol_ene=30, n_large_deviations=2,
                 eshift=np.full(n, -76.0), walltime=np.linspace(0.1, 5.0, n))
    p = tmp_path / "afqmc.dat"
    inputs.write_afqmc_dat(str(p), tw, te, stats, dt=0.005, nsteps=50, nchol=60)
    lines = open(p).read().splitlines()
    rows = [l for l in lines if not l.startswith("#")]
    assert len(rows) == n
    assert "Using truncated Cholesky with 30 vectors" in lines[2]
    # step 40 x 50 x 0.005 = 10: blocks < 40 are equilibration
    assert rows[39].split()[5] == "-" and rows[40].split()[5] != "-"
    assert abs(float(rows[40].split()[5]) - te[40]) < 1e-8
    cum = (tw[40:42] * te[40:42]).sum() / tw[40:42].sum()
    assert abs(float(rows[41].split()[5]) - cum) < 1e-8
    assert lines[-1] == "# Number of large deviations:  2"
