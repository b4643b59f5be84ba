"""Failure detection on the GPU, with every failure made on the host side.

* A walker whose determinant holds a NaN or an Inf (written by the host) gets a
  non-finite importance function at its next step and is given weight 0, as the
  reference's phaseless projection does (DQMC/DQMCWalker.cpp:496-502); the
  other walkers' results equal those of a run without the bad entries, and the
  control-variate estimate stays finite with the dead walker in the batch.
* A live walker with a non-finite local energy at a device block's measurement
  (the reference stops the run there, DQMC/MixedEstimator.cpp:513-522) is
  reported as AFQMC_ERR_NAN by the next call that reads device state; the
  handle stays usable.
* A bounded device wait that nothing completes gives up after ~2 s, and the
  call returns AFQMC_ERR_TIMEOUT with the handle still usable.
No test here faults, traps or hangs the GPU.
"""
import numpy as np
import pytest

from oracle import afqmc_oracle as O
from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

AFQMC_ERR_NAN = 3
AFQMC_ERR_TIMEOUT = 4


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def small_system():
    s = S.make_system(28, 5, 84, 6161, "uhf")
    N, n = 28, 5
    oh = O.Hamiltonian(N, n, n, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, "uhf", s["phi_a"], s["phi_b"])
    return s, oh, ot


def handle(A, s, W, precision):
    N, n = s["norb"], s["nalpha"]
    gh = A.Hamiltonian(N, n, n, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    gt = A.UHF(gh, s["phi_a"], s["phi_b"])
    return A.DQMCWalkers(gh, gt, W, False, 0.005, precision=precision, seed=5)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_finite_walker_dies(A, precision):
    s, oh, ot = small_system()
    W = 16
    rng = np.random.default_rng(1)
    base = O._ref_dets(oh, ot.phi, False)
    dets = base[None] + 0.05 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))
    bad = dets.copy()
    bad[3, 4, 2] = np.nan
    bad[7, 0, 6] = np.inf
    xi = rng.standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, False).real
    out = []
    for d in (dets, bad):
        wk = handle(A, s, W, precision)
        wk.set_det(d)
        wk.propagate_phaseless(xi, e0)
        out.append(wk.get_det())
        if d is bad:
            sw, _, _ = wk.population()
            assert np.isfinite(sw)
            wk.sync()
        wk.close()
    (d0, o0, w0), (d1, o1, w1) = out
    assert w1[3] == 0.0 and w1[7] == 0.0
    keep = np.ones(W, bool)
    keep[[3, 7]] = False
    assert np.all(np.isfinite(w1)) and np.all(w1[keep] > 0)
    assert np.array_equal(w1[keep], w0[keep])
    assert np.array_equal(d1[keep], d0[keep])


def test_control_variate_with_a_dead_non_finite_walker(A):
    """The estimate skips dead walkers: one with a NaN determinant (weight 0
    after its step) leaves every reported estimate finite."""
    from vmc_gb300.cv import ControlVariate
    s, oh, ot = small_system()
    W = 64
    wk = handle(A, s, W, "mixed")
    e0 = wk.ham_and_overlap().real.mean()
    wk.set_energy_estimate(e0, e0)
    cv = ControlVariate(wk, hidden=64, den=8, seed=2)
    for st in range(12):
        wk.propagate_phaseless(None)
        cv.collect()
    cv.train(epochs=2, batch=64, lr=1e-3)
    d, o, w = wk.get_det()
    d[5, 3, 1] = np.nan
    wk.set_det(d, weights=w)
    wk.propagate_phaseless(None)
    _, _, w2 = wk.get_det()
    assert w2[5] == 0.0
    cv.measure(tag=1, slot=0)
    r = cv.results(1)[0]
    assert np.all(np.isfinite(r)), r
    wk.close()


def test_non_finite_local_energy_reported(A):
    s, oh, ot = small_system()
    W = 8
    wk = handle(A, s, W, "fp64")
    base = O._ref_dets(oh, ot.phi, False)
    d = np.repeat(base[None], W, axis=0)
    d[2, 1, 1] = np.nan
    wk.set_det(d, weights=np.ones(W))  # walker 2 live, with a non-finite E_L
    e0 = O.hf_energy(ot, oh, ot.phi, False).real
    wk.block_setup(nsteps=1, e_est=e0)
    wk.block_end(comb=False)           # enqueued; the error is recorded on the device
    with pytest.raises(A.AfqmcError) as ei:
        wk.sync()
    assert ei.value.code == AFQMC_ERR_NAN
    # the error was taken; the handle works on
    d[2] = base
    wk.set_det(d)
    wk.propagate_phaseless(np.zeros((W, oh.nchol)), e0)
    wk.sync()
    wk.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bounded_wait_times_out(A, precision):
    s, oh, ot = small_system()
    W = 8
    wk = handle(A, s, W, precision)
    rc, msg = wk.check_wait_timeout()
    assert rc == AFQMC_ERR_TIMEOUT, (rc, msg)
    assert "timed out" in msg
    # the context and the handle are still usable
    e0 = O.hf_energy(ot, oh, ot.phi, False).real
    wk.propagate_phaseless(np.zeros((W, oh.nchol)), e0)
    wk.sync()
    _, _, w = wk.get_det()
    assert np.all(np.isfinite(w)) and np.all(w > 0)
    wk.close()
