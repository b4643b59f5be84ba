"""GPU parity of the FP64 form against the FP64 oracle, through the C ABI.

Every comparison uses the same seeded inputs on both sides; the bar is
relative error <= 1e-10 (max |gpu - oracle| / max |oracle|) for walker dets,
overlaps, weights and local energies, and <= 1e-12 for one-shot contractions.
"""
import numpy as np
import pytest

from oracle import afqmc_oracle as O
from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-10
TOL_ONE = 1e-12


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def make_case(kind):
    """(oracle ham, oracle trial, gpu ham, gpu trial, rhf_walker)."""
    if kind == "rhf_rhf":
        s = S.workload("cfg1")
        na = nb = 5
        trial_kind, rw = "rhf", True
    elif kind == "uhf_uhf":
        s = S.make_system(24, 6, 60, 777, "uhf")
        na, nb = 6, 4
        trial_kind, rw = "uhf", False
    elif kind == "rhf_uwalk":
        s = S.make_system(22, 5, 50, 778, "rhf")
        na = nb = 5
        trial_kind, rw = "rhf", False
    elif kind == "uhf_rwalk":
        s = S.make_system(22, 5, 50, 779, "uhf")
        na = nb = 5
        trial_kind, rw = "uhf", True
    else:
        raise ValueError(kind)
    N = s["norb"]
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, trial_kind, s["phi_a"][:, :na], s["phi_b"][:, :nb])
    return s, oh, ot, rw, na, nb


def gpu_objects(A, s, oh, ot, rw, nwalk, precision="fp64"):
    gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1, oh.h1mod, oh.chol)
    gt = A.RHF(gh, ot.phi[0]) if ot.kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
    wk = A.DQMCWalkers(gh, gt, nwalk, rw, 0.005, precision=precision)
    return gh, gt, wk


def random_dets(oh, ot, rw, W, seed):
    rng = np.random.default_rng(seed)
    base = O._ref_dets(oh, ot.phi, rw)
    noise = rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape)
    return base[None] + 0.15 * noise


CASES = ["rhf_rhf", "uhf_uhf", "rhf_uwalk", "uhf_rwalk"]


@pytest.mark.parametrize("kind", CASES)
def test_contractions(A, kind):
    s, oh, ot, rw, na, nb = make_case(kind)
    W = 37
    _, _, wk = gpu_objects(A, s, oh, ot, rw, W)
    dets = random_dets(oh, ot, rw, W, 1)
    wk.set_det(dets)
    ow = O.Walkers(oh, rw, dets)
    g_dets, g_ovl, g_w = wk.get_det()
    assert rel(g_dets, dets) == 0.0
    assert rel(g_ovl, O.overlap(ot, ow)) < TOL_ONE
    assert rel(wk.force_bias(), O.force_bias(ot, ow, oh)) < TOL_ONE
    assert rel(wk.ham_and_overlap(), O.local_energy(ot, ow, oh)) < TOL_ONE
    wk.set_nchol_ene(oh.nchol // 2)
    assert rel(wk.ham_and_overlap(), O.local_energy(ot, ow, oh, oh.nchol // 2)) < TOL_ONE


@pytest.mark.parametrize("kind", CASES)
def test_prop_setup(A, kind):
    s, oh, ot, rw, na, nb = make_case(kind)
    _, _, wk = gpu_objects(A, s, oh, ot, rw, 4)
    prop = O.Propagator(oh, ot.phi, 0.005, mode="fp64")
    mf, pc, ex = wk.prop_info()
    assert rel(mf, prop.mf) < 1e-13
    assert abs(pc - prop.prop_constant) / abs(prop.prop_constant) < 1e-13
    assert rel(ex[0], prop.expm[0]) < 1e-13


@pytest.mark.parametrize("kind", CASES)
def test_steps_fp64(A, kind):
    """12 steps with injected fields, ortho every 4, FP64 vs the FP64 oracle."""
    s, oh, ot, rw, na, nb = make_case(kind)
    W = 24
    _, _, wk = gpu_objects(A, s, oh, ot, rw, W)
    prop = O.Propagator(oh, ot.phi, 0.005, mode="fp64")
    dets = random_dets(oh, ot, rw, W, 2) * 0.3 + O._ref_dets(oh, ot.phi, rw)[None] * 0.7
    wk.set_det(dets)
    ow = O.Walkers(oh, rw, dets)
    ow.overlaps = O.overlap(ot, ow)
    rng = np.random.default_rng(3)
    eshift = O.hf_energy(ot, oh, ot.phi, rw).real
    for st in range(1, 13):
        xi = rng.standard_normal((W, oh.nchol))
        wk.propagate_phaseless(xi, eshift)
        O.step(ot, oh, prop, ow, xi, eshift, weight_cap=max(100.0, W / 10.0))
        if st % 4 == 0:
            wk.orthogonalize()
            O.orthogonalize(ow)
        g_dets, g_ovl, g_w = wk.get_det()
        assert rel(g_w, ow.weights) < TOL_STEP, st
        assert rel(g_ovl, ow.overlaps) < TOL_STEP, st
        assert rel(g_dets, ow.dets) < TOL_STEP, st
    assert rel(wk.ham_and_overlap(), O.local_energy(ot, ow, oh)) < TOL_STEP


def test_dead_walkers_untouched(A):
    s, oh, ot, rw, na, nb = make_case("uhf_uhf")
    W = 8
    _, _, wk = gpu_objects(A, s, oh, ot, rw, W)
    dets = random_dets(oh, ot, rw, W, 5)
    w0 = np.ones(W)
    w0[[1, 5]] = 0.0
    wk.set_det(dets, weights=w0)
    d0, o0, _ = wk.get_det()
    wk.propagate_phaseless(np.random.default_rng(0).standard_normal((W, oh.nchol)), -10.0)
    d1, o1, w1 = wk.get_det()
    for w in (1, 5):
        assert np.array_equal(d1[w], d0[w]) and o1[w] == o0[w] and w1[w] == 0.0


def test_population_control(A):
    s, oh, ot, rw, na, nb = make_case("rhf_rhf")
    W = 16
    _, _, wk = gpu_objects(A, s, oh, ot, rw, W)
    wk.set_energy_estimate(-20.0, -20.0)
    wk.propagate_phaseless(np.random.default_rng(1).standard_normal((W, oh.nchol)))
    sw, es, nc = wk.population()
    _, _, w = wk.get_det()
    assert abs(sw - w.sum()) < 1e-12 * W
    assert abs(es - (-20.0 - 0.1 * np.log(w.sum() / W) / 0.005)) < 1e-9


def test_device_rng_step_runs(A):
    s, oh, ot, rw, na, nb = make_case("uhf_uhf")
    W = 64
    _, _, wk = gpu_objects(A, s, oh, ot, rw, W)
    wk.set_energy_estimate(O.hf_energy(ot, oh, ot.phi, rw).real, O.hf_energy(ot, oh, ot.phi, rw).real)
    for _ in range(20):
        wk.propagate_phaseless(None)
    d, o, w = wk.get_det()
    assert np.all(np.isfinite(d)) and np.all(np.isfinite(w))
    assert (w > 0).sum() > W // 2
