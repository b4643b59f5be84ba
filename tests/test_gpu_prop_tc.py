"""Tensor-core propagator (tcgen05, split BF16 in three MMA passes, FP32
accumulation in TMEM) against the FP32 shared-memory propagator and the FP64
oracle.

Tolerances: one step of walker determinants and weights within 5e-5 relative
of the FP64 oracle and of the FP32 propagator (each of the seven products per
step drops only the lo.lo term, 2^-16 of the product); the mixed-estimator
energy after 100 steps with identical fields within 0.1 mEh of the oracle.
Cases cover RHF and UHF walkers, more columns than one pass holds (two
column passes of different widths) and N = 128 (every TMEM lane in use).
"""
import numpy as np
import pytest

from oracle import afqmc_oracle as O
from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


SYSTEMS = {
    "uhf": (40, 7, 6, 150, 4242, "uhf", False),
    "rhf": (36, 6, 6, 130, 4343, "rhf", True),
    "wide": (100, 30, 28, 260, 4444, "uhf", False),   # 58 columns: passes of 40 and 18
    "n128": (128, 10, 10, 300, 4545, "uhf", False),
}


def system(name):
    N, na, nb, G, seed, kind, rw = SYSTEMS[name]
    s = S.make_system(N, max(na, nb), G, seed, kind)
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    return oh, ot, rw


def walkers(A, oh, ot, rw, W, prop):
    gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1, oh.h1mod, oh.chol)
    gt = A.RHF(gh, ot.phi[0]) if ot.kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
    wk = A.DQMCWalkers(gh, gt, W, rw, 0.005, precision="mixed")
    A.set_tuning(wk, prop=prop)
    return wk


def start_dets(oh, ot, rw, W, seed):
    rng = np.random.default_rng(seed)
    base = O._ref_dets(oh, ot.phi, rw)
    return base[None] + 0.1 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))


@pytest.mark.parametrize("name", ["uhf", "rhf", "wide", "n128"])
def test_one_step_tensor_propagator(A, name):
    oh, ot, rw = system(name)
    W = 96
    dets = start_dets(oh, ot, rw, W, 2)
    xi = np.random.default_rng(3).standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    out = {}
    for prop in ("tensor", "smem"):
        wk = walkers(A, oh, ot, rw, W, prop)
        wk.set_det(dets)
        wk.propagate_phaseless(xi, e0)
        out[prop] = wk.get_det()
    ow = O.Walkers(oh, rw, dets)
    ow.overlaps = O.overlap(ot, ow)
    O.step(ot, oh, O.Propagator(oh, ot.phi, 0.005, mode="fp64"), ow, xi, e0, 1e9)
    d, _, w = out["tensor"]
    assert rel(d, ow.dets) < 5e-5, rel(d, ow.dets)
    assert rel(w, ow.weights) < 5e-5, rel(w, ow.weights)
    assert rel(d, out["smem"][0]) < 5e-5
    assert rel(w, out["smem"][2]) < 5e-5


def test_dead_walkers_untouched(A):
    oh, ot, rw = system("uhf")
    W = 64
    wk = walkers(A, oh, ot, rw, W, "tensor")
    dets = start_dets(oh, ot, rw, W, 7)
    wts = np.ones(W)
    wts[::3] = 0.0
    wk.set_det(dets, weights=wts)
    d0, _, _ = wk.get_det()
    wk.propagate_phaseless(np.random.default_rng(8).standard_normal((W, oh.nchol)),
                           O.hf_energy(ot, oh, ot.phi, rw).real)
    d, _, w = wk.get_det()
    assert np.array_equal(d[::3], d0[::3])
    assert np.all(w[::3] == 0.0)
    assert not np.array_equal(d[1::3], d0[1::3])


def test_energy_error_tensor_propagator(A):
    """100 steps (ortho every 5) with identical fields: the mixed form with the
    tensor-core propagator within 0.1 mEh of the FP64 oracle."""
    oh, ot, rw = system("uhf")
    W = 64
    wk = walkers(A, oh, ot, rw, W, "tensor")
    dets = np.repeat(O._ref_dets(oh, ot.phi, rw)[None], W, axis=0)
    wk.set_det(dets)
    ow = O.Walkers(oh, rw, dets)
    ow.overlaps = O.overlap(ot, ow)
    prop = O.Propagator(oh, ot.phi, 0.005, mode="fp64")
    rng = np.random.default_rng(4)
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    es = e0
    for st in range(1, 101):
        xi = rng.standard_normal((W, oh.nchol))
        wk.propagate_phaseless(xi, es)
        O.step(ot, oh, prop, ow, xi, es, 1e9)
        es = e0 - 0.1 * np.log(ow.weights.sum() / W) / 0.005
        if st % 5 == 0:
            wk.orthogonalize()
            O.orthogonalize(ow)
    _, _, w = wk.get_det()
    el_g = wk.ham_and_overlap().real
    el_o = O.local_energy(ot, ow, oh).real
    e_g = (w * el_g).sum() / w.sum()
    e_o = (ow.weights * el_o).sum() / ow.weights.sum()
    assert abs(e_g - e_o) < 1e-4, (e_g, e_o)


def test_tensor_choice_limits(A):
    """The MN-major variant covers N <= 128 and the tensor-core choice N <= 512
    (streamed tiles above 128); beyond them the choice is refused."""
    for N, tensor_ok in ((136, True), (520, False)):
        s = S.make_system(N, 4, 40, 4646, "uhf")
        gh = A.Hamiltonian(N, 4, 4, s["ecore"], s["h1"], s["h1mod"], s["chol"])
        gt = A.UHF(gh, s["phi_a"][:, :4], s["phi_b"][:, :4])
        wk = A.DQMCWalkers(gh, gt, 8, False, 0.005, precision="mixed")
        with pytest.raises(Exception):
            A.set_tuning(wk, prop="tensor_mn")
        if tensor_ok:
            A.set_tuning(wk, prop="tensor")
        else:
            with pytest.raises(Exception):
                A.set_tuning(wk, prop="tensor")
        wk.close()


@pytest.mark.parametrize("name", ["uhf", "rhf", "wide", "n128"])
def test_mn_major_walker_operand_equals_k_major(A, name):
    """The propagator with the walker operand stored MN-major (16-byte chunk
    stores) forms the same BF16 splits, issues the same MMAs in the same order
    and sums the same FP32 values as the K-major one: the steps are equal."""
    oh, ot, rw = system(name)
    W = 96
    dets = start_dets(oh, ot, rw, W, 12)
    w0 = np.ones(W)
    w0[::5] = 0.0
    xi = np.random.default_rng(13).standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    out = {}
    for prop in ("tensor", "tensor_mn"):
        wk = walkers(A, oh, ot, rw, W, prop)
        wk.set_det(dets, weights=w0)
        for _ in range(3):
            wk.propagate_phaseless(xi, e0)
        out[prop] = wk.get_det()
        wk.close()
    (d3, o3, w3), (d4, o4, w4) = out["tensor"], out["tensor_mn"]
    assert rel(d4, d3) <= 1e-12 and rel(w4, w3) <= 1e-12, (rel(d4, d3), rel(w4, w3))
    assert np.array_equal(d4[::5], dets[::5])
