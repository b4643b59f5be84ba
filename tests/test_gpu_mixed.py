"""Mixed-precision form (tcgen05 split-BF16 Cholesky contractions, FP32
propagator, FP64 overlap/QR/weights) against the FP64 oracle.

Tolerances are stated per result: force bias 2e-5 relative (split BF16 keeps
~16 significant bits per product, FP32 accumulation), one-step walker dets
2e-6, and the mixed-estimator energy after 100 steps with identical fields
within 0.1 mEh of the FP64 oracle; the same one-step and local-energy bounds
for a system with more than 32 occupied orbitals per spin.
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


def system(kind):
    if kind == "uhf":
        s = S.make_system(40, 7, 150, 4242, "uhf")
        na, nb, rw = 7, 6, False
    else:
        s = S.make_system(36, 6, 130, 4343, "rhf")
        na = nb = 6
        rw = True
    N = s["norb"]
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    return oh, ot, rw


def gpu(A, oh, ot, rw, W, precision):
    gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1, oh.h1mod, oh.chol)
    gt = A.RHF(gh, ot.phi[0]) if ot.kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
    return A.DQMCWalkers(gh, gt, W, rw, 0.005, precision=precision)


def start_dets(oh, ot, rw, W, seed):
    rng = np.random.default_rng(seed)
    base = O._ref_dets(oh, ot.phi, rw)
    return base[None] + 0.1 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))


@pytest.mark.parametrize("kind", ["uhf", "rhf"])
def test_force_bias_tensor_core(A, kind):
    oh, ot, rw = system(kind)
    W = 200  # several 128-row tiles, last one partial
    wk = gpu(A, oh, ot, rw, W, "mixed")
    dets = start_dets(oh, ot, rw, W, 1)
    wk.set_det(dets)
    fb = wk.force_bias()
    ref = O.force_bias(ot, O.Walkers(oh, rw, dets), oh)
    assert rel(fb, ref) < 2e-5


@pytest.mark.parametrize("kind", ["uhf", "rhf"])
def test_one_step_mixed(A, kind):
    oh, ot, rw = system(kind)
    W = 150
    wk = gpu(A, oh, ot, rw, W, "mixed")
    dets = start_dets(oh, ot, rw, W, 2)
    wk.set_det(dets)
    ow = O.Walkers(oh, rw, dets)
    ow.overlaps = O.overlap(ot, ow)
    prop = O.Propagator(oh, ot.phi, 0.005, mode="fp64")
    xi = np.random.default_rng(3).standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    wk.propagate_phaseless(xi, e0)
    O.step(ot, oh, prop, ow, xi, e0, 1e9)
    d, o, w = wk.get_det()
    assert rel(d, ow.dets) < 2e-6
    assert rel(w, ow.weights) < 2e-6


@pytest.mark.parametrize("kind", ["uhf", "rhf"])
def test_local_energy_tensor_core(A, kind):
    """Exchange + Coulomb on tcgen05 (split BF16), one-body in FP64: every
    walker's E_L within 2e-5 Eh of the FP64 oracle, also with a truncated
    Cholesky count (ncholEne)."""
    oh, ot, rw = system(kind)
    W = 45  # several walker tiles, the last one partial
    wk = gpu(A, oh, ot, rw, W, "mixed")
    dets = start_dets(oh, ot, rw, W, 5)
    wk.set_det(dets)
    ow = O.Walkers(oh, rw, dets)
    el = wk.ham_and_overlap()
    ref = O.local_energy(ot, ow, oh)
    assert np.abs(el - ref).max() < 2e-5, np.abs(el - ref).max()
    wk.set_nchol_ene(oh.nchol // 3)
    el = wk.ham_and_overlap()
    ref = O.local_energy(ot, ow, oh, oh.nchol // 3)
    assert np.abs(el - ref).max() < 2e-5, np.abs(el - ref).max()


def test_energy_error_vs_fp64_oracle(A):
    """100 steps (ortho every 5) with identical fields: mixed-estimator energy
    sum_w w E_L / sum_w w of the mixed form within 0.1 mEh of the FP64 oracle."""
    oh, ot, rw = system("uhf")
    W = 64
    wk = gpu(A, oh, ot, rw, W, "mixed")
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
    d, o, w = wk.get_det()
    el_g = wk.ham_and_overlap().real
    el_o = O.local_energy(ot, ow, oh).real
    e_g = (w * el_g).sum() / w.sum()
    e_o = (ow.weights * el_o).sum() / ow.weights.sum()
    assert abs(e_g - e_o) < 1e-4, (e_g, e_o)


def test_mixed_many_occupied_orbitals(A):
    """More than 32 occupied orbitals per spin (N = 96, 40 alpha and 38 beta):
    overlap and theta by the block Gauss-Jordan kernel, the tensor-core
    propagator in two column passes per walker, the exchange with its wide
    walker chunks, Cholesky-QR.  One step with identical fields against the
    FP64 oracle, with bounds that follow the size: dets 4e-6 per element (N =
    96 terms per product in FP32; 1.9e-6 measured); weights 5e-7 per occupied
    orbital (a weight is a ratio of determinants over all 78 columns, each
    carrying the ~1e-6 of the FP32 propagation: 2.0e-5 measured); every
    walker's E_L within 2e-6 of |E_L| (|E_L| ~ 310 Eh here; 6.9e-7 measured).
    After the QR the stored overlaps are the oracle's overlaps of the stored
    dets to 1e-10 (8e-14 measured)."""
    s = S.make_system(96, 40, 200, 4747, "uhf")
    na, nb, rw = 40, 38, False
    oh = O.Hamiltonian(96, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    W = 24
    wk = gpu(A, oh, ot, rw, W, "mixed")
    A.set_tuning(wk, prop="tensor")
    dets = start_dets(oh, ot, rw, W, 6)
    wk.set_det(dets)
    ow = O.Walkers(oh, rw, dets)
    ow.overlaps = O.overlap(ot, ow)
    prop = O.Propagator(oh, ot.phi, 0.005, mode="fp64")
    xi = np.random.default_rng(7).standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    wk.propagate_phaseless(xi, e0)
    O.step(ot, oh, prop, ow, xi, e0, 1e9)
    d, o, w = wk.get_det()
    el = wk.ham_and_overlap()
    ref = O.local_energy(ot, O.Walkers(oh, rw, d), oh)
    wk.orthogonalize()
    dq, oq, _ = wk.get_det()
    refq = O.overlap(ot, O.Walkers(oh, rw, dq))
    assert rel(d, ow.dets) < 4e-6
    assert rel(w, ow.weights) < 5e-7 * (na + nb)
    assert np.abs(el - ref).max() < 2e-6 * np.abs(ref).max(), np.abs(el - ref).max()
    assert np.abs(oq / refq - 1).max() < 1e-10
