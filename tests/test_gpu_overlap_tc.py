"""Tensor-core overlap matrices (exact BF16 slices, the Ozaki scheme) against
the FP64 overlap and the FP64 oracle.

* Overlaps of perturbed walkers (det of M = Phi^T psi per channel) within
  1e-11 relative of the oracle and of the FP64-M kernel, for the RHF and UHF
  walkers, N <= 64 (one 64-wide K panel per slice), N = 100 and N = 128: FP64
  walkers (integer slicing of the bits) and, after one step, walkers of FP32
  numbers (FP32 slicing).
* One step with identical fields: weights within 1e-9 relative of the FP64-M
  kernel (the same FP32 propagation either way).
* 100 steps with the mixed form's fastest kernels (tensor-core propagator,
  tensor-core M, Cholesky-QR): mixed-estimator energy within 0.1 mEh of the
  FP64 oracle.
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


SYSTEMS = {
    "uhf": (40, 7, 6, 150, 4242, "uhf", False),
    "rhf": (36, 6, 6, 130, 4343, "rhf", True),
    "n100": (100, 16, 15, 260, 4444, "uhf", False),
    "n128": (128, 10, 10, 300, 4545, "uhf", False),
}


def system(name):
    N, na, nb, G, seed, kind, rw = SYSTEMS[name]
    s = S.make_system(N, max(na, nb), G, seed, kind)
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    return oh, ot, rw


def walkers(A, oh, ot, rw, W, **tuning):
    gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1, oh.h1mod, oh.chol)
    gt = A.RHF(gh, ot.phi[0]) if ot.kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
    wk = A.DQMCWalkers(gh, gt, W, rw, 0.005, precision="mixed")
    A.set_tuning(wk, **tuning)
    return wk


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.mark.parametrize("name", ["uhf", "rhf", "n100", "n128"])
def test_overlap_tc_matches_fp64(A, name):
    oh, ot, rw = system(name)
    W = 80
    rng = np.random.default_rng(3)
    base = O._ref_dets(oh, ot.phi, rw)
    dets = base[None] + 0.2 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))
    xi = rng.standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    out = {}
    for ovl in (3, 1):
        wk = walkers(A, oh, ot, rw, W, ovl=ovl)
        wk.set_det(dets)
        _, o, _ = wk.get_det()
        fb = wk.force_bias()
        wk.propagate_phaseless(xi, e0)
        d1, o1_, w1 = wk.get_det()
        if ovl == 3:
            # after a step the walkers hold FP32 numbers: the FP32 slicing path
            ref1 = O.overlap(ot, O.Walkers(oh, rw, d1))
            assert np.abs(o1_ / ref1 - 1).max() < 1e-11, np.abs(o1_ / ref1 - 1).max()
        out[ovl] = (o, fb, w1)
    ref = O.overlap(ot, O.Walkers(oh, rw, dets))
    o3, fb3, w3 = out[3]
    o1, fb1, w1 = out[1]
    assert np.abs(o3 / ref - 1).max() < 1e-11, np.abs(o3 / ref - 1).max()
    assert np.abs(o3 / o1 - 1).max() < 1e-11
    assert rel(fb3, fb1) < 1e-6
    assert np.abs(w3 - w1).max() <= 1e-9 * np.abs(w1).max()


def test_energy_error_fast_kernels(A):
    oh, ot, rw = system("uhf")
    W = 64
    wk = walkers(A, oh, ot, rw, W, prop="tensor", ovl=3, qr="cholesky")
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
