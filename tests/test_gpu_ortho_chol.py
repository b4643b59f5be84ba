"""Cholesky-QR orthonormalisation of the mixed form against the Householder QR
with the reference's (Eigen's) column convention.

The two factorisations give the same Q up to the sign of each column: the
Cholesky-QR's Gram matrix, Cholesky factor and R^-1 are FP32, so its Q is
orthonormal to ~3e-7 and is checked against Householder's to 1e-6.  What keeps
the walk exact is that the stored overlap is the overlap of the returned Q:
checked against the FP64 oracle's overlap of those dets to 1e-10 (above 128
orbitals, where the mixed form's overlap comes from the FP32 copy of the
walker, the QR's factor is checked to 1e-10).  Every physical quantity is
unchanged: the local energies after either QR are within 2e-5 Eh of the FP64
oracle's energies of the walkers before it (the mixed form's local-energy
tolerance), and one further step with identical fields gives the same weights
to 1e-6 relative.
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


@pytest.mark.parametrize("kind", ["uhf", "rhf", "large"])
def test_cholesky_qr_equals_householder_up_to_column_signs(A, kind):
    """"large": N = 300 with 45 + 44 electrons, whose spin block does not fit
    shared memory as FP32 pairs: the variant that keeps it in L2."""
    if kind == "uhf":
        s = S.make_system(40, 7, 150, 4242, "uhf")
        na, nb, rw = 7, 6, False
    elif kind == "large":
        s = S.make_system(300, 45, 40, 4141, "uhf")
        na, nb, rw = 45, 44, False
    else:
        s = S.make_system(36, 6, 130, 4343, "rhf")
        na = nb = 6
        rw = True
    N = s["norb"]
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    W = 12 if kind == "large" else 48
    rng = np.random.default_rng(5)
    base = O._ref_dets(oh, ot.phi, rw)
    dets = base[None] + 0.1 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))
    el_ref = O.local_energy(ot, O.Walkers(oh, rw, dets), oh).real
    out = {}
    for qr in ("householder", "cholesky"):
        gh = A.Hamiltonian(N, na, nb, oh.ecore, oh.h1, oh.h1mod, oh.chol)
        gt = A.RHF(gh, ot.phi[0]) if ot.kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
        wk = A.DQMCWalkers(gh, gt, W, rw, 0.005, precision="mixed")
        A.set_tuning(wk, qr=qr)
        wk.set_det(dets)
        wk.orthogonalize()
        d, o, w = wk.get_det()
        el = wk.ham_and_overlap().real
        xi = np.random.default_rng(9).standard_normal((W, oh.nchol))
        e0 = O.hf_energy(ot, oh, ot.phi, rw).real
        wk.propagate_phaseless(xi, e0)
        _, _, w1 = wk.get_det()
        out[qr] = (d, o, el, w1)
    dh, oh_, elh, w1h = out["householder"]
    dc, oc, elc, w1c = out["cholesky"]
    qh, qc = dh, dc  # (W, N, columns): alpha columns, then beta for the unrestricted walker
    dq, dg = 0.0, 0.0
    for w in range(W):
        sgn = np.sign(np.einsum("pj,pj->j", qh[w].conj(), qc[w]).real)
        assert np.all(np.abs(sgn) == 1)
        dq = max(dq, np.abs(qc[w] - qh[w] * sgn[None]).max())
        # orthonormal columns per spin block
        blocks = [(0, na)] if rw else [(0, na), (na, na + nb)]
        for a, b in blocks:
            g = qc[w][:, a:b].conj().T @ qc[w][:, a:b]
            dg = max(dg, np.abs(g - np.eye(b - a)).max())
    print("cholesky-qr: |Q - Q_householder| %.2e, |Q^H Q - I| %.2e" % (dq, dg))
    assert dq < 1e-6 and dg < 1e-6
    ref_o = O.overlap(ot, O.Walkers(oh, rw, dc))
    ref_h = O.overlap(ot, O.Walkers(oh, rw, dh))
    if N > 128:
        # above 128 orbitals the mixed form's overlap is that of the FP32 copy
        # of the walker (~1e-7 from the FP64 dets' own); what the QR must keep
        # is the factor: both factorisations multiply the stored overlap by
        # det R^-1 exactly, so the two stay in the ratio of the FP64 overlaps
        assert np.abs(oc / ref_o - 1).max() < 1e-5
        assert np.abs((oc / oh_) / (ref_o / ref_h) - 1).max() < 1e-10
    else:
        assert np.abs(oc / ref_o - 1).max() < 1e-10
        assert np.abs(oh_ / ref_h - 1).max() < 1e-10
    tol_el = max(2e-5, 2e-7 * np.abs(el_ref).max())  # FP32-grade exchange: relative for large |E_L|
    if N > 128:
        # 45 + 44 electrons in 300 orbitals: the mixed form's local energy is
        # within 1e-6 of |E_L| of the FP64 value, before and after either QR
        tol_el = 1e-6 * np.abs(el_ref).max()
        assert np.abs(elc - elh).max() < tol_el
    assert np.abs(elh - el_ref).max() < tol_el
    assert np.abs(elc - el_ref).max() < tol_el
    assert np.abs(w1c - w1h).max() <= 1e-6 * np.abs(w1h).max()
