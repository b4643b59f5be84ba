"""The oracle's 1-RDM estimator on CPU: every walker's sample has trace equal
to the number of electrons (theta (Phi^T theta) = theta and tr(Phi^T theta) =
n per spin), and the reference's walker-by-walker running mean
(MixedEstimator.cpp:493-508) equals the plain weighted mean."""
import numpy as np

from oracle import afqmc_oracle as O
from vmc_gb300 import synthetic as S


def test_one_rdm_samples_and_running_mean():
    s = S.make_system(12, 3, 20, 41, "uhf")
    N, na, nb = 12, 3, 2
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, "uhf", s["phi_a"][:, :na], s["phi_b"][:, :nb])
    rng = np.random.default_rng(0)
    base = O._ref_dets(oh, ot.phi, False)
    d = base[None] + 0.3 * (rng.standard_normal((9,) + base.shape) + 1j * rng.standard_normal((9,) + base.shape))
    w = rng.random(9)
    w[4] = 0.0
    wk = O.Walkers(oh, False, d, weights=w)
    samp = O.one_rdm_samples(ot, wk, "r")
    assert samp.shape == (9, 1, N, N)
    assert np.allclose(np.trace(samp[:, 0], axis1=1, axis2=2), na + nb, atol=1e-10)
    acc = O.OneRDM(N, "r")
    acc.add(ot, wk)
    live = w != 0
    direct = (w[live, None, None, None] * samp[live]).sum(0) / w[live].sum()
    assert np.allclose(acc.rdm, direct, atol=1e-13) and abs(acc.cum - w.sum()) < 1e-14
    su = O.one_rdm_samples(ot, wk, "u")
    assert np.allclose(su[:, 0] + su[:, 1], samp[:, 0], atol=1e-12)
    assert np.allclose(np.trace(su[:, 1], axis1=1, axis2=2), nb, atol=1e-10)
