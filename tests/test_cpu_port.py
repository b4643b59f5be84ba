"""The C++ restatement of the walker step (oracle/cpu_step.cpp, the CPU
baseline) against the numpy oracle, on CPU.

FP64 VHS: one step (force bias, fields, VHS, propagator, overlap, importance
function, weight) and the local energy equal the numpy oracle's FP64 mode to
1e-12 relative; after the QR the columns are orthonormal and the stored
overlaps are the overlaps of the stored dets.  The reference's FP32 VHS (the
timed configuration): the same step within 1e-5 relative of the oracle's "ref"
mode (the FP32 sums run in a different order).  Both trial/walker pairings of
the benchmarks: UHF trial with UHF walkers, RHF trial with restricted walkers."""
import numpy as np
import pytest

from oracle import afqmc_oracle as O
from oracle import cpu_port as C
from vmc_gb300 import synthetic as S


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def setup(kind, mode):
    if kind == "uhf":
        s = S.make_system(18, 4, 40, 901, "uhf")
        na, nb, rw = 4, 3, False
    else:
        s = S.make_system(16, 4, 36, 902, "rhf")
        na = nb = 4
        rw = True
    N = s["norb"]
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    prop = O.Propagator(oh, ot.phi, 0.01, mode=mode)
    return oh, ot, prop, rw


@pytest.mark.parametrize("kind", ["uhf", "rhf"])
@pytest.mark.parametrize("mode", ["fp64", "ref"])
def test_cpu_port_step_matches_oracle(kind, mode):
    oh, ot, prop, rw = setup(kind, mode)
    W = 11
    rng = np.random.default_rng(3)
    base = O._ref_dets(oh, ot.phi, rw)
    dets = base[None] + 0.1 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))
    w0 = np.ones(W)
    w0[4] = 0.0
    xi = rng.standard_normal((W, oh.nchol))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    cw = C.CpuWalkers(oh, ot, prop, rw, W, nthreads=3)
    cw.set_walkers(dets, weights=w0)
    ow = O.Walkers(oh, rw, dets.copy(), weights=w0.copy())
    ow.overlaps = O.overlap(ot, ow)
    _, o0, _ = cw.get_walkers()
    assert rel(o0, ow.overlaps) < 1e-12
    sw = cw.step(xi, e0, 100.0)
    O.step(ot, oh, prop, ow, xi, e0, 100.0)
    d, o, w = cw.get_walkers()
    tol = 1e-12 if mode == "fp64" else 1e-5
    assert abs(sw - ow.weights.sum()) <= tol * ow.weights.sum()
    assert rel(d, ow.dets) < tol and rel(o, ow.overlaps) < tol and rel(w, ow.weights) < tol
    assert w[4] == 0.0 and np.array_equal(d[4], dets[4])
    el = cw.local_energy()
    live = w != 0
    ref = O.local_energy(ot, ow, oh)
    assert rel(el[live], ref[live]) < (1e-12 if mode == "fp64" else 1e-6)
    cw.orthonormalize()
    dq, oq, _ = cw.get_walkers()
    for k in range(W):
        blocks = [dq[k]] if rw else [dq[k][:, :oh.nalpha], dq[k][:, oh.nalpha:]]
        for b in blocks:
            assert np.allclose(b.conj().T @ b, np.eye(b.shape[1]), atol=1e-12)
    assert rel(oq, O.overlap(ot, O.Walkers(oh, rw, dq))) < 1e-12
    cw.close()


def test_cpu_port_timed_loop_runs():
    oh, ot, prop, rw = setup("uhf", "ref")
    cw = C.CpuWalkers(oh, ot, prop, rw, 16, nthreads=2)
    cw.set_walkers(np.repeat(O._ref_dets(oh, ot.phi, rw)[None], 16, axis=0))
    out = cw.run_timed(6, 5, 3, O.hf_energy(ot, oh, ot.phi, rw).real)
    assert out[3] == 6 * 16 and out[0] > 0 and out[1] > 0 and out[2] > 0
    _, _, w = cw.get_walkers()
    assert np.all(np.isfinite(w)) and (w > 0).sum() > 8
    cw.close()
