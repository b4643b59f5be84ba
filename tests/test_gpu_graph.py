"""CUDA-graph replay: a captured block of device-field steps reproduces the
same steps launched one by one, bit for bit, for one system and for several
systems of uneven orbital counts advancing in one graph."""
import numpy as np
import pytest

from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def make(A, s, W, precision, seed):
    n = s["nalpha"]
    gh = A.Hamiltonian(s["norb"], n, n, 0.0, s["h1"], s["h1mod"], s["chol"])
    gt = A.UHF(gh, s["phi_a"], s["phi_b"])
    wk = A.DQMCWalkers(gh, gt, W, False, 0.005, precision=precision, seed=seed)
    e0 = wk.ham_and_overlap().real.mean()
    wk.set_energy_estimate(e0, e0)
    return wk


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_replay_equals_steps(A, precision):
    s = S.make_system(36, 6, 100, 31, "uhf")
    a = make(A, s, 96, precision, 5)
    b = make(A, s, 96, precision, 5)
    for k in range(10):
        a.propagate_phaseless(None)
        if (k + 1) % 5 == 0:
            a.orthogonalize()
    g = A.StepGraph([b], 5, ortho_every=5)
    g.launch()
    g.launch()
    da, oa, wa = a.get_det()
    db, ob, wb = b.get_det()
    assert np.array_equal(da, db) and np.array_equal(oa, ob) and np.array_equal(wa, wb)
    g.close()


def test_uneven_systems_in_one_graph(A):
    systems = [S.make_system(n, max(2, round(n / 6)), 3 * n, 100 + n, "uhf") for n in (40, 72, 100, 150)]
    solo = [make(A, s, 64, "mixed", 9 + i) for i, s in enumerate(systems)]
    batch = [make(A, s, 64, "mixed", 9 + i) for i, s in enumerate(systems)]
    for w in solo:
        for k in range(10):
            w.propagate_phaseless(None)
            if (k + 1) % 5 == 0:
                w.orthogonalize()
    g = A.StepGraph(batch, 10, ortho_every=5)
    g.launch()
    for a, b in zip(solo, batch):
        da, oa, wa = a.get_det()
        db, ob, wb = b.get_det()
        assert np.array_equal(da, db) and np.array_equal(wa, wb)
        assert np.all(np.isfinite(da))
    g.close()


def test_autotune_choices_and_cache(A, tmp_path):
    """The autotuner picks valid variants, caches them, and the tuned handle
    steps like an untuned one (same fields) within the mixed form's tolerance."""
    s = S.make_system(48, 8, 160, 41, "uhf")
    a = make(A, s, 300, "mixed", 3)
    b = make(A, s, 300, "mixed", 3)
    cache = str(tmp_path / "tune.txt")
    ch, rep = A.autotune(b, cache)
    assert ch["bn_fb"] in (64, 128, 256) and ch["bn_vhs"] in (64, 128, 256)
    assert ch["prop"] in (1, 2, 3, 4) and ch["ovl"] in (1, 2, 3, 4) and ch["qr"] in (1, 2)
    c = make(A, s, 300, "mixed", 3)
    ch2, rep2 = A.autotune(c, cache)
    assert ch2 == ch and rep2.startswith("cached")
    for k in range(6):
        a.propagate_phaseless(None)
        b.propagate_phaseless(None)
    da, oa, wa = a.get_det()
    db, ob, wb = b.get_det()
    assert np.abs(da - db).max() / np.abs(da).max() < 1e-5
    assert np.abs(wa - wb).max() / np.abs(wa).max() < 1e-5
