"""CPU-side checks of the C ABI library: it loads, exports every entry point
that include/afqmc.h declares, its host-only parts behave, and with no GPU the
device entry points fail with an error instead of falling back to the CPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from vmc_gb300 import afqmc as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "afqmc.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(afqmc_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built():
    if not os.path.exists(A.LIB_PATH):
        from vmc_gb300 import build
        build.build()
    return A.lib()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("afqmc_create", "afqmc_step", "afqmc_force_bias", "afqmc_local_energy",
              "afqmc_orthonormalize", "afqmc_run", "afqmc_set_walkers", "afqmc_get_walkers"):
        assert s in syms


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(A.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_reference_order_rng_matches_oracle(built):
    """afqmc_refrng_* (product) and the oracle's fieldgen both replay
    mt19937 + per-walker normal_distribution: same stream, dead walkers skipped."""
    from oracle import afqmc_oracle as O
    w = np.array([1.0, 0.0, 2.0, 1e-9, 0.5])
    a, b = A.RefRNG(4321, 5), O.RankRNG(4321, 5)
    for _ in range(3):
        x, y = a.draw_step(w, 7), b.draw_step(w, 7)
        assert np.array_equal(x, y)
        assert np.all(x[1] == 0) and np.all(x[3] == 0)
    assert a.uniform() == b.uniform()


def test_create_without_gpu_fails_loudly(built):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    N, n, G = 4, 2, 3
    ham = A.Hamiltonian(N, n, n, 0.0, np.eye(N), np.eye(N), np.zeros((G, N, N)))
    tr = A.RHF(ham, np.eye(N)[:, :n])
    with pytest.raises(A.AfqmcError) as e:
        A.DQMCWalkers(ham, tr, 4, True, 0.01)
    assert e.value.code in (2,)


def test_create_rejects_bad_arguments(built):
    N, n, G = 4, 2, 3
    ham = A.Hamiltonian(N, n, n - 1, 0.0, np.eye(N), np.eye(N), np.zeros((G, N, N)))
    tr = A.RHF(ham, np.eye(N)[:, :n])
    with pytest.raises(A.AfqmcError) as e:
        A.DQMCWalkers(ham, tr, 4, False, 0.01)  # RHF trial needs nalpha == nbeta
    assert e.value.code == 5
    with pytest.raises(A.AfqmcError) as e:
        A.DQMCWalkers(ham, A.UHF(ham, np.eye(N)[:, :n], np.eye(N)[:, :1]), 0, False, 0.01)
    assert e.value.code == 1
