"""The allocation-free orthonormalisation entry point against the handle's own.

afqmc_orthonormalize_noalloc serves callers that cannot allocate GPU memory
when they call it (hosts whose device memory belongs to another allocator,
loops that must stay out of cudaMalloc / cudaFree, which synchronise the
device): it runs the same Householder QR on the caller's device buffers with
its Q workspace in a fixed device array.  This test calls it through the C ABI twice in a row, on
two different walker sets, and checks each result against afqmc_orthonormalize
of a handle holding the same walkers, within the FP64 tolerance of the other
parity tests (1e-12 relative).  The second walker set is large enough to go
through the fixed workspace in two batches.  A restricted walker (one spin
block, overlap divided by the squared diagonal product) is checked the same
way.

This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_noalloc_orthonormalize_matches_handle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from vmc_gb300 import afqmc as A
    L = A.lib()
    f = L.afqmc_orthonormalize_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p]

    s = S.make_system(30, 6, 20, 99, "uhf")
    N, na, nb = 30, 6, 5
    gh = A.Hamiltonian(N, na, nb, 0.0, s["h1"], s["h1mod"], s["chol"])
    gt = A.UHF(gh, s["phi_a"][:, :na], s["phi_b"][:, :nb])
    base = np.concatenate([s["phi_a"][:, :na], s["phi_b"][:, :nb]], axis=1)
    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream().cuda_stream
    # 1700 walkers x 11 columns x 30 rows > 2^19: two batches through the workspace
    for call, W in enumerate([40, 1700]):
        dets = base[None] + 0.3 * (rng.standard_normal((W, N, na + nb)) + 1j * rng.standard_normal((W, N, na + nb)))
        wk = A.DQMCWalkers(gh, gt, W, False, 0.005, precision="fp64")
        wk.set_det(dets)
        _, ovl0, _ = wk.get_det()
        wk.orthogonalize()
        d_ref, o_ref, _ = wk.get_det()
        wk.close()

        # the caller's own device buffers, library layout [W][ncols][N]
        d_dev = torch.from_numpy(np.ascontiguousarray(dets.transpose(0, 2, 1))).to("cuda")
        o_dev = torch.from_numpy(ovl0.copy()).to("cuda")
        torch.cuda.synchronize()
        rc = f(d_dev.data_ptr(), o_dev.data_ptr(), W, N, na, nb, 0, stream)
        assert rc == 0, L.afqmc_last_error(None).decode()
        torch.cuda.synchronize()
        d_out = d_dev.cpu().numpy().transpose(0, 2, 1)
        o_out = o_dev.cpu().numpy()
        assert rel(d_out, d_ref) < TOL, (call, rel(d_out, d_ref))
        assert rel(o_out, o_ref) < TOL, (call, rel(o_out, o_ref))
        # Q has orthonormal columns per spin block
        q = d_out[0, :, :na]
        assert np.allclose(q.conj().T @ q, np.eye(na), atol=1e-12)


def test_noalloc_restricted_walker():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from vmc_gb300 import afqmc as A
    L = A.lib()
    f = L.afqmc_orthonormalize_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p]
    s = S.make_system(26, 5, 20, 98, "rhf")
    N, n, W = 26, 5, 33
    gh = A.Hamiltonian(N, n, n, 0.0, s["h1"], s["h1mod"], s["chol"])
    gt = A.RHF(gh, s["phi_a"][:, :n])
    rng = np.random.default_rng(8)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        dets = s["phi_a"][None, :, :n] + 0.3 * (rng.standard_normal((W, N, n)) + 1j * rng.standard_normal((W, N, n)))
        wk = A.DQMCWalkers(gh, gt, W, True, 0.005, precision="fp64")
        wk.set_det(dets)
        _, ovl0, _ = wk.get_det()
        wk.orthogonalize()
        d_ref, o_ref, _ = wk.get_det()
        wk.close()
        d_dev = torch.from_numpy(np.ascontiguousarray(dets.transpose(0, 2, 1))).to("cuda")
        o_dev = torch.from_numpy(ovl0.copy()).to("cuda")
        torch.cuda.synchronize()
        rc = f(d_dev.data_ptr(), o_dev.data_ptr(), W, N, n, n, 1, stream)
        assert rc == 0, L.afqmc_last_error(None).decode()
        torch.cuda.synchronize()
        d_out = d_dev.cpu().numpy().transpose(0, 2, 1)
        o_out = o_dev.cpu().numpy()
        assert rel(d_out, d_ref[:, :, :n]) < TOL, (call, rel(d_out, d_ref[:, :, :n]))
        assert rel(o_out, o_ref) < TOL, (call, rel(o_out, o_ref))


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from vmc_gb300 import afqmc as A
    L = A.lib()
    f = L.afqmc_orthonormalize_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p]
    d = torch.zeros(2, dtype=torch.complex128, device="cuda")
    # one walker det of 128 x 4100 complex exceeds the 2^19 workspace
    rc = f(d.data_ptr(), d.data_ptr(), 1, 4100, 128, 128, 0, None)
    assert rc == 1
    assert "exceeds the fixed scratch" in L.afqmc_last_error(None).decode()
