"""ctypes front end of oracle/cpu_step.cpp, the C++ restatement of the
reference's walker step (test infrastructure: bench.py's CPU baseline and the
reference arm; tests/ check it against the numpy oracle).

``CpuWalkers(ham, trial, prop, rhf_walker, W)`` takes the numpy oracle's
Hamiltonian, trial and Propagator (its set-up: rotated Cholesky, FP32 packed
Cholesky, mean-field shifts, exp(-dt/2 h1')) and keeps W walkers in C++.
Restricted integrals only (the benchmark workloads).
"""
import ctypes
import os

import numpy as np

from . import afqmc_oracle as O

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


class _Case(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("G", ctypes.c_int), ("Gene", ctypes.c_int),
                ("nchan", ctypes.c_int), ("mult", ctypes.c_int), ("ncw", ctypes.c_int), ("nce", ctypes.c_int),
                ("ch_n", ctypes.c_int * 2), ("ch_psi_off", ctypes.c_int * 2), ("ch_col_off", ctypes.c_int * 2),
                ("nblk", ctypes.c_int), ("blk_c0", ctypes.c_int * 2), ("blk_nc", ctypes.c_int * 2),
                ("vhs_fp64", ctypes.c_int),
                ("dt", ctypes.c_double), ("ecore", ctypes.c_double), ("pc_re", ctypes.c_double),
                ("pc_im", ctypes.c_double),
                ("phi", ctypes.c_void_p), ("rot", ctypes.c_void_p), ("rotT", ctypes.c_void_p),
                ("h1phi", ctypes.c_void_p), ("L32", ctypes.c_void_p), ("L64", ctypes.c_void_p),
                ("B_re", ctypes.c_void_p), ("B_im", ctypes.c_void_p), ("mf_re", ctypes.c_void_p),
                ("mf_im", ctypes.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        so = os.path.join(_HERE, "_build", "libcpustep.so")
        if not os.path.exists(so):
            O.build()
        L = ctypes.CDLL(so)
        vp = ctypes.c_void_p
        L.cpu_create.restype = vp
        L.cpu_create.argtypes = [ctypes.POINTER(_Case), ctypes.c_int, ctypes.c_uint64, ctypes.c_int]
        L.cpu_destroy.argtypes = [vp]
        L.cpu_nthreads.argtypes = [vp]
        L.cpu_set_walkers.argtypes = [vp, vp, vp, vp]
        L.cpu_get_walkers.argtypes = [vp, vp, vp, vp]
        L.cpu_step.restype = ctypes.c_double
        L.cpu_step.argtypes = [vp, vp, ctypes.c_double, ctypes.c_double]
        L.cpu_orthonormalize.argtypes = [vp]
        L.cpu_local_energy.argtypes = [vp, vp]
        L.cpu_run_timed.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class CpuWalkers:
    def __init__(self, ham, trial, prop, rhf_walker, W, nthreads=0, seed=1, nchol_ene=None):
        if ham.int_type != "r":
            raise ValueError("the C++ step covers restricted integrals")
        N, G = ham.norb, ham.nchol
        na, nb = ham.nalpha, ham.nbeta
        ow = O.Walkers(ham, rhf_walker, np.zeros((1, N, na if rhf_walker else na + nb), complex))
        chans, mult = O.channels(trial, ow)
        phis, rots, h1phis, ns, psi_off = [], [], [], [], []
        for (_, s) in chans:
            n = trial.phi[s].shape[1]
            phis.append(trial.phi[s].T)                      # [n][N]
            rots.append(trial.rot[s])                        # [G][n][N]
            h1phis.append(trial.h1phi[s].T)                  # [n][N]
            ns.append(n)
            psi_off.append(0 if (rhf_walker or s == 0) else na)
        self.keep = []

        def arr(a, dt=np.float64):
            a = np.ascontiguousarray(a, dtype=dt)
            self.keep.append(a)
            return a
        phi = arr(np.concatenate(phis, axis=0))
        rot = arr(np.concatenate(rots, axis=1).reshape(G, -1))
        rotT = arr(rot.T)
        h1phi = arr(np.concatenate(h1phis, axis=0))
        L32 = arr(prop.packed[0] if prop.mode == "ref" else ham.float_chol[0], np.float32)
        L64 = arr(ham.packed_chol[0])
        B = prop.expm[0].T  # column major
        c = _Case()
        c.N, c.G, c.Gene = N, G, int(nchol_ene or ham.nchol_ene)
        c.nchan, c.mult = len(chans), mult
        c.ncw = na if rhf_walker else na + nb
        c.nce = sum(ns)
        col = 0
        for i, n in enumerate(ns):
            c.ch_n[i], c.ch_psi_off[i], c.ch_col_off[i] = n, psi_off[i], col
            col += n
        if rhf_walker:
            c.nblk, c.blk_c0[0], c.blk_nc[0] = 1, 0, na
        else:
            c.nblk = 2
            c.blk_c0[0], c.blk_nc[0], c.blk_c0[1], c.blk_nc[1] = 0, na, na, nb
        c.vhs_fp64 = 0 if prop.mode == "ref" else 1
        c.dt, c.ecore = prop.dt, ham.ecore
        c.pc_re, c.pc_im = prop.prop_constant.real, prop.prop_constant.imag
        c.phi, c.rot, c.rotT, c.h1phi = phi.ctypes.data, rot.ctypes.data, rotT.ctypes.data, h1phi.ctypes.data
        c.L32, c.L64 = L32.ctypes.data, L64.ctypes.data
        Br, Bi = arr(B.real), arr(B.imag)
        c.B_re, c.B_im = Br.ctypes.data, Bi.ctypes.data
        mr, mi = arr(prop.mf.real), arr(prop.mf.imag)
        c.mf_re, c.mf_im = mr.ctypes.data, mi.ctypes.data
        self.case = c
        self.N, self.W, self.ncw, self.G = N, W, c.ncw, G
        self.h = lib().cpu_create(ctypes.byref(c), W, seed, int(nthreads))
        self.nthreads = lib().cpu_nthreads(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().cpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_walkers(self, dets, overlaps=None, weights=None):
        """dets (W, N, ncw) complex, the oracle's layout."""
        d = np.ascontiguousarray(np.asarray(dets, complex).transpose(0, 2, 1))
        o = None if overlaps is None else np.ascontiguousarray(overlaps, complex)
        w = None if weights is None else np.ascontiguousarray(weights, np.float64)
        lib().cpu_set_walkers(self.h, d.ctypes.data, _p(o), _p(w))

    def get_walkers(self):
        d = np.zeros((self.W, self.ncw, self.N), complex)
        o = np.zeros(self.W, complex)
        w = np.zeros(self.W)
        lib().cpu_get_walkers(self.h, d.ctypes.data, o.ctypes.data, w.ctypes.data)
        return d.transpose(0, 2, 1), o, w

    def step(self, xi, eshift, weight_cap=np.inf):
        x = None if xi is None else np.ascontiguousarray(xi, np.float64)
        return lib().cpu_step(self.h, _p(x), float(eshift), float(min(weight_cap, 1e300)))

    def orthonormalize(self):
        lib().cpu_orthonormalize(self.h)

    def local_energy(self):
        e = np.zeros(self.W, complex)
        lib().cpu_local_energy(self.h, e.ctypes.data)
        return e

    def run_timed(self, nsteps, ortho_every, energy_every, e_est, weight_cap=100.0):
        """(seconds in steps, in QR, in energies, walker-steps)."""
        out = np.zeros(4)
        lib().cpu_run_timed(self.h, int(nsteps), int(ortho_every), int(energy_every), float(e_est),
                            float(weight_cap), out.ctypes.data)
        return out
