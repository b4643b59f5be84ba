"""CPU oracle for the phaseless AFQMC walker step (test infrastructure).

This module is the checker, not the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it.  It
restates, in numpy (complex128, batched over walkers), the algorithm of the
reference's DQMC phaseless path:

* ``Hamiltonian``: DQMC/Hamiltonian.cpp:9-42 (integrals), :179-219
  (``floattenCholesky``: packed lower triangle in FP32), :52-133
  (``rotateCholesky``: half-rotated tensors Phi^T L_g).
* trials: DQMC/RHF.cpp:9-101 and DQMC/UHF.cpp (overlap, force bias, local energy).
* ``prep_prop``: DQMC/DQMCWalker.cpp:32-103 (restricted integrals) and :106-187
  (``intType "u"``): mean-field shifts, h1', propagation constant, exp(-dt/2 h1').
* ``step``: DQMC/DQMCWalker.cpp:441-503 / :506-554 (force bias, shifted fields,
  VHS, Taylor propagator, overlap ratio, phaseless importance function) and
  DQMC/MixedEstimator.cpp:461-468 (weight update and cap).
* ``orthogonalize``: DQMC/DQMCWalker.cpp:295-326 (Householder QR, Eigen's sign
  convention: real R diagonal beta = -sign(Re c0) * ||x||).
* ``run``: DQMC/MixedEstimator.cpp:309-660 (population control, measurement with
  the local-energy clamp, comb reconfiguration), with MPI ranks emulated.

Two precisions are offered.  ``mode="ref"`` reproduces the reference's own mixed
precision: the mean-field shifts use the FP32 packed Cholesky copy
(DQMCWalker.cpp:72-84, active because the RHF/UHF left trial sets ``rotFlag``)
and the VHS is an FP32 product of the FP32 packed Cholesky vectors with the
fields rounded to complex<float> (DQMCWalker.cpp:454, :406-421).  ``mode="fp64"``
is the same algorithm with those FP32 parts in FP64 (still from the packed lower
triangle); it is the FP64 oracle for the GPU's FP64 form.

Layouts.  ``chol[g, i, j]`` equals the reference's ``chol[g](i, j)`` (the HDF5
``/chol`` dataset is read as column-major maps, integral.cpp:636-642).  Walker
dets are ``(W, N, ncols)`` complex128 with the alpha columns first, then beta
(absent for the restricted walker).
"""
import ctypes
import os

import numpy as np
import scipy.linalg

_HERE = os.path.dirname(os.path.abspath(__file__))


# ---------------------------------------------------------------------------
# reference-order random fields (std::mt19937 + per-walker normal_distribution)
# ---------------------------------------------------------------------------
_fg_lib = None


def fieldgen_lib():
    """Load (building if needed) the C++ replay of the reference's RNG order."""
    global _fg_lib
    if _fg_lib is None:
        so = os.path.join(_HERE, "_build", "libfieldgen.so")
        if not os.path.exists(so):
            build()
        lib = ctypes.CDLL(so)
        lib.fg_create.restype = ctypes.c_void_p
        lib.fg_create.argtypes = [ctypes.c_uint, ctypes.c_int]
        lib.fg_destroy.argtypes = [ctypes.c_void_p]
        lib.fg_draw.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.fg_draw_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_int, ctypes.c_void_p]
        lib.fg_uniform.restype = ctypes.c_double
        lib.fg_uniform.argtypes = [ctypes.c_void_p]
        _fg_lib = lib
    return _fg_lib


def build():
    """Compile the oracle's C++ helper into oracle/_build (plain g++)."""
    import subprocess
    out = os.path.join(_HERE, "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libfieldgen.so")
    tmp = so + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC",
                           os.path.join(_HERE, "fieldgen.cpp"), "-o", tmp])
    os.replace(tmp, so)
    # the C++ restatement of the walker step (CPU baseline; oracle/cpu_port.py)
    so = os.path.join(out, "libcpustep.so")
    tmp = so + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fcx-limited-range", "-shared", "-fPIC",
                           os.path.join(_HERE, "cpu_step.cpp"), "-o", tmp])
    os.replace(tmp, so)


class RankRNG:
    """One MPI rank's generator: mt19937(seed + rank) and nwalk normal streams."""

    def __init__(self, seed, nwalk):
        self.lib = fieldgen_lib()
        self.h = self.lib.fg_create(seed, nwalk)
        self.nwalk = nwalk

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.fg_destroy(self.h)
            self.h = None

    def draw_step(self, weights, nfields):
        """Fields for one step: rows of walkers with weight <= 1e-8 stay zero."""
        out = np.zeros((self.nwalk, nfields))
        w = np.ascontiguousarray(weights, dtype=np.float64)
        self.lib.fg_draw_step(self.h, self.nwalk, w.ctypes.data, nfields, out.ctypes.data)
        return out

    def uniform(self):
        return self.lib.fg_uniform(self.h)


# ---------------------------------------------------------------------------
# Hamiltonian and trials
# ---------------------------------------------------------------------------
def tri_size(n):
    return n * (n + 1) // 2


def pack_lower(mats):
    """Packed lower triangle, index i*(i+1)/2 + j for j <= i (Hamiltonian.cpp:189-199)."""
    n = mats.shape[-1]
    ii, jj = np.tril_indices(n)
    return mats[..., ii, jj]


def unpack_sym(packed, n):
    """Symmetric matrix from the packed lower triangle (DQMCWalker.cpp:74-83, :414-420)."""
    ii, jj = np.tril_indices(n)
    out = np.zeros(packed.shape[:-1] + (n, n), dtype=packed.dtype)
    out[..., ii, jj] = packed
    out[..., jj, ii] = packed
    return out


class Hamiltonian:
    """Restatement of DQMC/Hamiltonian.h:8-22.

    int_type "r": h1, h1mod (N,N); chol (G,N,N).
    int_type "u": h1u, h1umod (2,N,N); cholu (2,G,N,N).
    """

    def __init__(self, norb, nalpha, nbeta, ecore, h1=None, h1mod=None, chol=None,
                 int_type="r", h1u=None, h1umod=None, cholu=None):
        self.norb, self.nalpha, self.nbeta = int(norb), int(nalpha), int(nbeta)
        self.ecore = float(ecore)
        self.int_type = int_type
        if int_type == "r":
            self.h1 = np.asarray(h1, dtype=np.float64)
            self.h1mod = np.asarray(h1mod, dtype=np.float64)
            self.chol = np.asarray(chol, dtype=np.float64)
            self.nchol = self.chol.shape[0]
            # spin-resolved views so the rest of the code is written once
            self.h1s = np.stack([self.h1, self.h1])
            self.h1mods = np.stack([self.h1mod, self.h1mod])
            self.chols = np.stack([self.chol, self.chol])
        elif int_type == "u":
            self.h1s = np.asarray(h1u, dtype=np.float64)
            self.h1mods = np.asarray(h1umod, dtype=np.float64)
            self.chols = np.asarray(cholu, dtype=np.float64)
            self.nchol = self.chols.shape[1]
        else:
            raise ValueError("int_type must be 'r' or 'u'")
        self.nchol_ene = self.nchol
        # floattenCholesky (Hamiltonian.cpp:179-219): FP32 packed lower triangle
        nsp = 1 if int_type == "r" else 2
        self.float_chol = pack_lower(self.chols[:nsp]).astype(np.float32)  # (nsp, G, T)
        self.packed_chol = pack_lower(self.chols[:nsp])                     # FP64 twin

    @classmethod
    def from_fcidump(cls, d, int_type="r"):
        """From ``vmc_gb300.hdf5.read_fcidump_chol`` output (integral.cpp:589-741)."""
        n = d["norb"]
        if int_type == "r":
            chol = d["chol"].transpose(0, 2, 1)  # column-major maps
            return cls(n, d["nalpha"], d["nbeta"], d["ecore"], d["h1"], d["h1mod"], chol)
        cholu = d["cholu"].transpose(0, 1, 3, 2)
        return cls(n, d["nalpha"], d["nbeta"], d["ecore"], int_type="u",
                   h1u=d["h1u"], h1umod=d["h1umod"], cholu=cholu)


class Trial:
    """RHF (DQMC/RHF.cpp) or UHF (DQMC/UHF.cpp) left trial with rotated Cholesky.

    ``phi``: list of two real (N, n_sigma) orbital blocks.  For RHF both are the
    same block (RHF.cpp:13, the first nalpha columns of rhf.txt).
    """

    def __init__(self, ham, kind, phi_a, phi_b=None):
        self.kind = kind
        phi_a = np.asarray(phi_a, dtype=np.float64)
        phi_b = phi_a if phi_b is None else np.asarray(phi_b, dtype=np.float64)
        if kind == "rhf":
            phi_b = phi_a[:, :ham.nbeta]
        self.phi = [phi_a, phi_b]
        # rotateCholesky (Hamiltonian.cpp:52-84 restricted, :88-133 two-spin):
        # rot[s][g] = Phi_s^T L_{s,g}, shape (n_s, N)
        self.rot = [np.einsum("pi,gpq->giq", self.phi[s], ham.chols[s]) for s in range(2)]
        # h1 * Phi_s, used for the one-body energy sum_pq G_s[p,q] h1[p,q]
        self.h1phi = [ham.h1s[s] @ self.phi[s] for s in range(2)]

    @classmethod
    def rhf_from_file(cls, ham, path):
        mat = np.loadtxt(path).reshape(ham.norb, ham.norb)  # input.cpp:376-384
        return cls(ham, "rhf", mat[:, :ham.nalpha])

    @classmethod
    def uhf_from_file(cls, ham, path):
        mat = np.loadtxt(path).reshape(ham.norb, 2 * ham.norb)  # UHF.cpp reads N x 2N
        return cls(ham, "uhf", mat[:, :ham.nalpha], mat[:, ham.norb:ham.norb + ham.nbeta])


# ---------------------------------------------------------------------------
# walker batch
# ---------------------------------------------------------------------------
class Walkers:
    """A batch of DQMCWalker objects (DQMC/DQMCWalker.h:7-46), stored as arrays."""

    def __init__(self, ham, rhf_walker, dets, overlaps=None, weights=None):
        self.rhf = bool(rhf_walker)
        self.na, self.nb = ham.nalpha, ham.nbeta
        self.dets = np.array(dets, dtype=np.complex128)  # (W, N, ncols)
        W = self.dets.shape[0]
        self.overlaps = np.ones(W, complex) if overlaps is None else np.array(overlaps, complex)
        self.weights = np.ones(W) if weights is None else np.array(weights, float)

    @property
    def nwalk(self):
        return self.dets.shape[0]

    def spin_det(self, s):
        if self.rhf or s == 0:
            return self.dets[:, :, :self.na]
        return self.dets[:, :, self.na:self.na + self.nb]

    def copy(self):
        w = Walkers.__new__(Walkers)
        w.rhf, w.na, w.nb = self.rhf, self.na, self.nb
        w.dets, w.overlaps, w.weights = self.dets.copy(), self.overlaps.copy(), self.weights.copy()
        return w


def channels(trial, walkers):
    """Trial contractions as (walker det, Phi, rotated Cholesky) channels.

    RHF trial with the restricted walker is one channel counted twice
    (RHF.cpp:34-39, :54-61, :104-131); every other pairing has two channels
    (RHF.cpp:27-31, :42-51, :70-101; UHF.cpp overlap/forceBias/hamAndOverlap).
    Returns (list of (det_index, spin), multiplicity).
    """
    if trial.kind == "rhf" and walkers.rhf:
        return [(0, 0)], 2
    return [(0 if walkers.rhf else 0, 0), (0 if walkers.rhf else 1, 1)], 1


def _spin_dets(walkers, trial):
    chans, mult = channels(trial, walkers)
    out = []
    for (dummy, s) in chans:
        det = walkers.spin_det(0) if walkers.rhf else walkers.spin_det(s)
        out.append((s, det))
    return out, mult


def overlap(trial, walkers):
    """<Psi_T|phi> = prod_s det(Phi_s^T psi_s)^mult (RHF.cpp:27-39, UHF.cpp overlap)."""
    chans, mult = _spin_dets(walkers, trial)
    o = np.ones(walkers.nwalk, complex)
    for s, det in chans:
        o = o * np.linalg.det(np.einsum("pi,wpj->wij", trial.phi[s], det)) ** mult
    return o


def thetas(trial, walkers):
    """theta_s = psi_s (Phi_s^T psi_s)^{-1}, (W, N, n_s) per channel (RHF.cpp:46-47)."""
    chans, mult = _spin_dets(walkers, trial)
    out = []
    for s, det in chans:
        m = np.einsum("pi,wpj->wij", trial.phi[s], det)
        out.append((s, det @ np.linalg.inv(m)))
    return out, mult


def force_bias(trial, walkers, ham, nchol=None):
    """fb_g = mult * sum_s sum_{i,p} theta_s[p,i] rot_s[g][i,p] (RHF.cpp:42-61, UHF.cpp:45-65)."""
    th, mult = thetas(trial, walkers)
    G = ham.nchol if nchol is None else nchol
    fb = np.zeros((walkers.nwalk, G), complex)
    for s, t in th:
        fb += np.einsum("wpi,gip->wg", t, trial.rot[s][:G])
    return mult * fb


def local_energy(trial, walkers, ham, nchol_ene=None):
    """hamAndOverlap / overlap (RHF.cpp:70-131, UHF.cpp:75-140).

    E = ecore + mult sum_s tr(G_s h1_s)
          + 1/2 sum_{g < ncholEne} [(mult sum_s c_sg)^2 - mult sum_s sum_ij f_sg[i,j] f_sg[j,i]]
    with f_sg = rot_s[g] theta_s and c_sg = tr f_sg.  Returns complex (W,).
    """
    G = ham.nchol_ene if nchol_ene is None else nchol_ene
    th, mult = thetas(trial, walkers)
    e = np.full(walkers.nwalk, ham.ecore, complex)
    csum = np.zeros((walkers.nwalk, G), complex)
    exch = np.zeros(walkers.nwalk, complex)
    for s, t in th:
        e += mult * np.einsum("wpi,pi->w", t, trial.h1phi[s])
        f = np.einsum("gip,wpj->wgij", trial.rot[s][:G], t)
        csum += np.einsum("wgii->wg", f)
        exch += np.einsum("wgij,wgji->w", f, f)
    e += 0.5 * ((mult * csum) ** 2).sum(axis=1) - 0.5 * mult * exch
    return e


def hf_energy(trial, ham, ref_phi, rhf_walker, nchol_ene=None):
    """Energy of the reference determinant (MixedEstimator.cpp:338-354)."""
    dets = _ref_dets(ham, ref_phi, rhf_walker)
    w = Walkers(ham, rhf_walker, dets[None])
    return local_energy(trial, w, ham, nchol_ene)[0]


def _ref_dets(ham, ref_phi, rhf_walker):
    a, b = ref_phi
    if rhf_walker:
        return a[:, :ham.nalpha].astype(complex)
    return np.concatenate([a[:, :ham.nalpha], b[:, :ham.nbeta]], axis=1).astype(complex)


# ---------------------------------------------------------------------------
# prepProp
# ---------------------------------------------------------------------------
class Propagator:
    """DQMCWalker::prepPropR/U (DQMCWalker.cpp:32-103, :106-187), phaseless branch.

    ``ref_phi``: the two real reference blocks used for the mean-field Green's
    function G_s = ref_s (ref_s^T ref_s)^{-1} ref_s^T (DQMCWalker.cpp:59-65).
    ``green``: optional (2, N, N) override (the reference's spinRDM.0.0.txt).
    """

    def __init__(self, ham, ref_phi, dt, mode="ref", green=None):
        self.dt, self.mode = float(dt), mode
        N = ham.norb
        if green is None:
            green = []
            for s in range(2):
                r = np.asarray(ref_phi[s], dtype=np.float64)
                green.append(r @ np.linalg.inv(r.T @ r) @ r.T)
            green = np.stack(green)
        nsp = 1 if ham.int_type == "r" else 2
        if mode == "ref":
            Lsym = unpack_sym(ham.float_chol.astype(np.float64), N)  # (nsp, G, N, N)
        else:
            Lsym = unpack_sym(ham.packed_chol, N)
        Ls = [Lsym[0], Lsym[0]] if nsp == 1 else [Lsym[0], Lsym[1]]
        # mf_g = i * sum_s sum_pq G_s[p,q] L_{s,g}[p,q]   (DQMCWalker.cpp:85-87)
        mf = 1j * sum(np.einsum("pq,gpq->g", green[s], Ls[s]) for s in range(2))
        self.mf = mf
        # constant = ene0 - ecore - sum mf^2/2 ; propConstant = constant - ene0
        self.prop_constant = -ham.ecore - np.sum(mf ** 2) / 2.0
        self.h1p = [ham.h1mods[s] - np.einsum("g,gpq->pq", mf, 1j * Ls[s]) for s in range(2)]
        self.expm = [scipy.linalg.expm(-self.dt * self.h1p[s] / 2.0) for s in range(2)]
        self.packed = ham.float_chol if mode == "ref" else ham.packed_chol  # (nsp, G, T)
        self.nsp = nsp
        self.norb = N


# ---------------------------------------------------------------------------
# the phaseless step
# ---------------------------------------------------------------------------
def vhs(prop, fields, sp):
    """V = sqrt(dt) (i L.Re(x) - L.Im(x)) from packed L (DQMCWalker.cpp:406-421, :461-462)."""
    L = prop.packed[sp]  # (G, T)
    if prop.mode == "ref":
        f = fields.astype(np.complex64)
        pr = (f.real.astype(np.float32) @ L).astype(np.float32)
        pi = (f.imag.astype(np.float32) @ L).astype(np.float32)
        packed = (-pi).astype(np.float64) + 1j * pr.astype(np.float64)
    else:
        pr = fields.real @ L
        pi = fields.imag @ L
        packed = -pi + 1j * pr
    return np.sqrt(prop.dt) * unpack_sym(packed, prop.norb)


def apply_exp(v, det, terms=5):
    """det + sum_{k=1}^{5} V^k det / k! by the iteration temp = V temp / k (DQMCWalker.cpp:424-431)."""
    temp = det.copy()
    out = det.copy()
    for k in range(1, terms + 1):
        temp = v @ temp / k
        out = out + temp
    return out


def shifted_fields(prop, fb, xi):
    """x_g = xi_g - s_g, s_g = -sqrt(dt)(i fb_g - mf_g); shift and fbTerm (DQMCWalker.cpp:451-457)."""
    sdt = np.sqrt(prop.dt)
    fs = -sdt * (1j * fb - prop.mf[None, :])
    x = xi - fs
    shift = (x * prop.mf[None, :]).sum(axis=1)
    fbterm = (xi * fs - fs * fs / 2.0).sum(axis=1)
    return x, shift, fbterm


def step(trial, ham, prop, walkers, xi, eshift, weight_cap=np.inf):
    """One propagatePhaseless over the batch plus the weight update and cap.

    DQMCWalker.cpp:441-503 (restricted integrals) / :506-554 ("u"), and
    MixedEstimator.cpp:461-468.  Walkers with weight <= 1e-8 are not touched.
    ``xi``: (W, G) standard normals (rows of dead walkers are ignored).
    Returns the number of weights zeroed by the cap.
    """
    live = walkers.weights > 1.0e-8
    if not live.any():
        return 0
    sub = walkers.copy()
    idx = np.nonzero(live)[0]
    sub.dets, sub.overlaps, sub.weights = walkers.dets[idx], walkers.overlaps[idx], walkers.weights[idx]
    fb = force_bias(trial, sub, ham)
    x, shift, fbterm = shifted_fields(prop, fb, xi[idx])
    sdt = np.sqrt(prop.dt)
    na, nb = walkers.na, walkers.nb
    if prop.nsp == 1:
        v = vhs(prop, x, 0)
        vs = [v, v]
    else:
        vs = [vhs(prop, x, 0), vhs(prop, x, 1)]
    dets = sub.dets
    blocks = [(0, 0, na)] if walkers.rhf else [(0, 0, na), (1, na, na + nb)]
    new = dets.copy()
    for s, c0, c1 in blocks:
        d = prop.expm[s] @ dets[:, :, c0:c1]
        d = apply_exp(vs[s], d)
        new[:, :, c0:c1] = prop.expm[s] @ d
    sub.dets = new
    o_new = overlap(trial, sub)
    ratio = o_new / sub.overlaps
    imp = np.exp(-sdt * shift + fbterm + prop.dt * (eshift + prop.prop_constant)) * ratio
    theta = np.angle(np.exp(-sdt * shift) * ratio)
    with np.errstate(invalid="ignore"):
        val = np.abs(imp) * np.cos(theta)
    val = np.where((val < 1.0e-3) | (val > 100.0) | np.isnan(val), 0.0, val)
    walkers.dets[idx] = new
    walkers.overlaps[idx] = o_new
    w = walkers.weights[idx] * val
    capped = w > weight_cap
    w[capped] = 0.0
    walkers.weights[idx] = w
    return int(capped.sum())


def householder_qr(a):
    """Householder QR of one complex (m, n) matrix with Eigen's conventions.

    Reflector for column k (Householder.h makeHouseholder): c0 = x[0],
    beta = -sign(Re c0) * ||x||, tau = (beta - c0) / beta, v = [1, x[1:] / (c0 - beta)];
    a tail of squared norm <= the smallest normal number and Im(c0)^2 <= that
    number gives tau = 0, beta = c0.  Q = prod_k (I - conj(tau_k) v_k v_k^H)
    restricted to the first n columns; R's diagonal is the betas (real).
    Returns (Q (m, n), rdiag (n,)).
    """
    a = np.array(a, dtype=np.complex128)
    m, n = a.shape
    tiny = np.finfo(np.float64).tiny
    vs, taus, rdiag = [], [], []
    for k in range(n):
        x = a[k:, k]
        c0 = x[0]
        tail = np.vdot(x[1:], x[1:]).real
        if tail <= tiny and c0.imag ** 2 <= tiny:
            tau, beta, v = 0.0, c0.real, np.zeros(m - k, complex)
            v[0] = 1.0
        else:
            beta = np.sqrt(abs(c0) ** 2 + tail)
            if c0.real >= 0:
                beta = -beta
            v = np.empty(m - k, complex)
            v[0] = 1.0
            v[1:] = x[1:] / (c0 - beta)
            tau = np.conj((beta - c0) / beta)
        # apply H = I - tau v v^H to the remaining columns
        if k + 1 < n:
            sub = a[k:, k + 1:]
            a[k:, k + 1:] = sub - tau * np.outer(v, v.conj() @ sub)
        vs.append(v)
        taus.append(tau)
        rdiag.append(beta)
    q = np.zeros((m, n), complex)
    q[:n, :n] = np.eye(n)
    for k in reversed(range(n)):
        v = vs[k]
        q[k:, :] -= np.conj(taus[k]) * np.outer(v, v.conj() @ q[k:, :])
    return q, np.array(rdiag, dtype=complex)


def orthogonalize(walkers):
    """DQMCWalker::orthogonalize, phaseless branch (DQMCWalker.cpp:295-326)."""
    na, nb = walkers.na, walkers.nb
    for w in range(walkers.nwalk):
        fac = 1.0 + 0j
        blocks = [(0, na)] if walkers.rhf else [(0, na), (na, na + nb)]
        for c0, c1 in blocks:
            q, rd = householder_qr(walkers.dets[w, :, c0:c1])
            walkers.dets[w, :, c0:c1] = q
            fac *= np.prod(rd)
        walkers.overlaps[w] /= (fac * fac) if walkers.rhf else fac


# ---------------------------------------------------------------------------
# the driver (calcMixedEstimatorLongProp) with emulated MPI ranks
# ---------------------------------------------------------------------------
def one_rdm_samples(trial, walkers, int_type="r"):
    """Each walker's 1-RDM sample, real part: (psi_s (Phi_s^T psi_s)^-1 Phi_s^T)^T
    per spin (RHF.cpp:64-67, UHF.cpp:68-72).  Restricted integrals: the sum over
    the two spins, shape (W, 1, N, N); unrestricted: (W, 2, N, N).  The
    restricted walker's second spin is its first (DQMCWalker.cpp:487), which the
    channel multiplicity counts."""
    th, mult = thetas(trial, walkers)
    W, N = walkers.nwalk, walkers.dets.shape[1]
    nout = 1 if int_type == "r" else 2
    out = np.zeros((W, nout, N, N))
    for s, t in th:
        samp = np.einsum("pi,wqi->wpq", trial.phi[s], t).real  # [p][q] = sum_i Phi[p, i] theta[q, i]
        if nout == 1:
            out[:, 0] += mult * samp
        else:
            out[:, s] += samp
            if mult == 2:
                out[:, 1 - s] += samp
    return out


class OneRDM:
    """The reference's running weighted mean of the 1-RDM samples over live
    walkers and measurements (MixedEstimator.cpp:488-510), updated walker by
    walker: rdm <- (rdm cum + w sample) / (cum + w), cum <- cum + w."""

    def __init__(self, N, int_type="r"):
        self.rdm = np.zeros((1 if int_type == "r" else 2, N, N))
        self.cum = 0.0
        self.int_type = int_type

    def add(self, trial, walkers):
        live = np.nonzero(walkers.weights != 0.0)[0]
        if len(live) == 0:
            return
        sub = walkers.copy()
        sub.dets = walkers.dets[live]
        samples = one_rdm_samples(trial, sub, self.int_type)
        for j, w in enumerate(live):
            wt = walkers.weights[w]
            self.rdm = (self.rdm * self.cum + wt * samples[j]) / (self.cum + wt)
            self.cum += wt


def truncate_cholesky(trial, ham, ref_phi, rhf_walker, threshold):
    """ncholEne / delta selection (MixedEstimator.cpp:363-384)."""
    e_ref = hf_energy(trial, ham, ref_phi, rhf_walker, ham.nchol)
    G = ham.nchol
    for frac in (0.3, 0.4, 0.5, 0.6, 0.7):
        n = int(frac * G)
        e_t = hf_energy(trial, ham, ref_phi, rhf_walker, n)
        if abs(e_ref - e_t) < threshold:
            return n, (e_ref - e_t).real, e_ref
    return G, 0.0, e_ref


def run(ham, trial, ref_phi, rhf_walker, seed, nprocs=1, nwalk=20, dt=0.005, nsteps=50,
        nsweeps=50, ortho_steps=20, cholesky_threshold=1e-3, burn_iter=0,
        weight_cap=-1.0, mode="ref", max_steps=None, right_phi=None, one_rdm=False):
    """Restatement of calcMixedEstimatorLongProp (MixedEstimator.cpp:309-660).

    Emulates ``nprocs`` MPI ranks in lockstep: rank r has mt19937(seed + r) and
    ``nwalk`` walkers; the sums of MixedEstimator.cpp:420, :473, :536 run over
    all ranks; the comb (:559-635) gathers in rank order and draws zeta from rank
    0's generator.  Returns (totalWeights, totalEnergies) per block, i.e. the
    samples.dat columns (:678-683).  one_rdm: the info dict also holds the
    mixed 1-RDM ("one_rdm", "rdm_weight") accumulated at the measurements after
    equilibration (:491-510).
    """
    nchol_ene, delta, e_ref = truncate_cholesky(trial, ham, ref_phi, rhf_walker, cholesky_threshold)
    ham.nchol_ene = nchol_ene
    prop = Propagator(ham, ref_phi, dt, mode=mode)
    right = ref_phi if right_phi is None else right_phi
    init = _ref_dets(ham, right, rhf_walker)
    P = nprocs
    wk = Walkers(ham, rhf_walker, np.repeat(init[None], P * nwalk, axis=0))
    wk.overlaps = overlap(trial, wk)
    eloc = local_energy(trial, wk, ham).real
    rngs = [RankRNG(seed + r, nwalk) for r in range(P)]
    tot_w = np.zeros(nsweeps)
    tot_e = np.zeros(nsweeps)
    tot_w[0] = nwalk * P
    tot_e[0] = eloc.sum() / tot_w[0] + delta
    avg_e = avg_e_eql = tot_e[0]
    num_eql = den_eql = num = den = 0.0
    eshift = tot_e[0]
    e_est = tot_e[0]
    cap = weight_cap if weight_cap > 0 else max(100.0, nwalk / 10.0)
    nlarge = 0
    rdm = OneRDM(ham.norb, ham.int_type) if one_rdm else None
    last = nsweeps * nsteps if max_steps is None else min(nsweeps * nsteps, max_steps + 1)
    for st in range(1, last):
        if st * dt < 10.0:
            avg_e = avg_e_eql
        xi = np.concatenate([rngs[r].draw_step(wk.weights[r * nwalk:(r + 1) * nwalk], ham.nchol)
                             for r in range(P)])
        nlarge += step(trial, ham, prop, wk, xi, eshift, cap)
        total_weight = wk.weights.sum()
        eshift = e_est - 0.1 * np.log(total_weight / (nwalk * P)) / dt
        if st % ortho_steps == 0:
            orthogonalize(wk)
        if st % nsteps == 0:
            block = st // nsteps
            if rdm is not None and st * dt > 10.0 and st > burn_iter * nsteps:
                rdm.add(trial, wk)
            el = np.zeros(wk.nwalk)
            live = wk.weights != 0.0
            if live.any():
                sub = wk.copy()
                sub.dets = wk.dets[live]
                el[live] = local_energy(trial, sub, ham).real + delta
            dev = live & (np.abs(el - avg_e) > np.sqrt(2.0 / dt))
            nlarge += int(dev.sum())
            el = np.where(dev, np.where(el > avg_e, avg_e + np.sqrt(2.0 / dt), avg_e - np.sqrt(2.0 / dt)), el)
            tot_w[block] = total_weight
            tot_e[block] = (el * wk.weights).sum() / total_weight
            if st * dt < 10.0 or st < burn_iter * nsteps:
                num_eql += tot_e[block] * tot_w[block]
                den_eql += tot_w[block]
                avg_e_eql = num_eql / den_eql
            else:
                num += tot_e[block] * tot_w[block]
                den += tot_w[block]
                avg_e = num / den
            e_est = 0.9 * e_est + 0.1 * tot_e[block]
            # comb (MixedEstimator.cpp:583-621)
            cum = np.cumsum(wk.weights)
            total = cum[-1]
            zeta = rngs[0].uniform()
            z = (np.arange(P * nwalk) + zeta) / nwalk / P
            index = np.searchsorted(cum, z * total, side="left")
            wk.dets = wk.dets[index]
            wk.overlaps = wk.overlaps[index]
            wk.weights = np.full(P * nwalk, total / P / nwalk)
    info = {"nchol_ene": nchol_ene, "delta": delta, "e_ref": e_ref, "nlarge": nlarge}
    if rdm is not None:
        info.update(one_rdm=rdm.rdm, rdm_weight=rdm.cum)
    return tot_w, tot_e, info
