"""Host-side mirror of the reference's DQMC objects over the C ABI (include/afqmc.h).

``Hamiltonian``, ``RHF`` / ``UHF`` and ``DQMCWalkers`` follow the reference's
DQMC/Hamiltonian.h:8-22, DQMC/RHF.cpp, DQMC/UHF.cpp and DQMC/DQMCWalker.h:7-46,
batched: one ``DQMCWalkers`` object holds every walker of a rank on the GPU and
each method acts on all of them at once (the per-walker loops of
DQMC/MixedEstimator.cpp:398-416, :461-468, :478-480, :489-533 become one call).

All arithmetic runs in the CUDA library ``_lib/libafqmc_gb300.so`` (built by
``vmc_gb300.build``); there is no CPU fallback.  Loading fails with an error
when the library is absent.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libafqmc_gb300.so")

AFQMC_OK = 0
ERRORS = {1: "ARG", 2: "CUDA", 3: "NAN", 4: "TIMEOUT", 5: "UNSUPPORTED", 6: "STATE"}
INT_R, INT_U = 0, 1
TRIAL_RHF, TRIAL_UHF = 0, 1
PRECISION = {"fp64": 0, "mixed": 1, "ref32": 2}


class AfqmcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("afqmc error %s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class _Ham(ctypes.Structure):
    _fields_ = [("norb", ctypes.c_int), ("nalpha", ctypes.c_int), ("nbeta", ctypes.c_int),
                ("nchol", ctypes.c_int), ("int_type", ctypes.c_int), ("ecore", ctypes.c_double),
                ("h1", ctypes.c_void_p), ("h1mod", ctypes.c_void_p), ("chol", ctypes.c_void_p)]


class _Trial(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("phi_a", ctypes.c_void_p), ("phi_b", ctypes.c_void_p)]


class _Opts(ctypes.Structure):
    _fields_ = [("nwalk", ctypes.c_int), ("rhf_walker", ctypes.c_int), ("precision", ctypes.c_int),
                ("device", ctypes.c_int), ("dt", ctypes.c_double), ("ref_a", ctypes.c_void_p),
                ("ref_b", ctypes.c_void_p), ("green", ctypes.c_void_p), ("weight_cap", ctypes.c_double),
                ("pop_target", ctypes.c_double), ("seed", ctypes.c_uint64)]


_lib = None


def lib():
    """The loaded CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("CUDA library %s not built: run python -m vmc_gb300.build" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        L.afqmc_last_error.restype = ctypes.c_char_p
        L.afqmc_last_error.argtypes = [vp]
        L.afqmc_create.argtypes = [ctypes.POINTER(_Ham), ctypes.POINTER(_Trial), ctypes.POINTER(_Opts),
                                   ctypes.POINTER(vp)]
        for name, args in [("afqmc_destroy", [vp]),
                           ("afqmc_sizes", [vp] + [ctypes.POINTER(ip)] * 5),
                           ("afqmc_set_walkers", [vp, vp, vp, vp]),
                           ("afqmc_get_walkers", [vp, vp, vp, vp]),
                           ("afqmc_force_bias", [vp, vp]),
                           ("afqmc_step", [vp, vp, vp]),
                           ("afqmc_set_energy_estimate", [vp, ctypes.c_double, vp]),
                           ("afqmc_population", [vp, dp, dp, ctypes.POINTER(ctypes.c_long)]),
                           ("afqmc_orthonormalize", [vp]),
                           ("afqmc_set_nchol_ene", [vp, ip]),
                           ("afqmc_local_energy", [vp, vp]),
                           ("afqmc_prop_info", [vp, vp, vp, vp]),
                           ("afqmc_enable_timing", [vp, ip]),
                           ("afqmc_stage_time", [vp, ctypes.c_char_p, dp]),
                           ("afqmc_launch_count", [vp, ctypes.POINTER(ctypes.c_long)]),
                           ("afqmc_sync", [vp]),
                           ("afqmc_check_wait_timeout", [vp]),
                           ("afqmc_rdm_enable", [vp, ip]),
                           ("afqmc_rdm_reset", [vp]),
                           ("afqmc_rdm_accumulate", [vp]),
                           ("afqmc_timer_start", [vp]),
                           ("afqmc_timer_stop", [vp, dp]),
                           ("afqmc_run", [vp, ctypes.POINTER(_RunOpts), vp, vp, ctypes.POINTER(_RunStats)]),
                           ("afqmc_refrng_draw_step", [vp, vp, ip, vp])]:
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.afqmc_refrng_create.restype = vp
        L.afqmc_refrng_create.argtypes = [ctypes.c_uint, ip]
        L.afqmc_refrng_destroy.restype = None
        L.afqmc_refrng_destroy.argtypes = [vp]
        L.afqmc_refrng_uniform.restype = ctypes.c_double
        L.afqmc_refrng_uniform.argtypes = [vp]
        _lib = L
    return _lib


class _RunOpts(ctypes.Structure):
    _fields_ = [("nprocs", ctypes.c_int), ("nsteps", ctypes.c_int), ("nsweeps", ctypes.c_int),
                ("ortho_steps", ctypes.c_int), ("burn_iter", ctypes.c_int), ("seed", ctypes.c_uint),
                ("field_source", ctypes.c_int), ("comb", ctypes.c_int),
                ("cholesky_threshold", ctypes.c_double), ("max_steps", ctypes.c_long),
                ("device_blocks", ctypes.c_int)]


class _RunStats(ctypes.Structure):
    _fields_ = [("nchol_ene", ctypes.c_int), ("delta", ctypes.c_double), ("e_ref", ctypes.c_double),
                ("n_large_deviations", ctypes.c_long)]


class RefRNG:
    """One emulated rank's reference-order field stream (afqmc_refrng_*)."""

    def __init__(self, seed, nwalk):
        self.L = lib()
        self.h = self.L.afqmc_refrng_create(int(seed), int(nwalk))
        self.nwalk = nwalk

    def draw_step(self, weights, nfields):
        out = np.zeros((self.nwalk, nfields))
        w = np.ascontiguousarray(weights, dtype=np.float64)
        rc = self.L.afqmc_refrng_draw_step(self.h, w.ctypes.data, int(nfields), out.ctypes.data)
        if rc != AFQMC_OK:
            raise AfqmcError(rc, "refrng_draw_step")
        return out

    def uniform(self):
        return self.L.afqmc_refrng_uniform(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.afqmc_refrng_destroy(self.h)
            self.h = None


def _ptr(a):
    return None if a is None else a.ctypes.data


class Hamiltonian:
    """DQMC/Hamiltonian.h:8-22: one-body h1, h1Mod, Cholesky vectors, ecore.

    ``chol[g, i, j]`` is the reference's ``chol[g](i, j)``.  For ``int_type="u"``
    pass ``h1``/``h1mod`` of shape (2, N, N) and ``chol`` of shape (2, G, N, N)."""

    def __init__(self, norb, nalpha, nbeta, ecore, h1, h1mod, chol, int_type="r"):
        self.norb, self.nalpha, self.nbeta = int(norb), int(nalpha), int(nbeta)
        self.ecore = float(ecore)
        self.int_type = int_type
        nsp = 1 if int_type == "r" else 2
        N = self.norb
        self.h1 = np.ascontiguousarray(np.asarray(h1, dtype=np.float64).reshape(nsp, N, N))
        self.h1mod = np.ascontiguousarray(np.asarray(h1mod, dtype=np.float64).reshape(nsp, N, N))
        chol = np.asarray(chol, dtype=np.float64)
        self.nchol = chol.shape[-3]
        self.chol = np.ascontiguousarray(chol.reshape(nsp, self.nchol, N, N))


class RHF:
    """Restricted left trial (DQMC/RHF.cpp:9-17): first nalpha columns of rhf.txt."""
    kind = TRIAL_RHF

    def __init__(self, ham, phi):
        self.phi_a = np.ascontiguousarray(np.asarray(phi, dtype=np.float64)[:, :ham.nalpha])
        self.phi_b = self.phi_a[:, :ham.nbeta].copy()


class UHF:
    """Unrestricted left trial (DQMC/UHF.cpp): alpha and beta orbital blocks."""
    kind = TRIAL_UHF

    def __init__(self, ham, phi_a, phi_b):
        self.phi_a = np.ascontiguousarray(np.asarray(phi_a, dtype=np.float64)[:, :ham.nalpha])
        self.phi_b = np.ascontiguousarray(np.asarray(phi_b, dtype=np.float64)[:, :ham.nbeta])


class DQMCWalkers:
    """All walkers of one rank on the GPU (batched DQMC/DQMCWalker.h:7-46).

    ``rhf_walker``: one spin determinant per walker (``DQMCWalker(true, ...)``).
    ``ref``: (ref_a, ref_b) reference determinants for the mean-field shifts
    (the rhf.txt/uhf.txt blocks of DQMC/MixedEstimator.cpp:338-350); default the trial.
    ``precision``: "fp64", "mixed" or "ref32" (the reference's own FP32 VHS).
    """

    def __init__(self, ham, trial, nwalk, rhf_walker, dt, precision="fp64", ref=None, green=None,
                 weight_cap=-1.0, pop_target=-1.0, seed=12345, device=0):
        L = lib()
        self.ham, self.trial = ham, trial
        self.nwalk, self.rhf_walker = int(nwalk), bool(rhf_walker)
        self.precision = precision
        self._keep = []
        h = _Ham(ham.norb, ham.nalpha, ham.nbeta, ham.nchol, INT_R if ham.int_type == "r" else INT_U,
                 ham.ecore, _ptr(ham.h1), _ptr(ham.h1mod), _ptr(ham.chol))
        t = _Trial(trial.kind, _ptr(trial.phi_a), _ptr(trial.phi_b))
        ref_a = ref_b = None
        if ref is not None:
            ref_a = np.ascontiguousarray(np.asarray(ref[0], dtype=np.float64)[:, :ham.nalpha])
            ref_b = np.ascontiguousarray(np.asarray(ref[1], dtype=np.float64)[:, :ham.nbeta])
        g = None if green is None else np.ascontiguousarray(green, dtype=np.float64)
        self._keep += [ref_a, ref_b, g]
        o = _Opts(self.nwalk, int(self.rhf_walker), PRECISION[precision], int(device), float(dt),
                  _ptr(ref_a), _ptr(ref_b), _ptr(g), float(weight_cap), float(pop_target), int(seed))
        hp = ctypes.c_void_p()
        rc = L.afqmc_create(ctypes.byref(h), ctypes.byref(t), ctypes.byref(o), ctypes.byref(hp))
        if rc != AFQMC_OK:
            raise AfqmcError(rc, L.afqmc_last_error(None).decode())
        self.h = hp
        self.ser = ham.norb * (ham.nalpha + ham.nbeta)

    def _check(self, rc):
        if rc != AFQMC_OK:
            raise AfqmcError(rc, lib().afqmc_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().afqmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- walker state (DQMCWalker::setDet / getDet, DQMCWalker.cpp:251-290) ---
    def set_det(self, dets, overlaps=None, weights=None):
        """dets: (W, N, ncols) complex (alpha columns then beta) or serial (W, N*(na+nb))."""
        d = np.asarray(dets, dtype=np.complex128)
        if d.ndim == 3:
            d = self.to_serial(d)
        d = np.ascontiguousarray(d.reshape(self.nwalk, self.ser))
        o = None if overlaps is None else np.ascontiguousarray(overlaps, dtype=np.complex128)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        self._check(lib().afqmc_set_walkers(self.h, _ptr(d), _ptr(o), _ptr(w)))

    def get_det(self):
        d = np.zeros((self.nwalk, self.ser), np.complex128)
        o = np.zeros(self.nwalk, np.complex128)
        w = np.zeros(self.nwalk)
        self._check(lib().afqmc_get_walkers(self.h, _ptr(d), _ptr(o), _ptr(w)))
        return self.from_serial(d), o, w

    def weights(self):
        """The walker weights alone (no determinant copy)."""
        w = np.zeros(self.nwalk)
        self._check(lib().afqmc_get_walkers(self.h, None, None, _ptr(w)))
        return w

    def to_serial(self, d):
        N, na, nb = self.ham.norb, self.ham.nalpha, self.ham.nbeta
        a = d[:, :, :na]
        b = d[:, :, :nb] if self.rhf_walker else d[:, :, na:na + nb]
        return np.concatenate([a.reshape(len(d), -1), b.reshape(len(d), -1)], axis=1)

    def from_serial(self, s):
        N, na, nb = self.ham.norb, self.ham.nalpha, self.ham.nbeta
        a = s[:, :N * na].reshape(-1, N, na)
        if self.rhf_walker:
            return a
        b = s[:, N * na:].reshape(-1, N, nb)
        return np.concatenate([a, b], axis=2)

    # --- trial contractions ---
    def force_bias(self):
        fb = np.zeros((self.nwalk, self.ham.nchol), np.complex128)
        self._check(lib().afqmc_force_bias(self.h, _ptr(fb)))
        return fb

    def ham_and_overlap(self):
        """Local energies E_L (complex, one per walker); hamAndOverlap[0]/[1]."""
        e = np.zeros(self.nwalk, np.complex128)
        self._check(lib().afqmc_local_energy(self.h, _ptr(e)))
        return e

    local_energy = ham_and_overlap

    def set_nchol_ene(self, n):
        self._check(lib().afqmc_set_nchol_ene(self.h, int(n)))

    # --- propagation ---
    def propagate_phaseless(self, xi=None, eshift=None):
        """One step of every live walker; xi (W, G) host normals or None (device RNG)."""
        x = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        e = None if eshift is None else np.array([eshift], dtype=np.float64)
        self._check(lib().afqmc_step(self.h, _ptr(x), _ptr(e)))

    def orthogonalize(self):
        self._check(lib().afqmc_orthonormalize(self.h))

    def comb(self, zeta, nprocs=1):
        """Comb reconfiguration on the device (MixedEstimator.cpp:583-621)."""
        L = lib()
        L.afqmc_comb.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        self._check(L.afqmc_comb(self.h, float(zeta), int(nprocs)))

    def block_setup(self, nsteps, e_est, avg_e=None, delta=0.0, burn_steps=0, zetas=None, nprocs=1):
        """Start device-resident blocks (afqmc_block_setup)."""
        L = lib()
        L.afqmc_block_setup.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_long, ctypes.c_void_p,
                                        ctypes.c_int]
        z = None if zetas is None else np.ascontiguousarray(zetas, dtype=np.float64)
        self._check(L.afqmc_block_setup(self.h, int(nprocs), int(nsteps), float(e_est),
                                        float(e_est if avg_e is None else avg_e), float(delta), int(burn_steps),
                                        _ptr(z), 0 if z is None else len(z)))

    def block_end(self, comb=True):
        L = lib()
        L.afqmc_block_end.argtypes = [ctypes.c_void_p, ctypes.c_int]
        self._check(L.afqmc_block_end(self.h, int(bool(comb))))

    def block_results(self, nblocks):
        """(total_weights, block energies, clamped local energies) of the first nblocks blocks."""
        L = lib()
        L.afqmc_block_results.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.POINTER(ctypes.c_long)]
        tw, te, n = np.zeros(nblocks), np.zeros(nblocks), ctypes.c_long()
        self._check(L.afqmc_block_results(self.h, int(nblocks), tw.ctypes.data, te.ctypes.data, ctypes.byref(n)))
        return tw, te, n.value

    def set_energy_estimate(self, e_est, eshift=None):
        e = None if eshift is None else np.array([eshift], dtype=np.float64)
        self._check(lib().afqmc_set_energy_estimate(self.h, float(e_est), _ptr(e)))

    def population(self):
        s, e, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
        self._check(lib().afqmc_population(self.h, ctypes.byref(s), ctypes.byref(e), ctypes.byref(n)))
        return s.value, e.value, n.value

    def prop_info(self):
        G, N = self.ham.nchol, self.ham.norb
        nsp = 1 if self.ham.int_type == "r" else 2
        mf = np.zeros(G, np.complex128)
        pc = np.zeros(1, np.complex128)
        ex = np.zeros((nsp, N, N), np.complex128)
        self._check(lib().afqmc_prop_info(self.h, _ptr(mf), _ptr(pc), _ptr(ex)))
        return mf, pc[0], ex

    def enable_timing(self, on=True):
        self._check(lib().afqmc_enable_timing(self.h, int(on)))

    def stage_time(self, stage):
        ms = ctypes.c_double()
        self._check(lib().afqmc_stage_time(self.h, stage.encode(), ctypes.byref(ms)))
        return ms.value

    def walker_steps(self):
        """Walker-steps propagated so far (live walkers only; afqmc_walker_steps)."""
        v = ctypes.c_double()
        L = lib()
        L.afqmc_walker_steps.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        self._check(L.afqmc_walker_steps(self.h, ctypes.byref(v)))
        return v.value

    def launch_count(self):
        c = ctypes.c_long()
        self._check(lib().afqmc_launch_count(self.h, ctypes.byref(c)))
        return c.value

    def sync(self):
        self._check(lib().afqmc_sync(self.h))

    # --- mixed 1-RDM estimator (MixedEstimator.cpp:488-510) ---
    def rdm_enable(self, on=True):
        self._check(lib().afqmc_rdm_enable(self.h, int(bool(on))))

    def rdm_reset(self):
        self._check(lib().afqmc_rdm_reset(self.h))

    def rdm_accumulate(self):
        self._check(lib().afqmc_rdm_accumulate(self.h))

    def rdm(self):
        """(rdm, cumulative weight): rdm (1, N, N) spin-summed for restricted
        integrals, (2, N, N) up / down for unrestricted ones."""
        N = self.ham.norb
        nout = 1 if self.ham.int_type == "r" else 2
        r = np.zeros((nout, N, N))
        cw = ctypes.c_double()
        L = lib()
        L.afqmc_rdm_get.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        self._check(L.afqmc_rdm_get(self.h, r.ctypes.data, ctypes.byref(cw)))
        return r, cw.value

    def check_wait_timeout(self):
        """Run one bounded device wait that nothing completes (afqmc_check_wait_timeout);
        returns the status code (AFQMC_ERR_TIMEOUT = 4 expected) and the message."""
        rc = lib().afqmc_check_wait_timeout(self.h)
        return rc, (lib().afqmc_last_error(self.h) or b"").decode()

    def timer_start(self):
        self._check(lib().afqmc_timer_start(self.h))

    def timer_stop(self):
        ms = ctypes.c_double()
        self._check(lib().afqmc_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value

    def run(self, nsteps=50, nsweeps=50, ortho_steps=20, seed=4321, nprocs=1, burn_iter=0,
            field_source="reference", comb=True, cholesky_threshold=1e-3, max_steps=0, device_blocks=False,
            block_info=False):
        """calcMixedEstimatorLongProp from the current walkers (DQMC/MixedEstimator.cpp:309-660).

        Returns (total_weights, total_energies, stats) -- the samples.dat columns.
        block_info: stats also holds "eshift" and "walltime" per block (the other
        afqmc.dat columns; inputs.write_afqmc_dat)."""
        o = _RunOpts(int(nprocs), int(nsteps), int(nsweeps), int(ortho_steps), int(burn_iter), int(seed),
                     0 if field_source == "reference" else 1, int(bool(comb)), float(cholesky_threshold),
                     int(max_steps), int(bool(device_blocks)))
        tw = np.zeros(nsweeps)
        te = np.zeros(nsweeps)
        st = _RunStats()
        if block_info:
            es, wl = np.zeros(nsweeps), np.zeros(nsweeps)
            L = lib()
            L.afqmc_run_blocks.argtypes = [ctypes.c_void_p, ctypes.POINTER(_RunOpts)] + [ctypes.c_void_p] * 4 + \
                [ctypes.POINTER(_RunStats)]
            self._check(L.afqmc_run_blocks(self.h, ctypes.byref(o), tw.ctypes.data, te.ctypes.data, es.ctypes.data,
                                           wl.ctypes.data, ctypes.byref(st)))
        else:
            self._check(lib().afqmc_run(self.h, ctypes.byref(o), tw.ctypes.data, te.ctypes.data,
                                        ctypes.byref(st)))
        out = dict(nchol_ene=st.nchol_ene, delta=st.delta, e_ref=st.e_ref, n_large_deviations=st.n_large_deviations)
        if block_info:
            out.update(eshift=es, walltime=wl)
        return tw, te, out


def from_reference_inputs(ham_arrays, trials, cfg, nprocs=1, precision="ref32", device=0, green=None):
    """Build ``DQMCWalkers`` the way executables/DQMC.cpp:74-153 does for the
    RHF/UHF phaseless path.

    ham_arrays: dict with norb, nalpha, nbeta, ecore and h1/h1mod/chol (int "r")
    or h1u/h1umod/cholu (int "u"), ``chol[g, i, j]`` = reference ``chol[g](i, j)``.
    trials: {"rhf": ("rhf", phi)} and/or {"uhf": ("uhf", phi_a, phi_b)} -- the
    rhf.txt / uhf.txt contents.  cfg: the afqmc.json dict.  The left trial is
    cfg["wavefunction"]["left"]; the walkers start at the right trial's
    determinant (waveRight.getSample); the mean-field reference is rhf.txt for
    the restricted walker and uhf.txt otherwise (MixedEstimator.cpp:338-350).
    green: optional [2][norb][norb] mean-field Green's function replacing the
    reference determinant's in the mean-field shifts (the spinRDM.0.0.txt
    override, DQMCWalker.cpp:39-58; inputs.read_spin_rdm)."""
    left = trials[cfg["wavefunction"]["left"]]
    right = trials[cfg["wavefunction"]["right"]]
    it = cfg["system"].get("intType", "r")
    if it == "r":
        ham = Hamiltonian(ham_arrays["norb"], ham_arrays["nalpha"], ham_arrays["nbeta"], ham_arrays["ecore"],
                          ham_arrays["h1"], ham_arrays["h1mod"], ham_arrays["chol"])
    else:
        ham = Hamiltonian(ham_arrays["norb"], ham_arrays["nalpha"], ham_arrays["nbeta"], ham_arrays["ecore"],
                          ham_arrays["h1u"], ham_arrays["h1umod"], ham_arrays["cholu"], int_type="u")

    def mk(t):
        return RHF(ham, t[1]) if t[0] == "rhf" else UHF(ham, t[1], t[2])

    s = cfg["sampling"]
    rhf_walker = ham.nalpha == ham.nbeta and right[0] != "uhf"
    ref_t = mk(trials["rhf" if rhf_walker else "uhf"])
    nwalk = int(s.get("nwalk", 100))
    wk = DQMCWalkers(ham, mk(left), nwalk * nprocs, rhf_walker, float(s.get("dt", 0.1)), precision=precision,
                     ref=(ref_t.phi_a, ref_t.phi_b), green=green, weight_cap=max(100.0, nwalk / 10.0),
                     pop_target=nwalk * nprocs, device=device)
    rt = mk(right)
    init = np.concatenate([rt.phi_a, rt.phi_b], axis=1) if not rhf_walker else rt.phi_a
    wk.set_det(np.repeat(init[None].astype(np.complex128), nwalk * nprocs, axis=0))
    return wk


# ---------------------------------------------------------------------------
# learned control variate
# ---------------------------------------------------------------------------
CV_NF = 67


def _bind_cv(L):
    if getattr(L, "_cv_bound", False):
        return
    vp, ip = ctypes.c_void_p, ctypes.c_int
    for name, args in [("afqmc_mlp_create", [ip, ip, ip, ip, ctypes.c_uint64, ctypes.POINTER(vp)]),
                       ("afqmc_mlp_destroy", [vp]),
                       ("afqmc_mlp_nparams", [vp, ctypes.POINTER(ctypes.c_long)]),
                       ("afqmc_mlp_params", [vp, vp, vp]),
                       ("afqmc_mlp_loss_grad", [vp, vp, vp, ip, ctypes.POINTER(ctypes.c_double), vp]),
                       ("afqmc_mlp_predict", [vp, vp, ip, vp]),
                       ("afqmc_mlp_train", [vp, vp, vp, ip, ip, ip, ctypes.c_float, ctypes.c_uint64,
                                            ctypes.POINTER(ctypes.c_double)]),
                       ("afqmc_cv_features", [vp, vp]),
                       ("afqmc_local_energy_subset", [vp, vp, ip, vp]),
                       ("afqmc_cv_attach", [vp, vp, vp, vp, ctypes.c_float, ctypes.c_float, ip]),
                       ("afqmc_cv_measure", [vp, ctypes.c_uint64, ip]),
                       ("afqmc_cv_results", [vp, vp, ip]),
                       ("afqmc_cv_result_post", [vp, ip]),
                       ("afqmc_cv_result_take", [vp, vp])]:
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.afqmc_mlp_last_error.restype = ctypes.c_char_p
    L.afqmc_mlp_last_error.argtypes = [vp]
    L._cv_bound = True


class MLP:
    """GPU MLP n_in -> hidden -> hidden -> 1 (SiLU), trained by the library's kernels."""

    def __init__(self, n_in=CV_NF, hidden=256, max_batch=4096, seed=1, device=0):
        L = lib()
        _bind_cv(L)
        h = ctypes.c_void_p()
        rc = L.afqmc_mlp_create(n_in, hidden, max_batch, device, seed, ctypes.byref(h))
        if rc != AFQMC_OK:
            raise AfqmcError(rc, "afqmc_mlp_create")
        self.h, self.n_in, self.hidden = h, n_in, hidden
        n = ctypes.c_long()
        L.afqmc_mlp_nparams(h, ctypes.byref(n))
        self.nparams = n.value

    def _check(self, rc):
        if rc != AFQMC_OK:
            raise AfqmcError(rc, lib().afqmc_mlp_last_error(self.h).decode())

    def get_params(self):
        p = np.zeros(self.nparams, np.float32)
        self._check(lib().afqmc_mlp_params(self.h, p.ctypes.data, None))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(lib().afqmc_mlp_params(self.h, None, p.ctypes.data))

    def split(self, p):
        """Flat parameters -> [W1, b1, W2, b2, w3, b3]."""
        H, I = self.hidden, self.n_in
        o = [0, H * I, H * I + H, H * I + H + H * H, H * I + 2 * H + H * H, H * I + 3 * H + H * H]
        return [p[o[0]:o[1]].reshape(H, I), p[o[1]:o[2]], p[o[2]:o[3]].reshape(H, H), p[o[3]:o[4]],
                p[o[4]:o[5]], p[o[5]:o[5] + 1]]

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = ctypes.c_double()
        g = np.zeros(self.nparams, np.float32)
        self._check(lib().afqmc_mlp_loss_grad(self.h, x.ctypes.data, t.ctypes.data, len(t), ctypes.byref(loss),
                                              g.ctypes.data))
        return loss.value, g

    def predict(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros(len(x), np.float32)
        self._check(lib().afqmc_mlp_predict(self.h, x.ctypes.data, len(x), y.ctypes.data))
        return y

    def train(self, x, t, epochs=20, batch=256, lr=1e-3, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(lib().afqmc_mlp_train(self.h, x.ctypes.data, t.ctypes.data, len(t), epochs, batch, lr, seed,
                                          ctypes.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            lib().afqmc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cv_features(wk):
    L = lib()
    _bind_cv(L)
    f = np.zeros((wk.nwalk, CV_NF), np.float32)
    wk._check(L.afqmc_cv_features(wk.h, f.ctypes.data))
    return f


def local_energy_subset(wk, idx):
    L = lib()
    _bind_cv(L)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    e = np.zeros(len(idx), np.complex128)
    wk._check(L.afqmc_local_energy_subset(wk.h, idx.ctypes.data, len(idx), e.ctypes.data))
    return e


class StepGraph:
    """nsteps device-field steps of one or several DQMCWalkers as one CUDA graph
    (afqmc_graph_*): each replay advances every system by nsteps."""

    def __init__(self, walkers, nsteps, ortho_every=5, cv_every=0, block_end=None):
        """block_end: None (steps only), or "measure" / "comb" to end each
        replay with the device-resident block end (afqmc_graph_capture_blocks)."""
        L = lib()
        vp = ctypes.c_void_p
        L.afqmc_graph_capture.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(vp)]
        L.afqmc_graph_capture_blocks.argtypes = L.afqmc_graph_capture.argtypes
        L.afqmc_graph_launch.argtypes = [vp]
        L.afqmc_graph_destroy.argtypes = [vp]
        L.afqmc_graph_nodes.argtypes = [vp, ctypes.POINTER(ctypes.c_long)]
        L.afqmc_graph_last_error.restype = ctypes.c_char_p
        self.walkers = list(walkers)
        arr = (vp * len(self.walkers))(*[w.h for w in self.walkers])
        g = vp()
        if block_end is None:
            rc = L.afqmc_graph_capture(arr, len(self.walkers), nsteps, ortho_every, cv_every, ctypes.byref(g))
        else:
            rc = L.afqmc_graph_capture_blocks(arr, len(self.walkers), nsteps, ortho_every,
                                              1 if block_end == "comb" else 0, ctypes.byref(g))
        if rc != AFQMC_OK:
            raise AfqmcError(rc, L.afqmc_graph_last_error().decode())
        self.g = g
        self.nsteps = nsteps

    def launch(self):
        rc = lib().afqmc_graph_launch(self.g)
        if rc != AFQMC_OK:
            raise AfqmcError(rc, lib().afqmc_graph_last_error().decode())

    def nodes(self):
        n = ctypes.c_long()
        lib().afqmc_graph_nodes(self.g, ctypes.byref(n))
        return n.value

    def close(self):
        if getattr(self, "g", None):
            lib().afqmc_graph_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(wk, cache_path=None):
    """Run the library's autotuner on a DQMCWalkers handle; returns (choices, report)."""
    L = lib()
    L.afqmc_autotune.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
    L.afqmc_tuning.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 5
    buf = ctypes.create_string_buffer(2048)
    wk._check(L.afqmc_autotune(wk.h, cache_path.encode() if cache_path else None, buf, 2048))
    v = [ctypes.c_int() for _ in range(5)]
    L.afqmc_tuning(wk.h, *[ctypes.byref(x) for x in v])
    return (dict(bn_fb=v[0].value, bn_vhs=v[1].value, prop=v[2].value, ovl=v[3].value, qr=v[4].value),
            buf.value.decode())


PROP_VARIANTS = {"smem": 1, "chunked": 2, "tensor": 3, "tensor_mn": 4}
QR_VARIANTS = {"householder": 1, "cholesky": 2}


def set_tuning(wk, bn_fb=0, bn_vhs=0, prop=0, ovl=0, qr=0):
    """Choose kernel variants directly (0 keeps the current choice); `prop` and
    `qr` may be names of PROP_VARIANTS / QR_VARIANTS.  Raises on a choice the
    handle cannot run."""
    L = lib()
    L.afqmc_set_tuning.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 5
    prop = PROP_VARIANTS.get(prop, prop)
    qr = QR_VARIANTS.get(qr, qr)
    wk._check(L.afqmc_set_tuning(wk.h, bn_fb, bn_vhs, prop, ovl, qr))
