/*
 * afqmc.h -- C ABI of the GB300-native phaseless AFQMC walker step.
 *
 * One handle = one system (Hamiltonian + left trial) and one batch of walkers
 * resident on one GPU.  Every entry point returns an int status
 * (AFQMC_OK = 0); afqmc_last_error() gives the message.  Nothing calls exit().
 * A handle is used by one host thread at a time; its work runs in order on the
 * handle's own CUDA stream, and every call returns after that work finished
 * unless its comment says otherwise.
 *
 * Interfaces replaced (reference paths are relative to the reference checkout):
 *   Hamiltonian ctor + floattenCholesky + rotateCholesky
 *       DQMC/Hamiltonian.cpp:9-42, :179-219, :52-133   -> afqmc_create
 *   RHF / UHF left trial (Wavefunction plug-in)
 *       DQMC/Wavefunction.h:7-20, DQMC/RHF.cpp:9-17, DQMC/UHF.cpp -> afqmc_trial
 *   DQMCWalker::prepProp (mean-field shifts, exp(-dt/2 h1'))
 *       DQMC/DQMCWalker.cpp:32-103, :106-187            -> afqmc_create
 *   DQMCWalker::setDet / getDet (serial layout)
 *       DQMC/DQMCWalker.cpp:251-290                      -> afqmc_set_walkers / afqmc_get_walkers
 *   DQMCWalker::forceBias -> RHF/UHF::forceBias
 *       DQMC/DQMCWalker.cpp:569-576, DQMC/RHF.cpp:42-61  -> afqmc_force_bias
 *   the per-walker loop of propagatePhaseless + weight update and cap
 *       DQMC/MixedEstimator.cpp:461-468, DQMC/DQMCWalker.cpp:441-554 -> afqmc_step
 *   population-control shift
 *       DQMC/MixedEstimator.cpp:472-475                  -> afqmc_step (device eshift)
 *   DQMCWalker::orthogonalize
 *       DQMC/DQMCWalker.cpp:295-326                      -> afqmc_orthonormalize
 *   DQMCWalker::hamAndOverlap -> RHF/UHF::hamAndOverlap
 *       DQMC/DQMCWalker.cpp:592-601, DQMC/RHF.cpp:70-131 -> afqmc_local_energy
 *   Hamiltonian::setNcholEne
 *       DQMC/Hamiltonian.cpp:45-48                       -> afqmc_set_nchol_ene
 */
#ifndef AFQMC_GB300_H
#define AFQMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define AFQMC_OK 0
#define AFQMC_ERR_ARG 1          /* bad argument or size */
#define AFQMC_ERR_CUDA 2         /* a CUDA runtime call failed */
#define AFQMC_ERR_NAN 3          /* non-finite local energy */
#define AFQMC_ERR_TIMEOUT 4      /* a bounded device wait gave up */
#define AFQMC_ERR_UNSUPPORTED 5  /* combination not implemented */
#define AFQMC_ERR_STATE 6        /* call made in the wrong state */

/* integral type: DQMC/Hamiltonian.cpp:20-31 ("r" restricted, "u" unrestricted) */
#define AFQMC_INT_R 0
#define AFQMC_INT_U 1

/* left-trial kind */
#define AFQMC_TRIAL_RHF 0
#define AFQMC_TRIAL_UHF 1

/* arithmetic of the step */
#define AFQMC_PREC_FP64 0   /* everything in FP64 (the FP64 oracle's algorithm) */
#define AFQMC_PREC_MIXED 1  /* tensor-core Cholesky contractions, FP32 propagator, FP64 QR/LU/weights */
#define AFQMC_PREC_REF32 2  /* FP64 except the reference's own FP32 parts: FP32 VHS from the
                               FP32 packed Cholesky copy with complex<float> fields, and
                               mean-field shifts from that FP32 copy (DQMCWalker.cpp:72-84, :406-421) */

typedef struct afqmc_ham {
  int norb, nalpha, nbeta, nchol;
  int int_type;        /* AFQMC_INT_R or AFQMC_INT_U */
  double ecore;
  /* nsp = 1 (INT_R) or 2 (INT_U: up then down) */
  const double* h1;    /* [nsp][norb][norb] row-major */
  const double* h1mod; /* [nsp][norb][norb] row-major, h1 - 1/2 sum_g L_g L_g */
  const double* chol;  /* [nsp][nchol][norb][norb]; chol[g][i][j] = reference chol[g](i, j) */
} afqmc_ham;

typedef struct afqmc_trial {
  int kind;            /* AFQMC_TRIAL_RHF or AFQMC_TRIAL_UHF */
  const double* phi_a; /* [norb][nalpha] row-major real orbitals */
  const double* phi_b; /* [norb][nbeta]  (UHF only; RHF uses the first nbeta columns of phi_a) */
} afqmc_trial;

typedef struct afqmc_opts {
  int nwalk;           /* walkers in this handle */
  int rhf_walker;      /* 1: one spin det per walker (DQMCWalker(true, ...)); 0: two */
  int precision;       /* AFQMC_PREC_* */
  int device;          /* CUDA device ordinal */
  double dt;
  const double* ref_a; /* mean-field reference det [norb][nalpha] (rhf.txt / uhf.txt block);
                          NULL: the trial's orbitals */
  const double* ref_b; /* [norb][nbeta]; NULL with ref_a set: first nbeta columns of ref_a */
  const double* green; /* optional [2][norb][norb] mean-field Green's function (the reference's
                          spinRDM.0.0.txt override, DQMCWalker.cpp:39-58); NULL: from ref */
  double weight_cap;   /* <= 0: max(100, nwalk / 10) as MixedEstimator.cpp:452-454 */
  double pop_target;   /* walkers of the whole population (nwalk x ranks); <= 0: nwalk */
  uint64_t seed;       /* device Philox seed for fields when no host fields are given */
} afqmc_opts;

typedef struct afqmc_handle afqmc_handle;

/* Message of the last failure of h (or of the last failed afqmc_create if h is NULL). */
const char* afqmc_last_error(const afqmc_handle* h);

int afqmc_create(const afqmc_ham* ham, const afqmc_trial* trial, const afqmc_opts* opts,
                 afqmc_handle** out);
int afqmc_destroy(afqmc_handle* h);

/* Sizes: serial det length N*(nalpha+nbeta) per walker, as DQMCWalker::getDet. */
int afqmc_sizes(const afqmc_handle* h, int* norb, int* nalpha, int* nbeta, int* nchol, int* nwalk);

/* Walker state through host buffers (complex = interleaved re, im doubles).
 * dets:     [nwalk][N*(nalpha+nbeta)] in the reference's serial layout
 *           (row-major alpha block, then row-major beta block; DQMCWalker.cpp:272-290).
 *           For the restricted walker only the alpha block is read; both are written.
 * overlaps: [nwalk] complex; NULL on set: computed as <Psi_T|phi>.
 * weights:  [nwalk]; NULL on set: 1.  */
int afqmc_set_walkers(afqmc_handle* h, const double* dets, const double* overlaps,
                      const double* weights);
int afqmc_get_walkers(afqmc_handle* h, double* dets, double* overlaps, double* weights);

/* Force bias of every walker: fb [nwalk][nchol] complex. */
int afqmc_force_bias(afqmc_handle* h, double* fb);

/* One phaseless step of every live walker (weight > 1e-8), then the weight cap.
 * xi:     [nwalk][nchol] standard normals in host memory (rows of dead walkers
 *         ignored), or NULL to draw them on the device (Philox, key = seed).
 * eshift: if non-NULL, the energy shift for this step; if NULL, the device value
 *         left by the previous step's population control,
 *         eshift = e_estimate - 0.1 ln(sum_w / pop_target) / dt.
 * Asynchronous: returns once the work is queued on the handle's stream (and,
 * with host fields, once they have been copied, so the caller may refill its
 * buffer).  Host fields go to the device on the handle's copy stream, into one
 * of two device buffers used in turn; the copy waits only for the step two
 * back to have read that buffer, so it overlaps the previous step when the
 * caller issues this step before waiting for the previous one's results. */
int afqmc_step(afqmc_handle* h, const double* xi, const double* eshift);

/* Set the energy estimate used by the device population control, and optionally
 * the current eshift (NULL leaves it). */
int afqmc_set_energy_estimate(afqmc_handle* h, double e_estimate, const double* eshift);

/* Sum of weights after the last step, and the eshift the next step will use. */
int afqmc_population(afqmc_handle* h, double* sum_w, double* eshift_next, long* n_capped);

/* Householder QR of every walker det (all walkers, as the reference), psi <- Q,
 * overlap /= prod diag(R) (squared for the restricted walker). */
int afqmc_orthonormalize(afqmc_handle* h);

/* Number of Cholesky vectors used by the local energy (Hamiltonian::setNcholEne). */
int afqmc_set_nchol_ene(afqmc_handle* h, int nchol_ene);

/* Local energy E_L = <Psi_T|H|phi>/<Psi_T|phi> of every walker: eloc [nwalk] complex. */
int afqmc_local_energy(afqmc_handle* h, double* eloc);

/* Mean-field data from set-up: mf [nchol] complex, prop_constant (complex),
 * expm [nsp][N][N] complex row-major = exp(-dt/2 h1'_s).  Any pointer may be NULL. */
int afqmc_prop_info(afqmc_handle* h, double* mf, double* prop_constant, double* expm);

/* Milliseconds of device time of the named stage over all steps since the last
 * reset ("fb", "fields", "vhs", "prop", "overlap", "weights", "ortho", "energy"),
 * when timing was enabled with afqmc_enable_timing(h, 1). */
int afqmc_enable_timing(afqmc_handle* h, int on);
int afqmc_stage_time(afqmc_handle* h, const char* stage, double* ms);

/* Walker-steps propagated since creation: the sum over steps of the walkers
 * that were live (weight > 1e-8) when the step began; dead walkers are not
 * propagated and not counted.  Synchronises the handle's stream. */
int afqmc_walker_steps(afqmc_handle* h, double* propagated);

/* Kernels launched by this handle since creation (device work items). */
int afqmc_launch_count(const afqmc_handle* h, long* count);

/* Device-time stopwatch on the handle's stream (CUDA events): start, then stop
 * returns the milliseconds between the two points of the stream. */
int afqmc_timer_start(afqmc_handle* h);
int afqmc_timer_stop(afqmc_handle* h, double* ms);

/* Failure-detection check: runs, on the handle's stream, one bounded device
 * wait of the kind the tensor-core pipelines use (an mbarrier wait that gives
 * up after ~2 s, records a code and returns instead of hanging) on a barrier
 * that nothing arrives at.  Returns AFQMC_ERR_TIMEOUT once that wait has run
 * out, with the handle still usable; no copy or tensor memory is involved.
 * No counterpart in the reference (its CPU path has no device waits). */
int afqmc_check_wait_timeout(afqmc_handle* h);

/* Synchronise the handle's stream. */
int afqmc_sync(afqmc_handle* h);

/* ---- host driver: calcMixedEstimatorLongProp (DQMC/MixedEstimator.cpp:309-660) ---- */
typedef struct afqmc_run_opts {
  int nprocs;        /* emulated MPI ranks; the handle holds nprocs x nwalk walkers, rank r
                        owning walkers [r nwalk, (r + 1) nwalk) */
  int nsteps;        /* steps per block (sampling.nsteps) */
  int nsweeps;       /* blocks (sampling.stochasticIter) */
  int ortho_steps;   /* sampling.orthoSteps */
  int burn_iter;     /* sampling.burnIter */
  unsigned seed;     /* sampling.seed; rank r draws from std::mt19937(seed + r) */
  int field_source;  /* 0: the reference's order (host mt19937, one normal_distribution per
                        walker, dead walkers draw nothing); 1: device Philox stream */
  int comb;          /* 1: comb reconfiguration after every measurement (as the reference) */
  double cholesky_threshold;  /* sampling.choleskyThreshold (energy Cholesky truncation) */
  long max_steps;    /* > 0: stop after this many steps */
  int device_blocks; /* 1 (field_source 1 only): each block -- its steps, QR cadence, measurement and
                        comb -- is one CUDA-graph replay with all scalars on the device; needs
                        nsteps to be a multiple of ortho_steps */
} afqmc_run_opts;

typedef struct afqmc_run_stats {
  int nchol_ene;            /* Cholesky vectors used for the energy */
  double delta;             /* energy correction of the truncation */
  double e_ref;             /* energy of the reference determinant */
  long n_large_deviations;  /* capped weights + clamped local energies */
} afqmc_run_stats;

/* Run the phaseless AFQMC loop from the walkers currently in h (set them with
 * afqmc_set_walkers first, e.g. to the right trial's determinant).  Writes the
 * samples.dat columns: total_weights[nsweeps], total_energies[nsweeps]. */
int afqmc_run(afqmc_handle* h, const afqmc_run_opts* opts, double* total_weights, double* total_energies,
              afqmc_run_stats* stats);

/* afqmc_run, and per block the two other columns of the reference's afqmc.dat
 * rows (MixedEstimator.cpp:423-425, :530-544): block_eshift[nsweeps], the
 * energy shift of the measured step (row 0: the initial energy), and
 * block_wall[nsweeps], seconds since the walker set-up began (with
 * device_blocks this waits for each block).  Either pointer may be NULL. */
int afqmc_run_blocks(afqmc_handle* h, const afqmc_run_opts* opts, double* total_weights, double* total_energies,
                     double* block_eshift, double* block_wall, afqmc_run_stats* stats);

/* ---- mixed one-body reduced density matrix ----
 * The reference's weighted mixed estimate of the 1-RDM: the mean over live
 * walkers and measurements, weighted by the walker weights, of each walker's
 * sample (psi_s (Phi_s^T psi_s)^-1 Phi_s^T)^T, real part (DQMC/RHF.cpp:64-67,
 * DQMC/UHF.cpp:68-72, DQMC/MixedEstimator.cpp:488-510, written by :52-110).
 * afqmc_rdm_enable(h, 1) allocates the running sums (once) and makes afqmc_run
 * (both paths) and afqmc_block_end add every measurement after equilibration
 * (step dt > 10 and step > burnIter nsteps, counted from afqmc_block_setup on
 * the device); afqmc_rdm_accumulate adds the current walkers unconditionally
 * (asynchronous).  afqmc_rdm_get writes rdm [nout][norb][norb] row-major
 * (nout = 1, the sum over spins, for AFQMC_INT_R; 2, up then down, for
 * AFQMC_INT_U) and the cumulative weight; either pointer may be NULL.  For a
 * trial/integral pairing whose reference trial has no matching override (UHF
 * trial with restricted integrals, RHF trial with unrestricted ones), the
 * reference leaves its sample at zero; this library returns the same
 * spin-summed or per-spin estimate as for the other pairings. */
int afqmc_rdm_enable(afqmc_handle* h, int on);
int afqmc_rdm_reset(afqmc_handle* h);
int afqmc_rdm_accumulate(afqmc_handle* h);
int afqmc_rdm_get(afqmc_handle* h, double* rdm, double* cumulative_weight);

/* The reference's field order for one emulated rank: std::mt19937(seed) and nwalk
 * std::normal_distribution<double>(0, 1) objects (DQMC/DQMCWalker.h:18). */
typedef struct afqmc_refrng afqmc_refrng;
afqmc_refrng* afqmc_refrng_create(unsigned seed, int nwalk);
void afqmc_refrng_destroy(afqmc_refrng* r);
/* out[w][g] for walkers with weights[w] > 1e-8, in walker order; zeros for the others. */
int afqmc_refrng_draw_step(afqmc_refrng* r, const double* weights, int nfields, double* out);
/* std::uniform_real_distribution<double>(0, 1) draw (the comb's zeta). */
double afqmc_refrng_uniform(afqmc_refrng* r);

/* ---- learned control variate (no counterpart in the reference) ----
 * A small MLP n_in -> hidden -> hidden -> 1 (SiLU) trained on the GPU by
 * hand-written kernels (forward with BF16-rounded weights and FP32
 * accumulation, backward, Adam on FP32 master weights).  Parameters are one
 * flat FP32 array: W1 [hidden][n_in] | b1 [hidden] | W2 [hidden][hidden] |
 * b2 [hidden] | w3 [hidden] | b3 [1].  Host buffers throughout. */
typedef struct afqmc_mlp afqmc_mlp;
int afqmc_mlp_create(int n_in, int hidden, int max_batch, int device, uint64_t seed, afqmc_mlp** out);
int afqmc_mlp_destroy(afqmc_mlp* m);
const char* afqmc_mlp_last_error(const afqmc_mlp* m);
int afqmc_mlp_nparams(const afqmc_mlp* m, long* n);
/* get (non-NULL) and/or set (non-NULL) the flat parameter array */
int afqmc_mlp_params(afqmc_mlp* m, float* get, const float* set);
/* mean-squared-error loss of x [B][n_in] against t [B] and its gradient [nparams] */
int afqmc_mlp_loss_grad(afqmc_mlp* m, const float* x, const float* t, int B, double* loss, float* grad);
int afqmc_mlp_predict(afqmc_mlp* m, const float* x, int B, float* y);
/* Adam (lr) over shuffled mini-batches of a dataset x [n][n_in], t [n]; final_loss = MSE over all n */
int afqmc_mlp_train(afqmc_mlp* m, const float* x, const float* t, int n, int epochs, int batch, float lr,
                    uint64_t seed, double* final_loss);

/* Control variate on a handle (mixed precision form):
 * features of the current walkers, host [nwalk][67]: Re fb_g (g < 64), one-body
 * energy, log|overlap|, arg overlap (raw, not standardised). */
int afqmc_cv_features(afqmc_handle* h, float* feats);
/* exact local energies of the walkers idx[0..m) (host), eloc [m] complex */
int afqmc_local_energy_subset(afqmc_handle* h, const int* idx, int m, double* eloc);
/* use the trained MLP m (67 inputs, max_batch >= nwalk) with the feature mean /
 * std and target mean / std of its training set; exact energies on 1 walker of
 * every block of den */
int afqmc_cv_attach(afqmc_handle* h, afqmc_mlp* m, const float* mean, const float* stdv, float ymean, float ystd,
                    int den);
/* asynchronous control-variate measurement of the current walkers into result
 * slot `slot` (< 4096): {E_cv = sum_w w f / sum_w w + sum_S w (E - f) / sum_S w,
 * E_cv in Horvitz-Thompson form, E_subsample (Horvitz-Thompson), E_subsample
 * (ratio), sum of weights, sum of subsample weights}; `tag` seeds the subsample */
int afqmc_cv_measure(afqmc_handle* h, uint64_t tag, int slot);
int afqmc_cv_results(afqmc_handle* h, double* out, int nslots);
/* asynchronous reads of single slots, first in first out (at most 8 posted):
 * post enqueues a copy of slot `slot` after the work already issued on the
 * handle; take waits for the oldest posted copy only and writes its 6 doubles
 * to out.  A caller that issues step k + 1 (whose host fields then reach the
 * device while step k runs) before taking step k's estimate keeps the device
 * busy between steps. */
int afqmc_cv_result_post(afqmc_handle* h, int slot);
int afqmc_cv_result_take(afqmc_handle* h, double* out);

/* ---- autotuner ----
 * Time the candidate tile shapes and kernel variants of this handle's size class
 * on its own data (tensor-core GEMM N-tiles 64/128/256 for the force bias and
 * the VHS, propagator with V in shared memory or column-chunked, overlap with a
 * warp or a CTA per matrix) and keep the fastest.  cache_path (nullable): text
 * file of earlier choices, read first and appended to.  report (nullable)
 * receives the timings. */
int afqmc_autotune(afqmc_handle* h, const char* cache_path, char* report, int report_len);
int afqmc_tuning(const afqmc_handle* h, int* bn_fb, int* bn_vhs, int* prop, int* ovl, int* qr);
/* Set the choices directly (a value <= 0 keeps the current one).  bn_*: 64, 128
 * or 256; prop: 1 V in shared memory (N <= 128), 2 column-chunked, 3 tensor
 * core (N <= 512; streamed tiles above 128), 4 tensor core with the walker
 * operand stored MN-major (N <= 128); ovl: 1 warp per matrix, 2 CTA per matrix
 * (FP64 Gauss-Jordan), 3 warp per matrix with M = Phi^T psi formed on the
 * tensor cores from exact BF16 slices (mixed form, N <= 128, n <= 32;
 * FP64-grade), 4 CTA per matrix in double-FP32 (mixed form; the default there
 * above 32 electrons per channel); qr (walker
 * orthonormalisation): 1 Householder with the reference's (Eigen's) column
 * signs, 2 Cholesky-QR in FP64 (mixed form; the same Q up to column signs,
 * which the overlaps carry, so every physical result is unchanged; the
 * default there).  An unavailable choice is AFQMC_ERR_ARG. */
int afqmc_set_tuning(afqmc_handle* h, int bn_fb, int bn_vhs, int prop, int ovl, int qr);

/* ---- device-resident blocks (MixedEstimator.cpp:483-635 without the host) ----
 * afqmc_block_setup starts a run's device state: nprocs emulated ranks (the
 * comb's P), nsteps per block, the energy estimate and running average the
 * driver starts from, the truncation correction delta, burn_steps (steps
 * measured into the equilibration average besides those with step*dt < 10),
 * and optionally the comb zetas of the first nzeta blocks (the reference draws
 * them from rank 0's generator); later blocks draw zeta from the device Philox
 * stream.  Steps are counted from this call. */
int afqmc_block_setup(afqmc_handle* h, int nprocs, int nsteps, double e_estimate, double avg_e, double delta,
                      long burn_steps, const double* zetas, int nzeta);
/* End of a block, enqueued on the handle's stream (capturable, no host sync):
 * exact local energies of all walkers, the clamped weighted block energy into
 * the block ring, the running averages and energy estimate, and with comb != 0
 * the comb reconfiguration.  A non-finite energy of a live walker is reported
 * as AFQMC_ERR_NAN by the next call that reads device state. */
int afqmc_block_end(afqmc_handle* h, int comb);
/* The first nblocks ring entries (total weight, block energy: samples.dat rows
 * 1..nblocks) and the clamped local energies counted since afqmc_block_setup. */
int afqmc_block_results(afqmc_handle* h, int nblocks, double* total_weights, double* total_energies, long* n_large);
/* Comb reconfiguration alone, on the device, with the given zeta in [0, 1) over
 * nprocs emulated ranks (MixedEstimator.cpp:583-621). */
int afqmc_comb(afqmc_handle* h, double zeta, int nprocs);

/* ---- CUDA-graph replay (one or several systems) ----
 * Capture nsteps device-field steps of each of the n handles (QR every
 * ortho_every steps, control-variate measurement every cv_every steps when a
 * network is attached; 0 disables) into one graph whose per-system branches run
 * concurrently; afqmc_graph_launch replays it (every handle advances nsteps).
 * Population control runs on the device (afqmc_set_energy_estimate). */
typedef struct afqmc_graph afqmc_graph;
int afqmc_graph_capture(afqmc_handle** hs, int n, int nsteps, int ortho_every, int cv_every, afqmc_graph** out);
/* As afqmc_graph_capture, and each handle's branch ends with afqmc_block_end
 * (comb as given): one replay is one whole block of the run. */
int afqmc_graph_capture_blocks(afqmc_handle** hs, int n, int nsteps, int ortho_every, int comb, afqmc_graph** out);
int afqmc_graph_launch(afqmc_graph* g);
int afqmc_graph_nodes(const afqmc_graph* g, long* nodes);
int afqmc_graph_destroy(afqmc_graph* g);
const char* afqmc_graph_last_error(void);

/* ---- allocation-free orthonormalisation ----
 * No counterpart in the reference.  For callers that cannot allocate GPU
 * memory when they call it: hosts whose device memory belongs to another
 * allocator (a framework's caching pool, a service that budgets the whole GPU
 * up front), and latency-bound loops that must stay out of the allocator,
 * whose cudaMalloc / cudaFree synchronise the device.  Same Householder QR as
 * afqmc_orthonormalize, on caller-owned device buffers:
 *   dets:     device, [nwalk][ncols][norb] complex double, column-major per walker
 *             (ncols = nalpha for rhf_walker, else nalpha + nbeta, alpha first); in/out
 *   overlaps: device, [nwalk] complex double; divided by prod diag(R) (squared
 *             for the restricted walker); in/out
 *   stream:   cudaStream_t to launch on (NULL: the default stream); asynchronous.
 * The Q workspace is a fixed device array of 2^19 complex doubles (8 MiB) that
 * every GPU loading the library keeps until exit; walkers go through it in
 * batches, and one walker's det (norb x ncols) must fit, else AFQMC_ERR_ARG.
 * The first call on a device looks up the array's address (with that device
 * current) and should come before any stream capture; after cudaDeviceReset
 * that address is stale, so do not call this again on a reset device.  All
 * calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller.  Nothing is allocated (no cudaMalloc / cudaFree).
 * A CUDA error already pending when it is called is returned as
 * AFQMC_ERR_CUDA with a message saying so.  On failure the message is
 * afqmc_last_error(NULL). */
int afqmc_orthonormalize_noalloc(void* dets, void* overlaps, int nwalk, int norb, int nalpha, int nbeta,
                                 int rhf_walker, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* AFQMC_GB300_H */
