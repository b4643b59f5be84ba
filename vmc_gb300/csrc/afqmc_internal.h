// Internal declarations shared by the C-ABI layer and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <complex>
#include <string>
#include <vector>

#include "../../include/afqmc.h"

namespace afqmc {

using cplx = std::complex<double>;

// A trial "channel": one (walker det block, trial orbital block) pair of the
// trial contractions.  RHF trial x restricted walker is one channel counted
// twice (mult = 2, DQMC/RHF.cpp:34-39, :54-61, :104-131); all other pairings
// have two channels with mult = 1.
struct Channel {
  int psi_off;  // first walker-det column of this channel
  int n;        // occupied orbitals
  int col_off;  // first column in the channel-ordered arrays (phi, rot, theta, h1phi)
  int lspin;    // which Cholesky / h1 spin block it contracts with (0 unless int_type U)
};

// A column chunk of the walker det for the propagator: columns [c0, c0 + nc)
// all in walker spin block `spin` (which selects V and exp(-dt/2 h1')).
struct PropChunk {
  int c0, nc, spin;
};

constexpr int PROP_CH = 8;   // walker-det columns per propagator CTA
constexpr int QR_MAXN = 128; // largest nocc the QR kernel handles

// Device scalars of the population control and of device-resident blocks
// (slots of Handle::scal): energy shift, energy estimate, sum of weights after
// the last step, capped weights; running block averages (production / before
// the end of equilibration), truncation correction delta, clamped local
// energies, step counter at the start of the run, equilibration steps, the
// next block slot, emulated ranks, and the number of host-given comb zetas.
enum {
  S_ESHIFT = 0, S_EEST = 1, S_SUMW = 2, S_NCAP = 3,
  S_AVGE = 4, S_AVGE_EQL = 5, S_NUM = 6, S_DEN = 7, S_NUM_EQL = 8, S_DEN_EQL = 9,
  S_DELTA = 10, S_NLARGE = 11, S_STEP0 = 12, S_BURN = 13, S_BLOCK = 14, S_NPROCS = 15, S_NZETA = 16,
  S_NLIVE = 20,  // walker-steps propagated since the handle was created (live walkers, w > 1e-8)
  S_NSLOTS = 24
};
constexpr int BLK_MAX = 65536;  // block ring capacity (samples of one run)
constexpr int WT_MAXPARTS = 1024;  // CTAs of the weight update (partial sums)
constexpr int CV_EST_THREADS = 256, CV_EST_MAX_CTAS = 64;  // the control-variate estimate's grid
constexpr int DERR_NAN_ENERGY = 100;  // d_err code: non-finite local energy in a device block

// Stage names for timing.
enum Stage { ST_FB = 0, ST_FIELDS, ST_VHS, ST_PROP, ST_OVERLAP, ST_WEIGHTS, ST_ORTHO, ST_ENERGY, ST_N };

}  // namespace afqmc

struct afqmc_handle {
  // sizes
  int N = 0, na = 0, nb = 0, G = 0, T = 0, nsp = 1, int_type = 0;
  int nwalk = 0, rhf_walker = 0, precision = 0, device = 0;
  int nsm = 0;          // SMs of the device (persistent grids)
  int ncw = 0;          // walker det columns (na, or na + nb)
  int nchan = 0, mult = 1, nce = 0;
  afqmc::Channel chan[2];
  std::vector<afqmc::PropChunk> chunks, chunks32;
  int nspV = 1;         // distinct VHS matrices per walker (1 for INT_R, 2 for INT_U)
  double dt = 0, ecore = 0, weight_cap = 0, pop_target = 0;
  uint64_t seed = 0, step_counter = 0;
  int nchol_ene = 0;
  afqmc::cplx prop_constant;
  std::vector<afqmc::cplx> mf_host;    // [G]
  std::vector<afqmc::cplx> expm_host;  // [nsp][N][N] row-major
  std::vector<double> ref_serial;      // mean-field reference det, serial layout N*(na+nb)
  cudaStream_t stream = nullptr;
  std::string err;
  long launches = 0;
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[afqmc::ST_N];
  std::vector<cudaEvent_t> ev_pool;
  double stage_ms[afqmc::ST_N] = {0};
  cudaEvent_t timer[2] = {nullptr, nullptr};

  // device buffers (FP64 form)
  double2* psi = nullptr;     // [W][ncw][N]          walker dets, column-major per walker
  double* phi = nullptr;      // [nce][N]             channel trial orbitals
  double* rot = nullptr;      // [G][nce*N]           rot[g][(col)*N + p] = (Phi^T L_g)[i, p]
  double* h1phi = nullptr;    // [nce][N]             (h1 Phi)[p, i]
  float2* h1phi32 = nullptr;  // [nce][N]             double-FP32 copy (mixed form: features, one-body energy)
  float2* phi2 = nullptr;     // [nce][N]             double-FP32 copy of phi (mixed form: overlap matrices)
  double* LT = nullptr;       // [nsp][T][G]          packed lower-triangle Cholesky, FP64
  float* LT32 = nullptr;      // [nsp][T][G]          FP32 copy (REF32)
  int2* tri = nullptr;        // [T]                  packed index -> (i, j), j <= i
  double2* expm = nullptr;    // [nsp][N][N]          column-major exp(-dt/2 h1'_s)
  double2* mf = nullptr;      // [G]
  double* theta = nullptr;    // [W][2][nce*N]        re / im planes (FP64 and reference forms)
  float* theta32 = nullptr;   // [W][2][nce*N]        the same in FP32 (mixed form, where it is formed in FP32)
  double2* det = nullptr;     // [W][2]               det(Phi_s^T psi_s) per channel
  double2* ovlp = nullptr;    // [W]
  double* weights = nullptr;  // [W]
  double* fb = nullptr;       // [W][2][G]
  double* xi = nullptr;       // [W][G]
  double* x = nullptr;        // [W][2][G]
  float* x32 = nullptr;       // [W][2][G]
  double2* shift = nullptr;   // [W]
  double2* fbterm = nullptr;  // [W]
  double* V = nullptr;        // [W][nspV][2][N*N]    full VHS matrices, re / im planes
  double2* qwork = nullptr;   // [W][ncw][N]          QR scratch (Q)
  double2* epart = nullptr;   // [W][nechunk]         local-energy partial sums
  double2* eloc = nullptr;    // [W]
  double* scal = nullptr;     // [S_NSLOTS]
  double* host_pinned = nullptr;  // pinned staging for xi: two buffers of W G doubles, used in turn
  size_t host_pinned_bytes = 0;   // bytes of one buffer
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};  // recorded after each buffer's copy to the device
  int stage_next = 0;
  // host fields reach the device on their own stream, into two device buffers
  // used in turn (xi and xi1), so a copy waits only for the fields kernel that
  // last read its buffer, not for the device's previous step
  cudaStream_t copy_stream = nullptr;
  double* xi1 = nullptr;                             // [W][G] second device field buffer
  double* xi_cur = nullptr;                          // the buffer this step's fields kernel reads
  cudaEvent_t xi_copied[2] = {nullptr, nullptr};     // the copy into buffer b is done
  cudaEvent_t xi_read[2] = {nullptr, nullptr};       // the fields kernel that read buffer b is done
  int xi_next = 0;
  // asynchronous reads of control-variate results: a FIFO of pinned 6-double
  // slots, each with the event of its device-to-host copy
  double* res_pinned = nullptr;                      // [RES_RING][6]
  cudaEvent_t res_ev[8] = {};
  int res_head = 0, res_count = 0;
  int nechunk = 0;
  afqmc::PropChunk* d_chunks = nullptr;
  int nchunks = 0;

  // mixed-precision form
  int* d_err = nullptr;              // error code of bounded device waits (0 = none)
  int kf_pad = 0, kv_pad = 0;        // padded split-K lengths of the force-bias / VHS GEMMs
  int kf_seg = 0;                    // force bias: nce N rounded up to 64; kf_pad = 3 kf_seg
  __nv_bfloat16* rotA = nullptr;     // [G][kf_pad]       [hi | hi | lo] of rot, segments kf_seg apart
  __nv_bfloat16* LTA = nullptr;      // [nsp][T][kv_pad]  [hi | hi | lo] of LT
  __nv_bfloat16* thetaB = nullptr;   // [2W][2 kf_seg]    [hi | lo] of theta planes (the GEMM reads hi twice)
  __nv_bfloat16* xB = nullptr;       // [2W][kv_pad]      [hi | lo | hi] of field planes
  float* fb32 = nullptr;             // [W][2][G]
  float* V32 = nullptr;              // [W][nspV][2][T]   packed VHS, re / im planes
  bool real_expm = false;            // exp(-dt/2 h1') has no imaginary part (real trial)
  float* expm32 = nullptr;           // [nsp][2][N*N]     re / im planes, column-major
  afqmc::PropChunk* d_chunks32 = nullptr;
  int nchunks32 = 0;
  CUtensorMap tm_rot, tm_LT[2];
  CUtensorMap tm_theta_bn[3], tm_x_bn[3];  // B operands with box heights 64, 128, 256
  // autotuned choices (afqmc_autotune): GEMM N-tiles; propagator 0 auto / 1 SMEM / 2 chunked / 3 tcgen05 /
  // 4 tcgen05 with the walker operand MN-major (N <= 128);
  // overlap 0 auto / 1 warp per matrix / 2 block per matrix (FP64) / 3 warp per matrix, M on the tensor cores /
  // 4 block per matrix in double-FP32 (mixed form)
  int tune_bn_fb = 128, tune_bn_vhs = 128, tune_prop = 0, tune_ovl = 0;
  int tune_qr = 0;  // walker QR: 0 auto (Cholesky-QR in the mixed form when it fits), 1 Householder, 2 Cholesky-QR
  int tune_prop_best = 0, tune_ovl_best = 0;
  // mixed local energy
  int ke_pad = 0;                    // padded split-K (3N) of the exchange GEMM
  __nv_bfloat16* rotE = nullptr;     // [G][nce][ke_pad]  [hi | hi | lo] of rot along p
  __nv_bfloat16* thetaE = nullptr;   // [2W][nce][ke_pad] [hi | lo | hi] of theta along p
  double2* xc = nullptr;             // [W][2][Gene][2]   exchange X and Coulomb c per (w, s, g)
  int ex_gbox[2] = {1, 1}, ex_wbox[2] = {1, 1};
  CUtensorMap tm_rotE[2], tm_thE[2];
  unsigned long long* d_step = nullptr;  // device step counter of the Philox field stream
  bool fb_current = false;               // fb32 holds the force bias of the current theta
  bool thetaB_from_lu = false;           // the overlap LU wrote thetaB (the split of the current theta)
  float2* psi32 = nullptr;               // [W][ncw][N] FP32 copy of psi (mixed form)
  // device-resident blocks: comb scratch, the block ring and host-given zetas
  double* wpart = nullptr;      // [WT_MAXPARTS][2] partial sums of the weight update
  unsigned int* wt_cnt = nullptr;  // CTAs of the weight update finished (the last one resets it to 0)
  double* comb_cum = nullptr;   // [W]
  int* comb_idx = nullptr;      // [W]
  double2* comb_ovl = nullptr;  // [W]
  double* blk = nullptr;        // [BLK_MAX][2] total weight, block energy
  double* blk_zeta = nullptr;   // [BLK_MAX]
  __nv_bfloat16* pt_img = nullptr;
  uint2* pt_voff = nullptr;  // [T] swizzled scatter offsets of the packed triangle (tensor-core propagator)
  // tensor-core propagator for 128 < N <= 512: the B - I tile image per spin
  // and one V-image scratch slot per persistent CTA
  uint8_t* pb_img = nullptr;
  uint8_t* pb_scratch = nullptr;
  int pb_slots = 0;
  // tensor-core overlap matrices (exact BF16 slices): trial-orbital scales
  // [channel][BNP], the swizzled trial-slice images [channel][bytes], and M
  double* ovl_tau = nullptr;
  uint8_t* ovl_bimg = nullptr;
  float4* ovl_M = nullptr;  // [W][2][nmax][nmax] double-FP32 (re hi, re lo, im hi, im lo)
  float4* mf32 = nullptr;   // [G] mean field as double-FP32 (re hi, re lo, im hi, im lo)
  // control variate
  float* cv_x = nullptr;             // [W][67] features
  float* cv_f = nullptr;             // [W]     network outputs (standard units) of the local energies
  int* cv_idx = nullptr;             // [W]     subsample
  double2* cv_esub = nullptr;        // [W]     exact energies of the subsample
  float* cv_ms = nullptr;            // [2][67] feature mean / std
  double* cv_out = nullptr;          // [cv_nslots][4]
  double* cv_part = nullptr;         // [CV_EST_MAX_CTAS][8] per-CTA sums of the estimate
  unsigned int* cv_cnt = nullptr;    // CTAs of the estimate finished (the last one resets it to 0)
  int cv_nslots = 4096, cv_den = 8;
  float cv_ymean = 0.f, cv_ystd = 1.f;
  struct afqmc_mlp* cv_mlp = nullptr;
  cudaStream_t cv_side = nullptr;      // the subsample's exact energies, beside the force bias
  cudaEvent_t cv_fork = nullptr, cv_join = nullptr;
  // mixed 1-RDM estimator: running sums of sum_w w Re theta_w [nce*N] and of
  // the weights (slot nce*N), per-chunk partial sums, trial orbitals on the host
  bool rdm_on = false;
  double* rdm_acc = nullptr;   // [nce*N + 1]
  double* rdm_part = nullptr;  // [RDM_CHUNKS][nce*N + 1]
  std::vector<double> phi_host;  // [nce][N] channel trial orbitals
};

namespace afqmc {

// ---- kernels (kernels_fp64.cu) ----
void launch_overlap_theta(afqmc_handle* h, bool only_live);
void launch_force_bias(afqmc_handle* h);
void launch_fields(afqmc_handle* h, bool device_rng);
void launch_vhs(afqmc_handle* h);
void launch_propagate(afqmc_handle* h);
void launch_weights(afqmc_handle* h);
void launch_ortho(afqmc_handle* h);
void launch_local_energy(afqmc_handle* h);
void launch_init_overlap(afqmc_handle* h);
void launch_psi_to_f32(afqmc_handle* h);

// ---- kernels (kernels_mixed.cu) ----
bool setup_mixed(afqmc_handle* h);
bool setup_prop_tc(afqmc_handle* h);
bool ovl_tc_wanted(const afqmc_handle* h);
bool ovl_tc_available(const afqmc_handle* h);
int ovl_kp(const afqmc_handle* h);
int ovl_bnp(const afqmc_handle* h);
size_t ovl_bimg_bytes(const afqmc_handle* h);
bool setup_ovl_tc(afqmc_handle* h);
void launch_overlap_m_tc(afqmc_handle* h);
bool prop_tc_available(const afqmc_handle* h);
void launch_propagate_tc(afqmc_handle* h);
bool prop_tc2_available(const afqmc_handle* h);  // N <= 128, MN-major X operand
void launch_propagate_tc2(afqmc_handle* h);
size_t prop_tcb_img_bytes(int N);  // one matrix's tile image, 128 < N <= 512
bool prop_tcb_supported(int N);
bool setup_prop_tcb(afqmc_handle* h);
bool prop_tcb_available(const afqmc_handle* h);
void launch_propagate_tcb(afqmc_handle* h);
void launch_block_end(afqmc_handle* h, int comb);
bool ortho_chol_available(const afqmc_handle* h);
void launch_ortho_chol(afqmc_handle* h);
// the step's orthonormalisation: QR of every walker and whatever it invalidates
void launch_ortho_refresh(afqmc_handle* h);
int take_device_error(afqmc_handle* h);  // AFQMC_OK, or the status of a recorded device error (cleared)
void launch_force_bias_mixed(afqmc_handle* h);
void launch_fields_mixed(afqmc_handle* h, bool device_rng);
void launch_vhs_mixed(afqmc_handle* h);
void launch_propagate_mixed(afqmc_handle* h);
void split_rows(afqmc_handle* h, const double* src, long lds, int rows, int K, int kpad, int pattern, int seg,
                int nseg,
                __nv_bfloat16* dst);
void split_rows(afqmc_handle* h, const float* src, long lds, int rows, int K, int kpad, int pattern, int seg,
                int nseg,
                __nv_bfloat16* dst);
void launch_local_energy_mixed(afqmc_handle* h);
void launch_wait_probe(afqmc_handle* h);  // one bounded mbarrier wait that nothing completes
// ---- mixed 1-RDM estimator (afqmc_rdm.cu) ----
// add sum_w w Re theta_w of the live walkers to the running sums; gated: only
// when the step counted on the device satisfies step dt > 10 and step > burn
void launch_rdm_accumulate(afqmc_handle* h, bool gated);

// error helper used by kernels' launchers
bool check_launch(afqmc_handle* h, const char* what);

// Raise `kernel`'s dynamic shared-memory limit to at least `bytes` on the
// current device.  The attribute belongs to one device, so the set-up is
// remembered per (kernel, device), under a lock: handles on different devices
// or host threads each get it.  Returns false if CUDA refused it.
bool smem_optin_fn(const void* kernel, int bytes);
template <class F>
inline bool smem_optin(F* kernel, int bytes) {
  return smem_optin_fn((const void*)kernel, bytes);
}

}  // namespace afqmc
