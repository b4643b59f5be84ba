// Autotuner: per size class (device, N, nalpha, nbeta, nchol, walkers, spin
// blocks, precision) it times the candidate tile shapes and kernel variants
// on the handle's own data and keeps the fastest:
//   * N-tile (64 / 128 / 256) of the tensor-core force-bias and VHS GEMMs,
//   * propagator: tensor core (tcgen05, split BF16), walker V resident in
//     shared memory (FP32), or column-chunked with V streamed from L2 (FP32),
//   * overlap / inverse: one warp per matrix with M = Phi^T psi in FP64 or on
//     the tensor cores (exact BF16 slices), or one CTA per matrix.
// Choices are cached in a text file (one "key value..." line per size class),
// so later handles of the same class skip the timing.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <fstream>
#include <sstream>
#include <string>

#include "afqmc_internal.h"

namespace afqmc {
void launch_fb_gemm(afqmc_handle* h, int bn);
void launch_vhs_gemm(afqmc_handle* h, int bn);
void launch_theta_split(afqmc_handle* h);
}  // namespace afqmc

namespace {

template <class F>
float time_ms(afqmc_handle* h, F f, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  f();  // warm-up
  cudaEventRecord(a, h->stream);
  for (int r = 0; r < reps; ++r) f();
  cudaEventRecord(b, h->stream);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

std::string tune_key(afqmc_handle* h) {
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, h->device);
  std::ostringstream k;
  std::string name = p.name;
  for (auto& c : name)
    if (c == ' ') c = '_';
  k << name << "|N" << h->N << "|na" << h->na << "|nb" << h->nb << "|G" << h->G << "|W" << h->nwalk << "|sp"
    << h->nspV << "|p" << h->precision << "|rw" << h->rhf_walker;
  return k.str();
}

}  // namespace

extern "C" {

int afqmc_autotune(afqmc_handle* h, const char* cache_path, char* report, int report_len) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  const std::string key = tune_key(h);
  if (cache_path) {
    std::ifstream in(cache_path);
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream ls(line);
      std::string k;
      int a, b, c, d;
      if (ls >> k >> a >> b >> c >> d && k == key) {
        h->tune_bn_fb = a;
        h->tune_bn_vhs = b;
        h->tune_prop = c;
        h->tune_ovl = d;
        if (report) snprintf(report, report_len, "cached %s: fb_bn=%d vhs_bn=%d prop=%d ovl=%d", key.c_str(), a, b, c, d);
        return AFQMC_OK;
      }
    }
  }
  std::ostringstream rep;
  const bool mixed = h->precision == AFQMC_PREC_MIXED;
  if (mixed) {
    afqmc::launch_theta_split(h);
    const int bns[3] = {64, 128, 256};
    float best = 1e30f;
    for (int bn : bns) {
      const float t = time_ms(h, [&] { afqmc::launch_fb_gemm(h, bn); }, 3);
      rep << "fb_bn" << bn << "=" << t << "ms ";
      if (t < best) { best = t; h->tune_bn_fb = bn; }
    }
    best = 1e30f;
    for (int bn : bns) {
      const float t = time_ms(h, [&] { afqmc::launch_vhs_gemm(h, bn); }, 3);
      rep << "vhs_bn" << bn << "=" << t << "ms ";
      if (t < best) { best = t; h->tune_bn_vhs = bn; }
    }
    // propagator variants on a snapshot of the walkers (restored after each run)
    const size_t bytes = (size_t)h->nwalk * h->ncw * h->N * sizeof(double2);
    cudaMemcpyAsync(h->qwork, h->psi, bytes, cudaMemcpyDeviceToDevice, h->stream);
    best = 1e30f;
    const int cands[4] = {4, 3, 1, 2};
    for (int c : cands) {
      if ((c == 1 && h->N > 128) || (c == 3 && !afqmc::prop_tc_available(h)) ||
          (c == 4 && !afqmc::prop_tc2_available(h)))
        continue;
      h->tune_prop = c;
      const float t = time_ms(h, [&] {
        afqmc::launch_propagate_mixed(h);
        cudaMemcpyAsync(h->psi, h->qwork, bytes, cudaMemcpyDeviceToDevice, h->stream);
      }, 2);
      rep << "prop" << (c == 1 ? "_smem" : c == 2 ? "_chunk" : c == 3 ? "_tc" : "_tc_mn") << "=" << t << "ms ";
      if (t < best) { best = t; h->tune_prop_best = c; }
    }
    h->tune_prop = h->tune_prop_best;
    afqmc::launch_psi_to_f32(h);  // the FP32 copy follows the restored walkers
  }
  {
    const int nmax = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
    float best = 1e30f;
    const int cands[4] = {3, 1, 4, 2};
    for (int c : cands) {
      if (c == 1 && (nmax > 32 || (size_t)nmax * h->N * 8 + 4 * ((size_t)nmax * nmax * 24 + 4 * nmax + 16) > 160 * 1024))
        continue;
      if (c == 3 && !afqmc::ovl_tc_available(h)) continue;
      if (c == 4 && h->precision != AFQMC_PREC_MIXED) continue;
      h->tune_ovl = c;
      const float t = time_ms(h, [&] { afqmc::launch_overlap_theta(h, false); }, 3);
      rep << "ovl" << (c == 1 ? "_warp" : c == 2 ? "_block" : c == 3 ? "_tc" : "_block_df32") << "=" << t << "ms ";
      if (t < best) { best = t; h->tune_ovl_best = c; }
    }
    h->tune_ovl = h->tune_ovl_best;
    afqmc::launch_overlap_theta(h, false);  // theta / det of the current walkers again
  }
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = std::string("autotune: ") + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  if (cache_path) {
    std::ofstream out(cache_path, std::ios::app);
    out << key << " " << h->tune_bn_fb << " " << h->tune_bn_vhs << " " << h->tune_prop << " " << h->tune_ovl << "\n";
  }
  rep << "-> fb_bn=" << h->tune_bn_fb << " vhs_bn=" << h->tune_bn_vhs << " prop=" << h->tune_prop
      << " ovl=" << h->tune_ovl;
  if (report) snprintf(report, report_len, "%s", rep.str().c_str());
  return AFQMC_OK;
}

int afqmc_set_tuning(afqmc_handle* h, int bn_fb, int bn_vhs, int prop, int ovl, int qr) {
  if (!h) return AFQMC_ERR_ARG;
  auto bn_ok = [](int b) { return b <= 0 || b == 64 || b == 128 || b == 256; };
  const bool mixed = h->precision == AFQMC_PREC_MIXED;
  if (!bn_ok(bn_fb) || !bn_ok(bn_vhs) || prop > 4 || ovl > 4 || (ovl == 4 && !mixed) || ((bn_fb > 0 || bn_vhs > 0 || prop > 0) && !mixed) ||
      (ovl == 3 && !afqmc::ovl_tc_available(h)) ||
      ((prop == 1) && h->N > 128) || (prop == 3 && !afqmc::prop_tc_available(h)) ||
      (prop == 4 && !afqmc::prop_tc2_available(h)) || qr > 2 ||
      (qr == 2 && !afqmc::ortho_chol_available(h))) {
    h->err = "afqmc_set_tuning: choice not available for this handle";
    return AFQMC_ERR_ARG;
  }
  if (ovl == 1 || ovl == 3) {
    const int nmax = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
    if (nmax > 32) {
      h->err = "afqmc_set_tuning: warp overlap needs at most 32 electrons per channel";
      return AFQMC_ERR_ARG;
    }
  }
  if (bn_fb > 0) h->tune_bn_fb = bn_fb;
  if (bn_vhs > 0) h->tune_bn_vhs = bn_vhs;
  if (prop > 0) h->tune_prop = prop;
  if (ovl > 0) h->tune_ovl = ovl;
  if (qr > 0) h->tune_qr = qr;
  h->fb_current = false;
  return AFQMC_OK;
}

int afqmc_tuning(const afqmc_handle* h, int* bn_fb, int* bn_vhs, int* prop, int* ovl, int* qr) {
  if (!h) return AFQMC_ERR_ARG;
  if (bn_fb) *bn_fb = h->tune_bn_fb;
  if (bn_vhs) *bn_vhs = h->tune_bn_vhs;
  if (prop) *prop = h->tune_prop;
  if (ovl) *ovl = h->tune_ovl;
  if (qr) *qr = h->tune_qr == 0 ? (afqmc::ortho_chol_available(h) ? 2 : 1) : h->tune_qr;
  return AFQMC_OK;
}

}  // extern "C"
