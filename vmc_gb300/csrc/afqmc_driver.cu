// Host driver of the phaseless AFQMC run, written over the C ABI.
//
// Restates calcMixedEstimatorLongProp (DQMC/MixedEstimator.cpp:309-660): energy
// of the reference determinant and Cholesky truncation for the energy
// (:338-384), initial local energies (:398-421), the step loop with population
// control (:455-475), orthonormalisation cadence (:478-480), measurement with
// the local-energy clamp (:483-556) and comb reconfiguration (:559-635).
//
// MPI ranks are emulated inside one handle: the handle holds nprocs x nwalk
// walkers, rank r owning walkers [r nwalk, (r+1) nwalk); the sums that the
// reference takes with MPI_Allreduce run over all of them, and the comb gathers
// them in rank order.  With the reference-order field source each rank has its
// own std::mt19937(seed + r) and one std::normal_distribution per walker
// (executables/DQMC.cpp:58, DQMC/DQMCWalker.h:18), so a run reproduces the
// reference's samples.dat for the same inputs.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <random>
#include <string>
#include <vector>

#include "afqmc_internal.h"

struct afqmc_refrng {
  std::mt19937 gen;
  std::vector<std::normal_distribution<double>> normals;
};

extern "C" {

afqmc_refrng* afqmc_refrng_create(unsigned seed, int nwalk) {
  if (nwalk <= 0) return nullptr;
  afqmc_refrng* r = new afqmc_refrng();
  r->gen = std::mt19937(seed);
  r->normals.assign(nwalk, std::normal_distribution<double>(0.0, 1.0));
  return r;
}

void afqmc_refrng_destroy(afqmc_refrng* r) { delete r; }

int afqmc_refrng_draw_step(afqmc_refrng* r, const double* weights, int nfields, double* out) {
  if (!r || !weights || !out || nfields <= 0) return AFQMC_ERR_ARG;
  const int nw = (int)r->normals.size();
  for (int w = 0; w < nw; ++w) {
    double* o = out + (size_t)w * nfields;
    if (weights[w] > 1.0e-8) {
      for (int g = 0; g < nfields; ++g) o[g] = r->normals[w](r->gen);
    } else {
      for (int g = 0; g < nfields; ++g) o[g] = 0.0;
    }
  }
  return AFQMC_OK;
}

double afqmc_refrng_uniform(afqmc_refrng* r) {
  std::uniform_real_distribution<double> u(0.0, 1.0);
  return u(r->gen);
}

static int run_impl(afqmc_handle* h, const afqmc_run_opts* o, double* total_weights, double* total_energies,
                    double* block_eshift, double* block_wall, afqmc_run_stats* stats) {
  if (!h || !o || !total_weights || !total_energies) return AFQMC_ERR_ARG;
  // wall clock of the afqmc.dat rows: from the start of the walker set-up, as
  // the reference's calcInitTime (MixedEstimator.cpp:397)
  const auto t_start = std::chrono::steady_clock::now();
  const auto wall = [&]() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  };
  const int P = o->nprocs > 0 ? o->nprocs : 1;
  if (h->nwalk % P != 0) {
    h->err = "nwalk of the handle must be a multiple of nprocs";
    return AFQMC_ERR_ARG;
  }
  if (o->nsteps <= 0 || o->nsweeps <= 0 || o->ortho_steps <= 0) {
    h->err = "nsteps, nsweeps and ortho_steps must be positive";
    return AFQMC_ERR_ARG;
  }
  const int nwalk = h->nwalk / P, W = h->nwalk, G = h->G;
  const double dt = h->dt;
  const size_t ser = (size_t)h->N * (h->na + h->nb);
  int rc;
#define RUN(call)                  \
  do {                             \
    if ((rc = (call)) != AFQMC_OK) \
      return rc;                   \
  } while (0)

  // initial walkers (set by the caller) and the mean-field reference determinant
  std::vector<double> init_dets(2 * ser * W), init_ovlp(2 * W), wts(W);
  RUN(afqmc_get_walkers(h, init_dets.data(), nullptr, nullptr));
  std::vector<double> ref_dets(2 * ser * W, 0.0);
  for (int w = 0; w < W; ++w)
    for (size_t e = 0; e < ser; ++e) ref_dets[2 * (w * ser + e)] = h->ref_serial[e];
  RUN(afqmc_set_walkers(h, ref_dets.data(), nullptr, nullptr));
  std::vector<double> el(2 * W);
  RUN(afqmc_set_nchol_ene(h, G));
  RUN(afqmc_local_energy(h, el.data()));
  const double e_ref_re = el[0], e_ref_im = el[1];
  int nchol_ene = G;
  double delta = 0.0;
  const double fr[5] = {0.3, 0.4, 0.5, 0.6, 0.7};
  for (int i = 0; i < 5; ++i) {
    const int n = (int)(fr[i] * G);
    RUN(afqmc_set_nchol_ene(h, n));
    RUN(afqmc_local_energy(h, el.data()));
    const double dr = e_ref_re - el[0], di = e_ref_im - el[1];
    if (hypot(dr, di) < o->cholesky_threshold) {
      nchol_ene = n;
      delta = dr;
      break;
    }
  }
  RUN(afqmc_set_nchol_ene(h, nchol_ene));
  RUN(afqmc_set_walkers(h, init_dets.data(), nullptr, nullptr));
  RUN(afqmc_local_energy(h, el.data()));

  const int nsweeps = o->nsweeps, nsteps = o->nsteps;
  for (int b = 0; b < nsweeps; ++b) total_weights[b] = total_energies[b] = 0.0;
  double wsum_e = 0.0;
  for (int w = 0; w < W; ++w) wsum_e += el[2 * w];
  total_weights[0] = (double)nwalk * P;
  total_energies[0] = wsum_e / total_weights[0] + delta;
  if (block_eshift) {
    for (int b = 0; b < nsweeps; ++b) block_eshift[b] = 0.0;
    block_eshift[0] = total_energies[0];  // row 0 prints the initial energy in the eshift column
  }
  if (block_wall) {
    for (int b = 0; b < nsweeps; ++b) block_wall[b] = 0.0;
    block_wall[0] = wall();
  }

  std::vector<afqmc_refrng*> rngs;
  for (int r = 0; r < P; ++r) rngs.push_back(afqmc_refrng_create(o->seed + (unsigned)r, nwalk));
  struct Guard {
    std::vector<afqmc_refrng*>& v;
    ~Guard() { for (auto* r : v) afqmc_refrng_destroy(r); }
  } guard{rngs};

  double eshift = total_energies[0];
  double e_est = total_energies[0];
  double avg_e = total_energies[0], avg_e_eql = total_energies[0];
  double num = 0.0, den = 0.0, num_eql = 0.0, den_eql = 0.0;
  long nlarge = 0;
  RUN(afqmc_set_energy_estimate(h, e_est, &eshift));
  std::vector<double> xi(o->field_source == 0 ? (size_t)W * G : 0);
  std::vector<double> dets(2 * ser * W), ovl(2 * W), ndets(2 * ser * W), novl(2 * W), cum(W);
  const long last = o->max_steps > 0 ? std::min<long>((long)nsweeps * nsteps, (long)o->max_steps + 1)
                                     : (long)nsweeps * nsteps;
  RUN(afqmc_get_walkers(h, nullptr, nullptr, wts.data()));
  if (o->device_blocks) {
    // Whole blocks as graph replays with the device-resident block end; the
    // comb zetas are drawn here in the reference's order (rank 0's generator,
    // one per measurement) and handed to the device up front.
    if (o->field_source != 1 || nsteps % o->ortho_steps != 0) {
      h->err = "device_blocks needs field_source 1 and nsteps a multiple of ortho_steps";
      return AFQMC_ERR_ARG;
    }
    const long nblk = (last - 1) / nsteps;  // measured blocks: steps nsteps, 2 nsteps, ... < last
    if (nblk > afqmc::BLK_MAX) {
      h->err = "device_blocks: too many blocks";
      return AFQMC_ERR_ARG;
    }
    std::vector<double> zetas(o->comb ? nblk : 0);
    for (auto& z : zetas) z = afqmc_refrng_uniform(rngs[0]);
    RUN(afqmc_block_setup(h, P, nsteps, e_est, avg_e, delta, (long)o->burn_iter * nsteps, zetas.data(),
                          (int)zetas.size()));
    if (nblk > 0) {
      afqmc_graph* g = nullptr;
      afqmc_handle* hs[1] = {h};
      RUN(afqmc_graph_capture_blocks(hs, 1, nsteps, o->ortho_steps, o->comb, &g));
      for (long b = 0; b < nblk && rc == AFQMC_OK; ++b) {
        rc = afqmc_graph_launch(g);
        if (rc == AFQMC_OK && block_wall) {  // one wait per block, only when its time is asked for
          rc = afqmc_sync(h);
          if (b + 1 < nsweeps) block_wall[b + 1] = wall();
        }
      }
      afqmc_graph_destroy(g);
      if (rc != AFQMC_OK) {
        h->err = afqmc_graph_last_error();
        return rc;
      }
    }
    for (long step = nblk * nsteps + 1; step < last; ++step) {  // steps after the last measurement
      RUN(afqmc_step(h, nullptr, nullptr));
      if (step % o->ortho_steps == 0) RUN(afqmc_orthonormalize(h));
    }
    std::vector<double> bw(nblk), be(nblk);
    RUN(afqmc_block_results(h, (int)nblk, bw.data(), be.data(), &nlarge));
    double est = e_est;
    for (long b = 0; b < nblk; ++b)
      if (b + 1 < nsweeps) {
        total_weights[b + 1] = bw[b];
        total_energies[b + 1] = be[b];
        // the eshift of the measured step: the estimate before this block's
        // update and the block's total weight (MixedEstimator.cpp:474, :545)
        if (block_eshift) block_eshift[b + 1] = est - 0.1 * log(bw[b] / ((double)nwalk * P)) / dt;
        est = 0.9 * est + 0.1 * be[b];
      }
  }
  for (long step = o->device_blocks ? last : 1; step < last; ++step) {
    if (step * dt < 10.0) avg_e = avg_e_eql;
    if (o->field_source == 0) {
      for (int r = 0; r < P; ++r)
        afqmc_refrng_draw_step(rngs[r], wts.data() + (size_t)r * nwalk, G, xi.data() + (size_t)r * nwalk * G);
      RUN(afqmc_step(h, xi.data(), nullptr));
    } else {
      RUN(afqmc_step(h, nullptr, nullptr));
    }
    const bool ortho = step % o->ortho_steps == 0;
    const bool measure = step % nsteps == 0;
    double total_weight = 0.0;
    if (o->field_source == 0 || measure) {
      RUN(afqmc_population(h, &total_weight, &eshift, nullptr));
    }
    if (ortho) RUN(afqmc_orthonormalize(h));
    if (o->field_source == 0 || measure) RUN(afqmc_get_walkers(h, nullptr, nullptr, wts.data()));
    if (measure) {
      const int block = (int)(step / nsteps);
      RUN(afqmc_local_energy(h, el.data()));
      double wE = 0.0;
      for (int w = 0; w < W; ++w) {
        double e = 0.0;
        if (wts[w] != 0.0) {
          e = el[2 * w] + delta;
          if (isnan(e) || isinf(e)) {
            h->err = "non-finite local energy of walker " + std::to_string(w);
            return AFQMC_ERR_NAN;
          }
          if (fabs(e - avg_e) > sqrt(2.0 / dt)) {
            ++nlarge;
            e = e > avg_e ? avg_e + sqrt(2.0 / dt) : avg_e - sqrt(2.0 / dt);
          }
        }
        wE += e * wts[w];
      }
      if (block < nsweeps) {
        total_weights[block] = total_weight;
        total_energies[block] = wE / total_weight;
        if (block_eshift) block_eshift[block] = eshift;
        if (block_wall) block_wall[block] = wall();
      }
      const double tb = wE / total_weight;
      if (step * dt < 10.0 || step < (long)o->burn_iter * nsteps) {
        num_eql += tb * total_weight;
        den_eql += total_weight;
        avg_e_eql = num_eql / den_eql;
      } else {
        num += tb * total_weight;
        den += total_weight;
        avg_e = num / den;
      }
      e_est = 0.9 * e_est + 0.1 * tb;
      // mixed 1-RDM of the measured walkers, after equilibration (MixedEstimator.cpp:491)
      if (h->rdm_on && step * dt > 10.0 && step > (long)o->burn_iter * nsteps) {
        afqmc::launch_rdm_accumulate(h, false);
        if (cudaGetLastError() != cudaSuccess) {
          h->err = "1-RDM accumulation launch failed";
          return AFQMC_ERR_CUDA;
        }
      }
      if (o->comb) {
        RUN(afqmc_get_walkers(h, dets.data(), ovl.data(), nullptr));
        cum[0] = wts[0];
        for (int w = 1; w < W; ++w) cum[w] = cum[w - 1] + wts[w];
        const double tot = cum[W - 1];
        const double zeta = afqmc_refrng_uniform(rngs[0]);
        for (int w = 0; w < W; ++w) {
          const double z = (w + zeta) / nwalk / P;
          const int idx = (int)(std::lower_bound(cum.begin(), cum.end(), z * tot) - cum.begin());
          const int src = std::min(idx, W - 1);
          memcpy(ndets.data() + 2 * (size_t)w * ser, dets.data() + 2 * (size_t)src * ser, 2 * ser * sizeof(double));
          novl[2 * w] = ovl[2 * src];
          novl[2 * w + 1] = ovl[2 * src + 1];
        }
        for (int w = 0; w < W; ++w) wts[w] = tot / P / nwalk;
        RUN(afqmc_set_walkers(h, ndets.data(), novl.data(), wts.data()));
      }
      // the device recomputes eshift from the new estimate after the next step
      RUN(afqmc_set_energy_estimate(h, e_est, &eshift));
    }
  }
  if (stats) {
    stats->nchol_ene = nchol_ene;
    stats->delta = delta;
    stats->e_ref = e_ref_re;
    stats->n_large_deviations = nlarge;
    long capped = 0;
    afqmc_population(h, nullptr, nullptr, &capped);
    stats->n_large_deviations += capped;
  }
  return AFQMC_OK;
#undef RUN
}

int afqmc_run(afqmc_handle* h, const afqmc_run_opts* o, double* total_weights, double* total_energies,
              afqmc_run_stats* stats) {
  return run_impl(h, o, total_weights, total_energies, nullptr, nullptr, stats);
}

int afqmc_run_blocks(afqmc_handle* h, const afqmc_run_opts* o, double* total_weights, double* total_energies,
                     double* block_eshift, double* block_wall, afqmc_run_stats* stats) {
  return run_impl(h, o, total_weights, total_energies, block_eshift, block_wall, stats);
}

}  // extern "C"
