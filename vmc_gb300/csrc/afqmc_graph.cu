// CUDA-graph replay of blocks of steps, for one system or several systems of
// uneven sizes at once.
//
// A graph holds `nsteps` device-field steps of every handle (force bias,
// fields, VHS, propagator, overlap, weights; QR every `ortho_every` steps; the
// control-variate measurement every `cv_every` steps when a network is
// attached), optionally followed by the device-resident block end
// (measurement, energy estimate, comb).  Each handle's kernels run on its own stream, forked from and
// joined to the first handle's stream during capture, so the systems' kernels
// are independent branches of the one graph and run concurrently; a replay is
// one cudaGraphLaunch.  The device step counter of the Philox field stream
// and the population-control scalars live in device memory, so replays draw
// new fields and keep the population shift current without the host.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "afqmc_internal.h"

struct afqmc_graph {
  std::vector<afqmc_handle*> hs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> evs;
  size_t nodes = 0;
  int nsteps = 0;
  std::string err;
};

namespace {
thread_local std::string g_graph_err;
}

namespace afqmc {

void enqueue_step(afqmc_handle* h) {
  const bool mixed = h->precision == AFQMC_PREC_MIXED;
  if (mixed) {
    launch_force_bias_mixed(h);
    launch_fields_mixed(h, true);
    launch_vhs_mixed(h);
    launch_propagate_mixed(h);
  } else {
    launch_force_bias(h);
    launch_fields(h, true);
    launch_vhs(h);
    launch_propagate(h);
  }
  launch_overlap_theta(h, true);
  launch_weights(h);
}

void enqueue_ortho(afqmc_handle* h) { launch_ortho_refresh(h); }

}  // namespace afqmc

extern "C" {

int afqmc_cv_measure(afqmc_handle* h, uint64_t tag, int slot);

const char* afqmc_graph_last_error(void) { return g_graph_err.c_str(); }

}  // extern "C"

namespace {
// block_end < 0: steps only; 0 / 1: each branch ends with the block end without / with the comb
int capture(afqmc_handle** hs, int n, int nsteps, int ortho_every, int cv_every, int block_end, afqmc_graph** out) {
  if (!hs || n <= 0 || nsteps <= 0 || !out) {
    g_graph_err = "bad arguments";
    return AFQMC_ERR_ARG;
  }
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!hs[i] || hs[i]->device != hs[0]->device) {
      g_graph_err = "all handles must exist and share one device";
      return AFQMC_ERR_ARG;
    }
  cudaSetDevice(hs[0]->device);
  afqmc_graph* g = new afqmc_graph();
  g->hs.assign(hs, hs + n);
  g->nsteps = nsteps;
  auto bail = [&](const char* what, cudaError_t e) {
    g_graph_err = std::string(what) + ": " + cudaGetErrorString(e);
    if (g->graph) cudaGraphDestroy(g->graph);
    for (auto ev : g->evs) cudaEventDestroy(ev);
    delete g;
    return AFQMC_ERR_CUDA;
  };
  // every handle's pending work finishes before the capture starts
  for (int i = 0; i < n; ++i) {
    cudaError_t e = cudaStreamSynchronize(hs[i]->stream);
    if (e != cudaSuccess) return bail("stream sync", e);
  }
  // events: [0] fork, [1, n) joins of the capture, [n + i] pre-launch records, [2n] launch done
  g->evs.resize(2 * n + 1);
  for (auto& ev : g->evs) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaStream_t s0 = hs[0]->stream;
  std::vector<long> launches0(n);
  for (int i = 0; i < n; ++i) launches0[i] = hs[i]->launches;  // captured kernels are counted per replay
  cudaError_t e = cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return bail("cudaStreamBeginCapture", e);
  cudaEventRecord(g->evs[0], s0);
  for (int i = 1; i < n; ++i) cudaStreamWaitEvent(hs[i]->stream, g->evs[0], 0);
  for (int i = 0; i < n; ++i) {
    afqmc_handle* h = hs[i];
    h->fb_current = false;  // a replay must not rely on work outside the graph
    for (int k = 0; k < nsteps; ++k) {
      afqmc::enqueue_step(h);
      if (ortho_every > 0 && (k + 1) % ortho_every == 0) afqmc::enqueue_ortho(h);
      if (cv_every > 0 && h->cv_mlp && (k + 1) % cv_every == 0) afqmc_cv_measure(h, (uint64_t)k, k % h->cv_nslots);
    }
    if (block_end >= 0) afqmc::launch_block_end(h, block_end);
    if (i > 0) {
      cudaEventRecord(g->evs[i], h->stream);
      cudaStreamWaitEvent(s0, g->evs[i], 0);
    }
  }
  e = cudaStreamEndCapture(s0, &g->graph);
  for (int i = 0; i < n; ++i) hs[i]->launches = launches0[i];
  if (e != cudaSuccess) return bail("cudaStreamEndCapture", e);
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) return bail("cudaGraphInstantiate", e);
  cudaGraphGetNodes(g->graph, nullptr, &g->nodes);
  *out = g;
  return AFQMC_OK;
}
}  // namespace

extern "C" {

int afqmc_graph_capture(afqmc_handle** hs, int n, int nsteps, int ortho_every, int cv_every, afqmc_graph** out) {
  return capture(hs, n, nsteps, ortho_every, cv_every, -1, out);
}

int afqmc_graph_capture_blocks(afqmc_handle** hs, int n, int nsteps, int ortho_every, int comb, afqmc_graph** out) {
  return capture(hs, n, nsteps, ortho_every, 0, comb ? 1 : 0, out);
}

// One replay: every handle advances nsteps steps.  Ordered after each handle's
// earlier work, and each handle's later work is ordered after it.
int afqmc_graph_launch(afqmc_graph* g) {
  if (!g) return AFQMC_ERR_ARG;
  const int n = (int)g->hs.size();
  cudaStream_t s0 = g->hs[0]->stream;
  cudaSetDevice(g->hs[0]->device);
  for (int i = 1; i < n; ++i) {
    cudaEventRecord(g->evs[n + i], g->hs[i]->stream);
    cudaStreamWaitEvent(s0, g->evs[n + i], 0);
  }
  cudaError_t e = cudaGraphLaunch(g->exec, s0);
  if (e != cudaSuccess) {
    g_graph_err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  cudaEventRecord(g->evs[2 * n], s0);
  for (int i = 0; i < n; ++i) {
    g->hs[i]->launches += (long)g->nodes / n;
    if (i > 0) cudaStreamWaitEvent(g->hs[i]->stream, g->evs[2 * n], 0);
  }
  return AFQMC_OK;
}

int afqmc_graph_nodes(const afqmc_graph* g, long* nodes) {
  if (!g || !nodes) return AFQMC_ERR_ARG;
  *nodes = (long)g->nodes;
  return AFQMC_OK;
}

int afqmc_graph_destroy(afqmc_graph* g) {
  if (!g) return AFQMC_ERR_ARG;
  cudaSetDevice(g->hs[0]->device);
  cudaStreamSynchronize(g->hs[0]->stream);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (auto ev : g->evs) cudaEventDestroy(ev);
  delete g;
  return AFQMC_OK;
}

}  // extern "C"
