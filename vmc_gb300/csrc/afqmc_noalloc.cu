// Allocation-free Householder orthonormalisation of walker determinants.
//
// This entry point has no counterpart in the reference.  It exists for callers
// that cannot allocate GPU memory at the time they call it: hosts whose device
// memory is owned by another allocator (a framework's caching pool, a service
// that budgets every byte of the GPU up front), and latency-bound loops that
// must not enter the allocator, whose cudaMalloc / cudaFree synchronise the
// device.  The caller passes the walker determinants and overlaps in its own
// device memory; the Q workspace of the QR lives in a fixed file-scope device
// array, so nothing is allocated.
//
// The array holds AFQMC_NOALLOC_QR_SCRATCH complex doubles (8 MiB); every GPU
// that loads this library keeps it until the process exits.  Walkers are
// processed in batches that fit in it, so nwalk is unbounded, but one walker's
// determinant (norb x (nalpha + nbeta) complex) must fit.  Every call shares the
// array and it keeps the last call's contents (the kernel rewrites the part it
// uses before reading it), so calls that overlap on the GPU -- on different
// streams, or from different host threads -- race on it and must be serialised
// by the caller.  The first call on a device looks up the array's device
// address with that device current and keeps it; cudaDeviceReset discards the
// library's device memory, so the kept address is stale after a reset and the
// entry point must not be used on that device again in the same process.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "afqmc_internal.h"

namespace afqmc {
void launch_ortho_buffers(double2* psi, double2* qwork, double2* ovlp, int nwalk, int N, int ncw, int na, int nb,
                          int rhf_walker, cudaStream_t stream);
void set_global_error(const std::string& msg);  // read back with afqmc_last_error(NULL)
}

#define AFQMC_NOALLOC_QR_SCRATCH (1 << 19)

static __device__ __align__(256) double2 g_qr_scratch[AFQMC_NOALLOC_QR_SCRATCH];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double2* g_scratch_addr[kMaxDevices] = {nullptr};
int noalloc_fail(int code, const std::string& m) {
  afqmc::set_global_error("afqmc_orthonormalize_noalloc: " + m);
  return code;
}

}  // namespace

extern "C" {

int afqmc_orthonormalize_noalloc(void* dets, void* overlaps, int nwalk, int norb, int nalpha, int nbeta,
                                 int rhf_walker, void* stream) {
  if (!dets || !overlaps) return noalloc_fail(AFQMC_ERR_ARG, "null device buffer");
  if (nwalk <= 0 || norb <= 0 || nalpha <= 0 || nbeta < 0 || nalpha > norb || nbeta > norb)
    return noalloc_fail(AFQMC_ERR_ARG, "bad sizes");
  if (std::max(nalpha, nbeta) > afqmc::QR_MAXN)
    return noalloc_fail(AFQMC_ERR_ARG, "nocc above the QR kernel's limit of 128");
  if (rhf_walker && nalpha != nbeta) return noalloc_fail(AFQMC_ERR_ARG, "restricted walker needs nalpha == nbeta");
  const int ncw = rhf_walker ? nalpha : nalpha + nbeta;
  const long per_walker = (long)ncw * norb;
  if (per_walker > AFQMC_NOALLOC_QR_SCRATCH)
    return noalloc_fail(AFQMC_ERR_ARG, "one walker determinant (" + std::to_string(per_walker) +
                                           " complex) exceeds the fixed scratch of " +
                                           std::to_string(AFQMC_NOALLOC_QR_SCRATCH) + " complex");
  // an error left pending by earlier, unrelated work is reported as such, not
  // as a failure of this call's launches
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return noalloc_fail(AFQMC_ERR_CUDA, std::string("an earlier CUDA error is pending: ") + cudaGetErrorString(e));
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(AFQMC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(AFQMC_ERR_ARG, "device ordinal out of range");
  double2* scratch;
  {
    // first call on this device (with it current): look up the device address
    // of the array; this first call should come before any stream capture
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_qr_scratch);
      if (e != cudaSuccess)
        return noalloc_fail(AFQMC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = (double2*)p;
    }
    scratch = g_scratch_addr[dev];
  }
  const int batch = (int)std::min<long>(nwalk, AFQMC_NOALLOC_QR_SCRATCH / per_walker);
  cudaStream_t st = (cudaStream_t)stream;
  for (int w0 = 0; w0 < nwalk; w0 += batch) {
    const int nw = std::min(batch, nwalk - w0);
    afqmc::launch_ortho_buffers((double2*)dets + (size_t)w0 * per_walker, scratch, (double2*)overlaps + w0, nw,
                                norb, ncw, nalpha, nbeta, rhf_walker ? 1 : 0, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(AFQMC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  }
  return AFQMC_OK;
}

}  // extern "C"
