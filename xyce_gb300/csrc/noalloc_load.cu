// noalloc_load.cu — xg_load_noalloc: the Newton load without any device
// allocation in the call.
//
// The regular load (xg_load) keeps its per-load stamp terms in a buffer the
// circuit allocated at set-up.  Some callers cannot allocate device memory at
// the point where they load: host simulators that hand the GPU a fixed memory
// budget up front and forbid allocation afterwards, and real-time loops that
// must never block in the allocator.
// This entry point runs the same evaluation and fixed-order reduction kernels,
// but the stamp terms live in one fixed device array defined in this file, and
// the results are written to a buffer the caller passes in.
//
// The array holds at most kScratchTerms doubles (16 MiB); every GPU that loads
// this library keeps it reserved until the process exits.  All calls share it,
// so two calls whose work overlaps on the GPU (different streams, or
// different circuits loaded concurrently) race on it: serialise them.  Every
// term a load reads is written earlier in the same call, so nothing in the
// array needs to start at zero.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "xg.h"
#include "xg_internal.h"

namespace {

constexpr int64_t kScratchTerms = 2 * 1024 * 1024;  // 16 MiB of FP64 terms

static __device__ __align__(256) double g_term_scratch[kScratchTerms];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device
// with that device current and kept for the life of the process (a
// cudaDeviceReset invalidates it; the library must be reloaded after one).
// In host code the array's name only stands in for the symbol; the kernels
// must be given this address.
int scratch_on(int device, double **out) {
  if (device < 0 || device >= kMaxDevices) return XG_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_term_scratch);
    if (e != cudaSuccess) {
      xg::set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return XG_ERR_CUDA;
    }
    g_scratch_addr[device] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[device];
  return XG_OK;
}

}  // namespace

extern "C" int xg_load_noalloc(xg_circuit *c, const xg_load_flags *flags, double *dev_out,
                               int64_t dev_out_len) {
  xg::CircuitView v;
  if (!c || !flags || !dev_out || xg::circuit_view(c, &v) != XG_OK) {
    xg::set_error("xg_load_noalloc: null argument");
    return XG_ERR_ARG;
  }
  const xg::Plan &P = *v.plan;
  if (dev_out_len < P.n_out) {
    xg::set_error("xg_load_noalloc: output buffer shorter than the circuit's outputs");
    return XG_ERR_ARG;
  }
  if (P.n_terms > kScratchTerms) {
    xg::set_error("xg_load_noalloc: circuit needs " + std::to_string(P.n_terms) +
                  " stamp terms; the fixed scratch array holds " +
                  std::to_string(kScratchTerms) + " (use xg_load)");
    return XG_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(v.device);
  if (e != cudaSuccess) {
    xg::set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return XG_ERR_CUDA;
  }
  double *scratch = nullptr;
  int rc = scratch_on(v.device, &scratch);
  if (rc) return rc;
  xg::LoadIO io = v.io;
  io.terms = scratch;
  xg::Flags f{flags->dcop, flags->tranop, flags->acop, flags->transient, flags->init_jct,
              flags->init_fix, flags->newton_iter, flags->inputop, flags->pdt, flags->time,
              flags->init_tran};
  for (int k = 0; k < P.n_order; ++k) {
    const int t = P.order[k];
    const xg::TypeData &T = P.T[t];
    if (!T.n) continue;
    xg::DevType dt{T.n, T.nterm, T.sta0, T.sto0, T.term0, T.d_params, T.d_lid};
    rc = v.fma ? xg::fast::launch_eval(t, dt, v.opt, f, io, v.stream)
               : xg::exact::launch_eval(t, dt, v.opt, f, io, v.stream);
    if (rc) {
      xg::set_error("xg_load_noalloc: evaluation kernel launch failed");
      return rc;
    }
  }
  const xg::ReduceArgs ra = xg::reduce_args(P, scratch, v.red, dev_out, 0,
                                            P.n_out);
  rc = v.fma ? xg::fast::launch_reduce(ra, v.stream) : xg::exact::launch_reduce(ra, v.stream);
  if (rc) xg::set_error("xg_load_noalloc: reduction kernel launch failed");
  return rc;
}
