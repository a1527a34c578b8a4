// api.cpp — the C ABI of libxg (include/xg.h): context and circuit lifetime,
// device-resident vectors, and the Newton-load entry points.
//
// The entry points mirror the reference's load interface:
//   xg_update_state       <- Device::updateState            (N_DEV_Device.h:200-265)
//   xg_load_dae_vectors   <- Device::loadDAEVectors
//   xg_load_dae_matrices  <- Device::loadDAEMatrices
// driven in DeviceMgr's order (N_DEV_DeviceMgr.C:2201-2661).  Each returns an
// int status (the reference's bool success) and never throws.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "xg.h"
#include "xg_internal.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? XG_ERR_OOM : XG_ERR_CUDA;
}

#define CK(call)                                          \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
  } while (0)

xg_device_options default_options() {
  xg_device_options o;
  o.gmin = 1e-12;
  o.temp = 300.15;
  o.tnom = 300.15;
  o.voltlim = 1;
  o.newmeyer = 0;
  o.fma = 0;
  return o;
}

}  // namespace

struct xg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  xg_device_options opt = default_options();
};

struct xg_circuit {
  xg_ctx *ctx = nullptr;
  xg_device_options opt;
  xg::Plan plan;
  // the LU analysis of the last transient's first Newton matrix, kept for the
  // next transient on this circuit (see circuit_lu_take)
  xg_lu *lu_cache = nullptr;
  uint64_t lu_cache_key = 0;
  double *d_sol[3] = {nullptr, nullptr, nullptr};
  double *d_sta[3] = {nullptr, nullptr, nullptr};
  double *d_sto[3] = {nullptr, nullptr, nullptr};
  double *d_out = nullptr;       // [F | Q | dFdxdVp | dQdxdVp | dFdx | dQdx]
  double *d_terms = nullptr;     // per-load stamp terms
  int64_t *d_red_ptr = nullptr;
  uint32_t *d_red_idx = nullptr;   // reduction entry -> term
  int64_t *d_long_out = nullptr; // outputs reduced by a warp each
  xg::EllBucket *d_ell = nullptr;    // the others as ELL buckets
  uint32_t *d_ell_out = nullptr, *d_ell_idx = nullptr;
  double *d_diode_vd = nullptr;  // Diode Instance::Vd carried between loads
  double *d_b3_mem = nullptr;    // BSIM3 members carried between loads
  bool state_done = false;
};
// Members carried between loads per BSIM3 instance (bsim3_eval.cuh, B3Mem).
static const int kB3MemPerInstance = 20;

namespace {

template <typename T>
int dalloc(T **p, int64_t count) {
  *p = nullptr;
  if (count <= 0) count = 1;
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)count);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  return XG_OK;
}

void free_circuit(xg_circuit *c) {
  if (c->lu_cache) xg_lu_destroy(c->lu_cache);
  c->lu_cache = nullptr;
  for (int k = 0; k < 3; ++k) {
    cudaFree(c->d_sol[k]);
    cudaFree(c->d_sta[k]);
    cudaFree(c->d_sto[k]);
  }
  cudaFree(c->d_out);
  cudaFree(c->d_terms);
  cudaFree(c->d_red_ptr);
  cudaFree(c->d_long_out);
  cudaFree(c->d_ell);
  cudaFree(c->d_ell_out);
  cudaFree(c->d_ell_idx);
  cudaFree(c->d_red_idx);
  cudaFree(c->d_diode_vd);
  cudaFree(c->d_b3_mem);
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    cudaFree(c->plan.T[t].d_params);
    cudaFree(c->plan.T[t].d_lid);
  }
}

int64_t vec_len(const xg_circuit *c, int id) {
  const xg::Plan &P = c->plan;
  switch (id) {
    case XG_VEC_SOL_NEXT: case XG_VEC_SOL_CURR: case XG_VEC_SOL_LAST:
    case XG_VEC_F: case XG_VEC_Q: case XG_VEC_DFDXDVP: case XG_VEC_DQDXDVP:
      return (int64_t)P.n_unknowns + 1;
    case XG_VEC_STA_NEXT: case XG_VEC_STA_CURR: case XG_VEC_STA_LAST: return P.n_state;
    case XG_VEC_STO_NEXT: case XG_VEC_STO_CURR: case XG_VEC_STO_LAST: return P.n_store;
    case XG_VEC_DFDX: case XG_VEC_DQDX: return P.nnz;
  }
  return -1;
}

double *vec_ptr(xg_circuit *c, int id) {
  const xg::Plan &P = c->plan;
  const int64_t W = (int64_t)P.n_unknowns + 1;
  switch (id) {
    case XG_VEC_SOL_NEXT: return c->d_sol[0];
    case XG_VEC_SOL_CURR: return c->d_sol[1];
    case XG_VEC_SOL_LAST: return c->d_sol[2];
    case XG_VEC_STA_NEXT: return c->d_sta[0];
    case XG_VEC_STA_CURR: return c->d_sta[1];
    case XG_VEC_STA_LAST: return c->d_sta[2];
    case XG_VEC_STO_NEXT: return c->d_sto[0];
    case XG_VEC_STO_CURR: return c->d_sto[1];
    case XG_VEC_STO_LAST: return c->d_sto[2];
    case XG_VEC_F: return c->d_out;
    case XG_VEC_Q: return c->d_out + W;
    case XG_VEC_DFDXDVP: return c->d_out + 2 * W;
    case XG_VEC_DQDXDVP: return c->d_out + 3 * W;
    case XG_VEC_DFDX: return c->d_out + P.n_vec_out;
    case XG_VEC_DQDX: return c->d_out + P.n_vec_out + P.nnz;
  }
  return nullptr;
}

int set_device(const xg_ctx *ctx) {
  CK(cudaSetDevice(ctx->device));
  return XG_OK;
}

}  // namespace

namespace xg {

void set_error(const std::string &msg) { g_err = msg; }

xg_lu *circuit_lu_take(xg_circuit *c, uint64_t key) {
  xg_lu *lu = c->lu_cache;
  c->lu_cache = nullptr;
  if (lu && c->lu_cache_key == key) return lu;
  if (lu) xg_lu_destroy(lu);
  return nullptr;
}

void circuit_lu_keep(xg_circuit *c, xg_lu *lu, uint64_t key) {
  if (c->lu_cache && c->lu_cache != lu) xg_lu_destroy(c->lu_cache);
  c->lu_cache = lu;
  c->lu_cache_key = key;
}

int circuit_reset_members(xg_circuit *c) {
  if (!c) return XG_ERR_ARG;
  const xg::Plan &P = c->plan;
  cudaStream_t s = c->ctx->stream;
  if (c->d_diode_vd && P.T[XG_DEV_DIODE].n)
    CK(cudaMemsetAsync(c->d_diode_vd, 0, sizeof(double) * P.T[XG_DEV_DIODE].n, s));
  if (c->d_b3_mem && P.T[XG_DEV_BSIM3].n)
    CK(cudaMemsetAsync(c->d_b3_mem, 0, sizeof(double) * kB3MemPerInstance * P.T[XG_DEV_BSIM3].n, s));
  c->state_done = false;
  return XG_OK;
}

static std::atomic<long long> g_launches{0};
void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

int sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

int ctx_info(xg_ctx *ctx, int *device, void **stream) {
  if (!ctx) return XG_ERR_ARG;
  *device = ctx->device;
  *stream = ctx->stream;
  return XG_OK;
}

int ctx_options(xg_ctx *ctx, xg_device_options *o) {
  if (!ctx || !o) return XG_ERR_ARG;
  *o = ctx->opt;
  return XG_OK;
}

int circuit_view(xg_circuit *c, CircuitView *v) {
  if (!c || !v) return XG_ERR_ARG;
  v->ctx = c->ctx;
  v->plan = &c->plan;
  v->device = c->ctx->device;
  v->stream = (void *)c->ctx->stream;
  v->fma = c->opt.fma;
  v->opt = DevOptions{c->opt.gmin, c->opt.voltlim};
  v->io = LoadIO{c->d_sol[0], c->d_sta[1], c->d_sto[1], c->d_sta[0], c->d_sto[0], c->d_terms,
                 c->d_diode_vd, c->d_b3_mem, c->d_sta[1]};
  v->red = ReduceLists{c->d_red_ptr, c->d_red_idx, c->d_long_out, c->d_ell, c->d_ell_out, c->d_ell_idx};
  return XG_OK;
}

ReduceArgs reduce_args(const Plan &P, const double *terms, const ReduceLists &L, double *out, int64_t o0,
                       int64_t o1) {
  auto lo = std::lower_bound(P.long_out.begin(), P.long_out.end(), o0);
  auto hi = std::lower_bound(P.long_out.begin(), P.long_out.end(), o1);
  ReduceArgs a{terms, L.red_ptr, L.red_idx, L.long_out + (lo - P.long_out.begin()), (int64_t)(hi - lo),
               out, o0, o1};
  // the short outputs of [o0, o1) (the vector part, the matrix part or both)
  // as buckets
  a.ell = L.ell;
  a.b0 = o0 >= P.n_vec_out ? P.n_ell_vec : 0;
  a.b1 = o1 <= P.n_vec_out ? P.n_ell_vec : (int)P.ell.size();
  a.ell_block0 = a.ell_blocks = 0;
  if (a.b1 > a.b0) {
    const EllBucket &last = P.ell[(size_t)a.b1 - 1];
    a.ell_block0 = P.ell[(size_t)a.b0].block0;
    a.ell_blocks = last.block0 + (last.m + kEllPerBlock - 1) / kEllPerBlock - a.ell_block0;
  }
  a.ell_out = L.ell_out;
  a.ell_idx = L.ell_idx;
  return a;
}

}  // namespace xg

extern "C" {

int xg_abi_version(void) { return XG_ABI_VERSION; }

const char *xg_last_error(void) { return g_err.c_str(); }

long long xg_launch_count(void) { return xg::g_launches.load(std::memory_order_relaxed); }

const char *xg_status_string(int status) {
  switch (status) {
    case XG_OK: return "ok";
    case XG_ERR_ARG: return "bad argument";
    case XG_ERR_CUDA: return "CUDA error";
    case XG_ERR_OOM: return "out of memory";
    case XG_ERR_SINGULAR: return "singular matrix";
    case XG_ERR_NAN: return "non-finite value";
    case XG_ERR_TIMEOUT: return "device wait timed out";
    case XG_ERR_STATE: return "call out of order";
    case XG_ERR_UNSUPPORTED: return "unsupported";
    case XG_ERR_NOCONV: return "Newton iteration did not converge";
  }
  return "unknown status";
}

int xg_ctx_create(int cuda_device, xg_ctx **out) {
  if (!out) return fail(XG_ERR_ARG, "null output pointer");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  if (cuda_device < 0 || cuda_device >= ndev) return fail(XG_ERR_ARG, "no such CUDA device");
  xg_ctx *ctx = new (std::nothrow) xg_ctx();
  if (!ctx) return fail(XG_ERR_OOM, "host allocation");
  ctx->device = cuda_device;
  e = cudaSetDevice(cuda_device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    return cuda_fail(e, "stream create");
  }
  *out = ctx;
  return XG_OK;
}

int xg_ctx_destroy(xg_ctx *ctx) {
  if (!ctx) return XG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return XG_OK;
}

int xg_ctx_set_options(xg_ctx *ctx, const xg_device_options *opt) {
  if (!ctx || !opt) return fail(XG_ERR_ARG, "null argument");
  if (opt->newmeyer) return fail(XG_ERR_UNSUPPORTED, "newmeyer=1 is not supported");
  ctx->opt = *opt;
  return XG_OK;
}

int xg_ctx_get_options(const xg_ctx *ctx, xg_device_options *opt) {
  if (!ctx || !opt) return fail(XG_ERR_ARG, "null argument");
  *opt = ctx->opt;
  return XG_OK;
}

int xg_ctx_synchronize(xg_ctx *ctx) {
  if (!ctx) return fail(XG_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(ctx->stream));
  return XG_OK;
}

int xg_ctx_stream(xg_ctx *ctx, void **stream_out) {
  if (!ctx || !stream_out) return fail(XG_ERR_ARG, "null argument");
  *stream_out = (void *)ctx->stream;
  return XG_OK;
}

int xg_circuit_create(xg_ctx *ctx, const xg_netlist *nl, xg_circuit **out) {
  if (!ctx || !nl || !out) return fail(XG_ERR_ARG, "null argument");
  *out = nullptr;
  int rc = set_device(ctx);
  if (rc) return rc;
  xg_circuit *c = new (std::nothrow) xg_circuit();
  if (!c) return fail(XG_ERR_OOM, "host allocation");
  c->ctx = ctx;
  c->opt = ctx->opt;
  std::string err;
  try {
    rc = xg::build_plan(nl, &c->opt, &c->plan, &err);
  } catch (const std::bad_alloc &) {
    rc = XG_ERR_OOM;
    err = "host allocation during setup";
  }
  if (rc) {
    delete c;
    return fail(rc, err);
  }
  xg::Plan &P = c->plan;
  const int64_t W = (int64_t)P.n_unknowns + 1;
  for (int k = 0; k < 3 && !rc; ++k) {
    rc = dalloc(&c->d_sol[k], W);
    if (!rc) rc = dalloc(&c->d_sta[k], P.n_state);
    if (!rc) rc = dalloc(&c->d_sto[k], P.n_store);
  }
  if (!rc) rc = dalloc(&c->d_out, P.n_out);
  if (!rc) rc = dalloc(&c->d_terms, P.n_terms);
  if (!rc) rc = dalloc(&c->d_red_ptr, P.n_out + 1);
  if (!rc) rc = dalloc(&c->d_red_idx, (int64_t)P.red_idx.size());
  if (!rc && !P.red_idx.empty() &&
      cudaMemcpy(c->d_red_idx, P.red_idx.data(), P.red_idx.size() * sizeof(uint32_t),
                 cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(XG_ERR_CUDA, "copy red_idx");
  if (!rc) rc = dalloc(&c->d_long_out, (int64_t)P.long_out.size());
  if (!rc && !P.ell.empty()) {
    rc = dalloc(&c->d_ell, (int64_t)P.ell.size());
    if (!rc) rc = dalloc(&c->d_ell_out, (int64_t)P.ell_out.size());
    if (!rc) rc = dalloc(&c->d_ell_idx, (int64_t)P.ell_idx.size());
    if (!rc && (cudaMemcpy(c->d_ell, P.ell.data(), P.ell.size() * sizeof(xg::EllBucket),
                           cudaMemcpyHostToDevice) != cudaSuccess ||
                (!P.ell_out.empty() &&
                 cudaMemcpy(c->d_ell_out, P.ell_out.data(), P.ell_out.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice) != cudaSuccess) ||
                (!P.ell_idx.empty() &&
                 cudaMemcpy(c->d_ell_idx, P.ell_idx.data(), P.ell_idx.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice) != cudaSuccess)))
      rc = fail(XG_ERR_CUDA, "copy ELL lists");
  }
  if (!rc && !P.long_out.empty() &&
      cudaMemcpy(c->d_long_out, P.long_out.data(), P.long_out.size() * sizeof(int64_t),
                 cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(XG_ERR_CUDA, "copy long_out");
  if (!rc) rc = dalloc(&c->d_diode_vd, P.T[XG_DEV_DIODE].n);
  if (!rc) rc = dalloc(&c->d_b3_mem, (int64_t)kB3MemPerInstance * P.T[XG_DEV_BSIM3].n);
  for (int t = 0; t < XG_NUM_DEV_TYPES && !rc; ++t) {
    xg::TypeData &T = P.T[t];
    if (!T.n) continue;
    rc = dalloc(&T.d_params, (int64_t)T.params.size());
    if (!rc) rc = dalloc(&T.d_lid, (int64_t)T.lid.size());
    if (!rc && cudaMemcpy(T.d_params, T.params.data(), T.params.size() * sizeof(double),
                          cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(XG_ERR_CUDA, "copy params");
    if (!rc && cudaMemcpy(T.d_lid, T.lid.data(), T.lid.size() * sizeof(int),
                          cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(XG_ERR_CUDA, "copy lids");
  }
  if (!rc && cudaMemcpy(c->d_red_ptr, P.red_ptr.data(), P.red_ptr.size() * sizeof(int64_t),
                        cudaMemcpyHostToDevice) != cudaSuccess) rc = fail(XG_ERR_CUDA, "copy red_ptr");
  if (!rc) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
      e = cudaMemset(c->d_sol[k], 0, W * sizeof(double));
      if (e == cudaSuccess && P.n_state) e = cudaMemset(c->d_sta[k], 0, P.n_state * sizeof(double));
      if (e == cudaSuccess && P.n_store) e = cudaMemset(c->d_sto[k], 0, P.n_store * sizeof(double));
    }
    if (e == cudaSuccess) e = cudaMemset(c->d_out, 0, P.n_out * sizeof(double));
    if (e == cudaSuccess && P.T[XG_DEV_DIODE].n)
      e = cudaMemset(c->d_diode_vd, 0, P.T[XG_DEV_DIODE].n * sizeof(double));
    if (e == cudaSuccess && P.T[XG_DEV_BSIM3].n)
      e = cudaMemset(c->d_b3_mem, 0,
                     (size_t)kB3MemPerInstance * P.T[XG_DEV_BSIM3].n * sizeof(double));
    if (e != cudaSuccess) rc = cuda_fail(e, "initialise vectors");
  }
  if (rc) {
    free_circuit(c);
    delete c;
    return rc;
  }
  // The host copies of the reduction lists are no longer needed.
  std::vector<uint32_t>().swap(P.red_idx);
  std::vector<uint32_t>().swap(P.ell_out);
  std::vector<uint32_t>().swap(P.ell_idx);
  std::vector<int64_t>().swap(P.short_order);
  *out = c;
  return XG_OK;
}

int xg_circuit_destroy(xg_circuit *c) {
  if (!c) return XG_OK;
  cudaSetDevice(c->ctx->device);
  cudaStreamSynchronize(c->ctx->stream);
  free_circuit(c);
  delete c;
  return XG_OK;
}

int xg_circuit_get_info(const xg_circuit *c, xg_circuit_info *info) {
  if (!c || !info) return fail(XG_ERR_ARG, "null argument");
  const xg::Plan &P = c->plan;
  std::memset(info, 0, sizeof *info);
  info->n_unknowns = P.n_unknowns;
  info->n_state = P.n_state;
  info->n_store = P.n_store;
  info->nnz = P.nnz;
  info->n_terms = P.n_terms;
  info->scratch_bytes = P.n_terms * (int64_t)sizeof(double);
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) info->n_instances[t] = P.T[t].n;
  return XG_OK;
}

int xg_circuit_get_pattern(const xg_circuit *c, int *host_rowptr, int *host_colidx) {
  if (!c || !host_rowptr || !host_colidx) return fail(XG_ERR_ARG, "null argument");
  const xg::Plan &P = c->plan;
  std::memcpy(host_rowptr, P.rowptr.data(), P.rowptr.size() * sizeof(int));
  std::memcpy(host_colidx, P.colidx.data(), P.colidx.size() * sizeof(int));
  return XG_OK;
}

int xg_circuit_get_params(const xg_circuit *c, int dev_type, double *host_out, int *n_params,
                          int *n_instances) {
  if (!c || dev_type < 0 || dev_type >= XG_NUM_DEV_TYPES) return fail(XG_ERR_ARG, "bad argument");
  const xg::TypeData &T = c->plan.T[dev_type];
  if (n_params) *n_params = T.np;
  if (n_instances) *n_instances = T.n;
  if (host_out && !T.params.empty())
    std::memcpy(host_out, T.params.data(), T.params.size() * sizeof(double));
  return XG_OK;
}

int xg_setup_params(const xg_netlist *nl, const xg_device_options *opt, int dev_type,
                    double *host_out, int *n_params, int *n_instances) {
  if (!nl || dev_type < 0 || dev_type >= XG_NUM_DEV_TYPES) return fail(XG_ERR_ARG, "bad argument");
  xg_device_options o = opt ? *opt : default_options();
  xg::Plan plan;
  std::string err;
  int rc;
  try {
    rc = xg::build_plan(nl, &o, &plan, &err, /*params_only=*/true);
  } catch (const std::bad_alloc &) {
    return fail(XG_ERR_OOM, "host allocation during setup");
  }
  if (rc) return fail(rc, err);
  const xg::TypeData &T = plan.T[dev_type];
  if (n_params) *n_params = T.np;
  if (n_instances) *n_instances = T.n;
  if (host_out && !T.params.empty())
    std::memcpy(host_out, T.params.data(), T.params.size() * sizeof(double));
  return XG_OK;
}

int xg_vec_size(const xg_circuit *c, int vec_id, int64_t *n) {
  if (!c || !n) return fail(XG_ERR_ARG, "null argument");
  int64_t len = vec_len(c, vec_id);
  if (len < 0) return fail(XG_ERR_ARG, "bad vector id");
  *n = len;
  return XG_OK;
}

int xg_vec_upload(xg_circuit *c, int vec_id, const double *host_src) {
  if (!c || !host_src) return fail(XG_ERR_ARG, "null argument");
  int64_t len = vec_len(c, vec_id);
  if (len < 0) return fail(XG_ERR_ARG, "bad vector id");
  int rc = set_device(c->ctx);
  if (rc) return rc;
  double *d = vec_ptr(c, vec_id);
  if (len) CK(cudaMemcpyAsync(d, host_src, len * sizeof(double), cudaMemcpyHostToDevice, c->ctx->stream));
  if (vec_id <= XG_VEC_SOL_LAST)  // ground holds 0 whatever the caller passed
    CK(cudaMemsetAsync(d + c->plan.n_unknowns, 0, sizeof(double), c->ctx->stream));
  CK(cudaStreamSynchronize(c->ctx->stream));
  return XG_OK;
}

int xg_vec_download(xg_circuit *c, int vec_id, double *host_dst) {
  if (!c || !host_dst) return fail(XG_ERR_ARG, "null argument");
  int64_t len = vec_len(c, vec_id);
  if (len < 0) return fail(XG_ERR_ARG, "bad vector id");
  int rc = set_device(c->ctx);
  if (rc) return rc;
  if (len)
    CK(cudaMemcpyAsync(host_dst, vec_ptr(c, vec_id), len * sizeof(double), cudaMemcpyDeviceToHost,
                       c->ctx->stream));
  CK(cudaStreamSynchronize(c->ctx->stream));
  return XG_OK;
}

int xg_vec_device_ptr(xg_circuit *c, int vec_id, double **dev_ptr) {
  if (!c || !dev_ptr) return fail(XG_ERR_ARG, "null argument");
  if (vec_len(c, vec_id) < 0) return fail(XG_ERR_ARG, "bad vector id");
  *dev_ptr = vec_ptr(c, vec_id);
  return XG_OK;
}

int xg_rotate_history(xg_circuit *c) {
  if (!c) return fail(XG_ERR_ARG, "null argument");
  int rc = set_device(c->ctx);
  if (rc) return rc;
  const xg::Plan &P = c->plan;
  double **v[3] = {c->d_sol, c->d_sta, c->d_sto};
  int64_t len[3] = {(int64_t)P.n_unknowns + 1, P.n_state, P.n_store};
  for (int k = 0; k < 3; ++k) {
    double *oldlast = v[k][2];
    v[k][2] = v[k][1];
    v[k][1] = v[k][0];
    v[k][0] = oldlast;
    if (len[k])
      CK(cudaMemcpyAsync(v[k][0], v[k][1], len[k] * sizeof(double), cudaMemcpyDeviceToDevice,
                         c->ctx->stream));
  }
  return XG_OK;
}

int xg_update_state(xg_circuit *c, const xg_load_flags *flags) {
  if (!c || !flags) return fail(XG_ERR_ARG, "null argument");
  int rc = set_device(c->ctx);
  if (rc) return rc;
  xg::Plan &P = c->plan;
  xg::DevOptions o{c->opt.gmin, c->opt.voltlim};
  xg::Flags f{flags->dcop, flags->tranop, flags->acop, flags->transient, flags->init_jct,
              flags->init_fix, flags->newton_iter, flags->inputop, flags->pdt, flags->time,
              flags->init_tran};
  xg::LoadIO io{c->d_sol[0], c->d_sta[1], c->d_sto[1], c->d_sta[0], c->d_sto[0], c->d_terms,
                c->d_diode_vd, c->d_b3_mem, c->d_sta[1]};
  for (int k = 0; k < P.n_order; ++k) {
    int t = P.order[k];
    const xg::TypeData &T = P.T[t];
    if (!T.n) continue;
    xg::DevType dt{T.n, T.nterm, T.sta0, T.sto0, T.term0, T.d_params, T.d_lid};
    rc = c->opt.fma ? xg::fast::launch_eval(t, dt, o, f, io, c->ctx->stream)
                    : xg::exact::launch_eval(t, dt, o, f, io, c->ctx->stream);
    if (rc) return fail(rc, rc == XG_ERR_CUDA ? "eval kernel launch failed" : "unsupported device type");
  }
  c->state_done = true;
  return XG_OK;
}

static int reduce_range(xg_circuit *c, int64_t o0, int64_t o1) {
  xg::CircuitView v;
  xg::circuit_view(c, &v);
  const xg::ReduceArgs a = xg::reduce_args(c->plan, c->d_terms, v.red, c->d_out, o0, o1);
  int rc = c->opt.fma ? xg::fast::launch_reduce(a, c->ctx->stream)
                      : xg::exact::launch_reduce(a, c->ctx->stream);
  return rc ? fail(rc, "reduce kernel launch failed") : XG_OK;
}

int xg_load_dae_vectors(xg_circuit *c) {
  if (!c) return fail(XG_ERR_ARG, "null argument");
  if (!c->state_done) return fail(XG_ERR_STATE, "xg_update_state must come first");
  int rc = set_device(c->ctx);
  if (rc) return rc;
  return reduce_range(c, 0, c->plan.n_vec_out);
}

int xg_load_dae_matrices(xg_circuit *c) {
  if (!c) return fail(XG_ERR_ARG, "null argument");
  if (!c->state_done) return fail(XG_ERR_STATE, "xg_update_state must come first");
  int rc = set_device(c->ctx);
  if (rc) return rc;
  return reduce_range(c, c->plan.n_vec_out, c->plan.n_out);
}

int xg_load(xg_circuit *c, const xg_load_flags *flags) {
  int rc = xg_update_state(c, flags);
  if (rc) return rc;
  return reduce_range(c, 0, c->plan.n_out);
}

}  // extern "C"
