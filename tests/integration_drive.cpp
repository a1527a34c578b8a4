// integration_drive.cpp — test driver for the drop-in layer (integration/):
// runs GpuLoad::load over stand-in solver-state, vector and CSR-matrix types
// shaped like Xyce's (vector[lid], matrix[row][offset]) and DirectSolver on
// host CSR systems, behind a C interface the GPU tests call through ctypes.
// Test infrastructure only.
#include <N_DEV_GpuLoad.h>
#include <xg_direct_solver.h>

#include <cstring>
#include <memory>
#include <vector>

namespace {

struct State {  // the SolverState fields GpuLoad reads (N_DEV_SolverState.h:85-160)
  bool dcopFlag = false, tranopFlag = false, acopFlag = false, transientFlag = false;
  bool initJctFlag = false, initFixFlag = false, inputOPFlag = false, initTranFlag = false;
  int newtonIter = 0;
  double pdt = 0.0, currTime = 0.0;
};
struct Vec {
  double *d;
  double &operator[](int i) { return d[i]; }
  const double &operator[](int i) const { return d[i]; }
};
struct Mat {  // CSR rows addressed as row pointer + offset (N_LAS_Matrix::operator[])
  const int *rowptr;
  double *val;
  double *operator[](int r) { return val + rowptr[r]; }
};

std::unique_ptr<xg_integration::DirectSolver> g_solver;

}  // namespace

extern "C" {

// One load through GpuLoad with xg's own numbering as the "Xyce" numbering
// (identity maps); flags_i = {dcop, tranop, acop, transient, init_jct,
// init_fix, newton_iter, inputop, init_tran}, flags_d = {pdt, time}.
// F, Q: n_unknowns each; dFdx, dQdx: nnz each on xg's pattern.
int drive_gpuload(const xg_netlist *nl, const xg_device_options *opt, const int *flags_i,
                  const double *flags_d, const double *sol, double *F, double *Q, double *dFdx,
                  double *dQdx) {
  // xg's pattern first, to build the non-zero maps
  xg_ctx *ctx = nullptr;
  xg_circuit *ckt = nullptr;
  xg_circuit_info info{};
  if (xg_ctx_create(0, &ctx) || xg_circuit_create(ctx, nl, &ckt)) return -1;
  xg_circuit_get_info(ckt, &info);
  std::vector<int> rowptr(size_t(info.n_unknowns) + 1), col(size_t(info.nnz));
  xg_circuit_get_pattern(ckt, rowptr.data(), col.data());
  xg_circuit_destroy(ckt);
  xg_ctx_destroy(ctx);
  std::vector<int> lid(size_t(info.n_unknowns)), nz_row(size_t(info.nnz)), nz_off(size_t(info.nnz));
  for (int k = 0; k < info.n_unknowns; ++k) {
    lid[k] = k;
    for (int p = rowptr[k]; p < rowptr[k + 1]; ++p) {
      nz_row[p] = k;
      nz_off[p] = p - rowptr[k];
    }
  }
  try {
    xg_integration::GpuLoad g(*nl, *opt, 0, lid, nz_row, nz_off);
    State ss;
    ss.dcopFlag = flags_i[0];
    ss.tranopFlag = flags_i[1];
    ss.acopFlag = flags_i[2];
    ss.transientFlag = flags_i[3];
    ss.initJctFlag = flags_i[4];
    ss.initFixFlag = flags_i[5];
    ss.newtonIter = flags_i[6];
    ss.inputOPFlag = flags_i[7];
    ss.initTranFlag = flags_i[8];
    ss.pdt = flags_d[0];
    ss.currTime = flags_d[1];
    std::vector<double> x(sol, sol + info.n_unknowns);
    Vec vs{x.data()}, vf{F}, vq{Q};
    Mat mf{rowptr.data(), dFdx}, mq{rowptr.data(), dQdx};
    return g.load(ss, vs, vf, vq, mf, mq) ? 0 : -2;
  } catch (...) {
    return -3;
  }
}

// DirectSolver on one process-wide instance, so that successive calls can
// reuse factors; reset drops it.
void drive_direct_reset(int fp32) { g_solver.reset(new xg_integration::DirectSolver(0, fp32 != 0, 2)); }

int drive_direct_solve(int n, const int *rowptr, const int *col, const double *val, const double *b,
                       double *x, int reuse, int *singular, int *refactored, int *analyses) {
  if (!g_solver) drive_direct_reset(0);
  const int rc = g_solver->solve(n, rowptr, col, val, b, x, reuse != 0);
  *singular = g_solver->singular();
  *refactored = g_solver->refactored();
  *analyses = g_solver->analyses();
  return rc;
}

void drive_direct_free(void) { g_solver.reset(); }

}  // extern "C"
