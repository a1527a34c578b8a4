// xg_internal.h — structures shared by the host setup (setup.cpp), the C ABI
// (api.cpp) and the load kernels (load_kernels.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "xg.h"
#include "xg_params.h"

namespace xg {

// Where a stamp term lands.  Vector outputs address (kind, LID slot j);
// matrix outputs address (kind, row LID slot j, col LID slot j2).  LID slots
// index the instance's LID list (terminals then internal unknowns).
enum OutKind : int8_t { OUT_F = 0, OUT_Q, OUT_DFDXDVP, OUT_DQDXDVP, OUT_DFDX, OUT_DQDX };

struct TermDef {
  OutKind kind;
  int8_t row;   // LID slot of the equation (row)
  int8_t col;   // LID slot of the unknown (column), matrices only
};

// Per-type static description: LIDs per instance and the ordered stamp
// terms the load kernel writes (the statement order of the reference Master
// loops).  Defined in setup.cpp.
struct TypeLayout {
  int nlid;
  int nterm;
  const TermDef *terms;
  int np;
  int nsta, nsto;
};
const TypeLayout &type_layout(int dev_type);

// Per-type data prepared by setup.
struct TypeData {
  int n = 0;                   // instances
  int np = 0, nlid = 0, nterm = 0, nsta = 0, nsto = 0;
  int sta0 = 0, sto0 = 0;      // first state / store slot
  int64_t term0 = 0;           // first term in the per-load term buffer
  std::vector<double> params;  // SoA: params[k * n + i]
  std::vector<int> lid;        // SoA: lid[j * n + i]; ground = n_unknowns
  // device copies
  double *d_params = nullptr;
  int *d_lid = nullptr;
};

struct Flags;

// Device-side view of one device type, passed to kernels by value.
struct DevType {
  int n;
  int nterm;
  int sta0, sto0;
  int64_t term0;
  const double *p;   // SoA params
  const int *lid;    // SoA LIDs
  // Batched loads of independent circuits: the circuit of each instance and
  // the per-circuit load flags (null: every instance uses the launch's flags).
  // An instance whose circuit is negative (an unused place in a slot) or whose
  // circuit's flags say skip (a finished request) is not evaluated.
  const int *cid = nullptr;
  const Flags *cflags = nullptr;
};

struct DevOptions {
  double gmin;
  int voltlim;
};

struct Flags {
  int dcop, tranop, acop, transient, init_jct, init_fix, newton_iter, inputop;
  double pdt, time;
  int init_tran;
  int skip;  // batched loads: the circuit is not evaluated (it has finished)
};

// Vectors the load kernels read and write (device pointers).
struct LoadIO {
  const double *sol;        // next solution, n_unknowns + 1 (ground = 0)
  const double *sta_curr, *sto_curr;
  double *sta, *sto;        // next state / store (sto holds previous iterate on entry)
  double *terms;            // per-load stamp terms, term q of instance i at term0 + q*n + i
  double *diode_vd;         // Diode Instance::Vd carried between loads
  double *b3_mem;           // BSIM3 members carried between loads, [k*n + i]
  double *sta_curr_w;       // current state, written on the first transient step
};

// The short outputs, grouped by term count (a sliced ELL layout): bucket b holds m outputs of c terms each; its output numbers are
// ell_out[out0 .. out0+m) and term j of its k-th output is term
// ell_idx[idx0 + j*m + k], so a thread per output reads its term numbers
// coalesced with its neighbours' and has all of them in flight at once.
// block0: the bucket's first block in a launch over all buckets (a block
// takes kEllPerBlock outputs).
struct EllBucket {
  int64_t out0, idx0, block0;
  int32_t m, c;
};
constexpr int kEllThreads = 256;
constexpr int kEllPerThread = 2;  // outputs per thread (their loads interleaved)
constexpr int kEllPerBlock = kEllThreads * kEllPerThread;

// Everything setup derives from a netlist (host side).
struct Plan {
  int n_nodes = 0, n_unknowns = 0, n_state = 0, n_store = 0;
  int order[XG_NUM_DEV_TYPES];
  int n_order = 0;
  TypeData T[XG_NUM_DEV_TYPES];
  // solved Jacobian pattern (ground excluded)
  std::vector<int> rowptr, colidx;
  int64_t nnz = 0;
  // output space: [F | Q | dFdxdVp | dQdxdVp] (n_unknowns+1 each) then dFdx, dQdx (nnz each)
  int64_t n_out = 0, n_vec_out = 0;
  int64_t n_terms = 0;
  // fixed-order reduction: red_ptr[o]..red_ptr[o+1] are the term indices
  // summed, in reference order, into output o
  std::vector<int64_t> red_ptr;
  std::vector<uint32_t> red_idx;
  // Terms are written in [q][i] order (a warp's stores fill whole sectors)
  // and output o gathers terms red_idx[red_ptr[o]..red_ptr[o+1]).
  // outputs summing more than kLongSegment terms (a supply node's row), in
  // ascending order: reduced by a warp each instead of a thread
  std::vector<int64_t> long_out;
  // the other outputs, vector outputs first, then matrix outputs, each part
  // sorted by term count: a warp then sums segments of one length
  std::vector<int64_t> short_order;
  int64_t n_short_vec = 0;    // short outputs in [0, n_vec_out)
  // the short outputs as ELL buckets, the vector part's (n_ell_vec of them)
  // first, then the matrix part's
  std::vector<EllBucket> ell;
  int n_ell_vec = 0;
  std::vector<uint32_t> ell_out, ell_idx;
};
constexpr int64_t kLongSegment = 64;


// The reduction's device data and the long outputs inside [o0, o1).
struct ReduceArgs {
  const double *terms;
  const int64_t *red_ptr;
  const uint32_t *red_idx;    // term of each reduction entry
  const int64_t *long_out;    // device, the sub-range of long outputs in [o0, o1)
  int64_t n_long;
  double *out;
  int64_t o0, o1;
  // the short outputs of [o0, o1) as buckets [b0, b1) of the ELL lists,
  // ell_blocks blocks from block ell_block0 on
  const EllBucket *ell;
  int b0, b1;
  int64_t ell_block0, ell_blocks;
  const uint32_t *ell_out, *ell_idx;
};

// A circuit's reduction lists on the device.
struct ReduceLists {
  const int64_t *red_ptr;
  const uint32_t *red_idx;
  const int64_t *long_out;     // device copy of plan->long_out
  const EllBucket *ell;        // the short outputs' ELL lists
  const uint32_t *ell_out, *ell_idx;
};

// setup.cpp
// params_only: stop after the per-instance parameter blocks (no numbering,
// pattern or term plan).
int build_plan(const xg_netlist *nl, const xg_device_options *opt, Plan *plan, std::string *err,
               bool params_only = false);

// Read-only view of a circuit's device data (api.cpp), for entry points
// implemented in other translation units.
struct CircuitView {
  xg_ctx *ctx;
  const Plan *plan;
  int device;
  void *stream;
  int fma;
  DevOptions opt;
  LoadIO io;                   // terms = the circuit's own term buffer
  ReduceLists red;
};
int circuit_view(xg_circuit *c, CircuitView *v);
// ReduceArgs for outputs [o0, o1) of a circuit's plan (long outputs located
// on the host copy, addressed in the device copy).
ReduceArgs reduce_args(const Plan &P, const double *terms, const ReduceLists &L, double *out, int64_t o0,
                       int64_t o1);
void set_error(const std::string &msg);
// Kernel launches of this library, counted at every launch site (api.cpp).
void count_launches(int k);
// Streaming multiprocessors of the current CUDA device (queried once per
// device); grids are sized in multiples of it.
int sm_count();
// Zero the members carried between loads (diode Vd, BSIM3 charges/caps).
int circuit_reset_members(xg_circuit *c);
// A transient keeps its LU analysis in the circuit when it ends; the next
// transient on the circuit takes it back when its first Newton matrix is the
// same (key: a hash of the values and the precision), the case in which a
// fresh analysis would find the same pivot order.  Otherwise the kept one is
// destroyed and nullptr returned.
xg_lu *circuit_lu_take(xg_circuit *c, uint64_t key);
void circuit_lu_keep(xg_circuit *c, xg_lu *lu, uint64_t key);
// The device and stream of a context (api.cpp).
int ctx_info(xg_ctx *ctx, int *device, void **stream);
// The device options a context's circuits are set up and loaded with.
int ctx_options(xg_ctx *ctx, xg_device_options *o);
// Breakpoints of the PULSE sources (both corners of each edge, every period,
// up to tstop) and tstop itself, sorted and unique (tran.cu).  lo/hi, when
// given, restrict the sources to instances [lo[0], hi[0]) of VSRC and
// [lo[1], hi[1]) of ISRC: one request of a batch.
std::vector<double> pulse_breakpoints(const Plan &P, double tstop, const int *lo = nullptr,
                                      const int *hi = nullptr);

// load_kernels.cu (two builds: bit-exact and FMA-contracted)
namespace exact {
int launch_eval(int dev_type, const DevType &t, const DevOptions &o, const Flags &f,
                const LoadIO &io, void *stream);
int launch_reduce(const ReduceArgs &a, void *stream);
}  // namespace exact
namespace fast {
int launch_eval(int dev_type, const DevType &t, const DevOptions &o, const Flags &f,
                const LoadIO &io, void *stream);
int launch_reduce(const ReduceArgs &a, void *stream);
}  // namespace fast

}  // namespace xg
