// N_DEV_GpuLoad.h — the device-load half of the drop-in: xg's fused GPU
// Newton load in place of DeviceMgr's loops over every device Master.
//
// Reference interface replaced: DeviceMgr::updateState, loadDAEVectors and
// loadDAEMatrices (src/DeviceModelPKG/Core/src/N_DEV_DeviceMgr.C:2201-2285,
// 2520-2661, 2329-2479), which call Device::updateState / loadDAEVectors /
// loadDAEMatrices (src/DeviceModelPKG/Core/include/N_DEV_Device.h:200-265)
// for every Master in turn.  A maintainer adds this header under
// src/DeviceModelPKG/Core/include, lets DeviceMgr own one GpuLoad when a
// device option asks for it, and at the top of DeviceMgr::loadDAEVectors:
//
//     if (gpuLoad_)
//       return gpuLoad_->load(solState_, *nextSolVectorPtr, *daeFVectorPtr,
//                             *daeQVectorPtr, *dFdxMatrixPtr, *dQdxMatrixPtr);
//
// with updateState and loadDAEMatrices returning true at once while gpuLoad_
// is set (the fused call has done their work).  load() is a template over
// the solver-state, vector and matrix types so that the same code runs over
// Xyce's Xyce::Device::SolverState, N_LAS_Vector and N_LAS_Matrix, whose
// access it uses is the devices' own: vector[lid] and matrix[row][offset]
// (N_LAS_Matrix.C:863-879, the row pointer plus the offsets cached by
// registerJacLIDs).
//
// Set-up maps xg's numbering to Xyce's: lid[k] is the Xyce local id of xg
// unknown k, and for the k-th non-zero of xg's pattern (xg_circuit_get_
// pattern) nz_row[k] / nz_offset[k] give its Xyce row and its position in
// that row.  State and store vectors stay on the GPU (xg_rotate_history
// rotates them after an accepted step); F, Q, dF/dx and dQ/dx come back to
// the host for a host-side linear solve.  Every call returns bool, as the
// reference's load path does; set-up errors throw.
#ifndef Xyce_N_DEV_GpuLoad_h
#define Xyce_N_DEV_GpuLoad_h

#include <xg.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace xg_integration {

class GpuLoad {
 public:
  GpuLoad(const xg_netlist &nl, const xg_device_options &opt, int cuda_device,
          std::vector<int> lid, std::vector<int> nz_row, std::vector<int> nz_offset)
      : lid_(std::move(lid)), nzrow_(std::move(nz_row)), nzoff_(std::move(nz_offset)) {
    check(xg_ctx_create(cuda_device, &ctx_), "xg_ctx_create");
    if (int rc = xg_ctx_set_options(ctx_, &opt)) {
      xg_ctx_destroy(ctx_);
      check(rc, "xg_ctx_set_options");
    }
    if (int rc = xg_circuit_create(ctx_, &nl, &ckt_)) {
      xg_ctx_destroy(ctx_);
      check(rc, "xg_circuit_create");
    }
    xg_circuit_get_info(ckt_, &info_);
    if (int(lid_.size()) != info_.n_unknowns || int64_t(nzrow_.size()) != info_.nnz ||
        nzoff_.size() != nzrow_.size()) {
      release();
      throw std::invalid_argument("GpuLoad: numbering maps do not match the circuit");
    }
    x_.assign(size_t(info_.n_unknowns) + 1, 0.0);  // ground last, zero
    v_.resize(size_t(info_.n_unknowns) + 1);
    m_.resize(size_t(info_.nnz));
  }
  ~GpuLoad() { release(); }
  GpuLoad(const GpuLoad &) = delete;
  GpuLoad &operator=(const GpuLoad &) = delete;

  const xg_circuit_info &info() const { return info_; }
  xg_circuit *circuit() { return ckt_; }

  // updateState + loadDAEVectors + loadDAEMatrices for every device, one
  // call.  F and Q rows and the two matrices' entries of xg's pattern are
  // overwritten (the reference's caller zeroes them first; every entry the
  // load touches is written here).
  template <class SolverState, class Vector, class Matrix>
  bool load(const SolverState &ss, const Vector &sol, Vector &F, Vector &Q, Matrix &dFdx,
            Matrix &dQdx) {
    for (int k = 0; k < info_.n_unknowns; ++k) x_[k] = sol[lid_[k]];
    if (xg_vec_upload(ckt_, XG_VEC_SOL_NEXT, x_.data())) return false;
    xg_load_flags fl;
    fl.dcop = ss.dcopFlag;
    fl.tranop = ss.tranopFlag;
    fl.acop = ss.acopFlag;
    fl.transient = ss.transientFlag;
    fl.init_jct = ss.initJctFlag;
    fl.init_fix = ss.initFixFlag;
    fl.newton_iter = ss.newtonIter;
    fl.inputop = ss.inputOPFlag;
    fl.pdt = ss.pdt;
    fl.time = ss.currTime;
    fl.init_tran = ss.initTranFlag;
    if (xg_load(ckt_, &fl)) return false;
    return scatter(XG_VEC_F, F) && scatter(XG_VEC_Q, Q) && scatter_matrix(XG_VEC_DFDX, dFdx) &&
           scatter_matrix(XG_VEC_DQDX, dQdx);
  }

 private:
  static void check(int rc, const char *what) {
    if (rc) throw std::runtime_error(std::string(what) + ": " + xg_last_error());
  }
  template <class Vector>
  bool scatter(int id, Vector &v) {
    if (xg_vec_download(ckt_, id, v_.data())) return false;
    for (int k = 0; k < info_.n_unknowns; ++k) v[lid_[k]] = v_[k];
    return true;
  }
  template <class Matrix>
  bool scatter_matrix(int id, Matrix &m) {
    if (xg_vec_download(ckt_, id, m_.data())) return false;
    for (int64_t k = 0; k < info_.nnz; ++k) m[nzrow_[k]][nzoff_[k]] = m_[k];
    return true;
  }
  void release() {
    if (ckt_) xg_circuit_destroy(ckt_);
    if (ctx_) xg_ctx_destroy(ctx_);
    ckt_ = nullptr;
    ctx_ = nullptr;
  }

  xg_ctx *ctx_ = nullptr;
  xg_circuit *ckt_ = nullptr;
  xg_circuit_info info_{};
  std::vector<int> lid_, nzrow_, nzoff_;
  std::vector<double> x_, v_, m_;
};

}  // namespace xg_integration

#endif  // Xyce_N_DEV_GpuLoad_h
