// xref_tia.C — drives the reference's own time-integration and Newton
// convergence code, compiled from its unmodified sources, on plain arrays:
// the golden maker of the transient oracle's pin.  Test infrastructure only:
// the product never links this.
//
// Reference code run (src/TimeIntegrationPKG/src, src/NonlinearSolverPKG/src):
//   N_TIA_OneStep::updateCoeffs       N_TIA_OneStep.C:1355-1480
//   N_TIA_OneStep::obtainPredictor    N_TIA_OneStep.C:115-205
//   N_TIA_OneStep::obtainResidual     N_TIA_OneStep.C:215-290
//   N_TIA_OneStep::obtainJacobian     N_TIA_OneStep.C:297-352
//   N_TIA_DataStore::setErrorWtVector N_TIA_DataStore.C:1200-1370
//   N_TIA_DataStore::WRMS_errorNorm   N_TIA_DataStore.C:1380-1400
//   N_TIA_OneStep::computeErrorEstimate's product ck * WRMS_errorNorm
//                                     (include/N_TIA_OneStep.h:97)
//   N_NLS_DampedNewton::converged_    N_NLS_DampedNewton.C:1787-1919
//
// What it supplies in place of Trilinos (which the reference needs and this
// tree does not have): the N_LAS_MultiVector / N_LAS_Vector / N_LAS_Matrix
// members those functions call, over caller arrays, with the Epetra
// operations they wrap (N_LAS_MultiVector.C:257-860, N_LAS_Matrix.C:835-853):
// Update(a, A, b, B, 0) = a*A + b*B, Scale, Abs, PutScalar, NormInf,
// NormWeighted = sqrt(sum((x_i / w_i)^2) / n), copy; and this = a*A + b*B
// over the values of a matrix.  The reference's objects (data store, step
// error control, parameters, Newton solver) are not constructed through
// their Trilinos-bound constructors: the members the functions read are set
// on zeroed storage, as the device harness does for the load.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <list>
#include <map>
#include <new>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#define private public
#define protected public
#include <Xyce_config.h>
#include <N_IO_OutputMgr.h>
#include <N_LAS_BlockVector.h>
#include <N_LAS_Matrix.h>
#include <N_LAS_MultiVector.h>
#include <N_PDS_ParMap.h>
#include <N_LAS_Vector.h>
#include <N_LOA_Loader.h>
#include <N_NLS_DampedNewton.h>
#include <N_NLS_ParamMgr.h>
#include <N_TIA_DataStore.h>
#include <N_TIA_OneStep.h>
#include <N_TIA_StepErrorControl.h>
#include <N_TIA_TIAParams.h>
#undef private
#undef protected

#define XREF_API extern "C" __attribute__((visibility("default")))

// ---------------------------------------------------------------------------
// Vector and matrix stand-ins
// ---------------------------------------------------------------------------
namespace {
struct Arr {
  double *d;
  int64_t n;
};
std::map<const void *, Arr> g_arr;
const Arr &arr(const void *p) { return g_arr.at(p); }
}  // namespace

double &N_LAS_Vector::operator[](int i) { return g_arr.at(this).d[i]; }
const double &N_LAS_Vector::operator[](int i) const { return g_arr.at(this).d[i]; }
N_LAS_MultiVector &N_LAS_MultiVector::operator=(const N_LAS_MultiVector &right) {
  const Arr &a = arr(this), &b = arr(&right);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = b.d[i];
  return *this;
}
void N_LAS_MultiVector::scale(const double s) {
  const Arr &a = arr(this);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = s * a.d[i];
}
void N_LAS_MultiVector::daxpy(const N_LAS_MultiVector &y, const double s, const N_LAS_MultiVector &x) {
  const Arr &a = arr(this), &ya = arr(&y), &xa = arr(&x);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = 1.0 * ya.d[i] + s * xa.d[i];
}
void N_LAS_MultiVector::linearCombo(const double s, const N_LAS_MultiVector &x, const double t,
                                    const N_LAS_MultiVector &y) {
  const Arr &a = arr(this), &xa = arr(&x), &ya = arr(&y);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = s * xa.d[i] + t * ya.d[i];
}
void N_LAS_MultiVector::putScalar(const double s) {
  const Arr &a = arr(this);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = s;
}
void N_LAS_MultiVector::absValue(const N_LAS_MultiVector &A) {
  const Arr &a = arr(this), &b = arr(&A);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = std::fabs(b.d[i]);
}
int N_LAS_MultiVector::infNorm(double *result) const {
  const Arr &a = arr(this);
  double m = 0.0;
  for (int64_t i = 0; i < a.n; ++i) m = std::fabs(a.d[i]) > m ? std::fabs(a.d[i]) : m;
  *result = m;
  return 0;
}
int N_LAS_MultiVector::wRMSNorm(const N_LAS_MultiVector &weights, double *result) const {
  const Arr &a = arr(this), &w = arr(&weights);
  double s = 0.0;
  for (int64_t i = 0; i < a.n; ++i) {
    const double t = a.d[i] / w.d[i];
    s += t * t;
  }
  *result = std::sqrt(s / double(a.n));
  return 0;
}
void N_LAS_MultiVector::update(double s, const N_LAS_MultiVector &A, double t) {
  const Arr &a = arr(this), &b = arr(&A);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = s * b.d[i] + t * a.d[i];
}
void N_LAS_MultiVector::linearCombo(const double s, const N_LAS_MultiVector &x, const double t,
                                    const N_LAS_MultiVector &y, const double u,
                                    const N_LAS_MultiVector &z) {
  const Arr &a = arr(this), &xa = arr(&x), &ya = arr(&y), &za = arr(&z);
  for (int64_t i = 0; i < a.n; ++i) a.d[i] = s * xa.d[i] + t * ya.d[i] + u * za.d[i];
}
void N_LAS_Matrix::linearCombo(const double s, const N_LAS_Matrix &A, const double t,
                               const N_LAS_Matrix &B) {
  const Arr &a = arr(this), &x = arr(&A), &y = arr(&B);
  for (int64_t k = 0; k < a.n; ++k) a.d[k] = s * x.d[k] + t * y.d[k];
}

// Construction of a vector the functions receive: the reference's virtual
// calls (putScalar) need a real object, but its constructors need Epetra.
// These definitions build one without a Trilinos vector; the harness binds
// its storage (g_arr) instead.
N_LAS_MultiVector::N_LAS_MultiVector(Epetra_MultiVector *, bool)
    : aMultiVector_(0), oMultiVector_(0), importer_(0), exporter_(0), viewTransform_(0),
      isOwned_(false) {}
N_LAS_Vector::N_LAS_Vector(Epetra_Vector *v, bool owned)
    : N_LAS_MultiVector(reinterpret_cast<Epetra_MultiVector *>(v), owned) {}
N_LAS_MultiVector::~N_LAS_MultiVector() {}

// Members that reference code linked here names on paths the entry points
// never take (block vectors of multi-time analyses, output, parallel maps,
// packing): defined so the library links; each aborts if ever reached.
N_LAS_MultiVector::N_LAS_MultiVector(const N_LAS_MultiVector &) : Packable() { std::abort(); }
int N_LAS_MultiVector::packedByteCount() const { std::abort(); }
void N_LAS_MultiVector::pack(char *, int, int &, N_PDS_Comm *) const { std::abort(); }
void N_LAS_MultiVector::unpack(char *, int, int &, N_PDS_Comm *) { std::abort(); }
void N_LAS_MultiVector::addScalar(const double) { std::abort(); }
void N_LAS_MultiVector::writeToFile(char *, bool) { std::abort(); }
void N_LAS_MultiVector::readFromFile(char *) { std::abort(); }
void N_LAS_MultiVector::printPetraObject(std::ostream &) const { std::abort(); }
void N_LAS_BlockVector::printPetraObject(std::ostream &) const { std::abort(); }
int N_PDS_ParMap::globalToLocalIndex(const int &) { std::abort(); }
void Xyce::IO::OutputMgr::outputDCOP(N_LAS_Vector &) { std::abort(); }
void Xyce::IO::OutputMgr::output(const double &, const int, const int,
                                 const std::vector<N_ANP_SweepParam> &, const int, const int,
                                 const std::vector<N_ANP_SweepParam> &, N_LAS_Vector *,
                                 N_LAS_Vector *, N_LAS_Vector *, const std::vector<double> &,
                                 const std::vector<double> &, const std::vector<double> &,
                                 const std::vector<double> &, const std::vector<double> &, bool) {
  std::abort();
}

namespace {

template <class T>
struct Raw {  // zeroed storage for a reference object whose constructor needs Trilinos
  alignas(T) unsigned char buf[sizeof(T)];
  Raw() { std::memset(buf, 0, sizeof buf); }
  T *get() { return reinterpret_cast<T *>(buf); }
};

struct Vec {  // one bound vector
  Raw<N_LAS_Vector> obj;
  Vec() { new (obj.get()) N_LAS_Vector(static_cast<Epetra_Vector *>(0), false); }
  N_LAS_Vector *bind(double *d, int64_t n) {
    g_arr[obj.get()] = Arr{d, n};
    return obj.get();
  }
  ~Vec() {
    g_arr.erase(obj.get());
    obj.get()->~N_LAS_Vector();
  }
};
struct Mat {
  Raw<N_LAS_Matrix> obj;
  N_LAS_Matrix *bind(double *d, int64_t n) {
    g_arr[obj.get()] = Arr{d, n};
    return obj.get();
  }
  ~Mat() { g_arr.erase(obj.get()); }
};

// The integrator: zeroed data store, step error control and parameters, and
// a OneStep constructed on them (its constructor only reads the parameters'
// order limits, N_TIA_OneStep.C:89-104).
struct Integrator {
  Raw<N_TIA_TIAParams> params;
  Raw<N_TIA_StepErrorControl> sec;
  Raw<N_TIA_DataStore> ds;
  N_TIA_OneStep *method = nullptr;
  Integrator() {
    params.get()->maxOrder = 2;
    params.get()->minOrder = 1;
    N_TIA_StepErrorControl &c = *sec.get();
    for (std::vector<double> *v : {&c.alpha_, &c.sigma_, &c.gamma_, &c.beta_, &c.psi_})
      new (v) std::vector<double>(6, 0.0);
    new (&ds.get()->xHistory) std::vector<N_LAS_Vector *>();
    new (&ds.get()->qHistory) std::vector<N_LAS_Vector *>();
    new (&ds.get()->sHistory) std::vector<N_LAS_Vector *>();
    new (&ds.get()->stoHistory) std::vector<N_LAS_Vector *>();
    new (&ds.get()->stoLeadCurrQCompHistory) std::vector<N_LAS_Vector *>();
    method = new N_TIA_OneStep(*params.get(), *sec.get(), *ds.get());
  }
  ~Integrator() {
    delete method;
    typedef std::vector<double> D;
    N_TIA_StepErrorControl &c = *sec.get();
    for (D *v : {&c.alpha_, &c.sigma_, &c.gamma_, &c.beta_, &c.psi_}) v->~D();
    typedef std::vector<N_LAS_Vector *> V;
    ds.get()->xHistory.~V();
    ds.get()->qHistory.~V();
    ds.get()->sHistory.~V();
    ds.get()->stoHistory.~V();
    ds.get()->stoLeadCurrQCompHistory.~V();
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// Entry points
// ---------------------------------------------------------------------------

// updateCoeffs: in psi[3] (the step history), order, h, h_sum; out psi,
// beta[3], *alphas, *ck.
XREF_API void xref_tia_update_coeffs(int order, double h, double h_sum, double *psi, double *beta,
                                     double *alphas, double *ck) {
  Integrator I;
  N_TIA_StepErrorControl &sec = *I.sec.get();
  sec.currentOrder_ = order;
  sec.currentTimeStep = h;
  sec.currentTimeStepSum = h_sum;
  for (int k = 0; k < 3; ++k) sec.psi_[k] = psi[k];
  I.method->N_TIA_OneStep::updateCoeffs();
  for (int k = 0; k < 3; ++k) {
    psi[k] = sec.psi_[k];
    beta[k] = sec.beta_[k];
  }
  *alphas = sec.alphas_;
  *ck = sec.ck_;
}

// obtainPredictor: xn0 = xh0 + sum_i beta[i] xh_i (i = 1..order), qn0 = qh0.
XREF_API void xref_tia_predictor(int n, int order, const double *beta, double *xh0, double *xh1,
                                 double *xh2, double *qh0, double *xn0, double *qn0) {
  Integrator I;
  N_TIA_StepErrorControl &sec = *I.sec.get();
  N_TIA_DataStore &ds = *I.ds.get();
  sec.currentOrder_ = order;
  for (int k = 0; k < 3; ++k) sec.beta_[k] = beta[k];
  std::vector<double> zero(size_t(n) + 1, 0.0), scratch(8 * (size_t(n) + 1), 0.0);
  Vec vx[3], vq, vxn0, vqn0, vs[8];
  ds.xHistory = {vx[0].bind(xh0, n), vx[1].bind(xh1, n), vx[2].bind(xh2, n)};
  ds.qHistory = {vq.bind(qh0, n)};
  for (int k = 0; k < 8; ++k) vs[k].bind(&scratch[k * (size_t(n) + 1)], n);
  ds.sHistory = {vs[0].obj.get()};
  ds.stoHistory = {vs[1].obj.get()};
  ds.stoLeadCurrQCompHistory = {vs[2].obj.get()};
  ds.xn0Ptr = vxn0.bind(xn0, n);
  ds.qn0Ptr = vqn0.bind(qn0, n);
  ds.sn0Ptr = vs[3].obj.get();
  ds.ston0Ptr = vs[4].obj.get();
  ds.stoQCn0Ptr = vs[5].obj.get();
  ds.spn0Ptr = vs[6].obj.get();
  ds.stopn0Ptr = vs[7].obj.get();
  ds.stoQCpn0Ptr = vs[6].obj.get();
  ds.nextSolutionPtr = vs[7].obj.get();
  I.method->N_TIA_OneStep::obtainPredictor();
}

// obtainResidual: rhs = -[(Q - qn0)/h + f F + f qhist2] + limiter terms, in
// the reference's operation order; dqdxdvp is scaled in place by
// -alphas/h, as the reference's data store vector is.
XREF_API void xref_tia_residual(int n, int order, double h, double alphas, int limiter,
                                double *Q, double *qn0, double *F, double *qhist2,
                                double *dfdxdvp, double *dqdxdvp, double *rhs) {
  Integrator I;
  N_TIA_StepErrorControl &sec = *I.sec.get();
  N_TIA_DataStore &ds = *I.ds.get();
  sec.currentOrder_ = order;
  sec.currentTimeStep = h;
  sec.alphas_ = alphas;
  ds.limiterFlag = limiter != 0;
  Vec vr, vq, vqn0, vf, vh[3], vfp, vqp;
  ds.RHSVectorPtr = vr.bind(rhs, n);
  ds.daeQVectorPtr = vq.bind(Q, n);
  ds.qn0Ptr = vqn0.bind(qn0, n);
  ds.daeFVectorPtr = vf.bind(F, n);
  ds.qHistory = {vh[0].bind(qhist2, n), vh[1].bind(qhist2, n), vh[2].bind(qhist2, n)};
  ds.dFdxdVpVectorPtr = vfp.bind(dfdxdvp, n);
  ds.dQdxdVpVectorPtr = vqp.bind(dqdxdvp, n);
  ds.nextSolutionPtr = vf.obj.get();
  I.method->N_TIA_OneStep::obtainResidual();
}

// obtainJacobian: jac = (-alphas/h) dQdx + f dFdx over nnz matrix values.
XREF_API void xref_tia_jacobian(int64_t nnz, int order, double h, double alphas, double *dqdx,
                                double *dfdx, double *jac) {
  Integrator I;
  N_TIA_StepErrorControl &sec = *I.sec.get();
  N_TIA_DataStore &ds = *I.ds.get();
  sec.currentOrder_ = order;
  sec.currentTimeStep = h;
  sec.alphas_ = alphas;
  Mat mq, mf, mj;
  ds.dQdxMatrixPtr = mq.bind(dqdx, nnz);
  ds.dFdxMatrixPtr = mf.bind(dfdx, nnz);
  ds.JMatrixPtr = mj.bind(jac, nnz);
  I.method->N_TIA_OneStep::obtainJacobian();
}

// setErrorWtVector (newLte, no fast tests: every unknown a voltage
// variable) then computeErrorEstimate = ck * WRMS_errorNorm.  x_curr: the
// current (accepted) solution; corr, q_corr: the Newton corrections (x -
// predictor) of the solution and of Q; q: Q; reltol, abstol per unknown.
// Returns the estimate; errwt / qerrwt receive the weights.
XREF_API double xref_tia_error_estimate(int n, double ck, int new_lte, double *x_curr, double *corr,
                                        double *q, double *q_corr, double *reltol, double *abstol,
                                        double *errwt, double *qerrwt) {
  Integrator I;
  N_TIA_TIAParams &tp = *I.params.get();
  N_TIA_StepErrorControl &sec = *I.sec.get();
  N_TIA_DataStore &ds = *I.ds.get();
  tp.newLte = new_lte != 0;
  tp.fastTests = false;
  sec.ck_ = ck;
  ds.tiaParamsPtr_ = &tp;
  Vec vc, vcorr, vq, vqc, vr, va, vw, vqw;
  ds.currSolutionPtr = vc.bind(x_curr, n);
  ds.newtonCorrectionPtr = vcorr.bind(corr, n);
  ds.daeQVectorPtr = vq.bind(q, n);
  ds.qNewtonCorrectionPtr = vqc.bind(q_corr, n);
  ds.relErrTolPtr = vr.bind(reltol, n);
  ds.absErrTolPtr = va.bind(abstol, n);
  ds.errWtVecPtr = vw.bind(errwt, n);
  ds.qErrWtVecPtr = vqw.bind(qerrwt, n);
  new (&ds.indexVVars) std::vector<int>();
  new (&ds.indexIVars) std::vector<int>();
  new (&ds.indexMaskedVars) std::vector<int>();
  new (&ds.innerErrorInfoVec) decltype(ds.innerErrorInfoVec)();
  ds.indexVVars.resize(size_t(n));
  for (int k = 0; k < n; ++k) ds.indexVVars[k] = k;
  ds.numVVars = n;
  ds.numIVars = 0;
  ds.numMaskedVars = 0;
  ds.solutionSize = n;
  ds.indexVecsInitialized = true;
  ds.N_TIA_DataStore::setErrorWtVector();
  // computeErrorEstimate is sec.ck_ * ds.WRMS_errorNorm() (N_TIA_OneStep.h:97),
  // a virtual call on the data store, whose vtable comes with a constructor
  // this harness cannot run: the same product, with the norm called directly
  const double est = sec.ck_ * ds.N_TIA_DataStore::WRMS_errorNorm();
  typedef std::vector<int> VI;
  ds.indexVVars.~VI();
  ds.indexIVars.~VI();
  ds.indexMaskedVars.~VI();
  typedef decltype(ds.innerErrorInfoVec) VE;
  ds.innerErrorInfoVec.~VE();
  return est;
}

namespace {
// The loader the convergence test asks whether devices converged: Xyce's
// default answers (N_LOA_Loader.h:273-276, both true) for the circuit case.
struct ConvergedLoader : N_LOA_Loader {
  bool setParam(std::string &, double) { return false; }
  double getParamAndReduce(const std::string &) { return 0.0; }
  bool getParamAndReduce(const std::string &, double &) { return false; }
  bool initializeProblem(N_LAS_Vector *, N_LAS_Vector *, N_LAS_Vector *, N_LAS_Vector *,
                         N_LAS_Vector *, N_LAS_Vector *, N_LAS_Vector *, N_LAS_Vector *,
                         N_LAS_Vector *, N_LAS_Vector *, N_LAS_Vector *, N_LAS_Vector *,
                         N_LAS_Vector *, N_LAS_Vector *) {
    return false;
  }
};
}  // namespace

// DampedNewton::converged_ on the solver's state after a Newton step.
// transient: 1 for a transient step's solve (AnalysisMode TRANSIENT), else
// DC.  count / tmp_rate carry the stall counter between calls (in and out).
XREF_API int xref_nls_converged(int transient, int step, int max_step, double rhs_tol,
                                double dx_tol, double small_update_tol, double max_norm_rhs,
                                double wt_norm_dx, double step_length, double norm_rhs_rel,
                                double conv_rate, int *count, double *tmp_rate) {
  Raw<N_NLS_DampedNewton> dn;
  Raw<N_NLS_ParamMgr> pm;
  N_NLS_DampedNewton &s = *dn.get();
  new (&s.nlParams) N_NLS_NLParams(transient ? TRANSIENT : DC_OP, *static_cast<N_IO_CmdParse *>(0));
  s.nlParams.setMaxNewtonStep(max_step);
  s.nlParams.setRHSTol(rhs_tol);
  s.nlParams.setDeltaXTol(dx_tol);
  s.nlParams.setSmallUpdateTol(small_update_tol);
  s.nlParams.setEnforceDeviceConvFlag(false);
  pm.get()->currentMode_ = transient ? TRANSIENT : DC_OP;
  s.nlpMgrPtr_ = pm.get();
  ConvergedLoader loader;
  s.loaderPtr_ = &loader;
  new (&s.retCodes_) N_NLS_ReturnCodes();
  s.nlStep_ = unsigned(step);
  s.maxNormRHS_ = max_norm_rhs;
  s.wtNormDX_ = wt_norm_dx;
  s.stepLength_ = step_length;
  s.normRHS_rel_ = norm_rhs_rel;
  s.resConvRate_ = conv_rate;
  s.count = *count;
  s.tmpConvRate = *tmp_rate;
  const int r = s.N_NLS_DampedNewton::converged_();
  *count = s.count;
  *tmp_rate = s.tmpConvRate;
  return r;
}

namespace {
// History vectors of one integrator, bound to caller arrays: hist[0..2] the
// solution history, hist[3..5] the charge history; the state and store
// histories the reference also rotates are bound to scratch.
struct History {
  Vec x[3], q[3], sto[3], stoqc[3], s0, scratch[4];
  std::vector<double> tmp;
  void bind(N_TIA_DataStore &ds, int n, double *const *hist) {
    tmp.assign(12 * (size_t(n) + 1), 0.0);
    double *t = tmp.data();
    ds.xHistory = {x[0].bind(hist[0], n), x[1].bind(hist[1], n), x[2].bind(hist[2], n)};
    ds.qHistory = {q[0].bind(hist[3], n), q[1].bind(hist[4], n), q[2].bind(hist[5], n)};
    for (int k = 0; k < 3; ++k) {
      sto[k].bind(t + (2 * k) * (n + 1), n);
      stoqc[k].bind(t + (2 * k + 1) * (n + 1), n);
    }
    ds.stoHistory = {sto[0].obj.get(), sto[1].obj.get(), sto[2].obj.get()};
    ds.stoLeadCurrQCompHistory = {stoqc[0].obj.get(), stoqc[1].obj.get(), stoqc[2].obj.get()};
    ds.sHistory = {s0.bind(t + 6 * (n + 1), n)};
    for (int k = 0; k < 4; ++k) scratch[k].bind(t + (7 + k) * (n + 1), n);
    ds.nextStorePtr = scratch[0].obj.get();
    ds.nextStoreLeadCurrQCompPtr = scratch[1].obj.get();
    ds.nextStatePtr = scratch[2].obj.get();
  }
};

void step_control_setup(Integrator &I, const double *in) {
  N_TIA_TIAParams &tp = *I.params.get();
  N_TIA_StepErrorControl &sec = *I.sec.get();
  tp.errorAnalysisOption = 0;
  tp.constantStepSize = false;
  sec.tolAimFac_ = 0.5;
  sec.r_factor_ = 1.0;  // the build without Xyce_USE_Q_NORM (N_TIA_StepErrorControl.C:164-168)
  sec.r_safety_ = 2.0;
  sec.r_fudge_ = 0.0001;
  sec.r_min_ = 0.25;
  sec.r_max_ = 0.9;
  sec.r_hincr_test_ = 2.0;
  sec.r_hincr_ = 2.0;
  sec.max_LET_fail_ = 15;
  sec.newOrder_ = 1;
  sec.currentOrder_ = int(in[0]);
  sec.usedOrder_ = int(in[0]);
  sec.numberOfSteps_ = int(in[1]);
  sec.nef_ = int(in[2]);
  sec.estOverTol_ = in[3];
  sec.currentTimeStep = in[4];
  sec.currentTime = in[5];
  sec.nextTime = in[6];
  sec.stopTime = in[7];
  sec.minTimeStep = in[8];
  sec.maxTimeStep = in[9];
  sec.lastTimeStep = in[10];
  sec.currentTimeStepSum = in[11];
  for (int k = 0; k < 3; ++k) sec.psi_[k] = in[12 + k];
  sec.newtonConvergenceStatus = int(in[15]);
  sec.savedTimeStep = in[16];
}

void step_control_result(Integrator &I, double *out) {
  const N_TIA_StepErrorControl &sec = *I.sec.get();
  out[0] = sec.currentOrder_;
  out[1] = sec.numberOfSteps_;
  out[2] = sec.nef_;
  out[3] = sec.currentTimeStep;
  out[4] = sec.currentTime;
  out[5] = sec.nextTime;
  out[6] = sec.lastTimeStep;
  out[7] = sec.currentTimeStepSum;
  out[8] = sec.savedTimeStep;
  for (int k = 0; k < 3; ++k) out[9 + k] = sec.psi_[k];
}
}  // namespace

// OneStep::completeStep (N_TIA_OneStep.C:1945-2190) after an accepted step:
// the next order and step, the time advanced and the solution and charge
// histories rotated (updateHistory, :1209-1300).  in[17]: order,
// steps taken, error-test failures, estOverTol, h, t, t_next, stop time,
// min step, max step, last step, h_sum, psi[3], Newton status, saved step.
// hist[6]: x history 0..2 then Q history 0..2 (n each, updated in place);
// x_next, Q, F: the accepted point.  out[12]: order, steps, failures, h,
// t, t_next, last step, h_sum, saved step, psi[3].
XREF_API void xref_tia_complete_step(int n, const double *in, double *const *hist, double *x_next,
                                     double *Q, double *F, double *out) {
  Integrator I;
  N_TIA_DataStore &ds = *I.ds.get();
  step_control_setup(I, in);
  History H;
  H.bind(ds, n, hist);
  Vec vx, vq, vf;
  ds.nextSolutionPtr = vx.bind(x_next, n);
  ds.daeQVectorPtr = vq.bind(Q, n);
  ds.daeFVectorPtr = vf.bind(F, n);
  I.method->N_TIA_OneStep::completeStep();
  step_control_result(I, out);
}

// OneStep::rejectStep (N_TIA_OneStep.C:1695-1930) after a failed step (a
// Newton failure when the Newton status is <= 0, else the local error
// test): the retry's order and step.  in / out as xref_tia_complete_step.
XREF_API void xref_tia_reject_step(const double *in, double *out) {
  Integrator I;
  step_control_setup(I, in);
  I.sec.get()->stepAttemptStatus = false;
  I.method->N_TIA_OneStep::rejectStep();
  step_control_result(I, out);
}
