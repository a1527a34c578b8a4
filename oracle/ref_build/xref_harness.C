// xref_harness.C — drives the reference Xyce device code (compiled from the
// reference's own sources, untouched) through exactly the calls DeviceMgr makes
// for one Newton load, on a circuit given in the xg_netlist format of
// include/xg.h.  Test infrastructure only: the product never links this.
//
// What it replaces from the reference (which cannot be built here: it needs
// Trilinos/Epetra):
//   * DeviceMgr::addDeviceModel / addDeviceInstance   N_DEV_DeviceMgr.C:923-1200
//   * Topology LID + Jacobian-offset registration      N_TOP_CktGraphBasic.C:1092-1142
//   * DeviceMgr::updateState / loadDAEVectors / loadDAEMatrices, the order of
//     calls and the raw-pointer publication in ExternData
//                                                      N_DEV_DeviceMgr.C:2201-2661
//   * a CSR-backed N_LAS_Matrix::operator[] and N_LAS_Vector::operator[]
//     (N_LAS_Matrix.C:863-879) in place of Epetra.
//
// Ground is the trailing index of every solution vector and the trailing
// row/column of the matrices (SOLUTION_OVERLAP_GND, N_LAS_Builder.C:334-341).

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <vector>

// Derived per-instance parameters are read straight out of the reference's
// Instance objects to pin the engine's own setup code.
#define private public
#define protected public
#include <Xyce_config.h>
#include <N_DEV_Capacitor.h>
#include <N_DEV_Const.h>
#include <N_DEV_Configuration.h>
#include <N_DEV_DeviceBlock.h>
#include <N_DEV_DeviceMaster.h>
#include <N_DEV_DeviceOptions.h>
#include <N_DEV_Diode.h>
#include <N_DEV_ISRC.h>
#include <N_DEV_ExternData.h>
#include <N_DEV_MOSFET1.h>
#include <N_DEV_MOSFET_B3.h>
#include <N_DEV_MatrixLoadData.h>
#include <N_DEV_Param.h>
#include <N_DEV_Resistor.h>
#include <N_DEV_SolverState.h>
#include <N_DEV_SourceData.h>
#include <N_DEV_Vsrc.h>
#include <N_LAS_Matrix.h>
#include <N_LAS_Vector.h>
#undef private
#undef protected

#include "xg.h"
#include "xg_params.h"

using namespace Xyce::Device;

// ---------------------------------------------------------------------------
// Epetra stand-ins: the devices only ever index rows/elements.
// ---------------------------------------------------------------------------
namespace {
struct Csr {
  int nrows = 0;                  // includes the ground row
  std::vector<int> rowptr, col;   // ascending columns per row
  std::vector<double> val;
};
std::map<const void *, double *> g_vec;
std::map<const void *, Csr *> g_mat;
}  // namespace

double &N_LAS_Vector::operator[](int index) { return g_vec.at(this)[index]; }
const double &N_LAS_Vector::operator[](int index) const { return g_vec.at(this)[index]; }
double *N_LAS_Matrix::operator[](int row) {
  Csr *m = g_mat.at(this);
  return &m->val[m->rowptr[row]];
}
double *const N_LAS_Matrix::operator[](int row) const {
  Csr *m = g_mat.at(this);
  return &m->val[m->rowptr[row]];
}

// Members named by reference code that is linked but never reached on the
// load path (numerical-Jacobian dumps, command-line option parsing).
int N_LAS_Matrix::getLocalNumRows() const { std::abort(); }
void N_LAS_Matrix::replaceLocalRow(int, int, double *, int *) { std::abort(); }
bool N_LAS_Matrix::putLocalRow(int, int, const double *, const int *) { std::abort(); }
#include <N_IO_CmdParse.h>
bool Xyce::IO::CmdParse::argExists(const std::string &) const { return false; }
std::string Xyce::IO::CmdParse::getArgumentValue(const std::string &) const { return ""; }

namespace {

template <class T>
struct RawObj {  // storage for an object whose constructor needs Epetra
  alignas(T) unsigned char buf[sizeof(T)];
  T *get() { return reinterpret_cast<T *>(buf); }
};

struct VecSlot {
  RawObj<N_LAS_Vector> obj;
  std::vector<double> data;
  void bind(size_t n) {
    data.assign(n, 0.0);
    g_vec[obj.get()] = data.data();
  }
};

struct DevEntry {
  int type;
  Device *device = nullptr;
  std::vector<DeviceInstance *> inst;
};

bool g_registered = false;
void register_once() {
  if (g_registered) return;
  Resistor::registerDevice();
  Capacitor::registerDevice();
  Vsrc::registerDevice();
  ISRC::registerDevice();
  Diode::registerDevice();
  MOSFET1::registerDevice();
  MOSFET_B3::registerDevice();
  g_registered = true;
}

const char *letter_of(int type) {
  switch (type) {
    case XG_DEV_RES: return "R";
    case XG_DEV_CAP: return "C";
    case XG_DEV_VSRC: return "V";
    case XG_DEV_ISRC: return "I";
    case XG_DEV_DIODE: return "D";
    default: return "M";
  }
}

}  // namespace

struct XRef {
  DeviceOptions opts;
  SolverState ss;
  MatrixLoadData mld;
  ExternData ext;
  // The devices never touch the command line; FactoryBlock only stores a reference.
  alignas(16) unsigned char cmd[256];
  std::unique_ptr<FactoryBlock> fb;
  std::vector<DevEntry> devs;   // in load order
  int n_nodes = 0, n_unknowns = 0, n_state = 0, n_store = 0;
  Csr dfdx, dqdx;
  RawObj<N_LAS_Matrix> dfdx_obj, dqdx_obj;
  VecSlot sol[3], sta[3], sto[3], f, q, dfdxdvp, dqdxdvp, stadot, lead_f, lead_q, flag;
  std::string err;
};

static int node_lid(const XRef &x, int node) { return node < 0 ? x.n_unknowns : node; }

static Device *make_device(XRef &x, int type, const std::string &model_type_name, int level) {
  ModelTypeId mt;
  if (type == XG_DEV_MOS1 || type == XG_DEV_BSIM3 || type == XG_DEV_DIODE)
    mt = Configuration::getModelType(model_type_name, level);
  else
    mt = Configuration::getModelGroup(letter_of(type));
  return Configuration::createDevice(mt, *x.fb);
}

extern "C" {

// Builds the circuit: models, instances, LIDs, Jacobian pattern and offsets.
int xref_build(const xg_netlist *nl, const xg_device_options *opt, XRef **out) {
  register_once();
  XRef *x = new XRef();
  if (opt) {
    x->opts.gmin = opt->gmin;
    x->opts.voltageLimiterFlag = opt->voltlim != 0;
    x->opts.newMeyerFlag = opt->newmeyer != 0;
    x->opts.tnom = opt->tnom;
    x->opts.temp = Xyce::Util::Param("TEMP", opt->temp);
  }
  x->fb.reset(new FactoryBlock(x->opts, x->ss, x->mld, x->ext, *reinterpret_cast<Xyce::IO::CmdParse *>(x->cmd)));
  x->n_nodes = nl->n_nodes;

  std::vector<int> order;
  if (nl->type_order && nl->n_type_order > 0)
    order.assign(nl->type_order, nl->type_order + nl->n_type_order);
  else
    for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) order.push_back(t);

  // One Device (Master) per type, created in load order.
  std::map<int, DevEntry *> by_type;
  x->devs.reserve(order.size());
  for (int t : order) {
    int count = 0;
    switch (t) {
      case XG_DEV_RES: count = nl->res.n; break;
      case XG_DEV_CAP: count = nl->cap.n; break;
      case XG_DEV_VSRC: count = nl->vsrc.n; break;
      case XG_DEV_ISRC: count = nl->isrc.n; break;
      case XG_DEV_DIODE: count = nl->diode.n; break;
      case XG_DEV_MOS1: count = nl->mos1.n; break;
      case XG_DEV_BSIM3: count = nl->bsim3.n; break;
      default: count = 0;
    }
    if (count == 0) continue;
    DevEntry e;
    e.type = t;
    x->devs.push_back(e);
    by_type[t] = &x->devs.back();
  }

  // Models.
  std::vector<std::string> model_names(nl->n_models);
  for (int mi = 0; mi < nl->n_models; ++mi) {
    const xg_model_desc &md = nl->models[mi];
    char nm[32];
    snprintf(nm, sizeof nm, "MOD%d", mi);
    model_names[mi] = nm;
    std::string tname;
    int level = 1;
    if (md.type == XG_DEV_DIODE) { tname = "D"; level = 1; }
    else if (md.type == XG_DEV_MOS1) { tname = md.polarity < 0 ? "PMOS" : "NMOS"; level = 1; }
    else if (md.type == XG_DEV_BSIM3) { tname = md.polarity < 0 ? "PMOS" : "NMOS"; level = 9; }
    else continue;
    auto it = by_type.find(md.type);
    if (it == by_type.end()) continue;  // model without instances
    DevEntry &e = *it->second;
    if (!e.device) e.device = make_device(*x, md.type, tname, level);
    ModelBlock mb(nm, tname, level);
    for (int p = 0; p < md.n_params; ++p)
      mb.params.push_back(Param(std::string(md.names[p]), md.values[p], true));
    e.device->addModel(mb, *x->fb);
  }
  for (auto &e : x->devs)
    if (!e.device) e.device = make_device(*x, e.type, "", 1);

  // Instances.
  auto add = [&](DevEntry &e, const std::string &name, const std::string &model,
                 std::vector<Param> params, int next) {
    InstanceBlock ib(name);
    ib.setModelName(model);
    ib.params = params;
    ib.iNumNodes = next;
    ib.numExtVars = next;
    ib.numIntVars = 0;
    ib.modelFlag = !model.empty();
    DeviceInstance *di = e.device->addInstance(ib, *x->fb);
    e.inst.push_back(di);
  };
  std::vector<std::vector<std::vector<int>>> ext_nodes(x->devs.size());
  for (size_t k = 0; k < x->devs.size(); ++k) {
    DevEntry &e = x->devs[k];
    auto &en = ext_nodes[k];
    char nm[48];
    switch (e.type) {
      case XG_DEV_RES:
        for (int i = 0; i < nl->res.n; ++i) {
          snprintf(nm, sizeof nm, "R%d", i);
          add(e, nm, "", {Param("R", nl->res.value[i], true)}, 2);
          en.push_back({nl->res.p[i], nl->res.m[i]});
        }
        break;
      case XG_DEV_CAP:
        for (int i = 0; i < nl->cap.n; ++i) {
          snprintf(nm, sizeof nm, "C%d", i);
          add(e, nm, "", {Param("C", nl->cap.value[i], true)}, 2);
          en.push_back({nl->cap.p[i], nl->cap.m[i]});
        }
        break;
      case XG_DEV_VSRC:
      case XG_DEV_ISRC: {
        const xg_src_desc &sd = e.type == XG_DEV_VSRC ? nl->vsrc : nl->isrc;
        for (int i = 0; i < sd.n; ++i) {
          snprintf(nm, sizeof nm, "%s%d", e.type == XG_DEV_VSRC ? "V" : "I", i);
          const double *w = sd.wave + 7 * i;
          std::vector<Param> ps;
          if (sd.kind[i] == XG_SRC_PULSE) {
            ps.push_back(Param("DCV0", w[0], true));
            ps.push_back(Param("DCSOURCETYPE", (int)_DC_DATA, true));
            ps.push_back(Param("TRANSIENTSOURCETYPE", (int)_PULSE_DATA, true));
            const char *tags[7] = {"V1", "V2", "TD", "TR", "TF", "PW", "PER"};
            for (int j = 0; j < 7; ++j) ps.push_back(Param(tags[j], w[j], true));
          } else {
            ps.push_back(Param("DCV0", w[0], true));
            ps.push_back(Param("DCSOURCETYPE", (int)_DC_DATA, true));
          }
          add(e, nm, "", ps, 2);
          en.push_back({sd.p[i], sd.m[i]});
        }
        break;
      }
      case XG_DEV_DIODE:
        for (int i = 0; i < nl->diode.n; ++i) {
          snprintf(nm, sizeof nm, "D%d", i);
          std::vector<Param> ps;
          if (nl->diode.area) ps.push_back(Param("AREA", nl->diode.area[i], true));
          add(e, nm, model_names[nl->diode.model[i]], ps, 2);
          en.push_back({nl->diode.a[i], nl->diode.c[i]});
        }
        break;
      case XG_DEV_MOS1:
      case XG_DEV_BSIM3: {
        const xg_mos_desc &md = e.type == XG_DEV_MOS1 ? nl->mos1 : nl->bsim3;
        for (int i = 0; i < md.n; ++i) {
          snprintf(nm, sizeof nm, "M%d", i);
          std::vector<Param> ps;
          ps.push_back(Param("W", md.w[i], true));
          ps.push_back(Param("L", md.l[i], true));
          if (md.ad) ps.push_back(Param("AD", md.ad[i], true));
          if (md.as) ps.push_back(Param("AS", md.as[i], true));
          if (md.pd) ps.push_back(Param("PD", md.pd[i], true));
          if (md.ps) ps.push_back(Param("PS", md.ps[i], true));
          if (md.nrd) ps.push_back(Param("NRD", md.nrd[i], true));
          if (md.nrs) ps.push_back(Param("NRS", md.nrs[i], true));
          if (md.m) ps.push_back(Param("M", md.m[i], true));
          add(e, nm, model_names[md.model[i]], ps, 4);
          en.push_back({md.d[i], md.g[i], md.s[i], md.b[i]});
        }
        break;
      }
    }
  }

  // LIDs: circuit nodes, then internal unknowns by type order / instance.
  int next_lid = nl->n_nodes;
  std::vector<std::vector<int>> ext_lids_all, int_lids_all;
  for (size_t k = 0; k < x->devs.size(); ++k)
    for (size_t i = 0; i < x->devs[k].inst.size(); ++i) {
      DeviceInstance *di = x->devs[k].inst[i];
      std::vector<int> il(di->getNumIntVars());
      for (auto &v : il) v = next_lid++;
      int_lids_all.push_back(il);
    }
  x->n_unknowns = next_lid;
  {
    size_t flat = 0;
    for (size_t k = 0; k < x->devs.size(); ++k)
      for (size_t i = 0; i < x->devs[k].inst.size(); ++i, ++flat) {
        std::vector<int> el;
        for (int nd : ext_nodes[k][i]) el.push_back(node_lid(*x, nd));
        x->devs[k].inst[i]->registerLIDs(int_lids_all[flat], el);
        ext_lids_all.push_back(el);
      }
  }
  // State / store LIDs.
  int sta = 0, sto = 0;
  for (auto &e : x->devs)
    for (DeviceInstance *di : e.inst) {
      std::vector<int> sl(di->getNumStateVars()), tl(di->getNumStoreVars());
      for (auto &v : sl) v = sta++;
      for (auto &v : tl) v = sto++;
      di->registerStateLIDs(sl);
      di->registerStoreLIDs(tl);
    }
  x->n_state = sta;
  x->n_store = sto;

  // Jacobian pattern from every instance's stamp (ground included).
  const int nr = x->n_unknowns + 1;
  std::vector<std::set<int>> rows(nr);
  std::vector<std::vector<int>> lids_all;
  {
    size_t flat = 0;
    for (auto &e : x->devs)
      for (DeviceInstance *di : e.inst) {
        std::vector<int> lids = ext_lids_all[flat];
        lids.insert(lids.end(), int_lids_all[flat].begin(), int_lids_all[flat].end());
        lids_all.push_back(lids);
        ++flat;
        const auto &st = di->jacobianStamp();
        for (size_t r = 0; r < st.size(); ++r)
          for (int c : st[r]) rows[lids[r]].insert(lids[c]);
      }
  }
  for (Csr *m : {&x->dfdx, &x->dqdx}) {
    m->nrows = nr;
    m->rowptr.assign(nr + 1, 0);
    for (int r = 0; r < nr; ++r) m->rowptr[r + 1] = m->rowptr[r] + (int)rows[r].size();
    m->col.clear();
    for (int r = 0; r < nr; ++r) m->col.insert(m->col.end(), rows[r].begin(), rows[r].end());
    m->val.assign(m->col.size(), 0.0);
  }
  g_mat[x->dfdx_obj.get()] = &x->dfdx;
  g_mat[x->dqdx_obj.get()] = &x->dqdx;
  {
    size_t flat = 0;
    for (auto &e : x->devs)
      for (DeviceInstance *di : e.inst) {
        const std::vector<int> &lids = lids_all[flat++];
        const auto &st = di->jacobianStamp();
        std::vector<std::vector<int>> off(st.size());
        for (size_t r = 0; r < st.size(); ++r) {
          int gr = lids[r];
          for (int c : st[r]) {
            int gc = lids[c];
            auto b = x->dfdx.col.begin() + x->dfdx.rowptr[gr];
            auto en = x->dfdx.col.begin() + x->dfdx.rowptr[gr + 1];
            off[r].push_back((int)(std::lower_bound(b, en, gc) - b));
          }
        }
        di->registerJacLIDs(off);
      }
  }

  // Vectors.
  for (int i = 0; i < 3; ++i) {
    x->sol[i].bind(nr);
    x->sta[i].bind(std::max(1, x->n_state));
    x->sto[i].bind(std::max(1, x->n_store));
  }
  for (VecSlot *v : {&x->f, &x->q, &x->dfdxdvp, &x->dqdxdvp, &x->flag}) v->bind(nr);
  x->stadot.bind(std::max(1, x->n_state));
  x->lead_f.bind(std::max(1, x->n_store));
  x->lead_q.bind(std::max(1, x->n_store));
  ExternData &ext = x->ext;
  ext.dFdxMatrixPtr = x->dfdx_obj.get();
  ext.dQdxMatrixPtr = x->dqdx_obj.get();
  ext.nextSolVectorPtr = x->sol[0].obj.get();
  ext.currSolVectorPtr = x->sol[1].obj.get();
  ext.lastSolVectorPtr = x->sol[2].obj.get();
  ext.nextStaVectorPtr = x->sta[0].obj.get();
  ext.currStaVectorPtr = x->sta[1].obj.get();
  ext.lastStaVectorPtr = x->sta[2].obj.get();
  ext.nextStoVectorPtr = x->sto[0].obj.get();
  ext.currStoVectorPtr = x->sto[1].obj.get();
  ext.lastStoVectorPtr = x->sto[2].obj.get();
  ext.daeFVectorPtr = x->f.obj.get();
  ext.daeQVectorPtr = x->q.obj.get();
  ext.dFdxdVpVectorPtr = x->dfdxdvp.obj.get();
  ext.dQdxdVpVectorPtr = x->dqdxdvp.obj.get();
  ext.nextStaDerivVectorPtr = x->stadot.obj.get();
  ext.flagSolVectorPtr = x->flag.obj.get();
  ext.nextSolVectorRawPtr = x->sol[0].data.data();
  ext.currSolVectorRawPtr = x->sol[1].data.data();
  ext.lastSolVectorRawPtr = x->sol[2].data.data();
  ext.nextStaVectorRawPtr = x->sta[0].data.data();
  ext.currStaVectorRawPtr = x->sta[1].data.data();
  ext.lastStaVectorRawPtr = x->sta[2].data.data();
  ext.nextStoVectorRawPtr = x->sto[0].data.data();
  ext.currStoVectorRawPtr = x->sto[1].data.data();
  ext.lastStoVectorRawPtr = x->sto[2].data.data();
  ext.daeFVectorRawPtr = x->f.data.data();
  ext.daeQVectorRawPtr = x->q.data.data();
  ext.dFdxdVpVectorRawPtr = x->dfdxdvp.data.data();
  ext.dQdxdVpVectorRawPtr = x->dqdxdvp.data.data();
  ext.nextStaDerivVectorRawPtr = x->stadot.data.data();
  ext.storeLeadCurrQCompRawPtr = x->lead_q.data.data();

  // First loadDAEMatrices call publishes the matrix pointers
  // (DeviceMgr::setupRawMatrixPointers_, N_DEV_DeviceMgr.C:3732-3744).
  for (auto &e : x->devs)
    for (DeviceInstance *di : e.inst) di->setupPointers();
  *out = x;
  return 0;
}

int xref_free(XRef *x) {
  if (!x) return 0;
  g_mat.erase(x->dfdx_obj.get());
  g_mat.erase(x->dqdx_obj.get());
  for (auto *v : {&x->sol[0], &x->sol[1], &x->sol[2], &x->sta[0], &x->sta[1], &x->sta[2],
                  &x->sto[0], &x->sto[1], &x->sto[2], &x->f, &x->q, &x->dfdxdvp, &x->dqdxdvp,
                  &x->stadot, &x->lead_f, &x->lead_q, &x->flag})
    g_vec.erase(v->obj.get());
  // Device objects are leaked deliberately: their destructors reach into
  // global registries this harness never fully populates.
  delete x;
  return 0;
}

int xref_sizes(const XRef *x, int *n_unknowns, int *n_state, int *n_store, int64_t *nnz_gnd) {
  *n_unknowns = x->n_unknowns;
  *n_state = x->n_state;
  *n_store = x->n_store;
  *nnz_gnd = (int64_t)x->dfdx.col.size();
  return 0;
}

// Pattern including the ground row/column (row n_unknowns, col n_unknowns).
int xref_pattern(const XRef *x, int *rowptr, int *col) {
  std::copy(x->dfdx.rowptr.begin(), x->dfdx.rowptr.end(), rowptr);
  std::copy(x->dfdx.col.begin(), x->dfdx.col.end(), col);
  return 0;
}

// Derived per-instance parameters read from the reference's Instance objects,
// in the column layout of include/xg_params.h (column k of instance i at
// out[k*n + i]).  Values the reference recomputes at every load from setup
// constants (DrainSatCur, SourceSatCur, Beta: N_DEV_MOSFET1.C:2650-2665;
// Isat, Vt, Gspr: N_DEV_Diode.C:911-915) are formed here by those same
// expressions.  Returns the number of instances (0 if the type is absent).
int xref_params(XRef *x, int type, double *out, int *n_params) {
  for (auto &e : x->devs) {
    if (e.type != type) continue;
    const int n = (int)e.inst.size();
    for (int i = 0; i < n; ++i) {
      double v[256] = {0};
      int np = 0;
      if (type == XG_DEV_MOS1) {
        MOSFET1::Instance &m = *static_cast<MOSFET1::Instance *>(e.inst[i]);
        const MOSFET1::Model &mo = m.model_;
        np = XG_M1_NPARAMS;
        v[XG_M1_DTYPE] = mo.dtype;
        v[XG_M1_GAMMA] = mo.gamma;
        v[XG_M1_LAMBDA] = mo.lambda;
        v[XG_M1_MJ] = mo.bulkJctBotGradingCoeff;
        v[XG_M1_MJSW] = mo.bulkJctSideGradingCoeff;
        if ((m.tSatCurDens == 0) || (m.drainArea == 0) || (m.sourceArea == 0)) {
          v[XG_M1_DRAINSATCUR] = m.tSatCur;
          v[XG_M1_SOURCESATCUR] = m.tSatCur;
        } else {
          v[XG_M1_DRAINSATCUR] = m.tSatCurDens * m.drainArea;
          v[XG_M1_SOURCESATCUR] = m.tSatCurDens * m.sourceArea;
        }
        v[XG_M1_BETA] = m.tTransconductance * m.w / m.EffectiveLength;
        v[XG_M1_TVTO] = m.tVto;
        v[XG_M1_SOURCEVCRIT] = m.sourceVcrit;
        v[XG_M1_DRAINVCRIT] = m.drainVcrit;
        v[XG_M1_VT] = m.vt;
        v[XG_M1_TPHI] = m.tPhi;
        v[XG_M1_TVBI] = m.tVbi;
        v[XG_M1_CBS] = m.Cbs;
        v[XG_M1_CBSSW] = m.Cbssw;
        v[XG_M1_CBD] = m.Cbd;
        v[XG_M1_CBDSW] = m.Cbdsw;
        v[XG_M1_TDEPCAP] = m.tDepCap;
        v[XG_M1_TBULKPOT] = m.tBulkPot;
        v[XG_M1_F2S] = m.f2s;
        v[XG_M1_F3S] = m.f3s;
        v[XG_M1_F4S] = m.f4s;
        v[XG_M1_F2D] = m.f2d;
        v[XG_M1_F3D] = m.f3d;
        v[XG_M1_F4D] = m.f4d;
        v[XG_M1_OXIDECAP] = m.OxideCap;
        v[XG_M1_CGSO] = m.GateSourceOverlapCap;
        v[XG_M1_CGDO] = m.GateDrainOverlapCap;
        v[XG_M1_CGBO] = m.GateBulkOverlapCap;
        v[XG_M1_GD] = m.drainConductance;
        v[XG_M1_GS] = m.sourceConductance;
        v[XG_M1_M] = m.numberParallel;
        v[XG_M1_ICVDS] = m.icVDS;
        v[XG_M1_ICVGS] = m.icVGS;
        v[XG_M1_ICVBS] = m.icVBS;
        v[XG_M1_FLAGS] = (m.OFF ? 1 : 0) | (m.IC_GIVEN ? 2 : 0);
      } else if (type == XG_DEV_DIODE) {
        Diode::Instance &d = *static_cast<Diode::Instance *>(e.inst[i]);
        const Diode::Model &mo = d.model_;
        np = XG_D_NPARAMS;
        v[XG_D_M] = mo.M;
        v[XG_D_BV] = mo.BV;
        v[XG_D_N] = mo.N;
        v[XG_D_TT] = mo.TT;
        v[XG_D_F2] = mo.F2;
        v[XG_D_F3] = mo.F3;
        v[XG_D_ISAT] = d.tSatCur * d.Area;
        v[XG_D_VT] = CONSTKoverQ * d.Temp;
        v[XG_D_GSPR] = d.tCOND * d.Area;
        v[XG_D_TVCRIT] = d.tVcrit;
        v[XG_D_TIRF] = d.tIRF;
        v[XG_D_TBRKDWNV] = d.tBrkdwnV;
        v[XG_D_TJCTCAP] = d.tJctCap;
        v[XG_D_TJCTPOT] = d.tJctPot;
        v[XG_D_TDEPCAP] = d.tDepCap;
        v[XG_D_TF1] = d.tF1;
        v[XG_D_AREA] = d.Area;
        v[XG_D_INITCOND] = d.InitCond;
        v[XG_D_FLAGS] = (mo.BVGiven ? 1 : 0) | (d.InitCondGiven ? 2 : 0) | (d.off ? 4 : 0);
      } else if (type == XG_DEV_RES) {
        np = XG_R_NPARAMS;
        v[XG_R_G] = static_cast<Resistor::Instance *>(e.inst[i])->G;
      } else if (type == XG_DEV_CAP) {
        np = XG_C_NPARAMS;
        v[XG_C_C] = static_cast<Capacitor::Instance *>(e.inst[i])->C;
      } else if (type == XG_DEV_BSIM3) {
        // Raw columns only (0..XG_B3_NRAW-1); the hoisted constants after
        // them are checked through the load results.
        MOSFET_B3::Instance &b = *static_cast<MOSFET_B3::Instance *>(e.inst[i]);
        const MOSFET_B3::Model &mo = b.model_;
        const MOSFET_B3::SizeDependParam &p = *b.paramPtr;
        np = XG_B3_NRAW;
        v[XG_B3_DTYPE] = mo.dtype;
        v[XG_B3_MOBMOD] = mo.mobMod;
        v[XG_B3_CAPMOD] = mo.capMod;
        v[XG_B3_XPART] = mo.xpart;
        v[XG_B3_TOX] = mo.tox;
        v[XG_B3_COX] = mo.cox;
        v[XG_B3_FACTOR1] = mo.factor1;
        v[XG_B3_VCRIT] = mo.vcrit;
        v[XG_B3_NJ] = mo.jctEmissionCoeff;
        v[XG_B3_IJTH] = mo.ijth;
        v[XG_B3_MJ] = mo.bulkJctBotGradingCoeff;
        v[XG_B3_MJSW] = mo.bulkJctSideGradingCoeff;
        v[XG_B3_MJSWG] = mo.bulkJctGateSideGradingCoeff;
        v[XG_B3_TNOM] = mo.tnom;
        v[XG_B3_TEMP] = b.temp;
        v[XG_B3_VTM] = b.vtm;
        v[XG_B3_JSTEMP] = b.jctTempSatCurDensity;
        v[XG_B3_JSWTEMP] = b.jctSidewallTempSatCurDensity;
        v[XG_B3_CJTEMP] = b.unitAreaJctCapTemp;
        v[XG_B3_CJSWTEMP] = b.unitLengthSidewallJctCapTemp;
        v[XG_B3_CJSWGTEMP] = b.unitLengthGateSidewallJctCapTemp;
        v[XG_B3_PHIB] = b.PhiBTemp;
        v[XG_B3_PHIBSW] = b.PhiBSWTemp;
        v[XG_B3_PHIBSWG] = b.PhiBSWGTemp;
        v[XG_B3_VJSM] = b.vjsm;
        v[XG_B3_ISEVJSM] = b.IsEvjsm;
        v[XG_B3_VJDM] = b.vjdm;
        v[XG_B3_ISEVJDM] = b.IsEvjdm;
        v[XG_B3_AD] = b.drainArea;
        v[XG_B3_AS] = b.sourceArea;
        v[XG_B3_PD] = b.drainPerimeter;
        v[XG_B3_PS] = b.sourcePerimeter;
        v[XG_B3_GD] = b.drainConductance;
        v[XG_B3_GS] = b.sourceConductance;
        v[XG_B3_M] = b.numberParallel;
        v[XG_B3_FLAGS] = b.OFF ? 1 : 0;
        v[XG_B3_VTH0] = p.vth0;
        v[XG_B3_VBSC] = p.vbsc;
        v[XG_B3_PHI] = p.phi;
        v[XG_B3_PHIS3] = p.phis3;
        v[XG_B3_SQRTPHI] = p.sqrtPhi;
        v[XG_B3_XDEP0] = p.Xdep0;
        v[XG_B3_LEFF] = p.leff;
        v[XG_B3_WEFF] = p.weff;
        v[XG_B3_VBI] = p.vbi;
        v[XG_B3_DVT0] = p.dvt0;
        v[XG_B3_DVT1] = p.dvt1;
        v[XG_B3_DVT2] = p.dvt2;
        v[XG_B3_DVT0W] = p.dvt0w;
        v[XG_B3_DVT1W] = p.dvt1w;
        v[XG_B3_DVT2W] = p.dvt2w;
        v[XG_B3_NLX] = p.nlx;
        v[XG_B3_K1] = p.k1;
        v[XG_B3_K1OX] = p.k1ox;
        v[XG_B3_K2OX] = p.k2ox;
        v[XG_B3_K3] = p.k3;
        v[XG_B3_K3B] = p.k3b;
        v[XG_B3_KT1] = p.kt1;
        v[XG_B3_KT1L] = p.kt1l;
        v[XG_B3_KT2] = p.kt2;
        v[XG_B3_W0] = p.w0;
        v[XG_B3_ETA0] = p.eta0;
        v[XG_B3_ETAB] = p.etab;
        v[XG_B3_THETA0VB0] = p.theta0vb0;
        v[XG_B3_NFACTOR] = p.nfactor;
        v[XG_B3_CDSC] = p.cdsc;
        v[XG_B3_CDSCB] = p.cdscb;
        v[XG_B3_CDSCD] = p.cdscd;
        v[XG_B3_CIT] = p.cit;
        v[XG_B3_VFB] = p.vfb;
        v[XG_B3_NGATE] = p.ngate;
        v[XG_B3_VOFF] = p.voff;
        v[XG_B3_CDEP0] = p.cdep0;
        v[XG_B3_DWG] = p.dwg;
        v[XG_B3_DWB] = p.dwb;
        v[XG_B3_PRWG] = p.prwg;
        v[XG_B3_PRWB] = p.prwb;
        v[XG_B3_RDS0] = p.rds0;
        v[XG_B3_XJ] = p.xj;
        v[XG_B3_A0] = p.a0;
        v[XG_B3_B0] = p.b0;
        v[XG_B3_B1] = p.b1;
        v[XG_B3_AGS] = p.ags;
        v[XG_B3_KETA] = p.keta;
        v[XG_B3_UA] = p.ua;
        v[XG_B3_UB] = p.ub;
        v[XG_B3_UC] = p.uc;
        v[XG_B3_U0TEMP] = p.u0temp;
        v[XG_B3_VSATTEMP] = p.vsattemp;
        v[XG_B3_A1] = p.a1;
        v[XG_B3_A2] = p.a2;
        v[XG_B3_DELTA] = p.delta;
        v[XG_B3_PCLM] = p.pclm;
        v[XG_B3_LITL] = p.litl;
        v[XG_B3_THETAROUT] = p.thetaRout;
        v[XG_B3_PDIBLB] = p.pdiblb;
        v[XG_B3_PVAG] = p.pvag;
        v[XG_B3_PSCBE1] = p.pscbe1;
        v[XG_B3_PSCBE2] = p.pscbe2;
        v[XG_B3_ALPHA0] = p.alpha0;
        v[XG_B3_ALPHA1] = p.alpha1;
        v[XG_B3_BETA0] = p.beta0;
        v[XG_B3_VFBCV] = p.vfbcv;
        v[XG_B3_WEFFCV] = p.weffCV;
        v[XG_B3_LEFFCV] = p.leffCV;
        v[XG_B3_ABULKCVFACTOR] = p.abulkCVfactor;
        v[XG_B3_NOFF] = p.noff;
        v[XG_B3_VOFFCV] = p.voffcv;
        v[XG_B3_VFBZB] = p.vfbzb;
        v[XG_B3_ACDE] = p.acde;
        v[XG_B3_LDEB] = p.ldeb;
        v[XG_B3_MOIN] = p.moin;
        v[XG_B3_CGDO] = p.cgdo;
        v[XG_B3_CGSO] = p.cgso;
        v[XG_B3_CGBO] = p.cgbo;
        v[XG_B3_CKAPPA] = p.ckappa;
        v[XG_B3_CGDL] = p.cgdl;
        v[XG_B3_CGSL] = p.cgsl;
      } else if (type == XG_DEV_VSRC || type == XG_DEV_ISRC) {
        // PulseData / ConstData parameters (N_DEV_SourceData.C:1033-1045, 2065-2070)
        SourceData *tran, *dc;
        int tran_type;
        if (type == XG_DEV_VSRC) {
          Vsrc::Instance &s = *static_cast<Vsrc::Instance *>(e.inst[i]);
          tran = s.Data_ptr; dc = s.dcData_ptr; tran_type = s.TRANSIENTSOURCETYPE;
        } else {
          ISRC::Instance &s = *static_cast<ISRC::Instance *>(e.inst[i]);
          tran = s.Data_ptr; dc = s.dcData_ptr; tran_type = s.TRANSIENTSOURCETYPE;
        }
        np = XG_V_NPARAMS;
        double w[16] = {0};
        if (tran && tran_type == _PULSE_DATA) {
          v[XG_V_KIND] = XG_SRC_PULSE;
          tran->getParams(w);
          for (int k = 0; k < 7; ++k) v[XG_V_V1 + k] = w[k];
        } else {
          v[XG_V_KIND] = XG_SRC_DC;
          if (dc) dc->getParams(w);
          v[XG_V_V1] = w[0];
        }
      } else {
        return -1;
      }
      if (n_params) *n_params = np;
      if (out)
        for (int k = 0; k < np; ++k) out[(size_t)k * n + i] = v[k];
    }
    return n;
  }
  return 0;
}

// One Newton load.  Vectors in: sol next/curr/last (n_unknowns+1), sta
// next/curr/last (n_state), sto next/curr/last (n_store; next = previous
// Newton iterate).  Out: F, Q, dFdxdVp, dQdxdVp, sta_next, sto_next, dfdx and
// dqdx values on the ground-inclusive pattern.
int xref_load(XRef *x, const xg_load_flags *fl, const double *const *in_vecs, double *f,
              double *q, double *dfdxdvp, double *dqdxdvp, double *sta_next,
              double *sto_next, double *dfdx, double *dqdx) {
  SolverState &ss = x->ss;
  ss.dcopFlag = fl->dcop != 0;
  ss.tranopFlag = fl->tranop != 0;
  ss.acopFlag = fl->acop != 0;
  ss.transientFlag = fl->transient != 0;
  ss.initJctFlag = fl->init_jct != 0;
  ss.initFixFlag = fl->init_fix != 0;
  ss.newtonIter = fl->newton_iter;
  ss.inputOPFlag = fl->inputop != 0;
  ss.pdt = fl->pdt;
  ss.currTime = fl->time;
  ss.initTranFlag = fl->init_tran != 0;
  const int nr = x->n_unknowns + 1;
  for (int i = 0; i < 3; ++i) std::copy(in_vecs[i], in_vecs[i] + nr, x->sol[i].data.begin());
  for (int i = 0; i < 3; ++i)
    if (x->n_state) std::copy(in_vecs[3 + i], in_vecs[3 + i] + x->n_state, x->sta[i].data.begin());
  for (int i = 0; i < 3; ++i)
    if (x->n_store) std::copy(in_vecs[6 + i], in_vecs[6 + i] + x->n_store, x->sto[i].data.begin());
  x->sol[0].data[nr - 1] = 0.0;
  // The caller zeroes the outputs (N_TIA_Assembler.C:156-161).
  for (VecSlot *v : {&x->f, &x->q, &x->dfdxdvp, &x->dqdxdvp})
    std::fill(v->data.begin(), v->data.end(), 0.0);
  std::fill(x->dfdx.val.begin(), x->dfdx.val.end(), 0.0);
  std::fill(x->dqdx.val.begin(), x->dqdx.val.end(), 0.0);

  double *solp = x->sol[0].data.data();
  double *stap = x->sta[0].data.data();
  double *stop = x->sto[0].data.data();
  for (auto &e : x->devs) e.device->updateSources();
  for (auto &e : x->devs) e.device->updateState(solp, stap, stop);
  for (auto &e : x->devs) e.device->updateSecondaryState(x->stadot.data.data(), stop);
  for (auto &e : x->devs)
    e.device->loadDAEVectors(solp, x->f.data.data(), x->q.data.data(), x->lead_f.data.data(),
                             x->lead_q.data.data());
  for (auto &e : x->devs) e.device->loadDAEMatrices(*x->dfdx_obj.get(), *x->dqdx_obj.get());

  std::copy(x->f.data.begin(), x->f.data.end(), f);
  std::copy(x->q.data.begin(), x->q.data.end(), q);
  std::copy(x->dfdxdvp.data.begin(), x->dfdxdvp.data.end(), dfdxdvp);
  std::copy(x->dqdxdvp.data.begin(), x->dqdxdvp.data.end(), dqdxdvp);
  if (x->n_state) std::copy(x->sta[0].data.begin(), x->sta[0].data.begin() + x->n_state, sta_next);
  if (x->n_store) std::copy(x->sto[0].data.begin(), x->sto[0].data.begin() + x->n_store, sto_next);
  std::copy(x->dfdx.val.begin(), x->dfdx.val.end(), dfdx);
  std::copy(x->dqdx.val.begin(), x->dqdx.val.end(), dqdx);
  return 0;
}

}  // extern "C"
