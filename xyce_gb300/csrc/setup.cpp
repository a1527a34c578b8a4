// setup.cpp — host-side circuit setup: model cards, per-instance derived
// parameters, unknown/state numbering, the Jacobian pattern, and the plan of
// stamp terms and their fixed-order reduction.
//
// Restates the reference's setup path for the supported devices:
//   Model constructors + Model::processParams     (MOSFET1 :3786-3866, :3890-3990;
//                                                  Diode :1772-1790, :1826-1900)
//   Instance constructors + updateTemperature     (MOSFET1 :1170-1262, :3437-3680;
//                                                  Diode :380-400, :1335-1500)
//   Resistor::updateTemperature :847-863, Capacitor, Vsrc PulseData params
//   Topology registerLIDs / registerJacLIDs       (N_TOP_CktGraphBasic.C:1092-1142)
// (all OpenModels paths are src/DeviceModelPKG/OpenModels/src/N_DEV_*.C).
// Compiled with -ffp-contract=off so every derived parameter is rounded as the
// reference computes it.

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "xg_internal.h"
#include "xg_bsim3_setup.h"

namespace xg {

// ---- constants (src/DeviceModelPKG/Core/include/N_DEV_Const.h) -------------
static const double kQ = 1.6021918e-19;      // CONSTQ
static const double kBoltz = 1.3806226e-23;  // CONSTboltz
static const double kRefTemp = 300.15;       // CONSTREFTEMP
static const double kCtoK = 273.15;          // CONSTCtoK
static inline double KoverQ() { return kBoltz / kQ; }  // CONSTKoverQ
static inline double Root2() { return std::sqrt(2.0); }  // CONSTroot2

// ---- stamp term tables (statement order of each Master load loop) ----------
// Resistor: N_DEV_Resistor.C:1094-1135.  LID slots: 0 pos, 1 neg.
static const TermDef kResTerms[] = {
    {OUT_F, 0, 0}, {OUT_F, 1, 0},
    {OUT_DFDX, 0, 0}, {OUT_DFDX, 0, 1}, {OUT_DFDX, 1, 0}, {OUT_DFDX, 1, 1}};
// Capacitor: N_DEV_Capacitor.C:1881-2040.  LID slots: 0 pos, 1 neg.
static const TermDef kCapTerms[] = {
    {OUT_Q, 0, 0}, {OUT_Q, 1, 0},
    {OUT_DQDX, 0, 0}, {OUT_DQDX, 0, 1}, {OUT_DQDX, 1, 0}, {OUT_DQDX, 1, 1}};
// Vsrc: N_DEV_Vsrc.C:1002-1045.  LID slots: 0 pos, 1 neg, 2 branch.
static const TermDef kVsrcTerms[] = {
    {OUT_F, 0, 0}, {OUT_F, 1, 0}, {OUT_F, 2, 0}, {OUT_F, 2, 0},
    {OUT_DFDX, 0, 2}, {OUT_DFDX, 1, 2}, {OUT_DFDX, 2, 0}, {OUT_DFDX, 2, 1}};
// ISRC: N_DEV_ISRC.C:774-800 (F only, an empty Jacobian stamp).  LID slots: 0 pos, 1 neg.
static const TermDef kIsrcTerms[] = {{OUT_F, 0, 0}, {OUT_F, 1, 0}};
// Diode: N_DEV_Diode.C:2034-2128.  LID slots: 0 pos, 1 neg, 2 pos'.
static const TermDef kDiodeTerms[] = {
    {OUT_F, 0, 0}, {OUT_F, 1, 0}, {OUT_F, 2, 0},
    {OUT_Q, 1, 0}, {OUT_Q, 2, 0},
    {OUT_DFDXDVP, 1, 0}, {OUT_DFDXDVP, 2, 0}, {OUT_DQDXDVP, 1, 0}, {OUT_DQDXDVP, 2, 0},
    {OUT_DFDX, 0, 0}, {OUT_DFDX, 0, 2}, {OUT_DFDX, 1, 1}, {OUT_DFDX, 1, 2},
    {OUT_DFDX, 2, 0}, {OUT_DFDX, 2, 1}, {OUT_DFDX, 2, 2},
    {OUT_DQDX, 1, 1}, {OUT_DQDX, 1, 2}, {OUT_DQDX, 2, 1}, {OUT_DQDX, 2, 2}};
// MOSFET1: N_DEV_MOSFET1.C:4202-4722 (newMeyer off).
// LID slots: 0 d, 1 g, 2 s, 3 b, 4 d', 5 s'.
static const TermDef kMos1Terms[] = {
    {OUT_F, 0, 0}, {OUT_F, 1, 0}, {OUT_F, 2, 0}, {OUT_F, 3, 0}, {OUT_F, 4, 0}, {OUT_F, 5, 0},
    {OUT_Q, 1, 0}, {OUT_Q, 3, 0}, {OUT_Q, 4, 0}, {OUT_Q, 5, 0},
    {OUT_DFDXDVP, 3, 0}, {OUT_DFDXDVP, 4, 0}, {OUT_DFDXDVP, 5, 0},
    {OUT_DQDXDVP, 1, 0}, {OUT_DQDXDVP, 3, 0}, {OUT_DQDXDVP, 4, 0}, {OUT_DQDXDVP, 5, 0},
    {OUT_DFDX, 0, 0}, {OUT_DFDX, 0, 4}, {OUT_DFDX, 2, 2}, {OUT_DFDX, 2, 5},
    {OUT_DFDX, 3, 3}, {OUT_DFDX, 3, 4}, {OUT_DFDX, 3, 5},
    {OUT_DFDX, 4, 0}, {OUT_DFDX, 4, 1}, {OUT_DFDX, 4, 3}, {OUT_DFDX, 4, 4}, {OUT_DFDX, 4, 5},
    {OUT_DFDX, 5, 1}, {OUT_DFDX, 5, 2}, {OUT_DFDX, 5, 3}, {OUT_DFDX, 5, 4}, {OUT_DFDX, 5, 5},
    {OUT_DQDX, 1, 1}, {OUT_DQDX, 1, 3}, {OUT_DQDX, 1, 4}, {OUT_DQDX, 1, 5},
    {OUT_DQDX, 3, 1}, {OUT_DQDX, 3, 3}, {OUT_DQDX, 3, 4}, {OUT_DQDX, 3, 5},
    {OUT_DQDX, 4, 1}, {OUT_DQDX, 4, 3}, {OUT_DQDX, 4, 4},
    {OUT_DQDX, 5, 1}, {OUT_DQDX, 5, 3}, {OUT_DQDX, 5, 5}};

#define NT(a) int(sizeof(a) / sizeof((a)[0]))
const TypeLayout &type_layout(int t) {
  static const TypeLayout L[XG_NUM_DEV_TYPES] = {
      {2, NT(kResTerms), kResTerms, XG_R_NPARAMS, 0, 0},
      {2, NT(kCapTerms), kCapTerms, XG_C_NPARAMS, 1, 0},
      {3, NT(kVsrcTerms), kVsrcTerms, XG_V_NPARAMS, 0, 0},
      {2, NT(kIsrcTerms), kIsrcTerms, XG_V_NPARAMS, 0, 0},
      {3, NT(kDiodeTerms), kDiodeTerms, XG_D_NPARAMS, 0, 1},
      {6, NT(kMos1Terms), kMos1Terms, XG_M1_NPARAMS, 8, 5},
      {b3_nlid(), b3_nterm(), b3_terms(), XG_B3_NPARAMS, 12, 5},
  };
  return L[t];
}

// Runs f(i, scratch, err) for i in [0, n) on the host's cores, in fixed
// chunks of 1,024, each worker with its own scratch of np doubles.  Returns
// the error of the lowest failing i, as the serial loop would.  Set-up of a
// batch union or a million-device netlist is per model and per instance.
template <class F>
int parallel_rows(int n, int np, F f, std::string *err) {
  constexpr int kChunk = 1024;
  const int nchunks = (n + kChunk - 1) / kChunk;
  const int hw = int(std::thread::hardware_concurrency());
  const int nt = std::max(1, std::min(std::min(nchunks, 16), hw > 0 ? hw : 1));
  std::vector<int> rc(size_t(std::max(nchunks, 1)), 0);
  std::vector<std::string> msg(size_t(std::max(nchunks, 1)));
  std::atomic<int> next{0};
  auto work = [&]() {
    std::vector<double> tmp(size_t(std::max(np, 1)));
    for (int c = next++; c < nchunks; c = next++)
      for (int i = c * kChunk; i < std::min(n, (c + 1) * kChunk); ++i) {
        const int r = f(i, tmp.data(), &msg[size_t(c)]);
        if (r) {
          rc[size_t(c)] = r;
          break;
        }
      }
  };
  std::vector<std::thread> pool;
  for (int k = 1; k < nt; ++k) pool.emplace_back(work);
  work();
  for (auto &th : pool) th.join();
  for (int c = 0; c < nchunks; ++c)
    if (rc[size_t(c)]) {
      *err = msg[size_t(c)];
      return rc[size_t(c)];
    }
  return XG_OK;
}

// ---- model cards -----------------------------------------------------------
namespace {

std::string upper(const char *s) {
  std::string r(s);
  for (auto &ch : r) ch = (char)std::toupper((unsigned char)ch);
  return r;
}

struct Card {
  std::map<std::string, double> v;
  bool given(const char *k) const { return v.count(k) != 0; }
  double get(const char *k, double def) const {
    auto it = v.find(k);
    return it == v.end() ? def : it->second;
  }
};

Card read_card(const xg_model_desc &m) {
  Card c;
  for (int i = 0; i < m.n_params; ++i) c.v[upper(m.names[i])] = m.values[i];
  return c;
}

// MOSFET level-1 model after Model::Model + Model::processParams.
struct Mos1Model {
  int dtype;
  double model_l, model_w, vt0, transconductance, gamma, phi, lambda;
  double drainResistance, sourceResistance, capBD, capBS, jctSatCur, bulkJctPotential;
  double cgso, cgdo, cgbo, sheetResistance, bulkCapFactor, bulkJctBotGradingCoeff;
  double sideWallCapFactor, bulkJctSideGradingCoeff, jctSatCurDensity, oxideThickness;
  double latDiff, surfaceMobility, fwdCapDepCoeff, substrateDoping, surfaceStateDensity;
  double tnom, gateType;
  bool capBDGiven, capBSGiven, bulkCapFactorGiven, sideWallCapFactorGiven, rshGiven;
  // processParams outputs
  double fact1, vtnom, egfet1, pbfact1, oxideCapFactor;
};

int make_mos1_model(const xg_model_desc &md, const xg_device_options &opt, Mos1Model *m,
                    std::string *err) {
  static const char *known[] = {"L", "W", "VTO", "KP", "GAMMA", "PHI", "LAMBDA", "RD", "RS",
                                "CBD", "CBS", "IS", "PB", "CGSO", "CGDO", "CGBO", "RSH", "CJ",
                                "MJ", "CJSW", "MJSW", "JS", "TOX", "LD", "UO", "U0", "FC",
                                "NSUB", "NSS", "TNOM", "KF", "AF", "TPG", "LEVEL"};
  Card c = read_card(md);
  for (auto &kv : c.v)
    if (std::find_if(std::begin(known), std::end(known),
                     [&](const char *k) { return kv.first == k; }) == std::end(known)) {
      *err = "MOSFET level 1: unsupported model parameter " + kv.first;
      return XG_ERR_UNSUPPORTED;
    }
  m->dtype = md.polarity < 0 ? -1 : 1;
  m->model_l = c.get("L", 1e-4);
  m->model_w = c.get("W", 1e-4);
  m->vt0 = c.get("VTO", 0.0);
  m->transconductance = c.get("KP", 2e-5);
  m->gamma = c.get("GAMMA", 0.0);
  m->phi = c.get("PHI", 0.6);
  m->lambda = c.get("LAMBDA", 0.0);
  m->drainResistance = c.get("RD", 0.0);
  m->sourceResistance = c.get("RS", 0.0);
  m->capBD = c.get("CBD", 0.0);
  m->capBS = c.get("CBS", 0.0);
  m->jctSatCur = c.get("IS", 1e-14);
  m->bulkJctPotential = c.get("PB", 0.8);
  m->cgso = c.get("CGSO", 0.0);
  m->cgdo = c.get("CGDO", 0.0);
  m->cgbo = c.get("CGBO", 0.0);
  m->sheetResistance = c.get("RSH", 0.0);
  m->rshGiven = c.given("RSH");
  m->bulkCapFactor = c.get("CJ", 0.0);
  m->bulkCapFactorGiven = c.given("CJ");
  m->bulkJctBotGradingCoeff = c.get("MJ", 0.5);
  m->sideWallCapFactor = c.get("CJSW", 0.0);
  m->sideWallCapFactorGiven = c.given("CJSW");
  m->bulkJctSideGradingCoeff = c.get("MJSW", 0.5);
  m->jctSatCurDensity = c.get("JS", 0.0);
  m->oxideThickness = c.get("TOX", 1e-7);
  m->latDiff = c.get("LD", 0.0);
  m->surfaceMobility = c.get("UO", 600.0);
  if (c.given("U0")) m->surfaceMobility = c.get("U0", 600.0);
  m->fwdCapDepCoeff = c.get("FC", 0.5);
  m->substrateDoping = c.get("NSUB", 0.0);
  m->surfaceStateDensity = c.get("NSS", 0.0);
  m->gateType = c.get("TPG", 0.0);
  m->tnom = c.given("TNOM") ? c.get("TNOM", 27.0) + kCtoK : opt.tnom;
  m->capBDGiven = m->capBD != 0;
  m->capBSGiven = m->capBS != 0;

  // Model::processParams (N_DEV_MOSFET1.C:3786-3866)
  const double tnom = m->tnom;
  m->fact1 = tnom / kRefTemp;
  m->vtnom = tnom * KoverQ();
  double kt1 = kBoltz * tnom;
  m->egfet1 = 1.16 - (7.02e-4 * tnom * tnom) / (tnom + 1108);
  double arg1 = -m->egfet1 / (kt1 + kt1) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
  m->pbfact1 = -2 * m->vtnom * (1.5 * std::log(m->fact1) + kQ * arg1);
  if (!c.given("TOX") || m->oxideThickness == 0) {
    m->oxideCapFactor = 0;
  } else {
    m->oxideCapFactor = 3.9 * 8.854214871e-12 / m->oxideThickness;
    if (!c.given("KP")) {
      if (!c.given("UO") && !c.given("U0")) m->surfaceMobility = 600;
      m->transconductance = m->surfaceMobility * m->oxideCapFactor * 1e-4;
    }
    if (c.given("NSUB")) {
      if (m->substrateDoping * 1e6 > 1.45e16) {
        if (!c.given("PHI")) {
          m->phi = 2 * m->vtnom * std::log(m->substrateDoping * 1e6 / 1.45e16);
          m->phi = 0.1 > m->phi ? 0.1 : m->phi;  // Xycemax(0.1, phi)
        }
        double fermis = m->dtype * .5 * m->phi;
        double wkfng = 3.2;
        if (!c.given("TPG")) m->gateType = 1;
        if (m->gateType != 0) {
          double fermig = m->dtype * m->gateType * .5 * m->egfet1;
          wkfng = 3.25 + .5 * m->egfet1 - fermig;
        }
        double wkfngs = wkfng - (3.25 + .5 * m->egfet1 + fermis);
        if (!c.given("GAMMA"))
          m->gamma = std::sqrt(2 * 11.70 * 8.854214871e-12 * kQ * m->substrateDoping * 1e6) /
                     m->oxideCapFactor;
        if (!c.given("VTO")) {
          if (!c.given("NSS")) m->surfaceStateDensity = 0;
          double vfb = wkfngs - m->surfaceStateDensity * 1e4 * kQ / m->oxideCapFactor;
          m->vt0 = vfb + m->dtype * (m->gamma * std::sqrt(m->phi) + m->phi);
        }
      } else {
        *err = "MOSFET level 1: Nsub < Ni";
        return XG_ERR_ARG;
      }
    }
  }
  return XG_OK;
}

// Instance constructor + updateTemperature (N_DEV_MOSFET1.C:1170-1262, 3437-3680)
// + the per-load constants of updateIntermediateVars (:2650-2665).
void mos1_instance_params(const Mos1Model &mo, const xg_mos_desc &d, int i,
                          const xg_device_options &opt, double *out /* XG_M1_NPARAMS */) {
  const double temp = opt.temp;
  double l = d.l ? d.l[i] : mo.model_l;
  double w = d.w ? d.w[i] : mo.model_w;
  double drainArea = d.ad ? d.ad[i] : 0.0;      // DeviceOptions::defad
  double sourceArea = d.as ? d.as[i] : 0.0;     // DeviceOptions::defas
  double drainPerimeter = d.pd ? d.pd[i] : 0.0;
  double sourcePerimeter = d.ps ? d.ps[i] : 0.0;
  double drainSquares = d.nrd ? d.nrd[i] : 1.0;
  double sourceSquares = d.nrs ? d.nrs[i] : 1.0;
  double numberParallel = d.m ? d.m[i] : 1.0;

  double drainConductance, sourceConductance;
  if (mo.drainResistance != 0) drainConductance = 1 / mo.drainResistance;
  else if (mo.rshGiven) drainConductance = mo.sheetResistance != 0 ? 1 / (mo.sheetResistance * drainSquares) : 0;
  else drainConductance = 0;
  if (mo.sourceResistance != 0) sourceConductance = 1 / mo.sourceResistance;
  else if (mo.rshGiven) sourceConductance = mo.sheetResistance != 0 ? 1 / (mo.sheetResistance * sourceSquares) : 0;
  else sourceConductance = 0;

  double EffectiveLength = l - 2 * mo.latDiff;
  double GateSourceOverlapCap = mo.cgso * w;
  double GateDrainOverlapCap = mo.cgdo * w;
  double GateBulkOverlapCap = mo.cgbo * EffectiveLength;
  double OxideCap = mo.oxideCapFactor * EffectiveLength * w;

  // updateTemperature
  const double tnom = mo.tnom;
  double vt = temp * KoverQ();
  double ratio = temp / tnom;
  double fact2 = temp / kRefTemp;
  double kt = temp * kBoltz;
  double egfet = 1.16 - (7.02e-4 * temp * temp) / (temp + 1108);
  double arg = -egfet / (kt + kt) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
  double pbfact = -2 * vt * (1.5 * std::log(fact2) + kQ * arg);
  double ratio4 = ratio * std::sqrt(ratio);
  double tTransconductance = mo.transconductance / ratio4;
  double phio = (mo.phi - mo.pbfact1) / mo.fact1;
  double tPhi = fact2 * phio + pbfact;
  double tVbi = mo.vt0 - mo.dtype * (mo.gamma * std::sqrt(mo.phi)) + .5 * (mo.egfet1 - egfet) +
                mo.dtype * .5 * (tPhi - mo.phi);
  double tVto = tVbi + mo.dtype * mo.gamma * std::sqrt(tPhi);
  double tSatCur = mo.jctSatCur * std::exp(-egfet / vt + mo.egfet1 / mo.vtnom);
  double tSatCurDens = mo.jctSatCurDensity * std::exp(-egfet / vt + mo.egfet1 / mo.vtnom);
  double pbo = (mo.bulkJctPotential - mo.pbfact1) / mo.fact1;
  double gmaold = (mo.bulkJctPotential - pbo) / pbo;
  double capfact = 1 / (1 + mo.bulkJctBotGradingCoeff * (4e-4 * (mo.tnom - kRefTemp) - gmaold));
  double tCbd = mo.capBD * capfact;
  double tCbs = mo.capBS * capfact;
  double tCj = mo.bulkCapFactor * capfact;
  capfact = 1 / (1 + mo.bulkJctSideGradingCoeff * (4e-4 * (mo.tnom - kRefTemp) - gmaold));
  double tCjsw = mo.sideWallCapFactor * capfact;
  double tBulkPot = fact2 * pbo + pbfact;
  double gmanew = (tBulkPot - pbo) / pbo;
  capfact = (1 + mo.bulkJctBotGradingCoeff * (4e-4 * (temp - kRefTemp) - gmanew));
  tCbd *= capfact;
  tCbs *= capfact;
  tCj *= capfact;
  capfact = (1 + mo.bulkJctSideGradingCoeff * (4e-4 * (temp - kRefTemp) - gmanew));
  tCjsw *= capfact;
  double tDepCap = mo.fwdCapDepCoeff * tBulkPot;
  double sourceVcrit, drainVcrit;
  if ((mo.jctSatCurDensity == 0) || (drainArea == 0) || (sourceArea == 0)) {
    sourceVcrit = drainVcrit = vt * std::log(vt / (Root2() * mo.jctSatCur));
  } else {
    drainVcrit = vt * std::log(vt / (Root2() * mo.jctSatCurDensity * drainArea));
    sourceVcrit = vt * std::log(vt / (Root2() * mo.jctSatCurDensity * sourceArea));
  }
  const double MJ = mo.bulkJctBotGradingCoeff, MJSW = mo.bulkJctSideGradingCoeff;
  const double FC = mo.fwdCapDepCoeff;
  double czbd = mo.capBDGiven ? tCbd : (mo.bulkCapFactorGiven ? tCj * drainArea : 0);
  double czbdsw = mo.sideWallCapFactorGiven ? tCjsw * drainPerimeter : 0;
  arg = 1 - FC;
  double sarg = std::exp((-MJ) * std::log(arg));
  double sargsw = std::exp((-MJSW) * std::log(arg));
  double Cbd = czbd, Cbdsw = czbdsw;
  double f2d = czbd * (1 - FC * (1 + MJ)) * sarg / arg + czbdsw * (1 - FC * (1 + MJSW)) * sargsw / arg;
  double f3d = czbd * MJ * sarg / arg / tBulkPot + czbdsw * MJSW * sargsw / arg / tBulkPot;
  double f4d = czbd * tBulkPot * (1 - arg * sarg) / (1 - MJ) +
               czbdsw * tBulkPot * (1 - arg * sargsw) / (1 - MJSW) - f3d / 2 * (tDepCap * tDepCap) -
               tDepCap * f2d;
  double czbs = mo.capBSGiven ? tCbs : (mo.bulkCapFactorGiven ? tCj * sourceArea : 0);
  double czbssw = mo.sideWallCapFactorGiven ? tCjsw * sourcePerimeter : 0;
  double Cbs = czbs, Cbssw = czbssw;
  double f2s = czbs * (1 - FC * (1 + MJ)) * sarg / arg + czbssw * (1 - FC * (1 + MJSW)) * sargsw / arg;
  double f3s = czbs * MJ * sarg / arg / tBulkPot + czbssw * MJSW * sargsw / arg / tBulkPot;
  double f4s = czbs * tBulkPot * (1 - arg * sarg) / (1 - MJ) +
               czbssw * tBulkPot * (1 - arg * sargsw) / (1 - MJSW) - f3s / 2 * (tDepCap * tDepCap) -
               tDepCap * f2s;

  // updateIntermediateVars per-load constants (N_DEV_MOSFET1.C:2650-2665)
  double DrainSatCur, SourceSatCur;
  if ((tSatCurDens == 0) || (drainArea == 0) || (sourceArea == 0)) {
    DrainSatCur = tSatCur;
    SourceSatCur = tSatCur;
  } else {
    DrainSatCur = tSatCurDens * drainArea;
    SourceSatCur = tSatCurDens * sourceArea;
  }
  double Beta = tTransconductance * w / EffectiveLength;

  out[XG_M1_DTYPE] = mo.dtype;
  out[XG_M1_GAMMA] = mo.gamma;
  out[XG_M1_LAMBDA] = mo.lambda;
  out[XG_M1_MJ] = MJ;
  out[XG_M1_MJSW] = MJSW;
  out[XG_M1_DRAINSATCUR] = DrainSatCur;
  out[XG_M1_SOURCESATCUR] = SourceSatCur;
  out[XG_M1_BETA] = Beta;
  out[XG_M1_TVTO] = tVto;
  out[XG_M1_SOURCEVCRIT] = sourceVcrit;
  out[XG_M1_DRAINVCRIT] = drainVcrit;
  out[XG_M1_VT] = vt;
  out[XG_M1_TPHI] = tPhi;
  out[XG_M1_TVBI] = tVbi;
  out[XG_M1_CBS] = Cbs;
  out[XG_M1_CBSSW] = Cbssw;
  out[XG_M1_CBD] = Cbd;
  out[XG_M1_CBDSW] = Cbdsw;
  out[XG_M1_TDEPCAP] = tDepCap;
  out[XG_M1_TBULKPOT] = tBulkPot;
  out[XG_M1_F2S] = f2s;
  out[XG_M1_F3S] = f3s;
  out[XG_M1_F4S] = f4s;
  out[XG_M1_F2D] = f2d;
  out[XG_M1_F3D] = f3d;
  out[XG_M1_F4D] = f4d;
  out[XG_M1_OXIDECAP] = OxideCap;
  out[XG_M1_CGSO] = GateSourceOverlapCap;
  out[XG_M1_CGDO] = GateDrainOverlapCap;
  out[XG_M1_CGBO] = GateBulkOverlapCap;
  out[XG_M1_GD] = drainConductance;
  out[XG_M1_GS] = sourceConductance;
  out[XG_M1_M] = numberParallel;
  out[XG_M1_ICVDS] = 0.0;
  out[XG_M1_ICVGS] = 0.0;
  out[XG_M1_ICVBS] = 0.0;
  out[XG_M1_FLAGS] = 0.0;
}

// Diode, level 1.
struct DiodeModel {
  double IS, RS, COND, N, TT, CJO, VJ, M, EG, XTI, FC, BV, IBV, IRF, TNOM, F2, F3;
  bool BVGiven;
};

int make_diode_model(const xg_model_desc &md, const xg_device_options &opt, DiodeModel *m,
                     std::string *err) {
  static const char *known[] = {"IS", "JS", "RS", "N", "TT", "CJO", "CJ", "CJ0", "VJ", "M",
                                "EG", "XTI", "FC", "BV", "VB", "IBV", "IRF", "TNOM", "KF",
                                "AF", "LEVEL"};
  Card c = read_card(md);
  for (auto &kv : c.v)
    if (std::find_if(std::begin(known), std::end(known),
                     [&](const char *k) { return kv.first == k; }) == std::end(known)) {
      *err = "diode: unsupported model parameter " + kv.first;
      return XG_ERR_UNSUPPORTED;
    }
  if (c.given("LEVEL") && c.get("LEVEL", 1) != 1) {
    *err = "diode: only level 1 is supported";
    return XG_ERR_UNSUPPORTED;
  }
  m->IS = c.given("IS") ? c.get("IS", 1e-14) : c.get("JS", 1e-14);
  m->RS = c.get("RS", 0.0);
  m->N = c.get("N", 1.0);
  m->TT = c.get("TT", 0.0);
  m->CJO = c.given("CJO") ? c.get("CJO", 0) : (c.given("CJ") ? c.get("CJ", 0) : c.get("CJ0", 0.0));
  m->VJ = c.get("VJ", 1.0);
  m->M = c.get("M", 0.5);
  m->EG = c.get("EG", 1.11);
  m->XTI = c.get("XTI", 3.0);
  m->FC = c.get("FC", 0.5);
  m->BVGiven = c.given("BV") || c.given("VB");
  m->BV = c.given("BV") ? c.get("BV", 1e99) : c.get("VB", 1e99);
  m->IBV = c.get("IBV", 1.0e-3);
  m->IRF = c.get("IRF", 1.0);
  m->TNOM = c.given("TNOM") ? c.get("TNOM", 27.0) + kCtoK : opt.tnom;
  // Model::processParams (N_DEV_Diode.C:1772-1790)
  if (m->M > 0.9) m->M = 0.9;
  if (m->EG < 0.1) m->EG = 0.1;
  if (m->FC > 0.95) m->FC = 0.95;
  m->COND = m->RS == 0.0 ? 0.0 : 1.0 / m->RS;
  double xfc = std::log(1.0 - m->FC);
  m->F2 = std::exp((1.0 + m->M) * xfc);
  m->F3 = 1.0 - m->FC * (1.0 + m->M);
  return XG_OK;
}

// Diode Instance::updateTemperature (N_DEV_Diode.C:1335-1500), level 1.
void diode_instance_params(const DiodeModel &mo, const xg_diode_desc &d, int i,
                           const xg_device_options &opt, double *out) {
  const double CONSTe = std::exp(1.0);
  const double Area = d.area ? d.area[i] : 1.0;
  const double Temp = opt.temp;
  double vtnom = KoverQ() * mo.TNOM;
  double xfc = std::log(1.0 - mo.FC);
  double vt = KoverQ() * Temp;
  double fact2 = Temp / kRefTemp;
  double egfet = 1.16 - (7.02e-4 * Temp * Temp) / (Temp + 1108.0);
  double arg = -egfet / (2.0 * kBoltz * Temp) + 1.1150877 / (kBoltz * (kRefTemp + kRefTemp));
  double pbfact = -2.0 * vt * (1.5 * std::log(fact2) + kQ * arg);
  double egfet1 = 1.16 - (7.02e-4 * mo.TNOM * mo.TNOM) / (mo.TNOM + 1108.0);
  double arg1 = -egfet1 / (2.0 * kBoltz * mo.TNOM) + 1.1150877 / (2.0 * kBoltz * kRefTemp);
  double fact1 = mo.TNOM / kRefTemp;
  double pbfact1 = -2.0 * vtnom * (1.5 * std::log(fact1) + kQ * arg1);
  double pbo = (mo.VJ - pbfact1) / fact1;
  double gmaold = (mo.VJ - pbo) / pbo;
  double tJctCap = mo.CJO / (1.0 + mo.M * (4.0e-4 * (mo.TNOM - kRefTemp) - gmaold));
  double tJctPot = pbfact + fact2 * pbo;
  double gmanew = (tJctPot - pbo) / pbo;
  tJctCap *= 1.0 + mo.M * (4.0e-4 * (Temp - kRefTemp) - gmanew);
  double tSatCur = mo.IS * std::exp(((Temp / mo.TNOM) - 1.0) * mo.EG / (mo.N * vt) +
                                    mo.XTI / mo.N * std::log(Temp / mo.TNOM));
  double tF1 = tJctPot * (1.0 - std::exp((1.0 - mo.M) * xfc)) / (1.0 - mo.M);
  double tDepCap = mo.FC * tJctPot;
  double vte = mo.N * vt;
  double tVcrit = vte * std::log(vte / (Root2() * tSatCur));
  double tCOND = mo.COND;
  double tIRF = mo.IRF * std::pow(fact2, 1.6);
  double tempBV = mo.BV;
  double tBrkdwnV = 0.0;
  if (mo.BVGiven) {
    double IRFactor = tIRF;
    double cbv = mo.IBV;
    double a1 = 3.0 * vte / (CONSTe * tempBV);
    a1 = a1 * a1 * a1;
    double cthreshlow = tSatCur * IRFactor * (1 - a1);
    double cthreshhigh = tSatCur * IRFactor * (1 - 1.0 / (CONSTe * CONSTe * CONSTe)) *
                         std::exp(-1.0 * (3.0 * vte - tempBV) / vte);
    if (cbv >= cthreshhigh) {
      tBrkdwnV = 3.0 * vte;
    } else if (cbv <= cthreshlow) {
      tBrkdwnV = tempBV;
    } else {
      double xbv = tempBV;
      for (int it = 0; it < 8; it++) {
        double a2 = 3.0 * vte / (CONSTe * xbv);
        a2 = a2 * a2 * a2;
        xbv = tempBV - vte * std::log(cbv / (tSatCur * IRFactor)) + vte * std::log(1 - a2);
      }
      tBrkdwnV = xbv;
    }
  }
  out[XG_D_M] = mo.M;
  out[XG_D_BV] = mo.BV;
  out[XG_D_N] = mo.N;
  out[XG_D_TT] = mo.TT;
  out[XG_D_F2] = mo.F2;
  out[XG_D_F3] = mo.F3;
  out[XG_D_ISAT] = tSatCur * Area;
  out[XG_D_VT] = KoverQ() * Temp;
  out[XG_D_GSPR] = tCOND * Area;
  out[XG_D_TVCRIT] = tVcrit;
  out[XG_D_TIRF] = tIRF;
  out[XG_D_TBRKDWNV] = tBrkdwnV;
  out[XG_D_TJCTCAP] = tJctCap;
  out[XG_D_TJCTPOT] = tJctPot;
  out[XG_D_TDEPCAP] = tDepCap;
  out[XG_D_TF1] = tF1;
  out[XG_D_AREA] = Area;
  out[XG_D_INITCOND] = 0.0;
  out[XG_D_FLAGS] = mo.BVGiven ? 1.0 : 0.0;
}

int count_of(const xg_netlist *nl, int t) {
  switch (t) {
    case XG_DEV_RES: return nl->res.n;
    case XG_DEV_CAP: return nl->cap.n;
    case XG_DEV_VSRC: return nl->vsrc.n;
    case XG_DEV_ISRC: return nl->isrc.n;
    case XG_DEV_DIODE: return nl->diode.n;
    case XG_DEV_MOS1: return nl->mos1.n;
    case XG_DEV_BSIM3: return nl->bsim3.n;
  }
  return 0;
}

bool node_ok(int node, int n_nodes) { return node >= -1 && node < n_nodes; }

}  // namespace

// ---- the plan ---------------------------------------------------------------
int build_plan(const xg_netlist *nl, const xg_device_options *opt, Plan *plan, std::string *err,
               bool params_only) {
  Plan &P = *plan;
  if (!nl || !opt || nl->n_nodes < 0) { *err = "null netlist/options"; return XG_ERR_ARG; }
  if (opt->newmeyer) { *err = "newmeyer=1 is not supported"; return XG_ERR_UNSUPPORTED; }
  P.n_nodes = nl->n_nodes;
  if (nl->type_order && nl->n_type_order > 0) {
    if (nl->n_type_order > XG_NUM_DEV_TYPES) { *err = "type_order too long"; return XG_ERR_ARG; }
    P.n_order = nl->n_type_order;
    bool seen[XG_NUM_DEV_TYPES] = {};
    for (int k = 0; k < P.n_order; ++k) {
      int t = nl->type_order[k];
      if (t < 0 || t >= XG_NUM_DEV_TYPES || seen[t]) { *err = "bad type_order"; return XG_ERR_ARG; }
      seen[t] = true;
      P.order[k] = t;
    }
    for (int t = 0; t < XG_NUM_DEV_TYPES; ++t)
      if (!seen[t] && count_of(nl, t)) { *err = "type_order misses a used type"; return XG_ERR_ARG; }
  } else {
    P.n_order = XG_NUM_DEV_TYPES;
    for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) P.order[t] = t;
  }

  // Models.
  std::vector<Mos1Model> mos1_models(nl->n_models);
  std::vector<DiodeModel> diode_models(nl->n_models);
  std::vector<B3Model> b3_models(nl->n_models);
  std::vector<int> model_ok(nl->n_models, 0);
  {
    int rc = parallel_rows(nl->n_models, 0, [&](int mi, double *, std::string *e) {
      const xg_model_desc &md = nl->models[mi];
      int r = XG_OK;
      if (md.type == XG_DEV_MOS1) r = make_mos1_model(md, *opt, &mos1_models[mi], e);
      else if (md.type == XG_DEV_DIODE) r = make_diode_model(md, *opt, &diode_models[mi], e);
      else if (md.type == XG_DEV_BSIM3) r = b3_make_model(md, *opt, &b3_models[mi], e);
      else { *e = "model of unsupported device type"; r = XG_ERR_UNSUPPORTED; }
      if (!r) model_ok[mi] = md.type;
      return r;
    }, err);
    if (rc) return rc;
  }
  auto check_model = [&](int mi, int type) {
    return mi >= 0 && mi < nl->n_models && model_ok[mi] == type;
  };

  // Per-type parameter blocks + node checks.
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    TypeData &T = P.T[t];
    const TypeLayout &L = type_layout(t);
    T.n = count_of(nl, t);
    T.np = L.np;
    T.nlid = L.nlid;
    T.nterm = L.nterm;
    T.nsta = L.nsta;
    T.nsto = L.nsto;
    if (!T.n) continue;
    T.params.assign((size_t)T.np * T.n, 0.0);
    auto row = [&](int i, double *tmp, std::string *e) -> int {
      auto bad_node = [&]() {
        *e = "node index out of range";
        return XG_ERR_ARG;
      };
      switch (t) {
        case XG_DEV_RES: {
          if (!node_ok(nl->res.p[i], P.n_nodes) || !node_ok(nl->res.m[i], P.n_nodes)) return bad_node();
          double R = nl->res.value[i], factor = 1.0;  // N_DEV_Resistor.C:852-860
          tmp[XG_R_G] = (R * factor != 0.0) ? 1.0 / (R * factor) : 0.0;
          break;
        }
        case XG_DEV_CAP:
          if (!node_ok(nl->cap.p[i], P.n_nodes) || !node_ok(nl->cap.m[i], P.n_nodes)) return bad_node();
          tmp[XG_C_C] = nl->cap.value[i];
          break;
        case XG_DEV_VSRC:
        case XG_DEV_ISRC: {
          // Same source data for both (N_DEV_SourceData.C): the DC value, or PULSE's seven.
          const xg_src_desc &d = t == XG_DEV_VSRC ? nl->vsrc : nl->isrc;
          if (!node_ok(d.p[i], P.n_nodes) || !node_ok(d.m[i], P.n_nodes)) return bad_node();
          const double *w = d.wave + 7 * (size_t)i;
          int kind = d.kind[i];
          if (kind != XG_SRC_DC && kind != XG_SRC_PULSE) { *e = "bad source kind"; return XG_ERR_ARG; }
          tmp[XG_V_KIND] = kind;
          for (int k = 0; k < 7; ++k) tmp[XG_V_V1 + k] = kind == XG_SRC_PULSE || k == 0 ? w[k] : 0.0;
          break;
        }
        case XG_DEV_DIODE: {
          if (!node_ok(nl->diode.a[i], P.n_nodes) || !node_ok(nl->diode.c[i], P.n_nodes)) return bad_node();
          int mi = nl->diode.model[i];
          if (!check_model(mi, XG_DEV_DIODE)) { *e = "diode references a non-diode model"; return XG_ERR_ARG; }
          diode_instance_params(diode_models[mi], nl->diode, i, *opt, tmp);
          break;
        }
        case XG_DEV_MOS1: {
          const xg_mos_desc &d = nl->mos1;
          if (!node_ok(d.d[i], P.n_nodes) || !node_ok(d.g[i], P.n_nodes) ||
              !node_ok(d.s[i], P.n_nodes) || !node_ok(d.b[i], P.n_nodes)) return bad_node();
          int mi = d.model[i];
          if (!check_model(mi, XG_DEV_MOS1)) { *e = "MOSFET references a non-level-1 model"; return XG_ERR_ARG; }
          mos1_instance_params(mos1_models[mi], d, i, *opt, tmp);
          break;
        }
        case XG_DEV_BSIM3: {
          const xg_mos_desc &d = nl->bsim3;
          if (!node_ok(d.d[i], P.n_nodes) || !node_ok(d.g[i], P.n_nodes) ||
              !node_ok(d.s[i], P.n_nodes) || !node_ok(d.b[i], P.n_nodes)) return bad_node();
          int mi = d.model[i];
          if (!check_model(mi, XG_DEV_BSIM3)) { *e = "MOSFET references a non-BSIM3 model"; return XG_ERR_ARG; }
          int rc = b3_instance_params(b3_models[mi], d, i, *opt, tmp, e);
          if (rc) return rc;
          break;
        }
      }
      for (int k = 0; k < T.np; ++k) T.params[(size_t)k * T.n + i] = tmp[k];
      return XG_OK;
    };
    const int rc = parallel_rows(T.n, T.np, row, err);
    if (rc) return rc;
  }
  if (params_only) return XG_OK;

  // LIDs: circuit nodes, then internal unknowns in type order / instance order.
  int next = P.n_nodes;
  std::vector<std::vector<int>> lid_aos(XG_NUM_DEV_TYPES);
  for (int k = 0; k < P.n_order; ++k) {
    int t = P.order[k];
    TypeData &T = P.T[t];
    if (!T.n) continue;
    std::vector<int> &A = lid_aos[t];
    A.assign((size_t)T.nlid * T.n, -1);
    for (int i = 0; i < T.n; ++i) {
      int *Ls = &A[(size_t)i * T.nlid];
      auto prm = [&](int kk) { return T.params[(size_t)kk * T.n + i]; };
      switch (t) {
        case XG_DEV_RES: Ls[0] = nl->res.p[i]; Ls[1] = nl->res.m[i]; break;
        case XG_DEV_CAP: Ls[0] = nl->cap.p[i]; Ls[1] = nl->cap.m[i]; break;
        case XG_DEV_VSRC: Ls[0] = nl->vsrc.p[i]; Ls[1] = nl->vsrc.m[i]; Ls[2] = next++; break;
        case XG_DEV_ISRC: Ls[0] = nl->isrc.p[i]; Ls[1] = nl->isrc.m[i]; break;
        case XG_DEV_DIODE:
          Ls[0] = nl->diode.a[i]; Ls[1] = nl->diode.c[i];
          Ls[2] = prm(XG_D_GSPR) != 0.0 ? next++ : Ls[0];
          break;
        case XG_DEV_MOS1:
          Ls[0] = nl->mos1.d[i]; Ls[1] = nl->mos1.g[i]; Ls[2] = nl->mos1.s[i]; Ls[3] = nl->mos1.b[i];
          Ls[4] = prm(XG_M1_GD) != 0.0 ? next++ : Ls[0];
          Ls[5] = prm(XG_M1_GS) != 0.0 ? next++ : Ls[2];
          break;
        case XG_DEV_BSIM3: {
          int ext[4] = {nl->bsim3.d[i], nl->bsim3.g[i], nl->bsim3.s[i], nl->bsim3.b[i]};
          b3_assign_lids(T.params.data(), T.n, i, ext, &next, Ls);
          break;
        }
      }
    }
  }
  P.n_unknowns = next;
  const int gnd = P.n_unknowns;
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    TypeData &T = P.T[t];
    if (!T.n) continue;
    T.lid.assign((size_t)T.nlid * T.n, 0);
    for (int i = 0; i < T.n; ++i)
      for (int j = 0; j < T.nlid; ++j) {
        int v = lid_aos[t][(size_t)i * T.nlid + j];
        T.lid[(size_t)j * T.n + i] = v < 0 ? gnd : v;
      }
  }

  // State / store numbering.
  int sta = 0, sto = 0;
  for (int k = 0; k < P.n_order; ++k) {
    int t = P.order[k];
    TypeData &T = P.T[t];
    if (!T.n) continue;
    T.sta0 = sta;
    T.sto0 = sto;
    if (t == XG_DEV_DIODE) {
      // One state slot per diode whose CJO == 0 (N_DEV_Diode.C:392-393).  The
      // load never reads or writes it; it only shifts the slots that follow.
      T.nsta = 0;
      for (int i = 0; i < T.n; ++i) sta += T.params[(size_t)XG_D_TJCTCAP * T.n + i] == 0.0 ? 1 : 0;
    } else {
      sta += T.nsta * T.n;
    }
    sto += T.nsto * T.n;
  }
  P.n_state = sta;
  P.n_store = sto;

  const int64_t W = (int64_t)P.n_unknowns + 1;
  // Jacobian pattern from every matrix term (ground excluded): the terms'
  // columns bucketed by row (a counting sort), then each row's few columns
  // sorted and made unique, rows in parallel.
  {
    std::vector<int64_t> rcount((size_t)P.n_unknowns + 1, 0);
    auto each_matrix_term = [&](auto &&fn) {
      for (int k = 0; k < P.n_order; ++k) {
        const int t = P.order[k];
        const TypeData &T = P.T[t];
        if (!T.n) continue;
        const TypeLayout &L = type_layout(t);
        for (int i = 0; i < T.n; ++i)
          for (int q = 0; q < L.nterm; ++q) {
            const TermDef &td = L.terms[q];
            if (td.kind != OUT_DFDX && td.kind != OUT_DQDX) continue;
            const int r = T.lid[(size_t)td.row * T.n + i], c = T.lid[(size_t)td.col * T.n + i];
            if (r == gnd || c == gnd) continue;
            fn(r, c);
          }
      }
    };
    each_matrix_term([&](int r, int) { rcount[(size_t)r + 1]++; });
    for (int r = 0; r < P.n_unknowns; ++r) rcount[(size_t)r + 1] += rcount[(size_t)r];
    std::vector<int> cols((size_t)rcount[(size_t)P.n_unknowns]);
    {
      std::vector<int64_t> fill(rcount.begin(), rcount.end() - 1);
      each_matrix_term([&](int r, int c) { cols[(size_t)fill[(size_t)r]++] = c; });
    }
    std::vector<int> ulen((size_t)P.n_unknowns, 0);
    int rc = parallel_rows(P.n_unknowns, 0, [&](int r, double *, std::string *) {
      int *b = cols.data() + rcount[(size_t)r], *e = cols.data() + rcount[(size_t)r + 1];
      std::sort(b, e);
      ulen[(size_t)r] = int(std::unique(b, e) - b);
      return 0;
    }, err);
    if (rc) return rc;
    P.nnz = 0;
    for (int r = 0; r < P.n_unknowns; ++r) P.nnz += ulen[(size_t)r];
    if (P.nnz >= (int64_t)1 << 31) { *err = "pattern too large"; return XG_ERR_ARG; }
    P.rowptr.assign((size_t)P.n_unknowns + 1, 0);
    for (int r = 0; r < P.n_unknowns; ++r) P.rowptr[(size_t)r + 1] = P.rowptr[(size_t)r] + ulen[(size_t)r];
    P.colidx.resize((size_t)P.nnz);
    rc = parallel_rows(P.n_unknowns, 0, [&](int r, double *, std::string *) {
      std::copy_n(cols.data() + rcount[(size_t)r], ulen[(size_t)r], P.colidx.data() + P.rowptr[(size_t)r]);
      return 0;
    }, err);
    if (rc) return rc;
  }

  // Term plan.
  P.n_vec_out = 4 * W;
  P.n_out = P.n_vec_out + 2 * P.nnz;
  int64_t term = 0;
  for (int k = 0; k < P.n_order; ++k) {
    int t = P.order[k];
    TypeData &T = P.T[t];
    if (!T.n) continue;
    T.term0 = term;
    term += (int64_t)T.n * T.nterm;
  }
  P.n_terms = term;
  if (P.n_terms + 1 >= ((int64_t)1 << 32)) { *err = "too many stamp terms"; return XG_ERR_ARG; }

  // Fixed-order reduction lists: a counting sort by output, stable in the
  // reference's (type, instance, statement) order.
  auto slot_of = [&](int r, int c) -> int64_t {
    const int *b = P.colidx.data() + P.rowptr[r];
    const int *e = P.colidx.data() + P.rowptr[r + 1];
    const int *it = std::lower_bound(b, e, c);
    return (int64_t)(it - P.colidx.data());
  };
  // The output of every term (-1: none), instances in parallel; kept per
  // instance in statement order so the counting passes read it in sequence.
  std::vector<int64_t> out_of((size_t)P.n_terms);
  for (int k = 0; k < P.n_order; ++k) {
    const int t = P.order[k];
    const TypeData &T = P.T[t];
    if (!T.n) continue;
    const TypeLayout &L = type_layout(t);
    int rc = parallel_rows(T.n, 0, [&](int i, double *, std::string *) {
      int64_t *o_i = out_of.data() + T.term0 + (int64_t)i * L.nterm;
      for (int q = 0; q < L.nterm; ++q) {
        const TermDef &td = L.terms[q];
        int64_t o = -1;
        const int r = T.lid[(size_t)td.row * T.n + i];
        if (r != gnd) {
          if (td.kind <= OUT_DQDXDVP) {
            o = (int64_t)td.kind * W + r;
          } else {
            const int c = T.lid[(size_t)td.col * T.n + i];
            if (c != gnd) o = P.n_vec_out + (td.kind == OUT_DQDX ? P.nnz : 0) + slot_of(r, c);
          }
        }
        o_i[q] = o;
      }
      return 0;
    }, err);
    if (rc) return rc;
  }
  std::vector<int64_t> &cnt = P.red_ptr;
  cnt.assign((size_t)P.n_out + 1, 0);
  int64_t kept = 0;
  for (int64_t j = 0; j < P.n_terms; ++j)
    if (out_of[(size_t)j] >= 0) {
      cnt[(size_t)out_of[(size_t)j] + 1]++;
      ++kept;
    }
  for (int64_t o = 0; o < P.n_out; ++o) cnt[(size_t)o + 1] += cnt[(size_t)o];
  P.red_idx.resize((size_t)kept);
  {
    // the (type, instance, statement) order of the reference's loads
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int k = 0; k < P.n_order; ++k) {
      const int t = P.order[k];
      const TypeData &T = P.T[t];
      if (!T.n) continue;
      const int nterm = type_layout(t).nterm;
      for (int i = 0; i < T.n; ++i) {
        const int64_t *o_i = out_of.data() + T.term0 + (int64_t)i * nterm;
        for (int q = 0; q < nterm; ++q)
          if (o_i[q] >= 0)
            P.red_idx[(size_t)fill[(size_t)o_i[q]]++] = (uint32_t)(T.term0 + (int64_t)q * T.n + i);
      }
    }
  }
  P.long_out.clear();
  P.short_order.clear();
  for (int64_t o = 0; o < P.n_out; ++o) {
    const int64_t len = P.red_ptr[(size_t)o + 1] - P.red_ptr[(size_t)o];
    if (len > kLongSegment) P.long_out.push_back(o);
    else P.short_order.push_back(o);
  }
  auto mid = std::lower_bound(P.short_order.begin(), P.short_order.end(), P.n_vec_out);
  P.n_short_vec = mid - P.short_order.begin();
  // stable counting sort of each part by term count (0..kLongSegment)
  auto bucket = [&](std::vector<int64_t>::iterator b, std::vector<int64_t>::iterator e) {
    std::vector<int64_t> cnt(kLongSegment + 2, 0), tmp(b, e);
    for (int64_t o : tmp) cnt[(size_t)(P.red_ptr[(size_t)o + 1] - P.red_ptr[(size_t)o]) + 1]++;
    for (size_t k = 1; k < cnt.size(); ++k) cnt[k] += cnt[k - 1];
    for (int64_t o : tmp) *(b + cnt[(size_t)(P.red_ptr[(size_t)o + 1] - P.red_ptr[(size_t)o])]++) = o;
  };
  bucket(P.short_order.begin(), mid);
  bucket(mid, P.short_order.end());
  // the short outputs as ELL buckets, one per run of equal term counts in
  // each part (short_order is grouped that way)
  P.ell.clear();
  P.ell_out.clear();
  P.ell_idx.clear();
  P.n_ell_vec = 0;
  {
    int64_t blocks = 0;
    auto part = [&](int64_t s0, int64_t s1) {
      for (int64_t k = s0; k < s1;) {
        const int64_t o0 = P.short_order[(size_t)k];
        const int32_t c = int32_t(P.red_ptr[(size_t)o0 + 1] - P.red_ptr[(size_t)o0]);
        int64_t e = k + 1;
        while (e < s1) {
          const int64_t o = P.short_order[(size_t)e];
          if (P.red_ptr[(size_t)o + 1] - P.red_ptr[(size_t)o] != c) break;
          ++e;
        }
        const int64_t m = e - k;
        EllBucket b{(int64_t)P.ell_out.size(), (int64_t)P.ell_idx.size(), blocks, int32_t(m), c};
        P.ell.push_back(b);
        for (int64_t q = k; q < e; ++q) P.ell_out.push_back((uint32_t)P.short_order[(size_t)q]);
        for (int32_t j = 0; j < c; ++j)
          for (int64_t q = k; q < e; ++q)
            P.ell_idx.push_back(P.red_idx[(size_t)(P.red_ptr[(size_t)P.short_order[(size_t)q]] + j)]);
        blocks += (m + kEllPerBlock - 1) / kEllPerBlock;
        k = e;
      }
    };
    part(0, P.n_short_vec);
    P.n_ell_vec = (int)P.ell.size();
    part(P.n_short_vec, (int64_t)P.short_order.size());
  }
  return XG_OK;
}

}  // namespace xg
