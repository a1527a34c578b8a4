// bsim3_setup.cpp — BSIM3 v3.2 host setup: model card defaults and
// Model::processParams, the size-dependent parameters and temperature update
// of each instance, and the per-instance parameter block the load kernel
// reads (include/xg_params.h, enum xg_b3_param).
//
// Restates src/DeviceModelPKG/OpenModels/src/N_DEV_MOSFET_B3.C:
//   parameter table and defaults          Traits::loadModelParameters :204-1845
//   Model::Model, Model::processParams    :8603-9105, :8488-8570
//   Instance::Instance, processParams     :1845-1880, :1890-2492
//   Instance::updateTemperature           :3611-4516 (SizeDependParam built
//                                          per instance: the reference's
//                                          (L, W) list cache only avoids
//                                          recomputing identical values)
// Compiled with -ffp-contract=off.

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xg_b3_hoist.h"
#include "xg_bsim3_setup.h"

namespace xg {

namespace {

// ---- constants (src/DeviceModelPKG/Core/include/N_DEV_Const.h) -------------
const double kQ = 1.6021918e-19;
const double kBoltz = 1.3806226e-23;
const double kRefTemp = 300.15;
const double kCtoK = 273.15;
const double kEpsOx = 3.453133e-11;
const double kEpsSi = 1.03594e-10;
const double kNi0 = 1.45e10;
const double kExpThreshold = 34.0;
const double kMinExp = 1.713908431e-15;
inline double KoverQ() { return kBoltz / kQ; }
inline double Vt0() { return kBoltz * (27.0 + kCtoK) / kQ; }  // CONSTvt0

// ---- parameter table --------------------------------------------------------
// Binnable parameters: each has L-, W- and P-prefixed length/width/area
// coefficients (default 0) and is evaluated per instance as
// X + LX*Inv_L + WX*Inv_W + PX*Inv_LW (updateTemperature :3837-4251).
struct Def {
  const char *name;
  double def;
};
const Def kBinnable[] = {
    {"CDSC", 2.4e-4}, {"CDSCB", 0.0}, {"CDSCD", 0.0}, {"CIT", 0.0}, {"NFACTOR", 1.0},
    {"XJ", 0.15e-6}, {"VSAT", 8.0e4}, {"AT", 3.3e4}, {"A0", 1.0}, {"AGS", 0.0}, {"A1", 0.0},
    {"A2", 1.0}, {"KETA", -0.047}, {"NSUB", 6.0e16}, {"NCH", 1.7e17}, {"NGATE", 0.0},
    {"GAMMA1", 0.0}, {"GAMMA2", 0.0}, {"VBX", 0.0}, {"VBM", -3.0}, {"XT", 1.55e-7},
    {"VFB", 0.0}, {"K1", 0.0}, {"KT1", -0.11}, {"KT1L", 0.0}, {"K2", 0.0}, {"KT2", 0.022},
    {"K3", 80.0}, {"K3B", 0.0}, {"W0", 2.5e-6}, {"NLX", 1.74e-7}, {"DVT0", 2.2},
    {"DVT1", 0.53}, {"DVT2", -0.032}, {"DVT0W", 0.0}, {"DVT1W", 5.3e6}, {"DVT2W", -0.032},
    {"DROUT", 0.56}, {"DSUB", 0.0}, {"VTH0", 0.0}, {"UA", 2.25e-9}, {"UA1", 4.31e-9},
    {"UB", 5.87e-19}, {"UB1", -7.61e-18}, {"UC", 0.0}, {"UC1", 0.0}, {"U0", 0.0},
    {"UTE", -1.5}, {"VOFF", -0.08}, {"DELTA", 0.01}, {"RDSW", 0.0}, {"PRWG", 0.0},
    {"PRWB", 0.0}, {"PRT", 0.0}, {"ETA0", 0.08}, {"ETAB", -0.07}, {"PCLM", 1.3},
    {"PDIBLC1", 0.39}, {"PDIBLC2", 0.0086}, {"PDIBLCB", 0.0}, {"PSCBE1", 4.24e8},
    {"PSCBE2", 1.0e-5}, {"PVAG", 0.0}, {"WR", 1.0}, {"DWG", 0.0}, {"DWB", 0.0}, {"B0", 0.0},
    {"B1", 0.0}, {"ALPHA0", 0.0}, {"ALPHA1", 0.0}, {"BETA0", 30.0}, {"ELM", 5.0},
    {"CGSL", 0.0}, {"CGDL", 0.0}, {"CKAPPA", 0.6}, {"CF", 0.0}, {"CLC", 0.1e-6},
    {"CLE", 0.6}, {"VFBCV", -1.0}, {"ACDE", 1.0}, {"MOIN", 15.0}, {"NOFF", 1.0},
    {"VOFFCV", 0.0}};
// Parameters without size dependence.
const Def kPlain[] = {
    {"TOX", 150.e-10}, {"TOXM", 0.0}, {"IJTH", 0.1}, {"TCJ", 0.0}, {"TCJSW", 0.0},
    {"TCJSWG", 0.0}, {"TPB", 0.0}, {"TPBSW", 0.0}, {"TPBSWG", 0.0}, {"TNOM", 0.0},
    {"CGSO", 0.0}, {"CGDO", 0.0}, {"CGBO", 0.0}, {"XPART", 0.0}, {"RSH", 0.0},
    {"JS", 1.e-4}, {"JSW", 0.0}, {"MJ", 0.5}, {"MJSW", 0.33}, {"CJ", 5.e-4},
    {"CJSW", 5.e-10}, {"MJSWG", 0.0}, {"CJSWG", 0.0}, {"NJ", 1.0}, {"XTI", 3.0},
    {"PB", 1.0}, {"PBSW", 1.0}, {"PBSWG", 0.0}, {"LINT", 0.0}, {"LL", 0.0}, {"LLC", 0.0},
    {"LLN", 0.0}, {"LW", 0.0}, {"LWC", 0.0}, {"LWN", 0.0}, {"LWL", 0.0}, {"LWLC", 0.0},
    {"WINT", 0.0}, {"WL", 0.0}, {"WLC", 0.0}, {"WLN", 0.0}, {"WW", 0.0}, {"WWC", 0.0},
    {"WWN", 0.0}, {"WWL", 0.0}, {"WWLC", 0.0}, {"DWC", 0.0}, {"DLC", 0.0}, {"MOBMOD", 1},
    {"BINUNIT", 1}, {"CAPMOD", 3}, {"NOIMOD", 1}, {"L", 5.e-6}, {"W", 5.e-6}, {"LMAX", 1.0},
    {"LMIN", 0.0}, {"WMAX", 1.0}, {"WMIN", 0.0}, {"NOIA", 0.0}, {"NOIB", 0.0},
    {"NOIC", 0.0}, {"EM", 4.1e7}, {"EF", 1.0}, {"AF", 1.0}, {"KF", 0.0},
    {"PARAMCHK", 0}, {"USEFRINGE", 0}, {"LEVEL", 9}, {"VERSION", 3.2}};

std::string up(const char *s) {
  std::string r(s);
  for (auto &c : r) c = (char)std::toupper((unsigned char)c);
  return r;
}

// Stamp terms in the statement order of Master::loadDAEVectors
// (:9306-9653) and the pointer-path Master::loadDAEMatrices (:9654-9939),
// nqsMod = 0, no initial conditions.  LID slots: 0 d, 1 g, 2 s, 3 b, 4 d', 5 s'.
const TermDef kB3Terms[] = {
    {OUT_F, 0, 0}, {OUT_F, 2, 0}, {OUT_F, 3, 0}, {OUT_F, 4, 0}, {OUT_F, 5, 0},
    {OUT_DFDXDVP, 3, 0}, {OUT_DFDXDVP, 4, 0}, {OUT_DFDXDVP, 5, 0},
    {OUT_Q, 1, 0}, {OUT_Q, 3, 0}, {OUT_Q, 4, 0}, {OUT_Q, 5, 0},
    {OUT_DQDXDVP, 1, 0}, {OUT_DQDXDVP, 3, 0}, {OUT_DQDXDVP, 4, 0}, {OUT_DQDXDVP, 5, 0},
    {OUT_DFDX, 0, 0}, {OUT_DFDX, 0, 4}, {OUT_DFDX, 2, 2}, {OUT_DFDX, 2, 5},
    {OUT_DFDX, 3, 1}, {OUT_DFDX, 3, 3}, {OUT_DFDX, 3, 4}, {OUT_DFDX, 3, 5},
    {OUT_DFDX, 4, 0}, {OUT_DFDX, 4, 3}, {OUT_DFDX, 4, 1}, {OUT_DFDX, 4, 4}, {OUT_DFDX, 4, 5},
    {OUT_DFDX, 5, 1}, {OUT_DFDX, 5, 3}, {OUT_DFDX, 5, 2}, {OUT_DFDX, 5, 4}, {OUT_DFDX, 5, 5},
    {OUT_DQDX, 1, 1}, {OUT_DQDX, 1, 3}, {OUT_DQDX, 1, 4}, {OUT_DQDX, 1, 5},
    {OUT_DQDX, 3, 1}, {OUT_DQDX, 3, 3}, {OUT_DQDX, 3, 4}, {OUT_DQDX, 3, 5},
    {OUT_DQDX, 4, 3}, {OUT_DQDX, 4, 1}, {OUT_DQDX, 4, 4}, {OUT_DQDX, 4, 5},
    {OUT_DQDX, 5, 1}, {OUT_DQDX, 5, 3}, {OUT_DQDX, 5, 4}, {OUT_DQDX, 5, 5}};

}  // namespace

int b3_nlid() { return 6; }
int b3_nterm() { return int(sizeof(kB3Terms) / sizeof(kB3Terms[0])); }
const TermDef *b3_terms() { return kB3Terms; }

int b3_make_model(const xg_model_desc &md, const xg_device_options &opt, B3Model *m,
                  std::string *err) {
  B3Model &M = *m;
  M.dtype = md.polarity < 0 ? -1 : 1;
  for (const Def &d : kBinnable) {
    M.v[d.name] = d.def;
    const std::string n(d.name);
    M.v["L" + n] = 0.0;
    M.v["W" + n] = 0.0;
    M.v["P" + n] = 0.0;
  }
  for (const Def &d : kPlain) M.v[d.name] = d.def;
  for (int i = 0; i < md.n_params; ++i) {
    std::string k = up(md.names[i]);
    if (!M.v.count(k)) {
      *err = "BSIM3: unsupported model parameter " + k;
      return XG_ERR_UNSUPPORTED;
    }
    M.v[k] = md.values[i];
    M.given[k] = true;
  }
  if (M.g("LEVEL") && M["LEVEL"] != 9 && M["LEVEL"] != 49) {
    *err = "BSIM3: LEVEL must be 9 or 49";
    return XG_ERR_UNSUPPORTED;
  }
  const int mobMod = (int)M["MOBMOD"], capMod = (int)M["CAPMOD"];
  if (mobMod < 1 || mobMod > 3 || capMod < 0 || capMod > 3) {
    *err = "BSIM3: MOBMOD must be 1..3 and CAPMOD 0..3";
    return XG_ERR_UNSUPPORTED;
  }
  // Model::Model (:9064-9102)
  M.tnom = M.g("TNOM") ? M["TNOM"] + kCtoK : opt.tnom;
  if (!M.g("VTH0")) M.v["VTH0"] = (M.dtype == 1) ? 0.7 : -0.7;
  if (!M.g("UC")) M.v["UC"] = (mobMod == 3) ? -0.0465 : -0.0465e-9;
  if (!M.g("UC1")) M.v["UC1"] = (mobMod == 3) ? -0.056 : -0.056e-9;
  if (!M.g("U0")) M.v["U0"] = (M.dtype == 1) ? 0.067 : 0.025;

  // Model::processParams (:8488-8570)
  auto &v = M.v;
  const double tox = v["TOX"];
  M.cox = 3.453133e-11 / tox;
  if (!M.g("TOXM")) v["TOXM"] = tox;
  if (!M.g("DSUB")) v["DSUB"] = v["DROUT"];
  if (!M.g("LLC")) v["LLC"] = v["LL"];
  if (!M.g("LWC")) v["LWC"] = v["LW"];
  if (!M.g("LWLC")) v["LWLC"] = v["LWL"];
  if (!M.g("WLC")) v["WLC"] = v["WL"];
  if (!M.g("WWL")) v["WWLC"] = v["WWL"];
  if (!M.g("WWLC")) v["WWLC"] = v["WWL"];
  if (!M.g("DWC")) v["DWC"] = v["WINT"];
  if (!M.g("DLC")) v["DLC"] = v["LINT"];
  if (!M.g("CF")) {
    double C1 = 2.0 * kEpsOx;
    double C5 = M_PI;
    double C2 = 1.0 + (0.4e-6 / tox);
    double C3 = std::log(C2);
    v["CF"] = C1 * C3 / C5;
  }
  if (!M.g("CGDO")) {
    if (M.g("DLC") && (v["DLC"] > 0.0)) v["CGDO"] = v["DLC"] * M.cox - v["CGDL"];
    else v["CGDO"] = 0.6 * v["XJ"] * M.cox;
  }
  if (!M.g("CGSO")) {
    if (M.g("DLC") && (v["DLC"] > 0.0)) v["CGSO"] = v["DLC"] * M.cox - v["CGSL"];
    else v["CGSO"] = 0.6 * v["XJ"] * M.cox;
  }
  if (!M.g("CGBO")) v["CGBO"] = 2.0 * v["DWC"] * M.cox;
  if (!M.g("CJSWG")) v["CJSWG"] = v["CJSW"];
  if (!M.g("PBSWG")) v["PBSWG"] = v["PBSW"];
  if (!M.g("MJSWG")) v["MJSWG"] = v["MJSW"];
  if (v["PB"] < 0.1) v["PB"] = 0.1;
  if (v["PBSW"] < 0.1) v["PBSW"] = 0.1;
  if (v["PBSWG"] < 0.1) v["PBSWG"] = 0.1;
  M.vcrit = Vt0() * std::log(Vt0() / (std::sqrt(2.0) * 1.0e-14));
  M.factor1 = std::sqrt(kEpsSi / kEpsOx * tox);
  const double tnom = M.tnom;
  M.Vtm0 = KoverQ() * tnom;
  M.Eg0 = 1.16 - 7.02e-4 * tnom * tnom / (tnom + 1108.0);
  M.ni = kNi0 * (tnom / kRefTemp) * std::sqrt(tnom / kRefTemp) *
         std::exp(21.5565981 - M.Eg0 / (2.0 * M.Vtm0));
  return XG_OK;
}

int b3_instance_params(const B3Model &M, const xg_mos_desc &d, int i,
                       const xg_device_options &opt, double *out, std::string *err) {
  const auto &v = M.v;
  auto V = [&](const char *k) { return v.at(k); };
  std::memset(out, 0, sizeof(double) * XG_B3_NPARAMS);
  // Instance::Instance (:2471-2492) and processParams (:1845-1880)
  const double temp = opt.temp;
  const double l = d.l ? d.l[i] : V("L");
  const double w = d.w ? d.w[i] : V("W");
  const double drainArea = d.ad ? d.ad[i] : 0.0;
  const double sourceArea = d.as ? d.as[i] : 0.0;
  const double drainPerimeter = d.pd ? d.pd[i] : 0.0;
  const double sourcePerimeter = d.ps ? d.ps[i] : 0.0;
  const double drainSquares = d.nrd ? d.nrd[i] : 1.0;
  const double sourceSquares = d.nrs ? d.nrs[i] : 1.0;
  const double numberParallel = d.m ? d.m[i] : 1.0;
  double drainConductance = V("RSH") * drainSquares;
  drainConductance = drainConductance > 0.0 ? 1.0 / drainConductance : 0.0;
  double sourceConductance = V("RSH") * sourceSquares;
  sourceConductance = sourceConductance > 0.0 ? 1.0 / sourceConductance : 0.0;

  // updateTemperature (:3639-3727)
  const double Tnom = M.tnom;
  const double TRatio = temp / Tnom;
  const double vtm = KoverQ() * temp;
  const double Eg = 1.16 - 7.02e-4 * temp * temp / (temp + 1108.0);
  double jctTempSatCurDensity, jctSidewallTempSatCurDensity;
  if (temp != Tnom) {
    double T0 = M.Eg0 / M.Vtm0 - Eg / vtm + V("XTI") * std::log(temp / Tnom);
    double T1 = std::exp(T0 / V("NJ"));
    jctTempSatCurDensity = V("JS") * T1;
    jctSidewallTempSatCurDensity = V("JSW") * T1;
  } else {
    jctTempSatCurDensity = V("JS");
    jctSidewallTempSatCurDensity = V("JSW");
  }
  if (jctTempSatCurDensity < 0.0) jctTempSatCurDensity = 0.0;
  if (jctSidewallTempSatCurDensity < 0.0) jctSidewallTempSatCurDensity = 0.0;
  const double delTemp = temp - Tnom;
  double unitAreaJctCapTemp = 0.0, unitLengthSidewallJctCapTemp = 0.0,
         unitLengthGateSidewallJctCapTemp = 0.0;
  double T0 = V("TCJ") * delTemp;
  if (T0 >= -1.0) unitAreaJctCapTemp = V("CJ") * (1.0 + T0);
  T0 = V("TCJSW") * delTemp;
  if (T0 >= -1.0) unitLengthSidewallJctCapTemp = V("CJSW") * (1.0 + T0);
  T0 = V("TCJSWG") * delTemp;
  if (T0 >= -1.0) unitLengthGateSidewallJctCapTemp = V("CJSWG") * (1.0 + T0);
  double PhiBTemp = V("PB") - V("TPB") * delTemp;
  if (PhiBTemp < 0.01) PhiBTemp = 0.01;
  double PhiBSWTemp = V("PBSW") - V("TPBSW") * delTemp;
  if (PhiBSWTemp <= 0.01) PhiBSWTemp = 0.01;
  double PhiBSWGTemp = V("PBSWG") - V("TPBSWG") * delTemp;
  if (PhiBSWGTemp <= 0.01) PhiBSWGTemp = 0.01;

  // SizeDependParam (:3757-4470)
  const double Ldrn = l, Wdrn = w;
  T0 = std::pow(Ldrn, V("LLN"));
  double T1 = std::pow(Wdrn, V("LWN"));
  double tmp1 = V("LL") / T0 + V("LW") / T1 + V("LWL") / (T0 * T1);
  const double dl = V("LINT") + tmp1;
  double tmp2 = V("LLC") / T0 + V("LWC") / T1 + V("LWLC") / (T0 * T1);
  const double dlc = V("DLC") + tmp2;
  double T2 = std::pow(Ldrn, V("WLN"));
  double T3 = std::pow(Wdrn, V("WWN"));
  tmp1 = V("WL") / T2 + V("WW") / T3 + V("WWL") / (T2 * T3);
  const double dw = V("WINT") + tmp1;
  tmp2 = V("WLC") / T2 + V("WWC") / T3 + V("WWLC") / (T2 * T3);
  const double dwc = V("DWC") + tmp2;
  const double leff = l - 2.0 * dl;
  const double weff = w - 2.0 * dw;
  const double leffCV = l - 2.0 * dlc;
  const double weffCV = w - 2.0 * dwc;
  if (leff <= 0.0 || weff <= 0.0 || leffCV <= 0.0 || weffCV <= 0.0) {
    *err = "BSIM3: effective channel length or width <= 0";
    return XG_ERR_ARG;
  }
  double Inv_L, Inv_W, Inv_LW;
  if (V("BINUNIT") == 1) {
    Inv_L = 1.0e-6 / leff;
    Inv_W = 1.0e-6 / weff;
    Inv_LW = 1.0e-12 / (leff * weff);
  } else {
    Inv_L = 1.0 / leff;
    Inv_W = 1.0 / weff;
    Inv_LW = 1.0 / (leff * weff);
  }
  auto bin = [&](const char *k) {
    const std::string n(k);
    return v.at(n) + v.at("L" + n) * Inv_L + v.at("W" + n) * Inv_W + v.at("P" + n) * Inv_LW;
  };
  double cdsc = bin("CDSC"), cdscb = bin("CDSCB"), cdscd = bin("CDSCD"), cit = bin("CIT");
  double nfactor = bin("NFACTOR"), xj = bin("XJ"), vsat = bin("VSAT"), at = bin("AT");
  double a0 = bin("A0"), ags = bin("AGS"), a1 = bin("A1"), a2 = bin("A2"), keta = bin("KETA");
  double nsub = bin("NSUB"), npeak = bin("NCH"), ngate = bin("NGATE");
  double gamma1 = bin("GAMMA1"), gamma2 = bin("GAMMA2"), vbx = bin("VBX"), vbm = bin("VBM");
  double xt = bin("XT"), vfb = bin("VFB"), k1 = bin("K1"), kt1 = bin("KT1"), kt1l = bin("KT1L");
  double k2 = bin("K2"), kt2 = bin("KT2"), k3 = bin("K3"), k3b = bin("K3B"), w0 = bin("W0");
  double nlx = bin("NLX"), dvt0 = bin("DVT0"), dvt1 = bin("DVT1"), dvt2 = bin("DVT2");
  double dvt0w = bin("DVT0W"), dvt1w = bin("DVT1W"), dvt2w = bin("DVT2W");
  double drout = bin("DROUT"), dsub = bin("DSUB"), vth0 = bin("VTH0");
  double ua = bin("UA"), ua1 = bin("UA1"), ub = bin("UB"), ub1 = bin("UB1");
  double uc = bin("UC"), uc1 = bin("UC1"), u0 = bin("U0"), ute = bin("UTE");
  double voff = bin("VOFF"), delta = bin("DELTA"), rdsw = bin("RDSW"), prwg = bin("PRWG");
  double prwb = bin("PRWB"), prt = bin("PRT"), eta0 = bin("ETA0"), etab = bin("ETAB");
  double pclm = bin("PCLM"), pdibl1 = bin("PDIBLC1"), pdibl2 = bin("PDIBLC2");
  double pdiblb = bin("PDIBLCB"), pscbe1 = bin("PSCBE1"), pscbe2 = bin("PSCBE2");
  double pvag = bin("PVAG"), wr = bin("WR"), dwg = bin("DWG"), dwb = bin("DWB");
  double b0 = bin("B0"), b1 = bin("B1"), alpha0 = bin("ALPHA0"), alpha1 = bin("ALPHA1");
  double beta0 = bin("BETA0"), elm = bin("ELM"), cgsl = bin("CGSL"), cgdl = bin("CGDL");
  double ckappa = bin("CKAPPA"), cf = bin("CF"), clc = bin("CLC"), cle = bin("CLE");
  double vfbcv = bin("VFBCV"), acde = bin("ACDE"), moin = bin("MOIN"), noff = bin("NOFF");
  double voffcv = bin("VOFFCV");
  (void)elm;
  const double abulkCVfactor = 1.0 + std::pow((clc / leffCV), cle);
  T0 = (TRatio - 1.0);
  ua = ua + ua1 * T0;
  ub = ub + ub1 * T0;
  uc = uc + uc1 * T0;
  if (u0 > 1.0) u0 = u0 / 1.0e4;
  const double u0temp = u0 * std::pow(TRatio, ute);
  const double vsattemp = vsat - at * T0;
  const double rds0 = (rdsw + prt * T0) / std::pow(weff * 1E6, wr);
  const double tox = V("TOX"), cox = M.cox;
  const double p_cgdo = (V("CGDO") + cf) * weffCV;
  const double p_cgso = (V("CGSO") + cf) * weffCV;
  const double p_cgbo = V("CGBO") * leffCV;
  if (!M.g("NCH") && M.g("GAMMA1")) {
    T0 = gamma1 * cox;
    npeak = 3.021E22 * T0 * T0;
  }
  const double Vtm0 = M.Vtm0, ni = M.ni;
  const double phi = 2.0 * Vtm0 * std::log(npeak / ni);
  const double sqrtPhi = std::sqrt(phi);
  const double phis3 = sqrtPhi * phi;
  const double Xdep0 = std::sqrt(2.0 * kEpsSi / (kQ * npeak * 1.0e6)) * sqrtPhi;
  const double litl = std::sqrt(3.0 * xj * tox);
  const double vbi = Vtm0 * std::log(1.0e20 * npeak / (ni * ni));
  const double cdep0 = std::sqrt(kQ * kEpsSi * npeak * 1.0e6 / 2.0 / phi);
  const double ldeb = std::sqrt(kEpsSi * Vtm0 / (kQ * npeak * 1.0e6)) / 3.0;
  acde *= std::pow((npeak / 2.0e16), -0.25);
  if (M.g("K1") || M.g("K2")) {
    if (!M.g("K1")) k1 = 0.53;
    if (!M.g("K2")) k2 = -0.0186;
  } else {
    if (!M.g("VBX")) vbx = phi - 7.7348e-4 * npeak * xt * xt;
    if (vbx > 0.0) vbx = -vbx;
    if (vbm > 0.0) vbm = -vbm;
    if (!M.g("GAMMA1")) gamma1 = 5.753e-12 * std::sqrt(npeak) / cox;
    if (!M.g("GAMMA2")) gamma2 = 5.753e-12 * std::sqrt(nsub) / cox;
    T0 = gamma1 - gamma2;
    T1 = std::sqrt(phi - vbx) - sqrtPhi;
    T2 = std::sqrt(phi * (phi - vbm)) - phi;
    k2 = T0 * T1 / (2.0 * T2 + vbm);
    k1 = gamma2 - 2.0 * k2 * std::sqrt(phi - vbm);
  }
  double vbsc;
  if (k2 < 0.0) {
    T0 = 0.5 * k1 / k2;
    vbsc = 0.9 * (phi - T0 * T0);
    if (vbsc > -3.0) vbsc = -3.0;
    else if (vbsc < -30.0) vbsc = -30.0;
  } else {
    vbsc = -30.0;
  }
  if (vbsc > vbm) vbsc = vbm;
  const int dtype = M.dtype;
  if (!M.g("VFB")) {
    if (M.g("VTH0")) vfb = dtype * vth0 - phi - k1 * sqrtPhi;
    else vfb = -1.0;
  }
  if (!M.g("VTH0")) vth0 = dtype * (vfb + phi + k1 * sqrtPhi);
  const double toxm = V("TOXM");
  const double k1ox = k1 * tox / toxm;
  const double k2ox = k2 * tox / toxm;
  T1 = std::sqrt(kEpsSi / kEpsOx * tox * Xdep0);
  T0 = std::exp(-0.5 * dsub * leff / T1);
  const double theta0vb0 = (T0 + 2.0 * T0 * T0);
  T0 = std::exp(-0.5 * drout * leff / T1);
  T2 = (T0 + 2.0 * T0 * T0);
  const double thetaRout = pdibl1 * T2 + pdibl2;
  double tmp = std::sqrt(Xdep0);
  tmp1 = vbi - phi;
  tmp2 = M.factor1 * tmp;
  T0 = -0.5 * dvt1w * weff * leff / tmp2;
  if (T0 > -kExpThreshold) {
    T1 = std::exp(T0);
    T2 = T1 * (1.0 + 2.0 * T1);
  } else {
    T1 = kMinExp;
    T2 = T1 * (1.0 + 2.0 * T1);
  }
  T0 = dvt0w * T2;
  T2 = T0 * tmp1;
  T0 = -0.5 * dvt1 * leff / tmp2;
  if (T0 > -kExpThreshold) {
    T1 = std::exp(T0);
    T3 = T1 * (1.0 + 2.0 * T1);
  } else {
    T1 = kMinExp;
    T3 = T1 * (1.0 + 2.0 * T1);
  }
  T3 = dvt0 * T3 * tmp1;
  double T4 = tox * phi / (weff + w0);
  T0 = std::sqrt(1.0 + nlx / leff);
  double T5 = k1ox * (T0 - 1.0) * sqrtPhi + (kt1 + kt1l / leff) * (TRatio - 1.0);
  double tmp3 = dtype * vth0 - T2 - T3 + k3 * T4 + T5;
  const double vfbzb = tmp3 - phi - k1 * sqrtPhi;

  // Junction saturation currents (:4475-4511)
  const double Nvtm = vtm * V("NJ");
  const double ijth = V("IJTH");
  double SourceSatCurrent, DrainSatCurrent, vjsm = 0.0, IsEvjsm = 0.0, vjdm = 0.0, IsEvjdm = 0.0;
  if ((sourceArea <= 0.0) && (sourcePerimeter <= 0.0)) SourceSatCurrent = 1.0e-14;
  else SourceSatCurrent = sourceArea * jctTempSatCurDensity + sourcePerimeter * jctSidewallTempSatCurDensity;
  if ((SourceSatCurrent > 0.0) && (ijth > 0.0)) {
    vjsm = Nvtm * std::log(ijth / SourceSatCurrent + 1.0);
    IsEvjsm = SourceSatCurrent * std::exp(vjsm / Nvtm);
  }
  if ((drainArea <= 0.0) && (drainPerimeter <= 0.0)) DrainSatCurrent = 1.0e-14;
  else DrainSatCurrent = drainArea * jctTempSatCurDensity + drainPerimeter * jctSidewallTempSatCurDensity;
  if ((DrainSatCurrent > 0.0) && (ijth > 0.0)) {
    vjdm = Nvtm * std::log(ijth / DrainSatCurrent + 1.0);
    IsEvjdm = DrainSatCurrent * std::exp(vjdm / Nvtm);
  }

  // Junction capacitances per instance (updateIntermediateVars :6983-7007)
  const double czbd = unitAreaJctCapTemp * drainArea;
  const double czbs = unitAreaJctCapTemp * sourceArea;
  double czbdsw, czbdswg, czbssw, czbsswg;
  if (drainPerimeter < weff) {
    czbdswg = unitLengthGateSidewallJctCapTemp * drainPerimeter;
    czbdsw = 0.0;
  } else {
    czbdsw = unitLengthSidewallJctCapTemp * (drainPerimeter - weff);
    czbdswg = unitLengthGateSidewallJctCapTemp * weff;
  }
  if (sourcePerimeter < weff) {
    czbssw = 0.0;
    czbsswg = unitLengthGateSidewallJctCapTemp * sourcePerimeter;
  } else {
    czbssw = unitLengthSidewallJctCapTemp * (sourcePerimeter - weff);
    czbsswg = unitLengthGateSidewallJctCapTemp * weff;
  }

  double *o = out;
  o[XG_B3_DTYPE] = dtype;
  o[XG_B3_MOBMOD] = V("MOBMOD");
  o[XG_B3_CAPMOD] = V("CAPMOD");
  o[XG_B3_XPART] = V("XPART");
  o[XG_B3_TOX] = tox;
  o[XG_B3_COX] = cox;
  o[XG_B3_FACTOR1] = M.factor1;
  o[XG_B3_VCRIT] = M.vcrit;
  o[XG_B3_NJ] = V("NJ");
  o[XG_B3_IJTH] = ijth;
  o[XG_B3_MJ] = V("MJ");
  o[XG_B3_MJSW] = V("MJSW");
  o[XG_B3_MJSWG] = V("MJSWG");
  o[XG_B3_TNOM] = Tnom;
  o[XG_B3_TEMP] = temp;
  o[XG_B3_VTM] = vtm;
  o[XG_B3_JSTEMP] = jctTempSatCurDensity;
  o[XG_B3_JSWTEMP] = jctSidewallTempSatCurDensity;
  o[XG_B3_CJTEMP] = unitAreaJctCapTemp;
  o[XG_B3_CJSWTEMP] = unitLengthSidewallJctCapTemp;
  o[XG_B3_CJSWGTEMP] = unitLengthGateSidewallJctCapTemp;
  o[XG_B3_PHIB] = PhiBTemp;
  o[XG_B3_PHIBSW] = PhiBSWTemp;
  o[XG_B3_PHIBSWG] = PhiBSWGTemp;
  o[XG_B3_VJSM] = vjsm;
  o[XG_B3_ISEVJSM] = IsEvjsm;
  o[XG_B3_VJDM] = vjdm;
  o[XG_B3_ISEVJDM] = IsEvjdm;
  o[XG_B3_AD] = drainArea;
  o[XG_B3_AS] = sourceArea;
  o[XG_B3_PD] = drainPerimeter;
  o[XG_B3_PS] = sourcePerimeter;
  o[XG_B3_GD] = drainConductance;
  o[XG_B3_GS] = sourceConductance;
  o[XG_B3_M] = numberParallel;
  o[XG_B3_FLAGS] = 0.0;
  o[XG_B3_VTH0] = vth0;
  o[XG_B3_VBSC] = vbsc;
  o[XG_B3_PHI] = phi;
  o[XG_B3_PHIS3] = phis3;
  o[XG_B3_SQRTPHI] = sqrtPhi;
  o[XG_B3_XDEP0] = Xdep0;
  o[XG_B3_LEFF] = leff;
  o[XG_B3_WEFF] = weff;
  o[XG_B3_VBI] = vbi;
  o[XG_B3_DVT0] = dvt0;
  o[XG_B3_DVT1] = dvt1;
  o[XG_B3_DVT2] = dvt2;
  o[XG_B3_DVT0W] = dvt0w;
  o[XG_B3_DVT1W] = dvt1w;
  o[XG_B3_DVT2W] = dvt2w;
  o[XG_B3_NLX] = nlx;
  o[XG_B3_K1] = k1;
  o[XG_B3_K1OX] = k1ox;
  o[XG_B3_K2OX] = k2ox;
  o[XG_B3_K3] = k3;
  o[XG_B3_K3B] = k3b;
  o[XG_B3_KT1] = kt1;
  o[XG_B3_KT1L] = kt1l;
  o[XG_B3_KT2] = kt2;
  o[XG_B3_W0] = w0;
  o[XG_B3_ETA0] = eta0;
  o[XG_B3_ETAB] = etab;
  o[XG_B3_THETA0VB0] = theta0vb0;
  o[XG_B3_NFACTOR] = nfactor;
  o[XG_B3_CDSC] = cdsc;
  o[XG_B3_CDSCB] = cdscb;
  o[XG_B3_CDSCD] = cdscd;
  o[XG_B3_CIT] = cit;
  o[XG_B3_VFB] = vfb;
  o[XG_B3_NGATE] = ngate;
  o[XG_B3_VOFF] = voff;
  o[XG_B3_CDEP0] = cdep0;
  o[XG_B3_DWG] = dwg;
  o[XG_B3_DWB] = dwb;
  o[XG_B3_PRWG] = prwg;
  o[XG_B3_PRWB] = prwb;
  o[XG_B3_RDS0] = rds0;
  o[XG_B3_XJ] = xj;
  o[XG_B3_A0] = a0;
  o[XG_B3_B0] = b0;
  o[XG_B3_B1] = b1;
  o[XG_B3_AGS] = ags;
  o[XG_B3_KETA] = keta;
  o[XG_B3_UA] = ua;
  o[XG_B3_UB] = ub;
  o[XG_B3_UC] = uc;
  o[XG_B3_U0TEMP] = u0temp;
  o[XG_B3_VSATTEMP] = vsattemp;
  o[XG_B3_A1] = a1;
  o[XG_B3_A2] = a2;
  o[XG_B3_DELTA] = delta;
  o[XG_B3_PCLM] = pclm;
  o[XG_B3_LITL] = litl;
  o[XG_B3_THETAROUT] = thetaRout;
  o[XG_B3_PDIBLB] = pdiblb;
  o[XG_B3_PVAG] = pvag;
  o[XG_B3_PSCBE1] = pscbe1;
  o[XG_B3_PSCBE2] = pscbe2;
  o[XG_B3_ALPHA0] = alpha0;
  o[XG_B3_ALPHA1] = alpha1;
  o[XG_B3_BETA0] = beta0;
  o[XG_B3_VFBCV] = vfbcv;
  o[XG_B3_WEFFCV] = weffCV;
  o[XG_B3_LEFFCV] = leffCV;
  o[XG_B3_ABULKCVFACTOR] = abulkCVfactor;
  o[XG_B3_NOFF] = noff;
  o[XG_B3_VOFFCV] = voffcv;
  o[XG_B3_VFBZB] = vfbzb;
  o[XG_B3_ACDE] = acde;
  o[XG_B3_LDEB] = ldeb;
  o[XG_B3_MOIN] = moin;
  o[XG_B3_CGDO] = p_cgdo;
  o[XG_B3_CGSO] = p_cgso;
  o[XG_B3_CGBO] = p_cgbo;
  o[XG_B3_CKAPPA] = ckappa;
  o[XG_B3_CGDL] = cgdl;
  o[XG_B3_CGSL] = cgsl;
  o[XG_B3_SSAT] = SourceSatCurrent;
  o[XG_B3_DSAT] = DrainSatCurrent;
  o[XG_B3_NVTM] = Nvtm;
  o[XG_B3_CZBD] = czbd;
  o[XG_B3_CZBS] = czbs;
  o[XG_B3_CZBDSW] = czbdsw;
  o[XG_B3_CZBDSWG] = czbdswg;
  o[XG_B3_CZBSSW] = czbssw;
  o[XG_B3_CZBSSWG] = czbsswg;
  xg_b3_hoist(o);
  return XG_OK;
}

// Instance::registerLIDs (:2840-2856): d' then s' when RSH makes them
// internal nodes.
void b3_assign_lids(const double *params, int n, int i, const int *ext, int *next, int *lids) {
  lids[0] = ext[0];
  lids[1] = ext[1];
  lids[2] = ext[2];
  lids[3] = ext[3];
  lids[4] = params[(size_t)XG_B3_GD * n + i] != 0.0 ? (*next)++ : ext[0];
  lids[5] = params[(size_t)XG_B3_GS * n + i] != 0.0 ? (*next)++ : ext[2];
}

}  // namespace xg
