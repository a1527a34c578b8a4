/*
 * xgo_b3setup.c — the oracle's BSIM3 v3.2 set-up (TEST INFRASTRUCTURE ONLY;
 * see xgo.h): model cards and the per-instance parameter block of
 * include/xg_params.h (enum xg_b3_param), computed on the CPU.
 *
 * Restates src/DeviceModelPKG/OpenModels/src/N_DEV_MOSFET_B3.C:
 *   parameter table and defaults        Traits::loadModelParameters :204-1845
 *   Model::Model, Model::processParams  :9064-9102, :8488-8570
 *   Instance ctor and processParams     :2471-2492, :1845-1880
 *   Instance::updateTemperature         :3611-4516 (the size-dependent
 *                                       parameters of each instance; the
 *                                       reference's (L, W) cache only avoids
 *                                       recomputing identical values)
 *   junction capacitances of updateIntermediateVars :6983-7007 (the hoisted
 *                                       columns after XG_B3_NRAW)
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xg_b3_hoist.h"
#include "xgo_internal.h"

#define K_Q 1.6021918e-19
#define K_BOLTZ 1.3806226e-23
#define K_REFTEMP 300.15
#define K_CTOK 273.15
#define K_EPSOX 3.453133e-11
#define K_EPSSI 1.03594e-10
#define K_NI0 1.45e10
#define EXP_THRESHOLD 34.0
#define MIN_EXP 1.713908431e-15
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Binnable parameters: value X + LX/Leff + WX/Weff + PX/(Leff Weff). */
enum {
  B_CDSC, B_CDSCB, B_CDSCD, B_CIT, B_NFACTOR, B_XJ, B_VSAT, B_AT, B_A0, B_AGS, B_A1, B_A2,
  B_KETA, B_NSUB, B_NCH, B_NGATE, B_GAMMA1, B_GAMMA2, B_VBX, B_VBM, B_XT, B_VFB, B_K1, B_KT1,
  B_KT1L, B_K2, B_KT2, B_K3, B_K3B, B_W0, B_NLX, B_DVT0, B_DVT1, B_DVT2, B_DVT0W, B_DVT1W,
  B_DVT2W, B_DROUT, B_DSUB, B_VTH0, B_UA, B_UA1, B_UB, B_UB1, B_UC, B_UC1, B_U0, B_UTE, B_VOFF,
  B_DELTA, B_RDSW, B_PRWG, B_PRWB, B_PRT, B_ETA0, B_ETAB, B_PCLM, B_PDIBLC1, B_PDIBLC2,
  B_PDIBLCB, B_PSCBE1, B_PSCBE2, B_PVAG, B_WR, B_DWG, B_DWB, B_B0, B_B1, B_ALPHA0, B_ALPHA1,
  B_BETA0, B_ELM, B_CGSL, B_CGDL, B_CKAPPA, B_CF, B_CLC, B_CLE, B_VFBCV, B_ACDE, B_MOIN, B_NOFF,
  B_VOFFCV, B_N
};
static const struct { const char *name; double def; } kBin[B_N] = {
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

/* Parameters without size dependence. */
enum {
  Q_TOX, Q_TOXM, Q_IJTH, Q_TCJ, Q_TCJSW, Q_TCJSWG, Q_TPB, Q_TPBSW, Q_TPBSWG, Q_TNOM, Q_CGSO,
  Q_CGDO, Q_CGBO, Q_XPART, Q_RSH, Q_JS, Q_JSW, Q_MJ, Q_MJSW, Q_CJ, Q_CJSW, Q_MJSWG, Q_CJSWG,
  Q_NJ, Q_XTI, Q_PB, Q_PBSW, Q_PBSWG, Q_LINT, Q_LL, Q_LLC, Q_LLN, Q_LW, Q_LWC, Q_LWN, Q_LWL,
  Q_LWLC, Q_WINT, Q_WL, Q_WLC, Q_WLN, Q_WW, Q_WWC, Q_WWN, Q_WWL, Q_WWLC, Q_DWC, Q_DLC,
  Q_MOBMOD, Q_BINUNIT, Q_CAPMOD, Q_NOIMOD, Q_L, Q_W, Q_LMAX, Q_LMIN, Q_WMAX, Q_WMIN, Q_NOIA,
  Q_NOIB, Q_NOIC, Q_EM, Q_EF, Q_AF, Q_KF, Q_PARAMCHK, Q_USEFRINGE, Q_LEVEL, Q_VERSION, Q_N
};
static const struct { const char *name; double def; } kPlain[Q_N] = {
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

typedef struct {
  int dtype;
  double bin[B_N][4];          /* X, LX, WX, PX */
  unsigned char bin_given[B_N];
  double q[Q_N];
  unsigned char q_given[Q_N];
  double cox, vcrit, factor1, Vtm0, Eg0, ni, tnom;
} b3card_t;

/* Card entry `name` into the model; 0, or -1 when the name is unknown. */
static int b3_put(b3card_t *M, const char *name, double v) {
  for (int k = 0; k < B_N; ++k)
    if (xgo_card_eq(name, kBin[k].name)) {
      M->bin[k][0] = v;
      M->bin_given[k] = 1;
      return 0;
    }
  for (int k = 0; k < Q_N; ++k)
    if (xgo_card_eq(name, kPlain[k].name)) {
      M->q[k] = v;
      M->q_given[k] = 1;
      return 0;
    }
  const char c = name[0];
  const int col = (c == 'L' || c == 'l') ? 1 : (c == 'W' || c == 'w') ? 2 : (c == 'P' || c == 'p') ? 3 : 0;
  if (col)
    for (int k = 0; k < B_N; ++k)
      if (xgo_card_eq(name + 1, kBin[k].name)) {
        M->bin[k][col] = v;
        return 0;
      }
  return -1;
}

static int b3_card(const xg_model_desc *md, const xg_device_options *opt, b3card_t *M) {
  memset(M, 0, sizeof *M);
  M->dtype = md->polarity < 0 ? -1 : 1;
  for (int k = 0; k < B_N; ++k) M->bin[k][0] = kBin[k].def;
  for (int k = 0; k < Q_N; ++k) M->q[k] = kPlain[k].def;
  for (int i = 0; i < md->n_params; ++i)
    if (b3_put(M, md->names[i], md->values[i])) return XG_ERR_UNSUPPORTED;
  if (M->q_given[Q_LEVEL] && M->q[Q_LEVEL] != 9 && M->q[Q_LEVEL] != 49) return XG_ERR_UNSUPPORTED;
  const int mobMod = (int)M->q[Q_MOBMOD], capMod = (int)M->q[Q_CAPMOD];
  if (mobMod < 1 || mobMod > 3 || capMod < 0 || capMod > 3) return XG_ERR_UNSUPPORTED;
  double *q = M->q;
  /* Model::Model (:9064-9102) */
  M->tnom = M->q_given[Q_TNOM] ? q[Q_TNOM] + K_CTOK : opt->tnom;
  if (!M->bin_given[B_VTH0]) M->bin[B_VTH0][0] = M->dtype == 1 ? 0.7 : -0.7;
  if (!M->bin_given[B_UC]) M->bin[B_UC][0] = mobMod == 3 ? -0.0465 : -0.0465e-9;
  if (!M->bin_given[B_UC1]) M->bin[B_UC1][0] = mobMod == 3 ? -0.056 : -0.056e-9;
  if (!M->bin_given[B_U0]) M->bin[B_U0][0] = M->dtype == 1 ? 0.067 : 0.025;
  /* Model::processParams (:8488-8570) */
  const double tox = q[Q_TOX];
  M->cox = 3.453133e-11 / tox;
  if (!M->q_given[Q_TOXM]) q[Q_TOXM] = tox;
  if (!M->bin_given[B_DSUB]) M->bin[B_DSUB][0] = M->bin[B_DROUT][0];
  if (!M->q_given[Q_LLC]) q[Q_LLC] = q[Q_LL];
  if (!M->q_given[Q_LWC]) q[Q_LWC] = q[Q_LW];
  if (!M->q_given[Q_LWLC]) q[Q_LWLC] = q[Q_LWL];
  if (!M->q_given[Q_WLC]) q[Q_WLC] = q[Q_WL];
  if (!M->q_given[Q_WWL]) q[Q_WWLC] = q[Q_WWL];
  if (!M->q_given[Q_WWLC]) q[Q_WWLC] = q[Q_WWL];
  if (!M->q_given[Q_DWC]) q[Q_DWC] = q[Q_WINT];
  if (!M->q_given[Q_DLC]) q[Q_DLC] = q[Q_LINT];
  if (!M->bin_given[B_CF]) {
    const double C1 = 2.0 * K_EPSOX, C5 = M_PI, C2 = 1.0 + (0.4e-6 / tox), C3 = log(C2);
    M->bin[B_CF][0] = C1 * C3 / C5;
  }
  if (!M->q_given[Q_CGDO]) {
    if (M->q_given[Q_DLC] && q[Q_DLC] > 0.0) q[Q_CGDO] = q[Q_DLC] * M->cox - M->bin[B_CGDL][0];
    else q[Q_CGDO] = 0.6 * M->bin[B_XJ][0] * M->cox;
  }
  if (!M->q_given[Q_CGSO]) {
    if (M->q_given[Q_DLC] && q[Q_DLC] > 0.0) q[Q_CGSO] = q[Q_DLC] * M->cox - M->bin[B_CGSL][0];
    else q[Q_CGSO] = 0.6 * M->bin[B_XJ][0] * M->cox;
  }
  if (!M->q_given[Q_CGBO]) q[Q_CGBO] = 2.0 * q[Q_DWC] * M->cox;
  if (!M->q_given[Q_CJSWG]) q[Q_CJSWG] = q[Q_CJSW];
  if (!M->q_given[Q_PBSWG]) q[Q_PBSWG] = q[Q_PBSW];
  if (!M->q_given[Q_MJSWG]) q[Q_MJSWG] = q[Q_MJSW];
  if (q[Q_PB] < 0.1) q[Q_PB] = 0.1;
  if (q[Q_PBSW] < 0.1) q[Q_PBSW] = 0.1;
  if (q[Q_PBSWG] < 0.1) q[Q_PBSWG] = 0.1;
  const double vt0 = K_BOLTZ * (27.0 + K_CTOK) / K_Q; /* CONSTvt0 */
  M->vcrit = vt0 * log(vt0 / (sqrt(2.0) * 1.0e-14));
  M->factor1 = sqrt(K_EPSSI / K_EPSOX * tox);
  const double tnom = M->tnom;
  M->Vtm0 = K_BOLTZ / K_Q * tnom;
  M->Eg0 = 1.16 - 7.02e-4 * tnom * tnom / (tnom + 1108.0);
  M->ni = K_NI0 * (tnom / K_REFTEMP) * sqrt(tnom / K_REFTEMP) * exp(21.5565981 - M->Eg0 / (2.0 * M->Vtm0));
  return XG_OK;
}

static double at_or(const double *a, int i, double def) { return a ? a[i] : def; }

/* One instance: Instance ctor + updateTemperature (:3639-4511) + the
 * junction capacitances; o has XG_B3_NPARAMS entries. */
static int b3_instance(const b3card_t *M, const xg_mos_desc *d, int i, double temp, double *o) {
  const double *q = M->q;
  memset(o, 0, sizeof(double) * XG_B3_NPARAMS);
  const double l = at_or(d->l, i, q[Q_L]), w = at_or(d->w, i, q[Q_W]);
  const double AD = at_or(d->ad, i, 0.0), AS = at_or(d->as, i, 0.0);
  const double PD = at_or(d->pd, i, 0.0), PS = at_or(d->ps, i, 0.0);
  const double NRD = at_or(d->nrd, i, 1.0), NRS = at_or(d->nrs, i, 1.0);
  const double Mult = at_or(d->m, i, 1.0);
  double gd = q[Q_RSH] * NRD;
  gd = gd > 0.0 ? 1.0 / gd : 0.0;
  double gs = q[Q_RSH] * NRS;
  gs = gs > 0.0 ? 1.0 / gs : 0.0;

  /* temperature (:3639-3727) */
  const double Tnom = M->tnom, TRatio = temp / Tnom;
  const double vtm = K_BOLTZ / K_Q * temp;
  const double Eg = 1.16 - 7.02e-4 * temp * temp / (temp + 1108.0);
  double Js, Jsw;
  if (temp != Tnom) {
    const double T0 = M->Eg0 / M->Vtm0 - Eg / vtm + q[Q_XTI] * log(temp / Tnom);
    const double T1 = exp(T0 / q[Q_NJ]);
    Js = q[Q_JS] * T1;
    Jsw = q[Q_JSW] * T1;
  } else {
    Js = q[Q_JS];
    Jsw = q[Q_JSW];
  }
  if (Js < 0.0) Js = 0.0;
  if (Jsw < 0.0) Jsw = 0.0;
  const double dT = temp - Tnom;
  double cj = 0.0, cjsw = 0.0, cjswg = 0.0, T0;
  T0 = q[Q_TCJ] * dT;
  if (T0 >= -1.0) cj = q[Q_CJ] * (1.0 + T0);
  T0 = q[Q_TCJSW] * dT;
  if (T0 >= -1.0) cjsw = q[Q_CJSW] * (1.0 + T0);
  T0 = q[Q_TCJSWG] * dT;
  if (T0 >= -1.0) cjswg = q[Q_CJSWG] * (1.0 + T0);
  double phib = q[Q_PB] - q[Q_TPB] * dT;
  if (phib < 0.01) phib = 0.01;
  double phibsw = q[Q_PBSW] - q[Q_TPBSW] * dT;
  if (phibsw <= 0.01) phibsw = 0.01;
  double phibswg = q[Q_PBSWG] - q[Q_TPBSWG] * dT;
  if (phibswg <= 0.01) phibswg = 0.01;

  /* size dependence (:3757-4470) */
  T0 = pow(l, q[Q_LLN]);
  double T1 = pow(w, q[Q_LWN]);
  double tmp1 = q[Q_LL] / T0 + q[Q_LW] / T1 + q[Q_LWL] / (T0 * T1);
  const double dl = q[Q_LINT] + tmp1;
  double tmp2 = q[Q_LLC] / T0 + q[Q_LWC] / T1 + q[Q_LWLC] / (T0 * T1);
  const double dlc = q[Q_DLC] + tmp2;
  double T2 = pow(l, q[Q_WLN]);
  double T3 = pow(w, q[Q_WWN]);
  tmp1 = q[Q_WL] / T2 + q[Q_WW] / T3 + q[Q_WWL] / (T2 * T3);
  const double dw = q[Q_WINT] + tmp1;
  tmp2 = q[Q_WLC] / T2 + q[Q_WWC] / T3 + q[Q_WWLC] / (T2 * T3);
  const double dwc = q[Q_DWC] + tmp2;
  const double leff = l - 2.0 * dl, weff = w - 2.0 * dw;
  const double leffCV = l - 2.0 * dlc, weffCV = w - 2.0 * dwc;
  if (leff <= 0.0 || weff <= 0.0 || leffCV <= 0.0 || weffCV <= 0.0) return XG_ERR_ARG;
  double iL, iW, iLW;
  if (q[Q_BINUNIT] == 1) {
    iL = 1.0e-6 / leff;
    iW = 1.0e-6 / weff;
    iLW = 1.0e-12 / (leff * weff);
  } else {
    iL = 1.0 / leff;
    iW = 1.0 / weff;
    iLW = 1.0 / (leff * weff);
  }
  double b[B_N];
  for (int k = 0; k < B_N; ++k)
    b[k] = M->bin[k][0] + M->bin[k][1] * iL + M->bin[k][2] * iW + M->bin[k][3] * iLW;
  const double abulkCVfactor = 1.0 + pow((b[B_CLC] / leffCV), b[B_CLE]);
  T0 = (TRatio - 1.0);
  const double ua = b[B_UA] + b[B_UA1] * T0, ub = b[B_UB] + b[B_UB1] * T0;
  const double uc = b[B_UC] + b[B_UC1] * T0;
  double u0 = b[B_U0];
  if (u0 > 1.0) u0 = u0 / 1.0e4;
  const double u0temp = u0 * pow(TRatio, b[B_UTE]);
  const double vsattemp = b[B_VSAT] - b[B_AT] * T0;
  const double rds0 = (b[B_RDSW] + b[B_PRT] * T0) / pow(weff * 1E6, b[B_WR]);
  const double tox = q[Q_TOX], cox = M->cox;
  const double cf = b[B_CF];
  const double p_cgdo = (q[Q_CGDO] + cf) * weffCV, p_cgso = (q[Q_CGSO] + cf) * weffCV;
  const double p_cgbo = q[Q_CGBO] * leffCV;
  double npeak = b[B_NCH], gamma1 = b[B_GAMMA1], gamma2 = b[B_GAMMA2];
  double vbx = b[B_VBX], vbm = b[B_VBM], k1 = b[B_K1], k2 = b[B_K2], vfb = b[B_VFB];
  double vth0 = b[B_VTH0], acde = b[B_ACDE];
  if (!M->bin_given[B_NCH] && M->bin_given[B_GAMMA1]) {
    T0 = gamma1 * cox;
    npeak = 3.021E22 * T0 * T0;
  }
  const double Vtm0 = M->Vtm0, ni = M->ni;
  const double phi = 2.0 * Vtm0 * log(npeak / ni);
  const double sqrtPhi = sqrt(phi), phis3 = sqrtPhi * phi;
  const double Xdep0 = sqrt(2.0 * K_EPSSI / (K_Q * npeak * 1.0e6)) * sqrtPhi;
  const double litl = sqrt(3.0 * b[B_XJ] * tox);
  const double vbi = Vtm0 * log(1.0e20 * npeak / (ni * ni));
  const double cdep0 = sqrt(K_Q * K_EPSSI * npeak * 1.0e6 / 2.0 / phi);
  const double ldeb = sqrt(K_EPSSI * Vtm0 / (K_Q * npeak * 1.0e6)) / 3.0;
  acde *= pow((npeak / 2.0e16), -0.25);
  if (M->bin_given[B_K1] || M->bin_given[B_K2]) {
    if (!M->bin_given[B_K1]) k1 = 0.53;
    if (!M->bin_given[B_K2]) k2 = -0.0186;
  } else {
    if (!M->bin_given[B_VBX]) vbx = phi - 7.7348e-4 * npeak * b[B_XT] * b[B_XT];
    if (vbx > 0.0) vbx = -vbx;
    if (vbm > 0.0) vbm = -vbm;
    if (!M->bin_given[B_GAMMA1]) gamma1 = 5.753e-12 * sqrt(npeak) / cox;
    if (!M->bin_given[B_GAMMA2]) gamma2 = 5.753e-12 * sqrt(b[B_NSUB]) / cox;
    T0 = gamma1 - gamma2;
    T1 = sqrt(phi - vbx) - sqrtPhi;
    T2 = sqrt(phi * (phi - vbm)) - phi;
    k2 = T0 * T1 / (2.0 * T2 + vbm);
    k1 = gamma2 - 2.0 * k2 * sqrt(phi - vbm);
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
  const int dtype = M->dtype;
  if (!M->bin_given[B_VFB]) {
    if (M->bin_given[B_VTH0]) vfb = dtype * vth0 - phi - k1 * sqrtPhi;
    else vfb = -1.0;
  }
  if (!M->bin_given[B_VTH0]) vth0 = dtype * (vfb + phi + k1 * sqrtPhi);
  const double toxm = q[Q_TOXM];
  const double k1ox = k1 * tox / toxm, k2ox = k2 * tox / toxm;
  T1 = sqrt(K_EPSSI / K_EPSOX * tox * Xdep0);
  T0 = exp(-0.5 * b[B_DSUB] * leff / T1);
  const double theta0vb0 = (T0 + 2.0 * T0 * T0);
  T0 = exp(-0.5 * b[B_DROUT] * leff / T1);
  T2 = (T0 + 2.0 * T0 * T0);
  const double thetaRout = b[B_PDIBLC1] * T2 + b[B_PDIBLC2];
  const double sqXd = sqrt(Xdep0);
  tmp1 = vbi - phi;
  tmp2 = M->factor1 * sqXd;
  T0 = -0.5 * b[B_DVT1W] * weff * leff / tmp2;
  T1 = T0 > -EXP_THRESHOLD ? exp(T0) : MIN_EXP;
  T2 = T1 * (1.0 + 2.0 * T1);
  T0 = b[B_DVT0W] * T2;
  T2 = T0 * tmp1;
  T0 = -0.5 * b[B_DVT1] * leff / tmp2;
  T1 = T0 > -EXP_THRESHOLD ? exp(T0) : MIN_EXP;
  T3 = T1 * (1.0 + 2.0 * T1);
  T3 = b[B_DVT0] * T3 * tmp1;
  const double T4 = tox * phi / (weff + b[B_W0]);
  T0 = sqrt(1.0 + b[B_NLX] / leff);
  const double T5 = k1ox * (T0 - 1.0) * sqrtPhi + (b[B_KT1] + b[B_KT1L] / leff) * (TRatio - 1.0);
  const double tmp3 = dtype * vth0 - T2 - T3 + b[B_K3] * T4 + T5;
  const double vfbzb = tmp3 - phi - k1 * sqrtPhi;

  /* junction saturation currents (:4475-4511) */
  const double Nvtm = vtm * q[Q_NJ], ijth = q[Q_IJTH];
  double ssat, dsat, vjsm = 0.0, isevjsm = 0.0, vjdm = 0.0, isevjdm = 0.0;
  ssat = (AS <= 0.0 && PS <= 0.0) ? 1.0e-14 : AS * Js + PS * Jsw;
  if (ssat > 0.0 && ijth > 0.0) {
    vjsm = Nvtm * log(ijth / ssat + 1.0);
    isevjsm = ssat * exp(vjsm / Nvtm);
  }
  dsat = (AD <= 0.0 && PD <= 0.0) ? 1.0e-14 : AD * Js + PD * Jsw;
  if (dsat > 0.0 && ijth > 0.0) {
    vjdm = Nvtm * log(ijth / dsat + 1.0);
    isevjdm = dsat * exp(vjdm / Nvtm);
  }
  /* junction capacitances (updateIntermediateVars :6983-7007) */
  double czbdsw, czbdswg, czbssw, czbsswg;
  if (PD < weff) {
    czbdswg = cjswg * PD;
    czbdsw = 0.0;
  } else {
    czbdsw = cjsw * (PD - weff);
    czbdswg = cjswg * weff;
  }
  if (PS < weff) {
    czbssw = 0.0;
    czbsswg = cjswg * PS;
  } else {
    czbssw = cjsw * (PS - weff);
    czbsswg = cjswg * weff;
  }

  o[XG_B3_DTYPE] = dtype;
  o[XG_B3_MOBMOD] = q[Q_MOBMOD];
  o[XG_B3_CAPMOD] = q[Q_CAPMOD];
  o[XG_B3_XPART] = q[Q_XPART];
  o[XG_B3_TOX] = tox;
  o[XG_B3_COX] = cox;
  o[XG_B3_FACTOR1] = M->factor1;
  o[XG_B3_VCRIT] = M->vcrit;
  o[XG_B3_NJ] = q[Q_NJ];
  o[XG_B3_IJTH] = ijth;
  o[XG_B3_MJ] = q[Q_MJ];
  o[XG_B3_MJSW] = q[Q_MJSW];
  o[XG_B3_MJSWG] = q[Q_MJSWG];
  o[XG_B3_TNOM] = Tnom;
  o[XG_B3_TEMP] = temp;
  o[XG_B3_VTM] = vtm;
  o[XG_B3_JSTEMP] = Js;
  o[XG_B3_JSWTEMP] = Jsw;
  o[XG_B3_CJTEMP] = cj;
  o[XG_B3_CJSWTEMP] = cjsw;
  o[XG_B3_CJSWGTEMP] = cjswg;
  o[XG_B3_PHIB] = phib;
  o[XG_B3_PHIBSW] = phibsw;
  o[XG_B3_PHIBSWG] = phibswg;
  o[XG_B3_VJSM] = vjsm;
  o[XG_B3_ISEVJSM] = isevjsm;
  o[XG_B3_VJDM] = vjdm;
  o[XG_B3_ISEVJDM] = isevjdm;
  o[XG_B3_AD] = AD;
  o[XG_B3_AS] = AS;
  o[XG_B3_PD] = PD;
  o[XG_B3_PS] = PS;
  o[XG_B3_GD] = gd;
  o[XG_B3_GS] = gs;
  o[XG_B3_M] = Mult;
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
  o[XG_B3_DVT0] = b[B_DVT0];
  o[XG_B3_DVT1] = b[B_DVT1];
  o[XG_B3_DVT2] = b[B_DVT2];
  o[XG_B3_DVT0W] = b[B_DVT0W];
  o[XG_B3_DVT1W] = b[B_DVT1W];
  o[XG_B3_DVT2W] = b[B_DVT2W];
  o[XG_B3_NLX] = b[B_NLX];
  o[XG_B3_K1] = k1;
  o[XG_B3_K1OX] = k1ox;
  o[XG_B3_K2OX] = k2ox;
  o[XG_B3_K3] = b[B_K3];
  o[XG_B3_K3B] = b[B_K3B];
  o[XG_B3_KT1] = b[B_KT1];
  o[XG_B3_KT1L] = b[B_KT1L];
  o[XG_B3_KT2] = b[B_KT2];
  o[XG_B3_W0] = b[B_W0];
  o[XG_B3_ETA0] = b[B_ETA0];
  o[XG_B3_ETAB] = b[B_ETAB];
  o[XG_B3_THETA0VB0] = theta0vb0;
  o[XG_B3_NFACTOR] = b[B_NFACTOR];
  o[XG_B3_CDSC] = b[B_CDSC];
  o[XG_B3_CDSCB] = b[B_CDSCB];
  o[XG_B3_CDSCD] = b[B_CDSCD];
  o[XG_B3_CIT] = b[B_CIT];
  o[XG_B3_VFB] = vfb;
  o[XG_B3_NGATE] = b[B_NGATE];
  o[XG_B3_VOFF] = b[B_VOFF];
  o[XG_B3_CDEP0] = cdep0;
  o[XG_B3_DWG] = b[B_DWG];
  o[XG_B3_DWB] = b[B_DWB];
  o[XG_B3_PRWG] = b[B_PRWG];
  o[XG_B3_PRWB] = b[B_PRWB];
  o[XG_B3_RDS0] = rds0;
  o[XG_B3_XJ] = b[B_XJ];
  o[XG_B3_A0] = b[B_A0];
  o[XG_B3_B0] = b[B_B0];
  o[XG_B3_B1] = b[B_B1];
  o[XG_B3_AGS] = b[B_AGS];
  o[XG_B3_KETA] = b[B_KETA];
  o[XG_B3_UA] = ua;
  o[XG_B3_UB] = ub;
  o[XG_B3_UC] = uc;
  o[XG_B3_U0TEMP] = u0temp;
  o[XG_B3_VSATTEMP] = vsattemp;
  o[XG_B3_A1] = b[B_A1];
  o[XG_B3_A2] = b[B_A2];
  o[XG_B3_DELTA] = b[B_DELTA];
  o[XG_B3_PCLM] = b[B_PCLM];
  o[XG_B3_LITL] = litl;
  o[XG_B3_THETAROUT] = thetaRout;
  o[XG_B3_PDIBLB] = b[B_PDIBLCB];
  o[XG_B3_PVAG] = b[B_PVAG];
  o[XG_B3_PSCBE1] = b[B_PSCBE1];
  o[XG_B3_PSCBE2] = b[B_PSCBE2];
  o[XG_B3_ALPHA0] = b[B_ALPHA0];
  o[XG_B3_ALPHA1] = b[B_ALPHA1];
  o[XG_B3_BETA0] = b[B_BETA0];
  o[XG_B3_VFBCV] = b[B_VFBCV];
  o[XG_B3_WEFFCV] = weffCV;
  o[XG_B3_LEFFCV] = leffCV;
  o[XG_B3_ABULKCVFACTOR] = abulkCVfactor;
  o[XG_B3_NOFF] = b[B_NOFF];
  o[XG_B3_VOFFCV] = b[B_VOFFCV];
  o[XG_B3_VFBZB] = vfbzb;
  o[XG_B3_ACDE] = acde;
  o[XG_B3_LDEB] = ldeb;
  o[XG_B3_MOIN] = b[B_MOIN];
  o[XG_B3_CGDO] = p_cgdo;
  o[XG_B3_CGSO] = p_cgso;
  o[XG_B3_CGBO] = p_cgbo;
  o[XG_B3_CKAPPA] = b[B_CKAPPA];
  o[XG_B3_CGDL] = b[B_CGDL];
  o[XG_B3_CGSL] = b[B_CGSL];
  o[XG_B3_SSAT] = ssat;
  o[XG_B3_DSAT] = dsat;
  o[XG_B3_NVTM] = Nvtm;
  o[XG_B3_CZBD] = cj * AD;
  o[XG_B3_CZBS] = cj * AS;
  o[XG_B3_CZBDSW] = czbdsw;
  o[XG_B3_CZBDSWG] = czbdswg;
  o[XG_B3_CZBSSW] = czbssw;
  o[XG_B3_CZBSSWG] = czbsswg;
  xg_b3_hoist(o);
  return XG_OK;
}

int xgo_b3_setup(const xg_netlist *nl, const xg_device_options *opt, double *out) {
  const xg_mos_desc *d = &nl->bsim3;
  const int n = d->n;
  b3card_t *cards = (b3card_t *)calloc((size_t)nl->n_models + 1, sizeof *cards);
  if (!cards) return XG_ERR_OOM;
  int rc = XG_OK;
  for (int k = 0; k < nl->n_models && rc == XG_OK; ++k)
    if (nl->models[k].type == XG_DEV_BSIM3) rc = b3_card(&nl->models[k], opt, &cards[k]);
  double o[XG_B3_NPARAMS];
  for (int i = 0; i < n && rc == XG_OK; ++i) {
    const int mi = d->model[i];
    if (mi < 0 || mi >= nl->n_models || nl->models[mi].type != XG_DEV_BSIM3) {
      rc = XG_ERR_ARG;
      break;
    }
    rc = b3_instance(&cards[mi], d, i, opt->temp, o);
    for (int k = 0; k < XG_B3_NPARAMS; ++k) out[(int64_t)k * n + i] = o[k];
  }
  free(cards);
  return rc;
}
