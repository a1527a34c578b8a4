/*
 * xgo_setup.c — the oracle's own circuit set-up (TEST INFRASTRUCTURE ONLY;
 * see xgo.h): model cards and per-instance parameter blocks of every device
 * type, in the column layout of include/xg_params.h, computed here on the
 * CPU so that nothing the oracle runs comes from the engine.  Pinned by the
 * tests to the parameter blocks the reference itself derived (the golden
 * fixtures' params.* arrays, and oracle/_ref where it is built).
 *
 * Restates, from src/DeviceModelPKG/OpenModels/src/:
 *   N_DEV_MOSFET1.C  Model::Model/processParams :3730-3866, Instance ctor
 *                    :1170-1262, updateTemperature :3437-3680, and the
 *                    per-load constants of updateIntermediateVars :2650-2665
 *   N_DEV_Diode.C    Model::processParams :1772-1790, updateTemperature
 *                    :1335-1500 (level 1)
 *   N_DEV_Resistor.C :852-860, N_DEV_Capacitor.C, N_DEV_Vsrc.C / N_DEV_ISRC.C
 *                    with N_DEV_SourceData.C (DC, PULSE)
 * BSIM3 v3.2 is in xgo_b3setup.c.
 *
 * Compiled with -ffp-contract=off like the rest of the oracle.
 */
#include <ctype.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xgo_internal.h"

#define K_Q 1.6021918e-19        /* CONSTQ      (N_DEV_Const.h) */
#define K_BOLTZ 1.3806226e-23    /* CONSTboltz  */
#define K_REFTEMP 300.15         /* CONSTREFTEMP */
#define K_CTOK 273.15            /* CONSTCtoK   */

static double koverq(void) { return K_BOLTZ / K_Q; }

/* ---- model cards ------------------------------------------------------------ */

int xgo_card_eq(const char *a, const char *b) {
  for (; *a && *b; ++a, ++b)
    if (toupper((unsigned char)*a) != toupper((unsigned char)*b)) return 0;
  return *a == 0 && *b == 0;
}

/* The value of parameter `key` on the card, or `def` when it is not given. */
static int card_given(const xg_model_desc *m, const char *key, double *v) {
  for (int i = 0; i < m->n_params; ++i)
    if (xgo_card_eq(m->names[i], key)) {
      if (v) *v = m->values[i];
      return 1;
    }
  return 0;
}
static double card(const xg_model_desc *m, const char *key, double def) {
  double v = def;
  card_given(m, key, &v);
  return v;
}
static int card_known(const xg_model_desc *m, const char *const *known, int nk) {
  for (int i = 0; i < m->n_params; ++i) {
    int ok = 0;
    for (int k = 0; k < nk && !ok; ++k) ok = xgo_card_eq(m->names[i], known[k]);
    if (!ok) return 0;
  }
  return 1;
}

/* ---- MOSFET level 1 --------------------------------------------------------- */

typedef struct {
  int dtype;
  double l, w, vto, kp, gamma, phi, lambda, rd, rs, cbd, cbs, is, pb, cgso, cgdo, cgbo, rsh;
  double cj, mj, cjsw, mjsw, js, tox, ld, uo, fc, nsub, nss, tpg, tnom;
  int g_rsh, g_cj, g_cjsw;
  double fact1, vtnom, egfet1, pbfact1, oxcap;
} m1card_t;

/* Model::Model defaults (Traits::loadModelParameters) and processParams
 * (N_DEV_MOSFET1.C:3786-3866). */
static int m1_card(const xg_model_desc *md, const xg_device_options *opt, m1card_t *m) {
  static const char *const known[] = {
      "L", "W", "VTO", "KP", "GAMMA", "PHI", "LAMBDA", "RD", "RS", "CBD", "CBS", "IS", "PB",
      "CGSO", "CGDO", "CGBO", "RSH", "CJ", "MJ", "CJSW", "MJSW", "JS", "TOX", "LD", "UO", "U0",
      "FC", "NSUB", "NSS", "TNOM", "KF", "AF", "TPG", "LEVEL"};
  if (!card_known(md, known, (int)(sizeof known / sizeof known[0]))) return XG_ERR_UNSUPPORTED;
  memset(m, 0, sizeof *m);
  m->dtype = md->polarity < 0 ? -1 : 1;
  m->l = card(md, "L", 1e-4);
  m->w = card(md, "W", 1e-4);
  m->vto = card(md, "VTO", 0.0);
  m->kp = card(md, "KP", 2e-5);
  m->gamma = card(md, "GAMMA", 0.0);
  m->phi = card(md, "PHI", 0.6);
  m->lambda = card(md, "LAMBDA", 0.0);
  m->rd = card(md, "RD", 0.0);
  m->rs = card(md, "RS", 0.0);
  m->cbd = card(md, "CBD", 0.0);
  m->cbs = card(md, "CBS", 0.0);
  m->is = card(md, "IS", 1e-14);
  m->pb = card(md, "PB", 0.8);
  m->cgso = card(md, "CGSO", 0.0);
  m->cgdo = card(md, "CGDO", 0.0);
  m->cgbo = card(md, "CGBO", 0.0);
  m->rsh = card(md, "RSH", 0.0);
  m->g_rsh = card_given(md, "RSH", NULL);
  m->cj = card(md, "CJ", 0.0);
  m->g_cj = card_given(md, "CJ", NULL);
  m->mj = card(md, "MJ", 0.5);
  m->cjsw = card(md, "CJSW", 0.0);
  m->g_cjsw = card_given(md, "CJSW", NULL);
  m->mjsw = card(md, "MJSW", 0.5);
  m->js = card(md, "JS", 0.0);
  m->tox = card(md, "TOX", 1e-7);
  m->ld = card(md, "LD", 0.0);
  m->uo = card(md, "UO", 600.0);
  card_given(md, "U0", &m->uo);
  m->fc = card(md, "FC", 0.5);
  m->nsub = card(md, "NSUB", 0.0);
  m->nss = card(md, "NSS", 0.0);
  m->tpg = card(md, "TPG", 0.0);
  m->tnom = card_given(md, "TNOM", &m->tnom) ? m->tnom + K_CTOK : opt->tnom;

  const double tnom = m->tnom;
  m->fact1 = tnom / K_REFTEMP;
  m->vtnom = tnom * koverq();
  const double kt1 = K_BOLTZ * tnom;
  m->egfet1 = 1.16 - (7.02e-4 * tnom * tnom) / (tnom + 1108);
  const double arg1 = -m->egfet1 / (kt1 + kt1) + 1.1150877 / (K_BOLTZ * (K_REFTEMP + K_REFTEMP));
  m->pbfact1 = -2 * m->vtnom * (1.5 * log(m->fact1) + K_Q * arg1);
  if (!card_given(md, "TOX", NULL) || m->tox == 0) {
    m->oxcap = 0;
  } else {
    m->oxcap = 3.9 * 8.854214871e-12 / m->tox;
    if (!card_given(md, "KP", NULL)) {
      if (!card_given(md, "UO", NULL) && !card_given(md, "U0", NULL)) m->uo = 600;
      m->kp = m->uo * m->oxcap * 1e-4;
    }
    if (card_given(md, "NSUB", NULL)) {
      if (m->nsub * 1e6 > 1.45e16) {
        if (!card_given(md, "PHI", NULL)) {
          m->phi = 2 * m->vtnom * log(m->nsub * 1e6 / 1.45e16);
          if (m->phi < 0.1) m->phi = 0.1;
        }
        const double fermis = m->dtype * .5 * m->phi;
        double wkfng = 3.2;
        if (!card_given(md, "TPG", NULL)) m->tpg = 1;
        if (m->tpg != 0) {
          const double fermig = m->dtype * m->tpg * .5 * m->egfet1;
          wkfng = 3.25 + .5 * m->egfet1 - fermig;
        }
        const double wkfngs = wkfng - (3.25 + .5 * m->egfet1 + fermis);
        if (!card_given(md, "GAMMA", NULL))
          m->gamma = sqrt(2 * 11.70 * 8.854214871e-12 * K_Q * m->nsub * 1e6) / m->oxcap;
        if (!card_given(md, "VTO", NULL)) {
          if (!card_given(md, "NSS", NULL)) m->nss = 0;
          const double vfb = wkfngs - m->nss * 1e4 * K_Q / m->oxcap;
          m->vto = vfb + m->dtype * (m->gamma * sqrt(m->phi) + m->phi);
        }
      } else {
        return XG_ERR_ARG; /* Nsub < Ni */
      }
    }
  }
  return XG_OK;
}

static double opt_at(const double *a, int i, double def) { return a ? a[i] : def; }

/* Instance ctor (:1170-1262) + updateTemperature (:3437-3680) + the per-load
 * constants of updateIntermediateVars (:2650-2665). */
static void m1_instance(const m1card_t *mo, const xg_mos_desc *d, int i, double temp, double *o) {
  const double l = opt_at(d->l, i, mo->l), w = opt_at(d->w, i, mo->w);
  const double AD = opt_at(d->ad, i, 0.0), AS = opt_at(d->as, i, 0.0);
  const double PD = opt_at(d->pd, i, 0.0), PS = opt_at(d->ps, i, 0.0);
  const double NRD = opt_at(d->nrd, i, 1.0), NRS = opt_at(d->nrs, i, 1.0);
  const double M = opt_at(d->m, i, 1.0);
  double gd = 0, gs = 0;
  if (mo->rd != 0) gd = 1 / mo->rd;
  else if (mo->g_rsh) gd = mo->rsh != 0 ? 1 / (mo->rsh * NRD) : 0;
  if (mo->rs != 0) gs = 1 / mo->rs;
  else if (mo->g_rsh) gs = mo->rsh != 0 ? 1 / (mo->rsh * NRS) : 0;
  const double Leff = l - 2 * mo->ld;

  const double tnom = mo->tnom;
  const double vt = temp * koverq();
  const double ratio = temp / tnom;
  const double fact2 = temp / K_REFTEMP;
  const double kt = temp * K_BOLTZ;
  const double egfet = 1.16 - (7.02e-4 * temp * temp) / (temp + 1108);
  double arg = -egfet / (kt + kt) + 1.1150877 / (K_BOLTZ * (K_REFTEMP + K_REFTEMP));
  const double pbfact = -2 * vt * (1.5 * log(fact2) + K_Q * arg);
  const double ratio4 = ratio * sqrt(ratio);
  const double tKP = mo->kp / ratio4;
  const double phio = (mo->phi - mo->pbfact1) / mo->fact1;
  const double tPhi = fact2 * phio + pbfact;
  const double tVbi = mo->vto - mo->dtype * (mo->gamma * sqrt(mo->phi)) + .5 * (mo->egfet1 - egfet) +
                      mo->dtype * .5 * (tPhi - mo->phi);
  const double tVto = tVbi + mo->dtype * mo->gamma * sqrt(tPhi);
  const double tIs = mo->is * exp(-egfet / vt + mo->egfet1 / mo->vtnom);
  const double tJs = mo->js * exp(-egfet / vt + mo->egfet1 / mo->vtnom);
  const double pbo = (mo->pb - mo->pbfact1) / mo->fact1;
  const double gmaold = (mo->pb - pbo) / pbo;
  double capfact = 1 / (1 + mo->mj * (4e-4 * (mo->tnom - K_REFTEMP) - gmaold));
  double tCbd = mo->cbd * capfact, tCbs = mo->cbs * capfact, tCj = mo->cj * capfact;
  capfact = 1 / (1 + mo->mjsw * (4e-4 * (mo->tnom - K_REFTEMP) - gmaold));
  double tCjsw = mo->cjsw * capfact;
  const double tPb = fact2 * pbo + pbfact;
  const double gmanew = (tPb - pbo) / pbo;
  capfact = (1 + mo->mj * (4e-4 * (temp - K_REFTEMP) - gmanew));
  tCbd *= capfact;
  tCbs *= capfact;
  tCj *= capfact;
  capfact = (1 + mo->mjsw * (4e-4 * (temp - K_REFTEMP) - gmanew));
  tCjsw *= capfact;
  const double tDepCap = mo->fc * tPb;
  double svcrit, dvcrit;
  if (mo->js == 0 || AD == 0 || AS == 0) {
    svcrit = dvcrit = vt * log(vt / (sqrt(2.0) * mo->is));
  } else {
    dvcrit = vt * log(vt / (sqrt(2.0) * mo->js * AD));
    svcrit = vt * log(vt / (sqrt(2.0) * mo->js * AS));
  }
  const double MJ = mo->mj, MJSW = mo->mjsw, FC = mo->fc;
  const double czbd = mo->cbd != 0 ? tCbd : (mo->g_cj ? tCj * AD : 0);
  const double czbdsw = mo->g_cjsw ? tCjsw * PD : 0;
  arg = 1 - FC;
  const double sarg = exp((-MJ) * log(arg)), sargsw = exp((-MJSW) * log(arg));
  const double f2d = czbd * (1 - FC * (1 + MJ)) * sarg / arg + czbdsw * (1 - FC * (1 + MJSW)) * sargsw / arg;
  const double f3d = czbd * MJ * sarg / arg / tPb + czbdsw * MJSW * sargsw / arg / tPb;
  const double f4d = czbd * tPb * (1 - arg * sarg) / (1 - MJ) + czbdsw * tPb * (1 - arg * sargsw) / (1 - MJSW) -
                     f3d / 2 * (tDepCap * tDepCap) - tDepCap * f2d;
  const double czbs = mo->cbs != 0 ? tCbs : (mo->g_cj ? tCj * AS : 0);
  const double czbssw = mo->g_cjsw ? tCjsw * PS : 0;
  const double f2s = czbs * (1 - FC * (1 + MJ)) * sarg / arg + czbssw * (1 - FC * (1 + MJSW)) * sargsw / arg;
  const double f3s = czbs * MJ * sarg / arg / tPb + czbssw * MJSW * sargsw / arg / tPb;
  const double f4s = czbs * tPb * (1 - arg * sarg) / (1 - MJ) + czbssw * tPb * (1 - arg * sargsw) / (1 - MJSW) -
                     f3s / 2 * (tDepCap * tDepCap) - tDepCap * f2s;
  double dsat, ssat;
  if (tJs == 0 || AD == 0 || AS == 0) {
    dsat = ssat = tIs;
  } else {
    dsat = tJs * AD;
    ssat = tJs * AS;
  }
  o[XG_M1_DTYPE] = mo->dtype;
  o[XG_M1_GAMMA] = mo->gamma;
  o[XG_M1_LAMBDA] = mo->lambda;
  o[XG_M1_MJ] = MJ;
  o[XG_M1_MJSW] = MJSW;
  o[XG_M1_DRAINSATCUR] = dsat;
  o[XG_M1_SOURCESATCUR] = ssat;
  o[XG_M1_BETA] = tKP * w / Leff;
  o[XG_M1_TVTO] = tVto;
  o[XG_M1_SOURCEVCRIT] = svcrit;
  o[XG_M1_DRAINVCRIT] = dvcrit;
  o[XG_M1_VT] = vt;
  o[XG_M1_TPHI] = tPhi;
  o[XG_M1_TVBI] = tVbi;
  o[XG_M1_CBS] = czbs;
  o[XG_M1_CBSSW] = czbssw;
  o[XG_M1_CBD] = czbd;
  o[XG_M1_CBDSW] = czbdsw;
  o[XG_M1_TDEPCAP] = tDepCap;
  o[XG_M1_TBULKPOT] = tPb;
  o[XG_M1_F2S] = f2s;
  o[XG_M1_F3S] = f3s;
  o[XG_M1_F4S] = f4s;
  o[XG_M1_F2D] = f2d;
  o[XG_M1_F3D] = f3d;
  o[XG_M1_F4D] = f4d;
  o[XG_M1_OXIDECAP] = mo->oxcap * Leff * w;
  o[XG_M1_CGSO] = mo->cgso * w;
  o[XG_M1_CGDO] = mo->cgdo * w;
  o[XG_M1_CGBO] = mo->cgbo * Leff;
  o[XG_M1_GD] = gd;
  o[XG_M1_GS] = gs;
  o[XG_M1_M] = M;
  o[XG_M1_ICVDS] = o[XG_M1_ICVGS] = o[XG_M1_ICVBS] = 0.0;
  o[XG_M1_FLAGS] = 0.0;
}

/* ---- diode, level 1 ----------------------------------------------------------- */

typedef struct {
  double IS, RS, COND, N, TT, CJO, VJ, M, EG, XTI, FC, BV, IBV, IRF, TNOM, F2, F3;
  int bv_given;
} dcard_t;

static int d_card(const xg_model_desc *md, const xg_device_options *opt, dcard_t *m) {
  static const char *const known[] = {"IS", "JS", "RS", "N", "TT", "CJO", "CJ", "CJ0", "VJ", "M",
                                      "EG", "XTI", "FC", "BV", "VB", "IBV", "IRF", "TNOM", "KF",
                                      "AF", "LEVEL"};
  if (!card_known(md, known, (int)(sizeof known / sizeof known[0]))) return XG_ERR_UNSUPPORTED;
  if (card(md, "LEVEL", 1) != 1) return XG_ERR_UNSUPPORTED;
  memset(m, 0, sizeof *m);
  m->IS = card_given(md, "IS", NULL) ? card(md, "IS", 1e-14) : card(md, "JS", 1e-14);
  m->RS = card(md, "RS", 0.0);
  m->N = card(md, "N", 1.0);
  m->TT = card(md, "TT", 0.0);
  m->CJO = card_given(md, "CJO", NULL) ? card(md, "CJO", 0)
                                       : (card_given(md, "CJ", NULL) ? card(md, "CJ", 0) : card(md, "CJ0", 0));
  m->VJ = card(md, "VJ", 1.0);
  m->M = card(md, "M", 0.5);
  m->EG = card(md, "EG", 1.11);
  m->XTI = card(md, "XTI", 3.0);
  m->FC = card(md, "FC", 0.5);
  m->bv_given = card_given(md, "BV", NULL) || card_given(md, "VB", NULL);
  m->BV = card_given(md, "BV", NULL) ? card(md, "BV", 1e99) : card(md, "VB", 1e99);
  m->IBV = card(md, "IBV", 1.0e-3);
  m->IRF = card(md, "IRF", 1.0);
  m->TNOM = card_given(md, "TNOM", &m->TNOM) ? m->TNOM + K_CTOK : opt->tnom;
  /* Model::processParams (N_DEV_Diode.C:1772-1790) */
  if (m->M > 0.9) m->M = 0.9;
  if (m->EG < 0.1) m->EG = 0.1;
  if (m->FC > 0.95) m->FC = 0.95;
  m->COND = m->RS == 0.0 ? 0.0 : 1.0 / m->RS;
  const double xfc = log(1.0 - m->FC);
  m->F2 = exp((1.0 + m->M) * xfc);
  m->F3 = 1.0 - m->FC * (1.0 + m->M);
  return XG_OK;
}

/* Instance::updateTemperature (N_DEV_Diode.C:1335-1500), level 1. */
static void d_instance(const dcard_t *mo, const xg_diode_desc *d, int i, double Temp, double *o) {
  const double e1 = exp(1.0);
  const double Area = opt_at(d->area, i, 1.0);
  const double vtnom = koverq() * mo->TNOM;
  const double xfc = log(1.0 - mo->FC);
  const double vt = koverq() * Temp;
  const double fact2 = Temp / K_REFTEMP;
  const double egfet = 1.16 - (7.02e-4 * Temp * Temp) / (Temp + 1108.0);
  const double arg = -egfet / (2.0 * K_BOLTZ * Temp) + 1.1150877 / (K_BOLTZ * (K_REFTEMP + K_REFTEMP));
  const double pbfact = -2.0 * vt * (1.5 * log(fact2) + K_Q * arg);
  const double egfet1 = 1.16 - (7.02e-4 * mo->TNOM * mo->TNOM) / (mo->TNOM + 1108.0);
  const double arg1 = -egfet1 / (2.0 * K_BOLTZ * mo->TNOM) + 1.1150877 / (2.0 * K_BOLTZ * K_REFTEMP);
  const double fact1 = mo->TNOM / K_REFTEMP;
  const double pbfact1 = -2.0 * vtnom * (1.5 * log(fact1) + K_Q * arg1);
  const double pbo = (mo->VJ - pbfact1) / fact1;
  const double gmaold = (mo->VJ - pbo) / pbo;
  double tCj = mo->CJO / (1.0 + mo->M * (4.0e-4 * (mo->TNOM - K_REFTEMP) - gmaold));
  const double tPot = pbfact + fact2 * pbo;
  const double gmanew = (tPot - pbo) / pbo;
  tCj *= 1.0 + mo->M * (4.0e-4 * (Temp - K_REFTEMP) - gmanew);
  const double tIs = mo->IS * exp(((Temp / mo->TNOM) - 1.0) * mo->EG / (mo->N * vt) +
                                  mo->XTI / mo->N * log(Temp / mo->TNOM));
  const double tF1 = tPot * (1.0 - exp((1.0 - mo->M) * xfc)) / (1.0 - mo->M);
  const double vte = mo->N * vt;
  const double tVcrit = vte * log(vte / (sqrt(2.0) * tIs));
  const double tIRF = mo->IRF * pow(fact2, 1.6);
  double tBV = 0.0;
  if (mo->bv_given) {
    const double BV = mo->BV, cbv = mo->IBV;
    double a1 = 3.0 * vte / (e1 * BV);
    a1 = a1 * a1 * a1;
    const double lo = tIs * tIRF * (1 - a1);
    const double hi = tIs * tIRF * (1 - 1.0 / (e1 * e1 * e1)) * exp(-1.0 * (3.0 * vte - BV) / vte);
    if (cbv >= hi) {
      tBV = 3.0 * vte;
    } else if (cbv <= lo) {
      tBV = BV;
    } else {
      double xbv = BV;
      for (int it = 0; it < 8; it++) {
        double a2 = 3.0 * vte / (e1 * xbv);
        a2 = a2 * a2 * a2;
        xbv = BV - vte * log(cbv / (tIs * tIRF)) + vte * log(1 - a2);
      }
      tBV = xbv;
    }
  }
  o[XG_D_M] = mo->M;
  o[XG_D_BV] = mo->BV;
  o[XG_D_N] = mo->N;
  o[XG_D_TT] = mo->TT;
  o[XG_D_F2] = mo->F2;
  o[XG_D_F3] = mo->F3;
  o[XG_D_ISAT] = tIs * Area;
  o[XG_D_VT] = koverq() * Temp;
  o[XG_D_GSPR] = mo->COND * Area;
  o[XG_D_TVCRIT] = tVcrit;
  o[XG_D_TIRF] = tIRF;
  o[XG_D_TBRKDWNV] = tBV;
  o[XG_D_TJCTCAP] = tCj;
  o[XG_D_TJCTPOT] = tPot;
  o[XG_D_TDEPCAP] = mo->FC * tPot;
  o[XG_D_TF1] = tF1;
  o[XG_D_AREA] = Area;
  o[XG_D_INITCOND] = 0.0;
  o[XG_D_FLAGS] = mo->bv_given ? 1.0 : 0.0;
}

/* ---- entry point ------------------------------------------------------------- */

static int count_t(const xg_netlist *nl, int t) {
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

static int np_t(int t) {
  switch (t) {
    case XG_DEV_RES: return XG_R_NPARAMS;
    case XG_DEV_CAP: return XG_C_NPARAMS;
    case XG_DEV_VSRC: case XG_DEV_ISRC: return XG_V_NPARAMS;
    case XG_DEV_DIODE: return XG_D_NPARAMS;
    case XG_DEV_MOS1: return XG_M1_NPARAMS;
    case XG_DEV_BSIM3: return XG_B3_NPARAMS;
  }
  return 0;
}

int xgo_setup_params(const xg_netlist *nl, const xg_device_options *opt, int t, double *out,
                     int *n_params, int *n_instances) {
  if (!nl || !opt || t < 0 || t >= XG_NUM_DEV_TYPES) return XG_ERR_ARG;
  const int n = count_t(nl, t), np = np_t(t);
  if (n_params) *n_params = np;
  if (n_instances) *n_instances = n;
  if (!out || !n) return XG_OK;
  double tmp[XG_B3_NPARAMS + 8];
  int rc = XG_OK;
  if (t == XG_DEV_BSIM3) return xgo_b3_setup(nl, opt, out);
  m1card_t *m1 = NULL;
  dcard_t *dc = NULL;
  if (t == XG_DEV_MOS1 || t == XG_DEV_DIODE) {
    m1 = (m1card_t *)calloc((size_t)nl->n_models + 1, sizeof *m1);
    dc = (dcard_t *)calloc((size_t)nl->n_models + 1, sizeof *dc);
    for (int k = 0; k < nl->n_models && rc == XG_OK; ++k) {
      const xg_model_desc *md = &nl->models[k];
      if (md->type == XG_DEV_MOS1 && t == XG_DEV_MOS1) rc = m1_card(md, opt, &m1[k]);
      if (md->type == XG_DEV_DIODE && t == XG_DEV_DIODE) rc = d_card(md, opt, &dc[k]);
    }
  }
  for (int i = 0; i < n && rc == XG_OK; ++i) {
    memset(tmp, 0, sizeof tmp);
    switch (t) {
      case XG_DEV_RES: {
        const double R = nl->res.value[i];
        tmp[XG_R_G] = R != 0.0 ? 1.0 / R : 0.0;
        break;
      }
      case XG_DEV_CAP:
        tmp[XG_C_C] = nl->cap.value[i];
        break;
      case XG_DEV_VSRC:
      case XG_DEV_ISRC: {
        const xg_src_desc *d = t == XG_DEV_VSRC ? &nl->vsrc : &nl->isrc;
        const int kind = d->kind[i];
        if (kind != XG_SRC_DC && kind != XG_SRC_PULSE) { rc = XG_ERR_ARG; break; }
        tmp[XG_V_KIND] = kind;
        for (int k = 0; k < 7; ++k)
          tmp[XG_V_V1 + k] = kind == XG_SRC_PULSE || k == 0 ? d->wave[7 * (size_t)i + k] : 0.0;
        break;
      }
      case XG_DEV_DIODE: {
        const int mi = nl->diode.model[i];
        if (mi < 0 || mi >= nl->n_models || nl->models[mi].type != XG_DEV_DIODE) { rc = XG_ERR_ARG; break; }
        d_instance(&dc[mi], &nl->diode, i, opt->temp, tmp);
        break;
      }
      case XG_DEV_MOS1: {
        const int mi = nl->mos1.model[i];
        if (mi < 0 || mi >= nl->n_models || nl->models[mi].type != XG_DEV_MOS1) { rc = XG_ERR_ARG; break; }
        m1_instance(&m1[mi], &nl->mos1, i, opt->temp, tmp);
        break;
      }
    }
    for (int k = 0; k < np; ++k) out[(int64_t)k * n + i] = tmp[k];
  }
  free(m1);
  free(dc);
  return rc;
}
