/*
 * xgo_bsim3.c — BSIM3 v3.2 load loops of the oracle (TEST INFRASTRUCTURE
 * ONLY; see xgo.h).  Restates, statement for statement, from
 * src/DeviceModelPKG/OpenModels/src/N_DEV_MOSFET_B3.C:
 *   Instance::updateIntermediateVars   :4526-7273 (nqsMod = 0)
 *   Instance::setupCapacitors_oldDAE / _newDAE  :7574-7898
 *   Instance::auxChargeCalculations    :7477-7573
 *   Master::updateState                :9229-9305
 *   Master::loadDAEVectors             :9306-9653
 *   Master::loadDAEMatrices (pointer)  :9654-9939
 * The per-instance inputs are the parameter block of include/xg_params.h.
 * Members the reference only refreshes when charges are computed (the CAP*
 * capacitances, the Qeqq*_Jdxp limiter charges and qg/qb/qd/qbs/qbd) carry
 * over from one load to the next here as they do there.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xgo_internal.h"

#define EXP_THRESHOLD 34.0
#define MAX_EXP 5.834617425e14
#define MIN_EXP 1.713908431e-15
#define DELTA_1 0.02
#define DELTA_3 0.02
#define DELTA_4 0.02
#define EPSSI 1.03594e-10
#define KQ 1.6021918e-19
#define KBOLTZ 1.3806226e-23
#define CTOK 273.15

typedef struct { /* carried across loads */
  double CAPcggb, CAPcgdb, CAPcgsb, CAPcdgb, CAPcddb, CAPcdsb, CAPcsgb, CAPcsdb, CAPcssb;
  double CAPcbgb, CAPcbdb, CAPcbsb;
  double Qeqqg_Jdxp, Qeqqb_Jdxp, Qeqqd_Jdxp;
  double qg, qb, qd, qbs, qbd;
} b3mem_t;

typedef struct { /* produced by updateState, read by the vector/matrix loads */
  double vbs, vgs, vds, vbd, vgd, vgb, vbs_orig, vgs_orig, vds_orig, vbd_orig, vgd_orig;
  double von, gbs, gbd, cbs, cbd, gm, gds, gmbs, gbbs, gbgs, gbds, cd, csub;
  double Idrain, Isource, dxpart, sxpart, T1global;
  double ddxpart_dVd, ddxpart_dVg, ddxpart_dVb, ddxpart_dVs;
  double dsxpart_dVd, dsxpart_dVg, dsxpart_dVb, dsxpart_dVs;
  double ggtg, ggtd, ggtb, ggts;
  double Gm, Gmbs; /* signed by mode, set in loadDAEVectors (:9317-9345) */
  int mode, origFlag, ChargeComputationNeeded;
} b3m_t;

int xgo_b3_nparams(void) { return XG_B3_NPARAMS; }
void *xgo_b3_members_alloc(int n) { return calloc((size_t)n + 1, sizeof(b3mem_t)); }
void xgo_b3_members_reset(void *m, int n) { memset(m, 0, sizeof(b3mem_t) * ((size_t)n + 1)); }
int xgo_b3_nlid(void) { return 6; }
int xgo_b3_nint(const xgo_type *T, int i) {
  return (P(T, XG_B3_GD, i) != 0.0) + (P(T, XG_B3_GS, i) != 0.0);
}
/* Instance::registerLIDs (:2840-2856) */
void xgo_b3_lids(const xgo_type *T, int i, const int *ext, int *next, int *lid) {
  lid[0] = ext[0]; lid[1] = ext[1]; lid[2] = ext[2]; lid[3] = ext[3];
  lid[4] = P(T, XG_B3_GD, i) != 0.0 ? (*next)++ : ext[0];
  lid[5] = P(T, XG_B3_GS, i) != 0.0 ? (*next)++ : ext[2];
}
int xgo_b3_stamps(const xgo_type *T, int i, int *r, int *k) {
  const int *L = T->lid + (int64_t)i * 6;
  int d = L[0], g = L[1], s = L[2], b = L[3], dp = L[4], sp = L[5], n = 0;
#define ST(a, c) (r[n] = (a), k[n] = (c), ++n)
  ST(d, d); ST(d, dp); ST(s, s); ST(s, sp); ST(b, g); ST(b, b); ST(b, dp); ST(b, sp);
  ST(dp, d); ST(dp, b); ST(dp, g); ST(dp, dp); ST(dp, sp);
  ST(sp, g); ST(sp, b); ST(sp, s); ST(sp, dp); ST(sp, sp);
  ST(g, g); ST(g, b); ST(g, dp); ST(g, sp);
#undef ST
  return n;
}

static double dmin(double a, double b) { return a < b ? a : b; }

static b3m_t *b3_members(xgo_circuit *c) {
  xgo_type *T = &c->T[XG_DEV_BSIM3];
  if (!T->m) T->m = calloc((size_t)T->n + 1, sizeof(b3m_t));
  return (b3m_t *)T->m;
}

/* updateIntermediateVars + Master::updateState for one instance. */
static void b3_update(xgo_circuit *c, int i, xgo_io *io, b3m_t *m, b3mem_t *mem) {
  const xgo_type *T = &c->T[XG_DEV_BSIM3];
  const xg_load_flags *fl = io->fl;
  const int *L = T->lid + (int64_t)i * 6;
  const int li_Drain = L[0], li_Gate = L[1], li_Source = L[2], li_Bulk = L[3];
  const int li_DrainPrime = L[4], li_SourcePrime = L[5];
#define PP(k) P(T, k, i)
  const int dtype = (int)PP(XG_B3_DTYPE);
  const int mobMod = (int)PP(XG_B3_MOBMOD), capMod = (int)PP(XG_B3_CAPMOD);
  const double xpart = PP(XG_B3_XPART), tox = PP(XG_B3_TOX), cox = PP(XG_B3_COX);
  const double factor1 = PP(XG_B3_FACTOR1);
  const double gmin = c->opt.gmin;
  const int OFF = ((int)PP(XG_B3_FLAGS)) & 1;
  double *sto = io->sto + T->sto0 + (int64_t)i * 5;
  double *sta = io->sta + T->sta0 + (int64_t)i * 12;
  const double *csto = io->sto_curr + T->sto0 + (int64_t)i * 5;
  enum { O_VBD, O_VBS, O_VGS, O_VDS, O_VON };
  enum { S_QB, S_QG, S_QD, S_QBS, S_QBD };

  double SourceSatCurrent, DrainSatCurrent, vgdo, VgstNVt, ExpVgst;
  double czbd, czbdsw, czbdswg, czbs, czbssw, czbsswg, evbd, evbs, arg, sarg;
  double Vfbeff, dVfbeff_dVg, dVfbeff_dVb, V3, V4, MJ, MJSW, MJSWG;
  double Vds, Vgs, Vbs, Vgs_eff, dVgs_eff_dVg, Vfb, Phis, dPhis_dVb, sqrtPhis, dsqrtPhis_dVb;
  double Vth, dVth_dVb, dVth_dVd, Vgst, dVgst_dVg, dVgst_dVb, Nvtm, Vtm;
  double n, dn_dVb, dn_dVd, voffcv, noff, dnoff_dVd, dnoff_dVb;
  double ExpArg, V0, CoxWLcen, QovCox, LINK, DeltaPhi, dDeltaPhi_dVg, dDeltaPhi_dVd, dDeltaPhi_dVb;
  double Cox, Tox, Tcen, dTcen_dVg, dTcen_dVd, dTcen_dVb, Ccen, Coxeff, dCoxeff_dVg, dCoxeff_dVd, dCoxeff_dVb;
  double Denomi, dDenomi_dVg, dDenomi_dVd, dDenomi_dVb, ueff, dueff_dVg, dueff_dVd, dueff_dVb;
  double Esat, Vdsat, EsatL, dEsatL_dVg, dEsatL_dVd, dEsatL_dVb;
  double dVdsat_dVg, dVdsat_dVb, dVdsat_dVd, Vasat, dAlphaz_dVg, dAlphaz_dVb;
  double dVasat_dVg, dVasat_dVb, dVasat_dVd, Va, dVa_dVd, dVa_dVg, dVa_dVb;
  double Vbseff, dVbseff_dVb, VbseffCV, dVbseffCV_dVb, Arg1, One_Third_CoxWL, Two_Third_CoxWL, Alphaz;
  double T0, dT0_dVg, dT0_dVd, dT0_dVb, T1, dT1_dVg, dT1_dVd, dT1_dVb, T2, dT2_dVg, dT2_dVd, dT2_dVb;
  double T3, dT3_dVg, dT3_dVd, dT3_dVb, T4, T5, T6, T7, T8, T9, T10, T11, T12;
  double tmp, Abulk, dAbulk_dVb, Abulk0, dAbulk0_dVb;
  double VACLM, dVACLM_dVg, dVACLM_dVd, dVACLM_dVb, VADIBL, dVADIBL_dVg, dVADIBL_dVd, dVADIBL_dVb;
  double Xdep, dXdep_dVb, lt1, dlt1_dVb, ltw, dltw_dVb, Delt_vth, dDelt_vth_dVb, Theta0, dTheta0_dVb;
  double TempRatio, tmp1, tmp2, tmp3, tmp4, DIBL_Sft, dDIBL_Sft_dVd, Lambda, dLambda_dVg, a1;
  double Vgsteff, dVgsteff_dVg, dVgsteff_dVd, dVgsteff_dVb, Vdseff, dVdseff_dVg, dVdseff_dVd, dVdseff_dVb;
  double VdseffCV, dVdseffCV_dVg, dVdseffCV_dVd, dVdseffCV_dVb, diffVds, dAbulk_dVg;
  double beta, dbeta_dVg, dbeta_dVd, dbeta_dVb, gche, dgche_dVg, dgche_dVd, dgche_dVb;
  double fgche1, dfgche1_dVg, dfgche1_dVd, dfgche1_dVb, fgche2, dfgche2_dVg, dfgche2_dVd, dfgche2_dVb;
  double Idl, dIdl_dVg, dIdl_dVd, dIdl_dVb, Idsa, dIdsa_dVg, dIdsa_dVd, dIdsa_dVb, Ids, Gm, Gds, Gmb, Isub;
  double Gbd, Gbg, Gbb, VASCBE, dVASCBE_dVg, dVASCBE_dVd, dVASCBE_dVb, CoxWovL;
  double Rds, dRds_dVg, dRds_dVb, WVCox, WVCoxRds, Vgst2Vtm, VdsatCV, dVdsatCV_dVg, dVdsatCV_dVb;
  double Leff, Weff, dWeff_dVg, dWeff_dVb, AbulkCV, dAbulkCV_dVb, qinoi;
  double Cgg1, Cgb1, Cgd1, Cbg1, Cbb1, Cbd1, Qac0, Qsub0, dQac0_dVg, dQac0_dVb, dQsub0_dVg, dQsub0_dVd, dQsub0_dVb;
  double von_local, vbs_old, vbd_old, vgs_old, vds_old;
  double qgate, qdrn, qsrc, qbulk, cggb, cgsb, cgdb, cdgb, cdsb, cddb, cbgb, cbsb, cbdb;
  double Cgg, Cgd, Cgb, Cbg, Cbd, Cbb, Csg, Csd, Csb, CoxWL, qinv;
  double qgdo, qgso, cgdo, cgso, capbs, capbd, qbs, qbd, gbs, gbd, cbs, cbd;
  (void)qinv;
  int Check = 1;
  int ChargeComputationNeeded = (fl->tranop || fl->acop || fl->transient) ? 1 : 0;
  int mode;

  const double *sol = io->sol;
  double Vd = sol[li_Drain], Vg = sol[li_Gate], Vs = sol[li_Source], Vb = sol[li_Bulk];
  double Vsp = sol[li_SourcePrime], Vdp = sol[li_DrainPrime];
  double Vddp = Vd - Vdp, Vssp = Vs - Vsp, Vbsp = Vb - Vsp, Vgsp = Vg - Vsp;
  double Vdpsp = Vdp - Vsp;
  double vbs = dtype * Vbsp, vgs = dtype * Vgsp, vds = dtype * Vdpsp;
  double vbd = vbs - vds, vgd = vgs - vds, vgb;
  int origFlag = 1;
  const double vgs_orig = vgs, vds_orig = vds, vbs_orig = vbs, vbd_orig = vbd, vgd_orig = vgd;

  if (fl->init_jct && !OFF && c->opt.voltlim) {
    /* inputOP with an all-zero flag vector takes the same branch */
    vbs = 0.0;
    vgs = dtype * PP(XG_B3_VTH0) + 0.1;
    vds = 0.1;
    origFlag = 0;
    vbd = vbs - vds;
    vgd = vgs - vds;
  } else if ((fl->init_fix || fl->init_jct) && OFF) {
    vbs = vgs = vds = 0;
  }
  if (fl->newton_iter == 0) {
    if (!fl->dcop) {
      vbs_old = csto[O_VBS]; vbd_old = csto[O_VBD]; vgs_old = csto[O_VGS];
      vds_old = csto[O_VDS]; von_local = csto[O_VON];
    } else {
      vbs_old = vbs; vbd_old = vbd; vgs_old = vgs; vds_old = vds; von_local = 0.0;
    }
  } else {
    vbs_old = sto[O_VBS]; vbd_old = sto[O_VBD]; vgs_old = sto[O_VGS];
    vds_old = sto[O_VDS]; von_local = sto[O_VON];
  }
  vgdo = vgs_old - vds_old;
  if (c->opt.voltlim && !(fl->init_fix && OFF)) {
    const double vt0 = KBOLTZ * (27.0 + CTOK) / KQ;
    const double vcrit = PP(XG_B3_VCRIT);
    if (fl->newton_iter >= 0) {
      if (vds_old >= 0.0) {
        vgs = xgo_fetlim(vgs, vgs_old, von_local);
        vds = vgs - vgd;
        vds = xgo_limvds(vds, vds_old);
        vgd = vgs - vds;
      } else {
        vgd = xgo_fetlim(vgd, vgdo, von_local);
        vds = vgs - vgd;
        vds = -xgo_limvds(-vds, -vds_old);
        vgs = vgd + vds;
      }
      if (vds >= 0.0) {
        vbs = xgo_pnjlim(vbs, vbs_old, vt0, vcrit, &Check);
        vbd = vbs - vds;
      } else {
        vbd = xgo_pnjlim(vbd, vbd_old, vt0, vcrit, &Check);
        vbs = vbd + vds;
      }
    }
    if (vgs_orig != vgs || vds_orig != vds || vbs_orig != vbs || vbd_orig != vbd || vgd_orig != vgd)
      origFlag = 0;
  }
  vbd = vbs - vds;
  vgd = vgs - vds;
  vgb = vgs - vbs;

  const double vtm = PP(XG_B3_VTM);
  Nvtm = vtm * PP(XG_B3_NJ);
  const double sourceArea = PP(XG_B3_AS), sourcePerimeter = PP(XG_B3_PS);
  const double drainArea = PP(XG_B3_AD), drainPerimeter = PP(XG_B3_PD);
  const double jctTempSatCurDensity = PP(XG_B3_JSTEMP);
  const double jctSidewallTempSatCurDensity = PP(XG_B3_JSWTEMP);
  const double ijth = PP(XG_B3_IJTH);
  if ((sourceArea <= 0.0) && (sourcePerimeter <= 0.0)) SourceSatCurrent = 1.0e-14;
  else SourceSatCurrent = sourceArea * jctTempSatCurDensity + sourcePerimeter * jctSidewallTempSatCurDensity;
  if (SourceSatCurrent <= 0.0) {
    gbs = gmin;
    cbs = gbs * vbs;
  } else if (ijth == 0.0) {
    evbs = exp(vbs / Nvtm);
    gbs = SourceSatCurrent * evbs / Nvtm + gmin;
    cbs = SourceSatCurrent * (evbs - 1.0) + gmin * vbs;
  } else if (vbs < PP(XG_B3_VJSM)) {
    evbs = exp(vbs / Nvtm);
    gbs = SourceSatCurrent * evbs / Nvtm + gmin;
    cbs = SourceSatCurrent * (evbs - 1.0) + gmin * vbs;
  } else {
    T0 = PP(XG_B3_ISEVJSM) / Nvtm;
    gbs = T0 + gmin;
    cbs = PP(XG_B3_ISEVJSM) - SourceSatCurrent + T0 * (vbs - PP(XG_B3_VJSM)) + gmin * vbs;
  }
  if ((drainArea <= 0.0) && (drainPerimeter <= 0.0)) DrainSatCurrent = 1.0e-14;
  else DrainSatCurrent = drainArea * jctTempSatCurDensity + drainPerimeter * jctSidewallTempSatCurDensity;
  if (DrainSatCurrent <= 0.0) {
    gbd = gmin;
    cbd = gbd * vbd;
  } else if (ijth == 0.0) {
    evbd = exp(vbd / Nvtm);
    gbd = DrainSatCurrent * evbd / Nvtm + gmin;
    cbd = DrainSatCurrent * (evbd - 1.0) + gmin * vbd;
  } else if (vbd < PP(XG_B3_VJDM)) {
    evbd = exp(vbd / Nvtm);
    gbd = DrainSatCurrent * evbd / Nvtm + gmin;
    cbd = DrainSatCurrent * (evbd - 1.0) + gmin * vbd;
  } else {
    T0 = PP(XG_B3_ISEVJDM) / Nvtm;
    gbd = T0 + gmin;
    cbd = PP(XG_B3_ISEVJDM) - DrainSatCurrent + T0 * (vbd - PP(XG_B3_VJDM)) + gmin * vbd;
  }

  if (vds >= 0.0) {
    mode = 1; Vds = vds; Vgs = vgs; Vbs = vbs;
  } else {
    mode = -1; Vds = -vds; Vgs = vgd; Vbs = vbd;
  }

  const double vbsc = PP(XG_B3_VBSC), phi = PP(XG_B3_PHI), phis3 = PP(XG_B3_PHIS3);
  const double sqrtPhi = PP(XG_B3_SQRTPHI), Xdep0 = PP(XG_B3_XDEP0);
  T0 = Vbs - vbsc - 0.001;
  double T1global = sqrt(T0 * T0 - 0.004 * vbsc);
  Vbseff = vbsc + 0.5 * (T0 + T1global);
  dVbseff_dVb = 0.5 * (1.0 + T0 / T1global);
  if (Vbseff < Vbs) Vbseff = Vbs;
  if (Vbseff > 0.0) {
    T0 = phi / (phi + Vbseff);
    Phis = phi * T0;
    dPhis_dVb = -T0 * T0;
    sqrtPhis = phis3 / (phi + 0.5 * Vbseff);
    dsqrtPhis_dVb = -0.5 * sqrtPhis * sqrtPhis / phis3;
  } else {
    Phis = phi - Vbseff;
    dPhis_dVb = -1.0;
    sqrtPhis = sqrt(Phis);
    dsqrtPhis_dVb = -0.5 / sqrtPhis;
  }
  Xdep = Xdep0 * sqrtPhis / sqrtPhi;
  dXdep_dVb = (Xdep0 / sqrtPhi) * dsqrtPhis_dVb;
  Leff = PP(XG_B3_LEFF);
  Vtm = vtm;
  T3 = sqrt(Xdep);
  V0 = PP(XG_B3_VBI) - phi;
  const double dvt2 = PP(XG_B3_DVT2), dvt2w = PP(XG_B3_DVT2W);
  T0 = dvt2 * Vbseff;
  if (T0 >= -0.5) {
    T1 = 1.0 + T0;
    T2 = dvt2;
  } else {
    T4 = 1.0 / (3.0 + 8.0 * T0);
    T1 = (1.0 + 3.0 * T0) * T4;
    T2 = dvt2 * T4 * T4;
  }
  lt1 = factor1 * T3 * T1;
  dlt1_dVb = factor1 * (0.5 / T3 * T1 * dXdep_dVb + T3 * T2);
  T0 = dvt2w * Vbseff;
  if (T0 >= -0.5) {
    T1 = 1.0 + T0;
    T2 = dvt2w;
  } else {
    T4 = 1.0 / (3.0 + 8.0 * T0);
    T1 = (1.0 + 3.0 * T0) * T4;
    T2 = dvt2w * T4 * T4;
  }
  ltw = factor1 * T3 * T1;
  dltw_dVb = factor1 * (0.5 / T3 * T1 * dXdep_dVb + T3 * T2);
  T0 = -0.5 * PP(XG_B3_DVT1) * Leff / lt1;
  if (T0 > -EXP_THRESHOLD) {
    T1 = exp(T0);
    Theta0 = T1 * (1.0 + 2.0 * T1);
    dT1_dVb = -T0 / lt1 * T1 * dlt1_dVb;
    dTheta0_dVb = (1.0 + 4.0 * T1) * dT1_dVb;
  } else {
    T1 = MIN_EXP;
    Theta0 = T1 * (1.0 + 2.0 * T1);
    dTheta0_dVb = 0.0;
  }
  double thetavth = PP(XG_B3_DVT0) * Theta0;
  Delt_vth = thetavth * V0;
  dDelt_vth_dVb = PP(XG_B3_DVT0) * dTheta0_dVb * V0;
  const double weff = PP(XG_B3_WEFF);
  T0 = -0.5 * PP(XG_B3_DVT1W) * weff * Leff / ltw;
  if (T0 > -EXP_THRESHOLD) {
    T1 = exp(T0);
    T2 = T1 * (1.0 + 2.0 * T1);
    dT1_dVb = -T0 / ltw * T1 * dltw_dVb;
    dT2_dVb = (1.0 + 4.0 * T1) * dT1_dVb;
  } else {
    T1 = MIN_EXP;
    T2 = T1 * (1.0 + 2.0 * T1);
    dT2_dVb = 0.0;
  }
  T0 = PP(XG_B3_DVT0W) * T2;
  T2 = T0 * V0;
  dT2_dVb = PP(XG_B3_DVT0W) * dT2_dVb * V0;
  TempRatio = PP(XG_B3_TEMP) / PP(XG_B3_TNOM) - 1.0;
  const double k1ox = PP(XG_B3_K1OX), kt2 = PP(XG_B3_KT2);
  T0 = sqrt(1.0 + PP(XG_B3_NLX) / Leff);
  T1 = k1ox * (T0 - 1.0) * sqrtPhi + (PP(XG_B3_KT1) + PP(XG_B3_KT1L) / Leff + kt2 * Vbseff) * TempRatio;
  tmp2 = tox * phi / (weff + PP(XG_B3_W0));
  const double etab = PP(XG_B3_ETAB), theta0vb0 = PP(XG_B3_THETA0VB0);
  T3 = PP(XG_B3_ETA0) + etab * Vbseff;
  if (T3 < 1.0e-4) {
    T9 = 1.0 / (3.0 - 2.0e4 * T3);
    T3 = (2.0e-4 - T3) * T9;
    T4 = T9 * T9;
  } else {
    T4 = 1.0;
  }
  dDIBL_Sft_dVd = T3 * theta0vb0;
  DIBL_Sft = dDIBL_Sft_dVd * Vds;
  const double k2ox = PP(XG_B3_K2OX), k3b = PP(XG_B3_K3B);
  Vth = dtype * PP(XG_B3_VTH0) - PP(XG_B3_K1) * sqrtPhi + k1ox * sqrtPhis - k2ox * Vbseff - Delt_vth -
        T2 + (PP(XG_B3_K3) + k3b * Vbseff) * tmp2 + T1 - DIBL_Sft;
  double von = Vth;
  dVth_dVb = k1ox * dsqrtPhis_dVb - k2ox - dDelt_vth_dVb - dT2_dVb + k3b * tmp2 -
             etab * Vds * theta0vb0 * T4 + kt2 * TempRatio;
  dVth_dVd = -dDIBL_Sft_dVd;

  const double cdscb = PP(XG_B3_CDSCB), cdscd = PP(XG_B3_CDSCD);
  tmp2 = PP(XG_B3_NFACTOR) * EPSSI / Xdep;
  tmp3 = PP(XG_B3_CDSC) + cdscb * Vbseff + cdscd * Vds;
  tmp4 = (tmp2 + tmp3 * Theta0 + PP(XG_B3_CIT)) / cox;
  if (tmp4 >= -0.5) {
    n = 1.0 + tmp4;
    dn_dVb = (-tmp2 / Xdep * dXdep_dVb + tmp3 * dTheta0_dVb + cdscb * Theta0) / cox;
    dn_dVd = cdscd * Theta0 / cox;
  } else {
    T0 = 1.0 / (3.0 + 8.0 * tmp4);
    n = (1.0 + 3.0 * tmp4) * T0;
    T0 *= T0;
    dn_dVb = (-tmp2 / Xdep * dXdep_dVb + tmp3 * dTheta0_dVb + cdscb * Theta0) / cox * T0;
    dn_dVd = cdscd * Theta0 / cox * T0;
  }

  T0 = PP(XG_B3_VFB) + phi;
  const double ngate = PP(XG_B3_NGATE);
  if ((ngate > 1.e18) && (ngate < 1.e25) && (Vgs > T0)) {
    T1 = 1.0e6 * KQ * EPSSI * ngate / (cox * cox);
    T4 = sqrt(1.0 + 2.0 * (Vgs - T0) / T1);
    T2 = T1 * (T4 - 1.0);
    T3 = 0.5 * T2 * T2 / T1;
    T7 = 1.12 - T3 - 0.05;
    T6 = sqrt(T7 * T7 + 0.224);
    T5 = 1.12 - 0.5 * (T7 + T6);
    Vgs_eff = Vgs - T5;
    dVgs_eff_dVg = 1.0 - (0.5 - 0.5 / T4) * (1.0 + T7 / T6);
  } else {
    Vgs_eff = Vgs;
    dVgs_eff_dVg = 1.0;
  }
  Vgst = Vgs_eff - Vth;

  const double voff = PP(XG_B3_VOFF), cdep0 = PP(XG_B3_CDEP0);
  T10 = 2.0 * n * Vtm;
  VgstNVt = Vgst / T10;
  ExpArg = (2.0 * voff - Vgst) / T10;
  if (VgstNVt > EXP_THRESHOLD) {
    Vgsteff = Vgst;
    dVgsteff_dVg = dVgs_eff_dVg;
    dVgsteff_dVd = -dVth_dVd;
    dVgsteff_dVb = -dVth_dVb;
  } else if (ExpArg > EXP_THRESHOLD) {
    T0 = (Vgst - voff) / (n * Vtm);
    ExpVgst = exp(T0);
    Vgsteff = Vtm * cdep0 / cox * ExpVgst;
    dVgsteff_dVg = Vgsteff / (n * Vtm);
    dVgsteff_dVd = -dVgsteff_dVg * (dVth_dVd + T0 * Vtm * dn_dVd);
    dVgsteff_dVb = -dVgsteff_dVg * (dVth_dVb + T0 * Vtm * dn_dVb);
    dVgsteff_dVg *= dVgs_eff_dVg;
  } else {
    ExpVgst = exp(VgstNVt);
    T1 = T10 * log(1.0 + ExpVgst);
    dT1_dVg = ExpVgst / (1.0 + ExpVgst);
    dT1_dVb = -dT1_dVg * (dVth_dVb + Vgst / n * dn_dVb) + T1 / n * dn_dVb;
    dT1_dVd = -dT1_dVg * (dVth_dVd + Vgst / n * dn_dVd) + T1 / n * dn_dVd;
    dT2_dVg = -cox / (Vtm * cdep0) * exp(ExpArg);
    T2 = 1.0 - T10 * dT2_dVg;
    dT2_dVd = -dT2_dVg * (dVth_dVd - 2.0 * Vtm * ExpArg * dn_dVd) + (T2 - 1.0) / n * dn_dVd;
    dT2_dVb = -dT2_dVg * (dVth_dVb - 2.0 * Vtm * ExpArg * dn_dVb) + (T2 - 1.0) / n * dn_dVb;
    Vgsteff = T1 / T2;
    T3 = T2 * T2;
    dVgsteff_dVg = (T2 * dT1_dVg - T1 * dT2_dVg) / T3 * dVgs_eff_dVg;
    dVgsteff_dVd = (T2 * dT1_dVd - T1 * dT2_dVd) / T3;
    dVgsteff_dVb = (T2 * dT1_dVb - T1 * dT2_dVb) / T3;
  }

  const double dwg = PP(XG_B3_DWG), dwb = PP(XG_B3_DWB);
  T9 = sqrtPhis - sqrtPhi;
  Weff = weff - 2.0 * (dwg * Vgsteff + dwb * T9);
  dWeff_dVg = -2.0 * dwg;
  dWeff_dVb = -2.0 * dwb * dsqrtPhis_dVb;
  if (Weff < 2.0e-8) {
    T0 = 1.0 / (6.0e-8 - 2.0 * Weff);
    Weff = 2.0e-8 * (4.0e-8 - Weff) * T0;
    T0 *= T0 * 4.0e-16;
    dWeff_dVg *= T0;
    dWeff_dVb *= T0;
  }
  const double prwg = PP(XG_B3_PRWG), prwb = PP(XG_B3_PRWB), rds0 = PP(XG_B3_RDS0);
  T0 = prwg * Vgsteff + prwb * T9;
  if (T0 >= -0.9) {
    Rds = rds0 * (1.0 + T0);
    dRds_dVg = rds0 * prwg;
    dRds_dVb = rds0 * prwb * dsqrtPhis_dVb;
  } else {
    T1 = 1.0 / (17.0 + 20.0 * T0);
    Rds = rds0 * (0.8 + T0) * T1;
    T1 *= T1;
    dRds_dVg = rds0 * prwg * T1;
    dRds_dVb = rds0 * prwb * dsqrtPhis_dVb * T1;
  }

  T1 = 0.5 * k1ox / sqrtPhis;
  dT1_dVb = -T1 / sqrtPhis * dsqrtPhis_dVb;
  T9 = sqrt(PP(XG_B3_XJ) * Xdep);
  tmp1 = Leff + 2.0 * T9;
  T5 = Leff / tmp1;
  const double a0 = PP(XG_B3_A0);
  tmp2 = a0 * T5;
  tmp3 = weff + PP(XG_B3_B1);
  tmp4 = PP(XG_B3_B0) / tmp3;
  T2 = tmp2 + tmp4;
  dT2_dVb = -T9 / tmp1 / Xdep * dXdep_dVb;
  T6 = T5 * T5;
  T7 = T5 * T6;
  Abulk0 = 1.0 + T1 * T2;
  dAbulk0_dVb = T1 * tmp2 * dT2_dVb + T2 * dT1_dVb;
  T8 = PP(XG_B3_AGS) * a0 * T7;
  dAbulk_dVg = -T1 * T8;
  Abulk = Abulk0 + dAbulk_dVg * Vgsteff;
  dAbulk_dVb = dAbulk0_dVb - T8 * Vgsteff * (dT1_dVb + 3.0 * T1 * dT2_dVb);
  if (Abulk0 < 0.1) {
    T9 = 1.0 / (3.0 - 20.0 * Abulk0);
    Abulk0 = (0.2 - Abulk0) * T9;
    dAbulk0_dVb *= T9 * T9;
  }
  if (Abulk < 0.1) {
    T9 = 1.0 / (3.0 - 20.0 * Abulk);
    Abulk = (0.2 - Abulk) * T9;
    T10 = T9 * T9;
    dAbulk_dVb *= T10;
    dAbulk_dVg *= T10;
  }
  const double keta = PP(XG_B3_KETA);
  T2 = keta * Vbseff;
  if (T2 >= -0.9) {
    T0 = 1.0 / (1.0 + T2);
    dT0_dVb = -keta * T0 * T0;
  } else {
    T1 = 1.0 / (0.8 + T2);
    T0 = (17.0 + 20.0 * T2) * T1;
    dT0_dVb = -keta * T1 * T1;
  }
  dAbulk_dVg *= T0;
  dAbulk_dVb = dAbulk_dVb * T0 + Abulk * dT0_dVb;
  dAbulk0_dVb = dAbulk0_dVb * T0 + Abulk0 * dT0_dVb;
  Abulk *= T0;
  Abulk0 *= T0;

  const double ua = PP(XG_B3_UA), ub = PP(XG_B3_UB), uc = PP(XG_B3_UC);
  if (mobMod == 1) {
    T0 = Vgsteff + Vth + Vth;
    T2 = ua + uc * Vbseff;
    T3 = T0 / tox;
    T5 = T3 * (T2 + ub * T3);
    dDenomi_dVg = (T2 + 2.0 * ub * T3) / tox;
    dDenomi_dVd = dDenomi_dVg * 2.0 * dVth_dVd;
    dDenomi_dVb = dDenomi_dVg * 2.0 * dVth_dVb + uc * T3;
  } else if (mobMod == 2) {
    T5 = Vgsteff / tox * (ua + uc * Vbseff + ub * Vgsteff / tox);
    dDenomi_dVg = (ua + uc * Vbseff + 2.0 * ub * Vgsteff / tox) / tox;
    dDenomi_dVd = 0.0;
    dDenomi_dVb = Vgsteff * uc / tox;
  } else {
    T0 = Vgsteff + Vth + Vth;
    T2 = 1.0 + uc * Vbseff;
    T3 = T0 / tox;
    T4 = T3 * (ua + ub * T3);
    T5 = T4 * T2;
    dDenomi_dVg = (ua + 2.0 * ub * T3) * T2 / tox;
    dDenomi_dVd = dDenomi_dVg * 2.0 * dVth_dVd;
    dDenomi_dVb = dDenomi_dVg * 2.0 * dVth_dVb + uc * T4;
  }
  if (T5 >= -0.8) {
    Denomi = 1.0 + T5;
  } else {
    T9 = 1.0 / (7.0 + 10.0 * T5);
    Denomi = (0.6 + T5) * T9;
    T9 *= T9;
    dDenomi_dVg *= T9;
    dDenomi_dVd *= T9;
    dDenomi_dVb *= T9;
  }
  ueff = PP(XG_B3_U0TEMP) / Denomi;
  T9 = -ueff / Denomi;
  dueff_dVg = T9 * dDenomi_dVg;
  dueff_dVd = T9 * dDenomi_dVd;
  dueff_dVb = T9 * dDenomi_dVb;

  const double vsattemp = PP(XG_B3_VSATTEMP);
  WVCox = Weff * vsattemp * cox;
  WVCoxRds = WVCox * Rds;
  Esat = 2.0 * vsattemp / ueff;
  EsatL = Esat * Leff;
  T0 = -EsatL / ueff;
  dEsatL_dVg = T0 * dueff_dVg;
  dEsatL_dVd = T0 * dueff_dVd;
  dEsatL_dVb = T0 * dueff_dVb;

  a1 = PP(XG_B3_A1);
  const double a2 = PP(XG_B3_A2);
  if (a1 == 0.0) {
    Lambda = a2;
    dLambda_dVg = 0.0;
  } else if (a1 > 0.0) {
    T0 = 1.0 - a2;
    T1 = T0 - a1 * Vgsteff - 0.0001;
    T2 = sqrt(T1 * T1 + 0.0004 * T0);
    Lambda = a2 + T0 - 0.5 * (T1 + T2);
    dLambda_dVg = 0.5 * a1 * (1.0 + T1 / T2);
  } else {
    T1 = a2 + a1 * Vgsteff - 0.0001;
    T2 = sqrt(T1 * T1 + 0.0004 * a2);
    Lambda = 0.5 * (T1 + T2);
    dLambda_dVg = 0.5 * a1 * (1.0 + T1 / T2);
  }
  Vgst2Vtm = Vgsteff + 2.0 * Vtm;
  if (Rds > 0) {
    tmp2 = dRds_dVg / Rds + dWeff_dVg / Weff;
    tmp3 = dRds_dVb / Rds + dWeff_dVb / Weff;
  } else {
    tmp2 = dWeff_dVg / Weff;
    tmp3 = dWeff_dVb / Weff;
  }
  if ((Rds == 0.0) && (Lambda == 1.0)) {
    T0 = 1.0 / (Abulk * EsatL + Vgst2Vtm);
    tmp1 = 0.0;
    T1 = T0 * T0;
    T2 = Vgst2Vtm * T0;
    T3 = EsatL * Vgst2Vtm;
    Vdsat = T3 * T0;
    dT0_dVg = -(Abulk * dEsatL_dVg + EsatL * dAbulk_dVg + 1.0) * T1;
    dT0_dVd = -(Abulk * dEsatL_dVd) * T1;
    dT0_dVb = -(Abulk * dEsatL_dVb + dAbulk_dVb * EsatL) * T1;
    dVdsat_dVg = T3 * dT0_dVg + T2 * dEsatL_dVg + EsatL * T0;
    dVdsat_dVd = T3 * dT0_dVd + T2 * dEsatL_dVd;
    dVdsat_dVb = T3 * dT0_dVb + T2 * dEsatL_dVb;
  } else {
    tmp1 = dLambda_dVg / (Lambda * Lambda);
    T9 = Abulk * WVCoxRds;
    T8 = Abulk * T9;
    T7 = Vgst2Vtm * T9;
    T6 = Vgst2Vtm * WVCoxRds;
    T0 = 2.0 * Abulk * (T9 - 1.0 + 1.0 / Lambda);
    dT0_dVg = 2.0 * (T8 * tmp2 - Abulk * tmp1 + (2.0 * T9 + 1.0 / Lambda - 1.0) * dAbulk_dVg);
    dT0_dVb = 2.0 * (T8 * (2.0 / Abulk * dAbulk_dVb + tmp3) + (1.0 / Lambda - 1.0) * dAbulk_dVb);
    dT0_dVd = 0.0;
    T1 = Vgst2Vtm * (2.0 / Lambda - 1.0) + Abulk * EsatL + 3.0 * T7;
    dT1_dVg = (2.0 / Lambda - 1.0) - 2.0 * Vgst2Vtm * tmp1 + Abulk * dEsatL_dVg +
              EsatL * dAbulk_dVg + 3.0 * (T9 + T7 * tmp2 + T6 * dAbulk_dVg);
    dT1_dVb = Abulk * dEsatL_dVb + EsatL * dAbulk_dVb + 3.0 * (T6 * dAbulk_dVb + T7 * tmp3);
    dT1_dVd = Abulk * dEsatL_dVd;
    T2 = Vgst2Vtm * (EsatL + 2.0 * T6);
    dT2_dVg = EsatL + Vgst2Vtm * dEsatL_dVg + T6 * (4.0 + 2.0 * Vgst2Vtm * tmp2);
    dT2_dVb = Vgst2Vtm * (dEsatL_dVb + 2.0 * T6 * tmp3);
    dT2_dVd = Vgst2Vtm * dEsatL_dVd;
    T3 = sqrt(T1 * T1 - 2.0 * T0 * T2);
    Vdsat = (T1 - T3) / T0;
    dT3_dVg = (T1 * dT1_dVg - 2.0 * (T0 * dT2_dVg + T2 * dT0_dVg)) / T3;
    dT3_dVd = (T1 * dT1_dVd - 2.0 * (T0 * dT2_dVd + T2 * dT0_dVd)) / T3;
    dT3_dVb = (T1 * dT1_dVb - 2.0 * (T0 * dT2_dVb + T2 * dT0_dVb)) / T3;
    (void)dT3_dVg; (void)dT3_dVd; (void)dT3_dVb;
    dVdsat_dVg = (dT1_dVg - (T1 * dT1_dVg - dT0_dVg * T2 - T0 * dT2_dVg) / T3 - Vdsat * dT0_dVg) / T0;
    dVdsat_dVb = (dT1_dVb - (T1 * dT1_dVb - dT0_dVb * T2 - T0 * dT2_dVb) / T3 - Vdsat * dT0_dVb) / T0;
    dVdsat_dVd = (dT1_dVd - (T1 * dT1_dVd - T0 * dT2_dVd) / T3) / T0;
  }

  const double delta = PP(XG_B3_DELTA);
  T1 = Vdsat - Vds - delta;
  dT1_dVg = dVdsat_dVg;
  dT1_dVd = dVdsat_dVd - 1.0;
  dT1_dVb = dVdsat_dVb;
  T2 = sqrt(T1 * T1 + 4.0 * delta * Vdsat);
  T0 = T1 / T2;
  T3 = 2.0 * delta / T2;
  dT2_dVg = T0 * dT1_dVg + T3 * dVdsat_dVg;
  dT2_dVd = T0 * dT1_dVd + T3 * dVdsat_dVd;
  dT2_dVb = T0 * dT1_dVb + T3 * dVdsat_dVb;
  Vdseff = Vdsat - 0.5 * (T1 + T2);
  dVdseff_dVg = dVdsat_dVg - 0.5 * (dT1_dVg + dT2_dVg);
  dVdseff_dVd = dVdsat_dVd - 0.5 * (dT1_dVd + dT2_dVd);
  dVdseff_dVb = dVdsat_dVb - 0.5 * (dT1_dVb + dT2_dVb);
  if (Vds == 0.0) {
    Vdseff = 0.0;
    dVdseff_dVg = 0.0;
    dVdseff_dVb = 0.0;
  }

  tmp4 = 1.0 - 0.5 * Abulk * Vdsat / Vgst2Vtm;
  T9 = WVCoxRds * Vgsteff;
  T8 = T9 / Vgst2Vtm;
  T0 = EsatL + Vdsat + 2.0 * T9 * tmp4;
  T7 = 2.0 * WVCoxRds * tmp4;
  dT0_dVg = dEsatL_dVg + dVdsat_dVg + T7 * (1.0 + tmp2 * Vgsteff) -
            T8 * (Abulk * dVdsat_dVg - Abulk * Vdsat / Vgst2Vtm + Vdsat * dAbulk_dVg);
  dT0_dVb = dEsatL_dVb + dVdsat_dVb + T7 * tmp3 * Vgsteff - T8 * (dAbulk_dVb * Vdsat + Abulk * dVdsat_dVb);
  dT0_dVd = dEsatL_dVd + dVdsat_dVd - T8 * Abulk * dVdsat_dVd;
  T9 = WVCoxRds * Abulk;
  T1 = 2.0 / Lambda - 1.0 + T9;
  dT1_dVg = -2.0 * tmp1 + WVCoxRds * (Abulk * tmp2 + dAbulk_dVg);
  dT1_dVb = dAbulk_dVb * WVCoxRds + T9 * tmp3;
  Vasat = T0 / T1;
  dVasat_dVg = (dT0_dVg - Vasat * dT1_dVg) / T1;
  dVasat_dVb = (dT0_dVb - Vasat * dT1_dVb) / T1;
  dVasat_dVd = dT0_dVd / T1;
  if (Vdseff > Vds) Vdseff = Vds;
  diffVds = Vds - Vdseff;

  const double pclm = PP(XG_B3_PCLM), litl = PP(XG_B3_LITL);
  if ((pclm > 0.0) && (diffVds > 1.0e-10)) {
    T0 = 1.0 / (pclm * Abulk * litl);
    dT0_dVb = -T0 / Abulk * dAbulk_dVb;
    dT0_dVg = -T0 / Abulk * dAbulk_dVg;
    T2 = Vgsteff / EsatL;
    T1 = Leff * (Abulk + T2);
    dT1_dVg = Leff * ((1.0 - T2 * dEsatL_dVg) / EsatL + dAbulk_dVg);
    dT1_dVb = Leff * (dAbulk_dVb - T2 * dEsatL_dVb / EsatL);
    dT1_dVd = -T2 * dEsatL_dVd / Esat;
    T9 = T0 * T1;
    VACLM = T9 * diffVds;
    dVACLM_dVg = T0 * dT1_dVg * diffVds - T9 * dVdseff_dVg + T1 * diffVds * dT0_dVg;
    dVACLM_dVb = (dT0_dVb * T1 + T0 * dT1_dVb) * diffVds - T9 * dVdseff_dVb;
    dVACLM_dVd = T0 * dT1_dVd * diffVds + T9 * (1.0 - dVdseff_dVd);
  } else {
    VACLM = MAX_EXP;
    dVACLM_dVd = dVACLM_dVg = dVACLM_dVb = 0.0;
  }
  const double thetaRout = PP(XG_B3_THETAROUT), pdiblb = PP(XG_B3_PDIBLB);
  if (thetaRout > 0.0) {
    T8 = Abulk * Vdsat;
    T0 = Vgst2Vtm * T8;
    dT0_dVg = Vgst2Vtm * Abulk * dVdsat_dVg + T8 + Vgst2Vtm * Vdsat * dAbulk_dVg;
    dT0_dVb = Vgst2Vtm * (dAbulk_dVb * Vdsat + Abulk * dVdsat_dVb);
    dT0_dVd = Vgst2Vtm * Abulk * dVdsat_dVd;
    T1 = Vgst2Vtm + T8;
    dT1_dVg = 1.0 + Abulk * dVdsat_dVg + Vdsat * dAbulk_dVg;
    dT1_dVb = Abulk * dVdsat_dVb + dAbulk_dVb * Vdsat;
    dT1_dVd = Abulk * dVdsat_dVd;
    T9 = T1 * T1;
    T2 = thetaRout;
    VADIBL = (Vgst2Vtm - T0 / T1) / T2;
    dVADIBL_dVg = (1.0 - dT0_dVg / T1 + T0 * dT1_dVg / T9) / T2;
    dVADIBL_dVb = (-dT0_dVb / T1 + T0 * dT1_dVb / T9) / T2;
    dVADIBL_dVd = (-dT0_dVd / T1 + T0 * dT1_dVd / T9) / T2;
    T7 = pdiblb * Vbseff;
    if (T7 >= -0.9) {
      T3 = 1.0 / (1.0 + T7);
      VADIBL *= T3;
      dVADIBL_dVg *= T3;
      dVADIBL_dVb = (dVADIBL_dVb - VADIBL * pdiblb) * T3;
      dVADIBL_dVd *= T3;
    } else {
      T4 = 1.0 / (0.8 + T7);
      T3 = (17.0 + 20.0 * T7) * T4;
      dVADIBL_dVg *= T3;
      dVADIBL_dVb = dVADIBL_dVb * T3 - VADIBL * pdiblb * T4 * T4;
      dVADIBL_dVd *= T3;
      VADIBL *= T3;
    }
  } else {
    VADIBL = MAX_EXP;
    dVADIBL_dVd = dVADIBL_dVg = dVADIBL_dVb = 0.0;
  }
  T8 = PP(XG_B3_PVAG) / EsatL;
  T9 = T8 * Vgsteff;
  if (T9 > -0.9) {
    T0 = 1.0 + T9;
    dT0_dVg = T8 * (1.0 - Vgsteff * dEsatL_dVg / EsatL);
    dT0_dVb = -T9 * dEsatL_dVb / EsatL;
    dT0_dVd = -T9 * dEsatL_dVd / EsatL;
  } else {
    T1 = 1.0 / (17.0 + 20.0 * T9);
    T0 = (0.8 + T9) * T1;
    T1 *= T1;
    dT0_dVg = T8 * (1.0 - Vgsteff * dEsatL_dVg / EsatL) * T1;
    T9 *= T1 / EsatL;
    dT0_dVb = -T9 * dEsatL_dVb;
    dT0_dVd = -T9 * dEsatL_dVd;
  }
  tmp1 = VACLM * VACLM;
  tmp2 = VADIBL * VADIBL;
  tmp3 = VACLM + VADIBL;
  T1 = VACLM * VADIBL / tmp3;
  tmp3 *= tmp3;
  dT1_dVg = (tmp1 * dVADIBL_dVg + tmp2 * dVACLM_dVg) / tmp3;
  dT1_dVd = (tmp1 * dVADIBL_dVd + tmp2 * dVACLM_dVd) / tmp3;
  dT1_dVb = (tmp1 * dVADIBL_dVb + tmp2 * dVACLM_dVb) / tmp3;
  Va = Vasat + T0 * T1;
  dVa_dVg = dVasat_dVg + T1 * dT0_dVg + T0 * dT1_dVg;
  dVa_dVd = dVasat_dVd + T1 * dT0_dVd + T0 * dT1_dVd;
  dVa_dVb = dVasat_dVb + T1 * dT0_dVb + T0 * dT1_dVb;

  const double pscbe1 = PP(XG_B3_PSCBE1), pscbe2 = PP(XG_B3_PSCBE2);
  if (pscbe2 > 0.0) {
    if (diffVds > pscbe1 * litl / EXP_THRESHOLD) {
      T0 = pscbe1 * litl / diffVds;
      VASCBE = Leff * exp(T0) / pscbe2;
      T1 = T0 * VASCBE / diffVds;
      dVASCBE_dVg = T1 * dVdseff_dVg;
      dVASCBE_dVd = -T1 * (1.0 - dVdseff_dVd);
      dVASCBE_dVb = T1 * dVdseff_dVb;
    } else {
      VASCBE = MAX_EXP * Leff / pscbe2;
      dVASCBE_dVg = dVASCBE_dVd = dVASCBE_dVb = 0.0;
    }
  } else {
    VASCBE = MAX_EXP;
    dVASCBE_dVg = dVASCBE_dVd = dVASCBE_dVb = 0.0;
  }

  CoxWovL = cox * Weff / Leff;
  beta = ueff * CoxWovL;
  dbeta_dVg = CoxWovL * dueff_dVg + beta * dWeff_dVg / Weff;
  dbeta_dVd = CoxWovL * dueff_dVd;
  dbeta_dVb = CoxWovL * dueff_dVb + beta * dWeff_dVb / Weff;
  T0 = 1.0 - 0.5 * Abulk * Vdseff / Vgst2Vtm;
  dT0_dVg = -0.5 * (Abulk * dVdseff_dVg - Abulk * Vdseff / Vgst2Vtm + Vdseff * dAbulk_dVg) / Vgst2Vtm;
  dT0_dVd = -0.5 * Abulk * dVdseff_dVd / Vgst2Vtm;
  dT0_dVb = -0.5 * (Abulk * dVdseff_dVb + dAbulk_dVb * Vdseff) / Vgst2Vtm;
  fgche1 = Vgsteff * T0;
  dfgche1_dVg = Vgsteff * dT0_dVg + T0;
  dfgche1_dVd = Vgsteff * dT0_dVd;
  dfgche1_dVb = Vgsteff * dT0_dVb;
  T9 = Vdseff / EsatL;
  fgche2 = 1.0 + T9;
  dfgche2_dVg = (dVdseff_dVg - T9 * dEsatL_dVg) / EsatL;
  dfgche2_dVd = (dVdseff_dVd - T9 * dEsatL_dVd) / EsatL;
  dfgche2_dVb = (dVdseff_dVb - T9 * dEsatL_dVb) / EsatL;
  gche = beta * fgche1 / fgche2;
  dgche_dVg = (beta * dfgche1_dVg + fgche1 * dbeta_dVg - gche * dfgche2_dVg) / fgche2;
  dgche_dVd = (beta * dfgche1_dVd + fgche1 * dbeta_dVd - gche * dfgche2_dVd) / fgche2;
  dgche_dVb = (beta * dfgche1_dVb + fgche1 * dbeta_dVb - gche * dfgche2_dVb) / fgche2;
  T0 = 1.0 + gche * Rds;
  T9 = Vdseff / T0;
  Idl = gche * T9;
  dIdl_dVg = (gche * dVdseff_dVg + T9 * dgche_dVg) / T0 - Idl * gche / T0 * dRds_dVg;
  dIdl_dVd = (gche * dVdseff_dVd + T9 * dgche_dVd) / T0;
  dIdl_dVb = (gche * dVdseff_dVb + T9 * dgche_dVb - Idl * dRds_dVb * gche) / T0;
  T9 = diffVds / Va;
  T0 = 1.0 + T9;
  Idsa = Idl * T0;
  dIdsa_dVg = T0 * dIdl_dVg - Idl * (dVdseff_dVg + T9 * dVa_dVg) / Va;
  dIdsa_dVd = T0 * dIdl_dVd + Idl * (1.0 - dVdseff_dVd - T9 * dVa_dVd) / Va;
  dIdsa_dVb = T0 * dIdl_dVb - Idl * (dVdseff_dVb + T9 * dVa_dVb) / Va;
  T9 = diffVds / VASCBE;
  T0 = 1.0 + T9;
  Ids = Idsa * T0;
  Gm = T0 * dIdsa_dVg - Idsa * (dVdseff_dVg + T9 * dVASCBE_dVg) / VASCBE;
  Gds = T0 * dIdsa_dVd + Idsa * (1.0 - dVdseff_dVd - T9 * dVASCBE_dVd) / VASCBE;
  Gmb = T0 * dIdsa_dVb - Idsa * (dVdseff_dVb + T9 * dVASCBE_dVb) / VASCBE;
  Gds += Gm * dVgsteff_dVd;
  Gmb += Gm * dVgsteff_dVb;
  Gm *= dVgsteff_dVg;
  Gmb *= dVbseff_dVb;

  const double alpha0 = PP(XG_B3_ALPHA0), alpha1 = PP(XG_B3_ALPHA1), beta0 = PP(XG_B3_BETA0);
  tmp = alpha0 + alpha1 * Leff;
  if ((tmp <= 0.0) || (beta0 <= 0.0)) {
    Isub = Gbd = Gbb = Gbg = 0.0;
  } else {
    T2 = tmp / Leff;
    if (diffVds > beta0 / EXP_THRESHOLD) {
      T0 = -beta0 / diffVds;
      T1 = T2 * diffVds * exp(T0);
      T3 = T1 / diffVds * (T0 - 1.0);
      dT1_dVg = T3 * dVdseff_dVg;
      dT1_dVd = T3 * (dVdseff_dVd - 1.0);
      dT1_dVb = T3 * dVdseff_dVb;
    } else {
      T3 = T2 * MIN_EXP;
      T1 = T3 * diffVds;
      dT1_dVg = -T3 * dVdseff_dVg;
      dT1_dVd = T3 * (1.0 - dVdseff_dVd);
      dT1_dVb = -T3 * dVdseff_dVb;
    }
    Isub = T1 * Idsa;
    Gbg = T1 * dIdsa_dVg + Idsa * dT1_dVg;
    Gbd = T1 * dIdsa_dVd + Idsa * dT1_dVd;
    Gbb = T1 * dIdsa_dVb + Idsa * dT1_dVb;
    Gbd += Gbg * dVgsteff_dVd;
    Gbb += Gbg * dVgsteff_dVb;
    Gbg *= dVgsteff_dVg;
    Gbb *= dVbseff_dVb;
  }
  const double cdrain = Ids;
  m->gds = Gds; m->gm = Gm; m->gmbs = Gmb;
  m->gbbs = Gbb; m->gbgs = Gbg; m->gbds = Gbd;
  m->csub = Isub;

  /* ---- charges: capMod 0-3 (:5994-6959) ---- */
  cgdo = PP(XG_B3_CGDO);
  cgso = PP(XG_B3_CGSO);
  const double weffCV = PP(XG_B3_WEFFCV), leffCV = PP(XG_B3_LEFFCV);
  const double abulkCVfactor = PP(XG_B3_ABULKCVFACTOR);
  qgate = qdrn = qsrc = qbulk = 0.0;
  cggb = cgsb = cgdb = cdgb = cdsb = cddb = cbgb = cbsb = cbdb = 0.0;
  if ((xpart < 0) || (!ChargeComputationNeeded)) {
    qgate = qdrn = qsrc = qbulk = 0.0;
    cggb = cgsb = cgdb = 0.0;
    cdgb = cdsb = cddb = 0.0;
    cbgb = cbsb = cbdb = 0.0;
    goto finished;
  } else if (capMod == 0) {
    if (Vbseff < 0.0) {
      Vbseff = Vbs;
      dVbseff_dVb = 1.0;
    } else {
      Vbseff = phi - Phis;
      dVbseff_dVb = -dPhis_dVb;
    }
    Vfb = PP(XG_B3_VFBCV);
    Vth = Vfb + phi + k1ox * sqrtPhis;
    Vgst = Vgs_eff - Vth;
    dVth_dVb = k1ox * dsqrtPhis_dVb;
    dVgst_dVb = -dVth_dVb;
    dVgst_dVg = dVgs_eff_dVg;
    (void)dVgst_dVb; (void)dVgst_dVg;
    CoxWL = cox * weffCV * leffCV;
    Arg1 = Vgs_eff - Vbseff - Vfb;
    if (Arg1 <= 0.0) {
      qgate = CoxWL * Arg1;
      qbulk = -qgate;
      qdrn = 0.0;
      cggb = CoxWL * dVgs_eff_dVg;
      cgdb = 0.0;
      cgsb = CoxWL * (dVbseff_dVb - dVgs_eff_dVg);
      cdgb = 0.0; cddb = 0.0; cdsb = 0.0;
      cbgb = -CoxWL * dVgs_eff_dVg;
      cbdb = 0.0;
      cbsb = -cgsb;
      qinv = 0.0;
    } else if (Vgst <= 0.0) {
      T1 = 0.5 * k1ox;
      T2 = sqrt(T1 * T1 + Arg1);
      qgate = CoxWL * k1ox * (T2 - T1);
      qbulk = -qgate;
      qdrn = 0.0;
      T0 = CoxWL * T1 / T2;
      cggb = T0 * dVgs_eff_dVg;
      cgdb = 0.0;
      cgsb = T0 * (dVbseff_dVb - dVgs_eff_dVg);
      cdgb = 0.0; cddb = 0.0; cdsb = 0.0;
      cbgb = -cggb;
      cbdb = 0.0;
      cbsb = -cgsb;
      qinv = 0.0;
    } else {
      One_Third_CoxWL = CoxWL / 3.0;
      Two_Third_CoxWL = 2.0 * One_Third_CoxWL;
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      Vdsat = Vgst / AbulkCV;
      dVdsat_dVg = dVgs_eff_dVg / AbulkCV;
      dVdsat_dVb = -(Vdsat * dAbulkCV_dVb + dVth_dVb) / AbulkCV;
      if (xpart > 0.5) {
        if (Vdsat <= Vds) {
          T1 = Vdsat / 3.0;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - T1);
          T2 = -Two_Third_CoxWL * Vgst;
          qbulk = -(qgate + T2);
          qdrn = 0.0;
          cggb = One_Third_CoxWL * (3.0 - dVdsat_dVg) * dVgs_eff_dVg;
          T2 = -One_Third_CoxWL * dVdsat_dVb;
          cgsb = -(cggb + T2);
          cgdb = 0.0;
          cdgb = 0.0; cddb = 0.0; cdsb = 0.0;
          cbgb = -(cggb - Two_Third_CoxWL * dVgs_eff_dVg);
          T3 = -(T2 + Two_Third_CoxWL * dVth_dVb);
          cbsb = -(cbgb + T3);
          cbdb = 0.0;
          qinv = -(qgate + qbulk);
        } else {
          Alphaz = Vgst / Vdsat;
          T1 = 2.0 * Vdsat - Vds;
          T2 = Vds / (3.0 * T1);
          T3 = T2 * Vds;
          T9 = 0.25 * CoxWL;
          T4 = T9 * Alphaz;
          T7 = 2.0 * Vds - T1 - 3.0 * T3;
          T8 = T3 - T1 - 2.0 * Vds;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - 0.5 * (Vds - T3));
          T10 = T4 * T8;
          qdrn = T4 * T7;
          qbulk = -(qgate + qdrn + T10);
          T5 = T3 / T1;
          cggb = CoxWL * (1.0 - T5 * dVdsat_dVg) * dVgs_eff_dVg;
          T11 = -CoxWL * T5 * dVdsat_dVb;
          cgdb = CoxWL * (T2 - 0.5 + 0.5 * T5);
          cgsb = -(cggb + T11 + cgdb);
          T6 = 1.0 / Vdsat;
          dAlphaz_dVg = T6 * (1.0 - Alphaz * dVdsat_dVg);
          dAlphaz_dVb = -T6 * (dVth_dVb + Alphaz * dVdsat_dVb);
          T7 = T9 * T7;
          T8 = T9 * T8;
          T9 = 2.0 * T4 * (1.0 - 3.0 * T5);
          cdgb = (T7 * dAlphaz_dVg - T9 * dVdsat_dVg) * dVgs_eff_dVg;
          T12 = T7 * dAlphaz_dVb - T9 * dVdsat_dVb;
          cddb = T4 * (3.0 - 6.0 * T2 - 3.0 * T5);
          cdsb = -(cdgb + T12 + cddb);
          T9 = 2.0 * T4 * (1.0 + T5);
          T10 = (T8 * dAlphaz_dVg - T9 * dVdsat_dVg) * dVgs_eff_dVg;
          T11 = T8 * dAlphaz_dVb - T9 * dVdsat_dVb;
          T12 = T4 * (2.0 * T2 + T5 - 1.0);
          T0 = -(T10 + T11 + T12);
          cbgb = -(cggb + cdgb + T10);
          cbdb = -(cgdb + cddb + T12);
          cbsb = -(cgsb + cdsb + T0);
          qinv = -(qgate + qbulk);
        }
      } else if (xpart < 0.5) {
        if (Vds >= Vdsat) {
          T1 = Vdsat / 3.0;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - T1);
          T2 = -Two_Third_CoxWL * Vgst;
          qbulk = -(qgate + T2);
          qdrn = 0.4 * T2;
          cggb = One_Third_CoxWL * (3.0 - dVdsat_dVg) * dVgs_eff_dVg;
          T2 = -One_Third_CoxWL * dVdsat_dVb;
          cgsb = -(cggb + T2);
          cgdb = 0.0;
          T3 = 0.4 * Two_Third_CoxWL;
          cdgb = -T3 * dVgs_eff_dVg;
          cddb = 0.0;
          T4 = T3 * dVth_dVb;
          cdsb = -(T4 + cdgb);
          cbgb = -(cggb - Two_Third_CoxWL * dVgs_eff_dVg);
          T3 = -(T2 + Two_Third_CoxWL * dVth_dVb);
          cbsb = -(cbgb + T3);
          cbdb = 0.0;
          qinv = -(qgate + qbulk);
        } else {
          Alphaz = Vgst / Vdsat;
          T1 = 2.0 * Vdsat - Vds;
          T2 = Vds / (3.0 * T1);
          T3 = T2 * Vds;
          T9 = 0.25 * CoxWL;
          T4 = T9 * Alphaz;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - 0.5 * (Vds - T3));
          T5 = T3 / T1;
          cggb = CoxWL * (1.0 - T5 * dVdsat_dVg) * dVgs_eff_dVg;
          tmp = -CoxWL * T5 * dVdsat_dVb;
          cgdb = CoxWL * (T2 - 0.5 + 0.5 * T5);
          cgsb = -(cggb + cgdb + tmp);
          T6 = 1.0 / Vdsat;
          dAlphaz_dVg = T6 * (1.0 - Alphaz * dVdsat_dVg);
          dAlphaz_dVb = -T6 * (dVth_dVb + Alphaz * dVdsat_dVb);
          T6 = 8.0 * Vdsat * Vdsat - 6.0 * Vdsat * Vds + 1.2 * Vds * Vds;
          T8 = T2 / T1;
          T7 = Vds - T1 - T8 * T6;
          qdrn = T4 * T7;
          T7 *= T9;
          tmp = T8 / T1;
          tmp1 = T4 * (2.0 - 4.0 * tmp * T6 + T8 * (16.0 * Vdsat - 6.0 * Vds));
          cdgb = (T7 * dAlphaz_dVg - tmp1 * dVdsat_dVg) * dVgs_eff_dVg;
          T10 = T7 * dAlphaz_dVb - tmp1 * dVdsat_dVb;
          cddb = T4 * (2.0 - (1.0 / (3.0 * T1 * T1) + 2.0 * tmp) * T6 + T8 * (6.0 * Vdsat - 2.4 * Vds));
          cdsb = -(cdgb + T10 + cddb);
          T7 = 2.0 * (T1 + T3);
          qbulk = -(qgate - T4 * T7);
          T7 *= T9;
          T0 = 4.0 * T4 * (1.0 - T5);
          T12 = (-T7 * dAlphaz_dVg - cdgb - T0 * dVdsat_dVg) * dVgs_eff_dVg;
          T11 = -T7 * dAlphaz_dVb - T10 - T0 * dVdsat_dVb;
          T10 = -4.0 * T4 * (T2 - 0.5 + 0.5 * T5) - cddb;
          tmp = -(T10 + T11 + T12);
          cbgb = -(cggb + cdgb + T12);
          cbdb = -(cgdb + cddb + T11);
          cbsb = -(cgsb + cdsb + tmp);
          qinv = -(qgate + qbulk);
        }
      } else {
        if (Vds >= Vdsat) {
          T1 = Vdsat / 3.0;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - T1);
          T2 = -Two_Third_CoxWL * Vgst;
          qbulk = -(qgate + T2);
          qdrn = 0.5 * T2;
          cggb = One_Third_CoxWL * (3.0 - dVdsat_dVg) * dVgs_eff_dVg;
          T2 = -One_Third_CoxWL * dVdsat_dVb;
          cgsb = -(cggb + T2);
          cgdb = 0.0;
          cdgb = -One_Third_CoxWL * dVgs_eff_dVg;
          cddb = 0.0;
          T4 = One_Third_CoxWL * dVth_dVb;
          cdsb = -(T4 + cdgb);
          cbgb = -(cggb - Two_Third_CoxWL * dVgs_eff_dVg);
          T3 = -(T2 + Two_Third_CoxWL * dVth_dVb);
          cbsb = -(cbgb + T3);
          cbdb = 0.0;
          qinv = -(qgate + qbulk);
        } else {
          Alphaz = Vgst / Vdsat;
          T1 = 2.0 * Vdsat - Vds;
          T2 = Vds / (3.0 * T1);
          T3 = T2 * Vds;
          T9 = 0.25 * CoxWL;
          T4 = T9 * Alphaz;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - 0.5 * (Vds - T3));
          T5 = T3 / T1;
          cggb = CoxWL * (1.0 - T5 * dVdsat_dVg) * dVgs_eff_dVg;
          tmp = -CoxWL * T5 * dVdsat_dVb;
          cgdb = CoxWL * (T2 - 0.5 + 0.5 * T5);
          cgsb = -(cggb + cgdb + tmp);
          T6 = 1.0 / Vdsat;
          dAlphaz_dVg = T6 * (1.0 - Alphaz * dVdsat_dVg);
          dAlphaz_dVb = -T6 * (dVth_dVb + Alphaz * dVdsat_dVb);
          T7 = T1 + T3;
          qdrn = -T4 * T7;
          qbulk = -(qgate + qdrn + qdrn);
          T7 *= T9;
          T0 = T4 * (2.0 * T5 - 2.0);
          cdgb = (T0 * dVdsat_dVg - T7 * dAlphaz_dVg) * dVgs_eff_dVg;
          T12 = T0 * dVdsat_dVb - T7 * dAlphaz_dVb;
          cddb = T4 * (1.0 - 2.0 * T2 - T5);
          cdsb = -(cdgb + T12 + cddb);
          cbgb = -(cggb + 2.0 * cdgb);
          cbdb = -(cgdb + 2.0 * cddb);
          cbsb = -(cgsb + 2.0 * cdsb);
          qinv = -(qgate + qbulk);
        }
      }
    }
  } else {
    if (Vbseff < 0.0) {
      VbseffCV = Vbseff;
      dVbseffCV_dVb = 1.0;
    } else {
      VbseffCV = phi - Phis;
      dVbseffCV_dVb = -dPhis_dVb;
    }
    CoxWL = cox * weffCV * leffCV;
    noff = n * PP(XG_B3_NOFF);
    dnoff_dVd = PP(XG_B3_NOFF) * dn_dVd;
    dnoff_dVb = PP(XG_B3_NOFF) * dn_dVb;
    T0 = Vtm * noff;
    voffcv = PP(XG_B3_VOFFCV);
    VgstNVt = (Vgst - voffcv) / T0;
    if (VgstNVt > EXP_THRESHOLD) {
      Vgsteff = Vgst - voffcv;
      dVgsteff_dVg = dVgs_eff_dVg;
      dVgsteff_dVd = -dVth_dVd;
      dVgsteff_dVb = -dVth_dVb;
    } else if (VgstNVt < -EXP_THRESHOLD) {
      Vgsteff = T0 * log(1.0 + MIN_EXP);
      dVgsteff_dVg = 0.0;
      dVgsteff_dVd = Vgsteff / noff;
      dVgsteff_dVb = dVgsteff_dVd * dnoff_dVb;
      dVgsteff_dVd *= dnoff_dVd;
    } else {
      ExpVgst = exp(VgstNVt);
      Vgsteff = T0 * log(1.0 + ExpVgst);
      dVgsteff_dVg = ExpVgst / (1.0 + ExpVgst);
      dVgsteff_dVd = -dVgsteff_dVg * (dVth_dVd + (Vgst - voffcv) / noff * dnoff_dVd) +
                     Vgsteff / noff * dnoff_dVd;
      dVgsteff_dVb = -dVgsteff_dVg * (dVth_dVb + (Vgst - voffcv) / noff * dnoff_dVb) +
                     Vgsteff / noff * dnoff_dVb;
      dVgsteff_dVg *= dVgs_eff_dVg;
    }
    if (capMod == 1) {
      Vfb = PP(XG_B3_VFBZB);
      Arg1 = Vgs_eff - VbseffCV - Vfb - Vgsteff;
      if (Arg1 <= 0.0) {
        qgate = CoxWL * Arg1;
        Cgg = CoxWL * (dVgs_eff_dVg - dVgsteff_dVg);
        Cgd = -CoxWL * dVgsteff_dVd;
        Cgb = -CoxWL * (dVbseffCV_dVb + dVgsteff_dVb);
      } else {
        T0 = 0.5 * k1ox;
        T1 = sqrt(T0 * T0 + Arg1);
        T2 = CoxWL * T0 / T1;
        qgate = CoxWL * k1ox * (T1 - T0);
        Cgg = T2 * (dVgs_eff_dVg - dVgsteff_dVg);
        Cgd = -T2 * dVgsteff_dVd;
        Cgb = -T2 * (dVbseffCV_dVb + dVgsteff_dVb);
      }
      qbulk = -qgate;
      Cbg = -Cgg;
      Cbd = -Cgd;
      Cbb = -Cgb;
      One_Third_CoxWL = CoxWL / 3.0;
      Two_Third_CoxWL = 2.0 * One_Third_CoxWL;
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      VdsatCV = Vgsteff / AbulkCV;
      if (VdsatCV < Vds) {
        dVdsatCV_dVg = 1.0 / AbulkCV;
        dVdsatCV_dVb = -VdsatCV * dAbulkCV_dVb / AbulkCV;
        T0 = Vgsteff - VdsatCV / 3.0;
        dT0_dVg = 1.0 - dVdsatCV_dVg / 3.0;
        dT0_dVb = -dVdsatCV_dVb / 3.0;
        qgate += CoxWL * T0;
        Cgg1 = CoxWL * dT0_dVg;
        Cgb1 = CoxWL * dT0_dVb + Cgg1 * dVgsteff_dVb;
        Cgd1 = Cgg1 * dVgsteff_dVd;
        Cgg1 *= dVgsteff_dVg;
        Cgg += Cgg1;
        Cgb += Cgb1;
        Cgd += Cgd1;
        T0 = VdsatCV - Vgsteff;
        dT0_dVg = dVdsatCV_dVg - 1.0;
        dT0_dVb = dVdsatCV_dVb;
        qbulk += One_Third_CoxWL * T0;
        Cbg1 = One_Third_CoxWL * dT0_dVg;
        Cbb1 = One_Third_CoxWL * dT0_dVb + Cbg1 * dVgsteff_dVb;
        Cbd1 = Cbg1 * dVgsteff_dVd;
        Cbg1 *= dVgsteff_dVg;
        Cbg += Cbg1;
        Cbb += Cbb1;
        Cbd += Cbd1;
        if (xpart > 0.5) T0 = -Two_Third_CoxWL;
        else if (xpart < 0.5) T0 = -0.4 * CoxWL;
        else T0 = -One_Third_CoxWL;
        qsrc = T0 * Vgsteff;
        Csg = T0 * dVgsteff_dVg;
        Csb = T0 * dVgsteff_dVb;
        Csd = T0 * dVgsteff_dVd;
        Cgb *= dVbseff_dVb;
        Cbb *= dVbseff_dVb;
        Csb *= dVbseff_dVb;
      } else {
        T0 = AbulkCV * Vds;
        T1 = 12.0 * (Vgsteff - 0.5 * T0 + 1.e-20);
        T2 = Vds / T1;
        T3 = T0 * T2;
        dT3_dVg = -12.0 * T2 * T2 * AbulkCV;
        dT3_dVd = 6.0 * T0 * (4.0 * Vgsteff - T0) / T1 / T1 - 0.5;
        dT3_dVb = 12.0 * T2 * T2 * dAbulkCV_dVb * Vgsteff;
        qgate += CoxWL * (Vgsteff - 0.5 * Vds + T3);
        Cgg1 = CoxWL * (1.0 + dT3_dVg);
        Cgb1 = CoxWL * dT3_dVb + Cgg1 * dVgsteff_dVb;
        Cgd1 = CoxWL * dT3_dVd + Cgg1 * dVgsteff_dVd;
        Cgg1 *= dVgsteff_dVg;
        Cgg += Cgg1;
        Cgb += Cgb1;
        Cgd += Cgd1;
        qbulk += CoxWL * (1.0 - AbulkCV) * (0.5 * Vds - T3);
        Cbg1 = -CoxWL * ((1.0 - AbulkCV) * dT3_dVg);
        Cbb1 = -CoxWL * ((1.0 - AbulkCV) * dT3_dVb + (0.5 * Vds - T3) * dAbulkCV_dVb) + Cbg1 * dVgsteff_dVb;
        Cbd1 = -CoxWL * (1.0 - AbulkCV) * dT3_dVd + Cbg1 * dVgsteff_dVd;
        Cbg1 *= dVgsteff_dVg;
        Cbg += Cbg1;
        Cbb += Cbb1;
        Cbd += Cbd1;
        if (xpart > 0.5) {
          T1 = T1 + T1;
          qsrc = -CoxWL * (0.5 * Vgsteff + 0.25 * T0 - T0 * T0 / T1);
          Csg = -CoxWL * (0.5 + 24.0 * T0 * Vds / T1 / T1 * AbulkCV);
          Csb = -CoxWL * (0.25 * Vds * dAbulkCV_dVb - 12.0 * T0 * Vds / T1 / T1 * (4.0 * Vgsteff - T0) * dAbulkCV_dVb) +
                Csg * dVgsteff_dVb;
          Csd = -CoxWL * (0.25 * AbulkCV - 12.0 * AbulkCV * T0 / T1 / T1 * (4.0 * Vgsteff - T0)) +
                Csg * dVgsteff_dVd;
          Csg *= dVgsteff_dVg;
        } else if (xpart < 0.5) {
          T1 = T1 / 12.0;
          T2 = 0.5 * CoxWL / (T1 * T1);
          T3 = Vgsteff * (2.0 * T0 * T0 / 3.0 + Vgsteff * (Vgsteff - 4.0 * T0 / 3.0)) - 2.0 * T0 * T0 * T0 / 15.0;
          qsrc = -T2 * T3;
          T4 = 4.0 / 3.0 * Vgsteff * (Vgsteff - T0) + 0.4 * T0 * T0;
          Csg = -2.0 * qsrc / T1 - T2 * (Vgsteff * (3.0 * Vgsteff - 8.0 * T0 / 3.0) + 2.0 * T0 * T0 / 3.0);
          Csb = (qsrc / T1 * Vds + T2 * T4 * Vds) * dAbulkCV_dVb + Csg * dVgsteff_dVb;
          Csd = (qsrc / T1 + T2 * T4) * AbulkCV + Csg * dVgsteff_dVd;
          Csg *= dVgsteff_dVg;
        } else {
          qsrc = -0.5 * (qgate + qbulk);
          Csg = -0.5 * (Cgg1 + Cbg1);
          Csb = -0.5 * (Cgb1 + Cbb1);
          Csd = -0.5 * (Cgd1 + Cbd1);
        }
        Cgb *= dVbseff_dVb;
        Cbb *= dVbseff_dVb;
        Csb *= dVbseff_dVb;
      }
      qdrn = -(qgate + qbulk + qsrc);
      cggb = Cgg;
      cgsb = -(Cgg + Cgd + Cgb);
      cgdb = Cgd;
      cdgb = -(Cgg + Cbg + Csg);
      cdsb = (Cgg + Cgd + Cgb + Cbg + Cbd + Cbb + Csg + Csd + Csb);
      cddb = -(Cgd + Cbd + Csd);
      cbgb = Cbg;
      cbsb = -(Cbg + Cbd + Cbb);
      cbdb = Cbd;
      qinv = -(qgate + qbulk);
    } else if (capMod == 2) {
      Vfb = PP(XG_B3_VFBZB);
      V3 = Vfb - Vgs_eff + VbseffCV - DELTA_3;
      if (Vfb <= 0.0) {
        T0 = sqrt(V3 * V3 - 4.0 * DELTA_3 * Vfb);
        T2 = -DELTA_3 / T0;
      } else {
        T0 = sqrt(V3 * V3 + 4.0 * DELTA_3 * Vfb);
        T2 = DELTA_3 / T0;
      }
      T1 = 0.5 * (1.0 + V3 / T0);
      Vfbeff = Vfb - 0.5 * (V3 + T0);
      dVfbeff_dVg = T1 * dVgs_eff_dVg;
      dVfbeff_dVb = -T1 * dVbseffCV_dVb;
      Qac0 = CoxWL * (Vfbeff - Vfb);
      dQac0_dVg = CoxWL * dVfbeff_dVg;
      dQac0_dVb = CoxWL * dVfbeff_dVb;
      T0 = 0.5 * k1ox;
      T3 = Vgs_eff - Vfbeff - VbseffCV - Vgsteff;
      if (k1ox == 0.0) {
        T1 = 0.0;
        T2 = 0.0;
      } else if (T3 < 0.0) {
        T1 = T0 + T3 / k1ox;
        T2 = CoxWL;
      } else {
        T1 = sqrt(T0 * T0 + T3);
        T2 = CoxWL * T0 / T1;
      }
      Qsub0 = CoxWL * k1ox * (T1 - T0);
      dQsub0_dVg = T2 * (dVgs_eff_dVg - dVfbeff_dVg - dVgsteff_dVg);
      dQsub0_dVd = -T2 * dVgsteff_dVd;
      dQsub0_dVb = -T2 * (dVfbeff_dVb + dVbseffCV_dVb + dVgsteff_dVb);
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      VdsatCV = Vgsteff / AbulkCV;
      V4 = VdsatCV - Vds - DELTA_4;
      T0 = sqrt(V4 * V4 + 4.0 * DELTA_4 * VdsatCV);
      VdseffCV = VdsatCV - 0.5 * (V4 + T0);
      T1 = 0.5 * (1.0 + V4 / T0);
      T2 = DELTA_4 / T0;
      T3 = (1.0 - T1 - T2) / AbulkCV;
      dVdseffCV_dVg = T3;
      dVdseffCV_dVd = T1;
      dVdseffCV_dVb = -T3 * VdsatCV * dAbulkCV_dVb;
      if (Vds == 0.0) {
        VdseffCV = 0.0;
        dVdseffCV_dVg = 0.0;
        dVdseffCV_dVb = 0.0;
      }
      T0 = AbulkCV * VdseffCV;
      T1 = 12.0 * (Vgsteff - 0.5 * T0 + 1e-20);
      T2 = VdseffCV / T1;
      T3 = T0 * T2;
      T4 = (1.0 - 12.0 * T2 * T2 * AbulkCV);
      T5 = (6.0 * T0 * (4.0 * Vgsteff - T0) / (T1 * T1) - 0.5);
      T6 = 12.0 * T2 * T2 * Vgsteff;
      qinoi = -CoxWL * (Vgsteff - 0.5 * T0 + AbulkCV * T3);
      qgate = CoxWL * (Vgsteff - 0.5 * VdseffCV + T3);
      Cgg1 = CoxWL * (T4 + T5 * dVdseffCV_dVg);
      Cgd1 = CoxWL * T5 * dVdseffCV_dVd + Cgg1 * dVgsteff_dVd;
      Cgb1 = CoxWL * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Cgg1 * dVgsteff_dVb;
      Cgg1 *= dVgsteff_dVg;
      T7 = 1.0 - AbulkCV;
      qbulk = CoxWL * T7 * (0.5 * VdseffCV - T3);
      T4 = -T7 * (T4 - 1.0);
      T5 = -T7 * T5;
      T6 = -(T7 * T6 + (0.5 * VdseffCV - T3));
      Cbg1 = CoxWL * (T4 + T5 * dVdseffCV_dVg);
      Cbd1 = CoxWL * T5 * dVdseffCV_dVd + Cbg1 * dVgsteff_dVd;
      Cbb1 = CoxWL * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Cbg1 * dVgsteff_dVb;
      Cbg1 *= dVgsteff_dVg;
      if (xpart > 0.5) {
        T1 = T1 + T1;
        qsrc = -CoxWL * (0.5 * Vgsteff + 0.25 * T0 - T0 * T0 / T1);
        T7 = (4.0 * Vgsteff - T0) / (T1 * T1);
        T4 = -(0.5 + 24.0 * T0 * T0 / (T1 * T1));
        T5 = -(0.25 * AbulkCV - 12.0 * AbulkCV * T0 * T7);
        T6 = -(0.25 * VdseffCV - 12.0 * T0 * VdseffCV * T7);
        Csg = CoxWL * (T4 + T5 * dVdseffCV_dVg);
        Csd = CoxWL * T5 * dVdseffCV_dVd + Csg * dVgsteff_dVd;
        Csb = CoxWL * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Csg * dVgsteff_dVb;
        Csg *= dVgsteff_dVg;
      } else if (xpart < 0.5) {
        T1 = T1 / 12.0;
        T2 = 0.5 * CoxWL / (T1 * T1);
        T3 = Vgsteff * (2.0 * T0 * T0 / 3.0 + Vgsteff * (Vgsteff - 4.0 * T0 / 3.0)) - 2.0 * T0 * T0 * T0 / 15.0;
        qsrc = -T2 * T3;
        T7 = 4.0 / 3.0 * Vgsteff * (Vgsteff - T0) + 0.4 * T0 * T0;
        T4 = -2.0 * qsrc / T1 - T2 * (Vgsteff * (3.0 * Vgsteff - 8.0 * T0 / 3.0) + 2.0 * T0 * T0 / 3.0);
        T5 = (qsrc / T1 + T2 * T7) * AbulkCV;
        T6 = (qsrc / T1 * VdseffCV + T2 * T7 * VdseffCV);
        Csg = (T4 + T5 * dVdseffCV_dVg);
        Csd = T5 * dVdseffCV_dVd + Csg * dVgsteff_dVd;
        Csb = (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Csg * dVgsteff_dVb;
        Csg *= dVgsteff_dVg;
      } else {
        qsrc = -0.5 * (qgate + qbulk);
        Csg = -0.5 * (Cgg1 + Cbg1);
        Csb = -0.5 * (Cgb1 + Cbb1);
        Csd = -0.5 * (Cgd1 + Cbd1);
      }
      qgate += Qac0 + Qsub0;
      qbulk -= (Qac0 + Qsub0);
      qdrn = -(qgate + qbulk + qsrc);
      Cgg = dQac0_dVg + dQsub0_dVg + Cgg1;
      Cgd = dQsub0_dVd + Cgd1;
      Cgb = dQac0_dVb + dQsub0_dVb + Cgb1;
      Cbg = Cbg1 - dQac0_dVg - dQsub0_dVg;
      Cbd = Cbd1 - dQsub0_dVd;
      Cbb = Cbb1 - dQac0_dVb - dQsub0_dVb;
      Cgb *= dVbseff_dVb;
      Cbb *= dVbseff_dVb;
      Csb *= dVbseff_dVb;
      cggb = Cgg;
      cgsb = -(Cgg + Cgd + Cgb);
      cgdb = Cgd;
      cdgb = -(Cgg + Cbg + Csg);
      cdsb = (Cgg + Cgd + Cgb + Cbg + Cbd + Cbb + Csg + Csd + Csb);
      cddb = -(Cgd + Cbd + Csd);
      cbgb = Cbg;
      cbsb = -(Cbg + Cbd + Cbb);
      cbdb = Cbd;
      qinv = qinoi;
    } else if (capMod == 3) {
      const double vfbzb = PP(XG_B3_VFBZB), acde = PP(XG_B3_ACDE), ldeb = PP(XG_B3_LDEB);
      V3 = vfbzb - Vgs_eff + VbseffCV - DELTA_3;
      if (vfbzb <= 0.0) {
        T0 = sqrt(V3 * V3 - 4.0 * DELTA_3 * vfbzb);
        T2 = -DELTA_3 / T0;
      } else {
        T0 = sqrt(V3 * V3 + 4.0 * DELTA_3 * vfbzb);
        T2 = DELTA_3 / T0;
      }
      T1 = 0.5 * (1.0 + V3 / T0);
      Vfbeff = vfbzb - 0.5 * (V3 + T0);
      dVfbeff_dVg = T1 * dVgs_eff_dVg;
      dVfbeff_dVb = -T1 * dVbseffCV_dVb;
      Cox = cox;
      Tox = 1.0e8 * tox;
      T0 = (Vgs_eff - VbseffCV - vfbzb) / Tox;
      dT0_dVg = dVgs_eff_dVg / Tox;
      dT0_dVb = -dVbseffCV_dVb / Tox;
      tmp = T0 * acde;
      if ((-EXP_THRESHOLD < tmp) && (tmp < EXP_THRESHOLD)) {
        Tcen = ldeb * exp(tmp);
        dTcen_dVg = acde * Tcen;
        dTcen_dVb = dTcen_dVg * dT0_dVb;
        dTcen_dVg *= dT0_dVg;
      } else if (tmp <= -EXP_THRESHOLD) {
        Tcen = ldeb * MIN_EXP;
        dTcen_dVg = dTcen_dVb = 0.0;
      } else {
        Tcen = ldeb * MAX_EXP;
        dTcen_dVg = dTcen_dVb = 0.0;
      }
      LINK = 1.0e-3 * tox;
      V3 = ldeb - Tcen - LINK;
      V4 = sqrt(V3 * V3 + 4.0 * LINK * ldeb);
      Tcen = ldeb - 0.5 * (V3 + V4);
      T1 = 0.5 * (1.0 + V3 / V4);
      dTcen_dVg *= T1;
      dTcen_dVb *= T1;
      Ccen = EPSSI / Tcen;
      T2 = Cox / (Cox + Ccen);
      Coxeff = T2 * Ccen;
      T3 = -Ccen / Tcen;
      dCoxeff_dVg = T2 * T2 * T3;
      dCoxeff_dVb = dCoxeff_dVg * dTcen_dVb;
      dCoxeff_dVg *= dTcen_dVg;
      CoxWLcen = CoxWL * Coxeff / Cox;
      Qac0 = CoxWLcen * (Vfbeff - vfbzb);
      QovCox = Qac0 / Coxeff;
      dQac0_dVg = CoxWLcen * dVfbeff_dVg + QovCox * dCoxeff_dVg;
      dQac0_dVb = CoxWLcen * dVfbeff_dVb + QovCox * dCoxeff_dVb;
      T0 = 0.5 * k1ox;
      T3 = Vgs_eff - Vfbeff - VbseffCV - Vgsteff;
      if (k1ox == 0.0) {
        T1 = 0.0;
        T2 = 0.0;
      } else if (T3 < 0.0) {
        T1 = T0 + T3 / k1ox;
        T2 = CoxWLcen;
      } else {
        T1 = sqrt(T0 * T0 + T3);
        T2 = CoxWLcen * T0 / T1;
      }
      Qsub0 = CoxWLcen * k1ox * (T1 - T0);
      QovCox = Qsub0 / Coxeff;
      dQsub0_dVg = T2 * (dVgs_eff_dVg - dVfbeff_dVg - dVgsteff_dVg) + QovCox * dCoxeff_dVg;
      dQsub0_dVd = -T2 * dVgsteff_dVd;
      dQsub0_dVb = -T2 * (dVfbeff_dVb + dVbseffCV_dVb + dVgsteff_dVb) + QovCox * dCoxeff_dVb;
      const double moin = PP(XG_B3_MOIN);
      if (k1ox <= 0.0) {
        Denomi = 0.25 * moin * Vtm;
        T0 = 0.5 * sqrtPhi;
      } else {
        Denomi = moin * Vtm * k1ox * k1ox;
        T0 = k1ox * sqrtPhi;
      }
      T1 = 2.0 * T0 + Vgsteff;
      DeltaPhi = Vtm * log(1.0 + T1 * Vgsteff / Denomi);
      dDeltaPhi_dVg = 2.0 * Vtm * (T1 - T0) / (Denomi + T1 * Vgsteff);
      dDeltaPhi_dVd = dDeltaPhi_dVg * dVgsteff_dVd;
      dDeltaPhi_dVb = dDeltaPhi_dVg * dVgsteff_dVb;
      (void)dDeltaPhi_dVd; (void)dDeltaPhi_dVb;
      T3 = 4.0 * (Vth - vfbzb - phi);
      Tox += Tox;
      if (T3 >= 0.0) {
        T0 = (Vgsteff + T3) / Tox;
        dT0_dVd = (dVgsteff_dVd + 4.0 * dVth_dVd) / Tox;
        dT0_dVb = (dVgsteff_dVb + 4.0 * dVth_dVb) / Tox;
      } else {
        T0 = (Vgsteff + 1.0e-20) / Tox;
        dT0_dVd = dVgsteff_dVd / Tox;
        dT0_dVb = dVgsteff_dVb / Tox;
      }
      tmp = exp(0.7 * log(T0));
      T1 = 1.0 + tmp;
      T2 = 0.7 * tmp / (T0 * Tox);
      Tcen = 1.9e-9 / T1;
      dTcen_dVg = -1.9e-9 * T2 / T1 / T1;
      dTcen_dVd = Tox * dTcen_dVg;
      dTcen_dVb = dTcen_dVd * dT0_dVb;
      dTcen_dVd *= dT0_dVd;
      dTcen_dVg *= dVgsteff_dVg;
      Ccen = EPSSI / Tcen;
      T0 = Cox / (Cox + Ccen);
      Coxeff = T0 * Ccen;
      T1 = -Ccen / Tcen;
      dCoxeff_dVg = T0 * T0 * T1;
      dCoxeff_dVd = dCoxeff_dVg * dTcen_dVd;
      dCoxeff_dVb = dCoxeff_dVg * dTcen_dVb;
      dCoxeff_dVg *= dTcen_dVg;
      CoxWLcen = CoxWL * Coxeff / Cox;
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      VdsatCV = (Vgsteff - DeltaPhi) / AbulkCV;
      V4 = VdsatCV - Vds - DELTA_4;
      T0 = sqrt(V4 * V4 + 4.0 * DELTA_4 * VdsatCV);
      VdseffCV = VdsatCV - 0.5 * (V4 + T0);
      T1 = 0.5 * (1.0 + V4 / T0);
      T2 = DELTA_4 / T0;
      T3 = (1.0 - T1 - T2) / AbulkCV;
      T4 = T3 * (1.0 - dDeltaPhi_dVg);
      dVdseffCV_dVg = T4;
      dVdseffCV_dVd = T1;
      dVdseffCV_dVb = -T3 * VdsatCV * dAbulkCV_dVb;
      if (Vds == 0.0) {
        VdseffCV = 0.0;
        dVdseffCV_dVg = 0.0;
        dVdseffCV_dVb = 0.0;
      }
      T0 = AbulkCV * VdseffCV;
      T1 = Vgsteff - DeltaPhi;
      T2 = 12.0 * (T1 - 0.5 * T0 + 1.0e-20);
      T3 = T0 / T2;
      T4 = 1.0 - 12.0 * T3 * T3;
      T5 = AbulkCV * (6.0 * T0 * (4.0 * T1 - T0) / (T2 * T2) - 0.5);
      T6 = T5 * VdseffCV / AbulkCV;
      qgate = qinoi = CoxWLcen * (T1 - T0 * (0.5 - T3));
      QovCox = qgate / Coxeff;
      Cgg1 = CoxWLcen * (T4 * (1.0 - dDeltaPhi_dVg) + T5 * dVdseffCV_dVg);
      Cgd1 = CoxWLcen * T5 * dVdseffCV_dVd + Cgg1 * dVgsteff_dVd + QovCox * dCoxeff_dVd;
      Cgb1 = CoxWLcen * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Cgg1 * dVgsteff_dVb + QovCox * dCoxeff_dVb;
      Cgg1 = Cgg1 * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      T7 = 1.0 - AbulkCV;
      T8 = T2 * T2;
      T9 = 12.0 * T7 * T0 * T0 / (T8 * AbulkCV);
      T10 = T9 * (1.0 - dDeltaPhi_dVg);
      T11 = -T7 * T5 / AbulkCV;
      T12 = -(T9 * T1 / AbulkCV + VdseffCV * (0.5 - T0 / T2));
      qbulk = CoxWLcen * T7 * (0.5 * VdseffCV - T0 * VdseffCV / T2);
      QovCox = qbulk / Coxeff;
      Cbg1 = CoxWLcen * (T10 + T11 * dVdseffCV_dVg);
      Cbd1 = CoxWLcen * T11 * dVdseffCV_dVd + Cbg1 * dVgsteff_dVd + QovCox * dCoxeff_dVd;
      Cbb1 = CoxWLcen * (T11 * dVdseffCV_dVb + T12 * dAbulkCV_dVb) + Cbg1 * dVgsteff_dVb + QovCox * dCoxeff_dVb;
      Cbg1 = Cbg1 * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      if (xpart > 0.5) {
        qsrc = -CoxWLcen * (T1 / 2.0 + T0 / 4.0 - 0.5 * T0 * T0 / T2);
        QovCox = qsrc / Coxeff;
        T2 += T2;
        T3 = T2 * T2;
        T7 = -(0.25 - 12.0 * T0 * (4.0 * T1 - T0) / T3);
        T4 = -(0.5 + 24.0 * T0 * T0 / T3) * (1.0 - dDeltaPhi_dVg);
        T5 = T7 * AbulkCV;
        T6 = T7 * VdseffCV;
        Csg = CoxWLcen * (T4 + T5 * dVdseffCV_dVg);
        Csd = CoxWLcen * T5 * dVdseffCV_dVd + Csg * dVgsteff_dVd + QovCox * dCoxeff_dVd;
        Csb = CoxWLcen * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Csg * dVgsteff_dVb + QovCox * dCoxeff_dVb;
        Csg = Csg * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      } else if (xpart < 0.5) {
        T2 = T2 / 12.0;
        T3 = 0.5 * CoxWLcen / (T2 * T2);
        T4 = T1 * (2.0 * T0 * T0 / 3.0 + T1 * (T1 - 4.0 * T0 / 3.0)) - 2.0 * T0 * T0 * T0 / 15.0;
        qsrc = -T3 * T4;
        QovCox = qsrc / Coxeff;
        T8 = 4.0 / 3.0 * T1 * (T1 - T0) + 0.4 * T0 * T0;
        T5 = -2.0 * qsrc / T2 - T3 * (T1 * (3.0 * T1 - 8.0 * T0 / 3.0) + 2.0 * T0 * T0 / 3.0);
        T6 = AbulkCV * (qsrc / T2 + T3 * T8);
        T7 = T6 * VdseffCV / AbulkCV;
        Csg = T5 * (1.0 - dDeltaPhi_dVg) + T6 * dVdseffCV_dVg;
        Csd = Csg * dVgsteff_dVd + T6 * dVdseffCV_dVd + QovCox * dCoxeff_dVd;
        Csb = Csg * dVgsteff_dVb + T6 * dVdseffCV_dVb + T7 * dAbulkCV_dVb + QovCox * dCoxeff_dVb;
        Csg = Csg * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      } else {
        qsrc = -0.5 * qgate;
        Csg = -0.5 * Cgg1;
        Csd = -0.5 * Cgd1;
        Csb = -0.5 * Cgb1;
      }
      qgate += Qac0 + Qsub0 - qbulk;
      qbulk -= (Qac0 + Qsub0);
      qdrn = -(qgate + qbulk + qsrc);
      Cbg = Cbg1 - dQac0_dVg - dQsub0_dVg;
      Cbd = Cbd1 - dQsub0_dVd;
      Cbb = Cbb1 - dQac0_dVb - dQsub0_dVb;
      Cgg = Cgg1 - Cbg;
      Cgd = Cgd1 - Cbd;
      Cgb = Cgb1 - Cbb;
      Cgb *= dVbseff_dVb;
      Cbb *= dVbseff_dVb;
      Csb *= dVbseff_dVb;
      cggb = Cgg;
      cgsb = -(Cgg + Cgd + Cgb);
      cgdb = Cgd;
      cdgb = -(Cgg + Cbg + Csg);
      cdsb = (Cgg + Cgd + Cgb + Cbg + Cbd + Cbb + Csg + Csd + Csb);
      cddb = -(Cgd + Cbd + Csd);
      cbgb = Cbg;
      cbsb = -(Cbg + Cbd + Cbb);
      cbdb = Cbd;
      qinv = -qinoi;
    }
  }

finished:
  m->cd = cdrain;
  capbs = capbd = qbs = qbd = 0.0;
  if (ChargeComputationNeeded) {
    czbd = PP(XG_B3_CJTEMP) * drainArea;
    czbs = PP(XG_B3_CJTEMP) * sourceArea;
    if (drainPerimeter < weff) {
      czbdswg = PP(XG_B3_CJSWGTEMP) * drainPerimeter;
      czbdsw = 0.0;
    } else {
      czbdsw = PP(XG_B3_CJSWTEMP) * (drainPerimeter - weff);
      czbdswg = PP(XG_B3_CJSWGTEMP) * weff;
    }
    if (sourcePerimeter < weff) {
      czbssw = 0.0;
      czbsswg = PP(XG_B3_CJSWGTEMP) * sourcePerimeter;
    } else {
      czbssw = PP(XG_B3_CJSWTEMP) * (sourcePerimeter - weff);
      czbsswg = PP(XG_B3_CJSWGTEMP) * weff;
    }
    MJ = PP(XG_B3_MJ);
    MJSW = PP(XG_B3_MJSW);
    MJSWG = PP(XG_B3_MJSWG);
    const double PhiBTemp = PP(XG_B3_PHIB), PhiBSWTemp = PP(XG_B3_PHIBSW);
    const double PhiBSWGTemp = PP(XG_B3_PHIBSWG);
    if (vbs == 0.0) {
      qbs = 0.0;
      capbs = czbs + czbssw + czbsswg;
    } else if (vbs < 0.0) {
      if (czbs > 0.0) {
        arg = 1.0 - vbs / PhiBTemp;
        if (MJ == 0.5) sarg = 1.0 / sqrt(arg);
        else sarg = exp(-MJ * log(arg));
        qbs = PhiBTemp * czbs * (1.0 - arg * sarg) / (1.0 - MJ);
        capbs = czbs * sarg;
      } else {
        qbs = 0.0;
        capbs = 0.0;
      }
      if (czbssw > 0.0) {
        arg = 1.0 - vbs / PhiBSWTemp;
        if (MJSW == 0.5) sarg = 1.0 / sqrt(arg);
        else sarg = exp(-MJSW * log(arg));
        qbs += PhiBSWTemp * czbssw * (1.0 - arg * sarg) / (1.0 - MJSW);
        capbs += czbssw * sarg;
      }
      if (czbsswg > 0.0) {
        arg = 1.0 - vbs / PhiBSWGTemp;
        if (MJSWG == 0.5) sarg = 1.0 / sqrt(arg);
        else sarg = exp(-MJSWG * log(arg));
        qbs += PhiBSWGTemp * czbsswg * (1.0 - arg * sarg) / (1.0 - MJSWG);
        capbs += czbsswg * sarg;
      }
    } else {
      T0 = czbs + czbssw + czbsswg;
      T1 = vbs * (czbs * MJ / PhiBTemp + czbssw * MJSW / PhiBSWTemp + czbsswg * MJSWG / PhiBSWGTemp);
      qbs = vbs * (T0 + 0.5 * T1);
      capbs = T0 + T1;
    }
    if (vbd == 0.0) {
      qbd = 0.0;
      capbd = czbd + czbdsw + czbdswg;
    } else if (vbd < 0.0) {
      if (czbd > 0.0) {
        arg = 1.0 - vbd / PhiBTemp;
        if (MJ == 0.5) sarg = 1.0 / sqrt(arg);
        else sarg = exp(-MJ * log(arg));
        qbd = PhiBTemp * czbd * (1.0 - arg * sarg) / (1.0 - MJ);
        capbd = czbd * sarg;
      } else {
        qbd = 0.0;
        capbd = 0.0;
      }
      if (czbdsw > 0.0) {
        arg = 1.0 - vbd / PhiBSWTemp;
        if (MJSW == 0.5) sarg = 1.0 / sqrt(arg);
        else sarg = exp(-MJSW * log(arg));
        qbd += PhiBSWTemp * czbdsw * (1.0 - arg * sarg) / (1.0 - MJSW);
        capbd += czbdsw * sarg;
      }
      if (czbdswg > 0.0) {
        arg = 1.0 - vbd / PhiBSWGTemp;
        if (MJSWG == 0.5) sarg = 1.0 / sqrt(arg);
        else sarg = exp(-MJSWG * log(arg));
        qbd += PhiBSWGTemp * czbdswg * (1.0 - arg * sarg) / (1.0 - MJSWG);
        capbd += czbdswg * sarg;
      }
    } else {
      T0 = czbd + czbdsw + czbdswg;
      T1 = vbd * (czbd * MJ / PhiBTemp + czbdsw * MJSW / PhiBSWTemp + czbdswg * MJSWG / PhiBSWGTemp);
      qbd = vbd * (T0 + 0.5 * T1);
      capbd = T0 + T1;
    }
  }

  m->ggtg = m->ggtd = m->ggtb = m->ggts = 0.0;
  if (ChargeComputationNeeded) {
    const double ckappa = PP(XG_B3_CKAPPA), cgdl = PP(XG_B3_CGDL), cgsl = PP(XG_B3_CGSL);
    if (capMod == 0) {
      cgdo = PP(XG_B3_CGDO);
      qgdo = PP(XG_B3_CGDO) * vgd;
      cgso = PP(XG_B3_CGSO);
      qgso = PP(XG_B3_CGSO) * vgs;
    } else if (capMod == 1) {
      if (vgd < 0.0) {
        T1 = sqrt(1.0 - 4.0 * vgd / ckappa);
        cgdo = PP(XG_B3_CGDO) + weffCV * cgdl / T1;
        qgdo = PP(XG_B3_CGDO) * vgd - weffCV * 0.5 * cgdl * ckappa * (T1 - 1.0);
      } else {
        cgdo = PP(XG_B3_CGDO) + weffCV * cgdl;
        qgdo = (weffCV * cgdl + PP(XG_B3_CGDO)) * vgd;
      }
      if (vgs < 0.0) {
        T1 = sqrt(1.0 - 4.0 * vgs / ckappa);
        cgso = PP(XG_B3_CGSO) + weffCV * cgsl / T1;
        qgso = PP(XG_B3_CGSO) * vgs - weffCV * 0.5 * cgsl * ckappa * (T1 - 1.0);
      } else {
        cgso = PP(XG_B3_CGSO) + weffCV * cgsl;
        qgso = (weffCV * cgsl + PP(XG_B3_CGSO)) * vgs;
      }
    } else {
      T0 = vgd + DELTA_1;
      T1 = sqrt(T0 * T0 + 4.0 * DELTA_1);
      T2 = 0.5 * (T0 - T1);
      T3 = weffCV * cgdl;
      T4 = sqrt(1.0 - 4.0 * T2 / ckappa);
      cgdo = PP(XG_B3_CGDO) + T3 - T3 * (1.0 - 1.0 / T4) * (0.5 - 0.5 * T0 / T1);
      qgdo = (PP(XG_B3_CGDO) + T3) * vgd - T3 * (T2 + 0.5 * ckappa * (T4 - 1.0));
      T0 = vgs + DELTA_1;
      T1 = sqrt(T0 * T0 + 4.0 * DELTA_1);
      T2 = 0.5 * (T0 - T1);
      T3 = weffCV * cgsl;
      T4 = sqrt(1.0 - 4.0 * T2 / ckappa);
      cgso = PP(XG_B3_CGSO) + T3 - T3 * (1.0 - 1.0 / T4) * (0.5 - 0.5 * T0 / T1);
      qgso = (PP(XG_B3_CGSO) + T3) * vgs - T3 * (T2 + 0.5 * ckappa * (T4 - 1.0));
    }
    /* setupCapacitors_oldDAE: charge sums and partition (:7640-7898), nqsMod 0 */
    const double cgbo = PP(XG_B3_CGBO);
    double qgd, qgs, qgb;
    if (mode > 0) {
      qgd = qgdo;
      qgs = qgso;
      qgb = cgbo * vgb;
      qgate += qgd + qgs + qgb;
      qbulk -= qgb;
      qdrn -= qgd;
      qsrc = -(qgate + qbulk + qdrn);
      m->sxpart = 0.6;
      m->dxpart = 0.4;
    } else {
      qgd = qgdo;
      qgs = qgso;
      qgb = cgbo * vgb;
      qgate += qgd + qgs + qgb;
      qbulk -= qgb;
      qsrc = qdrn - qgs;
      qdrn = -(qgate + qbulk + qsrc);
      m->sxpart = 0.4;
      m->dxpart = 0.6;
    }
    /* setupCapacitors_newDAE (:7574-7638), nqsMod 0 */
    if (mode > 0) {
      mem->CAPcggb = (cggb + cgdo + cgso + cgbo);
      mem->CAPcgdb = (cgdb - cgdo);
      mem->CAPcgsb = (cgsb - cgso);
      mem->CAPcdgb = (cdgb - cgdo);
      mem->CAPcddb = (cddb + capbd + cgdo);
      mem->CAPcdsb = cdsb;
      mem->CAPcsgb = -(cggb + cbgb + cdgb + cgso);
      mem->CAPcsdb = -(cgdb + cbdb + cddb);
      mem->CAPcssb = (capbs + cgso - (cgsb + cbsb + cdsb));
      mem->CAPcbgb = (cbgb - cgbo);
      mem->CAPcbdb = (cbdb - capbd);
      mem->CAPcbsb = (cbsb - capbs);
    } else {
      mem->CAPcggb = (cggb + cgdo + cgso + cgbo);
      mem->CAPcgdb = (cgsb - cgdo);
      mem->CAPcgsb = (cgdb - cgso);
      mem->CAPcdgb = -(cggb + cbgb + cdgb + cgdo);
      mem->CAPcddb = (capbd + cgdo - (cgsb + cbsb + cdsb));
      mem->CAPcdsb = -(cgdb + cbdb + cddb);
      mem->CAPcsgb = (cdgb - cgso);
      mem->CAPcsdb = cdsb;
      mem->CAPcssb = (cddb + capbs + cgso);
      mem->CAPcbgb = (cbgb - cgbo);
      mem->CAPcbdb = (cbsb - capbd);
      mem->CAPcbsb = (cbdb - capbs);
    }
    mem->qg = qgate;
    mem->qd = qdrn - qbd;
    mem->qb = qbulk + qbd + qbs;
    mem->qbs = qbs;
    mem->qbd = qbd;
  }
  m->ddxpart_dVd = m->ddxpart_dVg = m->ddxpart_dVb = m->ddxpart_dVs = 0.0;
  m->dsxpart_dVd = m->dsxpart_dVg = m->dsxpart_dVb = m->dsxpart_dVs = 0.0;
  m->Idrain = PP(XG_B3_GD) * Vddp;
  m->Isource = PP(XG_B3_GS) * Vssp;
  m->T1global = T1;
  m->vbs = vbs; m->vgs = vgs; m->vds = vds; m->vbd = vbd; m->vgd = vgd; m->vgb = vgb;
  m->vbs_orig = vbs_orig; m->vgs_orig = vgs_orig; m->vds_orig = vds_orig;
  m->vbd_orig = vbd_orig; m->vgd_orig = vgd_orig;
  m->von = von; m->gbs = gbs; m->gbd = gbd; m->cbs = cbs; m->cbd = cbd;
  m->mode = mode; m->origFlag = origFlag; m->ChargeComputationNeeded = ChargeComputationNeeded;

  /* Master::updateState store / state writes (:9240-9275) */
  sto[O_VBS] = vbs;
  sto[O_VGS] = vgs;
  sto[O_VDS] = vds;
  sto[O_VBD] = vbd;
  sto[O_VON] = von;
  sta[S_QB] = mem->qb;
  sta[S_QG] = mem->qg;
  sta[S_QD] = mem->qd;
  sta[S_QBS] = mem->qbs;
  sta[S_QBD] = mem->qbd;
  if (!fl->dcop && fl->init_tran && fl->newton_iter == 0) {
    double *csta = (double *)(io->sta_curr + T->sta0 + (int64_t)i * 12);
    csta[S_QB] = mem->qb;
    csta[S_QG] = mem->qg;
    csta[S_QD] = mem->qd;
    csta[S_QBS] = mem->qbs;
    csta[S_QBD] = mem->qbd;
  }
#undef PP
}

void xgo_b3_update_state(xgo_circuit *c, int i0, int i1, xgo_io *io) {
  b3m_t *m = b3_members(c);
  b3mem_t *mem = (b3mem_t *)c->b3_member;
  for (int i = i0; i < i1; ++i) b3_update(c, i, io, &m[i], &mem[i]);
}

/* Master::loadDAEVectors (:9306-9653) with auxChargeCalculations (:7477-7573). */
void xgo_b3_load_vectors(xgo_circuit *c, int i0, int i1, xgo_io *io) {
  const xgo_type *T = &c->T[XG_DEV_BSIM3];
  b3m_t *ms = b3_members(c);
  b3mem_t *mems = (b3mem_t *)c->b3_member;
  for (int i = i0; i < i1; ++i) {
    b3m_t *mi = &ms[i];
    b3mem_t *mem = &mems[i];
    const int *L = T->lid + (int64_t)i * 6;
    const int li_Drain = L[0], li_Gate = L[1], li_Source = L[2], li_Bulk = L[3];
    const int li_DrainPrime = L[4], li_SourcePrime = L[5];
    const int dtype = (int)P(T, XG_B3_DTYPE, i);
    const double numberParallel = P(T, XG_B3_M, i);
    const double drainConductance = P(T, XG_B3_GD, i), sourceConductance = P(T, XG_B3_GS, i);
    double cdreq_Jdxp = 0.0, ceqbd_Jdxp = 0.0, ceqbs_Jdxp = 0.0;
    double Gm, Gmbs, FwdSum, RevSum, cdreq, ceqbd, ceqbs;
    if (mi->mode >= 0) {
      Gm = mi->gm; Gmbs = mi->gmbs; FwdSum = Gm + Gmbs; RevSum = 0.0;
      cdreq = dtype * (mi->cd);
      ceqbd = -dtype * (mi->csub);
      ceqbs = 0.0;
    } else {
      Gm = -mi->gm; Gmbs = -mi->gmbs; FwdSum = 0.0; RevSum = -(Gm + Gmbs);
      cdreq = -dtype * (mi->cd);
      ceqbs = -dtype * (mi->csub);
      ceqbd = 0.0;
    }
    (void)FwdSum; (void)RevSum;
    if (dtype > 0) {
      ceqbs += (mi->cbs);
      ceqbd += (mi->cbd);
    } else {
      ceqbs -= (mi->cbs);
      ceqbd -= (mi->cbd);
    }
    if (drainConductance != 0.0) io->f[li_Drain] += mi->Idrain * numberParallel;
    if (sourceConductance != 0.0) io->f[li_Source] += mi->Isource * numberParallel;
    io->f[li_Bulk] += (ceqbs + ceqbd) * numberParallel;
    io->f[li_DrainPrime] += (-(ceqbd - cdreq) - mi->Idrain) * numberParallel;
    io->f[li_SourcePrime] += (-(cdreq + ceqbs) - mi->Isource) * numberParallel;
    if (c->opt.voltlim && !mi->origFlag) {
      double tmp;
      if (mi->mode >= 0) {
        tmp = dtype * (-mi->gds * (mi->vds - mi->vds_orig) - Gm * (mi->vgs - mi->vgs_orig) -
                       Gmbs * (mi->vbs - mi->vbs_orig));
        cdreq_Jdxp += tmp;
        cdreq += tmp;
        tmp = -dtype * (-mi->gbds * (mi->vds - mi->vds_orig) - mi->gbgs * (mi->vgs - mi->vgs_orig) -
                        mi->gbbs * (mi->vbs - mi->vbs_orig));
        ceqbd_Jdxp += tmp;
        ceqbd += tmp;
      } else {
        tmp = -dtype * (mi->gds * (mi->vds - mi->vds_orig) + Gm * (mi->vgd - mi->vgd_orig) +
                        Gmbs * (mi->vbd - mi->vbd_orig));
        cdreq_Jdxp += tmp;
        cdreq += tmp;
        tmp = -dtype * (mi->gbds * (mi->vds - mi->vds_orig) - mi->gbgs * (mi->vgd - mi->vgd_orig) -
                        mi->gbbs * (mi->vbd - mi->vbd_orig));
        ceqbd_Jdxp += tmp;
        ceqbd += tmp;
      }
      if (dtype > 0) {
        ceqbs_Jdxp += (-mi->gbs * (mi->vbs - mi->vbs_orig));
        ceqbs += (-mi->gbs * (mi->vbs - mi->vbs_orig));
        ceqbd_Jdxp += (-mi->gbd * (mi->vbd - mi->vbd_orig));
        ceqbd += (-mi->gbd * (mi->vbd - mi->vbd_orig));
      } else {
        ceqbs_Jdxp -= (-mi->gbs * (mi->vbs - mi->vbs_orig));
        ceqbs -= (-mi->gbs * (mi->vbs - mi->vbs_orig));
        ceqbd_Jdxp -= (-mi->gbd * (mi->vbd - mi->vbd_orig));
        ceqbd -= (-mi->gbd * (mi->vbd - mi->vbd_orig));
      }
      io->dfdxdvp[li_Bulk] += -(ceqbs_Jdxp + ceqbd_Jdxp) * numberParallel;
      io->dfdxdvp[li_DrainPrime] += (ceqbd_Jdxp - cdreq_Jdxp) * numberParallel;
      io->dfdxdvp[li_SourcePrime] += (cdreq_Jdxp + ceqbs_Jdxp) * numberParallel;
    }
    /* auxChargeCalculations */
    if (!mi->ChargeComputationNeeded) {
      mi->sxpart = (1.0 - (mi->dxpart = (mi->mode > 0) ? 0.4 : 0.6));
    } else {
      double vgb_orig = mi->vgs_orig - mi->vbs_orig;
      mem->Qeqqg_Jdxp = 0.0;
      if (!mi->origFlag)
        mem->Qeqqg_Jdxp = -mem->CAPcggb * (mi->vgb - vgb_orig) + mem->CAPcgdb * (mi->vbd - mi->vbd_orig) +
                          mem->CAPcgsb * (mi->vbs - mi->vbs_orig);
      mem->Qeqqb_Jdxp = 0.0;
      if (!mi->origFlag)
        mem->Qeqqb_Jdxp = -mem->CAPcbgb * (mi->vgb - vgb_orig) + mem->CAPcbdb * (mi->vbd - mi->vbd_orig) +
                          mem->CAPcbsb * (mi->vbs - mi->vbs_orig);
      mem->Qeqqd_Jdxp = 0.0;
      if (!mi->origFlag)
        mem->Qeqqd_Jdxp = -mem->CAPcdgb * (mi->vgb - vgb_orig) + mem->CAPcddb * (mi->vbd - mi->vbd_orig) +
                          mem->CAPcdsb * (mi->vbs - mi->vbs_orig);
    }
    double Qeqqg, Qeqqb, Qeqqd;
    if (dtype > 0) {
      Qeqqg = mem->qg; Qeqqb = mem->qb; Qeqqd = mem->qd;
    } else {
      Qeqqg = -mem->qg; Qeqqb = -mem->qb; Qeqqd = -mem->qd;
    }
    io->q[li_Gate] += Qeqqg * numberParallel;
    io->q[li_Bulk] += (Qeqqb) * numberParallel;
    io->q[li_DrainPrime] += (-(-Qeqqd)) * numberParallel;
    io->q[li_SourcePrime] += (-(+Qeqqg + Qeqqb + Qeqqd)) * numberParallel;
    if (c->opt.voltlim) {
      if (dtype <= 0) {
        mem->Qeqqg_Jdxp = -mem->Qeqqg_Jdxp;
        mem->Qeqqb_Jdxp = -mem->Qeqqb_Jdxp;
        mem->Qeqqd_Jdxp = -mem->Qeqqd_Jdxp;
      }
      if (!mi->origFlag) {
        io->dqdxdvp[li_Gate] += -mem->Qeqqg_Jdxp * numberParallel;
        io->dqdxdvp[li_Bulk] += -(+mem->Qeqqb_Jdxp) * numberParallel;
        io->dqdxdvp[li_DrainPrime] += (-mem->Qeqqd_Jdxp) * numberParallel;
        io->dqdxdvp[li_SourcePrime] += (+mem->Qeqqg_Jdxp + mem->Qeqqb_Jdxp + mem->Qeqqd_Jdxp) * numberParallel;
      }
    }
    mi->Gm = Gm;
    mi->Gmbs = Gmbs;
  }
}

/* Master::loadDAEMatrices, pointer path (:9654-9939). */
void xgo_b3_load_matrices(xgo_circuit *c, int i0, int i1, xgo_io *io) {
  const xgo_type *T = &c->T[XG_DEV_BSIM3];
  const xg_load_flags *fl = io->fl;
  b3m_t *ms = b3_members(c);
  b3mem_t *mems = (b3mem_t *)c->b3_member;
  for (int i = i0; i < i1; ++i) {
    const b3m_t *mi = &ms[i];
    const b3mem_t *mem = &mems[i];
    const int *L = T->lid + (int64_t)i * 6;
    const int d = L[0], g = L[1], s = L[2], b = L[3], dp = L[4], sp = L[5];
    const double M = P(T, XG_B3_M, i);
    const double GD = P(T, XG_B3_GD, i), GS = P(T, XG_B3_GS, i);
    double *F = io->dfdx, *Q = io->dqdx;
    /* FwdSum/RevSum and the gb* partition are set with Gm/Gmbs in
     * loadDAEVectors (:9315-9353) */
    const double Gm = mi->Gm, Gmbs = mi->Gmbs;
    double FwdSum, RevSum, gbbdp, gbbsp, gbdpg, gbdpdp, gbdpb, gbdpsp, gbspg, gbspdp, gbspb, gbspsp;
    if (mi->mode >= 0) {
      FwdSum = Gm + Gmbs; RevSum = 0.0;
      gbbdp = -mi->gbds;
      gbbsp = (mi->gbds + mi->gbgs + mi->gbbs);
      gbdpg = mi->gbgs; gbdpdp = mi->gbds; gbdpb = mi->gbbs;
      gbdpsp = -(gbdpg + gbdpdp + gbdpb);
      gbspg = 0.0; gbspdp = 0.0; gbspb = 0.0; gbspsp = 0.0;
    } else {
      FwdSum = 0.0; RevSum = -(Gm + Gmbs);
      gbbsp = -mi->gbds;
      gbbdp = (mi->gbds + mi->gbgs + mi->gbbs);
      gbdpg = 0.0; gbdpsp = 0.0; gbdpb = 0.0; gbdpdp = 0.0;
      gbspg = mi->gbgs; gbspsp = mi->gbds; gbspb = mi->gbbs;
      gbspdp = -(gbspg + gbspsp + gbspb);
    }
    const double dxpart = mi->dxpart, sxpart = mi->sxpart, T1g = mi->T1global;
    xgo_madd(c, F, d, d, GD * M);
    xgo_msub(c, F, d, dp, GD * M);
    xgo_madd(c, F, s, s, GS * M);
    xgo_msub(c, F, s, sp, GS * M);
    xgo_madd(c, F, b, g, (-mi->gbgs) * M);
    xgo_madd(c, F, b, b, (mi->gbd + mi->gbs - mi->gbbs) * M);
    xgo_madd(c, F, b, dp, (-mi->gbd + gbbdp) * M);
    xgo_madd(c, F, b, sp, (-mi->gbs + gbbsp) * M);
    xgo_msub(c, F, dp, d, GD * M);
    xgo_msub(c, F, dp, b, (mi->gbd - Gmbs - dxpart * mi->ggtb - T1g * mi->ddxpart_dVb - gbdpb) * M);
    xgo_madd(c, F, dp, g, (Gm + dxpart * mi->ggtg + T1g * mi->ddxpart_dVg + gbdpg) * M);
    xgo_madd(c, F, dp, dp, (GD + mi->gds + mi->gbd + RevSum + dxpart * mi->ggtd + T1g * mi->ddxpart_dVd + gbdpdp) * M);
    xgo_msub(c, F, dp, sp, (mi->gds + FwdSum - dxpart * mi->ggts - T1g * mi->ddxpart_dVs - gbdpsp) * M);
    xgo_madd(c, F, sp, g, (-Gm + sxpart * mi->ggtg + T1g * mi->dsxpart_dVg + gbspg) * M);
    xgo_msub(c, F, sp, b, (mi->gbs + Gmbs - sxpart * mi->ggtb - T1g * mi->dsxpart_dVb - gbspb) * M);
    xgo_msub(c, F, sp, s, GS * M);
    xgo_msub(c, F, sp, dp, (mi->gds + RevSum - sxpart * mi->ggtd - T1g * mi->dsxpart_dVd - gbspdp) * M);
    xgo_madd(c, F, sp, sp, (GS + mi->gds + mi->gbs + FwdSum + sxpart * mi->ggts + T1g * mi->dsxpart_dVs + gbspsp) * M);
    if (!(!fl->dcop && fl->init_tran && fl->newton_iter == 0)) {
      xgo_madd(c, Q, g, g, (mem->CAPcggb) * M);
      xgo_msub(c, Q, g, b, (mem->CAPcggb + mem->CAPcgdb + mem->CAPcgsb) * M);
      xgo_madd(c, Q, g, dp, (mem->CAPcgdb) * M);
      xgo_madd(c, Q, g, sp, (mem->CAPcgsb) * M);
      xgo_madd(c, Q, b, g, (mem->CAPcbgb) * M);
      xgo_madd(c, Q, b, b, (-mem->CAPcbgb - mem->CAPcbdb - mem->CAPcbsb) * M);
      xgo_madd(c, Q, b, dp, (mem->CAPcbdb) * M);
      xgo_madd(c, Q, b, sp, (mem->CAPcbsb) * M);
      xgo_msub(c, Q, dp, b, (+mem->CAPcdgb + mem->CAPcddb + mem->CAPcdsb) * M);
      xgo_madd(c, Q, dp, g, (mem->CAPcdgb) * M);
      xgo_madd(c, Q, dp, dp, (+mem->CAPcddb) * M);
      xgo_msub(c, Q, dp, sp, (-mem->CAPcdsb) * M);
      xgo_madd(c, Q, sp, g, (mem->CAPcsgb) * M);
      xgo_msub(c, Q, sp, b, (+mem->CAPcsgb + mem->CAPcsdb + mem->CAPcssb) * M);
      xgo_msub(c, Q, sp, dp, (-mem->CAPcsdb) * M);
      xgo_madd(c, Q, sp, sp, (+mem->CAPcssb) * M);
    }
  }
  (void)dmin;
}
