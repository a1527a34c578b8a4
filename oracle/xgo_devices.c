/*
 * xgo_devices.c — per-device-type load loops of the oracle
 * (TEST INFRASTRUCTURE ONLY; see xgo.h).  Each function restates one
 * reference Master method, statement for statement, over an instance range.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xgo_internal.h"

#define XGO_MAX_EXP_ARG 100.0 /* CONSTMAX_EXP_ARG, N_DEV_Const.h:106 */

static double dmin(double a, double b) { return a < b ? a : b; } /* Xycemin */
static double dmax(double a, double b) { return a > b ? a : b; } /* Xycemax */

/* ---- members carried from updateState to the vector/matrix loads ---------- */
typedef struct {
  double cbs, cbd, capbs, capbd, Capgs, Capgd, Capgb, qbs, qbd, qgs, qgd, qgb;
  double Idrain, Isource, cdreq, gbd, gbs, gds, Gm, Gmbs, revsum, nrmsum;
  double vbd, vbs, vds, vgs, vgd, Vgb, vbd_orig, vbs_orig, vds_orig, vgs_orig, vgd_orig;
  int mode, origFlag;
} m1m_t;

typedef struct {
  double Vp, Vpp, Vd, Vd_orig, Id, Gd, Qd, Cd;
} dm_t;

typedef struct { double i0; } rm_t;
typedef struct { double q0; } cm_t;
typedef struct { double srcCurrent, srcDrop, srcBC; } vm_t;

static void *members(xgo_circuit *c, int t, size_t sz) {
  xgo_type *T = &c->T[t];
  if (!T->m) T->m = calloc((size_t)T->n + 1, sz);
  return T->m;
}

/* ---- topology ------------------------------------------------------------- */

int xgo_nlid(int t) {
  switch (t) {
    case XG_DEV_RES: case XG_DEV_CAP: case XG_DEV_ISRC: return 2;
    case XG_DEV_VSRC: case XG_DEV_DIODE: return 3;
    case XG_DEV_MOS1: return 6;
    case XG_DEV_BSIM3: return xgo_b3_nlid();
  }
  return 0;
}

/* Circuit nodes are their own LIDs; internal unknowns are numbered in the
 * order each instance's registerLIDs consumes its intLIDVec. */
void xgo_assign_lids(xgo_circuit *c, const xg_netlist *nl, int t, int i, int *next) {
  xgo_type *T = &c->T[t];
  int *L = T->lid + (int64_t)i * T->nlid;
  switch (t) {
    case XG_DEV_RES: L[0] = nl->res.p[i]; L[1] = nl->res.m[i]; break;
    case XG_DEV_CAP: L[0] = nl->cap.p[i]; L[1] = nl->cap.m[i]; break;
    case XG_DEV_VSRC: /* N_DEV_Vsrc.C registerLIDs: li_Bra = intLIDVec[0] */
      L[0] = nl->vsrc.p[i]; L[1] = nl->vsrc.m[i]; L[2] = (*next)++; break;
    case XG_DEV_ISRC: /* N_DEV_ISRC.C:430-431: two external nodes, no internal */
      L[0] = nl->isrc.p[i]; L[1] = nl->isrc.m[i]; break;
    case XG_DEV_DIODE: /* N_DEV_Diode.C:456-459: li_Pri internal iff RS != 0 */
      L[0] = nl->diode.a[i]; L[1] = nl->diode.c[i];
      L[2] = (P(T, XG_D_GSPR, i) != 0.0) ? (*next)++ : L[0];
      break;
    case XG_DEV_MOS1: /* N_DEV_MOSFET1.C:1322-1330: d' then s' */
      L[0] = nl->mos1.d[i]; L[1] = nl->mos1.g[i]; L[2] = nl->mos1.s[i]; L[3] = nl->mos1.b[i];
      L[4] = P(T, XG_M1_GD, i) != 0.0 ? (*next)++ : L[0];
      L[5] = P(T, XG_M1_GS, i) != 0.0 ? (*next)++ : L[2];
      break;
    case XG_DEV_BSIM3: {
      int ext[4] = {nl->bsim3.d[i], nl->bsim3.g[i], nl->bsim3.s[i], nl->bsim3.b[i]};
      xgo_b3_lids(T, i, ext, next, L);
      break;
    }
  }
}

int xgo_nsta(const xgo_circuit *c, int t) {
  switch (t) {
    case XG_DEV_CAP: return 1;
    case XG_DEV_DIODE: /* per instance, counted in xgo_build */
      (void)c;
      return 0;
    case XG_DEV_MOS1: return 8;
    case XG_DEV_BSIM3: return 12;
  }
  return 0;
}

int xgo_nsto(int t) {
  switch (t) {
    case XG_DEV_DIODE: return 1;
    case XG_DEV_MOS1: return 5;
    case XG_DEV_BSIM3: return 5;
  }
  return 0;
}

int xgo_max_stamps(int t) {
  switch (t) {
    case XG_DEV_RES: case XG_DEV_CAP: case XG_DEV_VSRC: return 4;
    case XG_DEV_DIODE: return 7;
    case XG_DEV_MOS1: return 22;
    case XG_DEV_BSIM3: return 64;
  }
  return 0;
}

int xgo_stamps(const xgo_circuit *c, int t, int i, int *r, int *k) {
  const xgo_type *T = &c->T[t];
  const int *L = T->lid + (int64_t)i * T->nlid;
  int n = 0;
#define ST(a, b) (r[n] = (a), k[n] = (b), ++n)
  switch (t) {
    case XG_DEV_RES: case XG_DEV_CAP:
      ST(L[0], L[0]); ST(L[0], L[1]); ST(L[1], L[0]); ST(L[1], L[1]); break;
    case XG_DEV_VSRC:
      ST(L[0], L[2]); ST(L[1], L[2]); ST(L[2], L[0]); ST(L[2], L[1]); break;
    case XG_DEV_DIODE:
      ST(L[0], L[0]); ST(L[0], L[2]); ST(L[1], L[1]); ST(L[1], L[2]);
      ST(L[2], L[0]); ST(L[2], L[1]); ST(L[2], L[2]); break;
    case XG_DEV_MOS1: {
      int d = L[0], g = L[1], s = L[2], b = L[3], dp = L[4], sp = L[5];
      ST(d, d); ST(d, dp); ST(g, g); ST(g, b); ST(g, dp); ST(g, sp); ST(s, s); ST(s, sp);
      ST(b, g); ST(b, b); ST(b, dp); ST(b, sp); ST(dp, d); ST(dp, g); ST(dp, b); ST(dp, dp);
      ST(dp, sp); ST(sp, g); ST(sp, s); ST(sp, b); ST(sp, dp); ST(sp, sp);
      break;
    }
    case XG_DEV_BSIM3: return xgo_b3_stamps(T, i, r, k);
  }
#undef ST
  return n;
}

/* ---- PULSE source, PulseData::updateSource (N_DEV_SourceData.C:928-1031),
 *      break-point tolerance bpTol = 0 (SolverState default) ---------------- */
static double pulse_value(const xgo_type *T, int i, double t) {
  const double bpTol = 0.0;
  double V1 = P(T, XG_V_V1, i), V2 = P(T, XG_V_V2, i), TD = P(T, XG_V_TD, i);
  double TR = P(T, XG_V_TR, i), TF = P(T, XG_V_TF, i), PW = P(T, XG_V_PW, i);
  double PER = P(T, XG_V_PER, i);
  double time = t, basetime = 0;
  time -= TD;
  if (time > PER && PER != 0.0) {
    basetime = PER * floor(time / PER);
    time -= basetime;
  }
  if (time <= 0 || (time > (TR + PW + TF) && (fabs(time - (TR + PW + TF)) > bpTol)))
    return V1;
  if ((time > TR && fabs(time - TR) > bpTol) && (time < (TR + PW) || fabs(time - (TR + PW)) < bpTol))
    return V2;
  if (time > 0 && (time < TR || fabs(time - TR) < bpTol))
    return TR != 0.0 ? V1 + (V2 - V1) * (time) / TR : V1;
  return TF != 0.0 ? V2 + (V1 - V2) * (time - (TR + PW)) / TF : V2;
}

/* ---- MOSFET level 1 ------------------------------------------------------- */

/* Instance::updateIntermediateVars (N_DEV_MOSFET1.C:2618-3427) followed by the
 * store/state writes of Master::updateState (:4103-4192); newMeyer off. */
static void mos1_update(xgo_circuit *c, int i, xgo_io *io, m1m_t *m) {
  const xgo_type *T = &c->T[XG_DEV_MOS1];
  const xg_load_flags *fl = io->fl;
  const int *L = T->lid + (int64_t)i * 6;
  const int li_d = L[0], li_g = L[1], li_s = L[2], li_b = L[3], li_dp = L[4], li_sp = L[5];
  const int dtype = (int)P(T, XG_M1_DTYPE, i);
  const double gamma = P(T, XG_M1_GAMMA, i), lambda = P(T, XG_M1_LAMBDA, i);
  const double MJ = P(T, XG_M1_MJ, i), MJSW = P(T, XG_M1_MJSW, i);
  const double DrainSatCur = P(T, XG_M1_DRAINSATCUR, i), SourceSatCur = P(T, XG_M1_SOURCESATCUR, i);
  const double Beta = P(T, XG_M1_BETA, i), tVto = P(T, XG_M1_TVTO, i);
  const double sourceVcrit = P(T, XG_M1_SOURCEVCRIT, i), drainVcrit = P(T, XG_M1_DRAINVCRIT, i);
  const double vt = P(T, XG_M1_VT, i), tPhi = P(T, XG_M1_TPHI, i), tVbi = P(T, XG_M1_TVBI, i);
  const double Cbs = P(T, XG_M1_CBS, i), Cbssw = P(T, XG_M1_CBSSW, i);
  const double Cbd = P(T, XG_M1_CBD, i), Cbdsw = P(T, XG_M1_CBDSW, i);
  const double tDepCap = P(T, XG_M1_TDEPCAP, i), tBulkPot = P(T, XG_M1_TBULKPOT, i);
  const double f2s = P(T, XG_M1_F2S, i), f3s = P(T, XG_M1_F3S, i), f4s = P(T, XG_M1_F4S, i);
  const double f2d = P(T, XG_M1_F2D, i), f3d = P(T, XG_M1_F3D, i), f4d = P(T, XG_M1_F4D, i);
  const double OxideCap = P(T, XG_M1_OXIDECAP, i);
  const double GateSourceOverlapCap = P(T, XG_M1_CGSO, i);
  const double GateDrainOverlapCap = P(T, XG_M1_CGDO, i);
  const double GateBulkOverlapCap = P(T, XG_M1_CGBO, i);
  const double drainConductance = P(T, XG_M1_GD, i), sourceConductance = P(T, XG_M1_GS, i);
  const int flags = (int)P(T, XG_M1_FLAGS, i);
  const int OFF = flags & 1, IC_GIVEN = (flags >> 1) & 1;
  const double gmin = c->opt.gmin;
  const int voltlim = c->opt.voltlim;
  const double *sol = io->sol;
  double *sta = io->sta + T->sta0 + (int64_t)i * 8;
  double *sto = io->sto + T->sto0 + (int64_t)i * 5;
  const double *csta = io->sta_curr + T->sta0 + (int64_t)i * 8;
  const double *csto = io->sto_curr + T->sto0 + (int64_t)i * 5;
  enum { S_QGS, S_QGD, S_QGB, S_CAPGS, S_CAPGD, S_CAPGB, S_QBD, S_QBS };
  enum { O_VBD, O_VBS, O_VGS, O_VDS, O_VON };

  double Von, Vdsat, evbs, evbd, sarg, sargsw, arg;
  double vbs_old, vbd_old, vgs_old, vds_old, vgd_old;
  double capgs, capgd, capgb, gm, gds, gmbs, cdrain;
  int Check = 1;

  double Vd = sol[li_d], Vg = sol[li_g], Vs = sol[li_s], Vb = sol[li_b];
  double Vsp = sol[li_sp], Vdp = sol[li_dp];
  double Vddp = Vd - Vdp, Vssp = Vs - Vsp, Vbsp = Vb - Vsp;
  double Vgsp = Vg - Vsp, Vdpsp = Vdp - Vsp;
  double vbs = dtype * Vbsp, vgs = dtype * Vgsp, vds = dtype * Vdpsp;
  double vbd = vbs - vds, vgd = vgs - vds;
  double Vgb;
  int origFlag = 1;
  const double vgs_orig = vgs, vds_orig = vds, vbs_orig = vbs, vbd_orig = vbd, vgd_orig = vgd;

  if (fl->init_jct && !OFF && voltlim) {
    if (IC_GIVEN) {
      vds = dtype * P(T, XG_M1_ICVDS, i);
      vgs = dtype * P(T, XG_M1_ICVGS, i);
      vbs = dtype * P(T, XG_M1_ICVBS, i);
      vbd = vbs - vds;
      vgd = vgs - vds;
      origFlag = 0;
    } else {
      /* inputOP with an all-zero flag vector takes the same branch */
      vbs = -1;
      vgs = dtype * tVto;
      vds = 0;
      vbd = vbs - vds;
      vgd = vgs - vds;
    }
  } else if ((fl->init_fix || fl->init_jct) && OFF) {
    vbs = vgs = vds = 0;
    vbd = vgd = 0;
  }

  if (fl->newton_iter == 0) {
    if (!fl->dcop) {
      vbs_old = csto[O_VBS];
      vbd_old = csto[O_VBD];
      vgs_old = csto[O_VGS];
      vds_old = csto[O_VDS];
      Von = dtype * csto[O_VON];
    } else {
      vbs_old = vbs;
      vbd_old = vbd;
      vgs_old = vgs;
      vds_old = vds;
      Von = 0.0;
    }
    vgd_old = vgs_old - vds_old;
  } else {
    vbs_old = sto[O_VBS];
    vbd_old = sto[O_VBD];
    vgs_old = sto[O_VGS];
    vds_old = sto[O_VDS];
    Von = dtype * sto[O_VON];
    vgd_old = vgs_old - vds_old;
  }

  if (voltlim) {
    if (!(fl->init_fix && OFF)) {
      if (vds_old >= 0) {
        vgs = xgo_fetlim(vgs, vgs_old, Von);
        vds = vgs - vgd;
        vds = xgo_limvds(vds, vds_old);
        vgd = vgs - vds;
      } else {
        vgd = xgo_fetlim(vgd, vgd_old, Von);
        vds = vgs - vgd;
        vds = -xgo_limvds(-vds, -vds_old);
        vgs = vgd + vds;
      }
      if (vds >= 0.0) {
        vbs = xgo_pnjlim(vbs, vbs_old, vt, sourceVcrit, &Check);
        vbd = vbs - vds;
      } else {
        vbd = xgo_pnjlim(vbd, vbd_old, vt, drainVcrit, &Check);
        vbs = vbd + vds;
      }
    }
  }
  vbd = vbs - vds;
  vgd = vgs - vds;
  Vgb = vgs - vbs;
  if (vgs_orig != vgs || vds_orig != vds || vbs_orig != vbs || vbd_orig != vbd || vgd_orig != vgd)
    origFlag = 0;

  double gbs, cbs, gbd, cbd;
  if (vbs <= 0) {
    gbs = SourceSatCur / vt;
    gbs += gmin;
    cbs = gbs * vbs;
  } else {
    evbs = exp(dmin(XGO_MAX_EXP_ARG, vbs / vt));
    gbs = (SourceSatCur * evbs / vt + gmin);
    cbs = (SourceSatCur * (evbs - 1) + gmin * vbs);
  }
  if (vbd <= 0) {
    gbd = DrainSatCur / vt;
    gbd += gmin;
    cbd = gbd * vbd;
  } else {
    evbd = exp(dmin(XGO_MAX_EXP_ARG, vbd / vt));
    gbd = (DrainSatCur * evbd / vt + gmin);
    cbd = (DrainSatCur * (evbd - 1) + gmin * vbd);
  }
  const int mode = (vds >= 0) ? 1 : -1;
  {
    double betap, vgst;
    const double vbx = mode == 1 ? vbs : vbd;
    if (vbx <= 0) {
      sarg = sqrt(tPhi - vbx);
    } else {
      sarg = sqrt(tPhi);
      sarg = sarg - vbx / (sarg + sarg);
      sarg = dmax(0.0, sarg);
    }
    Von = (tVbi * dtype) + gamma * sarg;
    vgst = (mode == 1 ? vgs : vgd) - Von;
    Vdsat = dmax(vgst, 0.0);
    if (sarg <= 0) arg = 0;
    else arg = gamma / (sarg + sarg);
    if (vgst <= 0) {
      cdrain = 0; gm = 0; gds = 0; gmbs = 0;
    } else {
      betap = Beta * (1 + lambda * (vds * mode));
      if (vgst <= (vds * mode)) {
        cdrain = betap * vgst * vgst * .5;
        gm = betap * vgst;
        gds = lambda * Beta * vgst * vgst * .5;
        gmbs = gm * arg;
      } else {
        cdrain = betap * (vds * mode) * (vgst - .5 * (vds * mode));
        gm = betap * (vds * mode);
        gds = betap * (vgst - (vds * mode)) + lambda * Beta * (vds * mode) * (vgst - .5 * (vds * mode));
        gmbs = gm * arg;
      }
    }
  }
  const double von = dtype * Von;

  double qbs, capbs, qbd, capbd;
  if (Cbs != 0 || Cbssw != 0) {
    if (vbs < tDepCap) {
      arg = 1 - vbs / tBulkPot;
      if (MJ == MJSW) {
        if (MJ == .5) sarg = sargsw = 1 / sqrt(arg);
        else sarg = sargsw = exp(-MJ * log(arg));
      } else {
        if (MJ == .5) sarg = 1 / sqrt(arg);
        else sarg = exp(-MJ * log(arg));
        if (MJSW == .5) sargsw = 1 / sqrt(arg);
        else sargsw = exp(-MJSW * log(arg));
      }
      qbs = tBulkPot * (Cbs * (1 - arg * sarg) / (1 - MJ) + Cbssw * (1 - arg * sargsw) / (1 - MJSW));
      capbs = Cbs * sarg + Cbssw * sargsw;
    } else {
      qbs = f4s + vbs * (f2s + vbs * (f3s / 2));
      capbs = f2s + f3s * vbs;
    }
  } else {
    qbs = 0;
    capbs = 0;
  }
  if (Cbd != 0 || Cbdsw != 0) {
    if (vbd < tDepCap) {
      arg = 1 - vbd / tBulkPot;
      if (MJ == .5 && MJSW == .5) {
        sarg = sargsw = 1 / sqrt(arg);
      } else {
        if (MJ == .5) sarg = 1 / sqrt(arg);
        else sarg = exp(-MJ * log(arg));
        if (MJSW == .5) sargsw = 1 / sqrt(arg);
        else sargsw = exp(-MJSW * log(arg));
      }
      qbd = tBulkPot * (Cbd * (1 - arg * sarg) / (1 - MJ) + Cbdsw * (1 - arg * sargsw) / (1 - MJSW));
      capbd = Cbd * sarg + Cbdsw * sargsw;
    } else {
      qbd = f4d + vbd * (f2d + vbd * f3d / 2);
      capbd = f2d + vbd * f3d;
    }
  } else {
    qbd = 0;
    capbd = 0;
  }

  if (mode > 0)
    xgo_qmeyer(vgs, vgd, Vgb, Von, Vdsat, &capgs, &capgd, &capgb, tPhi, OxideCap);
  else
    xgo_qmeyer(vgd, vgs, Vgb, Von, Vdsat, &capgd, &capgs, &capgb, tPhi, OxideCap);

  double Capgs, Capgd, Capgb;
  if (fl->dcop) {
    Capgs = 2.0 * capgs + GateSourceOverlapCap;
    Capgd = 2.0 * capgd + GateDrainOverlapCap;
    Capgb = 2.0 * capgb + GateBulkOverlapCap;
  } else {
    Capgs = (capgs + csta[S_CAPGS] + GateSourceOverlapCap);
    Capgd = (capgd + csta[S_CAPGD] + GateDrainOverlapCap);
    Capgb = (capgb + csta[S_CAPGB] + GateBulkOverlapCap);
  }
  Capgs *= (Capgs < 0.0) ? -1.0 : 1.0;
  Capgd *= (Capgd < 0.0) ? -1.0 : 1.0;
  Capgb *= (Capgb < 0.0) ? -1.0 : 1.0;

  m->Idrain = drainConductance * Vddp;
  m->Isource = sourceConductance * Vssp;
  if (mode >= 0) {
    m->Gm = gm; m->Gmbs = gmbs;
    m->nrmsum = m->Gm + m->Gmbs;
    m->revsum = 0;
    m->cdreq = dtype * cdrain;
  } else {
    m->Gm = -gm; m->Gmbs = -gmbs;
    m->nrmsum = 0;
    m->revsum = -(m->Gm + m->Gmbs);
    m->cdreq = -(dtype) * cdrain;
  }
  m->cbs = cbs; m->cbd = cbd; m->gbs = gbs; m->gbd = gbd; m->gds = gds;
  m->capbs = capbs; m->capbd = capbd; m->qbs = qbs; m->qbd = qbd;
  m->Capgs = Capgs; m->Capgd = Capgd; m->Capgb = Capgb;
  m->vbd = vbd; m->vbs = vbs; m->vds = vds; m->vgs = vgs; m->vgd = vgd; m->Vgb = Vgb;
  m->vbd_orig = vbd_orig; m->vbs_orig = vbs_orig; m->vds_orig = vds_orig;
  m->vgs_orig = vgs_orig; m->vgd_orig = vgd_orig;
  m->mode = mode; m->origFlag = origFlag;

  /* Master::updateState store/state writes (N_DEV_MOSFET1.C:4117-4190). */
  sto[O_VBD] = vbd; sto[O_VBS] = vbs; sto[O_VGS] = vgs; sto[O_VDS] = vds; sto[O_VON] = von;
  sta[S_CAPGS] = capgs; sta[S_CAPGD] = capgd; sta[S_CAPGB] = capgb;
  double qgs, qgd, qgb;
  if (fl->dcop) {
    qgs = Capgs * vgs;
    qgd = Capgd * vgd;
    qgb = Capgb * Vgb;
  } else {
    qgs = csta[S_QGS];
    qgd = csta[S_QGD];
    qgb = csta[S_QGB];
    double vgs1 = csto[O_VGS], vbs1 = csto[O_VBS], vds1 = csto[O_VDS];
    double vgb1 = vgs1 - vbs1, vgd1 = vgs1 - vds1;
    qgs += Capgs * (vgs - vgs1);
    qgd += Capgd * (vgd - vgd1);
    qgb += Capgb * ((vgs - vbs) - vgb1);
  }
  m->qgs = qgs; m->qgd = qgd; m->qgb = qgb;
  sta[S_QGS] = qgs; sta[S_QGD] = qgd; sta[S_QGB] = qgb;
  sta[S_QBD] = qbd; sta[S_QBS] = qbs;
}

/* Master::loadDAEVectors (N_DEV_MOSFET1.C:4202-4430), newMeyer off. */
static void mos1_vectors(xgo_circuit *c, int i, xgo_io *io, const m1m_t *mi) {
  const xgo_type *T = &c->T[XG_DEV_MOS1];
  const xg_load_flags *fl = io->fl;
  const int *L = T->lid + (int64_t)i * 6;
  const int li_d = L[0], li_g = L[1], li_s = L[2], li_b = L[3], li_dp = L[4], li_sp = L[5];
  const int Dtype = (int)P(T, XG_M1_DTYPE, i);
  const double numberParallel = P(T, XG_M1_M, i);
  const double drainConductance = P(T, XG_M1_GD, i), sourceConductance = P(T, XG_M1_GS, i);
  const double gmin1 = c->opt.gmin;
  double *fVec = io->f, *qVec = io->q;
  double ceqbs = Dtype * (mi->cbs), ceqbd = Dtype * (mi->cbd);
  double ceqgb = 0.0, ceqgs = 0.0, ceqgd = 0.0, coef;

  if (drainConductance != 0.0) fVec[li_d] += mi->Idrain * numberParallel;
  coef = (ceqgs + ceqgd + ceqgb);
  fVec[li_g] += coef * numberParallel;
  if (sourceConductance != 0.0) fVec[li_s] += mi->Isource * numberParallel;
  coef = ceqbs + ceqbd - ceqgb;
  fVec[li_b] += coef * numberParallel;
  coef = -mi->Idrain - (ceqbd - mi->cdreq + ceqgd);
  fVec[li_dp] += coef * numberParallel;
  coef = -mi->Isource - (ceqbs + mi->cdreq + ceqgs);
  fVec[li_sp] += coef * numberParallel;

  double Qeqbs = Dtype * (mi->qbs), Qeqbd = Dtype * (mi->qbd), Qeqgb = Dtype * (mi->qgb);
  double Qeqgs = Dtype * (mi->qgs), Qeqgd = Dtype * (mi->qgd);
  coef = (Qeqgs + Qeqgd + Qeqgb);
  qVec[li_g] += coef * numberParallel;
  coef = Qeqbs + Qeqbd - Qeqgb;
  qVec[li_b] += coef * numberParallel;
  coef = -(Qeqbd + Qeqgd);
  qVec[li_dp] += coef * numberParallel;
  coef = -(Qeqbs + Qeqgs);
  qVec[li_sp] += coef * numberParallel;

  if (!mi->origFlag) {
    double dvgs = mi->vgs - mi->vgs_orig, dvgd = mi->vgd - mi->vgd_orig;
    double dvbs = mi->vbs - mi->vbs_orig, dvbd = mi->vbd - mi->vbd_orig;
    double dvds = mi->vds - mi->vds_orig;
    double coef_Jdxp4 = Dtype * (+((mi->gbd - gmin1)) * (dvbd) + ((mi->gbs - gmin1)) * (dvbs));
    double coef_Jdxp5 = Dtype * (-((mi->gbd - gmin1)) * (dvbd) + mi->gds * (dvds) +
                                 mi->Gm * ((mi->mode > 0) ? dvgs : dvgd) +
                                 mi->Gmbs * ((mi->mode > 0) ? dvbs : dvbd));
    double coef_Jdxp6 = Dtype * (-((mi->gbs - gmin1)) * (dvbs) - mi->gds * (dvds) -
                                 mi->Gm * ((mi->mode > 0) ? dvgs : dvgd) -
                                 mi->Gmbs * ((mi->mode > 0) ? dvbs : dvbd));
    io->dfdxdvp[li_b] += coef_Jdxp4 * numberParallel;
    io->dfdxdvp[li_dp] += coef_Jdxp5 * numberParallel;
    io->dfdxdvp[li_sp] += coef_Jdxp6 * numberParallel;
    double gcgd = 0.0, gcgs = 0.0, gcgb = 0.0, gcbs = 0.0, gcbd = 0.0;
    if (fl->tranop || fl->acop || fl->transient) {
      gcgd = mi->Capgd; gcgs = mi->Capgs; gcgb = mi->Capgb;
      gcbs = mi->capbs; gcbd = mi->capbd;
    }
    double coef_Jdxp2 = Dtype * (gcgd * (dvgd) + gcgs * (dvgs) +
                                 gcgb * (mi->vgs - mi->vgs_orig - mi->vbs + mi->vbs_orig));
    double qJdxp4 = Dtype * (-(gcgb) * (mi->vgs - mi->vgs_orig - mi->vbs + mi->vbs_orig) +
                             (gcgb) * (dvbd) + (gcbs) * (dvbs));
    double qJdxp5 = Dtype * (-(gcgd) * (dvgd) - (gcbd) * (dvbd));
    double qJdxp6 = Dtype * (-gcgs * (dvgs) - (gcbs) * (dvbs));
    io->dqdxdvp[li_g] += coef_Jdxp2 * numberParallel;
    io->dqdxdvp[li_b] += qJdxp4 * numberParallel;
    io->dqdxdvp[li_dp] += qJdxp5 * numberParallel;
    io->dqdxdvp[li_sp] += qJdxp6 * numberParallel;
  }
}

/* Master::loadDAEMatrices, pointer path (N_DEV_MOSFET1.C:4441-4722), newMeyer off. */
static void mos1_matrices(xgo_circuit *c, int i, xgo_io *io, const m1m_t *mi) {
  const xgo_type *T = &c->T[XG_DEV_MOS1];
  const xg_load_flags *fl = io->fl;
  const int *L = T->lid + (int64_t)i * 6;
  const int d = L[0], g = L[1], s = L[2], b = L[3], dp = L[4], sp = L[5];
  const double M = P(T, XG_M1_M, i);
  const double GD = P(T, XG_M1_GD, i), GS = P(T, XG_M1_GS, i);
  double *F = io->dfdx, *Q = io->dqdx;
  xgo_madd(c, F, d, d, GD * M);
  xgo_msub(c, F, d, dp, GD * M);
  xgo_madd(c, F, s, s, GS * M);
  xgo_msub(c, F, s, sp, GS * M);
  xgo_madd(c, F, b, b, (mi->gbs + mi->gbd) * M);
  xgo_msub(c, F, b, dp, mi->gbd * M);
  xgo_msub(c, F, b, sp, mi->gbs * M);
  xgo_msub(c, F, dp, d, GD * M);
  xgo_madd(c, F, dp, g, (mi->Gm) * M);
  xgo_madd(c, F, dp, b, (-mi->gbd + mi->Gmbs) * M);
  xgo_madd(c, F, dp, dp, (GD + mi->gds + mi->gbd + mi->revsum) * M);
  xgo_madd(c, F, dp, sp, (-mi->gds - mi->nrmsum) * M);
  xgo_msub(c, F, sp, g, (mi->Gm) * M);
  xgo_msub(c, F, sp, s, GS * M);
  xgo_msub(c, F, sp, b, (mi->gbs + mi->Gmbs) * M);
  xgo_msub(c, F, sp, dp, (mi->gds + mi->revsum) * M);
  xgo_madd(c, F, sp, sp, (GS + mi->gds + mi->gbs + mi->nrmsum) * M);

  double gcgd = 0.0, gcgs = 0.0, gcgb = 0.0, gcbs = 0.0, gcbd = 0.0;
  if (fl->tranop || fl->acop || fl->transient) {
    gcgd = mi->Capgd; gcgs = mi->Capgs; gcgb = mi->Capgb;
    gcbs = mi->capbs; gcbd = mi->capbd;
  }
  xgo_madd(c, Q, g, g, (gcgd + gcgs + gcgb) * M);
  xgo_msub(c, Q, g, b, gcgb * M);
  xgo_msub(c, Q, g, dp, gcgd * M);
  xgo_msub(c, Q, g, sp, gcgs * M);
  xgo_msub(c, Q, b, g, gcgb * M);
  xgo_madd(c, Q, b, b, (+gcbs + gcbd + gcgb) * M);
  xgo_msub(c, Q, b, dp, +gcbd * M);
  xgo_msub(c, Q, b, sp, +gcbs * M);
  xgo_madd(c, Q, dp, g, -gcgd * M);
  xgo_madd(c, Q, dp, b, -gcbd * M);
  xgo_madd(c, Q, dp, dp, (+gcbd + gcgd) * M);
  xgo_msub(c, Q, sp, g, gcgs * M);
  xgo_msub(c, Q, sp, b, +gcbs * M);
  xgo_madd(c, Q, sp, sp, (+gcbs + gcgs) * M);
}

/* ---- diode, level 1 (lambertW off) ---------------------------------------- */

/* Master::updateState (N_DEV_Diode.C:2007-2020) -> updateIntermediateVars
 * (:873-1331, level 1 branch). */
static void diode_update(xgo_circuit *c, int i, xgo_io *io, dm_t *m) {
  const xgo_type *T = &c->T[XG_DEV_DIODE];
  const xg_load_flags *fl = io->fl;
  const int *L = T->lid + (int64_t)i * 3;
  const int li_Pos = L[0], li_Neg = L[1], li_Pri = L[2];
  double *sto = io->sto + T->sto0 + i;
  const double *csto = io->sto_curr + T->sto0 + i;
  const double gmin = c->opt.gmin;
  const double M = P(T, XG_D_M, i), BV = P(T, XG_D_BV, i), N = P(T, XG_D_N, i);
  const double TT = P(T, XG_D_TT, i), F2 = P(T, XG_D_F2, i), F3 = P(T, XG_D_F3, i);
  const double tVcrit = P(T, XG_D_TVCRIT, i), tIRF = P(T, XG_D_TIRF, i);
  const double tBrkdwnV = P(T, XG_D_TBRKDWNV, i), tJctCap = P(T, XG_D_TJCTCAP, i);
  const double tJctPot = P(T, XG_D_TJCTPOT, i), tDepCap = P(T, XG_D_TDEPCAP, i);
  const double tF1 = P(T, XG_D_TF1, i), Area = P(T, XG_D_AREA, i);
  const int flags = (int)P(T, XG_D_FLAGS, i);
  const int BVGiven = flags & 1, InitCondGiven = (flags >> 1) & 1, off = (flags >> 2) & 1;

  sto[0] = c->diode_vd[i]; /* stoVec[li_storevd] = di.Vd, before the update */

  const double *solVec = io->sol;
  double Vpp = solVec[li_Pri], Vn = solVec[li_Neg], Vp = solVec[li_Pos];
  double Vd = Vpp - Vn;
  double Isat = P(T, XG_D_ISAT, i);
  double Vt = P(T, XG_D_VT, i);
  double Vte = N * Vt;
  double Vd_old;
  const double Vd_orig = Vd;
  if (fl->newton_iter == 0) {
    if (fl->init_jct && c->opt.voltlim) {
      if (InitCondGiven) Vd = P(T, XG_D_INITCOND, i);
      else if (off) Vd = 0.0;
      else Vd = tVcrit;
    }
    Vd_old = Vd;
    if (!fl->dcop) Vd_old = csto[0];
  } else {
    Vd_old = sto[0];
  }
  if (c->opt.voltlim) {
    int ichk = 0;
    if (fl->newton_iter >= 0) {
      if (BVGiven && (Vd < dmin(0.0, -BV + 10.0 * Vte))) {
        double Vdtmp = -(BV + Vd);
        Vdtmp = xgo_pnjlim(Vdtmp, -(Vd_old + BV), Vte, tVcrit, &ichk);
        Vd = -(Vdtmp + BV);
      } else {
        Vd = xgo_pnjlim(Vd, Vd_old, Vte, tVcrit, &ichk);
      }
    }
  }
  double Id, Gd;
  {
    double IRfactor;
    if (Vd >= -3.0 * Vte) IRfactor = 1.0;
    else IRfactor = tIRF;
    Isat *= IRfactor;
    if (Vd >= -3.0 * Vte) {
      double arg1 = Vd / Vte;
      arg1 = dmin(XGO_MAX_EXP_ARG, arg1);
      double evd = exp(arg1);
      Id = Isat * (evd - 1.0) + gmin * Vd;
      Gd = Isat * evd / Vte + gmin;
    } else if (!tBrkdwnV || (Vd >= -tBrkdwnV)) {
      double arg = 3.0 * Vte / (Vd * exp(1.0));
      arg = arg * arg * arg;
      Id = -Isat * (1.0 + arg) + gmin * Vd;
      Gd = Isat * 3.0 * arg / Vd + gmin;
    } else {
      double arg1 = -(tBrkdwnV + Vd) / Vte;
      arg1 = dmin(XGO_MAX_EXP_ARG, arg1);
      double evrev = exp(arg1);
      double arg2 = 3.0 * Vte / (exp(1.0) * tBrkdwnV);
      arg2 = arg2 * arg2 * arg2;
      double Isat_tBrkdwnV = Isat * (1 - arg2);
      Id = -Isat_tBrkdwnV * evrev + gmin * Vd;
      Gd = Isat_tBrkdwnV * evrev / Vte + gmin;
    }
  }
  double Vc = Vd, Qd, Cd;
  if (tJctCap != 0.0) {
    double Czero = tJctCap * Area;
    if (Vc < tDepCap) {
      double arg = 1.0 - Vc / tJctPot;
      double arg1 = -M * log(arg);
      arg1 = dmin(XGO_MAX_EXP_ARG, arg1);
      double sarg = exp(arg1);
      Qd = TT * Id + tJctPot * Czero * (1.0 - arg * sarg) / (1.0 - M);
      Cd = TT * Gd + Czero * sarg;
    } else {
      double Czof2 = Czero / F2;
      double MotJctPot = M / tJctPot;
      Qd = TT * Id + Czero * tF1 +
           Czof2 * (F3 * (Vc - tDepCap) + (0.5 * MotJctPot) * (Vc * Vc - tDepCap * tDepCap));
      Cd = TT * Gd + Czof2 * (F3 + MotJctPot * Vc);
    }
  } else {
    Qd = 0.0;
    Cd = 0.0;
  }
  m->Vp = Vp; m->Vpp = Vpp; m->Vd = Vd; m->Vd_orig = Vd_orig;
  m->Id = Id; m->Gd = Gd; m->Qd = Qd; m->Cd = Cd;
  c->diode_vd[i] = Vd;
}

/* Master::loadDAEVectors (N_DEV_Diode.C:2034-2086). */
static void diode_vectors(xgo_circuit *c, int i, xgo_io *io, const dm_t *di) {
  const xgo_type *T = &c->T[XG_DEV_DIODE];
  const int *L = T->lid + (int64_t)i * 3;
  const int li_Pos = L[0], li_Neg = L[1], li_Pri = L[2];
  const double Gspr = P(T, XG_D_GSPR, i);
  double Ir = Gspr * (di->Vp - di->Vpp);
  io->f[li_Pos] -= -Ir;
  io->f[li_Neg] -= di->Id;
  io->f[li_Pri] -= (-di->Id + Ir);
  io->q[li_Neg] -= di->Qd;
  io->q[li_Pri] -= -di->Qd;
  if (c->opt.voltlim) {
    double Vd_diff = di->Vd - di->Vd_orig;
    double Cd_Jdxp = -(di->Cd) * Vd_diff;
    double Gd_Jdxp = -(di->Gd) * Vd_diff;
    io->dfdxdvp[li_Neg] += Gd_Jdxp;
    io->dfdxdvp[li_Pri] -= Gd_Jdxp;
    io->dqdxdvp[li_Neg] += Cd_Jdxp;
    io->dqdxdvp[li_Pri] -= Cd_Jdxp;
  }
}

/* Master::loadDAEMatrices (N_DEV_Diode.C:2088-2128). */
static void diode_matrices(xgo_circuit *c, int i, xgo_io *io, const dm_t *di) {
  const xgo_type *T = &c->T[XG_DEV_DIODE];
  const int *L = T->lid + (int64_t)i * 3;
  const int p = L[0], n = L[1], r = L[2];
  const double Gspr = P(T, XG_D_GSPR, i);
  double *F = io->dfdx, *Q = io->dqdx;
  xgo_madd(c, F, p, p, Gspr);
  xgo_msub(c, F, p, r, Gspr);
  xgo_madd(c, F, n, n, di->Gd);
  xgo_msub(c, F, n, r, di->Gd);
  xgo_msub(c, F, r, p, Gspr);
  xgo_msub(c, F, r, n, di->Gd);
  xgo_madd(c, F, r, r, Gspr + di->Gd);
  xgo_madd(c, Q, n, n, di->Cd);
  xgo_msub(c, Q, n, r, di->Cd);
  xgo_msub(c, Q, r, n, di->Cd);
  xgo_madd(c, Q, r, r, di->Cd);
}

/* ---- dispatch ------------------------------------------------------------- */

void xgo_update_state(xgo_circuit *c, int t, int i0, int i1, xgo_io *io) {
  xgo_type *T = &c->T[t];
  const double *sol = io->sol;
  switch (t) {
    case XG_DEV_RES: { /* N_DEV_Resistor.C:1073-1085 */
      rm_t *m = (rm_t *)members(c, t, sizeof(rm_t));
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        m[i].i0 = (sol[L[0]] - sol[L[1]]) * P(T, XG_R_G, i);
      }
      break;
    }
    case XG_DEV_CAP: { /* N_DEV_Capacitor.C:1821-1850 (constant C, no IC) */
      cm_t *m = (cm_t *)members(c, t, sizeof(cm_t));
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        double vcap = sol[L[0]] - sol[L[1]];
        m[i].q0 = P(T, XG_C_C, i) * vcap;
        io->sta[T->sta0 + i] = m[i].q0;
      }
      break;
    }
    case XG_DEV_VSRC: { /* N_DEV_Vsrc.C:941-1000 */
      vm_t *m = (vm_t *)members(c, t, sizeof(vm_t));
      const xg_load_flags *fl = io->fl;
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 3;
        double source;
        if ((fl->tranop || fl->transient) && P(T, XG_V_KIND, i) == XG_SRC_PULSE)
          source = pulse_value(T, i, fl->time);
        else
          source = P(T, XG_V_V1, i);
        m[i].srcCurrent = sol[L[2]];
        m[i].srcDrop = (sol[L[0]] - sol[L[1]]);
        m[i].srcBC = source;
      }
      break;
    }
    case XG_DEV_DIODE: {
      dm_t *m = (dm_t *)members(c, t, sizeof(dm_t));
      for (int i = i0; i < i1; ++i) diode_update(c, i, io, &m[i]);
      break;
    }
    case XG_DEV_MOS1: {
      m1m_t *m = (m1m_t *)members(c, t, sizeof(m1m_t));
      for (int i = i0; i < i1; ++i) mos1_update(c, i, io, &m[i]);
      break;
    }
    case XG_DEV_BSIM3: xgo_b3_update_state(c, i0, i1, io); break;
  }
}

void xgo_load_vectors(xgo_circuit *c, int t, int i0, int i1, xgo_io *io) {
  xgo_type *T = &c->T[t];
  switch (t) {
    case XG_DEV_RES: { /* N_DEV_Resistor.C:1094-1110 */
      const rm_t *m = (const rm_t *)T->m;
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        io->f[L[0]] += m[i].i0;
        io->f[L[1]] += -m[i].i0;
      }
      break;
    }
    case XG_DEV_CAP: { /* N_DEV_Capacitor.C:1881-1990 */
      const cm_t *m = (const cm_t *)T->m;
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        io->q[L[0]] += m[i].q0;
        io->q[L[1]] += -m[i].q0;
      }
      break;
    }
    case XG_DEV_ISRC: { /* N_DEV_ISRC.C:774-800: F only, no matrix entries */
      const xg_load_flags *fl = io->fl;
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        double source;
        if ((fl->tranop || fl->transient) && P(T, XG_V_KIND, i) == XG_SRC_PULSE)
          source = pulse_value(T, i, fl->time);
        else
          source = P(T, XG_V_V1, i);
        io->f[L[0]] += source;
        io->f[L[1]] -= source;
      }
      break;
    }
    case XG_DEV_VSRC: { /* N_DEV_Vsrc.C:1002-1021 */
      const vm_t *m = (const vm_t *)T->m;
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 3;
        io->f[L[0]] += m[i].srcCurrent;
        io->f[L[1]] += -m[i].srcCurrent;
        io->f[L[2]] += m[i].srcDrop;
        io->f[L[2]] -= m[i].srcBC;
      }
      break;
    }
    case XG_DEV_DIODE: {
      const dm_t *m = (const dm_t *)T->m;
      for (int i = i0; i < i1; ++i) diode_vectors(c, i, io, &m[i]);
      break;
    }
    case XG_DEV_MOS1: {
      const m1m_t *m = (const m1m_t *)T->m;
      for (int i = i0; i < i1; ++i) mos1_vectors(c, i, io, &m[i]);
      break;
    }
    case XG_DEV_BSIM3: xgo_b3_load_vectors(c, i0, i1, io); break;
  }
}

void xgo_load_matrices(xgo_circuit *c, int t, int i0, int i1, xgo_io *io) {
  xgo_type *T = &c->T[t];
  switch (t) {
    case XG_DEV_RES: /* N_DEV_Resistor.C:1119-1135 */
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        double G = P(T, XG_R_G, i);
        xgo_madd(c, io->dfdx, L[0], L[0], G);
        xgo_msub(c, io->dfdx, L[0], L[1], G);
        xgo_msub(c, io->dfdx, L[1], L[0], G);
        xgo_madd(c, io->dfdx, L[1], L[1], G);
      }
      break;
    case XG_DEV_CAP: /* N_DEV_Capacitor.C:2002-2040 */
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 2;
        double C = P(T, XG_C_C, i);
        xgo_madd(c, io->dqdx, L[0], L[0], C);
        xgo_msub(c, io->dqdx, L[0], L[1], C);
        xgo_msub(c, io->dqdx, L[1], L[0], C);
        xgo_madd(c, io->dqdx, L[1], L[1], C);
      }
      break;
    case XG_DEV_VSRC: /* N_DEV_Vsrc.C:1023-1045 */
      for (int i = i0; i < i1; ++i) {
        const int *L = T->lid + (int64_t)i * 3;
        xgo_madd(c, io->dfdx, L[0], L[2], 1.0);
        xgo_msub(c, io->dfdx, L[1], L[2], 1.0);
        xgo_madd(c, io->dfdx, L[2], L[0], 1.0);
        xgo_msub(c, io->dfdx, L[2], L[1], 1.0);
      }
      break;
    case XG_DEV_DIODE: {
      const dm_t *m = (const dm_t *)T->m;
      for (int i = i0; i < i1; ++i) diode_matrices(c, i, io, &m[i]);
      break;
    }
    case XG_DEV_MOS1: {
      const m1m_t *m = (const m1m_t *)T->m;
      for (int i = i0; i < i1; ++i) mos1_matrices(c, i, io, &m[i]);
      break;
    }
    case XG_DEV_BSIM3: xgo_b3_load_matrices(c, i0, i1, io); break;
  }
}
