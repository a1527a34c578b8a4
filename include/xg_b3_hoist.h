/*
 * xg_b3_hoist.h — the instance-constant columns of the BSIM3 parameter block
 * (include/xg_params.h, the entries after XG_B3_CZBSSWG), formed from the
 * block's other columns of one instance.
 *
 * Each is a subexpression of the reference's per-load evaluation
 * (src/DeviceModelPKG/OpenModels/src/N_DEV_MOSFET_B3.C,
 * Instance::updateIntermediateVars :4526-7273) that depends on instance
 * parameters only.  It is written here with the same operations in the same
 * order as it stands there, so a kernel that reads the column instead of
 * recomputing it produces the same bits; compile with -ffp-contract=off.
 * Set-up fills these columns once per instance; the evaluation then saves
 * their divides, square roots and products on every load.  The trailing
 * reciprocal columns serve the kernel's fused-multiply-add build only, which
 * multiplies by them where the reference divides.
 */
#ifndef XG_B3_HOIST_H
#define XG_B3_HOIST_H

#include <math.h>

#include "xg_params.h"

#define XG_B3_EXP_THRESHOLD 34.0 /* CONSTEXP_THRESHOLD */
#define XG_B3_EPSSI 1.03594e-10  /* CONSTEPSSI */

/* o: one instance's XG_B3_NPARAMS values, the raw columns filled. */
static inline void xg_b3_hoist(double *o) {
  const double phi = o[XG_B3_PHI], sqrtPhi = o[XG_B3_SQRTPHI], leff = o[XG_B3_LEFF];
  const double weff = o[XG_B3_WEFF], tox = o[XG_B3_TOX], cox = o[XG_B3_COX];
  const double vtm = o[XG_B3_VTM], k1ox = o[XG_B3_K1OX];
  const double TempRatio = o[XG_B3_TEMP] / o[XG_B3_TNOM] - 1.0;
  const double toxphi_w = tox * phi / (o[XG_B3_WEFF] + o[XG_B3_W0]);
  o[XG_B3_XDEP0_SQRTPHI] = o[XG_B3_XDEP0] / sqrtPhi;
  o[XG_B3_V0] = o[XG_B3_VBI] - phi;
  o[XG_B3_DVT1_LEFF] = -0.5 * o[XG_B3_DVT1] * leff;
  o[XG_B3_DVT1W_WL] = -0.5 * o[XG_B3_DVT1W] * weff * leff;
  o[XG_B3_TRATIO] = TempRatio;
  o[XG_B3_K1OX_NLX] = k1ox * (sqrt(1.0 + o[XG_B3_NLX] / leff) - 1.0) * sqrtPhi;
  o[XG_B3_KT1_L] = o[XG_B3_KT1] + o[XG_B3_KT1L] / leff;
  o[XG_B3_TOXPHI_W] = toxphi_w;
  o[XG_B3_VTH_BASE] = (int)o[XG_B3_DTYPE] * o[XG_B3_VTH0] - o[XG_B3_K1] * sqrtPhi;
  o[XG_B3_K3B_TOXPHI] = o[XG_B3_K3B] * toxphi_w;
  o[XG_B3_KT2_TRATIO] = o[XG_B3_KT2] * TempRatio;
  o[XG_B3_NFACTOR_EPSSI] = o[XG_B3_NFACTOR] * XG_B3_EPSSI;
  o[XG_B3_VFB_PHI] = o[XG_B3_VFB] + phi;
  o[XG_B3_VTMCDEP_COX] = vtm * o[XG_B3_CDEP0] / cox;
  o[XG_B3_MCOX_VTMCDEP] = -cox / (vtm * o[XG_B3_CDEP0]);
  o[XG_B3_B0_W] = o[XG_B3_B0] / (weff + o[XG_B3_B1]);
  o[XG_B3_AGS_A0] = o[XG_B3_AGS] * o[XG_B3_A0];
  o[XG_B3_VSAT2] = 2.0 * o[XG_B3_VSATTEMP];
  const double isub_a = o[XG_B3_ALPHA0] + o[XG_B3_ALPHA1] * leff;
  o[XG_B3_ISUB_A] = isub_a;
  o[XG_B3_ISUB_T2] = isub_a / leff;
  o[XG_B3_BETA0_ET] = o[XG_B3_BETA0] / XG_B3_EXP_THRESHOLD;
  o[XG_B3_PSCBE1_LITL] = o[XG_B3_PSCBE1] * o[XG_B3_LITL];
  o[XG_B3_PSCBE1_LITL_ET] = o[XG_B3_PSCBE1] * o[XG_B3_LITL] / XG_B3_EXP_THRESHOLD;
  o[XG_B3_COXWL] = cox * o[XG_B3_WEFFCV] * o[XG_B3_LEFFCV];
  o[XG_B3_D3_VFBZB] = 4.0 * 0.02 /* DELTA_3 */ * o[XG_B3_VFBZB];
  o[XG_B3_TOX8] = 1.0e8 * tox;
  const double link = 1.0e-3 * tox;
  o[XG_B3_LINK] = link;
  o[XG_B3_LINK4_LDEB] = 4.0 * link * o[XG_B3_LDEB];
  if (k1ox <= 0.0) {
    o[XG_B3_DPHI_DENOMI] = 0.25 * o[XG_B3_MOIN] * vtm;
    o[XG_B3_DPHI_T0] = 0.5 * sqrtPhi;
  } else {
    o[XG_B3_DPHI_DENOMI] = o[XG_B3_MOIN] * vtm * k1ox * k1ox;
    o[XG_B3_DPHI_T0] = k1ox * sqrtPhi;
  }
  o[XG_B3_VTM2] = 2.0 * vtm;
  const double pb = o[XG_B3_PHIB], pbsw = o[XG_B3_PHIBSW], pbswg = o[XG_B3_PHIBSWG];
  o[XG_B3_QBS0] = pb * o[XG_B3_CZBS];
  o[XG_B3_QBSSW0] = pbsw * o[XG_B3_CZBSSW];
  o[XG_B3_QBSSWG0] = pbswg * o[XG_B3_CZBSSWG];
  o[XG_B3_QBD0] = pb * o[XG_B3_CZBD];
  o[XG_B3_QBDSW0] = pbsw * o[XG_B3_CZBDSW];
  o[XG_B3_QBDSWG0] = pbswg * o[XG_B3_CZBDSWG];
  o[XG_B3_OMMJ] = 1.0 - o[XG_B3_MJ];
  o[XG_B3_OMMJSW] = 1.0 - o[XG_B3_MJSW];
  o[XG_B3_OMMJSWG] = 1.0 - o[XG_B3_MJSWG];
  o[XG_B3_CBS_F] = o[XG_B3_CZBS] * o[XG_B3_MJ] / pb;
  o[XG_B3_CBSSW_F] = o[XG_B3_CZBSSW] * o[XG_B3_MJSW] / pbsw;
  o[XG_B3_CBSSWG_F] = o[XG_B3_CZBSSWG] * o[XG_B3_MJSWG] / pbswg;
  o[XG_B3_CBD_F] = o[XG_B3_CZBD] * o[XG_B3_MJ] / pb;
  o[XG_B3_CBDSW_F] = o[XG_B3_CZBDSW] * o[XG_B3_MJSW] / pbsw;
  o[XG_B3_CBDSWG_F] = o[XG_B3_CZBDSWG] * o[XG_B3_MJSWG] / pbswg;
  const double cgdl_w = o[XG_B3_WEFFCV] * o[XG_B3_CGDL];
  const double cgsl_w = o[XG_B3_WEFFCV] * o[XG_B3_CGSL];
  o[XG_B3_CGDL_W] = cgdl_w;
  o[XG_B3_CGSL_W] = cgsl_w;
  o[XG_B3_CGDO_T] = o[XG_B3_CGDO] + cgdl_w;
  o[XG_B3_CGSO_T] = o[XG_B3_CGSO] + cgsl_w;
  o[XG_B3_HALF_CKAPPA] = 0.5 * o[XG_B3_CKAPPA];
  o[XG_B3_R_NVTM] = 1.0 / o[XG_B3_NVTM];
  o[XG_B3_R_SQRTPHI] = 1.0 / sqrtPhi;
  o[XG_B3_R_PHIS3] = 1.0 / o[XG_B3_PHIS3];
  o[XG_B3_R_COX] = 1.0 / cox;
  o[XG_B3_R_TOX] = 1.0 / tox;
  o[XG_B3_R_LEFF] = 1.0 / leff;
  o[XG_B3_R_THETAROUT] = 1.0 / o[XG_B3_THETAROUT];
  o[XG_B3_R_TOX8] = 1.0 / o[XG_B3_TOX8];
  o[XG_B3_R_PSCBE2] = 1.0 / o[XG_B3_PSCBE2];
  o[XG_B3_R_DPHI_DENOMI] = 1.0 / o[XG_B3_DPHI_DENOMI];
  o[XG_B3_R_CKAPPA] = 1.0 / o[XG_B3_CKAPPA];
  o[XG_B3_R_PHIB] = 1.0 / pb;
  o[XG_B3_R_PHIBSW] = 1.0 / pbsw;
  o[XG_B3_R_PHIBSWG] = 1.0 / pbswg;
  o[XG_B3_R_OMMJ] = 1.0 / o[XG_B3_OMMJ];
  o[XG_B3_R_OMMJSW] = 1.0 / o[XG_B3_OMMJSW];
  o[XG_B3_R_OMMJSWG] = 1.0 / o[XG_B3_OMMJSWG];
}

#endif /* XG_B3_HOIST_H */
