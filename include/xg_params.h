/*
 * xg_params.h — layout of the per-instance parameter blocks that circuit setup
 * derives on the host (the reference's Instance constructor, processParams and
 * updateTemperature) and that the load kernels read, one structure-of-arrays
 * column per entry: column k of device type T holds parameter k of every
 * instance of T.  xg_circuit_get_params() returns these blocks.
 *
 * Each name is the reference member it holds (file:line of the computation).
 */
#ifndef XG_PARAMS_H
#define XG_PARAMS_H

#ifdef __cplusplus
extern "C" {
#endif

/* MOSFET level 1 — N_DEV_MOSFET1.C ctor :1175-1250, updateTemperature :3437-3680,
 * updateIntermediateVars :2650-2665 (sat currents, Beta). */
enum xg_mos1_param {
  XG_M1_DTYPE = 0,          /* model_.dtype (+1 / -1)                    */
  XG_M1_GAMMA,              /* model_.gamma                              */
  XG_M1_LAMBDA,             /* model_.lambda                             */
  XG_M1_MJ,                 /* model_.bulkJctBotGradingCoeff             */
  XG_M1_MJSW,               /* model_.bulkJctSideGradingCoeff            */
  XG_M1_DRAINSATCUR,        /* DrainSatCur                               */
  XG_M1_SOURCESATCUR,       /* SourceSatCur                              */
  XG_M1_BETA,               /* tTransconductance * w / EffectiveLength   */
  XG_M1_TVTO,
  XG_M1_SOURCEVCRIT,
  XG_M1_DRAINVCRIT,
  XG_M1_VT,
  XG_M1_TPHI,
  XG_M1_TVBI,
  XG_M1_CBS, XG_M1_CBSSW, XG_M1_CBD, XG_M1_CBDSW,
  XG_M1_TDEPCAP,
  XG_M1_TBULKPOT,
  XG_M1_F2S, XG_M1_F3S, XG_M1_F4S, XG_M1_F2D, XG_M1_F3D, XG_M1_F4D,
  XG_M1_OXIDECAP,
  XG_M1_CGSO,               /* GateSourceOverlapCap                      */
  XG_M1_CGDO,               /* GateDrainOverlapCap                       */
  XG_M1_CGBO,               /* GateBulkOverlapCap                        */
  XG_M1_GD,                 /* drainConductance                          */
  XG_M1_GS,                 /* sourceConductance                         */
  XG_M1_M,                  /* numberParallel                            */
  XG_M1_ICVDS, XG_M1_ICVGS, XG_M1_ICVBS,
  XG_M1_FLAGS,              /* bit0 OFF, bit1 IC given (as a double)     */
  XG_M1_NPARAMS
};

/* Junction diode, level 1 — N_DEV_Diode.C updateTemperature :1335-1500,
 * Model::processParams :1772-1790, updateIntermediateVars :873-1331. */
enum xg_diode_param {
  XG_D_M = 0,               /* model_.M (grading, clipped to 0.9)        */
  XG_D_BV,                  /* model_.BV                                 */
  XG_D_N,                   /* model_.N                                  */
  XG_D_TT,                  /* model_.TT                                 */
  XG_D_F2, XG_D_F3,         /* model_.F2, model_.F3                      */
  XG_D_ISAT,                /* tSatCur * Area                            */
  XG_D_VT,                  /* CONSTKoverQ * Temp                        */
  XG_D_GSPR,                /* tCOND * Area                              */
  XG_D_TVCRIT,
  XG_D_TIRF,
  XG_D_TBRKDWNV,
  XG_D_TJCTCAP,
  XG_D_TJCTPOT,
  XG_D_TDEPCAP,
  XG_D_TF1,
  XG_D_AREA,
  XG_D_INITCOND,
  XG_D_FLAGS,               /* bit0 BV given, bit1 IC given, bit2 off    */
  XG_D_NPARAMS
};

/* BSIM3 v3.2 — N_DEV_MOSFET_B3.C.  Columns 0..XG_B3_NRAW-1 are reference
 * members: the instance's SizeDependParam (updateTemperature :3736-4470), the
 * model constants the evaluation reads (Model::processParams :8488-8570) and
 * the instance temperature values (:3639-3727, :4472-4511).  The columns after
 * XG_B3_NRAW are instance constants the evaluation would otherwise recompute
 * at every load, formed on the host by the same expressions. */
enum xg_b3_param {
  /* model */
  XG_B3_DTYPE = 0, XG_B3_MOBMOD, XG_B3_CAPMOD, XG_B3_XPART, XG_B3_TOX, XG_B3_COX,
  XG_B3_FACTOR1, XG_B3_VCRIT, XG_B3_NJ, XG_B3_IJTH, XG_B3_MJ, XG_B3_MJSW, XG_B3_MJSWG,
  XG_B3_TNOM,
  /* instance temperature / geometry */
  XG_B3_TEMP, XG_B3_VTM, XG_B3_JSTEMP, XG_B3_JSWTEMP, XG_B3_CJTEMP, XG_B3_CJSWTEMP,
  XG_B3_CJSWGTEMP, XG_B3_PHIB, XG_B3_PHIBSW, XG_B3_PHIBSWG, XG_B3_VJSM, XG_B3_ISEVJSM,
  XG_B3_VJDM, XG_B3_ISEVJDM, XG_B3_AD, XG_B3_AS, XG_B3_PD, XG_B3_PS, XG_B3_GD, XG_B3_GS,
  XG_B3_M, XG_B3_FLAGS /* bit0 OFF */,
  /* SizeDependParam */
  XG_B3_VTH0, XG_B3_VBSC, XG_B3_PHI, XG_B3_PHIS3, XG_B3_SQRTPHI, XG_B3_XDEP0, XG_B3_LEFF,
  XG_B3_WEFF, XG_B3_VBI, XG_B3_DVT0, XG_B3_DVT1, XG_B3_DVT2, XG_B3_DVT0W, XG_B3_DVT1W,
  XG_B3_DVT2W, XG_B3_NLX, XG_B3_K1, XG_B3_K1OX, XG_B3_K2OX, XG_B3_K3, XG_B3_K3B, XG_B3_KT1,
  XG_B3_KT1L, XG_B3_KT2, XG_B3_W0, XG_B3_ETA0, XG_B3_ETAB, XG_B3_THETA0VB0, XG_B3_NFACTOR,
  XG_B3_CDSC, XG_B3_CDSCB, XG_B3_CDSCD, XG_B3_CIT, XG_B3_VFB, XG_B3_NGATE, XG_B3_VOFF,
  XG_B3_CDEP0, XG_B3_DWG, XG_B3_DWB, XG_B3_PRWG, XG_B3_PRWB, XG_B3_RDS0, XG_B3_XJ, XG_B3_A0,
  XG_B3_B0, XG_B3_B1, XG_B3_AGS, XG_B3_KETA, XG_B3_UA, XG_B3_UB, XG_B3_UC, XG_B3_U0TEMP,
  XG_B3_VSATTEMP, XG_B3_A1, XG_B3_A2, XG_B3_DELTA, XG_B3_PCLM, XG_B3_LITL, XG_B3_THETAROUT,
  XG_B3_PDIBLB, XG_B3_PVAG, XG_B3_PSCBE1, XG_B3_PSCBE2, XG_B3_ALPHA0, XG_B3_ALPHA1,
  XG_B3_BETA0, XG_B3_VFBCV, XG_B3_WEFFCV, XG_B3_LEFFCV, XG_B3_ABULKCVFACTOR, XG_B3_NOFF,
  XG_B3_VOFFCV, XG_B3_VFBZB, XG_B3_ACDE, XG_B3_LDEB, XG_B3_MOIN, XG_B3_CGDO, XG_B3_CGSO,
  XG_B3_CGBO, XG_B3_CKAPPA, XG_B3_CGDL, XG_B3_CGSL,
  XG_B3_NRAW,
  /* instance constants hoisted out of the per-load evaluation */
  XG_B3_SSAT = XG_B3_NRAW,  /* SourceSatCurrent                        */
  XG_B3_DSAT,               /* DrainSatCurrent                         */
  XG_B3_NVTM,               /* vtm * NJ                                */
  XG_B3_CZBD, XG_B3_CZBS, XG_B3_CZBDSW, XG_B3_CZBDSWG, XG_B3_CZBSSW, XG_B3_CZBSSWG,
  /* Instance-constant subexpressions of updateIntermediateVars, each formed
   * with the same operations in the same order as the evaluation would
   * (so the results keep their bits):                                     */
  XG_B3_XDEP0_SQRTPHI,      /* Xdep0 / sqrtPhi                          */
  XG_B3_V0,                 /* vbi - phi                                */
  XG_B3_DVT1_LEFF,          /* -0.5 * dvt1 * Leff                       */
  XG_B3_DVT1W_WL,           /* -0.5 * dvt1w * weff * Leff               */
  XG_B3_TRATIO,             /* temp / tnom - 1                          */
  XG_B3_K1OX_NLX,           /* k1ox * (sqrt(1 + nlx / Leff) - 1) * sqrtPhi */
  XG_B3_KT1_L,              /* kt1 + kt1l / Leff                        */
  XG_B3_TOXPHI_W,           /* tox * phi / (weff + w0)                  */
  XG_B3_VTH_BASE,           /* dtype * vth0 - k1 * sqrtPhi              */
  XG_B3_K3B_TOXPHI,         /* k3b * (tox * phi / (weff + w0))          */
  XG_B3_KT2_TRATIO,         /* kt2 * (temp / tnom - 1)                  */
  XG_B3_NFACTOR_EPSSI,      /* nfactor * EPSSI                          */
  XG_B3_VFB_PHI,            /* vfb + phi                                */
  XG_B3_VTMCDEP_COX,        /* vtm * cdep0 / cox                        */
  XG_B3_MCOX_VTMCDEP,       /* -cox / (vtm * cdep0)                     */
  XG_B3_B0_W,               /* b0 / (weff + b1)                         */
  XG_B3_AGS_A0,             /* ags * a0                                 */
  XG_B3_VSAT2,              /* 2 * vsattemp                             */
  XG_B3_ISUB_A,             /* alpha0 + alpha1 * Leff                   */
  XG_B3_ISUB_T2,            /* (alpha0 + alpha1 * Leff) / Leff          */
  XG_B3_BETA0_ET,           /* beta0 / EXP_THRESHOLD                    */
  XG_B3_PSCBE1_LITL,        /* pscbe1 * litl                            */
  XG_B3_PSCBE1_LITL_ET,     /* pscbe1 * litl / EXP_THRESHOLD            */
  XG_B3_COXWL,              /* cox * weffCV * leffCV                    */
  XG_B3_D3_VFBZB,           /* 4 * DELTA_3 * vfbzb                      */
  XG_B3_TOX8,               /* 1e8 * tox                                */
  XG_B3_LINK,               /* 1e-3 * tox                               */
  XG_B3_LINK4_LDEB,         /* 4 * LINK * ldeb                          */
  XG_B3_DPHI_DENOMI,        /* moin vtm k1ox^2 (k1ox > 0), else 0.25 moin vtm */
  XG_B3_DPHI_T0,            /* k1ox sqrtPhi (k1ox > 0), else 0.5 sqrtPhi */
  XG_B3_VTM2,               /* 2 * vtm                                  */
  XG_B3_QBS0, XG_B3_QBSSW0, XG_B3_QBSSWG0,   /* PhiB*Temp * czbs, czbssw, czbsswg */
  XG_B3_QBD0, XG_B3_QBDSW0, XG_B3_QBDSWG0,   /* ... * czbd, czbdsw, czbdswg      */
  XG_B3_OMMJ, XG_B3_OMMJSW, XG_B3_OMMJSWG,   /* 1 - MJ, 1 - MJSW, 1 - MJSWG      */
  XG_B3_CBS_F, XG_B3_CBSSW_F, XG_B3_CBSSWG_F,/* czbs * MJ / PhiBTemp, ...       */
  XG_B3_CBD_F, XG_B3_CBDSW_F, XG_B3_CBDSWG_F,/* czbd * MJ / PhiBTemp, ...       */
  XG_B3_CGDL_W, XG_B3_CGSL_W,                /* weffCV * cgdl, weffCV * cgsl    */
  XG_B3_CGDO_T, XG_B3_CGSO_T,                /* cgdo + weffCV cgdl, cgso + ...  */
  XG_B3_HALF_CKAPPA,                         /* 0.5 * ckappa                    */
  /* Reciprocals of per-instance divisors, read only by the FMA build of the
   * kernel, which multiplies by them instead of dividing:                 */
  XG_B3_R_NVTM, XG_B3_R_SQRTPHI, XG_B3_R_PHIS3, XG_B3_R_COX, XG_B3_R_TOX,
  XG_B3_R_LEFF, XG_B3_R_THETAROUT, XG_B3_R_TOX8, XG_B3_R_PSCBE2,
  XG_B3_R_DPHI_DENOMI, XG_B3_R_CKAPPA, XG_B3_R_PHIB, XG_B3_R_PHIBSW,
  XG_B3_R_PHIBSWG, XG_B3_R_OMMJ, XG_B3_R_OMMJSW, XG_B3_R_OMMJSWG,
  XG_B3_NPARAMS
};

/* Linear elements: one value each. */
enum xg_res_param { XG_R_G = 0, XG_R_NPARAMS };          /* 1/R       */
enum xg_cap_param { XG_C_C = 0, XG_C_NPARAMS };          /* C         */
enum xg_src_param { XG_V_KIND = 0, XG_V_V1, XG_V_V2, XG_V_TD, XG_V_TR, XG_V_TF,
                    XG_V_PW, XG_V_PER, XG_V_NPARAMS };   /* PULSE/DC  */

#ifdef __cplusplus
}
#endif

#endif /* XG_PARAMS_H */
