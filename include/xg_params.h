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

/* Linear elements: one value each. */
enum xg_res_param { XG_R_G = 0, XG_R_NPARAMS };          /* 1/R       */
enum xg_cap_param { XG_C_C = 0, XG_C_NPARAMS };          /* C         */
enum xg_src_param { XG_V_KIND = 0, XG_V_V1, XG_V_V2, XG_V_TD, XG_V_TR, XG_V_TF,
                    XG_V_PW, XG_V_PER, XG_V_NPARAMS };   /* PULSE/DC  */

#ifdef __cplusplus
}
#endif

#endif /* XG_PARAMS_H */
