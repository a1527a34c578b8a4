// bsim3_eval.cuh — the BSIM3 v3.2 Newton-load kernel, included by
// load_kernels.cu inside namespace xg::XG_NS (built bit-exact and with FMA).
//
// One thread per instance evaluates, in FP64, what the reference computes in
// src/DeviceModelPKG/OpenModels/src/N_DEV_MOSFET_B3.C:
//   Instance::updateIntermediateVars   :4526-7273 (nqsMod = 0; capMod 0-3;
//                                       mobMod 1-3; all charge partitions)
//   setupCapacitors_oldDAE / _newDAE   :7574-7898
//   Master::updateState                :9229-9305
//   Master::loadDAEVectors + auxChargeCalculations :9306-9653, :7477-7573
//   Master::loadDAEMatrices (pointer)  :9654-9939
// and writes the 50 stamp terms of the instance in that statement order.
// Terms that the reference adds as structural zeros (the non-quasi-static
// charge-partition derivatives, all zero for nqsMod = 0) are left out: adding
// +-0 never changes a sum's value.
//
// Members the reference refreshes only when charges are computed (CAP*
// capacitances, Qeqq*_Jdxp limiter charges, qg/qb/qd/qbs/qbd) live in a
// device array carried from one load to the next, laid out [k*n + i].

// src/DeviceModelPKG/Core/include/N_DEV_Const.h
constexpr double EXP_THRESHOLD = 34.0;          // CONSTEXP_THRESHOLD
constexpr double MAX_EXP = 5.834617425e14;      // CONSTMAX_EXP
constexpr double MIN_EXP = 1.713908431e-15;     // CONSTMIN_EXP
constexpr double DELTA_1 = 0.02, DELTA_3 = 0.02, DELTA_4 = 0.02;
constexpr double EPSSI = 1.03594e-10;           // CONSTEPSSI
constexpr double KQ = 1.6021918e-19;            // CONSTQ
constexpr double KBOLTZ = 1.3806226e-23;        // CONSTboltz
constexpr double CTOK = 273.15;                 // CONSTCtoK

// Quotients.  The bit-exact build divides wherever the reference divides.
// The FMA build (XG_FAST_DIV) multiplies by reciprocals instead: formed once
// where several quotients share a denominator, read from the parameter block
// where it is an instance constant, and otherwise taken by Newton-Raphson
// from the hardware's approximation (xg::fast_rcp, four fused multiply-adds
// against IEEE division's longer sequence); each quotient lands within ~1-2
// ulp, inside the tolerance that build is held to.  A literal divisor
// becomes a multiply by its reciprocal, folded at compile time.
//   B3_RCOL(name, k)   declares a reciprocal read from parameter column k
//   B3_RCP(name, x)    declares the reciprocal of x (FMA build only)
//   B3_DIV(a, b, rb)   a / b, or a * rb
//   B3_Q(a, b)         a / b, or a * fast_rcp(b)
//   B3_DIVK(a, k)      a / k for a literal k, or a * (1 / k)
//   B3_RSQRT(x)        1 / sqrt(x), or CUDA's rsqrt (within 1 ulp)
#if XG_FAST_DIV
#define B3_RCOL(name, k) const double name = PRM(k)
#define B3_RCP(name, x) const double name = xg::fast_rcp(x)
#define B3_DIV(a, b, rb) ((a) * (rb))
#define B3_Q(a, b) ((a) * xg::fast_rcp(b))
#define B3_DIVK(a, k) ((a) * (1.0 / (k)))
#define B3_RSQRT(x) rsqrt(x)
#else
#define B3_RCOL(name, k) (void)0
#define B3_RCP(name, x) (void)0
#define B3_DIV(a, b, rb) ((a) / (b))
#define B3_Q(a, b) ((a) / (b))
#define B3_DIVK(a, k) ((a) / (k))
#define B3_RSQRT(x) (1.0 / sqrt(x))
#endif

enum B3Mem {
  B3M_CAPCGGB = 0, B3M_CAPCGDB, B3M_CAPCGSB, B3M_CAPCDGB, B3M_CAPCDDB, B3M_CAPCDSB,
  B3M_CAPCSGB, B3M_CAPCSDB, B3M_CAPCSSB, B3M_CAPCBGB, B3M_CAPCBDB, B3M_CAPCBSB,
  B3M_QJG, B3M_QJB, B3M_QJD, B3M_QG, B3M_QB, B3M_QD, B3M_QBS, B3M_QBD, B3M_N
};

struct B3MemRegs {
  double CAPcggb, CAPcgdb, CAPcgsb, CAPcdgb, CAPcddb, CAPcdsb, CAPcsgb, CAPcsdb, CAPcssb;
  double CAPcbgb, CAPcbdb, CAPcbsb, Qeqqg_Jdxp, Qeqqb_Jdxp, Qeqqd_Jdxp, qg, qb, qd, qbs, qbd;
};

struct B3Local {
  double gds, gm, gmbs, gbbs, gbgs, gbds, csub, cd, ggtg, ggtd, ggtb, ggts, sxpart, dxpart;
};

__global__ void __launch_bounds__(128) bsim3_kernel(DevType t, DevOptions o, Flags f, LoadIO io) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_flags(t, i, f)) return;
  const int nI = t.n;  // instances ("n" is the subthreshold swing below)
  const double *__restrict__ p = t.p;
#define PRM(k) __ldg(p + (int64_t)(k) * nI + i)
  const int li_Drain = __ldg(t.lid + i), li_Gate = __ldg(t.lid + nI + i);
  const int li_Source = __ldg(t.lid + 2 * nI + i), li_Bulk = __ldg(t.lid + 3 * nI + i);
  const int li_DrainPrime = __ldg(t.lid + 4 * nI + i), li_SourcePrime = __ldg(t.lid + 5 * nI + i);
  const int dtype = (int)PRM(XG_B3_DTYPE);
  const int mobMod = (int)PRM(XG_B3_MOBMOD), capMod = (int)PRM(XG_B3_CAPMOD);
  const double xpart = PRM(XG_B3_XPART), tox = PRM(XG_B3_TOX), cox = PRM(XG_B3_COX);
  const double factor1 = PRM(XG_B3_FACTOR1);
  const double gmin = o.gmin;
  const int OFF = ((int)PRM(XG_B3_FLAGS)) & 1;
  double *sto = io.sto + t.sto0 + (int64_t)i * 5;
  double *sta = io.sta + t.sta0 + (int64_t)i * 12;
  const double *csto = io.sto_curr + t.sto0 + (int64_t)i * 5;
  enum { O_VBD, O_VBS, O_VGS, O_VDS, O_VON };
  enum { S_QB, S_QG, S_QD, S_QBS, S_QBD };
  double *memp = io.b3_mem + i;
  B3MemRegs mem;
  mem.CAPcggb = memp[(int64_t)B3M_CAPCGGB * nI];
  mem.CAPcgdb = memp[(int64_t)B3M_CAPCGDB * nI];
  mem.CAPcgsb = memp[(int64_t)B3M_CAPCGSB * nI];
  mem.CAPcdgb = memp[(int64_t)B3M_CAPCDGB * nI];
  mem.CAPcddb = memp[(int64_t)B3M_CAPCDDB * nI];
  mem.CAPcdsb = memp[(int64_t)B3M_CAPCDSB * nI];
  mem.CAPcsgb = memp[(int64_t)B3M_CAPCSGB * nI];
  mem.CAPcsdb = memp[(int64_t)B3M_CAPCSDB * nI];
  mem.CAPcssb = memp[(int64_t)B3M_CAPCSSB * nI];
  mem.CAPcbgb = memp[(int64_t)B3M_CAPCBGB * nI];
  mem.CAPcbdb = memp[(int64_t)B3M_CAPCBDB * nI];
  mem.CAPcbsb = memp[(int64_t)B3M_CAPCBSB * nI];
  mem.Qeqqg_Jdxp = memp[(int64_t)B3M_QJG * nI];
  mem.Qeqqb_Jdxp = memp[(int64_t)B3M_QJB * nI];
  mem.Qeqqd_Jdxp = memp[(int64_t)B3M_QJD * nI];
  mem.qg = memp[(int64_t)B3M_QG * nI];
  mem.qb = memp[(int64_t)B3M_QB * nI];
  mem.qd = memp[(int64_t)B3M_QD * nI];
  mem.qbs = memp[(int64_t)B3M_QBS * nI];
  mem.qbd = memp[(int64_t)B3M_QBD * nI];
  B3Local m;
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
  int ChargeComputationNeeded = (f.tranop || f.acop || f.transient) ? 1 : 0;
  int mode;

  const double *sol = io.sol;
  double Vd = sol[li_Drain], Vg = sol[li_Gate], Vs = sol[li_Source], Vb = sol[li_Bulk];
  double Vsp = sol[li_SourcePrime], Vdp = sol[li_DrainPrime];
  double Vddp = Vd - Vdp, Vssp = Vs - Vsp, Vbsp = Vb - Vsp, Vgsp = Vg - Vsp;
  double Vdpsp = Vdp - Vsp;
  double vbs = dtype * Vbsp, vgs = dtype * Vgsp, vds = dtype * Vdpsp;
  double vbd = vbs - vds, vgd = vgs - vds, vgb;
  int origFlag = 1;
  const double vgs_orig = vgs, vds_orig = vds, vbs_orig = vbs, vbd_orig = vbd, vgd_orig = vgd;

  if (f.init_jct && !OFF && o.voltlim) {
    /* inputOP with an all-zero flag vector takes the same branch */
    vbs = 0.0;
    vgs = dtype * PRM(XG_B3_VTH0) + 0.1;
    vds = 0.1;
    origFlag = 0;
    vbd = vbs - vds;
    vgd = vgs - vds;
  } else if ((f.init_fix || f.init_jct) && OFF) {
    vbs = vgs = vds = 0;
  }
  if (f.newton_iter == 0) {
    if (!f.dcop) {
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
  if (o.voltlim && !(f.init_fix && OFF)) {
    const double vt0 = KBOLTZ * (27.0 + CTOK) / KQ;
    const double vcrit = PRM(XG_B3_VCRIT);
    if (f.newton_iter >= 0) {
      if (vds_old >= 0.0) {
        vgs = fetlim(vgs, vgs_old, von_local);
        vds = vgs - vgd;
        vds = limvds(vds, vds_old);
        vgd = vgs - vds;
      } else {
        vgd = fetlim(vgd, vgdo, von_local);
        vds = vgs - vgd;
        vds = -limvds(-vds, -vds_old);
        vgs = vgd + vds;
      }
      if (vds >= 0.0) {
        vbs = pnjlim(vbs, vbs_old, vt0, vcrit, &Check);
        vbd = vbs - vds;
      } else {
        vbd = pnjlim(vbd, vbd_old, vt0, vcrit, &Check);
        vbs = vbd + vds;
      }
    }
    if (vgs_orig != vgs || vds_orig != vds || vbs_orig != vbs || vbd_orig != vbd || vgd_orig != vgd)
      origFlag = 0;
  }
  vbd = vbs - vds;
  vgd = vgs - vds;
  vgb = vgs - vbs;

  const double vtm = PRM(XG_B3_VTM);
  Nvtm = PRM(XG_B3_NVTM);  // vtm * NJ
  B3_RCOL(rNvtm, XG_B3_R_NVTM);
  const double ijth = PRM(XG_B3_IJTH);
  // area * Js + perimeter * Jsw, or 1e-14 with neither (set-up, :4475-4511)
  SourceSatCurrent = PRM(XG_B3_SSAT);
  if (SourceSatCurrent <= 0.0) {
    gbs = gmin;
    cbs = gbs * vbs;
  } else if (ijth == 0.0) {
    evbs = exp(B3_DIV(vbs, Nvtm, rNvtm));
    gbs = B3_DIV(SourceSatCurrent * evbs, Nvtm, rNvtm) + gmin;
    cbs = SourceSatCurrent * (evbs - 1.0) + gmin * vbs;
  } else if (vbs < PRM(XG_B3_VJSM)) {
    evbs = exp(B3_DIV(vbs, Nvtm, rNvtm));
    gbs = B3_DIV(SourceSatCurrent * evbs, Nvtm, rNvtm) + gmin;
    cbs = SourceSatCurrent * (evbs - 1.0) + gmin * vbs;
  } else {
    T0 = B3_DIV(PRM(XG_B3_ISEVJSM), Nvtm, rNvtm);
    gbs = T0 + gmin;
    cbs = PRM(XG_B3_ISEVJSM) - SourceSatCurrent + T0 * (vbs - PRM(XG_B3_VJSM)) + gmin * vbs;
  }
  DrainSatCurrent = PRM(XG_B3_DSAT);
  if (DrainSatCurrent <= 0.0) {
    gbd = gmin;
    cbd = gbd * vbd;
  } else if (ijth == 0.0) {
    evbd = exp(B3_DIV(vbd, Nvtm, rNvtm));
    gbd = B3_DIV(DrainSatCurrent * evbd, Nvtm, rNvtm) + gmin;
    cbd = DrainSatCurrent * (evbd - 1.0) + gmin * vbd;
  } else if (vbd < PRM(XG_B3_VJDM)) {
    evbd = exp(B3_DIV(vbd, Nvtm, rNvtm));
    gbd = B3_DIV(DrainSatCurrent * evbd, Nvtm, rNvtm) + gmin;
    cbd = DrainSatCurrent * (evbd - 1.0) + gmin * vbd;
  } else {
    T0 = B3_DIV(PRM(XG_B3_ISEVJDM), Nvtm, rNvtm);
    gbd = T0 + gmin;
    cbd = PRM(XG_B3_ISEVJDM) - DrainSatCurrent + T0 * (vbd - PRM(XG_B3_VJDM)) + gmin * vbd;
  }

  if (vds >= 0.0) {
    mode = 1; Vds = vds; Vgs = vgs; Vbs = vbs;
  } else {
    mode = -1; Vds = -vds; Vgs = vgd; Vbs = vbd;
  }

  const double vbsc = PRM(XG_B3_VBSC), phi = PRM(XG_B3_PHI), phis3 = PRM(XG_B3_PHIS3);
  const double sqrtPhi = PRM(XG_B3_SQRTPHI), Xdep0 = PRM(XG_B3_XDEP0);
  B3_RCOL(rPhis3, XG_B3_R_PHIS3);
  B3_RCOL(rSqrtPhi, XG_B3_R_SQRTPHI);
  T0 = Vbs - vbsc - 0.001;
  double T1global = sqrt(T0 * T0 - 0.004 * vbsc);
  Vbseff = vbsc + 0.5 * (T0 + T1global);
  dVbseff_dVb = 0.5 * (1.0 + B3_Q(T0, T1global));
  if (Vbseff < Vbs) Vbseff = Vbs;
  if (Vbseff > 0.0) {
    T0 = B3_Q(phi, (phi + Vbseff));
    Phis = phi * T0;
    dPhis_dVb = -T0 * T0;
    sqrtPhis = B3_Q(phis3, (phi + 0.5 * Vbseff));
    dsqrtPhis_dVb = B3_DIV(-0.5 * sqrtPhis * sqrtPhis, phis3, rPhis3);
  } else {
    Phis = phi - Vbseff;
    dPhis_dVb = -1.0;
    sqrtPhis = sqrt(Phis);
    dsqrtPhis_dVb = B3_Q(-0.5, sqrtPhis);
  }
  Xdep = B3_DIV(Xdep0 * sqrtPhis, sqrtPhi, rSqrtPhi);
  dXdep_dVb = PRM(XG_B3_XDEP0_SQRTPHI) * dsqrtPhis_dVb;
  Leff = PRM(XG_B3_LEFF);
  Vtm = vtm;
  T3 = sqrt(Xdep);
  B3_RCP(rSqXdep, T3);
  V0 = PRM(XG_B3_V0);
  const double dvt2 = PRM(XG_B3_DVT2), dvt2w = PRM(XG_B3_DVT2W);
  T0 = dvt2 * Vbseff;
  if (T0 >= -0.5) {
    T1 = 1.0 + T0;
    T2 = dvt2;
  } else {
    T4 = B3_Q(1.0, (3.0 + 8.0 * T0));
    T1 = (1.0 + 3.0 * T0) * T4;
    T2 = dvt2 * T4 * T4;
  }
  lt1 = factor1 * T3 * T1;
  dlt1_dVb = factor1 * (B3_DIV(0.5, T3, rSqXdep) * T1 * dXdep_dVb + T3 * T2);
  T0 = dvt2w * Vbseff;
  if (T0 >= -0.5) {
    T1 = 1.0 + T0;
    T2 = dvt2w;
  } else {
    T4 = B3_Q(1.0, (3.0 + 8.0 * T0));
    T1 = (1.0 + 3.0 * T0) * T4;
    T2 = dvt2w * T4 * T4;
  }
  ltw = factor1 * T3 * T1;
  dltw_dVb = factor1 * (B3_DIV(0.5, T3, rSqXdep) * T1 * dXdep_dVb + T3 * T2);
  B3_RCP(rlt1, lt1);
  T0 = B3_DIV(PRM(XG_B3_DVT1_LEFF), lt1, rlt1);
  if (T0 > -EXP_THRESHOLD) {
    T1 = exp(T0);
    Theta0 = T1 * (1.0 + 2.0 * T1);
    dT1_dVb = B3_DIV(-T0, lt1, rlt1) * T1 * dlt1_dVb;
    dTheta0_dVb = (1.0 + 4.0 * T1) * dT1_dVb;
  } else {
    T1 = MIN_EXP;
    Theta0 = T1 * (1.0 + 2.0 * T1);
    dTheta0_dVb = 0.0;
  }
  double thetavth = PRM(XG_B3_DVT0) * Theta0;
  Delt_vth = thetavth * V0;
  dDelt_vth_dVb = PRM(XG_B3_DVT0) * dTheta0_dVb * V0;
  const double weff = PRM(XG_B3_WEFF);
  B3_RCP(rltw, ltw);
  T0 = B3_DIV(PRM(XG_B3_DVT1W_WL), ltw, rltw);
  if (T0 > -EXP_THRESHOLD) {
    T1 = exp(T0);
    T2 = T1 * (1.0 + 2.0 * T1);
    dT1_dVb = B3_DIV(-T0, ltw, rltw) * T1 * dltw_dVb;
    dT2_dVb = (1.0 + 4.0 * T1) * dT1_dVb;
  } else {
    T1 = MIN_EXP;
    T2 = T1 * (1.0 + 2.0 * T1);
    dT2_dVb = 0.0;
  }
  T0 = PRM(XG_B3_DVT0W) * T2;
  T2 = T0 * V0;
  dT2_dVb = PRM(XG_B3_DVT0W) * dT2_dVb * V0;
  TempRatio = PRM(XG_B3_TRATIO);
  const double k1ox = PRM(XG_B3_K1OX), kt2 = PRM(XG_B3_KT2);
  T1 = PRM(XG_B3_K1OX_NLX) + (PRM(XG_B3_KT1_L) + kt2 * Vbseff) * TempRatio;
  tmp2 = PRM(XG_B3_TOXPHI_W);
  const double etab = PRM(XG_B3_ETAB), theta0vb0 = PRM(XG_B3_THETA0VB0);
  T3 = PRM(XG_B3_ETA0) + etab * Vbseff;
  if (T3 < 1.0e-4) {
    T9 = B3_Q(1.0, (3.0 - 2.0e4 * T3));
    T3 = (2.0e-4 - T3) * T9;
    T4 = T9 * T9;
  } else {
    T4 = 1.0;
  }
  dDIBL_Sft_dVd = T3 * theta0vb0;
  DIBL_Sft = dDIBL_Sft_dVd * Vds;
  const double k2ox = PRM(XG_B3_K2OX), k3b = PRM(XG_B3_K3B);
  Vth = PRM(XG_B3_VTH_BASE) + k1ox * sqrtPhis - k2ox * Vbseff - Delt_vth -
        T2 + (PRM(XG_B3_K3) + k3b * Vbseff) * tmp2 + T1 - DIBL_Sft;
  double von = Vth;
  dVth_dVb = k1ox * dsqrtPhis_dVb - k2ox - dDelt_vth_dVb - dT2_dVb + PRM(XG_B3_K3B_TOXPHI) -
             etab * Vds * theta0vb0 * T4 + PRM(XG_B3_KT2_TRATIO);
  dVth_dVd = -dDIBL_Sft_dVd;

  const double cdscb = PRM(XG_B3_CDSCB), cdscd = PRM(XG_B3_CDSCD);
  B3_RCP(rXdep, Xdep);
  B3_RCOL(rcox, XG_B3_R_COX);
  tmp2 = B3_DIV(PRM(XG_B3_NFACTOR_EPSSI), Xdep, rXdep);
  tmp3 = PRM(XG_B3_CDSC) + cdscb * Vbseff + cdscd * Vds;
  tmp4 = B3_DIV(tmp2 + tmp3 * Theta0 + PRM(XG_B3_CIT), cox, rcox);
  if (tmp4 >= -0.5) {
    n = 1.0 + tmp4;
    dn_dVb = B3_DIV(B3_DIV(-tmp2, Xdep, rXdep) * dXdep_dVb + tmp3 * dTheta0_dVb + cdscb * Theta0, cox, rcox);
    dn_dVd = B3_DIV(cdscd * Theta0, cox, rcox);
  } else {
    T0 = B3_Q(1.0, (3.0 + 8.0 * tmp4));
    n = (1.0 + 3.0 * tmp4) * T0;
    T0 *= T0;
    dn_dVb = B3_DIV(B3_DIV(-tmp2, Xdep, rXdep) * dXdep_dVb + tmp3 * dTheta0_dVb + cdscb * Theta0, cox, rcox) * T0;
    dn_dVd = B3_DIV(cdscd * Theta0, cox, rcox) * T0;
  }

  T0 = PRM(XG_B3_VFB_PHI);
  const double ngate = PRM(XG_B3_NGATE);
  if ((ngate > 1.e18) && (ngate < 1.e25) && (Vgs > T0)) {
    T1 = B3_Q(1.0e6 * KQ * EPSSI * ngate, (cox * cox));
    T4 = sqrt(1.0 + B3_Q(2.0 * (Vgs - T0), T1));
    T2 = T1 * (T4 - 1.0);
    T3 = B3_Q(0.5 * T2 * T2, T1);
    T7 = 1.12 - T3 - 0.05;
    T6 = sqrt(T7 * T7 + 0.224);
    T5 = 1.12 - 0.5 * (T7 + T6);
    Vgs_eff = Vgs - T5;
    dVgs_eff_dVg = 1.0 - (0.5 - B3_Q(0.5, T4)) * (1.0 + B3_Q(T7, T6));
  } else {
    Vgs_eff = Vgs;
    dVgs_eff_dVg = 1.0;
  }
  Vgst = Vgs_eff - Vth;

  const double voff = PRM(XG_B3_VOFF), cdep0 = PRM(XG_B3_CDEP0);
  T10 = 2.0 * n * Vtm;
  B3_RCP(rT10, T10);
  VgstNVt = B3_DIV(Vgst, T10, rT10);
  ExpArg = B3_DIV(2.0 * voff - Vgst, T10, rT10);
  if (VgstNVt > EXP_THRESHOLD) {
    Vgsteff = Vgst;
    dVgsteff_dVg = dVgs_eff_dVg;
    dVgsteff_dVd = -dVth_dVd;
    dVgsteff_dVb = -dVth_dVb;
  } else if (ExpArg > EXP_THRESHOLD) {
    T0 = B3_Q((Vgst - voff), (n * Vtm));
    ExpVgst = exp(T0);
    Vgsteff = PRM(XG_B3_VTMCDEP_COX) * ExpVgst;
    dVgsteff_dVg = B3_Q(Vgsteff, (n * Vtm));
    dVgsteff_dVd = -dVgsteff_dVg * (dVth_dVd + T0 * Vtm * dn_dVd);
    dVgsteff_dVb = -dVgsteff_dVg * (dVth_dVb + T0 * Vtm * dn_dVb);
    dVgsteff_dVg *= dVgs_eff_dVg;
  } else {
    ExpVgst = exp(VgstNVt);
    T1 = T10 * log(1.0 + ExpVgst);
    dT1_dVg = B3_Q(ExpVgst, (1.0 + ExpVgst));
    B3_RCP(rn, n);
    dT1_dVb = -dT1_dVg * (dVth_dVb + B3_DIV(Vgst, n, rn) * dn_dVb) + B3_DIV(T1, n, rn) * dn_dVb;
    dT1_dVd = -dT1_dVg * (dVth_dVd + B3_DIV(Vgst, n, rn) * dn_dVd) + B3_DIV(T1, n, rn) * dn_dVd;
    dT2_dVg = PRM(XG_B3_MCOX_VTMCDEP) * exp(ExpArg);
    T2 = 1.0 - T10 * dT2_dVg;
    dT2_dVd = -dT2_dVg * (dVth_dVd - 2.0 * Vtm * ExpArg * dn_dVd) + B3_DIV(T2 - 1.0, n, rn) * dn_dVd;
    dT2_dVb = -dT2_dVg * (dVth_dVb - 2.0 * Vtm * ExpArg * dn_dVb) + B3_DIV(T2 - 1.0, n, rn) * dn_dVb;
    Vgsteff = B3_Q(T1, T2);
    T3 = T2 * T2;
    B3_RCP(rT3, T3);
    dVgsteff_dVg = B3_DIV(T2 * dT1_dVg - T1 * dT2_dVg, T3, rT3) * dVgs_eff_dVg;
    dVgsteff_dVd = B3_DIV(T2 * dT1_dVd - T1 * dT2_dVd, T3, rT3);
    dVgsteff_dVb = B3_DIV(T2 * dT1_dVb - T1 * dT2_dVb, T3, rT3);
  }

  const double dwg = PRM(XG_B3_DWG), dwb = PRM(XG_B3_DWB);
  T9 = sqrtPhis - sqrtPhi;
  Weff = weff - 2.0 * (dwg * Vgsteff + dwb * T9);
  dWeff_dVg = -2.0 * dwg;
  dWeff_dVb = -2.0 * dwb * dsqrtPhis_dVb;
  if (Weff < 2.0e-8) {
    T0 = B3_Q(1.0, (6.0e-8 - 2.0 * Weff));
    Weff = 2.0e-8 * (4.0e-8 - Weff) * T0;
    T0 *= T0 * 4.0e-16;
    dWeff_dVg *= T0;
    dWeff_dVb *= T0;
  }
  const double prwg = PRM(XG_B3_PRWG), prwb = PRM(XG_B3_PRWB), rds0 = PRM(XG_B3_RDS0);
  T0 = prwg * Vgsteff + prwb * T9;
  if (T0 >= -0.9) {
    Rds = rds0 * (1.0 + T0);
    dRds_dVg = rds0 * prwg;
    dRds_dVb = rds0 * prwb * dsqrtPhis_dVb;
  } else {
    T1 = B3_Q(1.0, (17.0 + 20.0 * T0));
    Rds = rds0 * (0.8 + T0) * T1;
    T1 *= T1;
    dRds_dVg = rds0 * prwg * T1;
    dRds_dVb = rds0 * prwb * dsqrtPhis_dVb * T1;
  }

  B3_RCP(rSqrtPhis, sqrtPhis);
  T1 = B3_DIV(0.5 * k1ox, sqrtPhis, rSqrtPhis);
  dT1_dVb = B3_DIV(-T1, sqrtPhis, rSqrtPhis) * dsqrtPhis_dVb;
  T9 = sqrt(PRM(XG_B3_XJ) * Xdep);
  tmp1 = Leff + 2.0 * T9;
  B3_RCP(rtmp1, tmp1);
  T5 = B3_DIV(Leff, tmp1, rtmp1);
  const double a0 = PRM(XG_B3_A0);
  tmp2 = a0 * T5;
  tmp4 = PRM(XG_B3_B0_W);  // b0 / (weff + b1)
  T2 = tmp2 + tmp4;
  dT2_dVb = B3_DIV(B3_DIV(-T9, tmp1, rtmp1), Xdep, rXdep) * dXdep_dVb;
  T6 = T5 * T5;
  T7 = T5 * T6;
  Abulk0 = 1.0 + T1 * T2;
  dAbulk0_dVb = T1 * tmp2 * dT2_dVb + T2 * dT1_dVb;
  T8 = PRM(XG_B3_AGS_A0) * T7;
  dAbulk_dVg = -T1 * T8;
  Abulk = Abulk0 + dAbulk_dVg * Vgsteff;
  dAbulk_dVb = dAbulk0_dVb - T8 * Vgsteff * (dT1_dVb + 3.0 * T1 * dT2_dVb);
  if (Abulk0 < 0.1) {
    T9 = B3_Q(1.0, (3.0 - 20.0 * Abulk0));
    Abulk0 = (0.2 - Abulk0) * T9;
    dAbulk0_dVb *= T9 * T9;
  }
  if (Abulk < 0.1) {
    T9 = B3_Q(1.0, (3.0 - 20.0 * Abulk));
    Abulk = (0.2 - Abulk) * T9;
    T10 = T9 * T9;
    dAbulk_dVb *= T10;
    dAbulk_dVg *= T10;
  }
  const double keta = PRM(XG_B3_KETA);
  T2 = keta * Vbseff;
  if (T2 >= -0.9) {
    T0 = B3_Q(1.0, (1.0 + T2));
    dT0_dVb = -keta * T0 * T0;
  } else {
    T1 = B3_Q(1.0, (0.8 + T2));
    T0 = (17.0 + 20.0 * T2) * T1;
    dT0_dVb = -keta * T1 * T1;
  }
  dAbulk_dVg *= T0;
  dAbulk_dVb = dAbulk_dVb * T0 + Abulk * dT0_dVb;
  dAbulk0_dVb = dAbulk0_dVb * T0 + Abulk0 * dT0_dVb;
  Abulk *= T0;
  Abulk0 *= T0;

  const double ua = PRM(XG_B3_UA), ub = PRM(XG_B3_UB), uc = PRM(XG_B3_UC);
  B3_RCOL(rtox, XG_B3_R_TOX);
  if (mobMod == 1) {
    T0 = Vgsteff + Vth + Vth;
    T2 = ua + uc * Vbseff;
    T3 = B3_DIV(T0, tox, rtox);
    T5 = T3 * (T2 + ub * T3);
    dDenomi_dVg = B3_DIV(T2 + 2.0 * ub * T3, tox, rtox);
    dDenomi_dVd = dDenomi_dVg * 2.0 * dVth_dVd;
    dDenomi_dVb = dDenomi_dVg * 2.0 * dVth_dVb + uc * T3;
  } else if (mobMod == 2) {
    T5 = B3_DIV(Vgsteff, tox, rtox) * (ua + uc * Vbseff + B3_DIV(ub * Vgsteff, tox, rtox));
    dDenomi_dVg = B3_DIV(ua + uc * Vbseff + B3_DIV(2.0 * ub * Vgsteff, tox, rtox), tox, rtox);
    dDenomi_dVd = 0.0;
    dDenomi_dVb = B3_DIV(Vgsteff * uc, tox, rtox);
  } else {
    T0 = Vgsteff + Vth + Vth;
    T2 = 1.0 + uc * Vbseff;
    T3 = B3_DIV(T0, tox, rtox);
    T4 = T3 * (ua + ub * T3);
    T5 = T4 * T2;
    dDenomi_dVg = B3_DIV((ua + 2.0 * ub * T3) * T2, tox, rtox);
    dDenomi_dVd = dDenomi_dVg * 2.0 * dVth_dVd;
    dDenomi_dVb = dDenomi_dVg * 2.0 * dVth_dVb + uc * T4;
  }
  if (T5 >= -0.8) {
    Denomi = 1.0 + T5;
  } else {
    T9 = B3_Q(1.0, (7.0 + 10.0 * T5));
    Denomi = (0.6 + T5) * T9;
    T9 *= T9;
    dDenomi_dVg *= T9;
    dDenomi_dVd *= T9;
    dDenomi_dVb *= T9;
  }
  B3_RCP(rDenomi, Denomi);
  ueff = B3_DIV(PRM(XG_B3_U0TEMP), Denomi, rDenomi);
  T9 = B3_DIV(-ueff, Denomi, rDenomi);
  dueff_dVg = T9 * dDenomi_dVg;
  dueff_dVd = T9 * dDenomi_dVd;
  dueff_dVb = T9 * dDenomi_dVb;

  const double vsattemp = PRM(XG_B3_VSATTEMP);
  WVCox = Weff * vsattemp * cox;
  WVCoxRds = WVCox * Rds;
  B3_RCP(rueff, ueff);
  Esat = B3_DIV(PRM(XG_B3_VSAT2), ueff, rueff);
  EsatL = Esat * Leff;
  B3_RCP(rEsatL, EsatL);
  T0 = B3_DIV(-EsatL, ueff, rueff);
  dEsatL_dVg = T0 * dueff_dVg;
  dEsatL_dVd = T0 * dueff_dVd;
  dEsatL_dVb = T0 * dueff_dVb;

  a1 = PRM(XG_B3_A1);
  const double a2 = PRM(XG_B3_A2);
  if (a1 == 0.0) {
    Lambda = a2;
    dLambda_dVg = 0.0;
  } else if (a1 > 0.0) {
    T0 = 1.0 - a2;
    T1 = T0 - a1 * Vgsteff - 0.0001;
    T2 = sqrt(T1 * T1 + 0.0004 * T0);
    Lambda = a2 + T0 - 0.5 * (T1 + T2);
    dLambda_dVg = 0.5 * a1 * (1.0 + B3_Q(T1, T2));
  } else {
    T1 = a2 + a1 * Vgsteff - 0.0001;
    T2 = sqrt(T1 * T1 + 0.0004 * a2);
    Lambda = 0.5 * (T1 + T2);
    dLambda_dVg = 0.5 * a1 * (1.0 + B3_Q(T1, T2));
  }
  Vgst2Vtm = Vgsteff + PRM(XG_B3_VTM2);
  B3_RCP(rVgst2Vtm, Vgst2Vtm);
  B3_RCP(rWeff, Weff);
  if (Rds > 0) {
    B3_RCP(rRds, Rds);
    tmp2 = B3_DIV(dRds_dVg, Rds, rRds) + B3_DIV(dWeff_dVg, Weff, rWeff);
    tmp3 = B3_DIV(dRds_dVb, Rds, rRds) + B3_DIV(dWeff_dVb, Weff, rWeff);
  } else {
    tmp2 = B3_DIV(dWeff_dVg, Weff, rWeff);
    tmp3 = B3_DIV(dWeff_dVb, Weff, rWeff);
  }
  if ((Rds == 0.0) && (Lambda == 1.0)) {
    T0 = B3_Q(1.0, (Abulk * EsatL + Vgst2Vtm));
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
    tmp1 = B3_Q(dLambda_dVg, (Lambda * Lambda));
    T9 = Abulk * WVCoxRds;
    T8 = Abulk * T9;
    T7 = Vgst2Vtm * T9;
    T6 = Vgst2Vtm * WVCoxRds;
    T0 = 2.0 * Abulk * (T9 - 1.0 + B3_Q(1.0, Lambda));
    dT0_dVg = 2.0 * (T8 * tmp2 - Abulk * tmp1 + (2.0 * T9 + B3_Q(1.0, Lambda) - 1.0) * dAbulk_dVg);
    dT0_dVb = 2.0 * (T8 * (B3_Q(2.0, Abulk) * dAbulk_dVb + tmp3) + (B3_Q(1.0, Lambda) - 1.0) * dAbulk_dVb);
    dT0_dVd = 0.0;
    T1 = Vgst2Vtm * (B3_Q(2.0, Lambda) - 1.0) + Abulk * EsatL + 3.0 * T7;
    dT1_dVg = (B3_Q(2.0, Lambda) - 1.0) - 2.0 * Vgst2Vtm * tmp1 + Abulk * dEsatL_dVg +
              EsatL * dAbulk_dVg + 3.0 * (T9 + T7 * tmp2 + T6 * dAbulk_dVg);
    dT1_dVb = Abulk * dEsatL_dVb + EsatL * dAbulk_dVb + 3.0 * (T6 * dAbulk_dVb + T7 * tmp3);
    dT1_dVd = Abulk * dEsatL_dVd;
    T2 = Vgst2Vtm * (EsatL + 2.0 * T6);
    dT2_dVg = EsatL + Vgst2Vtm * dEsatL_dVg + T6 * (4.0 + 2.0 * Vgst2Vtm * tmp2);
    dT2_dVb = Vgst2Vtm * (dEsatL_dVb + 2.0 * T6 * tmp3);
    dT2_dVd = Vgst2Vtm * dEsatL_dVd;
    T3 = sqrt(T1 * T1 - 2.0 * T0 * T2);
    B3_RCP(rT0v, T0);
    B3_RCP(rT3v, T3);
    Vdsat = B3_DIV(T1 - T3, T0, rT0v);
    dT3_dVg = B3_Q((T1 * dT1_dVg - 2.0 * (T0 * dT2_dVg + T2 * dT0_dVg)), T3);
    dT3_dVd = B3_Q((T1 * dT1_dVd - 2.0 * (T0 * dT2_dVd + T2 * dT0_dVd)), T3);
    dT3_dVb = B3_Q((T1 * dT1_dVb - 2.0 * (T0 * dT2_dVb + T2 * dT0_dVb)), T3);
    (void)dT3_dVg; (void)dT3_dVd; (void)dT3_dVb;
    dVdsat_dVg = B3_DIV(dT1_dVg - B3_DIV(T1 * dT1_dVg - dT0_dVg * T2 - T0 * dT2_dVg, T3, rT3v) - Vdsat * dT0_dVg, T0, rT0v);
    dVdsat_dVb = B3_DIV(dT1_dVb - B3_DIV(T1 * dT1_dVb - dT0_dVb * T2 - T0 * dT2_dVb, T3, rT3v) - Vdsat * dT0_dVb, T0, rT0v);
    dVdsat_dVd = B3_DIV(dT1_dVd - B3_DIV(T1 * dT1_dVd - T0 * dT2_dVd, T3, rT3v), T0, rT0v);
  }

  const double delta = PRM(XG_B3_DELTA);
  T1 = Vdsat - Vds - delta;
  dT1_dVg = dVdsat_dVg;
  dT1_dVd = dVdsat_dVd - 1.0;
  dT1_dVb = dVdsat_dVb;
  T2 = sqrt(T1 * T1 + 4.0 * delta * Vdsat);
  B3_RCP(rT2d, T2);
  T0 = B3_DIV(T1, T2, rT2d);
  T3 = B3_DIV(2.0 * delta, T2, rT2d);
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

  tmp4 = 1.0 - B3_DIV(0.5 * Abulk * Vdsat, Vgst2Vtm, rVgst2Vtm);
  T9 = WVCoxRds * Vgsteff;
  T8 = B3_DIV(T9, Vgst2Vtm, rVgst2Vtm);
  T0 = EsatL + Vdsat + 2.0 * T9 * tmp4;
  T7 = 2.0 * WVCoxRds * tmp4;
  dT0_dVg = dEsatL_dVg + dVdsat_dVg + T7 * (1.0 + tmp2 * Vgsteff) -
            T8 * (Abulk * dVdsat_dVg - B3_DIV(Abulk * Vdsat, Vgst2Vtm, rVgst2Vtm) + Vdsat * dAbulk_dVg);
  dT0_dVb = dEsatL_dVb + dVdsat_dVb + T7 * tmp3 * Vgsteff - T8 * (dAbulk_dVb * Vdsat + Abulk * dVdsat_dVb);
  dT0_dVd = dEsatL_dVd + dVdsat_dVd - T8 * Abulk * dVdsat_dVd;
  T9 = WVCoxRds * Abulk;
  T1 = B3_Q(2.0, Lambda) - 1.0 + T9;
  dT1_dVg = -2.0 * tmp1 + WVCoxRds * (Abulk * tmp2 + dAbulk_dVg);
  dT1_dVb = dAbulk_dVb * WVCoxRds + T9 * tmp3;
  B3_RCP(rT1a, T1);
  Vasat = B3_DIV(T0, T1, rT1a);
  dVasat_dVg = B3_DIV(dT0_dVg - Vasat * dT1_dVg, T1, rT1a);
  dVasat_dVb = B3_DIV(dT0_dVb - Vasat * dT1_dVb, T1, rT1a);
  dVasat_dVd = B3_DIV(dT0_dVd, T1, rT1a);
  if (Vdseff > Vds) Vdseff = Vds;
  diffVds = Vds - Vdseff;

  const double pclm = PRM(XG_B3_PCLM), litl = PRM(XG_B3_LITL);
  if ((pclm > 0.0) && (diffVds > 1.0e-10)) {
    T0 = B3_Q(1.0, (pclm * Abulk * litl));
    B3_RCP(rAbulk, Abulk);
    dT0_dVb = B3_DIV(-T0, Abulk, rAbulk) * dAbulk_dVb;
    dT0_dVg = B3_DIV(-T0, Abulk, rAbulk) * dAbulk_dVg;
    T2 = B3_DIV(Vgsteff, EsatL, rEsatL);
    T1 = Leff * (Abulk + T2);
    dT1_dVg = Leff * (B3_DIV(1.0 - T2 * dEsatL_dVg, EsatL, rEsatL) + dAbulk_dVg);
    dT1_dVb = Leff * (dAbulk_dVb - B3_DIV(T2 * dEsatL_dVb, EsatL, rEsatL));
    dT1_dVd = B3_Q(-T2 * dEsatL_dVd, Esat);
    T9 = T0 * T1;
    VACLM = T9 * diffVds;
    dVACLM_dVg = T0 * dT1_dVg * diffVds - T9 * dVdseff_dVg + T1 * diffVds * dT0_dVg;
    dVACLM_dVb = (dT0_dVb * T1 + T0 * dT1_dVb) * diffVds - T9 * dVdseff_dVb;
    dVACLM_dVd = T0 * dT1_dVd * diffVds + T9 * (1.0 - dVdseff_dVd);
  } else {
    VACLM = MAX_EXP;
    dVACLM_dVd = dVACLM_dVg = dVACLM_dVb = 0.0;
  }
  const double thetaRout = PRM(XG_B3_THETAROUT), pdiblb = PRM(XG_B3_PDIBLB);
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
    B3_RCP(rT1r, T1);
    B3_RCP(rT9r, T9);
    B3_RCOL(rthetaRout, XG_B3_R_THETAROUT);
    VADIBL = B3_DIV(Vgst2Vtm - B3_DIV(T0, T1, rT1r), T2, rthetaRout);
    dVADIBL_dVg = B3_DIV(1.0 - B3_DIV(dT0_dVg, T1, rT1r) + B3_DIV(T0 * dT1_dVg, T9, rT9r), T2, rthetaRout);
    dVADIBL_dVb = B3_DIV(B3_DIV(-dT0_dVb, T1, rT1r) + B3_DIV(T0 * dT1_dVb, T9, rT9r), T2, rthetaRout);
    dVADIBL_dVd = B3_DIV(B3_DIV(-dT0_dVd, T1, rT1r) + B3_DIV(T0 * dT1_dVd, T9, rT9r), T2, rthetaRout);
    T7 = pdiblb * Vbseff;
    if (T7 >= -0.9) {
      T3 = B3_Q(1.0, (1.0 + T7));
      VADIBL *= T3;
      dVADIBL_dVg *= T3;
      dVADIBL_dVb = (dVADIBL_dVb - VADIBL * pdiblb) * T3;
      dVADIBL_dVd *= T3;
    } else {
      T4 = B3_Q(1.0, (0.8 + T7));
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
  T8 = B3_DIV(PRM(XG_B3_PVAG), EsatL, rEsatL);
  T9 = T8 * Vgsteff;
  if (T9 > -0.9) {
    T0 = 1.0 + T9;
    dT0_dVg = T8 * (1.0 - B3_DIV(Vgsteff * dEsatL_dVg, EsatL, rEsatL));
    dT0_dVb = B3_DIV(-T9 * dEsatL_dVb, EsatL, rEsatL);
    dT0_dVd = B3_DIV(-T9 * dEsatL_dVd, EsatL, rEsatL);
  } else {
    T1 = B3_Q(1.0, (17.0 + 20.0 * T9));
    T0 = (0.8 + T9) * T1;
    T1 *= T1;
    dT0_dVg = T8 * (1.0 - B3_DIV(Vgsteff * dEsatL_dVg, EsatL, rEsatL)) * T1;
    T9 *= B3_DIV(T1, EsatL, rEsatL);
    dT0_dVb = -T9 * dEsatL_dVb;
    dT0_dVd = -T9 * dEsatL_dVd;
  }
  tmp1 = VACLM * VACLM;
  tmp2 = VADIBL * VADIBL;
  tmp3 = VACLM + VADIBL;
  T1 = B3_Q(VACLM * VADIBL, tmp3);
  tmp3 *= tmp3;
  B3_RCP(rtmp3, tmp3);
  dT1_dVg = B3_DIV(tmp1 * dVADIBL_dVg + tmp2 * dVACLM_dVg, tmp3, rtmp3);
  dT1_dVd = B3_DIV(tmp1 * dVADIBL_dVd + tmp2 * dVACLM_dVd, tmp3, rtmp3);
  dT1_dVb = B3_DIV(tmp1 * dVADIBL_dVb + tmp2 * dVACLM_dVb, tmp3, rtmp3);
  Va = Vasat + T0 * T1;
  dVa_dVg = dVasat_dVg + T1 * dT0_dVg + T0 * dT1_dVg;
  dVa_dVd = dVasat_dVd + T1 * dT0_dVd + T0 * dT1_dVd;
  dVa_dVb = dVasat_dVb + T1 * dT0_dVb + T0 * dT1_dVb;

  const double pscbe1 = PRM(XG_B3_PSCBE1), pscbe2 = PRM(XG_B3_PSCBE2);
  if (pscbe2 > 0.0) {
    if (diffVds > PRM(XG_B3_PSCBE1_LITL_ET)) {
      B3_RCP(rdiff, diffVds);
      T0 = B3_DIV(PRM(XG_B3_PSCBE1_LITL), diffVds, rdiff);
      VASCBE = B3_DIV(Leff * exp(T0), pscbe2, PRM(XG_B3_R_PSCBE2));
      T1 = B3_DIV(T0 * VASCBE, diffVds, rdiff);
      dVASCBE_dVg = T1 * dVdseff_dVg;
      dVASCBE_dVd = -T1 * (1.0 - dVdseff_dVd);
      dVASCBE_dVb = T1 * dVdseff_dVb;
    } else {
      VASCBE = B3_Q(MAX_EXP * Leff, pscbe2);
      dVASCBE_dVg = dVASCBE_dVd = dVASCBE_dVb = 0.0;
    }
  } else {
    VASCBE = MAX_EXP;
    dVASCBE_dVg = dVASCBE_dVd = dVASCBE_dVb = 0.0;
  }

  CoxWovL = B3_DIV(cox * Weff, Leff, PRM(XG_B3_R_LEFF));
  beta = ueff * CoxWovL;
  dbeta_dVg = CoxWovL * dueff_dVg + B3_DIV(beta * dWeff_dVg, Weff, rWeff);
  dbeta_dVd = CoxWovL * dueff_dVd;
  dbeta_dVb = CoxWovL * dueff_dVb + B3_DIV(beta * dWeff_dVb, Weff, rWeff);
  T0 = 1.0 - B3_DIV(0.5 * Abulk * Vdseff, Vgst2Vtm, rVgst2Vtm);
  dT0_dVg = B3_DIV(-0.5 * (Abulk * dVdseff_dVg - B3_DIV(Abulk * Vdseff, Vgst2Vtm, rVgst2Vtm) + Vdseff * dAbulk_dVg),
                   Vgst2Vtm, rVgst2Vtm);
  dT0_dVd = B3_DIV(-0.5 * Abulk * dVdseff_dVd, Vgst2Vtm, rVgst2Vtm);
  dT0_dVb = B3_DIV(-0.5 * (Abulk * dVdseff_dVb + dAbulk_dVb * Vdseff), Vgst2Vtm, rVgst2Vtm);
  fgche1 = Vgsteff * T0;
  dfgche1_dVg = Vgsteff * dT0_dVg + T0;
  dfgche1_dVd = Vgsteff * dT0_dVd;
  dfgche1_dVb = Vgsteff * dT0_dVb;
  T9 = B3_DIV(Vdseff, EsatL, rEsatL);
  fgche2 = 1.0 + T9;
  dfgche2_dVg = B3_DIV(dVdseff_dVg - T9 * dEsatL_dVg, EsatL, rEsatL);
  dfgche2_dVd = B3_DIV(dVdseff_dVd - T9 * dEsatL_dVd, EsatL, rEsatL);
  dfgche2_dVb = B3_DIV(dVdseff_dVb - T9 * dEsatL_dVb, EsatL, rEsatL);
  B3_RCP(rfgche2, fgche2);
  gche = B3_DIV(beta * fgche1, fgche2, rfgche2);
  dgche_dVg = B3_DIV(beta * dfgche1_dVg + fgche1 * dbeta_dVg - gche * dfgche2_dVg, fgche2, rfgche2);
  dgche_dVd = B3_DIV(beta * dfgche1_dVd + fgche1 * dbeta_dVd - gche * dfgche2_dVd, fgche2, rfgche2);
  dgche_dVb = B3_DIV(beta * dfgche1_dVb + fgche1 * dbeta_dVb - gche * dfgche2_dVb, fgche2, rfgche2);
  T0 = 1.0 + gche * Rds;
  B3_RCP(rT0i, T0);
  T9 = B3_DIV(Vdseff, T0, rT0i);
  Idl = gche * T9;
  dIdl_dVg = B3_DIV(gche * dVdseff_dVg + T9 * dgche_dVg, T0, rT0i) - B3_DIV(Idl * gche, T0, rT0i) * dRds_dVg;
  dIdl_dVd = B3_DIV(gche * dVdseff_dVd + T9 * dgche_dVd, T0, rT0i);
  dIdl_dVb = B3_DIV(gche * dVdseff_dVb + T9 * dgche_dVb - Idl * dRds_dVb * gche, T0, rT0i);
  B3_RCP(rVa, Va);
  T9 = B3_DIV(diffVds, Va, rVa);
  T0 = 1.0 + T9;
  Idsa = Idl * T0;
  dIdsa_dVg = T0 * dIdl_dVg - B3_DIV(Idl * (dVdseff_dVg + T9 * dVa_dVg), Va, rVa);
  dIdsa_dVd = T0 * dIdl_dVd + B3_DIV(Idl * (1.0 - dVdseff_dVd - T9 * dVa_dVd), Va, rVa);
  dIdsa_dVb = T0 * dIdl_dVb - B3_DIV(Idl * (dVdseff_dVb + T9 * dVa_dVb), Va, rVa);
  B3_RCP(rVASCBE, VASCBE);
  T9 = B3_DIV(diffVds, VASCBE, rVASCBE);
  T0 = 1.0 + T9;
  Ids = Idsa * T0;
  Gm = T0 * dIdsa_dVg - B3_DIV(Idsa * (dVdseff_dVg + T9 * dVASCBE_dVg), VASCBE, rVASCBE);
  Gds = T0 * dIdsa_dVd + B3_DIV(Idsa * (1.0 - dVdseff_dVd - T9 * dVASCBE_dVd), VASCBE, rVASCBE);
  Gmb = T0 * dIdsa_dVb - B3_DIV(Idsa * (dVdseff_dVb + T9 * dVASCBE_dVb), VASCBE, rVASCBE);
  Gds += Gm * dVgsteff_dVd;
  Gmb += Gm * dVgsteff_dVb;
  Gm *= dVgsteff_dVg;
  Gmb *= dVbseff_dVb;

  const double beta0 = PRM(XG_B3_BETA0);
  tmp = PRM(XG_B3_ISUB_A);  // alpha0 + alpha1 * Leff
  if ((tmp <= 0.0) || (beta0 <= 0.0)) {
    Isub = Gbd = Gbb = Gbg = 0.0;
  } else {
    T2 = PRM(XG_B3_ISUB_T2);
    if (diffVds > PRM(XG_B3_BETA0_ET)) {
      B3_RCP(rdiffI, diffVds);
      T0 = B3_DIV(-beta0, diffVds, rdiffI);
      T1 = T2 * diffVds * exp(T0);
      T3 = B3_DIV(T1, diffVds, rdiffI) * (T0 - 1.0);
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
  m.gds = Gds; m.gm = Gm; m.gmbs = Gmb;
  m.gbbs = Gbb; m.gbgs = Gbg; m.gbds = Gbd;
  m.csub = Isub;

  /* ---- charges: capMod 0-3 (:5994-6959) ---- */
  cgdo = PRM(XG_B3_CGDO);
  cgso = PRM(XG_B3_CGSO);
  const double weffCV = PRM(XG_B3_WEFFCV), leffCV = PRM(XG_B3_LEFFCV);
  const double abulkCVfactor = PRM(XG_B3_ABULKCVFACTOR);
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
    Vfb = PRM(XG_B3_VFBCV);
    Vth = Vfb + phi + k1ox * sqrtPhis;
    Vgst = Vgs_eff - Vth;
    dVth_dVb = k1ox * dsqrtPhis_dVb;
    dVgst_dVb = -dVth_dVb;
    dVgst_dVg = dVgs_eff_dVg;
    (void)dVgst_dVb; (void)dVgst_dVg;
    CoxWL = PRM(XG_B3_COXWL);
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
      T0 = B3_Q(CoxWL * T1, T2);
      cggb = T0 * dVgs_eff_dVg;
      cgdb = 0.0;
      cgsb = T0 * (dVbseff_dVb - dVgs_eff_dVg);
      cdgb = 0.0; cddb = 0.0; cdsb = 0.0;
      cbgb = -cggb;
      cbdb = 0.0;
      cbsb = -cgsb;
      qinv = 0.0;
    } else {
      One_Third_CoxWL = B3_DIVK(CoxWL, 3.0);
      Two_Third_CoxWL = 2.0 * One_Third_CoxWL;
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      Vdsat = B3_Q(Vgst, AbulkCV);
      dVdsat_dVg = B3_Q(dVgs_eff_dVg, AbulkCV);
      dVdsat_dVb = B3_Q(-(Vdsat * dAbulkCV_dVb + dVth_dVb), AbulkCV);
      if (xpart > 0.5) {
        if (Vdsat <= Vds) {
          T1 = B3_DIVK(Vdsat, 3.0);
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
          Alphaz = B3_Q(Vgst, Vdsat);
          T1 = 2.0 * Vdsat - Vds;
          T2 = B3_Q(Vds, (3.0 * T1));
          T3 = T2 * Vds;
          T9 = 0.25 * CoxWL;
          T4 = T9 * Alphaz;
          T7 = 2.0 * Vds - T1 - 3.0 * T3;
          T8 = T3 - T1 - 2.0 * Vds;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - 0.5 * (Vds - T3));
          T10 = T4 * T8;
          qdrn = T4 * T7;
          qbulk = -(qgate + qdrn + T10);
          T5 = B3_Q(T3, T1);
          cggb = CoxWL * (1.0 - T5 * dVdsat_dVg) * dVgs_eff_dVg;
          T11 = -CoxWL * T5 * dVdsat_dVb;
          cgdb = CoxWL * (T2 - 0.5 + 0.5 * T5);
          cgsb = -(cggb + T11 + cgdb);
          T6 = B3_Q(1.0, Vdsat);
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
          T1 = B3_DIVK(Vdsat, 3.0);
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
          Alphaz = B3_Q(Vgst, Vdsat);
          T1 = 2.0 * Vdsat - Vds;
          T2 = B3_Q(Vds, (3.0 * T1));
          T3 = T2 * Vds;
          T9 = 0.25 * CoxWL;
          T4 = T9 * Alphaz;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - 0.5 * (Vds - T3));
          T5 = B3_Q(T3, T1);
          cggb = CoxWL * (1.0 - T5 * dVdsat_dVg) * dVgs_eff_dVg;
          tmp = -CoxWL * T5 * dVdsat_dVb;
          cgdb = CoxWL * (T2 - 0.5 + 0.5 * T5);
          cgsb = -(cggb + cgdb + tmp);
          T6 = B3_Q(1.0, Vdsat);
          dAlphaz_dVg = T6 * (1.0 - Alphaz * dVdsat_dVg);
          dAlphaz_dVb = -T6 * (dVth_dVb + Alphaz * dVdsat_dVb);
          T6 = 8.0 * Vdsat * Vdsat - 6.0 * Vdsat * Vds + 1.2 * Vds * Vds;
          T8 = B3_Q(T2, T1);
          T7 = Vds - T1 - T8 * T6;
          qdrn = T4 * T7;
          T7 *= T9;
          tmp = B3_Q(T8, T1);
          tmp1 = T4 * (2.0 - 4.0 * tmp * T6 + T8 * (16.0 * Vdsat - 6.0 * Vds));
          cdgb = (T7 * dAlphaz_dVg - tmp1 * dVdsat_dVg) * dVgs_eff_dVg;
          T10 = T7 * dAlphaz_dVb - tmp1 * dVdsat_dVb;
          cddb = T4 * (2.0 - (B3_Q(1.0, (3.0 * T1 * T1)) + 2.0 * tmp) * T6 + T8 * (6.0 * Vdsat - 2.4 * Vds));
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
          T1 = B3_DIVK(Vdsat, 3.0);
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
          Alphaz = B3_Q(Vgst, Vdsat);
          T1 = 2.0 * Vdsat - Vds;
          T2 = B3_Q(Vds, (3.0 * T1));
          T3 = T2 * Vds;
          T9 = 0.25 * CoxWL;
          T4 = T9 * Alphaz;
          qgate = CoxWL * (Vgs_eff - Vfb - phi - 0.5 * (Vds - T3));
          T5 = B3_Q(T3, T1);
          cggb = CoxWL * (1.0 - T5 * dVdsat_dVg) * dVgs_eff_dVg;
          tmp = -CoxWL * T5 * dVdsat_dVb;
          cgdb = CoxWL * (T2 - 0.5 + 0.5 * T5);
          cgsb = -(cggb + cgdb + tmp);
          T6 = B3_Q(1.0, Vdsat);
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
    CoxWL = PRM(XG_B3_COXWL);
    noff = n * PRM(XG_B3_NOFF);
    dnoff_dVd = PRM(XG_B3_NOFF) * dn_dVd;
    dnoff_dVb = PRM(XG_B3_NOFF) * dn_dVb;
    T0 = Vtm * noff;
    voffcv = PRM(XG_B3_VOFFCV);
    VgstNVt = B3_Q((Vgst - voffcv), T0);
    if (VgstNVt > EXP_THRESHOLD) {
      Vgsteff = Vgst - voffcv;
      dVgsteff_dVg = dVgs_eff_dVg;
      dVgsteff_dVd = -dVth_dVd;
      dVgsteff_dVb = -dVth_dVb;
    } else if (VgstNVt < -EXP_THRESHOLD) {
      Vgsteff = T0 * log(1.0 + MIN_EXP);
      dVgsteff_dVg = 0.0;
      dVgsteff_dVd = B3_Q(Vgsteff, noff);
      dVgsteff_dVb = dVgsteff_dVd * dnoff_dVb;
      dVgsteff_dVd *= dnoff_dVd;
    } else {
      ExpVgst = exp(VgstNVt);
      Vgsteff = T0 * log(1.0 + ExpVgst);
      dVgsteff_dVg = B3_Q(ExpVgst, (1.0 + ExpVgst));
      B3_RCP(rnoff, noff);
      dVgsteff_dVd = -dVgsteff_dVg * (dVth_dVd + B3_DIV(Vgst - voffcv, noff, rnoff) * dnoff_dVd) +
                     B3_DIV(Vgsteff, noff, rnoff) * dnoff_dVd;
      dVgsteff_dVb = -dVgsteff_dVg * (dVth_dVb + B3_DIV(Vgst - voffcv, noff, rnoff) * dnoff_dVb) +
                     B3_DIV(Vgsteff, noff, rnoff) * dnoff_dVb;
      dVgsteff_dVg *= dVgs_eff_dVg;
    }
    if (capMod == 1) {
      Vfb = PRM(XG_B3_VFBZB);
      Arg1 = Vgs_eff - VbseffCV - Vfb - Vgsteff;
      if (Arg1 <= 0.0) {
        qgate = CoxWL * Arg1;
        Cgg = CoxWL * (dVgs_eff_dVg - dVgsteff_dVg);
        Cgd = -CoxWL * dVgsteff_dVd;
        Cgb = -CoxWL * (dVbseffCV_dVb + dVgsteff_dVb);
      } else {
        T0 = 0.5 * k1ox;
        T1 = sqrt(T0 * T0 + Arg1);
        T2 = B3_Q(CoxWL * T0, T1);
        qgate = CoxWL * k1ox * (T1 - T0);
        Cgg = T2 * (dVgs_eff_dVg - dVgsteff_dVg);
        Cgd = -T2 * dVgsteff_dVd;
        Cgb = -T2 * (dVbseffCV_dVb + dVgsteff_dVb);
      }
      qbulk = -qgate;
      Cbg = -Cgg;
      Cbd = -Cgd;
      Cbb = -Cgb;
      One_Third_CoxWL = B3_DIVK(CoxWL, 3.0);
      Two_Third_CoxWL = 2.0 * One_Third_CoxWL;
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      VdsatCV = B3_Q(Vgsteff, AbulkCV);
      if (VdsatCV < Vds) {
        dVdsatCV_dVg = B3_Q(1.0, AbulkCV);
        dVdsatCV_dVb = B3_Q(-VdsatCV * dAbulkCV_dVb, AbulkCV);
        T0 = Vgsteff - B3_DIVK(VdsatCV, 3.0);
        dT0_dVg = 1.0 - B3_DIVK(dVdsatCV_dVg, 3.0);
        dT0_dVb = B3_DIVK(-dVdsatCV_dVb, 3.0);
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
        T2 = B3_Q(Vds, T1);
        T3 = T0 * T2;
        dT3_dVg = -12.0 * T2 * T2 * AbulkCV;
        dT3_dVd = B3_Q(B3_Q(6.0 * T0 * (4.0 * Vgsteff - T0), T1), T1) - 0.5;
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
          qsrc = -CoxWL * (0.5 * Vgsteff + 0.25 * T0 - B3_Q(T0 * T0, T1));
          Csg = -CoxWL * (0.5 + B3_Q(B3_Q(24.0 * T0 * Vds, T1), T1) * AbulkCV);
          Csb = -CoxWL * (0.25 * Vds * dAbulkCV_dVb - B3_Q(B3_Q(12.0 * T0 * Vds, T1), T1) * (4.0 * Vgsteff - T0) * dAbulkCV_dVb) +
                Csg * dVgsteff_dVb;
          Csd = -CoxWL * (0.25 * AbulkCV - B3_Q(B3_Q(12.0 * AbulkCV * T0, T1), T1) * (4.0 * Vgsteff - T0)) +
                Csg * dVgsteff_dVd;
          Csg *= dVgsteff_dVg;
        } else if (xpart < 0.5) {
          T1 = B3_DIVK(T1, 12.0);
          T2 = B3_Q(0.5 * CoxWL, (T1 * T1));
          T3 = Vgsteff * (B3_DIVK(2.0 * T0 * T0, 3.0) + Vgsteff * (Vgsteff - B3_DIVK(4.0 * T0, 3.0))) - B3_DIVK(2.0 * T0 * T0 * T0, 15.0);
          qsrc = -T2 * T3;
          T4 = B3_DIVK(4.0, 3.0) * Vgsteff * (Vgsteff - T0) + 0.4 * T0 * T0;
          Csg = B3_Q(-2.0 * qsrc, T1) - T2 * (Vgsteff * (3.0 * Vgsteff - B3_DIVK(8.0 * T0, 3.0)) + B3_DIVK(2.0 * T0 * T0, 3.0));
          Csb = (B3_Q(qsrc, T1) * Vds + T2 * T4 * Vds) * dAbulkCV_dVb + Csg * dVgsteff_dVb;
          Csd = (B3_Q(qsrc, T1) + T2 * T4) * AbulkCV + Csg * dVgsteff_dVd;
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
      Vfb = PRM(XG_B3_VFBZB);
      V3 = Vfb - Vgs_eff + VbseffCV - DELTA_3;
      if (Vfb <= 0.0) {
        T0 = sqrt(V3 * V3 - PRM(XG_B3_D3_VFBZB));  // 4 DELTA_3 Vfb, Vfb = vfbzb
        T2 = B3_Q(-DELTA_3, T0);
      } else {
        T0 = sqrt(V3 * V3 + PRM(XG_B3_D3_VFBZB));
        T2 = B3_Q(DELTA_3, T0);
      }
      T1 = 0.5 * (1.0 + B3_Q(V3, T0));
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
        T1 = T0 + B3_Q(T3, k1ox);
        T2 = CoxWL;
      } else {
        T1 = sqrt(T0 * T0 + T3);
        T2 = B3_Q(CoxWL * T0, T1);
      }
      Qsub0 = CoxWL * k1ox * (T1 - T0);
      dQsub0_dVg = T2 * (dVgs_eff_dVg - dVfbeff_dVg - dVgsteff_dVg);
      dQsub0_dVd = -T2 * dVgsteff_dVd;
      dQsub0_dVb = -T2 * (dVfbeff_dVb + dVbseffCV_dVb + dVgsteff_dVb);
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      VdsatCV = B3_Q(Vgsteff, AbulkCV);
      V4 = VdsatCV - Vds - DELTA_4;
      T0 = sqrt(V4 * V4 + 4.0 * DELTA_4 * VdsatCV);
      VdseffCV = VdsatCV - 0.5 * (V4 + T0);
      T1 = 0.5 * (1.0 + B3_Q(V4, T0));
      T2 = B3_Q(DELTA_4, T0);
      T3 = B3_Q((1.0 - T1 - T2), AbulkCV);
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
      T2 = B3_Q(VdseffCV, T1);
      T3 = T0 * T2;
      T4 = (1.0 - 12.0 * T2 * T2 * AbulkCV);
      T5 = (B3_Q(6.0 * T0 * (4.0 * Vgsteff - T0), (T1 * T1)) - 0.5);
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
        qsrc = -CoxWL * (0.5 * Vgsteff + 0.25 * T0 - B3_Q(T0 * T0, T1));
        T7 = B3_Q((4.0 * Vgsteff - T0), (T1 * T1));
        T4 = -(0.5 + B3_Q(24.0 * T0 * T0, (T1 * T1)));
        T5 = -(0.25 * AbulkCV - 12.0 * AbulkCV * T0 * T7);
        T6 = -(0.25 * VdseffCV - 12.0 * T0 * VdseffCV * T7);
        Csg = CoxWL * (T4 + T5 * dVdseffCV_dVg);
        Csd = CoxWL * T5 * dVdseffCV_dVd + Csg * dVgsteff_dVd;
        Csb = CoxWL * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Csg * dVgsteff_dVb;
        Csg *= dVgsteff_dVg;
      } else if (xpart < 0.5) {
        T1 = B3_DIVK(T1, 12.0);
        T2 = B3_Q(0.5 * CoxWL, (T1 * T1));
        T3 = Vgsteff * (B3_DIVK(2.0 * T0 * T0, 3.0) + Vgsteff * (Vgsteff - B3_DIVK(4.0 * T0, 3.0))) - B3_DIVK(2.0 * T0 * T0 * T0, 15.0);
        qsrc = -T2 * T3;
        T7 = B3_DIVK(4.0, 3.0) * Vgsteff * (Vgsteff - T0) + 0.4 * T0 * T0;
        T4 = B3_Q(-2.0 * qsrc, T1) - T2 * (Vgsteff * (3.0 * Vgsteff - B3_DIVK(8.0 * T0, 3.0)) + B3_DIVK(2.0 * T0 * T0, 3.0));
        T5 = (B3_Q(qsrc, T1) + T2 * T7) * AbulkCV;
        T6 = (B3_Q(qsrc, T1) * VdseffCV + T2 * T7 * VdseffCV);
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
      const double vfbzb = PRM(XG_B3_VFBZB), acde = PRM(XG_B3_ACDE), ldeb = PRM(XG_B3_LDEB);
      V3 = vfbzb - Vgs_eff + VbseffCV - DELTA_3;
      if (vfbzb <= 0.0) {
        T0 = sqrt(V3 * V3 - PRM(XG_B3_D3_VFBZB));
      } else {
        T0 = sqrt(V3 * V3 + PRM(XG_B3_D3_VFBZB));
      }
      B3_RCP(rT0f, T0);
      T2 = B3_DIV(vfbzb <= 0.0 ? -DELTA_3 : DELTA_3, T0, rT0f);
      T1 = 0.5 * (1.0 + B3_DIV(V3, T0, rT0f));
      Vfbeff = vfbzb - 0.5 * (V3 + T0);
      dVfbeff_dVg = T1 * dVgs_eff_dVg;
      dVfbeff_dVb = -T1 * dVbseffCV_dVb;
      Cox = cox;
      Tox = PRM(XG_B3_TOX8);
      B3_RCOL(rTox, XG_B3_R_TOX8);
      T0 = B3_DIV(Vgs_eff - VbseffCV - vfbzb, Tox, rTox);
      dT0_dVg = B3_DIV(dVgs_eff_dVg, Tox, rTox);
      dT0_dVb = B3_DIV(-dVbseffCV_dVb, Tox, rTox);
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
      LINK = PRM(XG_B3_LINK);
      V3 = ldeb - Tcen - LINK;
      V4 = sqrt(V3 * V3 + PRM(XG_B3_LINK4_LDEB));
      Tcen = ldeb - 0.5 * (V3 + V4);
      T1 = 0.5 * (1.0 + B3_Q(V3, V4));
      dTcen_dVg *= T1;
      dTcen_dVb *= T1;
      B3_RCP(rTcen, Tcen);
      Ccen = B3_DIV(EPSSI, Tcen, rTcen);
      T2 = B3_Q(Cox, (Cox + Ccen));
      Coxeff = T2 * Ccen;
      T3 = B3_DIV(-Ccen, Tcen, rTcen);
      dCoxeff_dVg = T2 * T2 * T3;
      dCoxeff_dVb = dCoxeff_dVg * dTcen_dVb;
      dCoxeff_dVg *= dTcen_dVg;
      CoxWLcen = B3_DIV(CoxWL * Coxeff, Cox, rcox);
      Qac0 = CoxWLcen * (Vfbeff - vfbzb);
      B3_RCP(rCoxeff, Coxeff);
      QovCox = B3_DIV(Qac0, Coxeff, rCoxeff);
      dQac0_dVg = CoxWLcen * dVfbeff_dVg + QovCox * dCoxeff_dVg;
      dQac0_dVb = CoxWLcen * dVfbeff_dVb + QovCox * dCoxeff_dVb;
      T0 = 0.5 * k1ox;
      T3 = Vgs_eff - Vfbeff - VbseffCV - Vgsteff;
      if (k1ox == 0.0) {
        T1 = 0.0;
        T2 = 0.0;
      } else if (T3 < 0.0) {
        T1 = T0 + B3_Q(T3, k1ox);
        T2 = CoxWLcen;
      } else {
        T1 = sqrt(T0 * T0 + T3);
        T2 = B3_Q(CoxWLcen * T0, T1);
      }
      Qsub0 = CoxWLcen * k1ox * (T1 - T0);
      QovCox = B3_DIV(Qsub0, Coxeff, rCoxeff);
      dQsub0_dVg = T2 * (dVgs_eff_dVg - dVfbeff_dVg - dVgsteff_dVg) + QovCox * dCoxeff_dVg;
      dQsub0_dVd = -T2 * dVgsteff_dVd;
      dQsub0_dVb = -T2 * (dVfbeff_dVb + dVbseffCV_dVb + dVgsteff_dVb) + QovCox * dCoxeff_dVb;
      Denomi = PRM(XG_B3_DPHI_DENOMI);  // moin Vtm k1ox^2, or 0.25 moin Vtm
      T0 = PRM(XG_B3_DPHI_T0);          // k1ox sqrtPhi, or 0.5 sqrtPhi
      T1 = 2.0 * T0 + Vgsteff;
      DeltaPhi = Vtm * log(1.0 + B3_DIV(T1 * Vgsteff, Denomi, PRM(XG_B3_R_DPHI_DENOMI)));
      dDeltaPhi_dVg = B3_Q(PRM(XG_B3_VTM2) * (T1 - T0), (Denomi + T1 * Vgsteff));
      dDeltaPhi_dVd = dDeltaPhi_dVg * dVgsteff_dVd;
      dDeltaPhi_dVb = dDeltaPhi_dVg * dVgsteff_dVb;
      (void)dDeltaPhi_dVd; (void)dDeltaPhi_dVb;
      T3 = 4.0 * (Vth - vfbzb - phi);
      Tox += Tox;
      // the doubled Tox's reciprocal is 0.5 / Tox exactly
      if (T3 >= 0.0) {
        T0 = B3_DIV(Vgsteff + T3, Tox, 0.5 * rTox);
        dT0_dVd = B3_DIV(dVgsteff_dVd + 4.0 * dVth_dVd, Tox, 0.5 * rTox);
        dT0_dVb = B3_DIV(dVgsteff_dVb + 4.0 * dVth_dVb, Tox, 0.5 * rTox);
      } else {
        T0 = B3_DIV(Vgsteff + 1.0e-20, Tox, 0.5 * rTox);
        dT0_dVd = B3_DIV(dVgsteff_dVd, Tox, 0.5 * rTox);
        dT0_dVb = B3_DIV(dVgsteff_dVb, Tox, 0.5 * rTox);
      }
      tmp = exp(0.7 * log(T0));
      T1 = 1.0 + tmp;
      T2 = B3_Q(0.7 * tmp, (T0 * Tox));
      B3_RCP(rT1c, T1);
      Tcen = B3_DIV(1.9e-9, T1, rT1c);
      dTcen_dVg = B3_DIV(B3_DIV(-1.9e-9 * T2, T1, rT1c), T1, rT1c);
      dTcen_dVd = Tox * dTcen_dVg;
      dTcen_dVb = dTcen_dVd * dT0_dVb;
      dTcen_dVd *= dT0_dVd;
      dTcen_dVg *= dVgsteff_dVg;
      B3_RCP(rTcen2, Tcen);
      Ccen = B3_DIV(EPSSI, Tcen, rTcen2);
      T0 = B3_Q(Cox, (Cox + Ccen));
      Coxeff = T0 * Ccen;
      T1 = B3_DIV(-Ccen, Tcen, rTcen2);
      dCoxeff_dVg = T0 * T0 * T1;
      dCoxeff_dVd = dCoxeff_dVg * dTcen_dVd;
      dCoxeff_dVb = dCoxeff_dVg * dTcen_dVb;
      dCoxeff_dVg *= dTcen_dVg;
      CoxWLcen = B3_DIV(CoxWL * Coxeff, Cox, rcox);
      AbulkCV = Abulk0 * abulkCVfactor;
      dAbulkCV_dVb = abulkCVfactor * dAbulk0_dVb;
      B3_RCP(rAbulkCV, AbulkCV);
      B3_RCP(rCoxeff2, Coxeff);
      VdsatCV = B3_DIV(Vgsteff - DeltaPhi, AbulkCV, rAbulkCV);
      V4 = VdsatCV - Vds - DELTA_4;
      T0 = sqrt(V4 * V4 + 4.0 * DELTA_4 * VdsatCV);
      VdseffCV = VdsatCV - 0.5 * (V4 + T0);
      B3_RCP(rT0g, T0);
      T1 = 0.5 * (1.0 + B3_DIV(V4, T0, rT0g));
      T2 = B3_DIV(DELTA_4, T0, rT0g);
      T3 = B3_DIV(1.0 - T1 - T2, AbulkCV, rAbulkCV);
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
      B3_RCP(rT2h, T2);
      T3 = B3_DIV(T0, T2, rT2h);
      T4 = 1.0 - 12.0 * T3 * T3;
      T5 = AbulkCV * (B3_DIV(6.0 * T0 * (4.0 * T1 - T0), T2 * T2, rT2h * rT2h) - 0.5);
      T6 = B3_DIV(T5 * VdseffCV, AbulkCV, rAbulkCV);
      qgate = qinoi = CoxWLcen * (T1 - T0 * (0.5 - T3));
      QovCox = B3_DIV(qgate, Coxeff, rCoxeff2);
      Cgg1 = CoxWLcen * (T4 * (1.0 - dDeltaPhi_dVg) + T5 * dVdseffCV_dVg);
      Cgd1 = CoxWLcen * T5 * dVdseffCV_dVd + Cgg1 * dVgsteff_dVd + QovCox * dCoxeff_dVd;
      Cgb1 = CoxWLcen * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Cgg1 * dVgsteff_dVb + QovCox * dCoxeff_dVb;
      Cgg1 = Cgg1 * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      T7 = 1.0 - AbulkCV;
      T8 = T2 * T2;
      T9 = B3_DIV(12.0 * T7 * T0 * T0, T8 * AbulkCV, rT2h * rT2h * rAbulkCV);
      T10 = T9 * (1.0 - dDeltaPhi_dVg);
      T11 = B3_DIV(-T7 * T5, AbulkCV, rAbulkCV);
      T12 = -(B3_DIV(T9 * T1, AbulkCV, rAbulkCV) + VdseffCV * (0.5 - B3_DIV(T0, T2, rT2h)));
      qbulk = CoxWLcen * T7 * (0.5 * VdseffCV - B3_DIV(T0 * VdseffCV, T2, rT2h));
      QovCox = B3_DIV(qbulk, Coxeff, rCoxeff2);
      Cbg1 = CoxWLcen * (T10 + T11 * dVdseffCV_dVg);
      Cbd1 = CoxWLcen * T11 * dVdseffCV_dVd + Cbg1 * dVgsteff_dVd + QovCox * dCoxeff_dVd;
      Cbb1 = CoxWLcen * (T11 * dVdseffCV_dVb + T12 * dAbulkCV_dVb) + Cbg1 * dVgsteff_dVb + QovCox * dCoxeff_dVb;
      Cbg1 = Cbg1 * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      if (xpart > 0.5) {
        qsrc = -CoxWLcen * (B3_DIVK(T1, 2.0) + B3_DIVK(T0, 4.0) - B3_DIV(0.5 * T0 * T0, T2, rT2h));
        QovCox = B3_DIV(qsrc, Coxeff, rCoxeff2);
        T2 += T2;
        T3 = T2 * T2;
        T7 = -(0.25 - B3_Q(12.0 * T0 * (4.0 * T1 - T0), T3));
        T4 = -(0.5 + B3_Q(24.0 * T0 * T0, T3)) * (1.0 - dDeltaPhi_dVg);
        T5 = T7 * AbulkCV;
        T6 = T7 * VdseffCV;
        Csg = CoxWLcen * (T4 + T5 * dVdseffCV_dVg);
        Csd = CoxWLcen * T5 * dVdseffCV_dVd + Csg * dVgsteff_dVd + QovCox * dCoxeff_dVd;
        Csb = CoxWLcen * (T5 * dVdseffCV_dVb + T6 * dAbulkCV_dVb) + Csg * dVgsteff_dVb + QovCox * dCoxeff_dVb;
        Csg = Csg * dVgsteff_dVg + QovCox * dCoxeff_dVg;
      } else if (xpart < 0.5) {
        T2 = B3_DIVK(T2, 12.0);
        B3_RCP(rT2x, T2);
        T3 = B3_DIV(0.5 * CoxWLcen, T2 * T2, rT2x * rT2x);
        T4 = T1 * (B3_DIVK(2.0 * T0 * T0, 3.0) + T1 * (T1 - B3_DIVK(4.0 * T0, 3.0))) -
             B3_DIVK(2.0 * T0 * T0 * T0, 15.0);
        qsrc = -T3 * T4;
        QovCox = B3_DIV(qsrc, Coxeff, rCoxeff2);
        T8 = B3_DIVK(4.0, 3.0) * T1 * (T1 - T0) + 0.4 * T0 * T0;
        T5 = B3_DIV(-2.0 * qsrc, T2, rT2x) -
             T3 * (T1 * (3.0 * T1 - B3_DIVK(8.0 * T0, 3.0)) + B3_DIVK(2.0 * T0 * T0, 3.0));
        T6 = AbulkCV * (B3_DIV(qsrc, T2, rT2x) + T3 * T8);
        T7 = B3_DIV(T6 * VdseffCV, AbulkCV, rAbulkCV);
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
  m.cd = cdrain;
  capbs = capbd = qbs = qbd = 0.0;
  if (ChargeComputationNeeded) {
    // bottom and sidewall junction capacitances (:6983-7007), from set-up
    czbd = PRM(XG_B3_CZBD);
    czbs = PRM(XG_B3_CZBS);
    czbdsw = PRM(XG_B3_CZBDSW);
    czbdswg = PRM(XG_B3_CZBDSWG);
    czbssw = PRM(XG_B3_CZBSSW);
    czbsswg = PRM(XG_B3_CZBSSWG);
    MJ = PRM(XG_B3_MJ);
    MJSW = PRM(XG_B3_MJSW);
    MJSWG = PRM(XG_B3_MJSWG);
    const double PhiBTemp = PRM(XG_B3_PHIB), PhiBSWTemp = PRM(XG_B3_PHIBSW);
    const double PhiBSWGTemp = PRM(XG_B3_PHIBSWG);
    if (vbs == 0.0) {
      qbs = 0.0;
      capbs = czbs + czbssw + czbsswg;
    } else if (vbs < 0.0) {
      if (czbs > 0.0) {
        arg = 1.0 - B3_DIV(vbs, PhiBTemp, PRM(XG_B3_R_PHIB));
        if (MJ == 0.5) sarg = B3_RSQRT(arg);
        else sarg = exp(-MJ * log(arg));
        qbs = B3_DIV(PRM(XG_B3_QBS0) * (1.0 - arg * sarg), PRM(XG_B3_OMMJ), PRM(XG_B3_R_OMMJ));
        capbs = czbs * sarg;
      } else {
        qbs = 0.0;
        capbs = 0.0;
      }
      if (czbssw > 0.0) {
        arg = 1.0 - B3_DIV(vbs, PhiBSWTemp, PRM(XG_B3_R_PHIBSW));
        if (MJSW == 0.5) sarg = B3_RSQRT(arg);
        else sarg = exp(-MJSW * log(arg));
        qbs += B3_DIV(PRM(XG_B3_QBSSW0) * (1.0 - arg * sarg), PRM(XG_B3_OMMJSW), PRM(XG_B3_R_OMMJSW));
        capbs += czbssw * sarg;
      }
      if (czbsswg > 0.0) {
        arg = 1.0 - B3_DIV(vbs, PhiBSWGTemp, PRM(XG_B3_R_PHIBSWG));
        if (MJSWG == 0.5) sarg = B3_RSQRT(arg);
        else sarg = exp(-MJSWG * log(arg));
        qbs += B3_DIV(PRM(XG_B3_QBSSWG0) * (1.0 - arg * sarg), PRM(XG_B3_OMMJSWG), PRM(XG_B3_R_OMMJSWG));
        capbs += czbsswg * sarg;
      }
    } else {
      T0 = czbs + czbssw + czbsswg;
      T1 = vbs * (PRM(XG_B3_CBS_F) + PRM(XG_B3_CBSSW_F) + PRM(XG_B3_CBSSWG_F));
      qbs = vbs * (T0 + 0.5 * T1);
      capbs = T0 + T1;
    }
    if (vbd == 0.0) {
      qbd = 0.0;
      capbd = czbd + czbdsw + czbdswg;
    } else if (vbd < 0.0) {
      if (czbd > 0.0) {
        arg = 1.0 - B3_DIV(vbd, PhiBTemp, PRM(XG_B3_R_PHIB));
        if (MJ == 0.5) sarg = B3_RSQRT(arg);
        else sarg = exp(-MJ * log(arg));
        qbd = B3_DIV(PRM(XG_B3_QBD0) * (1.0 - arg * sarg), PRM(XG_B3_OMMJ), PRM(XG_B3_R_OMMJ));
        capbd = czbd * sarg;
      } else {
        qbd = 0.0;
        capbd = 0.0;
      }
      if (czbdsw > 0.0) {
        arg = 1.0 - B3_DIV(vbd, PhiBSWTemp, PRM(XG_B3_R_PHIBSW));
        if (MJSW == 0.5) sarg = B3_RSQRT(arg);
        else sarg = exp(-MJSW * log(arg));
        qbd += B3_DIV(PRM(XG_B3_QBDSW0) * (1.0 - arg * sarg), PRM(XG_B3_OMMJSW), PRM(XG_B3_R_OMMJSW));
        capbd += czbdsw * sarg;
      }
      if (czbdswg > 0.0) {
        arg = 1.0 - B3_DIV(vbd, PhiBSWGTemp, PRM(XG_B3_R_PHIBSWG));
        if (MJSWG == 0.5) sarg = B3_RSQRT(arg);
        else sarg = exp(-MJSWG * log(arg));
        qbd += B3_DIV(PRM(XG_B3_QBDSWG0) * (1.0 - arg * sarg), PRM(XG_B3_OMMJSWG), PRM(XG_B3_R_OMMJSWG));
        capbd += czbdswg * sarg;
      }
    } else {
      T0 = czbd + czbdsw + czbdswg;
      T1 = vbd * (PRM(XG_B3_CBD_F) + PRM(XG_B3_CBDSW_F) + PRM(XG_B3_CBDSWG_F));
      qbd = vbd * (T0 + 0.5 * T1);
      capbd = T0 + T1;
    }
  }

  m.ggtg = m.ggtd = m.ggtb = m.ggts = 0.0;
  if (ChargeComputationNeeded) {
    const double ckappa = PRM(XG_B3_CKAPPA), cgdl = PRM(XG_B3_CGDL), cgsl = PRM(XG_B3_CGSL);
    if (capMod == 0) {
      cgdo = PRM(XG_B3_CGDO);
      qgdo = PRM(XG_B3_CGDO) * vgd;
      cgso = PRM(XG_B3_CGSO);
      qgso = PRM(XG_B3_CGSO) * vgs;
    } else if (capMod == 1) {
      if (vgd < 0.0) {
        T1 = sqrt(1.0 - B3_Q(4.0 * vgd, ckappa));
        cgdo = PRM(XG_B3_CGDO) + B3_Q(weffCV * cgdl, T1);
        qgdo = PRM(XG_B3_CGDO) * vgd - weffCV * 0.5 * cgdl * ckappa * (T1 - 1.0);
      } else {
        cgdo = PRM(XG_B3_CGDO) + weffCV * cgdl;
        qgdo = (weffCV * cgdl + PRM(XG_B3_CGDO)) * vgd;
      }
      if (vgs < 0.0) {
        T1 = sqrt(1.0 - B3_Q(4.0 * vgs, ckappa));
        cgso = PRM(XG_B3_CGSO) + B3_Q(weffCV * cgsl, T1);
        qgso = PRM(XG_B3_CGSO) * vgs - weffCV * 0.5 * cgsl * ckappa * (T1 - 1.0);
      } else {
        cgso = PRM(XG_B3_CGSO) + weffCV * cgsl;
        qgso = (weffCV * cgsl + PRM(XG_B3_CGSO)) * vgs;
      }
    } else {
      T0 = vgd + DELTA_1;
      T1 = sqrt(T0 * T0 + 4.0 * DELTA_1);
      T2 = 0.5 * (T0 - T1);
      T3 = PRM(XG_B3_CGDL_W);  // weffCV * cgdl
      T4 = sqrt(1.0 - B3_DIV(4.0 * T2, ckappa, PRM(XG_B3_R_CKAPPA)));
      cgdo = PRM(XG_B3_CGDO_T) - T3 * (1.0 - B3_Q(1.0, T4)) * (0.5 - B3_Q(0.5 * T0, T1));
      qgdo = PRM(XG_B3_CGDO_T) * vgd - T3 * (T2 + PRM(XG_B3_HALF_CKAPPA) * (T4 - 1.0));
      T0 = vgs + DELTA_1;
      T1 = sqrt(T0 * T0 + 4.0 * DELTA_1);
      T2 = 0.5 * (T0 - T1);
      T3 = PRM(XG_B3_CGSL_W);  // weffCV * cgsl
      T4 = sqrt(1.0 - B3_DIV(4.0 * T2, ckappa, PRM(XG_B3_R_CKAPPA)));
      cgso = PRM(XG_B3_CGSO_T) - T3 * (1.0 - B3_Q(1.0, T4)) * (0.5 - B3_Q(0.5 * T0, T1));
      qgso = PRM(XG_B3_CGSO_T) * vgs - T3 * (T2 + PRM(XG_B3_HALF_CKAPPA) * (T4 - 1.0));
    }
    /* setupCapacitors_oldDAE: charge sums and partition (:7640-7898), nqsMod 0 */
    const double cgbo = PRM(XG_B3_CGBO);
    double qgd, qgs, qgb;
    if (mode > 0) {
      qgd = qgdo;
      qgs = qgso;
      qgb = cgbo * vgb;
      qgate += qgd + qgs + qgb;
      qbulk -= qgb;
      qdrn -= qgd;
      qsrc = -(qgate + qbulk + qdrn);
      m.sxpart = 0.6;
      m.dxpart = 0.4;
    } else {
      qgd = qgdo;
      qgs = qgso;
      qgb = cgbo * vgb;
      qgate += qgd + qgs + qgb;
      qbulk -= qgb;
      qsrc = qdrn - qgs;
      qdrn = -(qgate + qbulk + qsrc);
      m.sxpart = 0.4;
      m.dxpart = 0.6;
    }
    /* setupCapacitors_newDAE (:7574-7638), nqsMod 0 */
    if (mode > 0) {
      mem.CAPcggb = (cggb + cgdo + cgso + cgbo);
      mem.CAPcgdb = (cgdb - cgdo);
      mem.CAPcgsb = (cgsb - cgso);
      mem.CAPcdgb = (cdgb - cgdo);
      mem.CAPcddb = (cddb + capbd + cgdo);
      mem.CAPcdsb = cdsb;
      mem.CAPcsgb = -(cggb + cbgb + cdgb + cgso);
      mem.CAPcsdb = -(cgdb + cbdb + cddb);
      mem.CAPcssb = (capbs + cgso - (cgsb + cbsb + cdsb));
      mem.CAPcbgb = (cbgb - cgbo);
      mem.CAPcbdb = (cbdb - capbd);
      mem.CAPcbsb = (cbsb - capbs);
    } else {
      mem.CAPcggb = (cggb + cgdo + cgso + cgbo);
      mem.CAPcgdb = (cgsb - cgdo);
      mem.CAPcgsb = (cgdb - cgso);
      mem.CAPcdgb = -(cggb + cbgb + cdgb + cgdo);
      mem.CAPcddb = (capbd + cgdo - (cgsb + cbsb + cdsb));
      mem.CAPcdsb = -(cgdb + cbdb + cddb);
      mem.CAPcsgb = (cdgb - cgso);
      mem.CAPcsdb = cdsb;
      mem.CAPcssb = (cddb + capbs + cgso);
      mem.CAPcbgb = (cbgb - cgbo);
      mem.CAPcbdb = (cbsb - capbd);
      mem.CAPcbsb = (cbdb - capbs);
    }
    mem.qg = qgate;
    mem.qd = qdrn - qbd;
    mem.qb = qbulk + qbd + qbs;
    mem.qbs = qbs;
    mem.qbd = qbd;
  }
  const double Idrain = PRM(XG_B3_GD) * Vddp;
  const double Isource = PRM(XG_B3_GS) * Vssp;

  // Master::updateState store / state writes (:9240-9278)
  sto[O_VBS] = vbs;
  sto[O_VGS] = vgs;
  sto[O_VDS] = vds;
  sto[O_VBD] = vbd;
  sto[O_VON] = von;
  sta[S_QB] = mem.qb;
  sta[S_QG] = mem.qg;
  sta[S_QD] = mem.qd;
  sta[S_QBS] = mem.qbs;
  sta[S_QBD] = mem.qbd;
  const bool init_tran_step = !f.dcop && f.init_tran && f.newton_iter == 0;
  if (init_tran_step) {
    double *csta = io.sta_curr_w + t.sta0 + (int64_t)i * 12;
    csta[S_QB] = mem.qb;
    csta[S_QG] = mem.qg;
    csta[S_QD] = mem.qd;
    csta[S_QBS] = mem.qbs;
    csta[S_QBD] = mem.qbd;
  }

  // Master::loadDAEVectors (:9306-9653)
  const double numberParallel = PRM(XG_B3_M);
  const double drainConductance = PRM(XG_B3_GD), sourceConductance = PRM(XG_B3_GS);
#undef PRM
  double cdreq_Jdxp = 0.0, ceqbd_Jdxp = 0.0, ceqbs_Jdxp = 0.0;
  double Gmx, Gmbsx, FwdSum, RevSum, cdreq, ceqbd, ceqbs;
  double gbbdp, gbbsp, gbdpg, gbdpdp, gbdpb, gbdpsp, gbspg, gbspdp, gbspb, gbspsp;
  if (mode >= 0) {
    Gmx = m.gm; Gmbsx = m.gmbs; FwdSum = Gmx + Gmbsx; RevSum = 0.0;
    cdreq = dtype * (m.cd);
    ceqbd = -dtype * (m.csub);
    ceqbs = 0.0;
    gbbdp = -m.gbds;
    gbbsp = (m.gbds + m.gbgs + m.gbbs);
    gbdpg = m.gbgs; gbdpdp = m.gbds; gbdpb = m.gbbs;
    gbdpsp = -(gbdpg + gbdpdp + gbdpb);
    gbspg = 0.0; gbspdp = 0.0; gbspb = 0.0; gbspsp = 0.0;
  } else {
    Gmx = -m.gm; Gmbsx = -m.gmbs; FwdSum = 0.0; RevSum = -(Gmx + Gmbsx);
    cdreq = -dtype * (m.cd);
    ceqbs = -dtype * (m.csub);
    ceqbd = 0.0;
    gbbsp = -m.gbds;
    gbbdp = (m.gbds + m.gbgs + m.gbbs);
    gbdpg = 0.0; gbdpsp = 0.0; gbdpb = 0.0; gbdpdp = 0.0;
    gbspg = m.gbgs; gbspsp = m.gbds; gbspb = m.gbbs;
    gbspdp = -(gbspg + gbspsp + gbspb);
  }
  if (dtype > 0) {
    ceqbs += (cbs);
    ceqbd += (cbd);
  } else {
    ceqbs -= (cbs);
    ceqbd -= (cbd);
  }
  Terms T{io.terms + t.term0, nI};
  T.put(0, i, drainConductance != 0.0 ? Idrain * numberParallel : 0.0);
  T.put(1, i, sourceConductance != 0.0 ? Isource * numberParallel : 0.0);
  T.put(2, i, (ceqbs + ceqbd) * numberParallel);
  T.put(3, i, (-(ceqbd - cdreq) - Idrain) * numberParallel);
  T.put(4, i, (-(cdreq + ceqbs) - Isource) * numberParallel);
  const bool lim = o.voltlim && !origFlag;
  if (lim) {
    double tmpj;
    if (mode >= 0) {
      tmpj = dtype * (-m.gds * (vds - vds_orig) - Gmx * (vgs - vgs_orig) - Gmbsx * (vbs - vbs_orig));
      cdreq_Jdxp += tmpj;
      cdreq += tmpj;
      tmpj = -dtype * (-m.gbds * (vds - vds_orig) - m.gbgs * (vgs - vgs_orig) - m.gbbs * (vbs - vbs_orig));
      ceqbd_Jdxp += tmpj;
      ceqbd += tmpj;
    } else {
      tmpj = -dtype * (m.gds * (vds - vds_orig) + Gmx * (vgd - vgd_orig) + Gmbsx * (vbd - vbd_orig));
      cdreq_Jdxp += tmpj;
      cdreq += tmpj;
      tmpj = -dtype * (m.gbds * (vds - vds_orig) - m.gbgs * (vgd - vgd_orig) - m.gbbs * (vbd - vbd_orig));
      ceqbd_Jdxp += tmpj;
      ceqbd += tmpj;
    }
    if (dtype > 0) {
      ceqbs_Jdxp += (-gbs * (vbs - vbs_orig));
      ceqbs += (-gbs * (vbs - vbs_orig));
      ceqbd_Jdxp += (-gbd * (vbd - vbd_orig));
      ceqbd += (-gbd * (vbd - vbd_orig));
    } else {
      ceqbs_Jdxp -= (-gbs * (vbs - vbs_orig));
      ceqbs -= (-gbs * (vbs - vbs_orig));
      ceqbd_Jdxp -= (-gbd * (vbd - vbd_orig));
      ceqbd -= (-gbd * (vbd - vbd_orig));
    }
  }
  T.put(5, i, lim ? -(ceqbs_Jdxp + ceqbd_Jdxp) * numberParallel : 0.0);
  T.put(6, i, lim ? (ceqbd_Jdxp - cdreq_Jdxp) * numberParallel : 0.0);
  T.put(7, i, lim ? (cdreq_Jdxp + ceqbs_Jdxp) * numberParallel : 0.0);

  // auxChargeCalculations (:7477-7573)
  if (ChargeComputationNeeded) {
    const double vgb_orig = vgs_orig - vbs_orig;
    mem.Qeqqg_Jdxp = 0.0;
    mem.Qeqqb_Jdxp = 0.0;
    mem.Qeqqd_Jdxp = 0.0;
    if (!origFlag) {
      mem.Qeqqg_Jdxp = -mem.CAPcggb * (vgb - vgb_orig) + mem.CAPcgdb * (vbd - vbd_orig) +
                       mem.CAPcgsb * (vbs - vbs_orig);
      mem.Qeqqb_Jdxp = -mem.CAPcbgb * (vgb - vgb_orig) + mem.CAPcbdb * (vbd - vbd_orig) +
                       mem.CAPcbsb * (vbs - vbs_orig);
      mem.Qeqqd_Jdxp = -mem.CAPcdgb * (vgb - vgb_orig) + mem.CAPcddb * (vbd - vbd_orig) +
                       mem.CAPcdsb * (vbs - vbs_orig);
    }
  } else {
    m.sxpart = (1.0 - (m.dxpart = (mode > 0) ? 0.4 : 0.6));
  }
  double Qeqqg, Qeqqb, Qeqqd;
  if (dtype > 0) {
    Qeqqg = mem.qg; Qeqqb = mem.qb; Qeqqd = mem.qd;
  } else {
    Qeqqg = -mem.qg; Qeqqb = -mem.qb; Qeqqd = -mem.qd;
  }
  T.put(8, i, Qeqqg * numberParallel);
  T.put(9, i, (Qeqqb) * numberParallel);
  T.put(10, i, (-(-Qeqqd)) * numberParallel);
  T.put(11, i, (-(+Qeqqg + Qeqqb + Qeqqd)) * numberParallel);
  if (o.voltlim && dtype <= 0) {
    mem.Qeqqg_Jdxp = -mem.Qeqqg_Jdxp;
    mem.Qeqqb_Jdxp = -mem.Qeqqb_Jdxp;
    mem.Qeqqd_Jdxp = -mem.Qeqqd_Jdxp;
  }
  T.put(12, i, lim ? -mem.Qeqqg_Jdxp * numberParallel : 0.0);
  T.put(13, i, lim ? -(+mem.Qeqqb_Jdxp) * numberParallel : 0.0);
  T.put(14, i, lim ? (-mem.Qeqqd_Jdxp) * numberParallel : 0.0);
  T.put(15, i, lim ? (+mem.Qeqqg_Jdxp + mem.Qeqqb_Jdxp + mem.Qeqqd_Jdxp) * numberParallel : 0.0);

  // Master::loadDAEMatrices (:9654-9939)
  const double M = numberParallel;
  const double GD = drainConductance, GS = sourceConductance;
  T.put(16, i, GD * M);
  T.put(17, i, -(GD * M));
  T.put(18, i, GS * M);
  T.put(19, i, -(GS * M));
  T.put(20, i, (-m.gbgs) * M);
  T.put(21, i, (gbd + gbs - m.gbbs) * M);
  T.put(22, i, (-gbd + gbbdp) * M);
  T.put(23, i, (-gbs + gbbsp) * M);
  T.put(24, i, -(GD * M));
  T.put(25, i, -((gbd - Gmbsx - gbdpb) * M));
  T.put(26, i, (Gmx + gbdpg) * M);
  T.put(27, i, (GD + m.gds + gbd + RevSum + gbdpdp) * M);
  T.put(28, i, -((m.gds + FwdSum - gbdpsp) * M));
  T.put(29, i, (-Gmx + gbspg) * M);
  T.put(30, i, -((gbs + Gmbsx - gbspb) * M));
  T.put(31, i, -(GS * M));
  T.put(32, i, -((m.gds + RevSum - gbspdp) * M));
  T.put(33, i, (GS + m.gds + gbs + FwdSum + gbspsp) * M);
  if (init_tran_step) {
#pragma unroll
    for (int q = 34; q < 50; ++q) T.put(q, i, 0.0);
  } else {
    T.put(34, i, (mem.CAPcggb) * M);
    T.put(35, i, -((mem.CAPcggb + mem.CAPcgdb + mem.CAPcgsb) * M));
    T.put(36, i, (mem.CAPcgdb) * M);
    T.put(37, i, (mem.CAPcgsb) * M);
    T.put(38, i, (mem.CAPcbgb) * M);
    T.put(39, i, (-mem.CAPcbgb - mem.CAPcbdb - mem.CAPcbsb) * M);
    T.put(40, i, (mem.CAPcbdb) * M);
    T.put(41, i, (mem.CAPcbsb) * M);
    T.put(42, i, -((+mem.CAPcdgb + mem.CAPcddb + mem.CAPcdsb) * M));
    T.put(43, i, (mem.CAPcdgb) * M);
    T.put(44, i, (+mem.CAPcddb) * M);
    T.put(45, i, -((-mem.CAPcdsb) * M));
    T.put(46, i, (mem.CAPcsgb) * M);
    T.put(47, i, -((+mem.CAPcsgb + mem.CAPcsdb + mem.CAPcssb) * M));
    T.put(48, i, -((-mem.CAPcsdb) * M));
    T.put(49, i, (+mem.CAPcssb) * M);
  }

  memp[(int64_t)B3M_CAPCGGB * nI] = mem.CAPcggb;
  memp[(int64_t)B3M_CAPCGDB * nI] = mem.CAPcgdb;
  memp[(int64_t)B3M_CAPCGSB * nI] = mem.CAPcgsb;
  memp[(int64_t)B3M_CAPCDGB * nI] = mem.CAPcdgb;
  memp[(int64_t)B3M_CAPCDDB * nI] = mem.CAPcddb;
  memp[(int64_t)B3M_CAPCDSB * nI] = mem.CAPcdsb;
  memp[(int64_t)B3M_CAPCSGB * nI] = mem.CAPcsgb;
  memp[(int64_t)B3M_CAPCSDB * nI] = mem.CAPcsdb;
  memp[(int64_t)B3M_CAPCSSB * nI] = mem.CAPcssb;
  memp[(int64_t)B3M_CAPCBGB * nI] = mem.CAPcbgb;
  memp[(int64_t)B3M_CAPCBDB * nI] = mem.CAPcbdb;
  memp[(int64_t)B3M_CAPCBSB * nI] = mem.CAPcbsb;
  memp[(int64_t)B3M_QJG * nI] = mem.Qeqqg_Jdxp;
  memp[(int64_t)B3M_QJB * nI] = mem.Qeqqb_Jdxp;
  memp[(int64_t)B3M_QJD * nI] = mem.Qeqqd_Jdxp;
  memp[(int64_t)B3M_QG * nI] = mem.qg;
  memp[(int64_t)B3M_QB * nI] = mem.qb;
  memp[(int64_t)B3M_QD * nI] = mem.qd;
  memp[(int64_t)B3M_QBS * nI] = mem.qbs;
  memp[(int64_t)B3M_QBD * nI] = mem.qbd;
}
