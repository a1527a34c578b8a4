// load_kernels.cu — the Newton-load kernels for sm_103a.
//
// One thread per device instance evaluates the model in FP64 (updateState) and
// writes every stamp term of that instance (loadDAEVectors/loadDAEMatrices) to
// a per-load term buffer laid out term-major, term[term0 + q*n + i], so a warp
// stores 32 consecutive doubles per term.  A second kernel sums the terms of
// each output (F, Q, dFdxdVp, dQdxdVp rows and dF/dx, dQ/dx non-zeros) in the
// reference's order — device type, instance, statement — from a precomputed
// list, one thread per output.  No atomics: results are identical run to run.
//
// This file is compiled twice: with -fmad=false into namespace xg::exact (each
// product and sum rounded on its own, as the serial CPU load does) and with
// -fmad=true into xg::fast (contracted to FMA).  XG_NS names the namespace.
// The fast build also splits each long output (a supply rail collects a term
// from every device on it) over the 256 threads of a block, each thread
// summing every 256th term in order, and adds the thread sums in a fixed
// butterfly and warp order: a serial chain of dependent FP64 adds (and
// gathers) is the slowest thing a GB300 can be asked to do.  The result is the same on every run, but not the reference's
// rounding, which the exact build keeps.

#include <cuda_runtime.h>

#include <algorithm>

#include <cstdint>

#include "xg_fast_rcp.cuh"
#include "xg_internal.h"

#ifndef XG_NS
#error "compile with -DXG_NS=exact or -DXG_NS=fast"
#endif
#ifndef XG_SPLIT_SUMS
#define XG_SPLIT_SUMS 0
#endif

namespace xg {
namespace XG_NS {

namespace {

constexpr double kMaxExpArg = 100.0;             // CONSTMAX_EXP_ARG
constexpr double kE = 2.718281828459045;         // CONSTe = exp(1.0), correctly rounded

__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }  // Xycemin
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }  // Xycemax

template <typename T>
__device__ __forceinline__ T ld(const T *p) { return __ldg(p); }

// ---- SPICE3 limiting, DeviceSupport (N_DEV_DeviceSupport.C:186-430) --------
__device__ __forceinline__ double limvds(double vnew, double vold) {
  if (vold >= 3.5) {
    if (vnew > vold) vnew = dmin(vnew, (3.0 * vold) + 2.0);
    else if (vnew < 3.5) vnew = dmax(vnew, 2.0);
  } else {
    if (vnew > vold) vnew = dmin(vnew, 4.0);
    else vnew = dmax(vnew, -0.5);
  }
  return vnew;
}

__device__ __forceinline__ double pnjlim(double vnew, double vold, double vt, double vcrit,
                                         int *icheck) {
  if ((vnew > vcrit) && (fabs(vnew - vold) > (vt + vt))) {
    if (vold > 0) {
      double arg = 1 + (vnew - vold) / vt;
      vnew = arg > 0 ? vold + vt * log(arg) : vcrit;
    } else {
      vnew = vt * log(vnew / vt);
    }
    *icheck = 1;
  } else {
    *icheck = 0;
  }
  return vnew;
}

__device__ __forceinline__ double fetlim(double vnew, double vold, double vto) {
  double vtsthi = fabs(2 * (vold - vto)) + 2;
  double vtstlo = vtsthi / 2 + 2;
  double vtox = vto + 3.5;
  double delv = vnew - vold;
  if (vold >= vto) {
    if (vold >= vtox) {
      if (delv <= 0) {
        if (vnew >= vtox) {
          if (-delv > vtstlo) vnew = vold - vtstlo;
        } else {
          vnew = dmax(vnew, vto + 2.0);
        }
      } else if (delv >= vtsthi) {
        vnew = vold + vtsthi;
      }
    } else {
      vnew = delv <= 0 ? dmax(vnew, vto - 0.5) : dmin(vnew, vto + 4.0);
    }
  } else {
    if (delv <= 0) {
      if (-delv > vtsthi) vnew = vold - vtsthi;
    } else {
      double vtemp = vto + 0.5;
      if (vnew <= vtemp) {
        if (delv > vtstlo) vnew = vold + vtstlo;
      } else {
        vnew = vtemp;
      }
    }
  }
  return vnew;
}

// DeviceSupport::qmeyer (N_DEV_DeviceSupport.C:545-631)
__device__ __forceinline__ void qmeyer(double vgs, double vgd, double von, double vdsat,
                                       double &capgs, double &capgd, double &capgb, double phi,
                                       double cox) {
  double vgst = vgs - von;
  if (vgst <= -phi) {
    capgb = cox / 2; capgs = 0; capgd = 0;
  } else if (vgst <= -phi / 2) {
    capgb = -vgst * cox / (2 * phi); capgs = 0; capgd = 0;
  } else if (vgst <= 0) {
    capgb = -vgst * cox / (2 * phi);
    capgs = vgst * cox / (1.5 * phi) + cox / 3;
    capgd = 0;
  } else {
    double vds = vgs - vgd;
    if (vdsat <= vds) {
      capgs = cox / 3; capgd = 0; capgb = 0;
    } else {
      double vddif = 2.0 * vdsat - vds;
      double vddif1 = vdsat - vds;
      double vddif2 = vddif * vddif;
      capgd = cox * (1.0 - vdsat * vdsat / vddif2) / 3;
      capgs = cox * (1.0 - vddif1 * vddif1 / vddif2) / 3;
      capgb = 0;
    }
  }
}

// Term writer: term q of instance i at [q][i], so a warp's store of one term
// fills whole sectors; the reduction gathers them.
struct Terms {
  double *__restrict__ base;
  int n;
  __device__ __forceinline__ void put(int q, int i, double v) const { base[(int64_t)q * n + i] = v; }
};

// Batched loads: take instance i's circuit flags; false when the instance is
// not evaluated (no circuit: an unused place in a slot; or a finished one).
__device__ __forceinline__ bool instance_flags(const DevType &t, int i, Flags &f) {
  if (!t.cid) return true;
  const int c = __ldg(t.cid + i);
  if (c < 0) return false;
  if (!t.cflags) return true;
  f = t.cflags[c];
  return !f.skip;
}
__device__ __forceinline__ bool instance_live(const DevType &t, int i) {
  if (!t.cid) return true;
  const int c = __ldg(t.cid + i);
  return c >= 0 && !(t.cflags && t.cflags[c].skip);
}

// ---- resistor (N_DEV_Resistor.C:1073-1135) ---------------------------------
__global__ void __launch_bounds__(256) res_kernel(DevType t, LoadIO io) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_live(t, i)) return;
  const int n = t.n;
  int lp = ld(t.lid + i), ln = ld(t.lid + n + i);
  double G = ld(t.p + i);
  double i0 = (ld(io.sol + lp) - ld(io.sol + ln)) * G;
  Terms T{io.terms + t.term0, n};
  T.put(0, i, i0);
  T.put(1, i, -i0);
  T.put(2, i, G);
  T.put(3, i, -G);
  T.put(4, i, -G);
  T.put(5, i, G);
}

// ---- capacitor, constant C, no IC (N_DEV_Capacitor.C:1821-2040) -------------
__global__ void __launch_bounds__(256) cap_kernel(DevType t, LoadIO io) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_live(t, i)) return;
  const int n = t.n;
  int lp = ld(t.lid + i), ln = ld(t.lid + n + i);
  double C = ld(t.p + i);
  double vcap = ld(io.sol + lp) - ld(io.sol + ln);
  double q0 = C * vcap;
  io.sta[t.sta0 + i] = q0;
  Terms T{io.terms + t.term0, n};
  T.put(0, i, q0);
  T.put(1, i, -q0);
  T.put(2, i, C);
  T.put(3, i, -C);
  T.put(4, i, -C);
  T.put(5, i, C);
}

// PulseData::updateSource (N_DEV_SourceData.C:928-1031) with bpTol = 0.
__device__ double pulse_value(const double *p, int n, int i, double t) {
  const double bpTol = 0.0;
  double V1 = ld(p + XG_V_V1 * n + i), V2 = ld(p + XG_V_V2 * n + i);
  double TD = ld(p + XG_V_TD * n + i), TR = ld(p + XG_V_TR * n + i);
  double TF = ld(p + XG_V_TF * n + i), PW = ld(p + XG_V_PW * n + i);
  double PER = ld(p + XG_V_PER * n + i);
  double time = t - TD;
  if (time > PER && PER != 0.0) time -= PER * floor(time / PER);
  if (time <= 0 || (time > (TR + PW + TF) && (fabs(time - (TR + PW + TF)) > bpTol))) return V1;
  if ((time > TR && fabs(time - TR) > bpTol) && (time < (TR + PW) || fabs(time - (TR + PW)) < bpTol))
    return V2;
  if (time > 0 && (time < TR || fabs(time - TR) < bpTol))
    return TR != 0.0 ? V1 + (V2 - V1) * (time) / TR : V1;
  return TF != 0.0 ? V2 + (V1 - V2) * (time - (TR + PW)) / TF : V2;
}

// ---- independent voltage source (N_DEV_Vsrc.C:941-1045) ---------------------
__global__ void __launch_bounds__(256) vsrc_kernel(DevType t, Flags f, LoadIO io) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_flags(t, i, f)) return;
  const int n = t.n;
  int lp = ld(t.lid + i), ln = ld(t.lid + n + i), lb = ld(t.lid + 2 * n + i);
  double source;
  if ((f.tranop || f.transient) && ld(t.p + XG_V_KIND * n + i) == XG_SRC_PULSE)
    source = pulse_value(t.p, n, i, f.time);
  else
    source = ld(t.p + XG_V_V1 * n + i);
  double srcCurrent = ld(io.sol + lb);
  double srcDrop = (ld(io.sol + lp) - ld(io.sol + ln));
  Terms T{io.terms + t.term0, n};
  T.put(0, i, srcCurrent);
  T.put(1, i, -srcCurrent);
  T.put(2, i, srcDrop);
  T.put(3, i, -source);
  T.put(4, i, 1.0);
  T.put(5, i, -1.0);
  T.put(6, i, 1.0);
  T.put(7, i, -1.0);
}

// ---- independent current source (N_DEV_ISRC.C:774-800) ----------------------
// The source value goes into F at both terminals; there are no matrix entries.
__global__ void __launch_bounds__(256) isrc_kernel(DevType t, Flags f, LoadIO io) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_flags(t, i, f)) return;
  const int n = t.n;
  double source;
  if ((f.tranop || f.transient) && ld(t.p + XG_V_KIND * n + i) == XG_SRC_PULSE)
    source = pulse_value(t.p, n, i, f.time);
  else
    source = ld(t.p + XG_V_V1 * n + i);
  Terms T{io.terms + t.term0, n};
  T.put(0, i, source);
  T.put(1, i, -source);
}

// ---- junction diode, level 1 (N_DEV_Diode.C:873-1331, 2007-2128) ------------
__global__ void __launch_bounds__(256) diode_kernel(DevType t, DevOptions o, Flags f, LoadIO io) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_flags(t, i, f)) return;
  const int n = t.n;
  const double *p = t.p;
#define PRM(k) ld(p + (k) * n + i)
  const int li_Pos = ld(t.lid + i), li_Neg = ld(t.lid + n + i), li_Pri = ld(t.lid + 2 * n + i);
  const double gmin = o.gmin;
  const double M = PRM(XG_D_M), BV = PRM(XG_D_BV), N = PRM(XG_D_N), TT = PRM(XG_D_TT);
  const double tVcrit = PRM(XG_D_TVCRIT), tBrkdwnV = PRM(XG_D_TBRKDWNV);
  const double tJctCap = PRM(XG_D_TJCTCAP);
  const int flags = (int)PRM(XG_D_FLAGS);
  const int BVGiven = flags & 1, InitCondGiven = (flags >> 1) & 1, off = (flags >> 2) & 1;
  double *sto = io.sto + t.sto0 + i;

  // Master::updateState stores the previous limited Vd before the update.
  const double vd_member = io.diode_vd[i];
  *sto = vd_member;
  double Vpp = ld(io.sol + li_Pri), Vn = ld(io.sol + li_Neg), Vp = ld(io.sol + li_Pos);
  double Vd = Vpp - Vn;
  double Isat = PRM(XG_D_ISAT);
  double Vte = N * PRM(XG_D_VT);
  const double Vd_orig = Vd;
  double Vd_old;
  if (f.newton_iter == 0) {
    if (f.init_jct && o.voltlim) {
      if (InitCondGiven) Vd = PRM(XG_D_INITCOND);
      else if (off) Vd = 0.0;
      else Vd = tVcrit;
    }
    Vd_old = f.dcop ? Vd : ld(io.sto_curr + t.sto0 + i);
  } else {
    Vd_old = vd_member;
  }
  if (o.voltlim && f.newton_iter >= 0) {
    int ichk = 0;
    if (BVGiven && (Vd < dmin(0.0, -BV + 10.0 * Vte))) {
      double Vdtmp = -(BV + Vd);
      Vdtmp = pnjlim(Vdtmp, -(Vd_old + BV), Vte, tVcrit, &ichk);
      Vd = -(Vdtmp + BV);
    } else {
      Vd = pnjlim(Vd, Vd_old, Vte, tVcrit, &ichk);
    }
  }
  double Id, Gd;
  if (Vd >= -3.0 * Vte) {
    double evd = exp(dmin(kMaxExpArg, Vd / Vte));
    Id = Isat * (evd - 1.0) + gmin * Vd;
    Gd = Isat * evd / Vte + gmin;
  } else {
    Isat *= PRM(XG_D_TIRF);
    if (!tBrkdwnV || (Vd >= -tBrkdwnV)) {
      double arg = 3.0 * Vte / (Vd * kE);
      arg = arg * arg * arg;
      Id = -Isat * (1.0 + arg) + gmin * Vd;
      Gd = Isat * 3.0 * arg / Vd + gmin;
    } else {
      double evrev = exp(dmin(kMaxExpArg, -(tBrkdwnV + Vd) / Vte));
      double arg2 = 3.0 * Vte / (kE * tBrkdwnV);
      arg2 = arg2 * arg2 * arg2;
      double Isat_tBrkdwnV = Isat * (1 - arg2);
      Id = -Isat_tBrkdwnV * evrev + gmin * Vd;
      Gd = Isat_tBrkdwnV * evrev / Vte + gmin;
    }
  }
  double Qd = 0.0, Cd = 0.0;
  const double Vc = Vd;
  if (tJctCap != 0.0) {
    double Area = PRM(XG_D_AREA), tJctPot = PRM(XG_D_TJCTPOT), tDepCap = PRM(XG_D_TDEPCAP);
    double Czero = tJctCap * Area;
    if (Vc < tDepCap) {
      double arg = 1.0 - Vc / tJctPot;
      double sarg = exp(dmin(kMaxExpArg, -M * log(arg)));
      Qd = TT * Id + tJctPot * Czero * (1.0 - arg * sarg) / (1.0 - M);
      Cd = TT * Gd + Czero * sarg;
    } else {
      double F2 = PRM(XG_D_F2), F3 = PRM(XG_D_F3);
      double Czof2 = Czero / F2;
      double MotJctPot = M / tJctPot;
      Qd = TT * Id + Czero * PRM(XG_D_TF1) +
           Czof2 * (F3 * (Vc - tDepCap) + (0.5 * MotJctPot) * (Vc * Vc - tDepCap * tDepCap));
      Cd = TT * Gd + Czof2 * (F3 + MotJctPot * Vc);
    }
  }
  io.diode_vd[i] = Vd;

  // Master::loadDAEVectors / loadDAEMatrices
  const double Gspr = PRM(XG_D_GSPR);
#undef PRM
  double Ir = Gspr * (Vp - Vpp);
  Terms T{io.terms + t.term0, n};
  T.put(0, i, -(-Ir));
  T.put(1, i, -Id);
  T.put(2, i, -(-Id + Ir));
  T.put(3, i, -Qd);
  T.put(4, i, -(-Qd));
  double Gd_Jdxp = 0.0, Cd_Jdxp = 0.0;
  if (o.voltlim) {
    double Vd_diff = Vd - Vd_orig;
    Cd_Jdxp = -(Cd)*Vd_diff;
    Gd_Jdxp = -(Gd)*Vd_diff;
  }
  T.put(5, i, Gd_Jdxp);
  T.put(6, i, -Gd_Jdxp);
  T.put(7, i, Cd_Jdxp);
  T.put(8, i, -Cd_Jdxp);
  T.put(9, i, Gspr);
  T.put(10, i, -Gspr);
  T.put(11, i, Gd);
  T.put(12, i, -Gd);
  T.put(13, i, -Gspr);
  T.put(14, i, -Gd);
  T.put(15, i, Gspr + Gd);
  T.put(16, i, Cd);
  T.put(17, i, -Cd);
  T.put(18, i, -Cd);
  T.put(19, i, Cd);
}

// ---- MOSFET level 1 (N_DEV_MOSFET1.C:2618-3427, 4103-4722), newMeyer off ----
__global__ void __launch_bounds__(128) mos1_kernel(DevType t, DevOptions o, Flags f, LoadIO io) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n || !instance_flags(t, i, f)) return;
  const int n = t.n;
  const double *p = t.p;
#define PRM(k) ld(p + (k) * n + i)
  const int li_d = ld(t.lid + i), li_g = ld(t.lid + n + i), li_s = ld(t.lid + 2 * n + i);
  const int li_b = ld(t.lid + 3 * n + i), li_dp = ld(t.lid + 4 * n + i), li_sp = ld(t.lid + 5 * n + i);
  const int dtype = (int)PRM(XG_M1_DTYPE);
  const double gamma = PRM(XG_M1_GAMMA);
  const double vt = PRM(XG_M1_VT), tPhi = PRM(XG_M1_TPHI);
  const double gmin = o.gmin;
  const int flags = (int)PRM(XG_M1_FLAGS);
  const int OFF = flags & 1, IC_GIVEN = (flags >> 1) & 1;
  double *sta = io.sta + t.sta0 + (int64_t)i * 8;
  double *sto = io.sto + t.sto0 + (int64_t)i * 5;
  const double *csta = io.sta_curr + t.sta0 + (int64_t)i * 8;
  const double *csto = io.sto_curr + t.sto0 + (int64_t)i * 5;
  enum { S_QGS, S_QGD, S_QGB, S_CAPGS, S_CAPGD, S_CAPGB, S_QBD, S_QBS };
  enum { O_VBD, O_VBS, O_VGS, O_VDS, O_VON };

  const double Vd = ld(io.sol + li_d), Vg = ld(io.sol + li_g), Vs = ld(io.sol + li_s);
  const double Vb = ld(io.sol + li_b), Vsp = ld(io.sol + li_sp), Vdp = ld(io.sol + li_dp);
  const double Vddp = Vd - Vdp, Vssp = Vs - Vsp;
  double vbs = dtype * (Vb - Vsp), vgs = dtype * (Vg - Vsp), vds = dtype * (Vdp - Vsp);
  double vbd = vbs - vds, vgd = vgs - vds;
  const double vgs_orig = vgs, vds_orig = vds, vbs_orig = vbs, vbd_orig = vbd, vgd_orig = vgd;

  bool forced = false;  // origFlag cleared by the initial-condition branch
  if (f.init_jct && !OFF && o.voltlim) {
    if (IC_GIVEN) {
      forced = true;
      vds = dtype * PRM(XG_M1_ICVDS);
      vgs = dtype * PRM(XG_M1_ICVGS);
      vbs = dtype * PRM(XG_M1_ICVBS);
    } else {
      vbs = -1;
      vgs = dtype * PRM(XG_M1_TVTO);
      vds = 0;
    }
    vbd = vbs - vds;
    vgd = vgs - vds;
  } else if ((f.init_fix || f.init_jct) && OFF) {
    vbs = vgs = vds = 0;
    vbd = vgd = 0;
  }

  double Von, vbs_old, vbd_old, vgs_old, vds_old;
  if (f.newton_iter == 0) {
    if (!f.dcop) {
      vbs_old = ld(csto + O_VBS); vbd_old = ld(csto + O_VBD);
      vgs_old = ld(csto + O_VGS); vds_old = ld(csto + O_VDS);
      Von = dtype * ld(csto + O_VON);
    } else {
      vbs_old = vbs; vbd_old = vbd; vgs_old = vgs; vds_old = vds;
      Von = 0.0;
    }
  } else {
    vbs_old = sto[O_VBS]; vbd_old = sto[O_VBD];
    vgs_old = sto[O_VGS]; vds_old = sto[O_VDS];
    Von = dtype * sto[O_VON];
  }
  const double vgd_old = vgs_old - vds_old;

  if (o.voltlim && !(f.init_fix && OFF)) {
    int Check = 1;
    if (vds_old >= 0) {
      vgs = fetlim(vgs, vgs_old, Von);
      vds = vgs - vgd;
      vds = limvds(vds, vds_old);
      vgd = vgs - vds;
    } else {
      vgd = fetlim(vgd, vgd_old, Von);
      vds = vgs - vgd;
      vds = -limvds(-vds, -vds_old);
      vgs = vgd + vds;
    }
    if (vds >= 0.0) {
      vbs = pnjlim(vbs, vbs_old, vt, PRM(XG_M1_SOURCEVCRIT), &Check);
      vbd = vbs - vds;
    } else {
      vbd = pnjlim(vbd, vbd_old, vt, PRM(XG_M1_DRAINVCRIT), &Check);
      vbs = vbd + vds;
    }
  }
  vbd = vbs - vds;
  vgd = vgs - vds;
  const double Vgb = vgs - vbs;
  const bool origFlag = !(forced || vgs_orig != vgs || vds_orig != vds || vbs_orig != vbs ||
                          vbd_orig != vbd || vgd_orig != vgd);

  double gbs, cbs, gbd, cbd;
  {
    const double SourceSatCur = PRM(XG_M1_SOURCESATCUR), DrainSatCur = PRM(XG_M1_DRAINSATCUR);
    if (vbs <= 0) {
      gbs = SourceSatCur / vt;
      gbs += gmin;
      cbs = gbs * vbs;
    } else {
      double evbs = exp(dmin(kMaxExpArg, vbs / vt));
      gbs = (SourceSatCur * evbs / vt + gmin);
      cbs = (SourceSatCur * (evbs - 1) + gmin * vbs);
    }
    if (vbd <= 0) {
      gbd = DrainSatCur / vt;
      gbd += gmin;
      cbd = gbd * vbd;
    } else {
      double evbd = exp(dmin(kMaxExpArg, vbd / vt));
      gbd = (DrainSatCur * evbd / vt + gmin);
      cbd = (DrainSatCur * (evbd - 1) + gmin * vbd);
    }
  }
  const int mode = (vds >= 0) ? 1 : -1;
  double Vdsat, cdrain, gm, gds, gmbs;
  {
    const double vbx = mode == 1 ? vbs : vbd;
    double sarg;
    if (vbx <= 0) {
      sarg = sqrt(tPhi - vbx);
    } else {
      sarg = sqrt(tPhi);
      sarg = sarg - vbx / (sarg + sarg);
      sarg = dmax(0.0, sarg);
    }
    Von = (PRM(XG_M1_TVBI) * dtype) + gamma * sarg;
    double vgst = (mode == 1 ? vgs : vgd) - Von;
    Vdsat = dmax(vgst, 0.0);
    double arg = sarg <= 0 ? 0 : gamma / (sarg + sarg);
    if (vgst <= 0) {
      cdrain = 0; gm = 0; gds = 0; gmbs = 0;
    } else {
      const double lambda = PRM(XG_M1_LAMBDA), Beta = PRM(XG_M1_BETA);
      double betap = Beta * (1 + lambda * (vds * mode));
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

  double qbs = 0, capbs = 0, qbd = 0, capbd = 0;
  {
    const double Cbs = PRM(XG_M1_CBS), Cbssw = PRM(XG_M1_CBSSW);
    const double Cbd = PRM(XG_M1_CBD), Cbdsw = PRM(XG_M1_CBDSW);
    if (Cbs != 0 || Cbssw != 0 || Cbd != 0 || Cbdsw != 0) {
      const double MJ = PRM(XG_M1_MJ), MJSW = PRM(XG_M1_MJSW);
      const double tDepCap = PRM(XG_M1_TDEPCAP), tBulkPot = PRM(XG_M1_TBULKPOT);
      double sarg, sargsw, arg;
      if (Cbs != 0 || Cbssw != 0) {
        if (vbs < tDepCap) {
          arg = 1 - vbs / tBulkPot;
          if (MJ == MJSW) {
            sarg = sargsw = (MJ == .5) ? 1 / sqrt(arg) : exp(-MJ * log(arg));
          } else {
            sarg = (MJ == .5) ? 1 / sqrt(arg) : exp(-MJ * log(arg));
            sargsw = (MJSW == .5) ? 1 / sqrt(arg) : exp(-MJSW * log(arg));
          }
          qbs = tBulkPot * (Cbs * (1 - arg * sarg) / (1 - MJ) + Cbssw * (1 - arg * sargsw) / (1 - MJSW));
          capbs = Cbs * sarg + Cbssw * sargsw;
        } else {
          const double f2s = PRM(XG_M1_F2S), f3s = PRM(XG_M1_F3S);
          qbs = PRM(XG_M1_F4S) + vbs * (f2s + vbs * (f3s / 2));
          capbs = f2s + f3s * vbs;
        }
      }
      if (Cbd != 0 || Cbdsw != 0) {
        if (vbd < tDepCap) {
          arg = 1 - vbd / tBulkPot;
          if (MJ == .5 && MJSW == .5) {
            sarg = sargsw = 1 / sqrt(arg);
          } else {
            sarg = (MJ == .5) ? 1 / sqrt(arg) : exp(-MJ * log(arg));
            sargsw = (MJSW == .5) ? 1 / sqrt(arg) : exp(-MJSW * log(arg));
          }
          qbd = tBulkPot * (Cbd * (1 - arg * sarg) / (1 - MJ) + Cbdsw * (1 - arg * sargsw) / (1 - MJSW));
          capbd = Cbd * sarg + Cbdsw * sargsw;
        } else {
          const double f2d = PRM(XG_M1_F2D), f3d = PRM(XG_M1_F3D);
          qbd = PRM(XG_M1_F4D) + vbd * (f2d + vbd * f3d / 2);
          capbd = f2d + vbd * f3d;
        }
      }
    }
  }

  double capgs, capgd, capgb;
  const double OxideCap = PRM(XG_M1_OXIDECAP);
  if (mode > 0) qmeyer(vgs, vgd, Von, Vdsat, capgs, capgd, capgb, tPhi, OxideCap);
  else qmeyer(vgd, vgs, Von, Vdsat, capgd, capgs, capgb, tPhi, OxideCap);

  double Capgs, Capgd, Capgb;
  {
    const double cgso = PRM(XG_M1_CGSO), cgdo = PRM(XG_M1_CGDO), cgbo = PRM(XG_M1_CGBO);
    if (f.dcop) {
      Capgs = 2.0 * capgs + cgso;
      Capgd = 2.0 * capgd + cgdo;
      Capgb = 2.0 * capgb + cgbo;
    } else {
      Capgs = (capgs + ld(csta + S_CAPGS) + cgso);
      Capgd = (capgd + ld(csta + S_CAPGD) + cgdo);
      Capgb = (capgb + ld(csta + S_CAPGB) + cgbo);
    }
    Capgs *= (Capgs < 0.0) ? -1.0 : 1.0;
    Capgd *= (Capgd < 0.0) ? -1.0 : 1.0;
    Capgb *= (Capgb < 0.0) ? -1.0 : 1.0;
  }
  const double drainConductance = PRM(XG_M1_GD), sourceConductance = PRM(XG_M1_GS);
  const double Idrain = drainConductance * Vddp;
  const double Isource = sourceConductance * Vssp;
  double Gm, Gmbs, nrmsum, revsum, cdreq;
  if (mode >= 0) {
    Gm = gm; Gmbs = gmbs; nrmsum = Gm + Gmbs; revsum = 0; cdreq = dtype * cdrain;
  } else {
    Gm = -gm; Gmbs = -gmbs; nrmsum = 0; revsum = -(Gm + Gmbs); cdreq = -(dtype)*cdrain;
  }

  // Master::updateState store / state writes
  sto[O_VBD] = vbd; sto[O_VBS] = vbs; sto[O_VGS] = vgs; sto[O_VDS] = vds; sto[O_VON] = von;
  sta[S_CAPGS] = capgs; sta[S_CAPGD] = capgd; sta[S_CAPGB] = capgb;
  double qgs, qgd, qgb;
  if (f.dcop) {
    qgs = Capgs * vgs; qgd = Capgd * vgd; qgb = Capgb * Vgb;
  } else {
    qgs = ld(csta + S_QGS); qgd = ld(csta + S_QGD); qgb = ld(csta + S_QGB);
    double vgs1 = ld(csto + O_VGS), vbs1 = ld(csto + O_VBS), vds1 = ld(csto + O_VDS);
    double vgb1 = vgs1 - vbs1, vgd1 = vgs1 - vds1;
    qgs += Capgs * (vgs - vgs1);
    qgd += Capgd * (vgd - vgd1);
    qgb += Capgb * ((vgs - vbs) - vgb1);
  }
  sta[S_QGS] = qgs; sta[S_QGD] = qgd; sta[S_QGB] = qgb; sta[S_QBD] = qbd; sta[S_QBS] = qbs;

  // Master::loadDAEVectors
  const double numberParallel = PRM(XG_M1_M);
#undef PRM
  Terms T{io.terms + t.term0, n};
  const double ceqbs = dtype * (cbs), ceqbd = dtype * (cbd);
  const double ceqgb = 0.0, ceqgs = 0.0, ceqgd = 0.0;
  T.put(0, i, drainConductance != 0.0 ? Idrain * numberParallel : 0.0);
  T.put(1, i, (ceqgs + ceqgd + ceqgb) * numberParallel);
  T.put(2, i, sourceConductance != 0.0 ? Isource * numberParallel : 0.0);
  T.put(3, i, (ceqbs + ceqbd - ceqgb) * numberParallel);
  T.put(4, i, (-Idrain - (ceqbd - cdreq + ceqgd)) * numberParallel);
  T.put(5, i, (-Isource - (ceqbs + cdreq + ceqgs)) * numberParallel);
  const double Qeqbs = dtype * (qbs), Qeqbd = dtype * (qbd), Qeqgb = dtype * (qgb);
  const double Qeqgs = dtype * (qgs), Qeqgd = dtype * (qgd);
  T.put(6, i, (Qeqgs + Qeqgd + Qeqgb) * numberParallel);
  T.put(7, i, (Qeqbs + Qeqbd - Qeqgb) * numberParallel);
  T.put(8, i, (-(Qeqbd + Qeqgd)) * numberParallel);
  T.put(9, i, (-(Qeqbs + Qeqgs)) * numberParallel);
  const bool cap_on = f.tranop || f.acop || f.transient;
  const double gcgd = cap_on ? Capgd : 0.0, gcgs = cap_on ? Capgs : 0.0, gcgb = cap_on ? Capgb : 0.0;
  const double gcbs = cap_on ? capbs : 0.0, gcbd = cap_on ? capbd : 0.0;
  if (!origFlag) {
    const double dvgs = vgs - vgs_orig, dvgd = vgd - vgd_orig, dvbs = vbs - vbs_orig;
    const double dvbd = vbd - vbd_orig, dvds = vds - vds_orig;
    const double dvg = (mode > 0) ? dvgs : dvgd, dvb = (mode > 0) ? dvbs : dvbd;
    T.put(10, i, (dtype * (+((gbd - gmin)) * (dvbd) + ((gbs - gmin)) * (dvbs))) * numberParallel);
    T.put(11, i, (dtype * (-((gbd - gmin)) * (dvbd) + gds * (dvds) + Gm * dvg + Gmbs * dvb)) * numberParallel);
    T.put(12, i, (dtype * (-((gbs - gmin)) * (dvbs) - gds * (dvds) - Gm * dvg - Gmbs * dvb)) * numberParallel);
    const double dvgsb = vgs - vgs_orig - vbs + vbs_orig;
    T.put(13, i, (dtype * (gcgd * (dvgd) + gcgs * (dvgs) + gcgb * dvgsb)) * numberParallel);
    T.put(14, i, (dtype * (-(gcgb)*dvgsb + (gcgb) * (dvbd) + (gcbs) * (dvbs))) * numberParallel);
    T.put(15, i, (dtype * (-(gcgd) * (dvgd) - (gcbd) * (dvbd))) * numberParallel);
    T.put(16, i, (dtype * (-gcgs * (dvgs) - (gcbs) * (dvbs))) * numberParallel);
  } else {
#pragma unroll
    for (int q = 10; q <= 16; ++q) T.put(q, i, 0.0);
  }
  // Master::loadDAEMatrices (pointer path); `-=` stored as the negated term.
  const double M = numberParallel;
  T.put(17, i, drainConductance * M);
  T.put(18, i, -(drainConductance * M));
  T.put(19, i, sourceConductance * M);
  T.put(20, i, -(sourceConductance * M));
  T.put(21, i, (gbs + gbd) * M);
  T.put(22, i, -(gbd * M));
  T.put(23, i, -(gbs * M));
  T.put(24, i, -(drainConductance * M));
  T.put(25, i, (Gm)*M);
  T.put(26, i, (-gbd + Gmbs) * M);
  T.put(27, i, (drainConductance + gds + gbd + revsum) * M);
  T.put(28, i, (-gds - nrmsum) * M);
  T.put(29, i, -((Gm)*M));
  T.put(30, i, -(sourceConductance * M));
  T.put(31, i, -((gbs + Gmbs) * M));
  T.put(32, i, -((gds + revsum) * M));
  T.put(33, i, (sourceConductance + gds + gbs + nrmsum) * M);
  T.put(34, i, (gcgd + gcgs + gcgb) * M);
  T.put(35, i, -(gcgb * M));
  T.put(36, i, -(gcgd * M));
  T.put(37, i, -(gcgs * M));
  T.put(38, i, -(gcgb * M));
  T.put(39, i, (+gcbs + gcbd + gcgb) * M);
  T.put(40, i, -(+gcbd * M));
  T.put(41, i, -(+gcbs * M));
  T.put(42, i, -gcgd * M);
  T.put(43, i, -gcbd * M);
  T.put(44, i, (+gcbd + gcgd) * M);
  T.put(45, i, -(gcgs * M));
  T.put(46, i, -(+gcbs * M));
  T.put(47, i, (+gcbs + gcgs) * M);
}

#include "bsim3_eval.cuh"

// ---- fixed-order reduction ---------------------------------------------------
// Each output is the sum of its terms in the reference's statement order,
// s = ((0 + t1) + t2) + ..., so the result is bit-identical to a serial load.
// Short outputs take a thread each.  Outputs with more than kLongSegment
// terms (a supply node collects a term from every device on it) take a warp
// each: the warp gathers the terms, 256 at a time, into shared memory with
// independent loads, and one lane adds them in order.  Blocks [0, long_blocks)
// serve the long outputs, the rest the short ones.
constexpr int kRedThreads = 256;
constexpr int kRedWarps = kRedThreads / 32;
constexpr int kRedChunk = 256;

__global__ void __launch_bounds__(kRedThreads) reduce_kernel(ReduceArgs a, int long_blocks) {
  if ((int)blockIdx.x < long_blocks) {
#if XG_SPLIT_SUMS
    // a block per long output: every thread sums a strided share of its terms,
    // then a fixed butterfly per warp and the warps in order
    __shared__ double part[kRedWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t w = blockIdx.x; w < a.n_long; w += long_blocks) {
      const int64_t o = a.long_out[w];
      const int64_t b = __ldg(a.red_ptr + o), e = __ldg(a.red_ptr + o + 1);
      double s = 0.0;
#pragma unroll 4
      for (int64_t j = b + threadIdx.x; j < e; j += blockDim.x)
        s += __ldg(a.terms + __ldg(a.red_idx + j));
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
      if (lane == 0) part[wid] = s;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = part[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) t += part[k];
        a.out[o] = t;
      }
      __syncthreads();
    }
    return;
#else
    __shared__ double buf[kRedWarps][kRedChunk];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t w = (int64_t)blockIdx.x * kRedWarps + wid; w < a.n_long;
         w += (int64_t)long_blocks * kRedWarps) {
      const int64_t o = a.long_out[w];
      const int64_t b = __ldg(a.red_ptr + o), e = __ldg(a.red_ptr + o + 1);
      double s = 0.0;
      for (int64_t base = b; base < e; base += kRedChunk) {
        const int cnt = (int)(e - base < kRedChunk ? e - base : kRedChunk);
        for (int j = lane; j < cnt; j += 32)
          buf[wid][j] = __ldg(a.terms + __ldg(a.red_idx + base + j));
        __syncwarp();
        if (lane == 0)
          for (int j = 0; j < cnt; ++j) s += buf[wid][j];
        __syncwarp();
      }
      if (lane == 0) a.out[o] = s;
    }
    return;
#endif
  }
  // two short outputs per thread (kEllThreads apart), their bucket found by
  // the block; every term number loaded coalesced, the two outputs' term
  // loads interleaved so that twice as many are in flight, each output
  // summed in its own order
  static_assert(kEllPerThread == 2, "the loop below takes two outputs per thread");
  const int64_t g = a.ell_block0 + ((int64_t)blockIdx.x - long_blocks);
  int lo = a.b0, hi = a.b1 - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&a.ell[mid].block0) <= g) lo = mid;
    else hi = mid - 1;
  }
  const EllBucket B = a.ell[lo];
  const int64_t k0 = (g - B.block0) * kEllPerBlock + threadIdx.x, k1 = k0 + kEllThreads;
  if (k0 >= B.m) return;
  const uint32_t *ix = a.ell_idx + B.idx0;
  if (k1 < B.m) {
    double s0 = 0.0, s1 = 0.0;
#pragma unroll 4
    for (int j = 0; j < B.c; ++j) {
      const int64_t row = (int64_t)j * B.m;
      const double t0 = __ldg(a.terms + __ldg(ix + row + k0));
      const double t1 = __ldg(a.terms + __ldg(ix + row + k1));
      s0 += t0;
      s1 += t1;
    }
    a.out[__ldg(a.ell_out + B.out0 + k0)] = s0;
    a.out[__ldg(a.ell_out + B.out0 + k1)] = s1;
  } else {
    double s = 0.0;
#pragma unroll 8
    for (int j = 0; j < B.c; ++j) s += __ldg(a.terms + __ldg(ix + (int64_t)j * B.m + k0));
    a.out[__ldg(a.ell_out + B.out0 + k0)] = s;
  }
}

int grid_for(int64_t n, int block) { return (int)((n + block - 1) / block); }

}  // namespace

int launch_eval(int dev_type, const DevType &t, const DevOptions &o, const Flags &f,
                const LoadIO &io, void *stream) {
  if (t.n <= 0) return XG_OK;
  cudaStream_t s = (cudaStream_t)stream;
  switch (dev_type) {
    case XG_DEV_RES: res_kernel<<<grid_for(t.n, 256), 256, 0, s>>>(t, io); xg::count_launches(1); break;
    case XG_DEV_CAP: cap_kernel<<<grid_for(t.n, 256), 256, 0, s>>>(t, io); xg::count_launches(1); break;
    case XG_DEV_VSRC: vsrc_kernel<<<grid_for(t.n, 256), 256, 0, s>>>(t, f, io); xg::count_launches(1); break;
    case XG_DEV_ISRC: isrc_kernel<<<grid_for(t.n, 256), 256, 0, s>>>(t, f, io); xg::count_launches(1); break;
    case XG_DEV_DIODE: diode_kernel<<<grid_for(t.n, 256), 256, 0, s>>>(t, o, f, io); xg::count_launches(1); break;
    case XG_DEV_MOS1: mos1_kernel<<<grid_for(t.n, 128), 128, 0, s>>>(t, o, f, io); xg::count_launches(1); break;
    case XG_DEV_BSIM3: bsim3_kernel<<<grid_for(t.n, 128), 128, 0, s>>>(t, o, f, io); xg::count_launches(1); break;
    default: return XG_ERR_UNSUPPORTED;
  }
  return cudaGetLastError() == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

int launch_reduce(const ReduceArgs &a, void *stream) {
  if (a.n_long <= 0 && a.ell_blocks <= 0) return XG_OK;
  const int sms = sm_count();
  const int64_t grid = a.ell_blocks;  // one thread per short output
  static_assert(kEllThreads == kRedThreads, "the ELL buckets are cut in blocks of the reduction's size");
#if XG_SPLIT_SUMS
  const int long_blocks = (int)std::min<int64_t>(a.n_long, sms * 8);  // a block per long output
#else
  const int long_blocks = (int)std::min<int64_t>((a.n_long + kRedWarps - 1) / kRedWarps, sms * 8);
#endif
  if (grid + long_blocks <= 0) return XG_OK;
  reduce_kernel<<<(unsigned)(grid + long_blocks), kRedThreads, 0, (cudaStream_t)stream>>>(a, long_blocks);
  xg::count_launches(1);
  return cudaGetLastError() == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

}  // namespace XG_NS
}  // namespace xg
