/*
 * xgo_support.c — SPICE3 voltage limiting and Meyer capacitances
 * (TEST INFRASTRUCTURE ONLY; see xgo.h).  Restates
 * src/DeviceModelPKG/Core/src/N_DEV_DeviceSupport.C.
 */
#include <math.h>

#include "xgo_internal.h"

static double dmin(double a, double b) { return a < b ? a : b; }
static double dmax(double a, double b) { return a > b ? a : b; }

/* DeviceSupport::limvds, N_DEV_DeviceSupport.C:186-213 */
double xgo_limvds(double vnew, double vold) {
  if (vold >= 3.5) {
    if (vnew > vold) vnew = dmin(vnew, (3.0 * vold) + 2.0);
    else if (vnew < 3.5) vnew = dmax(vnew, 2.0);
  } else {
    if (vnew > vold) vnew = dmin(vnew, 4.0);
    else vnew = dmax(vnew, -0.5);
  }
  return vnew;
}

/* DeviceSupport::pnjlim, N_DEV_DeviceSupport.C:214-262 */
double xgo_pnjlim(double vnew, double vold, double vt, double vcrit, int *icheck) {
  if ((vnew > vcrit) && (fabs(vnew - vold) > (vt + vt))) {
    if (vold > 0) {
      double arg = 1 + (vnew - vold) / vt;
      if (arg > 0) vnew = vold + vt * log(arg);
      else vnew = vcrit;
    } else {
      vnew = vt * log(vnew / vt);
    }
    *icheck = 1;
  } else {
    *icheck = 0;
  }
  return vnew;
}

/* DeviceSupport::fetlim, N_DEV_DeviceSupport.C:337-430 */
double xgo_fetlim(double vnew, double vold, double vto) {
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
      } else {
        if (delv >= vtsthi) vnew = vold + vtsthi;
      }
    } else {
      if (delv <= 0) vnew = dmax(vnew, vto - 0.5);
      else vnew = dmin(vnew, vto + 4.0);
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

/* DeviceSupport::qmeyer, N_DEV_DeviceSupport.C:545-631 */
void xgo_qmeyer(double vgs, double vgd, double vgb, double von, double vdsat,
                double *capgs, double *capgd, double *capgb, double phi, double cox) {
  (void)vgb;
  double vgst = vgs - von;
  if (vgst <= -phi) {
    *capgb = cox / 2;
    *capgs = 0;
    *capgd = 0;
  } else if (vgst <= -phi / 2) {
    *capgb = -vgst * cox / (2 * phi);
    *capgs = 0;
    *capgd = 0;
  } else if (vgst <= 0) {
    *capgb = -vgst * cox / (2 * phi);
    *capgs = vgst * cox / (1.5 * phi) + cox / 3;
    *capgd = 0;
  } else {
    double vds = vgs - vgd;
    if (vdsat <= vds) {
      *capgs = cox / 3;
      *capgd = 0;
      *capgb = 0;
    } else {
      double vddif = 2.0 * vdsat - vds;
      double vddif1 = vdsat - vds;
      double vddif2 = vddif * vddif;
      *capgd = cox * (1.0 - vdsat * vdsat / vddif2) / 3;
      *capgs = cox * (1.0 - vddif1 * vddif1 / vddif2) / 3;
      *capgb = 0;
    }
  }
}
