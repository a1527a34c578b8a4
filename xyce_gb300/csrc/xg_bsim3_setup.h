// xg_bsim3_setup.h — BSIM3 v3.2 host setup interface (bsim3_setup.cpp).
#pragma once

#include <map>
#include <string>

#include "xg.h"
#include "xg_internal.h"

namespace xg {

enum { XG_B3_NPARAMS_ = XG_B3_NPARAMS };

// A BSIM3 model card after Model::Model and Model::processParams
// (N_DEV_MOSFET_B3.C:8488-8570, 8603-9105): every parameter by its netlist
// name, the given flags, and the derived model constants.
struct B3Model {
  int dtype = 1;
  std::map<std::string, double> v;   // every parameter, defaults filled in
  std::map<std::string, bool> given;
  bool g(const char *k) const {
    auto it = given.find(k);
    return it != given.end() && it->second;
  }
  double operator[](const char *k) const { return v.at(k); }
  // processParams outputs
  double cox = 0, vcrit = 0, factor1 = 0, Vtm0 = 0, Eg0 = 0, ni = 0, tnom = 0;
};

int b3_nlid();
int b3_nterm();
const TermDef *b3_terms();
int b3_make_model(const xg_model_desc &md, const xg_device_options &opt, B3Model *m,
                  std::string *err);
int b3_instance_params(const B3Model &m, const xg_mos_desc &d, int i,
                       const xg_device_options &opt, double *out, std::string *err);
void b3_assign_lids(const double *params, int n, int i, const int *ext, int *next, int *lids);

}  // namespace xg
