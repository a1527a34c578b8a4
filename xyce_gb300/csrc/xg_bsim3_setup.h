// xg_bsim3_setup.h — BSIM3 v3.2 host setup interface (bsim3_setup.cpp).
#pragma once

#include <string>

#include "xg.h"
#include "xg_internal.h"

namespace xg {

// Per-instance parameter block width for BSIM3 (see bsim3_setup.cpp for the
// column meanings).
enum { XG_B3_NPARAMS = 1 };

struct B3Model {
  int dtype = 1;
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
