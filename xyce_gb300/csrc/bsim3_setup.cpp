// bsim3_setup.cpp — BSIM3 v3.2 host setup (placeholder until the BSIM3 path lands).
#include "xg_bsim3_setup.h"

namespace xg {

int b3_nlid() { return 4; }
int b3_nterm() { return 0; }
const TermDef *b3_terms() { return nullptr; }

int b3_make_model(const xg_model_desc &, const xg_device_options &, B3Model *,
                  std::string *err) {
  *err = "BSIM3 is not available in this build";
  return XG_ERR_UNSUPPORTED;
}

int b3_instance_params(const B3Model &, const xg_mos_desc &, int, const xg_device_options &,
                       double *, std::string *err) {
  *err = "BSIM3 is not available in this build";
  return XG_ERR_UNSUPPORTED;
}

void b3_assign_lids(const double *, int, int, const int *ext, int *, int *lids) {
  for (int k = 0; k < 4; ++k) lids[k] = ext[k];
}

}  // namespace xg
