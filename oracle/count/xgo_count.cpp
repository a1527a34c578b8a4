// xgo_count.cpp — the operation counters of liboracle_count.so (TEST
// INFRASTRUCTURE ONLY): the oracle's load sources compiled as C++ over the
// counting scalar of xgo_count.hpp, one translation unit each
// (xgo_count_unit.cpp), export the same xgo_* load entry points as
// liboracle.so.  The counts are of the restated reference equations, so they
// are the algorithmic operations of a load, independent of how a GPU kernel
// evaluates them.
#include "xgo_count.hpp"

extern "C" {
unsigned long long xgo_count_ops[XC_NKIND];
void xgo_count_reset(void) { memset(xgo_count_ops, 0, sizeof xgo_count_ops); }
void xgo_count_get(unsigned long long *out) { memcpy(out, xgo_count_ops, sizeof xgo_count_ops); }
}
