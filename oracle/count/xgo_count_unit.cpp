// xgo_count_unit.cpp — one oracle source (XGO_UNIT, a quoted path) compiled
// over the counting scalar (TEST INFRASTRUCTURE ONLY; see xgo_count.cpp).
#include "xgo_count.hpp"

#define double xcnt
#include XGO_UNIT
