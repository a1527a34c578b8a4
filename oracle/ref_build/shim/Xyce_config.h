/* Minimal stand-in for the autoconf-generated Xyce_config.h: only what the
 * device, Core, Utility and ErrorHandling sources test for. Test
 * infrastructure for building the reference's device code; not product code. */
#ifndef XG_SHIM_XYCE_CONFIG_H
#define XG_SHIM_XYCE_CONFIG_H
#include <limits.h>
#include <float.h>
#define HAVE_CMATH 1
#define HAVE_CSTDIO 1
#define HAVE_CSTDLIB 1
#define HAVE_CSTRING 1
#define HAVE_CLIMITS 1
#define HAVE_IOSTREAM 1
#define HAVE_FSTREAM 1
#define HAVE_ALGORITHM 1
#define HAVE_UNORDERED_MAP 1
#endif
