/* Stand-in for Teuchos_Utils.hpp (Trilinos): included, not used, by the
 * reference's time-integration data store.  Test infrastructure only. */
#ifndef XG_SHIM_TEUCHOS_UTILS
#define XG_SHIM_TEUCHOS_UTILS
#endif
