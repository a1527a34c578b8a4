/* Stand-in declaration for Teuchos_SerialDenseMatrix.hpp (Trilinos): named by
 * reference output headers on no path the harnesses reach.  Test
 * infrastructure only. */
#ifndef XG_SHIM_TEUCHOS_SDM
#define XG_SHIM_TEUCHOS_SDM
namespace Teuchos { template <class OrdinalType, class ScalarType> class SerialDenseMatrix; }
#endif
