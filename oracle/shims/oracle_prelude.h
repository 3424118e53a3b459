/* Test-infrastructure shim (oracle build only), force-included before the
 * reference sources.
 * - src/Saphyre2/ns/real_array.h uses memset/memcpy without <cstring>.
 * - src/Saphyre2/ns/MatrixD.h needs boost::ublas, which is absent. Its only
 *   user on this path is Assemble_A_From_Av (IIterativeLinearSystemSolver.h:70-84),
 *   which the oracle never calls; a stand-in with the same element access
 *   lets the header compile. */
#ifndef ORACLE_PRELUDE_H
#define ORACLE_PRELUDE_H
#include <cstring>
#include <cstdlib>
#define S2_NS_MATRIX_D_H
namespace S2 { namespace ns {
typedef double RealD;
struct MatrixD { double& operator()(unsigned, unsigned) { static double s; return s; } };
struct VectorD { double& operator()(unsigned) { static double s; return s; } };
}}
#endif
