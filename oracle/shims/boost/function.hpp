/* Test-infrastructure shim (oracle build only).
 * The reference's solver interface (src/Saphyre2/ns/IIterativeLinearSystemSolver.h:26-27)
 * names boost::function for its two callbacks. boost is not installed here; the
 * callbacks are plain call-through glue with no arithmetic, so std::function
 * is an exact stand-in. */
#ifndef ORACLE_SHIM_BOOST_FUNCTION_HPP
#define ORACLE_SHIM_BOOST_FUNCTION_HPP
#include <functional>
namespace boost { using std::function; }
#endif
