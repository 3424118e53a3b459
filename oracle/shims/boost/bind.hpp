/* Test-infrastructure shim (oracle build only).
 * The reference's geometry headers (src/Geo/shape/TetSolidShape3.cpp and the
 * bounding-volume hierarchy it includes) name boost::bind for callbacks of
 * its collision queries, which the shape harness never calls. boost is not
 * installed here; std::bind is an exact stand-in. */
#ifndef ORACLE_SHIM_BOOST_BIND_HPP
#define ORACLE_SHIM_BOOST_BIND_HPP
#include <functional>
namespace boost { using std::bind; }
using namespace std::placeholders;
#endif
