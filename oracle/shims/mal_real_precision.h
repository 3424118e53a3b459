/* Test-infrastructure shim (oracle/_ref "dbl" variant only), force-included
 * before the reference sources.
 *
 * src/Mal/RealUtils.h:27,45,48,63 define Sqrt/Sin/Cos/ATan2 as templates that
 * evaluate through float: T(sqrt(float(x))). With Real = double that makes
 * the FP64 build compute its rotations at float precision, and near F = I the
 * squared cofactor column norm (about 1e-64) underflows to zero in float, so
 * Largest_Column_Normalized divides by zero and R is NaN: every scene that
 * starts at rest freezes. These explicit specialisations evaluate the four
 * functions the rotation path calls at the precision of Real (double). The
 * reference's integer-argument call Sqrt(3) in Fast_Eigenvalues is not a
 * double call and keeps its value 1. */
#ifndef ORACLE_MAL_REAL_PRECISION_H
#define ORACLE_MAL_REAL_PRECISION_H
#include <math.h>
#include <Mal/RealUtils.h>
namespace mal {
template <> inline double Sqrt<double>(double v) { return ::sqrt(v); }
template <> inline double Sin<double>(double v) { return ::sin(v); }
template <> inline double Cos<double>(double v) { return ::cos(v); }
template <> inline double ATan2<double>(double y, double x) { return ::atan2(y, x); }
}
#endif
