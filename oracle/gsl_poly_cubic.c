/* Test infrastructure: closed-form real roots of x^3 + a x^2 + b x + c = 0,
 * the contract of GNU GSL's gsl_poly_solve_cubic (roots returned in
 * ascending order, count returned). Restated from the published method:
 * depress with x = t - a/3, then Viete's trigonometric form when the
 * discriminant says three real roots, Cardano's formula otherwise.
 * Only ComputeDoC (TetrahedronElementSet3.cpp:586-743) calls it: the DAPD
 * rotation's time of collapse. Its result does not reach the MSVD path. Both
 * the reference build and the oracle restatement link this one file. */
#include <math.h>
#include "shims/gsl/gsl_poly.h"

static void sort3(double *r0, double *r1, double *r2)
{
    double t;
    if (*r0 > *r1) { t = *r0; *r0 = *r1; *r1 = t; }
    if (*r1 > *r2) { t = *r1; *r1 = *r2; *r2 = t; }
    if (*r0 > *r1) { t = *r0; *r0 = *r1; *r1 = t; }
}

int gsl_poly_solve_cubic(double a, double b, double c, double *x0, double *x1, double *x2)
{
    double q = (a * a - 3.0 * b) / 9.0;
    double r = (2.0 * a * a * a - 9.0 * a * b + 27.0 * c) / 54.0;
    double q3 = q * q * q;
    double shift = a / 3.0;
    if (r == 0.0 && q == 0.0) {
        *x0 = *x1 = *x2 = -shift;
        return 3;
    }
    if (r * r < q3) {
        /* three distinct real roots */
        double theta = acos(r / sqrt(q3));
        double m = -2.0 * sqrt(q);
        const double two_pi = 6.283185307179586;
        *x0 = m * cos(theta / 3.0) - shift;
        *x1 = m * cos((theta + two_pi) / 3.0) - shift;
        *x2 = m * cos((theta - two_pi) / 3.0) - shift;
        sort3(x0, x1, x2);
        return 3;
    }
    if (r * r == q3) {
        /* a double root */
        double sq = sqrt(q);
        if (r > 0) { *x0 = -2.0 * sq - shift; *x1 = sq - shift; *x2 = sq - shift; }
        else { *x0 = -sq - shift; *x1 = -sq - shift; *x2 = 2.0 * sq - shift; }
        sort3(x0, x1, x2);
        return 3;
    }
    {
        double s = cbrt(fabs(r) + sqrt(r * r - q3));
        double A = (r > 0) ? -s : s;
        double B = (A == 0.0) ? 0.0 : q / A;
        *x0 = (A + B) - shift;
        return 1;
    }
}
