/* Test-infrastructure shim (oracle build only).
 * src/Saphyre2/ms/fem/TetrahedronElementSet3.cpp:37-71 calls GNU GSL's
 * gsl_poly_solve_cubic (version unpinned: the reference vendors no copy and has
 * no lockfile). It is reached only from ComputeDoC (TES3.cpp:477-743), whose
 * result (the direction of collapse) is read by the PD/DAPD rotation modes and
 * not by the MSVD + truncated-differential path the oracle runs. The
 * definition in ../gsl_poly_cubic.c restates the published closed form
 * (Viete's trigonometric form for three real roots, Cardano otherwise). */
#ifndef ORACLE_SHIM_GSL_POLY_H
#define ORACLE_SHIM_GSL_POLY_H
#ifdef __cplusplus
extern "C" {
#endif
int gsl_poly_solve_cubic(double a, double b, double c, double *x0, double *x1, double *x2);
#ifdef __cplusplus
}
#endif
#endif
