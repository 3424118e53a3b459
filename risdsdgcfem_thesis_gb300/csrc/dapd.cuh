// dapd.cuh -- the DAPD rotation of the reference's element set
// (ms::fem::Params::eRM_DAPD), FP64, for the BeginEvaluation kernel in
// rotation.cu (compiled without fused multiply-adds, so that each product
// and sum rounds as in the reference).
//
//   UpdateDegeneration     TetrahedronElementSet3.cpp:477-533
//   ComputeDoC             TetrahedronElementSet3.cpp:589-743
//   ComputeRotations_DAPD  TetrahedronElementSet3.cpp:860-892
//   Compute_R_DAPD_Degenerate   Rotation.cpp:364-495
//   GRotation3x3_PolarDecomposition  Mal/GMatDecomposition.h:411-432
//
// Matrices are row-major double[9].
#pragma once
#include <stdint.h>

#include "msvd.cuh"

namespace femgb {

struct DapdParams {
    double thr;            // m_DegenerateThresholdDetF
    double fL, fNL, eNL;   // m_DAPD_L_Factor, m_DAPD_NL_Factor, m_DAPD_NL_Exponent (float32 values)
};

// Direction of collapse (TetrahedronElement3::DoC, TetrahedronElement3.h:28-38):
// V-F when vit0 == vit1 (the vertex opposite the collapsing face), E-E when
// vit0 < vit1 (vit0 = 0, vit1 the edge 0-vit1 crossing the opposite edge),
// none when vit0 > vit1.
__device__ __forceinline__ bool doc_valid(uchar2 d) { return d.x <= d.y; }
__device__ __forceinline__ uchar2 doc_none() { return make_uchar2(3, 0); }

// mal::Det (Mal/GMat.h:236-245)
__device__ __forceinline__ double det3_rm(const double* m)
{
    return m[0] * m[4] * m[8] - m[0] * m[7] * m[5] + m[3] * m[7] * m[2] - m[3] * m[1] * m[8] + m[6] * m[1] * m[5] -
           m[6] * m[4] * m[2];
}

// mal::Inverse of the transpose of H (Mal/GMat.h:291-313 applied to H^T)
__device__ __forceinline__ void inverse_transpose3(const double* h, double* r)
{
    const double m[9] = {h[0], h[3], h[6], h[1], h[4], h[7], h[2], h[5], h[8]};
    const double inv_det = 1.0 / det3_rm(m);
    r[0] = inv_det * (m[4] * m[8] - m[5] * m[7]);
    r[1] = inv_det * (m[2] * m[7] - m[1] * m[8]);
    r[2] = inv_det * (m[1] * m[5] - m[2] * m[4]);
    r[3] = inv_det * (m[5] * m[6] - m[3] * m[8]);
    r[4] = inv_det * (m[0] * m[8] - m[2] * m[6]);
    r[5] = inv_det * (m[2] * m[3] - m[0] * m[5]);
    r[6] = inv_det * (m[3] * m[7] - m[4] * m[6]);
    r[7] = inv_det * (m[1] * m[6] - m[0] * m[7]);
    r[8] = inv_det * (m[0] * m[4] - m[1] * m[3]);
}

// Newton polar iteration H <- (H + H^-T) / 2 while |H1 - H0|_F^2 > 0.01f, at
// most 10 iterations; the iterate is the rotation (not exactly orthonormal
// under the loose stopping test, as in the reference).
__device__ __forceinline__ void polar_newton(const double* H, double* R)
{
    double H0[9];
#pragma unroll
    for (int c = 0; c < 9; c++) H0[c] = H[c];
    const double prec_sq = (double)0.01f;
    for (int it = 0; it < 10; it++) {
        double Hit[9];
        inverse_transpose3(H0, Hit);
        double error = 0.0;
#pragma unroll
        for (int c = 0; c < 9; c++) {
            const double h1 = 0.5 * (H0[c] + Hit[c]);
            const double d = h1 - H0[c];
            error += d * d;
            H0[c] = h1;
        }
        if (!(error > prec_sq)) break;
    }
#pragma unroll
    for (int c = 0; c < 9; c++) R[c] = H0[c];
}

// Real roots of x^3 + a x^2 + b x + c = 0 in ascending order, and their
// count (the contract of GSL's gsl_poly_solve_cubic): depressed with
// x = t - a/3, Viete's trigonometric form for three real roots, Cardano's
// formula for one.
__device__ __forceinline__ int cubic_monic_roots(double a, double b, double c, double* r)
{
    const double q = (a * a - 3.0 * b) / 9.0;
    const double rr = (2.0 * a * a * a - 9.0 * a * b + 27.0 * c) / 54.0;
    const double q3 = q * q * q;
    const double shift = a / 3.0;
    if (rr == 0.0 && q == 0.0) {
        r[0] = r[1] = r[2] = -shift;
        return 3;
    }
    if (rr * rr < q3) {
        const double theta = ::acos(rr / ::sqrt(q3));
        const double m = -2.0 * ::sqrt(q);
        const double two_pi = 6.283185307179586;
        double x0 = m * ::cos(theta / 3.0) - shift;
        double x1 = m * ::cos((theta + two_pi) / 3.0) - shift;
        double x2 = m * ::cos((theta - two_pi) / 3.0) - shift;
        double t;
        if (x0 > x1) { t = x0; x0 = x1; x1 = t; }
        if (x1 > x2) { t = x1; x1 = x2; x2 = t; }
        if (x0 > x1) { t = x0; x0 = x1; x1 = t; }
        r[0] = x0; r[1] = x1; r[2] = x2;
        return 3;
    }
    if (rr * rr == q3) {
        const double sq = ::sqrt(q);
        if (rr > 0) { r[0] = -2.0 * sq - shift; r[1] = sq - shift; r[2] = sq - shift; }
        else { r[0] = -sq - shift; r[1] = -sq - shift; r[2] = 2.0 * sq - shift; }
        if (r[0] > r[1]) { double t = r[0]; r[0] = r[1]; r[1] = t; }
        if (r[1] > r[2]) { double t = r[1]; r[1] = r[2]; r[2] = t; }
        if (r[0] > r[1]) { double t = r[0]; r[0] = r[1]; r[1] = t; }
        return 3;
    }
    const double s = ::cbrt(::fabs(rr) + ::sqrt(rr * rr - q3));
    const double A = (rr > 0) ? -s : s;
    const double B = (A == 0.0) ? 0.0 : q / A;
    r[0] = (A + B) - shift;
    return 1;
}

// mal::GSolvePolynomialEq3 as TetrahedronElementSet3.cpp:49-70 defines it
// (the monic cubic for a != 0, else GSolvePolynomialEq2/Eq1 of
// Mal/GSolvePolynomialEq.h:11-40 with IsZero's epsilon 0.0001f).
__device__ __forceinline__ int solve_cubic(double a, double b, double c, double d, double* r)
{
    if (a != 0.0) return cubic_monic_roots(b / a, c / a, d / a, r);
    r[2] = 0.0;
    const double eps = (double)0.0001f;
    if (::fabs(b) <= eps) {
        if (::fabs(c) <= eps) return 0;
        r[0] = -d / c;
        r[1] = r[0];
        return 1;
    }
    const double disc = c * c - 4 * b * d;
    if (disc < 0) return 0;
    const double root = ::sqrt(disc);
    const double inv_divisor = 1.0 / (2.0 * b);
    double x1 = (-c - root) * inv_divisor, x2 = (-c + root) * inv_divisor;
    if (x1 > x2) { double t = x1; x1 = x2; x2 = t; }
    r[0] = x1;
    r[1] = x2;
    return (x1 == x2) ? 1 : 2;
}

__device__ __forceinline__ V3<double> vsub(V3<double> a, V3<double> b) { return mk<double>(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3<double> vadd(V3<double> a, V3<double> b) { return mk<double>(a.x + b.x, a.y + b.y, a.z + b.z); }

// ComputeDoC: the time of collapse t in (0, 1] where det F along the straight
// path a -> b reaches the threshold (a cubic in t), then the kind of
// collapse at that time.
__device__ __forceinline__ uchar2 compute_doc(const V3<double> a[4], const V3<double> b[4], double volume, double thr)
{
    const V3<double> d0 = vsub(b[0], a[0]), d1 = vsub(b[1], a[1]), d2 = vsub(b[2], a[2]), d3 = vsub(b[3], a[3]);
    const V3<double> d10 = vsub(d1, d0), d20 = vsub(d2, d0), d30 = vsub(d3, d0);
    const V3<double> a10 = vsub(a[1], a[0]), a20 = vsub(a[2], a[0]), a30 = vsub(a[3], a[0]);
    const double K = thr * 6.0 * volume;
    const double A = +d10.x * d20.y * d30.z + d20.x * d30.y * d10.z + d30.x * d10.y * d20.z
                     - d30.x * d20.y * d10.z - d20.x * d10.y * d30.z - d10.x * d30.y * d20.z;
    const double B = +(a10.x * d20.y * d30.z + d10.x * a20.y * d30.z + d10.x * d20.y * a30.z)
                     + (a20.x * d30.y * d10.z + d20.x * a30.y * d10.z + d20.x * d30.y * a10.z)
                     + (a30.x * d10.y * d20.z + d30.x * a10.y * d20.z + d30.x * d10.y * a20.z)
                     - (a30.x * d20.y * d10.z + d30.x * a20.y * d10.z + d30.x * d20.y * a10.z)
                     - (a20.x * d10.y * d30.z + d20.x * a10.y * d30.z + d20.x * d10.y * a30.z)
                     - (a10.x * d30.y * d20.z + d10.x * a30.y * d20.z + d10.x * d30.y * a20.z);
    const double C = +(a10.x * a20.y * d30.z + a10.x * d20.y * a30.z + d10.x * a20.y * a30.z)
                     + (a20.x * a30.y * d10.z + a20.x * d30.y * a10.z + d20.x * a30.y * a10.z)
                     + (a30.x * a10.y * d20.z + a30.x * d10.y * a20.z + d30.x * a10.y * a20.z)
                     - (a30.x * a20.y * d10.z + a30.x * d20.y * a10.z + d30.x * a20.y * a10.z)
                     - (a20.x * a10.y * d30.z + a20.x * d10.y * a30.z + d20.x * a10.y * a30.z)
                     - (a10.x * a30.y * d20.z + a10.x * d30.y * a20.z + d10.x * a30.y * a20.z);
    const double D = +a10.x * a20.y * a30.z + a20.x * a30.y * a10.z + a30.x * a10.y * a20.z
                     - a30.x * a20.y * a10.z - a20.x * a10.y * a30.z - a10.x * a30.y * a20.z - K;
    double roots[3] = {0.0, 0.0, 0.0};
    const int n = solve_cubic(A, B, C, D, roots);
    if (n <= 0) return doc_none();
    double toc = 2.0;
    int n01 = 0;
    for (int i = 0; i < n; i++)
        if (roots[i] > 0.0 && roots[i] <= 1.0 && roots[i] < toc) {
            toc = roots[i];
            n01++;
        }
    if (n01 != 1 && n01 != 3) return doc_none();
    const V3<double> q0 = vadd(a[0], scale(toc, d0)), q1 = vadd(a[1], scale(toc, d1));
    const V3<double> q2 = vadd(a[2], scale(toc, d2)), q3 = vadd(a[3], scale(toc, d3));
    const V3<double> e1 = vsub(q1, q0), e2 = vsub(q2, q0), e3 = vsub(q3, q0);
    // collapse normal: the right singular vector of the smallest singular value of [e1 e2 e3]
    const double Q[9] = {e1.x, e2.x, e3.x, e1.y, e2.y, e3.y, e1.z, e2.z, e3.z};
    V3<double> N;
    msvd_rotation<double>(Q, nullptr, nullptr, &N);
    double area[4];
    area[0] = ::fabs(dot0(N, cross(vsub(q2, q1), vsub(q3, q1))));
    area[1] = ::fabs(dot0(N, cross(e2, e3)));
    area[2] = ::fabs(dot0(N, cross(e1, e3)));
    area[3] = ::fabs(dot0(N, cross(e1, e2)));
    const double sum_area = area[0] + area[1] + area[2] + area[3];
    uchar2 doc = doc_none();
    for (int f = 0; f < 4; f++)
        if (::fabs(area[f] - 0.5 * sum_area) <= (double)0.0001f) doc = make_uchar2(f, f);
    if (!doc_valid(doc)) {
        if (dot0(cross(e1, e2), cross(e1, e3)) < 0.0) doc = make_uchar2(0, 1);
        else if (dot0(cross(e2, e1), cross(e2, e3)) < 0.0) doc = make_uchar2(0, 2);
        else if (dot0(cross(e3, e1), cross(e3, e2)) < 0.0) doc = make_uchar2(0, 3);
        else doc = make_uchar2(0, 0);
    }
    return doc;
}

// Compute_R_DAPD_Degenerate: move the collapsing vertex (V-F) or edge (E-E)
// along the unit collapse normal past the threshold by lambda_u (a Hermite
// spline in front of the collapse plane, linear plus power behind it), then
// the polar rotation of the projected F. R = I when the collapse normal is
// too short.
__device__ __forceinline__ void dapd_degenerate(double detF, uchar2 doc, V3<double> X[4], double volume,
                                                const double* Dinv, const DapdParams& p, double* R)
{
    // i0 (and i1 for E-E) move; ia is the vertex the offset w is measured from
    int i0, i1 = -1, ia;
    V3<double> axis;
    if (doc.x == doc.y) {
        i0 = doc.x;
        ia = (i0 + 1) & 3;
        const V3<double> x1 = X[ia], x2 = X[(i0 + 2) & 3], x3 = X[(i0 + 3) & 3];
        axis = cross(vsub(x2, x1), vsub(x3, x1));
    } else {
        const int v1 = doc.y;
        const int v2 = (v1 == 1) ? 2 : 1, v3 = (v1 == 3) ? 2 : 3;
        i0 = doc.x;
        i1 = v1;
        ia = v2;
        axis = cross(vsub(X[v1], X[i0]), vsub(X[v3], X[v2]));
    }
    const double len_sq = dot0(axis, axis);
    if (!(len_sq > (double)0.000001f)) {
#pragma unroll
        for (int c = 0; c < 9; c++) R[c] = (c % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    const double len = ::sqrt(len_sq);
    axis = scale(1.0 / len, axis);
    const double dha = p.thr * 6 * volume / len;
    double w = dot0(vsub(X[i0], X[ia]), axis);
    if (w * detF < 0) {
        w = -w;
        axis = mk<double>(-axis.x, -axis.y, -axis.z);
    }
    const double s = w / dha, t = 1.0 - s;
    const double lambda = (w > 0) ? p.fL * dha * ((2 - t) * t * t) : p.fL * dha * (t + p.fNL * ::pow(-s, p.eNL));
    X[i0] = vadd(X[i0], scale(lambda, axis));
    if (i1 >= 0) X[i1] = vadd(X[i1], scale(lambda, axis));
    double F[9], det_projF;
    deformation_gradient(X, Dinv, F, det_projF);
    polar_newton(F, R);
}

// BeginEvaluation's rotation under DAPD for one element: the direction of
// collapse is updated from the previous and current positions
// (UpdateDegeneration), then R is the polar rotation of F above the
// threshold, the DAPD rotation below it when a direction of collapse is
// known, and I otherwise.
__device__ __forceinline__ void dapd_rotation(const V3<double> xprev[4], V3<double> x[4], const double* Dinv,
                                              const double* F, double detF, double volume, const DapdParams& p,
                                              uchar2& doc, double* R)
{
    if (detF > p.thr) {
        doc = doc_none();
        polar_newton(F, R);
        return;
    }
    double Fp[9], detFp;
    deformation_gradient(xprev, Dinv, Fp, detFp);
    if (detFp > p.thr) doc = compute_doc(xprev, x, volume, p.thr);
    if (doc_valid(doc)) {
        dapd_degenerate(detF, doc, x, volume, Dinv, p, R);
    } else {
#pragma unroll
        for (int c = 0; c < 9; c++) R[c] = (c % 4 == 0) ? 1.0 : 0.0;
    }
}

}  // namespace femgb
