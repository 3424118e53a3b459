/* TEST INFRASTRUCTURE ONLY -- the oracle restatement. See fem_oracle.h.
 *
 * Written in plain C99 with the reference's evaluation order kept term for
 * term: every matrix-vector product is an accumulator started at zero and
 * summed over the column index (src/Mal/GMatUtils.h:12-23), every matrix
 * product likewise (src/Mal/GMat.h:133-145), division of a vector by a
 * scalar multiplies by the reciprocal (src/Mal/GVec.h:83), and Sqrt/Sin/
 * Cos/ATan2 go through float (src/Mal/RealUtils.h:27,45,48,63). Built with
 * -ffp-contract=off so no multiply-add is fused.
 */
#include "fem_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double v[3]; } vec3;
typedef struct { double m[3][3]; } mat3;

/* ---- Mal scalar semantics (src/Mal/RealUtils.h) -------------------------- */

/* Which scalar math the Mal functions use, per calling thread (set by every
 * public entry point from the solid): FEM_ORC_MATH_DOUBLE evaluates Sqrt/Sin/
 * Cos/ATan2 in double; FEM_ORC_MATH_FLOAT_LITERAL reproduces the reference
 * FP64 build as written, T(f(float(x))) with the host's float libm
 * (RealUtils.h:27,45,48,63). */
static __thread int g_math = FEM_ORC_MATH_DOUBLE;

static double mal_sqrt(double x)
{
    if (g_math == FEM_ORC_MATH_FLOAT_LITERAL) return (double)sqrtf((float)x);
    return sqrt(x);
}
static double mal_atan2(double y, double x)
{
    if (g_math == FEM_ORC_MATH_FLOAT_LITERAL) return (double)atan2f((float)y, (float)x);
    return atan2(y, x);
}
static double mal_cos(double x)
{
    if (g_math == FEM_ORC_MATH_FLOAT_LITERAL) return (double)cosf((float)x);
    return cos(x);
}
static double mal_sin(double x)
{
    if (g_math == FEM_ORC_MATH_FLOAT_LITERAL) return (double)sinf((float)x);
    return sin(x);
}

/* ---- Mal vector/matrix semantics ---------------------------------------- */

static vec3 v3(double a, double b, double c) { vec3 r; r.v[0] = a; r.v[1] = b; r.v[2] = c; return r; }
static vec3 v_add(vec3 a, vec3 b) { return v3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
static vec3 v_sub(vec3 a, vec3 b) { return v3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
static vec3 v_scale(double s, vec3 a) { return v3(s * a.v[0], s * a.v[1], s * a.v[2]); }
static vec3 v_neg(vec3 a) { return v3(-a.v[0], -a.v[1], -a.v[2]); }
/* GVec::operator* (dot), accumulator from zero (GVec.h:88) */
static double v_dot(vec3 a, vec3 b)
{
    double acc = 0;
    for (int i = 0; i < 3; i++) acc += a.v[i] * b.v[i];
    return acc;
}
/* GVec::operator% (GVec.h:89-91) */
static vec3 v_cross(vec3 a, vec3 b)
{
    return v3(a.v[1] * b.v[2] - a.v[2] * b.v[1],
              a.v[2] * b.v[0] - a.v[0] * b.v[2],
              a.v[0] * b.v[1] - a.v[1] * b.v[0]);
}
/* GVec::operator/ : multiply by the reciprocal (GVec.h:83) */
static vec3 v_div(vec3 a, double s) { double inv = 1.0 / s; return v_scale(inv, a); }
/* Norm = Sqrt(NormSq) (GVec.h:102-105); Normalized = v / Norm (GVec.h:97) */
static double v_norm(vec3 a) { return mal_sqrt(v_dot(a, a)); }
static vec3 v_normalized(vec3 a) { return v_div(a, v_norm(a)); }

/* Mat-vector product (GMatUtils.h:12-23) */
static vec3 m_mulv(const mat3* m, vec3 x)
{
    vec3 r;
    for (int i = 0; i < 3; i++) {
        double acc = 0;
        for (int j = 0; j < 3; j++) acc += m->m[i][j] * x.v[j];
        r.v[i] = acc;
    }
    return r;
}
/* Matrix product (GMat.h:133-145) */
static mat3 m_mul(const mat3* a, const mat3* b)
{
    mat3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double acc = 0;
            for (int k = 0; k < 3; k++) acc += a->m[i][k] * b->m[k][j];
            r.m[i][j] = acc;
        }
    return r;
}
static mat3 m_transposed(const mat3* a)
{
    mat3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = a->m[j][i];
    return r;
}
/* GMat3x3_From_Columns (GMatUtils.h:133-138) */
static mat3 m_from_columns(vec3 c0, vec3 c1, vec3 c2)
{
    mat3 r;
    for (int i = 0; i < 3; i++) { r.m[i][0] = c0.v[i]; r.m[i][1] = c1.v[i]; r.m[i][2] = c2.v[i]; }
    return r;
}
/* Det 3x3 (GMat.h:236-245) */
static double m_det(const mat3* a)
{
    const double (*m)[3] = a->m;
    return m[0][0] * m[1][1] * m[2][2]
         - m[0][0] * m[2][1] * m[1][2]
         + m[1][0] * m[2][1] * m[0][2]
         - m[1][0] * m[0][1] * m[2][2]
         + m[2][0] * m[0][1] * m[1][2]
         - m[2][0] * m[1][1] * m[0][2];
}
/* Inverse 3x3 (GMat.h:291-313) */
static mat3 m_inverse(const mat3* a)
{
    const double (*m)[3] = a->m;
    double inv_det = 1.0 / m_det(a);
    mat3 r;
    r.m[0][0] = inv_det * (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
    r.m[0][1] = inv_det * (m[0][2] * m[2][1] - m[0][1] * m[2][2]);
    r.m[0][2] = inv_det * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
    r.m[1][0] = inv_det * (m[1][2] * m[2][0] - m[1][0] * m[2][2]);
    r.m[1][1] = inv_det * (m[0][0] * m[2][2] - m[0][2] * m[2][0]);
    r.m[1][2] = inv_det * (m[0][2] * m[1][0] - m[0][0] * m[1][2]);
    r.m[2][0] = inv_det * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    r.m[2][1] = inv_det * (m[0][1] * m[2][0] - m[0][0] * m[2][1]);
    r.m[2][2] = inv_det * (m[0][0] * m[1][1] - m[0][1] * m[1][0]);
    return r;
}
static vec3 m_col(const mat3* a, int j) { return v3(a->m[0][j], a->m[1][j], a->m[2][j]); }

/* ---- MSVD rotation: GFastSVD3x3 (src/Mal/GMatDecomposition_SVD3x3_PhysBAM.h) */

typedef struct { double x11, x21, x31, x22, x32, x33; } sym3;
typedef struct { double x11, x21, x22; } sym2;

/* Orthogonal_Vector (PhysBAM.h:35-49) */
static vec3 orthogonal_vector(vec3 v)
{
    double ax = fabs(v.v[0]), ay = fabs(v.v[1]), az = fabs(v.v[2]);
    if (ax < ay)
        return (ax < az) ? v3(0, v.v[2], -v.v[1]) : v3(v.v[1], -v.v[0], 0);
    return (ay < az) ? v3(-v.v[2], 0, v.v[0]) : v3(v.v[1], -v.v[0], 0);
}

/* GSymmetricMat3x3::Cofactor_Matrix (PhysBAM.h:139-147) */
static sym3 sym3_cofactor(sym3 a)
{
    sym3 r;
    r.x11 = a.x22 * a.x33 - a.x32 * a.x32;
    r.x21 = a.x32 * a.x31 - a.x21 * a.x33;
    r.x31 = a.x21 * a.x32 - a.x22 * a.x31;
    r.x22 = a.x11 * a.x33 - a.x31 * a.x31;
    r.x32 = a.x21 * a.x31 - a.x11 * a.x32;
    r.x33 = a.x11 * a.x22 - a.x21 * a.x21;
    return r;
}

/* GSymmetricMat3x3::Largest_Column_Normalized (PhysBAM.h:149-156) */
static vec3 sym3_largest_column_normalized(sym3 a)
{
    double s11 = a.x11 * a.x11, s12 = a.x21 * a.x21, s13 = a.x31 * a.x31;
    double s22 = a.x22 * a.x22, s23 = a.x32 * a.x32, s33 = a.x33 * a.x33;
    double scale1 = s11 + s12 + s13, scale2 = s12 + s22 + s23, scale3 = s13 + s23 + s33;
    if (scale1 > scale2) {
        if (scale1 > scale3) return v_div(v3(a.x11, a.x21, a.x31), mal_sqrt(scale1));
    } else if (scale2 > scale3)
        return v_div(v3(a.x21, a.x22, a.x32), mal_sqrt(scale2));
    if (scale3 > 0) return v_div(v3(a.x31, a.x32, a.x33), mal_sqrt(scale3));
    return v3(1, 0, 0);
}

/* GSymmetricMat2x2::Largest_Column_Normalized (PhysBAM.h:75-82), on the
 * cofactor matrix (x22, -x21, x11) of a (PhysBAM.h:70-73). */
static void sym2_cofactor_largest_column_normalized(sym2 a, double out[2])
{
    double c11 = a.x22, c21 = -a.x21, c22 = a.x11;
    double s11 = c11 * c11, s12 = c21 * c21, s22 = c22 * c22;
    double scale1 = s11 + s12, scale2 = s12 + s22;
    if (scale1 > scale2) {
        double inv = 1.0 / mal_sqrt(scale1);
        out[0] = inv * c11; out[1] = inv * c21;
    } else if (scale2 > 0) {
        double inv = 1.0 / mal_sqrt(scale2);
        out[0] = inv * c21; out[1] = inv * c22;
    } else {
        out[0] = 1; out[1] = 0;
    }
}

/* Fast_Eigenvalues (PhysBAM.h:161-197). Note the reference's
 * cRootThree( Sqrt(3) ): Sqrt is a template on its argument type, the
 * argument is the int literal 3, so it evaluates int(sqrtf(3.0f)) == 1. The
 * restatement keeps that value. */
static void fast_eigenvalues(sym3 a, double lambda_out[3])
{
    const double one_third = 1.0 / 3.0;
    const double one_sixth = 1.0 / 6.0;
    const double root_three = 1.0; /* reference value, see above */
    double m = one_third * (a.x11 + a.x22 + a.x33);
    double a11 = a.x11 - m, a22 = a.x22 - m, a33 = a.x33 - m;
    double a12_sqr = a.x21 * a.x21, a13_sqr = a.x31 * a.x31, a23_sqr = a.x32 * a.x32;
    double p = one_sixth * (a11 * a11 + a22 * a22 + a33 * a33 + 2 * (a12_sqr + a13_sqr + a23_sqr));
    double q = .5 * (a11 * (a22 * a33 - a23_sqr) - a22 * a13_sqr - a33 * a12_sqr) + a.x21 * a.x31 * a.x32;
    double sqrt_p = mal_sqrt(p), disc = p * p * p - q * q;
    double disc_clamped = (0.0 > disc) ? 0.0 : disc; /* Max((T)0, disc), NumberUtils.h:35 */
    double phi = one_third * mal_atan2(mal_sqrt(disc_clamped), q);
    double c = mal_cos(phi), s = mal_sin(phi);
    double sqrt_p_cos = sqrt_p * c, root_three_sqrt_p_sin = root_three * sqrt_p * s;
    double l0 = m + 2 * sqrt_p_cos;
    double l1 = m - sqrt_p_cos - root_three_sqrt_p_sin;
    double l2 = m - sqrt_p_cos + root_three_sqrt_p_sin;
    if (l0 < l1) {
        if (l1 < l2) { lambda_out[0] = l2; lambda_out[1] = l1; lambda_out[2] = l0; }
        else if (l0 < l2) { lambda_out[0] = l1; lambda_out[1] = l2; lambda_out[2] = l0; }
        else { lambda_out[0] = l1; lambda_out[1] = l0; lambda_out[2] = l2; }
    } else {
        if (l1 > l2) { lambda_out[0] = l0; lambda_out[1] = l1; lambda_out[2] = l2; }
        else if (l0 > l2) { lambda_out[0] = l0; lambda_out[1] = l2; lambda_out[2] = l1; }
        else { lambda_out[0] = l2; lambda_out[1] = l0; lambda_out[2] = l1; }
    }
}

/* Fast_Eigenvectors (PhysBAM.h:199-236); returns V with eigenvectors as columns */
static mat3 fast_eigenvectors(sym3 A, const double lambda[3])
{
    int flipped = 0;
    double lf[3] = {lambda[0], lambda[1], lambda[2]};
    if (lambda[0] - lambda[1] < lambda[1] - lambda[2]) {
        lf[0] = lambda[2];
        lf[2] = lambda[0];
        flipped = 1;
    }
    sym3 am = A;
    am.x11 -= lf[0]; am.x22 -= lf[0]; am.x33 -= lf[0];
    vec3 v1 = sym3_largest_column_normalized(sym3_cofactor(am));
    vec3 v1o = v_normalized(orthogonal_vector(v1));
    vec3 ov0 = v1o, ov1 = v_cross(v1, v1o); /* other_v columns */
    /* Conjugate_With_Transpose(other_v, A): (A_full * other_v)^T other_v */
    double Af[3][3] = {{A.x11, A.x21, A.x31}, {A.x21, A.x22, A.x32}, {A.x31, A.x32, A.x33}};
    double C[3][2];
    for (int i = 0; i < 3; i++) {
        double acc0 = 0, acc1 = 0;
        for (int k = 0; k < 3; k++) acc0 += Af[i][k] * ov0.v[k];
        for (int k = 0; k < 3; k++) acc1 += Af[i][k] * ov1.v[k];
        C[i][0] = acc0; C[i][1] = acc1;
    }
    sym2 ar;
    ar.x11 = C[0][0] * ov0.v[0] + C[1][0] * ov0.v[1] + C[2][0] * ov0.v[2];
    ar.x21 = C[0][1] * ov0.v[0] + C[1][1] * ov0.v[1] + C[2][1] * ov0.v[2];
    ar.x22 = C[0][1] * ov1.v[0] + C[1][1] * ov1.v[1] + C[2][1] * ov1.v[2];
    ar.x11 -= lf[2];
    ar.x22 -= lf[2];
    double w[2];
    sym2_cofactor_largest_column_normalized(ar, w);
    vec3 v3v;
    for (int i = 0; i < 3; i++) {
        double acc = 0;
        acc += ov0.v[i] * w[0];
        acc += ov1.v[i] * w[1];
        v3v.v[i] = acc;
    }
    vec3 v2 = v_cross(v3v, v1);
    return flipped ? m_from_columns(v3v, v2, v_neg(v1)) : m_from_columns(v1, v2, v3v);
}

/* GFastSVD3x3 (PhysBAM.h:247-280) reduced to the U and V it returns, then
 * Compute_R_SVD's R = U * V^T (src/Saphyre2/ms/fem/Rotation.cpp:39-57). The
 * singular values do not enter R and are not formed. */
static mat3 rotation_msvd(const mat3* F)
{
    sym3 ne;
    const double (*f)[3] = F->m;
    ne.x11 = f[0][0] * f[0][0] + f[1][0] * f[1][0] + f[2][0] * f[2][0];
    ne.x21 = f[0][1] * f[0][0] + f[1][1] * f[1][0] + f[2][1] * f[2][0];
    ne.x31 = f[0][2] * f[0][0] + f[1][2] * f[1][0] + f[2][2] * f[2][0];
    ne.x22 = f[0][1] * f[0][1] + f[1][1] * f[1][1] + f[2][1] * f[2][1];
    ne.x32 = f[0][2] * f[0][1] + f[1][2] * f[1][1] + f[2][2] * f[2][1];
    ne.x33 = f[0][2] * f[0][2] + f[1][2] * f[1][2] + f[2][2] * f[2][2];
    double lambda[3];
    fast_eigenvalues(ne, lambda);
    mat3 V = fast_eigenvectors(ne, lambda);
    vec3 u0 = v_normalized(m_mulv(F, m_col(&V, 0)));
    vec3 o0 = v_normalized(orthogonal_vector(u0));
    vec3 o1 = v_cross(u0, o0);
    vec3 t = v_normalized(m_mulv(F, m_col(&V, 1)));
    double w[2];
    {
        double acc0 = 0, acc1 = 0;
        for (int k = 0; k < 3; k++) acc0 += o0.v[k] * t.v[k];
        for (int k = 0; k < 3; k++) acc1 += o1.v[k] * t.v[k];
        w[0] = acc0; w[1] = acc1;
    }
    vec3 u1;
    for (int i = 0; i < 3; i++) {
        double acc = 0;
        acc += o0.v[i] * w[0];
        acc += o1.v[i] * w[1];
        u1.v[i] = acc;
    }
    vec3 u2 = v_cross(u0, u1);
    mat3 U = m_from_columns(u0, u1, u2);
    mat3 Vt = m_transposed(&V);
    return m_mul(&U, &Vt);
}

/* Column 2 of V of GFastSVD3x3 (PhysBAM.h:247-272): the right singular
 * vector of the smallest singular value. */
static vec3 svd_smallest_right_vector(const mat3* F)
{
    sym3 ne;
    const double (*f)[3] = F->m;
    ne.x11 = f[0][0] * f[0][0] + f[1][0] * f[1][0] + f[2][0] * f[2][0];
    ne.x21 = f[0][1] * f[0][0] + f[1][1] * f[1][0] + f[2][1] * f[2][0];
    ne.x31 = f[0][2] * f[0][0] + f[1][2] * f[1][0] + f[2][2] * f[2][0];
    ne.x22 = f[0][1] * f[0][1] + f[1][1] * f[1][1] + f[2][1] * f[2][1];
    ne.x32 = f[0][2] * f[0][1] + f[1][2] * f[1][1] + f[2][2] * f[2][1];
    ne.x33 = f[0][2] * f[0][2] + f[1][2] * f[1][2] + f[2][2] * f[2][2];
    double lambda[3];
    fast_eigenvalues(ne, lambda);
    mat3 V = fast_eigenvectors(ne, lambda);
    return m_col(&V, 2);
}

static mat3 m_identity(void)
{
    mat3 I;
    memset(&I, 0, sizeof(I));
    I.m[0][0] = I.m[1][1] = I.m[2][2] = 1;
    return I;
}

/* ---- DAPD rotations (ms::fem::Params::eRM_DAPD) -------------------------- */

/* GRotation3x3_PolarDecomposition (Mal/GMatDecomposition.h:411-432): Newton
 * iterations H <- (H + H^-T) / 2 while |H1 - H0|_F^2 > 0.01f, at most 10. */
static mat3 polar_newton(const mat3* H)
{
    mat3 H0 = *H;
    double error;
    unsigned num_iter = 0;
    const double prec_sq = (double)0.01f;
    do {
        mat3 Ht = m_transposed(&H0);
        mat3 Hit = m_inverse(&Ht);
        mat3 H1;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) H1.m[i][j] = 0.5 * (H0.m[i][j] + Hit.m[i][j]);
        error = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double d = H1.m[i][j] - H0.m[i][j];
                error += d * d;
            }
        H0 = H1;
        num_iter++;
    } while (num_iter < 10 && error > prec_sq);
    return H0;
}

/* mal::IsZero with the default epsilon 0.0001f (Mal/RealUtils.h:110-114) */
static int is_zero(double x) { return fabs(x) <= (double)0.0001f; }

/* GSolvePolynomialEq1/Eq2 (Mal/GSolvePolynomialEq.h:11-40) */
static int solve_eq1(double a, double b, double* x)
{
    if (is_zero(a)) return 0;
    *x = -b / a;
    return 1;
}
static int solve_eq2(double a, double b, double c, double* x1, double* x2)
{
    if (is_zero(a)) {
        int n = solve_eq1(b, c, x1);
        *x2 = *x1;
        return n;
    }
    double disc = b * b - 4 * a * c;
    if (disc < 0) return 0;
    double root = mal_sqrt(disc);
    double inv_divisor = 1.0 / (2.0 * a);
    *x1 = (-b - root) * inv_divisor;
    *x2 = (-b + root) * inv_divisor;
    if (*x1 > *x2) { double t = *x1; *x1 = *x2; *x2 = t; }
    return (*x1 == *x2) ? 1 : 2;
}

int gsl_poly_solve_cubic(double a, double b, double c, double* x0, double* x1, double* x2);

/* mal::GSolvePolynomialEq3 as defined in TetrahedronElementSet3.cpp:49-70:
 * GSL's monic cubic solver for a != 0, else the quadratic. */
static int solve_eq3(double a, double b, double c, double d, double* x1, double* x2, double* x3)
{
    if (a != 0) return gsl_poly_solve_cubic(b / a, c / a, d / a, x1, x2, x3);
    *x3 = 0;
    return solve_eq2(b, c, d, x1, x2);
}

/* TetrahedronElement3::DoC (TetrahedronElement3.h:28-38): V-F when
 * vit0 == vit1, E-E when vit0 < vit1, invalid when vit0 > vit1. */
typedef struct { uint8_t vit0, vit1; } doc_t;
static const doc_t kDocInvalid = {3, 0};
static int doc_valid(doc_t d) { return d.vit0 <= d.vit1; }

/* ComputeDoC (TetrahedronElementSet3.cpp:589-743): the time of collapse t in
 * (0, 1] when det F along the straight path a -> b crosses the threshold
 * (a cubic in t), then the kind of collapse at that time: the face whose
 * unit-height prism volume along the collapse normal is half the total
 * (V-F, its opposite vertex), else the crossing edge pair (E-E). */
static doc_t compute_doc(vec3 a0, vec3 a1, vec3 a2, vec3 a3, vec3 b0, vec3 b1, vec3 b2, vec3 b3, double volume,
                         double thr)
{
    doc_t doc = kDocInvalid;
    vec3 d0 = v_sub(b0, a0), d1 = v_sub(b1, a1), d2 = v_sub(b2, a2), d3 = v_sub(b3, a3);
    vec3 d10 = v_sub(d1, d0), d20 = v_sub(d2, d0), d30 = v_sub(d3, d0);
    vec3 a10 = v_sub(a1, a0), a20 = v_sub(a2, a0), a30 = v_sub(a3, a0);
#define X(a_) ((a_).v[0])
#define Y(a_) ((a_).v[1])
#define Z(a_) ((a_).v[2])
    double K = thr * 6.0 * volume;
    double A = +X(d10) * Y(d20) * Z(d30) + X(d20) * Y(d30) * Z(d10) + X(d30) * Y(d10) * Z(d20)
               - X(d30) * Y(d20) * Z(d10) - X(d20) * Y(d10) * Z(d30) - X(d10) * Y(d30) * Z(d20);
    double B = +(X(a10) * Y(d20) * Z(d30) + X(d10) * Y(a20) * Z(d30) + X(d10) * Y(d20) * Z(a30))
               + (X(a20) * Y(d30) * Z(d10) + X(d20) * Y(a30) * Z(d10) + X(d20) * Y(d30) * Z(a10))
               + (X(a30) * Y(d10) * Z(d20) + X(d30) * Y(a10) * Z(d20) + X(d30) * Y(d10) * Z(a20))
               - (X(a30) * Y(d20) * Z(d10) + X(d30) * Y(a20) * Z(d10) + X(d30) * Y(d20) * Z(a10))
               - (X(a20) * Y(d10) * Z(d30) + X(d20) * Y(a10) * Z(d30) + X(d20) * Y(d10) * Z(a30))
               - (X(a10) * Y(d30) * Z(d20) + X(d10) * Y(a30) * Z(d20) + X(d10) * Y(d30) * Z(a20));
    double C = +(X(a10) * Y(a20) * Z(d30) + X(a10) * Y(d20) * Z(a30) + X(d10) * Y(a20) * Z(a30))
               + (X(a20) * Y(a30) * Z(d10) + X(a20) * Y(d30) * Z(a10) + X(d20) * Y(a30) * Z(a10))
               + (X(a30) * Y(a10) * Z(d20) + X(a30) * Y(d10) * Z(a20) + X(d30) * Y(a10) * Z(a20))
               - (X(a30) * Y(a20) * Z(d10) + X(a30) * Y(d20) * Z(a10) + X(d30) * Y(a20) * Z(a10))
               - (X(a20) * Y(a10) * Z(d30) + X(a20) * Y(d10) * Z(a30) + X(d20) * Y(a10) * Z(a30))
               - (X(a10) * Y(a30) * Z(d20) + X(a10) * Y(d30) * Z(a20) + X(d10) * Y(a30) * Z(a20));
    double D = +X(a10) * Y(a20) * Z(a30) + X(a20) * Y(a30) * Z(a10) + X(a30) * Y(a10) * Z(a20)
               - X(a30) * Y(a20) * Z(a10) - X(a20) * Y(a10) * Z(a30) - X(a10) * Y(a30) * Z(a20) - K;
#undef X
#undef Y
#undef Z
    double toc_r[3] = {0, 0, 0};
    int num_roots = solve_eq3(A, B, C, D, &toc_r[0], &toc_r[1], &toc_r[2]);
    if (num_roots <= 0) return doc;
    double toc = 2;
    int num_roots01 = 0;
    for (int i = 0; i < num_roots; i++)
        if (toc_r[i] > 0 && toc_r[i] <= 1 && toc_r[i] < toc) {
            toc = toc_r[i];
            num_roots01++;
        }
    if (num_roots01 != 1 && num_roots01 != 3) return doc;
    vec3 q0 = v_add(a0, v_scale(toc, d0)), q1 = v_add(a1, v_scale(toc, d1));
    vec3 q2 = v_add(a2, v_scale(toc, d2)), q3 = v_add(a3, v_scale(toc, d3));
    /* collapse normal: the right singular vector of the smallest singular
     * value (GSingularValueDecomposition_USVt = GFastSVD3x3, row 2 of V^T) */
    mat3 Q = m_from_columns(v_sub(q1, q0), v_sub(q2, q0), v_sub(q3, q0));
    vec3 N = svd_smallest_right_vector(&Q);
    double area[4];
    area[0] = fabs(v_dot(N, v_cross(v_sub(q2, q1), v_sub(q3, q1))));
    area[1] = fabs(v_dot(N, v_cross(v_sub(q2, q0), v_sub(q3, q0))));
    area[2] = fabs(v_dot(N, v_cross(v_sub(q1, q0), v_sub(q3, q0))));
    area[3] = fabs(v_dot(N, v_cross(v_sub(q1, q0), v_sub(q2, q0))));
    double sum_area = area[0] + area[1] + area[2] + area[3];
    for (int f = 0; f < 4; f++)
        if (fabs(area[f] - 0.5 * sum_area) <= (double)0.0001f) { doc.vit0 = (uint8_t)f; doc.vit1 = (uint8_t)f; }
    if (!doc_valid(doc)) {
        vec3 e1 = v_sub(q1, q0), e2 = v_sub(q2, q0), e3 = v_sub(q3, q0);
        if (v_dot(v_cross(e1, e2), v_cross(e1, e3)) < 0) { doc.vit0 = 0; doc.vit1 = 1; }
        else if (v_dot(v_cross(e2, e1), v_cross(e2, e3)) < 0) { doc.vit0 = 0; doc.vit1 = 2; }
        else if (v_dot(v_cross(e3, e1), v_cross(e3, e2)) < 0) { doc.vit0 = 0; doc.vit1 = 3; }
        else { doc.vit0 = 0; doc.vit1 = 0; }
    }
    return doc;
}

/* Compute_R_DAPD_Degenerate (Rotation.cpp:364-495): move the collapsing
 * vertex (V-F) or edge (E-E) along the collapse normal past the threshold by
 * the Hermite-spline / linear + power offset lambda_u, then the polar
 * rotation of the projected F. */
static mat3 dapd_degenerate(double detF, double thr, doc_t doc, vec3 p0, vec3 p1, vec3 p2, vec3 p3,
                            double volume, const mat3* inv_Dm, double fL, double fNL, double eNL)
{
    vec3 X[4] = {p0, p1, p2, p3};
    int i0, i1 = -1;
    vec3 axis;
    double w;
    if (doc.vit0 == doc.vit1) {
        int noc = doc.vit0;
        i0 = noc;
        vec3 x1 = X[(noc + 1) % 4], x2 = X[(noc + 2) % 4], x3 = X[(noc + 3) % 4];
        axis = v_cross(v_sub(x2, x1), v_sub(x3, x1));
        double len_sq = v_dot(axis, axis);
        if (!(len_sq > (double)0.000001f)) return m_identity();
        double len = mal_sqrt(len_sq);
        axis = v_div(axis, len);
        double dha = thr * 6 * volume / len;
        w = v_dot(v_sub(X[i0], x1), axis);
        if (w * detF < 0) { w = -w; axis = v_neg(axis); }
        double s_ = w / dha, t = 1.0 - s_;
        double lambda = (w > 0) ? fL * dha * ((2 - t) * t * t) : fL * dha * (t + fNL * pow(-s_, eNL));
        X[i0] = v_add(X[i0], v_scale(lambda, axis));
    } else {
        int v0 = doc.vit0, v1 = doc.vit1, v2, v3;
        switch (v1) {
        case 1: v2 = 2; v3 = 3; break;
        case 2: v2 = 1; v3 = 3; break;
        default: v2 = 1; v3 = 2; break;
        }
        i0 = v0;
        i1 = v1;
        axis = v_cross(v_sub(X[v1], X[v0]), v_sub(X[v3], X[v2]));
        double len_sq = v_dot(axis, axis);
        if (!(len_sq > (double)0.000001f)) return m_identity();
        double len = mal_sqrt(len_sq);
        axis = v_div(axis, len);
        double dha = thr * 6 * volume / len;
        w = v_dot(v_sub(X[v0], X[v2]), axis);
        if (w * detF < 0) { w = -w; axis = v_neg(axis); }
        double s_ = w / dha, t = 1.0 - s_;
        double lambda = (w > 0) ? fL * dha * ((2 - t) * t * t) : fL * dha * (t + fNL * pow(-s_, eNL));
        X[i0] = v_add(X[i0], v_scale(lambda, axis));
        X[i1] = v_add(X[i1], v_scale(lambda, axis));
    }
    mat3 projDs = m_from_columns(v_sub(X[1], X[0]), v_sub(X[2], X[0]), v_sub(X[3], X[0]));
    mat3 projF = m_mul(&projDs, inv_Dm);
    return polar_newton(&projF);
}

void orc_rotation_svd(const double* F_in, double* R_out, int math_mode)
{
    g_math = math_mode;
    mat3 F;
    memcpy(F.m, F_in, sizeof(F.m));
    mat3 R = rotation_msvd(&F);
    memcpy(R_out, R.m, sizeof(R.m));
}

/* ---- Element stiffness: TetrahedronElement3 (TetrahedronElement3.h:85-173) */

static mat3 compute_D(vec3 r0, vec3 r1, vec3 r2, vec3 r3)
{
    return m_from_columns(v_sub(r1, r0), v_sub(r2, r0), v_sub(r3, r0));
}

static double compute_volume(vec3 r0, vec3 r1, vec3 r2, vec3 r3)
{
    mat3 D = compute_D(r0, r1, r2, r3);
    return m_det(&D) / 6.0;
}

/* Compute_K = V * B^T (E B) with B from AFEM-16 (TetrahedronElement3.h:106-173);
 * K12 row-major 12x12. */
static double compute_K(vec3 r0, vec3 r1, vec3 r2, vec3 r3, double young, double poisson, double K[12][12])
{
    double volume = compute_volume(r0, r1, r2, r3);
    double x1 = r0.v[0], x2 = r1.v[0], x3 = r2.v[0], x4 = r3.v[0];
    double y1 = r0.v[1], y2 = r1.v[1], y3 = r2.v[1], y4 = r3.v[1];
    double z1 = r0.v[2], z2 = r1.v[2], z3 = r2.v[2], z4 = r3.v[2];
    double J[4][4];
    J[0][0] = x2 * (y3 * z4 - y4 * z3) + x3 * (y4 * z2 - y2 * z4) + x4 * (y2 * z3 - y3 * z2);
    J[1][0] = x1 * (y4 * z3 - y3 * z4) + x3 * (y1 * z4 - y4 * z1) + x4 * (y3 * z1 - y1 * z3);
    J[2][0] = x1 * (y2 * z4 - y4 * z2) + x2 * (y4 * z1 - y1 * z4) + x4 * (y1 * z2 - y2 * z1);
    J[3][0] = x1 * (y3 * z2 - y2 * z3) + x2 * (y1 * z3 - y3 * z1) + x3 * (y2 * z1 - y1 * z2);
    J[0][1] = (y4 - y2) * (z3 - z2) - (y3 - y2) * (z4 - z2); J[0][2] = (x3 - x2) * (z4 - z2) - (x4 - x2) * (z3 - z2); J[0][3] = (x4 - x2) * (y3 - y2) - (x3 - x2) * (y4 - y2);
    J[1][1] = (y3 - y1) * (z4 - z3) - (y3 - y4) * (z1 - z3); J[1][2] = (x4 - x3) * (z3 - z1) - (x1 - x3) * (z3 - z4); J[1][3] = (x3 - x1) * (y4 - y3) - (x3 - x4) * (y1 - y3);
    J[2][1] = (y2 - y4) * (z1 - z4) - (y1 - y4) * (z2 - z4); J[2][2] = (x1 - x4) * (z2 - z4) - (x2 - x4) * (z1 - z4); J[2][3] = (x2 - x4) * (y1 - y4) - (x1 - x4) * (y2 - y4);
    J[3][1] = (y1 - y3) * (z2 - z1) - (y1 - y2) * (z3 - z1); J[3][2] = (x2 - x1) * (z1 - z3) - (x3 - x1) * (z1 - z2); J[3][3] = (x1 - x3) * (y2 - y1) - (x1 - x2) * (y3 - y1);
    double s = 1.0 / (6.0 * volume);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) J[i][j] = s * J[i][j];
    double a[4], b[4], c[4];
    for (int i = 0; i < 4; i++) { a[i] = J[i][1]; b[i] = J[i][2]; c[i] = J[i][3]; }
    double B[6][12];
    memset(B, 0, sizeof(B));
    for (int n = 0; n < 4; n++) {
        B[0][3 * n] = a[n];
        B[1][3 * n + 1] = b[n];
        B[2][3 * n + 2] = c[n];
        B[3][3 * n] = b[n]; B[3][3 * n + 1] = a[n];
        B[4][3 * n + 1] = c[n]; B[4][3 * n + 2] = b[n];
        B[5][3 * n] = c[n]; B[5][3 * n + 2] = a[n];
    }
    double E[6][6];
    memset(E, 0, sizeof(E));
    double k = young / ((1.0 + poisson) * (1.0 - 2.0 * poisson));
    double k_nu = k * poisson, k1 = k * (1.0 - poisson), k2 = k * (0.5 - poisson);
    E[0][0] = k1; E[0][1] = k_nu; E[0][2] = k_nu;
    E[1][0] = k_nu; E[1][1] = k1; E[1][2] = k_nu;
    E[2][0] = k_nu; E[2][1] = k_nu; E[2][2] = k1;
    E[3][3] = k2; E[4][4] = k2; E[5][5] = k2;
    double EB[6][12];
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 12; j++) {
            double acc = 0;
            for (int kk = 0; kk < 6; kk++) acc += E[i][kk] * B[kk][j];
            EB[i][j] = acc;
        }
    for (int i = 0; i < 12; i++)
        for (int j = 0; j < 12; j++) {
            double acc = 0;
            for (int kk = 0; kk < 6; kk++) acc += B[kk][i] * EB[kk][j];
            K[i][j] = volume * acc;
        }
    return volume;
}

/* ---- Solid -------------------------------------------------------------- */

struct orc_solid {
    uint32_t N, T;
    int math;
    vec3* ref_pos;
    uint32_t* tets;       /* T*4 */
    double* volume;       /* T */
    mat3* inv_Dm;         /* T */
    mat3* K;              /* T*16, K[e*16 + 4*i + j] = K_ij */
    mat3* R;              /* T */
    double* detF;         /* T */
    vec3 *x, *prev_x, *v, *b, *y;
    double *r, *d, *q;    /* CG scratch, 3N */
    double inv_mass;      /* uniform */
    double total_volume;
    double density, dt, rel_eps, abs_eps;
    uint32_t max_iter;
    vec3 gravity;
    double rayleigh[2];
    double factor_M, factor_K;
    uint32_t n_knc;
    uint32_t* knc_nid;
    vec3 *knc_pos, *knc_vel;
    uint32_t last_iters;
    double last_rel, last_abs, elastic_energy, potential_energy;
    /* fully-implicit Euler (LeafDSH_Solid3D_FEM::Params, LeafDSH_Solid3D_FEM.h:110,233-241) */
    uint32_t integrator, nr_max_iter;
    double nr_abs_eps;
    vec3 *xk, *vk;        /* Newton iterates x_k, v_k (m_IE_vec_x_k, m_IE_vec_v_k) */
    uint32_t nr_iters;
    double nr_rel, nr_abs;
    /* rotation method (ms::fem::Params::m_RM) and the DAPD parameters
     * (m_DegenerateThresholdDetF, m_DAPD_L/NL_Factor, m_DAPD_NL_Exponent) */
    uint32_t rotation;
    double dapd_thr, dapd_L, dapd_NL, dapd_exp;
    doc_t* doc;           /* per-element direction of collapse (ElementCache3::m_DoC) */
    /* linear solver (LeafDSH_Solid3D_FEM::Params::m_SolverLS_Type) and the
     * MINRES work vectors v, v0, v1, w, w1, p, p0, p0_tmp (3N each) */
    uint32_t ls_solver;
    double* mr;
    /* material model (ms::fem::Params::m_MM): C_WRP or C_LCM; the set's Lame
     * parameters from the scalar E, nu (EndEdition, TetrahedronElementSet3.cpp:
     * 2116-2117) and each element's F of the last evaluation (ec.m_F) */
    uint32_t material;
    double lame_mu, lame_lambda;
    mat3* Fm;
    /* multi-solid Newton lock-step (NR_* phases): iterations since the last
     * NR_PreStep reset and LS iterations of the last NR_MidStep */
    uint32_t lock_nr_k, lock_ls_iters;
    /* ms::fem::Params::m_ECIE_k_factor (float32, default 1.0f): C_LCMH's
     * radius of its LCM/WRP blend (TetrahedronElementSet3.cpp:1895-1913) */
    double ecie_k;
    /* host threads of the element loops (orc_solid_set_threads); with more
     * than one, element products go to contrib[4e + i] and are applied node
     * by node in element order through the node -> (4e + i) list */
    int threads;
    uint32_t *node_ptr, *node_idx;
    vec3* contrib;
};

static vec3 load3(const double* p) { return v3(p[0], p[1], p[2]); }

orc_solid* orc_solid_create(uint32_t N, const double* rest, uint32_t T, const uint32_t* tets,
                            double E, double nu, const double* E_per, const double* nu_per,
                            double density, double damping_ratio, const double* gravity,
                            double dt, double rel_eps, double abs_eps, uint32_t max_iter,
                            int math_mode)
{
    if (N == 0 || T == 0) return NULL;
    orc_solid* s = (orc_solid*)calloc(1, sizeof(orc_solid));
    s->N = N; s->T = T; s->math = math_mode;
    s->ref_pos = (vec3*)malloc(sizeof(vec3) * N);
    s->tets = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)T);
    s->volume = (double*)malloc(sizeof(double) * T);
    s->inv_Dm = (mat3*)malloc(sizeof(mat3) * T);
    s->K = (mat3*)malloc(sizeof(mat3) * 16 * (size_t)T);
    s->R = (mat3*)malloc(sizeof(mat3) * T);
    s->detF = (double*)malloc(sizeof(double) * T);
    s->x = (vec3*)malloc(sizeof(vec3) * N);
    s->prev_x = (vec3*)malloc(sizeof(vec3) * N);
    s->v = (vec3*)calloc(N, sizeof(vec3));
    s->b = (vec3*)calloc(N, sizeof(vec3));
    s->y = (vec3*)calloc(N, sizeof(vec3));
    s->r = (double*)malloc(sizeof(double) * 3 * N);
    s->d = (double*)malloc(sizeof(double) * 3 * N);
    s->q = (double*)malloc(sizeof(double) * 3 * N);
    s->xk = (vec3*)calloc(N, sizeof(vec3));
    s->vk = (vec3*)calloc(N, sizeof(vec3));
    s->doc = (doc_t*)malloc(sizeof(doc_t) * T);
    for (uint32_t e = 0; e < T; e++) s->doc[e] = kDocInvalid;
    s->Fm = (mat3*)calloc(T, sizeof(mat3));
    s->material = FEM_ORC_MAT_C_WRP;
    s->ecie_k = (double)1.0f;
    /* LameParameters_From_YoungAndPoisson (TetrahedronElementSet3.cpp:181-186) */
    s->lame_mu = 0.5 * E / (1 + nu);
    s->lame_lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    s->rotation = FEM_ORC_ROT_MSVD;
    s->dapd_thr = (double)0.1f;
    s->dapd_L = 1;
    s->dapd_NL = 0;
    s->dapd_exp = 2;
    s->integrator = FEM_ORC_QIE_V;
    s->nr_max_iter = 3;
    s->nr_abs_eps = 1e-6;
    for (uint32_t i = 0; i < N; i++) s->ref_pos[i] = s->x[i] = s->prev_x[i] = load3(rest + 3 * i);
    memcpy(s->tets, tets, sizeof(uint32_t) * 4 * (size_t)T);
    /* EditableTetrahedronElementSet3::EndEdition (TetrahedronElementSet3.cpp:2113-2166) */
    double acc_total_volume = 0;
    for (uint32_t e = 0; e < T; e++) {
        const uint32_t* t = tets + 4 * (size_t)e;
        vec3 r0 = s->ref_pos[t[0]], r1 = s->ref_pos[t[1]], r2 = s->ref_pos[t[2]], r3 = s->ref_pos[t[3]];
        s->volume[e] = compute_volume(r0, r1, r2, r3);
        acc_total_volume += s->volume[e];
        double K[12][12];
        double Ee = E_per ? E_per[e] : E, nue = nu_per ? nu_per[e] : nu;
        compute_K(r0, r1, r2, r3, Ee, nue, K);
        for (int bi = 0; bi < 4; bi++)
            for (int bj = 0; bj < 4; bj++)
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) s->K[16 * (size_t)e + 4 * bi + bj].m[i][j] = K[3 * bi + i][3 * bj + j];
        mat3 Dm = compute_D(r0, r1, r2, r3);
        s->inv_Dm[e] = m_inverse(&Dm);
        /* CreateCache: R = I, detF = 1 (TetrahedronElementSet3.cpp:190-209) */
        memset(&s->R[e], 0, sizeof(mat3));
        s->R[e].m[0][0] = s->R[e].m[1][1] = s->R[e].m[2][2] = 1;
        s->detF[e] = 1;
    }
    s->total_volume = acc_total_volume;
    s->density = density; s->dt = dt; s->rel_eps = rel_eps; s->abs_eps = abs_eps;
    s->max_iter = max_iter;
    s->gravity = load3(gravity);
    /* RebuildMass: m = rho * sum(V) / N, stored as its reciprocal
     * (LeafDSH_Solid3D_FEM.cpp:1591-1611, ParticleSystem.h:80) */
    double total_mass = density * s->total_volume;
    double mass_per_node = total_mass / N;
    s->inv_mass = (double)1.0f / mass_per_node;
    /* RebuildRayleighCoeffsFromFreqs (LeafDSH_Solid3D_FEM.h:347-354) with
     * the default frequencies 0.1f and 10000.0f (Params.h:79) */
    {
        double f1 = (double)0.1f, f2 = (double)10000.0f;
        double o00 = 1.0 / f1, o01 = f1, o10 = 1.0 / f2, o11 = f2;
        double det = o00 * o11 - o10 * o01;
        double inv_det = 1.0 / det;
        double i00 = inv_det * o11, i01 = -inv_det * o01, i10 = -inv_det * o10, i11 = inv_det * o00;
        double z0 = 2 * damping_ratio, z1 = 2 * damping_ratio;
        double acc0 = 0, acc1 = 0;
        acc0 += i00 * z0; acc0 += i01 * z1;
        acc1 += i10 * z0; acc1 += i11 * z1;
        s->rayleigh[0] = acc0;
        s->rayleigh[1] = acc1;
    }
    return s;
}

void orc_solid_destroy(orc_solid* s)
{
    if (!s) return;
    free(s->ref_pos); free(s->tets); free(s->volume); free(s->inv_Dm); free(s->K); free(s->R);
    free(s->detF); free(s->x); free(s->prev_x); free(s->v); free(s->b); free(s->y);
    free(s->r); free(s->d); free(s->q); free(s->xk); free(s->vk); free(s->doc); free(s->mr); free(s->Fm);
    free(s->knc_nid); free(s->knc_pos); free(s->knc_vel);
    free(s->node_ptr); free(s->node_idx); free(s->contrib);
    free(s);
}

void orc_solid_set_threads(orc_solid* s, int threads)
{
    s->threads = threads > 1 ? threads : 1;
    if (s->threads > 1 && !s->contrib) {
        /* node -> (4e + i) entries in element order (the serial scatter's order) */
        const size_t n4 = 4 * (size_t)s->T;
        s->node_ptr = (uint32_t*)calloc((size_t)s->N + 1, sizeof(uint32_t));
        s->node_idx = (uint32_t*)malloc(sizeof(uint32_t) * n4);
        s->contrib = (vec3*)malloc(sizeof(vec3) * n4);
        for (size_t j = 0; j < n4; j++) s->node_ptr[s->tets[j] + 1]++;
        for (uint32_t n = 0; n < s->N; n++) s->node_ptr[n + 1] += s->node_ptr[n];
        uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)s->N + 1));
        memcpy(fill, s->node_ptr, sizeof(uint32_t) * ((size_t)s->N + 1));
        for (size_t j = 0; j < n4; j++) s->node_idx[fill[s->tets[j]]++] = (uint32_t)j;
        free(fill);
    }
}

double orc_solid_total_volume(const orc_solid* s) { return s->total_volume; }
double orc_solid_node_mass(const orc_solid* s) { return 1.0 / s->inv_mass; }
void orc_solid_rayleigh(const orc_solid* s, double* out2) { out2[0] = s->rayleigh[0]; out2[1] = s->rayleigh[1]; }

void orc_solid_element_K(const orc_solid* s, uint32_t e, double* K144)
{
    memcpy(K144, &s->K[16 * (size_t)e], sizeof(mat3) * 16);
}

void orc_solid_set_solver(orc_solid* s, double rel_eps, double abs_eps, uint32_t max_iter)
{
    s->rel_eps = rel_eps;
    s->abs_eps = abs_eps;
    s->max_iter = max_iter;
}

void orc_solid_set_knc(orc_solid* s, uint32_t count, const uint32_t* nodes, const double* targets)
{
    free(s->knc_nid); free(s->knc_pos); free(s->knc_vel);
    s->n_knc = count;
    s->knc_nid = (uint32_t*)malloc(sizeof(uint32_t) * (count ? count : 1));
    s->knc_pos = (vec3*)malloc(sizeof(vec3) * (count ? count : 1));
    s->knc_vel = (vec3*)calloc(count ? count : 1, sizeof(vec3));
    for (uint32_t k = 0; k < count; k++) {
        s->knc_nid[k] = nodes[k];
        s->knc_pos[k] = load3(targets + 3 * k);
    }
}

void orc_solid_set_knc_targets(orc_solid* s, const double* targets)
{
    for (uint32_t k = 0; k < s->n_knc; k++) s->knc_pos[k] = load3(targets + 3 * k);
}

void orc_solid_set_state(orc_solid* s, const double* x, const double* v)
{
    for (uint32_t i = 0; i < s->N; i++) {
        if (x) { s->x[i] = load3(x + 3 * i); s->prev_x[i] = s->x[i]; }
        if (v) s->v[i] = load3(v + 3 * i);
    }
}

void orc_solid_get_state(const orc_solid* s, double* x, double* v)
{
    for (uint32_t i = 0; i < s->N; i++)
        for (int c = 0; c < 3; c++) {
            if (x) x[3 * i + c] = s->x[i].v[c];
            if (v) v[3 * i + c] = s->v[i].v[c];
        }
}

/* BeginEvaluation for C_WRP + MSVD (TetrahedronElementSet3.cpp:219-281,777-792):
 * Ds, F = Ds * Dm^-1, det F, R. The degeneration bookkeeping (DoC) does not
 * feed this path and is not formed. */
typedef void (*orc_range_fn)(void* ctx, uint32_t lo, uint32_t hi);
static void parallel_for(int threads, uint32_t n, orc_range_fn fn, void* ctx);

typedef struct {
    orc_solid* s;
    const vec3 *xprev, *x;
} eval_ctx;

/* BeginEvaluation for elements [lo, hi) (each element's work is its own) */
static void begin_eval_range(void* p, uint32_t lo, uint32_t hi)
{
    const eval_ctx* c = (const eval_ctx*)p;
    orc_solid* s = c->s;
    const vec3 *xprev = c->xprev, *x = c->x;
    for (uint32_t e = lo; e < hi; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        mat3 Ds = compute_D(x[t[0]], x[t[1]], x[t[2]], x[t[3]]);
        mat3 F = m_mul(&Ds, &s->inv_Dm[e]);
        double detF = m_det(&F);
        s->detF[e] = detF;
        s->Fm[e] = F;
        if (s->rotation == FEM_ORC_ROT_MSVD) {
            s->R[e] = rotation_msvd(&F);
            continue;
        }
        /* UpdateDegeneration (TetrahedronElementSet3.cpp:477-533) */
        const double thr = s->dapd_thr;
        if (detF > thr) {
            s->doc[e] = kDocInvalid;
        } else {
            mat3 prevDs = compute_D(xprev[t[0]], xprev[t[1]], xprev[t[2]], xprev[t[3]]);
            mat3 prevF = m_mul(&prevDs, &s->inv_Dm[e]);
            if (m_det(&prevF) > thr)
                s->doc[e] = compute_doc(xprev[t[0]], xprev[t[1]], xprev[t[2]], xprev[t[3]], x[t[0]], x[t[1]],
                                        x[t[2]], x[t[3]], s->volume[e], thr);
        }
        /* ComputeRotations_DAPD (TetrahedronElementSet3.cpp:860-892) */
        if (detF > thr)
            s->R[e] = polar_newton(&F);
        else if (doc_valid(s->doc[e]))
            s->R[e] = dapd_degenerate(detF, thr, s->doc[e], x[t[0]], x[t[1]], x[t[2]], x[t[3]], s->volume[e],
                                      &s->inv_Dm[e], s->dapd_L, s->dapd_NL, s->dapd_exp);
        else
            s->R[e] = m_identity();
    }
}

static void begin_evaluation_at(orc_solid* s, const vec3* xprev, const vec3* x)
{
    eval_ctx c = {s, xprev, x};
    parallel_for(s->threads, s->T, begin_eval_range, &c);
}

/* BeginEvaluation(m_vecPos0, x): the previous positions feed the DAPD
 * collapse detection only. */
static void begin_evaluation(orc_solid* s) { begin_evaluation_at(s, s->prev_x, s->x); }

/* ---- C_LCM material (linear corotational, first Piola-Kirchhoff form) ---- */

static double m_trace(const mat3* a)
{
    double t = 0;
    for (int i = 0; i < 3; i++) t += a->m[i][i];
    return t;
}
static mat3 m_scale(double k, const mat3* a)
{
    mat3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = k * a->m[i][j];
    return r;
}
static mat3 m_add(const mat3* a, const mat3* b)
{
    mat3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = a->m[i][j] + b->m[i][j];
    return r;
}

/* -V P Dm^-T scattered as h0 = -h1-h2-h3, h1..h3 = columns (the force
 * accumulation of C_LCM_f_e / C_LCM_df_x) */
static void pk_scatter(const orc_solid* s, uint32_t e, const mat3* P, vec3* f)
{
    const uint32_t* t = s->tets + 4 * (size_t)e;
    mat3 mVP = m_scale(-s->volume[e], P);
    mat3 DmT = m_transposed(&s->inv_Dm[e]);
    mat3 H = m_mul(&mVP, &DmT);
    vec3 c0 = m_col(&H, 0), c1 = m_col(&H, 1), c2 = m_col(&H, 2);
    f[t[0]] = v_add(f[t[0]], v_sub(v_sub(v_neg(c0), c1), c2));
    f[t[1]] = v_add(f[t[1]], c0);
    f[t[2]] = v_add(f[t[2]], c1);
    f[t[3]] = v_add(f[t[3]], c2);
}

/* C_LCM_f_e (TetrahedronElementSet3.cpp:1154-1178):
 * P = R (2 mu (S - I) + lambda tr(S - I) I), S = R^T F */
static void lcm_f_e_acc(const orc_solid* s, vec3* f)
{
    const mat3 I = m_identity();
    for (uint32_t e = 0; e < s->T; e++) {
        mat3 Rt = m_transposed(&s->R[e]);
        mat3 S = m_mul(&Rt, &s->Fm[e]);
        mat3 SmI;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) SmI.m[i][j] = S.m[i][j] - I.m[i][j];
        mat3 A = m_scale(2 * s->lame_mu, &SmI);
        mat3 B = m_scale(s->lame_lambda * m_trace(&SmI), &I);
        mat3 AB = m_add(&A, &B);
        mat3 P = m_mul(&s->R[e], &AB);
        pk_scatter(s, e, &P, f);
    }
}

/* C_LCM_df_x with truncated differentials (TetrahedronElementSet3.cpp:
 * 1838-1873; Compute_dR_From_RM gives no dR term under eDM_Truncated):
 * dP = 2 mu dF + lambda tr(R^T dF) R, dF = dDs Dm^-1 */
static void lcm_df_x_acc(const orc_solid* s, const vec3* dx, vec3* df)
{
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        mat3 Rt = m_transposed(&s->R[e]);
        mat3 dDs = compute_D(dx[t[0]], dx[t[1]], dx[t[2]], dx[t[3]]);
        mat3 dF = m_mul(&dDs, &s->inv_Dm[e]);
        mat3 A = m_scale(2 * s->lame_mu, &dF);
        mat3 RtdF = m_mul(&Rt, &dF);
        mat3 B = m_scale(s->lame_lambda * m_trace(&RtdF), &s->R[e]);
        mat3 dP = m_add(&A, &B);
        pk_scatter(s, e, &dP, df);
    }
}

/* C_LCM_V (TetrahedronElementSet3.cpp:1489-1507) */
static double lcm_V(const orc_solid* s)
{
    const mat3 I = m_identity();
    double acc_V = 0;
    for (uint32_t e = 0; e < s->T; e++) {
        mat3 Rt = m_transposed(&s->R[e]);
        mat3 S = m_mul(&Rt, &s->Fm[e]);
        mat3 SmI;
        double nsq = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                SmI.m[i][j] = S.m[i][j] - I.m[i][j];
                nsq += SmI.m[i][j] * SmI.m[i][j];
            }
        double tr = m_trace(&SmI);
        acc_V += s->volume[e] * (s->lame_mu * nsq + 0.5 * s->lame_lambda * (tr * tr));
    }
    return acc_V;
}

static mat3 m_sub(const mat3* a, const mat3* b)
{
    mat3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = a->m[i][j] - b->m[i][j];
    return r;
}

/* Adjugate 3x3 (GMat.h:316-329) */
static mat3 m_adjugate(const mat3* a)
{
    const double (*m)[3] = a->m;
    mat3 r;
    r.m[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
    r.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]);
    r.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
    r.m[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]);
    r.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]);
    r.m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]);
    r.m[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    r.m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]);
    r.m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]);
    return r;
}

/* Inverse 3x3 with a given determinant (GMat.h:291-313) */
static mat3 m_inverse_det(const mat3* a, double determinant)
{
    const double (*m)[3] = a->m;
    double inv_det = 1.0 / determinant; /* mal::Rcp */
    mat3 r;
    r.m[0][0] = inv_det * (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
    r.m[0][1] = inv_det * (m[0][2] * m[2][1] - m[0][1] * m[2][2]);
    r.m[0][2] = inv_det * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
    r.m[1][0] = inv_det * (m[1][2] * m[2][0] - m[1][0] * m[2][2]);
    r.m[1][1] = inv_det * (m[0][0] * m[2][2] - m[0][2] * m[2][0]);
    r.m[1][2] = inv_det * (m[0][2] * m[1][0] - m[0][0] * m[1][2]);
    r.m[2][0] = inv_det * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    r.m[2][1] = inv_det * (m[0][1] * m[2][0] - m[0][0] * m[2][1]);
    r.m[2][2] = inv_det * (m[0][0] * m[1][1] - m[0][1] * m[1][0]);
    return r;
}

/* C_LCMH_df_x with truncated differentials (TetrahedronElementSet3.cpp:
 * 1875-1930): for m_ECIE_k_factor k > 0.1 the hybrid of LCM and WRP,
 *   w = Clamp01(Rcp(k) tr|S - I| / 3),
 *   dP = 2 mu (w dF + (1 - w) R sym(R^T dF)) + lambda tr(R^T dF) R;
 * otherwise C_LCM's dP (the WRP branch for k > 10 is unreachable: k > 0.1
 * is tested first). f_e and V are C_LCM's (:303-400). */
static void lcmh_df_x_acc(const orc_solid* s, const vec3* dx, vec3* df)
{
    const mat3 I = m_identity();
    const double k = s->ecie_k;
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        mat3 Rt = m_transposed(&s->R[e]);
        mat3 S = m_mul(&Rt, &s->Fm[e]);
        mat3 dDs = compute_D(dx[t[0]], dx[t[1]], dx[t[2]], dx[t[3]]);
        mat3 dF = m_mul(&dDs, &s->inv_Dm[e]);
        mat3 RtdF = m_mul(&Rt, &dF);
        mat3 dP;
        if ((float)k > 0.1) {
            const double cDimension = 3, cRadiusWRP = k;
            mat3 SmI = m_sub(&S, &I);
            mat3 A;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) A.m[i][j] = fabs(SmI.m[i][j]);
            double w = (1.0 / cRadiusWRP) * m_trace(&A) / cDimension;
            w = (w < 1.0) ? w : 1.0; /* mal::Clamp01 = Max(0, Min(w, 1)) */
            w = (0.0 > w) ? 0.0 : w;
            mat3 RtdFt = m_transposed(&RtdF);
            mat3 sum = m_add(&RtdF, &RtdFt);
            mat3 sym = m_scale(0.5, &sum);
            mat3 wdF = m_scale(w, &dF);
            mat3 oR = m_scale(1 - w, &s->R[e]);
            mat3 oRsym = m_mul(&oR, &sym);
            mat3 inner = m_add(&wdF, &oRsym);
            mat3 T1 = m_scale(2 * s->lame_mu, &inner);
            mat3 T2 = m_scale(s->lame_lambda * m_trace(&RtdF), &s->R[e]);
            dP = m_add(&T1, &T2);
        } else {
            mat3 A = m_scale(2 * s->lame_mu, &dF);
            mat3 B = m_scale(s->lame_lambda * m_trace(&RtdF), &s->R[e]);
            dP = m_add(&A, &B);
        }
        pk_scatter(s, e, &dP, df);
    }
}

/* C_CCM_f_e (TetrahedronElementSet3.cpp:1180-1206):
 * S = R^T F, P = R (2 mu (S - I) + lambda (det S - 1) adj(S)^T) */
static void ccm_f_e_acc(const orc_solid* s, vec3* f)
{
    const mat3 I = m_identity();
    for (uint32_t e = 0; e < s->T; e++) {
        mat3 Rt = m_transposed(&s->R[e]);
        mat3 S = m_mul(&Rt, &s->Fm[e]);
        double det_S = m_det(&S);
        mat3 SmI = m_sub(&S, &I);
        mat3 A = m_scale(2 * s->lame_mu, &SmI);
        mat3 adj = m_adjugate(&S);
        mat3 adjT = m_transposed(&adj);
        mat3 B = m_scale(s->lame_lambda * (det_S - 1), &adjT);
        mat3 AB = m_add(&A, &B);
        mat3 P = m_mul(&s->R[e], &AB);
        pk_scatter(s, e, &P, f);
    }
}

/* C_CCM_df_x with truncated differentials (TetrahedronElementSet3.cpp:
 * 1932-1970), with the reference's dDs built from nodes (0, 1, 2, 2) -- its
 * fourth argument repeats node 2 (:1948) -- and F^-1 regularised at det F = 0
 * by det F + Sign(det F) 1e-6f:
 *   dP = 2 mu dF + lambda ((2 J^2 - J) tr(F^-1 dF) F^-T
 *                          - (J^2 - J) F^-T dF^T F^-T),  J = det F */
static void ccm_df_x_acc(const orc_solid* s, const vec3* dx, vec3* df)
{
    const double reg = (double)1e-6f; /* REGULARIZE_CCM_PD_U_THRESHOLD (:35) */
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        mat3 dDs = compute_D(dx[t[0]], dx[t[1]], dx[t[2]], dx[t[2]]);
        mat3 dF = m_mul(&dDs, &s->inv_Dm[e]);
        mat3 dP = m_scale(2 * s->lame_mu, &dF);
        const double J = s->detF[e];
        const double sign = (J >= 0.0) ? 1.0 : -1.0; /* mal::Sign */
        mat3 invF = m_inverse_det(&s->Fm[e], J + sign * reg);
        mat3 invFt = m_transposed(&invF);
        mat3 invFdF = m_mul(&invF, &dF);
        mat3 X = m_scale((2 * (J * J) - J) * m_trace(&invFdF), &invFt);
        mat3 c2invFt = m_scale((J * J) - J, &invFt);
        mat3 dFt = m_transposed(&dF);
        mat3 Y1 = m_mul(&c2invFt, &dFt);
        mat3 Y = m_mul(&Y1, &invFt);
        mat3 XY = m_sub(&X, &Y);
        mat3 W = m_scale(s->lame_lambda, &XY);
        dP = m_add(&dP, &W);
        pk_scatter(s, e, &dP, df);
    }
}

/* ---- element loops over host threads ------------------------------------
 * Test infrastructure speed only: the oracle's serial scatter
 * f[t[i]] -= c_{e,i} runs element after element. With threads, each
 * element's four terms c_{e,i} are formed in parallel (they are independent)
 * and stored, then every node subtracts its terms in element order -- the
 * same operations in the same order per node, so results are bit-identical
 * to the serial loop for any thread count. */
typedef struct {
    orc_range_fn fn;
    void* ctx;
    uint32_t lo, hi;
    int math;
} orc_task;

static void* orc_task_run(void* p)
{
    orc_task* t = (orc_task*)p;
    g_math = t->math;
    t->fn(t->ctx, t->lo, t->hi);
    return NULL;
}

static void parallel_for(int threads, uint32_t n, orc_range_fn fn, void* ctx)
{
    enum { kMaxThreads = 64 };
    if (threads > kMaxThreads) threads = kMaxThreads;
    if (threads <= 1 || n < 1024) {
        fn(ctx, 0, n);
        return;
    }
    pthread_t th[kMaxThreads];
    orc_task task[kMaxThreads];
    int started[kMaxThreads];
    const uint32_t chunk = (n + (uint32_t)threads - 1) / (uint32_t)threads;
    for (int k = 0; k < threads; k++) {
        const uint32_t lo = (uint32_t)k * chunk;
        const uint32_t hi = lo + chunk < n ? lo + chunk : n;
        task[k].fn = fn;
        task[k].ctx = ctx;
        task[k].lo = lo < n ? lo : n;
        task[k].hi = hi;
        task[k].math = g_math;
        started[k] = 0;
        if (k > 0 && task[k].lo < task[k].hi)
            started[k] = pthread_create(&th[k], NULL, orc_task_run, &task[k]) == 0;
    }
    fn(ctx, task[0].lo, task[0].hi);
    for (int k = 1; k < threads; k++) {
        if (started[k])
            pthread_join(th[k], NULL);
        else if (task[k].lo < task[k].hi)
            fn(ctx, task[k].lo, task[k].hi);
    }
}

typedef struct {
    const orc_solid* s;
    const vec3* in;   /* x (with ref: f_e) or dx (df_x) */
    int with_ref;     /* 1: u = R^T x - r (C_f_e); 0: l = R^T dx (C_df_x) */
    vec3* out;
} wrp_ctx;

/* c_{e,i} = R sum_j K_ij (R^T in_j [- r_j]) for elements [lo, hi) */
static void wrp_terms_range(void* p, uint32_t lo, uint32_t hi)
{
    const wrp_ctx* c = (const wrp_ctx*)p;
    const orc_solid* s = c->s;
    for (uint32_t e = lo; e < hi; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        const mat3* K = &s->K[16 * (size_t)e];
        mat3 Rt = m_transposed(&s->R[e]);
        vec3 u[4];
        for (int i = 0; i < 4; i++) {
            u[i] = m_mulv(&Rt, c->in[t[i]]);
            if (c->with_ref) u[i] = v_sub(u[i], s->ref_pos[t[i]]);
        }
        for (int i = 0; i < 4; i++) {
            vec3 acc = v_add(v_add(v_add(m_mulv(&K[4 * i], u[0]), m_mulv(&K[4 * i + 1], u[1])),
                                   m_mulv(&K[4 * i + 2], u[2])), m_mulv(&K[4 * i + 3], u[3]));
            s->contrib[4 * (size_t)e + i] = m_mulv(&s->R[e], acc);
        }
    }
}

/* out[n] -= c_{e,i} over n's entries in element order, nodes [lo, hi) */
static void node_subtract_range(void* p, uint32_t lo, uint32_t hi)
{
    const wrp_ctx* c = (const wrp_ctx*)p;
    const orc_solid* s = c->s;
    for (uint32_t n = lo; n < hi; n++) {
        vec3 a = c->out[n];
        for (uint32_t j = s->node_ptr[n]; j < s->node_ptr[n + 1]; j++) a = v_sub(a, s->contrib[s->node_idx[j]]);
        c->out[n] = a;
    }
}

static void wrp_scatter_threaded(const orc_solid* s, const vec3* in, int with_ref, vec3* out)
{
    wrp_ctx c = {s, in, with_ref, out};
    parallel_for(s->threads, s->T, wrp_terms_range, &c);
    parallel_for(s->threads, s->N, node_subtract_range, &c);
}

/* C_f_e (TetrahedronElementSet3.cpp:1053-1096): f_i -= R sum_j K_ij (R^T x_j - r_j) */
static void f_e_acc(const orc_solid* s, const vec3* x, vec3* f)
{
    /* f_e dispatch (TetrahedronElementSet3.cpp:303-322): C_LCMH uses C_LCM's */
    if (s->material == FEM_ORC_MAT_C_LCM || s->material == FEM_ORC_MAT_C_LCMH) {
        lcm_f_e_acc(s, f);
        return;
    }
    if (s->material == FEM_ORC_MAT_C_CCM) {
        ccm_f_e_acc(s, f);
        return;
    }
    if (s->threads > 1) {
        wrp_scatter_threaded(s, x, 1, f);
        return;
    }
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        const mat3* K = &s->K[16 * (size_t)e];
        mat3 Rt = m_transposed(&s->R[e]);
        vec3 u[4];
        for (int i = 0; i < 4; i++) u[i] = v_sub(m_mulv(&Rt, x[t[i]]), s->ref_pos[t[i]]);
        for (int i = 0; i < 4; i++) {
            vec3 acc = v_add(v_add(v_add(m_mulv(&K[4 * i], u[0]), m_mulv(&K[4 * i + 1], u[1])),
                                   m_mulv(&K[4 * i + 2], u[2])), m_mulv(&K[4 * i + 3], u[3]));
            f[t[i]] = v_sub(f[t[i]], m_mulv(&s->R[e], acc));
        }
    }
}

/* C_df_x with truncated differentials (TetrahedronElementSet3.cpp:1761-1836):
 * df_i -= R sum_j K_ij R^T dx_j */
static void df_x_acc(const orc_solid* s, const vec3* dx, vec3* df)
{
    /* df_x dispatch (TetrahedronElementSet3.cpp:355-377) */
    if (s->material == FEM_ORC_MAT_C_LCM) {
        lcm_df_x_acc(s, dx, df);
        return;
    }
    if (s->material == FEM_ORC_MAT_C_LCMH) {
        lcmh_df_x_acc(s, dx, df);
        return;
    }
    if (s->material == FEM_ORC_MAT_C_CCM) {
        ccm_df_x_acc(s, dx, df);
        return;
    }
    if (s->threads > 1) {
        wrp_scatter_threaded(s, dx, 0, df);
        return;
    }
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        const mat3* K = &s->K[16 * (size_t)e];
        mat3 Rt = m_transposed(&s->R[e]);
        vec3 l[4];
        for (int i = 0; i < 4; i++) l[i] = m_mulv(&Rt, dx[t[i]]);
        for (int i = 0; i < 4; i++) {
            vec3 acc = v_add(v_add(v_add(m_mulv(&K[4 * i], l[0]), m_mulv(&K[4 * i + 1], l[1])),
                                   m_mulv(&K[4 * i + 2], l[2])), m_mulv(&K[4 * i + 3], l[3]));
            df[t[i]] = v_sub(df[t[i]], m_mulv(&s->R[e], acc));
        }
    }
}

/* C_V (TetrahedronElementSet3.cpp:1456-1488) */
static double elastic_V(const orc_solid* s)
{
    /* V dispatch (TetrahedronElementSet3.cpp:382-400): C_LCMH uses C_LCM_V;
     * C_CCM_V's body is compiled out (__TO_PORT_TO_3D) and returns 0 (:1509-1545) */
    if (s->material == FEM_ORC_MAT_C_LCM || s->material == FEM_ORC_MAT_C_LCMH) return lcm_V(s);
    if (s->material == FEM_ORC_MAT_C_CCM) return 0.0;
    double acc_twice_V = 0;
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        const mat3* K = &s->K[16 * (size_t)e];
        mat3 Rt = m_transposed(&s->R[e]);
        vec3 u[4];
        for (int i = 0; i < 4; i++) u[i] = v_sub(m_mulv(&Rt, s->x[t[i]]), s->ref_pos[t[i]]);
        for (int i = 0; i < 4; i++) {
            vec3 acc = v_add(v_add(v_add(m_mulv(&K[4 * i], u[0]), m_mulv(&K[4 * i + 1], u[1])),
                                   m_mulv(&K[4 * i + 2], u[2])), m_mulv(&K[4 * i + 3], u[3]));
            acc_twice_V += v_dot(u[i], acc);
        }
    }
    return 0.5 * acc_twice_V;
}

/* RecomputeEnergy, potential part (LeafDSH_Solid3D_FEM.cpp:1554-1584) */
static double potential_energy(const orc_solid* s)
{
    double pe = 0;
    for (uint32_t e = 0; e < s->T; e++) {
        const uint32_t* t = s->tets + 4 * (size_t)e;
        double element_mass = s->density * s->volume[e];
        vec3 sum = v_add(v_add(v_add(s->x[t[0]], s->x[t[1]]), s->x[t[2]]), s->x[t[3]]);
        pe += (element_mass / 4.0) * v_dot(sum, v_neg(s->gravity));
    }
    return pe;
}

/* LS_ZeroKNC (LeafDSH_Solid3D_FEM.cpp:1045-1053) */
static void zero_knc(const orc_solid* s, double* v)
{
    for (uint32_t k = 0; k < s->n_knc; k++) {
        uint32_t n = s->knc_nid[k];
        v[3 * n] = 0; v[3 * n + 1] = 0; v[3 * n + 2] = 0;
    }
}

/* LS_A_times_d (LeafDSH_Solid3D_FEM.cpp:1056-1079) */
static void a_times_d(const orc_solid* s, double factor_M, double factor_K, const double* d, double* q)
{
    const uint32_t n3 = 3 * s->N;
    memset(q, 0, sizeof(double) * n3);
    df_x_acc(s, (const vec3*)d, (vec3*)q);
    for (uint32_t i = 0; i < n3; i++) q[i] *= -factor_K;
    double mass = 1.0 / s->inv_mass;
    for (uint32_t i = 0; i < s->N; i++) {
        double factor = mass * factor_M;
        q[3 * i] += factor * d[3 * i];
        q[3 * i + 1] += factor * d[3 * i + 1];
        q[3 * i + 2] += factor * d[3 * i + 2];
    }
}

/* ILSS_CG::Solve (src/Saphyre2/ns/ILSS_CG.h:38-151) with the scalar
 * real_array kernels (src/Saphyre2/ns/real_array.h:91-113). */
static void cg_solve(orc_solid* s, double* x, const double* b)
{
    const uint32_t n = 3 * s->N;
    double *r = s->r, *d = s->d, *q = s->q;
    double abs_epsilon_sq = s->abs_eps * s->abs_eps;
    a_times_d(s, s->factor_M, s->factor_K, x, r);
    for (uint32_t i = 0; i < n; i++) r[i] = -1 * r[i] + b[i];
    zero_knc(s, r);
    memcpy(d, r, sizeof(double) * n);
    double delta_0 = 0;
    for (uint32_t i = 0; i < n; i++) delta_0 += r[i] * r[i];
    double delta_new = delta_0, delta_old = delta_0;
    uint32_t k = 0;
    double delta_target = (s->rel_eps * s->rel_eps) * delta_0;
    while (delta_new > abs_epsilon_sq && delta_new > delta_target && k < s->max_iter) {
        a_times_d(s, s->factor_M, s->factor_K, d, q);
        zero_knc(s, q);
        double dot_d_q = 0;
        for (uint32_t i = 0; i < n; i++) dot_d_q += d[i] * q[i];
        if (fabs(dot_d_q) < abs_epsilon_sq) break;
        double alpha = delta_new / dot_d_q;
        for (uint32_t i = 0; i < n; i++) x[i] += alpha * d[i];
        double neg_alpha = -alpha;
        for (uint32_t i = 0; i < n; i++) r[i] += neg_alpha * q[i];
        delta_old = delta_new;
        delta_new = 0;
        for (uint32_t i = 0; i < n; i++) delta_new += r[i] * r[i];
        double beta = delta_new / delta_old;
        for (uint32_t i = 0; i < n; i++) d[i] = beta * d[i] + r[i];
        zero_knc(s, d);
        k++;
    }
    s->last_iters = k;
    s->last_rel = (delta_0 > 0) ? mal_sqrt(delta_new / delta_0) : 0;
    s->last_abs = mal_sqrt(delta_new);
}

static void ls_solve(orc_solid* s, double* x, const double* b);

/* real_array::norm_2 (src/Saphyre2/ns/real_array.h:97-98) */
static double norm_2(const double* v, uint32_t n)
{
    double res = 0;
    for (uint32_t i = 0; i < n; i++) res += v[i] * v[i];
    return mal_sqrt(res);
}

/* Step_FullyImplicitEuler_dx (LeafDSH_Solid3D_FEM.cpp:1357-1552) with h = dt,
 * or h = 0 for the quasi-static variant (FixedStep, :958-959). The Newton
 * iterates live in xk/vk; the model's x, v stay x^n, v^n until the end. No
 * contacts, CGS or the commented-out f_d; f_p is empty in the reference
 * (TetrahedronElementSet3.cpp:350-353). Warm start on (the Params default). */
static void step_fie(orc_solid* s, double h)
{
    const uint32_t N = s->N;
    const double inv_dt = (h == 0) ? 0 : 1.0 / h;
    const double mass = 1.0 / s->inv_mass;
    for (uint32_t i = 0; i < N; i++) { s->xk[i] = s->x[i]; s->vk[i] = s->v[i]; }
    uint32_t nr_k = 0, ls_iters = 0;
    double nr_delta_new = 0, nr_delta_0 = -1;
    int converged1 = 0;
    s->last_iters = 0;
    s->last_rel = s->last_abs = 0;
    do {
        for (uint32_t i = 0; i < N; i++) s->b[i] = v3(0, 0, 0);
        for (uint32_t i = 0; i < N; i++) s->b[i] = v_add(s->b[i], v_scale(mass, s->gravity));
        f_e_acc(s, s->xk, s->b);
        for (uint32_t i = 0; i < N; i++)
            s->b[i] = v_add(s->b[i], v_scale(inv_dt * mass, v_sub(s->v[i], v_scale(inv_dt, v_sub(s->xk[i], s->x[i])))));
        if (nr_k == 0) for (uint32_t i = 0; i < N; i++) s->y[i] = v_scale(h, s->v[i]);
        else memset(s->y, 0, sizeof(vec3) * N);
        for (uint32_t k = 0; k < s->n_knc; k++) {
            uint32_t nid = s->knc_nid[k];
            /* the KNC velocity bookkeeping (:1448-1456) does not feed this integrator */
            vec3 vk = v_scale(inv_dt, v_sub(s->knc_pos[k], s->x[nid]));
            double norm_vk = v_norm(vk);
            if (norm_vk > (double)0.001f) {
                double clamp = (norm_vk < 50.0) ? norm_vk : 50.0;
                s->knc_vel[k] = v_scale(clamp, v_normalized(vk));
            } else {
                s->knc_vel[k] = v3(0, 0, 0);
            }
            s->b[nid] = v_sub(s->knc_pos[k], s->xk[nid]);
            s->y[nid] = v_sub(s->knc_pos[k], s->xk[nid]);
        }
        nr_delta_new = norm_2((const double*)s->b, 3 * N);
        if (nr_delta_0 < 0) nr_delta_0 = nr_delta_new;
        converged1 = nr_delta_new < s->nr_abs_eps;
        if (!converged1) {
            s->factor_M = inv_dt * inv_dt + inv_dt * s->rayleigh[0];
            s->factor_K = 1.0 + inv_dt * s->rayleigh[1];
            ls_solve(s, (double*)s->y, (const double*)s->b);
            ls_iters += s->last_iters;
            for (uint32_t i = 0; i < N; i++) s->xk[i] = v_add(s->xk[i], s->y[i]);
            for (uint32_t i = 0; i < N; i++) s->vk[i] = v_scale(inv_dt, v_sub(s->xk[i], s->x[i]));
            nr_delta_new = norm_2((const double*)s->y, 3 * N);
            nr_k++;
            begin_evaluation_at(s, s->x, s->xk);
        }
    } while (!converged1 && nr_k < s->nr_max_iter);
    s->nr_iters = nr_k;
    s->nr_rel = (nr_delta_0 > 0) ? nr_delta_new / nr_delta_0 : 0;
    s->nr_abs = nr_delta_new;
    s->last_iters = ls_iters;
    for (uint32_t i = 0; i < N; i++) { s->x[i] = s->xk[i]; s->v[i] = s->vk[i]; }
}

/* ---- multi-solid Newton lock-step (LeafDSH_Solid3D_FEM.cpp:2824-3039) ----
 * The phases SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update
 * (SS_AggregateDSH_Basic.cpp:229-300) interleaves over its solids. x, v stay
 * at x^n, v^n until NR_End; x_k, v_k are the iterates. NR_PreStep resets
 * x_k = x^n, v_k = v^n and the iteration count at every NR iteration, so
 * each iteration solves the first Newton system again with the element
 * forces and rotations of the previous iterate's BeginEvaluation (the
 * cache's positions are the x_k array, which then holds x^n again). */

/* NR_Init (:2824-2845): UpdateKNC (a no-op in the default kinematic mode),
 * BeginEvaluation(m_vecPos0, x), m_vecPos0 = x */
void orc_solid_nr_init(orc_solid* s, double dt)
{
    (void)dt;
    g_math = s->math;
    begin_evaluation(s);
    for (uint32_t i = 0; i < s->N; i++) s->prev_x[i] = s->x[i];
}

/* NR_PreStep (:2870-2890) */
void orc_solid_nr_prestep(orc_solid* s, double dt)
{
    (void)dt;
    for (uint32_t i = 0; i < s->N; i++) {
        s->xk[i] = s->x[i];
        s->vk[i] = s->v[i];
    }
    s->lock_nr_k = 0;
    s->lock_ls_iters = 0;
}

/* NR_MidStep (:2892-2990): b = m g + f_e + (1/h) m (v - (1/h)(x_k - x)),
 * warm start y = h v on the first iteration after a reset (always, since
 * NR_PreStep resets the count), position constraints as b = y = target -
 * x_k (the KNC velocity bookkeeping does not feed this integrator), then
 * the linear solve with factor_M = 1/h^2 + a0/h, factor_K = 1 + a1/h. */
void orc_solid_nr_midstep(orc_solid* s, double dt)
{
    g_math = s->math;
    const uint32_t N = s->N;
    const double inv_dt = (dt == 0) ? 0 : 1.0 / dt;
    const double mass = 1.0 / s->inv_mass;
    for (uint32_t i = 0; i < N; i++) s->b[i] = v3(0, 0, 0);
    for (uint32_t i = 0; i < N; i++) s->b[i] = v_add(s->b[i], v_scale(mass, s->gravity));
    f_e_acc(s, s->xk, s->b);
    for (uint32_t i = 0; i < N; i++)
        s->b[i] = v_add(s->b[i], v_scale(inv_dt * mass, v_sub(s->v[i], v_scale(inv_dt, v_sub(s->xk[i], s->x[i])))));
    if (s->lock_nr_k == 0) for (uint32_t i = 0; i < N; i++) s->y[i] = v_scale(dt, s->v[i]);
    else memset(s->y, 0, sizeof(vec3) * N);
    for (uint32_t k = 0; k < s->n_knc; k++) {
        uint32_t nid = s->knc_nid[k];
        vec3 vk = v_scale(inv_dt, v_sub(s->knc_pos[k], s->x[nid]));
        double norm_vk = v_norm(vk);
        if (norm_vk > (double)0.001f) {
            double clamp = (norm_vk < 50.0) ? norm_vk : 50.0;
            s->knc_vel[k] = v_scale(clamp, v_normalized(vk));
        } else {
            s->knc_vel[k] = v3(0, 0, 0);
        }
        s->b[nid] = v_sub(s->knc_pos[k], s->xk[nid]);
        s->y[nid] = v_sub(s->knc_pos[k], s->xk[nid]);
    }
    s->factor_M = inv_dt * inv_dt + inv_dt * s->rayleigh[0];
    s->factor_K = 1.0 + inv_dt * s->rayleigh[1];
    ls_solve(s, (double*)s->y, (const double*)s->b);
    s->lock_ls_iters += s->last_iters;
}

/* NR_PostStep (:2992-3020): x_k += y, v_k = (x_k - x)/h, BeginEvaluation(x, x_k) */
void orc_solid_nr_poststep(orc_solid* s, double dt)
{
    g_math = s->math;
    const double inv_dt = (dt == 0) ? 0 : 1.0 / dt;
    for (uint32_t i = 0; i < s->N; i++) s->xk[i] = v_add(s->xk[i], s->y[i]);
    for (uint32_t i = 0; i < s->N; i++) s->vk[i] = v_scale(inv_dt, v_sub(s->xk[i], s->x[i]));
    s->lock_nr_k++;
    begin_evaluation_at(s, s->x, s->xk);
}

/* NR_End (:2847-2868): x = x_k, v = v_k, RecomputeEnergy's potential term
 * (no air drag by default); NR_End evaluates no V, so the elastic energy
 * keeps its value */
void orc_solid_nr_end(orc_solid* s, double dt)
{
    (void)dt;
    g_math = s->math;
    for (uint32_t i = 0; i < s->N; i++) {
        s->x[i] = s->xk[i];
        s->v[i] = s->vk[i];
    }
    s->potential_energy = potential_energy(s);
}

/* SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update's body for one fixed step
 * (its contact calls left out): NR_Init for all; the largest nr_max_iter of
 * the solids NR iterations of (NR_PreStep, NR_MidStep for all; NR_PostStep
 * for all); NR_End for all -- every phase with the same dt. */
void orc_multi_lock_step(orc_solid** solids, uint32_t count, double dt)
{
    uint32_t max_nr_iter = 0;
    for (uint32_t i = 0; i < count; i++)
        max_nr_iter = solids[i]->nr_max_iter > max_nr_iter ? solids[i]->nr_max_iter : max_nr_iter;
    for (uint32_t i = 0; i < count; i++) orc_solid_nr_init(solids[i], dt);
    uint32_t nr_iter = 0;
    do {
        for (uint32_t i = 0; i < count; i++) {
            orc_solid_nr_prestep(solids[i], dt);
            orc_solid_nr_midstep(solids[i], dt);
        }
        for (uint32_t i = 0; i < count; i++) orc_solid_nr_poststep(solids[i], dt);
    } while (++nr_iter < max_nr_iter);
    for (uint32_t i = 0; i < count; i++) orc_solid_nr_end(solids[i], dt);
}

void orc_solid_last_lock_stats(const orc_solid* s, uint32_t* nr_k, uint32_t* ls_iters)
{
    *nr_k = s->lock_nr_k;
    *ls_iters = s->lock_ls_iters;
}

/* ILSS_MINRES::Solve (src/Saphyre2/ns/ILSS_MINRES.h:51-168): Paige-Saunders
 * MINRES without a preconditioner, the scalar real_array kernels
 * (src/Saphyre2/ns/real_array.h:91-113), the residual norm carried by the
 * Givens sines, stopping on |r|^2 <= abs^2, |r|^2 <= rel^2 |b|^2 or the
 * iteration cap. */
static void minres_solve(orc_solid* s, double* x, const double* b)
{
    const uint32_t n = 3 * s->N;
    double *v = s->mr, *v0 = v + n, *v1 = v0 + n, *w = v1 + n, *w1 = w + n, *p = w1 + n, *p0 = p + n,
           *p0_tmp = p0 + n;
    const double fM = s->factor_M, fK = s->factor_K;
    double abs_epsilon_sq = s->abs_eps * s->abs_eps;
    memset(v, 0, sizeof(double) * n);
    a_times_d(s, fM, fK, x, v1);
    for (uint32_t i = 0; i < n; i++) v1[i] = -1 * v1[i] + b[i];
    zero_knc(s, v1);
    double norm_r_sq = 0;
    for (uint32_t i = 0; i < n; i++) norm_r_sq += v1[i] * v1[i];
    memcpy(w1, v1, sizeof(double) * n);
    double beta_new_sq = 0;
    for (uint32_t i = 0; i < n; i++) beta_new_sq += v1[i] * w1[i];
    double beta_new = mal_sqrt(beta_new_sq);
    double beta_one = beta_new;
    {
        double inv = 1.0 / beta_new;
        for (uint32_t i = 0; i < n; i++) v1[i] *= inv;
        for (uint32_t i = 0; i < n; i++) w1[i] *= inv;
    }
    double c = 1.0, c_old = 1.0, sn = 0.0, sn_old = 0.0;
    memset(p0, 0, sizeof(double) * n);
    memset(p, 0, sizeof(double) * n);
    double eta = 1.0;
    uint32_t k = 0;
    double norm_b_sq = 0;
    for (uint32_t i = 0; i < n; i++) norm_b_sq += b[i] * b[i];
    double delta_target = (s->rel_eps * s->rel_eps) * norm_b_sq;
    while (norm_r_sq > abs_epsilon_sq && norm_r_sq > delta_target && k < s->max_iter) {
        double beta = beta_new;
        memcpy(v0, v, sizeof(double) * n);
        memcpy(v, v1, sizeof(double) * n);
        memcpy(w, w1, sizeof(double) * n);
        a_times_d(s, fM, fK, w, v1);
        zero_knc(s, v1);
        for (uint32_t i = 0; i < n; i++) v1[i] += -beta * v0[i];
        double alpha = 0;
        for (uint32_t i = 0; i < n; i++) alpha += v1[i] * w[i];
        for (uint32_t i = 0; i < n; i++) v1[i] += -alpha * v[i];
        memcpy(w1, v1, sizeof(double) * n);
        beta_new_sq = 0;
        for (uint32_t i = 0; i < n; i++) beta_new_sq += v1[i] * w1[i];
        beta_new = mal_sqrt(beta_new_sq);
        {
            double inv = 1.0 / beta_new;
            for (uint32_t i = 0; i < n; i++) v1[i] *= inv;
            for (uint32_t i = 0; i < n; i++) w1[i] *= inv;
        }
        const double r2 = sn * alpha + c * c_old * beta;
        const double r3 = sn_old * beta;
        const double r1_hat = c * alpha - c_old * sn * beta;
        const double r1 = mal_sqrt(r1_hat * r1_hat + beta_new_sq);
        c_old = c;
        sn_old = sn;
        c = r1_hat / r1;
        sn = beta_new / r1;
        memcpy(p0_tmp, p0, sizeof(double) * n);
        memcpy(p0, p, sizeof(double) * n);
        for (uint32_t i = 0; i < n; i++) p[i] = -r2 * p[i] + w[i];
        for (uint32_t i = 0; i < n; i++) p[i] += -r3 * p0_tmp[i];
        {
            double inv = 1.0 / r1;
            for (uint32_t i = 0; i < n; i++) p[i] *= inv;
        }
        {
            double coef = beta_one * c * eta;
            for (uint32_t i = 0; i < n; i++) x[i] += coef * p[i];
        }
        norm_r_sq *= sn * sn;
        eta = -sn * eta;
        k++;
    }
    s->last_iters = k;
    s->last_rel = mal_sqrt(norm_r_sq / norm_b_sq);
    s->last_abs = mal_sqrt(norm_r_sq);
}

/* LS_Solve's solver choice (LeafDSH_Solid3D_FEM.cpp:1136-1154) */
static void ls_solve(orc_solid* s, double* x, const double* b)
{
    if (s->ls_solver == FEM_ORC_LS_MINRES) minres_solve(s, x, b);
    else cg_solve(s, x, b);
}

/* FixedStep (LeafDSH_Solid3D_FEM.cpp:898-990) with
 * Step_QuasiImplicitEuler_v (LeafDSH_Solid3D_FEM.cpp:1205-1328) or
 * Step_FullyImplicitEuler_dx (:1357-1552). */
void orc_solid_fixed_step(orc_solid* s)
{
    g_math = s->math;
    const uint32_t N = s->N;
    const double dt = s->dt;
    begin_evaluation(s);
    for (uint32_t i = 0; i < N; i++) s->prev_x[i] = s->x[i];
    if (s->integrator != FEM_ORC_QIE_V) {
        step_fie(s, s->integrator == FEM_ORC_FIE_DX_QUASISTATIC ? 0.0 : dt);
        s->elastic_energy = elastic_V(s);
        s->potential_energy = potential_energy(s);
        return;
    }
    double inv_dt = 1.0 / dt;
    double mass = 1.0 / s->inv_mass;
    for (uint32_t i = 0; i < N; i++) s->b[i] = v3(0, 0, 0);
    for (uint32_t i = 0; i < N; i++) s->b[i] = v_add(s->b[i], v_scale(mass, s->gravity));
    f_e_acc(s, s->x, s->b);
    for (uint32_t i = 0; i < N; i++) s->b[i] = v_scale(dt, s->b[i]);
    for (uint32_t i = 0; i < N; i++) s->b[i] = v_add(s->b[i], v_scale(mass, s->v[i]));
    for (uint32_t i = 0; i < N; i++) s->y[i] = s->v[i];
    for (uint32_t k = 0; k < s->n_knc; k++) {
        uint32_t nid = s->knc_nid[k];
        vec3 vk = v_scale(inv_dt, v_sub(s->knc_pos[k], s->x[nid]));
        double norm_vk = v_norm(vk);
        if (norm_vk > (double)0.001f) {
            double clamp = (norm_vk < 50.0) ? norm_vk : 50.0;
            s->knc_vel[k] = v_scale(clamp, v_normalized(vk));
        } else {
            s->knc_vel[k] = v3(0, 0, 0);
        }
        s->b[nid] = s->knc_vel[k];
        s->y[nid] = s->knc_vel[k];
    }
    s->factor_M = 1.0 + dt * s->rayleigh[0];
    s->factor_K = dt * dt + dt * s->rayleigh[1];
    ls_solve(s, (double*)s->y, (const double*)s->b);
    for (uint32_t i = 0; i < N; i++) {
        s->v[i] = s->y[i];
        s->x[i] = v_add(s->x[i], v_scale(dt, s->y[i]));
    }
    s->elastic_energy = elastic_V(s);
    s->potential_energy = potential_energy(s);
}

void orc_solid_set_rotation(orc_solid* s, uint32_t method, double thr, double factor_L, double factor_NL,
                            double exponent_NL)
{
    s->rotation = method;
    s->dapd_thr = thr;
    /* float32 fields in the reference (Params.h:29) */
    s->dapd_L = (double)(float)factor_L;
    s->dapd_NL = (double)(float)factor_NL;
    s->dapd_exp = (double)(float)exponent_NL;
    for (uint32_t e = 0; e < s->T; e++) s->doc[e] = kDocInvalid;
}

void orc_solid_doc(const orc_solid* s, uint8_t* doc2)
{
    for (uint32_t e = 0; e < s->T; e++) {
        doc2[2 * (size_t)e] = s->doc[e].vit0;
        doc2[2 * (size_t)e + 1] = s->doc[e].vit1;
    }
}

void orc_solid_set_material(orc_solid* s, uint32_t material) { s->material = material; }
void orc_solid_set_ecie_k_factor(orc_solid* s, double k) { s->ecie_k = (double)(float)k; }

void orc_solid_set_ls_solver(orc_solid* s, uint32_t ls_solver)
{
    s->ls_solver = ls_solver;
    if (ls_solver == FEM_ORC_LS_MINRES && !s->mr) s->mr = (double*)malloc(sizeof(double) * 8 * 3 * (size_t)s->N);
}

void orc_solid_set_integrator(orc_solid* s, uint32_t integrator, uint32_t nr_max_iter, double nr_abs_eps)
{
    s->integrator = integrator;
    s->nr_max_iter = nr_max_iter;
    s->nr_abs_eps = nr_abs_eps;
}

void orc_solid_last_nr_stats(const orc_solid* s, uint32_t* nr_iters, double* nr_rel, double* nr_abs)
{
    if (nr_iters) *nr_iters = s->integrator == FEM_ORC_QIE_V ? 0 : s->nr_iters;
    if (nr_rel) *nr_rel = s->integrator == FEM_ORC_QIE_V ? 0 : s->nr_rel;
    if (nr_abs) *nr_abs = s->integrator == FEM_ORC_QIE_V ? 0 : s->nr_abs;
}

void orc_solid_last_stats(const orc_solid* s, uint32_t* iters, double* rel_res, double* abs_res,
                          double* elastic_energy, double* potential_energy)
{
    if (iters) *iters = s->last_iters;
    if (rel_res) *rel_res = s->last_rel;
    if (abs_res) *abs_res = s->last_abs;
    if (elastic_energy) *elastic_energy = s->elastic_energy;
    if (potential_energy) *potential_energy = s->potential_energy;
}

void orc_solid_begin_eval(orc_solid* s, const double* x)
{
    g_math = s->math;
    for (uint32_t i = 0; i < s->N; i++) s->x[i] = load3(x + 3 * i);
    begin_evaluation(s);
}

void orc_solid_rotations(const orc_solid* s, double* R_out)
{
    for (uint32_t e = 0; e < s->T; e++) memcpy(R_out + 9 * (size_t)e, s->R[e].m, sizeof(mat3));
}

void orc_solid_detF(const orc_solid* s, double* detF_out)
{
    memcpy(detF_out, s->detF, sizeof(double) * s->T);
}

void orc_solid_f_e(const orc_solid* s, double* f)
{
    f_e_acc(s, s->x, (vec3*)f);
}

void orc_solid_df_x(const orc_solid* s, const double* dx, double* df)
{
    df_x_acc(s, (const vec3*)dx, (vec3*)df);
}

double orc_solid_V(const orc_solid* s) { return elastic_V(s); }

void orc_solid_apply_A(const orc_solid* s, double factor_M, double factor_K, const double* d, double* q)
{
    a_times_d(s, factor_M, factor_K, d, q);
    zero_knc(s, q);
}
