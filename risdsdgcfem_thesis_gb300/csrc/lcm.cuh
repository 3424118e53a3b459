// lcm.cuh -- the first Piola-Kirchhoff materials of the reference's element
// set (ms::fem::Params::eMM_C_LCM, eMM_C_LCMH, eMM_C_CCM), per element, FP64,
// with Mal's rounding order (products accumulated from zero, Trace from zero,
// scalar * matrix element by element):
//
//   C_LCM_f_e   TetrahedronElementSet3.cpp:1154-1178
//     S = R^T F, P = R (2 mu (S - I) + lambda tr(S - I) I)
//   C_LCM_df_x  TetrahedronElementSet3.cpp:1838-1873 (truncated: no dR term)
//     dF = dDs Dm^-1, dP = 2 mu dF + lambda tr(R^T dF) R
//   C_LCM_V     TetrahedronElementSet3.cpp:1489-1507
//     V (mu |S - I|_F^2 + 0.5 lambda tr(S - I)^2)
//   C_LCMH_df_x TetrahedronElementSet3.cpp:1875-1930 (f_e, V: C_LCM's)
//     for m_ECIE_k_factor k > 0.1: w = Clamp01(tr|S - I| / (3 k)),
//     dP = 2 mu (w dF + (1 - w) R sym(R^T dF)) + lambda tr(R^T dF) R
//   C_CCM_f_e   TetrahedronElementSet3.cpp:1180-1206
//     P = R (2 mu (S - I) + lambda (det S - 1) adj(S)^T)
//   C_CCM_df_x  TetrahedronElementSet3.cpp:1932-1970, dDs from nodes
//     (0, 1, 2, 2) as the reference builds it (:1948), J = det F,
//     F^-1 with determinant J + Sign(J) 1e-6f:
//     dP = 2 mu dF + lambda ((2 J^2 - J) tr(F^-1 dF) F^-T - (J^2 - J) F^-T dF^T F^-T)
//   C_CCM_V     0 (its body is compiled out, :1509-1545)
//   with H = -V P Dm^-T and nodal forces (-h1-h2-h3, h1, h2, h3), h_j the
//   columns of H.
//
// Outputs follow the element products' convention of the solid's kernels:
// out[3 i + a] is MINUS node i's force contribution (the gathers subtract).
// Host-callable as well, so that the arithmetic can be checked on the CPU.
// Matrices are row-major double[9].
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define FEM_HD __host__ __device__ __forceinline__
#else
#define FEM_HD inline
#endif

namespace femgb {

FEM_HD void lcm_matmul(const double* a, const double* b, double* r)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double acc = 0.0;
            acc += a[3 * i + 0] * b[0 * 3 + j];
            acc += a[3 * i + 1] * b[1 * 3 + j];
            acc += a[3 * i + 2] * b[2 * 3 + j];
            r[3 * i + j] = acc;
        }
}

FEM_HD double lcm_trace(const double* a)
{
    double t = 0.0;
    t += a[0];
    t += a[4];
    t += a[8];
    return t;
}

// H = (-V P) Dm^-T ; out = -(node forces)
FEM_HD void lcm_pk_out(double V, const double* P, const double* Dinv, double* out)
{
    double mVP[9], DmT[9], H[9];
    const double mV = -V;
    for (int c = 0; c < 9; c++) mVP[c] = mV * P[c];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) DmT[3 * i + j] = Dinv[3 * j + i];
    lcm_matmul(mVP, DmT, H);
    for (int a = 0; a < 3; a++) {
        const double c0 = H[3 * a + 0], c1 = H[3 * a + 1], c2 = H[3 * a + 2];
        const double h0 = ((-c0) - c1) - c2;
        out[a] = -h0;
        out[3 + a] = -c0;
        out[6 + a] = -c1;
        out[9 + a] = -c2;
    }
}

// S - I with S = R^T F
FEM_HD void lcm_s_minus_i(const double* R, const double* F, double* SmI)
{
    double Rt[9], S[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Rt[3 * i + j] = R[3 * j + i];
    lcm_matmul(Rt, F, S);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) SmI[3 * i + j] = S[3 * i + j] - (i == j ? 1.0 : 0.0);
}

FEM_HD void lcm_force(const double* R, const double* F, const double* Dinv, double V, double mu, double lambda,
                      double* out)
{
    double SmI[9], AB[9], P[9];
    lcm_s_minus_i(R, F, SmI);
    const double two_mu = 2 * mu;
    const double lt = lambda * lcm_trace(SmI);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) AB[3 * i + j] = two_mu * SmI[3 * i + j] + lt * (i == j ? 1.0 : 0.0);
    lcm_matmul(R, AB, P);
    lcm_pk_out(V, P, Dinv, out);
}

// dl: the element's 4 nodal displacements (12 values, node-major)
FEM_HD void lcm_dforce(const double* R, const double* Dinv, double V, double mu, double lambda, const double* dl,
                       double* out)
{
    double dDs[9], dF[9], Rt[9], RtdF[9], dP[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) dDs[3 * i + j] = dl[3 * (j + 1) + i] - dl[i];
    lcm_matmul(dDs, Dinv, dF);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Rt[3 * i + j] = R[3 * j + i];
    lcm_matmul(Rt, dF, RtdF);
    const double two_mu = 2 * mu;
    const double lt = lambda * lcm_trace(RtdF);
    for (int c = 0; c < 9; c++) dP[c] = two_mu * dF[c] + lt * R[c];
    lcm_pk_out(V, dP, Dinv, out);
}

FEM_HD void lcm_transpose(const double* a, double* r)
{
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r[3 * i + j] = a[3 * j + i];
}

// Det and Adjugate 3x3 in Mal's term order (GMat.h:236-245, 316-329)
FEM_HD double lcm_det(const double* m)
{
    return m[0] * m[4] * m[8] - m[0] * m[7] * m[5] + m[3] * m[7] * m[2] - m[3] * m[1] * m[8] + m[6] * m[1] * m[5] -
           m[6] * m[4] * m[2];
}

FEM_HD void lcm_adjugate(const double* m, double* r)
{
    r[0] = (m[4] * m[8] - m[5] * m[7]);
    r[1] = (m[2] * m[7] - m[1] * m[8]);
    r[2] = (m[1] * m[5] - m[2] * m[4]);
    r[3] = (m[5] * m[6] - m[3] * m[8]);
    r[4] = (m[0] * m[8] - m[2] * m[6]);
    r[5] = (m[2] * m[3] - m[0] * m[5]);
    r[6] = (m[3] * m[7] - m[4] * m[6]);
    r[7] = (m[1] * m[6] - m[0] * m[7]);
    r[8] = (m[0] * m[4] - m[1] * m[3]);
}

// C_LCMH_df_x: the LCM/WRP blend of radius k (m_ECIE_k_factor)
FEM_HD void lcmh_dforce(const double* R, const double* F, const double* Dinv, double V, double mu, double lambda,
                        double k, const double* dl, double* out)
{
    double dDs[9], dF[9], Rt[9], RtdF[9], dP[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) dDs[3 * i + j] = dl[3 * (j + 1) + i] - dl[i];
    lcm_matmul(dDs, Dinv, dF);
    lcm_transpose(R, Rt);
    lcm_matmul(Rt, dF, RtdF);
    const double two_mu = 2 * mu;
    const double lt = lambda * lcm_trace(RtdF);
    if ((float)k > 0.1) {
        double S[9];
        lcm_matmul(Rt, F, S);
        double tr = 0.0;
        tr += fabs(S[0] - 1.0);
        tr += fabs(S[4] - 1.0);
        tr += fabs(S[8] - 1.0);
        double w = (1.0 / k) * tr / 3.0;
        w = (w < 1.0) ? w : 1.0;  // mal::Clamp01 = Max(0, Min(w, 1))
        w = (0.0 > w) ? 0.0 : w;
        double sym[9], oR[9], oRsym[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) sym[3 * i + j] = 0.5 * (RtdF[3 * i + j] + RtdF[3 * j + i]);
        const double one_w = 1 - w;
        for (int c = 0; c < 9; c++) oR[c] = one_w * R[c];
        lcm_matmul(oR, sym, oRsym);
        for (int c = 0; c < 9; c++) dP[c] = two_mu * (w * dF[c] + oRsym[c]) + lt * R[c];
    } else {
        for (int c = 0; c < 9; c++) dP[c] = two_mu * dF[c] + lt * R[c];
    }
    lcm_pk_out(V, dP, Dinv, out);
}

// C_CCM_f_e
FEM_HD void ccm_force(const double* R, const double* F, const double* Dinv, double V, double mu, double lambda,
                      double* out)
{
    double Rt[9], S[9], adj[9], AB[9], P[9];
    lcm_transpose(R, Rt);
    lcm_matmul(Rt, F, S);
    const double det_S = lcm_det(S);
    lcm_adjugate(S, adj);
    const double two_mu = 2 * mu;
    const double c = lambda * (det_S - 1);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            AB[3 * i + j] = two_mu * (S[3 * i + j] - (i == j ? 1.0 : 0.0)) + c * adj[3 * j + i];
    lcm_matmul(R, AB, P);
    lcm_pk_out(V, P, Dinv, out);
}

// C_CCM_df_x (dDs from nodes 0, 1, 2, 2, as the reference)
FEM_HD void ccm_dforce(const double* F, double J, const double* Dinv, double V, double mu, double lambda,
                       const double* dl, double* out)
{
    double dDs[9], dF[9], invF[9], invFt[9], invFdF[9], dFt[9], Y1[9], Y[9], c2i[9], dP[9];
    for (int i = 0; i < 3; i++) {
        dDs[3 * i + 0] = dl[3 + i] - dl[i];
        dDs[3 * i + 1] = dl[6 + i] - dl[i];
        dDs[3 * i + 2] = dl[6 + i] - dl[i];
    }
    lcm_matmul(dDs, Dinv, dF);
    const double reg = (double)1e-6f;            // REGULARIZE_CCM_PD_U_THRESHOLD
    const double sign = (J >= 0.0) ? 1.0 : -1.0;  // mal::Sign
    const double inv_det = 1.0 / (J + sign * reg);
    lcm_adjugate(F, invF);
    for (int c = 0; c < 9; c++) invF[c] = inv_det * invF[c];
    lcm_transpose(invF, invFt);
    lcm_matmul(invF, dF, invFdF);
    const double cx = (2 * (J * J) - J) * lcm_trace(invFdF);
    const double c2 = (J * J) - J;
    for (int c = 0; c < 9; c++) c2i[c] = c2 * invFt[c];
    lcm_transpose(dF, dFt);
    lcm_matmul(c2i, dFt, Y1);
    lcm_matmul(Y1, invFt, Y);
    const double two_mu = 2 * mu;
    for (int c = 0; c < 9; c++) dP[c] = two_mu * dF[c] + lambda * (cx * invFt[c] - Y[c]);
    lcm_pk_out(V, dP, Dinv, out);
}

// The P-K material of a solid: kind 1 C_LCM, 2 C_LCMH, 3 C_CCM (enum
// fem_material); mu and lambda from the set's scalar E and nu; k the
// C_LCMH blend radius.
struct PkMaterial {
    int kind;
    double mu, lambda, k;
};

FEM_HD void pk_force(const PkMaterial& m, const double* R, const double* F, const double* Dinv, double V,
                     double* out)
{
    if (m.kind == 3)
        ccm_force(R, F, Dinv, V, m.mu, m.lambda, out);
    else
        lcm_force(R, F, Dinv, V, m.mu, m.lambda, out);
}

FEM_HD void pk_dforce(const PkMaterial& m, const double* R, const double* F, double detF, const double* Dinv,
                      double V, const double* dl, double* out)
{
    if (m.kind == 2)
        lcmh_dforce(R, F, Dinv, V, m.mu, m.lambda, m.k, dl, out);
    else if (m.kind == 3)
        ccm_dforce(F, detF, Dinv, V, m.mu, m.lambda, dl, out);
    else
        lcm_dforce(R, Dinv, V, m.mu, m.lambda, dl, out);
}

FEM_HD double lcm_energy(const double* R, const double* F, double V, double mu, double lambda);

FEM_HD double pk_energy(const PkMaterial& m, const double* R, const double* F, double V)
{
    return m.kind == 3 ? 0.0 : lcm_energy(R, F, V, m.mu, m.lambda);
}

FEM_HD double lcm_energy(const double* R, const double* F, double V, double mu, double lambda)
{
    double SmI[9];
    lcm_s_minus_i(R, F, SmI);
    double nsq = 0.0;
    for (int c = 0; c < 9; c++) nsq += SmI[c] * SmI[c];
    const double tr = lcm_trace(SmI);
    return V * (mu * nsq + 0.5 * lambda * (tr * tr));
}

}  // namespace femgb
