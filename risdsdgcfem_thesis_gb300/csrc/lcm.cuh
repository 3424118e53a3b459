// lcm.cuh -- the C_LCM material of the reference's element set (linear
// corotational in first Piola-Kirchhoff form, ms::fem::Params::eMM_C_LCM),
// per element, FP64, with Mal's rounding order (products accumulated from
// zero, Trace from zero, scalar * matrix element by element):
//
//   C_LCM_f_e   TetrahedronElementSet3.cpp:1154-1178
//     S = R^T F, P = R (2 mu (S - I) + lambda tr(S - I) I)
//   C_LCM_df_x  TetrahedronElementSet3.cpp:1838-1873 (truncated: no dR term)
//     dF = dDs Dm^-1, dP = 2 mu dF + lambda tr(R^T dF) R
//   C_LCM_V     TetrahedronElementSet3.cpp:1489-1507
//     V (mu |S - I|_F^2 + 0.5 lambda tr(S - I)^2)
//   with H = -V P Dm^-T and nodal forces (-h1-h2-h3, h1, h2, h3), h_j the
//   columns of H.
//
// Outputs follow the element products' convention of the solid's kernels:
// out[3 i + a] is MINUS node i's force contribution (the gathers subtract).
// Host-callable as well, so that the arithmetic can be checked on the CPU.
// Matrices are row-major double[9].
#pragma once

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
