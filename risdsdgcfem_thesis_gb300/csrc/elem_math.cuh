// elem_math.cuh -- the per-element corotational product in strain form.
//
// K0 = V B^T E B (TetrahedronElement3::Compute_K, TetrahedronElement3.h:
// 157-173) applied without forming K0: with the shape-function gradients of
// nodes 1..3 the rows of Dm^-1 (node 0: minus their sum), the displacement
// gradient is H = [u1-u0, u2-u0, u3-u0] Dm^-1, the Voigt strain is
// (H00, H11, H22, H01+H10, H12+H21, H02+H20), the stress uses the E-matrix
// entries a_k1 = lambda+2mu, a_nu = lambda, a_k2 = mu (times V), and the
// nodal forces are sigma * grad N_i. R K0 R^T d rotates d into the element
// frame and the forces back.
#pragma once

namespace femgb {

// Values (displacements, forces) are of type S; the element's coefficients
// (R, Dm^-1, material scalars) of type C, by default the same. The mixed
// path's recomputed residual takes S = a double-float and C = float, the
// type its element data is stored in.

// Local-frame stress product: given H (displacement gradient in the element
// frame), returns P = sigma(H) * Dinv^T (columns = forces on nodes 1..3 in
// the element frame, V folded into the material scalars) and eps:sigma.
template <typename S, typename C = S>
__device__ __forceinline__ void stress_forces(const S* H, const C* Di, C k1, C knu, C k2, S* P, S& eps_sig)
{
    const S exx = H[0], eyy = H[4], ezz = H[8];
    const S gxy = H[1] + H[3], gyz = H[5] + H[7], gzx = H[2] + H[6];
    const S sxx = k1 * exx + knu * (eyy + ezz);
    const S syy = k1 * eyy + knu * (exx + ezz);
    const S szz = k1 * ezz + knu * (exx + eyy);
    const S txy = k2 * gxy, tyz = k2 * gyz, tzx = k2 * gzx;
    eps_sig = sxx * exx + syy * eyy + szz * ezz + txy * gxy + tyz * gyz + tzx * gzx;
    const S Sg[9] = {sxx, txy, tzx, txy, syy, tyz, tzx, tyz, szz};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int i = 0; i < 3; i++)
            P[3 * a + i] = Sg[3 * a] * Di[3 * i] + Sg[3 * a + 1] * Di[3 * i + 1] + Sg[3 * a + 2] * Di[3 * i + 2];
}

// Writes R * P (world frame) to out[4][3]: node 0 gets minus the sum.
template <typename S, typename C = S>
__device__ __forceinline__ void rotate_out(const C* R, const S* P, S* out)
{
    S Pw[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int i = 0; i < 3; i++) Pw[3 * a + i] = R[3 * a] * P[i] + R[3 * a + 1] * P[3 + i] + R[3 * a + 2] * P[6 + i];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        out[3 * (i + 1) + 0] = Pw[i];
        out[3 * (i + 1) + 1] = Pw[3 + i];
        out[3 * (i + 1) + 2] = Pw[6 + i];
    }
    out[0] = -(Pw[0] + Pw[1] + Pw[2]);
    out[1] = -(Pw[3] + Pw[4] + Pw[5]);
    out[2] = -(Pw[6] + Pw[7] + Pw[8]);
}

// Product R K0 R^T d for one element (world-frame nodal vectors d[4][3]).
template <typename S, typename C = S>
__device__ __forceinline__ void elem_RKRt(const C* R, const C* Di, C k1, C knu, C k2, const S* d, S* out)
{
    S D[9];  // columns d1-d0, d2-d0, d3-d0 ; D[3a+j]
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) D[3 * a + j] = d[3 * (j + 1) + a] - d[a];
    S Hw[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) Hw[3 * a + b] = D[3 * a] * Di[b] + D[3 * a + 1] * Di[3 + b] + D[3 * a + 2] * Di[6 + b];
    S H[9];  // R^T Hw
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) H[3 * a + b] = R[a] * Hw[b] + R[3 + a] * Hw[3 + b] + R[6 + a] * Hw[6 + b];
    S P[9], es;
    stress_forces(H, Di, k1, knu, k2, P, es);
    rotate_out(R, P, out);
}

// The C_LCM differential (C_LCM_df_x, TetrahedronElementSet3.cpp:1838-1873,
// truncated) with V folded into the Lame scalars, kl = V lambda and
// km = V mu: dF = dDs Dm^-1, dP = 2 km dF + kl tr(R^T dF) R, and the nodal
// products dP Dm^-T (node 0: minus their sum), the convention of
// elem_RKRt. For the mixed path's types; the FP64 batch takes lcm_dforce,
// the FP64 solid's own arithmetic.
template <typename S, typename C = S>
__device__ __forceinline__ void elem_lcm_dforce(const C* R, const C* Di, C kl, C km, const S* d, S* out)
{
    S dDs[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) dDs[3 * a + j] = d[3 * (j + 1) + a] - d[a];
    S dF[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) dF[3 * a + b] = dDs[3 * a] * Di[b] + dDs[3 * a + 1] * Di[3 + b] + dDs[3 * a + 2] * Di[6 + b];
    S tr = R[0] * dF[0];
#pragma unroll
    for (int c = 1; c < 9; c++) tr = tr + R[c] * dF[c];
    const C km2 = (C)2 * km;
    const S ktr = kl * tr;
    S dP[9];
#pragma unroll
    for (int c = 0; c < 9; c++) dP[c] = km2 * dF[c] + ktr * R[c];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        S acc0 = dP[3 * a] * Di[0] + dP[3 * a + 1] * Di[1] + dP[3 * a + 2] * Di[2];
        S acc1 = dP[3 * a] * Di[3] + dP[3 * a + 1] * Di[4] + dP[3 * a + 2] * Di[5];
        S acc2 = dP[3 * a] * Di[6] + dP[3 * a + 1] * Di[7] + dP[3 * a + 2] * Di[8];
        out[3 + a] = acc0;
        out[6 + a] = acc1;
        out[9 + a] = acc2;
        out[a] = -(acc0 + acc1 + acc2);
    }
}

// The C_LCMH differential (C_LCMH_df_x, TetrahedronElementSet3.cpp:
// 1875-1930) in the same folded form, with the element's blend weight w
// (Clamp01(tr|S - I| / (3 k)) at the last evaluation; 1 when k <= 0.1,
// where the reference takes C_LCM's): dP = 2 km (w dF + (1 - w) R
// sym(R^T dF)) + kl tr(R^T dF) R.
template <typename S, typename C = S>
__device__ __forceinline__ void elem_lcmh_dforce(const C* R, const C* Di, C kl, C km, C w, const S* d, S* out)
{
    S dDs[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int j = 0; j < 3; j++) dDs[3 * a + j] = d[3 * (j + 1) + a] - d[a];
    S dF[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) dF[3 * a + b] = dDs[3 * a] * Di[b] + dDs[3 * a + 1] * Di[3 + b] + dDs[3 * a + 2] * Di[6 + b];
    S RtdF[9];  // R^T dF
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) RtdF[3 * a + b] = R[a] * dF[b] + R[3 + a] * dF[3 + b] + R[6 + a] * dF[6 + b];
    const S ktr = kl * (RtdF[0] + RtdF[4] + RtdF[8]);
    const C km2 = (C)2 * km, ow = (C)1 - w;
    S sym[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) sym[3 * a + b] = (RtdF[3 * a + b] + RtdF[3 * b + a]) * (C)0.5;
    S dP[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const S Rs = R[3 * a] * sym[b] + R[3 * a + 1] * sym[3 + b] + R[3 * a + 2] * sym[6 + b];
            dP[3 * a + b] = km2 * (w * dF[3 * a + b] + ow * Rs) + ktr * R[3 * a + b];
        }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        S acc0 = dP[3 * a] * Di[0] + dP[3 * a + 1] * Di[1] + dP[3 * a + 2] * Di[2];
        S acc1 = dP[3 * a] * Di[3] + dP[3 * a + 1] * Di[4] + dP[3 * a + 2] * Di[5];
        S acc2 = dP[3 * a] * Di[6] + dP[3 * a + 1] * Di[7] + dP[3 * a + 2] * Di[8];
        out[3 + a] = acc0;
        out[6 + a] = acc1;
        out[9 + a] = acc2;
        out[a] = -(acc0 + acc1 + acc2);
    }
}

}  // namespace femgb
