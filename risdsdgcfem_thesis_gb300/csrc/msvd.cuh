// msvd.cuh -- per-tet rotation R = U V^T of the reference's MSVD method, as a
// device function over a 3x3 deformation gradient held in registers.
//
// Follows Compute_R_SVD (Saphyre2 ms/fem/Rotation.cpp:39-57), which calls
// GFastSVD3x3 (Mal/GMatDecomposition_SVD3x3_PhysBAM.h:247-280): eigen-
// decomposition of the normal equations F^T F by Smith's trigonometric
// formula (Fast_Eigenvalues, :161-197), eigenvectors by cofactor columns with
// the "flip" to the most separated eigenvalue (Fast_Eigenvectors, :199-236),
// U from F V, R = U V^T. The operation order matches the reference term for
// term so that, compiled without fused multiply-adds, an FP64 evaluation
// gives the reference's R bit for bit on the same F (up to the last ulp of
// the libm sin/cos/atan2).
//
// Two properties of the reference are kept on purpose:
//  * Fast_Eigenvalues scales the sine term by Sqrt(3) with an int argument,
//    which the reference's Sqrt template evaluates as int(sqrtf(3)) == 1.
//    The factor here is therefore 1, not sqrt(3).
//  * Sqrt/Sin/Cos/ATan2 are evaluated at the precision of T. (The reference's
//    FP64 build rounds them through float, which makes R NaN near F = I;
//    the restatement and this kernel use double there.)
//
// T is double (the FP64 path, bit-exact), float (the optional FP32 rotation
// of the mixed path) or DF, a double-float (the mixed path's default: about
// 48 bits on the FP32 pipe; GB300's FP64 rate made the FP64 rotation, with
// its FP64 sin/cos/atan2, a tenth of the mixed step).
#pragma once
#include <cuda_runtime.h>

#include "df.cuh"

namespace femgb {

// Per-type math: sqrt, abs, and eig_cos_sin(m, p, sqrt_p, q, c, s), the
// cosine and sine of phi = atan2(sqrt(max(p^3 - q^2, 0)), q) / 3
// (Fast_Eigenvalues, PhysBAM.h:169-173).
template <typename T> struct MathOf;
template <> struct MathOf<double> {
    static __device__ __forceinline__ double sqrt_(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double abs_(double x) { return ::fabs(x); }
    static __device__ __forceinline__ void eig_cos_sin(double, double p, double, double q, double& c, double& s)
    {
        const double disc = p * p * p - q * q;
        const double disc_c = (0.0 > disc) ? 0.0 : disc;
        const double phi = (1.0 / 3.0) * ::atan2(::sqrt(disc_c), q);
        c = ::cos(phi);
        s = ::sin(phi);
    }
};
template <> struct MathOf<float> {
    static __device__ __forceinline__ float sqrt_(float x) { return ::sqrtf(x); }
    static __device__ __forceinline__ float abs_(float x) { return ::fabsf(x); }
    static __device__ __forceinline__ void eig_cos_sin(float, float p, float, float q, float& c, float& s)
    {
        const float disc = p * p * p - q * q;
        const float disc_c = (0.f > disc) ? 0.f : disc;
        const float phi = (1.f / 3.f) * ::atan2f(::sqrtf(disc_c), q);
        c = ::cosf(phi);
        s = ::sinf(phi);
    }
};
template <> struct MathOf<DF> {
    static __device__ __forceinline__ DF sqrt_(DF x) { return df_sqrt(x); }
    static __device__ __forceinline__ DF abs_(DF x) { return df_abs(x); }
    // cos(theta) = q / p^(3/2) and sin(theta) = sqrt(1 - cos^2) (clamped):
    // the same angle as above in a form free of p^3 and q^2, which scale
    // with the sixth power of the deviation from isotropy and would leave
    // FP32's exponent range. theta lies in [0, pi], phi = theta / 3 in
    // [0, pi/3]. c = cos(phi) solves 4c^3 - 3c = cos(theta), s = sin(phi)
    // solves 3s - 4s^3 = sin(theta) (triple-angle identities): Newton steps
    // from the FP32 values, with the derivative's reciprocal at the FP32
    // guess (each step gains about seven digits). Where a derivative
    // vanishes (c = 1/2, s = 1/2) the other of the pair gives it through
    // c^2 + s^2 = 1, away from cancellation.
    // A nearly isotropic F^T F (sqrt(p) below 1e-7 m) returns NaN: the
    // later cofactor products there approach FP32's underflow, and the
    // caller re-solves such an F in FP64.
    static __device__ __forceinline__ void eig_cos_sin(DF m, DF p, DF sqrt_p, DF q, DF& c, DF& s)
    {
        if (!(sqrt_p.hi >= 1e-7f * ::fabsf(m.hi))) {
            c = s = DF(__int_as_float(0x7fffffff), 0.f);
            return;
        }
        DF ct = q / (p * sqrt_p);
        if (ct > DF(1.f, 0.f)) ct = DF(1.f, 0.f);
        if (ct < DF(-1.f, 0.f)) ct = DF(-1.f, 0.f);
        const DF one_m = (DF(1.f, 0.f) - ct) * (DF(1.f, 0.f) + ct);
        const DF st = one_m.hi > 0.f ? df_sqrt(one_m) : DF(0.f, 0.f);
        const float phf = ::atan2f(st.hi, ct.hi) * (1.f / 3.f);
        const float cf = ::cosf(phf), sf = ::sinf(phf);
        DF cc(cf, 0.f), ss(sf, 0.f);
        const bool c_newton = cf >= 0.6f, s_newton = sf <= 0.35f || sf >= 0.65f;
        if (c_newton) {
            const float inv = 1.f / (12.f * cf * cf - 3.f);
#pragma unroll
            for (int k = 0; k < 3; k++) cc = cc - ((DF(4.f, 0.f) * cc * cc - DF(3.f, 0.f)) * cc - ct) * inv;
        }
        if (s_newton) {
            const float inv = 1.f / (3.f - 12.f * sf * sf);
#pragma unroll
            for (int k = 0; k < 3; k++) ss = ss - ((DF(3.f, 0.f) - DF(4.f, 0.f) * ss * ss) * ss - st) * inv;
        }
        if (!c_newton) cc = df_sqrt(DF(1.f, 0.f) - ss * ss);
        if (!s_newton) ss = df_sqrt(DF(1.f, 0.f) - cc * cc);
        c = cc;
        s = ss;
    }
};

// Branch-tie tracking for the FP32 evaluation: the MSVD below takes discrete
// decisions (which column, which axis, which eigenvalue order, the flip)
// and, with the reference's eigenvalue formula, its rotation jumps when a
// decision flips. near_tie() marks a comparison whose two sides are within
// a relative margin of each other, where FP32 rounding may decide it
// differently from FP64; a caller re-solves such an F in FP64. FP64 calls
// pass no tracker and are unaffected.
template <typename T> __device__ __forceinline__ void near_tie(bool* amb, T a, T b, T scale)
{
    if (amb && MathOf<T>::abs_(a - b) <= T(2e-3) * scale) *amb = true;
}

template <typename T>
struct V3 {
    T x, y, z;
};

template <typename T> __device__ __forceinline__ V3<T> mk(T a, T b, T c) { V3<T> r; r.x = a; r.y = b; r.z = c; return r; }
template <typename T> __device__ __forceinline__ T dot0(V3<T> a, V3<T> b)
{
    // accumulator from zero, as GVec::operator* (Mal/GVec.h:88)
    T acc = T(0);
    acc += a.x * b.x;
    acc += a.y * b.y;
    acc += a.z * b.z;
    return acc;
}
template <typename T> __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b)
{
    return mk<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T> __device__ __forceinline__ V3<T> scale(T s, V3<T> a) { return mk<T>(s * a.x, s * a.y, s * a.z); }
template <typename T> __device__ __forceinline__ V3<T> normalized(V3<T> a)
{
    T n = MathOf<T>::sqrt_(dot0(a, a));
    T inv = T(1) / n;
    return scale(inv, a);
}
template <typename T> __device__ __forceinline__ V3<T> orthogonal_vector(V3<T> v, bool* amb = nullptr)
{
    T ax = MathOf<T>::abs_(v.x), ay = MathOf<T>::abs_(v.y), az = MathOf<T>::abs_(v.z);
    if (amb) {
        const T sum = ax + ay + az;
        near_tie(amb, ax, ay, sum);
        near_tie(amb, ax, az, sum);
        near_tie(amb, ay, az, sum);
    }
    if (ax < ay) return (ax < az) ? mk<T>(T(0), v.z, -v.y) : mk<T>(v.y, -v.x, T(0));
    return (ay < az) ? mk<T>(-v.z, T(0), v.x) : mk<T>(v.y, -v.x, T(0));
}
// M * v with the accumulator from zero (Mal/GMatUtils.h:12-23); M row-major
template <typename T> __device__ __forceinline__ V3<T> matvec0(const T* M, V3<T> v)
{
    V3<T> r;
    T acc;
    acc = T(0); acc += M[0] * v.x; acc += M[1] * v.y; acc += M[2] * v.z; r.x = acc;
    acc = T(0); acc += M[3] * v.x; acc += M[4] * v.y; acc += M[5] * v.z; r.y = acc;
    acc = T(0); acc += M[6] * v.x; acc += M[7] * v.y; acc += M[8] * v.z; r.z = acc;
    return r;
}

template <typename T> struct Sym3 { T x11, x21, x31, x22, x32, x33; };

template <typename T> __device__ __forceinline__ Sym3<T> cofactor(const Sym3<T>& a)
{
    Sym3<T> r;
    r.x11 = a.x22 * a.x33 - a.x32 * a.x32;
    r.x21 = a.x32 * a.x31 - a.x21 * a.x33;
    r.x31 = a.x21 * a.x32 - a.x22 * a.x31;
    r.x22 = a.x11 * a.x33 - a.x31 * a.x31;
    r.x32 = a.x21 * a.x31 - a.x11 * a.x32;
    r.x33 = a.x11 * a.x22 - a.x21 * a.x21;
    return r;
}

template <typename T> __device__ __forceinline__ V3<T> largest_column_normalized(const Sym3<T>& a, bool* amb = nullptr)
{
    T s11 = a.x11 * a.x11, s12 = a.x21 * a.x21, s13 = a.x31 * a.x31;
    T s22 = a.x22 * a.x22, s23 = a.x32 * a.x32, s33 = a.x33 * a.x33;
    T scale1 = s11 + s12 + s13, scale2 = s12 + s22 + s23, scale3 = s13 + s23 + s33;
    if (amb) {
        const T sum = scale1 + scale2 + scale3;
        near_tie(amb, scale1, scale2, sum);
        near_tie(amb, scale1, scale3, sum);
        near_tie(amb, scale2, scale3, sum);
    }
    if (scale1 > scale2) {
        if (scale1 > scale3) return scale(T(1) / MathOf<T>::sqrt_(scale1), mk<T>(a.x11, a.x21, a.x31));
    } else if (scale2 > scale3) {
        return scale(T(1) / MathOf<T>::sqrt_(scale2), mk<T>(a.x21, a.x22, a.x32));
    }
    if (scale3 > T(0)) return scale(T(1) / MathOf<T>::sqrt_(scale3), mk<T>(a.x31, a.x32, a.x33));
    return mk<T>(T(1), T(0), T(0));
}

// Rotation of one deformation gradient F (row-major 3x3) into R (row-major).
// With `amb`, *amb is set when a branch decision was a near tie (see
// near_tie); the arithmetic is the same with or without it. With
// `v_smallest`, only column 2 of V (the right singular vector of the
// smallest singular value) is formed, into *v_smallest, and R is not written.
template <typename T>
__device__ __forceinline__ void msvd_rotation(const T* F, T* R, bool* amb = nullptr, V3<T>* v_smallest = nullptr)
{
    // normal equations F^T F (PhysBAM.h:129-137)
    Sym3<T> ne;
    ne.x11 = F[0] * F[0] + F[3] * F[3] + F[6] * F[6];
    ne.x21 = F[1] * F[0] + F[4] * F[3] + F[7] * F[6];
    ne.x31 = F[2] * F[0] + F[5] * F[3] + F[8] * F[6];
    ne.x22 = F[1] * F[1] + F[4] * F[4] + F[7] * F[7];
    ne.x32 = F[2] * F[1] + F[5] * F[4] + F[8] * F[7];
    ne.x33 = F[2] * F[2] + F[5] * F[5] + F[8] * F[8];

    // Fast_Eigenvalues
    const T one_third = T(1) / T(3);
    const T one_sixth = T(1) / T(6);
    const T root_three = T(1);  // the reference's Sqrt(3) on an int argument
    T m = one_third * (ne.x11 + ne.x22 + ne.x33);
    T a11 = ne.x11 - m, a22 = ne.x22 - m, a33 = ne.x33 - m;
    T a12_sqr = ne.x21 * ne.x21, a13_sqr = ne.x31 * ne.x31, a23_sqr = ne.x32 * ne.x32;
    T p = one_sixth * (a11 * a11 + a22 * a22 + a33 * a33 + T(2) * (a12_sqr + a13_sqr + a23_sqr));
    T q = T(.5) * (a11 * (a22 * a33 - a23_sqr) - a22 * a13_sqr - a33 * a12_sqr) + ne.x21 * ne.x31 * ne.x32;
    T sqrt_p = MathOf<T>::sqrt_(p);
    T c, s;
    MathOf<T>::eig_cos_sin(m, p, sqrt_p, q, c, s);
    T sqrt_p_cos = sqrt_p * c, root_three_sqrt_p_sin = root_three * sqrt_p * s;
    T l0 = m + T(2) * sqrt_p_cos;
    T l1 = m - sqrt_p_cos - root_three_sqrt_p_sin;
    T l2 = m - sqrt_p_cos + root_three_sqrt_p_sin;
    if (amb) {
        // eigenvalue order and the flip test, relative to the spread
        const T spread = MathOf<T>::abs_(l0 - l1) + MathOf<T>::abs_(l1 - l2) + MathOf<T>::abs_(l0 - l2);
        near_tie(amb, l0, l1, spread);
        near_tie(amb, l1, l2, spread);
        near_tie(amb, l0, l2, spread);
    }
    T lam0, lam1, lam2;
    if (l0 < l1) {
        if (l1 < l2) { lam0 = l2; lam1 = l1; lam2 = l0; }
        else if (l0 < l2) { lam0 = l1; lam1 = l2; lam2 = l0; }
        else { lam0 = l1; lam1 = l0; lam2 = l2; }
    } else {
        if (l1 > l2) { lam0 = l0; lam1 = l1; lam2 = l2; }
        else if (l0 > l2) { lam0 = l0; lam1 = l2; lam2 = l1; }
        else { lam0 = l2; lam1 = l0; lam2 = l1; }
    }

    // Fast_Eigenvectors
    bool flipped = false;
    T lf0 = lam0, lf2 = lam2;
    near_tie(amb, lam0 - lam1, lam1 - lam2, lam0 - lam2);
    if (lam0 - lam1 < lam1 - lam2) { lf0 = lam2; lf2 = lam0; flipped = true; }
    Sym3<T> am = ne;
    am.x11 -= lf0; am.x22 -= lf0; am.x33 -= lf0;
    V3<T> v1 = largest_column_normalized(cofactor(am), amb);
    V3<T> o0 = normalized(orthogonal_vector(v1, amb));
    V3<T> o1 = cross(v1, o0);
    // C = A_full * other_v, then A_reduced = C^T other_v (symmetric)
    T C00, C10, C20, C01, C11, C21;
    {
        T acc;
        acc = T(0); acc += ne.x11 * o0.x; acc += ne.x21 * o0.y; acc += ne.x31 * o0.z; C00 = acc;
        acc = T(0); acc += ne.x11 * o1.x; acc += ne.x21 * o1.y; acc += ne.x31 * o1.z; C01 = acc;
        acc = T(0); acc += ne.x21 * o0.x; acc += ne.x22 * o0.y; acc += ne.x32 * o0.z; C10 = acc;
        acc = T(0); acc += ne.x21 * o1.x; acc += ne.x22 * o1.y; acc += ne.x32 * o1.z; C11 = acc;
        acc = T(0); acc += ne.x31 * o0.x; acc += ne.x32 * o0.y; acc += ne.x33 * o0.z; C20 = acc;
        acc = T(0); acc += ne.x31 * o1.x; acc += ne.x32 * o1.y; acc += ne.x33 * o1.z; C21 = acc;
    }
    T r11 = C00 * o0.x + C10 * o0.y + C20 * o0.z;
    T r21 = C01 * o0.x + C11 * o0.y + C21 * o0.z;
    T r22 = C01 * o1.x + C11 * o1.y + C21 * o1.z;
    r11 -= lf2;
    r22 -= lf2;
    // 2x2 cofactor (r22, -r21, r11), largest column normalised (PhysBAM.h:70-82)
    T w0, w1;
    {
        T c11 = r22, c21 = -r21, c22 = r11;
        T s11 = c11 * c11, s12 = c21 * c21, s22 = c22 * c22;
        T scale1 = s11 + s12, scale2 = s12 + s22;
        near_tie(amb, scale1, scale2, scale1 + scale2);
        if (scale1 > scale2) { T inv = T(1) / MathOf<T>::sqrt_(scale1); w0 = inv * c11; w1 = inv * c21; }
        else if (scale2 > T(0)) { T inv = T(1) / MathOf<T>::sqrt_(scale2); w0 = inv * c21; w1 = inv * c22; }
        else { w0 = T(1); w1 = T(0); }
    }
    V3<T> v3;
    {
        T acc;
        acc = T(0); acc += o0.x * w0; acc += o1.x * w1; v3.x = acc;
        acc = T(0); acc += o0.y * w0; acc += o1.y * w1; v3.y = acc;
        acc = T(0); acc += o0.z * w0; acc += o1.z * w1; v3.z = acc;
    }
    V3<T> v2 = cross(v3, v1);
    V3<T> c0, c1, c2;  // columns of V
    if (flipped) { c0 = v3; c1 = v2; c2 = mk<T>(-v1.x, -v1.y, -v1.z); }
    else { c0 = v1; c1 = v2; c2 = v3; }
    if (v_smallest) {
        *v_smallest = c2;
        return;
    }

    // U (GFastSVD3x3, PhysBAM.h:273-279)
    V3<T> u0 = normalized(matvec0(F, c0));
    V3<T> p0 = normalized(orthogonal_vector(u0));
    V3<T> p1 = cross(u0, p0);
    V3<T> t = normalized(matvec0(F, c1));
    T wa, wb;
    {
        T acc;
        acc = T(0); acc += p0.x * t.x; acc += p0.y * t.y; acc += p0.z * t.z; wa = acc;
        acc = T(0); acc += p1.x * t.x; acc += p1.y * t.y; acc += p1.z * t.z; wb = acc;
    }
    V3<T> u1;
    {
        T acc;
        acc = T(0); acc += p0.x * wa; acc += p1.x * wb; u1.x = acc;
        acc = T(0); acc += p0.y * wa; acc += p1.y * wb; u1.y = acc;
        acc = T(0); acc += p0.z * wa; acc += p1.z * wb; u1.z = acc;
    }
    V3<T> u2 = cross(u0, u1);

    // R = U * V^T ; U columns u0,u1,u2 ; V^T rows c0,c1,c2
    const T U[9] = {u0.x, u1.x, u2.x, u0.y, u1.y, u2.y, u0.z, u1.z, u2.z};
    const T Vt[9] = {c0.x, c0.y, c0.z, c1.x, c1.y, c1.z, c2.x, c2.y, c2.z};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            T acc = T(0);
            acc += U[3 * i + 0] * Vt[0 * 3 + j];
            acc += U[3 * i + 1] * Vt[1 * 3 + j];
            acc += U[3 * i + 2] * Vt[2 * 3 + j];
            R[3 * i + j] = acc;
        }
}

// Rotation of F in double-float arithmetic, rounded to FP32 (the mixed
// path's rotation). F is first scaled by a power of two that brings its
// largest entry into [0.5, 1): R = U V^T does not change under a positive
// scaling of F, and the double-float products stay inside FP32's exponent
// range. Returns false (R not set) when the double-float evaluation cannot
// be trusted -- a nearly isotropic F^T F (see MathOf<DF>) or a non-finite
// F -- and the caller re-solves in FP64.
__device__ __forceinline__ bool rotation_df(const double* F, float* Rf)
{
    double mx = 0.0;
#pragma unroll
    for (int c = 0; c < 9; c++) mx = ::fmax(mx, ::fabs(F[c]));
    if (!(mx > 0.0 && mx <= 1.7976931348623157e308)) return false;
    int e;
    (void)::frexp(mx, &e);
    const double sc = ::ldexp(1.0, -e);
    DF Fd[9], Rd[9];
#pragma unroll
    for (int c = 0; c < 9; c++) Fd[c] = DF(F[c] * sc);
    msvd_rotation(Fd, Rd);
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 9; c++) {
        Rf[c] = __double2float_rn(df_to_double(Rd[c]));
        ok = ok && Rf[c] == Rf[c];
    }
    return ok;
}

// F = Ds * Dm^-1 with Ds columns (x1-x0, x2-x0, x3-x0), and det F
// (TetrahedronElement3::Compute_D/Compute_F, TetrahedronElement3.h:92-104;
//  mal::Det, Mal/GMat.h:236-245).
template <typename T>
__device__ __forceinline__ void deformation_gradient(const V3<T> x[4], const T* Dinv, T* F, T& detF)
{
    T Ds[9];
    Ds[0] = x[1].x - x[0].x; Ds[1] = x[2].x - x[0].x; Ds[2] = x[3].x - x[0].x;
    Ds[3] = x[1].y - x[0].y; Ds[4] = x[2].y - x[0].y; Ds[5] = x[3].y - x[0].y;
    Ds[6] = x[1].z - x[0].z; Ds[7] = x[2].z - x[0].z; Ds[8] = x[3].z - x[0].z;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            T acc = T(0);
            acc += Ds[3 * i + 0] * Dinv[0 * 3 + j];
            acc += Ds[3 * i + 1] * Dinv[1 * 3 + j];
            acc += Ds[3 * i + 2] * Dinv[2 * 3 + j];
            F[3 * i + j] = acc;
        }
    detF = F[0] * F[4] * F[8] - F[0] * F[7] * F[5] + F[3] * F[7] * F[2]
         - F[3] * F[1] * F[8] + F[6] * F[1] * F[5] - F[6] * F[4] * F[2];
}

}  // namespace femgb
