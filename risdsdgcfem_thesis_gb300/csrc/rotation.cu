// rotation.cu -- BeginEvaluation of the element set: F = Ds Dm^-1, det F and
// the MSVD rotation per tet (TetrahedronElementSet3::BeginEvaluation,
// TetrahedronElementSet3.cpp:219-281, ComputeRotations_MSVD :777-792).
//
// This translation unit is compiled with --fmad=false: the FP64 rotation is
// then evaluated with the reference's rounding sequence (no fused
// multiply-adds), which makes the GPU rotations equal to the reference's on
// the same positions.
#include "batch_launch.h"
#include "bounds.cuh"
#include "dapd.cuh"
#include "fem_device.cuh"
#include "msvd.cuh"

namespace femgb {

__global__ void k_begin_eval_fp64(MeshView<double> m, const double* __restrict__ x, double* F_out,
                                  StepScalars* st)
{
    unsigned inverted = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        const int ids[4] = {(int)bounds_idx((uint32_t)t.x, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.y, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.z, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.w, m.N, kSiteElemNode)};
        V3<double> xs[4];
#pragma unroll
        for (int i = 0; i < 4; i++) xs[i] = mk<double>(x[3 * (size_t)ids[i]], x[3 * (size_t)ids[i] + 1], x[3 * (size_t)ids[i] + 2]);
        double Di[9];
#pragma unroll
        for (int c = 0; c < 9; c++) Di[c] = m.Dinv[c * (size_t)m.T + e];
        double F[9], detF;
        deformation_gradient(xs, Di, F, detF);
        double R[9];
        msvd_rotation(F, R);
#pragma unroll
        for (int c = 0; c < 9; c++) m.R[c * (size_t)m.T + e] = R[c];
        m.detF[e] = detF;
        if (F_out) {
#pragma unroll
            for (int c = 0; c < 9; c++) F_out[9 * (size_t)e + c] = F[c];
        }
        inverted += (detF <= 0.0) ? 1u : 0u;
    }
    // count of inverted elements (the reference's S2_MS_STAT m_Num_Degenerate)
    unsigned w = inverted;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&st->inverted, w);
}

void launch_begin_eval_fp64(const MeshView<double>& m, const double* x, double* F_out, StepScalars* st,
                            cudaStream_t s)
{
    prof_begin("begin_eval_msvd_fp64", s);
    k_begin_eval_fp64<<<grid_for(m.T), kBlock, 0, s>>>(m, x, F_out, st);
    prof_end("begin_eval_msvd_fp64", s);
    launch_counter()++;
}

// BeginEvaluation with the DAPD rotation (ComputeRotations_DAPD,
// TetrahedronElementSet3.cpp:860-892): xprev are the positions the previous
// evaluation's step started from (m_vecPos0), doc the per-element direction
// of collapse carried between evaluations. Elements above the threshold take
// the Newton polar rotation (a few 3x3 inverses); the collapse analysis runs
// only on elements at or below it.
__global__ void k_begin_eval_dapd_fp64(MeshView<double> m, const double* __restrict__ xprev,
                                       const double* __restrict__ x, uchar2* doc, DapdParams p, double* F_out,
                                       StepScalars* st)
{
    unsigned inverted = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        const int ids[4] = {(int)bounds_idx((uint32_t)t.x, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.y, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.z, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.w, m.N, kSiteElemNode)};
        V3<double> xs[4], xp[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const size_t n = 3 * (size_t)ids[i];
            xs[i] = mk<double>(x[n], x[n + 1], x[n + 2]);
            xp[i] = mk<double>(xprev[n], xprev[n + 1], xprev[n + 2]);
        }
        double Di[9];
#pragma unroll
        for (int c = 0; c < 9; c++) Di[c] = m.Dinv[c * (size_t)m.T + e];
        double F[9], detF;
        deformation_gradient(xs, Di, F, detF);
        uchar2 d = doc[e];
        double R[9];
        dapd_rotation(xp, xs, Di, F, detF, m.vol[e], p, d, R);
        doc[e] = d;
#pragma unroll
        for (int c = 0; c < 9; c++) m.R[c * (size_t)m.T + e] = R[c];
        m.detF[e] = detF;
        if (F_out) {
#pragma unroll
            for (int c = 0; c < 9; c++) F_out[9 * (size_t)e + c] = F[c];
        }
        inverted += (detF <= 0.0) ? 1u : 0u;
    }
    unsigned w = inverted;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(&st->inverted, w);
}

void launch_begin_eval_dapd_fp64(const MeshView<double>& m, const double* xprev, const double* x, uchar2* doc,
                                 const DapdParams& p, double* F_out, StepScalars* st, cudaStream_t s)
{
    prof_begin("begin_eval_dapd_fp64", s);
    k_begin_eval_dapd_fp64<<<grid_for(m.T), kBlock, 0, s>>>(m, xprev, x, doc, p, F_out, st);
    prof_end("begin_eval_dapd_fp64", s);
    launch_counter()++;
}

// ---------------------------------------------------------------------------
// Batched BeginEvaluation: block per element tile (one mesh per tile). F and
// det F in FP64 from FP64 positions and Dm^-1. The FP64 path takes the FP64
// rotation; the mixed path the double-float rotation, or, with the FP32
// option, the FP32 rotation unless det F <= the mesh's threshold or the
// check below fails, where F is re-solved in double-float arithmetic. Per-mesh counts of
// inverted elements and FP64 re-solves are added with integer atomics (one
// per tile), so they do not depend on scheduling.
// FP32 rotation of F for the mixed path. The result is not trusted -- the
// cause is returned for an FP64 re-solve -- when one of the MSVD's branch
// decisions was a near tie (FP32 rounding may decide it differently from
// FP64, and the rotation jumps with the decision), or, with tol > 0, when
// the rotation computed again for F plus a fixed 2^-14 relative change
// differs by more than tol (max entry).
enum { kRotKept = 0, kRotTie = 1, kRotCheck = 2 };
template <typename S>
__device__ __forceinline__ int rotation_fp32(const double* F, float tol, S* Rs)
{
    float Ff[9], Rf[9];
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 9; c++) {
        Ff[c] = (float)F[c];
        s = fmaxf(s, fabsf(Ff[c]));
    }
    bool tie = false;
    msvd_rotation(Ff, Rf, &tie);
    if (tie) return kRotTie;  // a branch decision FP32 may take differently from FP64
    if (tol > 0.f) {
        const float d = s * 6.103515625e-05f;  // 2^-14 of the largest entry
        const float P[9] = {1.f, -1.f, 0.f, 0.f, 1.f, -1.f, 1.f, 0.f, 1.f};
        float Fp[9], Rp[9];
#pragma unroll
        for (int c = 0; c < 9; c++) Fp[c] = Ff[c] + d * P[c];
        msvd_rotation(Fp, Rp);
        float diff = 0.f;
#pragma unroll
        for (int c = 0; c < 9; c++) diff = fmaxf(diff, fabsf(Rf[c] - Rp[c]));
        if (!(diff <= tol)) return kRotCheck;  // also when NaN
    }
#pragma unroll
    for (int c = 0; c < 9; c++) Rs[c] = (S)Rf[c];
    return kRotKept;
}

// Three resident blocks per SM (80 registers): the double-float MSVD's long
// dependency chains need the extra warps more than the registers.
template <typename S>
__global__ void __launch_bounds__(256, 3) k_begin_eval_batch(BatchView<S> b, const double* __restrict__ x,
                                                              int newton)
{
    __shared__ unsigned s_inv, s_res, s_cause[4];  // re-solves: det F, isotropic, tie, check
    const uint32_t n = b.list_count[0];
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t t = b.start_tiles[i];
        const TileMeta tm = b.tiles[t];
        // newton: the FIE meshes whose solve has just updated x_k
        // (BeginEvaluation(x^n, x_k), LeafDSH_Solid3D_FEM.cpp:1529; their
        // DAPD previous positions are x^n); otherwise the start section's
        if (newton ? ((!b.lock && b.mc[tm.mesh].integrator == kMeshQie) || !b.st[tm.mesh].finished)
                   : !mesh_starts(b, tm.mesh))
            continue;
        if (threadIdx.x == 0) { s_inv = 0; s_res = 0; s_cause[0] = s_cause[1] = s_cause[2] = s_cause[3] = 0; }
        __syncthreads();
        if (threadIdx.x < tm.ne) {
            const size_t e = tm.e0 + threadIdx.x;
            const size_t T = b.Ttot;
            const int4 g = b.gtets[e];
            const int ids[4] = {(int)bounds_idx((uint32_t)g.x, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.y, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.z, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.w, b.Ntot, kSiteBatchNode)};
            V3<double> xs[4];
#pragma unroll
            for (int i = 0; i < 4; i++)
                xs[i] = mk<double>(x[3 * (size_t)ids[i]], x[3 * (size_t)ids[i] + 1], x[3 * (size_t)ids[i] + 2]);
            double Di[9];
#pragma unroll
            for (int c = 0; c < 9; c++) Di[c] = b.Dinv64[c * T + e];
            double F[9], detF;
            deformation_gradient(xs, Di, F, detF);
            S Rs[9];
            const MeshConsts& mcm = b.mc[tm.mesh];
            if (b.prev_x && mcm.rotation == kMeshRotationDapd) {
                // DAPD in FP64 in either precision (ComputeRotations_DAPD,
                // TetrahedronElementSet3.cpp:860-892), from the positions at
                // the start of the mesh's previous step
                V3<double> xp[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const size_t n3 = 3 * (size_t)ids[i];
                    xp[i] = mk<double>(b.prev_x[n3], b.prev_x[n3 + 1], b.prev_x[n3 + 2]);
                }
                DapdParams dp;
                dp.thr = mcm.dapd_thr;
                dp.fL = mcm.dapd_fL;
                dp.fNL = mcm.dapd_fNL;
                dp.eNL = mcm.dapd_eNL;
                uchar2 d = b.doc[e];
                double R[9];
                dapd_rotation(xp, xs, Di, F, detF, b.vol[e], dp, d, R);
                b.doc[e] = d;
#pragma unroll
                for (int c = 0; c < 9; c++) Rs[c] = (S)R[c];
                if (sizeof(S) != sizeof(double)) atomicAdd(&s_res, 1u);
            } else if (sizeof(S) == sizeof(double)) {
                double R[9];
                msvd_rotation(F, R);
#pragma unroll
                for (int c = 0; c < 9; c++) Rs[c] = (S)R[c];
            } else {
                const bool degenerate = !(detF > b.mc[tm.mesh].degenerate_det_F);
                const int why = (b.mc[tm.mesh].rot_fp32 && !degenerate)
                                    ? rotation_fp32(F, b.mc[tm.mesh].rot_check, Rs)
                                    : kRotTie + kRotCheck + 1;  // no FP32 attempt
                if (why != kRotKept) {
                    // the double-float rotation, or the FP64 one for a
                    // degenerate element (det F <= the threshold) or a nearly
                    // isotropic F (counted as re-solves, by cause)
                    float Rf[9];
                    bool iso = false;
                    if (degenerate || (iso = !rotation_df(F, Rf))) {
                        double R[9];
                        msvd_rotation(F, R);
#pragma unroll
                        for (int c = 0; c < 9; c++) Rf[c] = (float)R[c];
                    }
#pragma unroll
                    for (int c = 0; c < 9; c++) Rs[c] = (S)Rf[c];
                    atomicAdd(&s_res, 1u);
                    if (degenerate) atomicAdd(&s_cause[0], 1u);
                    else if (iso) atomicAdd(&s_cause[1], 1u);
                    if (why == kRotTie) atomicAdd(&s_cause[2], 1u);
                    if (why == kRotCheck) atomicAdd(&s_cause[3], 1u);
                }
            }
#pragma unroll
            for (int c = 0; c < 9; c++) b.R[c * T + e] = Rs[c];
            if (b.blob) {
                unsigned char* base = b.blob + 16ull * b.blob_off16[t];
                const uint32_t ne4 = blob_ne4(tm.ne), i = threadIdx.x;
                *reinterpret_cast<float4*>(base + blob_comp_off(0, i, ne4)) =
                    make_float4((float)Rs[0], (float)Rs[1], (float)Rs[2], (float)Rs[3]);
                *reinterpret_cast<float4*>(base + blob_comp_off(4, i, ne4)) =
                    make_float4((float)Rs[4], (float)Rs[5], (float)Rs[6], (float)Rs[7]);
                *reinterpret_cast<float*>(base + blob_comp_off(8, i, ne4)) = (float)Rs[8];
            }
            b.detF[e] = detF;
            if (b.Fe && mcm.material != kTileMaterialWrp) {
                // the element cache's F, which the P-K materials' f_e, V
                // and differentials read
#pragma unroll
                for (int c = 0; c < 9; c++) b.Fe[c * T + e] = F[c];
                if (b.lcmh_w && mcm.material == kTileMaterialLcmh) {
                    // the mixed path's C_LCMH blend weight
                    // (TetrahedronElementSet3.cpp:1886-1897) on the stored
                    // rotation: w = Clamp01(tr|R^T F - I| / (3 k)); 1 when
                    // (float)k <= 0.1, where the differential is C_LCM's
                    double w = 1.0;
                    if ((float)mcm.ecie_k > 0.1f) {
                        double tr = 0.0;
#pragma unroll
                        for (int a = 0; a < 3; a++) {
                            double sa = 0.0;
#pragma unroll
                            for (int k = 0; k < 3; k++) sa += (double)Rs[3 * k + a] * F[3 * k + a];
                            tr += fabs(sa - 1.0);
                        }
                        w = (1.0 / mcm.ecie_k) * tr / 3.0;
                        w = (w < 1.0) ? w : 1.0;
                        w = (0.0 > w) ? 0.0 : w;
                    }
                    b.lcmh_w[e] = (float)w;
                }
            }
            if (detF <= 0.0) atomicAdd(&s_inv, 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (s_inv) atomicAdd(&b.st[tm.mesh].inverted, s_inv);
            if (s_res) atomicAdd(&b.st[tm.mesh].fp64_resolved, s_res);
            if (s_cause[0]) atomicAdd(&b.st[tm.mesh].res_det_F, s_cause[0]);
            if (s_cause[1]) atomicAdd(&b.st[tm.mesh].res_isotropic, s_cause[1]);
            if (s_cause[2]) atomicAdd(&b.st[tm.mesh].res_tie, s_cause[2]);
            if (s_cause[3]) atomicAdd(&b.st[tm.mesh].res_check, s_cause[3]);
        }
        __syncthreads();
    }
}

template <typename S>
void BatchLaunch<S>::begin_eval(const BatchView<S>& b, const double* x, int newton, cudaStream_t s)
{
    prof_begin("begin_eval_batch", s);
    k_begin_eval_batch<S><<<grid_tiles(b.ntiles), kTileElems, 0, s>>>(b, x, newton);
    prof_end("begin_eval_batch", s);
    launch_counter()++;
}

template void BatchLaunch<double>::begin_eval(const BatchView<double>&, const double*, int, cudaStream_t);
template void BatchLaunch<float>::begin_eval(const BatchView<float>&, const double*, int, cudaStream_t);

FEMGB_BOUNDS_ACCESSOR(bounds_read_rotation)

}  // namespace femgb
