// rotation.cu -- BeginEvaluation of the element set: F = Ds Dm^-1, det F and
// the MSVD rotation per tet (TetrahedronElementSet3::BeginEvaluation,
// TetrahedronElementSet3.cpp:219-281, ComputeRotations_MSVD :777-792).
//
// This translation unit is compiled with --fmad=false: the FP64 rotation is
// then evaluated with the reference's rounding sequence (no fused
// multiply-adds), which makes the GPU rotations equal to the reference's on
// the same positions.
#include "fem_device.cuh"
#include "msvd.cuh"

namespace femgb {

__global__ void k_begin_eval_fp64(MeshView<double> m, const double* __restrict__ x, double* F_out,
                                  StepScalars* st)
{
    unsigned inverted = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        const int ids[4] = {t.x, t.y, t.z, t.w};
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
    k_begin_eval_fp64<<<grid_for(m.T), kBlock, 0, s>>>(m, x, F_out, st);
    launch_counter()++;
}

}  // namespace femgb
