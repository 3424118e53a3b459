// fem_kernels.cu -- FP64 element products, node gathers and CG vector
// kernels of the corotational linear-tet implicit-Euler step.
//
// Element products use the strain form of K0 = V B^T E B
// (TetrahedronElement3::Compute_K, TetrahedronElement3.h:157-173): with
// Dm^-1 rows = gradients of the shape functions of nodes 1..3 and node 0's
// the negative sum, K0 u = V B^T sigma(eps(u)), eps = sym(H),
// H = [u1-u0, u2-u0, u3-u0] Dm^-1. Mathematically identical to the
// reference's 16 stored 3x3 blocks; 9+3 scalars per element instead of 144
// and about 140 FMA per product instead of 216.
//
// Scatter is atomics-free: each element writes its four nodal vectors to
// eout, and one thread per node sums its entries in element order (the order
// the reference's serial scatter adds them). Reductions are deterministic:
// warp shuffles, a fixed block tree, then one block summing the block
// partials in index order.
#include "bounds.cuh"
#include "lcm.cuh"
#include "fem_device.cuh"
#include "msvd.cuh"
#include "elem_math.cuh"

#include <cooperative_groups.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace femgb {

// ---- kernel timing (events on the launching stream) ----
namespace {
struct ProfSlot {
    std::vector<cudaEvent_t> starts, stops;
    double done_ms = 0.0;
    unsigned long long done_count = 0;
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::map<std::string, ProfSlot> g_prof;
std::vector<cudaEvent_t> g_event_pool;

cudaEvent_t pool_event()
{
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

bool prof_enabled() { return g_prof_on; }

void prof_begin(const char* name, cudaStream_t s)
{
    if (!g_prof_on) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e = pool_event();
    cudaEventRecord(e, s);
    g_prof[name].starts.push_back(e);
}

void prof_end(const char* name, cudaStream_t s)
{
    if (!g_prof_on) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEvent_t e = pool_event();
    cudaEventRecord(e, s);
    g_prof[name].stops.push_back(e);
}

// Folds completed event pairs into the totals (synchronises on the events).
static void prof_collect()
{
    for (auto& kv : g_prof) {
        ProfSlot& sl = kv.second;
        const size_t n = sl.stops.size() < sl.starts.size() ? sl.stops.size() : sl.starts.size();
        for (size_t i = 0; i < n; i++) {
            float ms = 0.f;
            cudaEventSynchronize(sl.stops[i]);
            cudaEventElapsedTime(&ms, sl.starts[i], sl.stops[i]);
            sl.done_ms += ms;
            sl.done_count++;
            g_event_pool.push_back(sl.starts[i]);
            g_event_pool.push_back(sl.stops[i]);
        }
        sl.starts.erase(sl.starts.begin(), sl.starts.begin() + n);
        sl.stops.erase(sl.stops.begin(), sl.stops.begin() + n);
    }
}

}  // namespace femgb

extern "C" int fem_profile_enable(int on)
{
    std::lock_guard<std::mutex> lk(femgb::g_prof_mu);
    femgb::prof_collect();
    femgb::g_prof_on = on != 0;
    if (on) femgb::g_prof.clear();
    return 0;
}

extern "C" int fem_profile_read(const char* kernel, double* total_ms, unsigned long long* launches)
{
    std::lock_guard<std::mutex> lk(femgb::g_prof_mu);
    femgb::prof_collect();
    auto it = femgb::g_prof.find(kernel ? kernel : "");
    if (total_ms) *total_ms = it == femgb::g_prof.end() ? 0.0 : it->second.done_ms;
    if (launches) *launches = it == femgb::g_prof.end() ? 0ull : it->second.done_count;
    return 0;
}

namespace femgb {

uint64_t& launch_counter()
{
    static uint64_t n = 0;
    return n;
}

uint32_t grid_for(uint32_t n)
{
    uint32_t g = (n + kBlock - 1) / kBlock;
    if (g < 1) g = 1;
    if (g > 4096) g = 4096;
    return g;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum with a fixed tree; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_sum(v);
    return v;
}

template <typename S>
__device__ __forceinline__ void load_elem(const MeshView<S>& m, uint32_t e, S* R, S* Di, S& k1, S& knu, S& k2)
{
    const size_t T = m.T;
#pragma unroll
    for (int c = 0; c < 9; c++) R[c] = m.R[c * T + e];
#pragma unroll
    for (int c = 0; c < 9; c++) Di[c] = m.Dinv[c * T + e];
    k1 = m.mat[e];
    knu = m.mat[T + e];
    k2 = m.mat[2 * T + e];
}

// ---- C_LCM element kernels (csrc/lcm.cuh): the material's force from the
// stored F of the last evaluation (T x 9, row-major per element), its
// truncated differential, its energy. Same eout convention as the C_WRP
// kernels below. ----

__device__ __forceinline__ void load_R_Dinv(const MeshView<double>& m, uint32_t e, double* R, double* Di)
{
    const size_t T = m.T;
#pragma unroll
    for (int c = 0; c < 9; c++) {
        R[c] = m.R[c * T + e];
        Di[c] = m.Dinv[c * T + e];
    }
}

__global__ void k_elem_lcm_force_fp64(MeshView<double> m, const double* __restrict__ F, PkMaterial mat,
                                      int write_out, double* energy_partials)
{
    double energy = 0.0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        double R[9], Di[9], Fl[9];
        load_R_Dinv(m, e, R, Di);
#pragma unroll
        for (int c = 0; c < 9; c++) Fl[c] = F[9 * (size_t)e + c];
        if (write_out) {
            double out[12];
            pk_force(mat, R, Fl, Di, m.vol[e], out);
            double* o = m.eout + 12 * (size_t)e;
#pragma unroll
            for (int c = 0; c < 12; c++) o[c] = out[c];
        }
        if (energy_partials) energy += pk_energy(mat, R, Fl, m.vol[e]);
    }
    if (energy_partials) {
        double s = block_sum(energy);
        if (threadIdx.x == 0) energy_partials[blockIdx.x] = s;
    }
}

__global__ void k_elem_lcm_spmv_fp64(MeshView<double> m, const double* __restrict__ d, const double* __restrict__ F,
                                     PkMaterial mat, const StepScalars* st, int check_done)
{
    if (check_done && st->done) return;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        const int ids[4] = {(int)bounds_idx((uint32_t)t.x, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.y, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.z, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.w, m.N, kSiteElemNode)};
        double R[9], Di[9], dl[12];
        load_R_Dinv(m, e, R, Di);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            dl[3 * i] = d[3 * (size_t)ids[i]];
            dl[3 * i + 1] = d[3 * (size_t)ids[i] + 1];
            dl[3 * i + 2] = d[3 * (size_t)ids[i] + 2];
        }
        double Fl[9];
        if (mat.kind != 1) {  // C_LCMH and C_CCM read F (and C_CCM det F)
#pragma unroll
            for (int c = 0; c < 9; c++) Fl[c] = F[9 * (size_t)e + c];
        }
        double out[12];
        pk_dforce(mat, R, Fl, mat.kind == 3 ? m.detF[e] : 0.0, Di, m.vol[e], dl, out);
        double* o = m.eout + 12 * (size_t)e;
#pragma unroll
        for (int c = 0; c < 12; c++) o[c] = out[c];
    }
}

// ---- element kernels ----

__global__ void k_elem_spmv_fp64(MeshView<double> m, const double* __restrict__ d, const StepScalars* st,
                                 int check_done)
{
    if (check_done && st->done) return;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        double R[9], Di[9], k1, knu, k2;
        load_elem(m, e, R, Di, k1, knu, k2);
        double dl[12];
        const int ids[4] = {(int)bounds_idx((uint32_t)t.x, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.y, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.z, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.w, m.N, kSiteElemNode)};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            dl[3 * i] = d[3 * (size_t)ids[i]];
            dl[3 * i + 1] = d[3 * (size_t)ids[i] + 1];
            dl[3 * i + 2] = d[3 * (size_t)ids[i] + 2];
        }
        double out[12];
        elem_RKRt(R, Di, k1, knu, k2, dl, out);
        double* o = m.eout + 12 * (size_t)e;
#pragma unroll
        for (int c = 0; c < 12; c++) o[c] = out[c];
    }
}

// R K0 (R^T x - r) per element (C_f_e's product); optional eout write and
// per-block elastic-energy partial 0.5 * u^T K0 u (C_V).
__global__ void k_elem_force_fp64(MeshView<double> m, const double* __restrict__ x, int write_out,
                                  double* energy_partials)
{
    double energy = 0.0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        double R[9], Di[9], k1, knu, k2;
        load_elem(m, e, R, Di, k1, knu, k2);
        const int ids[4] = {(int)bounds_idx((uint32_t)t.x, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.y, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.z, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.w, m.N, kSiteElemNode)};
        double u[12];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const size_t n = ids[i];
            const double xa = x[3 * n], xb = x[3 * n + 1], xc = x[3 * n + 2];
            // u_i = R^T x_i - r_i (accumulator from zero, as the reference)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                double acc = 0.0;
                acc += R[a] * xa;
                acc += R[3 + a] * xb;
                acc += R[6 + a] * xc;
                u[3 * i + a] = acc - m.rest[3 * n + a];
            }
        }
        double D[9];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int j = 0; j < 3; j++) D[3 * a + j] = u[3 * (j + 1) + a] - u[a];
        double H[9];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) H[3 * a + b] = D[3 * a] * Di[b] + D[3 * a + 1] * Di[3 + b] + D[3 * a + 2] * Di[6 + b];
        double P[9], es;
        stress_forces(H, Di, k1, knu, k2, P, es);
        energy += 0.5 * es;
        if (write_out) {
            double out[12];
            rotate_out(R, P, out);
            double* o = m.eout + 12 * (size_t)e;
#pragma unroll
            for (int c = 0; c < 12; c++) o[c] = out[c];
        }
    }
    if (energy_partials) {
        double s = block_sum(energy);
        if (threadIdx.x == 0) energy_partials[blockIdx.x] = s;
    }
}

// Potential energy term of RecomputeEnergy (LeafDSH_Solid3D_FEM.cpp:1554-1584):
// sum_e (rho V_e / 4) (x0+x1+x2+x3) . (-g)
__global__ void k_potential_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ x, double* partials)
{
    double acc = 0.0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < m.T; e += gridDim.x * blockDim.x) {
        const int4 t = m.tets[e];
        const int ids[4] = {(int)bounds_idx((uint32_t)t.x, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.y, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.z, m.N, kSiteElemNode),
                            (int)bounds_idx((uint32_t)t.w, m.N, kSiteElemNode)};
        double s[3] = {0, 0, 0};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int a = 0; a < 3; a++) s[a] += x[3 * (size_t)ids[i] + a];
        double em = c.density * m.vol[e];
        acc += (em / 4.0) * (s[0] * -c.gravity[0] + s[1] * -c.gravity[1] + s[2] * -c.gravity[2]);
    }
    double v = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// ---- node kernels ----

__device__ __forceinline__ void gather3(const MeshView<double>& m, uint32_t n, double& a0, double& a1, double& a2)
{
    const uint32_t beg = m.csr_ptr[n], end = m.csr_ptr[n + 1];
    for (uint32_t j = beg; j < end; j++) {
        const double* o = m.eout + 3 * (size_t)bounds_idx(m.csr_idx[j], 4ull * m.T, kSiteCsrEntry);
        a0 += o[0];
        a1 += o[1];
        a2 += o[2];
    }
}

// K u at node n for the solvers' node kernels: the assembled row when the
// solid has one (9 FMAs per block), else the gather of the element outputs
// of the product the solver launched before.
__device__ __forceinline__ void node_Ku(const MeshView<double>& m, const double* __restrict__ u, uint32_t n,
                                        double& a0, double& a1, double& a2)
{
    if (m.bsr_val) {
        const uint32_t beg = m.bsr_row[n], end = m.bsr_row[n + 1];
        for (uint32_t k = beg; k < end; k++) {
            const size_t j = 3 * (size_t)bounds_idx(m.bsr_col[k], m.N, kSiteBsrEntry);
            const double* A = m.bsr_val + 9 * (size_t)k;
            const double u0 = u[j], u1 = u[j + 1], u2 = u[j + 2];
            a0 = fma(A[0], u0, a0);
            a0 = fma(A[1], u1, a0);
            a0 = fma(A[2], u2, a0);
            a1 = fma(A[3], u0, a1);
            a1 = fma(A[4], u1, a1);
            a1 = fma(A[5], u2, a1);
            a2 = fma(A[6], u0, a2);
            a2 = fma(A[7], u1, a2);
            a2 = fma(A[8], u2, a2);
        }
    } else {
        gather3(m, n, a0, a1, a2);
    }
}

// One block of the assembled stiffness per thread (see
// launch_bsr_assemble_fp64). The element block in the element frame, from
// the strain form of elem_RKRt (g_i the shape gradients: rows of Dm^-1,
// node 0 minus their sum; k1 = V(lambda + 2 mu), knu = V lambda, k2 = V mu):
// K0[a][a] = k1 gi_a gj_a + k2 (gi.gj - gi_a gj_a),
// K0[a][b] = knu gi_a gj_b + k2 gj_a gi_b (a != b); the world block R K0 R^T.
__global__ void k_bsr_assemble_fp64(MeshView<double> m, uint32_t nnzb, const uint32_t* __restrict__ cptr,
                                    const uint32_t* __restrict__ contrib, double* __restrict__ val)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < nnzb; s += gridDim.x * blockDim.x) {
        double acc[9];
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] = 0.0;
        for (uint32_t k = cptr[s]; k < cptr[s + 1]; k++) {
            const uint32_t cb = contrib[k], e = bounds_idx(cb >> 4, m.T, kSiteBsrEntry);
            const uint32_t li = (cb >> 2) & 3u, lj = cb & 3u;
            double R[9], Di[9], k1, knu, k2;
            load_elem(m, e, R, Di, k1, knu, k2);
            double gi[3], gj[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double g0 = -(Di[c] + Di[3 + c] + Di[6 + c]);
                gi[c] = li == 0 ? g0 : (li == 1 ? Di[c] : (li == 2 ? Di[3 + c] : Di[6 + c]));
                gj[c] = lj == 0 ? g0 : (lj == 1 ? Di[c] : (lj == 2 ? Di[3 + c] : Di[6 + c]));
            }
            const double dot = gi[0] * gj[0] + gi[1] * gj[1] + gi[2] * gj[2];
            double K0[9];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    const double p = gi[a] * gj[b];
                    K0[3 * a + b] = a == b ? k1 * p + k2 * (dot - p) : knu * p + k2 * gj[a] * gi[b];
                }
            double T1[9];  // R K0
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++)
                    T1[3 * a + b] = R[3 * a] * K0[b] + R[3 * a + 1] * K0[3 + b] + R[3 * a + 2] * K0[6 + b];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++)
                    acc[3 * a + b] += T1[3 * a] * R[3 * b] + T1[3 * a + 1] * R[3 * b + 1] + T1[3 * a + 2] * R[3 * b + 2];
        }
        double* o = val + 9 * (size_t)s;
#pragma unroll
        for (int k = 0; k < 9; k++) o[k] = acc[k];
    }
}

// b = dt (m g + f_e) + m v ; y = v   (Step_QuasiImplicitEuler_v, :1211-1231)
__global__ void k_node_b_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ v, double* b, double* y)
{
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double f0 = 0, f1 = 0, f2 = 0;
        gather3(m, n, f0, f1, f2);
        const size_t i = 3 * (size_t)n;
        b[i] = (c.mass * c.gravity[0] - f0) * c.dt + c.mass * v[i];
        b[i + 1] = (c.mass * c.gravity[1] - f1) * c.dt + c.mass * v[i + 1];
        b[i + 2] = (c.mass * c.gravity[2] - f2) * c.dt + c.mass * v[i + 2];
        y[i] = v[i];
        y[i + 1] = v[i + 1];
        y[i + 2] = v[i + 2];
    }
}

// Position constraints -> clamped velocity, written to b and y
// (Step_QuasiImplicitEuler_v, LeafDSH_Solid3D_FEM.cpp:1268-1295).
__global__ void k_knc_fp64(uint32_t N, uint32_t count, const uint32_t* __restrict__ nodes,
                           const double* __restrict__ targets, const double* __restrict__ x, StepConsts c, double* b,
                           double* y)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const size_t n = bounds_idx(nodes[k], N, kSiteKncNode);
        V3<double> vk = mk<double>(c.inv_dt * (targets[3 * k] - x[3 * n]), c.inv_dt * (targets[3 * k + 1] - x[3 * n + 1]),
                                   c.inv_dt * (targets[3 * k + 2] - x[3 * n + 2]));
        double norm_vk = ::sqrt(dot0(vk, vk));
        V3<double> vel = mk<double>(0.0, 0.0, 0.0);
        if (norm_vk > (double)0.001f) {
            double cl = (norm_vk < 50.0) ? norm_vk : 50.0;
            vel = scale(cl, normalized(vk));
        }
        b[3 * n] = vel.x; b[3 * n + 1] = vel.y; b[3 * n + 2] = vel.z;
        y[3 * n] = vel.x; y[3 * n + 1] = vel.y; y[3 * n + 2] = vel.z;
    }
}

// r = S (b - A y) ; d = r ; partial |r|^2   (ILSS_CG.h:53-64)
__device__ __forceinline__ void fin_alpha(StepScalars* st, double total);
__device__ __forceinline__ void fin_beta(StepScalars* st, double total);

// The grid's total of the blocks' values (v in thread 0 of each), added in
// the block that finishes last: each block leaves its value in its slot and
// takes a ticket; the last one (true) adds the slots in order (a strided
// sum per thread, then the block tree) into thread 0's total and resets
// the ticket for the next kernel.
__device__ __forceinline__ bool grid_total_last(double v, double* partials, uint32_t* ticket, double& total)
{
    __shared__ bool last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc = 0.0;
    for (uint32_t i = threadIdx.x; i < gridDim.x; i += blockDim.x) acc += __ldcg(partials + i);
    total = block_sum(acc);
    if (threadIdx.x == 0) *ticket = 0;
    return true;
}

__global__ void k_node_residual_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ b,
                                     const double* __restrict__ y, double* r, double* d, double* partials)
{
    double acc = 0.0;
    const double mfm = c.mass * c.factor_M;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double s0 = 0, s1 = 0, s2 = 0;
        node_Ku(m, y, n, s0, s1, s2);
        const size_t i = 3 * (size_t)n;
        double r0 = 0, r1 = 0, r2 = 0;
        if (!m.fixed[n]) {
            r0 = b[i] - (c.factor_K * s0 + mfm * y[i]);
            r1 = b[i + 1] - (c.factor_K * s1 + mfm * y[i + 1]);
            r2 = b[i + 2] - (c.factor_K * s2 + mfm * y[i + 2]);
        }
        r[i] = r0; r[i + 1] = r1; r[i + 2] = r2;
        d[i] = r0; d[i + 1] = r1; d[i + 2] = r2;
        acc += r0 * r0 + r1 * r1 + r2 * r2;
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// q = S A d ; partial d.q   (ILSS_CG.h:90-96)
__global__ void k_node_q_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ d, double* q,
                              double* partials, StepScalars* st, cudaGraphConditionalHandle cond, int set_cond)
{
    if (st->done) return;
    double acc = 0.0;
    const double mfm = c.mass * c.factor_M;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double s0 = 0, s1 = 0, s2 = 0;
        node_Ku(m, d, n, s0, s1, s2);
        const size_t i = 3 * (size_t)n;
        double q0 = 0, q1 = 0, q2 = 0;
        if (!m.fixed[n]) {
            q0 = c.factor_K * s0 + mfm * d[i];
            q1 = c.factor_K * s1 + mfm * d[i + 1];
            q2 = c.factor_K * s2 + mfm * d[i + 2];
        }
        q[i] = q0; q[i + 1] = q1; q[i + 2] = q2;
        acc += d[i] * q0 + d[i + 1] * q1 + d[i + 2] * q2;
    }
    double total = 0.0;
    if (grid_total_last(block_sum(acc), partials, &st->fin_ticket, total) && threadIdx.x == 0) {
        fin_alpha(st, total);
        if (set_cond) cudaGraphSetConditional(cond, st->done ? 0u : 1u);
    }
}

// y += alpha d ; r -= alpha q ; partial |r|^2   (ILSS_CG.h:100-117)
__global__ void k_node_xr_fp64(uint32_t N, double* y, double* r, const double* __restrict__ d,
                               const double* __restrict__ q, double* partials, StepScalars* st,
                               cudaGraphConditionalHandle cond, int set_cond)
{
    if (st->done) return;
    const double alpha = st->alpha, na = -alpha;
    double acc = 0.0;
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        y[i] += alpha * d[i];
        double ri = r[i] + na * q[i];
        r[i] = ri;
        acc += ri * ri;
    }
    double total = 0.0;
    if (grid_total_last(block_sum(acc), partials, &st->fin_ticket, total) && threadIdx.x == 0) {
        fin_beta(st, total);
        if (set_cond) cudaGraphSetConditional(cond, st->done ? 0u : 1u);
    }
}

// d = S (beta d + r)   (ILSS_CG.h:133-137)
__global__ void k_node_d_fp64(uint32_t N, const uint8_t* __restrict__ fixed, double* d, const double* __restrict__ r,
                              const StepScalars* st)
{
    // Once the loop has ended (including an iteration that just ended it in
    // FIN_BETA) d is no longer read, so the update is skipped.
    if (st->done) return;
    const double beta = st->beta;
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const uint32_t n = i / 3;
        d[i] = fixed[n] ? 0.0 : beta * d[i] + r[i];
    }
}

// v = y ; x += dt y   (Step_QuasiImplicitEuler_v, :1322-1327)
__global__ void k_integrate_fp64(uint32_t N, double dt, double* x, double* v, const double* __restrict__ y)
{
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const double yi = y[i];
        v[i] = yi;
        x[i] = x[i] + dt * yi;
    }
}

// ---- fully-implicit Euler, Delta x form (LeafDSH_Solid3D_FEM.cpp:1357-1552) ----
// x holds the Newton iterate x_k, xn and vn the step's x^n and v^n; eout holds
// the element forces at x_k (k_elem_force_fp64 with the rotations of x_k).

// b = m g + f_e(x_k) + (inv_dt m) (v^n - inv_dt (x_k - x^n)) with f_p = 0 and
// f_d left out as in the reference (:1382-1401); y = dt v^n on the first
// Newton iteration (the warm start, :1406-1407), else 0.
__global__ void k_node_b_fie_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ x,
                                  const double* __restrict__ xn, const double* __restrict__ vn, int warm,
                                  double* b, double* y)
{
    const double im = c.inv_dt * c.mass;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double f[3] = {0, 0, 0};
        gather3(m, n, f[0], f[1], f[2]);
        const size_t i = 3 * (size_t)n;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double bf = c.mass * c.gravity[a] - f[a];
            b[i + a] = bf + im * (vn[i + a] - c.inv_dt * (x[i + a] - xn[i + a]));
            y[i + a] = warm ? c.dt * vn[i + a] : 0.0;
        }
    }
}

// Position constraints as Delta x rows: b = y = target - x_k (:1441-1465).
__global__ void k_knc_fie_fp64(uint32_t N, uint32_t count, const uint32_t* __restrict__ nodes,
                               const double* __restrict__ targets, const double* __restrict__ x, double* b,
                               double* y)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const size_t n = bounds_idx(nodes[k], N, kSiteKncNode);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double dx = targets[3 * k + a] - x[3 * n + a];
            b[3 * n + a] = dx;
            y[3 * n + a] = dx;
        }
    }
}

// partial sum of v_i^2 (real_array::sq_norm_2)
__global__ void k_sq_norm_fp64(uint32_t n, const double* __restrict__ v, double* partials)
{
    double acc = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += v[i] * v[i];
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// x_k += y ; v_k = inv_dt (x_k - x^n) ; partial |y|^2   (:1500-1512)
__global__ void k_fie_update_fp64(uint32_t N, double inv_dt, double* x, double* v, const double* __restrict__ xn,
                                  const double* __restrict__ y, double* partials)
{
    double acc = 0.0;
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const double yi = y[i];
        const double xi = x[i] + yi;
        x[i] = xi;
        v[i] = inv_dt * (xi - xn[i]);
        acc += yi * yi;
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// ---- MINRES (ILSS_MINRES::Solve, ILSS_MINRES.h:51-168), no preconditioner:
// w == v, w1 == v1. The host rotates the v0/v/v1 and p0/p buffers between
// iterations; every kernel is a no-op once the loop has ended.

// v1 = S (b - A y) ; partial |v1|^2   (:66-74)
__global__ void k_mr_init_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ b,
                               const double* __restrict__ y, double* v1, double* partials)
{
    double acc = 0.0;
    const double mfm = c.mass * c.factor_M;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double f[3] = {0, 0, 0};
        node_Ku(m, y, n, f[0], f[1], f[2]);
        const size_t i = 3 * (size_t)n;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double r = m.fixed[n] ? 0.0 : b[i + a] - (c.factor_K * f[a] + mfm * y[i + a]);
            v1[i + a] = r;
            acc += r * r;
        }
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// v1 *= 1/beta_new ; v = p = p0 = 0   (:82-95)
__global__ void k_mr_start_fp64(uint32_t N, double* v1, double* v, double* p, double* p0, const StepScalars* st)
{
    const double inv = 1.0 / st->mr.beta_new;
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        v1[i] *= inv;
        v[i] = 0.0;
        p[i] = 0.0;
        p0[i] = 0.0;
    }
}

// v1 = S A v - beta v0 ; partial v1.v   (:117-123)
__global__ void k_mr_q_fp64(MeshView<double> m, StepConsts c, const double* __restrict__ v,
                            const double* __restrict__ v0, double* v1, double* partials, const StepScalars* st)
{
    if (st->done) return;
    const double mfm = c.mass * c.factor_M;
    const double nb = -st->mr.beta_new;
    double acc = 0.0;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double f[3] = {0, 0, 0};
        node_Ku(m, v, n, f[0], f[1], f[2]);
        const size_t i = 3 * (size_t)n;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double q = m.fixed[n] ? 0.0 : c.factor_K * f[a] + mfm * v[i + a];
            const double w1 = q + nb * v0[i + a];
            v1[i + a] = w1;
            acc += w1 * v[i + a];
        }
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// v1 -= alpha v ; partial |v1|^2   (:125-129)
__global__ void k_mr_v1_fp64(uint32_t N, double* v1, const double* __restrict__ v, double* partials,
                             const StepScalars* st)
{
    if (st->done) return;
    const double na = -st->mr.alpha;
    double acc = 0.0;
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const double r = v1[i] + na * v[i];
        v1[i] = r;
        acc += r * r;
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// v1 *= 1/beta_new ; p_new = ((-r2) p + w + (-r3) p0) / r1 into p0's buffer ;
// y += beta_one c eta p_new   (:131-156)
__global__ void k_mr_update_fp64(uint32_t N, double* v1, const double* __restrict__ v,
                                 const double* __restrict__ p, double* p0, double* y, const StepScalars* st)
{
    if (st->done_prev) return;
    const MinresScalars mr = st->mr;
    const uint32_t n3 = 3 * N;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        v1[i] *= mr.inv_beta;
        double pn = mr.neg_r2 * p[i] + v[i];
        pn += mr.neg_r3 * p0[i];
        pn *= mr.inv_r1;
        p0[i] = pn;
        y[i] += mr.x_coef * pn;
    }
}

// q = S (factor_M M d + factor_K sum R K R^T d) using a fresh eout
__global__ void k_apply_A_fp64(MeshView<double> m, double factor_M, double factor_K, double mass,
                               const double* __restrict__ d, double* q)
{
    const double mfm = mass * factor_M;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double s0 = 0, s1 = 0, s2 = 0;
        gather3(m, n, s0, s1, s2);
        const size_t i = 3 * (size_t)n;
        if (m.fixed[n]) { q[i] = 0; q[i + 1] = 0; q[i + 2] = 0; continue; }
        q[i] = factor_K * s0 + mfm * d[i];
        q[i + 1] = factor_K * s1 + mfm * d[i + 1];
        q[i + 2] = factor_K * s2 + mfm * d[i + 2];
    }
}

// f += sign * sum(eout) per node
// Material triple of every element from one E, nu (k_c = a (1 - nu), a nu,
// a (0.5 - nu), formed on the host): mat[c][e] = V_e k_c, the product
// EditableTetrahedronElementSet3::SetParams re-bakes for every element
// (TetrahedronElementSet3.cpp:2168-2200).
__global__ void k_rebake_material_fp64(uint32_t T, const double* __restrict__ vol, double k0, double k1, double k2,
                                       double* mat)
{
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < T; e += gridDim.x * blockDim.x) {
        const double V = vol[e];
        mat[e] = V * k0;
        mat[(size_t)T + e] = V * k1;
        mat[2 * (size_t)T + e] = V * k2;
    }
}

void launch_rebake_material_fp64(uint32_t T, const double* vol, double k0, double k1, double k2, double* mat,
                                 cudaStream_t s)
{
    k_rebake_material_fp64<<<grid_for(T), kBlock, 0, s>>>(T, vol, k0, k1, k2, mat);
    launch_counter()++;
}

__global__ void k_gather_sum_fp64(MeshView<double> m, double sign, double* f)
{
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < m.N; n += gridDim.x * blockDim.x) {
        double s0 = 0, s1 = 0, s2 = 0;
        gather3(m, n, s0, s1, s2);
        f[3 * (size_t)n] += sign * s0;
        f[3 * (size_t)n + 1] += sign * s1;
        f[3 * (size_t)n + 2] += sign * s2;
    }
}

// ---- finalizers (one block) ----

__device__ __forceinline__ bool cg_continue(const StepScalars* st)
{
    return st->delta_new > st->abs_eps_sq && st->delta_new > st->delta_target && st->k < st->max_iter;
}

// ILSS_CG::Solve's scalar steps (ILSS_CG.h:53-151) on a reduced total: the
// start, alpha with the breakdown test, beta with the loop test, and the
// statistics at the end. Shared by the finaliser kernel and the one-block
// solver below.
__device__ __forceinline__ void fin_init(StepScalars* st, const StepConsts& c, double total)
{
    st->delta_0 = total;
    st->delta_new = total;
    st->delta_old = total;
    st->delta_target = c.rel_eps_sq * total;
    st->abs_eps_sq = c.abs_eps_sq;
    st->max_iter = c.max_iter;
    st->k = 0;
    st->status = 0;
    st->alpha = 0.0;
    st->beta = 0.0;
    st->done = cg_continue(st) ? 0u : 1u;
    if (!isfinite(total)) st->status = 3;  // FEM_E_NAN
}
__device__ __forceinline__ void fin_alpha(StepScalars* st, double total)
{
    if (st->done) return;
    st->dot_dq = total;
    if (::fabs(total) < st->abs_eps_sq) {  // breakdown: leave before the update (ILSS_CG.h:97)
        st->done = 1;
        return;
    }
    st->alpha = st->delta_new / total;
}
__device__ __forceinline__ void fin_beta(StepScalars* st, double total)
{
    if (st->done) return;
    st->delta_old = st->delta_new;
    st->delta_new = total;
    st->beta = total / st->delta_old;
    st->k += 1;
    st->total_iters += 1;
    st->done = cg_continue(st) ? 0u : 1u;
    if (!isfinite(total)) st->status = 3;
}
__device__ __forceinline__ void fin_stats(StepScalars* st)
{
    st->rel_residual = (st->delta_0 > 0) ? ::sqrt(st->delta_new / st->delta_0) : 0.0;
    st->abs_residual = ::sqrt(st->delta_new);
}

__global__ void k_finalize(int kind, const double* __restrict__ partials, uint32_t count, StepConsts c,
                           StepScalars* st, cudaGraphConditionalHandle cond, int set_cond)
{
    double acc = 0.0;
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) acc += partials[i];
    const double total = block_sum(acc);
    if (threadIdx.x != 0) return;
    switch (kind) {
    case FIN_INIT:
        fin_init(st, c, total);
        break;
    case FIN_ALPHA:
        fin_alpha(st, total);
        break;
    case FIN_BETA:
        fin_beta(st, total);
        break;
    case FIN_ENERGY_E:
        st->elastic_energy = total;
        break;
    case FIN_ENERGY_P:
        st->potential_energy = total;
        break;
    case FIN_SUM:
        st->host_sum = total;
        break;
    case FIN_MR_INIT: {
        // |r0|^2 (sq_norm_2 and dot(v1, w1) are the same sum); |b|^2 from the
        // FIN_SUM before; beta_one = |r0| (:74-107)
        MinresScalars& mr = st->mr;
        minres_start(mr, total);
        mr.norm_b_sq = st->host_sum;
        st->delta_0 = mr.norm_b_sq;
        st->delta_target = c.rel_eps_sq * mr.norm_b_sq;
        st->abs_eps_sq = c.abs_eps_sq;
        st->max_iter = c.max_iter;
        st->k = 0;
        st->status = 0;
        st->done = (mr.norm_r_sq > st->abs_eps_sq && mr.norm_r_sq > st->delta_target && st->k < st->max_iter) ? 0u : 1u;
        st->done_prev = st->done;
        if (!isfinite(total)) st->status = 3;
        break;
    }
    case FIN_MR_ALPHA:
        st->done_prev = st->done;
        if (st->done) break;
        st->mr.beta = st->mr.beta_new;
        st->mr.alpha = total;
        break;
    case FIN_MR_BETA: {
        if (st->done) break;
        MinresScalars& mr = st->mr;
        minres_givens(mr, total);  // Givens rotation (:135-144)
        st->delta_new = mr.norm_r_sq;
        st->k += 1;
        st->total_iters += 1;
        st->done = (mr.norm_r_sq > st->abs_eps_sq && mr.norm_r_sq > st->delta_target && st->k < st->max_iter) ? 0u : 1u;
        if (!isfinite(total) || !isfinite(mr.norm_r_sq)) st->status = 3;
        break;
    }
    case FIN_MR_STATS:
        st->rel_residual = ::sqrt(st->mr.norm_r_sq / st->mr.norm_b_sq);
        st->abs_residual = ::sqrt(st->mr.norm_r_sq);
        break;
    case FIN_STATS:
        fin_stats(st);
        break;
    }
    if (set_cond && (kind == FIN_INIT || kind == FIN_ALPHA || kind == FIN_BETA || kind == FIN_MR_INIT ||
                     kind == FIN_MR_ALPHA || kind == FIN_MR_BETA))
        cudaGraphSetConditional(cond, st->done ? 0u : 1u);
}

// elem_RKRt over three lanes of a warp (lane a of lanes 3g..3g+2 computes
// component a): u_i = R^T d_i, the element-frame gradient row a, the stress
// row a after exchanging the gradient's diagonal and column a, the force
// row a, and after exchanging the force rows component a of R P (node 0:
// minus the sum). About 50 FP64 instructions per lane against 140 for one
// lane; GB300 gives a warp's FP64 instruction about 64 clocks whatever the
// lanes, so a few warps of elements take a third of the time. Every lane of
// the warp must call it (invalid lanes with zeros); out4 = component a of
// nodes 0..3.
// Rc: column a of R; Rr: row a of R as (R[a][a], R[a][a+1], R[a][a+2])
// (indexes mod 3).
__device__ __forceinline__ void elem_RKRt_lanes(const double* Rc, const double* Rr, const double* Di, double k1,
                                                double knu, double k2, const double* d, uint32_t a, uint32_t base,
                                                double* out4)
{
    const uint32_t l1 = base + (a == 2 ? 0u : a + 1), l2 = base + (a == 0 ? 2u : a - 1);  // lanes of a+1, a+2 (mod 3)
    double u[4];
#pragma unroll
    for (int i = 0; i < 4; i++) u[i] = Rc[0] * d[3 * i] + Rc[1] * d[3 * i + 1] + Rc[2] * d[3 * i + 2];
    const double D0 = u[1] - u[0], D1 = u[2] - u[0], D2 = u[3] - u[0];
    double H[3];  // row a of the element-frame gradient
#pragma unroll
    for (int b = 0; b < 3; b++) H[b] = D0 * Di[b] + D1 * Di[3 + b] + D2 * Di[6 + b];
    // the lane of component b sends H[b][a'] for the receiver a' = b - 1 or b - 2
    const double Ha = a == 0 ? H[0] : (a == 1 ? H[1] : H[2]);
    const double send1 = a == 0 ? H[2] : (a == 1 ? H[0] : H[1]);  // to a - 1
    const double send2 = a == 0 ? H[1] : (a == 1 ? H[2] : H[0]);  // to a - 2
    const double e1 = __shfl_sync(0xffffffffu, Ha, l1), e2 = __shfl_sync(0xffffffffu, Ha, l2);
    const double c1 = __shfl_sync(0xffffffffu, send1, l1), c2 = __shfl_sync(0xffffffffu, send2, l2);
    const double h1 = a == 0 ? H[1] : (a == 1 ? H[2] : H[0]), h2 = a == 0 ? H[2] : (a == 1 ? H[0] : H[1]);
    const double saa = k1 * Ha + knu * (e1 + e2);
    const double s1 = k2 * (h1 + c1), s2 = k2 * (h2 + c2);
    double Sg[3];  // row a of the stress
    Sg[0] = a == 0 ? saa : (a == 1 ? s2 : s1);
    Sg[1] = a == 1 ? saa : (a == 2 ? s2 : s1);
    Sg[2] = a == 2 ? saa : (a == 0 ? s2 : s1);
    double P[3];
#pragma unroll
    for (int i = 0; i < 3; i++) P[i] = Sg[0] * Di[3 * i] + Sg[1] * Di[3 * i + 1] + Sg[2] * Di[3 * i + 2];
    double Q1[3], Q2[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        Q1[i] = __shfl_sync(0xffffffffu, P[i], l1);
        Q2[i] = __shfl_sync(0xffffffffu, P[i], l2);
    }
    double w[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        w[i] = Rr[0] * P[i] + Rr[1] * Q1[i] + Rr[2] * Q2[i];
        out4[i + 1] = w[i];
    }
    out4[0] = -(w[0] + w[1] + w[2]);
}

// The whole of ILSS_CG::Solve (ILSS_CG.h:38-151) for a C_WRP solid of up to
// kCgClusterMaxCtas x kCgClusterMaxThreads tets on one thread-block cluster,
// on chip. CTA r owns the elements [r ept, (r+1) ept) and the nodes
// [r npt, (r+1) npt): a thread (kSplit: three lanes, elem_RKRt_lanes)
// keeps one element's R, Dm^-1 and material scalars in registers and its
// element output in its CTA's shared memory; the CTA keeps its nodes' y,
// r, d, q, b, CSR rows and fixed flags. An element product reads its four
// nodes' d from the owning CTAs' shared memory (distributed shared memory);
// a node component's gather (one thread per component) reads its element
// corners' outputs the same way (ent: per CSR entry, the owning CTA << 24 |
// its local corner). A reduction sums each CTA's block total into a slot of
// every CTA, then every CTA adds the slots in rank order, so all CTAs take
// the same scalar steps and leave the loop together. Four cluster barriers
// per iteration: element outputs complete, d.q, |r|^2, the new d. y and the
// statistics are written back at the end; the loop ends on the solver's own
// tests (at most max_iter iterations).
template <int kSplit>
__global__ void __launch_bounds__(kCgClusterMaxThreads, 1)
    k_cg_cluster_fp64(MeshView<double> m, StepConsts c, CgClusterPlan p, const uint32_t* __restrict__ ent,
                      const double* __restrict__ b, double* y, StepScalars* st)
{
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    extern __shared__ __align__(16) unsigned char cl_smem[];
    const uint32_t tid = threadIdx.x, nt = blockDim.x, rank = cl.block_rank(), C = p.ctas;
    const uint32_t N = m.N, T = m.T;
    const uint32_t e0 = rank * p.ept, n0 = rank * p.npt;
    const uint32_t ne = e0 < T ? min(p.ept, T - e0) : 0u, nn = n0 < N ? min(p.npt, N - n0) : 0u, n3 = 3 * nn;
    const size_t v3 = 3 * (size_t)p.npt;
    double* eo = reinterpret_cast<double*>(cl_smem);  // [12 ept]
    double* vy = eo + 12 * (size_t)p.ept;               // [3 npt] each
    double* vr = vy + v3;
    double* vd = vr + v3;
    double* vq = vd + v3;
    double* vb = vq + v3;
    double* part = vb + v3;                                   // [3][kCgClusterMaxCtas]
    uint32_t* cptr = reinterpret_cast<uint32_t*>(part + 3 * kCgClusterMaxCtas);  // [npt + 1]
    uint32_t* cent = cptr + p.npt + 1;                                          // [ent_max]
    uint8_t* fx = reinterpret_cast<uint8_t*>(cent + p.ent_max);                 // [npt]
    __shared__ StepScalars sst;
    const double mfm = c.mass * c.factor_M;
    const uint32_t base = nn ? m.csr_ptr[n0] : 0u;
    for (uint32_t i = tid; i < n3; i += nt) {
        vy[i] = y[3 * (size_t)n0 + i];
        vb[i] = b[3 * (size_t)n0 + i];
    }
    for (uint32_t i = tid; i <= nn; i += nt) cptr[i] = nn ? m.csr_ptr[n0 + i] - base : 0u;
    const uint32_t ne_ent = nn ? min(m.csr_ptr[n0 + nn] - base, p.ent_max) : 0u;
    for (uint32_t i = tid; i < ne_ent; i += nt) cent[i] = ent[base + i];
    for (uint32_t i = tid; i < nn; i += nt) fx[i] = m.fixed[n0 + i];
    if (tid == 0) sst = *st;
    // this thread's element and where its nodes live: element tid, or with
    // kSplit lane 3g + a (a < 3, g < 10) of warp w takes component a of
    // element 10 w + g
    const uint32_t lane = tid & 31, ca = kSplit ? lane % 3 : 0u, cbase = lane - ca;
    const uint32_t le = kSplit ? (lane < 30 ? 10 * (tid >> 5) + lane / 3 : 0xffffffffu) : tid;
    const bool has_elem = le < ne;
    double R[9], Di[9], k1 = 0, knu = 0, k2 = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) R[k] = Di[k] = 0.0;
    double Rc[3] = {0, 0, 0}, Rr[3] = {0, 0, 0};  // kSplit: column a of R, row a from (a, a)
    uint32_t nr[4] = {0, 0, 0, 0}, nl[4] = {0, 0, 0, 0};
    if (has_elem) {
        load_elem(m, e0 + le, R, Di, k1, knu, k2);
        if constexpr (kSplit != 0) {
            double row[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                Rc[k] = ca == 0 ? R[3 * k] : (ca == 1 ? R[3 * k + 1] : R[3 * k + 2]);
                row[k] = ca == 0 ? R[k] : (ca == 1 ? R[3 + k] : R[6 + k]);
            }
            Rr[0] = ca == 0 ? row[0] : (ca == 1 ? row[1] : row[2]);
            Rr[1] = ca == 0 ? row[1] : (ca == 1 ? row[2] : row[0]);
            Rr[2] = ca == 0 ? row[2] : (ca == 1 ? row[0] : row[1]);
        }
        const int4 t = m.tets[e0 + le];
        const uint32_t ids[4] = {bounds_idx((uint32_t)t.x, N, kSiteElemNode), bounds_idx((uint32_t)t.y, N, kSiteElemNode),
                                 bounds_idx((uint32_t)t.z, N, kSiteElemNode), bounds_idx((uint32_t)t.w, N, kSiteElemNode)};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            nr[k] = ids[k] / p.npt;
            nl[k] = 3 * (ids[k] - nr[k] * p.npt);
        }
    }
    const double* pd[4];
#pragma unroll
    for (int k = 0; k < 4; k++) pd[k] = cl.map_shared_rank(vd, nr[k]) + nl[k];
    cl.sync();  // every CTA's y, d and CSR rows are in place
    auto elem_products = [&](const double* const* u) {
        double dl[12];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            dl[3 * k] = has_elem ? u[k][0] : 0.0;
            dl[3 * k + 1] = has_elem ? u[k][1] : 0.0;
            dl[3 * k + 2] = has_elem ? u[k][2] : 0.0;
        }
        if constexpr (kSplit != 0) {
            double o4[4];
            elem_RKRt_lanes(Rc, Rr, Di, k1, knu, k2, dl, ca, cbase, o4);
            if (has_elem)
#pragma unroll
                for (int k = 0; k < 4; k++) eo[12 * le + 3 * k + ca] = o4[k];
        } else if (has_elem) {
            double out[12];
            elem_RKRt(R, Di, k1, knu, k2, dl, out);
#pragma unroll
            for (int k = 0; k < 12; k++) eo[12 * le + k] = out[k];
        }
        cl.sync();  // all element outputs complete
    };
    // component a of node ln's element sum
    auto gather = [&](uint32_t ln, uint32_t a) {
        const uint32_t jend = min(cptr[ln + 1], ne_ent);
        double acc = 0.0;
#pragma unroll 4
        for (uint32_t j = cptr[ln]; j < jend; j++) {
            const uint32_t e = cent[j];
            acc += cl.map_shared_rank(eo, e >> 24)[3 * (e & 0xffffffu) + a];
        }
        return acc;
    };
    // the cluster's total of every thread's acc (valid in thread 0)
    // (each FP64 add costs a warp about 64 clocks: the CTA's warp totals and
    // the CTAs' totals are added in shuffle trees of log2 depth, the same
    // fixed trees in every CTA)
    __shared__ double wsum[kCgClusterMaxThreads / 32];
    const uint32_t nw = nt >> 5;
    const uint32_t wtop = nw > 1 ? 1u << (31 - __clz(nw - 1)) : 0u, ctop = C > 1 ? 1u << (31 - __clz(C - 1)) : 0u;
    auto cluster_total = [&](double acc, int slot) -> double {
        double v = warp_sum(acc);
        if (lane == 0) wsum[tid >> 5] = v;
        __syncthreads();
        if (tid < 32) {
            v = lane < nw ? wsum[lane] : 0.0;
            for (uint32_t o = wtop; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            v = __shfl_sync(0xffffffffu, v, 0);
            if (lane < C) cl.map_shared_rank(part, lane)[slot * kCgClusterMaxCtas + rank] = v;
        }
        cl.sync();
        double total = 0.0;
        if (tid < 32) {
            total = lane < C ? part[slot * kCgClusterMaxCtas + lane] : 0.0;
            for (uint32_t o = ctop; o >= 1; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
        }
        return total;
    };
    // r = S(b - A y), d = r, |r|^2
    {
        const double* py[4];
#pragma unroll
        for (int k = 0; k < 4; k++) py[k] = cl.map_shared_rank(vy, nr[k]) + nl[k];
        elem_products(py);
    }
    double acc = 0.0;
    for (uint32_t i = tid; i < n3; i += nt) {
        const uint32_t ln = i / 3;
        const double s = gather(ln, i - 3 * ln);
        const double ri = fx[ln] ? 0.0 : vb[i] - (c.factor_K * s + mfm * vy[i]);
        vr[i] = ri;
        vd[i] = ri;
        acc += ri * ri;
    }
    double total = cluster_total(acc, 0);
    if (tid == 0) fin_init(&sst, c, total);
    __syncthreads();
    while (!sst.done) {
        // q = S A d, d.q, alpha
        elem_products(pd);
        acc = 0.0;
        for (uint32_t i = tid; i < n3; i += nt) {
            const uint32_t ln = i / 3;
            const double s = gather(ln, i - 3 * ln);
            const double qi = fx[ln] ? 0.0 : c.factor_K * s + mfm * vd[i];
            vq[i] = qi;
            acc += vd[i] * qi;
        }
        total = cluster_total(acc, 1);
        if (tid == 0) fin_alpha(&sst, total);
        __syncthreads();
        if (sst.done) break;
        // y += alpha d, r -= alpha q, |r|^2, beta and the loop test
        const double alpha = sst.alpha, na = -alpha;
        acc = 0.0;
        for (uint32_t i = tid; i < n3; i += nt) {
            vy[i] += alpha * vd[i];
            const double ri = vr[i] + na * vq[i];
            vr[i] = ri;
            acc += ri * ri;
        }
        total = cluster_total(acc, 2);
        if (tid == 0) fin_beta(&sst, total);
        __syncthreads();
        if (sst.done) break;
        // d = S (beta d + r)
        const double beta = sst.beta;
        for (uint32_t i = tid; i < n3; i += nt) vd[i] = fx[i / 3] ? 0.0 : beta * vd[i] + vr[i];
        cl.sync();  // the new d is complete
    }
    for (uint32_t i = tid; i < n3; i += nt) y[3 * (size_t)n0 + i] = vy[i];
    if (rank == 0 && tid == 0) {
        fin_stats(&sst);
        *st = sst;
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

size_t cg_cluster_smem_bytes(uint32_t ept, uint32_t npt, uint32_t ent_max)
{
    return sizeof(double) * (12 * (size_t)ept + 15 * (size_t)npt + 3 * kCgClusterMaxCtas) +
           sizeof(uint32_t) * ((size_t)npt + 1 + ent_max) + npt;
}

namespace {
template <int kSplit>
cudaError_t cg_cluster_attrs()
{
    static const cudaError_t e = [] {
        cudaError_t r = cudaFuncSetAttribute(k_cg_cluster_fp64<kSplit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kCgClusterMaxSmem);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(k_cg_cluster_fp64<kSplit>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        return r;
    }();
    return e;
}
void cluster_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute& at, const CgClusterPlan& p, cudaStream_t s)
{
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = dim3(p.ctas);
    cfg.blockDim = dim3(p.threads);
    cfg.dynamicSmemBytes = p.smem;
    cfg.stream = s;
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = p.ctas;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
}
}  // namespace

bool cg_cluster_fits(const CgClusterPlan& p)
{
    if (p.ctas < 1 || p.ctas > kCgClusterMaxCtas || p.threads < 32 || p.threads > kCgClusterMaxThreads ||
        p.threads % 32 || p.smem > kCgClusterMaxSmem ||
        p.ept > (p.split ? 10 * (p.threads / 32) : p.threads) ||
        (p.split ? cg_cluster_attrs<1>() : cg_cluster_attrs<0>()) != cudaSuccess)
        return false;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at;
    cluster_config(cfg, at, p, nullptr);
    int n = 0;
    const cudaError_t e = p.split ? cudaOccupancyMaxActiveClusters(&n, k_cg_cluster_fp64<1>, &cfg)
                                  : cudaOccupancyMaxActiveClusters(&n, k_cg_cluster_fp64<0>, &cfg);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n >= 1;
}

cudaError_t launch_cg_cluster_fp64(const MeshView<double>& m, const StepConsts& c, const CgClusterPlan& p,
                                   const uint32_t* ent, const double* b, double* y, StepScalars* st, cudaStream_t s)
{
    cudaError_t e = p.split ? cg_cluster_attrs<1>() : cg_cluster_attrs<0>();
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute at;
    cluster_config(cfg, at, p, s);
    e = p.split ? cudaLaunchKernelEx(&cfg, k_cg_cluster_fp64<1>, m, c, p, ent, b, y, st)
                : cudaLaunchKernelEx(&cfg, k_cg_cluster_fp64<0>, m, c, p, ent, b, y, st);
    launch_counter()++;
    return e;
}

// ---- launchers ----

#define FEMGB_LAUNCH(kernel, grid, ...)                                   \
    do {                                                                  \
        kernel<<<(grid), kBlock, 0, s>>>(__VA_ARGS__);                    \
        launch_counter()++;                                               \
    } while (0)

void launch_elem_spmv_fp64(const MeshView<double>& m, const double* d, const StepScalars* st, int check_done,
                           cudaStream_t s)
{
    prof_begin("elem_spmv_fp64", s);
    FEMGB_LAUNCH(k_elem_spmv_fp64, grid_for(m.T), m, d, st, check_done);
    prof_end("elem_spmv_fp64", s);
}
void launch_elem_force_fp64(const MeshView<double>& m, const double* x, int write_out, double* energy_partials,
                            cudaStream_t s)
{
    FEMGB_LAUNCH(k_elem_force_fp64, grid_for(m.T), m, x, write_out, energy_partials);
}
void launch_node_b_fp64(const MeshView<double>& m, const StepConsts& c, const double* v, double* b, double* y,
                        cudaStream_t s)
{
    FEMGB_LAUNCH(k_node_b_fp64, grid_for(m.N), m, c, v, b, y);
}
void launch_knc_fp64(uint32_t N, uint32_t count, const uint32_t* nodes, const double* targets, const double* x,
                     const StepConsts& c, double* b, double* y, cudaStream_t s)
{
    if (count == 0) return;
    FEMGB_LAUNCH(k_knc_fp64, grid_for(count), N, count, nodes, targets, x, c, b, y);
}
void launch_node_residual_fp64(const MeshView<double>& m, const StepConsts& c, const double* b, const double* y,
                               double* r, double* d, double* partials, cudaStream_t s)
{
    FEMGB_LAUNCH(k_node_residual_fp64, grid_for(m.N), m, c, b, y, r, d, partials);
}
void launch_node_q_fp64(const MeshView<double>& m, const StepConsts& c, const double* d, double* q,
                        double* partials, StepScalars* st, cudaStream_t s, cudaGraphConditionalHandle cond,
                        int set_cond)
{
    prof_begin("node_q_fp64", s);
    FEMGB_LAUNCH(k_node_q_fp64, grid_for(m.N), m, c, d, q, partials, st, cond, set_cond);
    prof_end("node_q_fp64", s);
}
void launch_node_xr_fp64(uint32_t N, double* y, double* r, const double* d, const double* q, double* partials,
                         StepScalars* st, cudaStream_t s, cudaGraphConditionalHandle cond, int set_cond)
{
    FEMGB_LAUNCH(k_node_xr_fp64, grid_for(3 * N), N, y, r, d, q, partials, st, cond, set_cond);
}
void launch_node_d_fp64(uint32_t N, const uint8_t* fixed, double* d, const double* r, const StepScalars* st,
                        cudaStream_t s)
{
    FEMGB_LAUNCH(k_node_d_fp64, grid_for(3 * N), N, fixed, d, r, st);
}
void launch_integrate_fp64(uint32_t N, double dt, double* x, double* v, const double* y, cudaStream_t s)
{
    FEMGB_LAUNCH(k_integrate_fp64, grid_for(3 * N), N, dt, x, v, y);
}
void launch_node_b_fie_fp64(const MeshView<double>& m, const StepConsts& c, const double* x, const double* xn,
                            const double* vn, int warm, double* b, double* y, cudaStream_t s)
{
    FEMGB_LAUNCH(k_node_b_fie_fp64, grid_for(m.N), m, c, x, xn, vn, warm, b, y);
}
void launch_knc_fie_fp64(uint32_t N, uint32_t count, const uint32_t* nodes, const double* targets, const double* x,
                         double* b, double* y, cudaStream_t s)
{
    if (count == 0) return;
    FEMGB_LAUNCH(k_knc_fie_fp64, grid_for(count), N, count, nodes, targets, x, b, y);
}
void launch_sq_norm_fp64(uint32_t n, const double* v, double* partials, cudaStream_t s)
{
    FEMGB_LAUNCH(k_sq_norm_fp64, grid_for(n), n, v, partials);
}
void launch_fie_update_fp64(uint32_t N, double inv_dt, double* x, double* v, const double* xn, const double* y,
                            double* partials, cudaStream_t s)
{
    FEMGB_LAUNCH(k_fie_update_fp64, grid_for(3 * N), N, inv_dt, x, v, xn, y, partials);
}
void launch_bsr_assemble_fp64(const MeshView<double>& m, uint32_t nnzb, const uint32_t* cptr,
                              const uint32_t* contrib, double* val, cudaStream_t s)
{
    prof_begin("bsr_assemble_fp64", s);
    FEMGB_LAUNCH(k_bsr_assemble_fp64, grid_for(nnzb), m, nnzb, cptr, contrib, val);
    prof_end("bsr_assemble_fp64", s);
}
void launch_mr_init_fp64(const MeshView<double>& m, const StepConsts& c, const double* b, const double* y,
                         double* v1, double* partials, cudaStream_t s)
{
    FEMGB_LAUNCH(k_mr_init_fp64, grid_for(m.N), m, c, b, y, v1, partials);
}
void launch_mr_start_fp64(uint32_t N, double* v1, double* v, double* p, double* p0, const StepScalars* st,
                          cudaStream_t s)
{
    FEMGB_LAUNCH(k_mr_start_fp64, grid_for(3 * N), N, v1, v, p, p0, st);
}
void launch_mr_q_fp64(const MeshView<double>& m, const StepConsts& c, const double* v, const double* v0,
                      double* v1, double* partials, const StepScalars* st, cudaStream_t s)
{
    FEMGB_LAUNCH(k_mr_q_fp64, grid_for(m.N), m, c, v, v0, v1, partials, st);
}
void launch_mr_v1_fp64(uint32_t N, double* v1, const double* v, double* partials, const StepScalars* st,
                       cudaStream_t s)
{
    FEMGB_LAUNCH(k_mr_v1_fp64, grid_for(3 * N), N, v1, v, partials, st);
}
void launch_mr_update_fp64(uint32_t N, double* v1, const double* v, const double* p, double* p0, double* y,
                           const StepScalars* st, cudaStream_t s)
{
    FEMGB_LAUNCH(k_mr_update_fp64, grid_for(3 * N), N, v1, v, p, p0, y, st);
}
void launch_elem_lcm_force_fp64(const MeshView<double>& m, const double* F, const PkMaterial& mat, int write_out,
                                double* energy_partials, cudaStream_t s)
{
    FEMGB_LAUNCH(k_elem_lcm_force_fp64, grid_for(m.T), m, F, mat, write_out, energy_partials);
}
void launch_elem_lcm_spmv_fp64(const MeshView<double>& m, const double* d, const double* F, const PkMaterial& mat,
                               const StepScalars* st, int check_done, cudaStream_t s)
{
    FEMGB_LAUNCH(k_elem_lcm_spmv_fp64, grid_for(m.T), m, d, F, mat, st, check_done);
}
void launch_potential_fp64(const MeshView<double>& m, const StepConsts& c, const double* x, double* partials,
                           cudaStream_t s)
{
    FEMGB_LAUNCH(k_potential_fp64, grid_for(m.T), m, c, x, partials);
}
void launch_apply_A_fp64(const MeshView<double>& m, double factor_M, double factor_K, double mass,
                         const double* d, double* q, cudaStream_t s)
{
    FEMGB_LAUNCH(k_apply_A_fp64, grid_for(m.N), m, factor_M, factor_K, mass, d, q);
}
void launch_gather_sum_fp64(const MeshView<double>& m, double sign, double* f, cudaStream_t s)
{
    FEMGB_LAUNCH(k_gather_sum_fp64, grid_for(m.N), m, sign, f);
}
void launch_finalize(int kind, const double* partials, uint32_t count, const StepConsts& c, StepScalars* st,
                     cudaStream_t s, cudaGraphConditionalHandle cond, int set_cond)
{
    k_finalize<<<1, kFinalizeThreads, 0, s>>>(kind, partials, count, c, st, cond, set_cond);
    launch_counter()++;
}

FEMGB_BOUNDS_ACCESSOR(bounds_read_fem_kernels)

}  // namespace femgb
