// solid.cu -- host runtime of one device-resident solid: the C ABI in
// include/fem_tet.h for the FP64 drop-in path.
//
// Set-up restates EditableTetrahedronElementSet3::EndEdition
// (TetrahedronElementSet3.cpp:2113-2166) for the data the strain-form kernels
// need (Dm^-1, volume, the E-matrix entries times V), and the Leaf's
// RebuildMass / RebuildRayleighCoeffsFromFreqs (LeafDSH_Solid3D_FEM.cpp:
// 1591-1611, LeafDSH_Solid3D_FEM.h:347-354). The step orchestrates
// FixedStep + Step_QuasiImplicitEuler_v (LeafDSH_Solid3D_FEM.cpp:898-990,
// 1205-1328) and ILSS_CG::Solve (ILSS_CG.h:38-151) as kernels on the
// handle's stream; the CG loop runs in chunks of iterations whose kernels
// turn into no-ops once the device-side loop condition fails, and the host
// reads the condition once per chunk. The fully-implicit Euler integrator
// (Step_FullyImplicitEuler_dx, :1357-1552) runs its Newton loop on the host
// over the same kernels, reading |b_k| and |y_k| once per Newton iteration.
#include "../../include/fem_tet.h"
#include "bounds.cuh"
#include "dapd.cuh"
#include "fem_device.cuh"
#include "graph_capture.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace femgb;

namespace femgb {
thread_local std::string g_err;
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace femgb

namespace {

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(e_ == cudaErrorMemoryAllocation ? FEM_E_OOM : FEM_E_CUDA, "%s: %s (%s:%d)", #call, \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                          \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        n = count;
        return cudaMalloc(&p, sizeof(T) * (count ? count : 1));
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

// 3x3 helpers with the reference's rounding (Mal/GMat.h:236-313), host side.
double det3(const double* m)
{
    return m[0] * m[4] * m[8] - m[0] * m[7] * m[5] + m[3] * m[7] * m[2] - m[3] * m[1] * m[8] + m[6] * m[1] * m[5] -
           m[6] * m[4] * m[2];
}
void inverse3(const double* m, double* r)
{
    double inv_det = 1.0 / det3(m);
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

}  // namespace

struct fem_solid_s {
    uint32_t N = 0, T = 0;
    fem_params params{};
    StepConsts consts{};
    double node_mass = 0, total_volume = 0, rayleigh[2] = {0, 0};
    cudaStream_t stream = nullptr;
    // element data
    DevBuf<int4> tets;
    DevBuf<double> Dinv, mat, vol, R, detF, eout;
    DevBuf<uint32_t> csr_ptr, csr_idx;
    DevBuf<uint8_t> fixed;
    // the one-cluster CG of a small solid (ctas 0: none); cl_ent as csr_idx,
    // each entry as the owning CTA and its local corner
    CgClusterPlan cl_plan{};
    DevBuf<uint32_t> cl_ent;
    // the assembled stiffness (MeshView::bsr_*): pattern, per-slot
    // contributions and blocks; bsr_use: the solvers take it (set_bsr_use)
    DevBuf<uint32_t> bsr_row, bsr_col, bsr_cptr, bsr_contrib;
    DevBuf<double> bsr_val;
    uint32_t bsr_nnzb = 0;
    bool bsr_want = false, bsr_use = false;  // fem_solid_set_assembled; the solvers take it now
    // node vectors
    DevBuf<double> rest, x, v, y, b, r, d, q, tmp;
    DevBuf<double> xn, vn;  // FIE: x^n and v^n of the step (allocated for the FIE integrators only)
    // DAPD: the positions the previous step started from (m_vecPos0) and the
    // per-element direction of collapse (allocated for DAPD only)
    DevBuf<double> prev_x;
    DevBuf<uchar2> doc;
    DapdParams dapd{};
    // MINRES: the p and p0 vectors (v, v0, v1 reuse the CG's r, d, q)
    DevBuf<double> mr_p, mr_p0;
    // C_LCM: each element's F of the last evaluation (T x 9) and the set's
    // Lame parameters (from the scalar E, nu, as the reference's element set)
    DevBuf<double> Fe;
    double lame_mu = 0, lame_lambda = 0;
    // FIE statistics of the last step (host side; the Newton loop runs on the host)
    uint32_t nr_iters = 0, fie_cg_iters = 0;
    double nr_rel = 0, nr_abs = 0;
    bool fie_solved = false;
    // constraints
    DevBuf<uint32_t> knc_nodes;
    DevBuf<double> knc_targets;
    uint32_t knc_count = 0;
    std::vector<uint8_t> fixed_host;
    // reductions / scalars
    DevBuf<double> partials, partials2;
    DevBuf<StepScalars> st;
    StepScalars* st_host = nullptr;  // pinned
    bool evaluated = false;
    // multi-solid Newton lock-step (fem_solid_nr_*): the iterates x_k, v_k
    // (allocated by the first fem_solid_nr_init), the iterations since the
    // last NR_PreStep and the LS iterations of its NR_MidStep
    DevBuf<double> lk_x, lk_v;
    uint32_t lock_nr_k = 0, lock_ls_iters = 0;
    bool lock_stats = false;  // the last completed step was a lock-step (NR_End)
    // fem_solid_apply_A_noalloc: device address of the static scratch array,
    // looked up at creation (null for solids above FEM_NOALLOC_MAX_TETS)
    double* noalloc_scratch = nullptr;
    // the QIE_V step as one CUDA graph (its solver loop a WHILE node),
    // captured at the first step and again after a change of parameters or
    // constraints; FIE steps stay host-driven (their Newton tests)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    void drop_graph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }

    MeshView<double> view()
    {
        MeshView<double> m;
        m.N = N;
        m.T = T;
        m.tets = tets.p;
        m.Dinv = Dinv.p;
        m.mat = mat.p;
        m.R = R.p;
        m.detF = detF.p;
        m.vol = vol.p;
        m.rest = rest.p;
        m.csr_ptr = csr_ptr.p;
        m.csr_idx = csr_idx.p;
        m.fixed = fixed.p;
        m.eout = eout.p;
        if (bsr_use) {
            m.bsr_row = bsr_row.p;
            m.bsr_col = bsr_col.p;
            m.bsr_val = bsr_val.p;
        }
        return m;
    }

    void release()
    {
        DevBuf<double>* dbl[] = {&Dinv, &mat, &vol, &R, &detF, &eout, &bsr_val, &rest, &x, &v, &y, &b, &r, &d, &q, &tmp,
                                 &xn, &vn, &prev_x, &mr_p, &mr_p0, &Fe, &knc_targets, &partials, &partials2,
                                 &lk_x, &lk_v};
        for (auto* p : dbl) p->release();
        doc.release();
        tets.release();
        csr_ptr.release();
        csr_idx.release();
        cl_ent.release();
        bsr_row.release();
        bsr_col.release();
        bsr_cptr.release();
        bsr_contrib.release();
        fixed.release();
        knc_nodes.release();
        st.release();
        if (st_host) cudaFreeHost(st_host);
        st_host = nullptr;
        drop_graph();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

namespace {

int check_handle(fem_solid s)
{
    if (!s) return fail(FEM_E_ARG, "null solid handle");
    return FEM_OK;
}

bool uses_dapd(const fem_solid s) { return s->params.rotation == FEM_ROTATION_DAPD; }
// the first Piola-Kirchhoff materials (C_LCM, C_LCMH, C_CCM) keep F per element
bool uses_lcm(const fem_solid s) { return s->params.material != FEM_MATERIAL_C_WRP; }

PkMaterial pk_material(const fem_solid s)
{
    PkMaterial m;
    m.kind = (int)s->params.material;
    m.mu = s->lame_mu;
    m.lambda = s->lame_lambda;
    m.k = (double)(float)s->params.ecie_k_factor;  // float32 in the reference's Params
    return m;
}

// Parameters every entry point that takes a fem_params checks (enums in
// range, finite DAPD settings, a positive time step, the FP64 precision).
int check_params(const fem_params* params)
{
    if (!(params->fixed_dt > 0)) return fail(FEM_E_ARG, "fixed_dt must be > 0");
    if (params->precision != FEM_PRECISION_FP64)
        return fail(FEM_E_ARG, "precision %u: this entry point builds the FP64 path; use the batch API for mixed",
                    params->precision);
    if (params->integrator > FEM_INTEGRATOR_FIE_DX_QUASISTATIC)
        return fail(FEM_E_ARG, "integrator %u is not an enum fem_integrator value", params->integrator);
    if (params->integrator != FEM_INTEGRATOR_QIE_V && !(params->nr_abs_epsilon >= 0))
        return fail(FEM_E_ARG, "nr_abs_epsilon must be >= 0");
    if (params->ls_solver > FEM_LS_MINRES)
        return fail(FEM_E_ARG, "ls_solver %u is not an enum fem_ls_solver value", params->ls_solver);
    if (params->material > FEM_MATERIAL_C_CCM)
        return fail(FEM_E_ARG, "material %u is not an enum fem_material value", params->material);
    if (params->material == FEM_MATERIAL_C_LCMH && !std::isfinite(params->ecie_k_factor))
        return fail(FEM_E_ARG, "ecie_k_factor must be finite");
    if (params->rotation > FEM_ROTATION_DAPD)
        return fail(FEM_E_ARG, "rotation %u is not an enum fem_rotation value", params->rotation);
    if (params->rotation == FEM_ROTATION_DAPD &&
        !(std::isfinite(params->dapd_threshold_det_F) && std::isfinite(params->dapd_l_factor) &&
          std::isfinite(params->dapd_nl_factor) && std::isfinite(params->dapd_nl_exponent)))
        return fail(FEM_E_ARG, "DAPD threshold and factors must be finite");
    return FEM_OK;
}

// The step's constants from the solid's parameters and total volume:
// RebuildMass (m = rho sum V / N stored as its float-rounded reciprocal,
// LeafDSH_Solid3D_FEM.cpp:1591-1611), RebuildRayleighCoeffsFromFreqs with the
// default frequencies 0.1f and 1e4 (LeafDSH_Solid3D_FEM.h:347-354), the
// factors of Step_QuasiImplicitEuler_v (:1300-1301) and the CG settings.
void set_consts(fem_solid s)
{
    const fem_params* params = &s->params;
    const double total_mass = params->density * s->total_volume;
    const double mass_per_node = total_mass / s->N;
    const double inv_mass = (double)1.0f / mass_per_node;
    s->node_mass = 1.0 / inv_mass;
    {
        const double f1 = (double)0.1f, f2 = (double)10000.0f;
        const double o00 = 1.0 / f1, o01 = f1, o10 = 1.0 / f2, o11 = f2;
        const double inv_det = 1.0 / (o00 * o11 - o10 * o01);
        const double i00 = inv_det * o11, i01 = -inv_det * o01, i10 = -inv_det * o10, i11 = inv_det * o00;
        const double z = 2 * params->damping_ratio;
        double a0 = 0, a1 = 0;
        a0 += i00 * z; a0 += i01 * z;
        a1 += i10 * z; a1 += i11 * z;
        s->rayleigh[0] = a0;
        s->rayleigh[1] = a1;
    }
    StepConsts& c = s->consts;
    c.dt = params->fixed_dt;
    c.inv_dt = 1.0 / params->fixed_dt;
    c.mass = s->node_mass;
    c.factor_M = 1.0 + c.dt * s->rayleigh[0];
    c.factor_K = c.dt * c.dt + c.dt * s->rayleigh[1];
    for (int i = 0; i < 3; i++) c.gravity[i] = params->gravity[i];
    c.density = params->density;
    c.rel_eps_sq = params->ls_rel_epsilon * params->ls_rel_epsilon;
    c.abs_eps_sq = params->ls_abs_epsilon * params->ls_abs_epsilon;
    c.max_iter = params->ls_max_iter;
    // LameParameters_From_YoungAndPoisson on the set's E, nu
    // (TetrahedronElementSet3.cpp:181-186, 2116-2117, 2172-2173)
    const double E = params->young_modulus, nu = params->poisson_ratio;
    s->lame_mu = 0.5 * E / (1 + nu);
    s->lame_lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    s->dapd.thr = params->dapd_threshold_det_F;
    s->dapd.fL = (double)(float)params->dapd_l_factor;
    s->dapd.fNL = (double)(float)params->dapd_nl_factor;
    s->dapd.eNL = (double)(float)params->dapd_nl_exponent;
}

// TetrahedronElementSet3::BeginEvaluation(x0 = xprev, x): F, det F and the
// rotations at x; xprev feeds the DAPD collapse detection only. C_LCM keeps F.
void begin_eval(fem_solid s, const double* xprev, const double* x)
{
    MeshView<double> m = s->view();
    double* F_out = uses_lcm(s) ? s->Fe.p : nullptr;
    if (uses_dapd(s))
        launch_begin_eval_dapd_fp64(m, xprev, x, s->doc.p, s->dapd, F_out, s->st.p, s->stream);
    else
        launch_begin_eval_fp64(m, x, F_out, s->st.p, s->stream);
    if (s->bsr_use)  // the solvers' operator on the new rotations
        launch_bsr_assemble_fp64(m, s->bsr_nnzb, s->bsr_cptr.p, s->bsr_contrib.p, s->bsr_val.p, s->stream);
}

// The material's element force at x (C_f_e / C_LCM_f_e) into m.eout and/or
// its energy partials (C_V / C_LCM_V); C_LCM works from the stored F.
void elem_force(fem_solid s, const MeshView<double>& m, const double* x, int write_out, double* energy_partials)
{
    if (uses_lcm(s))
        launch_elem_lcm_force_fp64(m, s->Fe.p, pk_material(s), write_out, energy_partials, s->stream);
    else
        launch_elem_force_fp64(m, x, write_out, energy_partials, s->stream);
}

// The material's element differential of d (C_df_x / C_LCM_df_x) into m.eout.
void elem_spmv(fem_solid s, const MeshView<double>& m, const double* d, int check_done)
{
    if (uses_lcm(s))
        launch_elem_lcm_spmv_fp64(m, d, s->Fe.p, pk_material(s), s->st.p, check_done, s->stream);
    else
        launch_elem_spmv_fp64(m, d, s->st.p, check_done, s->stream);
}

// The solvers' product ahead of their node kernels: nothing when those take
// K u from the assembled stiffness (m.bsr_val), else the element outputs.
void solve_product(fem_solid s, const MeshView<double>& m, const double* d, int check_done)
{
    if (!m.bsr_val) elem_spmv(s, m, d, check_done);
}

// FixedStep's opening: BeginEvaluation(m_vecPos0, x), then m_vecPos0 = x
// (LeafDSH_Solid3D_FEM.cpp:927-935).
int open_step(fem_solid s)
{
    cudaStream_t st = s->stream;
    CK(cudaMemsetAsync(&s->st.p->inverted, 0, sizeof(uint32_t), st));
    begin_eval(s, s->prev_x.p, s->x.p);
    if (uses_dapd(s))
        CK(cudaMemcpyAsync(s->prev_x.p, s->x.p, sizeof(double) * 3 * (size_t)s->N, cudaMemcpyDeviceToDevice, st));
    return FEM_OK;
}

// A C_WRP solid with a one-cluster CG plan. GB300 gives a warp's FP64
// instruction about 64 clocks whatever its active lanes, and an SM about
// one every 19 clocks over all its warps: a 140-instruction element product
// takes about 9k clocks, so the plan spreads the elements thin (at most a
// few warps of them per SM) over up to 16 CTAs, and its iteration is four
// cluster barriers instead of six launches.
bool cg_on_cluster(const fem_solid s)
{
    return s->params.material == FEM_MATERIAL_C_WRP && s->cl_plan.ctas > 0;
}

// Whether the solvers take K u from the assembled stiffness (asked for by
// fem_solid_set_assembled and built): a C_WRP solid whose solve is not the
// one-cluster CG. GB300's
// FP64 element product is bound by the FP64 pipe at about 140 instructions
// per tet per iteration; the assembled rows take 9 FMAs per block, about
// 27 per tet, at the price of one assembly per evaluation (about 90 per
// element corner pair, 16 pairs per tet).
void set_bsr_use(fem_solid s)
{
    s->bsr_use = s->bsr_want && s->bsr_nnzb > 0 && s->params.material == FEM_MATERIAL_C_WRP &&
                 !(s->params.ls_solver != FEM_LS_MINRES && cg_on_cluster(s));
}

// The assembled stiffness's pattern and contributions (MeshView::bsr_*):
// row n holds n's neighbours through its elements and n itself, ascending;
// slot (n, j) sums the corner pairs (li of n, lj of j) of the elements
// holding both, in element order. ptr/idx: the node CSR of element corners.
int build_bsr(fem_solid s, const uint32_t* tets, const std::vector<uint32_t>& ptr, const std::vector<uint32_t>& idx)
{
    const uint32_t N = s->N, T = s->T;
    if ((uint64_t)T >= (1ull << 28)) return FEM_OK;  // contributions pack the element in 28 bits
    std::vector<uint32_t> brow(N + 1, 0), bcol, nb;
    bcol.reserve(16 * (size_t)N);
    for (uint32_t n = 0; n < N; n++) {
        nb.clear();
        nb.push_back(n);
        for (uint32_t j = ptr[n]; j < ptr[n + 1]; j++) {
            const size_t e = idx[j] >> 2;
            for (int k = 0; k < 4; k++) nb.push_back(tets[4 * e + k]);
        }
        std::sort(nb.begin(), nb.end());
        nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
        bcol.insert(bcol.end(), nb.begin(), nb.end());
        if (bcol.size() >= (1ull << 32)) return FEM_OK;
        brow[n + 1] = (uint32_t)bcol.size();
    }
    const size_t nnzb = bcol.size();
    auto slot_of = [&](uint32_t n, uint32_t col) {
        return (size_t)(std::lower_bound(bcol.begin() + brow[n], bcol.begin() + brow[n + 1], col) - bcol.begin());
    };
    std::vector<uint32_t> bcptr(nnzb + 1, 0), bcon(16 * (size_t)T);
    for (uint32_t n = 0; n < N; n++)
        for (uint32_t j = ptr[n]; j < ptr[n + 1]; j++)
            for (int lj = 0; lj < 4; lj++) bcptr[slot_of(n, tets[4 * (size_t)(idx[j] >> 2) + lj]) + 1]++;
    for (size_t k = 0; k < nnzb; k++) bcptr[k + 1] += bcptr[k];
    {
        std::vector<uint32_t> fill(bcptr.begin(), bcptr.end() - 1);
        for (uint32_t n = 0; n < N; n++)
            for (uint32_t j = ptr[n]; j < ptr[n + 1]; j++) {
                const uint32_t e = idx[j] >> 2, li = idx[j] & 3u;
                for (uint32_t lj = 0; lj < 4; lj++)
                    bcon[fill[slot_of(n, tets[4 * (size_t)e + lj])]++] = (e << 4) | (li << 2) | lj;
            }
    }
    cudaStream_t st = s->stream;
    CK(s->bsr_row.alloc(N + 1));
    CK(s->bsr_col.alloc(nnzb));
    CK(s->bsr_cptr.alloc(nnzb + 1));
    CK(s->bsr_contrib.alloc(bcon.size()));
    CK(s->bsr_val.alloc(9 * nnzb));
    CK(cudaMemcpyAsync(s->bsr_row.p, brow.data(), sizeof(uint32_t) * brow.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->bsr_col.p, bcol.data(), sizeof(uint32_t) * nnzb, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->bsr_cptr.p, bcptr.data(), sizeof(uint32_t) * bcptr.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(s->bsr_contrib.p, bcon.data(), sizeof(uint32_t) * bcon.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(s->bsr_val.p, 0, sizeof(double) * 9 * nnzb, st));
    CK(cudaStreamSynchronize(st));
    s->bsr_nnzb = (uint32_t)nnzb;
    return FEM_OK;
}

// The one-cluster CG plan of a solid (see cg_on_cluster). Up to 1,440 tets,
// three lanes per element (about 50 FP64 instructions each) and 30
// elements per CTA on ceil(T / 30) CTAs; beyond, one lane per element and
// 128 per CTA on ceil(T / 128). When a cluster of that size does not fit,
// the fewest CTAs below it that do, with at most kCgClusterMaxThreads
// threads; none when the solid is too large. ptr: the node CSR's row starts.
CgClusterPlan plan_cg_cluster(uint32_t N, uint32_t T, const std::vector<uint32_t>& ptr)
{
    if (T == 0 || N == 0) return CgClusterPlan{};
    auto try_plan = [&](uint32_t C, uint32_t split, CgClusterPlan& p) {
        p = CgClusterPlan{};
        p.ctas = C;
        p.split = split;
        p.ept = (T + C - 1) / C;
        p.npt = (N + C - 1) / C;
        uint32_t emax = 0;
        for (uint32_t r = 0; r < C; r++) {
            const uint32_t a = std::min(N, r * p.npt), b = std::min(N, (r + 1) * p.npt);
            emax = std::max(emax, ptr[b] - ptr[a]);
        }
        p.ent_max = emax;
        const uint32_t need = split ? 32 * ((p.ept + 9) / 10) : (p.ept + 31) / 32 * 32;
        p.threads = std::max<uint32_t>(128u, need);
        p.smem = cg_cluster_smem_bytes(p.ept, p.npt, p.ent_max);
        return p.threads <= kCgClusterMaxThreads && cg_cluster_fits(p);
    };
    CgClusterPlan p{};
    if (T <= 1440) {
        const uint32_t want = std::min<uint32_t>(kCgClusterMaxCtas, std::max<uint32_t>(1u, (T + 29) / 30));
        for (uint32_t C = want; C >= 1; C--)
            if (try_plan(C, 1, p)) return p;
    }
    const uint32_t want = std::min<uint32_t>(kCgClusterMaxCtas, std::max<uint32_t>(1u, (T + 127) / 128));
    for (uint32_t C = want; C >= 1; C--) {
        if ((T + C - 1) / C > kCgClusterMaxThreads) break;  // fewer CTAs only take more
        if (try_plan(C, 0, p)) return p;
    }
    return CgClusterPlan{};
}

// ILSS_CG::Solve (ILSS_CG.h:38-151) of A y = b from the warm start in y,
// with the factors of c, on the rotations of the last evaluation. Returns
// once the device-side loop condition has failed (the host reads it once per
// chunk of iterations).
int cg_solve(fem_solid s, const StepConsts& c, int chunk)
{
    cudaStream_t st = s->stream;
    MeshView<double> m = s->view();
    if (cg_on_cluster(s)) {
        CK(launch_cg_cluster_fp64(m, c, s->cl_plan, s->cl_ent.p, s->b.p, s->y.p, s->st.p, st));
        CK(cudaMemcpyAsync(s->st_host, s->st.p, sizeof(StepScalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CK(cudaGetLastError());
        return FEM_OK;
    }
    const uint32_t gN = grid_for(s->N), gV = grid_for(3 * s->N);
    solve_product(s, m, s->y.p, 0);
    launch_node_residual_fp64(m, c, s->b.p, s->y.p, s->r.p, s->d.p, s->partials.p, st);
    launch_finalize(FIN_INIT, s->partials.p, gN, c, s->st.p, st);
    for (;;) {
        for (int i = 0; i < chunk; i++) {
            solve_product(s, m, s->d.p, 1);
            launch_node_q_fp64(m, c, s->d.p, s->q.p, s->partials.p, s->st.p, st);
            launch_node_xr_fp64(s->N, s->y.p, s->r.p, s->d.p, s->q.p, s->partials.p, s->st.p, st);
            launch_node_d_fp64(s->N, s->fixed.p, s->d.p, s->r.p, s->st.p, st);
        }
        CK(cudaMemcpyAsync(s->st_host, s->st.p, sizeof(StepScalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (s->st_host->done) break;
    }
    launch_finalize(FIN_STATS, s->partials.p, 0, c, s->st.p, st);
    CK(cudaGetLastError());
    return FEM_OK;
}

// ILSS_MINRES::Solve (ILSS_MINRES.h:51-168) of A y = b from the warm start in
// y, with the factors of c: Lanczos vectors v0, v, v1 and directions p0, p
// rotated by pointer between iterations (the kernels of an iteration after the
// loop has ended are no-ops, so the rotation is harmless there).
int minres_solve(fem_solid s, const StepConsts& c, int chunk)
{
    cudaStream_t st = s->stream;
    MeshView<double> m = s->view();
    const uint32_t gN = grid_for(s->N), gV = grid_for(3 * s->N);
    double *v = s->r.p, *v0 = s->d.p, *v1 = s->q.p, *p = s->mr_p.p, *p0 = s->mr_p0.p;
    launch_sq_norm_fp64(3 * s->N, s->b.p, s->partials.p, st);
    launch_finalize(FIN_SUM, s->partials.p, gV, c, s->st.p, st);  // |b|^2
    solve_product(s, m, s->y.p, 0);
    launch_mr_init_fp64(m, c, s->b.p, s->y.p, v1, s->partials.p, st);
    launch_finalize(FIN_MR_INIT, s->partials.p, gN, c, s->st.p, st);
    launch_mr_start_fp64(s->N, v1, v, p, p0, s->st.p, st);
    for (;;) {
        for (int i = 0; i < chunk; i++) {
            double* t = v0;  // v0 <- v, v <- v1, v1 <- the old v0 buffer
            v0 = v;
            v = v1;
            v1 = t;
            solve_product(s, m, v, 1);
            launch_mr_q_fp64(m, c, v, v0, v1, s->partials.p, s->st.p, st);
            launch_finalize(FIN_MR_ALPHA, s->partials.p, gN, c, s->st.p, st);
            launch_mr_v1_fp64(s->N, v1, v, s->partials.p, s->st.p, st);
            launch_finalize(FIN_MR_BETA, s->partials.p, gV, c, s->st.p, st);
            launch_mr_update_fp64(s->N, v1, v, p, p0, s->y.p, s->st.p, st);
            t = p;  // the new p was written into p0's buffer
            p = p0;
            p0 = t;
        }
        CK(cudaMemcpyAsync(s->st_host, s->st.p, sizeof(StepScalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (s->st_host->done) break;
    }
    launch_finalize(FIN_MR_STATS, s->partials.p, 0, c, s->st.p, st);
    CK(cudaGetLastError());
    return FEM_OK;
}

// LS_Solve's solver choice (LeafDSH_Solid3D_FEM.cpp:1136-1154)
int ls_solve(fem_solid s, const StepConsts& c, int chunk)
{
    return s->params.ls_solver == FEM_LS_MINRES ? minres_solve(s, c, chunk) : cg_solve(s, c, chunk);
}

// The solver of ls_solve enqueued for capture into the step graph: the same
// kernels in the same order, the loop a WHILE node whose condition the
// finalisers set (the kernels of an iteration after the loop test failed
// are no-ops, as in the host-driven loop). The body is captured with
// s->stream pointing at the body's capture stream.
cudaError_t ls_solve_capture(fem_solid s, const StepConsts& c, cudaGraph_t top)
{
    cudaStream_t st = s->stream;
    MeshView<double> m = s->view();
    const uint32_t gN = grid_for(s->N), gV = grid_for(3 * s->N);
    if (s->params.ls_solver != FEM_LS_MINRES && cg_on_cluster(s))
        return launch_cg_cluster_fp64(m, c, s->cl_plan, s->cl_ent.p, s->b.p, s->y.p, s->st.p, st);
    cudaGraphConditionalHandle cond = 0;
    cudaError_t e = cudaGraphConditionalHandleCreate(&cond, top, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    if (s->params.ls_solver != FEM_LS_MINRES) {
        solve_product(s, m, s->y.p, 0);
        launch_node_residual_fp64(m, c, s->b.p, s->y.p, s->r.p, s->d.p, s->partials.p, st);
        launch_finalize(FIN_INIT, s->partials.p, gN, c, s->st.p, st, cond, 1);
        e = capture_conditional(st, cond, cudaGraphCondTypeWhile, [&](cudaStream_t bs, cudaGraph_t) {
            s->stream = bs;
            solve_product(s, m, s->d.p, 1);
            launch_node_q_fp64(m, c, s->d.p, s->q.p, s->partials.p, s->st.p, bs, cond, 1);
            launch_node_xr_fp64(s->N, s->y.p, s->r.p, s->d.p, s->q.p, s->partials.p, s->st.p, bs, cond, 1);
            launch_node_d_fp64(s->N, s->fixed.p, s->d.p, s->r.p, s->st.p, bs);
            s->stream = st;
            return cudaGetLastError();
        });
        if (e != cudaSuccess) return e;
        launch_finalize(FIN_STATS, s->partials.p, 0, c, s->st.p, st);
        return cudaGetLastError();
    }
    // MINRES: the host loop rotates v0, v, v1 (period 3) and p, p0
    // (period 2) between iterations; the body holds six iterations, after
    // which every buffer is back in its place
    double *v = s->r.p, *v0 = s->d.p, *v1 = s->q.p, *p = s->mr_p.p, *p0 = s->mr_p0.p;
    launch_sq_norm_fp64(3 * s->N, s->b.p, s->partials.p, st);
    launch_finalize(FIN_SUM, s->partials.p, gV, c, s->st.p, st);  // |b|^2
    solve_product(s, m, s->y.p, 0);
    launch_mr_init_fp64(m, c, s->b.p, s->y.p, v1, s->partials.p, st);
    launch_finalize(FIN_MR_INIT, s->partials.p, gN, c, s->st.p, st, cond, 1);
    launch_mr_start_fp64(s->N, v1, v, p, p0, s->st.p, st);
    e = capture_conditional(st, cond, cudaGraphCondTypeWhile, [&](cudaStream_t bs, cudaGraph_t) {
        s->stream = bs;
        for (int i = 0; i < 6; i++) {
            double* t = v0;  // v0 <- v, v <- v1, v1 <- the old v0 buffer
            v0 = v;
            v = v1;
            v1 = t;
            solve_product(s, m, v, 1);
            launch_mr_q_fp64(m, c, v, v0, v1, s->partials.p, s->st.p, bs);
            launch_finalize(FIN_MR_ALPHA, s->partials.p, gN, c, s->st.p, bs, cond, 1);
            launch_mr_v1_fp64(s->N, v1, v, s->partials.p, s->st.p, bs);
            launch_finalize(FIN_MR_BETA, s->partials.p, gV, c, s->st.p, bs, cond, 1);
            launch_mr_update_fp64(s->N, v1, v, p, p0, s->y.p, s->st.p, bs);
            t = p;  // the new p was written into p0's buffer
            p = p0;
            p0 = t;
        }
        s->stream = st;
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    launch_finalize(FIN_MR_STATS, s->partials.p, 0, c, s->st.p, st);
    return cudaGetLastError();
}

// Sum of `count` block partials into StepScalars::host_sum, read on the host.
int host_sum(fem_solid s, uint32_t count, double* out)
{
    cudaStream_t st = s->stream;
    launch_finalize(FIN_SUM, s->partials.p, count, s->consts, s->st.p, st);
    CK(cudaMemcpyAsync(&s->st_host->host_sum, &s->st.p->host_sum, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *out = s->st_host->host_sum;
    return FEM_OK;
}

// Elastic and potential energy at x with the current rotations
// (FixedStep's m_TES.V and RecomputeEnergy, LeafDSH_Solid3D_FEM.cpp:979,1554-1584).
void energy(fem_solid s)
{
    cudaStream_t st = s->stream;
    MeshView<double> m = s->view();
    const StepConsts& c = s->consts;
    const uint32_t gE = grid_for(s->T);
    elem_force(s, m, s->x.p, 0, s->partials2.p);
    launch_finalize(FIN_ENERGY_E, s->partials2.p, gE, c, s->st.p, st);
    launch_potential_fp64(m, c, s->x.p, s->partials2.p, st);
    launch_finalize(FIN_ENERGY_P, s->partials2.p, gE, c, s->st.p, st);
}

// One FixedStep with Step_FullyImplicitEuler_dx (LeafDSH_Solid3D_FEM.cpp:
// 1357-1552). x and v are the Newton iterates x_k and v_k in place; xn and vn
// keep x^n and v^n. Each Newton iteration: element forces at x_k, b_k, the
// constraint rows, |b_k| (the exit test), CG on
//   A = (1/h^2 + a0/h) M + (1 + a1/h) K(x_k),
// x_k += y, v_k = (x_k - x^n)/h, |y|, and BeginEvaluation at the new x_k.
// h = 0 (quasi-static) drops every 1/h term.
int step_fie(fem_solid s, int chunk)
{
    cudaStream_t st = s->stream;
    MeshView<double> m = s->view();
    const bool quasi = s->params.integrator == FEM_INTEGRATOR_FIE_DX_QUASISTATIC;
    StepConsts c = s->consts;
    c.dt = quasi ? 0.0 : s->consts.dt;
    c.inv_dt = quasi ? 0.0 : 1.0 / s->consts.dt;
    c.factor_M = c.inv_dt * c.inv_dt + c.inv_dt * s->rayleigh[0];
    c.factor_K = 1.0 + c.inv_dt * s->rayleigh[1];
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    const uint32_t gV = grid_for(3 * s->N);
    if (int e = open_step(s)) return e;
    CK(cudaMemcpyAsync(s->xn.p, s->x.p, bytes, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(s->vn.p, s->v.p, bytes, cudaMemcpyDeviceToDevice, st));
    uint32_t nr_k = 0, cg_iters = 0;
    double delta_new = 0.0, delta_0 = -1.0, sum = 0.0;
    bool converged = false, solved = false;
    do {
        elem_force(s, m, s->x.p, 1, nullptr);
        launch_node_b_fie_fp64(m, c, s->x.p, s->xn.p, s->vn.p, nr_k == 0 ? 1 : 0, s->b.p, s->y.p, st);
        launch_knc_fie_fp64(s->N, s->knc_count, s->knc_nodes.p, s->knc_targets.p, s->x.p, s->b.p, s->y.p, st);
        launch_sq_norm_fp64(3 * s->N, s->b.p, s->partials.p, st);
        if (int e = host_sum(s, gV, &sum)) return e;
        delta_new = std::sqrt(sum);
        if (delta_0 < 0) delta_0 = delta_new;
        if (!std::isfinite(delta_new)) return fail(FEM_E_NAN, "NaN or Inf in the Newton right-hand side");
        converged = delta_new < s->params.nr_abs_epsilon;
        if (!converged) {
            if (int e = ls_solve(s, c, chunk)) return e;
            cg_iters += s->st_host->k;
            solved = true;
            launch_fie_update_fp64(s->N, c.inv_dt, s->x.p, s->v.p, s->xn.p, s->y.p, s->partials.p, st);
            if (int e = host_sum(s, gV, &sum)) return e;
            delta_new = std::sqrt(sum);
            nr_k++;
            // BeginEvaluation(x^n, x_k) (:1529)
            CK(cudaMemsetAsync(&s->st.p->inverted, 0, sizeof(uint32_t), st));
            begin_eval(s, s->xn.p, s->x.p);
        }
    } while (!converged && nr_k < s->params.nr_max_iter);
    s->nr_iters = nr_k;
    s->fie_cg_iters = cg_iters;
    s->fie_solved = solved;
    s->nr_abs = delta_new;
    s->nr_rel = (delta_0 > 0) ? delta_new / delta_0 : 0.0;
    if (s->params.compute_energy) energy(s);
    CK(cudaGetLastError());
    return FEM_OK;
}

// One FixedStep's QIE_V pipeline after the opening: f_e, b, constraints,
// the solve, integration and energies.
void qie_head(fem_solid s)
{
    cudaStream_t st = s->stream;
    MeshView<double> m = s->view();
    const StepConsts& c = s->consts;
    elem_force(s, m, s->x.p, 1, nullptr);
    launch_node_b_fp64(m, c, s->v.p, s->b.p, s->y.p, st);
    launch_knc_fp64(s->N, s->knc_count, s->knc_nodes.p, s->knc_targets.p, s->x.p, c, s->b.p, s->y.p, st);
}
void qie_tail(fem_solid s)
{
    const StepConsts& c = s->consts;
    launch_integrate_fp64(s->N, c.dt, s->x.p, s->v.p, s->y.p, s->stream);
    if (s->params.compute_energy) energy(s);
}

// The QIE_V step as one graph: the opening, the pipeline and the solver's
// loop on the device.
int capture_step(fem_solid s)
{
    s->drop_graph();
    cudaStream_t st = s->stream;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    cudaGraph_t top = nullptr;
    cudaStreamCaptureStatus cs;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &top, nullptr, nullptr, nullptr);
    int rc = e == cudaSuccess ? open_step(s) : FEM_E_CUDA;
    if (rc == FEM_OK) {
        qie_head(s);
        e = ls_solve_capture(s, s->consts, top);
        if (e == cudaSuccess) qie_tail(s);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(st, &g);
    if (e == cudaSuccess) e = e2;
    if (rc != FEM_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (rc != FEM_OK) return rc;
        return fail(FEM_E_CUDA, "step graph capture: %s", cudaGetErrorString(e));
    }
    s->graph = g;
    CK(cudaGraphInstantiate(&s->exec, g, 0));
    return FEM_OK;
}

// One FixedStep on the device: QIE_V as the step graph (no host
// synchronisation); FIE with its Newton loop on the host.
int step_once(fem_solid s, int chunk)
{
    s->lock_stats = false;
    if (s->params.integrator != FEM_INTEGRATOR_QIE_V) return step_fie(s, chunk);
    if (!s->exec)
        if (int e = capture_step(s)) return e;
    CK(cudaGraphLaunch(s->exec, s->stream));
    return FEM_OK;
}
void fill_stats(fem_solid s, const StepScalars& h, fem_step_stats* out)
{
    out->cg_iterations = h.k;
    out->status = h.status;
    out->rel_residual = h.rel_residual;
    out->abs_residual = h.abs_residual;
    out->elastic_energy = h.elastic_energy;
    out->potential_energy = h.potential_energy;
    out->inverted_elements = h.inverted;
    out->fp64_resolved = h.fp64_resolved;
    out->total_cg_iterations = h.total_iters;
    out->nr_iterations = 0;
    out->pad = 0;
    out->nr_rel_residual = 0.0;
    out->nr_abs_residual = 0.0;
    out->resolved_det_F = out->resolved_isotropic = out->resolved_tie = out->resolved_check = 0;  // FP64: none
    if (s->lock_stats) {
        // the Leaf's m_Stats after NR_End: LS iterations since the last
        // NR_PreStep, m_NR_nr_k (reset by every NR_PreStep)
        out->cg_iterations = s->lock_ls_iters;
        out->nr_iterations = s->lock_nr_k;
        return;
    }
    if (s->params.integrator != FEM_INTEGRATOR_QIE_V) {
        out->cg_iterations = s->fie_cg_iters;
        if (!s->fie_solved) out->rel_residual = out->abs_residual = 0.0;
        out->nr_iterations = s->nr_iters;
        out->nr_rel_residual = s->nr_rel;
        out->nr_abs_residual = s->nr_abs;
    }
}

}  // namespace

extern "C" {

const char* fem_last_error(void) { return g_err.c_str(); }

uint64_t fem_kernel_launches(void) { return launch_counter(); }

int fem_device_info(int* device, int* sm_count, int* cc_major, int* cc_minor)
{
    int dev = 0, n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(FEM_E_NODEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    CK(cudaGetDevice(&dev));
    cudaDeviceProp p;
    CK(cudaGetDeviceProperties(&p, dev));
    if (device) *device = dev;
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return FEM_OK;
}

int fem_bounds_check_status(int* enabled, uint32_t* failures, uint32_t* site, uint32_t* index, uint32_t* limit)
{
#ifdef FEM_BOUNDS_CHECK
    const int on = 1;
#else
    const int on = 0;
#endif
    int (*const units[])(unsigned*) = {bounds_read_fem_kernels, bounds_read_rotation, bounds_read_batch_kernels,
                                       bounds_read_tile_pipe};
    unsigned total = 0, first[3] = {0u, 0u, 0u};
    for (auto rd : units) {
        unsigned w[4];
        if (rd(w) != 0) return fail(FEM_E_CUDA, "reading the index-check words failed");
        if (w[0] != 0u && total == 0u) {
            first[0] = w[1];
            first[1] = w[2];
            first[2] = w[3];
        }
        total += w[0];
    }
    if (enabled) *enabled = on;
    if (failures) *failures = total;
    if (site) *site = first[0];
    if (index) *index = first[1];
    if (limit) *limit = first[2];
    return FEM_OK;
}

int fem_params_default(fem_params* p)
{
    if (!p) return fail(FEM_E_ARG, "null params");
    std::memset(p, 0, sizeof(*p));
    p->fixed_dt = (double)0.001f;
    p->density = 1000.0;
    p->young_modulus = 1000.0;
    p->poisson_ratio = (double)0.25f;
    p->damping_ratio = 1.0;
    p->ls_rel_epsilon = 1e-3;
    p->ls_abs_epsilon = 1e-6;
    p->ls_max_iter = 20;
    p->precision = FEM_PRECISION_FP64;
    p->degenerate_det_F = 1e-3;
    p->rotation_check = 1e-3;
    p->refresh_every = 50;
    p->refresh_drop = 0.0;
    p->compute_energy = 1;
    // LeafDSH_Solid3D_FEM::Params (LeafDSH_Solid3D_FEM.h:209,233-241)
    p->integrator = FEM_INTEGRATOR_QIE_V;
    p->nr_max_iter = 3;
    p->nr_abs_epsilon = 1e-6;
    // ms::fem::Params (Params.h:85-95)
    p->ls_solver = FEM_LS_CG;  // LeafDSH_Solid3D_FEM::Params m_SolverLS_Type
    p->material = FEM_MATERIAL_C_WRP;  // ms::fem::Params m_MM
    p->ecie_k_factor = 1.0;            // ms::fem::Params m_ECIE_k_factor
    p->rotation = FEM_ROTATION_MSVD;
    p->dapd_threshold_det_F = (double)0.1f;
    p->dapd_l_factor = 1.0;
    p->dapd_nl_factor = 0.0;
    p->dapd_nl_exponent = 2.0;
    return FEM_OK;
}

namespace {
int apply_scratch(double** out);
}

int fem_solid_create(const double* rest_xyz, uint32_t N, const uint32_t* tets, uint32_t T, const fem_params* params,
                     const double* young_per_elem, const double* poisson_per_elem, fem_solid* out)
{
    if (!out) return fail(FEM_E_ARG, "null output handle");
    *out = nullptr;
    if (!rest_xyz || !tets || !params) return fail(FEM_E_ARG, "null rest/tets/params");
    if (N == 0 || T == 0) return fail(FEM_E_ARG, "empty mesh (N=%u, T=%u)", N, T);
    if (N > (1u << 30) || T > (1u << 29)) return fail(FEM_E_ARG, "mesh too large (N=%u, T=%u)", N, T);
    if (int e = check_params(params)) return e;
    for (size_t i = 0; i < 4 * (size_t)T; i++)
        if (tets[i] >= N) return fail(FEM_E_INDEX, "tet %zu names node %u >= N=%u", i / 4, tets[i], N);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FEM_E_NODEVICE, "no CUDA device");

    // ---- host set-up (EndEdition + RebuildMass + Rayleigh) ----
    std::vector<double> Dinv(9 * (size_t)T), mat(3 * (size_t)T), vol(T);
    double acc_total_volume = 0.0;
    for (uint32_t e = 0; e < T; e++) {
        const double* r0 = rest_xyz + 3 * (size_t)tets[4 * (size_t)e];
        const double* r1 = rest_xyz + 3 * (size_t)tets[4 * (size_t)e + 1];
        const double* r2 = rest_xyz + 3 * (size_t)tets[4 * (size_t)e + 2];
        const double* r3 = rest_xyz + 3 * (size_t)tets[4 * (size_t)e + 3];
        double D[9];
        for (int i = 0; i < 3; i++) {
            D[3 * i] = r1[i] - r0[i];
            D[3 * i + 1] = r2[i] - r0[i];
            D[3 * i + 2] = r3[i] - r0[i];
        }
        const double V = det3(D) / 6.0;
        if (!(V > 0.0)) return fail(FEM_E_DEGENERATE, "tet %u has rest volume %g <= 0", e, V);
        vol[e] = V;
        acc_total_volume += V;
        double Di[9];
        inverse3(D, Di);
        for (int c = 0; c < 9; c++) Dinv[(size_t)c * T + e] = Di[c];
        const double E = young_per_elem ? young_per_elem[e] : params->young_modulus;
        const double nu = poisson_per_elem ? poisson_per_elem[e] : params->poisson_ratio;
        // Compute_E (TetrahedronElement3.h:141-156)
        const double a = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
        mat[e] = V * (a * (1.0 - nu));
        mat[(size_t)T + e] = V * (a * nu);
        mat[2 * (size_t)T + e] = V * (a * (0.5 - nu));
    }
    fem_solid s = new (std::nothrow) fem_solid_s;
    if (!s) return fail(FEM_E_OOM, "host allocation failed");
    s->N = N;
    s->T = T;
    s->params = *params;
    s->total_volume = acc_total_volume;
    set_consts(s);

    // node -> (4e + slot) entries, element order
    std::vector<uint32_t> ptr(N + 1, 0), idx(4 * (size_t)T);
    for (size_t i = 0; i < 4 * (size_t)T; i++) ptr[tets[i] + 1]++;
    for (uint32_t n = 0; n < N; n++) ptr[n + 1] += ptr[n];
    {
        std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
        for (size_t i = 0; i < 4 * (size_t)T; i++) idx[fill[tets[i]]++] = (uint32_t)i;
    }
    std::vector<int4> t4(T);
    for (uint32_t e = 0; e < T; e++)
        t4[e] = make_int4((int)tets[4 * (size_t)e], (int)tets[4 * (size_t)e + 1], (int)tets[4 * (size_t)e + 2],
                          (int)tets[4 * (size_t)e + 3]);
    s->fixed_host.assign(N, 0);

    auto cleanup = [&](int code) {
        s->release();
        delete s;
        return code;
    };
#define CKC(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return cleanup(fail(e_ == cudaErrorMemoryAllocation ? FEM_E_OOM : FEM_E_CUDA, "%s: %s", #call, \
                                cudaGetErrorString(e_)));                                           \
    } while (0)
    CKC(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    const size_t n3 = 3 * (size_t)N;
    CKC(s->tets.alloc(T));
    CKC(s->Dinv.alloc(9 * (size_t)T));
    CKC(s->mat.alloc(3 * (size_t)T));
    CKC(s->vol.alloc(T));
    CKC(s->R.alloc(9 * (size_t)T));
    CKC(s->detF.alloc(T));
    CKC(s->eout.alloc(12 * (size_t)T));
    CKC(s->csr_ptr.alloc(N + 1));
    CKC(s->csr_idx.alloc(4 * (size_t)T));
    CKC(s->fixed.alloc(N));
    DevBuf<double>* vecs[] = {&s->rest, &s->x, &s->v, &s->y, &s->b, &s->r, &s->d, &s->q, &s->tmp};
    for (auto* vb : vecs) CKC(vb->alloc(n3));
    if (params->integrator != FEM_INTEGRATOR_QIE_V) {
        CKC(s->xn.alloc(n3));
        CKC(s->vn.alloc(n3));
    }
    if (params->material != FEM_MATERIAL_C_WRP) {
        CKC(s->Fe.alloc(9 * (size_t)T));
        CKC(cudaMemsetAsync(s->Fe.p, 0, sizeof(double) * 9 * (size_t)T, s->stream));
    }
    if (params->ls_solver == FEM_LS_MINRES) {
        CKC(s->mr_p.alloc(n3));
        CKC(s->mr_p0.alloc(n3));
    }
    if (params->rotation == FEM_ROTATION_DAPD) {
        CKC(s->prev_x.alloc(n3));
        CKC(s->doc.alloc(T));
    }
    CKC(s->partials.alloc(4096));
    CKC(s->partials2.alloc(4096));
    CKC(s->st.alloc(1));
    CKC(cudaMallocHost(&s->st_host, sizeof(StepScalars)));
    cudaStream_t st = s->stream;
    CKC(cudaMemcpyAsync(s->tets.p, t4.data(), sizeof(int4) * T, cudaMemcpyHostToDevice, st));
    CKC(cudaMemcpyAsync(s->Dinv.p, Dinv.data(), sizeof(double) * Dinv.size(), cudaMemcpyHostToDevice, st));
    CKC(cudaMemcpyAsync(s->mat.p, mat.data(), sizeof(double) * mat.size(), cudaMemcpyHostToDevice, st));
    CKC(cudaMemcpyAsync(s->vol.p, vol.data(), sizeof(double) * T, cudaMemcpyHostToDevice, st));
    CKC(cudaMemcpyAsync(s->csr_ptr.p, ptr.data(), sizeof(uint32_t) * (N + 1), cudaMemcpyHostToDevice, st));
    CKC(cudaMemcpyAsync(s->csr_idx.p, idx.data(), sizeof(uint32_t) * idx.size(), cudaMemcpyHostToDevice, st));
    s->cl_plan = plan_cg_cluster(N, T, ptr);
    if (s->cl_plan.ctas) {
        std::vector<uint32_t> ent(idx.size());
        for (size_t j = 0; j < idx.size(); j++) {
            const uint32_t e = idx[j] >> 2, r = e / s->cl_plan.ept;
            ent[j] = (r << 24) | (4 * (e - r * s->cl_plan.ept) + (idx[j] & 3));
        }
        CKC(s->cl_ent.alloc(ent.size()));
        CKC(cudaMemcpyAsync(s->cl_ent.p, ent.data(), sizeof(uint32_t) * ent.size(), cudaMemcpyHostToDevice, st));
        CKC(cudaStreamSynchronize(st));
    }
    set_bsr_use(s);
    CKC(cudaMemsetAsync(s->fixed.p, 0, N, st));
    CKC(cudaMemcpyAsync(s->rest.p, rest_xyz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
    CKC(cudaMemcpyAsync(s->x.p, rest_xyz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
    if (params->rotation == FEM_ROTATION_DAPD) {
        CKC(cudaMemcpyAsync(s->prev_x.p, rest_xyz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
        const std::vector<uchar2> none(T, make_uchar2(3, 0));  // no direction of collapse
        CKC(cudaMemcpyAsync(s->doc.p, none.data(), sizeof(uchar2) * T, cudaMemcpyHostToDevice, st));
        CKC(cudaStreamSynchronize(st));
    }
    CKC(cudaMemsetAsync(s->v.p, 0, sizeof(double) * n3, st));
    CKC(cudaMemsetAsync(s->y.p, 0, sizeof(double) * n3, st));
    CKC(cudaMemsetAsync(s->st.p, 0, sizeof(StepScalars), st));
    // R = I, det F = 1 until the first evaluation (CreateCache, TetrahedronElementSet3.cpp:190-209)
    {
        std::vector<double> Rh(9 * (size_t)T, 0.0), dh(T, 1.0);
        for (uint32_t e = 0; e < T; e++) Rh[e] = Rh[4 * (size_t)T + e] = Rh[8 * (size_t)T + e] = 1.0;
        CKC(cudaMemcpyAsync(s->R.p, Rh.data(), sizeof(double) * Rh.size(), cudaMemcpyHostToDevice, st));
        CKC(cudaMemcpyAsync(s->detF.p, dh.data(), sizeof(double) * T, cudaMemcpyHostToDevice, st));
        CKC(cudaStreamSynchronize(st));
    }
#undef CKC
    // the static scratch of fem_solid_apply_A_noalloc: its address is looked
    // up here, where allocating is expected, so that the no-alloc call never
    // loads its module (a failure is left for that call to report)
    if (T <= FEM_NOALLOC_MAX_TETS) {
        const std::string keep = g_err;
        if (apply_scratch(&s->noalloc_scratch) != FEM_OK) s->noalloc_scratch = nullptr;
        g_err = keep;
    }
    *out = s;
    return FEM_OK;
}

int fem_solid_destroy(fem_solid s)
{
    if (!s) return FEM_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->release();
    delete s;
    return FEM_OK;
}

int fem_solid_set_assembled(fem_solid s, int on)
{
    if (int e = check_handle(s)) return e;
    s->drop_graph();  // the step graph holds the operator's launches
    if (on && !s->bsr_nnzb) {
        const uint32_t N = s->N, T = s->T;
        std::vector<int4> t4(T);
        std::vector<uint32_t> tets(4 * (size_t)T), ptr(N + 1), idx(4 * (size_t)T);
        CK(cudaMemcpyAsync(t4.data(), s->tets.p, sizeof(int4) * T, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(ptr.data(), s->csr_ptr.p, sizeof(uint32_t) * (N + 1), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(idx.data(), s->csr_idx.p, sizeof(uint32_t) * idx.size(), cudaMemcpyDeviceToHost,
                           s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (uint32_t e = 0; e < T; e++) {
            tets[4 * (size_t)e] = (uint32_t)t4[e].x;
            tets[4 * (size_t)e + 1] = (uint32_t)t4[e].y;
            tets[4 * (size_t)e + 2] = (uint32_t)t4[e].z;
            tets[4 * (size_t)e + 3] = (uint32_t)t4[e].w;
        }
        if (int e = build_bsr(s, tets.data(), ptr, idx)) {
            s->bsr_row.release();
            s->bsr_col.release();
            s->bsr_cptr.release();
            s->bsr_contrib.release();
            s->bsr_val.release();
            s->bsr_nnzb = 0;
            return e;
        }
        // the current rotations' blocks, for a solve before the next evaluation
        MeshView<double> m = s->view();
        launch_bsr_assemble_fp64(m, s->bsr_nnzb, s->bsr_cptr.p, s->bsr_contrib.p, s->bsr_val.p, s->stream);
        CK(cudaStreamSynchronize(s->stream));
    }
    s->bsr_want = on != 0;
    set_bsr_use(s);
    return FEM_OK;
}

int fem_solid_get_sizes(fem_solid s, uint32_t* N, uint32_t* T)
{
    if (int e = check_handle(s)) return e;
    if (N) *N = s->N;
    if (T) *T = s->T;
    return FEM_OK;
}

int fem_solid_set_knc(fem_solid s, const uint32_t* nodes, const double* targets, uint32_t count)
{
    if (s) s->drop_graph();  // the step graph's constraint launch follows the count
    if (int e = check_handle(s)) return e;
    if (count && (!nodes || !targets)) return fail(FEM_E_ARG, "null constraint arrays");
    for (uint32_t k = 0; k < count; k++)
        if (nodes[k] >= s->N) return fail(FEM_E_INDEX, "constraint %u names node %u >= N=%u", k, nodes[k], s->N);
    CK(cudaStreamSynchronize(s->stream));
    s->knc_nodes.release();
    s->knc_targets.release();
    s->knc_count = count;
    std::fill(s->fixed_host.begin(), s->fixed_host.end(), 0);
    if (count) {
        CK(s->knc_nodes.alloc(count));
        CK(s->knc_targets.alloc(3 * (size_t)count));
        CK(cudaMemcpyAsync(s->knc_nodes.p, nodes, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->knc_targets.p, targets, sizeof(double) * 3 * count, cudaMemcpyHostToDevice,
                           s->stream));
        for (uint32_t k = 0; k < count; k++) s->fixed_host[nodes[k]] = 1;
    }
    CK(cudaMemcpyAsync(s->fixed.p, s->fixed_host.data(), s->N, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_set_knc_targets(fem_solid s, const double* targets)
{
    if (int e = check_handle(s)) return e;
    if (s->knc_count == 0) return FEM_OK;
    if (!targets) return fail(FEM_E_ARG, "null targets");
    CK(cudaMemcpyAsync(s->knc_targets.p, targets, sizeof(double) * 3 * s->knc_count, cudaMemcpyHostToDevice,
                       s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_set_state(fem_solid s, const double* x, const double* v)
{
    if (int e = check_handle(s)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    if (x) CK(cudaMemcpyAsync(s->x.p, x, bytes, cudaMemcpyHostToDevice, s->stream));
    // the previous-step positions restart at x (the Leaf's SetPos path keeps
    // m_vecPos0 in step with the model's positions)
    if (x && uses_dapd(s)) CK(cudaMemcpyAsync(s->prev_x.p, x, bytes, cudaMemcpyHostToDevice, s->stream));
    if (v) CK(cudaMemcpyAsync(s->v.p, v, bytes, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_set_params(fem_solid s, const fem_params* params)
{
    if (int e = check_handle(s)) return e;
    if (!params) return fail(FEM_E_ARG, "null params");
    if (int e = check_params(params)) return e;
    CK(cudaStreamSynchronize(s->stream));
    s->drop_graph();  // the step graph holds the constants and methods by value
    const fem_params old = s->params;
    const size_t n3 = 3 * (size_t)s->N;
    // buffers the new methods need (kept when a method is switched off)
    if (params->integrator != FEM_INTEGRATOR_QIE_V && !s->xn.p) {
        CK(s->xn.alloc(n3));
        CK(s->vn.alloc(n3));
    }
    if (params->ls_solver == FEM_LS_MINRES && !s->mr_p.p) {
        CK(s->mr_p.alloc(n3));
        CK(s->mr_p0.alloc(n3));
    }
    if (params->material != FEM_MATERIAL_C_WRP && !s->Fe.p) {
        CK(s->Fe.alloc(9 * (size_t)s->T));
        CK(cudaMemsetAsync(s->Fe.p, 0, sizeof(double) * 9 * (size_t)s->T, s->stream));
    }
    if (params->rotation == FEM_ROTATION_DAPD && old.rotation != FEM_ROTATION_DAPD) {
        // DAPD from here on: the previous positions start at the current
        // ones and no element has a direction of collapse yet (as a solid
        // created with DAPD, TetrahedronElementSet3.cpp:190-209)
        if (!s->prev_x.p) CK(s->prev_x.alloc(n3));
        if (!s->doc.p) CK(s->doc.alloc(s->T));
        CK(cudaMemcpyAsync(s->prev_x.p, s->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s->stream));
        const std::vector<uchar2> none(s->T, make_uchar2(3, 0));
        CK(cudaMemcpyAsync(s->doc.p, none.data(), sizeof(uchar2) * s->T, cudaMemcpyHostToDevice, s->stream));
    }
    s->params = *params;
    set_bsr_use(s);
    set_consts(s);
    // a new Young's modulus or Poisson ratio re-bakes every element from the
    // scalar values, as EditableTetrahedronElementSet3::SetParams does
    // (TetrahedronElementSet3.cpp:2168-2200); per-element values given at
    // creation are then replaced
    if (params->young_modulus != old.young_modulus || params->poisson_ratio != old.poisson_ratio) {
        const double E = params->young_modulus, nu = params->poisson_ratio;
        const double a = E / ((1.0 + nu) * (1.0 - 2.0 * nu));  // Compute_E (TetrahedronElement3.h:141-156)
        launch_rebake_material_fp64(s->T, s->vol.p, a * (1.0 - nu), a * nu, a * (0.5 - nu), s->mat.p, s->stream);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

// ---- multi-solid Newton lock-step (LeafDSH_Solid3D_FEM.cpp:2824-3039) ----
namespace {

// The factors of a lock-step phase of step dt (0: quasi-static)
// (NR_MidStep, :2960-2962).
StepConsts lock_consts(const fem_solid s, double dt)
{
    StepConsts c = s->consts;
    c.dt = dt;
    c.inv_dt = dt == 0 ? 0.0 : 1.0 / dt;
    c.factor_M = c.inv_dt * c.inv_dt + c.inv_dt * s->rayleigh[0];
    c.factor_K = 1.0 + c.inv_dt * s->rayleigh[1];
    return c;
}

int check_lock_dt(double dt)
{
    if (!(dt >= 0) || !std::isfinite(dt)) return fail(FEM_E_ARG, "dt must be finite and >= 0");
    return FEM_OK;
}

int check_lock_ready(fem_solid s)
{
    if (!s->lk_x.p) return fail(FEM_E_ARG, "fem_solid_nr_init must come first");
    return FEM_OK;
}

}  // namespace

int fem_solid_nr_init(fem_solid s, double dt)
{
    if (int e = check_handle(s)) return e;
    if (int e = check_lock_dt(dt)) return e;
    const size_t n3 = 3 * (size_t)s->N;
    if (!s->lk_x.p) {
        CK(s->lk_x.alloc(n3));
        CK(s->lk_v.alloc(n3));
    }
    s->lock_stats = false;
    // UpdateKNC (a no-op in the default kinematic mode), BeginEvaluation(
    // m_vecPos0, x), m_vecPos0 = x
    if (int e = open_step(s)) return e;
    CK(cudaGetLastError());
    return FEM_OK;
}

int fem_solid_nr_prestep(fem_solid s, double dt)
{
    if (int e = check_handle(s)) return e;
    if (int e = check_lock_dt(dt)) return e;
    if (int e = check_lock_ready(s)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    CK(cudaMemcpyAsync(s->lk_x.p, s->x.p, bytes, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->lk_v.p, s->v.p, bytes, cudaMemcpyDeviceToDevice, s->stream));
    s->lock_nr_k = 0;
    s->lock_ls_iters = 0;
    return FEM_OK;
}

int fem_solid_nr_midstep(fem_solid s, double dt)
{
    if (int e = check_handle(s)) return e;
    if (int e = check_lock_dt(dt)) return e;
    if (int e = check_lock_ready(s)) return e;
    const StepConsts c = lock_consts(s, dt);
    MeshView<double> m = s->view();
    // f_e at the positions of the cache, which are x_k's array (= x^n after
    // NR_PreStep), with the rotations of the last BeginEvaluation
    elem_force(s, m, s->lk_x.p, 1, nullptr);
    launch_node_b_fie_fp64(m, c, s->lk_x.p, s->x.p, s->v.p, s->lock_nr_k == 0 ? 1 : 0, s->b.p, s->y.p, s->stream);
    launch_knc_fie_fp64(s->N, s->knc_count, s->knc_nodes.p, s->knc_targets.p, s->lk_x.p, s->b.p, s->y.p, s->stream);
    if (int e = ls_solve(s, c, 8)) return e;
    s->lock_ls_iters += s->st_host->k;
    CK(cudaGetLastError());
    if (s->st_host->status == FEM_E_NAN) return fail(FEM_E_NAN, "NaN or Inf in the CG residual");
    return FEM_OK;
}

int fem_solid_nr_poststep(fem_solid s, double dt)
{
    if (int e = check_handle(s)) return e;
    if (int e = check_lock_dt(dt)) return e;
    if (int e = check_lock_ready(s)) return e;
    const StepConsts c = lock_consts(s, dt);
    launch_fie_update_fp64(s->N, c.inv_dt, s->lk_x.p, s->lk_v.p, s->x.p, s->y.p, s->partials.p, s->stream);
    s->lock_nr_k++;
    // EndEvaluation, BeginEvaluation(x, x_k)
    CK(cudaMemsetAsync(&s->st.p->inverted, 0, sizeof(uint32_t), s->stream));
    begin_eval(s, s->x.p, s->lk_x.p);
    CK(cudaGetLastError());
    return FEM_OK;
}

int fem_solid_nr_end(fem_solid s, double dt)
{
    if (int e = check_handle(s)) return e;
    if (int e = check_lock_dt(dt)) return e;
    if (int e = check_lock_ready(s)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    CK(cudaMemcpyAsync(s->x.p, s->lk_x.p, bytes, cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->v.p, s->lk_v.p, bytes, cudaMemcpyDeviceToDevice, s->stream));
    // RecomputeEnergy's potential term; NR_End evaluates no V, so the elastic
    // energy keeps its value (LeafDSH_Solid3D_FEM.cpp:2847-2868, 1554-1584)
    if (s->params.compute_energy) {
        MeshView<double> m = s->view();
        launch_potential_fp64(m, s->consts, s->x.p, s->partials2.p, s->stream);
        launch_finalize(FIN_ENERGY_P, s->partials2.p, grid_for(s->T), s->consts, s->st.p, s->stream);
    }
    s->lock_stats = true;
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_multi_step(fem_solid* solids, uint32_t count, double dt, uint32_t nsteps)
{
    if (!solids || count == 0) return fail(FEM_E_ARG, "no solids");
    for (uint32_t i = 0; i < count; i++)
        if (int e = check_handle(solids[i])) return e;
    uint32_t max_nr_iter = 0;
    for (uint32_t i = 0; i < count; i++) max_nr_iter = std::max(max_nr_iter, solids[i]->params.nr_max_iter);
    for (uint32_t step = 0; step < nsteps; step++) {
        for (uint32_t i = 0; i < count; i++)
            if (int e = fem_solid_nr_init(solids[i], dt)) return e;
        uint32_t nr_iter = 0;
        do {
            for (uint32_t i = 0; i < count; i++) {
                if (int e = fem_solid_nr_prestep(solids[i], dt)) return e;
                if (int e = fem_solid_nr_midstep(solids[i], dt)) return e;
            }
            for (uint32_t i = 0; i < count; i++)
                if (int e = fem_solid_nr_poststep(solids[i], dt)) return e;
        } while (++nr_iter < max_nr_iter);
        for (uint32_t i = 0; i < count; i++)
            if (int e = fem_solid_nr_end(solids[i], dt)) return e;
    }
    return FEM_OK;
}

int fem_solid_get_params(fem_solid s, fem_params* params)
{
    if (int e = check_handle(s)) return e;
    if (!params) return fail(FEM_E_ARG, "null params");
    *params = s->params;
    return FEM_OK;
}

int fem_solid_get_dapd_state(fem_solid s, double* prev_x, uint8_t* doc)
{
    if (int e = check_handle(s)) return e;
    if (!uses_dapd(s)) return fail(FEM_E_ARG, "the solid does not use the DAPD rotation");
    if (prev_x)
        CK(cudaMemcpyAsync(prev_x, s->prev_x.p, sizeof(double) * 3 * (size_t)s->N, cudaMemcpyDeviceToHost,
                           s->stream));
    if (doc) CK(cudaMemcpyAsync(doc, s->doc.p, sizeof(uchar2) * s->T, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_set_dapd_state(fem_solid s, const double* prev_x, const uint8_t* doc)
{
    if (int e = check_handle(s)) return e;
    if (!uses_dapd(s)) return fail(FEM_E_ARG, "the solid does not use the DAPD rotation");
    if (doc)
        for (uint32_t e = 0; e < s->T; e++) {
            const uint8_t a = doc[2 * (size_t)e], b = doc[2 * (size_t)e + 1];
            // none (3, 0), V-F (v, v) or E-E (a < b), vertex ids 0..3
            if (!((a == 3 && b == 0) || (a <= 3 && b <= 3 && a <= b)))
                return fail(FEM_E_ARG, "element %u: (%u, %u) is not a direction of collapse", e, a, b);
        }
    if (prev_x)
        CK(cudaMemcpyAsync(s->prev_x.p, prev_x, sizeof(double) * 3 * (size_t)s->N, cudaMemcpyHostToDevice,
                           s->stream));
    if (doc) CK(cudaMemcpyAsync(s->doc.p, doc, sizeof(uchar2) * s->T, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_get_state(fem_solid s, double* x, double* v)
{
    if (int e = check_handle(s)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    if (x) CK(cudaMemcpyAsync(x, s->x.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    if (v) CK(cudaMemcpyAsync(v, s->v.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_step_async(fem_solid s, uint32_t nsteps)
{
    if (int e = check_handle(s)) return e;
    for (uint32_t i = 0; i < nsteps; i++)
        if (int e = step_once(s, 8)) return e;
    return FEM_OK;
}

int fem_solid_synchronize(fem_solid s, fem_step_stats* stats)
{
    if (int e = check_handle(s)) return e;
    CK(cudaMemcpyAsync(s->st_host, s->st.p, sizeof(StepScalars), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (stats) fill_stats(s, *s->st_host, stats);
    if (s->st_host->status == FEM_E_NAN) return fail(FEM_E_NAN, "NaN or Inf in the CG residual");
    return FEM_OK;
}

int fem_solid_step(fem_solid s, uint32_t nsteps, fem_step_stats* stats)
{
    if (int e = fem_solid_step_async(s, nsteps)) return e;
    return fem_solid_synchronize(s, stats);
}

int fem_solid_step_host(fem_solid s, const double* x_in, const double* v_in, uint32_t nsteps, double* x_out,
                        double* v_out, fem_step_stats* stats)
{
    if (int e = check_handle(s)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    if (x_in) CK(cudaMemcpyAsync(s->x.p, x_in, bytes, cudaMemcpyHostToDevice, s->stream));
    if (v_in) CK(cudaMemcpyAsync(s->v.p, v_in, bytes, cudaMemcpyHostToDevice, s->stream));
    if (int e = fem_solid_step_async(s, nsteps)) return e;
    if (x_out) CK(cudaMemcpyAsync(x_out, s->x.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    if (v_out) CK(cudaMemcpyAsync(v_out, s->v.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    return fem_solid_synchronize(s, stats);
}

int fem_solid_stream(fem_solid s, void** stream)
{
    if (int e = check_handle(s)) return e;
    if (!stream) return fail(FEM_E_ARG, "null stream pointer");
    *stream = (void*)s->stream;
    return FEM_OK;
}

int fem_solid_begin_eval(fem_solid s, const double* x)
{
    if (int e = check_handle(s)) return e;
    if (!x) return fail(FEM_E_ARG, "null positions");
    CK(cudaMemcpyAsync(s->tmp.p, x, sizeof(double) * 3 * (size_t)s->N, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(&s->st.p->inverted, 0, sizeof(uint32_t), s->stream));
    begin_eval(s, s->prev_x.p, s->tmp.p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->stream));
    s->evaluated = true;
    return FEM_OK;
}

int fem_solid_get_rotations(fem_solid s, double* R, double* detF)
{
    if (int e = check_handle(s)) return e;
    const size_t T = s->T;
    if (R) {
        std::vector<double> soa(9 * T);
        CK(cudaMemcpyAsync(soa.data(), s->R.p, sizeof(double) * 9 * T, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (size_t e = 0; e < T; e++)
            for (int c = 0; c < 9; c++) R[9 * e + c] = soa[(size_t)c * T + e];
    }
    if (detF) {
        CK(cudaMemcpyAsync(detF, s->detF.p, sizeof(double) * T, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return FEM_OK;
}

int fem_solid_get_doc(fem_solid s, uint8_t* doc)
{
    if (int e = check_handle(s)) return e;
    if (!doc) return fail(FEM_E_ARG, "null output");
    if (!uses_dapd(s)) return fail(FEM_E_ARG, "the solid does not use the DAPD rotation");
    CK(cudaMemcpyAsync(doc, s->doc.p, sizeof(uchar2) * s->T, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_force_elastic(fem_solid s, double* f)
{
    if (int e = check_handle(s)) return e;
    if (!f) return fail(FEM_E_ARG, "null force array");
    if (!s->evaluated) return fail(FEM_E_ARG, "fem_solid_begin_eval must come first");
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    // positions of the last evaluation are in tmp
    CK(cudaMemcpyAsync(s->q.p, f, bytes, cudaMemcpyHostToDevice, s->stream));
    elem_force(s, s->view(), s->tmp.p, 1, nullptr);
    launch_gather_sum_fp64(s->view(), -1.0, s->q.p, s->stream);
    CK(cudaMemcpyAsync(f, s->q.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_df_x(fem_solid s, const double* dx, double* df)
{
    if (int e = check_handle(s)) return e;
    if (!dx || !df) return fail(FEM_E_ARG, "null arrays");
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    CK(cudaMemcpyAsync(s->d.p, dx, bytes, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->q.p, df, bytes, cudaMemcpyHostToDevice, s->stream));
    elem_spmv(s, s->view(), s->d.p, 0);
    launch_gather_sum_fp64(s->view(), -1.0, s->q.p, s->stream);
    CK(cudaMemcpyAsync(df, s->q.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_apply_A(fem_solid s, double factor_M, double factor_K, const double* d, double* q)
{
    if (int e = check_handle(s)) return e;
    if (!d || !q) return fail(FEM_E_ARG, "null arrays");
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    CK(cudaMemcpyAsync(s->d.p, d, bytes, cudaMemcpyHostToDevice, s->stream));
    elem_spmv(s, s->view(), s->d.p, 0);
    launch_apply_A_fp64(s->view(), factor_M, factor_K, s->node_mass, s->d.p, s->q.p, s->stream);
    CK(cudaMemcpyAsync(q, s->q.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}

int fem_solid_energy(fem_solid s, double* V)
{
    if (int e = check_handle(s)) return e;
    if (!V) return fail(FEM_E_ARG, "null output");
    if (!s->evaluated) return fail(FEM_E_ARG, "fem_solid_begin_eval must come first");
    elem_force(s, s->view(), s->tmp.p, 0, s->partials2.p);
    launch_finalize(FIN_ENERGY_E, s->partials2.p, grid_for(s->T), s->consts, s->st.p, s->stream);
    CK(cudaMemcpyAsync(s->st_host, s->st.p, sizeof(StepScalars), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *V = s->st_host->elastic_energy;
    return FEM_OK;
}

int fem_solid_mass_info(fem_solid s, double* node_mass, double* rayleigh2, double* total_volume)
{
    if (int e = check_handle(s)) return e;
    if (node_mass) *node_mass = s->node_mass;
    if (rayleigh2) {
        rayleigh2[0] = s->rayleigh[0];
        rayleigh2[1] = s->rayleigh[1];
    }
    if (total_volume) *total_volume = s->total_volume;
    return FEM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// fem_solid_apply_A_noalloc: the product of fem_solid_apply_A with its
// per-element scratch (12 doubles per tet, written by the element kernel and
// gathered per node) in a static device array instead of the solid's own
// buffer. It is meant for callers that cannot allocate device memory when
// they call it: a fixed-rate control or haptics loop, where cudaMalloc's
// implicit device synchronisation and unbounded latency would break the
// loop's deadline, or a process whose device memory is already reserved by
// another allocator (a framework's caching allocator, say). It calls no
// cudaMalloc, cudaFree or other allocating CUDA, torch or library routine.
//
// Limits and sharing:
//   * at most FEM_NOALLOC_MAX_TETS tets (the array is 12 * 65536 doubles,
//     6 MiB, per device); larger solids are rejected with FEM_E_ARG;
//   * every call on a device uses the same array, which keeps the last
//     call's contents. Nothing in it has to start at zero: the element
//     kernel writes all 12 T entries before the gather reads them. Calls
//     whose work overlaps on the GPU (several host threads calling at once,
//     on solids whose streams run concurrently) race on the array: serialise
//     them;
//   * set-up: host code cannot use the array's name as a device address, so
//     fem_solid_create looks the address up (cudaGetSymbolAddress, with the
//     solid's device current) for every solid small enough to use it, and
//     keeps it in the solid. The array lives in a module without kernels;
//     under CUDA's lazy module loading that first lookup loads the module,
//     which reserves its 6 MiB and may synchronise the device -- work done
//     inside fem_solid_create, which allocates anyway, so that the no-alloc
//     call itself never does it. Only if that lookup failed does the first
//     no-alloc call on the solid retry it (and then it should come before
//     any stream capture).
namespace {

static __device__ __align__(256) double g_apply_scratch[12ull * FEM_NOALLOC_MAX_TETS];

// Device address of the static scratch on the current device.
int apply_scratch(double** out)
{
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_apply_scratch);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(FEM_E_CUDA, "cudaGetSymbolAddress of the static scratch: %s", cudaGetErrorString(e));
    }
    *out = static_cast<double*>(p);
    return FEM_OK;
}

}  // namespace

extern "C" int fem_solid_apply_A_noalloc(fem_solid s, double factor_M, double factor_K, const double* d, double* q)
{
    if (int e = check_handle(s)) return e;
    if (!d || !q) return fail(FEM_E_ARG, "null arrays");
    if (s->T > FEM_NOALLOC_MAX_TETS)
        return fail(FEM_E_ARG, "solid has %u tets; fem_solid_apply_A_noalloc takes at most %u (static scratch)",
                    s->T, (unsigned)FEM_NOALLOC_MAX_TETS);
    if (!s->noalloc_scratch)
        if (int e = apply_scratch(&s->noalloc_scratch)) return e;
    MeshView<double> m = s->view();
    m.eout = s->noalloc_scratch;
    const size_t bytes = sizeof(double) * 3 * (size_t)s->N;
    CK(cudaMemcpyAsync(s->d.p, d, bytes, cudaMemcpyHostToDevice, s->stream));
    elem_spmv(s, m, s->d.p, 0);
    launch_apply_A_fp64(m, factor_M, factor_K, s->node_mass, s->d.p, s->q.p, s->stream);
    CK(cudaMemcpyAsync(q, s->q.p, bytes, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FEM_OK;
}
