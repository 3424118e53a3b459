// batch.cu -- host runtime of the tiled, batched step: the fem_batch_* part
// of include/fem_tet.h.
//
// A batch holds independent solids (the reference's many-solid scheme steps
// its Solid3D leaves one after another, SS_AggregateDSH_Basic.cpp:229-300;
// here they step together). Each solid keeps the reference's per-solid
// semantics: its own parameters, constraints, CG loop and stopping test
// (ILSS_CG.h:86-88), so its results do not depend on the other solids.
//
// Set-up (fem_batch_finalize): per mesh, elements are put in Morton order of
// their centroids and cut into tiles of at most tile_elems tets and 256
// local nodes (120 for the mixed path's tiles of up to 128 tets); the element data (Dm^-1, E-matrix entries times V, FP64 for
// the once-per-step kernels and in the path's type S for the CG products)
// follow that order. Node numbering is the caller's.
//
// Step: one CUDA graph per batch -- the once-per-step kernels, then a
// conditional while node whose body is one CG iteration of every mesh still
// iterating and whose condition the per-mesh finaliser sets on the device,
// then integration and energies. No host synchronisation inside a step.
#include "../../include/fem_tet.h"
#include "batch.cuh"
#include "batch_launch.h"
#include "graph_capture.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

using namespace femgb;

namespace femgb {
int batch_fail(int code, const char* fmt, ...);
}

namespace {

#define BCK(call)                                                                                          \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return batch_fail(e_ == cudaErrorMemoryAllocation ? FEM_E_OOM : FEM_E_CUDA, "%s: %s (%s:%d)", #call, \
                              cudaGetErrorString(e_), __FILE__, __LINE__);                                 \
    } while (0)

struct HostMesh {
    std::vector<double> rest;
    std::vector<uint32_t> tets;
    fem_params p;
    std::vector<double> E, nu;
    std::vector<uint32_t> knc_nodes;
    std::vector<double> knc_targets;
};

template <typename T>
struct Dev {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        n = count;
        return cudaMalloc(&p, sizeof(T) * (count ? count : 1));
    }
    cudaError_t upload(const std::vector<T>& h, cudaStream_t s)
    {
        if (h.empty()) return cudaSuccess;
        return cudaMemcpyAsync(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
    }
    size_t bytes() const { return sizeof(T) * n; }
};

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

uint32_t spread10(uint32_t v)
{
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}

}  // namespace

static_assert(kMeshRotationMsvd == FEM_ROTATION_MSVD && kMeshRotationDapd == FEM_ROTATION_DAPD,
              "per-mesh rotation values are enum fem_rotation's");
static_assert(kMeshSolverCg == FEM_LS_CG && kMeshSolverMinres == FEM_LS_MINRES, "solver ids follow fem_tet.h");
static_assert(kMeshQie == FEM_INTEGRATOR_QIE_V && kMeshFie == FEM_INTEGRATOR_FIE_DX &&
                  kMeshFieQuasi == FEM_INTEGRATOR_FIE_DX_QUASISTATIC,
              "integrator ids follow fem_tet.h");
static_assert(kTileMaterialWrp == FEM_MATERIAL_C_WRP && kTileMaterialLcm == FEM_MATERIAL_C_LCM &&
                  kTileMaterialLcmh == FEM_MATERIAL_C_LCMH && kTileMaterialCcm == FEM_MATERIAL_C_CCM,
              "per-tile material values are enum fem_material's");

struct fem_batch_s {
    fem_batch_options opt{};
    std::vector<HostMesh> meshes;
    bool finalized = false;
    uint32_t M = 0, ntiles = 0, nchunks = 0, K = 0;
    uint64_t Ntot = 0, Ttot = 0, nslots = 0;
    std::vector<MeshConsts> mc_host;
    std::vector<uint32_t> knc_base;   // per mesh first KNC entry
    cudaStream_t stream = nullptr;
    // device buffers (type-erased for S)
    Dev<TileMeta> tiles;
    Dev<ChunkMeta> chunks;
    Dev<MeshConsts> mc;
    Dev<StepScalars> st;
    Dev<uint8_t> active;
    Dev<int4> gtets;
    Dev<unsigned char> Dinv_s, mat_s, R_s;  // S-typed, raw bytes
    Dev<double> Dinv64, vol, detF;
    Dev<uint32_t> tile_nodes, lptr0, ov_ptr, ov_map, knc_node, knc_mesh;
    std::vector<uint32_t> perm_h, inv_h;  // batch node -> caller's node, and back (global ids)
    std::vector<uint32_t> eperm_h;        // batch element -> the caller's element index in its mesh
    Dev<uint32_t> perm;                   // perm_h on the device (whole-batch state transfers)
    Dev<double> stage_x, stage_v;         // caller-order staging for whole-batch transfers
    Dev<uchar4> lconn;
    Dev<uint16_t> lptr, lidx;
    Dev<uint8_t> fixed;
    Dev<double> rest, x, v, bvec, y, part64, cpart, tpart, knc_target;
    Dev<unsigned char> r_s, d_s, q_s, part_s, ydelta_s;  // S-typed
    Dev<unsigned> counter, any_flag, refresh_flag, mcount, err;
    Dev<unsigned> gbar;  // persistent loop: grid-barrier arrivals, generation, go flag
    Dev<double> prev_x;  // DAPD meshes: positions at the start of their last step (batch node order)
    Dev<uchar2> doc;     // DAPD meshes: direction of collapse per element (batch element order)
    Dev<double> Fe;      // C_LCM meshes: F of the last BeginEvaluation (SoA, batch element order)
    bool any_dapd = false;
    bool any_lcm = false;   // some mesh has a P-K material (C_LCM, C_LCMH, C_CCM)
    bool any_lcmh = false;
    Dev<float> lcmh_w;      // mixed C_LCMH meshes: the blend weight per element
    bool any_minres = false;
    bool any_fie = false;
    Dev<double> xn, vn;                  // FIE meshes: x^n, v^n of the step (lock-step: x_k, v_k)
    // the multi-solid Newton lock-step (fem_batch_nr_*)
    std::vector<double> ray0, ray1;      // per mesh: the Rayleigh coefficients a0, a1
    std::vector<double> vol_total;       // per mesh: rest volume summed in the reference's element order
    std::vector<uint8_t> elem_mat;       // per mesh: per-element E or nu were given (and not replaced since)
    std::vector<uint8_t> mat_scalar;     // per mesh: its element data hold values baked from the scalar E, nu
    Dev<MeshConsts> mc_lock;             // the meshes' constants with the lock-step's factors
    double lock_dt = -1.0;               // dt of mc_lock (-1: none yet)
    bool lock = false;                   // views use mc_lock and the lock-step's branches
    bool lock_open = false;              // between fem_batch_nr_init and fem_batch_nr_end
    bool lock_stats = false;             // the last call was fem_batch_nr_end (its statistics)
    Dev<unsigned char> mr_p_s, mr_p0_s;  // MINRES meshes: directions p, p0 (S-typed)
    Dev<double> cpart_b;                 // MINRES meshes: per-chunk |b|^2 partials
    Dev<unsigned char> blob;
    Dev<uint32_t> blob_off16;
    Dev<uint32_t> act_tiles, act_chunks, act_count;
    Dev<unsigned> list_dirty;
    Dev<unsigned> slice;                // [iteration budget of a launch (0 = none), iterations run]
    Dev<uint32_t> start_tiles, start_chunks, launch_tiles, launch_chunks, refresh_tiles, refresh_chunks, list_count;
    uint32_t slice_budget = 0;
    std::vector<uint8_t> mask_host;     // last active mask (empty = all start)
    StepScalars* st_host = nullptr;
    unsigned* err_host = nullptr;  // pinned copy of the error word (server readback)
    // step graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t device_bytes = 0;

    size_t S_size() const { return opt.precision == FEM_PRECISION_FP64 ? 8 : 4; }

    template <typename S>
    BatchView<S> view() const
    {
        BatchView<S> b;
        b.M = M;
        b.ntiles = ntiles;
        b.nchunks = nchunks;
        b.pipe_tile = opt.tile_elems <= (uint32_t)kPipeSmallTile ? kPipeSmallTile : kTileElems;
        b.fuse_alpha = opt.fuse_alpha ? 1u : 0u;
        b.has_lcm = any_lcmh ? 2u : any_lcm ? 1u : 0u;
        b.lock = lock ? 1u : 0u;
        b.Ntot = (uint32_t)Ntot;
        b.Ttot = (uint32_t)Ttot;
        b.nslots = nslots;
        b.tiles = tiles.p;
        b.chunks = chunks.p;
        b.mc = lock ? mc_lock.p : mc.p;
        b.st = st.p;
        b.active = active.p;
        b.gtets = gtets.p;
        b.Dinv = reinterpret_cast<const S*>(Dinv_s.p);
        b.mat = reinterpret_cast<const S*>(mat_s.p);
        b.R = reinterpret_cast<S*>(R_s.p);
        b.Dinv64 = Dinv64.p;
        b.vol = vol.p;
        b.detF = detF.p;
        b.tile_nodes = tile_nodes.p;
        b.lconn = lconn.p;
        b.lptr = lptr.p;
        b.lidx = lidx.p;
        b.lptr0 = lptr0.p;
        b.ov_ptr = ov_ptr.p;
        b.ov_map = ov_map.p;
        b.fixed = fixed.p;
        b.rest = rest.p;
        b.ydelta = opt.precision == FEM_PRECISION_MIXED ? reinterpret_cast<S*>(ydelta_s.p) : nullptr;
        b.blob = opt.precision == FEM_PRECISION_MIXED ? blob.p : nullptr;
        b.blob_off16 = blob_off16.p;
        b.prev_x = prev_x.p;
        b.doc = doc.p;
        b.Fe = Fe.p;
        b.lcmh_w = lcmh_w.p;
        b.mr_p = reinterpret_cast<S*>(mr_p_s.p);
        b.mr_p0 = reinterpret_cast<S*>(mr_p0_s.p);
        b.mr_v1 = reinterpret_cast<S*>(q_s.p);
        b.cpart_b = cpart_b.p;
        b.xn = xn.p;
        b.vn = vn.p;
        const bool mixed = opt.precision == FEM_PRECISION_MIXED;
        b.act_tiles = mixed ? act_tiles.p : nullptr;
        b.act_chunks = mixed ? act_chunks.p : nullptr;
        b.act_count = mixed ? act_count.p : nullptr;
        b.list_dirty = mixed ? list_dirty.p : nullptr;
        b.start_tiles = start_tiles.p;
        b.start_chunks = start_chunks.p;
        b.launch_tiles = launch_tiles.p;
        b.launch_chunks = launch_chunks.p;
        b.refresh_tiles = mixed ? refresh_tiles.p : nullptr;
        b.refresh_chunks = mixed ? refresh_chunks.p : nullptr;
        b.list_count = list_count.p;
        b.knc_node = knc_node.p;
        b.knc_mesh = knc_mesh.p;
        b.knc_target = knc_target.p;
        return b;
    }

    void release()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        tiles.release(); chunks.release(); mc.release(); st.release(); active.release(); gtets.release();
        Dinv_s.release(); mat_s.release(); R_s.release(); Dinv64.release(); vol.release(); detF.release();
        tile_nodes.release(); lptr0.release(); ov_ptr.release(); ov_map.release(); knc_node.release();
        perm.release(); stage_x.release(); stage_v.release();
        knc_mesh.release(); lconn.release(); lptr.release(); lidx.release(); fixed.release(); rest.release();
        x.release(); v.release(); bvec.release(); y.release(); part64.release(); cpart.release(); tpart.release();
        knc_target.release(); r_s.release(); d_s.release(); q_s.release(); part_s.release(); ydelta_s.release(); counter.release();
        any_flag.release(); refresh_flag.release(); mcount.release(); err.release(); gbar.release(); blob.release();
        prev_x.release(); doc.release(); Fe.release(); lcmh_w.release();
        mr_p_s.release(); mr_p0_s.release(); cpart_b.release(); xn.release(); vn.release(); mc_lock.release();
        blob_off16.release();
        act_tiles.release(); act_chunks.release(); act_count.release(); list_dirty.release(); slice.release();
        start_tiles.release(); start_chunks.release(); launch_tiles.release(); launch_chunks.release();
        refresh_tiles.release(); refresh_chunks.release();
        list_count.release();
        if (st_host) cudaFreeHost(st_host);
        st_host = nullptr;
        if (err_host) cudaFreeHost(err_host);
        err_host = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

namespace femgb {
void set_last_error(const char* msg);
int batch_fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    set_last_error(buf);
    return code;
}
// Server support (server.cu): queue the per-mesh statistics and the error
// word into pinned host memory on the batch's stream; they are valid once
// the stream has passed this point.
int batch_enqueue_readback(fem_batch b)
{
    cudaError_t e = cudaMemcpyAsync(b->st_host, b->st.p, sizeof(StepScalars) * b->M, cudaMemcpyDeviceToHost,
                                    b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->err_host, b->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream);
    if (e != cudaSuccess) return batch_fail(FEM_E_CUDA, "stats readback: %s", cudaGetErrorString(e));
    return FEM_OK;
}
unsigned batch_host_err(fem_batch b) { return b->err_host ? *b->err_host : 0u; }
}  // namespace femgb

namespace {

template <typename S>
std::vector<unsigned char> as_bytes(const std::vector<double>& src)
{
    std::vector<unsigned char> out(src.size() * sizeof(S));
    S* o = reinterpret_cast<S*>(out.data());
    for (size_t i = 0; i < src.size(); i++) o[i] = (S)src[i];
    return out;
}

// The parameter-dependent constants of a mesh from its params, its total
// rest volume (summed in the reference's element order) and node count:
// node mass (RebuildMass), Rayleigh coefficients (RebuildRayleighCoeffsFrom
// Freqs), the system factors of the integrator (Step_QuasiImplicitEuler_v,
// Step_FullyImplicitEuler_dx), tolerances and the method settings. The
// structural fields of c (ranges of nodes, elements, tiles, chunks,
// constraints) are left as they are; ray receives a0, a1.
void param_consts(MeshConsts& c, const fem_params& p, double acc_total_volume, uint32_t N, bool fp64, double* ray)
{
    const double total_mass = p.density * acc_total_volume;
    const double mass_per_node = total_mass / N;
    const double inv_mass = (double)1.0f / mass_per_node;
    {
        const double f1 = (double)0.1f, f2 = (double)10000.0f;
        const double o00 = 1.0 / f1, o01 = f1, o10 = 1.0 / f2, o11 = f2;
        const double inv_det = 1.0 / (o00 * o11 - o10 * o01);
        const double i00 = inv_det * o11, i01 = -inv_det * o01, i10 = -inv_det * o10, i11 = inv_det * o00;
        const double z = 2 * p.damping_ratio;
        double a0 = 0, a1 = 0;
        a0 += i00 * z; a0 += i01 * z;
        a1 += i10 * z; a1 += i11 * z;
        ray[0] = a0;
        ray[1] = a1;
    }
    c.dt = p.fixed_dt;
    c.inv_dt = 1.0 / p.fixed_dt;
    c.mass = 1.0 / inv_mass;
    c.factor_M = 1.0 + c.dt * ray[0];
    c.factor_K = c.dt * c.dt + c.dt * ray[1];
    c.integrator = p.integrator;
    c.nr_max_iter = p.nr_max_iter;
    c.nr_abs_eps = p.nr_abs_epsilon;
    if (p.integrator != FEM_INTEGRATOR_QIE_V) {
        // Step_FullyImplicitEuler_dx's system (LeafDSH_Solid3D_FEM.cpp:
        // 1357-1411): A = (1/h^2 + a0/h) M + (1 + a1/h) K; the
        // quasi-static variant drops every 1/h term
        const bool quasi = p.integrator == FEM_INTEGRATOR_FIE_DX_QUASISTATIC;
        c.dt = quasi ? 0.0 : p.fixed_dt;
        c.inv_dt = quasi ? 0.0 : 1.0 / p.fixed_dt;
        c.factor_M = c.inv_dt * c.inv_dt + c.inv_dt * ray[0];
        c.factor_K = 1.0 + c.inv_dt * ray[1];
    }
    for (int a = 0; a < 3; a++) c.gravity[a] = p.gravity[a];
    c.density = p.density;
    c.rel_eps_sq = p.ls_rel_epsilon * p.ls_rel_epsilon;
    c.abs_eps_sq = p.ls_abs_epsilon * p.ls_abs_epsilon;
    c.degenerate_det_F = p.degenerate_det_F;
    c.rot_check = (float)p.rotation_check;
    c.rot_fp32 = p.rotation_fp32 ? 1u : 0u;
    c.rotation = p.rotation;
    c.material = p.material;
    c.ecie_k = (double)(float)p.ecie_k_factor;  // float32 in the reference's Params
    // the element set's Lame pair (from its Params, TetrahedronElementSet3.cpp:143-148)
    c.lame_mu = 0.5 * p.young_modulus / (1 + p.poisson_ratio);
    c.lame_lambda = p.young_modulus * p.poisson_ratio / ((1.0 + p.poisson_ratio) * (1.0 - 2.0 * p.poisson_ratio));
    // the reference's DAPD factors are float (ms::fem::Params)
    c.dapd_thr = p.dapd_threshold_det_F;
    c.dapd_fL = (double)(float)p.dapd_l_factor;
    c.dapd_fNL = (double)(float)p.dapd_nl_factor;
    c.dapd_eNL = (double)(float)p.dapd_nl_exponent;
    c.solver = p.ls_solver;
    c.refresh_drop_sq = fp64 ? 0.0 : p.refresh_drop * p.refresh_drop;
    c.max_iter = p.ls_max_iter;
    c.refresh_every = fp64 ? 0u : p.refresh_every;
    c.fK_f = (float)c.factor_K;
    c.mfm_f = (float)(c.mass * c.factor_M);
}


// Enqueue one launch of the step on `s`:
//   reset (one block: which meshes start, continue or are left out)
//   IF some mesh starts: BeginEvaluation, f_e, b, constraints, A y, r0
//   WHILE some mesh iterates (and the launch's iteration budget is not
//         spent): one CG iteration (mixed: IF refresh { FP64 A y })
//   integration and energies of the meshes whose loop ended in this launch.
// With an FIE mesh in the batch the step has a Newton level:
//   reset
//   IF some mesh starts: BeginEvaluation
//   WHILE some mesh takes a Newton iteration (QIE meshes take one):
//     f_e, b_k, constraints, A y, r0 and the per-mesh |b_k| test
//     WHILE some mesh iterates: one CG (or MINRES) iteration
//     QIE: integration; FIE: x_k += y, v_k, |y|, the Newton count and
//     limit, BeginEvaluation(x^n, x_k); the next iteration's lists
//   energies.
// In graph capture the conditions are set on the device; outside capture the
// same kernels run with the loops on the host, in chunks, reading the
// meshes' flags.
template <typename S>
int enqueue_step(fem_batch B, cudaStream_t s, bool capture, int lock_phase = 0)
{
    const BatchView<S> b = B->view<S>();
    const bool mixed = B->opt.precision == FEM_PRECISION_MIXED;
    const bool newton = B->any_fie;
    S* r = reinterpret_cast<S*>(B->r_s.p);
    S* d = reinterpret_cast<S*>(B->d_s.p);
    S* q = reinterpret_cast<S*>(B->q_s.p);
    S* part = reinterpret_cast<S*>(B->part_s.p);
    using L = BatchLaunch<S>;
    cudaGraphConditionalHandle cond = 0, if_start = 0, nw = 0;
    cudaGraph_t top = nullptr;
    if (capture) {
        cudaStreamCaptureStatus cs;
        BCK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &top, nullptr, nullptr, nullptr));
        if (!newton) BCK(cudaGraphConditionalHandleCreate(&cond, top, 0, cudaGraphCondAssignDefault));
        BCK(cudaGraphConditionalHandleCreate(&if_start, top, 0, cudaGraphCondAssignDefault));
        if (newton) BCK(cudaGraphConditionalHandleCreate(&nw, top, 0, cudaGraphCondAssignDefault));
    }
    LoopSync ls;
    ls.mcount = B->mcount.p;
    ls.gcount = B->counter.p;
    ls.refresh_flag = B->refresh_flag.p;
    ls.body_runs = nullptr;
    ls.err = B->err.p;
    ls.slice = B->slice.p;
    ls.cond = cond;
    ls.set_cond = capture ? 1 : 0;
    LoopSync lb = ls;
    lb.body_runs = B->any_flag.p;
    // f_e, b, constraints, A y, r0 of the meshes in the start lists (the
    // lock-step's at its iterate x_k)
    const double* xk = B->lock ? B->xn.p : B->x.p;
    auto solve_start = [&](cudaStream_t ss) {
        L::tile_force(b, xk, B->part64.p, nullptr, ss);
        L::node_b(b, B->part64.p, B->v.p, B->x.p, B->bvec.p, B->y.p, ss);
        L::knc(b, B->K, xk, B->bvec.p, B->y.p, ss);
        L::tile_spmv_y64(b, B->y.p, B->part64.p, 0, nullptr, ss);
        L::node_residual(b, B->part64.p, B->bvec.p, B->y.p, r, d, B->cpart.p, ls, ss);
        if (B->any_minres) L::node_mr_finish(b, B->y.p, r, d, q, ls, ss);
    };
    // mixed: the tile product also writes each tile's share of d^T A d; one
    // fused node pass forms alpha from the shares and does the rest
    auto body_head = [&](cudaStream_t bs, cudaGraphConditionalHandle ifh, int set_if) {
        if constexpr (sizeof(S) == 4)
            launch_tile_spmv_pipe(b, d, r, part, reinterpret_cast<float2*>(B->tpart.p), ifh, set_if,
                                  set_if ? B->refresh_flag.p : nullptr, B->err.p, bs);
        else
            L::tile_spmv(b, d, r, part, ifh, 0, B->refresh_flag.p, bs);
    };
    auto body_tail = [&](cudaStream_t bs) {
        if constexpr (sizeof(S) == 4) {
            launch_node_update_fused(b, part, reinterpret_cast<const float2*>(B->tpart.p), B->part64.p, B->bvec.p,
                                     B->y.p, r, d, reinterpret_cast<float2*>(B->cpart.p), lb, bs);
        } else {
            L::node_q(b, part, d, q, nullptr, B->bvec.p, B->y.p, r, B->cpart.p, lb, bs);
            L::node_update(b, B->y.p, r, d, q, B->cpart.p, lb, bs);
        }
        // MINRES meshes: the iteration's vector and iterate updates, after
        // their loop test
        if (B->any_minres) L::node_mr_finish(b, B->y.p, r, d, q, ls, bs);
    };
    // the CG loop as a WHILE node after the capture point of `cs`
    auto capture_cg = [&](cudaStream_t cs) {
        return capture_conditional(cs, ls.cond, cudaGraphCondTypeWhile, [&](cudaStream_t bs, cudaGraph_t bodyg) {
            cudaGraphConditionalHandle ifh = 0;
            if (mixed) {
                const cudaError_t e = cudaGraphConditionalHandleCreate(&ifh, bodyg, 0, 0);
                if (e != cudaSuccess) return e;
            }
            body_head(bs, ifh, mixed ? 1 : 0);
            if (mixed) {
                // IF (some mesh refreshes this iteration) { FP64 product of y }
                const cudaError_t e = capture_conditional(bs, ifh, cudaGraphCondTypeIf, [&](cudaStream_t is, cudaGraph_t) {
                    L::tile_spmv_y64(b, B->y.p, B->part64.p, 1, nullptr, is);
                    return cudaGetLastError();
                });
                if (e != cudaSuccess) return e;
            }
            body_tail(bs);
            return cudaGetLastError();
        });
    };
    // the CG loop driven from the host: chunks of iterations, then read the
    // per-mesh flags
    auto host_cg = [&]() -> int {
        bool coop = false;
        if constexpr (sizeof(S) == 4) {
            if (B->opt.persistent_loop) {
                // every iteration of this launch in one cooperative kernel,
                // with about two tiles per block of the meshes taking part
                uint64_t tiles = 0;
                for (uint32_t m = 0; m < B->M; m++)
                    if (B->mask_host.empty() || B->mask_host[m] != 0) tiles += B->mc_host[m].ntiles;
                const uint32_t blocks = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1, (tiles + 1) / 2), 1u << 20);
                CoopLoopArgs a;
                a.d = d; a.r = r; a.part = part; a.tshare = reinterpret_cast<float2*>(B->tpart.p);
                a.part64 = B->part64.p; a.bv = B->bvec.p; a.y = B->y.p;
                a.cshare = reinterpret_cast<float2*>(B->cpart.p); a.err = B->err.p; a.gbar = B->gbar.p;
                a.ls = lb;
                a.ls.set_cond = 0;
                if (tiles <= cg_resident_capacity(B->M))
                    BCK(launch_cg_resident(b, a, (uint32_t)tiles, s));
                else
                    BCK(launch_cg_coop(b, a, blocks, s));
                coop = true;
            }
        }
        uint32_t budget = B->slice_budget, ran = 0;
        for (; !coop;) {
            BCK(cudaMemcpyAsync(B->st_host, B->st.p, sizeof(StepScalars) * B->M, cudaMemcpyDeviceToHost, s));
            BCK(cudaStreamSynchronize(s));
            bool any = false;
            for (uint32_t m = 0; m < B->M; m++) any |= !B->st_host[m].done;
            if (!any || (budget && ran >= budget)) break;
            for (int i = 0; i < 8 && !(budget && ran >= budget); i++, ran++) {
                body_head(s, 0, 0);
                if (mixed) L::tile_spmv_y64(b, B->y.p, B->part64.p, 1, B->refresh_flag.p, s);
                body_tail(s);
            }
        }
        return FEM_OK;
    };
    // after a solve: QIE integration or the FIE update, re-evaluation and
    // the next Newton iteration's lists
    auto after_solve = [&](cudaStream_t as) {
        L::integrate(b, B->x.p, B->v.p, B->y.p, B->cpart.p, ls, as);
        if (newton || B->lock) {
            L::begin_eval(b, xk, 1, as);
            L::newton_tail(b, ls, nw, as);
        }
    };
    if (lock_phase == 1) {  // NR_MidStep: the solve at x_k
        solve_start(s);
        return host_cg();
    }
    if (lock_phase == 2) {  // NR_PostStep: the update and the re-evaluation at x_k
        after_solve(s);
        BCK(cudaGetLastError());
        return FEM_OK;
    }
    L::reset_counts(b, ls, if_start, nw, newton ? 1 : 0, s);
    bool any_start = B->mask_host.empty();
    for (uint8_t a : B->mask_host) any_start |= a == 1;
    if (capture && !newton) {
        BCK(capture_conditional(s, if_start, cudaGraphCondTypeIf, [&](cudaStream_t ss, cudaGraph_t) {
            L::begin_eval(b, B->x.p, 0, ss);
            solve_start(ss);
            return cudaGetLastError();
        }));
        BCK(capture_cg(s));
        after_solve(s);
    } else if (capture) {
        BCK(capture_conditional(s, if_start, cudaGraphCondTypeIf, [&](cudaStream_t ss, cudaGraph_t) {
            L::begin_eval(b, B->x.p, 0, ss);
            return cudaGetLastError();
        }));
        BCK(capture_conditional(s, nw, cudaGraphCondTypeWhile, [&](cudaStream_t ns, cudaGraph_t nbody) {
            // the CG loop's condition belongs to the Newton body; the start
            // section's last kernel sets it
            cudaError_t e = cudaGraphConditionalHandleCreate(&ls.cond, nbody, 0, cudaGraphCondAssignDefault);
            if (e != cudaSuccess) return e;
            lb.cond = ls.cond;
            solve_start(ns);
            e = capture_cg(ns);
            if (e != cudaSuccess) return e;
            after_solve(ns);
            return cudaGetLastError();
        }));
    } else {
        if (any_start) {
            L::begin_eval(b, B->x.p, 0, s);
            solve_start(s);
        }
        if (int e = host_cg()) return e;
        after_solve(s);
        // further Newton iterations while some FIE mesh goes on
        while (newton) {
            BCK(cudaMemcpyAsync(B->st_host, B->st.p, sizeof(StepScalars) * B->M, cudaMemcpyDeviceToHost, s));
            BCK(cudaStreamSynchronize(s));
            bool go = false;
            for (uint32_t m = 0; m < B->M; m++) go |= B->st_host[m].nr_go != 0;
            if (!go) break;
            solve_start(s);
            if (int e = host_cg()) return e;
            after_solve(s);
        }
    }
    bool energy = false;
    for (auto& m : B->meshes) energy |= m.p.compute_energy != 0;
    if (energy) {
        L::tile_force(b, B->x.p, nullptr, B->tpart.p, s);
        L::fin_energy(b, FIN_ENERGY_E, B->tpart.p, s);
        L::tile_potential(b, B->x.p, B->tpart.p, s);
        L::fin_energy(b, FIN_ENERGY_P, B->tpart.p, s);
    }
    BCK(cudaGetLastError());
    return FEM_OK;
}

int build_graph(fem_batch B)
{
    if (B->exec) return FEM_OK;
    cudaStream_t s = B->stream;
    BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    int rc = B->opt.precision == FEM_PRECISION_FP64 ? enqueue_step<double>(B, s, true) : enqueue_step<float>(B, s, true);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc != FEM_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    BCK(e);
    B->graph = g;
    BCK(cudaGraphInstantiate(&B->exec, g, 0));
    return FEM_OK;
}

}  // namespace

extern "C" {

int fem_batch_options_default(fem_batch_options* o)
{
    if (!o) return batch_fail(FEM_E_ARG, "null options");
    std::memset(o, 0, sizeof(*o));
    o->precision = FEM_PRECISION_MIXED;
    o->tile_elems = kTileElems;
    o->reorder = 1;
    o->use_graph = 1;
    o->chunk_nodes = kChunkNodes;
    return FEM_OK;
}

int fem_batch_create(const fem_batch_options* opt, fem_batch* out)
{
    if (!out) return batch_fail(FEM_E_ARG, "null output handle");
    *out = nullptr;
    fem_batch_options o;
    fem_batch_options_default(&o);
    if (opt) o = *opt;
    if (o.precision != FEM_PRECISION_FP64 && o.precision != FEM_PRECISION_MIXED)
        return batch_fail(FEM_E_ARG, "unknown precision %u", o.precision);
    if (o.tile_elems == 0 || o.tile_elems > (uint32_t)kTileElems)
        return batch_fail(FEM_E_ARG, "tile_elems must be in [1, %d]", kTileElems);
    if (o.chunk_nodes == 0) o.chunk_nodes = kChunkNodes;
    if (o.chunk_nodes < 32 || o.chunk_nodes > 8192)
        return batch_fail(FEM_E_ARG, "chunk_nodes must be in [32, 8192]");
    if (o.persistent_loop && (o.precision != FEM_PRECISION_MIXED || o.tile_elems <= (uint32_t)kPipeSmallTile))
        return batch_fail(FEM_E_ARG, "persistent_loop needs the mixed precision and tile_elems > %d", kPipeSmallTile);
    fem_batch b = new (std::nothrow) fem_batch_s;
    if (!b) return batch_fail(FEM_E_OOM, "host allocation failed");
    b->opt = o;
    *out = b;
    return FEM_OK;
}

// The parameters a batch takes for a mesh (either precision unless said).
static int check_mesh_params(fem_batch b, const fem_params* p)
{
    if (!(p->fixed_dt > 0)) return batch_fail(FEM_E_ARG, "fixed_dt must be > 0");
    if (p->integrator != FEM_INTEGRATOR_QIE_V && p->integrator != FEM_INTEGRATOR_FIE_DX &&
        p->integrator != FEM_INTEGRATOR_FIE_DX_QUASISTATIC)
        return batch_fail(FEM_E_ARG, "unknown integrator %u", p->integrator);
    if (p->integrator != FEM_INTEGRATOR_QIE_V && b->opt.persistent_loop)
        return batch_fail(FEM_E_ARG, "the persistent loop takes QIE_V meshes only");
    if (p->integrator != FEM_INTEGRATOR_QIE_V && !(p->nr_abs_epsilon >= 0))
        return batch_fail(FEM_E_ARG, "nr_abs_epsilon must be >= 0");
    if (p->rotation != FEM_ROTATION_MSVD && p->rotation != FEM_ROTATION_DAPD)
        return batch_fail(FEM_E_ARG, "unknown rotation %u", p->rotation);
    if (p->rotation == FEM_ROTATION_DAPD &&
        !(std::isfinite(p->dapd_threshold_det_F) && std::isfinite(p->dapd_l_factor) &&
          std::isfinite(p->dapd_nl_factor) && std::isfinite(p->dapd_nl_exponent)))
        return batch_fail(FEM_E_ARG, "non-finite DAPD parameters");
    if (p->ls_solver != FEM_LS_CG && p->ls_solver != FEM_LS_MINRES)
        return batch_fail(FEM_E_ARG, "unknown ls_solver %u", p->ls_solver);
    if (p->ls_solver == FEM_LS_MINRES && b->opt.persistent_loop)
        return batch_fail(FEM_E_ARG, "the persistent loop takes CG meshes only");
    if (p->material > FEM_MATERIAL_C_CCM) return batch_fail(FEM_E_ARG, "unknown material %u", p->material);
    if (p->material == FEM_MATERIAL_C_CCM && b->opt.precision == FEM_PRECISION_MIXED)
        return batch_fail(FEM_E_ARG, "C_CCM runs in FP64 batches (its differential is not symmetric: CG diverges "
                                     "on it, in the reference too)");
    if (p->material == FEM_MATERIAL_C_LCMH && !std::isfinite(p->ecie_k_factor))
        return batch_fail(FEM_E_ARG, "ecie_k_factor must be finite");
    if (p->material != FEM_MATERIAL_C_WRP && b->opt.persistent_loop)
        return batch_fail(FEM_E_ARG, "the persistent loop takes C_WRP meshes only");
    return FEM_OK;
}

int fem_batch_add_mesh(fem_batch b, const double* rest, uint32_t N, const uint32_t* tets, uint32_t T,
                       const fem_params* p, const double* young_per_elem, const double* poisson_per_elem,
                       uint32_t* mesh_index)
{
    if (!b) return batch_fail(FEM_E_ARG, "null batch");
    if (b->finalized) return batch_fail(FEM_E_ARG, "batch already finalized");
    if (!rest || !tets || !p) return batch_fail(FEM_E_ARG, "null rest/tets/params");
    if (N == 0 || T == 0) return batch_fail(FEM_E_ARG, "empty mesh (N=%u, T=%u)", N, T);
    if (int e = check_mesh_params(b, p)) return e;
    for (size_t i = 0; i < 4 * (size_t)T; i++)
        if (tets[i] >= N) return batch_fail(FEM_E_INDEX, "tet %zu names node %u >= N=%u", i / 4, tets[i], N);
    HostMesh m;
    m.rest.assign(rest, rest + 3 * (size_t)N);
    m.tets.assign(tets, tets + 4 * (size_t)T);
    m.p = *p;
    if (young_per_elem) m.E.assign(young_per_elem, young_per_elem + T);
    if (poisson_per_elem) m.nu.assign(poisson_per_elem, poisson_per_elem + T);
    b->meshes.push_back(std::move(m));
    if (mesh_index) *mesh_index = (uint32_t)(b->meshes.size() - 1);
    return FEM_OK;
}

int fem_batch_set_knc(fem_batch b, uint32_t mesh, const uint32_t* nodes, const double* targets, uint32_t count)
{
    if (!b) return batch_fail(FEM_E_ARG, "null batch");
    if (b->finalized) return batch_fail(FEM_E_ARG, "constraint sets are fixed at finalize; use set_knc_targets");
    if (mesh >= b->meshes.size()) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    if (count && (!nodes || !targets)) return batch_fail(FEM_E_ARG, "null constraint arrays");
    HostMesh& m = b->meshes[mesh];
    const uint32_t N = (uint32_t)(m.rest.size() / 3);
    for (uint32_t k = 0; k < count; k++)
        if (nodes[k] >= N) return batch_fail(FEM_E_INDEX, "constraint %u names node %u >= N=%u", k, nodes[k], N);
    m.knc_nodes.assign(nodes, nodes + count);
    m.knc_targets.assign(targets, targets + 3 * (size_t)count);
    return FEM_OK;
}

int fem_batch_finalize(fem_batch b)
{
    if (!b) return batch_fail(FEM_E_ARG, "null batch");
    if (b->finalized) return FEM_OK;
    if (b->meshes.empty()) return batch_fail(FEM_E_ARG, "empty batch");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return batch_fail(FEM_E_NODEVICE, "no CUDA device");
    const bool fp64 = b->opt.precision == FEM_PRECISION_FP64;
    const uint32_t tile_cap = b->opt.tile_elems;
    b->eperm_h.clear();
    // local nodes per tile: the mixed path's small tiles hold fewer
    const size_t node_cap = (!fp64 && tile_cap <= (uint32_t)kPipeSmallTile) ? kPipeSmallNodes : kTileNodes;
    b->M = (uint32_t)b->meshes.size();

    std::vector<TileMeta> tiles;
    std::vector<ChunkMeta> chunks;
    std::vector<MeshConsts> mcs(b->M);
    b->ray0.clear();
    b->ray1.clear();
    b->vol_total.clear();
    b->elem_mat.clear();
    b->mat_scalar.clear();
    std::vector<int4> gtets;
    std::vector<double> vol, rest_all;
    std::vector<uchar4> lconn;
    std::vector<uint32_t> tile_nodes, lptr0;
    std::vector<uint16_t> lptr, lidx;
    std::vector<uint8_t> fixed;
    std::vector<uint32_t> knc_node, knc_mesh;
    std::vector<double> knc_target;
    std::vector<uint32_t> ov_node;   // node of each overflow partial slot, tile order
    std::vector<uint32_t> perm_h;    // batch node id -> caller's node id (both global)
    // element data collected AoS then transposed
    std::vector<double> Dinv_aos, mat_aos;

    uint64_t node0 = 0, elem0 = 0;
    for (uint32_t mi = 0; mi < b->M; mi++) {
        HostMesh& hm = b->meshes[mi];
        const uint32_t N = (uint32_t)(hm.rest.size() / 3), T = (uint32_t)(hm.tets.size() / 4);
        const fem_params& p = hm.p;
        // element order
        std::vector<uint32_t> order(T);
        for (uint32_t e = 0; e < T; e++) order[e] = e;
        if (b->opt.reorder) {
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (uint32_t n = 0; n < N; n++)
                for (int a = 0; a < 3; a++) {
                    lo[a] = std::min(lo[a], hm.rest[3 * (size_t)n + a]);
                    hi[a] = std::max(hi[a], hm.rest[3 * (size_t)n + a]);
                }
            double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
            if (!(ext > 0)) ext = 1.0;
            std::vector<uint64_t> key(T);
            for (uint32_t e = 0; e < T; e++) {
                double c[3] = {0, 0, 0};
                for (int i = 0; i < 4; i++)
                    for (int a = 0; a < 3; a++) c[a] += 0.25 * hm.rest[3 * (size_t)hm.tets[4 * (size_t)e + i] + a];
                uint32_t qv[3];
                for (int a = 0; a < 3; a++) {
                    double f = (c[a] - lo[a]) / ext * 1023.0;
                    qv[a] = (uint32_t)std::max(0.0, std::min(1023.0, f));
                }
                const uint32_t code = spread10(qv[0]) | (spread10(qv[1]) << 1) | (spread10(qv[2]) << 2);
                key[e] = ((uint64_t)code << 32) | e;
            }
            std::sort(key.begin(), key.end());
            for (uint32_t e = 0; e < T; e++) order[e] = (uint32_t)(key[e] & 0xffffffffu);
        }
        // per-element data in the new order
        double acc_total_volume = 0.0;
        std::vector<double> vol_orig(T);
        for (uint32_t e = 0; e < T; e++) {
            const uint32_t* t = &hm.tets[4 * (size_t)e];
            double D[9];
            for (int i = 0; i < 3; i++) {
                D[3 * i] = hm.rest[3 * (size_t)t[1] + i] - hm.rest[3 * (size_t)t[0] + i];
                D[3 * i + 1] = hm.rest[3 * (size_t)t[2] + i] - hm.rest[3 * (size_t)t[0] + i];
                D[3 * i + 2] = hm.rest[3 * (size_t)t[3] + i] - hm.rest[3 * (size_t)t[0] + i];
            }
            const double V = det3(D) / 6.0;
            if (!(V > 0.0)) return batch_fail(FEM_E_DEGENERATE, "mesh %u tet %u has rest volume %g <= 0", mi, e, V);
            vol_orig[e] = V;
            acc_total_volume += V;  // the reference's element order (EndEdition)
        }
        for (uint32_t k = 0; k < T; k++) {
            const uint32_t e = order[k];
            b->eperm_h.push_back(e);
            const uint32_t* t = &hm.tets[4 * (size_t)e];
            double D[9];
            for (int i = 0; i < 3; i++) {
                D[3 * i] = hm.rest[3 * (size_t)t[1] + i] - hm.rest[3 * (size_t)t[0] + i];
                D[3 * i + 1] = hm.rest[3 * (size_t)t[2] + i] - hm.rest[3 * (size_t)t[0] + i];
                D[3 * i + 2] = hm.rest[3 * (size_t)t[3] + i] - hm.rest[3 * (size_t)t[0] + i];
            }
            double Di[9];
            inverse3(D, Di);
            const double V = vol_orig[e];
            // the mixed path's P-K products take V lambda and V mu from the
            // element data: from the set's scalar E and nu (per-element
            // values would only re-bake K0, which they do not use; the FP64
            // products take V, mu and lambda directly)
            const bool scalar_mat = !fp64 && p.material != FEM_MATERIAL_C_WRP;
            const double E = (hm.E.empty() || scalar_mat) ? p.young_modulus : hm.E[e];
            const double nu = (hm.nu.empty() || scalar_mat) ? p.poisson_ratio : hm.nu[e];
            const double a = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
            for (int c = 0; c < 9; c++) Dinv_aos.push_back(Di[c]);
            mat_aos.push_back(V * (a * (1.0 - nu)));
            mat_aos.push_back(V * (a * nu));
            mat_aos.push_back(V * (a * (0.5 - nu)));
            vol.push_back(V);
            gtets.push_back(make_int4((int)(node0 + t[0]), (int)(node0 + t[1]), (int)(node0 + t[2]),
                                      (int)(node0 + t[3])));
        }
        // tiles
        MeshConsts& c = mcs[mi];
        c.tile0 = (uint32_t)tiles.size();
        std::vector<int32_t> stamp(N, -1), local(N, 0);
        std::vector<int32_t> intern(N, -1);  // caller's node -> batch node (tile order; by degree within a tile)
        uint32_t next_id = 0;
        uint32_t k = 0;
        while (k < T) {
            TileMeta tm;
            tm.mesh = mi;
            tm.e0 = (uint32_t)(elem0 + k);
            tm.n0 = (uint32_t)tile_nodes.size();
            tm.c0 = (uint32_t)lidx.size();
            const int32_t tid = (int32_t)tiles.size();
            std::vector<uint32_t> lnodes;
            uint32_t ne = 0;
            while (k < T && ne < tile_cap) {
                const uint32_t* t = &hm.tets[4 * (size_t)order[k]];
                uint32_t fresh = 0;
                for (int i = 0; i < 4; i++) {
                    bool seen = stamp[t[i]] == tid;
                    for (int j = 0; j < i; j++) seen |= (t[j] == t[i]);
                    fresh += seen ? 0 : 1;
                }
                if (lnodes.size() + fresh > node_cap) break;
                uchar4 lc;
                unsigned char li4[4];
                for (int i = 0; i < 4; i++) {
                    if (stamp[t[i]] != tid) {
                        stamp[t[i]] = tid;
                        local[t[i]] = (int32_t)lnodes.size();
                        lnodes.push_back(t[i]);
                    }
                    li4[i] = (unsigned char)local[t[i]];
                }
                lc.x = li4[0]; lc.y = li4[1]; lc.z = li4[2]; lc.w = li4[3];
                lconn.push_back(lc);
                ne++;
                k++;
            }
            tm.ne = (uint16_t)ne;
            tm.nn = (uint16_t)lnodes.size();
            // nodes first seen in this tile get the next batch ids and lead
            // the tile's local list; the others follow. Within each group
            // the nodes are ordered by their number of entries in the tile
            // (most first, ties in local order): one thread sums one node's
            // entries, and a warp then runs loops of similar length.
            {
                std::vector<uint32_t> owned, shared;
                std::vector<uint16_t> deg(lnodes.size(), 0);
                for (size_t el = lconn.size() - ne; el < lconn.size(); el++) {
                    const uchar4 lc = lconn[el];
                    deg[lc.x]++; deg[lc.y]++; deg[lc.z]++; deg[lc.w]++;
                }
                for (uint32_t u : lnodes) (intern[u] < 0 ? owned : shared).push_back(u);
                auto by_degree = [&](uint32_t a, uint32_t b2) { return deg[local[a]] > deg[local[b2]]; };
                std::stable_sort(owned.begin(), owned.end(), by_degree);
                std::stable_sort(shared.begin(), shared.end(), by_degree);
                for (uint32_t u : owned) intern[u] = (int32_t)next_id++;
                std::vector<unsigned char> remap(lnodes.size());
                for (size_t i = 0; i < owned.size(); i++) remap[local[owned[i]]] = (unsigned char)i;
                for (size_t i = 0; i < shared.size(); i++)
                    remap[local[shared[i]]] = (unsigned char)(owned.size() + i);
                for (size_t el = lconn.size() - ne; el < lconn.size(); el++) {
                    uchar4& lc = lconn[el];
                    lc.x = remap[lc.x];
                    lc.y = remap[lc.y];
                    lc.z = remap[lc.z];
                    lc.w = remap[lc.w];
                }
                tm.nown = (uint16_t)owned.size();
                tm.material = (uint16_t)hm.p.material;
                tm.own0 = owned.empty() ? 0u : (uint32_t)(node0 + intern[owned[0]]);
                tm.ov0 = (uint32_t)ov_node.size();
                for (uint32_t u : shared) ov_node.push_back((uint32_t)(node0 + intern[u]));
                lnodes = owned;
                lnodes.insert(lnodes.end(), shared.begin(), shared.end());
            }
            // tile-local CSR: local node -> (element << 2 | slot), element order
            std::vector<uint16_t> cnt(lnodes.size() + 1, 0);
            const size_t lc0 = lconn.size() - ne;
            for (uint32_t el = 0; el < ne; el++) {
                const uchar4 lc = lconn[lc0 + el];
                cnt[lc.x + 1]++; cnt[lc.y + 1]++; cnt[lc.z + 1]++; cnt[lc.w + 1]++;
            }
            for (size_t i = 0; i < lnodes.size(); i++) cnt[i + 1] += cnt[i];
            lptr0.push_back((uint32_t)lptr.size());
            for (size_t i = 0; i <= lnodes.size(); i++) lptr.push_back(cnt[i]);
            std::vector<uint16_t> fill(cnt.begin(), cnt.end() - 1), ent(4 * ne);
            for (uint32_t el = 0; el < ne; el++) {
                const uchar4 lc = lconn[lc0 + el];
                const unsigned char ids[4] = {lc.x, lc.y, lc.z, lc.w};
                for (int sl = 0; sl < 4; sl++) ent[fill[ids[sl]]++] = (uint16_t)((el << 2) | sl);
            }
            lidx.insert(lidx.end(), ent.begin(), ent.end());
            for (uint32_t n : lnodes) tile_nodes.push_back((uint32_t)(node0 + intern[n]));
            tiles.push_back(tm);
        }
        // nodes no tet names get the remaining ids (no tile writes their
        // partial: it stays zero)
        for (uint32_t u = 0; u < N; u++)
            if (intern[u] < 0) intern[u] = (int32_t)next_id++;
        for (uint32_t kk = 0; kk < T; kk++) {
            int4& g = gtets[elem0 + kk];
            g.x = (int)(node0 + intern[g.x - node0]);
            g.y = (int)(node0 + intern[g.y - node0]);
            g.z = (int)(node0 + intern[g.z - node0]);
            g.w = (int)(node0 + intern[g.w - node0]);
        }
        perm_h.resize(node0 + N);
        for (uint32_t u = 0; u < N; u++) perm_h[node0 + intern[u]] = (uint32_t)(node0 + u);
        c.ntiles = (uint32_t)tiles.size() - c.tile0;
        // node chunks
        c.chunk0 = (uint32_t)chunks.size();
        const uint32_t chunk = b->opt.chunk_nodes ? b->opt.chunk_nodes : (uint32_t)kChunkNodes;
        for (uint32_t n = 0; n < N; n += chunk) {
            ChunkMeta ch;
            ch.mesh = mi;
            ch.n0 = (uint32_t)(node0 + n);
            ch.n1 = (uint32_t)(node0 + std::min<uint32_t>(N, n + chunk));
            chunks.push_back(ch);
        }
        c.nchunks = (uint32_t)chunks.size() - c.chunk0;
        double ray[2];
        param_consts(c, p, acc_total_volume, N, fp64, ray);
        b->ray0.push_back(ray[0]);
        b->ray1.push_back(ray[1]);
        b->vol_total.push_back(acc_total_volume);
        const bool given = !hm.E.empty() || !hm.nu.empty();
        b->elem_mat.push_back(given ? 1u : 0u);
        b->mat_scalar.push_back(!given || (!fp64 && p.material != FEM_MATERIAL_C_WRP) ? 1u : 0u);
        if (p.integrator != FEM_INTEGRATOR_QIE_V) b->any_fie = true;
        if (c.material != kTileMaterialWrp) b->any_lcm = true;
        if (c.material == kTileMaterialLcmh) b->any_lcmh = true;
        if (p.rotation == FEM_ROTATION_DAPD) b->any_dapd = true;
        if (p.ls_solver == FEM_LS_MINRES) b->any_minres = true;
        c.node0 = (uint32_t)node0;
        c.N = N;
        c.elem0 = (uint32_t)elem0;
        c.T = T;
        c.knc0 = (uint32_t)knc_node.size();
        c.nknc = (uint32_t)hm.knc_nodes.size();
        // nodes, in batch order
        const size_t r0 = rest_all.size();
        rest_all.resize(r0 + 3 * (size_t)N);
        for (uint32_t u = 0; u < N; u++)
            for (int a = 0; a < 3; a++) rest_all[r0 + 3 * (size_t)intern[u] + a] = hm.rest[3 * (size_t)u + a];
        const size_t f0 = fixed.size();
        fixed.resize(f0 + N, 0);
        for (size_t kk = 0; kk < hm.knc_nodes.size(); kk++) {
            knc_node.push_back((uint32_t)(node0 + intern[hm.knc_nodes[kk]]));
            knc_mesh.push_back(mi);
            for (int a = 0; a < 3; a++) knc_target.push_back(hm.knc_targets[3 * kk + a]);
            fixed[f0 + intern[hm.knc_nodes[kk]]] = 1;
        }
        node0 += N;
        elem0 += T;
    }
    if (node0 >= (1ull << 31) || elem0 >= (1ull << 31)) return batch_fail(FEM_E_ARG, "batch too large");
    b->Ntot = node0;
    b->Ttot = elem0;
    b->ntiles = (uint32_t)tiles.size();
    b->nchunks = (uint32_t)chunks.size();
    b->K = (uint32_t)knc_node.size();
    b->nslots = b->Ntot + ov_node.size();  // owner slots (node order) + overflow slots
    b->mc_host = mcs;
    b->perm_h = perm_h;
    b->inv_h.assign(b->Ntot, 0);
    for (uint64_t i = 0; i < b->Ntot; i++) b->inv_h[perm_h[i]] = (uint32_t)i;
    // node -> overflow slots, tile order
    // a node's overflow entries get consecutive slots Ntot + [ov_ptr[n],
    // ov_ptr[n+1]), in tile order
    if (b->nslots >= (1ull << 32)) return batch_fail(FEM_E_ARG, "batch too large for partial slots");
    std::vector<uint32_t> ov_ptr(b->Ntot + 1, 0), ov_map(ov_node.size());
    for (uint32_t g : ov_node) ov_ptr[g + 1]++;
    for (uint64_t n = 0; n < b->Ntot; n++) ov_ptr[n + 1] += ov_ptr[n];
    {
        std::vector<uint32_t> fill(ov_ptr.begin(), ov_ptr.end() - 1);
        for (size_t kk = 0; kk < ov_node.size(); kk++) ov_map[kk] = (uint32_t)(b->Ntot + fill[ov_node[kk]]++);
    }
    // SoA transposes
    const size_t T = b->Ttot;
    std::vector<double> Dinv_soa(9 * T), mat_soa(3 * T);
    for (size_t e = 0; e < T; e++) {
        for (int c = 0; c < 9; c++) Dinv_soa[c * T + e] = Dinv_aos[9 * e + c];
        for (int c = 0; c < 3; c++) mat_soa[c * T + e] = mat_aos[3 * e + c];
    }
    // per-tile blobs for the pipelined mixed product (element data in FP32)
    std::vector<uint32_t> blob_off16_h;
    std::vector<unsigned char> blob_h;
    if (!fp64) {
        uint64_t total = 0;
        blob_off16_h.resize(b->ntiles);
        for (uint32_t t = 0; t < b->ntiles; t++) {
            blob_off16_h[t] = (uint32_t)(total / 16);
            total += blob_bytes(tiles[t].ne, tiles[t].nn, tiles[t].nown);
        }
        if (total / 16 >= (1ull << 32)) return batch_fail(FEM_E_ARG, "batch too large for tile blobs");
        blob_h.assign(total, 0);
        for (uint32_t t = 0; t < b->ntiles; t++) {
            const TileMeta& tm = tiles[t];
            unsigned char* base = blob_h.data() + 16ull * blob_off16_h[t];
            const uint32_t ne4 = blob_ne4(tm.ne);
            auto put = [&](uint32_t c, uint32_t i, float v) { std::memcpy(base + blob_comp_off(c, i, ne4), &v, 4); };
            for (uint32_t i = 0; i < tm.ne; i++) {
                const size_t e = tm.e0 + i;
                put(0, i, 1.f); put(4, i, 1.f); put(8, i, 1.f);  // R = I
                for (uint32_t c = 0; c < 9; c++) put(9 + c, i, (float)Dinv_soa[c * T + e]);
                put(18, i, (float)mat_soa[T + e]);      // V lambda
                put(19, i, (float)mat_soa[2 * T + e]);  // V mu
                const uchar4 lc = lconn[e];
                const uint32_t w = (uint32_t)lc.x | ((uint32_t)lc.y << 8) | ((uint32_t)lc.z << 16) | ((uint32_t)lc.w << 24);
                std::memcpy(base + blob_comp_off(20, i, ne4), &w, 4);
            }
            uint16_t* lp = reinterpret_cast<uint16_t*>(base + blob_lptr_off(tm.ne));
            const uint16_t* src_lp = lptr.data() + lptr0[t];
            for (uint32_t i = 0; i <= tm.nn; i++) lp[i] = src_lp[i];
            uint16_t* li = lp + (tm.nn + 1);
            for (uint32_t j = 0; j < 4u * tm.ne; j++) {
                const uint16_t v = lidx[tm.c0 + j];  // (element << 2 | slot) -> slot * ne4 + element
                li[j] = (uint16_t)((v & 3u) * ne4 + (v >> 2));
            }
            uint32_t* hdr = reinterpret_cast<uint32_t*>(base + blob_hdr_off(tm.ne, tm.nn));
            hdr[0] = tm.own0;
            std::memcpy(&hdr[1], &mcs[tm.mesh].fK_f, 4);
            std::memcpy(&hdr[2], &mcs[tm.mesh].mfm_f, 4);
            for (uint32_t i = tm.nown; i < tm.nn; i++) hdr[3 + i - tm.nown] = ov_map[tm.ov0 + i - tm.nown];
        }
    }
    std::vector<double> Rinit(9 * T, 0.0);
    for (size_t e = 0; e < T; e++) Rinit[e] = Rinit[4 * T + e] = Rinit[8 * T + e] = 1.0;

    // ---- device ----
    auto cleanup = [&](int code) {
        b->release();
        return code;
    };
#define BCKC(call)                                                                                        \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return cleanup(batch_fail(e_ == cudaErrorMemoryAllocation ? FEM_E_OOM : FEM_E_CUDA, "%s: %s", #call, \
                                      cudaGetErrorString(e_)));                                           \
    } while (0)
    BCKC(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    cudaStream_t s = b->stream;
    const size_t SB = b->S_size();
    const size_t N3 = 3 * b->Ntot;
    BCKC(b->tiles.alloc(b->ntiles));
    BCKC(b->chunks.alloc(b->nchunks));
    BCKC(b->mc.alloc(b->M));
    BCKC(b->st.alloc(b->M));
    BCKC(b->active.alloc(b->M));
    BCKC(b->gtets.alloc(T));
    BCKC(b->Dinv_s.alloc(9 * T * SB));
    BCKC(b->mat_s.alloc(3 * T * SB));
    BCKC(b->R_s.alloc(9 * T * SB));
    BCKC(b->Dinv64.alloc(9 * T));
    BCKC(b->vol.alloc(T));
    BCKC(b->detF.alloc(T));
    BCKC(b->tile_nodes.alloc(tile_nodes.size()));
    BCKC(b->lptr0.alloc(b->ntiles));
    BCKC(b->ov_ptr.alloc(b->Ntot + 1));
    BCKC(b->ov_map.alloc(ov_map.size()));
    BCKC(b->perm.alloc(b->Ntot));
    BCKC(b->knc_node.alloc(b->K));
    BCKC(b->knc_mesh.alloc(b->K));
    BCKC(b->knc_target.alloc(3 * (size_t)b->K));
    BCKC(b->lconn.alloc(T));
    BCKC(b->lptr.alloc(lptr.size()));
    BCKC(b->lidx.alloc(lidx.size()));
    BCKC(b->fixed.alloc(b->Ntot));
    BCKC(b->rest.alloc(N3));
    BCKC(b->x.alloc(N3));
    BCKC(b->v.alloc(N3));
    BCKC(b->bvec.alloc(N3));
    BCKC(b->y.alloc(N3));
    BCKC(b->r_s.alloc(N3 * SB));
    BCKC(b->d_s.alloc(N3 * SB));
    BCKC(b->q_s.alloc(N3 * SB));
    BCKC(b->part_s.alloc(3 * b->nslots * SB));
    BCKC(cudaMemsetAsync(b->part_s.p, 0, 3 * b->nslots * SB, s));  // slots of nodes no tet names stay zero
    BCKC(b->ydelta_s.alloc(N3 * SB));
    BCKC(cudaMemsetAsync(b->ydelta_s.p, 0, N3 * SB, s));
    BCKC(b->part64.alloc(3 * b->nslots));
    BCKC(cudaMemsetAsync(b->part64.p, 0, 3 * b->nslots * sizeof(double), s));
    BCKC(b->cpart.alloc(b->nchunks));
    BCKC(b->tpart.alloc(b->ntiles));
    BCKC(b->counter.alloc(1));
    BCKC(b->any_flag.alloc(1));
    BCKC(b->refresh_flag.alloc(1));
    BCKC(b->mcount.alloc(b->M));
    BCKC(b->err.alloc(2));  // [0] error word, [1] poll limit of the tile-copy waits
    BCKC(b->gbar.alloc(3));
    {
        const unsigned e0[2] = {0u, kDefaultWaitPolls};
        BCKC(cudaMemcpyAsync(b->err.p, e0, sizeof(e0), cudaMemcpyHostToDevice, s));
        BCKC(cudaStreamSynchronize(s));
    }
    BCKC(b->blob.alloc(blob_h.size()));
    BCKC(b->blob.upload(blob_h, s));
    BCKC(b->blob_off16.alloc(blob_off16_h.size()));
    BCKC(b->blob_off16.upload(blob_off16_h, s));
    BCKC(b->slice.alloc(2));
    BCKC(cudaMemsetAsync(b->slice.p, 0, 2 * sizeof(unsigned), s));
    BCKC(b->start_tiles.alloc(b->ntiles));
    BCKC(b->start_chunks.alloc(b->nchunks));
    BCKC(b->launch_tiles.alloc(b->ntiles));
    BCKC(b->launch_chunks.alloc(b->nchunks));
    if (!fp64) {
        BCKC(b->refresh_tiles.alloc(b->ntiles));
        BCKC(b->refresh_chunks.alloc(b->nchunks));
    }
    BCKC(b->list_count.alloc(6));
    BCKC(cudaMemsetAsync(b->list_count.p, 0, 6 * sizeof(uint32_t), s));
    if (!fp64) {
        BCKC(b->act_tiles.alloc(b->ntiles));
        BCKC(b->act_chunks.alloc(b->nchunks));
        BCKC(b->act_count.alloc(2));
        BCKC(b->list_dirty.alloc(1));
        BCKC(cudaMemsetAsync(b->act_count.p, 0, 2 * sizeof(uint32_t), s));
        BCKC(cudaMemsetAsync(b->list_dirty.p, 0, sizeof(unsigned), s));
    }
    if (!fp64) prepare_tile_pipe();
    BCKC(cudaMallocHost(&b->st_host, sizeof(StepScalars) * b->M));
    BCKC(cudaMallocHost(&b->err_host, sizeof(unsigned)));
    *b->err_host = 0;
    BCKC(b->tiles.upload(tiles, s));
    BCKC(b->chunks.upload(chunks, s));
    BCKC(b->mc.upload(mcs, s));
    BCKC(cudaMemsetAsync(b->st.p, 0, sizeof(StepScalars) * b->M, s));
    BCKC(cudaMemsetAsync(b->active.p, 1, b->M, s));
    BCKC(b->gtets.upload(gtets, s));
    {
        std::vector<unsigned char> tmp = fp64 ? as_bytes<double>(Dinv_soa) : as_bytes<float>(Dinv_soa);
        BCKC(b->Dinv_s.upload(tmp, s));
        BCKC(cudaStreamSynchronize(s));
        tmp = fp64 ? as_bytes<double>(mat_soa) : as_bytes<float>(mat_soa);
        BCKC(b->mat_s.upload(tmp, s));
        BCKC(cudaStreamSynchronize(s));
        tmp = fp64 ? as_bytes<double>(Rinit) : as_bytes<float>(Rinit);
        BCKC(b->R_s.upload(tmp, s));
        BCKC(cudaStreamSynchronize(s));
    }
    BCKC(b->Dinv64.upload(Dinv_soa, s));
    BCKC(b->vol.upload(vol, s));
    BCKC(b->tile_nodes.upload(tile_nodes, s));
    BCKC(b->lptr0.upload(lptr0, s));
    BCKC(b->ov_ptr.upload(ov_ptr, s));
    BCKC(b->ov_map.upload(ov_map, s));
    BCKC(b->perm.upload(perm_h, s));
    BCKC(b->knc_node.upload(knc_node, s));
    BCKC(b->knc_mesh.upload(knc_mesh, s));
    BCKC(b->knc_target.upload(knc_target, s));
    BCKC(b->lconn.upload(lconn, s));
    BCKC(b->lptr.upload(lptr, s));
    BCKC(b->lidx.upload(lidx, s));
    BCKC(b->fixed.upload(fixed, s));
    BCKC(b->rest.upload(rest_all, s));
    BCKC(b->x.upload(rest_all, s));
    if (b->any_lcm) {
        BCKC(b->Fe.alloc(9 * (size_t)b->Ttot));
        BCKC(cudaMemsetAsync(b->Fe.p, 0, sizeof(double) * 9 * (size_t)b->Ttot, s));
    }
    if (b->any_lcmh && !fp64) {
        BCKC(b->lcmh_w.alloc(b->Ttot));
        BCKC(cudaMemsetAsync(b->lcmh_w.p, 0, sizeof(float) * (size_t)b->Ttot, s));
    }
    if (b->any_minres) {
        BCKC(b->mr_p_s.alloc(N3 * SB));
        BCKC(b->mr_p0_s.alloc(N3 * SB));
        BCKC(cudaMemsetAsync(b->mr_p_s.p, 0, N3 * SB, s));
        BCKC(cudaMemsetAsync(b->mr_p0_s.p, 0, N3 * SB, s));
    }
    if (b->any_minres || b->any_fie) BCKC(b->cpart_b.alloc(b->nchunks));
    if (b->any_fie) {
        BCKC(b->xn.alloc(N3));
        BCKC(b->vn.alloc(N3));
    }
    std::vector<uchar2> doc_none;
    if (b->any_dapd) {
        // DAPD's previous positions start at the rest positions (Create,
        // LeafDSH_Solid3D_FEM.cpp:136-147), no element has a direction of
        // collapse
        BCKC(b->prev_x.alloc(N3));
        BCKC(cudaMemcpyAsync(b->prev_x.p, b->x.p, sizeof(double) * N3, cudaMemcpyDeviceToDevice, s));
        BCKC(b->doc.alloc(b->Ttot));
        doc_none.assign(b->Ttot, make_uchar2(3, 0));
        BCKC(b->doc.upload(doc_none, s));
    }
    BCKC(cudaMemsetAsync(b->v.p, 0, sizeof(double) * N3, s));
    BCKC(cudaMemsetAsync(b->y.p, 0, sizeof(double) * N3, s));
    BCKC(cudaMemsetAsync(b->counter.p, 0, sizeof(unsigned), s));
    BCKC(cudaMemsetAsync(b->any_flag.p, 0, sizeof(unsigned), s));
    BCKC(cudaMemsetAsync(b->refresh_flag.p, 0, sizeof(unsigned), s));
    BCKC(cudaMemsetAsync(b->mcount.p, 0, sizeof(unsigned) * b->M, s));
    BCKC(cudaStreamSynchronize(s));
#undef BCKC
    b->device_bytes = b->tiles.bytes() + b->chunks.bytes() + b->mc.bytes() + b->st.bytes() + b->active.bytes() +
                      b->gtets.bytes() + b->Dinv_s.bytes() + b->mat_s.bytes() + b->R_s.bytes() +
                      b->Dinv64.bytes() + b->vol.bytes() + b->detF.bytes() + b->tile_nodes.bytes() +
                      b->lptr0.bytes() + b->ov_ptr.bytes() + b->ov_map.bytes() + b->knc_node.bytes() +
                      b->perm.bytes() + b->prev_x.bytes() + b->doc.bytes() + b->Fe.bytes() + b->lcmh_w.bytes() + b->mr_p_s.bytes() +
                      b->mr_p0_s.bytes() + b->cpart_b.bytes() + b->xn.bytes() + b->vn.bytes() +
                      b->knc_mesh.bytes() + b->knc_target.bytes() + b->lconn.bytes() + b->lptr.bytes() +
                      b->lidx.bytes() + b->fixed.bytes() + b->rest.bytes() + b->x.bytes() + b->v.bytes() +
                      b->bvec.bytes() + b->y.bytes() + b->r_s.bytes() + b->d_s.bytes() + b->q_s.bytes() +
                      b->part_s.bytes() + b->ydelta_s.bytes() + b->part64.bytes() + b->cpart.bytes() +
                      b->tpart.bytes() + b->counter.bytes() + b->any_flag.bytes() + b->refresh_flag.bytes() +
                      b->mcount.bytes() + b->err.bytes() + b->blob.bytes() + b->blob_off16.bytes() +
                      b->act_tiles.bytes() + b->act_chunks.bytes() + b->act_count.bytes() + b->list_dirty.bytes() +
                      b->slice.bytes() + b->start_tiles.bytes() + b->start_chunks.bytes() +
                      b->launch_tiles.bytes() + b->launch_chunks.bytes() + b->refresh_tiles.bytes() +
                      b->refresh_chunks.bytes() + b->list_count.bytes();
    b->finalized = true;
    // host copies of the meshes are no longer needed beyond sizes
    for (auto& m : b->meshes) {
        std::vector<uint32_t>().swap(m.tets);
        std::vector<double>().swap(m.E);
        std::vector<double>().swap(m.nu);
    }
    if (b->opt.use_graph) {
        int rc = build_graph(b);
        if (rc != FEM_OK) return rc;
    }
    return FEM_OK;
}

int fem_batch_destroy(fem_batch b)
{
    if (!b) return FEM_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->release();
    delete b;
    return FEM_OK;
}

static int check_ready(fem_batch b)
{
    if (!b) return batch_fail(FEM_E_ARG, "null batch");
    if (!b->finalized) return batch_fail(FEM_E_ARG, "batch not finalized");
    return FEM_OK;
}

int fem_batch_info(fem_batch b, uint32_t* meshes, uint64_t* nodes, uint64_t* tets, uint32_t* tiles,
                   uint64_t* device_bytes)
{
    if (!b) return batch_fail(FEM_E_ARG, "null batch");
    if (meshes) *meshes = (uint32_t)b->meshes.size();
    if (nodes) *nodes = b->Ntot;
    if (tets) *tets = b->Ttot;
    if (tiles) *tiles = b->ntiles;
    if (device_bytes) *device_bytes = b->device_bytes;
    return FEM_OK;
}

int fem_batch_set_knc_targets(fem_batch b, uint32_t mesh, const double* targets)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    const MeshConsts& c = b->mc_host[mesh];
    if (c.nknc == 0) return FEM_OK;
    if (!targets) return batch_fail(FEM_E_ARG, "null targets");
    BCK(cudaMemcpyAsync(b->knc_target.p + 3 * (size_t)c.knc0, targets, sizeof(double) * 3 * c.nknc,
                        cudaMemcpyHostToDevice, b->stream));
    return FEM_OK;
}

// Per-mesh state transfers permute on the host between the caller's node
// order and the batch's (tile order).
int fem_batch_set_state(fem_batch b, uint32_t mesh, const double* x, const double* v)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    const MeshConsts& c = b->mc_host[mesh];
    const size_t off = 3 * (size_t)c.node0, bytes = sizeof(double) * 3 * c.N;
    std::vector<double> tmp(3 * (size_t)c.N);
    const double* src[2] = {x, v};
    double* dst[2] = {b->x.p, b->v.p};
    for (int k = 0; k < 2; k++) {
        if (!src[k]) continue;
        for (uint32_t u = 0; u < c.N; u++) {
            const size_t i = b->inv_h[c.node0 + u] - c.node0;
            for (int a = 0; a < 3; a++) tmp[3 * i + a] = src[k][3 * (size_t)u + a];
        }
        BCK(cudaMemcpyAsync(dst[k] + off, tmp.data(), bytes, cudaMemcpyHostToDevice, b->stream));
        // a DAPD mesh's previous positions restart at the new x, as on the
        // solid (fem_solid_set_state); fem_batch_set_dapd_state restores them
        if (k == 0 && c.rotation == FEM_ROTATION_DAPD && b->prev_x.p)
            BCK(cudaMemcpyAsync(b->prev_x.p + off, tmp.data(), bytes, cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    return FEM_OK;
}

int fem_batch_get_dapd_state(fem_batch b, uint32_t mesh, double* prev_x, uint8_t* doc)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    const MeshConsts& c = b->mc_host[mesh];
    if (c.rotation != FEM_ROTATION_DAPD || !b->prev_x.p)
        return batch_fail(FEM_E_ARG, "mesh %u does not use the DAPD rotation", mesh);
    if (prev_x) {
        std::vector<double> tmp(3 * (size_t)c.N);
        BCK(cudaMemcpyAsync(tmp.data(), b->prev_x.p + 3 * (size_t)c.node0, sizeof(double) * tmp.size(),
                            cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        for (uint32_t u = 0; u < c.N; u++) {
            const size_t i = b->inv_h[c.node0 + u] - c.node0;
            for (int a = 0; a < 3; a++) prev_x[3 * (size_t)u + a] = tmp[3 * i + a];
        }
    }
    if (doc) {
        std::vector<uchar2> tmp(c.T);
        BCK(cudaMemcpyAsync(tmp.data(), b->doc.p + c.elem0, sizeof(uchar2) * c.T, cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        const uint32_t* perm = b->eperm_h.data() + c.elem0;
        for (uint32_t i = 0; i < c.T; i++) {
            doc[2 * (size_t)perm[i]] = tmp[i].x;
            doc[2 * (size_t)perm[i] + 1] = tmp[i].y;
        }
    }
    return FEM_OK;
}

int fem_batch_set_dapd_state(fem_batch b, uint32_t mesh, const double* prev_x, const uint8_t* doc)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    const MeshConsts& c = b->mc_host[mesh];
    if (c.rotation != FEM_ROTATION_DAPD || !b->prev_x.p)
        return batch_fail(FEM_E_ARG, "mesh %u does not use the DAPD rotation", mesh);
    if (prev_x) {
        std::vector<double> tmp(3 * (size_t)c.N);
        for (uint32_t u = 0; u < c.N; u++) {
            const size_t i = b->inv_h[c.node0 + u] - c.node0;
            for (int a = 0; a < 3; a++) tmp[3 * i + a] = prev_x[3 * (size_t)u + a];
        }
        BCK(cudaMemcpyAsync(b->prev_x.p + 3 * (size_t)c.node0, tmp.data(), sizeof(double) * tmp.size(),
                            cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    if (doc) {
        std::vector<uchar2> tmp(c.T);
        const uint32_t* perm = b->eperm_h.data() + c.elem0;
        for (uint32_t i = 0; i < c.T; i++) {
            const uint8_t v0 = doc[2 * (size_t)perm[i]], v1 = doc[2 * (size_t)perm[i] + 1];
            // none (3, 0), V-F (v, v) or E-E (v0 < v1), vertex ids 0..3
            if (!((v0 == 3 && v1 == 0) || (v0 <= 3 && v1 <= 3 && v0 <= v1)))
                return batch_fail(FEM_E_ARG, "element %u: (%u, %u) is not a direction of collapse", perm[i], v0, v1);
            tmp[i] = make_uchar2(v0, v1);
        }
        BCK(cudaMemcpyAsync(b->doc.p + c.elem0, tmp.data(), sizeof(uchar2) * c.T, cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
    }
    return FEM_OK;
}

int fem_batch_set_params(fem_batch b, uint32_t mesh, const fem_params* params)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M || !params) return batch_fail(FEM_E_ARG, "bad mesh index or null params");
    if (int e = check_mesh_params(b, params)) return e;
    if (b->lock_open) return batch_fail(FEM_E_ARG, "a lock-step is open: fem_batch_nr_end first");
    if (params->integrator != FEM_INTEGRATOR_QIE_V && b->slice_budget)
        return batch_fail(FEM_E_ARG, "an FIE mesh in a batch with an iteration budget");
    const bool fp64 = b->opt.precision == FEM_PRECISION_FP64;
    const fem_params old = b->meshes[mesh].p;
    const bool pk_new = params->material != FEM_MATERIAL_C_WRP;
    const bool en_changed = params->young_modulus != old.young_modulus || params->poisson_ratio != old.poisson_ratio;
    // the mixed path's P-K products take the element data's V lambda and V
    // mu from the scalar E and nu: a mesh built with per-element values
    // cannot go back to them from a P-K material
    if (!fp64 && !pk_new && !en_changed && b->elem_mat[mesh] && b->mat_scalar[mesh])
        return batch_fail(FEM_E_ARG, "mesh %u: its per-element E, nu were replaced by the scalar ones for a P-K "
                                     "material", mesh);
    cudaStream_t s = b->stream;
    BCK(cudaStreamSynchronize(s));
    const size_t n3 = 3 * (size_t)b->Ntot;
    const size_t SB = b->S_size();
    MeshConsts c = b->mc_host[mesh];
    // buffers the new methods need (kept when a method is switched off)
    if (params->integrator != FEM_INTEGRATOR_QIE_V && !b->xn.p) {
        BCK(b->xn.alloc(n3));
        BCK(b->vn.alloc(n3));
    }
    if ((params->integrator != FEM_INTEGRATOR_QIE_V || params->ls_solver == FEM_LS_MINRES) && !b->cpart_b.p)
        BCK(b->cpart_b.alloc(b->nchunks));
    if (params->ls_solver == FEM_LS_MINRES && !b->mr_p_s.p) {
        BCK(b->mr_p_s.alloc(n3 * SB));
        BCK(b->mr_p0_s.alloc(n3 * SB));
        BCK(cudaMemsetAsync(b->mr_p_s.p, 0, n3 * SB, s));
        BCK(cudaMemsetAsync(b->mr_p0_s.p, 0, n3 * SB, s));
    }
    if (pk_new && !b->Fe.p) {
        BCK(b->Fe.alloc(9 * (size_t)b->Ttot));
        BCK(cudaMemsetAsync(b->Fe.p, 0, sizeof(double) * 9 * (size_t)b->Ttot, s));
    }
    if (params->material == FEM_MATERIAL_C_LCMH && !fp64 && !b->lcmh_w.p) {
        BCK(b->lcmh_w.alloc(b->Ttot));
        BCK(cudaMemsetAsync(b->lcmh_w.p, 0, sizeof(float) * (size_t)b->Ttot, s));
    }
    if (params->rotation == FEM_ROTATION_DAPD && old.rotation != FEM_ROTATION_DAPD) {
        // DAPD from here on: the mesh's previous positions start at its
        // current ones and none of its elements has a direction of collapse
        // (as a solid created with DAPD, TetrahedronElementSet3.cpp:190-209)
        if (!b->prev_x.p) {
            BCK(b->prev_x.alloc(n3));
            BCK(cudaMemcpyAsync(b->prev_x.p, b->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
        } else {
            BCK(cudaMemcpyAsync(b->prev_x.p + 3 * (size_t)c.node0, b->x.p + 3 * (size_t)c.node0,
                                sizeof(double) * 3 * (size_t)c.N, cudaMemcpyDeviceToDevice, s));
        }
        const std::vector<uchar2> none(b->doc.p ? c.T : b->Ttot, make_uchar2(3, 0));
        if (!b->doc.p) {
            BCK(b->doc.alloc(b->Ttot));
            BCK(cudaMemcpyAsync(b->doc.p, none.data(), sizeof(uchar2) * b->Ttot, cudaMemcpyHostToDevice, s));
        } else {
            BCK(cudaMemcpyAsync(b->doc.p + c.elem0, none.data(), sizeof(uchar2) * c.T, cudaMemcpyHostToDevice, s));
        }
        BCK(cudaStreamSynchronize(s));
    }
    if (params->integrator != FEM_INTEGRATOR_QIE_V) b->any_fie = true;
    if (params->ls_solver == FEM_LS_MINRES) b->any_minres = true;
    if (pk_new) b->any_lcm = true;
    if (params->material == FEM_MATERIAL_C_LCMH) b->any_lcmh = true;
    if (params->rotation == FEM_ROTATION_DAPD) b->any_dapd = true;
    // the constants (node mass, Rayleigh coefficients, system factors,
    // tolerances, methods), as a batch built with these parameters has them
    double ray[2];
    param_consts(c, *params, b->vol_total[mesh], c.N, fp64, ray);
    b->ray0[mesh] = ray[0];
    b->ray1[mesh] = ray[1];
    b->mc_host[mesh] = c;
    BCK(b->mc.upload(b->mc_host, s));
    // element data: re-baked from the scalar E and nu when they change (as
    // EditableTetrahedronElementSet3::SetParams does, replacing per-element
    // values), or when the mixed path's P-K products need them; the tiles
    // take the mesh's material
    const bool rebake = en_changed || (!fp64 && pk_new && !b->mat_scalar[mesh]);
    const double E = params->young_modulus, nu = params->poisson_ratio;
    const double a = E / ((1.0 + nu) * (1.0 - 2.0 * nu));  // Compute_E (TetrahedronElement3.h:141-156)
    if (fp64)
        launch_rebake_mesh(b->view<double>(), c.tile0, c.ntiles, a * (1.0 - nu), a * nu, a * (0.5 - nu),
                           rebake ? 1 : 0, (uint16_t)params->material, s);
    else
        launch_rebake_mesh(b->view<float>(), c.tile0, c.ntiles, a * (1.0 - nu), a * nu, a * (0.5 - nu),
                           rebake ? 1 : 0, (uint16_t)params->material, s);
    if (rebake) b->mat_scalar[mesh] = 1;
    if (en_changed) b->elem_mat[mesh] = 0;  // replaced by the scalar values
    if (!fp64) launch_blob_factors(b->view<float>(), s);
    b->meshes[mesh].p = *params;
    b->lock_dt = -1.0;  // the lock-step's constants are rebuilt at its next phase
    BCK(cudaGetLastError());
    BCK(cudaStreamSynchronize(s));
    // the step graph holds the forms the batch's methods need: capture anew
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (b->opt.use_graph) return build_graph(b);
    return FEM_OK;
}

int fem_batch_get_params(fem_batch b, uint32_t mesh, fem_params* params)
{
    if (!b) return batch_fail(FEM_E_ARG, "null batch");
    if (mesh >= b->meshes.size() || !params) return batch_fail(FEM_E_ARG, "bad mesh index or null params");
    *params = b->meshes[mesh].p;
    params->precision = b->opt.precision;
    return FEM_OK;
}

int fem_batch_get_state(fem_batch b, uint32_t mesh, double* x, double* v)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    const MeshConsts& c = b->mc_host[mesh];
    const size_t off = 3 * (size_t)c.node0, bytes = sizeof(double) * 3 * c.N;
    std::vector<double> tmp(3 * (size_t)c.N);
    double* dst[2] = {x, v};
    const double* src[2] = {b->x.p, b->v.p};
    for (int k = 0; k < 2; k++) {
        if (!dst[k]) continue;
        BCK(cudaMemcpyAsync(tmp.data(), src[k] + off, bytes, cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        for (uint32_t u = 0; u < c.N; u++) {
            const size_t i = b->inv_h[c.node0 + u] - c.node0;
            for (int a = 0; a < 3; a++) dst[k][3 * (size_t)u + a] = tmp[3 * i + a];
        }
    }
    return FEM_OK;
}

int fem_batch_get_rotations(fem_batch b, uint32_t mesh, double* R, double* detF)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M) return batch_fail(FEM_E_ARG, "mesh %u out of range", mesh);
    const MeshConsts& c = b->mc_host[mesh];
    const size_t T = b->Ttot, e0 = c.elem0, n = c.T;
    const uint32_t* perm = b->eperm_h.data() + e0;
    if (R) {
        const bool fp64 = b->opt.precision == FEM_PRECISION_FP64;
        const size_t sb = fp64 ? 8 : 4;
        std::vector<unsigned char> tmp(9 * n * sb);
        for (int k = 0; k < 9; k++)
            BCK(cudaMemcpyAsync(tmp.data() + k * n * sb, b->R_s.p + (k * T + e0) * sb, n * sb, cudaMemcpyDeviceToHost,
                                b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < n; i++)
            for (int k = 0; k < 9; k++) {
                double v;
                if (fp64) {
                    std::memcpy(&v, tmp.data() + (k * n + i) * 8, 8);
                } else {
                    float f;
                    std::memcpy(&f, tmp.data() + (k * n + i) * 4, 4);
                    v = f;
                }
                R[9 * (size_t)perm[i] + k] = v;
            }
    }
    if (detF) {
        std::vector<double> tmp(n);
        BCK(cudaMemcpyAsync(tmp.data(), b->detF.p + e0, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < n; i++) detF[perm[i]] = tmp[i];
    }
    return FEM_OK;
}

int fem_batch_use_graph(fem_batch b, int on)
{
    if (int e = check_ready(b)) return e;
    b->opt.use_graph = on ? 1u : 0u;
    if (on) return build_graph(b);
    return FEM_OK;
}

// Whole-batch state transfers go through caller-order staging buffers on
// the device (allocated at first use) and a permute kernel.
static int ensure_staging(fem_batch b)
{
    if (b->stage_x.p) return FEM_OK;
    const size_t n3 = 3 * (size_t)b->Ntot;
    cudaError_t e = b->stage_x.alloc(n3);
    if (e == cudaSuccess) e = b->stage_v.alloc(n3);
    if (e != cudaSuccess) {
        b->stage_x.release();
        b->stage_v.release();
        return batch_fail(e == cudaErrorMemoryAllocation ? FEM_E_OOM : FEM_E_CUDA, "staging buffers: %s",
                          cudaGetErrorString(e));
    }
    b->device_bytes += 2 * n3 * sizeof(double);
    return FEM_OK;
}

int fem_batch_set_state_all(fem_batch b, const double* x, const double* v)
{
    if (int e = check_ready(b)) return e;
    if (int e = ensure_staging(b)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)b->Ntot;
    if (x) {
        BCK(cudaMemcpyAsync(b->stage_x.p, x, bytes, cudaMemcpyHostToDevice, b->stream));
        launch_permute(b->perm.p, b->Ntot, b->stage_x.p, b->x.p, true, b->stream);
        // DAPD meshes' previous positions restart at the new x (the other
        // meshes never read them)
        if (b->prev_x.p) BCK(cudaMemcpyAsync(b->prev_x.p, b->x.p, bytes, cudaMemcpyDeviceToDevice, b->stream));
    }
    if (v) {
        BCK(cudaMemcpyAsync(b->stage_v.p, v, bytes, cudaMemcpyHostToDevice, b->stream));
        launch_permute(b->perm.p, b->Ntot, b->stage_v.p, b->v.p, true, b->stream);
    }
    BCK(cudaGetLastError());
    return FEM_OK;
}

int fem_batch_get_state_all(fem_batch b, double* x, double* v)
{
    if (int e = check_ready(b)) return e;
    if (int e = ensure_staging(b)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)b->Ntot;
    if (x) {
        launch_permute(b->perm.p, b->Ntot, b->x.p, b->stage_x.p, false, b->stream);
        BCK(cudaMemcpyAsync(x, b->stage_x.p, bytes, cudaMemcpyDeviceToHost, b->stream));
    }
    if (v) {
        launch_permute(b->perm.p, b->Ntot, b->v.p, b->stage_v.p, false, b->stream);
        BCK(cudaMemcpyAsync(v, b->stage_v.p, bytes, cudaMemcpyDeviceToHost, b->stream));
    }
    BCK(cudaStreamSynchronize(b->stream));
    return FEM_OK;
}

int fem_batch_step_host(fem_batch b, const double* x_in, const double* v_in, uint32_t nsteps, double* x_out,
                        double* v_out)
{
    if (int e = fem_batch_set_state_all(b, x_in, v_in)) return e;
    if (int e = fem_batch_step_async(b, nsteps)) return e;
    if (int e = fem_batch_get_state_all(b, x_out, v_out)) return e;
    return fem_batch_synchronize(b);
}

int fem_batch_set_active(fem_batch b, const uint8_t* mask)
{
    if (int e = check_ready(b)) return e;
    if (mask) {
        for (uint32_t m = 0; m < b->M; m++)
            if (mask[m] > 2) return batch_fail(FEM_E_ARG, "mask[%u] = %u (0, 1 or 2)", m, (unsigned)mask[m]);
        b->mask_host.assign(mask, mask + b->M);
        BCK(cudaMemcpyAsync(b->active.p, b->mask_host.data(), b->M, cudaMemcpyHostToDevice, b->stream));
    } else {
        b->mask_host.clear();
        BCK(cudaMemsetAsync(b->active.p, 1, b->M, b->stream));
    }
    return FEM_OK;
}

int fem_batch_set_slice(fem_batch b, uint32_t max_iterations)
{
    if (int e = check_ready(b)) return e;
    if (max_iterations && b->any_fie)
        return batch_fail(FEM_E_ARG, "iteration budgets are for QIE_V batches (a Newton step runs whole)");
    b->slice_budget = max_iterations;
    BCK(cudaMemcpyAsync(b->slice.p, &b->slice_budget, sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return FEM_OK;
}

int fem_batch_set_wait_limit(fem_batch b, uint32_t polls)
{
    if (int e = check_ready(b)) return e;
    const unsigned v = polls == FEM_WAIT_LIMIT_DEFAULT ? kDefaultWaitPolls : polls;
    BCK(cudaMemcpyAsync(b->err.p + 1, &v, sizeof(unsigned), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return FEM_OK;
}

int fem_batch_step_async(fem_batch b, uint32_t nsteps)
{
    if (int e = check_ready(b)) return e;
    if (b->lock_open) return batch_fail(FEM_E_ARG, "a lock-step is open: fem_batch_nr_end first");
    b->lock_stats = false;
    for (uint32_t i = 0; i < nsteps; i++) {
        if (b->exec && b->opt.use_graph && !b->opt.persistent_loop) {
            BCK(cudaGraphLaunch(b->exec, b->stream));
            launch_counter() += 0;  // kernels inside the graph are counted at capture
        } else {
            int rc = b->opt.precision == FEM_PRECISION_FP64 ? enqueue_step<double>(b, b->stream, false)
                                                            : enqueue_step<float>(b, b->stream, false);
            if (rc) return rc;
        }
    }
    return FEM_OK;
}

}  // extern "C"

// ---- the multi-solid Newton lock-step over the meshes of a batch ----

namespace {

int lock_check(fem_batch b, double dt, bool opened)
{
    if (int e = check_ready(b)) return e;
    if (!(dt >= 0) || !std::isfinite(dt)) return batch_fail(FEM_E_ARG, "dt must be finite and >= 0");
    if (b->slice_budget) return batch_fail(FEM_E_ARG, "the lock-step's solves run whole: no iteration budget");
    if (b->opt.persistent_loop) return batch_fail(FEM_E_ARG, "the lock-step runs with the kernel-per-phase CG loop");
    if (opened && !b->lock_open) return batch_fail(FEM_E_ARG, "fem_batch_nr_init must come first");
    return FEM_OK;
}

// The meshes' constants with the lock-step's factors for step dt (NR_MidStep,
// LeafDSH_Solid3D_FEM.cpp:2960-2962: the FIE system, 1/h = 0 when dt = 0).
int lock_consts(fem_batch b, double dt)
{
    if (b->lock_dt == dt && b->mc_lock.p) return FEM_OK;
    std::vector<MeshConsts> mcs = b->mc_host;
    for (uint32_t m = 0; m < b->M; m++) {
        MeshConsts& c = mcs[m];
        c.dt = dt;
        c.inv_dt = dt == 0 ? 0.0 : 1.0 / dt;
        c.factor_M = c.inv_dt * c.inv_dt + c.inv_dt * b->ray0[m];
        c.factor_K = 1.0 + c.inv_dt * b->ray1[m];
        c.fK_f = (float)c.factor_K;
        c.mfm_f = (float)(c.mass * c.factor_M);
    }
    if (!b->mc_lock.p) BCK(b->mc_lock.alloc(b->M));
    BCK(b->mc_lock.upload(mcs, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->lock_dt = dt;
    return FEM_OK;
}

// The mixed path's tile blobs carry FP32 copies of the factors: the
// lock-step's while it is open, the step's otherwise.
void blob_factors(fem_batch b, bool lock)
{
    if (b->opt.precision != FEM_PRECISION_MIXED) return;
    b->lock = lock;
    launch_blob_factors(b->view<float>(), b->stream);
    b->lock = false;
}

template <typename S>
int lock_run(fem_batch b, int phase)
{
    b->lock = true;
    const int rc = enqueue_step<S>(b, b->stream, false, phase);
    b->lock = false;
    return rc;
}

int lock_solve_phase(fem_batch b, int phase)
{
    return b->opt.precision == FEM_PRECISION_FP64 ? lock_run<double>(b, phase) : lock_run<float>(b, phase);
}

}  // namespace

extern "C" {

int fem_batch_nr_init(fem_batch b, double dt)
{
    if (int e = lock_check(b, dt, false)) return e;
    if (int e = lock_consts(b, dt)) return e;
    const size_t n3 = 3 * (size_t)b->Ntot;
    if (!b->xn.p) {
        BCK(b->xn.alloc(n3));
        BCK(b->vn.alloc(n3));
    }
    cudaStream_t s = b->stream;
    blob_factors(b, true);
    b->lock_open = true;
    b->lock_stats = false;
    b->lock = true;
    // the per-mesh counts and start lists of the meshes taking part; then
    // UpdateKNC (a no-op in the default kinematic mode), BeginEvaluation(
    // m_vecPos0, x), m_vecPos0 = x (LeafDSH_Solid3D_FEM.cpp:2824-2846)
    LoopSync ls{};
    ls.mcount = b->mcount.p;
    ls.gcount = b->counter.p;
    ls.err = b->err.p;
    if (b->opt.precision == FEM_PRECISION_FP64) {
        BatchLaunch<double>::reset_counts(b->view<double>(), ls, 0, 0, 0, s);
        BatchLaunch<double>::begin_eval(b->view<double>(), b->x.p, 0, s);
    } else {
        BatchLaunch<float>::reset_counts(b->view<float>(), ls, 0, 0, 0, s);
        BatchLaunch<float>::begin_eval(b->view<float>(), b->x.p, 0, s);
    }
    b->lock = false;
    if (b->any_dapd) BCK(cudaMemcpyAsync(b->prev_x.p, b->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    // the iterate starts at x^n (nr_end right after nr_init leaves x, v as they are)
    BCK(cudaMemcpyAsync(b->xn.p, b->x.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    BCK(cudaMemcpyAsync(b->vn.p, b->v.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s));
    BCK(cudaGetLastError());
    return FEM_OK;
}

int fem_batch_nr_prestep(fem_batch b, double dt)
{
    if (int e = lock_check(b, dt, true)) return e;
    if (int e = lock_consts(b, dt)) return e;
    blob_factors(b, true);
    const size_t bytes = sizeof(double) * 3 * (size_t)b->Ntot;
    cudaStream_t s = b->stream;
    // x_k = x^n, v_k = v^n; the iterate and solver counts restart
    // (LeafDSH_Solid3D_FEM.cpp:2869-2929)
    BCK(cudaMemcpyAsync(b->xn.p, b->x.p, bytes, cudaMemcpyDeviceToDevice, s));
    BCK(cudaMemcpyAsync(b->vn.p, b->v.p, bytes, cudaMemcpyDeviceToDevice, s));
    b->lock = true;
    if (b->opt.precision == FEM_PRECISION_FP64)
        BatchLaunch<double>::lock_phase(b->view<double>(), 0, s);
    else
        BatchLaunch<float>::lock_phase(b->view<float>(), 0, s);
    b->lock = false;
    BCK(cudaGetLastError());
    return FEM_OK;
}

int fem_batch_nr_midstep(fem_batch b, double dt)
{
    if (int e = lock_check(b, dt, true)) return e;
    if (int e = lock_consts(b, dt)) return e;
    blob_factors(b, true);
    if (int e = lock_solve_phase(b, 1)) return e;
    BCK(cudaMemcpyAsync(b->st_host, b->st.p, sizeof(StepScalars) * b->M, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    for (uint32_t m = 0; m < b->M; m++)
        if (b->st_host[m].status == FEM_E_NAN) return batch_fail(FEM_E_NAN, "NaN or Inf in the residual of mesh %u", m);
    return FEM_OK;
}

int fem_batch_nr_poststep(fem_batch b, double dt)
{
    if (int e = lock_check(b, dt, true)) return e;
    if (int e = lock_consts(b, dt)) return e;
    return lock_solve_phase(b, 2);
}

int fem_batch_nr_end(fem_batch b, double dt)
{
    if (int e = lock_check(b, dt, true)) return e;
    if (int e = lock_consts(b, dt)) return e;
    const size_t bytes = sizeof(double) * 3 * (size_t)b->Ntot;
    cudaStream_t s = b->stream;
    // x = x_k, v = v_k; RecomputeEnergy's potential term (NR_End evaluates
    // no V: the elastic energy keeps its value; LeafDSH_Solid3D_FEM.cpp:
    // 2847-2868, 1554-1584)
    BCK(cudaMemcpyAsync(b->x.p, b->xn.p, bytes, cudaMemcpyDeviceToDevice, s));
    BCK(cudaMemcpyAsync(b->v.p, b->vn.p, bytes, cudaMemcpyDeviceToDevice, s));
    bool energy = false;
    for (auto& m : b->meshes) energy |= m.p.compute_energy != 0;
    b->lock = true;
    if (b->opt.precision == FEM_PRECISION_FP64) {
        BatchLaunch<double>::lock_phase(b->view<double>(), 1, s);
        if (energy) {
            BatchLaunch<double>::tile_potential(b->view<double>(), b->x.p, b->tpart.p, s);
            BatchLaunch<double>::fin_energy(b->view<double>(), FIN_ENERGY_P, b->tpart.p, s);
        }
    } else {
        BatchLaunch<float>::lock_phase(b->view<float>(), 1, s);
        if (energy) {
            BatchLaunch<float>::tile_potential(b->view<float>(), b->x.p, b->tpart.p, s);
            BatchLaunch<float>::fin_energy(b->view<float>(), FIN_ENERGY_P, b->tpart.p, s);
        }
    }
    b->lock = false;
    blob_factors(b, false);
    b->lock_open = false;
    b->lock_stats = true;
    BCK(cudaMemcpyAsync(b->st_host, b->st.p, sizeof(StepScalars) * b->M, cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
    return FEM_OK;
}

int fem_batch_multi_step(fem_batch b, double dt, uint32_t nsteps)
{
    if (int e = lock_check(b, dt, false)) return e;
    uint32_t max_nr_iter = 0;
    for (uint32_t m = 0; m < b->M; m++)
        if (b->mask_host.empty() || b->mask_host[m] == 1)
            max_nr_iter = std::max(max_nr_iter, b->meshes[m].p.nr_max_iter);
    for (uint32_t step = 0; step < nsteps; step++) {
        if (int e = fem_batch_nr_init(b, dt)) return e;
        uint32_t nr_iter = 0;
        do {
            if (int e = fem_batch_nr_prestep(b, dt)) return e;
            if (int e = fem_batch_nr_midstep(b, dt)) return e;
            if (int e = fem_batch_nr_poststep(b, dt)) return e;
        } while (++nr_iter < max_nr_iter);
        if (int e = fem_batch_nr_end(b, dt)) return e;
    }
    return FEM_OK;
}

int fem_batch_synchronize(fem_batch b)
{
    if (int e = check_ready(b)) return e;
    BCK(cudaMemcpyAsync(b->st_host, b->st.p, sizeof(StepScalars) * b->M, cudaMemcpyDeviceToHost, b->stream));
    unsigned err = 0;
    if (b->err.p) BCK(cudaMemcpyAsync(&err, b->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    if (err) {
        // reported once: the next launches start with a clear word
        BCK(cudaMemsetAsync(b->err.p, 0, sizeof(unsigned), b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        return batch_fail(FEM_E_TIMEOUT, "a bounded device wait gave up (code %u: 1 tile copy, 2 copy drain, 3 grid "
                                         "barrier)", err);
    }
    for (uint32_t m = 0; m < b->M; m++)
        if (b->st_host[m].status == FEM_E_NAN) return batch_fail(FEM_E_NAN, "NaN or Inf in the CG residual of mesh %u", m);
    return FEM_OK;
}

int fem_batch_step(fem_batch b, uint32_t nsteps)
{
    if (int e = fem_batch_step_async(b, nsteps)) return e;
    return fem_batch_synchronize(b);
}

int fem_batch_finished(fem_batch b, uint8_t* flags)
{
    if (int e = check_ready(b)) return e;
    if (!flags) return batch_fail(FEM_E_ARG, "null flags");
    for (uint32_t m = 0; m < b->M; m++) {
        const StepScalars& h = b->st_host[m];
        flags[m] = h.step_done ? 1 : (h.done ? 0 : 2);
    }
    return FEM_OK;
}

int fem_batch_get_stats(fem_batch b, uint32_t mesh, fem_step_stats* out)
{
    if (int e = check_ready(b)) return e;
    if (mesh >= b->M || !out) return batch_fail(FEM_E_ARG, "bad mesh index or null output");
    const StepScalars& h = b->st_host[mesh];  // as of the last synchronize
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
    out->resolved_det_F = h.res_det_F;
    out->resolved_isotropic = h.res_isotropic;
    out->resolved_tie = h.res_tie;
    out->resolved_check = h.res_check;
    if (b->lock_stats) {
        // the Leaf's m_Stats after NR_End: solver iterations since the last
        // NR_PreStep, m_NR_nr_k (reset by every NR_PreStep)
        out->cg_iterations = h.fie_cg;
        out->nr_iterations = h.nr_k;
    } else if (b->mc_host[mesh].integrator != kMeshQie) {
        // the Leaf's FIE stats (m_SolverLS_NumIter summed over the Newton
        // iterations, m_SolverNR_NumIter, m_SolverNR_AbsPrec)
        out->cg_iterations = h.fie_cg;
        if (!h.nr_solved) out->rel_residual = out->abs_residual = 0.0;
        out->nr_iterations = h.nr_k;
        out->nr_abs_residual = h.nr_abs;
        out->nr_rel_residual = h.nr_delta0 > 0 ? h.nr_abs / h.nr_delta0 : 0.0;
    }
    return FEM_OK;
}

int fem_batch_kernel_launches(fem_batch b, uint32_t steps, uint64_t* launches)
{
    if (int e = check_ready(b)) return e;
    if (!launches) return batch_fail(FEM_E_ARG, "null output");
    unsigned body_runs = 0;
    BCK(cudaMemcpyAsync(&body_runs, b->any_flag.p, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    // kernels per step outside the CG loop, plus per executed CG iteration 3
    // (FP64 path) or 6 (mixed path: tile product, refresh product -- counted
    // in every iteration, an upper bound --, mesh alpha unless the node pass
    // forms it, node pass, mesh update)
    bool energy = false;
    for (auto& m : b->meshes) energy |= m.p.compute_energy != 0;
    const bool mixed = b->opt.precision == FEM_PRECISION_MIXED;
    const uint64_t fixed = 8 + (b->K ? 1 : 0) + (energy ? 4 : 0);
    const uint64_t per_iter = mixed ? (b->opt.fuse_alpha ? 5ull : 6ull) : 3ull;
    *launches = (uint64_t)steps * fixed + per_iter * body_runs;
    return FEM_OK;
}

int fem_batch_reset_launch_count(fem_batch b)
{
    if (int e = check_ready(b)) return e;
    BCK(cudaMemsetAsync(b->any_flag.p, 0, sizeof(unsigned), b->stream));
    return FEM_OK;
}

int fem_batch_stream(fem_batch b, void** stream)
{
    if (int e = check_ready(b)) return e;
    if (!stream) return batch_fail(FEM_E_ARG, "null stream pointer");
    *stream = (void*)b->stream;
    return FEM_OK;
}

}  // extern "C"
