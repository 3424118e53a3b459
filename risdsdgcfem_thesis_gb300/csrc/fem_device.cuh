// fem_device.cuh -- device-side data layout and launcher declarations shared
// by the kernels (fem_kernels.cu, rotation.cu) and the host runtime (solid.cu).
//
// Layout in HBM for one solid (T tets, N nodes):
//   tets      int4[T]          node ids of each tet
//   Dinv      S[9][T]          Dm^-1 of each tet, row-major, component-major
//                              arrays (coalesced per component)
//   mat       S[3][T]          V*(lambda+2mu), V*lambda, V*mu of each tet (the
//                              entries a_k1, a_nu, a_k2 of the reference's E
//                              matrix, TetrahedronElement3.h:141-156, times V)
//   R         S[9][T]          cached rotation, detF double[T]
//   node vectors (x, v, y, b, r, d, q, rest): AoS xyz, 3N scalars, the
//                              reference's Vec3 array layout
//   eout      S[T][4][3]       per-element nodal products, gathered per node
//   csr_ptr/csr_idx            node -> (4*e + slot) entries in element order,
//                              the order the reference scatters in
//   fixed     uint8[N]         1 where a kinematic node constraint zeroes the row
// S is double on the FP64 path and float on the mixed path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lcm.cuh"

namespace femgb {

// MINRES recurrence scalars (ILSS_MINRES::Solve, ILSS_MINRES.h:51-168).
struct MinresScalars {
    double norm_r_sq, norm_b_sq;     // |r|^2 carried by the Givens sines; |b|^2
    double beta, beta_new, beta_one;  // Lanczos norms (beta_one: of the initial residual)
    double alpha;
    double c, c_old, s, s_old, eta;   // Givens rotation state
    double inv_beta, neg_r2, neg_r3, inv_r1, x_coef;  // this iteration's update coefficients
};

// Device-resident CG and step scalars of one solid.
struct StepScalars {
    double delta_new, delta_old, delta_0, delta_target, abs_eps_sq;
    double alpha, beta, dot_dq;
    double elastic_energy, potential_energy;
    double rel_residual, abs_residual;
    uint32_t k, max_iter, done, status;
    uint32_t inverted, fp64_resolved, refresh_every;
    float beta_f;       // beta rounded to FP32 (mixed path)
    uint32_t finished;      // batch: the CG loop ended during this launch (cleared at launch start)
    uint32_t refresh_next;  // mixed: the next iteration recomputes r = b - A y in FP64
    double delta_refresh;   // mixed: |r|^2 right after the last FP64 residual
    uint32_t k_refresh;
    uint32_t confirm;       // mixed: this iteration only measures the FP64 residual (exit test)
    float alpha_f;          // mixed: this iteration's alpha in FP32 (0 on a confirm iteration)
    uint32_t brk;           // mixed: this iteration breaks down (|d.q| < abs^2) and leaves the loop
    uint32_t done_prev;     // MINRES: `done` as it was at the top of the current iteration
    uint32_t mr_pending;    // batch MINRES: 1 = this iteration's vector and iterate update is due,
                            // 2 = the start (or restart) residual is to be normalised
    // batch: the step's Newton level (QIE meshes make one pass of it)
    uint32_t nr_go;         // takes part in the next start section (b, constraints, r0)
    uint32_t nr_k;          // FIE: Newton iterations of this step so far
    uint32_t nr_solved;     // FIE: some linear solve ran in this step
    uint32_t step_done;     // the step ended during this launch (energy, completion flag)
    uint32_t fie_cg;        // FIE: linear-solver iterations summed over this step's Newton iterations
    double nr_delta0;       // FIE: |b_0| of this step
    double nr_abs;          // FIE: the last |b_k| or |y_k|
    unsigned long long total_iters;
    double host_sum;        // FIE: the last FIN_SUM total (|b_k|^2 or |y_k|^2), read by the host
    MinresScalars mr;       // MINRES solver state (FP64 solid)
    // mixed: rotations of this step by cause of their double-precision
    // re-solve: det F <= degenerate_det_F (FP64 MSVD), a nearly isotropic
    // F^T F (FP64 MSVD in place of double-float), and with FP32 rotations an
    // MSVD branch near a tie or a failed sensitivity check
    uint32_t res_det_F, res_isotropic, res_tie, res_check;
    uint32_t fin_ticket;    // FP64 solid: blocks of the running kernel done with their partial (0 between kernels)
};

// One MINRES iteration's Givens rotation and update coefficients from
// |v1|^2 after the Lanczos step (ILSS_MINRES.h:131-156): beta_new, the
// rotation (c, s), the coefficients of the direction and iterate updates,
// and the residual norm carried by the sines.
__device__ __forceinline__ void minres_givens(MinresScalars& mr, double beta_new_sq)
{
    mr.beta_new = ::sqrt(beta_new_sq);
    mr.inv_beta = 1.0 / mr.beta_new;
    const double r2 = mr.s * mr.alpha + mr.c * mr.c_old * mr.beta;
    const double r3 = mr.s_old * mr.beta;
    const double r1_hat = mr.c * mr.alpha - mr.c_old * mr.s * mr.beta;
    const double r1 = ::sqrt(r1_hat * r1_hat + beta_new_sq);
    mr.c_old = mr.c;
    mr.s_old = mr.s;
    mr.c = r1_hat / r1;
    mr.s = mr.beta_new / r1;
    mr.neg_r2 = -r2;
    mr.neg_r3 = -r3;
    mr.inv_r1 = 1.0 / r1;
    mr.x_coef = mr.beta_one * mr.c * mr.eta;
    mr.norm_r_sq *= mr.s * mr.s;
    mr.eta = -mr.s * mr.eta;
}

// MINRES start from the residual r0 (ILSS_MINRES.h:74-107): |r0|^2 and the
// Givens state of an empty Lanczos basis.
__device__ __forceinline__ void minres_start(MinresScalars& mr, double r0_sq)
{
    mr.norm_r_sq = r0_sq;
    mr.beta_new = ::sqrt(r0_sq);
    mr.beta_one = mr.beta_new;
    mr.inv_beta = 1.0 / mr.beta_new;
    mr.c = 1.0; mr.c_old = 1.0; mr.s = 0.0; mr.s_old = 0.0; mr.eta = 1.0;
}

template <typename S>
struct MeshView {
    uint32_t N, T;
    const int4* tets;
    const S* Dinv;     // [9][T]
    const S* mat;      // [3][T]
    S* R;              // [9][T]
    double* detF;      // [T]
    const double* vol; // [T]
    const double* rest;          // [3N] (double)
    const uint32_t* csr_ptr;     // [N+1]
    const uint32_t* csr_idx;     // [4T]
    const uint8_t* fixed;        // [N]
    S* eout;                     // [12T]
    // FP64 solid: the assembled stiffness K = sum_e R K0 R^T as 3x3 blocks
    // (row starts [N+1], columns [nnzb], blocks [nnzb][9] row-major); when
    // set, the solvers' node kernels take K u from it instead of gathering
    // the element outputs
    const uint32_t* bsr_row = nullptr;
    const uint32_t* bsr_col = nullptr;
    const double* bsr_val = nullptr;
};

struct StepConsts {
    double dt, inv_dt, mass, factor_M, factor_K;
    double gravity[3];
    double density;
    double rel_eps_sq, abs_eps_sq;
    uint32_t max_iter;
};

constexpr int kBlock = 256;
constexpr int kFinalizeThreads = 512;

// ---- launchers (fem_kernels.cu / rotation.cu) ----
void launch_begin_eval_fp64(const MeshView<double>& m, const double* x, double* F_out, StepScalars* st,
                            cudaStream_t s);
struct DapdParams;
void launch_begin_eval_dapd_fp64(const MeshView<double>& m, const double* xprev, const double* x, uchar2* doc,
                                 const DapdParams& p, double* F_out, StepScalars* st, cudaStream_t s);
void launch_elem_spmv_fp64(const MeshView<double>& m, const double* d, const StepScalars* st, int check_done,
                           cudaStream_t s);
void launch_elem_force_fp64(const MeshView<double>& m, const double* x, int write_out, double* energy_partials,
                            cudaStream_t s);
void launch_node_b_fp64(const MeshView<double>& m, const StepConsts& c, const double* v, double* b, double* y,
                        cudaStream_t s);
void launch_knc_fp64(uint32_t N, uint32_t count, const uint32_t* nodes, const double* targets, const double* x,
                     const StepConsts& c, double* b, double* y, cudaStream_t s);
void launch_node_residual_fp64(const MeshView<double>& m, const StepConsts& c, const double* b, const double* y,
                               double* r, double* d, double* partials, cudaStream_t s);
// The CG iteration's two reductions end in the kernel that makes their
// partials: the block that finishes last adds them (slot order) and takes
// the scalar step (alpha; beta and the loop test), and with set_cond sets
// the step graph's WHILE condition.
void launch_node_q_fp64(const MeshView<double>& m, const StepConsts& c, const double* d, double* q,
                        double* partials, StepScalars* st, cudaStream_t s, cudaGraphConditionalHandle cond = 0,
                        int set_cond = 0);
void launch_node_xr_fp64(uint32_t N, double* y, double* r, const double* d, const double* q, double* partials,
                         StepScalars* st, cudaStream_t s, cudaGraphConditionalHandle cond = 0, int set_cond = 0);
void launch_node_d_fp64(uint32_t N, const uint8_t* fixed, double* d, const double* r, const StepScalars* st,
                        cudaStream_t s);
void launch_integrate_fp64(uint32_t N, double dt, double* x, double* v, const double* y, cudaStream_t s);
// Fully-implicit Euler (Newton on Delta x) pieces, FP64 solid path.
void launch_node_b_fie_fp64(const MeshView<double>& m, const StepConsts& c, const double* x, const double* xn,
                            const double* vn, int warm, double* b, double* y, cudaStream_t s);
void launch_knc_fie_fp64(uint32_t N, uint32_t count, const uint32_t* nodes, const double* targets, const double* x, double* b,
                         double* y, cudaStream_t s);
void launch_sq_norm_fp64(uint32_t n, const double* v, double* partials, cudaStream_t s);
void launch_fie_update_fp64(uint32_t N, double inv_dt, double* x, double* v, const double* xn, const double* y,
                            double* partials, cudaStream_t s);
// C_LCM material (FP64 solid): element force and/or energy from the stored F,
// and the truncated differential of d.
void launch_elem_lcm_force_fp64(const MeshView<double>& m, const double* F, const PkMaterial& mat, int write_out,
                                double* energy_partials, cudaStream_t s);
void launch_elem_lcm_spmv_fp64(const MeshView<double>& m, const double* d, const double* F, const PkMaterial& mat,
                               const StepScalars* st, int check_done, cudaStream_t s);
// MINRES (FP64 solid). v1 = S (b - A y) and partial |v1|^2 from a fresh eout of y.
void launch_mr_init_fp64(const MeshView<double>& m, const StepConsts& c, const double* b, const double* y,
                         double* v1, double* partials, cudaStream_t s);
// v1 *= 1/beta_new ; v = p = p0 = 0
void launch_mr_start_fp64(uint32_t N, double* v1, double* v, double* p, double* p0, const StepScalars* st,
                          cudaStream_t s);
// v1 = S A w - beta v0 (w = v, eout of v) ; partial v1.v
void launch_mr_q_fp64(const MeshView<double>& m, const StepConsts& c, const double* v, const double* v0,
                      double* v1, double* partials, const StepScalars* st, cudaStream_t s);
// v1 -= alpha v ; partial |v1|^2
void launch_mr_v1_fp64(uint32_t N, double* v1, const double* v, double* partials, const StepScalars* st,
                       cudaStream_t s);
// v1 /= beta_new ; p0 <- (w - r2 p - r3 p0) / r1 (the new p, in p0's buffer) ; y += coef p_new
void launch_mr_update_fp64(uint32_t N, double* v1, const double* v, const double* p, double* p0, double* y,
                           const StepScalars* st, cudaStream_t s);
void launch_potential_fp64(const MeshView<double>& m, const StepConsts& c, const double* x, double* partials,
                           cudaStream_t s);
void launch_apply_A_fp64(const MeshView<double>& m, double factor_M, double factor_K, double mass,
                         const double* d, double* q, cudaStream_t s);
void launch_gather_sum_fp64(const MeshView<double>& m, double sign, double* f, cudaStream_t s);
void launch_rebake_material_fp64(uint32_t T, const double* vol, double k0, double k1, double k2, double* mat,
                                 cudaStream_t s);

// finalizers: one block, fixed-order sums of `count` block partials
enum FinalizeKind {
    FIN_INIT = 0, FIN_ALPHA = 1, FIN_BETA = 2, FIN_ENERGY_E = 3, FIN_ENERGY_P = 4, FIN_STATS = 5,
    FIN_SUM = 6,  // host_sum = total
    // MINRES: init (|r0|^2 = total, |b|^2 from host_sum), alpha, beta + Givens, stats
    FIN_MR_INIT = 7, FIN_MR_ALPHA = 8, FIN_MR_BETA = 9, FIN_MR_STATS = 10
};
// set_cond: the kinds that end a solver's loop test (init, alpha, beta and
// their MINRES forms) also set the step graph's WHILE condition `cond` to
// "the loop goes on"
void launch_finalize(int kind, const double* partials, uint32_t count, const StepConsts& c, StepScalars* st,
                     cudaStream_t s, cudaGraphConditionalHandle cond = 0, int set_cond = 0);

// The assembled stiffness's blocks (MeshView::bsr_*): block slot s sums, in
// element order, R K0[li][lj] R^T over its contributions contrib[cptr[s]..
// cptr[s+1]) = element << 4 | li << 2 | lj.
void launch_bsr_assemble_fp64(const MeshView<double>& m, uint32_t nnzb, const uint32_t* cptr,
                              const uint32_t* contrib, double* val, cudaStream_t s);

// The whole CG solve of a small C_WRP solid on one thread-block cluster
// (fem_kernels.cu): CTA r of `ctas` owns the elements [r ept, (r+1) ept) and
// the nodes [r npt, (r+1) npt); ent_max bounds a CTA's CSR entries; smem is
// its dynamic shared memory (cg_cluster_smem_bytes).
constexpr uint32_t kCgClusterMaxCtas = 16, kCgClusterMaxThreads = 512;
constexpr size_t kCgClusterMaxSmem = 200 * 1024;
// split: three lanes per element (ten elements per warp), else one.
struct CgClusterPlan {
    uint32_t ctas, threads, ept, npt, ent_max, split;
    size_t smem;
};
size_t cg_cluster_smem_bytes(uint32_t ept, uint32_t npt, uint32_t ent_max);
// The plan launches on this device (its cluster size, threads and shared
// memory give at least one resident cluster).
bool cg_cluster_fits(const CgClusterPlan& p);
// ent: per CSR entry, (CTA owning the corner's element) << 24 | (local
// element index * 4 + corner).
cudaError_t launch_cg_cluster_fp64(const MeshView<double>& m, const StepConsts& c, const CgClusterPlan& p,
                                   const uint32_t* ent, const double* b, double* y, StepScalars* st, cudaStream_t s);

uint32_t grid_for(uint32_t n);    // grid size of the grid-stride kernels
uint64_t& launch_counter();       // kernels launched by this library

// Optional per-kernel timing with CUDA events recorded on the launching
// stream around each launch of a named kernel (off unless enabled).
void prof_begin(const char* name, cudaStream_t s);
void prof_end(const char* name, cudaStream_t s);
bool prof_enabled();
}  // namespace femgb
