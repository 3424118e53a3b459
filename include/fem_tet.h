/* fem_tet.h -- C ABI of the GB300-native corotational linear-tetrahedral FEM
 * implicit-Euler step (the Saphyre2 LeafDSH_Solid3D_FEM / TetrahedronElementSet3 /
 * ILSS_CG path), implemented by libfemtet_gb300.so with hand-written sm_103a
 * kernels.
 *
 * Conventions
 *  - Plain pointers and sizes only. Host arrays are caller-owned and copied
 *    in or out during the call; device state is owned by the handle.
 *  - Node vectors are AoS xyz triples (N*3 doubles), the reference's Vec3
 *    array layout (Saphyre2 ParticleSystem m_vecPos/m_vecVel). Tets are T*4
 *    uint32 node ids (the reference uses uint16, TetrahedronElementSet3.h:73-74).
 *  - Every entry point returns an int status (FEM_OK on success);
 *    fem_last_error() gives the message of the last failure on the calling
 *    thread. The reference returns no errors (asserts only).
 *  - One CUDA stream per handle; a handle is thread-compatible, not
 *    thread-safe. All calls on a handle are synchronous unless named _async.
 */
#ifndef FEM_TET_H
#define FEM_TET_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum fem_status {
    FEM_OK = 0,
    FEM_E_ARG = 1,       /* bad argument (null pointer, zero size, out-of-range value) */
    FEM_E_INDEX = 2,     /* a tet or constraint names a node >= N */
    FEM_E_NAN = 3,       /* NaN/Inf reached the solver residual */
    FEM_E_OOM = 4,       /* device allocation failed */
    FEM_E_CUDA = 5,      /* CUDA runtime error (message in fem_last_error) */
    FEM_E_TIMEOUT = 6,   /* a bounded device-side wait gave up */
    FEM_E_NODEVICE = 7,  /* no CUDA device / extension not usable */
    FEM_E_DEGENERATE = 8 /* a tet has non-positive rest volume */
};

enum fem_precision {
    /* Plain FP64: every product, reduction and rotation in double. The
     * drop-in for the reference's FP64 step. */
    FEM_PRECISION_FP64 = 0,
    /* Mixed: FP32 element products and vector updates, FP64 dot products and
     * norms, FP64 residual refresh r = b - A x when |r| has fallen by
     * refresh_drop since the last one (or after refresh_every iterations),
     * FP32 rotations re-solved in FP64 where det F <=
     * degenerate_det_F or where the FP32 rotation is sensitive to rounding
     * (rotation_check). */
    FEM_PRECISION_MIXED = 1
};

/* Time integrators of LeafDSH_Solid3D_FEM::FixedStep
 * (LeafDSH_Solid3D_FEM.cpp:944-963; Params::EIntegratorType,
 * LeafDSH_Solid3D_FEM.h:110). */
enum fem_integrator {
    /* Step_QuasiImplicitEuler_v (LeafDSH_Solid3D_FEM.cpp:1205-1328): one
     * linearised solve for v^{n+1} per step. The reference default. */
    FEM_INTEGRATOR_QIE_V = 0,
    /* Step_FullyImplicitEuler_dx(dt) (LeafDSH_Solid3D_FEM.cpp:1357-1552):
     * Newton on Delta x = x^{n+1} - x^n, the rotations and the elastic force
     * re-evaluated at every Newton iterate, up to nr_max_iter iterations,
     * stopping when |b_k| < nr_abs_epsilon. On the solid and in batches of
     * either precision (a device-side Newton loop, each solid leaving on its
     * own test), and in servers (shards of their own that run whole
     * steps). */
    FEM_INTEGRATOR_FIE_DX = 1,
    /* Step_FullyImplicitEuler_dx(0): the same Newton loop without inertia
     * (quasi-static equilibrium; velocities become zero). As FIE_DX. */
    FEM_INTEGRATOR_FIE_DX_QUASISTATIC = 2
};

/* Linear solvers of the step (LeafDSH_Solid3D_FEM::Params::m_SolverLS_Type,
 * LS_Solve, LeafDSH_Solid3D_FEM.cpp:1136-1154). Both stop on |r|^2 <= abs^2,
 * on a relative test, or at ls_max_iter. */
enum fem_ls_solver {
    /* ns::ILSS_CG (ILSS_CG.h:38-151): relative test |r|^2 <= rel^2 |r0|^2,
     * breakdown when |d.q| < abs^2. The default. */
    FEM_LS_CG = 0,
    /* ns::ILSS_MINRES (ILSS_MINRES.h:51-168): Paige-Saunders MINRES without
     * a preconditioner; |r| carried by the Givens sines, relative test
     * |r|^2 <= rel^2 |b|^2. On the solid, in batches and servers (mixed
     * precision: FP32 Lanczos vectors; when the estimate passes, the FP64
     * residual of the iterate decides, restarting MINRES from it if needed). */
    FEM_LS_MINRES = 1
};

/* Material models of the element set (ms::fem::Params::m_MM, Params.h:48-62;
 * f_e / df_x / V dispatch, TetrahedronElementSet3.cpp:303-400). */
enum fem_material {
    /* C_WRP: warped stiffness f = -R K0 (R^T x - X), df = -R K0 R^T dx. The
     * default. */
    FEM_MATERIAL_C_WRP = 0,
    /* C_LCM: linear corotational in first Piola-Kirchhoff form,
     * P = R (2 mu (S - I) + lambda tr(S - I) I) with S = R^T F, its
     * differential without the dR term (truncated) and energy
     * V (mu |S - I|^2 + lambda/2 tr(S - I)^2) (TetrahedronElementSet3.cpp:
     * 1154-1178, 1838-1873, 1489-1507). mu and lambda come from the scalar
     * young_modulus and poisson_ratio, as the reference's element set takes
     * them from its Params even where per-element E, nu re-bake K0. On the
     * solid, in batches and servers of either precision. */
    FEM_MATERIAL_C_LCM = 1,
    /* C_LCMH: C_LCM's force and energy, and a differential that blends LCM
     * and warped stiffness per element by w = Clamp01(tr|S - I| / (3 k)),
     * k = ecie_k_factor: dP = 2 mu (w dF + (1 - w) R sym(R^T dF)) +
     * lambda tr(R^T dF) R for k > 0.1, C_LCM's dP otherwise
     * (TetrahedronElementSet3.cpp:1875-1930). On the solid, in batches and
     * servers of either precision (mixed: w of each element's last
     * evaluation, FP32 products). */
    FEM_MATERIAL_C_LCMH = 2,
    /* C_CCM: P = R (2 mu (S - I) + lambda (det S - 1) adj(S)^T) and the
     * reference's differential, which builds dDs from nodes (0, 1, 2, 2)
     * (TetrahedronElementSet3.cpp:1180-1206, 1932-1970; :1948): its A is not
     * symmetric positive definite, so CG diverges and the state runs to
     * Inf/NaN within steps, in the reference as here (FEM_E_NAN). Energy 0
     * (its body is compiled out of the reference). On the solid and in FP64
     * batches and servers. */
    FEM_MATERIAL_C_CCM = 3
};

/* Rotation methods of the element set (ms::fem::Params::ERotationMethod,
 * Params.h:63-67; ComputeRotations_*, TetrahedronElementSet3.cpp:267-278). */
enum fem_rotation {
    /* ComputeRotations_MSVD: R = U V^T of the PhysBAM-style SVD. The default. */
    FEM_ROTATION_MSVD = 0,
    /* ComputeRotations_DAPD (TetrahedronElementSet3.cpp:860-892): the Newton
     * polar rotation above dapd_threshold_det_F; at or below it, the rotation
     * of F with the collapsing vertex or edge moved along the collapse normal
     * (Rotation.cpp:364-495), the direction of collapse found from the
     * previous step's positions by the time-of-collapse cubic
     * (TetrahedronElementSet3.cpp:477-743) and kept while the element stays
     * degenerate; I where no direction is known. On the solid and in batches
     * and servers of either precision (there in FP64, per mesh). */
    FEM_ROTATION_DAPD = 1
};

/* Solid parameters. Mirrors bs::Solid3D::Params and Params_Extra
 * (Saphyre2 bs/Solid3D.h:27-85) for the fields this path reads:
 * FixedDT, Density, YoungModulus, PoissonRatio, DampingRatio, Gravity,
 * LS_Iter, LS_RelEpsilon, and the Leaf's LS abs epsilon, integrator and NR
 * settings (LeafDSH_Solid3D_FEM.h:209-241). Methods are fixed to the
 * reference defaults: material C_WRP, rotation MSVD, truncated
 * differentials, CG solver with warm start. */
typedef struct fem_params {
    double fixed_dt;          /* time step of one FixedStep [s] */
    double density;           /* rho [kg/m^3]; node mass = rho * sum(V_e) / N */
    double young_modulus;     /* E [Pa] (ignored where per-element E is given) */
    double poisson_ratio;     /* nu (ignored where per-element nu is given) */
    double damping_ratio;     /* zeta; Rayleigh coefficients from the reference's
                                 default frequencies 0.1 and 1e4 Hz */
    double gravity[3];        /* [m/s^2] */
    double ls_rel_epsilon;    /* CG stops when |r|^2 <= rel^2 |r0|^2 */
    double ls_abs_epsilon;    /* ... or |r|^2 <= abs^2 (and breaks if |d.q| < abs^2) */
    uint32_t ls_max_iter;     /* CG iteration cap per step */
    uint32_t precision;       /* enum fem_precision */
    double degenerate_det_F;  /* mixed only: elements with det F at or below this get the FP64
                                 rotation */
    uint32_t refresh_every;   /* mixed only: longest run of iterations between FP64
                                 residuals (0 = no periodic refresh) */
    uint32_t compute_energy;  /* 1: elastic and potential energy every step (as FixedStep) */
    double rotation_check;    /* mixed only, with rotation_fp32: an FP32 rotation is also
                                 re-solved when it moves by more than this (max entry)
                                 under a 2^-14 relative change of F; 0 = det F test only */
    double refresh_drop;      /* mixed only: the residual is recomputed in FP64 once |r|
                                 has fallen by this factor since the last time (reliable
                                 updates), and at least every refresh_every iterations;
                                 0 = by refresh_every alone */
    uint32_t rotation_fp32;   /* mixed only: 0 = every rotation re-solved at double
                                 precision (double-float arithmetic, about 48 bits; FP64
                                 where det F <= degenerate_det_F or F^T F is nearly
                                 isotropic); 1 = rotations in FP32, re-solved so where
                                 det F <= degenerate_det_F, a branch decision was a near
                                 tie or rotation_check flags them */
    uint32_t integrator;      /* enum fem_integrator; the batch and server paths take QIE_V only */
    uint32_t nr_max_iter;     /* FIE: Newton iteration cap per step (m_SolverNR_MaxIter) */
    uint32_t rotation;        /* enum fem_rotation; the batch and server paths take MSVD only */
    uint32_t ls_solver;       /* enum fem_ls_solver; the batch and server paths take CG only */
    double nr_abs_epsilon;    /* FIE: Newton stops once |b_k| < this (m_SolverNR_AbsEpsilon) */
    double dapd_threshold_det_F; /* DAPD: degenerate at or below this det F
                                    (m_DegenerateThresholdDetF, default 0.1f) */
    double dapd_l_factor;     /* DAPD: offset factors and exponent (m_DAPD_L_Factor 1, */
    double dapd_nl_factor;    /*   m_DAPD_NL_Factor 0, m_DAPD_NL_Exponent 2); float32 in the */
    double dapd_nl_exponent;  /*   reference, so they are rounded to float */
    uint32_t material;        /* enum fem_material; the batch and server paths take C_WRP only */
    uint32_t pad;
    double ecie_k_factor;     /* C_LCMH: blend radius k (m_ECIE_k_factor, float32 in the
                                 reference, default 1) */
} fem_params;

/* Per-step statistics (the Leaf's per-step LS stats, LeafDSH_Solid3D_FEM.h:597-622). */
typedef struct fem_step_stats {
    uint32_t cg_iterations;   /* ILSS_CG::GetNumIterations of the last step (FIE: summed over
                                 its Newton iterations, as m_SolverLS_NumIter) */
    uint32_t status;          /* enum fem_status of the last step */
    double rel_residual;      /* sqrt(delta_new / delta_0) (FIE: of the last solve; 0 if none ran) */
    double abs_residual;      /* sqrt(delta_new) */
    double elastic_energy;    /* TetrahedronElementSet3::V after the step */
    double potential_energy;  /* LeafDSH_Solid3D_FEM::RecomputeEnergy's potential term */
    uint32_t inverted_elements; /* elements with det F <= 0 at BeginEvaluation */
    uint32_t fp64_resolved;   /* mixed: elements whose rotation was re-solved at double
                                 precision (every element with rotation_fp32 = 0) */
    uint64_t total_cg_iterations; /* sum over the steps of this call */
    uint32_t nr_iterations;   /* FIE: Newton iterations of the last step (m_SolverNR_NumIter); 0 for QIE */
    uint32_t pad;
    double nr_rel_residual;   /* FIE: last |y_k| (or |b_k| when it converged) over the first |b_0| */
    double nr_abs_residual;   /* FIE: that last |y_k| or |b_k| (m_SolverNR_AbsPrec) */
    /* mixed: the re-solved rotations of fp64_resolved by cause. FP64 MSVD:
     * det F <= degenerate_det_F, or a nearly isotropic F^T F where the
     * double-float MSVD would lose its precision; with rotation_fp32 = 1
     * also why the FP32 rotation was not kept: an MSVD branch decision near
     * a tie, or the rotation_check sensitivity test (these two are re-solved
     * in double-float unless one of the first two applies) */
    uint32_t resolved_det_F, resolved_isotropic, resolved_tie, resolved_check;
} fem_step_stats;

typedef struct fem_solid_s* fem_solid;

/* Fills the reference defaults (fem::Params, LeafDSH_Solid3D_FEM::Params):
 * fixed_dt 0.001, density 1000, E 1000, nu 0.25, damping 1, gravity 0,
 * CG rel 1e-3, abs 1e-6, 20 iterations, FP64, threshold 1e-3, refresh 50,
 * energy on, rotation check 1e-3, refresh every 50 iterations (no drop rule),
 * QIE_V integrator, 3 Newton iterations with abs epsilon 1e-6, CG, MSVD
 * rotations (DAPD threshold 0.1f, factors 1, 0, 2), C_WRP material (C_LCMH
 * blend radius 1). */
int fem_params_default(fem_params* p);

/* Replaces: EditableTetrahedronElementSet3::BeginEdition/AddElement/EndEdition
 * (TetrahedronElementSet3.cpp:2084-2166), TetrahedronElementSet3::CreateCache
 * (:190-209) and LeafDSH_Solid3D_FEM::Create (LeafDSH_Solid3D_FEM.cpp:125-223).
 * rest_xyz: N*3; tets: T*4; young/poisson_per_elem: T each or null.
 * Node state starts at x = rest, v = 0 (Create, :136-143). */
int fem_solid_create(const double* rest_xyz, uint32_t N, const uint32_t* tets, uint32_t T,
                     const fem_params* params, const double* young_per_elem,
                     const double* poisson_per_elem, fem_solid* out);
int fem_solid_destroy(fem_solid s);
int fem_solid_get_sizes(fem_solid s, uint32_t* N, uint32_t* T);

/* Replaces: Solid3D::FixAllNodesInBoundaryPlane / CreateKinematicPointConstraint
 * -> KinematicNodeConstraintSet3::AddKNC (KinematicNodeConstraintSet3.h:32-40).
 * Sets the whole constraint list: position constraints on `nodes` with the
 * given targets (count*3). count == 0 clears it. */
int fem_solid_set_knc(fem_solid s, const uint32_t* nodes, const double* targets, uint32_t count);
/* Replaces: Solid3D::SetKinematicPointConstraint_Pos -> SetPosKNC
 * (KinematicNodeConstraintSet3.h:55-60) for every constraint (count*3). */
int fem_solid_set_knc_targets(fem_solid s, const double* targets);

/* State [pos|vel] (GLeafDSH_Model::QueryState / Solid3D::Dbg_SaveState);
 * either pointer may be null. set_state also sets the previous positions. */
int fem_solid_set_state(fem_solid s, const double* x, const double* v);
int fem_solid_get_state(fem_solid s, double* x, double* v);

/* Replaces: Solid3D::SetParamsExtra (bs/Solid3D.h:150; applied by the Leaf's
 * "set_params_extra", LeafDSH_Solid3D_FEM.cpp:380-492) and the Leaf's
 * run-time parameter rebuilds (RebuildMass, RebuildRayleighCoeffsFromFreqs,
 * RebuildFEM; LeafDSH_Solid3D_FEM.h:289-354) on a live solid, between steps.
 * Every field may change except precision (FP64): time step, density (node
 * mass), damping (Rayleigh coefficients), gravity, solver and tolerances,
 * integrator and Newton settings, material, rotation method and DAPD
 * settings, energy. Element data are kept unless young_modulus or
 * poisson_ratio change: then every element is re-baked from those scalar
 * values, as EditableTetrahedronElementSet3::SetParams does
 * (TetrahedronElementSet3.cpp:2168-2200), replacing per-element values.
 * Switching to DAPD starts it from the current positions with no direction
 * of collapse. Unlike the reference's set_params_extra, whose ls_rel_epsilon
 * goes through the Newton rebuild and is never applied
 * (LeafDSH_Solid3D_FEM.cpp:461), ls_rel_epsilon takes effect. */
int fem_solid_set_params(fem_solid s, const fem_params* params);
int fem_solid_get_params(fem_solid s, fem_params* params);
/* The FP64 solid's solver operator, an option of this library. The
 * reference's solvers apply the element set's product matrix-free
 * (ILSS_CG.h:38-151 over TetrahedronElementSet3's R K0 R^T products), and
 * so does this solid by default (on = 0). With on = 1 a C_WRP solid keeps
 * K = sum_e R K0 R^T as 3x3 blocks over the node graph, rebuilt at every
 * evaluation, and CG and MINRES take K u from its rows: about 24 FP64 FMAs
 * per tet and iteration against about 140, at the price of 76 B per block
 * (12.6 blocks per node on grid meshes) and one assembly per evaluation;
 * the sums run in another order, so other bits, within the same parity
 * tolerances. Other materials keep the element product, and so does the
 * one-cluster CG of solids of at most 8,192 tets. FEM_E_OOM when the blocks
 * do not fit. */
int fem_solid_set_assembled(fem_solid s, int on);

/* Replaces: the multi-solid Newton lock-step phases of the Leaf,
 * NR_Init / NR_PreStep / NR_MidStep / NR_PostStep / NR_End
 * (LeafDSH_Solid3D_FEM.cpp:2824-3039), which the aggregate scheme
 * SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update (SS_AggregateDSH_Basic.cpp:
 * 229-300) calls over all its solids so that contact terms between solids
 * can enter between them. dt is the phase's step (0: quasi-static); the
 * solid's integrator setting is not used. The solid's x, v stay x^n, v^n
 * until NR_End; x_k, v_k are the iterates:
 *   nr_init      BeginEvaluation at x (DAPD: against the previous
 *                positions), previous positions = x;
 *   nr_prestep   x_k = x, v_k = v, the iteration count reset to 0 -- at
 *                every NR iteration, as in the reference, so each iteration
 *                solves from x^n with the element forces and rotations of
 *                the previous iterate's evaluation;
 *   nr_midstep   b = m g + f_e + (1/dt) m (v - (1/dt)(x_k - x)), warm start
 *                y = dt v, constraint rows b = y = target - x_k, then the
 *                solid's linear solver with factor_M = 1/dt^2 + a0/dt,
 *                factor_K = 1 + a1/dt;
 *   nr_poststep  x_k += y, v_k = (x_k - x)/dt, BeginEvaluation(x, x_k);
 *   nr_end       x = x_k, v = v_k, the potential energy (the elastic energy
 *                keeps its value: NR_End evaluates none).
 * fem_solid_synchronize then reports the LS iterations and the iteration
 * count since the last nr_prestep (the Leaf's m_Stats). nr_init allocates
 * the iterates on first use. */
int fem_solid_nr_init(fem_solid s, double dt);
int fem_solid_nr_prestep(fem_solid s, double dt);
int fem_solid_nr_midstep(fem_solid s, double dt);
int fem_solid_nr_poststep(fem_solid s, double dt);
int fem_solid_nr_end(fem_solid s, double dt);
/* Replaces: the body of SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update
 * (SS_AggregateDSH_Basic.cpp:229-300) for nsteps fixed steps, its contact
 * calls left out: nr_init on every solid; then, the largest nr_max_iter of
 * the solids times, nr_prestep + nr_midstep on every solid and nr_poststep
 * on every solid; nr_end on every solid. The aggregate's time accumulator
 * (a step while the accumulated time exceeds the smallest fixed_dt) is the
 * caller's, as FixedStep is for fem_solid_step. */
int fem_multi_step(fem_solid* solids, uint32_t count, double dt, uint32_t nsteps);

/* DAPD state, for checkpoint and resume: the positions the last step started
 * from (m_vecPos0, N*3; the next BeginEvaluation's collapse test compares
 * against them) and each element's direction of collapse (T*2 bytes, as
 * fem_solid_get_doc). fem_solid_set_state resets the previous positions to
 * x, so a resume calls fem_solid_set_state, then fem_solid_set_dapd_state
 * with the saved values, and then steps as the uninterrupted run would.
 * Either pointer may be null. FEM_E_ARG when the solid does not use DAPD or
 * a direction is malformed. No counterpart call in the reference, which
 * keeps this state inside the element set (TetrahedronElementSet3.cpp:477-584). */
int fem_solid_get_dapd_state(fem_solid s, double* prev_x, uint8_t* doc);
int fem_solid_set_dapd_state(fem_solid s, const double* prev_x, const uint8_t* doc);

/* Replaces: LeafDSH_Solid3D_FEM::FixedStep (LeafDSH_Solid3D_FEM.cpp:898-990)
 * with Step_QuasiImplicitEuler_v (:1205-1328), nsteps times. stats may be null. */
int fem_solid_step(fem_solid s, uint32_t nsteps, fem_step_stats* stats);

/* Host-buffer round trip in one call: upload x,v (may be null = keep),
 * step nsteps, download x,v (may be null). */
int fem_solid_step_host(fem_solid s, const double* x_in, const double* v_in, uint32_t nsteps,
                        double* x_out, double* v_out, fem_step_stats* stats);

/* --- Element-level hooks (the IForce3 seam, TetrahedronElementSet3.h:29-58) --- */

/* Replaces TetrahedronElementSet3::BeginEvaluation (TetrahedronElementSet3.cpp:219-281):
 * F, det F and the rotation (MSVD, or DAPD against the solid's previous-step
 * positions) of every element at positions x (N*3). */
int fem_solid_begin_eval(fem_solid s, const double* x);
/* The cached rotations (T*9, row-major) and det F (T) of the last evaluation. */
int fem_solid_get_rotations(fem_solid s, double* R, double* detF);
/* DAPD: each element's direction of collapse (ElementCache3::m_DoC) as two
 * bytes (vit0, vit1): V-F when equal, E-E when vit0 < vit1, none = (3, 0).
 * T*2 bytes. FEM_E_ARG when the solid does not use DAPD. */
int fem_solid_get_doc(fem_solid s, uint8_t* doc);
/* f += f_e at the evaluated positions (C_f_e, TetrahedronElementSet3.cpp:1053-1096). N*3. */
int fem_solid_force_elastic(fem_solid s, double* f);
/* df += df_x(dx) = -R K0 R^T dx (C_df_x, TetrahedronElementSet3.cpp:1761-1836). N*3. */
int fem_solid_df_x(fem_solid s, const double* dx, double* df);
/* q = S (factor_M M d - factor_K df_x(d)) (LS_A_times_d + LS_ZeroKNC,
 * LeafDSH_Solid3D_FEM.cpp:1045-1079). N*3. */
int fem_solid_apply_A(fem_solid s, double factor_M, double factor_K, const double* d, double* q);
/* Elastic energy V at the evaluated positions (C_V, TetrahedronElementSet3.cpp:1456-1488). */
int fem_solid_energy(fem_solid s, double* V);
/* Uniform node mass and Rayleigh coefficients (RebuildMass, RebuildRayleighCoeffsFromFreqs). */
int fem_solid_mass_info(fem_solid s, double* node_mass, double* rayleigh2, double* total_volume);

/* No counterpart in the reference. The product of fem_solid_apply_A with its
 * per-element scratch in a static device array (12 doubles per tet, at most
 * FEM_NOALLOC_MAX_TETS tets: 6 MiB per device) instead of a device buffer,
 * for callers that cannot allocate device memory when they call it (a
 * fixed-rate control loop that cudaMalloc's implicit synchronisation would
 * stall, a process whose device memory another allocator has reserved). It
 * calls no allocating routine. Larger solids fail with FEM_E_ARG. All calls
 * on a device share the array and it keeps the last call's contents: calls
 * that overlap on the GPU race, so serialise them. Set-up happens in
 * fem_solid_create, which looks the array's device address up for every
 * solid of at most FEM_NOALLOC_MAX_TETS tets (the first lookup on a device
 * loads the array's module and reserves its 6 MiB there); only if that
 * lookup failed does the first call on the solid retry it, and that call
 * should then come before any stream capture. */
#define FEM_NOALLOC_MAX_TETS 65536u
int fem_solid_apply_A_noalloc(fem_solid s, double factor_M, double factor_K, const double* d, double* q);

/* --- Device-resident timing hooks (state stays in HBM) --- */
/* Enqueue nsteps on the handle's stream without synchronising and without
 * host copies; stats are left on the device. (The CG loop condition is read
 * once per chunk of iterations; the FIE integrators also read |b_k| and
 * |y_k| once per Newton iteration, so their steps return when done.) */
int fem_solid_step_async(fem_solid s, uint32_t nsteps);
int fem_solid_synchronize(fem_solid s, fem_step_stats* stats);
/* The handle's CUDA stream (a cudaStream_t) for event timing. */
int fem_solid_stream(fem_solid s, void** stream);

/* --- Batches: many independent solids stepped together (tiled path) ---
 *
 * The reference steps several solids one after another inside its
 * aggregate scheme (SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update,
 * SS_AggregateDSH_Basic.cpp:229-300); a batch steps them together on one GPU,
 * each with its own parameters, constraints and CG loop, so a solid's result
 * is the same alone and in any batch. One step of a batch is one CUDA graph
 * launch: the CG loop of every solid runs on the device until each has met
 * its own stopping test. */
typedef struct fem_batch_s* fem_batch;

typedef struct fem_batch_options {
    uint32_t precision;   /* enum fem_precision for every solid of the batch */
    uint32_t tile_elems;  /* elements per tile, 1..256 */
    uint32_t reorder;     /* 1: Morton order of element centroids before tiling */
    uint32_t use_graph;   /* 1: each step is one CUDA graph with a device-side CG loop */
    uint32_t chunk_nodes; /* nodes per node-pass work item, 32..8192 (0 = 1024) */
    uint32_t fuse_alpha;  /* mixed: 1 = every node-pass block forms its mesh's alpha from the
                             tile shares itself (one kernel fewer per CG iteration: shorter
                             iterations when few meshes run, more work when many do; the
                             same results either way) */
    uint32_t persistent_loop; /* mixed, tile_elems > 128: 1 = the CG iterations of a launch run
                             in one persistent cooperative kernel (the phases of an iteration
                             separated by bounded grid barriers; the fused alpha) sized to the
                             tiles of the meshes taking part, instead of four kernels per
                             iteration in a CUDA graph: much shorter iterations for a few small
                             meshes, the same results bit for bit. A grid barrier that gives up
                             is reported as FEM_E_TIMEOUT. */
} fem_batch_options;

int fem_batch_options_default(fem_batch_options* o);
int fem_batch_create(const fem_batch_options* opt, fem_batch* out);
/* Adds one solid (same inputs as fem_solid_create); returns its index. */
int fem_batch_add_mesh(fem_batch b, const double* rest_xyz, uint32_t N, const uint32_t* tets, uint32_t T,
                       const fem_params* params, const double* young_per_elem,
                       const double* poisson_per_elem, uint32_t* mesh_index);
/* Position constraints of one solid (before finalize). */
int fem_batch_set_knc(fem_batch b, uint32_t mesh, const uint32_t* nodes, const double* targets, uint32_t count);
/* Builds tiles and uploads everything; the batch is then device resident. */
int fem_batch_finalize(fem_batch b);
int fem_batch_destroy(fem_batch b);
int fem_batch_info(fem_batch b, uint32_t* meshes, uint64_t* nodes, uint64_t* tets, uint32_t* tiles,
                   uint64_t* device_bytes);
int fem_batch_set_knc_targets(fem_batch b, uint32_t mesh, const double* targets);
int fem_batch_set_state(fem_batch b, uint32_t mesh, const double* x, const double* v);
/* Replaces: Solid3D::SetParams / SetParamsExtra on one solid of an aggregate
 * (bs/Solid3D.h:96,150; LeafDSH_Solid3D_FEM.cpp:380-492) -- as
 * fem_solid_set_params, between steps, for mesh `mesh` of the batch: every
 * field may change except precision (the batch's). The mesh's constants
 * become those of a batch built with these parameters; a new
 * young_modulus or poisson_ratio re-bakes its elements from those scalar
 * values, replacing per-element ones; switching to DAPD starts it from the
 * mesh's current positions with no direction of collapse; buffers a new
 * method needs are allocated and the step graph is captured anew. On the
 * mixed path a P-K material takes its Lame pair from the element data, so
 * a mesh built with per-element E or nu whose data were re-baked for a P-K
 * material cannot return to C_WRP without new scalar values (FEM_E_ARG). The
 * batch's restrictions hold (C_CCM only in FP64 batches, the persistent
 * loop's, no FIE under an iteration budget); FEM_E_ARG while a lock-step is
 * open. */
int fem_batch_set_params(fem_batch b, uint32_t mesh, const fem_params* params);
/* The parameters mesh `mesh` steps with (its precision: the batch's). */
int fem_batch_get_params(fem_batch b, uint32_t mesh, fem_params* params);
int fem_batch_get_state(fem_batch b, uint32_t mesh, double* x, double* v);
/* The rotations (T*9, row-major, the caller's element order; the mixed path's
 * FP32 rotations widened to double) and det F (T) of mesh `mesh` as of its
 * last BeginEvaluation: the batch form of fem_solid_get_rotations (the
 * element set's cached R and det F, TetrahedronElementSet3.cpp:219-281).
 * Either pointer may be null. */
int fem_batch_get_rotations(fem_batch b, uint32_t mesh, double* R, double* detF);
/* A DAPD mesh's hidden state, as fem_solid_get/set_dapd_state: the positions
 * its last step started from (N*3) and the direction of collapse per element
 * (T*2), in the caller's node and element order. fem_batch_set_state resets
 * the previous positions to the new x (as on the solid), so a resume calls
 * fem_batch_set_state, then fem_batch_set_dapd_state. FEM_E_ARG for a mesh
 * that does not use DAPD. */
int fem_batch_get_dapd_state(fem_batch b, uint32_t mesh, double* prev_x, uint8_t* doc);
int fem_batch_set_dapd_state(fem_batch b, uint32_t mesh, const double* prev_x, const uint8_t* doc);
/* 1: steps run as the captured CUDA graph (device-side CG loop); 0: the same
 * kernels launched one by one with the CG loop on the host (per-kernel
 * profiling and timing). */
int fem_batch_use_graph(fem_batch b, int on);
/* All solids' states at once, concatenated in mesh order (sum N_m * 3). */
int fem_batch_set_state_all(fem_batch b, const double* x, const double* v);
int fem_batch_get_state_all(fem_batch b, double* x, double* v);
/* Host-buffer round trip: upload all states (null = keep), step, download. */
int fem_batch_step_host(fem_batch b, const double* x_in, const double* v_in, uint32_t nsteps, double* x_out,
                        double* v_out);
/* Which solids take part in the next launches (M bytes; null = all start):
 * 1 = start a step, 2 = continue a step that an iteration budget
 * (fem_batch_set_slice) interrupted, 0 = leave out (an interrupted step left
 * out is dropped). fem_batch_get_stats' `status`/`cg_iterations` then say
 * where each solid stands; a solid's step is complete when its CG loop has
 * ended (fem_batch_finished). */
int fem_batch_set_active(fem_batch b, const uint8_t* mask);
/* Iteration budget of each following launch (0 = run every CG loop to its
 * end, the default). With a budget, a launch stops after that many CG
 * iterations; solids whose loop has not ended continue in a later launch
 * (mask value 2) with bit-identical results. FEM_E_ARG in a batch with an
 * FIE solid (its Newton steps run whole). */
int fem_batch_set_slice(fem_batch b, uint32_t max_iterations);
/* Replaces: the Leaf's NR_Init / NR_PreStep / NR_MidStep / NR_PostStep /
 * NR_End (LeafDSH_Solid3D_FEM.cpp:2824-3039) on every solid of the batch
 * that takes part (fem_batch_set_active value 1; all by default) at once,
 * with the semantics of fem_solid_nr_* (the FIE system of step dt, 0 =
 * quasi-static; x, v stay x^n, v^n until nr_end; each nr_prestep restarts
 * the iterate at x^n), so a caller can add terms between the phases. Any
 * integrator, solver, rotation and material the batch takes; either
 * precision. nr_midstep returns once the solves have ended; nr_end
 * recomputes the potential energy only, and fem_batch_get_stats then reports
 * the solver iterations and iterate count since the last nr_prestep. Steps
 * (fem_batch_step*) are refused between nr_init and nr_end, and the phases
 * under an iteration budget or with fem_batch_options.persistent_loop. */
int fem_batch_nr_init(fem_batch b, double dt);
int fem_batch_nr_prestep(fem_batch b, double dt);
int fem_batch_nr_midstep(fem_batch b, double dt);
int fem_batch_nr_poststep(fem_batch b, double dt);
int fem_batch_nr_end(fem_batch b, double dt);
/* Replaces: SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update
 * (SS_AggregateDSH_Basic.cpp:229-300), its contact calls left out, over the
 * solids of the batch, nsteps times: nr_init; the largest nr_max_iter of
 * the solids times nr_prestep, nr_midstep, nr_poststep; nr_end (as
 * fem_multi_step over fem_solid handles). */
int fem_batch_multi_step(fem_batch b, double dt, uint32_t nsteps);
/* Per solid (M bytes): 1 if its step ended (its CG loop, or FIE Newton
 * loop, ended and the step was integrated) in the last launch; 2 if its loop
 * is still running; 0 otherwise. As of the last synchronize. */
int fem_batch_finished(fem_batch b, uint8_t* flags);
/* Poll limit of the device-side waits of the mixed path's tile product for
 * each tile's copy into shared memory (every wait on the device is bounded;
 * no counterpart in the reference, which has no device waits). A wait that
 * gives up sets the batch's error word: the CG loops stop at the end of that
 * iteration, the blocks drain their copies in flight, and the next
 * fem_batch_synchronize returns FEM_E_TIMEOUT once (the word is cleared). The
 * default (FEM_WAIT_LIMIT_DEFAULT) is 2^22 polls, far above any copy's
 * latency; 0 makes every such wait give up at once, which exercises that
 * error path. */
#define FEM_WAIT_LIMIT_DEFAULT 0xffffffffu
int fem_batch_set_wait_limit(fem_batch b, uint32_t polls);
int fem_batch_step_async(fem_batch b, uint32_t nsteps);
int fem_batch_synchronize(fem_batch b);
int fem_batch_step(fem_batch b, uint32_t nsteps);
/* Statistics of one solid's last step, as of the last synchronize. */
int fem_batch_get_stats(fem_batch b, uint32_t mesh, fem_step_stats* stats);
int fem_batch_stream(fem_batch b, void** stream);
/* Kernels launched by `steps` steps since the last reset (the CG-loop body
 * runs are counted on the device). */
int fem_batch_kernel_launches(fem_batch b, uint32_t steps, uint64_t* launches);
int fem_batch_reset_launch_count(fem_batch b);

/* --- Serving: step requests over device-resident scenes ---
 *
 * The reference steps a solid when its owner asks (bs::Solid3D::Update,
 * bs/Solid3D.cpp:61-104) and several solids one after another
 * (SS_AggregateDSH_Basic.cpp:229-300). A server keeps many scenes resident
 * on the GPU and serves requests of one FixedStep each:
 *  - scenes are registered, then admitted into device memory by
 *    fem_server_admit while the device bytes stay within hbm_budget_bytes;
 *    admitted scenes are grouped by size into shards (batches);
 *  - fem_server_submit queues a request; fem_server_pump (never blocking)
 *    harvests every shard launch that has finished, completes the requests
 *    whose step ended, and at once relaunches every idle shard that has
 *    steps running or requests waiting. A launch runs at most
 *    slice_iterations CG iterations: steps in flight continue in the next
 *    launch and requests that arrived meanwhile start there, so a request
 *    waits at most one slice to join; shards run concurrently on their own
 *    streams (continuous batching at CG-iteration granularity);
 *  - a scene's result is the same alone and in the mix (bit-identical).
 * A server is used from one host thread at a time. */
typedef struct fem_server_s* fem_server;

typedef struct fem_server_options {
    uint32_t precision;          /* enum fem_precision of every scene */
    uint32_t shard_max_scenes;   /* scenes per shard */
    uint64_t shard_max_tets;     /* tets per shard */
    uint64_t hbm_budget_bytes;   /* device bytes the resident scenes may hold */
    uint32_t slice_iterations;   /* CG iterations per shard launch; running steps
                                    continue in the next launch, requests that
                                    arrived meanwhile start there (0 = whole steps) */
    uint32_t chunk_nodes;        /* node chunk of the shards' node passes (as
                                    fem_batch_options.chunk_nodes; default 256: a
                                    lone request's iterations are shorter with more,
                                    smaller chunks) */
    uint32_t fuse_alpha;         /* as fem_batch_options.fuse_alpha for the shards
                                    (default 0: measured 3 % shorter iterations for a
                                    lone request against 7 % less capacity) */
    uint32_t persistent_loop;    /* as fem_batch_options.persistent_loop for the shards */
} fem_server_options;

typedef struct fem_server_completion {
    uint64_t tag;            /* as given to fem_server_submit */
    uint32_t scene;
    uint32_t status;         /* enum fem_status of the step */
    uint32_t cg_iterations;
    uint32_t fp64_resolved;  /* mixed: rotations re-solved at double precision in that step */
    double latency_us;       /* submit -> completion seen by fem_server_pump */
    double queue_us;         /* submit -> the launch that started its step */
    double device_us;        /* device time of the shard launches its step took part
                                in (shared with the other scenes of those launches) */
} fem_server_completion;

typedef struct fem_server_status {
    uint32_t resident_scenes, waiting_scenes, shards, busy_shards, max_busy_shards, pad;
    uint64_t device_bytes;      /* bytes held by the resident shards */
    uint64_t pending_requests;  /* submitted and not yet completed */
} fem_server_status;

/* Defaults: mixed precision, 2048 scenes and 3.2e7 tets per shard, 120 GiB,
 * 32 CG iterations per launch. */
int fem_server_options_default(fem_server_options* o);
int fem_server_create(const fem_server_options* opt, fem_server* out);
int fem_server_destroy(fem_server s);
/* Registers a scene (same inputs as fem_solid_create plus its position
 * constraints); it waits on the host until admitted. */
int fem_server_add_scene(fem_server s, const double* rest_xyz, uint32_t N, const uint32_t* tets, uint32_t T,
                         const fem_params* params, const double* young_per_elem, const double* poisson_per_elem,
                         const uint32_t* knc_nodes, const double* knc_targets, uint32_t knc_count,
                         uint32_t* scene);
/* Admits waiting scenes (smallest first) while the budget allows. */
int fem_server_admit(fem_server s, uint32_t* admitted);
/* Frees a scene with no request pending; a shard's memory is released when
 * its last scene goes. */
int fem_server_remove_scene(fem_server s, uint32_t scene);
/* Run-time parameter change of a scene with no request pending or in
 * flight (fem_batch_set_params on its shard when it is resident); a change
 * between QIE_V and the FIE integrators, which live in shards of different
 * kinds, needs the scene removed and added again (FEM_E_ARG). */
int fem_server_set_params(fem_server s, uint32_t scene, const fem_params* params);
int fem_server_submit(fem_server s, uint32_t scene, uint64_t tag);
/* Progress without blocking; writes up to cap completions. */
int fem_server_pump(fem_server s, fem_server_completion* out, uint32_t cap, uint32_t* n);
/* State of a resident scene (waits for its shard's step in flight); either
 * pointer may be null. */
int fem_server_get_state(fem_server s, uint32_t scene, double* x, double* v);
int fem_server_set_state(fem_server s, uint32_t scene, const double* x, const double* v);
int fem_server_get_status(fem_server s, fem_server_status* status);
/* One scene: state 0 waiting, 1 resident, 2 removed; its shard (~0u while
 * waiting); requests pending (including one in flight). */
int fem_server_scene_info(fem_server s, uint32_t scene, uint32_t* state, uint32_t* shard, uint32_t* pending);

/* --- Library --- */
const char* fem_last_error(void);
int fem_device_info(int* device, int* sm_count, int* cc_major, int* cc_minor);
/* Number of kernels this library has launched in the calling process. */
uint64_t fem_kernel_launches(void);
/* Kernel timing: while enabled, launches of the named hot kernels
 * ("elem_spmv_fp64", "node_q_fp64", ...) are bracketed by CUDA events on
 * their launching stream. fem_profile_enable(1) clears the totals;
 * fem_profile_read returns the summed event time and launch count. */
int fem_profile_enable(int on);
int fem_profile_read(const char* kernel, double* total_ms, unsigned long long* launches);
/* Index checks (a diagnostic build, no counterpart in the reference): in a
 * library compiled with -DFEM_BOUNDS_CHECK (libfemtet_gb300_bounds.so) every
 * data-dependent index the kernels read from a table -- node ids of
 * elements, node CSR entries, tile node lists and tile-local ids, partial
 * slots, constraint nodes -- is compared with its limit; a bad one is
 * counted, the first one's site (1 element node, 2 CSR entry, 3 constraint
 * node, 4 batch node, 5 tile-local node, 6 partial slot, 7 tile CSR entry),
 * index and limit are kept, and the access uses index 0 instead of faulting.
 * Reads and clears the counts of every kernel unit; *enabled is 1 in that
 * build, 0 in the normal one (where the counts are always 0). Any pointer
 * may be null. */
int fem_bounds_check_status(int* enabled, uint32_t* failures, uint32_t* site, uint32_t* index, uint32_t* limit);

/* --- Mesh ingest: TetGen .node / .ele (examples/tetgen2geo/main.cpp) --- */
/* Reads a TetGen tetrahedral mesh as the reference's converter does: the
 * first node id is the base of every id (0 or 1), positions are read as
 * float, node attributes, boundary markers and tet attributes are skipped,
 * tets with det(x1-x0, x2-x0, x3-x0) <= 0 (in float) are dropped as
 * EditableTetSolidShape3::AddTetrahedron drops them
 * (Geo/shape/TetSolidShape3.cpp:278-307), and natural_scale > 0 applies the
 * converter's "-nsac" option (center the float AABB of the nodes at the
 * origin, scale its largest extent to natural_scale). '#' comments are
 * skipped. Outputs: N*3 positions (float values as double) and T*4 base-0
 * ids in file order, ready for fem_solid_create. Call with rest and tets
 * null to get num_nodes / num_tets (after dropping) first; num_dropped may
 * be null. FEM_E_ARG for unreadable or malformed files, a dimension other
 * than 3, other than 4 nodes per tet, or short arrays; FEM_E_INDEX for an id
 * outside the .node file. Host only: needs no device. */
int fem_tetgen_read(const char* node_path, const char* ele_path, double natural_scale, double* rest,
                    uint32_t max_nodes, uint32_t* tets, uint32_t max_tets, uint32_t* num_nodes,
                    uint32_t* num_tets, uint32_t* num_dropped);

/* --- Tet-solid shapes (Geo/shape/TetSolidShape3.{h,cpp}) and shape files --- */
/* EditableTetSolidShape3::EndEdition's rebuild (TetSolidShape3.cpp:558-845)
 * of a mesh, which fixes the vertex and tet order a reference solid built
 * from the shape uses (LeafDSH_Solid3D_FEM.cpp:158-168): vertices no tet
 * uses are removed (the rest keep their order); each tet's neighbour across
 * the face opposite each of its vertices (~0u on the boundary); one
 * boundary face per unmatched face, oriented outwards (sign test in float);
 * vertex layers by distance from the boundary, tet layer = its lowest
 * vertex layer, tets reordered by layer (stable). Outputs (each may be
 * null): out_rest (num_nodes*3, the kept positions), out_tets (T*4, layer
 * order, new node ids), out_neighbors (T*4), out_tet_of (T: the input tet of
 * each output tet), out_node_of (num_nodes: the input node of each output
 * node), out_bfaces (num_bfaces*3, up to max_bfaces; at most 4 T),
 * out_layers ((first, count) pairs, up to max_layers; at most T + 1).
 * Positions are compared as float, as the reference's float shapes hold
 * them. FEM_E_INDEX for an id >= N. Host only. */
int fem_tetshape_rebuild(const double* rest, uint32_t N, const uint32_t* tets, uint32_t T, double* out_rest,
                         uint32_t* out_num_nodes, uint32_t* out_tets, uint32_t* out_neighbors, uint32_t* out_tet_of,
                         uint32_t* out_node_of, uint32_t* out_bfaces, uint32_t max_bfaces, uint32_t* out_num_bfaces,
                         uint32_t* out_layers, uint32_t max_layers, uint32_t* out_num_layers);
/* The shape file examples/tetgen2geo/main.cpp writes
 * (ShapeLibrary::Register_TetSolidShape3 + Save(path, text),
 * Geo/shape/ShapeLibrary.cpp:332-360, util/ItemStreamSerialization.cpp:14-182)
 * for a mesh: the shape after fem_tetshape_rebuild, positions as float, one
 * complex item "#1" with shape_type 21 (eShape_TetSolid3), version 3, the
 * counts and the baked arrays as hex bytes. At most 65534 nodes and tets
 * (the shape's uint16 ids): FEM_E_ARG above. Host only. */
int fem_geo_write(const char* path, const double* rest, uint32_t N, const uint32_t* tets, uint32_t T);
/* Reads the first tet-solid shape of a shape file (ShapeFactory's
 * eShape_TetSolid3 case, Geo/shape/ShapeFactory.cpp:188-201): its vertices
 * (float values as double) and tets (the shape's order, ready for
 * fem_solid_create) and neighbours (~0u = none). Call with null arrays to
 * get the counts. FEM_E_ARG for a missing or malformed file, a version other
 * than 3 or arrays that do not match the counts; FEM_E_INDEX for a vertex id
 * >= num_nodes. Host only. */
int fem_geo_read(const char* path, double* rest, uint32_t max_nodes, uint32_t* tets, uint32_t max_tets,
                 uint32_t* neighbors, uint32_t* num_nodes, uint32_t* num_tets);
/* The converter as a whole (examples/tetgen2geo/main.cpp with -nsac when
 * natural_scale > 0): fem_tetgen_read, then fem_geo_write. Host only. */
int fem_tetgen_to_geo(const char* node_path, const char* ele_path, double natural_scale, const char* geo_path);

#ifdef __cplusplus
}
#endif
#endif /* FEM_TET_H */
