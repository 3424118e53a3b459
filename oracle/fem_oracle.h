/* TEST INFRASTRUCTURE ONLY -- the oracle.
 *
 * A plain-C restatement of the reference's FP64 corotational linear-tet
 * implicit-Euler step (Saphyre2: TetrahedronElementSet3 with C_WRP + MSVD +
 * truncated differentials, ILSS_CG, LeafDSH_Solid3D_FEM::FixedStep with the
 * quasi-implicit Euler "v" integrator or the fully-implicit Euler "dx"
 * Newton integrator). Each function in fem_oracle.c cites
 * the reference file:line it follows and keeps the reference's operation
 * order, so that it reproduces the reference bit-for-bit on the same host.
 *
 * Pinning: tests compare it against the reference's own translation units
 * compiled by oracle/Makefile (oracle/_ref/libfemref*.so) on small meshes,
 * and the committed fixtures under tests/golden/ were generated from that
 * reference build.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker. The product path never does.
 *
 * Differences from the reference, all deliberate:
 *  - node and element indices are uint32 (the reference's are uint16,
 *    TetrahedronElementSet3.h:73-74), so large meshes run;
 *  - Mal's Sqrt/Sin/Cos/ATan2 evaluate through float in the reference even
 *    when Real is double (RealUtils.h:27,45,48,63). As written, that makes
 *    the FP64 rotation NaN for any F within about 1e-10 of the identity (the
 *    squared cofactor norm underflows in float), so every scene starting at
 *    rest freezes. FEM_ORC_MATH_DOUBLE (the default, and what the CUDA
 *    kernels do) evaluates the four functions in double;
 *    FEM_ORC_MATH_FLOAT_LITERAL reproduces the build as written. The
 *    reference's Sqrt(3) with an int argument (== 1, in every build) is kept
 *    in both modes.
 */
#ifndef FEM_ORACLE_H
#define FEM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { FEM_ORC_MATH_DOUBLE = 0, FEM_ORC_MATH_FLOAT_LITERAL = 1 };
/* ms::fem::Params::ERotationMethod values this oracle evaluates */
enum { FEM_ORC_ROT_MSVD = 0, FEM_ORC_ROT_DAPD = 1 };
/* ms::fem::Params::m_MM values this oracle evaluates */
enum { FEM_ORC_MAT_C_WRP = 0, FEM_ORC_MAT_C_LCM = 1, FEM_ORC_MAT_C_LCMH = 2, FEM_ORC_MAT_C_CCM = 3 };
/* LeafDSH_Solid3D_FEM::Params::m_SolverLS_Type values this oracle solves with */
enum { FEM_ORC_LS_CG = 0, FEM_ORC_LS_MINRES = 1 };
/* LeafDSH_Solid3D_FEM::Params::EIntegratorType values this oracle steps */
enum { FEM_ORC_QIE_V = 0, FEM_ORC_FIE_DX = 1, FEM_ORC_FIE_DX_QUASISTATIC = 2 };

typedef struct orc_solid orc_solid;

orc_solid* orc_solid_create(uint32_t N, const double* rest, uint32_t T, const uint32_t* tets,
                            double E, double nu, const double* E_per, const double* nu_per,
                            double density, double damping_ratio, const double* gravity,
                            double dt, double rel_eps, double abs_eps, uint32_t max_iter,
                            int math_mode);
void orc_solid_destroy(orc_solid* s);
double orc_solid_total_volume(const orc_solid* s);
double orc_solid_node_mass(const orc_solid* s);
void orc_solid_rayleigh(const orc_solid* s, double* out2);
void orc_solid_set_knc(orc_solid* s, uint32_t count, const uint32_t* nodes, const double* targets);
void orc_solid_set_solver(orc_solid* s, double rel_eps, double abs_eps, uint32_t max_iter);
void orc_solid_set_knc_targets(orc_solid* s, const double* targets);
void orc_solid_set_state(orc_solid* s, const double* x, const double* v);
void orc_solid_get_state(const orc_solid* s, double* x, double* v);
void orc_solid_fixed_step(orc_solid* s);
/* Host threads of the element loops (BeginEvaluation and the C_WRP f_e and
 * df_x scatters); 1 (the default) is the serial restatement. Results are
 * bit-identical for any count: element terms are formed in parallel and
 * applied node by node in element order. */
void orc_solid_set_threads(orc_solid* s, int threads);
/* Rotation method (FEM_ORC_ROT_*) with the DAPD degeneration threshold on
 * det F and the offset factors; resets every element's direction of collapse. */
void orc_solid_set_rotation(orc_solid* s, uint32_t method, double thr, double factor_L, double factor_NL,
                            double exponent_NL);
/* Per-element direction of collapse (vit0, vit1), T*2 bytes; (3, 0) = none. */
void orc_solid_doc(const orc_solid* s, uint8_t* doc2);
/* Material model (FEM_ORC_MAT_*); C_LCM's Lame parameters come from the
 * scalar E and nu given at creation, as the reference's element set's do. */
void orc_solid_set_material(orc_solid* s, uint32_t material);
/* C_LCMH's blend radius m_ECIE_k_factor (float32 in the reference; default 1). */
void orc_solid_set_ecie_k_factor(orc_solid* s, double k);
/* Linear solver of the step (FEM_ORC_LS_*). */
void orc_solid_set_ls_solver(orc_solid* s, uint32_t ls_solver);
/* Integrator (FEM_ORC_*), Newton iteration cap and |b_k| epsilon (FIE only). */
void orc_solid_set_integrator(orc_solid* s, uint32_t integrator, uint32_t nr_max_iter, double nr_abs_eps);
/* Newton iterations, |last| / |b_0| and |last| of the last FIE step (0 for QIE). */
void orc_solid_last_nr_stats(const orc_solid* s, uint32_t* nr_iters, double* nr_rel, double* nr_abs);
void orc_solid_last_stats(const orc_solid* s, uint32_t* iters, double* rel_res, double* abs_res,
                          double* elastic_energy, double* potential_energy);

/* The multi-solid Newton lock-step phases (LeafDSH_Solid3D_FEM.cpp:
 * 2824-3039) and the aggregate's loop of one fixed step over them
 * (SS_AggregateDSH_Basic.cpp:229-300, contacts left out). */
void orc_solid_nr_init(orc_solid* s, double dt);
void orc_solid_nr_prestep(orc_solid* s, double dt);
void orc_solid_nr_midstep(orc_solid* s, double dt);
void orc_solid_nr_poststep(orc_solid* s, double dt);
void orc_solid_nr_end(orc_solid* s, double dt);
void orc_multi_lock_step(orc_solid** solids, uint32_t count, double dt);
/* Iterations since the last NR_PreStep and LS iterations of its NR_MidStep. */
void orc_solid_last_lock_stats(const orc_solid* s, uint32_t* nr_k, uint32_t* ls_iters);

/* Element-level hooks (state: the positions given to begin_eval). */
void orc_solid_begin_eval(orc_solid* s, const double* x);
void orc_solid_rotations(const orc_solid* s, double* R_out);   /* T*9 row-major */
void orc_solid_detF(const orc_solid* s, double* detF_out);     /* T */
void orc_solid_f_e(const orc_solid* s, double* f);             /* f += f_e */
void orc_solid_df_x(const orc_solid* s, const double* dx, double* df); /* df += df_x(dx) */
double orc_solid_V(const orc_solid* s);
/* q = A d (LS_A_times_d) for the given factors, then the KNC projection. */
void orc_solid_apply_A(const orc_solid* s, double factor_M, double factor_K, const double* d, double* q);

/* The reference MSVD rotation of one F (row-major). */
void orc_rotation_svd(const double* F, double* R, int math_mode);

/* The per-element stiffness blocks K_ij (16 row-major 3x3, element e). */
void orc_solid_element_K(const orc_solid* s, uint32_t e, double* K144);

#ifdef __cplusplus
}
#endif
#endif
