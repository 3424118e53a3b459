/* Test infrastructure: the reference's own FP64 CPU implementation of the
 * corotational linear-tet implicit-Euler step, exposed through a small C ABI
 * so that tests can pin the oracle restatement (fem_oracle.c) against it.
 *
 * Only tests/ and bench.py's CPU-baseline leg load this library, and only as
 * a checker. It is built by oracle/Makefile from the reference sources where
 * they lie (TetrahedronElementSet3.cpp, Rotation.cpp) plus the header-only
 * solver (ILSS_CG.h); nothing of the reference is copied.
 *
 * What runs here is the reference's code:
 *   EditableTetrahedronElementSet3::BeginEdition/AddElement/EndEdition
 *       (src/Saphyre2/ms/fem/TetrahedronElementSet3.cpp:2084-2166)
 *   TetrahedronElementSet3::CreateCache/BeginEvaluation/f_e/df_x/V
 *       (TetrahedronElementSet3.cpp:190-281,291-377,1053-1096,1456-1488,1761-1836)
 *   ns::ILSS_CG::Solve (src/Saphyre2/ns/ILSS_CG.h:38-151)
 * What is restated (the Leaf does not compile with Real=double, see the
 * survey of the reference): the per-step driver of
 *   LeafDSH_Solid3D_FEM::FixedStep            (LeafDSH_Solid3D_FEM.cpp:898-990)
 *   LeafDSH_Solid3D_FEM::Step_QuasiImplicitEuler_v (:1205-1328)
 *   LeafDSH_Solid3D_FEM::LS_A_times_d / LS_ZeroKNC (:1045-1079)
 *   LeafDSH_Solid3D_FEM::RebuildMass          (:1591-1611)
 *   Params::RebuildRayleighCoeffsFromFreqs    (LeafDSH_Solid3D_FEM.h:347-354)
 * with contacts, air drag and the test modes at their defaults (off).
 *
 * Per-element materials: the reference bakes one (E, nu) per element set.
 * RebakePerElement re-runs the reference's own TetrahedronElement3::Compute_K
 * (TetrahedronElement3.h:157-173) per element and writes the 16 blocks the
 * same way EndEdition does (TetrahedronElementSet3.cpp:2136-2156).
 *
 * Index width: element_index_type/node_index_type are uint16 in the
 * reference (TetrahedronElementSet3.h:73-74), so meshes are limited to
 * 65535 nodes and elements here; ref_tes_create rejects larger ones.
 */
#include <Saphyre2/ms/fem/TetrahedronElementSet3.h>
#include <Saphyre2/ms/fem/TetrahedronElement3.h>
#include <Saphyre2/ms/fem/Rotation.h>
#include <Saphyre2/ns/ILSS_CG.h>
#include <Saphyre2/ns/ILSS_MINRES.h>
#include <vector>
#include <cstdint>
#include <cstring>

using namespace S2;

namespace {

typedef ms::fem::TetrahedronElementSet3 TES3;

class PerElementTES : public ms::fem::EditableTetrahedronElementSet3
{
public:
    // ms::fem::Params::m_RM and the DAPD parameters (Params.h:27-29,63-67),
    // set in place so that per-element materials stay baked.
    // ms::fem::Params::m_MM (Params.h:48-62): 0 C_WRP, 1 C_LCM, 2 C_LCMH, 3 C_CCM
    void SetMaterial(unsigned mm)
    {
        static const ms::fem::Params::EMaterialMethod kMM[4] = {ms::fem::Params::eMM_C_WRP, ms::fem::Params::eMM_C_LCM,
                                                                ms::fem::Params::eMM_C_LCMH, ms::fem::Params::eMM_C_CCM};
        m_Params.m_MM = kMM[mm < 4 ? mm : 0];
    }
    // ms::fem::Params::m_ECIE_k_factor (Params.h:30,89), C_LCMH's blend radius
    void SetEcieK(double k) { m_Params.m_ECIE_k_factor = float32(k); }
    void SetRotation(unsigned method, double thr, double factor_L, double factor_NL, double exponent_NL)
    {
        m_Params.m_RM = method ? ms::fem::Params::eRM_DAPD : ms::fem::Params::eRM_MSVD;
        m_Params.m_DegenerateThresholdDetF = Real(thr);
        m_Params.m_DAPD_L_Factor = float32(factor_L);
        m_Params.m_DAPD_NL_Factor = float32(factor_NL);
        m_Params.m_DAPD_NL_Exponent = float32(exponent_NL);
    }

    void RebakePerElement(const double* E, const double* nu)
    {
        TES3::LinearED* led = const_cast<TES3::LinearED*>(m_vecLED);
        for (unsigned e = 0; e < m_NumElements; e++) {
            const TES3::ElementData& ed = m_vecED[e];
            Mat12x12 K;
            ms::fem::TetrahedronElement3::Compute_K(m_vecRefPos[ed.m_vecNID[0]], m_vecRefPos[ed.m_vecNID[1]],
                                                    m_vecRefPos[ed.m_vecNID[2]], m_vecRefPos[ed.m_vecNID[3]],
                                                    Real(E[e]), Real(nu[e]), K);
            Mat3x3* blocks[4][4] = {
                {&led[e].m_K00, &led[e].m_K01, &led[e].m_K02, &led[e].m_K03},
                {&led[e].m_K10, &led[e].m_K11, &led[e].m_K12, &led[e].m_K13},
                {&led[e].m_K20, &led[e].m_K21, &led[e].m_K22, &led[e].m_K23},
                {&led[e].m_K30, &led[e].m_K31, &led[e].m_K32, &led[e].m_K33}};
            for (int bi = 0; bi < 4; bi++)
                for (int bj = 0; bj < 4; bj++)
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            (*blocks[bi][bj])(i, j) = K(3 * bi + i, 3 * bj + j);
        }
    }
};

struct RefKNC {
    unsigned nid;
    Vec3 pos, vel;
    bool is_position;
};

} // namespace

struct ref_tes {
    PerElementTES tes;
    ms::IForce3::ICache* cache;
    std::vector<Vec3> x, prev_x, v;
    std::vector<Real> inv_mass;
    unsigned N, T;
};

struct ref_solid {
    ref_tes* t;
    std::vector<RefKNC> knc;
    Real density, dt, rel_eps, abs_eps;
    unsigned max_iter;
    Vec3 gravity;
    Real rayleigh[2];
    Real total_time;
    Real elastic_energy, potential_energy;
    std::vector<Vec3> b, y;
    ns::ILSS_CG cg;
    ns::ILSS_MINRES minres;
    unsigned ls_solver;  // 0 CG, 1 MINRES (Params::m_SolverLS_Type)
    Real factor_M, factor_K;
    unsigned last_iters;
    Real last_rel, last_abs;
    // fully-implicit Euler (LeafDSH_Solid3D_FEM.h:110,233-241)
    unsigned integrator, nr_max_iter;
    Real nr_abs_eps;
    std::vector<Vec3> xk, vk;  // m_IE_vec_x_k, m_IE_vec_v_k
    unsigned nr_iters;
    Real nr_rel, nr_abs;
    // multi-solid Newton lock-step: m_NR_nr_k and the LS iterations since the
    // last NR_PreStep (m_Stats.m_SolverLS_NumIter)
    unsigned lock_nr_k = 0, lock_ls_iters = 0;
};

static Vec3 V3(const double* p) { return Vec3(Real(p[0]), Real(p[1]), Real(p[2])); }

extern "C" {

int ref_real_size(void) { return (int)sizeof(Real); }

/* Element set over N nodes / T tets; E_per/nu_per may be null (then the
 * scalar E, nu hold for all elements, as in the reference). */
ref_tes* ref_tes_create(unsigned N, const double* rest, unsigned T, const uint32_t* tets,
                        double E, double nu, const double* E_per, const double* nu_per)
{
    if (N > 65535u || T > 65535u || N == 0 || T == 0) return 0;
    ref_tes* h = new ref_tes;
    h->N = N; h->T = T;
    std::vector<Vec3> r(N);
    for (unsigned i = 0; i < N; i++) r[i] = V3(rest + 3 * i);
    ms::fem::Params p; // defaults: C_WRP, MSVD, Truncated (Params.h:74-98)
    p.m_YoungModulus = Real(E);
    p.m_PoissonRatio = Real(nu);
    h->tes.BeginEdition(N, &r[0], T, p);
    for (unsigned e = 0; e < T; e++)
        h->tes.AddElement(tets[4 * e], tets[4 * e + 1], tets[4 * e + 2], tets[4 * e + 3]);
    h->tes.EndEdition();
    if (E_per && nu_per) h->tes.RebakePerElement(E_per, nu_per);
    h->x = r; h->prev_x = r;
    h->v.assign(N, Vec3::Zero());
    h->inv_mass.assign(N, Real(1));
    h->cache = h->tes.CreateCache(&h->inv_mass[0]);
    return h;
}

void ref_tes_destroy(ref_tes* h)
{
    if (!h) return;
    h->tes.DestroyCache(h->cache);
    delete h;
}

double ref_tes_total_volume(ref_tes* h) { return h->tes.TotalVolume(); }

/* BeginEvaluation at positions x (N*3). ref_tes_rotations then reads the
 * per-element rotation R (row-major 3x3, T*9) through the element-to-world
 * transform, whose rotation part is the cached R under C_WRP
 * (TetrahedronElementSet3.cpp:426-441). */
void ref_tes_begin_eval(ref_tes* h, const double* x)
{
    for (unsigned i = 0; i < h->N; i++) h->x[i] = V3(x + 3 * i);
    h->tes.BeginEvaluation(h->cache, &h->prev_x[0], &h->x[0], &h->v[0], Real(0));
}

void ref_tes_rotations(ref_tes* h, double* R_out)
{
    for (unsigned e = 0; e < h->T; e++) {
        Transform3 tr = h->tes.GetTransformE2W(h->cache, e, &h->x[0]);
        const Mat3x3& R = tr.m_Rot;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) R_out[9 * e + 3 * i + j] = R(i, j);
    }
}

/* f += f_e(x) at the last begin_eval positions (accumulating, as IForce3). */
void ref_tes_f_e(ref_tes* h, double* f)
{
    std::vector<Vec3> acc(h->N);
    for (unsigned i = 0; i < h->N; i++) acc[i] = V3(f + 3 * i);
    h->tes.f_e(h->cache, &acc[0]);
    for (unsigned i = 0; i < h->N; i++)
        for (int c = 0; c < 3; c++) f[3 * i + c] = acc[i][c];
}

/* df += df_x(dx) = -R K0 R^T dx, accumulating. */
void ref_tes_df_x(ref_tes* h, const double* dx, double* df)
{
    std::vector<Vec3> d(h->N), acc(h->N);
    for (unsigned i = 0; i < h->N; i++) { d[i] = V3(dx + 3 * i); acc[i] = V3(df + 3 * i); }
    h->tes.df_x(h->cache, &d[0], &acc[0]);
    for (unsigned i = 0; i < h->N; i++)
        for (int c = 0; c < 3; c++) df[3 * i + c] = acc[i][c];
}

double ref_tes_V(ref_tes* h) { return h->tes.V(h->cache); }

/* The reference rotation of one deformation gradient (Rotation.cpp:39-57). */
void ref_rotation_svd(const double* F_in, double* R_out)
{
    Mat3x3 F;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) F(i, j) = Real(F_in[3 * i + j]);
    Mat3x3 R = ms::fem::Compute_R_SVD(F, mal::Det(F), Real(0.1f));
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) R_out[3 * i + j] = R(i, j);
}

/* Solid with the Leaf's state: uniform node mass from RebuildMass, Rayleigh
 * coefficients from the damping ratio, position KNCs with zero velocity. */
ref_solid* ref_solid_create(unsigned N, const double* rest, unsigned T, const uint32_t* tets,
                            double E, double nu, const double* E_per, const double* nu_per,
                            double density, double damping_ratio, const double* gravity,
                            double dt, double rel_eps, double abs_eps, unsigned max_iter)
{
    ref_tes* t = ref_tes_create(N, rest, T, tets, E, nu, E_per, nu_per);
    if (!t) return 0;
    ref_solid* s = new ref_solid;
    s->t = t;
    s->density = Real(density);
    s->dt = Real(dt);
    s->rel_eps = Real(rel_eps);
    s->abs_eps = Real(abs_eps);
    s->max_iter = max_iter;
    s->gravity = V3(gravity);
    s->total_time = 0;
    s->elastic_energy = s->potential_energy = 0;
    s->b.assign(N, Vec3::Zero());
    s->y.assign(N, Vec3::Zero());
    s->cg.Init(3 * N);
    s->minres.Init(3 * N);
    s->ls_solver = 0;
    s->last_iters = 0; s->last_rel = s->last_abs = 0;
    s->integrator = 0; s->nr_max_iter = 3; s->nr_abs_eps = Real(1e-6);
    s->xk.assign(N, Vec3::Zero());
    s->vk.assign(N, Vec3::Zero());
    s->nr_iters = 0; s->nr_rel = s->nr_abs = 0;
    // GParticleSystem::SetDscr(N, 666) then LeafDSH_Solid3D_FEM::RebuildMass
    // (ParticleSystem.h:46-58,80,154-159; LeafDSH_Solid3D_FEM.cpp:1591-1611)
    Real total_mass = s->density * t->tes.TotalVolume();
    Real mass_per_node = total_mass / N;
    for (unsigned i = 0; i < N; i++) t->inv_mass[i] = Real(1.0f) / mass_per_node;
    // Params::RebuildRayleighCoeffsFromFreqs (LeafDSH_Solid3D_FEM.h:347-354)
    // with ms::fem::Params' default frequencies (Params.h:79)
    ms::fem::Params fp;
    Mat2x2 Omega;
    Omega(0, 0) = mal::Rcp(fp.m_RayleighFreq1); Omega(0, 1) = fp.m_RayleighFreq1;
    Omega(1, 0) = mal::Rcp(fp.m_RayleighFreq2); Omega(1, 1) = fp.m_RayleighFreq2;
    const Real zr = Real(damping_ratio);
    Vec2 zeta(zr, zr);
    Vec2 coeff = mal::Inverse(Omega) * (2 * zeta);
    s->rayleigh[0] = coeff[0];
    s->rayleigh[1] = coeff[1];
    return s;
}

void ref_solid_destroy(ref_solid* s)
{
    if (!s) return;
    ref_tes_destroy(s->t);
    delete s;
}

void ref_solid_rayleigh(ref_solid* s, double* out) { out[0] = s->rayleigh[0]; out[1] = s->rayleigh[1]; }
double ref_solid_node_mass(ref_solid* s) { return Real(1) / s->t->inv_mass[0]; }

/* KinematicNodeConstraintSet3::AddKNC (KinematicNodeConstraintSet3.h:32-40):
 * position constraints at the given targets, zero velocity. */
void ref_solid_set_knc(ref_solid* s, unsigned count, const uint32_t* nodes, const double* targets)
{
    s->knc.resize(count);
    for (unsigned k = 0; k < count; k++) {
        s->knc[k].nid = nodes[k];
        s->knc[k].pos = V3(targets + 3 * k);
        s->knc[k].vel = Vec3::Zero();
        s->knc[k].is_position = true;
    }
}

/* KinematicNodeConstraintSet3::SetPosKNC for every constraint. */
void ref_solid_set_knc_targets(ref_solid* s, const double* targets)
{
    for (size_t k = 0; k < s->knc.size(); k++) {
        s->knc[k].pos = V3(targets + 3 * k);
        s->knc[k].is_position = true;
    }
}

void ref_solid_set_state(ref_solid* s, const double* x, const double* v)
{
    for (unsigned i = 0; i < s->t->N; i++) {
        if (x) { s->t->x[i] = V3(x + 3 * i); s->t->prev_x[i] = s->t->x[i]; }
        if (v) s->t->v[i] = V3(v + 3 * i);
    }
}

void ref_solid_get_state(ref_solid* s, double* x, double* v)
{
    for (unsigned i = 0; i < s->t->N; i++)
        for (int c = 0; c < 3; c++) {
            if (x) x[3 * i + c] = s->t->x[i][c];
            if (v) v[3 * i + c] = s->t->v[i][c];
        }
}

static void zero_knc(const ref_solid* s, Vec3* v)
{
    for (size_t k = 0; k < s->knc.size(); k++) v[s->knc[k].nid] = Vec3::Zero();
}

static void a_times_d(const ref_solid* s, Real* q, const Real* d)
{
    const unsigned n3 = 3 * s->t->N;
    ns::real_array::zero(q, n3);
    s->t->tes.df_x(s->t->cache, reinterpret_cast<const Vec3*>(d), reinterpret_cast<Vec3*>(q));
    ns::real_array::muleq(q, -s->factor_K, n3);
    for (unsigned i = 0; i < s->t->N; i++) {
        Real factor((Real(1) / s->t->inv_mass[i]) * s->factor_M);
        q[3 * i] += factor * d[3 * i];
        q[3 * i + 1] += factor * d[3 * i + 1];
        q[3 * i + 2] += factor * d[3 * i + 2];
    }
}

static void finish_step(ref_solid* s);

/* LS_Solve (LeafDSH_Solid3D_FEM.cpp:1081-1154): the chosen solver's Solve
 * with the Leaf's A*v and constraint delegates. */
static void ls_solve(ref_solid* s)
{
    ns::IIterativeLinearSystemSolver* ls = s->ls_solver ? static_cast<ns::IIterativeLinearSystemSolver*>(&s->minres)
                                                       : static_cast<ns::IIterativeLinearSystemSolver*>(&s->cg);
    ls->Solve([s](Real* Av, const Real* v) { a_times_d(s, Av, v); },
              [s](Real* v) { zero_knc(s, reinterpret_cast<Vec3*>(v)); },
              reinterpret_cast<Real*>(&s->y[0]), reinterpret_cast<const Real*>(&s->b[0]),
              s->rel_eps, s->abs_eps, s->max_iter);
    s->last_iters = ls->GetNumIterations();
    s->last_rel = ls->GetRelResidual();
    s->last_abs = ls->GetAbsResidual();
}

/* Restated Step_FullyImplicitEuler_dx (LeafDSH_Solid3D_FEM.cpp:1357-1552)
 * around the reference's element set and CG: contacts off, warm start on,
 * CG solver. h = 0 is the quasi-static variant (:958-959). */
static void step_fie(ref_solid* s, Real h)
{
    ref_tes* t = s->t;
    const unsigned N = t->N;
    const unsigned cN = 3 * N;
    Real inv_dt(h == 0 ? 0 : mal::Rcp(h));
    for (unsigned i = 0; i < N; i++) { s->xk[i] = t->x[i]; s->vk[i] = t->v[i]; }
    unsigned nr_k = 0, ls_iters = 0;
    Real nr_delta_new(0), nr_delta_0(-1);
    bool converged1 = false;
    s->last_iters = 0; s->last_rel = s->last_abs = 0;
    do {
        for (unsigned i = 0; i < N; i++) s->b[i] = Vec3::Zero();
        for (unsigned i = 0; i < N; i++) s->b[i] += (Real(1) / t->inv_mass[i]) * s->gravity;
        t->tes.f_e(t->cache, &s->b[0]);
        t->tes.f_p(t->cache, &s->b[0]);
        for (unsigned i = 0; i < N; i++)
            s->b[i] += inv_dt * (Real(1) / t->inv_mass[i]) * (t->v[i] - inv_dt * (s->xk[i] - t->x[i]));
        if (nr_k == 0) for (unsigned i = 0; i < N; i++) s->y[i] = h * t->v[i];
        else for (unsigned i = 0; i < N; i++) s->y[i] = Vec3::Zero();
        for (size_t k = 0; k < s->knc.size(); k++) {
            RefKNC& c = s->knc[k];
            if (c.is_position) {
                Vec3 vk((c.pos - t->x[c.nid]) * inv_dt);
                Real norm_vk(vk.Norm());
                if (norm_vk > Real(0.001f))
                    c.vel = mal::Min(norm_vk, Real(50.0f)) * vk.Normalized();
                else
                    c.vel = Vec3::Zero();
            }
            s->b[c.nid] = c.pos - s->xk[c.nid];
            s->y[c.nid] = c.pos - s->xk[c.nid];
        }
        nr_delta_new = ns::real_array::norm_2(reinterpret_cast<const Real*>(&s->b[0]), cN);
        if (nr_delta_0 < 0) nr_delta_0 = nr_delta_new;
        converged1 = nr_delta_new < s->nr_abs_eps;
        if (!converged1) {
            s->factor_M = mal::Sq(inv_dt) + inv_dt * s->rayleigh[0];
            s->factor_K = Real(1) + inv_dt * s->rayleigh[1];
            ls_solve(s);
            ls_iters += s->last_iters;
            ns::real_array::addeq(reinterpret_cast<Real*>(&s->xk[0]), reinterpret_cast<const Real*>(&s->y[0]), cN);
            for (unsigned i = 0; i < N; i++) s->vk[i] = inv_dt * (s->xk[i] - t->x[i]);
            nr_delta_new = ns::real_array::norm_2(reinterpret_cast<const Real*>(&s->y[0]), cN);
            if (nr_delta_0 < 0) nr_delta_0 = nr_delta_new;
            nr_k++;
            t->tes.EndEvaluation(t->cache);
            t->tes.BeginEvaluation(t->cache, &t->x[0], &s->xk[0], &s->vk[0], s->total_time);
        }
    } while (!converged1 && nr_k < s->nr_max_iter);
    s->nr_iters = nr_k;
    s->nr_rel = (nr_delta_0 > 0) ? nr_delta_new / nr_delta_0 : 0;
    s->nr_abs = nr_delta_new;
    s->last_iters = ls_iters;
    for (unsigned i = 0; i < N; i++) { t->x[i] = s->xk[i]; t->v[i] = s->vk[i]; }
}

/* Rotation method (0 MSVD, 1 DAPD) and DAPD parameters; call before the
 * first step (the caches' directions of collapse start invalid). */
void ref_tes_set_rotation(ref_tes* h, unsigned method, double thr, double factor_L, double factor_NL,
                          double exponent_NL)
{
    h->tes.SetRotation(method, thr, factor_L, factor_NL, exponent_NL);
}

void ref_solid_set_rotation(ref_solid* s, unsigned method, double thr, double factor_L, double factor_NL,
                            double exponent_NL)
{
    ref_tes_set_rotation(s->t, method, thr, factor_L, factor_NL, exponent_NL);
}

void ref_solid_set_ls_solver(ref_solid* s, unsigned ls_solver) { s->ls_solver = ls_solver; }

void ref_solid_set_material(ref_solid* s, unsigned material) { s->t->tes.SetMaterial(material); }
void ref_solid_set_ecie_k_factor(ref_solid* s, double k) { s->t->tes.SetEcieK(k); }

void ref_solid_set_integrator(ref_solid* s, unsigned integrator, unsigned nr_max_iter, double nr_abs_eps)
{
    s->integrator = integrator;
    s->nr_max_iter = nr_max_iter;
    s->nr_abs_eps = Real(nr_abs_eps);
}

void ref_solid_last_nr_stats(ref_solid* s, unsigned* nr_iters, double* nr_rel, double* nr_abs)
{
    const bool fie = s->integrator != 0;
    if (nr_iters) *nr_iters = fie ? s->nr_iters : 0;
    if (nr_rel) *nr_rel = fie ? s->nr_rel : 0;
    if (nr_abs) *nr_abs = fie ? s->nr_abs : 0;
}

/* One FixedStep(dt) of the Leaf with the QIE-v integrator, or with the FIE-dx
 * integrators (1: dt, 2: quasi-static). */
void ref_solid_fixed_step(ref_solid* s)
{
    ref_tes* t = s->t;
    const unsigned N = t->N;
    const Real dt = s->dt;
    t->tes.BeginEvaluation(t->cache, &t->prev_x[0], &t->x[0], &t->v[0], s->total_time);
    for (unsigned i = 0; i < N; i++) t->prev_x[i] = t->x[i];
    if (s->integrator != 0) {
        step_fie(s, s->integrator == 2 ? Real(0) : dt);
        finish_step(s);
        return;
    }
    // Step_QuasiImplicitEuler_v
    Real inv_dt(mal::Rcp(dt));
    for (unsigned i = 0; i < N; i++) s->b[i] = Vec3::Zero();
    for (unsigned i = 0; i < N; i++) s->b[i] += (Real(1) / t->inv_mass[i]) * s->gravity;
    t->tes.f_e(t->cache, &s->b[0]);
    for (unsigned i = 0; i < N; i++) s->b[i] *= dt;
    for (unsigned i = 0; i < N; i++) s->b[i] += (Real(1) / t->inv_mass[i]) * t->v[i];
    for (unsigned i = 0; i < N; i++) s->y[i] = t->v[i];
    for (size_t k = 0; k < s->knc.size(); k++) {
        RefKNC& c = s->knc[k];
        if (c.is_position) {
            Vec3 vk((c.pos - t->x[c.nid]) * inv_dt);
            Real norm_vk(vk.Norm());
            if (norm_vk > Real(0.001f))
                c.vel = mal::Min(norm_vk, Real(50.0f)) * vk.Normalized();
            else
                c.vel = Vec3::Zero();
        }
        s->b[c.nid] = c.vel;
        s->y[c.nid] = c.vel;
    }
    s->factor_M = Real(1) + dt * s->rayleigh[0];
    s->factor_K = mal::Sq(dt) + dt * s->rayleigh[1];
    ls_solve(s);
    for (unsigned i = 0; i < N; i++) {
        t->v[i] = s->y[i];
        t->x[i] = t->x[i] + dt * s->y[i];
    }
    finish_step(s);
}

/* The end of FixedStep after integration (LeafDSH_Solid3D_FEM.cpp:978-989):
 * elastic energy, EndEvaluation, RecomputeEnergy's potential term. */
// RecomputeEnergy (LeafDSH_Solid3D_FEM.cpp:1554-1584): potential part
static Real potential(ref_solid* s)
{
    ref_tes* t = s->t;
    Real pe(0);
    for (unsigned e = 0; e < t->T; e++) {
        unsigned nid[4];
        t->tes.GetNID(e, nid[0], nid[1], nid[2], nid[3]);
        Real element_mass(s->density * t->tes.Volume(e));
        pe += (element_mass / Real(4)) *
            mal::Dot(t->x[nid[0]] + t->x[nid[1]] + t->x[nid[2]] + t->x[nid[3]], -s->gravity);
    }
    return pe;
}

static void finish_step(ref_solid* s)
{
    ref_tes* t = s->t;
    const Real dt = s->dt;
    s->elastic_energy = t->tes.V(t->cache);
    t->tes.EndEvaluation(t->cache);
    s->potential_energy = potential(s);
    s->total_time += dt;
}

/* The multi-solid Newton lock-step phases, restated from
 * LeafDSH_Solid3D_FEM::NR_Init / NR_PreStep / NR_MidStep / NR_PostStep /
 * NR_End (LeafDSH_Solid3D_FEM.cpp:2824-3039) around the reference's element
 * set and solvers, contacts off, warm start on, default kinematic mode
 * (UpdateKNC a no-op). The element set's cache keeps the position array of
 * its last BeginEvaluation: after NR_PostStep that is xk, which the next
 * NR_PreStep resets to x. */
void ref_solid_nr_init(ref_solid* s, double)
{
    ref_tes* t = s->t;
    t->tes.BeginEvaluation(t->cache, &t->prev_x[0], &t->x[0], &t->v[0], s->total_time);
    for (unsigned i = 0; i < t->N; i++) t->prev_x[i] = t->x[i];
}

void ref_solid_nr_prestep(ref_solid* s, double)
{
    ref_tes* t = s->t;
    for (unsigned i = 0; i < t->N; i++) {
        s->xk[i] = t->x[i];
        s->vk[i] = t->v[i];
    }
    s->lock_nr_k = 0;
    s->lock_ls_iters = 0;
}

void ref_solid_nr_midstep(ref_solid* s, double dt_in)
{
    ref_tes* t = s->t;
    const unsigned N = t->N;
    const Real dt(dt_in);
    const Real inv_dt(dt == 0 ? 0 : mal::Rcp(dt));
    for (unsigned i = 0; i < N; i++) s->b[i] = Vec3::Zero();
    for (unsigned i = 0; i < N; i++) s->b[i] += (Real(1) / t->inv_mass[i]) * s->gravity;
    t->tes.f_e(t->cache, &s->b[0]);
    t->tes.f_p(t->cache, &s->b[0]);
    for (unsigned i = 0; i < N; i++)
        s->b[i] += inv_dt * (Real(1) / t->inv_mass[i]) * (t->v[i] - inv_dt * (s->xk[i] - t->x[i]));
    if (s->lock_nr_k == 0) for (unsigned i = 0; i < N; i++) s->y[i] = dt * t->v[i];
    else for (unsigned i = 0; i < N; i++) s->y[i] = Vec3::Zero();
    for (size_t k = 0; k < s->knc.size(); k++) {
        RefKNC& c = s->knc[k];
        if (c.is_position) {
            Vec3 vk((c.pos - t->x[c.nid]) * inv_dt);
            Real norm_vk(vk.Norm());
            if (norm_vk > Real(0.001f))
                c.vel = mal::Min(norm_vk, Real(50.0f)) * vk.Normalized();
            else
                c.vel = Vec3::Zero();
        }
        s->b[c.nid] = c.pos - s->xk[c.nid];
        s->y[c.nid] = c.pos - s->xk[c.nid];
    }
    s->factor_M = mal::Sq(inv_dt) + inv_dt * s->rayleigh[0];
    s->factor_K = Real(1) + inv_dt * s->rayleigh[1];
    ls_solve(s);
    s->lock_ls_iters += s->last_iters;
}

void ref_solid_nr_poststep(ref_solid* s, double dt_in)
{
    ref_tes* t = s->t;
    const Real dt(dt_in);
    const Real inv_dt(dt == 0 ? 0 : mal::Rcp(dt));
    ns::real_array::addeq(reinterpret_cast<Real*>(&s->xk[0]), reinterpret_cast<const Real*>(&s->y[0]), 3 * t->N);
    for (unsigned i = 0; i < t->N; i++) s->vk[i] = inv_dt * (s->xk[i] - t->x[i]);
    s->lock_nr_k++;
    t->tes.EndEvaluation(t->cache);
    t->tes.BeginEvaluation(t->cache, &t->x[0], &s->xk[0], &s->vk[0], s->total_time);
}

void ref_solid_nr_end(ref_solid* s, double)
{
    ref_tes* t = s->t;
    for (unsigned i = 0; i < t->N; i++) {
        t->x[i] = s->xk[i];
        t->v[i] = s->vk[i];
    }
    t->tes.EndEvaluation(t->cache);
    // RecomputeEnergy (LeafDSH_Solid3D_FEM.cpp:1554-1584): the potential
    // term; NR_End does not evaluate V, so the elastic energy keeps its value
    s->potential_energy = potential(s);
}

/* SS_AggregateDSH_Basic::MultiDSH_Solid3D_Update's body for one fixed step
 * (SS_AggregateDSH_Basic.cpp:229-300), contacts off. */
void ref_multi_lock_step(ref_solid** solids, unsigned count, double dt)
{
    unsigned max_nr_iter = 0;
    for (unsigned i = 0; i < count; i++) max_nr_iter = std::max(max_nr_iter, solids[i]->nr_max_iter);
    for (unsigned i = 0; i < count; i++) ref_solid_nr_init(solids[i], dt);
    unsigned nr_iter = 0;
    do {
        for (unsigned i = 0; i < count; i++) {
            ref_solid_nr_prestep(solids[i], dt);
            ref_solid_nr_midstep(solids[i], dt);
        }
        for (unsigned i = 0; i < count; i++) ref_solid_nr_poststep(solids[i], dt);
    } while (++nr_iter < max_nr_iter);
    for (unsigned i = 0; i < count; i++) ref_solid_nr_end(solids[i], dt);
}

void ref_solid_last_lock_stats(ref_solid* s, unsigned* nr_k, unsigned* ls_iters)
{
    *nr_k = s->lock_nr_k;
    *ls_iters = s->lock_ls_iters;
}

void ref_solid_last_stats(ref_solid* s, unsigned* iters, double* rel_res, double* abs_res,
                          double* elastic_energy, double* potential_energy)
{
    if (iters) *iters = s->last_iters;
    if (rel_res) *rel_res = s->last_rel;
    if (abs_res) *abs_res = s->last_abs;
    if (elastic_energy) *elastic_energy = s->elastic_energy;
    if (potential_energy) *potential_energy = s->potential_energy;
}

} // extern "C"
