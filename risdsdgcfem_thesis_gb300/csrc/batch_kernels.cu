// batch_kernels.cu -- kernels of the tiled, batched step (FP64 and mixed).
//
// One CG iteration (Saphyre2 ns/ILSS_CG.h:90-144) over every mesh whose loop
// is still running, in lock-step, is three kernels on the FP64 path (the
// mixed path runs its iteration as four kernels, tile_pipe.cu):
//   k_tile_spmv   one CTA per element tile: the tile's node values of the
//                 search direction d = S(r + beta d) are formed while staging
//                 r and d in shared memory, each thread forms one element's
//                 R K0 R^T d (elem_math.cuh), the 12 outputs go to shared
//                 memory, and each local node sums its entries in element
//                 order (tile-local CSR) into one partial per (tile, node).
//   k_node_q      per node: the same d (written back), q = S(fK sum(partials)
//                 + m fM d), FP64 d.q partials per node chunk; the last block
//                 of each mesh sums its partials in a fixed order and forms
//                 alpha (or stops the mesh on breakdown, ILSS_CG.h:97). On
//                 refresh iterations (mixed) also the true residual b - A y
//                 from the product of k_tile_spmv_y64 (double-float
//                 arithmetic, FP64 partial sums).
//   k_node_update y += alpha d (FP64), r -= alpha q, FP64 |r|^2 partials; the
//                 last block of each mesh forms beta and the mesh's loop test,
//                 and the last block of the grid sets the CUDA-graph while
//                 condition (any mesh still iterating) and the refresh flag.
// "Last block" uses per-mesh and per-grid arrival counters after a
// __threadfence (no waiting); the sums it forms do not depend on which block
// arrives last.
// The once-per-step kernels (elastic force, right-hand side, constraints,
// initial residual, integration, energies) follow
// Step_QuasiImplicitEuler_v (LeafDSH_Solid3D_FEM.cpp:1205-1328).
#include "active_list.cuh"
#include "batch.cuh"
#include "batch_launch.h"
#include "bounds.cuh"
#include "df.cuh"
#include "elem_math.cuh"
#include "msvd.cuh"
#include "lcm.cuh"
#include "refresh_product.cuh"

namespace femgb {

__device__ __forceinline__ double bwarp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double bblock_sum(double v)
{
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = bwarp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) v = bwarp_sum(v);
    return v;
}

// Block sum of one FP32 value per thread, for the FP64 reductions of the mixed
// path: within a warp the values are added as an unevaluated sum of two
// floats (Knuth's two-sum keeps each rounding error), which carries about
// 48 bits, then each warp's (hi, lo) is converted to double and the warps
// are added in FP64. The FP64 pipe of GB300 runs at a small fraction of the
// FP32 rate, so FP64 work per node is avoided; the tree is fixed, so the
// result does not depend on scheduling. Result valid in thread 0.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ double bblock_sum_f(float v)
{
    __shared__ double sh[32];
    float hi = v, lo = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
        float s, e;
        two_sum(hi, h2, s, e);
        e += lo + l2;
        hi = s + e;
        lo = e - (hi - s);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = (double)hi + (double)lo;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double w = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) w = bwarp_sum(w);
    return w;
}

template <typename S>
__device__ __forceinline__ double chunk_sum(S v);
template <>
__device__ __forceinline__ double chunk_sum<float>(float v) { return bblock_sum_f(v); }
template <>
__device__ __forceinline__ double chunk_sum<double>(double v) { return bblock_sum(v); }

// ---------------------------------------------------------------------------
// Element tile product of the new search direction: for each local node the
// tile stages d = S(r + beta d) (beta of the tile's mesh; zero rows stay zero
// because r and d are zero on constrained nodes), then part[tile node] = sum
// over the tile's elements of R K0 R^T d at that node, in S.
template <typename S>
__device__ __forceinline__ S dir_update(S beta, S d, S r);
template <>
__device__ __forceinline__ float dir_update<float>(float beta, float d, float r) { return __fmaf_rn(beta, d, r); }
template <>
__device__ __forceinline__ double dir_update<double>(double beta, double d, double r) { return __fma_rn(beta, d, r); }

template <typename S>
__global__ void __launch_bounds__(256) k_tile_spmv(BatchView<S> b, const S* __restrict__ dvec,
                                                   const S* __restrict__ rvec, S* __restrict__ part,
                                                   cudaGraphConditionalHandle if_refresh, int set_if,
                                                   const unsigned* __restrict__ refresh_flag)
{
    __shared__ S sd[3 * kTileNodes];
    __shared__ S so[12 * kTileElems];
    // the graph's IF node after this kernel runs the FP64 refresh product
    // only on iterations where some mesh refreshes its residual
    if (set_if && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(if_refresh, *refresh_flag ? 1u : 0u);
    const uint32_t t = blockIdx.x;
    if (t >= b.ntiles) return;
    const TileMeta tm = b.tiles[t];
    if (!mesh_running(b, tm.mesh)) return;
    const S beta = (S)b.st[tm.mesh].beta;
    const uint16_t* lp = b.lptr + b.lptr0[t];
    const uint16_t* li = b.lidx + tm.c0;
    // element data first: these loads are in flight while the tile stages
    // its node values
    const bool has_elem = threadIdx.x < tm.ne;
    const size_t e = tm.e0 + (has_elem ? threadIdx.x : 0);
    const size_t T = b.Ttot;
    S R[9], Di[9], k1 = 0, knu = 0, k2 = 0;
    uchar4 lc = make_uchar4(0, 0, 0, 0);
    if (has_elem) {
#pragma unroll
        for (int c = 0; c < 9; c++) R[c] = b.R[c * T + e];
#pragma unroll
        for (int c = 0; c < 9; c++) Di[c] = b.Dinv[c * T + e];
        k1 = b.mat[e];
        knu = b.mat[T + e];
        k2 = b.mat[2 * T + e];
        lc = b.lconn[e];
    }
    for (int i = threadIdx.x; i < tm.nn; i += blockDim.x) {
        const size_t g = bounds_idx(b.tile_nodes[tm.n0 + i], b.Ntot, kSiteBatchNode);
        sd[i] = dir_update<S>(beta, dvec[3 * g], rvec[3 * g]);
        sd[kTileNodes + i] = dir_update<S>(beta, dvec[3 * g + 1], rvec[3 * g + 1]);
        sd[2 * kTileNodes + i] = dir_update<S>(beta, dvec[3 * g + 2], rvec[3 * g + 2]);
    }
    __syncthreads();
    if (has_elem) {
        const int ids[4] = {(int)bounds_idx((uint32_t)lc.x, tm.nn, kSiteLocalNode),
                            (int)bounds_idx((uint32_t)lc.y, tm.nn, kSiteLocalNode),
                            (int)bounds_idx((uint32_t)lc.z, tm.nn, kSiteLocalNode),
                            (int)bounds_idx((uint32_t)lc.w, tm.nn, kSiteLocalNode)};
        S dl[12];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            dl[3 * i] = sd[ids[i]];
            dl[3 * i + 1] = sd[kTileNodes + ids[i]];
            dl[3 * i + 2] = sd[2 * kTileNodes + ids[i]];
        }
        S out[12];
        if (tm.material != kTileMaterialWrp)
            elem_pk(b, tm.material, tm.mesh, e, R, Di, knu, k2, dl, out);
        else
            elem_RKRt<S>(R, Di, k1, knu, k2, dl, out);
#pragma unroll
        for (int c = 0; c < 12; c++) so[c * kTileElems + threadIdx.x] = out[c];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < tm.nn; i += blockDim.x) {
        S a0 = 0, a1 = 0, a2 = 0;
        for (int j = lp[i]; j < lp[i + 1]; j++) {
            const int v = li[j], el = v >> 2, sl = v & 3;
            a0 += so[(3 * sl) * kTileElems + el];
            a1 += so[(3 * sl + 1) * kTileElems + el];
            a2 += so[(3 * sl + 2) * kTileElems + el];
        }
        const size_t o = 3 * tile_slot(b.ov_map, tm.own0, tm.ov0, tm.nown, i);
        part[o] = a0;
        part[o + 1] = a1;
        part[o + 2] = a2;
    }
}

template <typename S>
__global__ void __launch_bounds__(256) k_tile_spmv_y64(BatchView<S> b, const double* __restrict__ y,
                                                       double* __restrict__ part64, int mode,
                                                       const unsigned* __restrict__ flag)
{
    using V = typename Y64Value<S>::T;
    if (mode == SPMV_Y64_REFRESH && flag && !*flag) return;
    __shared__ V sd[3 * kTileNodes];
    __shared__ V so[12 * kTileElems];
    tile_spmv_y64_pass<S>(b, y, part64, mode, sd, so, blockIdx.x, gridDim.x);
}

// Elastic product at positions x (FP64): part64 = R K0 (R^T x - r) per tile
// node (C_f_e's product, TetrahedronElementSet3.cpp:1053-1096) and/or the
// per-tile elastic energy 0.5 u^T K0 u (C_V, :1456-1488).
template <typename S>
__global__ void __launch_bounds__(256) k_tile_force(BatchView<S> b, const double* __restrict__ x,
                                                    double* __restrict__ part64, double* __restrict__ tile_energy)
{
    // FP64 path: FP64. Mixed path: double-float values (about 48 bits; the
    // FP32 rotation and material scalars are exact in them, Dm^-1 comes from
    // its FP64 copy), FP64 partial sums: the mixed operator's FP32 element
    // data already bound its accuracy far above this evaluation's error
    using V = typename Y64Value<S>::T;
    __shared__ V so[12 * kTileElems];
    const uint32_t* list = part64 ? b.start_tiles : b.launch_tiles;
    const uint32_t n = b.list_count[part64 ? 0 : 2];
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t t = list[i];
        const TileMeta tm = b.tiles[t];
        // the force of a starting step, or the energy of a finished one
        if (part64 ? !mesh_starts(b, tm.mesh) : !b.st[tm.mesh].step_done) continue;
        double energy = 0.0;
        if (threadIdx.x < tm.ne && tm.material != kTileMaterialWrp) {
            // the P-K material's f_e and V (C_LCM_f_e / C_CCM_f_e, C_LCM_V,
            // TetrahedronElementSet3.cpp:1154-1206, 1489-1545) in FP64 in
            // either precision, on the F of the last BeginEvaluation (the
            // element cache's, as the reference's V() after a step also
            // reads it)
            const size_t e = tm.e0 + threadIdx.x;
            const size_t T = b.Ttot;
            const MeshConsts& mcm = b.mc[tm.mesh];
            double R[9], Di[9], F[9];
#pragma unroll
            for (int c = 0; c < 9; c++) R[c] = (double)b.R[c * T + e];
#pragma unroll
            for (int c = 0; c < 9; c++) Di[c] = b.Dinv64[c * T + e];
#pragma unroll
            for (int c = 0; c < 9; c++) F[c] = b.Fe[c * T + e];
            const PkMaterial pm{(int)tm.material, mcm.lame_mu, mcm.lame_lambda, mcm.ecie_k};
            energy = pk_energy(pm, R, F, b.vol[e]);
            if (part64) {
                double out[12];
                pk_force(pm, R, F, Di, b.vol[e], out);
#pragma unroll
                for (int c = 0; c < 12; c++) y64_set(so[c * kTileElems + threadIdx.x], out[c]);
            }
        } else if (threadIdx.x < tm.ne) {
            const size_t e = tm.e0 + threadIdx.x;
            const size_t T = b.Ttot;
            S R[9];
            V Di[9];
#pragma unroll
            for (int c = 0; c < 9; c++) R[c] = b.R[c * T + e];
#pragma unroll
            for (int c = 0; c < 9; c++) y64_set(Di[c], b.Dinv64[c * T + e]);
            V k1, knu, k2;
            y64_set(k1, (double)b.mat[e]);
            y64_set(knu, (double)b.mat[T + e]);
            y64_set(k2, (double)b.mat[2 * T + e]);
            const int4 g = b.gtets[e];
            const int ids[4] = {(int)bounds_idx((uint32_t)g.x, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.y, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.z, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.w, b.Ntot, kSiteBatchNode)};
            V u[12];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const size_t n = ids[i];
                V xa, xb, xc;
                y64_set(xa, x[3 * n]);
                y64_set(xb, x[3 * n + 1]);
                y64_set(xc, x[3 * n + 2]);
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    V acc{};
                    acc += R[a] * xa;
                    acc += R[3 + a] * xb;
                    acc += R[6 + a] * xc;
                    V r0;
                    y64_set(r0, b.rest[3 * n + a]);
                    u[3 * i + a] = acc - r0;
                }
            }
            V D[9];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int j = 0; j < 3; j++) D[3 * a + j] = u[3 * (j + 1) + a] - u[a];
            V H[9];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int c = 0; c < 3; c++) H[3 * a + c] = D[3 * a] * Di[c] + D[3 * a + 1] * Di[3 + c] + D[3 * a + 2] * Di[6 + c];
            V P[9], es;
            stress_forces(H, Di, k1, knu, k2, P, es);
            energy = 0.5 * y64_get(es);
            if (part64) {
                V out[12];
                rotate_out(R, P, out);
#pragma unroll
                for (int c = 0; c < 12; c++) so[c * kTileElems + threadIdx.x] = out[c];
            }
        }
        if (tile_energy) {
            const double s = bblock_sum(energy);
            if (threadIdx.x == 0) tile_energy[t] = s;
        }
        if (part64) {
            __syncthreads();
            const uint16_t* lp = b.lptr + b.lptr0[t];
            const uint16_t* li = b.lidx + tm.c0;
            for (int i = threadIdx.x; i < tm.nn; i += blockDim.x) {
                V a0{}, a1{}, a2{};
                for (int j = lp[i]; j < lp[i + 1]; j++) {
                    const int v = li[j], el = v >> 2, sl = v & 3;
                    a0 += so[(3 * sl) * kTileElems + el];
                    a1 += so[(3 * sl + 1) * kTileElems + el];
                    a2 += so[(3 * sl + 2) * kTileElems + el];
                }
                const size_t o = 3 * tile_slot(b.ov_map, tm.own0, tm.ov0, tm.nown, i);
                part64[o] = y64_get(a0);
                part64[o + 1] = y64_get(a1);
                part64[o + 2] = y64_get(a2);
            }
        }
        __syncthreads();
    }
}

// Potential energy term of RecomputeEnergy per tile (LeafDSH_Solid3D_FEM.cpp:1554-1584).
template <typename S>
__global__ void k_tile_potential(BatchView<S> b, const double* __restrict__ x, double* __restrict__ tile_pe)
{
    const uint32_t n = b.list_count[2];
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint32_t t = b.launch_tiles[i];
        const TileMeta tm = b.tiles[t];
        if (!b.st[tm.mesh].step_done) continue;
        const MeshConsts& c = b.mc[tm.mesh];
        double acc = 0.0;
        if (threadIdx.x < tm.ne) {
            const size_t e = tm.e0 + threadIdx.x;
            const int4 g = b.gtets[e];
            const int ids[4] = {(int)bounds_idx((uint32_t)g.x, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.y, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.z, b.Ntot, kSiteBatchNode),
                            (int)bounds_idx((uint32_t)g.w, b.Ntot, kSiteBatchNode)};
            double s[3] = {0, 0, 0};
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int a = 0; a < 3; a++) s[a] += x[3 * (size_t)ids[i] + a];
            const double em = c.density * b.vol[e];
            acc = (em / 4.0) * (s[0] * -c.gravity[0] + s[1] * -c.gravity[1] + s[2] * -c.gravity[2]);
        }
        const double v = bblock_sum(acc);
        if (threadIdx.x == 0) tile_pe[t] = v;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// node kernels: one block per node chunk (kChunkNodes nodes of one mesh,
// kNodeThreads threads striding it)

// Sum of a node's partials: its owner tile's (node order) first, then its
// overflow slots (contiguous, in tile order).
template <typename S, typename P>
__device__ __forceinline__ void sum_parts(const BatchView<S>& b, const P* __restrict__ part, size_t n, double& a0,
                                          double& a1, double& a2)
{
    a0 = (double)part[3 * n];
    a1 = (double)part[3 * n + 1];
    a2 = (double)part[3 * n + 2];
    const uint32_t j1 = bounds_idx(b.ov_ptr[n + 1], b.nslots - b.Ntot + 1, kSitePartialSlot);
    for (uint32_t j = b.ov_ptr[n]; j < j1; j++) {
        const size_t o = 3 * ((size_t)b.Ntot + j);
        a0 += (double)part[o];
        a1 += (double)part[o + 1];
        a2 += (double)part[o + 2];
    }
}

// QIE: b = dt (m g - f_e-product) + m v ; y = v.
// FIE (Step_FullyImplicitEuler_dx, LeafDSH_Solid3D_FEM.cpp:1412-1440): on
// the first Newton iteration x^n = x, v^n = v and the warm start
// y = h v^n (else 0); b_k = m g - f(x_k) + (m/h)(v^n - (x_k - x^n)/h)
// (quasi-static: 1/h = 0).
template <typename S>
__global__ void k_node_b(BatchView<S> b, const double* __restrict__ part64, const double* __restrict__ v,
                         const double* __restrict__ x, double* __restrict__ bv, double* __restrict__ y)
{
    const uint32_t nl = b.list_count[1];
    for (uint32_t il = blockIdx.x; il < nl; il += gridDim.x) {
        const uint32_t ci = b.start_chunks[il];
        const ChunkMeta ch = b.chunks[ci];
        if (!mesh_starts(b, ch.mesh)) continue;
        const MeshConsts& c = b.mc[ch.mesh];
        const bool opening = c.integrator == kMeshQie || b.st[ch.mesh].nr_k == 0;
        if (b.lock) {
            // NR_MidStep (LeafDSH_Solid3D_FEM.cpp:2930-2990): the FIE
            // right-hand side at the iterate x_k with x^n = x, v^n = v, warm
            // start h v^n on the phase's first solve since NR_PreStep
            const double im = c.inv_dt * c.mass;
            const bool warm = b.st[ch.mesh].nr_k == 0;
            for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
                double f[3];
                sum_parts(b, part64, n, f[0], f[1], f[2]);
                const size_t i = 3 * n;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const double bf = c.mass * c.gravity[a] - f[a];
                    bv[i + a] = bf + im * (v[i + a] - c.inv_dt * (b.xn[i + a] - x[i + a]));
                    y[i + a] = warm ? c.dt * v[i + a] : 0.0;
                    if (b.ydelta) b.ydelta[i + a] = 0;
                }
            }
            continue;
        }
        if (c.integrator != kMeshQie) {
            const double im = c.inv_dt * c.mass;
            for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
                double f[3];
                sum_parts(b, part64, n, f[0], f[1], f[2]);
                const size_t i = 3 * n;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    if (opening) {
                        b.xn[i + a] = x[i + a];
                        b.vn[i + a] = v[i + a];
                        if (b.prev_x && c.rotation == kMeshRotationDapd) b.prev_x[i + a] = x[i + a];
                    }
                    const double bf = c.mass * c.gravity[a] - f[a];
                    bv[i + a] = bf + im * (b.vn[i + a] - c.inv_dt * (x[i + a] - b.xn[i + a]));
                    y[i + a] = opening ? c.dt * b.vn[i + a] : 0.0;
                    if (b.ydelta) b.ydelta[i + a] = 0;
                }
            }
            continue;
        }
        // DAPD: this step's BeginEvaluation has read the previous positions;
        // the next one compares with this step's start (m_vecPos0 = x,
        // LeafDSH_Solid3D_FEM.cpp:927-935)
        const bool dapd = b.prev_x && c.rotation == kMeshRotationDapd;
        for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
            double f0, f1, f2;
            sum_parts(b, part64, n, f0, f1, f2);
            const size_t i = 3 * n;
            if (dapd) {
                b.prev_x[i] = x[i];
                b.prev_x[i + 1] = x[i + 1];
                b.prev_x[i + 2] = x[i + 2];
            }
            bv[i] = (c.mass * c.gravity[0] - f0) * c.dt + c.mass * v[i];
            bv[i + 1] = (c.mass * c.gravity[1] - f1) * c.dt + c.mass * v[i + 1];
            bv[i + 2] = (c.mass * c.gravity[2] - f2) * c.dt + c.mass * v[i + 2];
            y[i] = v[i];
            y[i + 1] = v[i + 1];
            y[i + 2] = v[i + 2];
            if (b.ydelta) {
                b.ydelta[i] = 0;
                b.ydelta[i + 1] = 0;
                b.ydelta[i + 2] = 0;
            }
        }
    }
}

// position constraints -> clamped velocity in b and y (LeafDSH_Solid3D_FEM.cpp:1268-1295)
template <typename S>
__global__ void k_knc(BatchView<S> b, uint32_t K, const double* __restrict__ x, double* __restrict__ bv,
                      double* __restrict__ y)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
        const uint32_t m = b.knc_mesh[k];
        if (!mesh_starts(b, m)) continue;
        const MeshConsts& c = b.mc[m];
        const size_t n = bounds_idx(b.knc_node[k], b.Ntot, kSiteKncNode);
        const double* tg = b.knc_target + 3 * (size_t)k;
        if (c.integrator != kMeshQie || b.lock) {
            // FIE: the constraint rows as Delta x, b = y = target - x_k
            // (LeafDSH_Solid3D_FEM.cpp:1441-1465)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const double dx = tg[a] - x[3 * n + a];
                bv[3 * n + a] = dx;
                y[3 * n + a] = dx;
            }
            continue;
        }
        V3<double> vk = mk<double>(c.inv_dt * (tg[0] - x[3 * n]), c.inv_dt * (tg[1] - x[3 * n + 1]),
                                   c.inv_dt * (tg[2] - x[3 * n + 2]));
        const double norm_vk = ::sqrt(dot0(vk, vk));
        V3<double> vel = mk<double>(0.0, 0.0, 0.0);
        if (norm_vk > (double)0.001f) {
            const double cl = (norm_vk < 50.0) ? norm_vk : 50.0;
            vel = scale(cl, normalized(vk));
        }
        bv[3 * n] = vel.x; bv[3 * n + 1] = vel.y; bv[3 * n + 2] = vel.z;
        y[3 * n] = vel.x; y[3 * n + 1] = vel.y; y[3 * n + 2] = vel.z;
    }
}

// ---------------------------------------------------------------------------
// Arrival counting. After a block has written its chunk partial, the block
// that completes a mesh's set of chunks sums them (fixed order) and updates
// the mesh's CG scalars; after a block has finished all its chunks, the block
// that completes the grid evaluates the batch-wide loop condition. Nothing
// waits: the last arrival does the work.
// The values other blocks must see (a chunk partial, a mesh's scalars) are
// written by thread 0, so thread 0 alone fences before arriving.
__device__ __forceinline__ bool arrive_last(unsigned* ctr, unsigned expected)
{
    __shared__ unsigned s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(ctr, 1u);
        s_last = (prev + 1u == expected) ? 1u : 0u;
        if (s_last) {
            *ctr = 0u;
            __threadfence();
        }
    }
    __syncthreads();
    return s_last != 0;
}

// Fixed-order sum of a mesh's chunk partials by the whole block (L1 bypassed:
// the partials were written by other blocks of this kernel).
__device__ __forceinline__ double mesh_partial_sum(const double* cpart, uint32_t c0, uint32_t n)
{
    double acc = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) acc += __ldcg(cpart + c0 + i);
    return bblock_sum(acc);
}

__device__ __forceinline__ bool cg_cont(const StepScalars& s)
{
    return s.delta_new > s.abs_eps_sq && s.delta_new > s.delta_target && s.k < s.max_iter;
}

__device__ __forceinline__ void finish_stats(StepScalars& s)
{
    s.rel_residual = (s.delta_0 > 0) ? ::sqrt(s.delta_new / s.delta_0) : 0.0;
    s.abs_residual = ::sqrt(s.delta_new);
}

// Last block of the grid: while condition (any mesh iterating), the refresh
// flag for the next iteration and, on the mixed path, the work lists of the
// meshes that iterate.
template <typename S>
__device__ void grid_tail(const BatchView<S>& b, const LoopSync& ls, bool iteration)
{
    if (!arrive_last(ls.gcount, gridDim.x)) return;
    if (b.act_tiles && (!iteration || *(volatile const unsigned*)b.list_dirty)) build_active_lists(b);  // FP64 tail: no lists
    int any = 0, refresh = 0, norf = 0;  // norf: a running mesh that does not refresh
    for (uint32_t i = threadIdx.x; i < b.M; i += blockDim.x) {
        volatile const StepScalars* sp = b.st + i;
        if (!sp->done) {
            any = 1;
            if (sp->refresh_next)
                refresh = 1;
            else
                norf = 1;
        }
    }
    any = __syncthreads_or(any);
    refresh = __syncthreads_or(refresh);
    norf = __syncthreads_or(norf);
    if (refresh && b.refresh_tiles) set_refresh_lists(b, !norf);
    if (threadIdx.x == 0) {
        if (ls.refresh_flag) *ls.refresh_flag = refresh ? 1u : 0u;
        if (ls.body_runs) *ls.body_runs += 1u;
        const bool stop = ls.err && *(volatile const unsigned*)ls.err;
        bool budget_left = true;
        if (ls.slice) {
            if (iteration) ls.slice[1] += 1u;
            budget_left = ls.slice[0] == 0u || ls.slice[1] < ls.slice[0];
        }
        if (ls.set_cond) cudaGraphSetConditional(ls.cond, (any && !stop && budget_left) ? 1u : 0u);
    }
}

// r = S(b - A y) with A y = fK sum(part64) + m fM y ; d = 0 ; |r|^2 ; the
// last block of a mesh starts its CG loop (ILSS_CG.h:53-73).
template <typename S>
__global__ void k_node_residual(BatchView<S> b, const double* __restrict__ part64, const double* __restrict__ bv,
                                const double* __restrict__ y, S* __restrict__ r, S* __restrict__ d,
                                double* __restrict__ cpart, LoopSync ls)
{
    const uint32_t nl = b.list_count[1];
    for (uint32_t il = blockIdx.x; il < nl; il += gridDim.x) {
        const uint32_t ci = b.start_chunks[il];
        const ChunkMeta ch = b.chunks[ci];
        if (!mesh_starts(b, ch.mesh)) continue;
        const MeshConsts& c = b.mc[ch.mesh];
        const double mfm = c.mass * c.factor_M;
        const bool minres = c.solver == kMeshSolverMinres;
        const bool fie = c.integrator != kMeshQie && !b.lock;  // the lock-step's solves have no |b_k| test
        const bool need_b = minres || fie;
        double acc = 0.0, acc_b = 0.0;
        for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
            const size_t i = 3 * n;
            S r0 = 0, r1 = 0, r2 = 0;
            if (!b.fixed[n]) {
                double s0, s1, s2;
                sum_parts(b, part64, n, s0, s1, s2);
                r0 = (S)(bv[i] - (c.factor_K * s0 + mfm * y[i]));
                r1 = (S)(bv[i + 1] - (c.factor_K * s1 + mfm * y[i + 1]));
                r2 = (S)(bv[i + 2] - (c.factor_K * s2 + mfm * y[i + 2]));
            }
            r[i] = r0; r[i + 1] = r1; r[i + 2] = r2;
            d[i] = 0; d[i + 1] = 0; d[i + 2] = 0;
            acc += (double)r0 * (double)r0 + (double)r1 * (double)r1 + (double)r2 * (double)r2;
            // |b| over every row, constrained ones too: MINRES's relative
            // test and FIE's Newton test
            if (need_b) acc_b += bv[i] * bv[i] + bv[i + 1] * bv[i + 1] + bv[i + 2] * bv[i + 2];
        }
        const double sum = bblock_sum(acc);
        const double sum_b = need_b ? bblock_sum(acc_b) : 0.0;
        if (threadIdx.x == 0) {
            cpart[ci] = sum;
            if (need_b) b.cpart_b[ci] = sum_b;
        }
        if (arrive_last(ls.mcount + ch.mesh, c.nchunks)) {
            const double total = mesh_partial_sum(cpart, c.chunk0, c.nchunks);
            const double total_b = need_b ? mesh_partial_sum(b.cpart_b, c.chunk0, c.nchunks) : 0.0;
            bool newton_ends = false;
            if (threadIdx.x == 0) {
                StepScalars& s = b.st[ch.mesh];
                if (b.lock) {
                } else if (c.integrator == kMeshQie) {
                    s.nr_go = 0;
                } else {
                    // the Newton test on |b_k| (LeafDSH_Solid3D_FEM.cpp:1466-1480):
                    // below the tolerance (or not finite) the loop ends
                    // without a solve
                    const double nb = ::sqrt(total_b);
                    if (s.nr_k == 0) s.nr_delta0 = nb;
                    s.nr_abs = nb;
                    if (!isfinite(nb) || nb < c.nr_abs_eps) {
                        newton_ends = true;
                        if (!isfinite(nb)) s.status = 3u;
                        s.done = 1;
                        s.nr_go = 0;
                        s.mr_pending = 0;
                        s.step_done = 1;
                    }
                }
            }
            if (threadIdx.x == 0 && !newton_ends && minres) {
                // ILSS_MINRES::Solve's start (ILSS_MINRES.h:66-107); the
                // next finishing pass normalises v = r0 / |r0|
                StepScalars& s = b.st[ch.mesh];
                minres_start(s.mr, total);
                s.mr.norm_b_sq = total_b;
                s.delta_0 = total_b;
                s.delta_new = total;
                s.delta_old = total;
                s.delta_target = c.rel_eps_sq * total_b;
                s.abs_eps_sq = c.abs_eps_sq;
                s.max_iter = c.max_iter;
                s.k = 0;
                s.status = (!isfinite(total)) ? 3u : 0u;
                s.alpha = 0.0;
                s.beta = 0.0;
                s.beta_f = 0.f;
                s.refresh_next = 0;
                s.delta_refresh = total;
                s.k_refresh = 0;
                s.confirm = 0;
                s.done = cg_cont(s) ? 0u : 1u;
                s.mr_pending = s.done ? 0u : 2u;
                if (s.done) {
                    finish_stats(s);
                    s.finished = 1;
                }
            } else if (threadIdx.x == 0 && !newton_ends) {
                StepScalars& s = b.st[ch.mesh];
                s.delta_0 = total;
                s.delta_new = total;
                s.delta_old = total;
                s.delta_target = c.rel_eps_sq * total;
                s.abs_eps_sq = c.abs_eps_sq;
                s.max_iter = c.max_iter;
                s.k = 0;
                s.status = (!isfinite(total)) ? 3u : 0u;
                s.alpha = 0.0;
                s.beta = 0.0;
                s.beta_f = 0.f;
                s.refresh_next = 0;  // r0 was formed from the FP64 product
                s.delta_refresh = total;
                s.k_refresh = 0;
                s.confirm = 0;
                s.done = cg_cont(s) ? 0u : 1u;
                if (s.done) {
                    finish_stats(s);
                    s.finished = 1;
                }
            }
        }
        __syncthreads();
    }
    grid_tail(b, ls, false);
}

// Sum of node n's tile partials: its owner slot, then its overflow slots.
template <typename S>
__device__ __forceinline__ void node_part_sum(const BatchView<S>& b, const S* part, size_t n, S& s0, S& s1, S& s2)
{
    s0 = part[3 * n];
    s1 = part[3 * n + 1];
    s2 = part[3 * n + 2];
    const uint32_t j1 = bounds_idx(b.ov_ptr[n + 1], b.nslots - b.Ntot + 1, kSitePartialSlot);
    for (uint32_t j = b.ov_ptr[n]; j < j1; j++) {
        const size_t o = 3 * ((size_t)b.Ntot + j);
        s0 += part[o];
        s1 += part[o + 1];
        s2 += part[o + 2];
    }
}

// MINRES, after the product of v (in r): v1 = S A v - beta v0 into q and
// v1.v; the last block of the mesh takes alpha = v1.v (ILSS_MINRES.h:
// 117-124).
template <typename S>
__device__ void node_q_minres(const BatchView<S>& b, const MeshConsts& c, const StepScalars& sm, uint32_t ci,
                              const ChunkMeta& ch, const S* part, const S* v, const S* v0, S* v1, double* cpart,
                              const LoopSync& ls)
{
    const S fK = (S)c.factor_K, mfm = (S)(c.mass * c.factor_M);
    const S nb = (S)(-sm.mr.beta_new);
    S acc = 0;
    for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
        const size_t i = 3 * n;
        S s[3] = {0, 0, 0};
        const bool fixed = b.fixed[n] != 0;
        if (!fixed) node_part_sum(b, part, n, s[0], s[1], s[2]);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const S qa = fixed ? (S)0 : fK * s[a] + mfm * v[i + a];
            const S w = qa + nb * v0[i + a];
            v1[i + a] = w;
            acc += w * v[i + a];
        }
    }
    const double sum = chunk_sum<S>(acc);
    if (threadIdx.x == 0) cpart[ci] = sum;
    if (arrive_last(ls.mcount + ch.mesh, c.nchunks)) {
        const double total = mesh_partial_sum(cpart, c.chunk0, c.nchunks);
        if (threadIdx.x == 0) {
            StepScalars& s = b.st[ch.mesh];
            s.mr.beta = s.mr.beta_new;
            s.mr.alpha = total;
        }
    }
}

// MINRES: v1 -= alpha v and |v1|^2; the last block of the mesh forms the
// Givens rotation, the residual estimate and the loop test (ILSS_MINRES.h:
// 125-160); the finishing pass then applies the iteration's updates.
template <typename S>
__device__ void node_update_minres(const BatchView<S>& b, const MeshConsts& c, const StepScalars& sm, uint32_t ci,
                                   const ChunkMeta& ch, const S* v, S* v1, double* cpart, const LoopSync& ls)
{
    const S na = (S)(-sm.mr.alpha);
    S acc = 0;
    for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const size_t i = 3 * n + a;
            const S w = v1[i] + na * v[i];
            v1[i] = w;
            acc += w * w;
        }
    }
    const double sum = chunk_sum<S>(acc);
    if (threadIdx.x == 0) cpart[ci] = sum;
    if (arrive_last(ls.mcount + ch.mesh, c.nchunks)) {
        const double total = mesh_partial_sum(cpart, c.chunk0, c.nchunks);
        if (threadIdx.x == 0) {
            StepScalars& s = b.st[ch.mesh];
            minres_givens(s.mr, total);
            s.delta_old = s.delta_new;
            s.delta_new = s.mr.norm_r_sq;
            s.k += 1;
            s.total_iters += 1;
            if (!isfinite(total) || !isfinite(s.mr.norm_r_sq)) s.status = 3u;
            s.mr_pending = 1u;
            s.done = cg_cont(s) ? 0u : 1u;
            if (s.done) {
                finish_stats(s);
                s.finished = 1;
            }
        }
    }
}

// d = S(r + beta d) written back ; q = S A d ; d.q ; last block of a mesh:
// alpha (ILSS_CG.h:90-98). On refresh iterations r becomes S(b - A y).
template <typename S>
__global__ void k_node_q(BatchView<S> b, const S* __restrict__ part, S* __restrict__ d, S* __restrict__ q,
                         const double* __restrict__ part64, const double* __restrict__ bv,
                         const double* __restrict__ y, S* __restrict__ r, double* __restrict__ cpart, LoopSync ls)
{
    {
        const uint32_t ci = blockIdx.x;
        if (ci >= b.nchunks) return;
        const ChunkMeta ch = b.chunks[ci];
        if (!mesh_running(b, ch.mesh)) return;
        const MeshConsts& c = b.mc[ch.mesh];
        const StepScalars& sm = b.st[ch.mesh];
        if (c.solver == kMeshSolverMinres) {
            node_q_minres(b, c, sm, ci, ch, part, r, d, q, cpart, ls);
            return;
        }
        const bool refresh = part64 && refresh_now(c, sm);
        const S beta = (S)sm.beta;
        const S fK = (S)c.factor_K, mfm = (S)(c.mass * c.factor_M);
        S acc = 0;
        for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
            const size_t i = 3 * n;
            S q0 = 0, q1 = 0, q2 = 0, dn0 = 0, dn1 = 0, dn2 = 0;
            if (!b.fixed[n]) {
                dn0 = dir_update<S>(beta, d[i], r[i]);
                dn1 = dir_update<S>(beta, d[i + 1], r[i + 1]);
                dn2 = dir_update<S>(beta, d[i + 2], r[i + 2]);
                S s0 = part[3 * n], s1 = part[3 * n + 1], s2 = part[3 * n + 2];
                const uint32_t j1 = bounds_idx(b.ov_ptr[n + 1], b.nslots - b.Ntot + 1, kSitePartialSlot);
                for (uint32_t j = b.ov_ptr[n]; j < j1; j++) {
                    const size_t o = 3 * ((size_t)b.Ntot + j);
                    s0 += part[o];
                    s1 += part[o + 1];
                    s2 += part[o + 2];
                }
                q0 = fK * s0 + mfm * dn0;
                q1 = fK * s1 + mfm * dn1;
                q2 = fK * s2 + mfm * dn2;
                if (refresh) {
                    double t0, t1, t2;
                    sum_parts(b, part64, n, t0, t1, t2);
                    const double mfm64 = c.mass * c.factor_M;
                    r[i] = (S)(bv[i] - (c.factor_K * t0 + mfm64 * y_full(b, y, i)));
                    r[i + 1] = (S)(bv[i + 1] - (c.factor_K * t1 + mfm64 * y_full(b, y, i + 1)));
                    r[i + 2] = (S)(bv[i + 2] - (c.factor_K * t2 + mfm64 * y_full(b, y, i + 2)));
                }
            }
            d[i] = dn0; d[i + 1] = dn1; d[i + 2] = dn2;
            q[i] = q0; q[i + 1] = q1; q[i + 2] = q2;
            acc += dn0 * q0 + dn1 * q1 + dn2 * q2;
        }
        const double sum = chunk_sum<S>(acc);
        if (threadIdx.x == 0) cpart[ci] = sum;
        if (arrive_last(ls.mcount + ch.mesh, c.nchunks)) {
            const double total = mesh_partial_sum(cpart, c.chunk0, c.nchunks);
            if (threadIdx.x == 0) {
                StepScalars& s = b.st[ch.mesh];
                s.dot_dq = total;
                if (::fabs(total) < s.abs_eps_sq) {  // breakdown: leave before the update
                    s.done = 1;
                    s.finished = 1;
                    finish_stats(s);
                } else {
                    s.alpha = s.delta_new / total;
                }
            }
        }
    }
}

// y += alpha d (FP64) ; r -= alpha q (in S) ; |r|^2 ; last block of a mesh:
// beta, k += 1 and the loop test (ILSS_CG.h:100-144).
template <typename S>
__global__ void k_node_update(BatchView<S> b, double* __restrict__ y, S* __restrict__ r, const S* __restrict__ d,
                              S* __restrict__ q, double* __restrict__ cpart, LoopSync ls)
{
    const uint32_t ci = blockIdx.x;
    const ChunkMeta ch = b.chunks[ci < b.nchunks ? ci : 0];
    if (ci < b.nchunks && mesh_running(b, ch.mesh) && b.mc[ch.mesh].solver == kMeshSolverMinres) {
        node_update_minres(b, b.mc[ch.mesh], b.st[ch.mesh], ci, ch, r, q, cpart, ls);
    } else if (ci < b.nchunks && mesh_running(b, ch.mesh)) {
        const MeshConsts& c = b.mc[ch.mesh];
        const double alpha = b.st[ch.mesh].alpha;
        const S alpha_s = (S)alpha, na = -alpha_s;
        S acc = 0;
        for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
            S rr = 0;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const size_t i = 3 * n + a;
                if (b.ydelta) b.ydelta[i] += alpha_s * d[i];
                else y[i] += alpha * (double)d[i];
                const S ri = r[i] + na * q[i];
                r[i] = ri;
                rr += ri * ri;
            }
            acc += rr;
        }
        const double sum = chunk_sum<S>(acc);
        if (threadIdx.x == 0) cpart[ci] = sum;
        if (arrive_last(ls.mcount + ch.mesh, c.nchunks)) {
            const double total = mesh_partial_sum(cpart, c.chunk0, c.nchunks);
            if (threadIdx.x == 0) {
                StepScalars& s = b.st[ch.mesh];
                s.delta_old = s.delta_new;
                s.delta_new = total;
                s.beta = total / s.delta_old;
                s.k += 1;
                s.total_iters += 1;
                if (!isfinite(total)) s.status = 3u;
                s.done = cg_cont(s) ? 0u : 1u;
                if (s.done) {
                    finish_stats(s);
                    s.finished = 1;
                }
            }
        }
    }
    grid_tail(b, ls, true);
}

// MINRES's finishing pass per chunk of a mesh with an update due, after the
// mesh's loop test (either precision):
//   mr_pending 2 (start or restart): v = r0 / |r0| (ILSS_MINRES.h:82-95),
//     v0 = p = p0 = 0;
//   mr_pending 1 (an iteration): p_new = (v - r2 p - r3 p0) / r1,
//     y += beta_one c eta p_new, p0 = p, p = p_new, v0 = v,
//     v = v1 / beta_new (ILSS_MINRES.h:131-156).
// The last block of the mesh clears the flag.
template <typename S>
__global__ void k_node_mr_finish(BatchView<S> b, double* __restrict__ y, S* __restrict__ r, S* __restrict__ d,
                                 const S* __restrict__ q, LoopSync ls)
{
    const uint32_t nl = b.list_count[3];
    for (uint32_t il = blockIdx.x; il < nl; il += gridDim.x) {
        const uint32_t ci = b.launch_chunks[il];
        const ChunkMeta ch = b.chunks[ci];
        const MeshConsts& c = b.mc[ch.mesh];
        if (c.solver != kMeshSolverMinres) continue;
        const StepScalars& sm = b.st[ch.mesh];
        const uint32_t pending = sm.mr_pending;
        if (!pending) continue;
        const MinresScalars mr = sm.mr;
        // the six vectors are distinct buffers: restrict lets the loads of
        // the next entries go ahead of this entry's stores
        S* __restrict__ p = b.mr_p;
        S* __restrict__ p0 = b.mr_p0;
        if (pending == 2u) {
            const S inv = (S)mr.inv_beta;
            for (size_t i = 3 * (size_t)ch.n0 + threadIdx.x; i < 3 * (size_t)ch.n1; i += blockDim.x) {
                r[i] *= inv;
                d[i] = 0;
                p[i] = 0;
                p0[i] = 0;
            }
        } else {
            const S inv = (S)mr.inv_beta, nr2 = (S)mr.neg_r2, nr3 = (S)mr.neg_r3, ir1 = (S)mr.inv_r1;
#pragma unroll 4
            for (size_t i = 3 * (size_t)ch.n0 + threadIdx.x; i < 3 * (size_t)ch.n1; i += blockDim.x) {
                const S v = r[i];
                const S pi = p[i];
                S pn = nr2 * pi + v;
                pn += nr3 * p0[i];
                pn *= ir1;
                p0[i] = pi;
                p[i] = pn;
                y[i] += mr.x_coef * (double)pn;
                d[i] = v;
                r[i] = q[i] * inv;
            }
        }
        if (arrive_last(ls.mcount + ch.mesh, c.nchunks) && threadIdx.x == 0) b.st[ch.mesh].mr_pending = 0u;
    }
}

// After a linear solve, per chunk of a mesh whose loop ended in it:
// QIE: v = y ; x += dt y, and the step is done.
// FIE (LeafDSH_Solid3D_FEM.cpp:1500-1529): x_k += y ; v_k = (x_k - x^n)/h ;
// |y|; the last block of the mesh counts the Newton iteration and decides
// whether the loop goes on (below the iteration limit); the step's
// BeginEvaluation at x_k follows in any case.
template <typename S>
__global__ void k_integrate(BatchView<S> b, double* __restrict__ x, double* __restrict__ v,
                            const double* __restrict__ y, double* __restrict__ cpart, LoopSync ls)
{
    const uint32_t nl = b.list_count[3];
    for (uint32_t il = blockIdx.x; il < nl; il += gridDim.x) {
        const uint32_t ci = b.launch_chunks[il];
        const ChunkMeta ch = b.chunks[ci];
        if (!b.st[ch.mesh].finished) continue;
        const MeshConsts& c = b.mc[ch.mesh];
        if (b.lock) {
            // NR_PostStep (LeafDSH_Solid3D_FEM.cpp:2991-3010): x_k += y,
            // v_k = (x_k - x^n)/h with x^n = x; the phase's counts
            for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const size_t i = 3 * n + a;
                    const double xi = b.xn[i] + y_full(b, y, i);
                    b.xn[i] = xi;
                    b.vn[i] = c.inv_dt * (xi - x[i]);
                }
            }
            if (arrive_last(ls.mcount + ch.mesh, c.nchunks) && threadIdx.x == 0) {
                StepScalars& s = b.st[ch.mesh];
                s.nr_k += 1;
                s.fie_cg += s.k;
                s.inverted = 0;  // counted again by the re-evaluation at x_k
            }
            continue;
        }
        if (c.integrator == kMeshQie) {
            const double dt = c.dt;
            for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const size_t i = 3 * n + a;
                    const double yi = y_full(b, y, i);
                    v[i] = yi;
                    x[i] = x[i] + dt * yi;
                }
            }
            if (threadIdx.x == 0) b.st[ch.mesh].step_done = 1;
            continue;
        }
        double acc = 0.0;
        for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const size_t i = 3 * n + a;
                const double yi = y_full(b, y, i);
                const double xi = x[i] + yi;
                x[i] = xi;
                v[i] = c.inv_dt * (xi - b.xn[i]);
                acc += yi * yi;
            }
        }
        const double sum = bblock_sum(acc);
        if (threadIdx.x == 0) cpart[ci] = sum;
        if (arrive_last(ls.mcount + ch.mesh, c.nchunks)) {
            const double total = mesh_partial_sum(cpart, c.chunk0, c.nchunks);
            if (threadIdx.x == 0) {
                StepScalars& s = b.st[ch.mesh];
                s.nr_abs = ::sqrt(total);
                s.nr_k += 1;
                s.fie_cg += s.k;
                s.nr_solved = 1;
                s.nr_go = s.nr_k < c.nr_max_iter ? 1u : 0u;
                if (!s.nr_go) s.step_done = 1;
                s.inverted = 0;  // counted again by the re-evaluation at x_k
            }
        }
    }
}

// The lock-step's per-mesh bookkeeping, one block: phase 0 (NR_PreStep)
// restarts the iterate count and the solver-iteration count of every mesh
// taking part; phase 1 (NR_End) marks their steps done.
template <typename S>
__global__ void k_lock_phase(BatchView<S> b, int phase)
{
    for (uint32_t m = threadIdx.x; m < b.M; m += blockDim.x) {
        StepScalars& s = b.st[m];
        if (b.active[m] != 1) continue;
        if (phase == 0) {
            s.nr_k = 0;
            s.fie_cg = 0;
            s.nr_go = 1;
            s.finished = 0;
        } else {
            s.step_done = 1;
        }
    }
}

// The mixed path's per-tile copies of the system factors (factor_K and
// m factor_M in FP32, in each tile blob's header) from the meshes' constants
// in the view: the lock-step's own, then the step's again.
__global__ void k_blob_factors(BatchView<float> b)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < b.ntiles; t += gridDim.x * blockDim.x) {
        const TileMeta tm = b.tiles[t];
        float* fac = reinterpret_cast<float*>(b.blob + 16ull * b.blob_off16[t] + blob_hdr_off(tm.ne, tm.nn) + 4u);
        fac[0] = b.mc[tm.mesh].fK_f;
        fac[1] = b.mc[tm.mesh].mfm_f;
    }
}

void launch_blob_factors(const BatchView<float>& b, cudaStream_t s)
{
    k_blob_factors<<<(b.ntiles + 255) / 256 < 1024 ? (b.ntiles + 255) / 256 : 1024, 256, 0, s>>>(b);
    launch_counter()++;
}

// One block, last kernel of a Newton iteration: the start lists of the next
// iteration (the FIE meshes going on), the finished flags cleared, and the
// Newton loop's condition.
template <typename S>
__global__ void k_newton_tail(BatchView<S> b, LoopSync ls, cudaGraphConditionalHandle newton)
{
    int go = 0;
    for (uint32_t m = threadIdx.x; m < b.M; m += blockDim.x) {
        StepScalars& s = b.st[m];
        s.finished = 0;
        go |= s.nr_go ? 1 : 0;
    }
    go = __syncthreads_or(go);
    build_mesh_lists(
        b, [&](uint32_t m) { return b.st[m].nr_go != 0u; }, b.start_tiles, b.start_chunks, b.list_count);
    if (threadIdx.x == 0) {
        const bool stop = ls.err && *(volatile const unsigned*)ls.err;
        if (ls.set_cond) cudaGraphSetConditional(newton, (go && !stop) ? 1u : 0u);
    }
}

// ---------------------------------------------------------------------------
// once-per-step bookkeeping

// One block, first kernel of a launch. active[m]: 1 starts a step, 2
// continues a step an iteration budget interrupted, 0 leaves the mesh out
// (a step left unfinished is dropped). Clears the finished flags and the
// launch's iteration count; sets the IF condition of the start-of-step
// kernels (some mesh starts) and the CG loop's while condition (some mesh
// continues); rebuilds the work lists when a running mesh was dropped.
template <typename S>
__global__ void k_reset_counts(BatchView<S> b, LoopSync ls, cudaGraphConditionalHandle if_start,
                               cudaGraphConditionalHandle newton, int newton_form)
{
    int start = 0, cont = 0, dropped = 0;
    for (uint32_t m = threadIdx.x; m < b.M; m += blockDim.x) {
        StepScalars& s = b.st[m];
        const uint8_t a = b.active[m];
        s.finished = 0;
        s.step_done = 0;
        s.nr_go = a == 1 ? 1u : 0u;
        if (a == 1) {
            s.inverted = 0;
            s.fp64_resolved = 0;
            s.res_det_F = s.res_isotropic = s.res_tie = s.res_check = 0;
            s.nr_k = 0;
            s.nr_solved = 0;
            s.fie_cg = 0;
            s.nr_delta0 = 0.0;
            s.nr_abs = 0.0;
            start = 1;
        } else if (a == 2) {
            cont |= s.done ? 0 : 1;
        } else {
            dropped |= s.done ? 0 : 1;
            s.done = 1;
        }
    }
    start = __syncthreads_or(start);
    cont = __syncthreads_or(cont);
    dropped = __syncthreads_or(dropped);
    if (dropped && b.act_tiles) build_active_lists(b);
    build_mesh_lists(
        b, [&](uint32_t m) { return b.active[m] == 1; }, b.start_tiles, b.start_chunks, b.list_count);
    build_mesh_lists(
        b, [&](uint32_t m) { return b.active[m] != 0; }, b.launch_tiles, b.launch_chunks, b.list_count + 2);
    if (threadIdx.x == 0) {
        if (ls.slice) ls.slice[1] = 0u;
        if (ls.set_cond) {
            cudaGraphSetConditional(if_start, start ? 1u : 0u);
            // with a Newton level, the CG loop's condition belongs to the
            // Newton body and is set there, by the start section
            if (newton_form)
                cudaGraphSetConditional(newton, (start || cont) ? 1u : 0u);
            else
                cudaGraphSetConditional(ls.cond, cont ? 1u : 0u);
        }
    }
}

// Per-mesh energies: one block per mesh, fixed-order sum of its tile partials.
template <typename S>
__global__ void k_fin_energy(BatchView<S> b, int kind, const double* __restrict__ tpart)
{
    for (uint32_t m = blockIdx.x; m < b.M; m += gridDim.x) {
        if (!b.st[m].step_done) continue;
        const MeshConsts& c = b.mc[m];
        double acc = 0.0;
        for (uint32_t i = threadIdx.x; i < c.ntiles; i += blockDim.x) acc += tpart[c.tile0 + i];
        const double total = bblock_sum(acc);
        if (threadIdx.x == 0) {
            if (kind == FIN_ENERGY_E) b.st[m].elastic_energy = total;
            else b.st[m].potential_energy = total;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// launchers

template <typename S>
void BatchLaunch<S>::tile_spmv(const BatchView<S>& b, const S* d, const S* r, S* part,
                               cudaGraphConditionalHandle if_refresh, int set_if, const unsigned* refresh_flag,
                               cudaStream_t s)
{
    prof_begin(sizeof(S) == 8 ? "tile_spmv_fp64" : "tile_spmv_mixed", s);
    k_tile_spmv<S><<<b.ntiles ? b.ntiles : 1, kTileElems, 0, s>>>(b, d, r, part, if_refresh, set_if, refresh_flag);
    prof_end(sizeof(S) == 8 ? "tile_spmv_fp64" : "tile_spmv_mixed", s);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::tile_spmv_y64(const BatchView<S>& b, const double* y, double* part64, int refresh,
                                   const unsigned* flag, cudaStream_t s)
{
    const char* name = sizeof(S) == 8 ? "y_product_fp64" : "y_product_mixed";
    prof_begin(name, s);
    k_tile_spmv_y64<S><<<grid_tiles(b.ntiles), kTileElems, 0, s>>>(b, y, part64,
                                                                   refresh ? SPMV_Y64_REFRESH : SPMV_Y64_ALL, flag);
    prof_end(name, s);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::tile_force(const BatchView<S>& b, const double* x, double* part64, double* tile_energy,
                                cudaStream_t s)
{
    prof_begin("tile_force", s);
    k_tile_force<S><<<grid_tiles(b.ntiles), kTileElems, 0, s>>>(b, x, part64, tile_energy);
    prof_end("tile_force", s);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::tile_potential(const BatchView<S>& b, const double* x, double* tile_pe, cudaStream_t s)
{
    k_tile_potential<S><<<grid_tiles(b.ntiles), kTileElems, 0, s>>>(b, x, tile_pe);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::node_b(const BatchView<S>& b, const double* part64, const double* v, const double* x, double* bv,
                            double* y, cudaStream_t s)
{
    k_node_b<S><<<grid_chunks(b.nchunks), kNodeThreads, 0, s>>>(b, part64, v, x, bv, y);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::knc(const BatchView<S>& b, uint32_t K, const double* x, double* bv, double* y, cudaStream_t s)
{
    if (!K) return;
    k_knc<S><<<(K + 255) / 256 < 1024 ? (K + 255) / 256 : 1024, 256, 0, s>>>(b, K, x, bv, y);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::node_residual(const BatchView<S>& b, const double* part64, const double* bv, const double* y,
                                   S* r, S* d, double* cpart, const LoopSync& ls, cudaStream_t s)
{
    k_node_residual<S><<<grid_chunks(b.nchunks), kNodeThreads, 0, s>>>(b, part64, bv, y, r, d, cpart, ls);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::node_q(const BatchView<S>& b, const S* part, S* d, S* q, const double* part64,
                            const double* bv, const double* y, S* r, double* cpart, const LoopSync& ls,
                            cudaStream_t s)
{
    prof_begin(sizeof(S) == 8 ? "node_q_fp64" : "node_q_mixed", s);
    k_node_q<S><<<b.nchunks ? b.nchunks : 1, kNodeThreads, 0, s>>>(b, part, d, q, part64, bv, y, r, cpart, ls);
    prof_end(sizeof(S) == 8 ? "node_q_fp64" : "node_q_mixed", s);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::node_update(const BatchView<S>& b, double* y, S* r, const S* d, S* q, double* cpart,
                                 const LoopSync& ls, cudaStream_t s)
{
    k_node_update<S><<<b.nchunks ? b.nchunks : 1, kNodeThreads, 0, s>>>(b, y, r, d, q, cpart, ls);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::node_mr_finish(const BatchView<S>& b, double* y, S* r, S* d, const S* q, const LoopSync& ls,
                                    cudaStream_t s)
{
    k_node_mr_finish<S><<<grid_chunks(b.nchunks), kNodeThreads, 0, s>>>(b, y, r, d, q, ls);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::integrate(const BatchView<S>& b, double* x, double* v, const double* y, double* cpart,
                               const LoopSync& ls, cudaStream_t s)
{
    k_integrate<S><<<grid_chunks(b.nchunks), kNodeThreads, 0, s>>>(b, x, v, y, cpart, ls);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::lock_phase(const BatchView<S>& b, int phase, cudaStream_t s)
{
    k_lock_phase<S><<<1, 256, 0, s>>>(b, phase);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::newton_tail(const BatchView<S>& b, const LoopSync& ls, cudaGraphConditionalHandle newton,
                                 cudaStream_t s)
{
    k_newton_tail<S><<<1, 256, 0, s>>>(b, ls, newton);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::fin_energy(const BatchView<S>& b, int kind, const double* tpart, cudaStream_t s)
{
    k_fin_energy<S><<<b.M < 4096 ? b.M : 4096, 256, 0, s>>>(b, kind, tpart);
    launch_counter()++;
}

template <typename S>
void BatchLaunch<S>::reset_counts(const BatchView<S>& b, const LoopSync& ls, cudaGraphConditionalHandle if_start,
                                   cudaGraphConditionalHandle newton, int newton_form, cudaStream_t s)
{
    k_reset_counts<S><<<1, 256, 0, s>>>(b, ls, if_start, newton, newton_form);
    launch_counter()++;
}

// One mesh's element material triple re-baked from scalar values (k0, k1,
// k2 = a (1 - nu), a nu, a (0.5 - nu), formed on the host):
// mat[c][e] = V_e k_c, rounded to the path's type, and on the mixed path the
// tile blobs' V lambda and V mu -- the values a batch built with those
// scalars holds (EditableTetrahedronElementSet3::SetParams,
// TetrahedronElementSet3.cpp:2168-2200). The mesh's tiles and element
// range; the material of its tiles set to `material`.
template <typename S>
__global__ void k_rebake_mesh(BatchView<S> b, uint32_t tile0, uint32_t ntiles, double k0, double k1, double k2,
                              int rebake, uint16_t material)
{
    S* mat = const_cast<S*>(b.mat);
    const size_t T = b.Ttot;
    for (uint32_t i = blockIdx.x; i < ntiles; i += gridDim.x) {
        const uint32_t t = tile0 + i;
        const TileMeta tm = b.tiles[t];
        if (threadIdx.x == 0) const_cast<TileMeta*>(b.tiles)[t].material = material;
        if (!rebake || threadIdx.x >= tm.ne) continue;
        const size_t e = tm.e0 + threadIdx.x;
        const double V = b.vol[e];
        const double m0 = V * k0, m1 = V * k1, m2 = V * k2;
        mat[e] = (S)m0;
        mat[T + e] = (S)m1;
        mat[2 * T + e] = (S)m2;
        if (b.blob) {
            unsigned char* base = b.blob + 16ull * b.blob_off16[t];
            const uint32_t ne4 = blob_ne4(tm.ne);
            *reinterpret_cast<float*>(base + blob_comp_off(18, threadIdx.x, ne4)) = (float)m1;
            *reinterpret_cast<float*>(base + blob_comp_off(19, threadIdx.x, ne4)) = (float)m2;
        }
    }
}

template <typename S>
void launch_rebake_mesh(const BatchView<S>& b, uint32_t tile0, uint32_t ntiles, double k0, double k1, double k2,
                        int rebake, uint16_t material, cudaStream_t s)
{
    if (!ntiles) return;
    k_rebake_mesh<S><<<ntiles < 1216u ? ntiles : 1216u, kTileElems, 0, s>>>(b, tile0, ntiles, k0, k1, k2, rebake,
                                                                          material);
    launch_counter()++;
}
template void launch_rebake_mesh<double>(const BatchView<double>&, uint32_t, uint32_t, double, double, double, int,
                                         uint16_t, cudaStream_t);
template void launch_rebake_mesh<float>(const BatchView<float>&, uint32_t, uint32_t, double, double, double, int,
                                        uint16_t, cudaStream_t);

__global__ void k_permute(const uint32_t* __restrict__ perm, uint64_t n, const double* __restrict__ src,
                          double* __restrict__ dst, int to_batch)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = perm[i];
        const uint64_t di = to_batch ? i : p, si = to_batch ? p : i;
#pragma unroll
        for (int a = 0; a < 3; a++) dst[3 * di + a] = src[3 * si + a];
    }
}

void launch_permute(const uint32_t* perm, uint64_t n, const double* src, double* dst, bool to_batch, cudaStream_t s)
{
    if (n == 0) return;
    const uint64_t blocks = (n + 255) / 256;
    k_permute<<<blocks < 152 * 16 ? (unsigned)blocks : 152u * 16u, 256, 0, s>>>(perm, n, src, dst, to_batch ? 1 : 0);
    launch_counter()++;
}

uint32_t grid_tiles(uint32_t ntiles)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    const uint32_t cap = (uint32_t)sms * 8u;
    return ntiles < cap ? (ntiles ? ntiles : 1) : cap;
}

uint32_t grid_chunks(uint32_t nchunks)
{
    const uint32_t cap = 152u * 8u;
    return nchunks < cap ? (nchunks ? nchunks : 1) : cap;
}

template struct BatchLaunch<double>;
template struct BatchLaunch<float>;

FEMGB_BOUNDS_ACCESSOR(bounds_read_batch_kernels)

}  // namespace femgb
