// refresh_product.cuh -- the product of the CG iterate y for the residual
// b - A y on the batch's tiles (k_tile_spmv_y64 and the persistent CG kernel
// of the mixed path run the same pass), and the per-mesh helpers it uses.
#pragma once
#include "active_list.cuh"
#include "batch.cuh"
#include "bounds.cuh"
#include "df.cuh"
#include "elem_math.cuh"
#include "lcm.cuh"

namespace femgb {

template <typename S>
__device__ __forceinline__ bool mesh_running(const BatchView<S>& b, uint32_t m)
{
    return !b.st[m].done;
}

// The CG iterate: FP64 y plus, on the mixed path, the FP32 sum of this
// step's alpha d increments (folded in at refresh and integration).
template <typename S>
__device__ __forceinline__ double y_full(const BatchView<S>& b, const double* y, size_t i)
{
    return b.ydelta ? y[i] + (double)b.ydelta[i] : y[i];
}

// Whether the mesh's next iteration recomputes its residual in FP64 (set by
// the last block of the mesh in the node pass, see refresh_decide).
__device__ __forceinline__ bool refresh_now(const MeshConsts&, const StepScalars& s) { return s.refresh_next != 0; }

// The P-K product of element e of `mesh` (the tile's material: C_LCM,
// C_LCMH or C_CCM): in FP64 the FP64 solid's own arithmetic (pk_dforce, on
// the F and det F of the last evaluation), otherwise the folded forms of
// elem_math.cuh on the element's V lambda and V mu (C_LCMH with its blend
// weight of the last evaluation; the mixed path takes no C_CCM).
template <typename S>
__device__ __forceinline__ void elem_pk(const BatchView<S>& b, uint32_t material, uint32_t mesh, size_t e,
                                        const double* R, const double* Di, double, double, const double* dl,
                                        double* out)
{
    const MeshConsts& c = b.mc[mesh];
    if (material == kTileMaterialLcm) {
        lcm_dforce(R, Di, b.vol[e], c.lame_mu, c.lame_lambda, dl, out);
        return;
    }
    double F[9];
    const size_t T = b.Ttot;
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = b.Fe[k * T + e];
    const PkMaterial m{(int)material, c.lame_mu, c.lame_lambda, c.ecie_k};
    pk_dforce(m, R, F, b.detF[e], Di, b.vol[e], dl, out);
}
template <typename S, typename V>
__device__ __forceinline__ void elem_pk(const BatchView<S>& b, uint32_t material, uint32_t, size_t e,
                                        const float* R, const float* Di, float kl, float km, const V* dl, V* out)
{
    if (material == kTileMaterialLcmh)
        elem_lcmh_dforce<V, float>(R, Di, kl, km, b.lcmh_w[e], dl, out);
    else
        elem_lcm_dforce<V, float>(R, Di, kl, km, dl, out);
}

// Product of the iterate y for the residual b - A y (same element data):
// mode SPMV_Y64_ALL for every active mesh (initial residual of a step);
// mode SPMV_Y64_REFRESH for meshes refreshing their residual this iteration,
// and only when the finaliser raised the batch's refresh flag (otherwise the
// launch returns at once). The FP64 path evaluates it in FP64. The mixed
// path, whose element data is FP32, evaluates it in double-float arithmetic
// (about 48 bits; FP64 would cost about 60 times the FP32 rate on this GPU)
// and writes FP64 partial sums, so its residual is accurate to about 1e-14
// of the magnitudes of the terms of A y.
enum { SPMV_Y64_ALL = 0, SPMV_Y64_REFRESH = 1 };

template <typename S>
struct Y64Value {
    using T = double;
};
template <>
struct Y64Value<float> {
    using T = DF;
};
__device__ __forceinline__ void y64_set(double& a, double v) { a = v; }
__device__ __forceinline__ void y64_set(DF& a, double v) { a = df_from_double(v); }
__device__ __forceinline__ double y64_get(double a) { return a; }
__device__ __forceinline__ double y64_get(DF a) { return df_to_double(a); }

// One pass of the product by this block over its entries block, block + G,
// ... of the mode's tile list; sd (3 kTileNodes values) and so (12
// kTileElems values) are the block's shared-memory staging.
template <typename S>
__device__ __forceinline__ void tile_spmv_y64_pass(const BatchView<S>& b, const double* y, double* part64, int mode,
                                                   typename Y64Value<S>::T* sd, typename Y64Value<S>::T* so,
                                                   const uint32_t block, const uint32_t G)
{
    using V = typename Y64Value<S>::T;
    // ALL: the meshes that start a step; REFRESH: the meshes that refresh in
    // this iteration (their work list on the mixed path, or the CG list when
    // all running meshes refresh)
    const uint32_t rc = (mode == SPMV_Y64_REFRESH && b.refresh_tiles) ? b.list_count[4] : 0u;
    const bool cg_list = rc == kRefreshUsesCgList;
    const uint32_t* list = mode == SPMV_Y64_ALL ? b.start_tiles : (cg_list ? b.act_tiles : b.refresh_tiles);
    const uint32_t n = mode == SPMV_Y64_ALL ? b.list_count[0]
                       : !b.refresh_tiles ? b.ntiles
                       : cg_list ? *(volatile const uint32_t*)b.act_count
                                 : rc;
    for (uint32_t i = block; i < n; i += G) {
        const uint32_t t = list_entry(list, i);
        const TileMeta tm = b.tiles[t];
        if (mode == SPMV_Y64_ALL && !mesh_starts(b, tm.mesh)) continue;
        if (mode == SPMV_Y64_REFRESH && (!mesh_running(b, tm.mesh) || !refresh_now(b.mc[tm.mesh], b.st[tm.mesh])))
            continue;
        const uint16_t* lp = b.lptr + b.lptr0[t];
        const uint16_t* li = b.lidx + tm.c0;
        for (int i = threadIdx.x; i < tm.nn; i += blockDim.x) {
            const size_t g = bounds_idx(b.tile_nodes[tm.n0 + i], b.Ntot, kSiteBatchNode);
            y64_set(sd[i], y_full(b, y, 3 * g));
            y64_set(sd[kTileNodes + i], y_full(b, y, 3 * g + 1));
            y64_set(sd[2 * kTileNodes + i], y_full(b, y, 3 * g + 2));
        }
        __syncthreads();
        if (threadIdx.x < tm.ne) {
            const size_t e = tm.e0 + threadIdx.x;
            const size_t T = b.Ttot;
            S R[9], Di[9];
#pragma unroll
            for (int c = 0; c < 9; c++) R[c] = b.R[c * T + e];
#pragma unroll
            for (int c = 0; c < 9; c++) Di[c] = b.Dinv[c * T + e];
            const S k1 = b.mat[e], knu = b.mat[T + e], k2 = b.mat[2 * T + e];
            const uchar4 lc = b.lconn[e];
            const int ids[4] = {(int)bounds_idx((uint32_t)lc.x, tm.nn, kSiteLocalNode),
                            (int)bounds_idx((uint32_t)lc.y, tm.nn, kSiteLocalNode),
                            (int)bounds_idx((uint32_t)lc.z, tm.nn, kSiteLocalNode),
                            (int)bounds_idx((uint32_t)lc.w, tm.nn, kSiteLocalNode)};
            V dl[12];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                dl[3 * i] = sd[ids[i]];
                dl[3 * i + 1] = sd[kTileNodes + ids[i]];
                dl[3 * i + 2] = sd[2 * kTileNodes + ids[i]];
            }
            V out[12];
            if (tm.material != kTileMaterialWrp)
                elem_pk(b, tm.material, tm.mesh, e, R, Di, knu, k2, dl, out);
            else
                elem_RKRt<V, S>(R, Di, k1, knu, k2, dl, out);
#pragma unroll
            for (int c = 0; c < 12; c++) so[c * kTileElems + threadIdx.x] = out[c];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < tm.nn; i += blockDim.x) {
            V a0{}, a1{}, a2{};
            for (int j = lp[i]; j < lp[i + 1]; j++) {
                const int v = li[j], el = v >> 2, sl = v & 3;
                a0 = a0 + so[(3 * sl) * kTileElems + el];
                a1 = a1 + so[(3 * sl + 1) * kTileElems + el];
                a2 = a2 + so[(3 * sl + 2) * kTileElems + el];
            }
            const size_t o = 3 * tile_slot(b.ov_map, tm.own0, tm.ov0, tm.nown, i);
            part64[o] = y64_get(a0);
            part64[o + 1] = y64_get(a1);
            part64[o + 2] = y64_get(a2);
        }
        __syncthreads();
    }
}

}  // namespace femgb
