// active_list.cuh -- work lists of a batch launch: the tiles and node chunks
// of a set of meshes, in mesh order.
//
//  * CG lists (mixed path): meshes whose CG loop is running. The last block
//    of a node pass rebuilds them when the set has changed; the tile product
//    and the node pass walk them instead of every tile and chunk of the
//    batch, so an iteration costs what its running meshes cost.
//  * start lists: meshes that start a step in this launch (active mask 1),
//    walked by the start-of-step kernels;
//  * launch lists: meshes that take part in this launch (mask 1 or 2),
//    walked by integration and energies.
// The start and launch lists are built by the launch's first kernel (one
// block).
#pragma once
#include "batch.cuh"

namespace femgb {

// Exclusive block scan of one value per thread (blockDim.x <= 1024, a
// multiple of 32); returns this thread's offset, *total the block's sum.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* sh, uint32_t* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < nw ? sh[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) sh[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t before = wid ? sh[wid - 1] : 0u;
    *total = sh[nw - 1];
    __syncthreads();
    return before + x - v;
}

// Tiles and chunks of the meshes m with pred(m), in mesh order, into
// tiles[] / chunks[] and their counts into count2[0..1]. Called by every
// thread of one block.
template <typename S, typename P>
__device__ void build_mesh_lists(const BatchView<S>& b, P pred, uint32_t* tiles, uint32_t* chunks,
                                 uint32_t* count2)
{
    __shared__ uint32_t sh[32];
    const uint32_t per = (b.M + blockDim.x - 1) / blockDim.x;
    const uint32_t m0 = threadIdx.x * per, m1 = min(b.M, m0 + per);
    uint32_t nt = 0, nc = 0;
    for (uint32_t m = m0; m < m1; m++) {
        if (pred(m)) {
            nt += b.mc[m].ntiles;
            nc += b.mc[m].nchunks;
        }
    }
    uint32_t tot_t, tot_c;
    uint32_t pt = block_excl_scan(nt, sh, &tot_t);
    uint32_t pc = block_excl_scan(nc, sh, &tot_c);
    for (uint32_t m = m0; m < m1; m++) {
        if (!pred(m)) continue;
        const MeshConsts& c = b.mc[m];
        for (uint32_t k = 0; k < c.ntiles; k++) tiles[pt++] = c.tile0 + k;
        for (uint32_t k = 0; k < c.nchunks; k++) chunks[pc++] = c.chunk0 + k;
    }
    if (threadIdx.x == 0) {
        count2[0] = tot_t;
        count2[1] = tot_c;
    }
    __syncthreads();
}

// The CG work lists: meshes whose loop is running. Called by every thread
// of one block, after every other block of the grid has finished its writes
// to the meshes' done flags.
template <typename S>
__device__ void build_active_lists(const BatchView<S>& b)
{
    build_mesh_lists(
        b, [&](uint32_t m) { return ((volatile const StepScalars*)(b.st + m))->done == 0u; }, b.act_tiles,
        b.act_chunks, b.act_count);
    if (threadIdx.x == 0) *b.list_dirty = 0u;
}

// The tiles of the meshes whose next iteration recomputes the residual in
// FP64 (walked by the FP64 product of y). Same calling rule as above.
template <typename S>
__device__ void build_refresh_lists(const BatchView<S>& b)
{
    build_mesh_lists(
        b,
        [&](uint32_t m) {
            volatile const StepScalars* sp = b.st + m;
            return sp->done == 0u && sp->refresh_next != 0u;
        },
        b.refresh_tiles, b.refresh_chunks, b.list_count + 4);
}

// list_count[4] when every running mesh refreshes: the refresh product walks
// the CG list itself (no copy; its per-tile test skips the meshes that have
// left their loop).
constexpr uint32_t kRefreshUsesCgList = 0xffffffffu;

// The refresh work list of the next iteration; `all` = every running mesh
// refreshes (then the CG list serves and nothing is copied: in a batch whose
// meshes started together that is every periodic refresh, while exit
// confirmations and staggered starts give short lists). Same calling rule
// as above.
template <typename S>
__device__ void set_refresh_lists(const BatchView<S>& b, bool all)
{
    if (all && b.act_tiles) {
        if (threadIdx.x == 0) b.list_count[4] = kRefreshUsesCgList;
        __syncthreads();
    } else {
        build_refresh_lists(b);
    }
}

// Entry i of a work list, or i itself when the launch has no list.
__device__ __forceinline__ uint32_t list_entry(const uint32_t* list, uint32_t i) { return list ? list[i] : i; }

}  // namespace femgb
