// bounds.cuh -- optional index checks of the kernels' data-dependent
// indices (node ids read from element tables, CSR entries, tile-local ids,
// partial slots, constraint nodes). Built in only with -DFEM_BOUNDS_CHECK
// (a separate library, build.build_bounds_check()): a bad index is then
// counted in a device error word, the first one's site, index and limit are
// kept, and the access uses index 0 instead, so a corrupted table shows up
// as a status instead of a memory fault. Without the define every check
// compiles to the index itself.
//
// Each translation unit that includes this header has its own error word
// (no relocatable device code); FEMGB_BOUNDS_ACCESSOR(name) defines the
// host function that reads and clears it, and fem_bounds_check_status sums
// them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace femgb {

// sites (the first failure's `site`)
enum BoundsSite : uint32_t {
    kSiteElemNode = 1,     // FP64 solid: node id of an element >= N
    kSiteCsrEntry = 2,     // FP64 solid: node CSR entry >= 4 T
    kSiteKncNode = 3,      // constraint node >= N (Ntot)
    kSiteBatchNode = 4,    // batch: node id (element table, tile node list) >= Ntot
    kSiteLocalNode = 5,    // batch: tile-local node id >= the tile's node count
    kSitePartialSlot = 6,  // batch: partial slot >= the batch's slot count
    kSiteTileEntry = 7,    // batch: tile-local CSR entry >= 4 ne4
    kSiteBsrEntry = 8,     // FP64 solid: assembled block's column >= N, or its element >= T
};

#ifdef FEM_BOUNDS_CHECK
static __device__ unsigned g_fem_bounds[4];  // failures, first site, index, limit

static __device__ __noinline__ void bounds_record(uint32_t site, uint64_t idx, uint64_t limit)
{
    if (atomicAdd(&g_fem_bounds[0], 1u) == 0u) {
        g_fem_bounds[1] = site;
        g_fem_bounds[2] = (unsigned)idx;
        g_fem_bounds[3] = (unsigned)limit;
    }
}

template <typename I>
__device__ __forceinline__ I bounds_idx(I idx, uint64_t limit, uint32_t site)
{
    if ((uint64_t)idx < limit) return idx;
    bounds_record(site, (uint64_t)idx, limit);
    return (I)0;
}

#define FEMGB_BOUNDS_ACCESSOR(name)                                                      \
    int name(unsigned* out)                                                              \
    {                                                                                    \
        static const unsigned zero[4] = {0u, 0u, 0u, 0u};                                \
        cudaError_t e = cudaMemcpyFromSymbol(out, g_fem_bounds, sizeof(unsigned) * 4);   \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_fem_bounds, zero, sizeof(zero));  \
        return e == cudaSuccess ? 0 : 1;                                                 \
    }
#else
template <typename I>
__device__ __forceinline__ I bounds_idx(I idx, uint64_t, uint32_t)
{
    return idx;
}

#define FEMGB_BOUNDS_ACCESSOR(name)            \
    int name(unsigned* out)                    \
    {                                          \
        out[0] = out[1] = out[2] = out[3] = 0; \
        return 0;                              \
    }
#endif

// the per-unit accessors (fem_kernels.cu, rotation.cu, batch_kernels.cu,
// tile_pipe.cu)
int bounds_read_fem_kernels(unsigned* out);
int bounds_read_rotation(unsigned* out);
int bounds_read_batch_kernels(unsigned* out);
int bounds_read_tile_pipe(unsigned* out);

}  // namespace femgb
