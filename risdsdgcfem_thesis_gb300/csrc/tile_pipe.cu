// tile_pipe.cu -- the mixed-precision element-tile product as a persistent,
// double-buffered pipeline: each tile's element data, tile-local CSR and
// node list form one contiguous 16-byte-aligned blob in HBM, copied into
// shared memory by one bulk asynchronous copy (cp.async.bulk, completion on
// an mbarrier) while the block computes the previous tile.
//
// Blob of a tile with ne elements (ne4 = ne rounded up to 4) and nn local
// nodes, all offsets from the blob start:
//   0                 float comp[22][ne4]: R (9), Dm^-1 (9), V(lambda+2mu),
//                     V lambda, V mu, local ids (uchar4 as one word)
//   88 ne4            uint16 lptr[nn+1]   tile-local CSR offsets
//   + 2(nn+1)         uint16 lidx[4 ne]   (slot << 8 | element), element order
//   (4-aligned)       uint32 nodes[nn]    global node id of each local node
//   size rounded up to 16.
//
// Waits on the mbarrier are bounded: a wait that gives up records an error
// code in the batch's error word and the block stops (after waiting, again
// bounded, for any copy it issued).
#include "batch.cuh"
#include "batch_launch.h"
#include "elem_math.cuh"

namespace femgb {

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: ~2^22 polls (each poll itself suspends for a hardware
// time slice), far above any copy's latency.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    for (uint32_t i = 0; i < (1u << 22); i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

}  // namespace

constexpr uint32_t kStageBytes = 26240;  // >= blob_bytes(256, 256), multiple of 128
static_assert(kStageBytes >= 26128, "stage must hold the largest tile blob");

__device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Shared memory: two blob stages, two gather stages (d and r of each local
// node, [6][256] floats), the staged direction sd4 and the outputs so4.
constexpr uint32_t kGatherBytes = 6u * kTileNodes * 4u;

__global__ void __launch_bounds__(256) k_tile_spmv_pipe(BatchView<float> b, const float* __restrict__ dvec,
                                                        const float* __restrict__ rvec, float* __restrict__ part,
                                                        cudaGraphConditionalHandle if_refresh, int set_if,
                                                        const unsigned* __restrict__ refresh_flag,
                                                        unsigned* __restrict__ err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    float* gbuf = reinterpret_cast<float*>(smem + 2 * kStageBytes);           // [2][6][256]
    float4* sd4 = reinterpret_cast<float4*>(smem + 2 * kStageBytes + 2 * kGatherBytes);
    float4* so4 = sd4 + kTileNodes;  // slot-major: so4[slot * 256 + element]
    uint64_t* bar = reinterpret_cast<uint64_t*>(so4 + 4 * kTileElems);

    if (set_if && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(if_refresh, *refresh_flag ? 1u : 0u);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto active = [&](uint32_t t) -> bool { return t < b.ntiles && !b.st[b.tiles[t].mesh].done; };
    auto issue_blob = [&](uint32_t t, int s) {
        const TileMeta tm = b.tiles[t];
        const uint32_t bytes = blob_bytes(tm.ne, tm.nn);
        mbar_expect_tx(&bar[s], bytes);
        bulk_copy_g2s(smem + s * kStageBytes, b.blob + 16ull * b.blob_off16[t], bytes, &bar[s]);
    };
    // d and r of local node i of a tile into gather stage s (this thread's copies)
    auto issue_gather = [&](uint32_t g, int s) {
        float* gs = gbuf + s * 6 * kTileNodes + threadIdx.x;
        const float* dp = dvec + 3 * (size_t)g;
        const float* rp = rvec + 3 * (size_t)g;
        cp_async4(gs, dp);
        cp_async4(gs + kTileNodes, dp + 1);
        cp_async4(gs + 2 * kTileNodes, dp + 2);
        cp_async4(gs + 3 * kTileNodes, rp);
        cp_async4(gs + 4 * kTileNodes, rp + 1);
        cp_async4(gs + 5 * kTileNodes, rp + 2);
    };

    uint32_t phase = 0u;    // bit s: parity of stage s's next completion
    uint32_t pending = 0u;  // bit s: a bulk copy into stage s is in flight
    uint32_t t = blockIdx.x;
    bool act = active(t);
    if (act) {
        const TileMeta tm = b.tiles[t];
        if (threadIdx.x == 0) issue_blob(t, 0);
        pending |= 1u;
        if (threadIdx.x < tm.nn) issue_gather(b.tile_nodes[tm.n0 + threadIdx.x], 0);
    }
    cp_async_commit();
    int s = 0;
    bool failed = false;
    for (; t < b.ntiles; t += gridDim.x) {
        const uint32_t tn = t + gridDim.x;
        // after a failed wait no new copies are issued
        const bool actn = !failed && active(tn);
        TileMeta tmn;
        uint32_t gn = 0;
        if (actn) {
            tmn = b.tiles[tn];
            if (threadIdx.x == 0) issue_blob(tn, s ^ 1);
            pending |= 1u << (s ^ 1);
            if (threadIdx.x < tmn.nn) gn = b.tile_nodes[tmn.n0 + threadIdx.x];  // used after this tile's compute
        }
        if (act) {
            // every thread polls; the block agrees on the outcome so the
            // barriers below stay uniform
            const bool ok = !failed && mbar_wait_bounded(&bar[s], (phase >> s) & 1u);
            if (__syncthreads_or(!ok)) {
                if (!failed && threadIdx.x == 0) atomicExch(err, 1u);
                failed = true;
            } else {
                phase ^= 1u << s;
                pending &= ~(1u << s);
            }
        }
        const TileMeta tm = b.tiles[t < b.ntiles ? t : 0];
        if (act && !failed) {
            cp_async_wait_all();  // this thread's gathers of tile t
            __syncthreads();
            const float beta = (float)b.st[tm.mesh].beta;
            const float* gs = gbuf + s * 6 * kTileNodes;
            if (threadIdx.x < tm.nn) {
                const int i = threadIdx.x;
                sd4[i] = make_float4(__fmaf_rn(beta, gs[i], gs[3 * kTileNodes + i]),
                                     __fmaf_rn(beta, gs[kTileNodes + i], gs[4 * kTileNodes + i]),
                                     __fmaf_rn(beta, gs[2 * kTileNodes + i], gs[5 * kTileNodes + i]), 0.f);
            }
            __syncthreads();
            const unsigned char* stage = smem + s * kStageBytes;
            const uint32_t ne4 = blob_ne4(tm.ne);
            const float* comp = reinterpret_cast<const float*>(stage);
            if (threadIdx.x < tm.ne) {
                const int i = threadIdx.x;
                float R[9], Di[9];
#pragma unroll
                for (int c = 0; c < 9; c++) R[c] = comp[c * ne4 + i];
#pragma unroll
                for (int c = 0; c < 9; c++) Di[c] = comp[(9 + c) * ne4 + i];
                const float k1 = comp[18 * ne4 + i], knu = comp[19 * ne4 + i], k2 = comp[20 * ne4 + i];
                const uint32_t lw = reinterpret_cast<const uint32_t*>(comp)[21 * ne4 + i];
                const int ids[4] = {(int)(lw & 0xff), (int)((lw >> 8) & 0xff), (int)((lw >> 16) & 0xff),
                                    (int)(lw >> 24)};
                float dl[12];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float4 v = sd4[ids[k]];
                    dl[3 * k] = v.x;
                    dl[3 * k + 1] = v.y;
                    dl[3 * k + 2] = v.z;
                }
                float out[12];
                elem_RKRt<float>(R, Di, k1, knu, k2, dl, out);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    so4[k * kTileElems + i] = make_float4(out[3 * k], out[3 * k + 1], out[3 * k + 2], 0.f);
            }
        }
        // the next tile's gathers go out while this tile reduces
        if (actn && threadIdx.x < tmn.nn) issue_gather(gn, s ^ 1);
        cp_async_commit();
        if (act && !failed) {
            __syncthreads();
            const unsigned char* stage = smem + s * kStageBytes;
            const uint16_t* lp = reinterpret_cast<const uint16_t*>(stage + blob_lptr_off(tm.ne));
            const uint16_t* li = lp + (tm.nn + 1);
            if (threadIdx.x < tm.nn) {
                const int i = threadIdx.x;
                float a0 = 0.f, a1 = 0.f, a2 = 0.f;
                for (int j = lp[i]; j < lp[i + 1]; j++) {
                    const float4 v = so4[li[j]];
                    a0 += v.x;
                    a1 += v.y;
                    a2 += v.z;
                }
                const size_t o = 3 * (size_t)(tm.n0 + i);
                part[o] = a0;
                part[o + 1] = a1;
                part[o + 2] = a2;
            }
        }
        __syncthreads();
        act = actn;
        s ^= 1;
    }
    // drain: every copy this block issued completes before it exits (bounded)
    cp_async_wait_all();
    if (failed) {
        for (int k = 0; k < 2; k++)
            if ((pending >> k) & 1u) (void)mbar_wait_bounded(&bar[k], (phase >> k) & 1u);
    }
}

uint32_t tile_pipe_smem_bytes()
{
    return 2 * kStageBytes + 2 * kGatherBytes + sizeof(float4) * (kTileNodes + 4 * kTileElems) + 2 * sizeof(uint64_t);
}

static int pipe_grid()
{
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_tile_spmv_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tile_pipe_smem_bytes());
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_spmv_pipe, 256, tile_pipe_smem_bytes());
        if (sms <= 0) sms = 152;
        if (per_sm <= 0) per_sm = 1;
        grid = sms * per_sm;
    }
    return grid;
}

void launch_tile_spmv_pipe(const BatchView<float>& b, const float* d, const float* r, float* part,
                           cudaGraphConditionalHandle if_refresh, int set_if, const unsigned* refresh_flag,
                           unsigned* err, cudaStream_t s)
{
    const int g = pipe_grid();
    const uint32_t grid = b.ntiles < (uint32_t)g ? (b.ntiles ? b.ntiles : 1) : (uint32_t)g;
    prof_begin("tile_spmv_mixed", s);
    k_tile_spmv_pipe<<<grid, 256, tile_pipe_smem_bytes(), s>>>(b, d, r, part, if_refresh, set_if, refresh_flag, err);
    prof_end("tile_spmv_mixed", s);
    launch_counter()++;
}

void prepare_tile_pipe() { (void)pipe_grid(); }

}  // namespace femgb
