// tile_pipe.cu -- one CG iteration of the mixed-precision path in three kernels
// (Saphyre2 ns/ILSS_CG.h:90-144, every running mesh of the batch in
// lock-step).
//
// k_tile_spmv_pipe: persistent, double-buffered element-tile product. Each
// tile's element data, tile-local CSR and node list form one contiguous
// 16-byte-aligned blob in HBM, copied into shared memory by one bulk
// asynchronous copy (cp.async.bulk, completion on an mbarrier) while the
// block computes the previous tile. The tile stages the new direction
// d = S(r + beta d) of its nodes, forms one element's R K0 R^T d per thread
// and sums the outputs per local node (tile-local CSR, element order) into
// one partial per (tile, node). The gathers of d and r for the next tile
// are issued into registers before the current tile is computed, so their
// latency overlaps a whole tile. The tile also forms its share of d^T A d:
//     fK * sum_e d_e . (R K0 R^T d)_e  +  m fM * sum_{nodes it owns} |d_n|^2,
// which sums to d^T S A d (ILSS_CG.h:91-96) because d is zero on constrained
// rows; a node is owned by the first tile (in tile order) that lists it, and
// its owner writes its partial in node order (the node pass reads it
// coalesced; shared nodes' other partials go to overflow slots).
//
// k_mesh_alpha: one warp per running mesh sums its tiles' shares (fixed
// order) and forms alpha, or the breakdown flag (ILSS_CG.h:97).
//
// k_node_update_fused: per node of the running meshes: d = S(r + beta d) (the
// values the tiles staged), q = S(fK sum(partials) + m fM d), y += alpha d
// (into the FP32 increment accumulator), r -= alpha q (on refresh iterations
// r is first recomputed as S(b - A y) from the product of y), and one
// (hi, lo) share of |r|^2 per node chunk; a mesh that breaks down leaves its
// loop before the update.
//
// k_mesh_update: one warp per running mesh sums its chunk shares (fixed
// order) and forms beta and the loop test (ILSS_CG.h:100-144); the last
// block of the grid sets the CUDA-graph while condition and the refresh
// flag. The per-mesh reductions thus need no arrival counters, fences or
// atomics inside the streaming kernels.
//
// Blob of a tile with ne elements (ne4 = ne rounded up to 4) and nn local
// nodes, offsets from the blob start:
//   0            element data, 21 FP32 components per element: R (9),
//                Dm^-1 (9), V lambda, V mu, local ids (uchar4 as one word), in
//                groups of four: float4 g[5][ne4] (components 0-19), then
//                uint32 [ne4] (component 20); V(lambda+2mu) = V lambda + 2 V mu
//   84 ne4       uint16 lptr[nn+1]      tile-local CSR offsets
//   + 2(nn+1)    uint16 lidx[4 ne]      slot * ne4 + element, element order
//   (4-aligned)  uint32 own0; float fK, m fM   partial slot of the first owned
//                                         node (local node i < nown -> part[own0 + i]);
//                                         the mesh's FP32 factors
//   + 12         uint32 ovslot[nn - nown] partial slots of the shared local nodes
//   size rounded up to 16. The batch node ids of the tile's local nodes
//   (its owned nodes first) are read from the batch's tile node list, ahead
//   of the blob.
//
// Every wait on an mbarrier is bounded: a wait that gives up records an error
// code in the batch's error word (err[0] = 1; its poll limit is err[1]); the
// block then issues no further copies and drains, again bounded (2^22 polls),
// the copies it has in flight, recording err[0] = 2 if even that drain gives
// up. The CG loop stops at the end of an iteration in which the error word is
// set.
#include "active_list.cuh"
#include "batch.cuh"
#include "batch_launch.h"
#include "bounds.cuh"
#include "elem_math.cuh"
#include "refresh_product.cuh"

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

// Bounded wait: at most `polls` polls (each poll itself suspends for a
// hardware time slice). The drain at the end of the kernel uses the full
// kDrainPolls; the waits for each tile's copy use the batch's limit
// (fem_batch_set_wait_limit, default kDrainPolls, far above any copy's
// latency; 0 makes every such wait give up at once, which exercises the
// error path without a stuck copy).
constexpr uint32_t kDrainPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t polls)
{
    for (uint32_t i = 0; i < polls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Unevaluated sum hi + lo of two floats (about 48 significant bits). The
// mixed path keeps its reductions in FP32 this way: GB300's FP64 pipe runs
// at a small fraction of the FP32 rate, and even a block's reduction tree
// in FP64 shows up in a kernel's time. Every tree below is fixed, so a sum
// does not depend on scheduling.
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 f2_add(F2 a, F2 b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    F2 r;
    r.hi = s + e;
    r.lo = e - (r.hi - s);
    return r;
}

__device__ __forceinline__ F2 warp_sum_f2(F2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        F2 w;
        w.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
        v = f2_add(v, w);
    }
    return v;
}

// This lane's part of a lane-strided sum of n (hi, lo) shares: k = lane,
// lane + 32, ... added in that order, the loads of each round of eight
// issued together (a mesh with hundreds of tiles would otherwise wait on a
// chain of dependent global loads).
__device__ __forceinline__ F2 lane_share_sum(const float2* p, uint32_t n, uint32_t lane)
{
    F2 a = {0.f, 0.f};
    for (uint32_t k0 = lane; k0 < n; k0 += 256u) {
        float2 w[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const uint32_t k = k0 + 32u * i;
            w[i] = k < n ? __ldcg(p + k) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int i = 0; i < 8; i++)
            if (k0 + 32u * i < n) a = f2_add(a, F2{w[i].x, w[i].y});
    }
    return a;
}

// Block sum, result valid in thread 0; every thread must call it.
__device__ __forceinline__ F2 block_sum_f2(F2 v, float2* sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    v = warp_sum_f2(v);
    if (lane == 0) sh[wid] = make_float2(v.hi, v.lo);
    __syncthreads();
    if (wid == 0) {
        const float2 w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : make_float2(0.f, 0.f);
        v.hi = w.x;
        v.lo = w.y;
        v = warp_sum_f2(v);
    }
    return v;
}

// Arrival of a block on a counter: the values other blocks must see are
// written by thread 0, which alone fences before arriving; the last arrival
// resets the counter. Every thread must call it.
__device__ __forceinline__ bool arrive_last_t(unsigned* ctr, unsigned expected, unsigned* s_last)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(ctr, 1u);
        *s_last = (prev + 1u == expected) ? 1u : 0u;
        if (*s_last) {
            *ctr = 0u;
            __threadfence();
        }
    }
    __syncthreads();
    return *s_last != 0;
}

// CG loop test (ILSS_CG.h:76-77, 140-143)
__device__ __forceinline__ bool cg_cont_t(const StepScalars& s)
{
    return s.delta_new > s.abs_eps_sq && s.delta_new > s.delta_target && s.k < s.max_iter;
}

__device__ __forceinline__ void finish_stats_t(StepScalars& s)
{
    s.rel_residual = (s.delta_0 > 0) ? ::sqrt(s.delta_new / s.delta_0) : 0.0;
    s.abs_residual = ::sqrt(s.delta_new);
}

}  // namespace

// Shared memory of a block of the TILE-thread kernel: two blob stages (a
// tile's element outputs overwrite its element data once every element has
// read it), the staged direction sd4[nodes], two mbarriers and the warps'
// shares and the previous tile's id. TILE = 256: 53.1 KB, four resident
// blocks per SM; TILE = 128 (at most 120 local nodes): 26.4 KB, eight (with
// the 1 KB each block reserves, 219 of the SM's 228 KB).
template <int TILE>
struct PipeShape {
    static constexpr uint32_t kNodes = TILE == kPipeSmallTile ? (uint32_t)kPipeSmallNodes : (uint32_t)kTileNodes;
    static constexpr uint32_t kStage = blob_bytes(TILE, kNodes, 0);  // a multiple of 16
    static constexpr uint32_t kSmem = 2 * kStage + 16u * kNodes + 16u + 8u * (TILE / 32) + 16u;
    static constexpr int kMinBlocks = TILE == kPipeSmallTile ? 8 : 4;
};
static_assert(PipeShape<256>::kStage == 25104 && PipeShape<128>::kStage == 12512, "stage sizes");
static_assert(8 * (((PipeShape<128>::kSmem + 127) & ~127u) + 1024) <= 233472, "eight small blocks per SM");

// What a block needs to know of one tile before its blob arrives.
struct TileLook {
    uint32_t tile;      // tile id
    uint32_t mesh, n0;  // the tile's mesh and first entry in the tile node list
    uint32_t sizes;     // ne | nn << 10 | nown << 20 | material << 30; 0: not an entry of the work list
    uint32_t boff;      // blob offset / 16
    uint32_t g;         // batch node id of this thread's local node
    uint32_t done;      // the mesh has left its loop (the list may still hold it)
    float beta;         // beta of the tile's mesh
};

__device__ __forceinline__ uint32_t look_ne(const TileLook& L) { return L.sizes & 0x3ffu; }
__device__ __forceinline__ uint32_t look_nn(const TileLook& L) { return (L.sizes >> 10) & 0x3ffu; }
__device__ __forceinline__ uint32_t look_nown(const TileLook& L) { return (L.sizes >> 20) & 0x3ffu; }
__device__ __forceinline__ bool look_lcm(const TileLook& L) { return (L.sizes >> 30) != kTileMaterialWrp; }
// A tile to do (valid once resolved).
__device__ __forceinline__ bool look_live(const TileLook& L) { return L.sizes != 0u && L.done == 0u; }

// First half of a look-up: entry i of the work list and the tile's metadata.
__device__ __forceinline__ void look_meta(const BatchView<float>& b, uint32_t i, uint32_t n, TileLook& L)
{
    L.sizes = 0u;
    L.done = 0u;
    if (i < n) {
        L.tile = b.act_tiles[i];
        const TileMeta tm = b.tiles[L.tile];
        L.mesh = tm.mesh;
        L.n0 = tm.n0;
        L.sizes = (uint32_t)tm.ne | ((uint32_t)tm.nn << 10) | ((uint32_t)tm.nown << 20) | ((uint32_t)tm.material << 30);
    }
}

// Second half: the loads that depend on the tile's metadata, all issued
// without waiting on one another (nothing here branches on a loaded value).
__device__ __forceinline__ void look_resolve(const BatchView<float>& b, TileLook& L)
{
    if (L.sizes == 0u) return;
    const StepScalars& st = b.st[L.mesh];
    L.done = st.done;
    L.beta = st.beta_f;
    L.boff = b.blob_off16[L.tile];
    L.g = threadIdx.x < look_nn(L) ? bounds_idx(__ldg(b.tile_nodes + L.n0 + threadIdx.x), b.Ntot, kSiteBatchNode)
                                   : 0u;
}

// A local node's sum of its element outputs (tile-local CSR entries
// [j, j1), element order). (Loading the indices and outputs of two or four
// entries together, to shorten the chain of dependent shared-memory loads,
// measured 1.5 times slower on the 1024-mesh batch: the extra registers
// spill.)
__device__ __forceinline__ void node_sum(const float4* so4, const uint16_t* li, int j, const int j1, uint32_t ne4,
                                         float& a0, float& a1, float& a2)
{
    for (; j < j1; j++) {
        const float4 v = so4[bounds_idx((uint32_t)li[j], 4u * ne4, kSiteTileEntry)];
        a0 += v.x;
        a1 += v.y;
        a2 += v.z;
    }
}

template <bool kCoherent>
__device__ __forceinline__ float ld_dir(const float* p)
{
    return kCoherent ? __ldcg(p) : __ldg(p);
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The block's two stage mbarriers (once per kernel; every thread calls it).
template <int TILE>
__device__ __forceinline__ void tile_pipe_init(unsigned char* smem)
{
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * PipeShape<TILE>::kStage + 16u * PipeShape<TILE>::kNodes);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
}

// One pass of the tile product by this block over its entries block,
// block + G, block + 2G, ... of the CG work list. `phase` carries the
// parities of the block's two stage mbarriers from one pass to the next (a
// persistent kernel runs a pass per CG iteration); every copy a pass issues
// has completed (or, after a wait gave up, been drained) when it returns.
// kCoherent: d and r are read through L2 (ld.global.cg) instead of the
// read-only path, for a kernel whose other phases write them (the
// persistent loop); the pointer parameters carry no __restrict__ for the
// same reason (the kernels that call a pass alone have it on theirs).
// kPk: the P-K products compiled in -- 0 none (C_WRP only), 1 C_LCM, 2 C_LCM
// and C_LCMH (each form only for batches that need it: the products' extra
// registers would otherwise cost the simpler forms).
template <int TILE, bool kCoherent = false, int kPk = 0>
__device__ __forceinline__ void tile_pipe_pass(const BatchView<float>& b, const float* dvec, const float* rvec,
                                               float* part, float2* tshare, unsigned* err,
                                               unsigned char* smem, uint32_t& phase, const uint32_t block,
                                               const uint32_t G, const uint32_t wait_polls)
{
    constexpr uint32_t kStageBytes = PipeShape<TILE>::kStage;
    float4* sd4 = reinterpret_cast<float4*>(smem + 2 * kStageBytes);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sd4 + PipeShape<TILE>::kNodes);
    float2* wsh = reinterpret_cast<float2*>(bar + 2);  // [TILE / 32] per-warp shares
    // the previous tile whose share thread 0 stores after barrier A (only
    // thread 0 uses it); ~0u: none
    uint32_t& s_prev = *reinterpret_cast<uint32_t*>(wsh + TILE / 32);
    const uint32_t tid = threadIdx.x;

    // Software pipeline over this block's entries i, i+G, i+2G, ... of the
    // work list. Per tile (cur, in stage s):
    //   stage the direction of its nodes in sd4 (from registers gathered one
    //   tile earlier) | wait for its blob; barrier A, which also ends every
    //   thread's reads of the other stage | thread 0 stores the previous
    //   tile's d^T A d share and issues the copy of the next tile's blob into
    //   the other stage | element products | the metadata of the tile after
    //   next is resolved and this thread's d and r of the next tile are
    //   gathered into registers | barrier B | outputs over the element data |
    //   barrier C | node sums.
    const uint32_t n_act = *(volatile const uint32_t*)b.act_count;
    uint32_t i = block;
    TileLook cur, nxt, n2;
    look_meta(b, i, n_act, cur);
    look_resolve(b, cur);
    look_meta(b, i + G, n_act, nxt);
    look_resolve(b, nxt);
    // phase, bit s: parity of stage s's next completion
    uint32_t pending = 0u;  // bit s: a copy into stage s is in flight
    int s = 0;
    bool failed = false;
    auto issue = [&](const TileLook& L, int st) {
        const uint32_t bytes = blob_bytes(look_ne(L), look_nn(L), look_nown(L));
        mbar_expect_tx(&bar[st], bytes);
        bulk_copy_g2s(smem + st * kStageBytes, b.blob + 16ull * L.boff, bytes, &bar[st]);
    };
    float cd0 = 0.f, cd1 = 0.f, cd2 = 0.f, cr0 = 0.f, cr1 = 0.f, cr2 = 0.f;
    if (look_live(cur)) {
        if (tid == 0) issue(cur, 0);
        pending |= 1u;
        if (tid < look_nn(cur)) {
            const size_t g = 3 * (size_t)cur.g;
            cd0 = ld_dir<kCoherent>(dvec + g); cd1 = ld_dir<kCoherent>(dvec + g + 1);
            cd2 = ld_dir<kCoherent>(dvec + g + 2);
            cr0 = ld_dir<kCoherent>(rvec + g); cr1 = ld_dir<kCoherent>(rvec + g + 1);
            cr2 = ld_dir<kCoherent>(rvec + g + 2);
        }
    }
    if (tid == 0) s_prev = ~0u;
    for (; i < n_act; i += G) {
        const bool live = look_live(cur), nlive = look_live(nxt);
        const uint32_t ne = look_ne(cur), nn = look_nn(cur);
        float dd = 0.f;  // |d|^2 of this thread's node when the tile owns it
        if (live && tid < nn) {
            const float dx = __fmaf_rn(cur.beta, cd0, cr0);
            const float dy = __fmaf_rn(cur.beta, cd1, cr1);
            const float dz = __fmaf_rn(cur.beta, cd2, cr2);
            sd4[tid] = make_float4(dx, dy, dz, 0.f);
            if (tid < look_nown(cur)) dd = dx * dx + dy * dy + dz * dz;
        }
        // barrier A: every thread polls; the block agrees on the outcome so
        // the barriers below stay uniform
        const bool wait = live && !failed;
        const bool ok = !wait || mbar_wait_bounded(&bar[s], (phase >> s) & 1u, wait_polls);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(err, 1u);
            failed = true;  // no new copies; the ones in flight are drained at the end
        } else if (wait) {
            phase ^= 1u << s;
            pending &= ~(1u << s);
        }
        if (tid == 0) {
            if (s_prev != ~0u) {
                F2 a = {0.f, 0.f};
                if (!failed)
                    for (int k = 0; k < (int)(blockDim.x >> 5); k++) a = f2_add(a, F2{wsh[k].x, wsh[k].y});
                tshare[s_prev] = make_float2(a.hi, a.lo);
            }
            s_prev = live ? cur.tile : ~0u;
            if (!failed && nlive) issue(nxt, s ^ 1);
        }
        if (!failed && nlive) pending |= 1u << (s ^ 1);
        const bool work = live && !failed;
        const unsigned char* stage = smem + s * kStageBytes;
        const uint32_t ne4 = blob_ne4(ne);
        const uint32_t* hdr = reinterpret_cast<const uint32_t*>(stage + blob_hdr_off(ne, nn));
        const float* fac = reinterpret_cast<const float*>(hdr + 1);  // fK, m fM
        float share = 0.f;  // this thread's part of the tile's d^T A d
        if (work) share = fac[1] * dd;  // the nodes the tile owns
        float out[12];
        if (work && tid < ne) {
            const float4* g4 = reinterpret_cast<const float4*>(stage) + tid;
            const float4 q0 = g4[0], q1 = g4[ne4], q2 = g4[2 * ne4], q3 = g4[3 * ne4], q4 = g4[4 * ne4];
            const uint32_t lw = reinterpret_cast<const uint32_t*>(stage + 80u * ne4)[tid];
            const float R[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
            const float Di[9] = {q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w, q4.x, q4.y};
            const float knu = q4.z, k2 = q4.w, k1 = __fmaf_rn(2.f, k2, knu);
            const int ids[4] = {(int)bounds_idx(lw & 0xffu, nn, kSiteLocalNode),
                                (int)bounds_idx((lw >> 8) & 0xffu, nn, kSiteLocalNode),
                                (int)bounds_idx((lw >> 16) & 0xffu, nn, kSiteLocalNode),
                                (int)bounds_idx(lw >> 24, nn, kSiteLocalNode)};
            float dl[12];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float4 v = sd4[ids[k]];
                dl[3 * k] = v.x;
                dl[3 * k + 1] = v.y;
                dl[3 * k + 2] = v.z;
            }
            if (kPk != 0 && look_lcm(cur)) {
                if (kPk == 2 && (cur.sizes >> 30) == kTileMaterialLcmh)
                    elem_lcmh_dforce<float>(R, Di, knu, k2, b.lcmh_w[b.tiles[cur.tile].e0 + tid], dl, out);
                else
                    elem_lcm_dforce<float>(R, Di, knu, k2, dl, out);
            }
            else
                elem_RKRt<float>(R, Di, k1, knu, k2, dl, out);
            float eq = 0.f;
#pragma unroll
            for (int k = 0; k < 12; k++) eq = __fmaf_rn(dl[k], out[k], eq);
            share = __fmaf_rn(fac[0], eq, share);
        }
        // the tile after next: looked up here, after the element products,
        // so that its values do not occupy registers during them
        look_meta(b, i + 2 * G, n_act, n2);
        look_resolve(b, n2);
        float nd0 = 0.f, nd1 = 0.f, nd2 = 0.f, nr0 = 0.f, nr1 = 0.f, nr2 = 0.f;
        if (nlive && tid < look_nn(nxt)) {
            const size_t g = 3 * (size_t)nxt.g;
            nd0 = ld_dir<kCoherent>(dvec + g); nd1 = ld_dir<kCoherent>(dvec + g + 1);
            nd2 = ld_dir<kCoherent>(dvec + g + 2);
            nr0 = ld_dir<kCoherent>(rvec + g); nr1 = ld_dir<kCoherent>(rvec + g + 1);
            nr2 = ld_dir<kCoherent>(rvec + g + 2);
        }
        if (work) {
            // barrier B: every element's data has been read; its space takes
            // the outputs, so4[slot * ne4 + element]
            __syncthreads();
            float4* so4 = reinterpret_cast<float4*>(smem + s * kStageBytes);
            if (tid < ne) {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    so4[k * ne4 + tid] = make_float4(out[3 * k], out[3 * k + 1], out[3 * k + 2], 0.f);
                // these generic-proxy writes precede the next bulk copy into
                // this stage (issued after a later barrier)
                fence_proxy_async_smem();
            }
            __syncthreads();  // barrier C
            if (tid < nn) {
                const uint16_t* lp = reinterpret_cast<const uint16_t*>(stage + blob_lptr_off(ne));
                const uint16_t* li = lp + (nn + 1);
                float a0 = 0.f, a1 = 0.f, a2 = 0.f;
                node_sum(so4, li, lp[tid], lp[tid + 1], ne4, a0, a1, a2);
                const uint32_t nown = look_nown(cur);
                const size_t o =
                    3 * (size_t)bounds_idx(tid < nown ? hdr[0] + tid : hdr[3 + tid - nown], b.nslots, kSitePartialSlot);
                part[o] = a0;
                part[o + 1] = a1;
                part[o + 2] = a2;
            }
            // the terms are non-negative (d_e^T R K0 R^T d_e and m fM |d|^2),
            // so a warp's FP32 tree sum is accurate to a few ulps; the warps'
            // sums are added as (hi, lo) pairs
            float w = share;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
            if ((tid & 31) == 0) wsh[tid >> 5] = make_float2(w, 0.f);
        }
        cur = nxt;
        nxt = n2;
        cd0 = nd0; cd1 = nd1; cd2 = nd2;
        cr0 = nr0; cr1 = nr1; cr2 = nr2;
        s ^= 1;
    }
    __syncthreads();
    if (tid == 0 && s_prev != ~0u) {
        F2 a = {0.f, 0.f};
        if (!failed)
            for (int k = 0; k < (int)(blockDim.x >> 5); k++) a = f2_add(a, F2{wsh[k].x, wsh[k].y});
        tshare[s_prev] = make_float2(a.hi, a.lo);
    }
    if (failed) {
        // every thread drains (the copies write this block's shared memory,
        // so no thread may leave while one is in flight)
        bool drained = true;
        for (int k = 0; k < 2; k++)
            if ((pending >> k) & 1u) {
                const bool ok = mbar_wait_bounded(&bar[k], (phase >> k) & 1u, kDrainPolls);
                if (ok) phase ^= 1u << k;
                drained &= ok;
            }
        if (!drained) atomicExch(err, 2u);
    }
}

template <int TILE, int kPk>
__global__ void __launch_bounds__(TILE, PipeShape<TILE>::kMinBlocks) k_tile_spmv_pipe(BatchView<float> b, const float* __restrict__ dvec,
                                                           const float* __restrict__ rvec, float* __restrict__ part,
                                                           float2* __restrict__ tshare,
                                                           cudaGraphConditionalHandle if_refresh, int set_if,
                                                           const unsigned* __restrict__ refresh_flag,
                                                           unsigned* __restrict__ err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    if (set_if && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(if_refresh, *refresh_flag ? 1u : 0u);
    tile_pipe_init<TILE>(smem);
    uint32_t phase = 0u;
    tile_pipe_pass<TILE, false, kPk>(b, dvec, rvec, part, tshare, err, smem, phase, blockIdx.x, gridDim.x,
                                      *(volatile const unsigned*)(err + 1));
}

// Per running mesh: d^T A d from its tiles' shares (fixed order), alpha and
// the breakdown test (ILSS_CG.h:91-97), once for the node pass's blocks of
// the mesh. One warp per mesh.
// d^T A d of mesh m from its tile shares, alpha and the breakdown test, by
// one warp (lane-strided sum, fixed order: the same bits wherever it runs).
// Valid in lane 0; `publish` writes them to the mesh's scalars.
struct MeshAlpha {
    double dq;
    float alpha;
    bool brk;
};
__device__ __forceinline__ MeshAlpha warp_mesh_alpha(const BatchView<float>& b, const float2* __restrict__ tshare,
                                                     uint32_t m, bool publish)
{
    const uint32_t lane = threadIdx.x & 31u;
    StepScalars& st = b.st[m];
    // every load that needs only the mesh id is issued before the shares
    const uint32_t tile0 = b.mc[m].tile0, ntiles = b.mc[m].ntiles;
    const bool confirm = st.confirm != 0;  // measure the FP64 residual only, no CG update
    const double abs_eps_sq = st.abs_eps_sq, delta_new = st.delta_new;
    const bool minres = b.mc[m].solver == kMeshSolverMinres;
    F2 a = lane_share_sum(tshare + tile0, ntiles, lane);
    a = warp_sum_f2(a);
    MeshAlpha r;
    r.dq = (double)a.hi + (double)a.lo;
    r.brk = !minres && !confirm && ::fabs(r.dq) < abs_eps_sq;  // leave before the update
    // MINRES: alpha = v^T A v (v is the product's operand; v1.v of the
    // reference's order is the same in exact arithmetic, since v0 is
    // orthogonal to v)
    r.alpha = confirm ? 0.f : minres ? (float)r.dq : (float)(delta_new / r.dq);
    if (publish && lane == 0) {
        st.dot_dq = r.dq;
        st.brk = r.brk ? 1u : 0u;
        st.alpha_f = r.alpha;
    }
    return r;
}

__global__ void __launch_bounds__(256) k_mesh_alpha(BatchView<float> b, const float2* __restrict__ tshare)
{
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < b.M; m += nw) {
        if (b.st[m].done) continue;
        (void)warp_mesh_alpha(b, tshare, m, true);
    }
}

// The node pass of chunk ci of a MINRES mesh (v in r, v0 in d, v1 into
// b.mr_v1): v1 = S A v - beta v0 - alpha v and its |v1|^2 share
// (ILSS_MINRES.h:117-130, alpha from the tile shares). On a confirming
// iteration (the residual estimate carried by the Givens sines has passed
// the test) the FP64 residual of the iterate goes into r instead, and its
// |r|^2 decides in the per-mesh update whether the mesh leaves or restarts.
__device__ __noinline__ void node_mr_chunk(const BatchView<float>& b, const float* part, const double* part64,
                                           const double* bv, const double* y, float* r, const float* d,
                                           float2* cshare, const uint32_t ci, const ChunkMeta ch,
                                           const float alpha_s)
{
    __shared__ float2 sh[32];
    const StepScalars& sm = b.st[ch.mesh];
    const MeshConsts& c = b.mc[ch.mesh];
    const bool confirm = sm.confirm != 0;
    const float nb = -(float)sm.mr.beta_new, na = -alpha_s;
    const float fK = c.fK_f, mfm = c.mfm_f;
    float* v1 = b.mr_v1;
    float acc = 0.f;
    for (size_t n = ch.n0 + threadIdx.x; n < ch.n1; n += blockDim.x) {
        const size_t i = 3 * n;
        if (b.fixed[n]) {
            if (!confirm) v1[i] = v1[i + 1] = v1[i + 2] = 0.f;
            continue;
        }
        float s0 = part[i], s1 = part[i + 1], s2 = part[i + 2];
        const uint32_t j0 = b.ov_ptr[n];
        const uint32_t j1 = bounds_idx(b.ov_ptr[n + 1], b.nslots - b.Ntot + 1, kSitePartialSlot);
        for (uint32_t j = j0; j < j1; j++) {
            const size_t o = 3 * ((size_t)b.Ntot + j);
            s0 += part[o];
            s1 += part[o + 1];
            s2 += part[o + 2];
        }
        if (confirm) {
            double t0 = part64[i], t1 = part64[i + 1], t2 = part64[i + 2];
            for (uint32_t j = j0; j < j1; j++) {
                const size_t o = 3 * ((size_t)b.Ntot + j);
                t0 += part64[o];
                t1 += part64[o + 1];
                t2 += part64[o + 2];
            }
            const double mfm64 = c.mass * c.factor_M;
            const float r0 = (float)(bv[i] - (c.factor_K * t0 + mfm64 * y_full(b, y, i)));
            const float r1 = (float)(bv[i + 1] - (c.factor_K * t1 + mfm64 * y_full(b, y, i + 1)));
            const float r2 = (float)(bv[i + 2] - (c.factor_K * t2 + mfm64 * y_full(b, y, i + 2)));
            r[i] = r0; r[i + 1] = r1; r[i + 2] = r2;
            acc += r0 * r0 + r1 * r1 + r2 * r2;
        } else {
            const float v0 = r[i], va = r[i + 1], vb = r[i + 2];
            float w0 = __fmaf_rn(nb, d[i], fK * s0 + mfm * v0);
            float w1 = __fmaf_rn(nb, d[i + 1], fK * s1 + mfm * va);
            float w2 = __fmaf_rn(nb, d[i + 2], fK * s2 + mfm * vb);
            w0 = __fmaf_rn(na, v0, w0);
            w1 = __fmaf_rn(na, va, w1);
            w2 = __fmaf_rn(na, vb, w2);
            v1[i] = w0; v1[i + 1] = w1; v1[i + 2] = w2;
            acc += w0 * w0 + w1 * w1 + w2 * w2;
        }
    }
    const F2 rr = block_sum_f2(F2{acc, 0.f}, sh);
    if (threadIdx.x == 0) cshare[ci] = make_float2(rr.hi, rr.lo);
}

// The node pass of chunk ci (every thread of the block calls it; fuse: the
// block forms its mesh's alpha from the tile shares itself).
__device__ __forceinline__ void node_update_chunk(const BatchView<float>& b, const float* part, const double* part64,
                                                  const double* bv, double* y, float* r, float* d, float2* cshare,
                                                  const float2* tshare, const uint32_t ci, const ChunkMeta& ch,
                                                  const bool fuse)
{
    __shared__ float2 sh[32];
    __shared__ float s_alpha;
    __shared__ int s_brk;
    const StepScalars& sm = b.st[ch.mesh];
    if (sm.done) return;  // left its loop; the list is rebuilt lazily
    const MeshConsts& c = b.mc[ch.mesh];
    bool brk;
    float alpha_s;
    if (fuse) {
        // this block forms its mesh's alpha (warp 0, the same sum as
        // k_mesh_alpha); the block of the mesh's first chunk publishes it
        if (threadIdx.x < 32) {
            const MeshAlpha ma = warp_mesh_alpha(b, tshare, ch.mesh, ci == c.chunk0);
            if (threadIdx.x == 0) {
                s_alpha = ma.alpha;
                s_brk = ma.brk ? 1 : 0;
            }
        }
        __syncthreads();
        brk = s_brk != 0;
        alpha_s = s_alpha;
    } else {
        brk = sm.brk != 0;
        alpha_s = sm.alpha_f;
    }
    if (c.solver == kMeshSolverMinres) {
        node_mr_chunk(b, part, part64, bv, y, r, d, cshare, ci, ch, alpha_s);
        return;
    }
    const bool confirm = sm.confirm != 0;
    const bool refresh = sm.refresh_next != 0;
    const float beta = sm.beta_f;
    const float na = -alpha_s;
    const float fK = c.fK_f, mfm = c.mfm_f;
    float acc = 0.f;
    // Software pipeline over this thread's nodes n, n + blockDim.x, ...: the
    // loads that need only the node id (constraint flag, d, r, the owner's
    // partial, the overflow range, the increment) are issued for the next
    // node before this node's dependent loads and its stores.
    struct Head {
        uint32_t fixed, j0, j1;
        float d[3], r[3], s[3], e[3];
    };
    auto load_head = [&](size_t n, Head& h) {
        const size_t i = 3 * n;
        h.fixed = b.fixed[n];
#pragma unroll
        for (int c3 = 0; c3 < 3; c3++) {
            h.d[c3] = d[i + c3];
            h.r[c3] = r[i + c3];
            h.s[c3] = part[i + c3];
            h.e[c3] = b.ydelta[i + c3];
        }
        h.j0 = b.ov_ptr[n];
        h.j1 = bounds_idx(b.ov_ptr[n + 1], b.nslots - b.Ntot + 1, kSitePartialSlot);
    };
    size_t n = ch.n0 + threadIdx.x;
    bool have = !brk && n < ch.n1;
    Head cur;
    if (have) load_head(n, cur);
    while (have) {
        const size_t nn = n + blockDim.x;
        const bool have_next = nn < ch.n1;
        Head nxt;
        if (have_next) load_head(nn, nxt);
        const size_t i = 3 * n;
        // every load is issued before the constraint flag is known; a
        // constrained row keeps d, r zero and y unchanged
        const bool fixed = cur.fixed != 0;
        const float d0 = __fmaf_rn(beta, cur.d[0], cur.r[0]);
        const float d1 = __fmaf_rn(beta, cur.d[1], cur.r[1]);
        const float d2 = __fmaf_rn(beta, cur.d[2], cur.r[2]);
        // the owner tile's partial (node order), then the overflow slots
        // (contiguous, tile order)
        float s0 = cur.s[0], s1 = cur.s[1], s2 = cur.s[2];
        const uint32_t j0 = cur.j0, j1 = cur.j1;
        float r0 = cur.r[0], r1 = cur.r[1], r2 = cur.r[2];
        float e0 = cur.e[0], e1 = cur.e[1], e2 = cur.e[2];
        // the first four overflow partials are loaded together, then
        // added in slot order (the rare rest one by one)
        float p[4][3];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const bool in = j0 + k < j1;
            const size_t o = 3 * ((size_t)b.Ntot + (in ? j0 + k : 0u));
            p[k][0] = in ? part[o] : 0.f;
            p[k][1] = in ? part[o + 1] : 0.f;
            p[k][2] = in ? part[o + 2] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (j0 + k < j1) {
                s0 += p[k][0];
                s1 += p[k][1];
                s2 += p[k][2];
            }
        }
        for (uint32_t j = j0 + 4; j < j1; j++) {
            const size_t o = 3 * ((size_t)b.Ntot + j);
            s0 += part[o];
            s1 += part[o + 1];
            s2 += part[o + 2];
        }
        if (!fixed) {
            const float q0 = fK * s0 + mfm * d0, q1 = fK * s1 + mfm * d1, q2 = fK * s2 + mfm * d2;
            if (refresh) {
                double t0 = part64[i], t1 = part64[i + 1], t2 = part64[i + 2];
                for (uint32_t j = j0; j < j1; j++) {
                    const size_t o = 3 * ((size_t)b.Ntot + j);
                    t0 += part64[o];
                    t1 += part64[o + 1];
                    t2 += part64[o + 2];
                }
                const double mfm64 = c.mass * c.factor_M;
                const double ya = y[i] + (double)e0, yb = y[i + 1] + (double)e1, yc = y[i + 2] + (double)e2;
                r0 = (float)(bv[i] - (c.factor_K * t0 + mfm64 * ya));
                r1 = (float)(bv[i + 1] - (c.factor_K * t1 + mfm64 * yb));
                r2 = (float)(bv[i + 2] - (c.factor_K * t2 + mfm64 * yc));
                // fold the FP32 increment into the FP64 iterate: later small
                // corrections then keep their bits (an FP32 sum that has grown
                // large would absorb them)
                y[i] = ya;
                y[i + 1] = yb;
                y[i + 2] = yc;
                e0 = e1 = e2 = 0.f;
            }
            if (!confirm) {
                r0 += na * q0;
                r1 += na * q1;
                r2 += na * q2;
                e0 = __fmaf_rn(alpha_s, d0, e0);
                e1 = __fmaf_rn(alpha_s, d1, e1);
                e2 = __fmaf_rn(alpha_s, d2, e2);
                d[i] = d0; d[i + 1] = d1; d[i + 2] = d2;
            }
            b.ydelta[i] = e0;
            b.ydelta[i + 1] = e1;
            b.ydelta[i + 2] = e2;
            r[i] = r0; r[i + 1] = r1; r[i + 2] = r2;
            acc += r0 * r0 + r1 * r1 + r2 * r2;
        }
        cur = nxt;
        n = nn;
        have = have_next;
    }
    const F2 rr = block_sum_f2(F2{acc, 0.f}, sh);
    if (threadIdx.x == 0) cshare[ci] = make_float2(rr.hi, rr.lo);
}

// The node pass by this block over its entries block, block + G, ... of the
// chunk work list.
__device__ __forceinline__ void node_update_pass(const BatchView<float>& b, const float* part, const double* part64,
                                                 const double* bv, double* y, float* r, float* d, float2* cshare,
                                                 const float2* tshare,
                                                 const uint32_t block, const uint32_t G, const bool fuse)
{
    const uint32_t n_act = *(volatile const uint32_t*)(b.act_count + 1);
    for (uint32_t ia = block; ia < n_act; ia += G) {
        const uint32_t ci = b.act_chunks[ia];
        const ChunkMeta ch = b.chunks[ci];
        node_update_chunk(b, part, part64, bv, y, r, d, cshare, tshare, ci, ch, fuse);
    }
}

__global__ void __launch_bounds__(256) k_node_update_fused(BatchView<float> b, const float* __restrict__ part,
                                                           const double* __restrict__ part64,
                                                           const double* __restrict__ bv,
                                                           double* __restrict__ y, float* __restrict__ r,
                                                           float* __restrict__ d, float2* __restrict__ cshare,
                                                           const float2* __restrict__ tshare)
{
    node_update_pass(b, part, part64, bv, y, r, d, cshare, tshare, blockIdx.x, gridDim.x, b.fuse_alpha != 0);
}

// A MINRES mesh's update from |v1|^2 (or, on a confirming iteration, the
// FP64 |r|^2): the Givens rotation, the residual estimate and the loop test
// (ILSS_MINRES.h:131-160). When the estimate passes, the next iteration
// measures the FP64 residual of the iterate (the FP32 Lanczos vectors carry
// the estimate only to FP32 accuracy); if that fails the test, MINRES
// restarts from it.
__device__ __forceinline__ void mesh_update_minres(const BatchView<float>& b, const MeshConsts& c, StepScalars& st,
                                                   const double total)
{
    if (st.confirm) {
        st.confirm = 0;
        st.refresh_next = 0;
        st.delta_old = st.delta_new;
        st.delta_new = total;
        if (!isfinite(total)) st.status = 3u;
        if (cg_cont_t(st)) {
            minres_start(st.mr, total);
            st.mr_pending = 2u;
            st.done = 0;
        } else {
            st.mr_pending = 0u;
            st.done = 1;
            st.finished = 1;
            atomicAdd(b.list_dirty, c.ntiles);
            finish_stats_t(st);
        }
        return;
    }
    st.mr.beta = st.mr.beta_new;
    st.mr.alpha = (double)st.alpha_f;
    minres_givens(st.mr, total);
    st.delta_old = st.delta_new;
    st.delta_new = st.mr.norm_r_sq;
    st.k += 1;
    st.total_iters += 1;
    const bool finite = isfinite(total) && isfinite(st.mr.norm_r_sq);
    if (!finite) st.status = 3u;
    st.mr_pending = 1u;
    bool cont = cg_cont_t(st);
    if (!cont && finite && st.k < st.max_iter) {
        cont = true;
        st.confirm = 1u;
        st.refresh_next = 1u;
    }
    st.done = cont ? 0u : 1u;
    if (st.done) {
        finish_stats_t(st);
        st.finished = 1;
        atomicAdd(b.list_dirty, c.ntiles);
    }
}

// Per running mesh, after the node pass: |r|^2 from its chunks' shares
// (fixed order), then beta, the reliable-update and exit-confirmation rules
// and the loop test (ILSS_CG.h:100-144). One warp per mesh; the last block
// of the grid then rebuilds the work lists, sets the CUDA-graph while
// condition and the refresh flag.
// The update of one mesh by one warp (any mesh: one that has left its loop
// returns at once).
__device__ __forceinline__ void mesh_update_one(const BatchView<float>& b, const float2* cshare, const uint32_t mesh)
{
    const uint32_t lane = threadIdx.x & 31u;
    // the mesh's scalars, copied before the first branch and before the
    // shares are summed (one round trip for all of them), updated in
    // registers and written back once
    const uint32_t done = b.st[mesh].done;
    const MeshConsts& c = b.mc[mesh];
    const uint32_t chunk0 = c.chunk0, nchunks = c.nchunks;
    StepScalars st;
    if (lane == 0) st = b.st[mesh];
    if (done) return;
    F2 tot = lane_share_sum(cshare + chunk0, nchunks, lane);
    tot = warp_sum_f2(tot);
    if (lane == 0 && c.solver == kMeshSolverMinres) {
        mesh_update_minres(b, c, st, (double)tot.hi + (double)tot.lo);
        b.st[mesh] = st;
        __threadfence();  // the mesh's scalars before the grid arrival that follows
    } else if (lane == 0) {
        const bool confirm = st.confirm != 0, brk = st.brk != 0;
        if (confirm) {
            // the FP64 residual of the current iterate decides: leave,
            // or go on from it -- with the recurrence's direction
            // (beta from the FP64 residual, reliable-update style),
            // unless the recursive residual had fallen to rounding
            // noise, then from the residual alone (beta = 0)
            const double total = (double)tot.hi + (double)tot.lo;
            const double rec = st.delta_new;  // recursive |r|^2 at the loop test
            st.confirm = 0;
            st.delta_old = rec;
            st.delta_new = total;
            st.delta_refresh = total;
            st.k_refresh = st.k;
            st.refresh_next = 0;
            if (!isfinite(total)) st.status = 3u;
            if (cg_cont_t(st)) {
                st.beta = (rec > 0.0 && total <= 1e3 * rec) ? total / rec : 0.0;
                st.beta_f = (float)st.beta;
                st.done = 0;
            } else {
                st.done = 1;
                st.finished = 1;
                atomicAdd(b.list_dirty, c.ntiles);
                finish_stats_t(st);
            }
        } else if (brk) {
            st.done = 1;
            st.finished = 1;
            atomicAdd(b.list_dirty, c.ntiles);
            finish_stats_t(st);
        } else {
            const double total = (double)tot.hi + (double)tot.lo;
            st.alpha = st.delta_new / st.dot_dq;
            st.delta_old = st.delta_new;
            st.delta_new = total;
            st.beta = total / st.delta_old;
            st.beta_f = (float)st.beta;
            st.k += 1;
            st.total_iters += 1;
            if (!isfinite(total)) st.status = 3u;
            // reliable updates: recompute the residual in FP64 once |r|
            // has fallen by refresh_drop since the last FP64 residual,
            // and at least every refresh_every iterations
            if (st.refresh_next) {
                st.delta_refresh = total;
                st.k_refresh = st.k;
            }
            st.refresh_next = ((c.refresh_drop_sq > 0.0 && total < c.refresh_drop_sq * st.delta_refresh) ||
                               (c.refresh_every > 0 && st.k - st.k_refresh >= c.refresh_every))
                                  ? 1u
                                  : 0u;
            bool cont = cg_cont_t(st);
            if (!cont && st.k_refresh != st.k && st.k < st.max_iter && total == total &&
                (c.refresh_every > 0 || c.refresh_drop_sq > 0.0)) {
                // converged on the FP32 recursive residual: the next
                // iteration measures the FP64 residual before the loop ends
                cont = true;
                st.refresh_next = 1u;
                st.confirm = 1u;
            }
            st.done = cont ? 0u : 1u;
            if (st.done) {
                finish_stats_t(st);
                st.finished = 1;
                atomicAdd(b.list_dirty, c.ntiles);
            }
        }
        b.st[mesh] = st;
        __threadfence();  // the mesh's scalars before the grid arrival that follows
    }
}

// Per running mesh (warp w of nw warps in all): the update above.
__device__ __forceinline__ void mesh_update_pass(const BatchView<float>& b, const float2* cshare,
                                                 const uint32_t w, const uint32_t nw)
{
    for (uint32_t mesh = w; mesh < b.M; mesh += nw) mesh_update_one(b, cshare, mesh);
}

// After every mesh's update, by one block (all its threads): work lists
// (when a mesh left its loop), refresh flag, slice count, and whether the
// loop goes on (the CUDA-graph while condition where there is one).
__device__ __forceinline__ bool loop_control(const BatchView<float>& b, const LoopSync& ls, bool rebuild = true)
{
    __shared__ unsigned s_go;
    // rebuild the CG lists once a quarter of their tiles belong to meshes that
    // have left their loop (the kernels skip those entries until then)
    if (rebuild && 4u * *(volatile const unsigned*)b.list_dirty >= *(volatile const uint32_t*)b.act_count)
        build_active_lists(b);
    int any = 0, rf = 0, norf = 0;  // norf: a running mesh that does not refresh
    for (uint32_t m = threadIdx.x; m < b.M; m += blockDim.x) {
        volatile const StepScalars* sp = b.st + m;
        if (!sp->done) {
            any = 1;
            if (sp->refresh_next)
                rf = 1;
            else
                norf = 1;
        }
    }
    any = __syncthreads_or(any);
    rf = __syncthreads_or(rf);
    norf = __syncthreads_or(norf);
    if (rf) set_refresh_lists(b, !norf);
    if (threadIdx.x == 0) {
        const bool stop = ls.err && *(volatile const unsigned*)ls.err;
        bool budget_left = true;
        if (ls.slice) {
            ls.slice[1] += 1u;
            budget_left = ls.slice[0] == 0u || ls.slice[1] < ls.slice[0];
        }
        if (ls.refresh_flag) *ls.refresh_flag = rf ? 1u : 0u;
        if (ls.body_runs) *ls.body_runs += 1u;
        if (ls.set_cond) cudaGraphSetConditional(ls.cond, (any && !stop && budget_left) ? 1u : 0u);
        s_go = (any && !stop && budget_left) ? 1u : 0u;
    }
    __syncthreads();
    return s_go != 0u;
}

__global__ void __launch_bounds__(256) k_mesh_update(BatchView<float> b, const float2* __restrict__ cshare, LoopSync ls)
{
    __shared__ unsigned s_last;
    mesh_update_pass(b, cshare, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5);
    // last block of the grid: the loop control
    if (!arrive_last_t(ls.gcount, gridDim.x, &s_last)) return;
    (void)loop_control(b, ls);
}

// ---------------------------------------------------------------------------
// The persistent form of the mixed CG loop: one cooperative launch runs the
// iterations of a launch (up to the slice budget) with the four phases of an
// iteration -- tile product, refresh product (when some mesh refreshes),
// node pass with the fused alpha, per-mesh update -- separated by grid
// barriers instead of kernel boundaries. It runs the same device code as the
// kernels above, in the same order per value, so its results are the same
// bits; what it saves is the launch and ramp of four kernels per iteration,
// which dominate an iteration of a small batch (a lone scene of a served
// shard).

// Bounded polls of a grid barrier (each poll sleeps about 20 ns after an L2 round trip): far above
// any phase of an iteration.
constexpr uint32_t kGridPolls = 1u << 22;

// Grid barrier of a cooperative launch over G blocks: gbar[0] counts
// arrivals (zeroed before the launch, never reset during it: generation g is
// complete at G g arrivals) and gbar[1] holds the last completed generation.
// The last block to arrive runs `last` (with all its threads) before it
// releases the others. A wait that gives up sets err[0] = 3 and returns
// false; the caller then leaves its loop.
template <typename F>
__device__ __forceinline__ bool grid_barrier(unsigned* gbar, uint32_t G, uint32_t& gen, unsigned* err, F&& last)
{
    __shared__ unsigned s_state;  // 1: this block arrived last; 2: gave up
    __syncthreads();
    gen++;
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&gbar[0], 1u);
        s_state = (prev + 1u == G * gen) ? 1u : 0u;
    }
    __syncthreads();
    const bool is_last = s_state == 1u;
    if (is_last) {
        last();
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicExch(&gbar[1], gen);
        }
    } else if (threadIdx.x == 0) {
        uint32_t polls = 0;
        while (*(volatile unsigned*)&gbar[1] < gen) {
            if (++polls > kGridPolls) {
                atomicExch(err, 3u);
                s_state = 2u;
                break;
            }
            __nanosleep(20);
        }
        __threadfence();
    }
    __syncthreads();
    return s_state != 2u;
}

// The phases as separate functions: each gets the registers for itself
// (inlined into one body they would share one allocation and spill).
template <int TILE>
__device__ __noinline__ void coop_tile_phase(const BatchView<float>& b, const CoopLoopArgs& a, unsigned char* smem,
                                             uint32_t& phase, uint32_t blk, uint32_t G, uint32_t wait_polls)
{
    tile_pipe_pass<TILE, true>(b, a.d, a.r, a.part, a.tshare, a.err, smem, phase, blk, G, wait_polls);
}
__device__ __noinline__ void coop_refresh_phase(const BatchView<float>& b, const CoopLoopArgs& a, unsigned char* smem,
                                                uint32_t blk, uint32_t G)
{
    // the product of y for the refreshing meshes, staged in the tile stages
    // (the tile product of this iteration is done)
    DF* sd = reinterpret_cast<DF*>(smem);
    DF* so = sd + 3 * kTileNodes;
    tile_spmv_y64_pass<float>(b, a.y, a.part64, SPMV_Y64_REFRESH, sd, so, blk, G);
}
__device__ __noinline__ void coop_node_phase(const BatchView<float>& b, const CoopLoopArgs& a, uint32_t blk,
                                             uint32_t G)
{
    node_update_pass(b, a.part, a.part64, a.bv, a.y, a.r, a.d, a.cshare, a.tshare, blk, G, true);
}
__device__ __noinline__ void coop_mesh_phase(const BatchView<float>& b, const CoopLoopArgs& a, uint32_t warp,
                                             uint32_t nwarps)
{
    mesh_update_pass(b, a.cshare, warp, nwarps);
}
__device__ __noinline__ void coop_loop_control(const BatchView<float>& b, const CoopLoopArgs& a)
{
    const bool go = loop_control(b, a.ls);
    if (threadIdx.x == 0) a.gbar[2] = go ? 1u : 0u;
}

// Whether any mesh's CG loop runs (the start of a step may have ended them
// all), by one block.
__device__ __noinline__ void coop_any_running(const BatchView<float>& b, const CoopLoopArgs& a)
{
    int any = 0;
    for (uint32_t m = threadIdx.x; m < b.M; m += blockDim.x) any |= (((volatile const StepScalars*)b.st) + m)->done ? 0 : 1;
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) a.gbar[2] = any ? 1u : 0u;
}

template <int TILE>
__global__ void __launch_bounds__(TILE, PipeShape<TILE>::kMinBlocks) k_cg_coop(BatchView<float> b, CoopLoopArgs a)
{
    extern __shared__ __align__(128) unsigned char smem[];
    tile_pipe_init<TILE>(smem);
    const uint32_t G = gridDim.x, blk = blockIdx.x;
    const uint32_t wait_polls = *(volatile const unsigned*)(a.err + 1);
    const uint32_t warp = (blk * blockDim.x + threadIdx.x) >> 5, nwarps = (G * blockDim.x) >> 5;
    uint32_t phase = 0u, gen = 0u;
    auto none = [] {};
    if (!grid_barrier(a.gbar, G, gen, a.err, [&] { coop_any_running(b, a); })) return;
    while (*(volatile const unsigned*)&a.gbar[2]) {
        coop_tile_phase<TILE>(b, a, smem, phase, blk, G, wait_polls);
        if (!grid_barrier(a.gbar, G, gen, a.err, none)) return;
        if (*(volatile const unsigned*)a.ls.refresh_flag) {
            coop_refresh_phase(b, a, smem, blk, G);
            if (!grid_barrier(a.gbar, G, gen, a.err, none)) return;
        }
        coop_node_phase(b, a, blk, G);
        if (!grid_barrier(a.gbar, G, gen, a.err, none)) return;
        coop_mesh_phase(b, a, warp, nwarps);
        if (!grid_barrier(a.gbar, G, gen, a.err, [&] { coop_loop_control(b, a); })) return;
    }
}
static_assert(sizeof(DF) * (3 * kTileNodes + 12 * kTileElems) <= PipeShape<kTileElems>::kSmem,
              "refresh staging fits the tile stages");

template <int TILE>
static int coop_max_blocks()
{
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_cg_coop<TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PipeShape<TILE>::kSmem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_coop<TILE>, TILE, PipeShape<TILE>::kSmem);
        grid = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    }
    return grid;
}

cudaError_t launch_cg_coop(const BatchView<float>& b, const CoopLoopArgs& a, uint32_t blocks, cudaStream_t s)
{
    // refresh staging is sized for 256-thread blocks
    if (b.pipe_tile == (uint32_t)kPipeSmallTile) return cudaErrorInvalidValue;
    const uint32_t maxg = (uint32_t)coop_max_blocks<kTileElems>();
    const uint32_t grid = blocks == 0 ? maxg : (blocks < maxg ? blocks : maxg);
    cudaError_t e = cudaMemsetAsync(a.gbar, 0, 3 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    BatchView<float> bv = b;
    CoopLoopArgs av = a;
    void* args[] = {&bv, &av};
    prof_begin("cg_coop", s);
    e = cudaLaunchCooperativeKernel((const void*)k_cg_coop<kTileElems>, dim3(grid), dim3(kTileElems), args,
                                    PipeShape<kTileElems>::kSmem, s);
    prof_end("cg_coop", s);
    launch_counter()++;
    return e;
}

// ---------------------------------------------------------------------------
// The resident-tile form of the persistent loop, for launches whose running
// tiles fit the GPU at two per block: each block keeps its tiles' blobs in
// its two stages for the whole launch (one bulk copy each, at the start) and
// their look-ups in registers, writes the element outputs to a separate
// area, and a CG iteration needs two grid barriers: after the tile product,
// and after the node pass, whose last block runs the per-mesh updates and
// the loop control. Per value it computes what the kernels above compute, in
// the same order, so the results are the same bits. What it removes is the
// per-iteration blob traffic and the chains of dependent global loads
// (work lists, tile metadata) that bound a small batch's iteration.
template <int TILE>
struct ResShape {
    static constexpr uint32_t kNodes = PipeShape<TILE>::kNodes;
    static constexpr uint32_t kStage = PipeShape<TILE>::kStage;
    static constexpr uint32_t kOut = 2 * kStage;            // float4 so4[4 TILE]; mesh list in the control
    static constexpr uint32_t kSd = kOut + 64u * TILE;      // float4 sd4[kNodes]
    static constexpr uint32_t kBar = kSd + 16u * kNodes;    // two mbarriers
    static constexpr uint32_t kSmem = kBar + 16u + 8u * (TILE / 32) + 16u;
    static constexpr int kMinBlocks = 3;
    static constexpr uint32_t kMaxMeshes = 64u * TILE / 4u;  // the control's mesh list in the output area
};
static_assert(3 * (((ResShape<256>::kSmem + 127) & ~127u) + 1024) <= 233472, "three resident blocks per SM");
static_assert(sizeof(DF) * 12 * kTileElems <= ResShape<kTileElems>::kStage &&
                  sizeof(DF) * 3 * kTileNodes <= 64u * kTileElems,
              "refresh staging fits stage 1 and the output area");

// One resident tile's product for this iteration (every thread calls it;
// a tile of a mesh that has left its loop is skipped as a whole).
template <int TILE>
__device__ __forceinline__ void resident_tile(const BatchView<float>& b, const float* dvec, const float* rvec,
                                              float* part, float2* tshare, const TileLook& L,
                                              const unsigned char* stage, unsigned char* smem)
{
    using RS = ResShape<TILE>;
    float4* sd4 = reinterpret_cast<float4*>(smem + RS::kSd);
    float4* so4 = reinterpret_cast<float4*>(smem + RS::kOut);
    float2* wsh = reinterpret_cast<float2*>(smem + RS::kBar + 16u);
    const uint32_t tid = threadIdx.x;
    const uint32_t ne = look_ne(L), nn = look_nn(L), nown = look_nown(L);
    // this thread's d and r and the mesh's flag and beta, loaded together
    float cd0 = 0.f, cd1 = 0.f, cd2 = 0.f, cr0 = 0.f, cr1 = 0.f, cr2 = 0.f;
    if (tid < nn) {
        const size_t g = 3 * (size_t)L.g;
        cd0 = __ldcg(dvec + g); cd1 = __ldcg(dvec + g + 1); cd2 = __ldcg(dvec + g + 2);
        cr0 = __ldcg(rvec + g); cr1 = __ldcg(rvec + g + 1); cr2 = __ldcg(rvec + g + 2);
    }
    const StepScalars* sp = b.st + L.mesh;
    const uint32_t done = *(volatile const uint32_t*)&sp->done;
    const float beta = *(volatile const float*)&sp->beta_f;
    if (done) return;  // uniform: every thread read the same flag after the last grid barrier
    float dd = 0.f;
    if (tid < nn) {
        const float dx = __fmaf_rn(beta, cd0, cr0);
        const float dy = __fmaf_rn(beta, cd1, cr1);
        const float dz = __fmaf_rn(beta, cd2, cr2);
        sd4[tid] = make_float4(dx, dy, dz, 0.f);
        if (tid < nown) dd = dx * dx + dy * dy + dz * dz;
    }
    __syncthreads();
    const uint32_t ne4 = blob_ne4(ne);
    const uint32_t* hdr = reinterpret_cast<const uint32_t*>(stage + blob_hdr_off(ne, nn));
    const float* fac = reinterpret_cast<const float*>(hdr + 1);  // fK, m fM
    float share = fac[1] * dd;
    if (tid < ne) {
        const float4* g4 = reinterpret_cast<const float4*>(stage) + tid;
        const float4 q0 = g4[0], q1 = g4[ne4], q2 = g4[2 * ne4], q3 = g4[3 * ne4], q4 = g4[4 * ne4];
        const uint32_t lw = reinterpret_cast<const uint32_t*>(stage + 80u * ne4)[tid];
        const float R[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
        const float Di[9] = {q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w, q4.x, q4.y};
        const float knu = q4.z, k2 = q4.w, k1 = __fmaf_rn(2.f, k2, knu);
        const int ids[4] = {(int)bounds_idx(lw & 0xffu, nn, kSiteLocalNode),
                            (int)bounds_idx((lw >> 8) & 0xffu, nn, kSiteLocalNode),
                            (int)bounds_idx((lw >> 16) & 0xffu, nn, kSiteLocalNode),
                            (int)bounds_idx(lw >> 24, nn, kSiteLocalNode)};
        float dl[12], out[12];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float4 v = sd4[ids[k]];
            dl[3 * k] = v.x;
            dl[3 * k + 1] = v.y;
            dl[3 * k + 2] = v.z;
        }
        elem_RKRt<float>(R, Di, k1, knu, k2, dl, out);
        float eq = 0.f;
#pragma unroll
        for (int k = 0; k < 12; k++) eq = __fmaf_rn(dl[k], out[k], eq);
        share = __fmaf_rn(fac[0], eq, share);
#pragma unroll
        for (int k = 0; k < 4; k++) so4[k * ne4 + tid] = make_float4(out[3 * k], out[3 * k + 1], out[3 * k + 2], 0.f);
    }
    __syncthreads();
    if (tid < nn) {
        const uint16_t* lp = reinterpret_cast<const uint16_t*>(stage + blob_lptr_off(ne));
        const uint16_t* li = lp + (nn + 1);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        node_sum(so4, li, lp[tid], lp[tid + 1], ne4, a0, a1, a2);
        const size_t o =
            3 * (size_t)bounds_idx(tid < nown ? hdr[0] + tid : hdr[3 + tid - nown], b.nslots, kSitePartialSlot);
        part[o] = a0;
        part[o + 1] = a1;
        part[o + 2] = a2;
    }
    float w = share;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
    if ((tid & 31) == 0) wsh[tid >> 5] = make_float2(w, 0.f);
    __syncthreads();
    if (tid == 0) {
        F2 a = {0.f, 0.f};
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) a = f2_add(a, F2{wsh[k].x, wsh[k].y});
        tshare[L.tile] = make_float2(a.hi, a.lo);
    }
    // the next tile's staging and outputs reuse sd4 and so4
    __syncthreads();
}

// The last block after the node pass: the update of every running mesh
// (a warp per mesh, from a list gathered in the output area), then the loop
// control (no list rebuild: a resident tile of a mesh that has left its
// loop is skipped where it lies).
template <int TILE>
__device__ __noinline__ void resident_control(const BatchView<float>& b, const CoopLoopArgs& a, unsigned char* smem)
{
    __shared__ unsigned s_n;
    uint32_t* list = reinterpret_cast<uint32_t*>(smem + ResShape<TILE>::kOut);
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
    for (uint32_t m = threadIdx.x; m < b.M; m += blockDim.x)
        if (!*(volatile const uint32_t*)&b.st[m].done) list[atomicAdd(&s_n, 1u)] = m;
    __syncthreads();
    const uint32_t n = s_n, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t i = warp; i < n; i += nw) mesh_update_one(b, a.cshare, list[i]);
    __syncthreads();
    const bool go = loop_control(b, a.ls, false);
    if (threadIdx.x == 0) a.gbar[2] = go ? 1u : 0u;
}

// The node pass: the block's chunks, looked up once per launch when they
// number at most two per block (the chunk list does not change during a
// resident launch), else the list walk of the other kernels.
struct ResidentChunks {
    uint32_t n;  // 0..2 cached; ~0u: walk the list
    uint32_t ci[2];
    ChunkMeta ch[2];
};
template <int TILE>
__device__ __noinline__ void resident_node_phase(const BatchView<float>& b, const CoopLoopArgs& a,
                                                 const ResidentChunks& rc, uint32_t blk, uint32_t G)
{
    if (rc.n == ~0u) {
        node_update_pass(b, a.part, a.part64, a.bv, a.y, a.r, a.d, a.cshare, a.tshare, blk, G, true);
        return;
    }
    for (uint32_t k = 0; k < rc.n; k++)
        node_update_chunk(b, a.part, a.part64, a.bv, a.y, a.r, a.d, a.cshare, a.tshare, rc.ci[k], rc.ch[k], true);
}

template <int TILE>
__device__ __noinline__ void resident_refresh_phase(const BatchView<float>& b, const CoopLoopArgs& a,
                                                    unsigned char* smem, uint32_t blk, uint32_t G)
{
    // staged in stage 1 and the output area (stage 1's blob is copied again after)
    DF* so = reinterpret_cast<DF*>(smem + ResShape<TILE>::kStage);
    DF* sd = reinterpret_cast<DF*>(smem + ResShape<TILE>::kOut);
    tile_spmv_y64_pass<float>(b, a.y, a.part64, SPMV_Y64_REFRESH, sd, so, blk, G);
}

template <int TILE>
__global__ void __launch_bounds__(TILE, ResShape<TILE>::kMinBlocks) k_cg_resident(BatchView<float> b, CoopLoopArgs a)
{
    using RS = ResShape<TILE>;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + RS::kBar);
    const uint32_t G = gridDim.x, blk = blockIdx.x, tid = threadIdx.x;
    const uint32_t wait_polls = *(volatile const unsigned*)(a.err + 1);
    const uint32_t n_act = *(volatile const uint32_t*)b.act_count;
    if (n_act > 2u * G) {
        // more running tiles than the launch was sized for: nothing runs
        if (blk == 0 && tid == 0) atomicExch(a.err, 4u);
        return;
    }
    TileLook L[2];
    look_meta(b, blk, n_act, L[0]);
    look_resolve(b, L[0]);
    look_meta(b, blk + G, n_act, L[1]);
    look_resolve(b, L[1]);
    ResidentChunks rc;
    {
        const uint32_t nch = *(volatile const uint32_t*)(b.act_count + 1);
        rc.n = nch > 2u * G ? ~0u : (blk < nch) + (blk + G < nch);
        for (uint32_t k = 0; k < 2; k++)
            if (rc.n != ~0u && k < rc.n) {
                rc.ci[k] = b.act_chunks[blk + k * G];
                rc.ch[k] = b.chunks[rc.ci[k]];
            }
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0u, pending = 0u;
    auto copy_blob = [&](int k) {
        if (tid == 0) {
            const uint32_t bytes = blob_bytes(look_ne(L[k]), look_nn(L[k]), look_nown(L[k]));
            mbar_expect_tx(&bar[k], bytes);
            bulk_copy_g2s(smem + k * RS::kStage, b.blob + 16ull * L[k].boff, bytes, &bar[k]);
        }
        pending |= 1u << k;
    };
    for (int k = 0; k < 2; k++)
        if (L[k].sizes) copy_blob(k);
    bool failed = false;
    // waits for stage k's copy, if one is in flight (every thread polls; the
    // block agrees on the outcome)
    auto await = [&](int k) {
        if (!((pending >> k) & 1u)) return;
        const bool ok = failed || mbar_wait_bounded(&bar[k], (phase >> k) & 1u, wait_polls);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(a.err, 1u);
            failed = true;
        } else {
            phase ^= 1u << k;
            pending &= ~(1u << k);
        }
    };
    uint32_t gen = 0u;
    auto none = [] {};
    bool run = grid_barrier(a.gbar, G, gen, a.err, [&] { coop_any_running(b, a); });
    while (run && *(volatile const unsigned*)&a.gbar[2]) {
        for (int k = 0; k < 2; k++) {
            if (!L[k].sizes) continue;
            await(k);
            if (!failed)
                resident_tile<TILE>(b, a.d, a.r, a.part, a.tshare, L[k], smem + k * RS::kStage, smem);
        }
        if (!grid_barrier(a.gbar, G, gen, a.err, none)) {
            run = false;
            break;
        }
        if (*(volatile const unsigned*)a.ls.refresh_flag) {
            await(1);  // stage 1 is about to be overwritten
            resident_refresh_phase<TILE>(b, a, smem, blk, G);
            // the staging writes precede the bulk copy into stage 1
            fence_proxy_async_smem();
            __syncthreads();
            if (L[1].sizes && !failed) copy_blob(1);
            if (!grid_barrier(a.gbar, G, gen, a.err, none)) {
                run = false;
                break;
            }
        }
        resident_node_phase<TILE>(b, a, rc, blk, G);
        if (!grid_barrier(a.gbar, G, gen, a.err, [&] { resident_control<TILE>(b, a, smem); })) {
            run = false;
            break;
        }
    }
    // no block leaves while a copy into its shared memory is in flight
    bool drained = true;
    for (int k = 0; k < 2; k++)
        if ((pending >> k) & 1u) drained &= mbar_wait_bounded(&bar[k], (phase >> k) & 1u, kDrainPolls);
    if (!drained) atomicExch(a.err, 2u);
}

template <int TILE>
static int resident_max_blocks()
{
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_cg_resident<TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)ResShape<TILE>::kSmem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_resident<TILE>, TILE, ResShape<TILE>::kSmem);
        grid = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    }
    return grid;
}

uint32_t cg_resident_capacity(uint32_t meshes)
{
    return meshes <= ResShape<kTileElems>::kMaxMeshes ? 2u * (uint32_t)resident_max_blocks<kTileElems>() : 0u;
}

cudaError_t launch_cg_resident(const BatchView<float>& b, const CoopLoopArgs& a, uint32_t tiles, cudaStream_t s)
{
    if (b.pipe_tile == (uint32_t)kPipeSmallTile || b.M > ResShape<kTileElems>::kMaxMeshes)
        return cudaErrorInvalidValue;
    const uint32_t maxg = (uint32_t)resident_max_blocks<kTileElems>();
    if (tiles > 2u * maxg) return cudaErrorInvalidValue;
    // one tile per block while they fit, else two
    const uint32_t grid = tiles == 0 ? 1u : (tiles <= maxg ? tiles : (tiles + 1) / 2);
    cudaError_t e = cudaMemsetAsync(a.gbar, 0, 3 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    BatchView<float> bv = b;
    CoopLoopArgs av = a;
    void* args[] = {&bv, &av};
    prof_begin("cg_resident", s);
    e = cudaLaunchCooperativeKernel((const void*)k_cg_resident<kTileElems>, dim3(grid), dim3(kTileElems), args,
                                    ResShape<kTileElems>::kSmem, s);
    prof_end("cg_resident", s);
    launch_counter()++;
    return e;
}

uint32_t tile_pipe_smem_bytes() { return PipeShape<256>::kSmem; }

template <int TILE, int kPk = 0>
static int pipe_grid()
{
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_tile_spmv_pipe<TILE, kPk>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)PipeShape<TILE>::kSmem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_spmv_pipe<TILE, kPk>, TILE,
                                                      PipeShape<TILE>::kSmem);
        if (sms <= 0) sms = 152;
        if (per_sm <= 0) per_sm = 1;
        grid = sms * per_sm;
    }
    return grid;
}

template <int TILE, int kPk>
static void launch_pipe_form(const BatchView<float>& b, const float* d, const float* r, float* part, float2* tshare,
                             cudaGraphConditionalHandle if_refresh, int set_if, const unsigned* refresh_flag,
                             unsigned* err, cudaStream_t s)
{
    const int g = pipe_grid<TILE, kPk>();
    const uint32_t grid = b.ntiles < (uint32_t)g ? (b.ntiles ? b.ntiles : 1) : (uint32_t)g;
    k_tile_spmv_pipe<TILE, kPk><<<grid, TILE, PipeShape<TILE>::kSmem, s>>>(b, d, r, part, tshare, if_refresh, set_if,
                                                                         refresh_flag, err);
}

void launch_tile_spmv_pipe(const BatchView<float>& b, const float* d, const float* r, float* part, float2* tshare,
                           cudaGraphConditionalHandle if_refresh, int set_if, const unsigned* refresh_flag,
                           unsigned* err, cudaStream_t s)
{
    // the form with the P-K products only for batches that hold such meshes
    // (b.has_lcm: 1 C_LCM, 2 also C_LCMH)
    const bool small = b.pipe_tile == (uint32_t)kPipeSmallTile;
    prof_begin("tile_spmv_mixed", s);
    if (small) {
        if (b.has_lcm == 2u)
            launch_pipe_form<kPipeSmallTile, 2>(b, d, r, part, tshare, if_refresh, set_if, refresh_flag, err, s);
        else if (b.has_lcm)
            launch_pipe_form<kPipeSmallTile, 1>(b, d, r, part, tshare, if_refresh, set_if, refresh_flag, err, s);
        else
            launch_pipe_form<kPipeSmallTile, 0>(b, d, r, part, tshare, if_refresh, set_if, refresh_flag, err, s);
    } else {
        if (b.has_lcm == 2u)
            launch_pipe_form<kTileElems, 2>(b, d, r, part, tshare, if_refresh, set_if, refresh_flag, err, s);
        else if (b.has_lcm)
            launch_pipe_form<kTileElems, 1>(b, d, r, part, tshare, if_refresh, set_if, refresh_flag, err, s);
        else
            launch_pipe_form<kTileElems, 0>(b, d, r, part, tshare, if_refresh, set_if, refresh_flag, err, s);
    }
    prof_end("tile_spmv_mixed", s);
    launch_counter()++;
}

// Grid of the node pass: the blocks that fit on the GPU at once, each
// walking the chunk list with a stride of the grid.
static int node_grid()
{
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_node_update_fused, kNodeThreads, 0);
        if (sms <= 0) sms = 152;
        if (per_sm <= 0) per_sm = 1;
        grid = sms * per_sm;
    }
    return grid;
}

void launch_node_update_fused(const BatchView<float>& b, const float* part, const float2* tshare,
                              const double* part64, const double* bv, double* y, float* r, float* d,
                              float2* cshare, const LoopSync& ls, cudaStream_t s)
{
    const uint32_t g = (uint32_t)node_grid();
    const uint32_t grid = b.nchunks < g ? (b.nchunks ? b.nchunks : 1) : g;
    if (!b.fuse_alpha) {
        prof_begin("mesh_alpha", s);
        k_mesh_alpha<<<(b.M * 32u + kNodeThreads - 1) / kNodeThreads, kNodeThreads, 0, s>>>(b, tshare);
        prof_end("mesh_alpha", s);
        launch_counter()++;
    }
    prof_begin("node_update_mixed", s);
    k_node_update_fused<<<grid, kNodeThreads, 0, s>>>(b, part, part64, bv, y, r, d, cshare, tshare);
    prof_end("node_update_mixed", s);
    launch_counter()++;
    prof_begin("mesh_update", s);
    k_mesh_update<<<(b.M * 32u + kNodeThreads - 1) / kNodeThreads, kNodeThreads, 0, s>>>(b, cshare, ls);
    prof_end("mesh_update", s);
    launch_counter()++;
}

void prepare_tile_pipe()
{
    (void)pipe_grid<kPipeSmallTile>();
    (void)pipe_grid<kTileElems>();
    (void)node_grid();
}

FEMGB_BOUNDS_ACCESSOR(bounds_read_tile_pipe)

}  // namespace femgb
