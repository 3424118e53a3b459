// batch_launch.h -- launchers of the batched kernels (batch_kernels.cu,
// rotation.cu), used by the batch runtime (batch.cu).
#pragma once
#include "batch.cuh"

namespace femgb {

uint32_t grid_tiles(uint32_t ntiles);
uint32_t tile_pipe_smem_bytes();
void prepare_tile_pipe();
uint32_t grid_chunks(uint32_t nchunks);
// Node-vector permutation between the caller's order and the batch's:
// to_batch: dst[i] = src[perm[i]]; otherwise dst[perm[i]] = src[i] (xyz each).
void launch_permute(const uint32_t* perm, uint64_t n, const double* src, double* dst, bool to_batch,
                    cudaStream_t s);

// Arrival counters and graph handle of the fused CG finalisation.
struct LoopSync {
    unsigned* mcount;        // [M] per-mesh chunk arrivals (FP64 path)
    unsigned* gcount;        // grid arrivals
    unsigned* refresh_flag;  // raised when a mesh refreshes its residual next iteration
    unsigned* body_runs;     // CG-loop body executions (launch accounting)
    const unsigned* err;     // batch error word: the loop stops once it is set
    unsigned* slice;         // [budget (0 = none), iterations run in this launch]
    cudaGraphConditionalHandle cond;
    int set_cond;
};

// Mixed path, one CG iteration (tile_pipe.cu): the tile product (with each
// tile's d^T A d share), then launch_node_update_fused: the per-mesh alpha,
// the node pass and the per-mesh update (beta, loop test, work lists).
void launch_tile_spmv_pipe(const BatchView<float>& b, const float* d, const float* r, float* part, float2* tshare,
                           cudaGraphConditionalHandle if_refresh, int set_if, const unsigned* refresh_flag,
                           unsigned* err, cudaStream_t s);
void launch_node_update_fused(const BatchView<float>& b, const float* part, const float2* tshare,
                              const double* part64, const double* bv, double* y, float* r, float* d,
                              float2* cshare, const LoopSync& ls, cudaStream_t s);

// One mesh's element material triple re-baked from scalar values (rebake;
// on the mixed path also its tile blobs' copies) and its tiles' material.
template <typename S>
void launch_rebake_mesh(const BatchView<S>& b, uint32_t tile0, uint32_t ntiles, double k0, double k1, double k2,
                        int rebake, uint16_t material, cudaStream_t s);

// Mixed path: rewrite each tile blob's FP32 system factors from b.mc.
void launch_blob_factors(const BatchView<float>& b, cudaStream_t s);

// Mixed path, the whole CG loop of a launch in one persistent cooperative
// kernel (tile_pipe.cu): per iteration the tile product, the refresh product
// when a mesh refreshes, the node pass with the fused alpha and the per-mesh
// update, separated by grid barriers; it ends when no mesh runs, the slice
// budget is spent or the error word is set. gbar: 3 device words.
struct CoopLoopArgs {
    float* d;
    float* r;
    float* part;
    float2* tshare;
    double* part64;
    const double* bv;
    double* y;
    float2* cshare;
    unsigned* err;
    unsigned* gbar;
    LoopSync ls;
};
// blocks: 0 = every block that fits the GPU; clamped to that.
cudaError_t launch_cg_coop(const BatchView<float>& b, const CoopLoopArgs& a, uint32_t blocks, cudaStream_t s);
// The resident-tile form (each block keeps up to two tiles' element data in
// shared memory for the whole launch): usable while the running tiles number
// at most cg_resident_capacity(meshes) (0 when the batch has too many meshes
// for its per-mesh control list); `tiles` bounds the running tiles.
uint32_t cg_resident_capacity(uint32_t meshes);
cudaError_t launch_cg_resident(const BatchView<float>& b, const CoopLoopArgs& a, uint32_t tiles, cudaStream_t s);

template <typename S>
struct BatchLaunch {
    // rotation.cu; newton: the re-evaluation at x_k of the FIE meshes that
    // have just updated (otherwise the meshes of the start section)
    static void begin_eval(const BatchView<S>& b, const double* x, int newton, cudaStream_t s);
    // newton: the Newton loop's while condition, set when newton_form (the
    // step has a Newton level: some mesh integrates with FIE)
    static void reset_counts(const BatchView<S>& b, const LoopSync& ls, cudaGraphConditionalHandle if_start,
                             cudaGraphConditionalHandle newton, int newton_form, cudaStream_t s);
    static void tile_spmv(const BatchView<S>& b, const S* d, const S* r, S* part,
                          cudaGraphConditionalHandle if_refresh, int set_if, const unsigned* refresh_flag,
                          cudaStream_t s);
    static void tile_spmv_y64(const BatchView<S>& b, const double* y, double* part64, int refresh,
                              const unsigned* flag, cudaStream_t s);
    static void tile_force(const BatchView<S>& b, const double* x, double* part64, double* tile_energy,
                           cudaStream_t s);
    static void tile_potential(const BatchView<S>& b, const double* x, double* tile_pe, cudaStream_t s);
    static void node_b(const BatchView<S>& b, const double* part64, const double* v, const double* x, double* bv,
                       double* y, cudaStream_t s);
    static void knc(const BatchView<S>& b, uint32_t K, const double* x, double* bv, double* y, cudaStream_t s);
    static void node_residual(const BatchView<S>& b, const double* part64, const double* bv, const double* y, S* r,
                              S* d, double* cpart, const LoopSync& ls, cudaStream_t s);
    static void node_q(const BatchView<S>& b, const S* part, S* d, S* q, const double* part64,
                       const double* bv, const double* y, S* r, double* cpart, const LoopSync& ls, cudaStream_t s);
    static void node_update(const BatchView<S>& b, double* y, S* r, const S* d, S* q, double* cpart,
                            const LoopSync& ls, cudaStream_t s);
    // MINRES meshes: the finishing pass of the start or of an iteration
    static void node_mr_finish(const BatchView<S>& b, double* y, S* r, S* d, const S* q, const LoopSync& ls,
                               cudaStream_t s);
    static void integrate(const BatchView<S>& b, double* x, double* v, const double* y, double* cpart,
                          const LoopSync& ls, cudaStream_t s);
    static void newton_tail(const BatchView<S>& b, const LoopSync& ls, cudaGraphConditionalHandle newton,
                            cudaStream_t s);
    // the lock-step's bookkeeping: 0 = NR_PreStep's counts, 1 = NR_End's
    static void lock_phase(const BatchView<S>& b, int phase, cudaStream_t s);
    static void fin_energy(const BatchView<S>& b, int kind, const double* tpart, cudaStream_t s);
};

}  // namespace femgb
