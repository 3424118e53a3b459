// batch.cuh -- device layout of a batch of independent solids stepped in
// lock-step (the tiled path; one solid is a batch of one).
//
// Meshes are concatenated: mesh m owns global nodes [node0, node0+N) and
// global elements [elem0, elem0+T). Elements are cut into tiles of at most
// tile_elems tets touching at most kTileNodes distinct nodes; a tile belongs
// to one mesh.
//
// Nodes are numbered inside the batch in the order they first appear in their
// mesh's tile sequence, by degree within a tile (the API permutes states to
// and from the caller's order). A tile's new nodes -- the nodes it owns --
// therefore have consecutive ids, and its local node list puts them first.
//
//   per tile     TileMeta: element range, its local node list (tile_nodes,
//                global ids, owned nodes first), its local connectivity
//                (lconn, uchar4 local ids) and a tile-local CSR (lptr/lidx)
//                giving, for each local node, the (element, slot) outputs to
//                sum, in element order
//   per element  Dinv/mat/R in the path's element type S (SoA), plus FP64
//                Dinv, volume and global ids for the once-per-step kernels
//   per node     x, v, b, y (FP64); r, d, q (S); rest (FP64); fixed flag
//   partials     one per (tile, local node): the owner tile's at part[node]
//                (node order, so the node pass reads it coalesced), a shared
//                node's other tiles' in overflow slots part[Ntot + j], j in
//                [ov_ptr[n], ov_ptr[n+1]) (contiguous per node, tile order);
//                ov_map gives the slot of each (tile, shared local node)
//
// All sums have a fixed order (a node's partials: owner first, then tile
// order), so a solid gives the same bits alone and in any batch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fem_device.cuh"

namespace femgb {

constexpr int kTileElems = 256;
constexpr int kTileNodes = 256;
constexpr int kChunkNodes = 1024;  // default node chunk (one work item of a node pass)
// The mixed path's pipelined tile product runs one thread per element: tiles
// of at most kPipeSmallTile tets use blocks of that many threads, with at most
// kPipeSmallNodes local nodes (so that eight blocks fit an SM's shared
// memory); larger tiles use kTileElems threads and up to kTileNodes nodes.
constexpr int kPipeSmallTile = 128;
constexpr int kPipeSmallNodes = 120;
constexpr int kNodeThreads = 256;  // threads per node-kernel block
// Default poll limit of the tile product's waits for a tile copy (each poll
// suspends for a hardware time slice: far above any copy's latency).
constexpr unsigned kDefaultWaitPolls = 1u << 22;

// Layout of a tile's blob (mixed path, see tile_pipe.cu): the element data,
// 21 FP32 components per element (R 0-8, Dm^-1 9-17, V lambda, V mu, local
// ids as one word; V(lambda+2mu) = V lambda + 2 V mu is formed in the
// kernel) grouped by four: group g < 5 holds components 4g..4g+3 as
// float4[ne4], component 20 follows as a word per element (one 16- or 4-byte
// load per group and element, consecutive elements in consecutive words);
// then uint16 lptr[nn+1], uint16 lidx[4 ne],
// and, 4-aligned, the header {uint32 own0, float fK, float m fM} (the partial
// slot of the first owned node, the mesh's FP32 factors) and uint32
// ovslot[nn - nown] (the partial slots of the shared local nodes).
__host__ __device__ constexpr uint32_t blob_ne4(uint32_t ne) { return (ne + 3u) & ~3u; }
// Byte offset of component c of element i.
__host__ __device__ constexpr uint32_t blob_comp_off(uint32_t c, uint32_t i, uint32_t ne4)
{
    return c < 20u ? 16u * ((c >> 2) * ne4 + i) + 4u * (c & 3u) : 80u * ne4 + 4u * i;
}
__host__ __device__ constexpr uint32_t blob_lptr_off(uint32_t ne) { return 84u * blob_ne4(ne); }
__host__ __device__ constexpr uint32_t blob_hdr_off(uint32_t ne, uint32_t nn)
{
    return (blob_lptr_off(ne) + 2u * (nn + 1u) + 8u * ne + 3u) & ~3u;
}
__host__ __device__ constexpr uint32_t blob_bytes(uint32_t ne, uint32_t nn, uint32_t nown)
{
    return (blob_hdr_off(ne, nn) + 12u + 4u * (nn - nown) + 15u) & ~15u;
}

// Per-mesh rotation methods (the values of enum fem_rotation).
constexpr uint32_t kMeshRotationMsvd = 0;
constexpr uint32_t kMeshRotationDapd = 1;

// The mesh's linear solver (LS_Solve's choice, LeafDSH_Solid3D_FEM.cpp:
// 1136-1154). A MINRES mesh keeps its Lanczos vectors in the CG buffers:
// v (the vector the tile product multiplies) in r, with beta = 0 so that the
// product's direction update r + beta d leaves it exact; v0 in d; v1 in q;
// and the directions p, p0 in their own buffers.
constexpr uint32_t kMeshSolverCg = 0;
constexpr uint32_t kMeshSolverMinres = 1;

// The mesh's integrator: QIE_V (one linear solve per step), or the
// fully-implicit Newton on Delta x (dynamic or quasi-static), whose steps
// loop over Newton iterations on the device, each mesh leaving the loop on
// its own |b_k| test or iteration limit.
constexpr uint32_t kMeshQie = 0;
constexpr uint32_t kMeshFie = 1;
constexpr uint32_t kMeshFieQuasi = 2;

struct TileMeta {
    uint32_t mesh;
    uint32_t e0;      // first element (global)
    uint32_t n0;      // first entry in tile_nodes
    uint32_t c0;      // first entry in lidx
    uint16_t ne, nn;  // elements, local nodes
    uint32_t own0;    // global id of the first owned node (local nodes [0, nown))
    uint32_t ov0;     // first entry in ov_map of the shared local nodes [nown, nn)
    uint16_t nown;
    uint16_t material;  // the mesh's kTileMaterial*
};

// Per-tile element products (the values of enum fem_material): C_WRP's
// stiffness product, or a first Piola-Kirchhoff material's differential
// (C_LCM, C_LCMH, C_CCM; csrc/lcm.cuh).
constexpr uint16_t kTileMaterialWrp = 0;
constexpr uint16_t kTileMaterialLcm = 1;
constexpr uint16_t kTileMaterialLcmh = 2;
constexpr uint16_t kTileMaterialCcm = 3;

// Partial slot of local node i of a tile: owned nodes write theirs in node
// order (slot = batch node id), shared nodes the overflow slot ov_map gives
// (Ntot + the entry's position in its node's overflow list, so each node's
// overflow partials are contiguous).
__host__ __device__ inline size_t tile_slot(const uint32_t* ov_map, uint32_t own0, uint32_t ov0, uint32_t nown,
                                            uint32_t i)
{
    return i < nown ? (size_t)own0 + i : (size_t)ov_map[ov0 + (i - nown)];
}

struct ChunkMeta {
    uint32_t mesh;
    uint32_t n0, n1;  // global node range
};

// Per-mesh constants.
struct MeshConsts {
    double dt, inv_dt, mass, factor_M, factor_K;
    double gravity[3];
    double density;
    double rel_eps_sq, abs_eps_sq;
    double degenerate_det_F;
    uint32_t max_iter, refresh_every;
    uint32_t node0, N, elem0, T;
    uint32_t tile0, ntiles, chunk0, nchunks;
    uint32_t knc0, nknc;
    float fK_f, mfm_f;  // factor_K and mass * factor_M rounded to FP32 (mixed path)
    float rot_check;    // mixed: FP64 re-solve when an FP32 rotation moves more than this under a small change of F
    uint32_t rot_fp32;  // mixed: 1 = FP32 rotations with FP64 re-solves, 0 = FP64 rotations
    double refresh_drop_sq;  // mixed: FP64 residual when |r|^2 fell below this times its value at the last one
    uint32_t rotation;       // kMeshRotationMsvd or kMeshRotationDapd (FP64 in either precision)
    uint32_t material;       // kTileMaterial* (the mesh's fem_material)
    double ecie_k;           // C_LCMH: the blend radius k (float32 in the reference)
    uint32_t solver;         // kMeshSolverCg or kMeshSolverMinres
    uint32_t integrator;     // kMeshQie, kMeshFie or kMeshFieQuasi
    uint32_t nr_max_iter;    // FIE: Newton iteration limit
    double nr_abs_eps;       // FIE: the Newton loop ends once |b_k| is below this
    double lame_mu, lame_lambda;  // C_LCM: from the mesh's scalar E and nu (per-element values re-bake only K0)
    double dapd_thr, dapd_fL, dapd_fNL, dapd_eNL;  // DAPD: threshold on det F, offset factors, exponent

};

template <typename S>
struct BatchView {
    uint32_t M, ntiles, nchunks, Ntot, Ttot;
    uint64_t nslots;               // partial slots: Ntot owner slots + the overflow slots
    double* prev_x;                // [3 Ntot] DAPD: positions at the start of each mesh's last step; null without DAPD
    uchar2* doc;                   // [Ttot] DAPD: direction of collapse per element (batch order)
    double* Fe;                    // [9 Ttot] P-K materials: F of the last BeginEvaluation (the element cache's), SoA; null without them
    float* lcmh_w;                 // [Ttot] mixed C_LCMH: the blend weight w of the last BeginEvaluation; null without it
    S* mr_p;                       // [3 Ntot] MINRES: direction p; null without a MINRES mesh
    S* mr_p0;                      // [3 Ntot] MINRES: the previous direction p0
    S* mr_v1;                      // [3 Ntot] MINRES: the Lanczos vector v1 (the q buffer)
    double* cpart_b;               // [nchunks] MINRES, FIE: per-chunk partials of |b|^2 at the start of a solve
    double* xn;                    // [3 Ntot] FIE: x^n, the positions at the start of the step (lock-step:
                                   // the iterate x_k); null without FIE or a lock-step
    double* vn;                    // [3 Ntot] FIE: v^n (lock-step: v_k)
    uint32_t pipe_tile;            // mixed: threads per block of the tile product (kPipeSmallTile or kTileElems)
    uint32_t fuse_alpha;           // mixed: the node pass forms alpha (no separate alpha kernel)
    uint32_t has_lcm;              // the P-K products some mesh takes: 0 none, 1 C_LCM (or C_CCM), 2 also C_LCMH
    uint32_t lock;                 // the multi-solid Newton lock-step's phases (x_k, v_k in xn, vn; x, v hold x^n, v^n)
    const TileMeta* tiles;
    const ChunkMeta* chunks;
    const MeshConsts* mc;
    StepScalars* st;               // [M]
    const uint8_t* active;         // [M] meshes taking part in this step
    // element data
    const int4* gtets;             // [Ttot] global node ids
    const S* Dinv;                 // [9][Ttot]
    const S* mat;                  // [3][Ttot]
    S* R;                          // [9][Ttot]
    const double* Dinv64;          // [9][Ttot]
    const double* vol;             // [Ttot]
    double* detF;                  // [Ttot]
    // tile structure
    const uint32_t* tile_nodes;    // [sum nn] global node id
    const uchar4* lconn;           // [Ttot] local ids within the tile
    const uint16_t* lptr;          // [sum (nn+1)] per tile: offsets into lidx (tile-relative)
    const uint16_t* lidx;          // [4 Ttot] (element-in-tile << 2 | slot), tile-relative
    const uint32_t* lptr0;         // [ntiles] base of each tile's lptr block
    // node data
    const uint32_t* ov_ptr;        // [Ntot+1] per node: its overflow slots Ntot + [ov_ptr[n], ov_ptr[n+1])
    const uint32_t* ov_map;        // [overflow entries] in tile order: the entry's partial slot
    const uint8_t* fixed;          // [Ntot]
    const double* rest;            // [3 Ntot]
    S* ydelta;                     // [3 Ntot] mixed: FP32 sum of this step's alpha d; null on FP64
    unsigned char* blob;           // mixed: per-tile blobs (element data, tile CSR, node list)
    const uint32_t* blob_off16;    // [ntiles] blob offset / 16
    // mixed: tiles and chunks of the meshes still iterating (active_list.cuh)
    uint32_t* act_tiles;           // [ntiles]
    uint32_t* act_chunks;          // [nchunks]
    uint32_t* act_count;           // [2] entries in act_tiles, act_chunks
    unsigned* list_dirty;          // tiles of the CG lists whose mesh has left its loop since the last rebuild
    // tiles and chunks of the meshes that start a step in this launch, and
    // of those that take part in it; list_count: start tiles, start chunks,
    // launch tiles, launch chunks
    uint32_t* start_tiles;         // [ntiles]
    uint32_t* start_chunks;        // [nchunks]
    uint32_t* launch_tiles;        // [ntiles]
    uint32_t* launch_chunks;       // [nchunks]
    uint32_t* refresh_tiles;       // [ntiles] mixed: meshes whose next iteration recomputes r in FP64
    uint32_t* refresh_chunks;      // [nchunks]
    uint32_t* list_count;          // [6] (+ refresh tiles, refresh chunks)
    // constraints
    const uint32_t* knc_node;      // [K] global node id
    const uint32_t* knc_mesh;      // [K]
    const double* knc_target;      // [3K]
};

// Whether mesh m takes part in the current start section (the opening of a
// step, or of a further Newton iteration of an FIE mesh).
template <typename S>
__device__ __forceinline__ bool mesh_starts(const BatchView<S>& b, uint32_t m)
{
    return b.st[m].nr_go != 0;
}

}  // namespace femgb
