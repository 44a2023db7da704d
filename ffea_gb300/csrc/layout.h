// layout.h -- the packed multi-blob layout in HBM, shared by host and device code.
//
// All blobs of a batch are concatenated.  Node-space arrays hold only the
// LINEAR nodes of each blob (the 4 corner nodes that carry mechanics); the
// secondary edge-midpoint nodes of FFEA's 10-node elements are reconstructed
// on output.  Each blob's node range is padded to a multiple of NODE_TILE and
// its element range to a multiple of ELEM_TILE so that every CTA of a
// node-space or element-space kernel belongs to exactly one blob; padding rows
// behave like pinned rows (zero force, identity matrix row).
#pragma once
#include <stdint.h>

#include "mrg32k3a.cuh"

namespace ffea {

constexpr int NODE_TILE = 256;   // rows per CTA of node-space kernels
constexpr int NODE_LANES = 4;    // threads per row of the node kernel (k_nodes)
constexpr int ELEM_TILE = 128;   // elements per CTA of the element kernel
constexpr int EDGE_TILE = 256;
constexpr int MAX_BLOBS = 1 << 20;
constexpr int CG_SEG_MAX_ROWS = 1024;  // rows of a CG segment (one per thread of a CG CTA)
constexpr int NOISE_RUN = 32;          // consecutive draws per thread of the noise kernel (one jump each)
constexpr int NOISE_THREADS = 128;     // threads per CTA of the noise kernel

enum SolverKind : int32_t { SOLVER_NOMASS = 0, SOLVER_MASS = 1, SOLVER_LUMPED = 2 };
enum Precision : int32_t { PREC_FP64 = 0, PREC_MIXED = 1 };

// node flag bits
constexpr uint8_t NODE_PINNED = 1;   // pinned or padding: identity row, zero force

// per-blob status bits
constexpr int32_t BLOB_FAIL_INVERSION = 1;
constexpr int32_t BLOB_FAIL_CG = 2;
constexpr int32_t BLOB_FAIL_NAN = 4;
constexpr int32_t BLOB_FAIL_TIMEOUT = 8;   // a grid barrier of the CG kernel gave up waiting

struct BlobParams {
    double dt, kT, epsilon2;
    int32_t max_iter;
    int32_t calc_noise, calc_stokes;
    int32_t solver;
    int32_t stream;            // index of the RNG stream this blob draws from
    uint32_t elem_draw_base;   // draw offset of element 0 within a step
    uint32_t node_draw_base;   // draw offset of node 0 (original numbering) within a step
    int32_t node_off, node_cnt, node_pad;   // padded linear-node range
    int32_t elem_off, elem_cnt, elem_pad;   // padded element range
    int32_t tile_off, tile_cnt;             // node tiles (CTAs) of this blob
    int32_t seg_off, seg_cnt;               // CG segments of this blob
    int32_t coarse_off, coarse_n;           // two-level: first coarse dof, number of coarse dofs (6 per segment)
    int32_t coarse_xoff;                    // offset of the blob's dense coarse matrices (coarse_n^2 floats)
    int32_t coarse_hxoff;                   // offset of the blob's FP16 scaled inverse (coarse_n rows of
                                            // coarse_n rounded up to 8 halves)
    int32_t num_nodes_total;                // N_t of the reference (linear + secondary)
    int32_t noise_node_off;                 // first node of the blob's node draws in the node-noise buffer
    int32_t true_residual;
    int32_t all_pinned;                     // every node pinned: no element step, no element draws (src/Blob.cpp:643-645)
};

// material table entry (meso units, tetra_element_linear fields)
struct Material {
    double rho, A, B, G, E;
};

// CG state of a blob during a solve
enum CgState : int32_t { CG_ACTIVE = 0, CG_VERIFY = 1, CG_RESTART = 2, CG_CONVERGED = 3, CG_FAILED = 4 };

// Per-blob CG scalars, FP64 (Chronopoulos-Gear recurrences).
struct CgScalars {
    double gamma;      // r . u   (u = D^-1 r)
    double delta;      // p . A p of the last update (w . u at the first)
    double ff;         // f . f   (rhs norm^2)
    double rr;         // r . r
    double alpha, beta;
    double true_relres2;   // ||b - A x||^2 / ||b||^2 of the last verification, -1 if none
    // mixed precision: the recurrences in FP32 (no FP64 instruction on the
    // per-iteration path; FP64 runs at 1/64 of the FP32 rate)
    float gamma_f, pap_f, alpha_f, beta_f;
    float stop_f;          // eps^2 f.f: stop when r.r < stop_f
    float floor_f;         // 1e-10 f.f: an FP32 recurrence that breaks down below this has converged as far as FP32 goes
    int32_t iters;         // matrix-vector products of this solve (the reference's iteration count)
    int32_t state;         // CgState
    int32_t restarts;
    int32_t reserved;      // (keeps the record a whole number of 8-byte words)
};

}  // namespace ffea
