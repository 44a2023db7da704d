// host_build.h -- host-side preprocessing of FFEA blobs into the packed layout.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"
#include "layout.h"

namespace ffea {

// How to rebuild the reference's node arrays of one blob.
struct BlobMap {
    int32_t num_nodes_total = 0;      // N_t
    int32_t num_elements = 0;
    std::vector<int32_t> lin_of_orig; // orig node -> global padded linear id, -1 for secondary
    std::vector<int32_t> topology;    // 10 * E original indices (midpoint reconstruction)
    std::vector<uint8_t> pinned_orig; // orig node pinned flag
    std::vector<double> drag_orig;    // orig node Stokes drag
};

struct HostBatch {
    int32_t num_blobs = 0;
    int32_t precision = PREC_MIXED;
    int32_t rng_mode = 0;
    int32_t nl_pad = 0, ne_pad = 0, n_edges = 0, n_tiles = 0, n_etiles = 0;
    int32_t any_mass = 0, any_nomass = 0, any_lumped = 0;
    std::vector<BlobParams> bp;
    std::vector<Material> materials;
    std::vector<uint16_t> mat_id;        // per padded element
    std::vector<int32_t> conn;           // 4 per padded element (global linear ids)
    std::vector<double> pos, vel;        // 3 per padded node
    std::vector<double> drag;            // per padded node
    std::vector<uint8_t> flags;          // per padded node
    std::vector<int32_t> orig;           // per padded node: original index in its blob, -1 padding
    std::vector<int32_t> gather_ptr, gather_idx;          // node -> (elem*4 + corner), element order
    std::vector<int32_t> fold_ptr, fold_sec;              // node -> secondary nodes folded onto it
    std::vector<double> fold_amp;                         // noise amplitude of each folded secondary node
    std::vector<double> node_amp;                         // per padded node: amplitude of its own noise
    std::vector<int32_t> edge_p, edge_q;                  // edges (p < q), sorted by (p, q)
    std::vector<int32_t> edge_cptr, edge_cidx;            // edge -> (elem*16 + a*4 + b), element order
    // SELL-32 layout of the node-node matrix: slices of 32 consecutive rows,
    // slot j of row r at entry slice_ptr[r/32] + 32*j + r%32, columns ascending
    std::vector<int32_t> slice_ptr, slice_len, sell_col;
    std::vector<int32_t> edge_pos_pq, edge_pos_qp;        // entry of (p,q) in row p and of (q,p) in row q
    std::vector<int32_t> tile_blob, etile_blob;
    // CG segments: contiguous row ranges of one blob, 32-row aligned, one
    // per CTA of the persistent CG kernel (or several per CTA)
    std::vector<int32_t> seg_row0, seg_rows, seg_blob;
    std::vector<int32_t> parts;                            // CG segments per blob
    // two-level preconditioner: segment of each padded row (-1 padding);
    // per row (x - c_s) / R_s of its segment at rest and the smoother weight;
    // per segment the sorted segments it couples to (itself included)
    std::vector<int32_t> seg_of_row;
    std::vector<float> phi;                                // 4 per padded row
    std::vector<int32_t> seg_nbr_ptr, seg_nbr;
    int64_t coarse_htotal = 0;                             // halves of the FP16 scaled inverses
    int32_t num_streams = 0;
    std::vector<uint32_t> stream_state;                   // 6 per stream
    std::vector<mrg::JumpMat> stream_step;                // per stream: A^(draws per step)
    // the noise kernel's runs of NOISE_RUN draws: prefix over (blob, kind)
    // pairs, kind 0 = element draws, 1 = node draws (2 * num_blobs + 1)
    std::vector<int32_t> noise_run_off;
    int64_t noise_nodes = 0;                              // nodes with node draws (all blobs)
    std::vector<BlobMap> maps;
};

// CG segments per blob for the given linear-node counts: at least enough of
// at most max_rows rows (a multiple of 32); when those fit `ctas`, segments
// are added where they are longest until there are `ctas` of them (each CTA
// then runs one, and the longest is as short as the 32-row granularity
// allows).
std::vector<int32_t> plan_parts(const std::vector<int32_t> &counts, int32_t ctas, int32_t max_rows);

// Build the packed batch for a persistent CG kernel of `cg_ctas` co-resident
// CTAs: each blob's linear nodes are numbered so that its CG segments
// (plan_parts) are compact blocks.  Returns false and sets err on invalid
// input.
bool build_batch(int32_t num_blobs, const ffea_gpu_mesh *meshes, const ffea_gpu_params *params, int32_t rng_mode,
                 int32_t cg_ctas, HostBatch &out, std::string &err);

// The CG segments of the batch (H.parts per blob, 32-row aligned row ranges):
// fills H.seg_* and H.bp[b].seg_off / seg_cnt; returns the number of segments.
int32_t plan_cg_segments(HostBatch &H);

// Coarse-space data of the two-level preconditioner for the planned
// segments (call after plan_cg_segments): seg_of_row, phi (smoother weight
// 1), seg_nbr_*, per blob coarse_off / coarse_n / coarse_xoff / coarse_hxoff
// (6 rigid modes per segment), and coarse_htotal.  Returns the total size of
// the per-blob dense coarse matrices (sum of coarse_n^2).
int64_t build_coarse(HostBatch &H);

// World::init's six seed words (src/World.cpp:299-305).
void ffea_seed_words(int32_t rng_seed, uint64_t out[6]);

}  // namespace ffea
