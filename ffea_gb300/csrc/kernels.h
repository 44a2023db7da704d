// kernels.h -- device buffers of a batch and the host-side launchers of its kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "layout.h"


namespace ffea {

// Device pointers of one packed batch.  Arrays typed `void *` hold the
// precision-dependent type T (float in PREC_MIXED, double in PREC_FP64).
struct DeviceBatch {
    int32_t num_blobs = 0, nl_pad = 0, ne_pad = 0, n_edges = 0, n_tiles = 0, n_etiles = 0, num_streams = 0;
    int32_t n_slices = 0, n_entries = 0;
    int32_t n_segs = 0;           // CG segments
    int32_t precision = PREC_MIXED;
    int32_t any_mass = 0, any_nomass = 0, any_lumped = 0;
    int32_t cg_grid = 0;          // CTAs of the persistent CG kernel
    int32_t cg_reg = 0;           // 1: one CG segment per CTA, row state kept in registers
    int32_t cg_local = 0;         // 1: every CTA reduces the dot products itself (few segments and blobs)
    int32_t cg_euler = 0;         // 1 (per launch): the CG kernel ends with the Euler update of the step
    int32_t cg_cache_slots = 0;   // REG: matrix slots per row whose values are copied to shared memory
    int32_t cg_cache_cols = 0;    // REG: matrix slots per row whose column indices are copied
    int32_t part_stride = 8;      // floats per segment slot of the CG partials (32 with the coarse space)
    // two-level preconditioner (REG and local reduction, NoMass, mixed precision)
    int32_t coarse = 0;           // 1: u = diag(omega) D^-1 r + P A_c^-1 P^T r
    int32_t coarse_nmax = 0;      // largest coarse dimension of a blob
    int32_t coarse_hmax = 0;      // memory-resident CG kernel: most coarse dofs of the blobs one CTA touches
    float4 *phi = nullptr;        // per padded row: rest offset from the segment centroid / R, smoother weight
    int32_t *seg_of_row = nullptr;
    int32_t *seg_nbr_ptr = nullptr, *seg_nbr = nullptr;   // segments coupled to each segment (itself included)
    float *coarse_A = nullptr, *coarse_X = nullptr;       // per blob: A_c and X ~ A_c^-1 (coarse_xoff)
    // memory-resident CG kernel: X read as S Xh S, S = diag(sqrt(X_ii)) per
    // coarse dof (coarse_off), Xh = S^-1 X S^-1 in FP16 (coarse_hxoff)
    uint16_t *coarse_Xh = nullptr;
    float *coarse_s = nullptr;
    float *coarse_T = nullptr, *coarse_Xn = nullptr;      // Newton-Schulz scratch (coarse_nmax^2)
    float *coarse_part = nullptr;                         // split-K partial products of the Newton-Schulz GEMMs
    float *coarse_asm = nullptr;                          // partial A_c blocks: 36 floats x CG_SEG_MAX_ROWS / 256 per neighbour entry
    int32_t cg_dyn_smem = 0;      // REG: dynamic shared memory bytes of that copy
    // blobs
    BlobParams *bp = nullptr;
    Material *mats = nullptr;
    void *mat_t = nullptr;        // the material table in T (MAT_T_STRIDE per material)
    int32_t *tile_blob = nullptr, *etile_blob = nullptr;
    int32_t *seg_row0 = nullptr, *seg_rows = nullptr, *seg_blob = nullptr;   // CG segments
    int32_t *seg_order = nullptr;  // memory-resident solve of several blobs: CTA c's segments are
                                   // seg_order[n_segs c / G .. n_segs (c + 1) / G) (NULL: in order)
    // RNG
    mrg::JumpMat *jump_table = nullptr;
    uint32_t *stream_state = nullptr;
    mrg::JumpMat *stream_step = nullptr;
    // the step's draws, generated up front (k_noise): element draws 7 T per
    // padded element, node draws 3 T per node in original numbering
    // (from bp.noise_node_off); runs of NOISE_RUN draws, prefix per (blob, kind)
    int32_t noise_runs = 0;
    int32_t *noise_run_off = nullptr;
    // each run's start state for the next step (6 planes of noise_runs
    // words) and the stream generation it belongs to; a stream's generation
    // changes when its state is set from outside (set_rng_state)
    uint32_t *noise_run_state = nullptr;
    uint32_t *noise_run_gen = nullptr;
    uint32_t *stream_gen = nullptr;
    void *elem_noise = nullptr;
    void *node_noise = nullptr;
    // nodes (FP64 state and rhs)
    double *pos = nullptr, *vel = nullptr, *drag = nullptr, *rhs = nullptr;
    double *ext = nullptr;        // external forces per row (folded; NULL until first set)
    double *lumped_inv = nullptr; // lumped-mass solver: inverse lumped mass per row
    float2 *pos_df = nullptr;     // mixed precision: positions as (hi, lo) FP32 pairs, kept with pos
    uint8_t *flags = nullptr;
    int32_t *orig = nullptr;
    int32_t *gather_ptr = nullptr, *gather_idx = nullptr;
    int32_t *fold_ptr = nullptr, *fold_sec = nullptr;
    void *fold_amp = nullptr;     // T: noise amplitude sqrt(24 kT drag / dt) of each folded secondary node
    void *node_amp = nullptr;     // T per padded node: the amplitude of its own draws
    // CG vectors, T-typed, 3 per padded node: solution x, residual r,
    // u = D^-1 r, w = A u, the recurrences s, p; Jacobi dinv
    void *x = nullptr, *r = nullptr, *u = nullptr, *w = nullptr, *p = nullptr, *s = nullptr, *dinv = nullptr;
    void *u4 = nullptr;           // CG kernel: u published for the neighbours, 4 T per padded node (x, y, z, 0)
    // elements
    int32_t *conn = nullptr;
    uint16_t *mat_id = nullptr;
    int8_t *det_sign = nullptr;
    void *jinv0 = nullptr, *vol0 = nullptr, *efrc = nullptr, *g = nullptr;
    // edges and the SELL-32 matrix
    int32_t *edge_p = nullptr, *edge_q = nullptr, *edge_cptr = nullptr, *edge_cidx = nullptr;
    int32_t *edge_pos_pq = nullptr, *edge_pos_qp = nullptr;
    int32_t *slice_ptr = nullptr, *slice_len = nullptr, *sell_col = nullptr;
    void *sell_val = nullptr;     // 9 T per entry: (slot base)*9 + k*32 + lane
    void *sell_mval = nullptr;    // mass matrix: 1 T per entry
    void *mass_diag = nullptr;    // T per node
    // reductions / status
    double *partials = nullptr;     // 4 per node tile (node kernel); CG: two buffers of part_stride floats per segment
    CgScalars *cg = nullptr;        // per blob
    double *last_sums = nullptr;    // per blob: r.u, w.u, r.r of the last reduction (written by CTA 0)
    unsigned int *counters = nullptr;  // one per reduction site
    unsigned int *bar = nullptr;    // grid barrier: arrival count, generation
    int32_t *status = nullptr;      // per blob failure bits
    int32_t *inverted = nullptr;    // per blob inverted-element count of the last step
    double *energy = nullptr;       // per blob: strain, kinetic
    double *epartials = nullptr;    // 2 per element tile
    unsigned long long *loop_count = nullptr;  // CG iterations executed by the persistent kernel (max over blobs)
};

// A position as a double-float pair (DeviceBatch::pos_df): hi = (float)p,
// lo = (float)(p - hi); the same bits on the host and the device.
__host__ __device__ inline float2 split_pos(double p)
{
    const float h = (float)p;
    return make_float2(h, (float)(p - (double)h));
}

// material table in the working precision T: no FP64 conversion per use
enum MatT { MAT_T_RHO = 0, MAT_T_A = 1, MAT_T_B = 2, MAT_T_G = 3, MAT_T_E = 4, MAT_T_STRIDE = 8 };

// reduction counter slots
enum CounterSlot { CNT_NODES = 0, CNT_ENERGY = 1, CNT_MEAS = 2, CNT_ANGMOM = 3, CNT_COUNT = 4 };

// Measurements (Blob::make_measurements) need the nodes in the reference's
// order, which the batch does not keep: per node (row, -1) for a corner node,
// (row_a, row_b) for an edge midpoint, (-1, -1) for a node of no element,
// with the positions at creation (Blob::set_pos_0), cut into tiles of
// MEAS_TILE nodes that each belong to one blob.
constexpr int MEAS_TILE = 128;
constexpr int MEAS_VALUES = 10;  // per blob: centroid xyz, RMSD, centre of mass xyz, angular momentum xyz
struct MeasView {
    const int2 *io_src = nullptr;
    const int64_t *io_off = nullptr;      // num_blobs + 1: first node of each blob
    const double *pos0 = nullptr;         // 3 per node
    const int32_t *tile_blob = nullptr;   // per node tile
    const int32_t *tile_first = nullptr;  // num_blobs + 1: first node tile of each blob
    int32_t n_tiles = 0;
    double *partials = nullptr;           // 4 per element tile, then 4 per node tile
    double *out = nullptr;                // MEAS_VALUES per blob
};

// element kernel modes
enum ElemMode { ELEM_STEP = 0, ELEM_MATRIX_ONLY = 1 };

constexpr int CG_THREADS = CG_SEG_MAX_ROWS;  // threads per CTA of the CG kernel = maximum rows of a segment
constexpr int CG_MAX_SEGS = 64;         // segments per CTA of the persistent kernel
constexpr int CG_LOCAL_MAX_BLOBS = 64;  // local reduction: blob records kept in shared memory
constexpr int CG_LOCAL_MAX_SEGS = 2048; // local reduction: partial sums every CTA reads per iteration
// memory-resident CG kernel (FP32): segment partials deferred in shared memory
constexpr int kDeferSegs = 16;  // segments per flush
constexpr int kDeferQ = 9;      // values per warp and segment: 3 dot terms + up to 6 restrictions
constexpr size_t kDeferBytes = sizeof(float) * kDeferSegs * kDeferQ * 32 + 16 * kDeferSegs;

// Launchers (all asynchronous on `s`).
void launch_rest_state(const DeviceBatch &d, cudaStream_t s);
void launch_mass_matrix(const DeviceBatch &d, cudaStream_t s);
void launch_lumped_mass(const DeviceBatch &d, cudaStream_t s);
void launch_elements(const DeviceBatch &d, cudaStream_t s, int mode);
void launch_assemble(const DeviceBatch &d, cudaStream_t s);
// the step's random draws (nothing when no blob draws)
void launch_noise(const DeviceBatch &d, cudaStream_t s);
void launch_nodes(const DeviceBatch &d, cudaStream_t s, int use_given_rhs);
// the persistent solve; with `euler` it also applies the step's Euler update
// (src/Blob.cpp:3937-3969) and RNG advance to the blobs whose solve converged
cudaError_t launch_cg(const DeviceBatch &d, cudaStream_t s, bool euler = false);
// The CG kernel's grid barrier with a target that no arrival reaches and the
// given spin limit, on `ctas` co-resident CTAs; *out counts the CTAs that
// reported the time-out (bar: 8 zeroed words, out: one zeroed int).
cudaError_t launch_barrier_timeout_selftest(unsigned int *bar, unsigned int spin_limit, int *out, int ctas,
                                            cudaStream_t s);
void launch_energies(const DeviceBatch &d, cudaStream_t s);
// centroid, RMSD, centre of mass and angular momentum of every blob into m.out
void launch_measurements(const DeviceBatch &d, const MeasView &m, cudaStream_t s);
void launch_apply(const DeviceBatch &d, cudaStream_t s, const double *in, double *out);
// standalone w = A u with one of the SpMV variants (0..3), for timing
void launch_spmv_variant(const DeviceBatch &d, cudaStream_t s, int variant);
void launch_rng_draws(const mrg::JumpMat *table, const uint32_t *state, uint64_t offset, int64_t count, double *out,
                      cudaStream_t s);
// Shared-memory plan of the register-resident CG kernel on the current
// device: column indices of JC slots per row (at most max_cols) and values of
// J slots (at most max_slots), plus x and D^-1 and extra_bytes (the coarse
// space); dyn_bytes is the dynamic shared memory that takes (also set as the
// kernel's limit).  -1 on error.
int cg_smem_plan(int precision, int max_slots, int max_cols, size_t extra_bytes, int *J, int *JC, size_t *dyn_bytes);
// Learned smoother weights (learned.cu): a 3-layer mesh message-passing
// network, hidden width 32, 8 input features per node.
constexpr int MPNN_FEATURES = 8;
constexpr int MPNN_HIDDEN = 32;
constexpr int MPNN_NUM_PARAMS = 2 * MPNN_HIDDEN * MPNN_FEATURES + MPNN_HIDDEN +
                                2 * (2 * MPNN_HIDDEN * MPNN_HIDDEN + MPNN_HIDDEN) + MPNN_HIDDEN + 1;
struct MpnnBuffers {
    float *x0 = nullptr;                    // features, 8 per padded row
    __nv_bfloat16 *h[3] = {nullptr, nullptr, nullptr};  // activations, 32 per padded row
    float *omega = nullptr;                 // per padded row
    float4 *v = nullptr, *e = nullptr;      // D^-1 f and z = M f
    float2 *gw = nullptr;                   // per row (Az.v, f.v): dL/d omega = k1 x - k2 y
    float *gvec = nullptr, *cvec = nullptr; // coarse P^T f and X P^T f
    double *cta_sums = nullptr, *scal = nullptr;   // 3 per forward CTA; loss, k1, k2
    float *dh = nullptr, *dh2 = nullptr, *dself = nullptr, *tbuf = nullptr;  // 32 per padded row
    float *partial = nullptr;               // per backward CTA: MPNN_NUM_PARAMS
    float *theta = nullptr, *grad = nullptr;
};
// forward pass (omega; write_phi: also the smoother weights of the solve),
// the loss of the last solve's (rhs, solution) pair, and the backward pass
// into grad_dev.  0 on success.
int mpnn_forward(const DeviceBatch &d, MpnnBuffers &B, const float *theta_dev, bool write_phi, cudaStream_t s);
int mpnn_loss(const DeviceBatch &d, MpnnBuffers &B, cudaStream_t s);
int mpnn_backward(const DeviceBatch &d, MpnnBuffers &B, const float *theta_dev, float *grad_dev, cudaStream_t s);

// Two-level preconditioner (coarse.cu): the coarse matrices of the current
// mesh, and `iterations` Newton-Schulz updates of X ~ A_c^-1 per blob
// (`init`: from I / ||A_c||_inf).  0 on success.
void launch_coarse_assemble(const DeviceBatch &d, cudaStream_t s);
int coarse_refresh(const DeviceBatch &d, const std::vector<BlobParams> &bps, cudaStream_t s, int iterations,
                   bool init);
// C = alpha A B + beta D over `batch` row-major n x n FP32 matrices n^2 apart
// (D may be null when beta = 0), enqueued on s.  part: split-K scratch of
// sgemm_splits(n, batch) * batch * n^2 floats, or null (no split).
void sgemm_batched(const float *A, const float *B, const float *D, float *C, int n, int batch, float alpha, float beta,
                   float *part, cudaStream_t s);
int sgemm_splits(int n, int batch);
// floats of split-K scratch the coarse refresh of these blobs needs (0: none)
size_t coarse_part_floats(const std::vector<BlobParams> &bps);
// CTAs of the persistent CG kernel (register-resident variant with dyn_bytes
// of dynamic shared memory, or not) that fit co-resident on the current
// device, 0 on error
int cg_max_grid(int precision, int reg, size_t dyn_bytes);
size_t cg_mem_defer_bytes(int precision);
size_t cg_mem_coarse_bytes(int coarse_hmax);
int cg_mem_smem_allow(int precision, size_t dyn_bytes);

int64_t kernel_launch_count();
void count_launches(int64_t n);

}  // namespace ffea
