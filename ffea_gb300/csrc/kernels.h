// kernels.h -- device buffers of a batch and the host-side launchers of its kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "layout.h"

namespace ffea {

// Device pointers of one packed batch.  Arrays typed `void *` hold the
// precision-dependent type T (float in PREC_MIXED, double in PREC_FP64).
struct DeviceBatch {
    int32_t num_blobs = 0, nl_pad = 0, ne_pad = 0, n_edges = 0, n_tiles = 0, n_etiles = 0, num_streams = 0;
    int32_t precision = PREC_MIXED;
    int32_t any_mass = 0, any_nomass = 0;
    // blobs
    BlobParams *bp = nullptr;
    Material *mats = nullptr;
    int32_t *tile_blob = nullptr, *etile_blob = nullptr;
    // RNG
    mrg::JumpMat *jump_table = nullptr;
    uint32_t *stream_state = nullptr;
    mrg::JumpMat *stream_step = nullptr;
    // nodes
    double *pos = nullptr, *vel = nullptr, *drag = nullptr, *rhs = nullptr, *x = nullptr, *r = nullptr;
    uint8_t *flags = nullptr;
    int32_t *orig = nullptr;
    int32_t *gather_ptr = nullptr, *gather_idx = nullptr;
    int32_t *fold_ptr = nullptr, *fold_sec = nullptr;
    double *fold_drag = nullptr;
    void *p = nullptr, *q = nullptr, *dinv = nullptr;
    // elements
    int32_t *conn = nullptr;
    uint16_t *mat_id = nullptr;
    int8_t *det_sign = nullptr;
    void *jinv0 = nullptr, *vol0 = nullptr, *efrc = nullptr, *g = nullptr;
    // edges
    int32_t *edge_p = nullptr, *edge_q = nullptr, *edge_cptr = nullptr, *edge_cidx = nullptr;
    int32_t *up_ptr = nullptr, *lo_ptr = nullptr, *lo_edge = nullptr;
    void *blocks = nullptr, *mass_edge = nullptr, *mass_diag = nullptr;
    // reductions / status
    double *partials = nullptr;     // 4 per node tile
    CgScalars *cg = nullptr;        // per blob
    unsigned int *counters = nullptr;  // one per reduction site
    int32_t *status = nullptr;      // per blob failure bits
    int32_t *inverted = nullptr;    // per blob inverted-element count of the last step
    double *energy = nullptr;       // per blob: strain, kinetic
    double *epartials = nullptr;    // 2 per element tile
    int32_t *any_running = nullptr; // host-visible "some blob still iterating" flag
};

// reduction counter slots
enum CounterSlot { CNT_NODES = 0, CNT_SPMV = 1, CNT_UPDATE = 2, CNT_ENERGY = 3, CNT_TRUERES = 4, CNT_COUNT = 8 };

// element kernel modes
enum ElemMode { ELEM_STEP = 0, ELEM_MATRIX_ONLY = 1 };

// Launchers (all asynchronous on `s`).  `cond` is a graph conditional handle
// (0 when not inside a conditional body).
void launch_rest_state(const DeviceBatch &d, cudaStream_t s);
void launch_mass_matrix(const DeviceBatch &d, cudaStream_t s);
void launch_elements(const DeviceBatch &d, cudaStream_t s, int mode);
void launch_assemble(const DeviceBatch &d, cudaStream_t s);
void launch_nodes(const DeviceBatch &d, cudaStream_t s, int use_given_rhs, unsigned long long cond);
void launch_cg_iteration(const DeviceBatch &d, cudaStream_t s, unsigned long long cond);
void launch_euler(const DeviceBatch &d, cudaStream_t s);
void launch_energies(const DeviceBatch &d, cudaStream_t s);
void launch_apply(const DeviceBatch &d, cudaStream_t s, const double *in, double *out);
void launch_true_residual(const DeviceBatch &d, cudaStream_t s);
void launch_rng_draws(const mrg::JumpMat *table, const uint32_t *state, uint64_t offset, int64_t count, double *out,
                      cudaStream_t s);

int64_t kernel_launch_count();

}  // namespace ffea
