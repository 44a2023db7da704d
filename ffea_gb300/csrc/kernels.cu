// kernels.cu -- sm_103a kernels of the FFEA blob update.
//
// One step of every blob in a batch is:
//   k_elements   per element: Jacobian, shape-function derivatives, volume,
//                inversion check, elastic + bulk + fluctuating (+ viscous for
//                the mass path) stress, nodal forces; writes the element's
//                scaled gradients g = sqrt(vol) dpsi for the assembly
//                (tetra_element_linear.cpp:193-489, Blob.cpp:638-735)
//   k_assemble   per mesh edge: the 3x3 viscosity block as a fixed-order sum
//                over the elements sharing the edge (NoMassCGSolver::init +
//                SparseMatrixFixedPattern::build, without pointer chasing)
//   k_nodes      per linear node: deterministic gather of element forces,
//                Stokes drag and noise, midpoint folding, pins, Jacobi
//                diagonal, and the CG start (Blob.cpp:3826-3928,
//                NoMassCGSolver.cpp:205-230)
//   k_spmv / k_update / k_pupdate    one Jacobi-PCG iteration
//                (NoMassCGSolver.cpp:165-197, ConjugateGradientSolver.cpp:206-232)
//   k_euler      velocity / position update and RNG stream advance
//                (Blob.cpp:3937-3969)
// Reductions are deterministic: a fixed butterfly inside each CTA, one
// partial per CTA, and a fixed-order per-blob sum done by the last CTA to
// finish.  No floating-point atomics are used anywhere.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>

#include "kernels.h"

namespace ffea {

static std::atomic<int64_t> g_launches{0};
int64_t kernel_launch_count() { return g_launches.load(); }
#define FFEA_LAUNCHED() g_launches.fetch_add(1, std::memory_order_relaxed)

namespace {

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum NV values over the CTA; result valid in thread 0.  Fixed order.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) smem[k * 32 + warp] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double t = lane < nw ? smem[k * 32 + lane] : 0.0;
            v[k] = warp_sum(t);
        }
    }
    __syncthreads();
}

// Returns true in every thread of the CTA that finished last.
__device__ __forceinline__ bool last_block(unsigned int *counter, unsigned int total)
{
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int prev = atomicAdd(counter, 1u);
        is_last = (prev == total - 1u);
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last != 0;
}

// Per-blob fixed-order sums of NV partials (stride 4 per tile) over the
// blob's node tiles; one warp per blob.  fin(b, sums) runs in lane 0.
template <int NV, typename Fin>
__device__ __forceinline__ void reduce_node_tiles(const DeviceBatch &d, Fin fin)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int b = warp; b < d.num_blobs; b += nw) {
        const int t0 = d.bp[b].tile_off, tc = d.bp[b].tile_cnt;
        double s[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) s[k] = 0.0;
        for (int t = lane; t < tc; t += 32)
#pragma unroll
            for (int k = 0; k < NV; k++) s[k] += __ldcg(&d.partials[4 * (size_t)(t0 + t) + k]);
#pragma unroll
        for (int k = 0; k < NV; k++) s[k] = warp_sum(s[k]);
        if (lane == 0) fin(b, s);
    }
}

__device__ __forceinline__ void set_condition(unsigned long long cond, unsigned int v)
{
    if (cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, v);
}

// ---------------------------------------------------------------- element math
template <typename T>
struct ElemGeom {
    T dpsi[12];  // d(psi_a)/dx_i at dpsi[4*i + a] (include/tetra_element_linear.h:120-131)
    T det, vol;
};

// calc_shape_function_derivatives_and_volume (src/tetra_element_linear.cpp:223-293)
template <typename T>
__device__ __forceinline__ void shape_functions(const T J[3][3], ElemGeom<T> &g)
{
    T *dpsi = g.dpsi;
    dpsi[1] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    dpsi[2] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    dpsi[3] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    dpsi[5] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
    dpsi[6] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
    dpsi[7] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
    dpsi[9] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
    dpsi[10] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
    dpsi[11] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
    g.det = J[0][0] * dpsi[1] + J[1][0] * dpsi[2] + J[2][0] * dpsi[3];
    g.vol = (T)(1.0 / 6.0) * fabs(g.det);
    const T inv = (T)1 / g.det;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        dpsi[4 * i + 1] *= inv;
        dpsi[4 * i + 2] *= inv;
        dpsi[4 * i + 3] *= inv;
        dpsi[4 * i] = -(dpsi[4 * i + 1] + dpsi[4 * i + 2] + dpsi[4 * i + 3]);
    }
}

template <typename T>
__device__ __forceinline__ void jacobian(const double *pos, int4 c, T J[3][3])
{
    const double x0 = pos[3 * (size_t)c.x], y0 = pos[3 * (size_t)c.x + 1], z0 = pos[3 * (size_t)c.x + 2];
    const int n[3] = {c.y, c.z, c.w};
#pragma unroll
    for (int r = 0; r < 3; r++) {
        J[r][0] = (T)(pos[3 * (size_t)n[r]] - x0);
        J[r][1] = (T)(pos[3 * (size_t)n[r] + 1] - y0);
        J[r][2] = (T)(pos[3 * (size_t)n[r] + 2] - z0);
    }
}

template <typename T>
__device__ __forceinline__ void load_g(const T *g, int el, int a, T out[3])
{
    const T *ge = g + 9 * (size_t)el;
    if (a > 0) {
        out[0] = ge[3 * (a - 1)];
        out[1] = ge[3 * (a - 1) + 1];
        out[2] = ge[3 * (a - 1) + 2];
    } else {
        out[0] = -(ge[0] + ge[3] + ge[6]);
        out[1] = -(ge[1] + ge[4] + ge[7]);
        out[2] = -(ge[2] + ge[5] + ge[8]);
    }
}

// ---------------------------------------------------------------- kernels
// Rest state (Blob::calc_rest_state_info, src/Blob.cpp:3760-3822, with
// mat3_invert src/mat_vec_fns.cpp:148-175), in FP64.
template <typename T>
__global__ void k_rest_state(DeviceBatch d)
{
    const int tile = blockIdx.x;
    const int b = d.etile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int le = tile * ELEM_TILE - bp.elem_off + threadIdx.x;
    if (le >= bp.elem_cnt) return;
    const int e = bp.elem_off + le;
    const int4 c = reinterpret_cast<const int4 *>(d.conn)[e];
    double J[3][3];
    jacobian<double>(d.pos, c, J);
    double mi[3][3];
    mi[0][0] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    mi[0][1] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    mi[0][2] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    mi[1][0] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
    mi[1][1] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
    mi[1][2] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
    mi[2][0] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
    mi[2][1] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
    mi[2][2] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
    const double det = J[0][0] * mi[0][0] + J[1][0] * mi[0][1] + J[2][0] * mi[0][2];
    const double inv = 1.0 / det;
    T *ji = static_cast<T *>(d.jinv0) + 9 * (size_t)e;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) ji[3 * i + k] = (T)(mi[i][k] * inv);
    static_cast<T *>(d.vol0)[e] = (T)((1.0 / 6.0) * fabs(det));
    d.det_sign[e] = det > 0 ? 1 : (det < 0 ? -1 : 0);
}

// The per-step element kernel.
template <typename T>
__global__ void __launch_bounds__(ELEM_TILE) k_elements(DeviceBatch d, int mode)
{
    const int tile = blockIdx.x;
    const int b = d.etile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int le = tile * ELEM_TILE - bp.elem_off + threadIdx.x;
    if (le >= bp.elem_cnt) return;
    if (mode == ELEM_STEP && d.status[b]) return;  // a failed blob stays at its failing step
    const int e = bp.elem_off + le;
    const int4 c = reinterpret_cast<const int4 *>(d.conn)[e];
    T J[3][3];
    jacobian<T>(d.pos, c, J);
    ElemGeom<T> geo;
    shape_functions<T>(J, geo);
    if (mode == ELEM_STEP) {
        const int8_t s = d.det_sign[e];
        if ((T)s * geo.det < (T)0) {  // inversion: last_det * det < 0 (src/tetra_element_linear.cpp:260)
            atomicAdd(&d.inverted[b], 1);
            atomicOr(&d.status[b], BLOB_FAIL_INVERSION);
            return;
        }
        if (geo.det != (T)0) d.det_sign[e] = geo.det > (T)0 ? 1 : -1;
    }
    const Material m = d.mats[d.mat_id[e]];
    const T A = (T)m.A, B = (T)m.B, G = (T)m.G, Eb = (T)m.E;
    const T vol = geo.vol;
    const T *dpsi = geo.dpsi;

    if (bp.solver == SOLVER_NOMASS) {
        // scaled gradients for the assembly: g_a = sqrt(vol) dpsi_a, corners 1..3
        const T sv = sqrt(vol);
        T *gout = static_cast<T *>(d.g) + 9 * (size_t)e;
#pragma unroll
        for (int a = 1; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) gout[3 * (a - 1) + i] = sv * dpsi[4 * i + a];
    }
    if (mode != ELEM_STEP) return;

    // deformation gradient: F = (J_inv_0 J)^T (mat3_mult_both_transposed, src/mat_vec_fns.cpp:104-111)
    const T *ji = static_cast<const T *>(d.jinv0) + 9 * (size_t)e;
    T Jinv0[3][3];
#pragma unroll
    for (int i = 0; i < 9; i++) Jinv0[i / 3][i % 3] = ji[i];
    T F[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) F[i][j] = J[0][i] * Jinv0[j][0] + J[1][i] * Jinv0[j][1] + J[2][i] * Jinv0[j][2];
    // shear + bulk elastic stress (src/tetra_element_linear.cpp:378-408)
    const T vol0 = static_cast<const T *>(d.vol0)[e];
    const T sscale = G * vol0 / vol;
    T S[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) S[i][j] = sscale * (F[i][0] * F[j][0] + F[i][1] * F[j][1] + F[i][2] * F[j][2]);
    const T c2 = Eb - G * (T)(2.0 / 3.0);
    const T cb = G * ((T)1 - vol0 / vol) + (T)0.5 * c2 * (vol / vol0 - vol0 / vol);
    S[0][0] -= G;
    S[1][1] -= G;
    S[2][2] -= G;
    S[0][0] += cb;
    S[1][1] += cb;
    S[2][2] += cb;
    // fluctuating stress: 7 draws at offset 7*element (src/tetra_element_linear.cpp:417-436)
    if (bp.calc_noise == 1) {
        uint32_t st[6];
#pragma unroll
        for (int i = 0; i < 6; i++) st[i] = d.stream_state[6 * bp.stream + i];
        mrg::jump(d.jump_table, bp.elem_draw_base + 7u * (uint32_t)le, st);
        T u[7];
#pragma unroll
        for (int k = 0; k < 7; k++) u[k] = (T)mrg::centred(st);
        const T cf = sqrt(((T)24 * (T)bp.kT) / (vol * (T)bp.dt));
        const T bf = sqrt(B) * u[0];
        const T s2a = sqrt((T)2 * A), sa = sqrt(A);
        S[0][0] += cf * (s2a * u[1] + bf);
        S[1][1] += cf * (s2a * u[2] + bf);
        S[2][2] += cf * (s2a * u[3] + bf);
        S[0][1] += cf * sa * u[4];
        S[0][2] += cf * sa * u[5];
        S[1][2] += cf * sa * u[6];
        S[1][0] = S[0][1];
        S[2][0] = S[0][2];
        S[2][1] = S[1][2];
    }
    if (bp.solver == SOLVER_MASS) {
        // viscous stress A (L + L^T) + B tr(L) I from the velocity gradient
        // L_ij = sum_b v_b,i dpsi_b,j; equal to viscosity_matrix * v
        // (src/tetra_element_linear.cpp:299-328, src/Blob.cpp:703-706)
        T L[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        const int cn[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const T v0 = (T)d.vel[3 * (size_t)cn[a]], v1 = (T)d.vel[3 * (size_t)cn[a] + 1],
                    v2 = (T)d.vel[3 * (size_t)cn[a] + 2];
#pragma unroll
            for (int j = 0; j < 3; j++) {
                L[0][j] += v0 * dpsi[4 * j + a];
                L[1][j] += v1 * dpsi[4 * j + a];
                L[2][j] += v2 * dpsi[4 * j + a];
            }
        }
        const T tr = L[0][0] + L[1][1] + L[2][2];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) S[i][j] += A * (L[i][j] + L[j][i]) + (i == j ? B * tr : (T)0);
    }
    // nodal forces: node_force[a] = -vol * S dpsi_a (src/tetra_element_linear.cpp:441-489)
    T *fo = static_cast<T *>(d.efrc) + 12 * (size_t)e;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++)
            fo[3 * a + i] = -(vol * (dpsi[a] * S[i][0] + dpsi[4 + a] * S[i][1] + dpsi[8 + a] * S[i][2]));
}

// Edge blocks of the viscosity matrix: K_pq = sum over elements e holding
// edge (p,q) of vol_e [A (delta_ik dpsi_a.dpsi_b + dpsi_a,k dpsi_b,i) + B dpsi_a,i dpsi_b,k]
// (include/tetra_element_linear.h:55-116 + add_diffusion_matrix).
template <typename T>
__global__ void __launch_bounds__(EDGE_TILE) k_assemble(DeviceBatch d)
{
    const int e = blockIdx.x * EDGE_TILE + threadIdx.x;
    if (e >= d.n_edges) return;
    T K[9];
#pragma unroll
    for (int i = 0; i < 9; i++) K[i] = (T)0;
    const T *g = static_cast<const T *>(d.g);
    for (int k = d.edge_cptr[e]; k < d.edge_cptr[e + 1]; k++) {
        const int ci = d.edge_cidx[k];
        const int el = ci >> 4, a = (ci >> 2) & 3, bb = ci & 3;
        T ga[3], gb[3];
        load_g<T>(g, el, a, ga);
        load_g<T>(g, el, bb, gb);
        const Material m = d.mats[d.mat_id[el]];
        const T A = (T)m.A, B = (T)m.B;
        const T gab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) K[3 * i + j] += A * ((i == j ? gab : (T)0) + ga[j] * gb[i]) + B * ga[i] * gb[j];
    }
    T *out = static_cast<T *>(d.blocks) + 9 * (size_t)e;
#pragma unroll
    for (int i = 0; i < 9; i++) out[i] = K[i];
}

// Mass matrix (ConjugateGradientSolver::init, src/ConjugateGradientSolver.cpp:62-204):
// per edge sum of 0.05 rho V0, per node sum of 0.1 rho V0; identity on pinned rows.
template <typename T>
__global__ void k_mass_matrix(DeviceBatch d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.n_edges) {
        double s = 0.0;
        for (int k = d.edge_cptr[i]; k < d.edge_cptr[i + 1]; k++) {
            const int el = d.edge_cidx[k] >> 4;
            s += .05 * d.mats[d.mat_id[el]].rho * (double)static_cast<const T *>(d.vol0)[el];
        }
        const bool pinned = (d.flags[d.edge_p[i]] | d.flags[d.edge_q[i]]) & NODE_PINNED;
        static_cast<T *>(d.mass_edge)[i] = pinned ? (T)0 : (T)s;
    }
    if (i < d.nl_pad) {
        double s = 0.0;
        for (int k = d.gather_ptr[i]; k < d.gather_ptr[i + 1]; k++) {
            const int el = d.gather_idx[k] >> 2;
            s += .1 * d.mats[d.mat_id[el]].rho * (double)static_cast<const T *>(d.vol0)[el];
        }
        const bool pinned = d.flags[i] & NODE_PINNED;
        static_cast<T *>(d.mass_diag)[i] = pinned ? (T)1 : (T)s;
        static_cast<T *>(d.dinv)[3 * (size_t)i] = pinned ? (T)1 : (T)(1.0 / s);
        static_cast<T *>(d.dinv)[3 * (size_t)i + 1] = pinned ? (T)1 : (T)(1.0 / s);
        static_cast<T *>(d.dinv)[3 * (size_t)i + 2] = pinned ? (T)1 : (T)(1.0 / s);
    }
}

// Node kernel: rhs and the CG start.
template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_nodes(DeviceBatch d, int use_given_rhs, unsigned long long cond)
{
    __shared__ double red[2 * 32];
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int row = tile * NODE_TILE + threadIdx.x;
    const int local = row - bp.node_off;
    const bool failed = d.status[b] != 0;
    const bool valid = local < bp.node_cnt && !(d.flags[row] & NODE_PINNED) && !failed;
    const bool nomass = bp.solver == SOLVER_NOMASS;
    double f[3] = {0.0, 0.0, 0.0};
    double D[3] = {0.0, 0.0, 0.0};
    const double drag = bp.calc_stokes == 1 ? d.drag[row] : 0.0;
    if (valid) {
        const T *ef = static_cast<const T *>(d.efrc);
        const T *g = static_cast<const T *>(d.g);
        for (int k = d.gather_ptr[row]; k < d.gather_ptr[row + 1]; k++) {
            const int gi = d.gather_idx[k];
            const int el = gi >> 2, a = gi & 3;
            if (!use_given_rhs) {
                f[0] += (double)ef[12 * (size_t)el + 3 * a];
                f[1] += (double)ef[12 * (size_t)el + 3 * a + 1];
                f[2] += (double)ef[12 * (size_t)el + 3 * a + 2];
            }
            if (nomass) {
                T ga[3];
                load_g<T>(g, el, a, ga);
                const Material m = d.mats[d.mat_id[el]];
                const T gg = ga[0] * ga[0] + ga[1] * ga[1] + ga[2] * ga[2];
#pragma unroll
                for (int i = 0; i < 3; i++) D[i] += (double)((T)m.A * (gg + ga[i] * ga[i]) + (T)m.B * ga[i] * ga[i]);
            }
        }
        if (!use_given_rhs) {
            if (!nomass && bp.calc_stokes == 1) {
#pragma unroll
                for (int i = 0; i < 3; i++) f[i] -= d.vel[3 * (size_t)row + i] * drag;
            }
            if (bp.calc_noise == 1 && bp.calc_stokes == 1) {
                const uint32_t *s0 = d.stream_state + 6 * bp.stream;
                if (drag != 0.0) {
                    uint32_t st[6];
#pragma unroll
                    for (int i = 0; i < 6; i++) st[i] = s0[i];
                    mrg::jump(d.jump_table, bp.node_draw_base + 3u * (uint32_t)d.orig[row], st);
                    const double amp = sqrt((24 * bp.kT * drag) / (bp.dt));
#pragma unroll
                    for (int i = 0; i < 3; i++) f[i] -= mrg::centred(st) * amp;
                }
                // secondary nodes with a drag: half of their force lands here
                for (int k = d.fold_ptr[row]; k < d.fold_ptr[row + 1]; k++) {
                    uint32_t st[6];
#pragma unroll
                    for (int i = 0; i < 6; i++) st[i] = s0[i];
                    mrg::jump(d.jump_table, bp.node_draw_base + 3u * (uint32_t)d.fold_sec[k], st);
                    const double amp = sqrt((24 * bp.kT * d.fold_drag[k]) / (bp.dt));
#pragma unroll
                    for (int i = 0; i < 3; i++) f[i] += 0.5 * (-(mrg::centred(st) * amp));
                }
            }
        }
    }
    if (use_given_rhs && valid) {
#pragma unroll
        for (int i = 0; i < 3; i++) f[i] = d.rhs[3 * (size_t)row + i];
    }
    T *dinv = static_cast<T *>(d.dinv);
    if (nomass) {
#pragma unroll
        for (int i = 0; i < 3; i++) dinv[3 * (size_t)row + i] = valid ? (T)(1.0 / (D[i] + drag)) : (T)1;
    }
    double rz = 0.0, ff = 0.0;
    T *p = static_cast<T *>(d.p);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const size_t k = 3 * (size_t)row + i;
        const double fi = valid ? f[i] : 0.0;
        if (!use_given_rhs) d.rhs[k] = fi;
        d.x[k] = 0.0;
        d.r[k] = fi;
        const double z = (double)dinv[k] * fi;
        p[k] = (T)z;
        rz += fi * z;
        ff += fi * fi;
    }
    double v[2] = {rz, ff};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        d.partials[4 * (size_t)tile] = v[0];
        d.partials[4 * (size_t)tile + 1] = v[1];
    }
    if (last_block(&d.counters[CNT_NODES], gridDim.x)) {
        __shared__ int running;
        if (threadIdx.x == 0) running = 0;
        __syncthreads();
        reduce_node_tiles<2>(d, [&](int bb, const double *s) {
            CgScalars &cg = d.cg[bb];
            cg.delta = s[0];
            cg.ff = s[1];
            cg.pq = cg.rr = cg.alpha = cg.beta = 0.0;
            cg.iters = 0;
            cg.true_relres2 = -1.0;
            const bool done = (d.status[bb] != 0) || s[1] == 0.0;
            cg.converged = done ? 1 : 0;
            cg.active = 1;
            if (!done) atomicOr(&running, 1);
        });
        __syncthreads();
        if (threadIdx.x == 0) {
            *d.any_running = running;
            set_condition(cond, running ? 1u : 0u);
            d.counters[CNT_NODES] = 0;
        }
    }
}

// q = A p for one row (difference form for the viscosity matrix), T arithmetic.
template <typename T>
__device__ __forceinline__ void row_apply(const DeviceBatch &d, int row, bool nomass, double drag, const T *p, T out[3])
{
    const T p0 = p[3 * (size_t)row], p1 = p[3 * (size_t)row + 1], p2 = p[3 * (size_t)row + 2];
    T a0 = 0, a1 = 0, a2 = 0;
    if (nomass) {
        const T *blk = static_cast<const T *>(d.blocks);
        // edges (row, q), q > row: K_pq = stored block
        for (int e = d.up_ptr[row]; e < d.up_ptr[row + 1]; e++) {
            const int qn = d.edge_q[e];
            const T d0 = p[3 * (size_t)qn] - p0, d1 = p[3 * (size_t)qn + 1] - p1, d2 = p[3 * (size_t)qn + 2] - p2;
            const T *K = blk + 9 * (size_t)e;
            a0 += K[0] * d0 + K[1] * d1 + K[2] * d2;
            a1 += K[3] * d0 + K[4] * d1 + K[5] * d2;
            a2 += K[6] * d0 + K[7] * d1 + K[8] * d2;
        }
        // edges (q, row), q < row: K_pq = (stored block)^T
        for (int k = d.lo_ptr[row]; k < d.lo_ptr[row + 1]; k++) {
            const int e = d.lo_edge[k];
            const int qn = d.edge_p[e];
            const T d0 = p[3 * (size_t)qn] - p0, d1 = p[3 * (size_t)qn + 1] - p1, d2 = p[3 * (size_t)qn + 2] - p2;
            const T *K = blk + 9 * (size_t)e;
            a0 += K[0] * d0 + K[3] * d1 + K[6] * d2;
            a1 += K[1] * d0 + K[4] * d1 + K[7] * d2;
            a2 += K[2] * d0 + K[5] * d1 + K[8] * d2;
        }
        const T dr = (T)drag;
        a0 += dr * p0;
        a1 += dr * p1;
        a2 += dr * p2;
    } else {
        const T *me = static_cast<const T *>(d.mass_edge);
        const T md = static_cast<const T *>(d.mass_diag)[row];
        a0 = md * p0;
        a1 = md * p1;
        a2 = md * p2;
        for (int e = d.up_ptr[row]; e < d.up_ptr[row + 1]; e++) {
            const int qn = d.edge_q[e];
            const T m = me[e];
            a0 += m * p[3 * (size_t)qn];
            a1 += m * p[3 * (size_t)qn + 1];
            a2 += m * p[3 * (size_t)qn + 2];
        }
        for (int k = d.lo_ptr[row]; k < d.lo_ptr[row + 1]; k++) {
            const int e = d.lo_edge[k];
            const int qn = d.edge_p[e];
            const T m = me[e];
            a0 += m * p[3 * (size_t)qn];
            a1 += m * p[3 * (size_t)qn + 1];
            a2 += m * p[3 * (size_t)qn + 2];
        }
    }
    out[0] = a0;
    out[1] = a1;
    out[2] = a2;
}

template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_spmv(DeviceBatch d)
{
    __shared__ double red[32];
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const bool run = d.cg[b].converged == 0;
    double pq = 0.0;
    if (run) {
        const int row = tile * NODE_TILE + threadIdx.x;
        const bool valid = (row - bp.node_off) < bp.node_cnt && !(d.flags[row] & NODE_PINNED);
        const T *p = static_cast<const T *>(d.p);
        T q[3] = {0, 0, 0};
        if (valid) {
            const double drag = bp.calc_stokes == 1 ? d.drag[row] : 0.0;
            row_apply<T>(d, row, bp.solver == SOLVER_NOMASS, drag, p, q);
            pq = (double)p[3 * (size_t)row] * (double)q[0] + (double)p[3 * (size_t)row + 1] * (double)q[1] +
                 (double)p[3 * (size_t)row + 2] * (double)q[2];
        }
        T *qo = static_cast<T *>(d.q);
        qo[3 * (size_t)row] = q[0];
        qo[3 * (size_t)row + 1] = q[1];
        qo[3 * (size_t)row + 2] = q[2];
    }
    double v[1] = {pq};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) d.partials[4 * (size_t)tile + 2] = v[0];
    if (last_block(&d.counters[CNT_SPMV], gridDim.x)) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            if (d.cg[bb].converged) continue;
            const int t0 = d.bp[bb].tile_off, tc = d.bp[bb].tile_cnt;
            double s = 0.0;
            for (int t = lane; t < tc; t += 32) s += __ldcg(&d.partials[4 * (size_t)(t0 + t) + 2]);
            s = warp_sum(s);
            if (lane == 0) {
                d.cg[bb].pq = s;
                d.cg[bb].alpha = d.cg[bb].delta / s;
            }
        }
        if (threadIdx.x == 0) d.counters[CNT_SPMV] = 0;
    }
}

template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_update(DeviceBatch d, unsigned long long cond)
{
    __shared__ double red[2 * 32];
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const bool run = d.cg[b].converged == 0;
    double rr = 0.0, rz = 0.0;
    if (run) {
        const int row = tile * NODE_TILE + threadIdx.x;
        const double alpha = d.cg[b].alpha;
        const T *p = static_cast<const T *>(d.p);
        const T *q = static_cast<const T *>(d.q);
        const T *dinv = static_cast<const T *>(d.dinv);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const size_t k = 3 * (size_t)row + i;
            d.x[k] += alpha * (double)p[k];
            const double r = d.r[k] + (-alpha) * (double)q[k];
            d.r[k] = r;
            rr += r * r;
            rz += r * ((double)dinv[k] * r);
        }
    }
    double v[2] = {rr, rz};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        d.partials[4 * (size_t)tile] = v[0];
        d.partials[4 * (size_t)tile + 1] = v[1];
    }
    if (last_block(&d.counters[CNT_UPDATE], gridDim.x)) {
        __shared__ int running;
        if (threadIdx.x == 0) running = 0;
        __syncthreads();
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            CgScalars &cg = d.cg[bb];
            if (cg.converged) continue;
            const int t0 = d.bp[bb].tile_off, tc = d.bp[bb].tile_cnt;
            double s0 = 0.0, s1 = 0.0;
            for (int t = lane; t < tc; t += 32) {
                s0 += __ldcg(&d.partials[4 * (size_t)(t0 + t)]);
                s1 += __ldcg(&d.partials[4 * (size_t)(t0 + t) + 1]);
            }
            s0 = warp_sum(s0);
            s1 = warp_sum(s1);
            if (lane == 0) {
                cg.iters += 1;
                cg.rr = s0;
                // residual2() = sum r^2 / sum f^2 (src/NoMassCGSolver.cpp:233-247)
                const double res = (cg.ff == 0.0) ? 0.0 : s0 / cg.ff;
                const int limit = d.bp[bb].solver == SOLVER_MASS ? d.bp[bb].max_iter - 1 : d.bp[bb].max_iter;
                if (res < d.bp[bb].epsilon2) {
                    cg.converged = 1;
                } else if (!(res == res) || cg.iters >= limit) {
                    cg.converged = 1;
                    atomicOr(&d.status[bb], (res == res) ? BLOB_FAIL_CG : (BLOB_FAIL_CG | BLOB_FAIL_NAN));
                } else {
                    cg.beta = s1 / cg.delta;
                    cg.delta = s1;
                    atomicOr(&running, 1);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            *d.any_running = running;
            set_condition(cond, running ? 1u : 0u);
            d.counters[CNT_UPDATE] = 0;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_pupdate(DeviceBatch d)
{
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    if (d.cg[b].converged) return;
    const double beta = d.cg[b].beta;
    const int row = tile * NODE_TILE + threadIdx.x;
    T *p = static_cast<T *>(d.p);
    const T *dinv = static_cast<const T *>(d.dinv);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const size_t k = 3 * (size_t)row + i;
        // vec3_scale_and_add: p = beta p + z (src/mat_vec_fns.cpp:265-275)
        p[k] = (T)(beta * (double)p[k] + (double)dinv[k] * d.r[k]);
    }
}

// Euler update (src/Blob.cpp:3937-3969) and the RNG advance to the next step.
__global__ void __launch_bounds__(NODE_TILE) k_euler(DeviceBatch d)
{
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int row = tile * NODE_TILE + threadIdx.x;
    if (row < d.num_streams) {  // the grid has at least 256 threads per blob
        const int s = row;
        bool advance = true;
        if (d.num_streams == d.num_blobs) advance = d.status[s] == 0;  // per-blob streams
        if (advance) {
            uint32_t st[6];
#pragma unroll
            for (int i = 0; i < 6; i++) st[i] = d.stream_state[6 * s + i];
            mrg::apply(d.stream_step[s], st);
#pragma unroll
            for (int i = 0; i < 6; i++) d.stream_state[6 * s + i] = st[i];
        }
    }
    if (row - bp.node_off >= bp.node_cnt || d.status[b]) return;
    const double dt = bp.dt;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const size_t k = 3 * (size_t)row + i;
        if (bp.solver == SOLVER_NOMASS) {
            const double x = d.x[k];
            d.vel[k] = x;
            d.pos[k] += x * dt;
        } else {
            const double v = d.vel[k] + d.x[k] * dt;
            d.vel[k] = v;
            d.pos[k] += v * dt;
        }
    }
}

// Strain (and kinetic) energy at the current state, FP64
// (Blob::make_measurements, src/Blob.cpp:1363-1432).
template <typename T>
__global__ void __launch_bounds__(ELEM_TILE) k_energies(DeviceBatch d)
{
    __shared__ double red[2 * 32];
    const int tile = blockIdx.x;
    const int b = d.etile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int le = tile * ELEM_TILE - bp.elem_off + threadIdx.x;
    double se = 0.0, ke = 0.0;
    if (le < bp.elem_cnt) {
        const int e = bp.elem_off + le;
        const int4 c = reinterpret_cast<const int4 *>(d.conn)[e];
        double J[3][3];
        jacobian<double>(d.pos, c, J);
        ElemGeom<double> geo;
        shape_functions<double>(J, geo);
        const T *ji = static_cast<const T *>(d.jinv0) + 9 * (size_t)e;
        double F[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                F[i][j] = J[0][i] * (double)ji[3 * j] + J[1][i] * (double)ji[3 * j + 1] + J[2][i] * (double)ji[3 * j + 2];
        double ff = 0;
        for (int i = 0; i < 9; i++) ff += F[i / 3][i % 3] * F[i / 3][i % 3];
        const Material m = d.mats[d.mat_id[e]];
        const double vol0 = (double)static_cast<const T *>(d.vol0)[e];
        const double C = m.E - (2.0 / 3.0) * m.G;
        const double t1 = geo.vol / vol0;
        se = vol0 * (m.G * (ff - 3) + 0.5 * C * (t1 * t1 - 1) - (C + 2 * m.G) * log(t1));
        if (bp.solver == SOLVER_MASS) {
            const int cn[4] = {c.x, c.y, c.z, c.w};
            for (int i = 0; i < 3; i++)
                for (int a = 0; a < 4; a++) {
                    double mv = 0;
                    for (int bq = 0; bq < 4; bq++) mv += (a == bq ? .1 : .05) * d.vel[3 * (size_t)cn[bq] + i];
                    ke += d.vel[3 * (size_t)cn[a] + i] * mv * (vol0 * m.rho);
                }
        }
    }
    double v[2] = {se, ke};
    block_sum<2>(v, red);
    if (threadIdx.x == 0) {
        d.epartials[2 * (size_t)tile] = v[0];
        d.epartials[2 * (size_t)tile + 1] = v[1];
    }
    if (last_block(&d.counters[CNT_ENERGY], gridDim.x)) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            const int t0 = d.bp[bb].elem_off / ELEM_TILE, tc = d.bp[bb].elem_pad / ELEM_TILE;
            double s0 = 0.0, s1 = 0.0;
            for (int t = lane; t < tc; t += 32) {
                s0 += __ldcg(&d.epartials[2 * (size_t)(t0 + t)]);
                s1 += __ldcg(&d.epartials[2 * (size_t)(t0 + t) + 1]);
            }
            s0 = warp_sum(s0);
            s1 = warp_sum(s1);
            if (lane == 0) {
                d.energy[2 * bb] = 0.5 * s0;
                d.energy[2 * bb + 1] = 0.5 * s1;
            }
        }
        if (threadIdx.x == 0) d.counters[CNT_ENERGY] = 0;
    }
}

// out = A in (FP64 vectors), pinned rows and padding excluded (callers handle them).
template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_apply(DeviceBatch d, const double *in, double *out)
{
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int row = tile * NODE_TILE + threadIdx.x;
    const bool valid = (row - bp.node_off) < bp.node_cnt && !(d.flags[row] & NODE_PINNED);
    double acc[3] = {0.0, 0.0, 0.0};
    if (valid) {
        const double drag = bp.calc_stokes == 1 ? d.drag[row] : 0.0;
        const double p0 = in[3 * (size_t)row], p1 = in[3 * (size_t)row + 1], p2 = in[3 * (size_t)row + 2];
        if (bp.solver == SOLVER_NOMASS) {
            const T *blk = static_cast<const T *>(d.blocks);
            for (int e = d.up_ptr[row]; e < d.up_ptr[row + 1]; e++) {
                const int qn = d.edge_q[e];
                const double d0 = in[3 * (size_t)qn] - p0, d1 = in[3 * (size_t)qn + 1] - p1, d2 = in[3 * (size_t)qn + 2] - p2;
                const T *K = blk + 9 * (size_t)e;
                acc[0] += (double)K[0] * d0 + (double)K[1] * d1 + (double)K[2] * d2;
                acc[1] += (double)K[3] * d0 + (double)K[4] * d1 + (double)K[5] * d2;
                acc[2] += (double)K[6] * d0 + (double)K[7] * d1 + (double)K[8] * d2;
            }
            for (int k = d.lo_ptr[row]; k < d.lo_ptr[row + 1]; k++) {
                const int e = d.lo_edge[k];
                const int qn = d.edge_p[e];
                const double d0 = in[3 * (size_t)qn] - p0, d1 = in[3 * (size_t)qn + 1] - p1, d2 = in[3 * (size_t)qn + 2] - p2;
                const T *K = blk + 9 * (size_t)e;
                acc[0] += (double)K[0] * d0 + (double)K[3] * d1 + (double)K[6] * d2;
                acc[1] += (double)K[1] * d0 + (double)K[4] * d1 + (double)K[7] * d2;
                acc[2] += (double)K[2] * d0 + (double)K[5] * d1 + (double)K[8] * d2;
            }
            acc[0] += drag * p0;
            acc[1] += drag * p1;
            acc[2] += drag * p2;
        } else {
            const T *me = static_cast<const T *>(d.mass_edge);
            const double md = (double)static_cast<const T *>(d.mass_diag)[row];
            acc[0] = md * p0;
            acc[1] = md * p1;
            acc[2] = md * p2;
            for (int e = d.up_ptr[row]; e < d.up_ptr[row + 1]; e++) {
                const int qn = d.edge_q[e];
                for (int i = 0; i < 3; i++) acc[i] += (double)me[e] * in[3 * (size_t)qn + i];
            }
            for (int k = d.lo_ptr[row]; k < d.lo_ptr[row + 1]; k++) {
                const int e = d.lo_edge[k];
                const int qn = d.edge_p[e];
                for (int i = 0; i < 3; i++) acc[i] += (double)me[e] * in[3 * (size_t)qn + i];
            }
        }
    }
    for (int i = 0; i < 3; i++) out[3 * (size_t)row + i] = acc[i];
}

// FP64 true residual of the last solve: || rhs - A x ||^2 / ||rhs||^2 per blob.
template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_true_residual(DeviceBatch d)
{
    __shared__ double red[32];
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int row = tile * NODE_TILE + threadIdx.x;
    const bool valid = (row - bp.node_off) < bp.node_cnt && !(d.flags[row] & NODE_PINNED) && d.status[b] == 0;
    double rr = 0.0;
    if (valid) {
        // A x with FP64 accumulation; x is FP64, blocks T.
        const double drag = bp.calc_stokes == 1 ? d.drag[row] : 0.0;
        const double *x = d.x;
        const double x0 = x[3 * (size_t)row], x1 = x[3 * (size_t)row + 1], x2 = x[3 * (size_t)row + 2];
        double a[3] = {0.0, 0.0, 0.0};
        if (bp.solver == SOLVER_NOMASS) {
            const T *blk = static_cast<const T *>(d.blocks);
            for (int e = d.up_ptr[row]; e < d.up_ptr[row + 1]; e++) {
                const int qn = d.edge_q[e];
                const double d0 = x[3 * (size_t)qn] - x0, d1 = x[3 * (size_t)qn + 1] - x1, d2 = x[3 * (size_t)qn + 2] - x2;
                const T *K = blk + 9 * (size_t)e;
                a[0] += (double)K[0] * d0 + (double)K[1] * d1 + (double)K[2] * d2;
                a[1] += (double)K[3] * d0 + (double)K[4] * d1 + (double)K[5] * d2;
                a[2] += (double)K[6] * d0 + (double)K[7] * d1 + (double)K[8] * d2;
            }
            for (int k = d.lo_ptr[row]; k < d.lo_ptr[row + 1]; k++) {
                const int e = d.lo_edge[k];
                const int qn = d.edge_p[e];
                const double d0 = x[3 * (size_t)qn] - x0, d1 = x[3 * (size_t)qn + 1] - x1, d2 = x[3 * (size_t)qn + 2] - x2;
                const T *K = blk + 9 * (size_t)e;
                a[0] += (double)K[0] * d0 + (double)K[3] * d1 + (double)K[6] * d2;
                a[1] += (double)K[1] * d0 + (double)K[4] * d1 + (double)K[7] * d2;
                a[2] += (double)K[2] * d0 + (double)K[5] * d1 + (double)K[8] * d2;
            }
            a[0] += drag * x0;
            a[1] += drag * x1;
            a[2] += drag * x2;
        } else {
            const T *me = static_cast<const T *>(d.mass_edge);
            const double md = (double)static_cast<const T *>(d.mass_diag)[row];
            a[0] = md * x0;
            a[1] = md * x1;
            a[2] = md * x2;
            for (int e = d.up_ptr[row]; e < d.up_ptr[row + 1]; e++)
                for (int i = 0; i < 3; i++) a[i] += (double)me[e] * x[3 * (size_t)d.edge_q[e] + i];
            for (int k = d.lo_ptr[row]; k < d.lo_ptr[row + 1]; k++) {
                const int e = d.lo_edge[k];
                for (int i = 0; i < 3; i++) a[i] += (double)me[e] * x[3 * (size_t)d.edge_p[e] + i];
            }
        }
        for (int i = 0; i < 3; i++) {
            const double r = d.rhs[3 * (size_t)row + i] - a[i];
            rr += r * r;
        }
    }
    double v[1] = {rr};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) d.partials[4 * (size_t)tile + 3] = v[0];
    if (last_block(&d.counters[CNT_TRUERES], gridDim.x)) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            const int t0 = d.bp[bb].tile_off, tc = d.bp[bb].tile_cnt;
            double s = 0.0;
            for (int t = lane; t < tc; t += 32) s += __ldcg(&d.partials[4 * (size_t)(t0 + t) + 3]);
            s = warp_sum(s);
            if (lane == 0) d.cg[bb].true_relres2 = d.cg[bb].ff == 0.0 ? 0.0 : s / d.cg[bb].ff;
        }
        if (threadIdx.x == 0) d.counters[CNT_TRUERES] = 0;
    }
}

__global__ void k_rng_draws(const mrg::JumpMat *table, const uint32_t *state, uint64_t offset, int64_t count,
                            double *out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint32_t st[6];
    for (int k = 0; k < 6; k++) st[k] = state[k];
    // offsets beyond 2^32 jump in 2^32 chunks via the top table level squared
    uint64_t off = offset + (uint64_t)i;
    while (off >> 32) {
        // A^(2^32) = (A^(2^24))^256 = table[3*256 + 255] * table[3*256 + 1]
        mrg::apply(table[(3 << 8) + 255], st);
        mrg::apply(table[(3 << 8) + 1], st);
        off -= (1ull << 32);
    }
    mrg::jump(table, (uint32_t)off, st);
    out[i] = mrg::u01(st);
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------- launchers
#define PREC_DISPATCH(d, KERNEL, GRID, BLOCK, STREAM, ...)                        \
    do {                                                                          \
        if ((d).precision == PREC_FP64)                                           \
            KERNEL<double><<<(GRID), (BLOCK), 0, (STREAM)>>>(__VA_ARGS__);        \
        else                                                                      \
            KERNEL<float><<<(GRID), (BLOCK), 0, (STREAM)>>>(__VA_ARGS__);         \
        FFEA_LAUNCHED();                                                          \
    } while (0)

void launch_rest_state(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_rest_state, d.n_etiles, ELEM_TILE, s, d);
}

void launch_mass_matrix(const DeviceBatch &d, cudaStream_t s)
{
    const int64_t n = d.n_edges > d.nl_pad ? d.n_edges : d.nl_pad;
    PREC_DISPATCH(d, k_mass_matrix, blocks_for(n, 256), 256, s, d);
}

void launch_elements(const DeviceBatch &d, cudaStream_t s, int mode)
{
    PREC_DISPATCH(d, k_elements, d.n_etiles, ELEM_TILE, s, d, mode);
}

void launch_assemble(const DeviceBatch &d, cudaStream_t s)
{
    if (d.n_edges == 0) return;
    PREC_DISPATCH(d, k_assemble, blocks_for(d.n_edges, EDGE_TILE), EDGE_TILE, s, d);
}

void launch_nodes(const DeviceBatch &d, cudaStream_t s, int use_given_rhs, unsigned long long cond)
{
    PREC_DISPATCH(d, k_nodes, d.n_tiles, NODE_TILE, s, d, use_given_rhs, cond);
}

void launch_cg_iteration(const DeviceBatch &d, cudaStream_t s, unsigned long long cond)
{
    PREC_DISPATCH(d, k_spmv, d.n_tiles, NODE_TILE, s, d);
    PREC_DISPATCH(d, k_update, d.n_tiles, NODE_TILE, s, d, cond);
    PREC_DISPATCH(d, k_pupdate, d.n_tiles, NODE_TILE, s, d);
}

void launch_euler(const DeviceBatch &d, cudaStream_t s)
{
    k_euler<<<d.n_tiles, NODE_TILE, 0, s>>>(d);
    FFEA_LAUNCHED();
}

void launch_energies(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_energies, d.n_etiles, ELEM_TILE, s, d);
}

void launch_apply(const DeviceBatch &d, cudaStream_t s, const double *in, double *out)
{
    PREC_DISPATCH(d, k_apply, d.n_tiles, NODE_TILE, s, d, in, out);
}

void launch_true_residual(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_true_residual, d.n_tiles, NODE_TILE, s, d);
}

void launch_rng_draws(const mrg::JumpMat *table, const uint32_t *state, uint64_t offset, int64_t count, double *out,
                      cudaStream_t s)
{
    if (count <= 0) return;
    k_rng_draws<<<blocks_for(count, 256), 256, 0, s>>>(table, state, offset, count, out);
    FFEA_LAUNCHED();
}

}  // namespace ffea
