// kernels.cu -- sm_103a kernels of the FFEA blob update.
//
// One step of every blob in a batch is:
//   k_elements   per element: Jacobian, shape-function derivatives, volume,
//                inversion check, elastic + bulk + fluctuating (+ viscous for
//                the mass path) stress, nodal forces; writes the element's
//                scaled gradients g = sqrt(vol) dpsi for the assembly
//                (tetra_element_linear.cpp:193-489, Blob.cpp:638-735)
//   k_assemble   per mesh edge: the 3x3 viscosity block as a fixed-order sum
//                over the elements sharing the edge, written into both rows of
//                the SELL-32 matrix (NoMassCGSolver::init + SparseMatrixFixedPattern::build)
//   k_nodes      per linear node: deterministic gather of element forces,
//                Stokes drag and noise, midpoint folding, pins, Jacobi
//                diagonal, and the CG start (Blob.cpp:3826-3928,
//                NoMassCGSolver.cpp:205-230)
//   k_cg         the whole Jacobi-PCG solve in one persistent cooperative
//                launch (NoMassCGSolver.cpp:165-197, ConjugateGradientSolver.cpp:206-232)
//   k_euler      velocity / position update and RNG stream advance
//                (Blob.cpp:3937-3969)
// Reductions are deterministic: fixed butterflies inside warps and CTAs, one
// partial per node tile, and fixed-order per-blob sums.  No floating-point
// atomics are used anywhere.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>

#include "kernels.h"

namespace ffea {

static std::atomic<int64_t> g_launches{0};
int64_t kernel_launch_count() { return g_launches.load(); }
void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
#define FFEA_LAUNCHED() g_launches.fetch_add(1, std::memory_order_relaxed)

namespace {

// ---------------------------------------------------------------- reductions
template <typename A>
__device__ __forceinline__ A warp_sum(A v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum NV per-thread values over the CTA; the butterfly inside each warp runs
// in W (float for the mixed path: GB300's FP64 rate is a small fraction of
// FP32), the per-warp results are summed in FP64.  Result valid in thread 0.
template <int NV, typename W>
__device__ __forceinline__ void block_sum(const W (&in)[NV], double (&out)[NV], double *smem)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        const W s = warp_sum<W>(in[k]);
        if (lane == 0) smem[k * 32 + warp] = (double)s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) out[k] = warp_sum<double>(lane < nw ? smem[k * 32 + lane] : 0.0);
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

// SELL-32 value index of component k (0..8 row-major 3x3) of entry `off`
__device__ __forceinline__ size_t sell_vidx(int off, int k)
{
    return (size_t)(off & ~31) * 9 + (size_t)k * 32 + (off & 31);
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

// Viscosity blocks: K_pq = sum over elements e holding edge (p,q) of
// vol_e [A (delta_ik dpsi_a.dpsi_b + dpsi_a,k dpsi_b,i) + B dpsi_a,i dpsi_b,k]
// (include/tetra_element_linear.h:55-116 + add_diffusion_matrix), written to
// row p as K_pq and to row q as K_pq^T.
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
    T *val = static_cast<T *>(d.sell_val);
    const int opq = d.edge_pos_pq[e], oqp = d.edge_pos_qp[e];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            val[sell_vidx(opq, 3 * i + j)] = K[3 * i + j];
            val[sell_vidx(oqp, 3 * j + i)] = K[3 * i + j];
        }
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
        T *mv = static_cast<T *>(d.sell_mval);
        mv[d.edge_pos_pq[i]] = pinned ? (T)0 : (T)s;
        mv[d.edge_pos_qp[i]] = pinned ? (T)0 : (T)s;
    }
    if (i < d.nl_pad) {
        double s = 0.0;
        for (int k = d.gather_ptr[i]; k < d.gather_ptr[i + 1]; k++) {
            const int el = d.gather_idx[k] >> 2;
            s += .1 * d.mats[d.mat_id[el]].rho * (double)static_cast<const T *>(d.vol0)[el];
        }
        const bool pinned = (d.flags[i] & NODE_PINNED) || s == 0.0;
        static_cast<T *>(d.mass_diag)[i] = pinned ? (T)1 : (T)s;
        T *dinv = static_cast<T *>(d.dinv);
#pragma unroll
        for (int c = 0; c < 3; c++) dinv[3 * (size_t)i + c] = pinned ? (T)1 : (T)(1.0 / s);
    }
}

// Node kernel: rhs and the CG start.
template <typename T>
__global__ void __launch_bounds__(NODE_TILE) k_nodes(DeviceBatch d, int use_given_rhs)
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
    // CG start (Chronopoulos-Gear form): x = 0, r = f, u = D^-1 r, p = s = w = 0
    T *x = static_cast<T *>(d.x), *r = static_cast<T *>(d.r), *u = static_cast<T *>(d.u);
    T *p = static_cast<T *>(d.p), *sv = static_cast<T *>(d.s), *w = static_cast<T *>(d.w);
    double gam = 0.0, ff = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const size_t k = 3 * (size_t)row + i;
        const double fi = valid ? f[i] : 0.0;
        if (!use_given_rhs) d.rhs[k] = fi;
        const T ri = (T)fi;
        const T ui = dinv[k] * ri;
        x[k] = (T)0;
        r[k] = ri;
        u[k] = ui;
        p[k] = (T)0;
        sv[k] = (T)0;
        w[k] = (T)0;
        gam += (double)ri * (double)ui;
        ff += fi * fi;
    }
    const double in[2] = {gam, ff};
    double sums[2];
    block_sum<2, double>(in, sums, red);
    if (threadIdx.x == 0) {
        d.partials[4 * (size_t)tile] = sums[0];
        d.partials[4 * (size_t)tile + 1] = sums[1];
    }
    if (last_block(&d.counters[CNT_NODES], gridDim.x)) {
        __shared__ unsigned int running;
        if (threadIdx.x == 0) running = 0;
        __syncthreads();
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            const int t0 = d.bp[bb].tile_off, tc = d.bp[bb].tile_cnt;
            double s0 = 0.0, s1 = 0.0;
            for (int t = lane; t < tc; t += 32) {
                s0 += __ldcg(&d.partials[4 * (size_t)(t0 + t)]);
                s1 += __ldcg(&d.partials[4 * (size_t)(t0 + t) + 1]);
            }
            s0 = warp_sum<double>(s0);
            s1 = warp_sum<double>(s1);
            if (lane == 0) {
                CgScalars &cg = d.cg[bb];
                cg.gamma = s0;
                cg.ff = s1;
                cg.delta = cg.rr = cg.alpha = cg.beta = 0.0;
                cg.iters = 0;
                cg.restarts = 0;
                cg.true_relres2 = -1.0;
                const bool done = (d.status[bb] != 0) || s1 == 0.0;
                cg.state = done ? CG_CONVERGED : CG_ACTIVE;
                if (!done) atomicAdd(&running, 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            d.bar[0] = 0;          // arrival count
            d.bar[2] = running;    // blobs still iterating
            d.bar[3] = running;
            d.bar[4] = 0;          // barrier time-out flag
            d.counters[CNT_NODES] = 0;
        }
    }
}

// ---------------------------------------------------------------- persistent CG
constexpr unsigned int kSpinLimit = 1u << 24;  // ~1 s of 64 ns sleeps, then give up
constexpr int kMaxRestarts = 4;

// Grid-wide barrier of the persistent kernel (all CTAs co-resident by the
// cooperative launch).  The last CTA to arrive publishes the running-blob
// count, so every CTA leaves with the same value.  A wait that exceeds the
// spin limit raises the time-out flag instead of hanging.
__device__ __forceinline__ unsigned int grid_barrier(unsigned int *bar, int *s_err, unsigned int *s_pub)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vb = bar;
        const unsigned int gen = vb[1];
        __threadfence();
        const unsigned int arrived = atomicAdd(&bar[0], 1u);
        if (arrived == gridDim.x - 1) {
            vb[3] = vb[2];
            vb[0] = 0;
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            unsigned int spins = 0;
            while (vb[1] == gen) {
                if (++spins > kSpinLimit || vb[4]) {
                    *s_err = 1;
                    atomicExch(&bar[4], 1u);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        *s_pub = vb[3];
    }
    __syncthreads();
    return *s_pub;
}

// q = A v for one row: NoMass in difference form sum_q K_pq (v_q - v_p) + drag v_p,
// mass sum_q m_pq v_q + m_pp v_p.  v is read through L2 (written by other CTAs).
template <typename T>
__device__ __forceinline__ void sell_row(const DeviceBatch &d, int row, bool nomass, T diag, const T *v, T out[3])
{
    const int sl = row >> 5, lane = row & 31;
    const int L = __ldg(&d.slice_len[sl]);
    const int base = __ldg(&d.slice_ptr[sl]);
    const T v0 = __ldcg(&v[3 * (size_t)row]), v1 = __ldcg(&v[3 * (size_t)row + 1]), v2 = __ldcg(&v[3 * (size_t)row + 2]);
    T a0 = diag * v0, a1 = diag * v1, a2 = diag * v2;
    if (nomass) {
        const T *val = static_cast<const T *>(d.sell_val);
#pragma unroll 2
        for (int j = 0; j < L; j++) {
            const int off = base + 32 * j + lane;
            const int q = __ldg(&d.sell_col[off]);
            const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
            T K[9];
#pragma unroll
            for (int k = 0; k < 9; k++) K[k] = __ldg(&val[vb + 32 * k]);
            const T d0 = __ldcg(&v[3 * (size_t)q]) - v0, d1 = __ldcg(&v[3 * (size_t)q + 1]) - v1,
                    d2 = __ldcg(&v[3 * (size_t)q + 2]) - v2;
            a0 += K[0] * d0 + K[1] * d1 + K[2] * d2;
            a1 += K[3] * d0 + K[4] * d1 + K[5] * d2;
            a2 += K[6] * d0 + K[7] * d1 + K[8] * d2;
        }
    } else {
        const T *mv = static_cast<const T *>(d.sell_mval);
#pragma unroll 2
        for (int j = 0; j < L; j++) {
            const int off = base + 32 * j + lane;
            const int q = __ldg(&d.sell_col[off]);
            const T m = __ldg(&mv[off]);
            a0 += m * __ldcg(&v[3 * (size_t)q]);
            a1 += m * __ldcg(&v[3 * (size_t)q + 1]);
            a2 += m * __ldcg(&v[3 * (size_t)q + 2]);
        }
    }
    out[0] = a0;
    out[1] = a1;
    out[2] = a2;
}

// b - A x for one row with FP64 products and accumulation (x is T).
template <typename T>
__device__ __forceinline__ void true_residual_row(const DeviceBatch &d, int row, bool nomass, double diag, const T *x,
                                                  double out[3])
{
    const int sl = row >> 5, lane = row & 31;
    const int L = __ldg(&d.slice_len[sl]);
    const int base = __ldg(&d.slice_ptr[sl]);
    const double x0 = (double)__ldcg(&x[3 * (size_t)row]), x1 = (double)__ldcg(&x[3 * (size_t)row + 1]),
                 x2 = (double)__ldcg(&x[3 * (size_t)row + 2]);
    double a0 = diag * x0, a1 = diag * x1, a2 = diag * x2;
    for (int j = 0; j < L; j++) {
        const int off = base + 32 * j + lane;
        const int q = __ldg(&d.sell_col[off]);
        const double y0 = (double)__ldcg(&x[3 * (size_t)q]), y1 = (double)__ldcg(&x[3 * (size_t)q + 1]),
                     y2 = (double)__ldcg(&x[3 * (size_t)q + 2]);
        if (nomass) {
            const T *val = static_cast<const T *>(d.sell_val);
            const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
            double K[9];
#pragma unroll
            for (int k = 0; k < 9; k++) K[k] = (double)__ldg(&val[vb + 32 * k]);
            const double d0 = y0 - x0, d1 = y1 - x1, d2 = y2 - x2;
            a0 += K[0] * d0 + K[1] * d1 + K[2] * d2;
            a1 += K[3] * d0 + K[4] * d1 + K[5] * d2;
            a2 += K[6] * d0 + K[7] * d1 + K[8] * d2;
        } else {
            const double m = (double)__ldg(&static_cast<const T *>(d.sell_mval)[off]);
            a0 += m * y0;
            a1 += m * y1;
            a2 += m * y2;
        }
    }
    out[0] = d.rhs[3 * (size_t)row] - a0;
    out[1] = d.rhs[3 * (size_t)row + 1] - a1;
    out[2] = d.rhs[3 * (size_t)row + 2] - a2;
}

// The whole solve of every blob: Chronopoulos-Gear PCG (one pair of
// reductions per iteration), x0 = 0, stopping on sum r^2 / sum f^2 < eps^2
// like residual2() (src/NoMassCGSolver.cpp:233-247).  With true_residual on,
// a recursive convergence is confirmed by an FP64 b - A x; a failed check
// restarts CG from that residual.  CTA c owns node tiles
// [n_tiles*c/G, n_tiles*(c+1)/G); thread t owns row t of each of its tiles.
template <typename T>
__global__ void __launch_bounds__(CG_THREADS) k_cg(DeviceBatch d)
{
    using W = T;
    __shared__ double red[4 * 32];
    __shared__ int s_nt, s_nb, s_err;
    __shared__ unsigned int s_pub;
    __shared__ int s_tslot[CG_MAX_TILES];
    __shared__ int s_blob[CG_MAX_TILES], s_state[CG_MAX_TILES], s_iters[CG_MAX_TILES], s_restarts[CG_MAX_TILES];
    __shared__ int s_owner[CG_MAX_TILES], s_limit[CG_MAX_TILES], s_tr[CG_MAX_TILES], s_nomass[CG_MAX_TILES];
    __shared__ double s_alpha[CG_MAX_TILES], s_beta[CG_MAX_TILES], s_gamma[CG_MAX_TILES], s_ff[CG_MAX_TILES];
    __shared__ double s_gnew[CG_MAX_TILES], s_eps2[CG_MAX_TILES], s_trr[CG_MAX_TILES], s_rr[CG_MAX_TILES];
    __shared__ double s_sum[2][CG_MAX_TILES];

    const int G = gridDim.x, c = blockIdx.x, tid = threadIdx.x;
    const int T0 = (int)(((long long)d.n_tiles * c) / G), T1 = (int)(((long long)d.n_tiles * (c + 1)) / G);
    if (tid == 0) {
        s_err = 0;
        int nb = 0;
        for (int j = 0; j < T1 - T0; j++) {
            const int b = d.tile_blob[T0 + j];
            if (nb == 0 || s_blob[nb - 1] != b) {
                const CgScalars cg = d.cg[b];
                const BlobParams &bp = d.bp[b];
                s_blob[nb] = b;
                s_state[nb] = cg.state;
                s_gamma[nb] = cg.gamma;
                s_ff[nb] = cg.ff;
                s_alpha[nb] = s_beta[nb] = 0.0;
                s_iters[nb] = 0;
                s_restarts[nb] = 0;
                s_trr[nb] = -1.0;
                s_rr[nb] = 0.0;
                s_owner[nb] = bp.tile_off == T0 + j;
                s_limit[nb] = bp.solver == SOLVER_MASS ? bp.max_iter - 1 : bp.max_iter;
                s_tr[nb] = bp.true_residual;
                s_nomass[nb] = bp.solver == SOLVER_NOMASS;
                s_eps2[nb] = bp.epsilon2;
                nb++;
            }
            s_tslot[j] = nb - 1;
        }
        s_nt = T1 - T0;
        s_nb = nb;
    }
    __syncthreads();
    const int nt = s_nt, nb = s_nb;
    T *x = static_cast<T *>(d.x), *r = static_cast<T *>(d.r), *u = static_cast<T *>(d.u);
    T *w = static_cast<T *>(d.w), *p = static_cast<T *>(d.p), *sv = static_cast<T *>(d.s);
    const T *dinv = static_cast<const T *>(d.dinv);

    // per-blob fixed-order sums of two partial slots; one warp per distinct
    // blob, 8 loads per lane in flight per pass (the partials live in L2)
    auto reduce2 = [&](int slot0) {
        const int lane = tid & 31, warp = tid >> 5;
        for (int k = warp; k < nb; k += CG_THREADS / 32) {
            const int b = s_blob[k];
            const int t0 = d.bp[b].tile_off, tc = d.bp[b].tile_cnt;
            double a0 = 0.0, a1 = 0.0;
            for (int base = 0; base < tc; base += 8 * 32) {
                double v0[8], v1[8];
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int t = base + 32 * q + lane;
                    const double2 pv = t < tc ? __ldcg(reinterpret_cast<const double2 *>(
                                                    &d.partials[4 * (size_t)(t0 + t) + slot0]))
                                              : make_double2(0.0, 0.0);
                    v0[q] = pv.x;
                    v1[q] = pv.y;
                }
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    a0 += v0[q];
                    a1 += v1[q];
                }
            }
            a0 = warp_sum<double>(a0);
            a1 = warp_sum<double>(a1);
            if (lane == 0) {
                s_sum[0][k] = a0;
                s_sum[1][k] = a1;
            }
        }
        __syncthreads();
    };
    auto finish_blob = [&](int k, int state, int bits) {
        s_state[k] = state;
        if (s_owner[k]) {
            atomicSub(&d.bar[2], 1u);
            if (bits) atomicOr(&d.status[s_blob[k]], bits);
        }
    };
    // SpMV phase for ACTIVE / RESTART blobs: w = A u, partial delta = w . u  -> slot 2;
    // VERIFY blobs: r = b - A x (FP64), u = D^-1 r, partials r.r -> slot 2, r.u -> slot 3
    auto spmv_phase = [&]() {
        for (int j = 0; j < nt; j++) {
            const int t = T0 + j, k = s_tslot[j], st = s_state[k];
            const int row = t * NODE_TILE + tid;
            const BlobParams &bp = d.bp[s_blob[k]];
            const bool valid = (row - bp.node_off) < bp.node_cnt && !(d.flags[row] & NODE_PINNED);
            W wd = 0, wg = 0;
            double vd = 0.0, vg = 0.0;
            if ((st == CG_ACTIVE || st == CG_RESTART) && valid) {
                const T diag = s_nomass[k] ? (T)(bp.calc_stokes == 1 ? d.drag[row] : 0.0)
                                           : static_cast<const T *>(d.mass_diag)[row];
                T q[3];
                sell_row<T>(d, row, s_nomass[k], diag, u, q);
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    w[3 * (size_t)row + i] = q[i];
                    wd += q[i] * __ldcg(&u[3 * (size_t)row + i]);
                }
            } else if (st == CG_VERIFY && valid) {
                const double diag = s_nomass[k] ? (bp.calc_stokes == 1 ? d.drag[row] : 0.0)
                                                : (double)static_cast<const T *>(d.mass_diag)[row];
                double rt[3];
                true_residual_row<T>(d, row, s_nomass[k], diag, x, rt);
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const size_t kk = 3 * (size_t)row + i;
                    const T ri = (T)rt[i];
                    const T ui = dinv[kk] * ri;
                    r[kk] = ri;
                    u[kk] = ui;
                    vd += rt[i] * rt[i];
                    vg += (double)ri * (double)ui;
                }
            }
            double out[2];
            if (st == CG_VERIFY) {
                const double in[2] = {vd, vg};
                block_sum<2, double>(in, out, red);
            } else {
                const W in[2] = {wd, wg};
                block_sum<2, W>(in, out, red);
            }
            if (tid == 0) {
                d.partials[4 * (size_t)t + 2] = out[0];
                d.partials[4 * (size_t)t + 3] = out[1];
            }
        }
    };

    // prologue: w0 = A u0, delta0, alpha0 = gamma0 / delta0
    spmv_phase();
    unsigned int running = grid_barrier(d.bar, &s_err, &s_pub);
    long long loops = 0;
    if (!s_err) {
        reduce2(2);
        if (tid == 0)
            for (int k = 0; k < nb; k++)
                if (s_state[k] == CG_ACTIVE) {
                    s_alpha[k] = s_gamma[k] / s_sum[0][k];
                    s_beta[k] = 0.0;
                }
        __syncthreads();
    }
    while (!s_err && running > 0) {
        // phase A: p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = D^-1 r
        for (int j = 0; j < nt; j++) {
            const int t = T0 + j, k = s_tslot[j];
            const int row = t * NODE_TILE + tid;
            W gam = 0, rr = 0;
            if (s_state[k] == CG_ACTIVE) {
                const T alpha = (T)s_alpha[k], beta = (T)s_beta[k];
                const bool first = s_beta[k] == 0.0;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const size_t kk = 3 * (size_t)row + i;
                    const T ui = u[kk], wi = w[kk];
                    const T pi = first ? ui : ui + beta * p[kk];
                    const T si = first ? wi : wi + beta * sv[kk];
                    p[kk] = pi;
                    sv[kk] = si;
                    x[kk] += alpha * pi;
                    const T ri = r[kk] - alpha * si;
                    r[kk] = ri;
                    const T un = dinv[kk] * ri;
                    u[kk] = un;
                    gam += ri * un;
                    rr += ri * ri;
                }
            }
            const W in[2] = {gam, rr};
            double out[2];
            block_sum<2, W>(in, out, red);
            if (tid == 0) {
                d.partials[4 * (size_t)t] = out[0];
                d.partials[4 * (size_t)t + 1] = out[1];
            }
        }
        loops++;
        running = grid_barrier(d.bar, &s_err, &s_pub);
        if (s_err || running == 0) break;
        reduce2(0);
        if (tid == 0) {
            for (int k = 0; k < nb; k++) {
                if (s_state[k] != CG_ACTIVE) continue;
                s_iters[k] += 1;
                const double rr = s_sum[1][k];
                s_rr[k] = rr;
                s_gnew[k] = s_sum[0][k];
                const double res = (s_ff[k] == 0.0) ? 0.0 : rr / s_ff[k];
                if (res < s_eps2[k]) {
                    if (s_tr[k]) s_state[k] = CG_VERIFY;
                    else finish_blob(k, CG_CONVERGED, 0);
                } else if (!(res == res)) {
                    finish_blob(k, CG_FAILED, BLOB_FAIL_CG | BLOB_FAIL_NAN);
                } else if (s_iters[k] >= s_limit[k]) {
                    finish_blob(k, CG_FAILED, BLOB_FAIL_CG);
                }
            }
        }
        __syncthreads();
        // phase B: w = A u (or the FP64 true residual for blobs being verified)
        spmv_phase();
        running = grid_barrier(d.bar, &s_err, &s_pub);
        if (s_err) break;
        reduce2(2);
        if (tid == 0) {
            for (int k = 0; k < nb; k++) {
                const int st = s_state[k];
                if (st == CG_ACTIVE) {
                    const double gnew = s_gnew[k], delta = s_sum[0][k];
                    const double beta = gnew / s_gamma[k];
                    s_alpha[k] = gnew / (delta - beta * gnew / s_alpha[k]);
                    s_beta[k] = beta;
                    s_gamma[k] = gnew;
                } else if (st == CG_RESTART) {
                    s_alpha[k] = s_gamma[k] / s_sum[0][k];
                    s_beta[k] = 0.0;
                    s_state[k] = CG_ACTIVE;
                } else if (st == CG_VERIFY) {
                    const double trr = s_sum[0][k];
                    s_trr[k] = (s_ff[k] == 0.0) ? 0.0 : trr / s_ff[k];
                    if (s_trr[k] < s_eps2[k]) {
                        finish_blob(k, CG_CONVERGED, 0);
                    } else if (s_restarts[k] >= kMaxRestarts || s_iters[k] >= s_limit[k]) {
                        finish_blob(k, CG_FAILED, BLOB_FAIL_CG);
                    } else {
                        s_restarts[k] += 1;
                        s_gamma[k] = s_sum[1][k];
                        s_state[k] = CG_RESTART;
                    }
                }
            }
        }
        __syncthreads();
        if (running == 0) break;
    }
    if (tid == 0) {
        if (s_err) {
            for (int k = 0; k < nb; k++) atomicOr(&d.status[s_blob[k]], BLOB_FAIL_CG | BLOB_FAIL_TIMEOUT);
        }
        for (int k = 0; k < nb; k++) {
            if (!s_owner[k]) continue;
            CgScalars &cg = d.cg[s_blob[k]];
            cg.state = s_state[k];
            cg.iters = s_iters[k];
            cg.restarts = s_restarts[k];
            cg.alpha = s_alpha[k];
            cg.beta = s_beta[k];
            cg.gamma = s_gamma[k];
            cg.rr = s_rr[k];
            cg.true_relres2 = s_trr[k];
        }
        if (c == 0) *d.loop_count += (unsigned long long)loops;
    }
}

// Euler update (src/Blob.cpp:3937-3969) and the RNG advance to the next step.
template <typename T>
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
    const T *x = static_cast<const T *>(d.x);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const size_t k = 3 * (size_t)row + i;
        const double xi = (double)x[k];
        if (bp.solver == SOLVER_NOMASS) {
            d.vel[k] = xi;
            d.pos[k] += xi * dt;
        } else {
            const double v = d.vel[k] + xi * dt;
            d.vel[k] = v;
            d.pos[k] += v * dt;
        }
    }
}

// out = A in (FP64 vectors and arithmetic); pinned rows and padding give 0.
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
        const bool nomass = bp.solver == SOLVER_NOMASS;
        const double diag = nomass ? (bp.calc_stokes == 1 ? d.drag[row] : 0.0)
                                   : (double)static_cast<const T *>(d.mass_diag)[row];
        const int sl = row >> 5, lane = row & 31;
        const int L = d.slice_len[sl], base = d.slice_ptr[sl];
        const double v0 = in[3 * (size_t)row], v1 = in[3 * (size_t)row + 1], v2 = in[3 * (size_t)row + 2];
        acc[0] = diag * v0;
        acc[1] = diag * v1;
        acc[2] = diag * v2;
        for (int j = 0; j < L; j++) {
            const int off = base + 32 * j + lane;
            const int q = d.sell_col[off];
            const double y0 = in[3 * (size_t)q], y1 = in[3 * (size_t)q + 1], y2 = in[3 * (size_t)q + 2];
            if (nomass) {
                const T *val = static_cast<const T *>(d.sell_val);
                double K[9];
                for (int k = 0; k < 9; k++) K[k] = (double)val[sell_vidx(off, k)];
                const double d0 = y0 - v0, d1 = y1 - v1, d2 = y2 - v2;
                acc[0] += K[0] * d0 + K[1] * d1 + K[2] * d2;
                acc[1] += K[3] * d0 + K[4] * d1 + K[5] * d2;
                acc[2] += K[6] * d0 + K[7] * d1 + K[8] * d2;
            } else {
                const double m = (double)static_cast<const T *>(d.sell_mval)[off];
                acc[0] += m * y0;
                acc[1] += m * y1;
                acc[2] += m * y2;
            }
        }
    }
    for (int i = 0; i < 3; i++) out[3 * (size_t)row + i] = acc[i];
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
    const double ein[2] = {se, ke};
    double v[2];
    block_sum<2, double>(ein, v, red);
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
            s0 = warp_sum<double>(s0);
            s1 = warp_sum<double>(s1);
            if (lane == 0) {
                d.energy[2 * bb] = 0.5 * s0;
                d.energy[2 * bb + 1] = 0.5 * s1;
            }
        }
        if (threadIdx.x == 0) d.counters[CNT_ENERGY] = 0;
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

void launch_nodes(const DeviceBatch &d, cudaStream_t s, int use_given_rhs)
{
    PREC_DISPATCH(d, k_nodes, d.n_tiles, NODE_TILE, s, d, use_given_rhs);
}

int cg_max_grid(int precision)
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    cudaError_t e = precision == PREC_FP64
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<double>, CG_THREADS, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<float>, CG_THREADS, 0);
    if (e != cudaSuccess) return 0;
    return sms * per_sm;
}

cudaError_t launch_cg(const DeviceBatch &d, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)d.cg_grid);
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FFEA_LAUNCHED();
    if (d.precision == PREC_FP64) return cudaLaunchKernelEx(&cfg, k_cg<double>, d);
    return cudaLaunchKernelEx(&cfg, k_cg<float>, d);
}

void launch_euler(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_euler, d.n_tiles, NODE_TILE, s, d);
}

void launch_energies(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_energies, d.n_etiles, ELEM_TILE, s, d);
}

void launch_apply(const DeviceBatch &d, cudaStream_t s, const double *in, double *out)
{
    PREC_DISPATCH(d, k_apply, d.n_tiles, NODE_TILE, s, d, in, out);
}

void launch_rng_draws(const mrg::JumpMat *table, const uint32_t *state, uint64_t offset, int64_t count, double *out,
                      cudaStream_t s)
{
    if (count <= 0) return;
    k_rng_draws<<<blocks_for(count, 256), 256, 0, s>>>(table, state, offset, count, out);
    FFEA_LAUNCHED();
}

}  // namespace ffea
