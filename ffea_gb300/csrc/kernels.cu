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
//                launch (NoMassCGSolver.cpp:165-197, ConjugateGradientSolver.cpp:206-232),
//                ending with the velocity / position update and the RNG
//                stream advance (Blob.cpp:3937-3969)
// Reductions are deterministic: fixed butterflies inside warps and CTAs, one
// partial per node tile, and fixed-order per-blob sums.  No floating-point
// atomics are used anywhere.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>

#include "kernels.h"

#include <algorithm>
#include <type_traits>

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

// Edge vectors of the element from the double-float copy of the positions
// (mixed precision): (hi_n - hi_0) + (lo_n - lo_0), within an FP32 rounding
// of the FP64 difference, with no FP64 instruction.  FP64 mode reads the
// FP64 positions.
template <typename T>
__device__ __forceinline__ void jacobian_t(const DeviceBatch &d, int4 c, T J[3][3])
{
    if constexpr (sizeof(T) == sizeof(double)) {
        jacobian<T>(d.pos, c, J);
    } else {
        const float2 *p = d.pos_df;
        const float2 a[3] = {p[3 * (size_t)c.x], p[3 * (size_t)c.x + 1], p[3 * (size_t)c.x + 2]};
        const int n[3] = {c.y, c.z, c.w};
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float2 q = p[3 * (size_t)n[r] + k];
                J[r][k] = (q.x - a[k].x) + (q.y - a[k].y);
            }
    }
}

// Double-float accumulation (Knuth's TwoSum, error-free in FP32): sums with
// ~48-bit precision on the FP32 pipes, which on GB300 run many times faster
// than FP64.
struct DF {
    float hi, lo;
};

__device__ __forceinline__ DF df_add(DF a, DF b)
{
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b.hi - bb);
    err += a.lo + b.lo;
    const float hi = s + err;
    return DF{hi, err - (hi - s)};
}

// Force sum of the node kernel: FP64 in FP64 mode; in mixed precision a
// double-float sum of the FP32 element forces, which keeps the FP64 pipes
// (1/64 of the FP32 rate on GB300) out of the per-corner loop.
// merge(o) adds another partial sum; xor_shfl(m) is lane ^ m's partial.
template <typename T> struct ForceSum {
    double v = 0.0;
    __device__ __forceinline__ void add(T x) { v += (double)x; }
    __device__ __forceinline__ void add_d(double x) { v += x; }
    __device__ __forceinline__ void merge(const ForceSum &o) { v += o.v; }
    __device__ __forceinline__ ForceSum xor_shfl(int m) const
    {
        ForceSum r;
        r.v = __shfl_xor_sync(0xffffffffu, v, m);
        return r;
    }
    __device__ __forceinline__ double value() const { return v; }
};
template <> struct ForceSum<float> {
    DF v{0.f, 0.f};
    __device__ __forceinline__ void add(float x) { v = df_add(v, DF{x, 0.f}); }
    __device__ __forceinline__ void add_d(double x)
    {
        const float h = (float)x;
        v = df_add(v, DF{h, (float)(x - (double)h)});
    }
    __device__ __forceinline__ void merge(const ForceSum &o) { v = df_add(v, o.v); }
    __device__ __forceinline__ ForceSum xor_shfl(int m) const
    {
        ForceSum r;
        r.v = DF{__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
        return r;
    }
    __device__ __forceinline__ double value() const { return (double)v.hi + (double)v.lo; }
};

// The scaled gradients g_a = sqrt(V) dpsi_a of one element, all four corners
// (12 values, corner 0 = -(g_1 + g_2 + g_3) formed when they are written),
// read as three 16-byte vectors: the assembly reads each element's gradients
// once per edge, and one vector load replaces four scalar ones.
template <typename T>
__device__ __forceinline__ void load_g4(const T *g, int el, T out[12]);
template <>
__device__ __forceinline__ void load_g4<float>(const float *g, int el, float out[12])
{
    const float4 *ge = reinterpret_cast<const float4 *>(g + 12 * (size_t)el);
#pragma unroll
    for (int v = 0; v < 3; v++) {
        const float4 q = __ldg(ge + v);
        out[4 * v] = q.x;
        out[4 * v + 1] = q.y;
        out[4 * v + 2] = q.z;
        out[4 * v + 3] = q.w;
    }
}
template <>
__device__ __forceinline__ void load_g4<double>(const double *g, int el, double out[12])
{
    const double2 *ge = reinterpret_cast<const double2 *>(g + 12 * (size_t)el);
#pragma unroll
    for (int v = 0; v < 6; v++) {
        const double2 q = __ldg(ge + v);
        out[2 * v] = q.x;
        out[2 * v + 1] = q.y;
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

// The step's random draws, ahead of the element and node kernels.  Each
// thread draws NOISE_RUN consecutive values from the start of its run, so
// the stream position is found once per 32 draws rather than once per
// element or node.  A run sits at the same offset in the stream every step,
// so its start state for the next step is this one advanced by the stream's
// draws per step (one product with A^(draws per step), the advance the step
// itself ends with); that state is kept, and only a run whose stream was set
// from outside since (a new generation) jumps from the stream state
// (mrg::jump, four table products).  Every secondary node's
// draws, which two linear nodes fold in, are made once.  The values are the
// same centred draws the consumers took from their own jumps: element e of a
// blob uses draws elem_draw_base + 7 le .. +6 (src/tetra_element_linear.cpp:417-436),
// node n uses node_draw_base + 3 n .. +2 in original numbering (src/Blob.cpp:3867-3899).
// One centred draw: FP64 as the reference computes it (FP64 mode); in mixed
// precision the FP32 value from the same integer state (mrg::centred_f),
// within 2 ulp of rounding the FP64 value, with no FP64 instruction.
template <typename T> __device__ __forceinline__ T draw(uint32_t *st);
template <> __device__ __forceinline__ double draw<double>(uint32_t *st) { return mrg::centred(st); }
template <> __device__ __forceinline__ float draw<float>(uint32_t *st) { return mrg::centred_f(st); }

template <typename T>
__global__ void __launch_bounds__(NOISE_THREADS) k_noise(DeviceBatch d)
{
    // each warp stages its 32 runs in shared memory (row per run, padded to
    // 33 so that both the per-run writes and the per-draw reads are
    // conflict-free for FP32), then stores run by run, one coalesced line
    // per run, instead of 32 scattered words per store instruction
    static_assert(NOISE_RUN == 32 && NOISE_THREADS % 32 == 0, "one lane per draw of a run");
    __shared__ T stage[NOISE_THREADS / 32][32][NOISE_RUN + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int run = blockIdx.x * blockDim.x + threadIdx.x;
    int cnt = 0;
    T *dst = nullptr;
    if (run < d.noise_runs) {
        // the (blob, kind) pair holding this run: the last prefix entry <= run
        int lo = 0, hi = 2 * d.num_blobs;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (d.noise_run_off[mid] <= run) lo = mid;
            else hi = mid;
        }
        const int b = lo >> 1, kind = lo & 1;
        if (d.status[b] == 0) {  // a failed blob takes no further step
            const BlobParams &bp = d.bp[b];
            const uint32_t first = (uint32_t)(run - d.noise_run_off[lo]) * NOISE_RUN;
            const uint32_t total = kind == 0 ? 7u * (uint32_t)bp.elem_cnt : 3u * (uint32_t)bp.num_nodes_total;
            cnt = (int)min((uint32_t)NOISE_RUN, total - first);
            dst = kind == 0 ? static_cast<T *>(d.elem_noise) + 7 * (size_t)bp.elem_off + first
                            : static_cast<T *>(d.node_noise) + 3 * (size_t)bp.noise_node_off + first;
            const int sm = bp.stream;
            const uint32_t gen = d.stream_gen[sm];
            const size_t R = (size_t)d.noise_runs;
            uint32_t st[6];
            if (d.noise_run_gen[run] == gen) {
#pragma unroll
                for (int i = 0; i < 6; i++) st[i] = d.noise_run_state[i * R + run];
            } else {
#pragma unroll
                for (int i = 0; i < 6; i++) st[i] = d.stream_state[6 * sm + i];
                mrg::jump(d.jump_table, (kind == 0 ? bp.elem_draw_base : bp.node_draw_base) + first, st);
            }
            // the run's start in the next step (a blob whose step fails takes
            // no further step, so its kept states are never read)
            uint32_t nx[6];
#pragma unroll
            for (int i = 0; i < 6; i++) nx[i] = st[i];
            mrg::apply(d.stream_step[sm], nx);
#pragma unroll
            for (int i = 0; i < 6; i++) d.noise_run_state[i * R + run] = nx[i];
            d.noise_run_gen[run] = gen;
            if (cnt == NOISE_RUN) {
                // a whole run, unrolled: the state words rotate by renaming
#pragma unroll
                for (int i = 0; i < NOISE_RUN; i++) stage[warp][lane][i] = draw<T>(st);
            } else {
                for (int i = 0; i < cnt; i++) stage[warp][lane][i] = draw<T>(st);
            }
        }
    }
    __syncwarp();
    for (int i = 0; i < 32; i++) {
        const int c = __shfl_sync(0xffffffffu, cnt, i);
        T *o = reinterpret_cast<T *>(__shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(dst), i));
        if (lane < c) o[lane] = stage[warp][i][lane];
    }
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
    // every node pinned: no element step and no element draws (src/Blob.cpp:643-645)
    if (mode == ELEM_STEP && bp.all_pinned) return;
    const int e = bp.elem_off + le;
    const int4 c = reinterpret_cast<const int4 *>(d.conn)[e];
    T J[3][3];
    jacobian_t<T>(d, c, J);
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
    const T *m = static_cast<const T *>(d.mat_t) + MAT_T_STRIDE * (size_t)d.mat_id[e];
    const T A = m[MAT_T_A], B = m[MAT_T_B], G = m[MAT_T_G], Eb = m[MAT_T_E];
    const T vol = geo.vol;
    const T *dpsi = geo.dpsi;

    if (bp.solver == SOLVER_NOMASS) {
        // scaled gradients for the assembly: g_a = sqrt(vol) dpsi_a of
        // corners 1..3, and corner 0 as minus their sum (the gradients of a
        // linear element's shape functions sum to zero)
        const T sv = sqrt(vol);
        T gv[12];
#pragma unroll
        for (int a = 1; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++) gv[3 * a + i] = sv * dpsi[4 * i + a];
#pragma unroll
        for (int i = 0; i < 3; i++) gv[i] = -(gv[3 + i] + gv[6 + i] + gv[9 + i]);
        T *gout = static_cast<T *>(d.g) + 12 * (size_t)e;
        if (sizeof(T) == 4) {
            float4 *o = reinterpret_cast<float4 *>(gout);
#pragma unroll
            for (int v = 0; v < 3; v++)
                o[v] = make_float4((float)gv[4 * v], (float)gv[4 * v + 1], (float)gv[4 * v + 2], (float)gv[4 * v + 3]);
        } else {
            double2 *o = reinterpret_cast<double2 *>(gout);
#pragma unroll
            for (int v = 0; v < 6; v++) o[v] = make_double2((double)gv[2 * v], (double)gv[2 * v + 1]);
        }
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
        const T *nz = static_cast<const T *>(d.elem_noise) + 7 * (size_t)e;  // k_noise
        T u[7];
#pragma unroll
        for (int k = 0; k < 7; k++) u[k] = nz[k];
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
    if (bp.solver != SOLVER_NOMASS) {
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
    // nodal forces: node_force[a] = -vol * S dpsi_a (src/tetra_element_linear.cpp:441-489),
    // one 4-vector per corner (x, y, z, 0) so that the node gather reads a
    // corner with one vector load
    T *fo = static_cast<T *>(d.efrc) + 16 * (size_t)e;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        T f[3];
#pragma unroll
        for (int i = 0; i < 3; i++) f[i] = -(vol * (dpsi[a] * S[i][0] + dpsi[4 + a] * S[i][1] + dpsi[8 + a] * S[i][2]));
        if (sizeof(T) == 4) {
            reinterpret_cast<float4 *>(fo)[a] = make_float4((float)f[0], (float)f[1], (float)f[2], 0.f);
        } else {
            reinterpret_cast<double2 *>(fo)[2 * a] = make_double2((double)f[0], (double)f[1]);
            reinterpret_cast<double2 *>(fo)[2 * a + 1] = make_double2((double)f[2], 0.0);
        }
    }
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
        T ge[12];
        load_g4<T>(g, el, ge);
        T ga[3], gb[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            // select corner a and b of the four (unrolled: no local memory)
            ga[i] = a == 0 ? ge[i] : a == 1 ? ge[3 + i] : a == 2 ? ge[6 + i] : ge[9 + i];
            gb[i] = bb == 0 ? ge[i] : bb == 1 ? ge[3 + i] : bb == 2 ? ge[6 + i] : ge[9 + i];
        }
        const T *m = static_cast<const T *>(d.mat_t) + MAT_T_STRIDE * (size_t)d.mat_id[el];
        const T A = m[MAT_T_A], B = m[MAT_T_B];
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

// Lumped masses (MassLumpedSolver::init, src/MassLumpedSolver.cpp:40-78):
// per corner row a quarter of rho vol_0 of every element holding it, summed
// in element order (the gather list's order), inverted; 1 on pinned rows.
template <typename T>
__global__ void k_lumped_mass(DeviceBatch d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nl_pad) return;
    const BlobParams &bp = d.bp[d.tile_blob[i / NODE_TILE]];
    if (bp.solver != SOLVER_LUMPED) return;
    double s = 0.0;
    for (int k = d.gather_ptr[i]; k < d.gather_ptr[i + 1]; k++) {
        const int el = d.gather_idx[k] >> 2;
        s += .25 * d.mats[d.mat_id[el]].rho * (double)static_cast<const T *>(d.vol0)[el];
    }
    if ((d.flags[i] & NODE_PINNED) || s == 0.0) s = 1.0;
    d.lumped_inv[i] = 1.0 / s;
}

// Node kernel: rhs and the CG start (for a lumped-mass blob the solve
// itself, x = M_lumped^-1 f, MassLumpedSolver::solve src/MassLumpedSolver.cpp:81-89).
template <typename T>
__global__ void __launch_bounds__(NODE_TILE * NODE_LANES) k_nodes(DeviceBatch d, int use_given_rhs)
{
    // NODE_LANES lanes per row: the lanes split the row's gather list
    // (entries q, q + NODE_LANES, ...), combine their partial sums in a fixed
    // order, then lanes 0..2 each finish one component.
    static_assert(NODE_LANES == 4, "the combine below is a two-step butterfly");
    __shared__ double red[2 * 32];
    const int tile = blockIdx.x;
    const int b = d.tile_blob[tile];
    const BlobParams &bp = d.bp[b];
    const int q = threadIdx.x & (NODE_LANES - 1);
    const int row = tile * NODE_TILE + threadIdx.x / NODE_LANES;
    const int local = row - bp.node_off;
    const bool failed = d.status[b] != 0;
    const bool valid = local < bp.node_cnt && !(d.flags[row] & NODE_PINNED) && !failed;
    const bool nomass = bp.solver == SOLVER_NOMASS;
    const double drag = bp.calc_stokes == 1 ? d.drag[row] : 0.0;
    ForceSum<T> fs[3];
    if (valid && !use_given_rhs) {
        // external forces first, as FFEA adds them to Blob::force before the
        // element contributions (src/World.cpp:1907, src/Blob.cpp:647)
        if (d.ext && q == 0) {
#pragma unroll
            for (int i = 0; i < 3; i++) fs[i].add_d(d.ext[3 * (size_t)row + i]);
        }
        const T *ef = static_cast<const T *>(d.efrc);
#pragma unroll 2
        for (int k = d.gather_ptr[row] + q; k < d.gather_ptr[row + 1]; k += NODE_LANES) {
            const int gi = d.gather_idx[k];  // (element << 2) | corner: the corner's 4-vector
            T f[3];
            if (sizeof(T) == 4) {
                const float4 v = __ldg(reinterpret_cast<const float4 *>(ef) + gi);
                f[0] = (T)v.x;
                f[1] = (T)v.y;
                f[2] = (T)v.z;
            } else {
                const double2 v0 = __ldg(reinterpret_cast<const double2 *>(ef) + 2 * (size_t)gi);
                const double2 v1 = __ldg(reinterpret_cast<const double2 *>(ef) + 2 * (size_t)gi + 1);
                f[0] = (T)v0.x;
                f[1] = (T)v0.y;
                f[2] = (T)v1.x;
            }
#pragma unroll
            for (int i = 0; i < 3; i++) fs[i].add(f[i]);
        }
    }
    // (lane 0 + lane 1) + (lane 2 + lane 3), the lower lane's partial first,
    // so every lane of the row ends with the same sum
#pragma unroll
    for (int m = 1; m < NODE_LANES; m <<= 1) {
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const ForceSum<T> o = fs[i].xor_shfl(m);
            if (q & m) {
                ForceSum<T> lo = o;
                lo.merge(fs[i]);
                fs[i] = lo;
            } else {
                fs[i].merge(o);
            }
        }
    }
    const int c = q < 3 ? q : 0;  // this lane's component (lane 3 repeats 0 and stores nothing)
    ForceSum<T> fc = c == 0 ? fs[0] : (c == 1 ? fs[1] : fs[2]);
    if (valid && !use_given_rhs) {
        if (!nomass && bp.calc_stokes == 1) fc.add_d(-(d.vel[3 * (size_t)row + c] * drag));
        if (bp.calc_noise == 1 && bp.calc_stokes == 1) {
            // draws from k_noise, amplitudes sqrt((24 kT drag) / dt) set up once
            const T *nz = static_cast<const T *>(d.node_noise) + 3 * (size_t)bp.noise_node_off;
            const T *na = static_cast<const T *>(d.node_amp), *fa = static_cast<const T *>(d.fold_amp);
            if (drag != 0.0) fc.add(-(nz[3 * (size_t)d.orig[row] + c] * na[row]));
            // secondary nodes with a drag: half of their force lands here
            for (int k = d.fold_ptr[row]; k < d.fold_ptr[row + 1]; k++)
                fc.add((T)0.5 * (-(nz[3 * (size_t)d.fold_sec[k] + c] * fa[k])));
        }
    }
    double f = fc.value();
    if (use_given_rhs && valid) f = d.rhs[3 * (size_t)row + c];
    const bool store = q < 3;
    T *dinv = static_cast<T *>(d.dinv);
    if (nomass && store) {
        // Jacobi diagonal of component c: zeta_p - sum_q K_pq[c][c] over the
        // row's assembled blocks (padding slots hold zeros).  The viscosity
        // diagonal block is minus the sum of the row's off-diagonal blocks,
        // as the gradients of a linear element's shape functions sum to zero.
        T Dc = (T)0;
        if (valid) {
            const int sl = row >> 5, L = d.slice_len[sl], base = d.slice_ptr[sl] + (row & 31);
            const T *val = static_cast<const T *>(d.sell_val);
            for (int j = 0; j < L; j++) Dc -= val[sell_vidx(base + 32 * j, 4 * c)];
        }
        dinv[3 * (size_t)row + c] = valid ? (T)1 / (Dc + (T)drag) : (T)1;
    }
    // CG start: x = 0, r = f, u = D^-1 r, w = s = p = 0
    T *x = static_cast<T *>(d.x), *r = static_cast<T *>(d.r), *u = static_cast<T *>(d.u);
    T *p = static_cast<T *>(d.p), *sv = static_cast<T *>(d.s), *w = static_cast<T *>(d.w);
    double gam = 0.0, ff = 0.0;
    const bool lumped = bp.solver == SOLVER_LUMPED;
    if (store) {
        const size_t k = 3 * (size_t)row + c;
        const double fi = valid ? f : 0.0;
        if (!use_given_rhs) d.rhs[k] = fi;
        const T ri = (T)fi;
        const T ui = dinv[k] * ri;
        x[k] = lumped ? (T)(fi * d.lumped_inv[row]) : (T)0;
        r[k] = ri;
        u[k] = ui;
        p[k] = (T)0;
        sv[k] = (T)0;
        w[k] = (T)0;
        gam = (double)ri * (double)ui;
        ff = fi * fi;
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
                cg.gamma_f = (float)s0;
                cg.pap_f = cg.alpha_f = cg.beta_f = 0.f;
                cg.stop_f = (float)(d.bp[bb].epsilon2 * s1);
                cg.floor_f = (float)(1e-10 * s1);
                cg.iters = 0;
                cg.restarts = 0;
                cg.true_relres2 = -1.0;
                // a lumped-mass blob has its solution already (no CG)
                const bool done = (d.status[bb] != 0) || s1 == 0.0 || d.bp[bb].solver == SOLVER_LUMPED;
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
            d.bar[5] = 0;          // arrivals at counting barriers (monotonic within a solve)
            d.counters[CNT_NODES] = 0;
        }
    }
}

// ---------------------------------------------------------------- persistent CG
constexpr unsigned int kSpinLimit = 1u << 24;  // ~1 s of 64 ns sleeps, then give up
constexpr int kMaxRestarts = 4;

// Grid-wide barrier on a counter that only grows during a solve: each CTA
// adds one and waits until the count reaches `target` (the number of CTAs
// times the barriers passed so far, including this one).  The waiters see the
// last arrival directly, one L2 round trip sooner than with a separate
// release word.  The CTAs are co-resident (cooperative launch); a wait that
// exceeds the spin limit raises the time-out flag instead of hanging.
__device__ __forceinline__ void counting_barrier(unsigned int *bar, unsigned int target, int *s_err,
                                                 unsigned int spin_limit = kSpinLimit)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        // release: the CTA's writes (ordered before this thread by the CTA
        // barrier) are visible to every CTA that acquires the count after it
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&bar[5]), "r"(1u));
        unsigned int spins = 0;
        for (;;) {
            unsigned int n;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(n) : "l"(&bar[5]));
            if ((int)(n - target) >= 0) break;
            // the time-out flag only every 16th poll: a poll is then one L2
            // round trip, not two, and the last arrival is seen sooner
            if ((++spins & 15) == 0 && (spins > spin_limit || ((volatile unsigned int *)bar)[4])) {
                *s_err = 1;
                atomicExch(&bar[4], 1u);
                break;
            }
            __nanosleep(32);
        }
    }
    __syncthreads();
}

// q = A v for one row: NoMass in difference form sum_q K_pq (v_q - v_p) + drag v_p,
// mass sum_q m_pq v_q + m_pp v_p.  v is read through L2 (written by other CTAs).
// Slots are processed in groups of 4: the column indices of a group are
// loaded together, then the 12 neighbour components, so a group costs about
// two L2 round trips instead of one or two per slot.
template <typename T>
__device__ __forceinline__ void sell_row(const DeviceBatch &d, int row, bool nomass, T diag, const T *v, T out[3])
{
    const int sl = row >> 5, lane = row & 31;
    const int L = __ldg(&d.slice_len[sl]);
    const int base = __ldg(&d.slice_ptr[sl]);
    const T v0 = __ldcg(&v[3 * (size_t)row]), v1 = __ldcg(&v[3 * (size_t)row + 1]), v2 = __ldcg(&v[3 * (size_t)row + 2]);
    T a0 = diag * v0, a1 = diag * v1, a2 = diag * v2;
    const T *val = static_cast<const T *>(d.sell_val);
    const T *mv = static_cast<const T *>(d.sell_mval);
    constexpr int GRP = 4;
    for (int j0 = 0; j0 < L; j0 += GRP) {
        int q[GRP];
#pragma unroll
        for (int g = 0; g < GRP; g++) q[g] = (j0 + g < L) ? __ldg(&d.sell_col[base + 32 * (j0 + g) + lane]) : row;
        T y[GRP][3];
#pragma unroll
        for (int g = 0; g < GRP; g++) {
            y[g][0] = __ldcg(&v[3 * (size_t)q[g]]);
            y[g][1] = __ldcg(&v[3 * (size_t)q[g] + 1]);
            y[g][2] = __ldcg(&v[3 * (size_t)q[g] + 2]);
        }
#pragma unroll
        for (int g = 0; g < GRP; g++) {
            if (j0 + g >= L) break;
            const int off = base + 32 * (j0 + g) + lane;
            if (nomass) {
                const size_t vb = (size_t)(base + 32 * (j0 + g)) * 9 + lane;
                T K[9];
#pragma unroll
                for (int k = 0; k < 9; k++) K[k] = __ldg(&val[vb + 32 * k]);
                const T d0 = y[g][0] - v0, d1 = y[g][1] - v1, d2 = y[g][2] - v2;
                a0 += K[0] * d0 + K[1] * d1 + K[2] * d2;
                a1 += K[3] * d0 + K[4] * d1 + K[5] * d2;
                a2 += K[6] * d0 + K[7] * d1 + K[8] * d2;
            } else {
                const T m = __ldg(&mv[off]);
                a0 += m * y[g][0];
                a1 += m * y[g][1];
                a2 += m * y[g][2];
            }
        }
    }
    out[0] = a0;
    out[1] = a1;
    out[2] = a2;
}

// Vector of 4 T: the published copy of u in the CG kernel (x, y, z, 0), one
// 16-byte (FP32) load per neighbour instead of three 4-byte loads that each
// touch the same sectors.
struct alignas(16) Dbl4 {
    double x, y, z, w;
};
template <typename T> struct Vec4T;
template <> struct Vec4T<float> { using type = float4; };
template <> struct Vec4T<double> { using type = Dbl4; };

__device__ __forceinline__ float4 ldcg4(const float4 *p) { return __ldcg(p); }

// Read-only loads of data streamed once per CG iteration (the matrix of the
// memory-resident solve, larger than L2) with the L2 evict-first priority,
// so that the vectors gathered and re-read every iteration keep their lines.
__device__ __forceinline__ uint64_t l2_evict_first()
{
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float ld_stream(const float *p, uint64_t pol)
{
    float v;
    asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ double ld_stream(const double *p, uint64_t pol)
{
    double v;
    asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int ld_stream(const int *p, uint64_t pol)
{
    int v;
    asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ Dbl4 ldcg4(const Dbl4 *p)
{
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    return Dbl4{a.x, a.y, b.x, b.y};
}

// On-chip copy of a CTA's matrix rows for one solve (register-resident CG
// variant): the column indices of slots j < JC (col[j * CG_THREADS + t] for
// thread t) and the 9 values of slots j < J as four pairs and a single
// (kv2[(4 j + m) * CG_THREADS + t], kv1[j * CG_THREADS + t]).  The matrix is
// constant during a solve; each slot held on chip saves its L2 reads in every
// iteration, and cached column indices take the index -> neighbour dependency
// off the critical path of the gathers.
template <typename T>
struct CgCache {
    using T2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
    const int *col = nullptr;
    const T2 *kv2 = nullptr;
    const T *kv1 = nullptr;
    int J = 0, JC = 0;
};

// One 3x3 block times a difference vector, added with explicit FMAs so that
// every code path gives the same bits.
template <typename T>
__device__ __forceinline__ void block_fma(const T K[9], T d0, T d1, T d2, T &a0, T &a1, T &a2)
{
    a0 = fma(K[2], d2, fma(K[1], d1, fma(K[0], d0, a0)));
    a1 = fma(K[5], d2, fma(K[4], d1, fma(K[3], d0, a1)));
    a2 = fma(K[8], d2, fma(K[7], d1, fma(K[6], d0, a2)));
}

// q = A u for one row of the CG kernel (sell_row's arithmetic): slots with
// values on chip in groups of 4 (only the neighbour loads go to L2), then the
// rest in groups of 2 (values and neighbours from L2, issued together).
template <typename T, bool MEM = false>
__device__ __forceinline__ void sell_row_cg(const DeviceBatch &d, int row, bool nomass, T diag,
                                            const typename Vec4T<T>::type *u4, T out[3], const CgCache<T> &cc)
{
    const int sl = row >> 5, lane = row & 31, t = threadIdx.x;
    const int L = __ldg(&d.slice_len[sl]);
    const int base = __ldg(&d.slice_ptr[sl]);
    const auto me = ldcg4(&u4[row]);
    T a0 = diag * me.x, a1 = diag * me.y, a2 = diag * me.z;
    auto col_of = [&](int j) {
        return j < cc.JC ? cc.col[j * CG_THREADS + t] : __ldg(&d.sell_col[base + 32 * j + lane]);
    };
    if (!nomass) {
        const T *mv = static_cast<const T *>(d.sell_mval);
        for (int j = 0; j < L; j++) {
            const auto y = ldcg4(&u4[col_of(j)]);
            const T m = __ldg(&mv[base + 32 * j + lane]);
            a0 = fma(m, y.x, a0);
            a1 = fma(m, y.y, a1);
            a2 = fma(m, y.z, a2);
        }
        out[0] = a0;
        out[1] = a1;
        out[2] = a2;
        return;
    }
    if constexpr (MEM) {
        // memory-resident kernel (no on-chip copy): the column indices of the
        // next group are loaded together with this group's values and
        // neighbours, so a group costs one memory round trip instead of two
        // (index, then neighbour).  Same slots, same FMA order: same bits.
        const T *val = static_cast<const T *>(d.sell_val);
        const uint64_t pol = l2_evict_first();
        constexpr int G2 = 2;
        int cn[G2];
#pragma unroll
        for (int g = 0; g < G2; g++) cn[g] = g < L ? ld_stream(&d.sell_col[base + 32 * g + lane], pol) : row;
        for (int j0 = 0; j0 < L; j0 += G2) {
            typename Vec4T<T>::type y[G2];
            T K[G2][9];
            int nx[G2];
#pragma unroll
            for (int g = 0; g < G2; g++) {
                const int j = j0 + g;
                y[g] = ldcg4(&u4[cn[g]]);
                const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
#pragma unroll
                for (int k = 0; k < 9; k++) K[g][k] = j < L ? ld_stream(&val[vb + 32 * k], pol) : (T)0;
                const int jn = j + G2;
                nx[g] = jn < L ? ld_stream(&d.sell_col[base + 32 * jn + lane], pol) : row;
            }
#pragma unroll
            for (int g = 0; g < G2; g++)
                if (j0 + g < L) block_fma(K[g], y[g].x - me.x, y[g].y - me.y, y[g].z - me.z, a0, a1, a2);
#pragma unroll
            for (int g = 0; g < G2; g++) cn[g] = nx[g];
        }
        out[0] = a0;
        out[1] = a1;
        out[2] = a2;
        return;
    }
    const int Jk = min(cc.J, L);
    constexpr int G1 = 4;
    for (int j0 = 0; j0 < Jk; j0 += G1) {
        typename Vec4T<T>::type y[G1];
#pragma unroll
        for (int g = 0; g < G1; g++) y[g] = ldcg4(&u4[j0 + g < Jk ? col_of(j0 + g) : row]);
#pragma unroll
        for (int g = 0; g < G1; g++) {
            const int j = j0 + g;
            if (j >= Jk) break;
            T K[9];
#pragma unroll
            for (int m = 0; m < 4; m++) {
                const auto kp = cc.kv2[(4 * j + m) * CG_THREADS + t];
                K[2 * m] = kp.x;
                K[2 * m + 1] = kp.y;
            }
            K[8] = cc.kv1[j * CG_THREADS + t];
            block_fma(K, y[g].x - me.x, y[g].y - me.y, y[g].z - me.z, a0, a1, a2);
        }
    }
    const T *val = static_cast<const T *>(d.sell_val);
    constexpr int G2 = 2;
    for (int j0 = Jk; j0 < L; j0 += G2) {
        typename Vec4T<T>::type y[G2];
        T K[G2][9];
#pragma unroll
        for (int g = 0; g < G2; g++) {
            const int j = j0 + g;
            y[g] = ldcg4(&u4[j < L ? col_of(j) : row]);
            const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
#pragma unroll
            for (int k = 0; k < 9; k++) K[g][k] = j < L ? __ldg(&val[vb + 32 * k]) : (T)0;
        }
#pragma unroll
        for (int g = 0; g < G2; g++)
            if (j0 + g < L) block_fma(K[g], y[g].x - me.x, y[g].y - me.y, y[g].z - me.z, a0, a1, a2);
    }
    out[0] = a0;
    out[1] = a1;
    out[2] = a2;
}

// Standalone w = A u over every row of every blob, for timing SpMV variants:
// TPR threads per row (slots j with j % TPR == sub), GROUPED = the grouped
// loads of sell_row (TPR 1 only).  NoMass blobs only; other rows are skipped.
template <typename T, int TPR, bool GROUPED>
__global__ void __launch_bounds__(256) k_spmv_variant(DeviceBatch d, const T *__restrict__ v, T *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int rows_per_warp = 32 / TPR;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int sub = lane / rows_per_warp;
    const int row = gwarp * rows_per_warp + (lane % rows_per_warp);
    if (row >= d.nl_pad) return;
    const int b = d.tile_blob[row / NODE_TILE];
    const BlobParams &bp = d.bp[b];
    const bool valid = (row - bp.node_off) < bp.node_cnt && !(d.flags[row] & NODE_PINNED) && bp.solver == SOLVER_NOMASS;
    T a[3] = {0, 0, 0};
    if (valid) {
        const T diag = (T)(bp.calc_stokes == 1 ? d.drag[row] : 0.0);
        if (TPR == 1 && GROUPED) {
            sell_row<T>(d, row, true, diag, v, a);
        } else {
            const int sl = row >> 5, rl = row & 31;
            const int L = __ldg(&d.slice_len[sl]);
            const int base = __ldg(&d.slice_ptr[sl]);
            const T v0 = __ldcg(&v[3 * (size_t)row]), v1 = __ldcg(&v[3 * (size_t)row + 1]), v2 = __ldcg(&v[3 * (size_t)row + 2]);
            if (sub == 0) {
                a[0] = diag * v0;
                a[1] = diag * v1;
                a[2] = diag * v2;
            }
            const T *val = static_cast<const T *>(d.sell_val);
#pragma unroll 2
            for (int j = sub; j < L; j += TPR) {
                const int off = base + 32 * j + rl;
                const int q = __ldg(&d.sell_col[off]);
                const size_t vb = (size_t)(base + 32 * j) * 9 + rl;
                T K[9];
#pragma unroll
                for (int k = 0; k < 9; k++) K[k] = __ldg(&val[vb + 32 * k]);
                const T d0 = __ldcg(&v[3 * (size_t)q]) - v0, d1 = __ldcg(&v[3 * (size_t)q + 1]) - v1,
                        d2 = __ldcg(&v[3 * (size_t)q + 2]) - v2;
                a[0] += K[0] * d0 + K[1] * d1 + K[2] * d2;
                a[1] += K[3] * d0 + K[4] * d1 + K[5] * d2;
                a[2] += K[6] * d0 + K[7] * d1 + K[8] * d2;
            }
        }
    }
#pragma unroll
    for (int o = rows_per_warp; o < 32; o <<= 1)
#pragma unroll
        for (int cc = 0; cc < 3; cc++) a[cc] += __shfl_xor_sync(0xffffffffu, a[cc], o);
    if (sub == 0)
#pragma unroll
        for (int cc = 0; cc < 3; cc++) out[3 * (size_t)row + cc] = a[cc];
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

// Per-row state of the CG recurrences (3 components each).
template <typename T>
struct RowState {
    T x[3], r[3], u[3], w[3], s[3], p[3], dinv[3];
};

// Fields of the row state (memory-resident variant: each phase moves only
// the fields it reads or writes).
enum RowField : int { RF_X = 1, RF_R = 2, RF_U = 4, RF_W = 8, RF_S = 16, RF_P = 32, RF_DINV = 64 };

template <typename T>
__device__ __forceinline__ void load_fields(const DeviceBatch &d, int row, RowState<T> &S, int m)
{
    const size_t o = 3 * (size_t)row;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (m & RF_X) S.x[c] = static_cast<const T *>(d.x)[o + c];
        if (m & RF_R) S.r[c] = static_cast<const T *>(d.r)[o + c];
        if (m & RF_U) S.u[c] = static_cast<const T *>(d.u)[o + c];
        if (m & RF_W) S.w[c] = static_cast<const T *>(d.w)[o + c];
        if (m & RF_S) S.s[c] = static_cast<const T *>(d.s)[o + c];
        if (m & RF_P) S.p[c] = static_cast<const T *>(d.p)[o + c];
        if (m & RF_DINV) S.dinv[c] = static_cast<const T *>(d.dinv)[o + c];
    }
}

template <typename T>
__device__ __forceinline__ void store_fields(const DeviceBatch &d, int row, const RowState<T> &S, int m)
{
    const size_t o = 3 * (size_t)row;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (m & RF_X) static_cast<T *>(d.x)[o + c] = S.x[c];
        if (m & RF_R) static_cast<T *>(d.r)[o + c] = S.r[c];
        if (m & RF_U) static_cast<T *>(d.u)[o + c] = S.u[c];
        if (m & RF_W) static_cast<T *>(d.w)[o + c] = S.w[c];
        if (m & RF_S) static_cast<T *>(d.s)[o + c] = S.s[c];
        if (m & RF_P) static_cast<T *>(d.p)[o + c] = S.p[c];
    }
}

template <typename T>
__device__ __forceinline__ void load_row(const DeviceBatch &d, int row, RowState<T> &S)
{
    const size_t o = 3 * (size_t)row;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        S.x[c] = static_cast<const T *>(d.x)[o + c];
        S.r[c] = static_cast<const T *>(d.r)[o + c];
        S.u[c] = static_cast<const T *>(d.u)[o + c];
        S.w[c] = static_cast<const T *>(d.w)[o + c];
        S.s[c] = static_cast<const T *>(d.s)[o + c];
        S.p[c] = static_cast<const T *>(d.p)[o + c];
        S.dinv[c] = static_cast<const T *>(d.dinv)[o + c];
    }
}

template <typename T>
__device__ __forceinline__ void store_row(const DeviceBatch &d, int row, const RowState<T> &S)
{
    const size_t o = 3 * (size_t)row;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        static_cast<T *>(d.x)[o + c] = S.x[c];
        static_cast<T *>(d.r)[o + c] = S.r[c];
        static_cast<T *>(d.u)[o + c] = S.u[c];
        static_cast<T *>(d.w)[o + c] = S.w[c];
        static_cast<T *>(d.s)[o + c] = S.s[c];
        static_cast<T *>(d.p)[o + c] = S.p[c];
    }
}

__device__ __forceinline__ DF df_warp_sum(DF v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = df_add(v, w);
    }
    return v;
}

// Sum of N values per lane over a warp (N a power of two, 2..32) by a
// transposed butterfly: at offsets 16, 8, ... each lane keeps half of its
// values and adds its partner's copy of that half (N/2 + N/4 + ... shuffles),
// then the remaining offsets add whole values.  Returns this lane's total of
// value index idx; every lane holding the same idx holds the same bits.
template <int N>
__device__ __forceinline__ float warp_sum_multi(float (&v)[N], int &idx)
{
    static_assert(N >= 2 && N <= 32 && (N & (N - 1)) == 0, "N must be a power of two in [2, 32]");
    const int lane = threadIdx.x & 31;
    idx = 0;
    int o = 16;
#pragma unroll
    for (int h = N / 2; h >= 1; h /= 2, o /= 2) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < h; k++) {
            const float send = upper ? v[k] : v[k + h];
            const float keep = upper ? v[k + h] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
        if (upper) idx += h;
    }
    float x = v[0];
#pragma unroll
    for (; o > 0; o /= 2) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Partial sums of a CG segment, written to its slot P of the partials
// buffer: three dot-product terms, each a (hi, lo) float pair in P[0..5]
// (mask selects which), and NX plain FP32 sums in P[ex_off ..] (the
// segment's coarse-space restrictions).  Per thread and per warp the dot
// terms run in W; then warp k of the CTA combines quantity k over the warps,
// the dot terms in double-float (FP32 pipes) or FP64, in parallel.
template <typename W, int NX>
__device__ __forceinline__ void seg_partials(float *P, const W (&in)[3], int mask, const float *ex, int ex_off,
                                             double *smem_raw)
{
    static_assert(CG_THREADS / 32 >= 3 + NX, "one warp per combined quantity");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    W *sw = reinterpret_cast<W *>(smem_raw);
    float *sxs = reinterpret_cast<float *>(smem_raw + 3 * 32);
    if (sizeof(W) == 4) {
        // all 3 + NX values in one transposed butterfly
        constexpr int NV = (3 + NX) <= 4 ? 4 : (3 + NX) <= 8 ? 8 : 16;
        float v[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = k < 3 ? (float)in[k] : k < 3 + NX ? ex[k - 3] : 0.f;
        int idx;
        const float t = warp_sum_multi<NV>(v, idx);
        if ((lane & (32 / NV - 1)) == 0) {
            if (idx < 3) sw[idx * 32 + warp] = (W)t;
            else if (idx < 3 + NX) sxs[(idx - 3) * 32 + warp] = t;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const W s = warp_sum<W>(in[k]);
            if (lane == 0) sw[k * 32 + warp] = s;
        }
#pragma unroll
        for (int k = 0; k < NX; k++) {
            const float s = warp_sum<float>(ex[k]);
            if (lane == 0) sxs[k * 32 + warp] = s;
        }
    }
    __syncthreads();
    if (warp < 3) {
        if (mask & (1 << warp)) {
            float hi, lo;
            if (sizeof(W) == 4) {
                const DF v = df_warp_sum(DF{lane < nw ? (float)sw[warp * 32 + lane] : 0.f, 0.f});
                hi = v.hi;
                lo = v.lo;
            } else {
                const double a = warp_sum<double>(lane < nw ? (double)sw[warp * 32 + lane] : 0.0);
                hi = (float)a;
                lo = (float)(a - (double)hi);
            }
            if (lane == 0) {
                P[2 * warp] = hi;
                P[2 * warp + 1] = lo;
            }
        }
    } else if (warp < 3 + NX) {
        const int k = warp - 3;
        const float v = warp_sum<float>(lane < nw ? sxs[k * 32 + lane] : 0.f);
        if (lane == 0) P[ex_off + k] = v;
    }
    __syncthreads();
}

// Dynamic shared memory of the CG kernel (layout in k_cg).
extern __shared__ __align__(16) unsigned char cg_dyn[];

// Deferred segment partials of the memory-resident CG kernel (FP32 sums).
// seg_partials ends every segment with two CTA barriers, so every warp waits
// for the slowest one before it starts on the next segment's rows.  Here the
// per-warp stage of seg_partials goes to shared memory with no barrier, the
// warps run on into the next segments, and flush_partials runs the
// cross-warp stage for up to kDeferSegs segments after one barrier.  The
// arithmetic and its order are those of seg_partials: the same bits.
// Region (start of the dynamic shared memory): kDeferSegs x kDeferQ x 32
// floats, then per deferred segment (slot, dot-term mask, NX, ex_off).
struct DeferView {
    float *buf;
    int4 *meta;
};

__device__ __forceinline__ DeferView defer_view()
{
    DeferView v;
    v.buf = reinterpret_cast<float *>(cg_dyn);
    v.meta = reinterpret_cast<int4 *>(v.buf + kDeferSegs * kDeferQ * 32);
    return v;
}

template <int NX>
__device__ __forceinline__ void seg_partials_defer(const DeferView &dv, int c, int seg, int mask, int ex_off,
                                                   const float (&in)[3], const float *ex)
{
    static_assert(3 + NX <= kDeferQ, "values per warp and segment");
    constexpr int NV = (3 + NX) <= 4 ? 4 : (3 + NX) <= 8 ? 8 : 16;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float v[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = k < 3 ? in[k] : k < 3 + NX ? ex[k - 3] : 0.f;
    int idx;
    const float t = warp_sum_multi<NV>(v, idx);
    if ((lane & (32 / NV - 1)) == 0 && idx < 3 + NX) dv.buf[(c * kDeferQ + idx) * 32 + warp] = t;
    if (threadIdx.x == 0) dv.meta[c] = make_int4(seg, mask, NX, ex_off);
}

// The cross-warp stage of seg_partials for the cnt deferred segments, into
// the partials buffer part (floats, stride floats per segment slot).
__device__ __forceinline__ void flush_partials(const DeferView &dv, int cnt, float *part, int stride)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    for (int p = warp; p < cnt * kDeferQ; p += nw) {
        const int c = p / kDeferQ, q = p % kDeferQ;
        const int4 m = dv.meta[c];
        float *P = part + (size_t)stride * m.x;
        const float *src = dv.buf + (c * kDeferQ + q) * 32;
        if (q < 3) {
            if (m.y & (1 << q)) {
                const DF v = df_warp_sum(DF{lane < nw ? src[lane] : 0.f, 0.f});
                if (lane == 0) {
                    P[2 * q] = v.hi;
                    P[2 * q + 1] = v.lo;
                }
            }
        } else if (q - 3 < m.z) {
            const float v = warp_sum<float>(lane < nw ? src[lane] : 0.f);
            if (lane == 0) P[m.w + q - 3] = v;
        }
    }
    __syncthreads();
}

// Loads of segment partials in flight per thread before they are added.
constexpr int kSumUnroll = 4;

// Adds the partials of segments s0 + first, s0 + first + stride, ... (< cnt)
// to a[0..2] in that order; kSumUnroll loads are issued before the adds.
__device__ __forceinline__ void add_seg_partials(const double *part, int slot4, int s0, int cnt, int first, int stride,
                                                 DF a[3])
{
    for (int t = first; t < cnt; t += kSumUnroll * stride) {
        float4 v01[kSumUnroll];
        float2 v2[kSumUnroll];
#pragma unroll
        for (int u = 0; u < kSumUnroll; u++) {
            const int tt = t + u * stride;
            if (tt < cnt) {
                v01[u] = __ldcg(reinterpret_cast<const float4 *>(part) + (size_t)slot4 * (s0 + tt));
                v2[u] = __ldcg(reinterpret_cast<const float2 *>(part) + 2 * (size_t)slot4 * (s0 + tt) + 2);
            } else {
                v01[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                v2[u] = make_float2(0.f, 0.f);
            }
        }
#pragma unroll
        for (int u = 0; u < kSumUnroll; u++) {
            a[0] = df_add(a[0], DF{v01[u].x, v01[u].y});
            a[1] = df_add(a[1], DF{v01[u].z, v01[u].w});
            a[2] = df_add(a[2], DF{v2[u].x, v2[u].y});
        }
    }
}

// Sum of the three partial slots over a blob's CG segments, by the calling
// warp (lane-strided, then a butterfly): fixed order, so deterministic.
__device__ __forceinline__ void warp_blob_sums(const DeviceBatch &d, const double *part, int b, DF out[3])
{
    DF a[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    add_seg_partials(part, d.part_stride / 4, d.bp[b].seg_off, d.bp[b].seg_cnt, threadIdx.x & 31, 32, a);
#pragma unroll
    for (int k = 0; k < 3; k++) out[k] = df_warp_sum(a[k]);
}

// The same for one blob with the whole CTA: thread-strided sums, a butterfly
// per warp, then warp 0 combines the warp sums of each quantity with a
// butterfly.  The result is valid in warp 0 only (every lane of it); the
// caller synchronises before reusing sm (2 * 3 * 32 floats).
__device__ __forceinline__ void block_blob_sums(const DeviceBatch &d, const double *part, int b, DF out[3],
                                                float *sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    DF a[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    add_seg_partials(part, d.part_stride / 4, d.bp[b].seg_off, d.bp[b].seg_cnt, threadIdx.x, blockDim.x, a);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const DF s = df_warp_sum(a[k]);
        if (lane == 0) {
            sm[2 * (k * 32 + warp)] = s.hi;
            sm[2 * (k * 32 + warp) + 1] = s.lo;
        }
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const DF v = lane < nw ? DF{sm[2 * (k * 32 + lane)], sm[2 * (k * 32 + lane) + 1]} : DF{0.f, 0.f};
            out[k] = df_warp_sum(v);
        }
    }
}

// One CG transition of a blob from its three sums:
//   ACTIVE   sums r.u, w.u, r.r: stop test, then alpha / beta of the next update
//   VERIFY   sums r.u, -, |b - A x|^2: converged, or restart from that residual
//   RESTART  sums r.u, w.u, -: alpha of the first restarted update, beta = 0
// Returns true when the blob stops (cg.state is then CONVERGED or FAILED) and
// sets *fail_bits to the failure bits (0 if none).
//
// FP64 precision runs the recurrence in FP64: alpha = r.u / (w.u - beta r.u /
// alpha_prev), beta = r.u / r.u_prev, stop when r.r / f.f < eps^2.  Mixed
// precision (`fast`) applies alpha and beta in FP32 anyway and runs it in
// FP32 as alpha = r.u / p.Ap with p.Ap = w.u - beta^2 (p.Ap)_prev (the same
// recurrence), stop when r.r < eps^2 f.f: FP64 arithmetic and conversions run
// at 1/64 of the FP32 rate and would sit on the critical path of every
// iteration.  VERIFY (once per solve) stays in FP64.
__device__ __forceinline__ bool transition_core(CgScalars &cg, const BlobParams &bp, const DF sums[3],
                                                int *fail_bits, bool fast)
{
    const int limit = bp.solver == SOLVER_MASS ? bp.max_iter - 1 : bp.max_iter;
    int finish = 0, bits = 0;
    if (cg.state == CG_ACTIVE) {
        bool conv, nan, breakdown = false, at_floor = false;
        if (fast) {
            const float g = sums[0].hi + sums[0].lo, dl = sums[1].hi + sums[1].lo, rr = sums[2].hi + sums[2].lo;
            conv = rr < cg.stop_f;
            nan = !(rr == rr) || !(g == g) || !(dl == dl);
            if (!(cg.iters > 0 && conv) && !nan && cg.iters < limit) {
                const float beta = cg.iters == 0 ? 0.f : g / cg.gamma_f;
                const float pap = cg.iters == 0 ? dl : fmaf(-beta * beta, cg.pap_f, dl);
                if (!(pap > 0.f) || !(g > 0.f)) {
                    // the FP32 recurrence broke down (p.Ap or r.u not
                    // positive, so alpha would not be finite).  Below the
                    // floor this is the precision limit of FP32 vectors
                    // (an epsilon tighter than FP32 can reach): stop there;
                    // above it, it is a failure.
                    breakdown = true;
                    at_floor = rr < cg.floor_f;
                } else {
                    cg.beta_f = beta;
                    cg.pap_f = pap;
                    cg.alpha_f = g / pap;
                    cg.gamma_f = g;
                }
            }
        } else {
            const double g = (double)sums[0].hi + (double)sums[0].lo, dl = (double)sums[1].hi + (double)sums[1].lo;
            const double rr = (double)sums[2].hi + (double)sums[2].lo;
            cg.rr = rr;
            const double res = (cg.ff == 0.0) ? 0.0 : rr / cg.ff;
            conv = res < bp.epsilon2;
            nan = !(res == res) || !(g == g) || !(dl == dl);
            if (!(cg.iters > 0 && conv) && !nan && cg.iters < limit) {
                if (cg.iters == 0) {
                    cg.beta = 0.0;
                    cg.alpha = g / dl;
                } else {
                    const double beta = g / cg.gamma;
                    cg.alpha = g / (dl - beta * g / cg.alpha);
                    cg.beta = beta;
                }
                cg.gamma = g;
            }
        }
        if ((cg.iters > 0 && conv) || (breakdown && at_floor)) {
            // with the true-residual check on, the FP64 b - A x decides
            // (converged, or a restart from it)
            if (bp.true_residual) cg.state = CG_VERIFY;
            else finish = CG_CONVERGED;
        } else if (breakdown) {
            finish = CG_FAILED;
            bits = BLOB_FAIL_CG;
        } else if (nan) {
            finish = CG_FAILED;
            bits = BLOB_FAIL_CG | BLOB_FAIL_NAN;
        } else if (cg.iters >= limit) {
            finish = CG_FAILED;
            bits = BLOB_FAIL_CG;
        } else {
            cg.iters += 1;
        }
    } else if (cg.state == CG_VERIFY) {
        const double tr = (double)sums[2].hi + (double)sums[2].lo;
        cg.true_relres2 = (cg.ff == 0.0) ? 0.0 : tr / cg.ff;
        if (cg.true_relres2 < bp.epsilon2) {
            finish = CG_CONVERGED;
        } else if (cg.restarts >= kMaxRestarts || cg.iters >= limit) {
            finish = CG_FAILED;
            bits = BLOB_FAIL_CG;
        } else {
            cg.restarts += 1;
            cg.gamma = (double)sums[0].hi + (double)sums[0].lo;
            cg.gamma_f = sums[0].hi + sums[0].lo;
            cg.state = CG_RESTART;
        }
    } else if (cg.state == CG_RESTART) {
        // r.u of the restarted u (phase B of the restart step recomputes it,
        // with the coarse correction where there is one)
        cg.state = CG_ACTIVE;
        cg.iters += 1;
        bool nan;
        if (fast) {
            cg.gamma_f = sums[0].hi + sums[0].lo;
            cg.beta_f = 0.f;
            cg.pap_f = sums[1].hi + sums[1].lo;
            cg.alpha_f = cg.gamma_f / cg.pap_f;
            nan = !(cg.alpha_f == cg.alpha_f);
        } else {
            cg.gamma = (double)sums[0].hi + (double)sums[0].lo;
            cg.beta = 0.0;
            cg.alpha = cg.gamma / ((double)sums[1].hi + (double)sums[1].lo);
            nan = !(cg.alpha == cg.alpha);
        }
        if (nan) {
            finish = CG_FAILED;
            bits = BLOB_FAIL_CG | BLOB_FAIL_NAN;
        }
    }
    if (finish) cg.state = finish;
    *fail_bits = bits;
    return finish != 0;
}

// The coefficients of the next update in the arithmetic type of the vectors.
template <typename T>
__device__ __forceinline__ void cg_coefs(const CgScalars &cg, T &alpha, T &beta);
template <>
__device__ __forceinline__ void cg_coefs<float>(const CgScalars &cg, float &alpha, float &beta)
{
    alpha = cg.alpha_f;
    beta = cg.beta_f;
}
template <>
__device__ __forceinline__ void cg_coefs<double>(const CgScalars &cg, double &alpha, double &beta)
{
    alpha = cg.alpha;
    beta = cg.beta;
}

// The iteration's reduced sums (r.u, w.u, r.r) as the transition received
// them, kept per blob for inspection of the reduction's accuracy.
__device__ __forceinline__ void record_sums(const DeviceBatch &d, int b, const DF sums[3])
{
#pragma unroll
    for (int i = 0; i < 3; i++) d.last_sums[3 * (size_t)b + i] = (double)sums[i].hi + (double)sums[i].lo;
}

// The transition run by the CTA that arrived last at a reducing barrier
// (exactly once per blob), on the blob's record in global memory.
__device__ __forceinline__ void cg_transition(const DeviceBatch &d, int b, const DF sums[3])
{
    // read through L2: the record may have been written by another SM's last CTA
    CgScalars cg;
    {
        static_assert(sizeof(CgScalars) % 8 == 0, "CgScalars must be 8-byte words");
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&d.cg[b]);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(&cg);
#pragma unroll
        for (int i = 0; i < (int)(sizeof(CgScalars) / 8); i++) dst[i] = __ldcg(src + i);
    }
    int bits;
    record_sums(d, b, sums);
    if (transition_core(cg, d.bp[b], sums, &bits, d.precision == PREC_MIXED)) {
        atomicSub(&d.bar[2], 1u);
        if (bits) atomicOr(&d.status[b], bits);
    }
    d.cg[b] = cg;
}

// Grid barrier whose last arriving CTA first reduces the partial sums of
// every busy blob and runs its CG transition, then publishes the count of
// blobs still iterating and releases the others.  Bounded waits as in
// counting_barrier.
__device__ __forceinline__ unsigned int reducing_barrier(const DeviceBatch &d, const double *part, int *s_err,
                                                         unsigned int *s_pub, int *s_last, float *sm)
{
    unsigned int *bar = d.bar;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vb = bar;
        s_last[1] = (int)vb[1];  // generation before arriving
        __threadfence();
        const unsigned int arrived = atomicAdd(&bar[0], 1u);
        s_last[0] = arrived == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last[0]) {
        __threadfence();
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (d.num_blobs < 8) {
            for (int b = 0; b < d.num_blobs; b++) {
                const int st = __ldcg(&d.cg[b].state);
                if (st == CG_CONVERGED || st == CG_FAILED) continue;
                DF sums[3];
                block_blob_sums(d, part, b, sums, sm);
                if (threadIdx.x == 0) cg_transition(d, b, sums);
                __syncthreads();  // sm reused by the next blob
            }
        } else {
            for (int b = warp; b < d.num_blobs; b += blockDim.x >> 5) {
                const int st = __ldcg(&d.cg[b].state);
                if (st == CG_CONVERGED || st == CG_FAILED) continue;
                DF sums[3];
                warp_blob_sums(d, part, b, sums);
                if (lane == 0) cg_transition(d, b, sums);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            volatile unsigned int *vb = bar;
            __threadfence();
            vb[3] = vb[2];
            vb[0] = 0;
            __threadfence();
            atomicAdd(&bar[1], 1u);
        }
    } else if (threadIdx.x == 0) {
        volatile unsigned int *vb = bar;
        const unsigned int gen = (unsigned int)s_last[1];
        unsigned int spins = 0;
        while (vb[1] == gen) {
            if (++spins > kSpinLimit || vb[4]) {
                *s_err = 1;
                atomicExch(&bar[4], 1u);
                break;
            }
            __nanosleep(32);
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        *s_pub = ((volatile unsigned int *)bar)[3];
    }
    __syncthreads();
    return *s_pub;
}

// Reduction without a serial step: after a plain grid barrier every CTA sums
// the partials of every busy blob itself, in the same fixed order, and runs
// the transitions on its own copy of the blob records in shared memory, so
// all CTAs reach bit-identical states.  CTA 0 alone records failure bits.
// Also refreshes the CTA's view (state, alpha, beta of its nb blobs) and
// returns the number of blobs still iterating.
//
// With the coarse space (coarse_n > 0; one blob per CTA) it also forms the
// CTA's coarse correction for the next update: thread j holds coarse dof j
// of the blob, with h_j = (P^T s)_j carried from iteration to iteration, and
// from the segment restrictions of this iteration (slot floats 8..: P^T r_k,
// 14..: P^T w_k) computes h = P^T w_k + beta h, g = P^T r_(k+1) = P^T r_k -
// alpha h with the new alpha and beta (after a failed true-residual check,
// RESTART: g = P^T r of the true residual), then c = X g over the CTA's six
// rows of X ~ A_c^-1 in one block reduction.
// The coarse-space region of the dynamic shared memory: per thread the rest
// offset and smoother weight (phi), the CTA's 6 rows of X, c (8 floats),
// 6 x 32 reduction floats, and (P^T s)_j per coarse dof j.  The addresses are
// recomputed from kernel parameters wherever they are used, so that they
// need no registers across the iteration.
struct CoarseView {
    float4 *phi;
    float *xrow, *cvec, *red6, *h;
};

template <typename T>
__device__ __forceinline__ CoarseView coarse_view(const DeviceBatch &d)
{
    using T2 = typename CgCache<T>::T2;
    size_t off = 12 * (size_t)CG_THREADS * sizeof(T) + (size_t)d.cg_cache_cols * CG_THREADS * sizeof(int) +
                 (size_t)d.cg_cache_slots * CG_THREADS * (4 * sizeof(T2) + sizeof(T));
    off = (off + 15) & ~(size_t)15;
    CoarseView v;
    v.phi = reinterpret_cast<float4 *>(cg_dyn + off);
    v.xrow = reinterpret_cast<float *>(v.phi + CG_THREADS);
    v.cvec = v.xrow + 6 * (size_t)d.coarse_nmax;
    v.red6 = v.cvec + 8;
    v.h = v.red6 + 6 * 32;
    return v;
}

// The on-chip matrix copy of the register-resident CG kernel (layout in
// k_cg), recomputed from kernel parameters where it is used.
template <typename T>
__device__ __forceinline__ CgCache<T> cg_cache_view(const DeviceBatch &d)
{
    using T2 = typename CgCache<T>::T2;
    CgCache<T> cc;
    cc.J = d.cg_cache_slots;
    cc.JC = d.cg_cache_cols;
    cc.col = reinterpret_cast<const int *>(cg_dyn + 12 * (size_t)CG_THREADS * sizeof(T));
    cc.kv2 = reinterpret_cast<const T2 *>(cc.col + (size_t)cc.JC * CG_THREADS);
    cc.kv1 = reinterpret_cast<const T *>(cc.kv2 + 4 * (size_t)cc.J * CG_THREADS);
    return cc;
}

// c = X g, g_j held by thread j (zero beyond n): a 6-value block reduction.
template <typename T>
__device__ __forceinline__ void coarse_apply(const DeviceBatch &d, int n, float g)
{
    const CoarseView cv = coarse_view<T>(d);
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
    float v[8];
#pragma unroll
    for (int l = 0; l < 8; l++) v[l] = (l < 6 && j < n) ? cv.xrow[l * n + j] * g : 0.f;
    int idx;
    const float t = warp_sum_multi<8>(v, idx);
    if ((lane & 3) == 0 && idx < 6) cv.red6[idx * 32 + warp] = t;
    __syncthreads();
    if (warp < 6) {
        const float u = warp_sum<float>(lane < (int)(blockDim.x >> 5) ? cv.red6[warp * 32 + lane] : 0.f);
        if (lane == 0) cv.cvec[warp] = u;
    }
    __syncthreads();
}

// Coarse space of the memory-resident CG kernel (several segments per CTA,
// any number of coarse dofs per blob).  Dynamic shared memory, after the
// deferred-partials region: c of each of the CTA's segments (8 floats),
// 32 x 8 reduction floats, the first coarse dof of each of the CTA's blobs in
// the next two arrays, then g and (P^T s)_j for every coarse dof of every
// blob the CTA touches (coarse_hmax floats each, blob after blob).  Every CTA that
// touches a blob carries its own copy of that blob's P^T s; all copies follow
// the same arithmetic on the same partial sums, so they hold the same bits.
struct CoarseMemView {
    float *cvec, *red, *g, *h;
    int *hoff;  // per blob k of the CTA: its first coarse dof in g and h
};

__device__ __forceinline__ CoarseMemView coarse_mem_view(const DeviceBatch &d)
{
    CoarseMemView v;
    v.cvec = reinterpret_cast<float *>(cg_dyn + kDeferBytes);
    v.red = v.cvec + 8 * CG_MAX_SEGS;
    v.hoff = reinterpret_cast<int *>(v.red + 8 * 32);
    v.g = reinterpret_cast<float *>(v.hoff + CG_MAX_SEGS);
    v.h = v.g + d.coarse_hmax;
    return v;
}

// Phi_p^T v = (v, d_p x v) into ex[0..5] for the rest offset f.xyz of row p
template <typename T>
__device__ __forceinline__ void restrict6_of(const float4 f, const T v[3], float *ex)
{
    const float v0 = (float)v[0], v1 = (float)v[1], v2 = (float)v[2];
    ex[0] = v0;
    ex[1] = v1;
    ex[2] = v2;
    ex[3] = f.y * v2 - f.z * v1;
    ex[4] = f.z * v0 - f.x * v2;
    ex[5] = f.x * v1 - f.y * v0;
}

// u = omega D^-1 r + Phi_p c for row p (f = rest offset and omega, c = its
// segment's coarse correction)
template <typename T>
__device__ __forceinline__ void coarse_u_of(const float4 f, const float *c, const T dinv[3], const T r[3], T u[3])
{
    const float cx = c[3], cy = c[4], cz = c[5];
    const T pc[3] = {(T)(c[0] + cy * f.z - cz * f.y), (T)(c[1] + cz * f.x - cx * f.z), (T)(c[2] + cx * f.y - cy * f.x)};
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = (T)f.w * dinv[k] * r[k] + pc[k];
}

// acc + sum_t h_t g_t over the eight FP16 values h of one 16-byte load
// (lowest address first), in order
__device__ __forceinline__ float dot8_half(const uint4 raw, const float (&g)[8], float acc)
{
    const unsigned int w[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        acc = fmaf(__half2float(__ushort_as_half((unsigned short)(w[q] & 0xffffu))), g[2 * q], acc);
        acc = fmaf(__half2float(__ushort_as_half((unsigned short)(w[q] >> 16))), g[2 * q + 1], acc);
    }
    return acc;
}

// The coarse corrections of the CTA's segments for the next update
// (memory-resident kernel), after the iteration's partial sums and the CG
// transitions.  First, for every blob k of the CTA (state ACTIVE or RESTART,
// or every blob in the prologue), from the restrictions in the partial slots
// (P^T r at float 8, P^T w at float 14), each blob in its own region:
//   restart / prologue: h = 0, g = P^T r
//   else:               h = P^T w + beta h, g = P^T r - alpha h  (= P^T r_(k+1))
// then, after one barrier, c_j = X_j g for every segment j of those blobs,
// X_j the segment's six rows of X ~ A_c^-1 (global memory, read once per
// iteration).  wps warps share a segment (lane-strided over its blob's coarse
// dofs, 6 sums per lane, a transposed butterfly per warp), then one thread per
// (segment, row) adds the wps warp sums in order: fixed order, so
// deterministic.  A CTA that holds segments of many blobs (a dealt batch)
// pays two barriers per round of 32 / wps segments, not per blob.
template <typename T>
__device__ __forceinline__ void coarse_mem_step(const DeviceBatch &d, const float *part, const int *s_sid, int nt,
                                                int nb, const int *s_blob, const int *s_tslot, const int *s_state,
                                                const T *s_alpha, const T *s_beta, bool prologue)
{
    const CoarseMemView cv = coarse_mem_view(d);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int hoff = 0;
    for (int k = 0; k < nb; k++) {
        const BlobParams &bp = d.bp[s_blob[k]];
        const int n = bp.coarse_n, st = s_state[k];
        if (tid == 0) cv.hoff[k] = hoff;
        if (n > 0 && (prologue || st == CG_ACTIVE || st == CG_RESTART)) {  // CTA-uniform
            const bool restart = prologue || st == CG_RESTART;
            const float a = (float)s_alpha[k], be = (float)s_beta[k];
            float *h = cv.h + hoff, *g = cv.g + hoff;
            for (int i = tid; i < n; i += blockDim.x) {
                const float *sl = part + (size_t)d.part_stride * (bp.seg_off + i / 6);
                const float pr = __ldcg(sl + 8 + i % 6);
                const float sc = d.coarse_Xh ? __ldg(&d.coarse_s[bp.coarse_off + i]) : 1.f;
                if (restart) {
                    h[i] = 0.f;
                    g[i] = sc * pr;
                } else {
                    const float hn = __ldcg(sl + 14 + i % 6) + be * h[i];
                    h[i] = hn;
                    g[i] = sc * (pr - a * hn);
                }
            }
        }
        hoff += n;
    }
    __syncthreads();
    int wps = 1;
    while (wps * 2 * nt <= 32) wps *= 2;
    const int per_round = 32 / wps;
    for (int q0 = 0; q0 < nt; q0 += per_round) {
        const int j = q0 + warp / wps, sub = warp % wps;
        // the row scale of the FP16 copy for the final sums below, loaded
        // ahead so that its latency overlaps the products
        float srow = 1.f;
        if (d.coarse_Xh && tid < 6 * per_round && q0 + tid / 6 < nt) {
            const int jj = q0 + tid / 6;
            const BlobParams &bp = d.bp[s_blob[s_tslot[jj]]];
            if (bp.coarse_n > 0) srow = __ldg(&d.coarse_s[bp.coarse_off + 6 * (s_sid[jj] - bp.seg_off) + tid % 6]);
        }
        float v[8];
#pragma unroll
        for (int l = 0; l < 8; l++) v[l] = 0.f;
        if (j < nt) {
            const int k = s_tslot[j], st = s_state[k];
            const BlobParams &bp = d.bp[s_blob[k]];
            const int n = bp.coarse_n;
            if (n > 0 && (prologue || st == CG_ACTIVE || st == CG_RESTART)) {  // warp-uniform
                const float *g = cv.g + cv.hoff[k];
                const float *Xr = d.coarse_X + bp.coarse_xoff + (size_t)(6 * (s_sid[j] - bp.seg_off)) * n;
                if (d.coarse_Xh) {
                    // the FP16 copy S^-1 X S^-1 (g holds S g): eight coarse
                    // dofs a lane and 16-byte load, rows padded to nh
                    const int nh = (n + 7) & ~7, n8 = nh >> 3;
                    const uint4 *X8 = reinterpret_cast<const uint4 *>(d.coarse_Xh + bp.coarse_hxoff +
                                                                      (size_t)(6 * (s_sid[j] - bp.seg_off)) * nh);
#pragma unroll 2
                    for (int i = sub * 32 + lane; i < n8; i += wps * 32) {
                        float gv[8];
#pragma unroll
                        for (int t = 0; t < 8; t++) gv[t] = 8 * i + t < n ? g[8 * i + t] : 0.f;
#pragma unroll
                        for (int l = 0; l < 6; l++) v[l] = dot8_half(__ldcg(X8 + (size_t)l * n8 + i), gv, v[l]);
                    }
                } else {
#pragma unroll 4
                    for (int i = sub * 32 + lane; i < n; i += wps * 32) {
                        const float gi = g[i];
#pragma unroll
                        for (int l = 0; l < 6; l++) v[l] = fmaf(__ldcg(Xr + (size_t)l * n + i), gi, v[l]);
                    }
                }
            }
        }
        int idx;
        const float t = warp_sum_multi<8>(v, idx);
        if ((lane & 3) == 0) cv.red[warp * 8 + idx] = t;
        __syncthreads();
        if (tid < 6 * per_round) {
            const int jj = tid / 6, l = tid % 6;
            if (q0 + jj < nt) {
                float sum = 0.f;
                for (int w = 0; w < wps; w++) sum += cv.red[(jj * wps + w) * 8 + l];
                cv.cvec[8 * (q0 + jj) + l] = sum * srow;
            }
        }
        __syncthreads();
    }
}

// L2 load issued where it stands (volatile asm keeps it ahead of the
// barriers that follow, so its latency overlaps the reduction's own loads)
__device__ __forceinline__ float ld_early(const float *p)
{
    float v;
    asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

template <typename T>
__device__ __forceinline__ unsigned int local_reduce(const DeviceBatch &d, const double *part, CgScalars *s_cg,
                                                     float *sm, unsigned int *s_run, int nb, const int *s_blob,
                                                     int *s_state, T *s_alpha, T *s_beta, int coarse_n)
{
    const int nbl = d.num_blobs, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr bool fast = sizeof(T) == 4;
    // coarse restrictions, loaded first so that they travel with the sums
    float ptr = 0.f, ptw = 0.f;
    int cb = -1;
    if (coarse_n) {
        cb = s_blob[0];
        const BlobParams &bp = d.bp[cb];
        const int j = threadIdx.x;
        if (j < bp.coarse_n) {
            const float *slot = reinterpret_cast<const float *>(part) + (size_t)d.part_stride * (bp.seg_off + j / 6);
            ptr = ld_early(slot + 8 + j % 6);
            ptw = ld_early(slot + 14 + j % 6);
        }
    }
    if (nbl < 8) {
        // one blob after the other with the whole CTA; thread 0 (in warp 0,
        // which holds the sums) runs every transition
        for (int b = 0; b < nbl; b++) {
            const int st = s_cg[b].state;
            if (st == CG_CONVERGED || st == CG_FAILED) continue;  // CTA-uniform
            DF sums[3];
            block_blob_sums(d, part, b, sums, sm);
            if (threadIdx.x == 0) {
                if (blockIdx.x == 0) record_sums(d, b, sums);
                int bits;
                if (transition_core(s_cg[b], d.bp[b], sums, &bits, fast) && bits && blockIdx.x == 0)
                    atomicOr(&d.status[b], bits);
            }
            if (b + 1 < nbl) __syncthreads();  // sm reused by the next blob
        }
    } else {
        for (int b = warp; b < nbl; b += blockDim.x >> 5) {
            const int st = s_cg[b].state;
            if (st == CG_CONVERGED || st == CG_FAILED) continue;  // warp-uniform
            DF sums[3];
            warp_blob_sums(d, part, b, sums);
            if (lane == 0) {
                if (blockIdx.x == 0) record_sums(d, b, sums);
                int bits;
                if (transition_core(s_cg[b], d.bp[b], sums, &bits, fast) && bits && blockIdx.x == 0)
                    atomicOr(&d.status[b], bits);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        unsigned int n = 0;
        for (int b = 0; b < nbl; b++) n += !(s_cg[b].state == CG_CONVERGED || s_cg[b].state == CG_FAILED);
        *s_run = n;
        for (int k = 0; k < nb; k++) {
            const CgScalars &cg = s_cg[s_blob[k]];
            s_state[k] = cg.state;
            cg_coefs<T>(cg, s_alpha[k], s_beta[k]);
        }
    }
    __syncthreads();
    if (coarse_n) {
        const CgScalars &cg = s_cg[cb];
        float g = 0.f;
        if (threadIdx.x < coarse_n) {
            float &h = coarse_view<T>(d).h[threadIdx.x];
            if (cg.state == CG_RESTART) {
                h = 0.f;
                g = ptr;
            } else {
                h = ptw + cg.beta_f * h;
                g = ptr - cg.alpha_f * h;
            }
        }
        coarse_apply<T>(d, coarse_n, g);
    }
    return *s_run;
}

// The whole solve of every blob in one cooperative launch: Jacobi-PCG in the
// Chronopoulos-Gear form (one SpMV and one group of dot products per
// iteration), x0 = 0, stopping on residual2() = sum r^2 / sum f^2 < eps^2
// after each update (src/NoMassCGSolver.cpp:180-189, :233-247).  Per
// iteration: phase A updates p, s, x, r and u = D^-1 r of the own rows; a
// grid barrier makes u visible; phase B computes w = A u; then r.u, r.r and
// w.u are summed per blob and each blob's CG state advances.  With few
// segments and blobs (cg_local) every CTA does that sum itself after a plain
// barrier, from partials double-buffered by iteration parity (a fast CTA's
// next phase A must not overwrite what a slow CTA is still summing); else a
// reducing barrier does it once, in the last CTA to arrive.  With
// true_residual on, a recursive convergence is confirmed by an FP64 b - A x
// and a failed check restarts the recurrences from that residual.
//
// Work split: the rows of each blob are cut into segments (32-row aligned, at
// most CG_THREADS rows); CTA c owns segments [n_segs*c/G, n_segs*(c+1)/G) and
// thread t row t of each.  With one segment per CTA (REG) the row state stays
// in registers for the whole solve; only u and x go to memory, for the
// neighbours.
template <typename T, bool REG>
__global__ void __launch_bounds__(CG_THREADS, 1) k_cg(DeviceBatch d)
{
    using W = T;
    __shared__ double red[3 * 32 + 9 * 32];  // 3 dot terms (W) and up to 18 FP32 sums per warp
    __shared__ float sm_df[2 * 3 * 32];
    __shared__ int s_nt, s_nb, s_err, s_last[2];
    __shared__ unsigned int s_pub;
    __shared__ int s_tslot[CG_MAX_SEGS], s_row0[CG_MAX_SEGS], s_rows[CG_MAX_SEGS];
    __shared__ int s_blob[CG_MAX_SEGS], s_state[CG_MAX_SEGS];
    __shared__ int s_sid[CG_MAX_SEGS];  // global index of the CTA's segment j
    __shared__ T s_alpha[CG_MAX_SEGS], s_beta[CG_MAX_SEGS];
    __shared__ CgScalars s_cg[CG_LOCAL_MAX_BLOBS];
    __shared__ unsigned int s_run;

    const int G = gridDim.x, c = blockIdx.x, tid = threadIdx.x;
    const bool local = d.cg_local;
    const int S0 = (int)(((long long)d.n_segs * c) / G), S1 = (int)(((long long)d.n_segs * (c + 1)) / G);
    if (tid == 0) {
        s_err = 0;
        int nb = 0;
        for (int j = 0; j < S1 - S0; j++) {
            // the CTA's segments: a range of the blob-ordered segments, or
            // its part of a list that deals every blob's segments over the
            // CTAs (memory-resident batches), sorted by segment
            const int sid = d.seg_order ? d.seg_order[S0 + j] : S0 + j;
            s_sid[j] = sid;
            const int b = d.seg_blob[sid];
            if (nb == 0 || s_blob[nb - 1] != b) s_blob[nb++] = b;
            s_tslot[j] = nb - 1;
            s_row0[j] = d.seg_row0[sid];
            s_rows[j] = d.seg_rows[sid];
        }
        s_nt = S1 - S0;
        s_nb = nb;
    }
    if (local)
        for (int b = tid; b < d.num_blobs; b += CG_THREADS) s_cg[b] = d.cg[b];
    __syncthreads();
    const int nt = s_nt, nb = s_nb;
    // the CG state of this CTA's blobs: its own records (local) or as
    // published by the last reducing barrier
    auto refresh = [&]() {
        for (int k = tid; k < nb; k += CG_THREADS) {
            if (local) {
                const CgScalars &cg = s_cg[s_blob[k]];
                s_state[k] = cg.state;
                cg_coefs<T>(cg, s_alpha[k], s_beta[k]);
            } else {
                const CgScalars *cg = &d.cg[s_blob[k]];
                s_state[k] = __ldcg(&cg->state);
                if (sizeof(T) == 4) {
                    s_alpha[k] = (T)__ldcg(&cg->alpha_f);
                    s_beta[k] = (T)__ldcg(&cg->beta_f);
                } else {
                    s_alpha[k] = (T)__ldcg(&cg->alpha);
                    s_beta[k] = (T)__ldcg(&cg->beta);
                }
            }
        }
        __syncthreads();
    };
    // partials buffer of the current iteration, and a segment's slot in it
    int parity = 0;
    auto part = [&]() { return d.partials + (size_t)parity * (d.part_stride / 2) * d.n_segs; };
    auto slot = [&](int seg) { return reinterpret_cast<float *>(part()) + (size_t)d.part_stride * seg; };
    refresh();
    using V4 = typename Vec4T<T>::type;
    using T2 = typename CgCache<T>::T2;
    // x and the published u in global memory: addresses from the kernel
    // parameters at each use (no registers held across the iteration)
    auto X = [&]() { return static_cast<T *>(d.x); };
    auto U4 = [&]() { return static_cast<V4 *>(d.u4); };

    // row of this thread in segment j, and whether it is a free (unpinned) row
    auto row_of = [&](int j, bool &valid) {
        const int row = s_row0[j] + tid;
        valid = tid < s_rows[j] && !(d.flags[row] & NODE_PINNED);
        return row;
    };
    auto diag_of = [&](int j, int row, bool &nomass) {
        const BlobParams &bp = d.bp[s_blob[s_tslot[j]]];
        nomass = bp.solver == SOLVER_NOMASS;
        return nomass ? (T)(bp.calc_stokes == 1 ? d.drag[row] : 0.0) : static_cast<const T *>(d.mass_diag)[row];
    };
    // REG: r, u, w of the CTA's only segment in registers; x, D^-1, p, s and
    // the on-chip matrix copy in dynamic shared memory (p and s are used in
    // phase A only; in registers they would be spilled around the SpMV):
    //   x[3 CG_THREADS] T | dinv[3 CG_THREADS] T | p[3 CG_THREADS] T |
    //   s[3 CG_THREADS] T | col[JC CG_THREADS] int | kv2[4 J CG_THREADS] T2 |
    //   kv1[J CG_THREADS] T | coarse region (coarse_view)
    RowState<T> reg;
    bool reg_valid = false, reg_nomass = true;
    T reg_diag = 0;
    T *sx = reinterpret_cast<T *>(cg_dyn);
    T *sdinv = sx + 3 * CG_THREADS;
    if (REG) {
        const CgCache<T> cc = cg_cache_view<T>(d);
        const int row = row_of(0, reg_valid);
        const size_t o = 3 * (size_t)row;
        if (tid < s_rows[0]) {
            reg_diag = diag_of(0, row, reg_nomass);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                reg.r[k] = static_cast<const T *>(d.r)[o + k];
                reg.u[k] = static_cast<const T *>(d.u)[o + k];
                reg.w[k] = static_cast<const T *>(d.w)[o + k];
                sx[(9 + k) * CG_THREADS + tid] = static_cast<const T *>(d.s)[o + k];
                sx[(6 + k) * CG_THREADS + tid] = static_cast<const T *>(d.p)[o + k];
                sx[k * CG_THREADS + tid] = static_cast<const T *>(d.x)[o + k];
                sdinv[k * CG_THREADS + tid] = static_cast<const T *>(d.dinv)[o + k];
            }
        }
        // every free row (NoMass or mass) reads its column indices from the
        // copy; only NoMass rows read values from it
        if (reg_valid) {
            const int sl = row >> 5, lane = row & 31;
            const int L = d.slice_len[sl], base = d.slice_ptr[sl];
            const T *val = static_cast<const T *>(d.sell_val);
            int *col = const_cast<int *>(cc.col);
            T2 *kv2 = const_cast<T2 *>(cc.kv2);
            T *kv1 = const_cast<T *>(cc.kv1);
            for (int j = 0; j < min(cc.JC, L); j++) col[j * CG_THREADS + tid] = d.sell_col[base + 32 * j + lane];
            for (int j = 0; reg_nomass && j < min(cc.J, L); j++) {
                const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    T2 kp;
                    kp.x = val[vb + 32 * (2 * m)];
                    kp.y = val[vb + 32 * (2 * m + 1)];
                    kv2[(4 * j + m) * CG_THREADS + tid] = kp;
                }
                kv1[j * CG_THREADS + tid] = val[vb + 32 * 8];
            }
        }
    }
    // two-level preconditioner (REG and local only): per row the rest offset
    // d_p and smoother weight, the CTA's 6 rows of X ~ A_c^-1, the blob's
    // coarse residual g and this segment's coarse correction c
    const bool coarse = REG && local && d.coarse;
    // the same preconditioner in the memory-resident kernel (coarse_mem_step)
    const bool mcoarse = !REG && d.coarse;
    // memory-resident kernel in FP32: segment partials deferred (flush_partials)
    constexpr bool kDefer = !REG && sizeof(T) == 4;
    int dcnt = 0;  // deferred segments not yet flushed (CTA-uniform)
    auto defer_flush = [&]() {
        if constexpr (kDefer) {
            if (dcnt) {
                flush_partials(defer_view(), dcnt, reinterpret_cast<float *>(part()), d.part_stride);
                dcnt = 0;
            }
        }
    };
    int coarse_n = 0;  // coarse dofs of the CTA's blob (0: no coarse space)
    if (coarse) {
        const CoarseView cv = coarse_view<T>(d);
        const BlobParams &bp = d.bp[s_blob[0]];
        coarse_n = bp.coarse_n;
        cv.h[tid] = 0.f;
        cv.phi[tid] = reg_valid ? d.phi[s_row0[0] + tid] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float *Xg = d.coarse_X + bp.coarse_xoff + (size_t)(6 * (s_sid[0] - bp.seg_off)) * bp.coarse_n;
        for (int k = tid; k < 6 * bp.coarse_n; k += CG_THREADS) cv.xrow[k] = Xg[k];
    }
    // u = omega D^-1 r + Phi_p c of the thread's row (REG, coarse)
    auto coarse_u = [&](RowState<T> &S) {
        const CoarseView cv = coarse_view<T>(d);
        const float4 f = cv.phi[tid];
        const float *cvec = cv.cvec;
        const float cx = cvec[3], cy = cvec[4], cz = cvec[5];
        const T pc[3] = {(T)(cvec[0] + cy * f.z - cz * f.y), (T)(cvec[1] + cz * f.x - cx * f.z),
                         (T)(cvec[2] + cx * f.y - cy * f.x)};
#pragma unroll
        for (int k = 0; k < 3; k++) S.u[k] = (T)f.w * sdinv[k * CG_THREADS + tid] * S.r[k] + pc[k];
    };
    // Phi_p^T v = (v, d_p x v) into ex[0..5]
    auto restrict6 = [&](const T v[3], float *ex) {
        const float4 f = coarse_view<T>(d).phi[tid];
        const float v0 = (float)v[0], v1 = (float)v[1], v2 = (float)v[2];
        ex[0] = v0;
        ex[1] = v1;
        ex[2] = v2;
        ex[3] = f.y * v2 - f.z * v1;
        ex[4] = f.z * v0 - f.x * v2;
        ex[5] = f.x * v1 - f.y * v0;
    };
    auto row_info = [&](int j, int &row, bool &valid, T &diag, bool &nomass) {
        if (REG) {
            row = s_row0[0] + tid;
            valid = reg_valid;
            diag = reg_diag;
            nomass = reg_nomass;
        } else {
            row = row_of(j, valid);
            if (valid) diag = diag_of(j, row, nomass);
        }
    };
    // x and D^-1 of the thread's row (component k)
    auto xref = [&](RowState<T> &S, int k) -> T & { return REG ? sx[k * CG_THREADS + tid] : S.x[k]; };
    auto pref = [&](RowState<T> &S, int k) -> T & { return REG ? sx[(6 + k) * CG_THREADS + tid] : S.p[k]; };
    auto sref = [&](RowState<T> &S, int k) -> T & { return REG ? sx[(9 + k) * CG_THREADS + tid] : S.s[k]; };
    auto dinv_of = [&](const RowState<T> &S, int k) -> T { return REG ? sdinv[k * CG_THREADS + tid] : S.dinv[k]; };
    // REG: x of the own rows to global memory (for the FP64 true residual and
    // the Euler update; the memory-resident variant keeps it there)
    auto publish_x = [&]() {
        if (REG && reg_valid) {
            const size_t o = 3 * (size_t)(s_row0[0] + tid);
#pragma unroll
            for (int k = 0; k < 3; k++) X()[o + k] = sx[k * CG_THREADS + tid];
        }
    };
    // phase A of segment j: p = u + beta p; s = w + beta s; x += alpha p;
    // r -= alpha s; u = D^-1 r.  Partials: slot 0 r.u, slot 2 r.r.
    auto phase_a = [&](int j) {
        const int k = s_tslot[j];
        if (coarse && s_state[k] == CG_RESTART) {
            // restart from the true residual: u = M r, published for phase B
            if (reg_valid) {
                coarse_u(reg);
                U4()[s_row0[0] + tid] = V4{reg.u[0], reg.u[1], reg.u[2], (T)0};
            }
            return;
        }
        if (mcoarse && s_state[k] == CG_RESTART) {
            // the same from the row state in memory
            int row;
            bool valid, nomass = true;
            T diag = 0;
            row_info(j, row, valid, diag, nomass);
            if (valid) {
                RowState<T> loc;
                load_fields<T>(d, row, loc, RF_R | RF_DINV);
                coarse_u_of<T>(d.phi[row], coarse_mem_view(d).cvec + 8 * j, loc.dinv, loc.r, loc.u);
                store_fields<T>(d, row, loc, RF_U);
                U4()[row] = V4{loc.u[0], loc.u[1], loc.u[2], (T)0};
            }
            return;
        }
        if (s_state[k] != CG_ACTIVE) return;  // CTA-uniform
        int row;
        bool valid, nomass = true;
        T diag = 0;
        row_info(j, row, valid, diag, nomass);
        W pg = 0, pr = 0;
        RowState<T> loc;
        RowState<T> &S = REG ? reg : loc;
        if (!REG && valid) {
            // u of the last iteration from its published copy (the plain u
            // array is not kept up to date by the memory-resident iteration)
            load_fields<T>(d, row, loc, RF_X | RF_R | RF_W | RF_S | RF_P | RF_DINV);
            const V4 uo = U4()[row];
            loc.u[0] = uo.x;
            loc.u[1] = uo.y;
            loc.u[2] = uo.z;
        }
        float4 fm = make_float4(0.f, 0.f, 0.f, 0.f);  // mcoarse: the row's rest offset and omega
        if (mcoarse && valid) fm = d.phi[row];
        if (valid) {
            const T a = s_alpha[k], b = s_beta[k];
            const bool first = b == (T)0;
#pragma unroll
            for (int cc2 = 0; cc2 < 3; cc2++) {
                const T pn = first ? S.u[cc2] : S.u[cc2] + b * pref(S, cc2);
                const T sn = first ? S.w[cc2] : S.w[cc2] + b * sref(S, cc2);
                pref(S, cc2) = pn;
                sref(S, cc2) = sn;
                xref(S, cc2) += a * pn;
                S.r[cc2] -= a * sn;
                S.u[cc2] = dinv_of(S, cc2) * S.r[cc2];
            }
            if (coarse) coarse_u(S);
            else if (mcoarse) coarse_u_of<T>(fm, coarse_mem_view(d).cvec + 8 * j, S.dinv, S.r, S.u);
#pragma unroll
            for (int cc2 = 0; cc2 < 3; cc2++) {
                pg += S.r[cc2] * S.u[cc2];
                pr += S.r[cc2] * S.r[cc2];
            }
            U4()[row] = V4{S.u[0], S.u[1], S.u[2], (T)0};
        }
        if (!REG && valid) store_fields<T>(d, row, loc, RF_X | RF_R | RF_S | RF_P);
        if constexpr (kDefer) {
            const float inf[3] = {(float)pg, 0.f, (float)pr};
            if (mcoarse) {
                float ex[6] = {0, 0, 0, 0, 0, 0};
                if (valid) restrict6_of<T>(fm, S.r, ex);
                seg_partials_defer<6>(defer_view(), dcnt, s_sid[j], 5, 8, inf, ex);
            } else {
                seg_partials_defer<0>(defer_view(), dcnt, s_sid[j], 5, 0, inf, nullptr);
            }
            if (++dcnt == kDeferSegs) defer_flush();
            return;
        }
        const W in[3] = {pg, (W)0, pr};
        if (coarse) {
            // restriction of the new r: slot floats 8..
            float ex[6] = {0, 0, 0, 0, 0, 0};
            if (valid) restrict6(S.r, ex);
            seg_partials<W, 6>(slot(s_sid[j]), in, 5, ex, 8, red);
        } else if (mcoarse) {
            float ex[6] = {0, 0, 0, 0, 0, 0};
            if (valid) restrict6_of<T>(fm, S.r, ex);
            seg_partials<W, 6>(slot(s_sid[j]), in, 5, ex, 8, red);
        } else {
            seg_partials<W, 0>(slot(s_sid[j]), in, 5, nullptr, 0, red);
        }
    };
    // phase B of segment j: ACTIVE / RESTART and the prologue: w = A u, slot 1
    // w.u (the prologue and RESTART also fill slots 0 and 2); VERIFY: the
    // FP64 b - A x becomes the new residual, slot 0 r.u, slot 2 |b - A x|^2.
    auto phase_b = [&](int j, bool prologue) {
        const int k = s_tslot[j], state = s_state[k];
        if (!(state == CG_ACTIVE || state == CG_VERIFY || state == CG_RESTART)) return;  // CTA-uniform
        int row;
        bool valid, nomass = true;
        T diag = 0;
        row_info(j, row, valid, diag, nomass);
        W pg = 0, pd = 0, pr = 0;
        double vr = 0.0, vg = 0.0;
        RowState<T> loc;
        RowState<T> &S = REG ? reg : loc;
        // an ACTIVE iteration only needs w.u here (r.u and r.r came from
        // phase A); the prologue and a restart also sum r.u and r.r
        const bool need_r = prologue || state != CG_ACTIVE;
        if (!REG && valid) {
            if (need_r) load_fields<T>(d, row, loc, RF_R | (state == CG_VERIFY ? RF_DINV : 0));
            if (state != CG_VERIFY) {
                const V4 uo = U4()[row];  // the u the product reads (published in phase A)
                loc.u[0] = uo.x;
                loc.u[1] = uo.y;
                loc.u[2] = uo.z;
            }
        }
        if (valid) {
            if (state != CG_VERIFY) {
                T au[3];
                sell_row_cg<T, !REG>(d, row, nomass, diag, static_cast<const V4 *>(d.u4), au,
                                     REG ? cg_cache_view<T>(d) : CgCache<T>{});
#pragma unroll
                for (int cc2 = 0; cc2 < 3; cc2++) {
                    S.w[cc2] = au[cc2];
                    pd += au[cc2] * S.u[cc2];
                }
                if (REG || need_r) {
#pragma unroll
                    for (int cc2 = 0; cc2 < 3; cc2++) {
                        pg += S.r[cc2] * S.u[cc2];
                        pr += S.r[cc2] * S.r[cc2];
                    }
                }
            } else {
                double rt[3];
                true_residual_row<T>(d, row, nomass, (double)diag, X(), rt);
#pragma unroll
                for (int cc2 = 0; cc2 < 3; cc2++) {
                    S.r[cc2] = (T)rt[cc2];
                    S.u[cc2] = dinv_of(S, cc2) * S.r[cc2];
                    vr += rt[cc2] * rt[cc2];
                    vg += (double)S.r[cc2] * (double)S.u[cc2];
                }
                U4()[row] = V4{S.u[0], S.u[1], S.u[2], (T)0};
            }
        }
        if (!REG && valid) store_fields<T>(d, row, loc, state == CG_VERIFY ? (RF_R | RF_U) : RF_W);
        if constexpr (kDefer) {
            if (!prologue && state == CG_ACTIVE) {
                const float inf[3] = {(float)pg, (float)pd, (float)pr};
                if (mcoarse) {
                    float ex[6] = {0, 0, 0, 0, 0, 0};
                    if (valid) restrict6_of<T>(d.phi[row], S.w, ex);
                    seg_partials_defer<6>(defer_view(), dcnt, s_sid[j], 2, 14, inf, ex);
                } else {
                    seg_partials_defer<0>(defer_view(), dcnt, s_sid[j], 2, 0, inf, nullptr);
                }
                if (++dcnt == kDeferSegs) defer_flush();
                return;
            }
        }
        if (mcoarse) {
            // the restrictions of the register-resident branch below, with
            // the rest offset from memory
            const float4 fm = valid ? d.phi[row] : make_float4(0.f, 0.f, 0.f, 0.f);
            float ex[12];
#pragma unroll
            for (int m = 0; m < 12; m++) ex[m] = 0.f;
            const bool full = prologue || state != CG_ACTIVE;
            if (valid) {
                if (full) restrict6_of<T>(fm, S.r, ex);
                if (state != CG_VERIFY) restrict6_of<T>(fm, S.w, ex + 6);
            }
            if (state == CG_VERIFY) {
                const double in[3] = {vg, 0.0, vr};
                seg_partials<double, 12>(slot(s_sid[j]), in, 5, ex, 8, red);
            } else if (full) {
                const W in[3] = {pg, pd, pr};
                seg_partials<W, 12>(slot(s_sid[j]), in, 7, ex, 8, red);
            } else {
                const W in[3] = {pg, pd, pr};
                seg_partials<W, 6>(slot(s_sid[j]), in, 2, ex + 6, 14, red);
            }
        } else if (coarse) {
            // restrictions: ACTIVE P^T w (slot floats 14..); the prologue,
            // RESTART and VERIFY restart the coarse recurrence: P^T r (8..)
            // and P^T w (14.., zero for VERIFY)
            float ex[12];
#pragma unroll
            for (int m = 0; m < 12; m++) ex[m] = 0.f;
            const bool full = prologue || state != CG_ACTIVE;
            if (valid) {
                if (full) restrict6(S.r, ex);
                if (state != CG_VERIFY) restrict6(S.w, ex + 6);
            }
            if (state == CG_VERIFY) {
                const double in[3] = {vg, 0.0, vr};
                seg_partials<double, 12>(slot(s_sid[j]), in, 5, ex, 8, red);
            } else if (full) {
                const W in[3] = {pg, pd, pr};
                seg_partials<W, 12>(slot(s_sid[j]), in, 7, ex, 8, red);
            } else {
                const W in[3] = {pg, pd, pr};
                seg_partials<W, 6>(slot(s_sid[j]), in, 2, ex + 6, 14, red);
            }
        } else if (state == CG_VERIFY) {
            const double in[3] = {vg, 0.0, vr};
            seg_partials<double, 0>(slot(s_sid[j]), in, 5, nullptr, 0, red);
        } else {
            const W in[3] = {pg, pd, pr};
            seg_partials<W, 0>(slot(s_sid[j]), in, (prologue || state == CG_RESTART) ? 7 : 2, nullptr, 0, red);
        }
    };

    unsigned int n_bar = 0;  // counting barriers passed
    // sums of the iteration's partials and the transitions; the running-blob count
    auto reduce = [&]() -> unsigned int {
        if (!local) return reducing_barrier(d, mcoarse ? part() : d.partials, &s_err, &s_pub, s_last, sm_df);
        counting_barrier(d.bar, (++n_bar) * (unsigned int)G, &s_err);
        if (s_err) return 0u;
        return local_reduce<T>(d, part(), s_cg, sm_df, &s_run, nb, s_blob, s_state, s_alpha, s_beta,
                               coarse_n);
    };
    if (coarse) {
        // u_0 = M r_0 needs P^T r_0 of every segment of the blob: restrict
        // into the second partials buffer, sum after a barrier, solve
        parity = 1;
        {
            float ex[6] = {0, 0, 0, 0, 0, 0};
            if (reg_valid) restrict6(reg.r, ex);
            const W none[3] = {(W)0, (W)0, (W)0};
            seg_partials<W, 6>(slot(s_sid[0]), none, 0, ex, 8, red);
        }
        counting_barrier(d.bar, (++n_bar) * (unsigned int)G, &s_err);
        if (!s_err) {
            const BlobParams &bp = d.bp[s_blob[0]];
            coarse_apply<T>(d, coarse_n, tid < coarse_n ? __ldcg(slot(bp.seg_off + tid / 6) + 8 + tid % 6) : 0.f);
            if (reg_valid) coarse_u(reg);
        }
        parity = 0;
    }
    if (mcoarse) {
        // the same with the row state in memory: P^T r_0 of every segment,
        // then c per segment and u_0 = M r_0 stored for the publication below
        parity = 1;
        for (int j = 0; j < nt; j++) {
            int row;
            bool valid, nomass = true;
            T diag = 0;
            row_info(j, row, valid, diag, nomass);
            float ex[6] = {0, 0, 0, 0, 0, 0};
            if (valid) {
                RowState<T> loc;
                load_fields<T>(d, row, loc, RF_R);
                restrict6_of<T>(d.phi[row], loc.r, ex);
            }
            const W none[3] = {(W)0, (W)0, (W)0};
            seg_partials<W, 6>(slot(s_sid[j]), none, 0, ex, 8, red);
        }
        counting_barrier(d.bar, (++n_bar) * (unsigned int)G, &s_err);
        if (!s_err) {
            coarse_mem_step<T>(d, reinterpret_cast<const float *>(part()), s_sid, nt, nb, s_blob, s_tslot, s_state,
                               s_alpha, s_beta, true);
            for (int j = 0; j < nt; j++) {
                int row;
                bool valid, nomass = true;
                T diag = 0;
                row_info(j, row, valid, diag, nomass);
                if (valid) {
                    RowState<T> loc;
                    load_fields<T>(d, row, loc, RF_R | RF_DINV);
                    coarse_u_of<T>(d.phi[row], coarse_mem_view(d).cvec + 8 * j, loc.dinv, loc.r, loc.u);
                    store_fields<T>(d, row, loc, RF_U);
                }
            }
        }
        parity = 0;
    }
    // publish u of the own rows for the neighbours (the k_nodes start value,
    // zero on pinned rows; with the coarse space u_0 = M r_0) before the
    // first product
    for (int j = 0; j < nt; j++) {
        const int row = s_row0[j] + tid;
        if (tid < s_rows[j]) {
            if (coarse) {
                U4()[row] = reg_valid ? V4{reg.u[0], reg.u[1], reg.u[2], (T)0} : V4{(T)0, (T)0, (T)0, (T)0};
            } else {
                const T *u = static_cast<const T *>(d.u) + 3 * (size_t)row;
                U4()[row] = V4{u[0], u[1], u[2], (T)0};
            }
        }
    }
    counting_barrier(d.bar, (++n_bar) * (unsigned int)G, &s_err);
    if (!s_err)
        for (int j = 0; j < nt; j++) phase_b(j, true);
    defer_flush();  // (the prologue defers nothing: a no-op)
    unsigned int running = s_err ? 0u : reduce();
    int loops = 0;
    while (!s_err && running > 0) {
        if (!local) refresh();  // the local reduction refreshed already
        // memory-resident coarse space: the corrections for this update, from
        // the partials just reduced (before the buffers swap)
        if (mcoarse)
            coarse_mem_step<T>(d, reinterpret_cast<const float *>(part()), s_sid, nt, nb, s_blob, s_tslot, s_state,
                               s_alpha, s_beta, false);
        if (local || mcoarse) parity ^= 1;
        if (REG && s_state[0] == CG_VERIFY) publish_x();
        for (int j = 0; j < nt; j++) phase_a(j);
        defer_flush();
        counting_barrier(d.bar, (++n_bar) * (unsigned int)G, &s_err);
        if (s_err) break;
        for (int j = 0; j < nt; j++) phase_b(j, false);
        defer_flush();
        loops++;
        running = reduce();
    }
    publish_x();
    if (d.cg_euler && !s_err) {
        // the step's Euler update (Blob::euler_integrate, src/Blob.cpp:3937-3969)
        // of the own rows, for blobs that had not failed before the solve and
        // whose solve converged (this CTA's copy of their state), and the
        // advance of every RNG stream by one step's draws (CTA 0)
        if (!local) refresh();
        for (int j = 0; j < nt; j++) {
            const int k = s_tslot[j], b = s_blob[k];
            const BlobParams &bp = d.bp[b];
            const int row = s_row0[j] + tid;
            if (tid >= s_rows[j] || row - bp.node_off >= bp.node_cnt) continue;
            if (s_state[k] != CG_CONVERGED || __ldcg(&d.status[b]) != 0) continue;
            const double dt = bp.dt;
#pragma unroll
            for (int cc2 = 0; cc2 < 3; cc2++) {
                const size_t kk = 3 * (size_t)row + cc2;
                const double xi = REG ? (double)sx[cc2 * CG_THREADS + tid] : (double)X()[kk];
                double pn;
                if (bp.solver == SOLVER_NOMASS) {
                    d.vel[kk] = xi;
                    pn = d.pos[kk] + xi * dt;
                } else {
                    const double v = d.vel[kk] + xi * dt;
                    d.vel[kk] = v;
                    pn = d.pos[kk] + v * dt;
                }
                d.pos[kk] = pn;
                if (d.pos_df) d.pos_df[kk] = split_pos(pn);
            }
        }
        if (c == 0) {
            __syncthreads();  // this CTA's status bits of the solve are visible to its threads
            for (int st = tid; st < d.num_streams; st += CG_THREADS) {
                if (d.num_streams == d.num_blobs && __ldcg(&d.status[st]) != 0) continue;  // per-blob streams
                uint32_t w[6];
#pragma unroll
                for (int i = 0; i < 6; i++) w[i] = d.stream_state[6 * st + i];
                mrg::apply(d.stream_step[st], w);
#pragma unroll
                for (int i = 0; i < 6; i++) d.stream_state[6 * st + i] = w[i];
            }
        }
    }
    if (local && c == 0)
        for (int b = tid; b < d.num_blobs; b += CG_THREADS) d.cg[b] = s_cg[b];
    if (tid == 0) {
        if (s_err)
            for (int k = 0; k < nb; k++) atomicOr(&d.status[s_blob[k]], BLOB_FAIL_CG | BLOB_FAIL_TIMEOUT);
        if (c == 0) *d.loop_count += (unsigned long long)loops;
    }
}

// Self-test of the grid barrier's time-out: every CTA arrives, but the target
// is one arrival more than the grid, so no wait can end; each waiter gives up
// after spin_limit sleeps, raises the time-out flag and returns.  out[0] =
// number of CTAs that reported the time-out.
__global__ void k_barrier_timeout_selftest(unsigned int *bar, unsigned int spin_limit, int *out)
{
    __shared__ int s_err;
    if (threadIdx.x == 0) s_err = 0;
    counting_barrier(bar, gridDim.x + 1, &s_err, spin_limit);
    if (threadIdx.x == 0 && s_err) atomicAdd(out, 1);
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
    if (valid && bp.solver == SOLVER_LUMPED) {
        // M in with the lumped masses (MassLumpedSolver::apply_matrix,
        // src/MassLumpedSolver.cpp:93-97, scales its result array in place by
        // the masses; this is the product it stands for)
        for (int i = 0; i < 3; i++) acc[i] = in[3 * (size_t)row + i] / d.lumped_inv[row];
    } else if (valid) {
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
        if (bp.solver != SOLVER_NOMASS) {
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

static_assert(MEAS_TILE == ELEM_TILE, "measurement kernels run element and node tiles in one grid");

// Element mass vol_0 rho (src/Blob.cpp:3797).
template <typename T>
__device__ __forceinline__ double element_mass(const DeviceBatch &d, int e)
{
    return (double)static_cast<const T *>(d.vol0)[e] * d.mats[d.mat_id[e]].rho;
}

// Sums of Blob::make_measurements over tiles, FP64.  Element tiles (blocks
// [0, n_etiles)) add Blob::get_CoM's terms, (m_e p_0 + p_1 + p_2 + p_3) / 4 --
// the element mass multiplies the first corner only, as the reference's
// parenthesisation has it (src/Blob.cpp:951-967); node tiles add the
// centroid over all N_t nodes and the squared displacement from the
// positions at creation (src/Blob.cpp:1488-1524, remTrans off).  A node of no
// element never moves and counts at its creation position.  The last block
// reduces each blob's tiles in a fixed order.
template <typename T>
__global__ void __launch_bounds__(ELEM_TILE) k_meas_sums(DeviceBatch d, MeasView m)
{
    __shared__ double red[4 * 32];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    const int t = blockIdx.x;
    if (t < d.n_etiles) {
        const BlobParams &bp = d.bp[d.etile_blob[t]];
        const int le = t * ELEM_TILE - bp.elem_off + threadIdx.x;
        if (le < bp.elem_cnt) {
            const int e = bp.elem_off + le;
            const int4 c = reinterpret_cast<const int4 *>(d.conn)[e];
            const double mass = element_mass<T>(d, e);
            for (int k = 0; k < 3; k++)
                v[k] = (mass * d.pos[3 * (size_t)c.x + k] + d.pos[3 * (size_t)c.y + k] + d.pos[3 * (size_t)c.z + k] +
                        d.pos[3 * (size_t)c.w + k]) / 4;
        }
    } else {
        const int nt = t - d.n_etiles;
        const int b = m.tile_blob[nt];
        const int64_t i0 = m.io_off[b], n = m.io_off[b + 1] - i0;
        const int64_t li = (int64_t)(nt - m.tile_first[b]) * MEAS_TILE + threadIdx.x;
        if (li < n) {
            const int64_t i = i0 + li;
            const int2 s = m.io_src[i];
            for (int k = 0; k < 3; k++) {
                const double p0 = m.pos0[3 * i + k];
                double p = p0;
                if (s.x >= 0 && s.y < 0)
                    p = d.pos[3 * (size_t)s.x + k];
                else if (s.x >= 0)
                    p = .5 * (d.pos[3 * (size_t)s.x + k] + d.pos[3 * (size_t)s.y + k]);
                v[k] = p;
                v[3] += (p - p0) * (p - p0);
            }
        }
    }
    double sum[4];
    block_sum<4, double>(v, sum, red);
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; k++) m.partials[4 * (size_t)t + k] = sum[k];
    if (last_block(&d.counters[CNT_MEAS], gridDim.x)) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            const BlobParams &bp = d.bp[bb];
            const int e0 = bp.elem_off / ELEM_TILE, ec = bp.elem_pad / ELEM_TILE;
            const int n0 = d.n_etiles + m.tile_first[bb], nc = m.tile_first[bb + 1] - m.tile_first[bb];
            double com[3] = {0.0, 0.0, 0.0}, cog[4] = {0.0, 0.0, 0.0, 0.0};
            for (int q = lane; q < ec; q += 32)
                for (int k = 0; k < 3; k++) com[k] += __ldcg(&m.partials[4 * (size_t)(e0 + q) + k]);
            for (int q = lane; q < nc; q += 32)
                for (int k = 0; k < 4; k++) cog[k] += __ldcg(&m.partials[4 * (size_t)(n0 + q) + k]);
            for (int k = 0; k < 3; k++) com[k] = warp_sum<double>(com[k]);
            for (int k = 0; k < 4; k++) cog[k] = warp_sum<double>(cog[k]);
            if (lane == 0) {
                const double nn = (double)(m.io_off[bb + 1] - m.io_off[bb]);
                double *o = m.out + MEAS_VALUES * (size_t)bb;
                for (int k = 0; k < 3; k++) o[k] = cog[k] / nn;
                o[3] = sqrt(cog[3] / nn);
                for (int k = 0; k < 3; k++) o[4 + k] = bp.elem_cnt ? com[k] / bp.elem_cnt : 0.0;
            }
        }
        if (threadIdx.x == 0) d.counters[CNT_MEAS] = 0;
    }
}

// Angular momentum about the centre of mass, sum over elements of
// m_e sum_ij MM_ij (r_j x v_i) with MM the linear element's mass matrix / m_e
// (0.1 diagonal, 0.05 off it); zero for CG_nomass (src/Blob.cpp:1434-1484).
template <typename T>
__global__ void __launch_bounds__(ELEM_TILE) k_meas_angmom(DeviceBatch d, MeasView m)
{
    __shared__ double red[3 * 32];
    const int t = blockIdx.x;
    const int b = d.etile_blob[t];
    const BlobParams &bp = d.bp[b];
    const int le = t * ELEM_TILE - bp.elem_off + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if (bp.solver != SOLVER_NOMASS && le < bp.elem_cnt) {
        const int e = bp.elem_off + le;
        const int4 c = reinterpret_cast<const int4 *>(d.conn)[e];
        const int cn[4] = {c.x, c.y, c.z, c.w};
        const double *com = m.out + MEAS_VALUES * (size_t)b + 4;
        double r[4][3], u[4][3];
        for (int i = 0; i < 4; i++)
            for (int k = 0; k < 3; k++) {
                r[i][k] = d.pos[3 * (size_t)cn[i] + k] - com[k];
                u[i][k] = d.vel[3 * (size_t)cn[i] + k];
            }
        double l[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                const double mm = i == j ? .1 : .05;
                l[0] += mm * (r[j][1] * u[i][2] - r[j][2] * u[i][1]);
                l[1] += mm * (r[j][2] * u[i][0] - r[j][0] * u[i][2]);
                l[2] += mm * (r[j][0] * u[i][1] - r[j][1] * u[i][0]);
            }
        const double mass = element_mass<T>(d, e);
        for (int k = 0; k < 3; k++) v[k] = mass * l[k];
    }
    double sum[3];
    block_sum<3, double>(v, sum, red);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++) m.partials[4 * (size_t)t + k] = sum[k];
    if (last_block(&d.counters[CNT_ANGMOM], gridDim.x)) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int bb = warp; bb < d.num_blobs; bb += nw) {
            const int e0 = d.bp[bb].elem_off / ELEM_TILE, ec = d.bp[bb].elem_pad / ELEM_TILE;
            double l[3] = {0.0, 0.0, 0.0};
            for (int q = lane; q < ec; q += 32)
                for (int k = 0; k < 3; k++) l[k] += __ldcg(&m.partials[4 * (size_t)(e0 + q) + k]);
            for (int k = 0; k < 3; k++) l[k] = warp_sum<double>(l[k]);
            if (lane == 0)
                for (int k = 0; k < 3; k++) m.out[MEAS_VALUES * (size_t)bb + 7 + k] = l[k];
        }
        if (threadIdx.x == 0) d.counters[CNT_ANGMOM] = 0;
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

void launch_lumped_mass(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_lumped_mass, blocks_for(d.nl_pad, 256), 256, s, d);
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

void launch_noise(const DeviceBatch &d, cudaStream_t s)
{
    if (d.noise_runs == 0) return;
    PREC_DISPATCH(d, k_noise, blocks_for(d.noise_runs, NOISE_THREADS), NOISE_THREADS, s, d);
}

void launch_nodes(const DeviceBatch &d, cudaStream_t s, int use_given_rhs)
{
    PREC_DISPATCH(d, k_nodes, d.n_tiles, NODE_TILE * NODE_LANES, s, d, use_given_rhs);
}

template <typename T>
static int cg_smem_plan_t(int max_slots, int max_cols, size_t extra_bytes, int *J, int *JC, size_t *dyn_bytes)
{
    int dev = 0, optin = 0;
    *J = *JC = 0;
    *dyn_bytes = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k_cg<T, true>) != cudaSuccess) return -1;
    const size_t reserve = 1024;  // per-CTA system use
    const size_t state = 12 * (size_t)CG_THREADS * sizeof(T);  // x, D^-1, p and s
    const size_t fixed = fa.sharedSizeBytes + reserve + state + extra_bytes;
    if ((size_t)optin < fixed) return -1;
    size_t room = optin - fixed;
    const size_t per_col = (size_t)CG_THREADS * sizeof(int), per_slot = (size_t)CG_THREADS * 9 * sizeof(T);
    *JC = (int)std::min<size_t>(room / per_col, (size_t)std::max(0, max_cols));
    room -= (size_t)*JC * per_col;
    *J = (int)std::min<size_t>(room / per_slot, (size_t)std::max(0, std::min(max_slots, *JC)));
    *dyn_bytes = state + (size_t)*JC * per_col + (size_t)*J * per_slot + extra_bytes;
    // the limit is a property of the kernel, shared by every handle: set it
    // to the device maximum so that no handle's plan lowers another's
    if (cudaFuncSetAttribute(k_cg<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - (int)fa.sharedSizeBytes) != cudaSuccess)
        return -1;
    return 0;
}

int cg_smem_plan(int precision, int max_slots, int max_cols, size_t extra_bytes, int *J, int *JC, size_t *dyn_bytes)
{
    return precision == PREC_FP64 ? cg_smem_plan_t<double>(max_slots, max_cols, extra_bytes, J, JC, dyn_bytes)
                                  : cg_smem_plan_t<float>(max_slots, max_cols, extra_bytes, J, JC, dyn_bytes);
}

// Dynamic shared memory of the memory-resident CG kernel with the coarse
// space (coarse_mem_view): its size for the given coarse dimensions, and
// whether the device allows it (the kernel's limit is raised to the device
// maximum, as for the register-resident kernel).
size_t cg_mem_defer_bytes(int precision) { return precision == PREC_FP64 ? 0 : kDeferBytes; }

size_t cg_mem_coarse_bytes(int coarse_hmax)
{
    // c per segment, reduction floats, blob offsets, then g and P^T s of the CTA's blobs
    return sizeof(float) * (8 * (size_t)CG_MAX_SEGS + 8 * 32 + (size_t)CG_MAX_SEGS + 2 * (size_t)coarse_hmax);
}

int cg_mem_smem_allow(int precision, size_t dyn_bytes)
{
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    cudaFuncAttributes fa;
    const void *fn = precision == PREC_FP64 ? (const void *)k_cg<double, false> : (const void *)k_cg<float, false>;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return -1;
    const size_t reserve = 1024;
    if (fa.sharedSizeBytes + reserve + dyn_bytes > (size_t)optin) return -1;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes) !=
        cudaSuccess)
        return -1;
    return 0;
}

int cg_max_grid(int precision, int reg, size_t dyn_bytes)
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    cudaError_t e;
    if (precision == PREC_FP64)
        e = reg ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<double, true>, CG_THREADS, dyn_bytes)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<double, false>, CG_THREADS, dyn_bytes);
    else
        e = reg ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<float, true>, CG_THREADS, dyn_bytes)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<float, false>, CG_THREADS, dyn_bytes);
    if (e != cudaSuccess) return 0;
    return sms * per_sm;
}

cudaError_t launch_barrier_timeout_selftest(unsigned int *bar, unsigned int spin_limit, int *out, int ctas,
                                            cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(32);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FFEA_LAUNCHED();
    return cudaLaunchKernelEx(&cfg, k_barrier_timeout_selftest, bar, spin_limit, out);
}

cudaError_t launch_cg(const DeviceBatch &dev, cudaStream_t s, bool euler)
{
    DeviceBatch d = dev;
    d.cg_euler = euler ? 1 : 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)d.cg_grid);
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = (size_t)d.cg_dyn_smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    FFEA_LAUNCHED();
    if (d.precision == PREC_FP64)
        return d.cg_reg ? cudaLaunchKernelEx(&cfg, k_cg<double, true>, d) : cudaLaunchKernelEx(&cfg, k_cg<double, false>, d);
    return d.cg_reg ? cudaLaunchKernelEx(&cfg, k_cg<float, true>, d) : cudaLaunchKernelEx(&cfg, k_cg<float, false>, d);
}

void launch_energies(const DeviceBatch &d, cudaStream_t s)
{
    PREC_DISPATCH(d, k_energies, d.n_etiles, ELEM_TILE, s, d);
}

void launch_measurements(const DeviceBatch &d, const MeasView &m, cudaStream_t s)
{
    PREC_DISPATCH(d, k_meas_sums, d.n_etiles + m.n_tiles, ELEM_TILE, s, d, m);
    PREC_DISPATCH(d, k_meas_angmom, d.n_etiles, ELEM_TILE, s, d, m);
}

template <typename T>
static void spmv_variant_dispatch(const DeviceBatch &d, cudaStream_t s, int variant)
{
    const T *v = static_cast<const T *>(d.u);
    T *o = static_cast<T *>(d.w);
    const int64_t rows = d.nl_pad;
    switch (variant) {
    case 0: k_spmv_variant<T, 1, true><<<blocks_for(rows, 256), 256, 0, s>>>(d, v, o); break;
    case 1: k_spmv_variant<T, 1, false><<<blocks_for(rows, 256), 256, 0, s>>>(d, v, o); break;
    case 2: k_spmv_variant<T, 2, false><<<blocks_for(rows * 2, 256), 256, 0, s>>>(d, v, o); break;
    default: k_spmv_variant<T, 4, false><<<blocks_for(rows * 4, 256), 256, 0, s>>>(d, v, o); break;
    }
    FFEA_LAUNCHED();
}

void launch_spmv_variant(const DeviceBatch &d, cudaStream_t s, int variant)
{
    if (d.precision == PREC_FP64) spmv_variant_dispatch<double>(d, s, variant);
    else spmv_variant_dispatch<float>(d, s, variant);
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
