// learned.cu -- the learned part of the two-level preconditioner: a mesh
// message-passing network that sets the per-node weight omega_p of the
// Jacobi term of M = diag(omega) D^-1 + P A_c^-1 P^T, its training gradient,
// and the loss it is trained on.
//
// Network (FP32 weights, BF16 stored activations, FP32 accumulation):
//   h0_p = features of row p (8, see k_features)
//   h(l+1)_p = ReLU(Ws_l h(l)_p + Wn_l mean_{q ~ p} h(l)_q + b_l),  l = 0, 1, 2,
//              hidden width 32, q ~ p the rows sharing a mesh edge with p
//   omega_p = 2 sigmoid(wo . h3_p + bo)  in (0, 2)
// Loss of one (rhs f, solution x) pair of the NoMass solve, on the matrix A
// and coarse inverse X of that solve: the A-norm error of the best multiple
// of one preconditioner application z = M f (one preconditioned steepest-
// descent step), relative to |x|_A:
//   L = min_tau |x - tau z|_A^2 / |x|_A^2 = 1 - (f.z)^2 / ((z.Az)(x.f)),
// invariant to the scale of M, as CG is (x.f = x.Ax).  With a = f.z,
// b = z.Az, c = x.f: dL/dz = (2a/(bc)) ((a/b) Az - f), and z_p depends on
// omega_p through omega_p (D^-1 f)_p, so dL/d omega_p = k1 (Az.v)_p - k2
// (f.v)_p with v = D^-1 f, k1 = 2a^2/(b^2 c), k2 = 2a/(bc); then the network
// backward.
// Every sum over rows is a fixed-order reduction (per-CTA partials, then a
// CTA-ordered sum): results do not depend on scheduling.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "kernels.h"

namespace ffea {

namespace {

constexpr int kHid = MPNN_HIDDEN, kFin = MPNN_FEATURES;
constexpr int kFwdThreads = 128;   // rows per CTA of the forward kernels
constexpr int kBwdThreads = 64;    // rows per CTA of the backward kernels

struct MpnnLayout {
    int ws[3], wn[3], b[3], wo, bo, total;
};

__host__ __device__ constexpr MpnnLayout mpnn_layout()
{
    MpnnLayout L{};
    int off = 0;
    for (int l = 0; l < 3; l++) {
        const int din = l == 0 ? kFin : kHid;
        L.ws[l] = off;
        off += kHid * din;
        L.wn[l] = off;
        off += kHid * din;
        L.b[l] = off;
        off += kHid;
    }
    L.wo = off;
    off += kHid;
    L.bo = off;
    off += 1;
    L.total = off;
    return L;
}
static_assert(mpnn_layout().total == MPNN_NUM_PARAMS, "parameter count");

__device__ __forceinline__ bool free_nomass_row(const DeviceBatch &d, int row, int &blob)
{
    if (row >= d.nl_pad) return false;
    blob = d.seg_of_row[row] >= 0 ? d.seg_blob[d.seg_of_row[row]] : -1;
    if (blob < 0) return false;
    const BlobParams &bp = d.bp[blob];
    return bp.solver == SOLVER_NOMASS && !(d.flags[row] & NODE_PINNED);
}

template <typename T>
__device__ __forceinline__ void load_K(const DeviceBatch &d, int base, int j, int lane, float K[9])
{
    const T *val = static_cast<const T *>(d.sell_val);
    const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
#pragma unroll
    for (int k = 0; k < 9; k++) K[k] = (float)val[vb + 32 * k];
}

// Eight scale-free features of row p from the current matrix and the coarse
// layout: drag / stiffness, neighbours in other segments, distance from the
// segment centroid, degree, off-diagonal weight, pinned neighbours,
// anisotropy of the diagonal block, and a constant.
template <typename T>
__global__ void __launch_bounds__(kFwdThreads) k_features(DeviceBatch d, float *x0)
{
    const int row = blockIdx.x * kFwdThreads + threadIdx.x;
    if (row >= d.nl_pad) return;
    float f[kFin] = {0, 0, 0, 0, 0, 0, 0, 0};
    int b;
    if (free_nomass_row(d, row, b)) {
        const BlobParams &bp = d.bp[b];
        const int sl = row >> 5, lane = row & 31;
        const int L = d.slice_len[sl], base = d.slice_ptr[sl];
        const int seg = d.seg_of_row[row];
        float S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, off = 0.f;
        int deg = 0, other = 0, pinned = 0;
        for (int j = 0; j < L; j++) {
            const int q = d.sell_col[base + 32 * j + lane];
            if (q == row) continue;
            float K[9];
            load_K<T>(d, base, j, lane, K);
            float n2 = 0.f;
#pragma unroll
            for (int m = 0; m < 9; m++) {
                S[m] -= K[m];
                n2 += K[m] * K[m];
            }
            off += sqrtf(n2);
            deg++;
            other += d.seg_of_row[q] != seg;
            pinned += (d.flags[q] & NODE_PINNED) != 0;
        }
        const float z = bp.calc_stokes == 1 ? (float)d.drag[row] : 0.f;
        S[0] += z;
        S[4] += z;
        S[8] += z;
        const float tr = fmaxf((S[0] + S[4] + S[8]) / 3.f, 1e-30f);
        const float4 ph = d.phi[row];
        const float od = sqrtf(S[1] * S[1] + S[2] * S[2] + S[3] * S[3] + S[5] * S[5] + S[6] * S[6] + S[7] * S[7]);
        const float inv = deg > 0 ? 1.f / deg : 0.f;
        f[0] = z / tr;
        f[1] = other * inv;
        f[2] = sqrtf(ph.x * ph.x + ph.y * ph.y + ph.z * ph.z);
        f[3] = deg / 16.f;
        f[4] = off / (3.f * tr);
        f[5] = pinned * inv;
        f[6] = od / tr;
        f[7] = 1.f;
    }
#pragma unroll
    for (int k = 0; k < kFin; k++) x0[(size_t)row * kFin + k] = f[k];
}

template <int DIN, bool BF>
__device__ __forceinline__ void load_act(const void *h, int row, float out[DIN])
{
    if (BF) {
        const __nv_bfloat162 *p = reinterpret_cast<const __nv_bfloat162 *>(h) + (size_t)row * (DIN / 2);
#pragma unroll
        for (int k = 0; k < DIN / 2; k++) {
            const float2 v = __bfloat1622float2(p[k]);
            out[2 * k] = v.x;
            out[2 * k + 1] = v.y;
        }
    } else {
        const float *p = reinterpret_cast<const float *>(h) + (size_t)row * DIN;
#pragma unroll
        for (int k = 0; k < DIN; k++) out[k] = p[k];
    }
}

// mean of the neighbours' activations (rows sharing a mesh edge; SELL padding
// slots hold the row itself and are skipped); returns the degree
template <int DIN, bool BF>
__device__ __forceinline__ int neighbour_mean(const DeviceBatch &d, const void *h, int row, float m[DIN])
{
#pragma unroll
    for (int k = 0; k < DIN; k++) m[k] = 0.f;
    const int sl = row >> 5, lane = row & 31;
    const int L = d.slice_len[sl], base = d.slice_ptr[sl];
    int deg = 0;
    for (int j = 0; j < L; j++) {
        const int q = d.sell_col[base + 32 * j + lane];
        if (q == row) continue;
        float v[DIN];
        load_act<DIN, BF>(h, q, v);
#pragma unroll
        for (int k = 0; k < DIN; k++) m[k] += v[k];
        deg++;
    }
    const float inv = deg > 0 ? 1.f / deg : 0.f;
#pragma unroll
    for (int k = 0; k < DIN; k++) m[k] *= inv;
    return deg;
}

// one message-passing layer: out = bf16(ReLU(Ws h + Wn mean(h_nbr) + b))
template <int DIN, bool BF>
__global__ void __launch_bounds__(kFwdThreads) k_layer(DeviceBatch d, const float *theta, int ws, int wn, int bo,
                                                       const void *hin, __nv_bfloat16 *hout)
{
    __shared__ float sWs[kHid * DIN], sWn[kHid * DIN], sb[kHid];
    for (int k = threadIdx.x; k < kHid * DIN; k += kFwdThreads) {
        sWs[k] = theta[ws + k];
        sWn[k] = theta[wn + k];
    }
    if (threadIdx.x < kHid) sb[threadIdx.x] = theta[bo + threadIdx.x];
    __syncthreads();
    const int row = blockIdx.x * kFwdThreads + threadIdx.x;
    if (row >= d.nl_pad) return;
    float h[DIN], m[DIN];
    load_act<DIN, BF>(hin, row, h);
    neighbour_mean<DIN, BF>(d, hin, row, m);
    __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(hout) + (size_t)row * (kHid / 2);
#pragma unroll 4
    for (int i = 0; i < kHid; i += 2) {
        float a0 = sb[i], a1 = sb[i + 1];
#pragma unroll
        for (int k = 0; k < DIN; k++) {
            a0 = fmaf(sWs[i * DIN + k], h[k], fmaf(sWn[i * DIN + k], m[k], a0));
            a1 = fmaf(sWs[(i + 1) * DIN + k], h[k], fmaf(sWn[(i + 1) * DIN + k], m[k], a1));
        }
        o[i / 2] = __floats2bfloat162_rn(fmaxf(a0, 0.f), fmaxf(a1, 0.f));
    }
}

// omega = 2 sigmoid(wo . h3 + bo); written to the smoother weight of free
// NoMass rows (other rows keep weight 1)
__global__ void __launch_bounds__(kFwdThreads) k_output(DeviceBatch d, const float *theta, const __nv_bfloat16 *h3,
                                                        float *omega, int write_phi)
{
    constexpr MpnnLayout L = mpnn_layout();
    const int row = blockIdx.x * kFwdThreads + threadIdx.x;
    if (row >= d.nl_pad) return;
    int b;
    if (!free_nomass_row(d, row, b)) {
        omega[row] = 1.f;
        return;
    }
    float h[kHid];
    load_act<kHid, true>(h3, row, h);
    float s = theta[L.bo];
#pragma unroll
    for (int i = 0; i < kHid; i++) s = fmaf(theta[L.wo + i], h[i], s);
    const float w = 2.f / (1.f + expf(-s));
    omega[row] = w;
    if (write_phi) d.phi[row].w = w;
}

// ---------------------------------------------------------------- loss
// P^T f per segment (one CTA of CG_SEG_MAX_ROWS threads per segment) and
// v = D^-1 f per row
template <typename T>
__global__ void __launch_bounds__(CG_SEG_MAX_ROWS) k_loss_restrict(DeviceBatch d, float4 *v, float *gvec)
{
    __shared__ float red[6][32];
    const int s = blockIdx.x, t = threadIdx.x;
    const int b = d.seg_blob[s];
    const BlobParams &bp = d.bp[b];
    const int row = d.seg_row0[s] + t;
    float ex[6] = {0, 0, 0, 0, 0, 0};
    if (t < d.seg_rows[s]) {
        float4 vv = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!(d.flags[row] & NODE_PINNED) && bp.solver == SOLVER_NOMASS) {
            const float f0 = (float)d.rhs[3 * (size_t)row], f1 = (float)d.rhs[3 * (size_t)row + 1],
                        f2 = (float)d.rhs[3 * (size_t)row + 2];
            const T *di = static_cast<const T *>(d.dinv) + 3 * (size_t)row;
            vv = make_float4((float)di[0] * f0, (float)di[1] * f1, (float)di[2] * f2, 0.f);
            const float4 ph = d.phi[row];
            ex[0] = f0;
            ex[1] = f1;
            ex[2] = f2;
            ex[3] = ph.y * f2 - ph.z * f1;
            ex[4] = ph.z * f0 - ph.x * f2;
            ex[5] = ph.x * f1 - ph.y * f0;
        }
        v[row] = vv;
    }
    const int lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int l = 0; l < 6; l++) {
        float x = ex[l];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[l][warp] = x;
    }
    __syncthreads();
    if (t < 6) {
        float x = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) x += red[t][w];
        gvec[bp.coarse_off + 6 * (s - bp.seg_off) + t] = x;
    }
}

// c = X g per blob (thread per coarse row)
__global__ void k_loss_coarse(DeviceBatch d, const float *gvec, float *cvec)
{
    const int b = blockIdx.y;
    const BlobParams &bp = d.bp[b];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (bp.solver != SOLVER_NOMASS || i >= bp.coarse_n) return;
    const float *X = d.coarse_X + bp.coarse_xoff + (size_t)i * bp.coarse_n;
    const float *g = gvec + bp.coarse_off;
    float a = 0.f;
    for (int j = 0; j < bp.coarse_n; j++) a = fmaf(X[j], g[j], a);
    cvec[bp.coarse_off + i] = a;
}

// z = M f = omega v + Phi_p c per row
__global__ void __launch_bounds__(kFwdThreads) k_loss_apply(DeviceBatch d, const float4 *v, const float *omega,
                                                            const float *cvec, float4 *z)
{
    const int row = blockIdx.x * kFwdThreads + threadIdx.x;
    if (row >= d.nl_pad) return;
    int b;
    float4 zv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (free_nomass_row(d, row, b)) {
        const BlobParams &bp = d.bp[b];
        const int s = d.seg_of_row[row];
        const float *c = cvec + bp.coarse_off + 6 * (s - bp.seg_off);
        const float4 ph = d.phi[row], vv = v[row];
        const float w = omega[row];
        zv.x = w * vv.x + c[0] + c[4] * ph.z - c[5] * ph.y;
        zv.y = w * vv.y + c[1] + c[5] * ph.x - c[3] * ph.z;
        zv.z = w * vv.z + c[2] + c[3] * ph.y - c[4] * ph.x;
    }
    z[row] = zv;
}

// A z per row (difference form); per row (Az.v, f.v) for the omega
// gradient; per CTA the sums f.z, z.Az, x.f
template <typename T>
__global__ void __launch_bounds__(kFwdThreads) k_loss_products(DeviceBatch d, const float4 *z, const float4 *v,
                                                               float2 *gw, double *cta_sums)
{
    __shared__ double red[3][kFwdThreads / 32];
    const int row = blockIdx.x * kFwdThreads + threadIdx.x;
    double fz = 0.0, zaz = 0.0, xf = 0.0;
    int b;
    if (free_nomass_row(d, row, b)) {
        const BlobParams &bp = d.bp[b];
        const int sl = row >> 5, lane = row & 31;
        const int L = d.slice_len[sl], base = d.slice_ptr[sl];
        const float4 zp = z[row];
        const float zeta = bp.calc_stokes == 1 ? (float)d.drag[row] : 0.f;
        float a0 = zeta * zp.x, a1 = zeta * zp.y, a2 = zeta * zp.z;
        for (int j = 0; j < L; j++) {
            const int q = d.sell_col[base + 32 * j + lane];
            if (q == row) continue;
            float K[9];
            load_K<T>(d, base, j, lane, K);
            const float4 zq = z[q];
            const float d0 = zq.x - zp.x, d1 = zq.y - zp.y, d2 = zq.z - zp.z;
            a0 += K[0] * d0 + K[1] * d1 + K[2] * d2;
            a1 += K[3] * d0 + K[4] * d1 + K[5] * d2;
            a2 += K[6] * d0 + K[7] * d1 + K[8] * d2;
        }
        const float4 vv = v[row];
        const double f0 = d.rhs[3 * (size_t)row], f1 = d.rhs[3 * (size_t)row + 1], f2 = d.rhs[3 * (size_t)row + 2];
        gw[row] = make_float2(a0 * vv.x + a1 * vv.y + a2 * vv.z, (float)(f0 * vv.x + f1 * vv.y + f2 * vv.z));
        fz = f0 * zp.x + f1 * zp.y + f2 * zp.z;
        zaz = (double)zp.x * a0 + (double)zp.y * a1 + (double)zp.z * a2;
        const T *x = static_cast<const T *>(d.x) + 3 * (size_t)row;
        xf = (double)x[0] * f0 + (double)x[1] * f1 + (double)x[2] * f2;
    } else if (row < d.nl_pad) {
        gw[row] = make_float2(0.f, 0.f);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
        zaz += __shfl_xor_sync(0xffffffffu, zaz, o);
        xf += __shfl_xor_sync(0xffffffffu, xf, o);
    }
    if (lane == 0) {
        red[0][warp] = fz;
        red[1][warp] = zaz;
        red[2][warp] = xf;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int w = 0; w < kFwdThreads / 32; w++) s += red[threadIdx.x][w];
        cta_sums[3 * blockIdx.x + threadIdx.x] = s;
    }
}

// a = f.z, b = z.Az, c = x.f summed over the CTAs in order; scal = (loss,
// k1, k2) with loss = 1 - a^2/(bc), k1 = 2a^2/(b^2 c), k2 = 2a/(bc)
__global__ void k_loss_total(const double *cta_sums, int n, double *scal)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = 0; i < n; i++) {
        a += cta_sums[3 * i];
        b += cta_sums[3 * i + 1];
        c += cta_sums[3 * i + 2];
    }
    const bool ok = b > 0.0 && c > 0.0;
    scal[0] = ok ? 1.0 - a * a / (b * c) : 0.0;
    scal[1] = ok ? 2.0 * a * a / (b * b * c) : 0.0;
    scal[2] = ok ? 2.0 * a / (b * c) : 0.0;
}

// ---------------------------------------------------------------- backward
// dL/d omega = k1 gw.x - k2 gw.y; dL/ds = dL/d omega * omega (1 - omega / 2);
// dH3 = dL/ds wo; per-CTA partials of dwo (32) and dbo (1) at
// partial[cta * MPNN_NUM_PARAMS + L.wo ..]
__global__ void __launch_bounds__(kBwdThreads) k_out_bwd(DeviceBatch d, const float *theta, const __nv_bfloat16 *h3,
                                                         const float *omega, const float2 *gw, const double *scal,
                                                         float *dh, float *partial)
{
    constexpr MpnnLayout L = mpnn_layout();
    __shared__ float sds[kBwdThreads], sh[kBwdThreads][kHid + 1];
    const int row = blockIdx.x * kBwdThreads + threadIdx.x;
    float ds = 0.f;
    float h[kHid];
#pragma unroll
    for (int i = 0; i < kHid; i++) h[i] = 0.f;
    if (row < d.nl_pad) {
        const float w = omega[row];
        const float2 g = gw[row];
        ds = ((float)scal[1] * g.x - (float)scal[2] * g.y) * w * (1.f - 0.5f * w);
        load_act<kHid, true>(h3, row, h);
#pragma unroll
        for (int i = 0; i < kHid; i++) dh[(size_t)row * kHid + i] = ds * theta[L.wo + i];
    }
    sds[threadIdx.x] = ds;
#pragma unroll
    for (int i = 0; i < kHid; i++) sh[threadIdx.x][i] = h[i];
    __syncthreads();
    float *P = partial + (size_t)blockIdx.x * MPNN_NUM_PARAMS;
    if (threadIdx.x < kHid) {
        float a = 0.f;
        for (int r = 0; r < kBwdThreads; r++) a = fmaf(sds[r], sh[r][threadIdx.x], a);
        P[L.wo + threadIdx.x] = a;
    } else if (threadIdx.x == kHid) {
        float a = 0.f;
        for (int r = 0; r < kBwdThreads; r++) a += sds[r];
        P[L.bo] = a;
    }
}

// backward of layer l: da = dh_out * (h_out > 0); dWs, dWn, db per-CTA
// partials; self part of dh_in (Ws^T da) and t = Wn^T da / deg for the
// neighbour gather
template <int DIN, bool BF>
__global__ void __launch_bounds__(kBwdThreads) k_layer_bwd(DeviceBatch d, const float *theta, int ws, int wn, int bo,
                                                           const void *hin, const __nv_bfloat16 *hout,
                                                           const float *dh_out, float *dh_in_self, float *tbuf,
                                                           float *partial)
{
    __shared__ float sda[kBwdThreads][kHid + 1], shin[kBwdThreads][DIN + 1], sm[kBwdThreads][DIN + 1];
    const int row = blockIdx.x * kBwdThreads + threadIdx.x;
    float da[kHid], h[DIN], m[DIN];
#pragma unroll
    for (int i = 0; i < kHid; i++) da[i] = 0.f;
#pragma unroll
    for (int k = 0; k < DIN; k++) h[k] = m[k] = 0.f;
    if (row < d.nl_pad) {
        float ho[kHid];
        load_act<kHid, true>(hout, row, ho);
#pragma unroll
        for (int i = 0; i < kHid; i++) da[i] = ho[i] > 0.f ? dh_out[(size_t)row * kHid + i] : 0.f;
        load_act<DIN, BF>(hin, row, h);
        const int deg = neighbour_mean<DIN, BF>(d, hin, row, m);
        const float inv = deg > 0 ? 1.f / deg : 0.f;
        if (dh_in_self) {
#pragma unroll
            for (int k = 0; k < DIN; k++) {
                float a = 0.f, t = 0.f;
#pragma unroll
                for (int i = 0; i < kHid; i++) {
                    a = fmaf(theta[ws + i * DIN + k], da[i], a);
                    t = fmaf(theta[wn + i * DIN + k], da[i], t);
                }
                dh_in_self[(size_t)row * DIN + k] = a;
                tbuf[(size_t)row * DIN + k] = t * inv;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < kHid; i++) sda[threadIdx.x][i] = da[i];
#pragma unroll
    for (int k = 0; k < DIN; k++) {
        shin[threadIdx.x][k] = h[k];
        sm[threadIdx.x][k] = m[k];
    }
    __syncthreads();
    float *P = partial + (size_t)blockIdx.x * MPNN_NUM_PARAMS;
    for (int e = threadIdx.x; e < 2 * kHid * DIN + kHid; e += kBwdThreads) {
        float a = 0.f;
        if (e < kHid * DIN) {
            const int i = e / DIN, k = e % DIN;
            for (int r = 0; r < kBwdThreads; r++) a = fmaf(sda[r][i], shin[r][k], a);
            P[ws + e] = a;
        } else if (e < 2 * kHid * DIN) {
            const int i = (e - kHid * DIN) / DIN, k = (e - kHid * DIN) % DIN;
            for (int r = 0; r < kBwdThreads; r++) a = fmaf(sda[r][i], sm[r][k], a);
            P[wn + (e - kHid * DIN)] = a;
        } else {
            const int i = e - 2 * kHid * DIN;
            for (int r = 0; r < kBwdThreads; r++) a += sda[r][i];
            P[bo + i] = a;
        }
    }
}

// dh_in[q] = self part + sum over neighbours p of t[p] (the mean's adjoint;
// the edge graph is symmetric)
template <int DIN>
__global__ void __launch_bounds__(kFwdThreads) k_gather_bwd(DeviceBatch d, const float *self_part, const float *tbuf,
                                                            float *dh_in)
{
    const int row = blockIdx.x * kFwdThreads + threadIdx.x;
    if (row >= d.nl_pad) return;
    float a[DIN];
#pragma unroll
    for (int k = 0; k < DIN; k++) a[k] = self_part[(size_t)row * DIN + k];
    const int sl = row >> 5, lane = row & 31;
    const int L = d.slice_len[sl], base = d.slice_ptr[sl];
    for (int j = 0; j < L; j++) {
        const int q = d.sell_col[base + 32 * j + lane];
        if (q == row) continue;
#pragma unroll
        for (int k = 0; k < DIN; k++) a[k] += tbuf[(size_t)q * DIN + k];
    }
#pragma unroll
    for (int k = 0; k < DIN; k++) dh_in[(size_t)row * DIN + k] = a[k];
}

// grad[e] = sum over CTAs of partial[cta][e] (parameter e), in CTA order
__global__ void k_sum_partials(const float *partial, int nctas, int lo, int hi, float *grad)
{
    const int e = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= hi) return;
    float a = 0.f;
    for (int c = 0; c < nctas; c++) a += partial[(size_t)c * MPNN_NUM_PARAMS + e];
    grad[e] = a;
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

}  // namespace

int mpnn_forward(const DeviceBatch &d, MpnnBuffers &B, const float *theta_dev, bool write_phi, cudaStream_t s)
{
    constexpr MpnnLayout L = mpnn_layout();
    const int nf = cdiv(d.nl_pad, kFwdThreads);
    if (d.precision == PREC_FP64)
        k_features<double><<<nf, kFwdThreads, 0, s>>>(d, B.x0);
    else
        k_features<float><<<nf, kFwdThreads, 0, s>>>(d, B.x0);
    k_layer<kFin, false><<<nf, kFwdThreads, 0, s>>>(d, theta_dev, L.ws[0], L.wn[0], L.b[0], B.x0, B.h[0]);
    k_layer<kHid, true><<<nf, kFwdThreads, 0, s>>>(d, theta_dev, L.ws[1], L.wn[1], L.b[1], B.h[0], B.h[1]);
    k_layer<kHid, true><<<nf, kFwdThreads, 0, s>>>(d, theta_dev, L.ws[2], L.wn[2], L.b[2], B.h[1], B.h[2]);
    k_output<<<nf, kFwdThreads, 0, s>>>(d, theta_dev, B.h[2], B.omega, write_phi ? 1 : 0);
    count_launches(5);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int mpnn_loss(const DeviceBatch &d, MpnnBuffers &B, cudaStream_t s)
{
    const int nf = cdiv(d.nl_pad, kFwdThreads);
    int nmax = 0;
    if (d.precision == PREC_FP64) {
        k_loss_restrict<double><<<d.n_segs, CG_SEG_MAX_ROWS, 0, s>>>(d, B.v, B.gvec);
    } else {
        k_loss_restrict<float><<<d.n_segs, CG_SEG_MAX_ROWS, 0, s>>>(d, B.v, B.gvec);
    }
    nmax = d.coarse_nmax;
    k_loss_coarse<<<dim3(cdiv(nmax, 128), d.num_blobs), 128, 0, s>>>(d, B.gvec, B.cvec);
    k_loss_apply<<<nf, kFwdThreads, 0, s>>>(d, B.v, B.omega, B.cvec, B.e);
    if (d.precision == PREC_FP64)
        k_loss_products<double><<<nf, kFwdThreads, 0, s>>>(d, B.e, B.v, B.gw, B.cta_sums);
    else
        k_loss_products<float><<<nf, kFwdThreads, 0, s>>>(d, B.e, B.v, B.gw, B.cta_sums);
    k_loss_total<<<1, 32, 0, s>>>(B.cta_sums, nf, B.scal);
    count_launches(6);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int mpnn_backward(const DeviceBatch &d, MpnnBuffers &B, const float *theta_dev, float *grad_dev, cudaStream_t s)
{
    constexpr MpnnLayout L = mpnn_layout();
    const int nb = cdiv(d.nl_pad, kBwdThreads), nf = cdiv(d.nl_pad, kFwdThreads);
    k_out_bwd<<<nb, kBwdThreads, 0, s>>>(d, theta_dev, B.h[2], B.omega, B.gw, B.scal, B.dh, B.partial);
    // layer 2: dh (32) -> dh_in for h[1]
    k_layer_bwd<kHid, true><<<nb, kBwdThreads, 0, s>>>(d, theta_dev, L.ws[2], L.wn[2], L.b[2], B.h[1], B.h[2], B.dh,
                                                        B.dself, B.tbuf, B.partial);
    k_gather_bwd<kHid><<<nf, kFwdThreads, 0, s>>>(d, B.dself, B.tbuf, B.dh2);
    k_layer_bwd<kHid, true><<<nb, kBwdThreads, 0, s>>>(d, theta_dev, L.ws[1], L.wn[1], L.b[1], B.h[0], B.h[1], B.dh2,
                                                        B.dself, B.tbuf, B.partial);
    k_gather_bwd<kHid><<<nf, kFwdThreads, 0, s>>>(d, B.dself, B.tbuf, B.dh);
    k_layer_bwd<kFin, false><<<nb, kBwdThreads, 0, s>>>(d, theta_dev, L.ws[0], L.wn[0], L.b[0], B.x0, B.h[0], B.dh,
                                                         nullptr, nullptr, B.partial);
    k_sum_partials<<<cdiv(MPNN_NUM_PARAMS, 128), 128, 0, s>>>(B.partial, nb, 0, MPNN_NUM_PARAMS, grad_dev);
    count_launches(7);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace ffea
