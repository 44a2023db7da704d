// coarse.cu -- the coarse space of the two-level CG preconditioner.
//
// Every CG segment (a compact block of one blob's rows, one per CTA of the
// persistent solve) is an aggregate with six rigid modes: the translations
// e_i and the rotations e_i x d_p, d_p = (x_p - c_s) / R_s the rest offset of
// row p from the segment centroid.  Phi_p (3 x 6) holds them, so that
// Phi_p^T v = (v, d_p x v) and Phi_p c = c_t + c_r x d_p.  The preconditioner
// is M = diag(omega) D^-1 + P A_c^-1 P^T with A_c = P^T A P, the coarse
// matrix of each blob (6 x segments square, dense).
//
//   k_coarse_assemble  A_c blocks (s, t) for the segments t coupled to s,
//   k_coarse_sum       at every refresh (the matrix changes with the mesh):
//                      partial blocks per quarter of a segment's rows, then
//                      their sum in a fixed order
//   coarse_refresh     X ~ A_c^-1 by Newton-Schulz, X <- 2X - X A_c X (two
//                      FP32 GEMMs, k_sgemm below) from the previous step's
//                      X; `init` starts from X = I / ||A_c||_inf and
//                      iterates to convergence; for the memory-resident
//                      CG kernel, then the FP16 copy it reads (k_coarse_half)
//
// The matrix enters in the same difference form as the solver's SpMV:
// (A v)_p = sum_q K_pq (v_q - v_p) + zeta_p v_p over the free rows.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "kernels.h"

namespace ffea {

namespace {

constexpr int kAsmThreads = 256;
constexpr int kAsmParts = CG_SEG_MAX_ROWS / kAsmThreads;  // CTAs per segment, one row per thread

// C (6 x 6, row-major) += Phi_p^T K Phi_q for rest offsets dp, dq.
__device__ __forceinline__ void add_block(float C[36], const float dp[3], const float K[9], const float dq[3])
{
#pragma unroll
    for (int m = 0; m < 6; m++) {
        // column m of Phi_q
        float c0, c1, c2;
        if (m < 3) {
            c0 = m == 0;
            c1 = m == 1;
            c2 = m == 2;
        } else if (m == 3) {  // e_x x d
            c0 = 0.f;
            c1 = -dq[2];
            c2 = dq[1];
        } else if (m == 4) {  // e_y x d
            c0 = dq[2];
            c1 = 0.f;
            c2 = -dq[0];
        } else {  // e_z x d
            c0 = -dq[1];
            c1 = dq[0];
            c2 = 0.f;
        }
        const float v0 = K[0] * c0 + K[1] * c1 + K[2] * c2;
        const float v1 = K[3] * c0 + K[4] * c1 + K[5] * c2;
        const float v2 = K[6] * c0 + K[7] * c1 + K[8] * c2;
        C[0 * 6 + m] += v0;
        C[1 * 6 + m] += v1;
        C[2 * 6 + m] += v2;
        C[3 * 6 + m] += dp[1] * v2 - dp[2] * v1;
        C[4 * 6 + m] += dp[2] * v0 - dp[0] * v2;
        C[5 * 6 + m] += dp[0] * v1 - dp[1] * v0;
    }
}

template <typename T>
__device__ __forceinline__ void load_K(const DeviceBatch &d, int base, int j, int lane, float K[9])
{
    const T *val = static_cast<const T *>(d.sell_val);
    const size_t vb = (size_t)(base + 32 * j) * 9 + lane;
#pragma unroll
    for (int k = 0; k < 9; k++) K[k] = (float)val[vb + 32 * k];
}

// Sums of 32 values per lane over a warp by a transposed butterfly (16 + 8
// + 4 + 2 + 1 shuffles): at each offset a lane keeps half of its values and
// adds its partner's copy of that half.  Lane l returns the warp total of
// value l (a fixed order per value: deterministic).
__device__ __forceinline__ float warp_sum32_transposed(float (&v)[36])
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool upper = (lane & h) != 0;
#pragma unroll
        for (int i = 0; i < h; i++) {
            const float send = upper ? v[i] : v[i + h];
            const float keep = upper ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    return v[0];
}

// Partial coarse blocks: CTA (s, part) of a NoMass blob's segment s takes
// rows part * 256 .. part * 256 + 255 of the segment, one row per thread.  A
// row's slots are sorted by column and segments are contiguous row ranges,
// so the slots of each coupled segment t form one run: a cursor per row walks
// them once over the targets.  Each (s, t) block of the CTA's rows is a
// fixed-order block reduction, written to part slot (k, part) of the
// segment's neighbour entry k; k_coarse_sum adds the parts in order.
template <typename T>
__global__ void __launch_bounds__(kAsmThreads) k_coarse_assemble(DeviceBatch d)
{
    const int s = blockIdx.x, part = blockIdx.y;
    const int b = d.seg_blob[s];
    const BlobParams &bp = d.bp[b];
    if (bp.solver != SOLVER_NOMASS) return;  // CTA-uniform
    const int r0 = d.seg_row0[s], nrows = d.seg_rows[s];
    const int lane32 = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ float red[36][kAsmThreads / 32];

    const int rr = part * kAsmThreads + threadIdx.x;
    const int p = r0 + rr;
    const bool active = rr < nrows && !(d.flags[p] & NODE_PINNED);
    float dp[3] = {0.f, 0.f, 0.f};
    int L = 0, base = 0;
    const int lane = p & 31;
    if (active) {
        const float4 fp = d.phi[p];
        dp[0] = fp.x;
        dp[1] = fp.y;
        dp[2] = fp.z;
        L = d.slice_len[p >> 5];
        base = d.slice_ptr[p >> 5];
    }
    int j = 0;
    for (int k = d.seg_nbr_ptr[s]; k < d.seg_nbr_ptr[s + 1]; k++) {
        const int t = d.seg_nbr[k];
        float C[36];
#pragma unroll
        for (int i = 0; i < 36; i++) C[i] = 0.f;
        if (active) {
            float K[9];
            if (t == s) {
                // diagonal of A in difference form: zeta_p I - sum_q K_pq
                float S[9];
#pragma unroll
                for (int m = 0; m < 9; m++) S[m] = 0.f;
                for (int jj = 0; jj < L; jj++) {
                    load_K<T>(d, base, jj, lane, K);
#pragma unroll
                    for (int m = 0; m < 9; m++) S[m] -= K[m];
                }
                const float z = bp.calc_stokes == 1 ? (float)d.drag[p] : 0.f;
                S[0] += z;
                S[4] += z;
                S[8] += z;
                add_block(C, dp, S, dp);
            }
            while (j < L) {
                const int q = d.sell_col[base + 32 * j + lane];
                const int tq = d.seg_of_row[q];
                if (tq > t) break;
                if (tq == t && q != p && !(d.flags[q] & NODE_PINNED)) {
                    load_K<T>(d, base, j, lane, K);
                    const float4 fq = d.phi[q];
                    const float dq[3] = {fq.x, fq.y, fq.z};
                    add_block(C, dp, K, dq);
                }
                j++;
            }
        }
        // fixed-order block reduction of the 36 entries: 32 by the transposed
        // butterfly, 4 by plain butterflies, then the warps in order
        float tail[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float v = C[32 + i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            tail[i] = v;
        }
        red[lane32][warp] = warp_sum32_transposed(C);
        if (lane32 < 4) red[32 + lane32][warp] = tail[lane32];
        __syncthreads();
        if (threadIdx.x < 36) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < kAsmThreads / 32; w++) v += red[threadIdx.x][w];
            d.coarse_asm[((size_t)k * kAsmParts + part) * 36 + threadIdx.x] = v;
        }
        __syncthreads();
    }
}

// A_c block (s, t) of every neighbour entry k of segment s: the sum of the
// kAsmParts partial blocks in part order.
__global__ void k_coarse_sum(DeviceBatch d)
{
    const int s = blockIdx.x;
    const int b = d.seg_blob[s];
    const BlobParams &bp = d.bp[b];
    if (bp.solver != SOLVER_NOMASS) return;
    const int nc = bp.coarse_n, ls = s - bp.seg_off;
    float *Ac = d.coarse_A + bp.coarse_xoff;
    const int k0 = d.seg_nbr_ptr[s], nk = d.seg_nbr_ptr[s + 1] - k0;
    for (int x = threadIdx.x; x < 36 * nk; x += blockDim.x) {
        const int k = k0 + x / 36, i = x % 36;
        float v = 0.f;
#pragma unroll
        for (int pt = 0; pt < kAsmParts; pt++) v += d.coarse_asm[((size_t)k * kAsmParts + pt) * 36 + i];
        const int li = i / 6, mi = i % 6, lt = d.seg_nbr[k] - bp.seg_off;
        Ac[(size_t)(6 * ls + li) * nc + (6 * lt + mi)] = v;
    }
}

// X <- (X + X^T) / 2 over n x n matrices, one per blockIdx.z, n^2 apart
// (src may alias nothing).
__global__ void k_symmetrize(const float *__restrict__ src, float *__restrict__ dst, int n)
{
    const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= n) return;
    const size_t o = (size_t)blockIdx.z * n * n;
    dst[o + (size_t)i * n + j] = 0.5f * (src[o + (size_t)i * n + j] + src[o + (size_t)j * n + i]);
}

// The scale of coarse dof i: sqrt(X_ii), 1 where that is not a positive
// finite number.
__device__ __forceinline__ float coarse_scale(float xii)
{
    return (xii > 0.f && xii < INFINITY) ? sqrtf(xii) : 1.f;
}

// Xh = S^-1 X S^-1 rounded to FP16 (unit diagonal, |entries| about 1 at most
// for an SPD X) with rows padded with zeros to nh halves, and s = diag(S);
// one n x n matrix per blockIdx.z (X n^2 apart, Xh n nh apart, s n apart).
// S Xh S is symmetric like X, and its entries keep FP16's relative precision
// whatever the magnitude of X.
__global__ void k_coarse_half(const float *__restrict__ X, __half *__restrict__ Xh, float *__restrict__ sv, int n,
                              int nh)
{
    const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || j >= nh) return;
    X += (size_t)blockIdx.z * n * n;
    Xh += (size_t)blockIdx.z * n * nh;
    const float si = coarse_scale(X[(size_t)i * n + i]);
    if (j == 0) sv[(size_t)blockIdx.z * n + i] = si;
    float v = 0.f;
    if (j < n) v = X[(size_t)i * n + j] / (si * coarse_scale(X[(size_t)j * n + j]));
    Xh[(size_t)i * nh + j] = __float2half_rn(v);
}

// X = I / ||A||_inf (the Newton-Schulz start, convergent for an SPD A), one
// n x n matrix per CTA, n^2 apart.
__global__ void k_scaled_identity(const float *__restrict__ A, float *__restrict__ X, int n)
{
    A += (size_t)blockIdx.x * n * n;
    X += (size_t)blockIdx.x * n * n;
    __shared__ float red[32];
    float m = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float r = 0.f;
        for (int j = 0; j < n; j++) r += fabsf(A[(size_t)i * n + j]);
        m = fmaxf(m, r);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float mm = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) mm = fmaxf(mm, red[w]);
        red[0] = mm > 0.f ? 1.f / mm : 1.f;
    }
    __syncthreads();
    const float a = red[0];
    for (size_t k = threadIdx.x; k < (size_t)n * n; k += blockDim.x) X[k] = (k / n == k % n) ? a : 0.f;
}

// C = alpha A B + beta D over n x n row-major matrices, one product per
// blockIdx.z (matrices n^2 apart; D may be null when beta = 0, and C may
// alias D).  A BM x BN tile of C per CTA of 256 threads, each thread a
// (BM/16) x (BN/16) register block split in two halves of rows and columns
// (so its shared-memory reads are float4 or float2 and conflict-free); K in steps of
// 16 through double-buffered shared memory, the next step's tile loaded into
// registers while the current one is multiplied.  Every C entry is a
// sequential FMA chain over k: deterministic.
//
// Split-K (splits > 1): blockIdx.z = product * splits + split; the CTA sums
// k over its chunk [split * kchunk, (split + 1) * kchunk) only and writes the
// raw partial tile to part (one n x n block per z); k_splitk_sum then adds
// the splits in order and applies alpha, beta and D.
template <int BM>
__global__ void __launch_bounds__(256, 2) k_sgemm(const float *__restrict__ A, const float *__restrict__ B,
                                               const float *D, float *C, int n, float alpha, float beta,
                                               int splits, int kchunk, float *__restrict__ part)
{
    constexpr int BK = 16, TM = BM / 16, H = TM / 2, LA = BM / 16, LB = BM / 16;
    constexpr int PAD = 4;
    __shared__ __align__(16) float As[2][BK][BM + PAD];
    __shared__ __align__(16) float Bs[2][BK][BM + PAD];
    const int prod = blockIdx.z / splits, sp = blockIdx.z % splits;
    const size_t off = (size_t)prod * n * n;
    A += off;
    B += off;
    C += off;
    if (D) D += off;
    const int kbeg = sp * kchunk, kend = min(n, kbeg + kchunk);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BM;
    float acc[TM][TM];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TM; j++) acc[i][j] = 0.f;
    float ra[LA], rb[LB];
    // A tile (BM x BK): element r at row tid/16 + 16 r, column tid%16;
    // B tile (BK x BM): row tid/BM + (256/BM) r, column tid%BM
    auto load = [&](int k0) {
#pragma unroll
        for (int r = 0; r < LA; r++) {
            const int row = i0 + (tid >> 4) + 16 * r, col = k0 + (tid & 15);
            ra[r] = (row < n && col < kend) ? A[(size_t)row * n + col] : 0.f;
        }
#pragma unroll
        for (int r = 0; r < LB; r++) {
            const int row = k0 + tid / BM + (256 / BM) * r, col = j0 + tid % BM;
            rb[r] = (row < kend && col < n) ? B[(size_t)row * n + col] : 0.f;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int r = 0; r < LA; r++) As[buf][tid & 15][(tid >> 4) + 16 * r] = ra[r];
#pragma unroll
        for (int r = 0; r < LB; r++) Bs[buf][tid / BM + (256 / BM) * r][tid % BM] = rb[r];
    };
    const int nk = (kend - kbeg + BK - 1) / BK;
    load(kbeg);
    store(0);
    __syncthreads();
    for (int kt = 0; kt < nk; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < nk) load(kbeg + (kt + 1) * BK);
#pragma unroll
        for (int k = 0; k < BK; k++) {
            float a[TM], b[TM];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float *pa = &As[buf][k][h * (BM / 2) + ty * H];
                const float *pb = &Bs[buf][k][h * (BM / 2) + tx * H];
                if constexpr (H % 4 == 0) {
#pragma unroll
                    for (int q = 0; q < H; q += 4) {
                        const float4 va = *reinterpret_cast<const float4 *>(pa + q);
                        const float4 vb = *reinterpret_cast<const float4 *>(pb + q);
                        a[h * H + q] = va.x;
                        a[h * H + q + 1] = va.y;
                        a[h * H + q + 2] = va.z;
                        a[h * H + q + 3] = va.w;
                        b[h * H + q] = vb.x;
                        b[h * H + q + 1] = vb.y;
                        b[h * H + q + 2] = vb.z;
                        b[h * H + q + 3] = vb.w;
                    }
                } else {
                    static_assert(H % 2 == 0, "register block halves must be even");
#pragma unroll
                    for (int q = 0; q < H; q += 2) {
                        const float2 va = *reinterpret_cast<const float2 *>(pa + q);
                        const float2 vb = *reinterpret_cast<const float2 *>(pb + q);
                        a[h * H + q] = va.x;
                        a[h * H + q + 1] = va.y;
                        b[h * H + q] = vb.x;
                        b[h * H + q + 1] = vb.y;
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TM; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (kt + 1 < nk) {
            store(buf ^ 1);
            __syncthreads();
        }
    }
#pragma unroll
    for (int i = 0; i < TM; i++) {
        const int row = i0 + (i / H) * (BM / 2) + ty * H + (i % H);
        if (row >= n) continue;
#pragma unroll
        for (int j = 0; j < TM; j++) {
            const int col = j0 + (j / H) * (BM / 2) + tx * H + (j % H);
            if (col >= n) continue;
            const size_t o = (size_t)row * n + col;
            if (splits > 1) {
                part[(size_t)blockIdx.z * n * n + o] = acc[i][j];
                continue;
            }
            float v = alpha * acc[i][j];
            if (beta != 0.f) v += beta * D[o];
            C[o] = v;
        }
    }
}

// The split-K epilogue: C = alpha (sum of the splits, in split order) + beta D.
__global__ void k_splitk_sum(const float *__restrict__ part, const float *D, float *C, int n, int splits,
                             float alpha, float beta)
{
    const size_t nn = (size_t)n * n;
    const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nn) return;
    const size_t prod = blockIdx.y;
    const float *p = part + prod * splits * nn + o;
    float acc = 0.f;
    for (int sp = 0; sp < splits; sp++) acc += p[(size_t)sp * nn];
    float v = alpha * acc;
    if (beta != 0.f) v += beta * D[prod * nn + o];
    C[prod * nn + o] = v;
}

}  // namespace

int sgemm_sms()
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

// K splits of a batched product: 1 when its 128 x 128 tiles fill the GPU,
// else enough to give about two tiles per SM (chunks of at least 128 k).
int sgemm_splits(int n, int batch)
{
    const long long tiles = (long long)((n + 127) / 128) * ((n + 127) / 128) * batch;
    const int sms = sgemm_sms();
    if (tiles >= sms || n < 256) return 1;
    const int want = (int)((2LL * sms + tiles - 1) / tiles);
    return std::max(1, std::min(want, n / 128));
}

// One batched product on stream s.  128 x 128 tiles when they fill the GPU
// or, for larger matrices, with the K dimension split (`part` then holds
// sgemm_splits(n, batch) n x n floats per product); 64 x 64 tiles for
// small matrices.
void sgemm_batched(const float *A, const float *B, const float *D, float *C, int n, int batch, float alpha, float beta,
                   float *part, cudaStream_t s)
{
    const long long tiles = (long long)((n + 127) / 128) * ((n + 127) / 128) * batch;
    const int splits = part ? sgemm_splits(n, batch) : 1;
    if (splits > 1) {
        const int kchunk = ((n + splits - 1) / splits + 15) / 16 * 16;
        dim3 grid((n + 127) / 128, (n + 127) / 128, batch * splits);
        k_sgemm<128><<<grid, 256, 0, s>>>(A, B, D, C, n, alpha, beta, splits, kchunk, part);
        const size_t nn = (size_t)n * n;
        dim3 g2((unsigned)((nn + 255) / 256), batch);
        k_splitk_sum<<<g2, 256, 0, s>>>(part, D, C, n, splits, alpha, beta);
        count_launches(2);
        return;
    }
    if (tiles >= sgemm_sms() || n >= 256) {
        dim3 grid((n + 127) / 128, (n + 127) / 128, batch);
        k_sgemm<128><<<grid, 256, 0, s>>>(A, B, D, C, n, alpha, beta, 1, n, nullptr);
    } else {
        dim3 grid((n + 63) / 64, (n + 63) / 64, batch);
        k_sgemm<64><<<grid, 256, 0, s>>>(A, B, D, C, n, alpha, beta, 1, n, nullptr);
    }
    count_launches(1);
}

void launch_coarse_assemble(const DeviceBatch &d, cudaStream_t s)
{
    if (!d.coarse || d.n_segs == 0) return;
    const dim3 grid(d.n_segs, kAsmParts);
    if (d.precision == PREC_FP64)
        k_coarse_assemble<double><<<grid, kAsmThreads, 0, s>>>(d);
    else
        k_coarse_assemble<float><<<grid, kAsmThreads, 0, s>>>(d);
    k_coarse_sum<<<d.n_segs, 256, 0, s>>>(d);
    count_launches(2);
}

// Runs of consecutive NoMass blobs with the same coarse dimension whose
// matrices lie n^2 apart: each run is updated by one batched product.
template <typename F>
void for_each_coarse_run(const std::vector<BlobParams> &bps, F f)
{
    for (size_t b0 = 0; b0 < bps.size();) {
        const BlobParams &bp = bps[b0];
        const int n = bp.coarse_n;
        size_t b1 = b0 + 1;
        if (bp.solver != SOLVER_NOMASS || n == 0) {
            b0 = b1;
            continue;
        }
        while (b1 < bps.size() && b1 - b0 < 65535 && bps[b1].solver == SOLVER_NOMASS && bps[b1].coarse_n == n &&
               (int64_t)bps[b1].coarse_xoff == (int64_t)bp.coarse_xoff + (int64_t)(b1 - b0) * n * n)
            b1++;
        f(bp, n, (int)(b1 - b0));
        b0 = b1;
    }
}

size_t coarse_part_floats(const std::vector<BlobParams> &bps)
{
    size_t need = 0;
    for_each_coarse_run(bps, [&](const BlobParams &, int n, int batch) {
        const int sp = sgemm_splits(n, batch);
        if (sp > 1) need = std::max(need, (size_t)sp * batch * n * n);
    });
    return need;
}

int coarse_refresh(const DeviceBatch &d, const std::vector<BlobParams> &bps, cudaStream_t s, int iterations,
                   bool init)
{
    if (!d.coarse) return 0;
    // a run of equal-size blobs (an ensemble of replicas) is updated by one
    // launch sequence of batched products
    for_each_coarse_run(bps, [&](const BlobParams &bp, int n, int batch) {
        float *A = d.coarse_A + bp.coarse_xoff, *X = d.coarse_X + bp.coarse_xoff;
        float *Tm = d.coarse_T, *Xn = d.coarse_Xn;
        if (init) {
            k_scaled_identity<<<batch, 1024, 0, s>>>(A, X, n);
            count_launches(1);
        }
        for (int it = 0; it < iterations; it++) {
            // T = A X; Xn = 2 X - X T; X = sym(Xn)
            sgemm_batched(A, X, nullptr, Tm, n, batch, 1.f, 0.f, d.coarse_part, s);
            sgemm_batched(X, Tm, X, Xn, n, batch, -1.f, 2.f, d.coarse_part, s);
            dim3 grid((n + 255) / 256, n, batch);
            k_symmetrize<<<grid, 256, 0, s>>>(Xn, X, n);
            count_launches(1);
        }
        if (d.coarse_Xh) {
            const int nh = (n + 7) / 8 * 8;
            dim3 grid((nh + 255) / 256, n, batch);
            k_coarse_half<<<grid, 256, 0, s>>>(X, reinterpret_cast<__half *>(d.coarse_Xh) + bp.coarse_hxoff,
                                               d.coarse_s + bp.coarse_off, n, nh);
            count_launches(1);
        }
    });
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace ffea
