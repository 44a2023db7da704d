// ssint.cu -- surface-surface Lennard-Jones interaction of FFEA on the GPU.
//
// Replaces VdW_solver::solve for "vdw_type = lennard-jones"
// (src/VdW_solver.cpp:168-210, 237-330, 338-394, 664-752) together with the
// nearest-neighbour grid it walks (NearestNeighbourLinkedListCube::
// build_nearest_neighbour_lookup, src/NearestNeighbourLinkedListCube.cpp:27-76)
// and the aggregation of face forces onto nodes (src/Blob.cpp:3841-3851).
//
// GPU layout and passes (one stream, no host round trip between them):
//   1. k_face_geom   one thread per active face: gathers its three corners,
//                    computes area, unit normal and centroid as
//                    Face::calc_area_normal_centroid (src/Face.cpp:197-219),
//                    bins the centroid into a cell (floor(c/h), wrapped once,
//                    LinkedListCube::pbc) and counts the cell's faces.
//   2. k_scan_local / k_scan_blocks   exclusive scan of the cell counts.
//   3. k_scatter     places every face in its cell's segment.
//   4. k_sort_cells  sorts each segment by face index (deterministic order):
//      k_sort_large  a thread per cell of up to 64 faces, a CTA per cell of up
//                    to 4096 (bitonic, in shared memory); a fuller cell makes
//                    the call an error (the grid is far too coarse).
//   5. k_pairs       one warp per face, in cell order so that neighbouring
//                    warps read the same cells: the lanes share the faces of
//                    the 27 cells around its own and integrate the LJ force
//                    of every partner the reference would pair with it; a
//                    fixed shuffle tree sums the lanes.  A pair (i, j) is evaluated
//                    from both sides, each side keeping only its own face's
//                    forces: twice the arithmetic of one evaluation, but no
//                    atomics on forces and a fixed summation order (the
//                    per-blob-pair energies use FP64 atomics, so their last
//                    bits may vary from run to run).  The pair
//                    is always evaluated with the lower pool index as FFEA's
//                    f1, so both sides reproduce FFEA's arithmetic.
//   6. k_node_gather one thread per node: sums its faces' corner forces in
//                    face order (a CSR built at creation).
// The file is compiled with -fmad=false so that every product and sum rounds
// as in the reference's FP64 code; cell binning and the normal test then
// decide exactly as FFEA does.  Two deliberate differences, both in the
// force of a pair, both changing it only at the rounding level: the unit
// direction of each point pair is (p - q) * (1/r) where FFEA divides by r,
// and the nine weighted terms per corner are regrouped through column sums
// of the (symmetric) force matrix.  Together they remove three FP64 divides
// per point pair and 216 of 243 products per pair side; the kernel is bound
// by the FP64 pipe.
#include <cuda_runtime.h>

#include <climits>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/ffea_gpu.h"

namespace ffea {
void set_last_error(const char *msg);  // api.cu
}

struct ffea_gpu_ssint {
    int num_nodes = 0, num_faces = 0, num_active = 0, num_types = 0, num_blobs = 0;
    int nx = 0, ny = 0, nz = 0, inc_self = 0;
    long long ncell = 0;
    int nblocks = 0;
    double h = 0.0;
    cudaStream_t stream = nullptr;
    // per active face, in the caller's face order
    int *d_corner = nullptr;    // 3 node indices
    int *d_blob = nullptr;
    int *d_type = nullptr;
    double *d_geo = nullptr;    // 16 doubles: corners (9), unit normal (3), area, pad
    int *d_cell = nullptr;      // -1: outside the box
    double *d_fforce = nullptr; // 9 doubles: force on each corner
    // grid
    int *d_count = nullptr;     // ncell
    int *d_start = nullptr;     // ncell, block-local exclusive prefix
    int *d_block = nullptr;     // nblocks, global prefix of each block
    int *d_sorted = nullptr;    // num_active faces in cell order
    // nodes
    int *d_node_ptr = nullptr;  // num_nodes + 1
    int *d_node_ent = nullptr;  // face * 3 + corner, face order
    double *d_emin = nullptr, *d_rmin = nullptr;
    double *d_pos = nullptr, *d_force = nullptr, *d_energy = nullptr;  // staging of the host entry point
    unsigned long long *d_stats = nullptr;  // [0] pairs, [1] out-of-box faces, [2] large cells, [3] oversized cells
    int *d_large = nullptr;                 // cells of more than kSortSmall faces (k_sort_large)
};

namespace {

constexpr int kScanBlock = 1024;

int fail(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ffea::set_last_error(buf);
    return FFEA_GPU_ERROR;
}

#define SSINT_CUDA(call)                                                                    \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return fail("%s: %s", #call, cudaGetErrorString(e_));        \
    } while (0)

// 3-point rule on a triangle (src/VdW_solver.cpp:61-71): weight kW, point k
// has barycentric coordinate eta(k, d).  Written as constant expressions so
// that, in the fully unrolled loops, products of constants such as
// kW * kW * eta fold at compile time (to the same double the reference
// computes at run time) instead of costing FP64 instructions per pair.
constexpr double kW = 0.333333333333333;
__host__ __device__ constexpr double eta(int k, int d) { return k == d ? 0.666666666666667 : 0.166666666666667; }

__device__ __forceinline__ int wrap(int x, int n)
{
    if (x < 0) return x + n;
    if (x >= n) return x - n;
    return x;
}

__global__ void k_face_geom(const double *__restrict__ pos, const int *__restrict__ corner, int nf, double h,
                            int nx, int ny, int nz, double *__restrict__ geo, int *__restrict__ cell,
                            int *__restrict__ count, unsigned long long *stats)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double v[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int n = corner[3 * f + k];
#pragma unroll
        for (int d = 0; d < 3; d++) v[k][d] = pos[3 * (long long)n + d];
    }
    double a[3], b[3], nrm[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        a[d] = v[1][d] - v[0][d];
        b[d] = v[2][d] - v[0][d];
    }
    nrm[0] = a[1] * b[2] - a[2] * b[1];
    nrm[1] = a[2] * b[0] - a[0] * b[2];
    nrm[2] = a[0] * b[1] - a[1] * b[0];
    const double mag = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    double *g = geo + 16 * (long long)f;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) g[3 * k + d] = v[k][d];
#pragma unroll
    for (int d = 0; d < 3; d++) g[9 + d] = nrm[d] / mag;
    g[12] = .5 * mag;
    int c[3];
    const int dims[3] = {nx, ny, nz};
    bool inside = true;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double cen = (1.0 / 3.0) * (v[0][d] + v[1][d] + v[2][d]);
        const double fl = floor(cen / h);
        // cells beyond int range (or a NaN centroid) are outside the box as well
        int x = (fl >= -2147483647.0 && fl <= 2147483647.0) ? (int)fl : -2147483647;
        x = (x < -dims[d] || x >= 2 * dims[d]) ? -1 : wrap(x, dims[d]);
        if (x < 0 || x >= dims[d]) inside = false;
        c[d] = x;
    }
    if (!inside) {
        cell[f] = -1;
        atomicAdd(&stats[1], 1ull);
        return;
    }
    const int id = (c[0] * ny + c[1]) * nz + c[2];
    cell[f] = id;
    atomicAdd(&count[id], 1);
}

__device__ __forceinline__ int warp_incl_scan(int v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-local exclusive scan of kScanBlock cells; the block's total to block_sum
__global__ void __launch_bounds__(kScanBlock) k_scan_local(const int *__restrict__ count, long long ncell,
                                                           int *__restrict__ start, int *__restrict__ block_sum)
{
    __shared__ int warp_tot[kScanBlock / 32];
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int v = i < ncell ? count[i] : 0;
    const int incl = warp_incl_scan(v, lane);
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int t = warp_incl_scan(warp_tot[lane], lane);
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int base = w ? warp_tot[w - 1] : 0;
    if (i < ncell) start[i] = base + incl - v;
    if (threadIdx.x == kScanBlock - 1) block_sum[blockIdx.x] = base + incl;
}

// exclusive scan of the block totals, in place, by one CTA
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(int *__restrict__ block, int nblocks)
{
    __shared__ int warp_tot[kScanBlock / 32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int v = i < nblocks ? block[i] : 0;
        const int incl = warp_incl_scan(v, lane);
        if (lane == 31) warp_tot[w] = incl;
        __syncthreads();
        if (w == 0) warp_tot[lane] = warp_incl_scan(warp_tot[lane], lane);
        __syncthreads();
        const int pre = (w ? warp_tot[w - 1] : 0) + incl - v;
        const int c = carry;
        if (i < nblocks) block[i] = c + pre;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry = c + pre + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) block[nblocks] = carry;  // faces binned in all
}

__device__ __forceinline__ int cell_begin(const int *start, const int *block, long long c)
{
    return start[c] + block[c / kScanBlock];
}

// block[nblocks] holds the number of faces binned, the end of the last cell
__device__ __forceinline__ int cell_end(const int *start, const int *block, long long c, long long ncell,
                                        int nblocks)
{
    return c + 1 < ncell ? cell_begin(start, block, c + 1) : block[nblocks];
}

__global__ void k_scatter(const int *__restrict__ cell, int nf, const int *__restrict__ start,
                          const int *__restrict__ block, int *__restrict__ count, int *__restrict__ sorted)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int c = cell[f];
    if (c < 0) return;
    const int slot = cell_begin(start, block, c) + atomicSub(&count[c], 1) - 1;
    sorted[slot] = f;
}

// Each cell's faces sorted by face index.  A cell of at most kSortSmall
// faces is insertion-sorted by its thread; a larger one, up to kSortMax
// faces, is listed for k_sort_large (one CTA per cell); a cell above that is
// counted in stats[3] and makes the call an error, so that a grid far too
// coarse for the mesh fails at once instead of one thread sorting many
// thousands of faces.
constexpr int kSortSmall = 64;
constexpr int kSortMax = 4096;
constexpr int kSortLargeCtas = 256;

__global__ void k_sort_cells(long long ncell, int nblocks, const int *__restrict__ start,
                             const int *__restrict__ block, int *__restrict__ sorted, int *__restrict__ large,
                             unsigned long long *stats)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int b = cell_begin(start, block, c);
    const int e = cell_end(start, block, c, ncell, nblocks);
    if (e - b > kSortMax) {
        atomicAdd(&stats[3], 1ull);
        return;
    }
    if (e - b > kSortSmall) {
        large[atomicAdd(&stats[2], 1ull)] = (int)c;
        return;
    }
    for (int i = b + 1; i < e; i++) {
        const int v = sorted[i];
        int j = i - 1;
        while (j >= b && sorted[j] > v) {
            sorted[j + 1] = sorted[j];
            j--;
        }
        sorted[j + 1] = v;
    }
}

// The listed large cells, one CTA each (grid-stride over the list): a
// bitonic sort in shared memory of the cell's face indices, padded to a
// power of two.
__global__ void __launch_bounds__(256) k_sort_large(long long ncell, int nblocks, const int *__restrict__ start,
                                                    const int *__restrict__ block, int *__restrict__ sorted,
                                                    const int *__restrict__ large,
                                                    const unsigned long long *__restrict__ stats)
{
    __shared__ int v[kSortMax];
    const int nl = (int)stats[2];
    for (int k = blockIdx.x; k < nl; k += gridDim.x) {
        const long long c = large[k];
        const int b = cell_begin(start, block, c);
        const int n = cell_end(start, block, c, ncell, nblocks) - b;  // kSortSmall < n <= kSortMax
        int m = 1;
        while (m < n) m <<= 1;
        for (int i = threadIdx.x; i < m; i += blockDim.x) v[i] = i < n ? sorted[b + i] : INT_MAX;
        __syncthreads();
        for (int size = 2; size <= m; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = threadIdx.x; i < m; i += blockDim.x) {
                    const int j = i ^ stride;
                    if (j > i) {
                        const bool up = (i & size) == 0;
                        const int a = v[i], bb = v[j];
                        if ((a > bb) == up) {
                            v[i] = bb;
                            v[j] = a;
                        }
                    }
                }
                __syncthreads();
            }
        for (int i = threadIdx.x; i < n; i += blockDim.x) sorted[b + i] = v[i];
        __syncthreads();
    }
}

// do_lj_interaction for f1 = A, f2 = B (src/VdW_solver.cpp:237-330 with
// calc_lj_force_pair_matrix / calc_lj_factors, :664-699, :736-752).  Adds
// force1 (A_SIDE) or force2 (!A_SIDE) to out[3][3] and returns the pair energy.
template <bool A_SIDE>
__device__ __forceinline__ double lj_pair(const double *A, const double *B, double emin, double rmin,
                                          double out[3][3])
{
    double p[3][3], q[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            p[k][d] = eta(k, 0) * A[d] + eta(k, 1) * A[3 + d] + eta(k, 2) * A[6 + d];
            q[k][d] = eta(k, 0) * B[d] + eta(k, 1) * B[3 + d] + eta(k, 2) * B[6 + d];
        }
    const double r2 = rmin * rmin;
    const double r4 = r2 * r2;
    const double r6 = r4 * r2;
    double fpm[3][3][3];
    double energy = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int l = k; l < 3; l++) {
            const double dx = p[k][0] - q[l][0], dy = p[k][1] - q[l][1], dz = p[k][2] - q[l][2];
            const double mag_r = sqrt(dx * dx + dy * dy + dz * dz);
            const double ri = 1. / mag_r;
            const double ri2 = ri * ri;
            const double ri4 = ri2 * ri2;
            const double ri6 = ri4 * ri2;
            const double ri7 = ri6 * ri;
            const double f6 = r6 * ri6;
            const double fm = 12 * ri7 * r6 * emin * (f6 - 1);
            const double e = kW * kW * emin * f6 * (f6 - 2);
            energy += (l == k) ? e : 2 * e;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                fpm[k][l][d] = fm * ((p[k][d] - q[l][d]) * ri);  // FFEA divides by mag_r: within 1 ulp
                fpm[l][k][d] = fpm[k][l][d];
            }
        }
    }
    const double apaq = A[12] * B[12];
    // FFEA sums W^2 eta * fpm over all nine (k, l) for each corner j.  The
    // matrix is symmetric, so both sides need only the column sums
    // S_l = sum_k fpm[k][l]: force1_j = sum_l W^2 eta_l[j] S_l and
    // force2_j = -sum_k W^2 eta_k[j] S_k.  Same terms, regrouped (27 products
    // per pair instead of 243; the sums round differently, within 1e-15).
    double S[3][3];
#pragma unroll
    for (int l = 0; l < 3; l++)
#pragma unroll
        for (int d = 0; d < 3; d++) S[l][d] = fpm[0][l][d] + fpm[1][l][d] + fpm[2][l][d];
#pragma unroll
    for (int j = 0; j < 3; j++) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double f = (kW * kW * eta(0, j)) * S[0][d] + (kW * kW * eta(1, j)) * S[1][d] +
                             (kW * kW * eta(2, j)) * S[2][d];
            out[j][d] += (A_SIDE ? f : -f) * apaq;
        }
    }
    return energy * apaq;
}

__constant__ int c_adj[27][3] = {{-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {-1, 0, 1},
                                 {-1, 1, -1},  {-1, 1, 0},  {-1, 1, 1},  {0, -1, -1}, {0, -1, 0}, {0, -1, 1},
                                 {0, 0, -1},   {0, 0, 0},   {0, 0, 1},   {0, 1, -1},  {0, 1, 0},  {0, 1, 1},
                                 {1, -1, -1},  {1, -1, 0},  {1, -1, 1},  {1, 0, -1},  {1, 0, 0},  {1, 0, 1},
                                 {1, 1, -1},   {1, 1, 0},   {1, 1, 1}};

constexpr int kPairWarps = 8;  // warps (faces) per CTA of k_pairs

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One warp per face i (faces taken in cell order): the candidates of the 27
// cells around i's cell are numbered 0..total-1 through a prefix sum over the
// cells, lane l tests candidates l, l + 32, ..., and the partners that pass
// are evaluated from a per-warp queue.  Each lane keeps face i's side of its
// pairs; a fixed shuffle tree sums the lanes.
__global__ void __launch_bounds__(32 * kPairWarps) k_pairs(
    const double *__restrict__ geo, const int *__restrict__ cell, const int *__restrict__ sorted,
    const int *__restrict__ start, const int *__restrict__ block, long long ncell, int nblocks, int nx, int ny,
    int nz, const int *__restrict__ fblob, const int *__restrict__ ftype, const double *__restrict__ emin,
    const double *__restrict__ rmin, int num_types, int num_blobs, int inc_self, double *__restrict__ fforce,
    double *__restrict__ energy, unsigned long long *stats)
{
    __shared__ int s_pre[kPairWarps][28];
    __shared__ int s_beg[kPairWarps][27];
    __shared__ int s_q[kPairWarps][64];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long w = (long long)blockIdx.x * kPairWarps + wi;
    if (w >= block[nblocks]) return;  // warp-uniform; faces outside the box are not binned
    if (stats[3]) return;             // a cell too full to sort: the call fails, nothing to evaluate
    const int i = sorted[w];
    const int ci = cell[i];
    const int cz = ci % nz, cy = (ci / nz) % ny, cx = ci / (nz * ny);
    int len = 0, beg = 0;
    if (lane < 27) {
        const int x = wrap(cx + c_adj[lane][0], nx), y = wrap(cy + c_adj[lane][1], ny),
                  z = wrap(cz + c_adj[lane][2], nz);
        const long long cc = ((long long)x * ny + y) * nz + z;
        beg = cell_begin(start, block, cc);
        len = cell_end(start, block, cc, ncell, nblocks) - beg;
    }
    const int incl = warp_incl_scan(len, lane);
    if (lane < 27) {
        s_beg[wi][lane] = beg;
        s_pre[wi][lane] = incl - len;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 26);
    __syncwarp();
    double A[13];
#pragma unroll
    for (int k = 0; k < 13; k++) A[k] = geo[16 * (long long)i + k];
    const int bi = fblob[i], ti = ftype[i];
    double out[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double e_acc = 0.0;
    int e_key = -1;
    unsigned long long npairs = 0;
    // one partner j: face i's side of the pair, FFEA's f1 being the lower index
    auto pair = [&](int j) {
        const double *G = geo + 16 * (long long)j;
        double B[13];
#pragma unroll
        for (int q = 0; q < 13; q++) B[q] = G[q];
        if (i < j) {
            const int tt = ti * num_types + ftype[j];
            const double en = lj_pair<true>(A, B, emin[tt], rmin[tt], out);
            const int key = bi * num_blobs + fblob[j];
            if (key != e_key) {
                if (e_key >= 0) atomicAdd(&energy[e_key], e_acc);
                e_key = key;
                e_acc = 0.0;
            }
            e_acc += en;
            npairs++;
        } else {
            const int tt = ftype[j] * num_types + ti;
            lj_pair<false>(B, A, emin[tt], rmin[tt], out);
        }
    };
    // The cheap tests (same face, same blob, normals facing the same way) run
    // over all candidates; the partners that pass are queued in shared memory
    // and evaluated 32 at a time, so every lane of the FP64 pair arithmetic
    // does useful work.
    int qn = 0;  // warp-uniform queue length, < 64
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        bool ok = false;
        int j = -1;
        if (k < total) {
            int c = 0;
            while (c < 26 && s_pre[wi][c + 1] <= k) c++;
            j = sorted[s_beg[wi][c] + (k - s_pre[wi][c])];
            const double *G = geo + 16 * (long long)j;
            ok = j != i && (inc_self || bi != fblob[j]) && !(A[9] * G[9] + A[10] * G[10] + A[11] * G[11] > 0.0);
        }
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (ok) s_q[wi][qn + __popc(m & ((1u << lane) - 1u))] = j;
        qn += __popc(m);
        __syncwarp();
        if (qn >= 32) {
            pair(s_q[wi][lane]);
            const int rest = qn - 32;
            const int moved = lane < rest ? s_q[wi][32 + lane] : 0;
            __syncwarp();
            if (lane < rest) s_q[wi][lane] = moved;
            qn = rest;
            __syncwarp();
        }
    }
    if (lane < qn) pair(s_q[wi][lane]);
    // energy: one atomic per distinct (blob, blob) key left in the warp
    for (;;) {
        const unsigned pending = __ballot_sync(0xffffffffu, e_key >= 0);
        if (!pending) break;
        const int lk = __shfl_sync(0xffffffffu, e_key, __ffs(pending) - 1);
        const double part = warp_sum_d(e_key == lk ? e_acc : 0.0);
        if (lane == 0) atomicAdd(&energy[lk], part);
        if (e_key == lk) e_key = -1;
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) out[k][d] = warp_sum_d(out[k][d]);
    unsigned long long np = npairs;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) np += __shfl_xor_sync(0xffffffffu, np, o);
    if (lane == 0) {
        if (np) atomicAdd(&stats[0], np);
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int d = 0; d < 3; d++) fforce[9 * (long long)i + 3 * k + d] = out[k][d];
    }
}

__global__ void k_node_gather(const int *__restrict__ ptr, const int *__restrict__ ent, int nn,
                              const double *__restrict__ fforce, const int *__restrict__ cell,
                              double *__restrict__ force)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    double f[3] = {0.0, 0.0, 0.0};
    for (int k = ptr[n]; k < ptr[n + 1]; k++) {
        const int fc = ent[k];
        if (cell[fc / 3] < 0) continue;
#pragma unroll
        for (int d = 0; d < 3; d++) f[d] += fforce[3 * (long long)fc + d];
    }
#pragma unroll
    for (int d = 0; d < 3; d++) force[3 * (long long)n + d] = f[d];
}

template <class T>
int dalloc(T **p, size_t n)
{
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return fail("cudaMalloc of %zu bytes: %s", sizeof(T) * n, cudaGetErrorString(e));
    return FFEA_GPU_OK;
}

}  // namespace

extern "C" int ffea_gpu_ssint_create(const ffea_gpu_ssint_desc *d, ffea_gpu_ssint_t **out)
{
    if (!d || !out) return fail("ffea_gpu_ssint_create: null argument");
    *out = nullptr;
    if (d->num_nodes < 0 || d->num_faces < 0 || d->num_types <= 0 || d->num_blobs <= 0)
        return fail("ffea_gpu_ssint_create: negative sizes, or no types or blobs");
    if ((d->num_faces && (!d->faces || !d->face_blob || !d->face_type)) || !d->emin || !d->rmin)
        return fail("ffea_gpu_ssint_create: null array");
    if (!(d->cell_size > 0.0)) return fail("ffea_gpu_ssint_create: cell_size must be positive");
    if (d->nx <= 0 || d->ny <= 0 || d->nz <= 0) return fail("ffea_gpu_ssint_create: grid dimensions must be positive");
    const long long ncell = (long long)d->nx * d->ny * d->nz;
    if (ncell > FFEA_GPU_SSINT_MAX_CELLS)
        return fail("ffea_gpu_ssint_create: %lld cells exceed the maximum %d", ncell, FFEA_GPU_SSINT_MAX_CELLS);
    std::vector<int> corner, blob, type;
    for (int f = 0; f < d->num_faces; f++) {
        if (d->face_type[f] < 0) continue;  // not ssint-active: not in the pool (src/Blob.cpp:1642-1648)
        if (d->face_type[f] >= d->num_types) return fail("face %d: interaction type %d >= num_types", f, d->face_type[f]);
        if (d->face_blob[f] < 0 || d->face_blob[f] >= d->num_blobs) return fail("face %d: blob %d out of range", f, d->face_blob[f]);
        for (int k = 0; k < 3; k++) {
            const int n = d->faces[3 * f + k];
            if (n < 0 || n >= d->num_nodes) return fail("face %d: node %d out of range", f, n);
            corner.push_back(n);
        }
        blob.push_back(d->face_blob[f]);
        type.push_back(d->face_type[f]);
    }
    const int na = (int)blob.size();
    // node -> (active face, corner) entries in face order
    std::vector<int> ptr(d->num_nodes + 1, 0), ent(3 * (size_t)na);
    for (int i = 0; i < 3 * na; i++) ptr[corner[i] + 1]++;
    for (int n = 0; n < d->num_nodes; n++) ptr[n + 1] += ptr[n];
    {
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int i = 0; i < 3 * na; i++) ent[fill[corner[i]]++] = i;
    }
    auto *s = new ffea_gpu_ssint();
    s->num_nodes = d->num_nodes;
    s->num_faces = d->num_faces;
    s->num_active = na;
    s->num_types = d->num_types;
    s->num_blobs = d->num_blobs;
    s->nx = d->nx;
    s->ny = d->ny;
    s->nz = d->nz;
    s->inc_self = d->inc_self ? 1 : 0;
    s->h = d->cell_size;
    s->ncell = ncell;
    s->nblocks = (int)((ncell + kScanBlock - 1) / kScanBlock);
    const int T2 = d->num_types * d->num_types;
    int rc = FFEA_GPU_OK;
    auto run = [&]() -> int {
        SSINT_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        if (dalloc(&s->d_corner, 3 * (size_t)na) || dalloc(&s->d_blob, na) || dalloc(&s->d_type, na) ||
            dalloc(&s->d_geo, 16 * (size_t)na) || dalloc(&s->d_cell, na) || dalloc(&s->d_fforce, 9 * (size_t)na) ||
            dalloc(&s->d_count, ncell) || dalloc(&s->d_start, ncell) || dalloc(&s->d_block, s->nblocks + 1) ||
            dalloc(&s->d_sorted, na) || dalloc(&s->d_node_ptr, d->num_nodes + 1) ||
            dalloc(&s->d_node_ent, 3 * (size_t)na) || dalloc(&s->d_emin, T2) || dalloc(&s->d_rmin, T2) ||
            dalloc(&s->d_pos, 3 * (size_t)d->num_nodes) || dalloc(&s->d_force, 3 * (size_t)d->num_nodes) ||
            dalloc(&s->d_energy, (size_t)d->num_blobs * d->num_blobs) || dalloc(&s->d_stats, 4) ||
            dalloc(&s->d_large, (size_t)na / (kSortSmall + 1) + 1))
            return FFEA_GPU_ERROR;
        if (na) {
            SSINT_CUDA(cudaMemcpy(s->d_corner, corner.data(), sizeof(int) * 3 * na, cudaMemcpyHostToDevice));
            SSINT_CUDA(cudaMemcpy(s->d_blob, blob.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
            SSINT_CUDA(cudaMemcpy(s->d_type, type.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
            SSINT_CUDA(cudaMemcpy(s->d_node_ent, ent.data(), sizeof(int) * 3 * na, cudaMemcpyHostToDevice));
        }
        SSINT_CUDA(cudaMemcpy(s->d_node_ptr, ptr.data(), sizeof(int) * (d->num_nodes + 1), cudaMemcpyHostToDevice));
        SSINT_CUDA(cudaMemcpy(s->d_emin, d->emin, sizeof(double) * T2, cudaMemcpyHostToDevice));
        SSINT_CUDA(cudaMemcpy(s->d_rmin, d->rmin, sizeof(double) * T2, cudaMemcpyHostToDevice));
        return FFEA_GPU_OK;
    };
    rc = run();
    if (rc != FFEA_GPU_OK) {
        ffea_gpu_ssint_destroy(s);
        return rc;
    }
    *out = s;
    return FFEA_GPU_OK;
}

extern "C" void ffea_gpu_ssint_destroy(ffea_gpu_ssint_t *s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    void *bufs[] = {s->d_corner, s->d_blob, s->d_type, s->d_geo, s->d_cell, s->d_fforce, s->d_count,
                    s->d_start, s->d_block, s->d_sorted, s->d_node_ptr, s->d_node_ent, s->d_emin, s->d_rmin,
                    s->d_pos, s->d_force, s->d_energy, s->d_stats, s->d_large};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

extern "C" void *ffea_gpu_ssint_stream(ffea_gpu_ssint_t *s) { return s ? (void *)s->stream : nullptr; }

extern "C" int ffea_gpu_ssint_forces_device(ffea_gpu_ssint_t *s, const double *pos, double *force, double *energy)
{
    if (!s || !pos || !force || !energy) return fail("ffea_gpu_ssint_forces_device: null argument");
    cudaStream_t st = s->stream;
    const int na = s->num_active;
    SSINT_CUDA(cudaMemsetAsync(energy, 0, sizeof(double) * s->num_blobs * s->num_blobs, st));
    SSINT_CUDA(cudaMemsetAsync(s->d_stats, 0, sizeof(unsigned long long) * 4, st));
    if (na == 0) {
        SSINT_CUDA(cudaMemsetAsync(force, 0, sizeof(double) * 3 * (size_t)s->num_nodes, st));
        return FFEA_GPU_OK;
    }
    SSINT_CUDA(cudaMemsetAsync(s->d_count, 0, sizeof(int) * s->ncell, st));
    const int fb = (na + 127) / 128;
    k_face_geom<<<fb, 128, 0, st>>>(pos, s->d_corner, na, s->h, s->nx, s->ny, s->nz, s->d_geo, s->d_cell,
                                    s->d_count, s->d_stats);
    k_scan_local<<<s->nblocks, kScanBlock, 0, st>>>(s->d_count, s->ncell, s->d_start, s->d_block);
    k_scan_blocks<<<1, kScanBlock, 0, st>>>(s->d_block, s->nblocks);
    k_scatter<<<fb, 128, 0, st>>>(s->d_cell, na, s->d_start, s->d_block, s->d_count, s->d_sorted);
    // faces outside the box are left out of the grid (and make the call an
    // error); the kernels below bound every segment by the scan's total
    k_sort_cells<<<(int)((s->ncell + 255) / 256), 256, 0, st>>>(s->ncell, s->nblocks, s->d_start, s->d_block,
                                                                s->d_sorted, s->d_large, s->d_stats);
    k_sort_large<<<kSortLargeCtas, 256, 0, st>>>(s->ncell, s->nblocks, s->d_start, s->d_block, s->d_sorted,
                                                 s->d_large, s->d_stats);
    k_pairs<<<(na + kPairWarps - 1) / kPairWarps, 32 * kPairWarps, 0, st>>>(s->d_geo, s->d_cell, s->d_sorted, s->d_start, s->d_block, s->ncell, s->nblocks, s->nx,
                                s->ny, s->nz, s->d_blob, s->d_type, s->d_emin, s->d_rmin, s->num_types,
                                s->num_blobs, s->inc_self, s->d_fforce, energy, s->d_stats);
    k_node_gather<<<(s->num_nodes + 255) / 256, 256, 0, st>>>(s->d_node_ptr, s->d_node_ent, s->num_nodes,
                                                              s->d_fforce, s->d_cell, force);
    SSINT_CUDA(cudaGetLastError());
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_ssint_synchronize(ffea_gpu_ssint_t *s, int64_t *pairs)
{
    if (!s) return fail("ffea_gpu_ssint_synchronize: null handle");
    unsigned long long st[4] = {0, 0, 0, 0};
    SSINT_CUDA(cudaMemcpyAsync(st, s->d_stats, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
    SSINT_CUDA(cudaStreamSynchronize(s->stream));
    if (pairs) *pairs = (int64_t)st[0];
    if (st[1]) return fail("%llu face centroids lie outside the interaction grid (FFEA reports this as an error)", st[1]);
    if (st[3])
        return fail("%llu grid cells hold more than %d faces each: the interaction grid is too coarse for this mesh "
                    "(use more, smaller cells)", st[3], kSortMax);
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_ssint_forces(ffea_gpu_ssint_t *s, const double *pos, double *force, double *energy,
                                     int64_t *pairs)
{
    if (!s || !pos || !force || !energy) return fail("ffea_gpu_ssint_forces: null argument");
    const size_t nb = sizeof(double) * 3 * (size_t)s->num_nodes;
    SSINT_CUDA(cudaMemcpyAsync(s->d_pos, pos, nb, cudaMemcpyHostToDevice, s->stream));
    if (ffea_gpu_ssint_forces_device(s, s->d_pos, s->d_force, s->d_energy)) return FFEA_GPU_ERROR;
    SSINT_CUDA(cudaMemcpyAsync(force, s->d_force, nb, cudaMemcpyDeviceToHost, s->stream));
    SSINT_CUDA(cudaMemcpyAsync(energy, s->d_energy, sizeof(double) * s->num_blobs * s->num_blobs,
                               cudaMemcpyDeviceToHost, s->stream));
    return ffea_gpu_ssint_synchronize(s, pairs);
}
