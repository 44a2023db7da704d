// ssint.cu -- surface-surface interactions of FFEA on the GPU.
//
// Replaces VdW_solver::solve for "vdw_type = lennard-jones"
// (src/VdW_solver.cpp:168-210, 237-330, 338-394, 664-752), "steric"
// (Steric_solver, src/VdW_solver.cpp:458-486), "ljsteric" (LJSteric_solver:
// steric where the faces' element tetrahedra overlap, Lennard-Jones
// elsewhere) and "gensoft" (GenSoftSSINT_solver, src/VdW_solver.cpp:488-563,
// 701-771), together with the nearest-neighbour grid they walk
// (NearestNeighbourLinkedListCube::build_nearest_neighbour_lookup,
// src/NearestNeighbourLinkedListCube.cpp:27-76) and the aggregation of face
// forces onto nodes (src/Blob.cpp:3841-3851).  The steric types first run
// k_steric (overlap volume of the two element tetrahedra by convex clipping,
// its forward-difference gradient and FFEA's barycentric weights, between
// steps 4 and 5 below), whose force lands on the four nodes of each face's
// element; k_pairs then skips the pairs k_steric handled.
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
    int type = FFEA_GPU_SSINT_LJ;
    double steric_factor = 0.0, steric_dr = 0.0;
    long long ncell = 0;
    int nblocks = 0;
    double h = 0.0;
    cudaStream_t stream = nullptr;
    // per active face, in the caller's face order
    int *d_corner = nullptr;    // 4 node indices: the corners, then the element's fourth node (-1: none)
    int *d_blob = nullptr;
    int *d_type = nullptr;
    double *d_geo = nullptr;    // 16 doubles: corners (9), unit normal (3), area, fourth node (3)
    int *d_cell = nullptr;      // -1: outside the box
    double *d_fforce = nullptr; // 12 doubles: force on each corner and on the fourth node
    double *d_corr = nullptr;   // periodic blob corrections (num_blobs^2 x 3), when set
    int has_corr = 0, sticky = 0;
    int *d_stlist = nullptr;    // steric types: the partners whose tetrahedra overlap (MAX_STERIC_PARTNERS each)
    int *d_stcnt = nullptr;     // their number per face
    // grid
    int *d_count = nullptr;     // ncell
    int *d_start = nullptr;     // ncell, block-local exclusive prefix
    int *d_block = nullptr;     // nblocks, global prefix of each block
    int *d_sorted = nullptr;    // num_active faces in cell order
    // nodes
    int *d_node_ptr = nullptr;  // num_nodes + 1
    int *d_node_ent = nullptr;  // face * 4 + corner (3: the fourth node), face order
    double *d_emin = nullptr, *d_rmin = nullptr, *d_k0 = nullptr;
    double *d_pos = nullptr, *d_force = nullptr, *d_energy = nullptr;  // staging of the host entry point
    unsigned long long *d_stats = nullptr;  // [0] pairs, [1] out-of-box faces, [2] large cells, [3] oversized cells,
                                            // [4] faces with too many steric partners
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
        const int n = corner[4 * f + k];
#pragma unroll
        for (int d = 0; d < 3; d++) v[k][d] = pos[3 * (long long)n + d];
    }
    const int apex = corner[4 * f + 3];
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
#pragma unroll
    for (int d = 0; d < 3; d++) g[13 + d] = apex >= 0 ? pos[3 * (long long)apex + d] : 0.0;
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

// The integrated point-pair potentials of one face pair, for f1 = A, f2 = B:
//   POT_LJ    do_lj_interaction (src/VdW_solver.cpp:237-330) with
//             calc_lj_force_pair_matrix / calc_lj_factors (:664-699, :736-752);
//   POT_SOFT  do_gensoft_interaction (:488-563) with
//             calc_gensoft_force_pair_matrix / calc_gensoft_factors (:701-734, :754-771).
// Adds force1 (A_SIDE) or force2 (!A_SIDE) to out[0..2] and returns the pair
// energy.  k0: the soft potential's k0 (unused by POT_LJ).
constexpr int POT_LJ = 0, POT_SOFT = 1;

template <int POT, bool A_SIDE>
__device__ __forceinline__ double pot_pair(const double *A, const double *B, double emin, double rmin, double k0,
                                           double out[4][3])
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
            double fm, e;
            if constexpr (POT == POT_LJ) {
                const double ri2 = ri * ri;
                const double ri4 = ri2 * ri2;
                const double ri6 = ri4 * ri2;
                const double ri7 = ri6 * ri;
                const double f6 = r6 * ri6;
                fm = 12 * ri7 * r6 * emin * (f6 - 1);
                e = kW * kW * emin * f6 * (f6 - 2);
            } else {
                const double mag_r_2 = mag_r * mag_r;
                const double gf2 = mag_r_2 / r2;
                const double gf3 = gf2 * mag_r / rmin;
                const double k0rm = k0 * rmin;
                const double k0rm2 = k0rm * rmin;
                const double epsonrm = emin / rmin;
                fm = 2 * (k0rm - 6 * epsonrm) * gf3 + 3 * (4 * epsonrm - k0rm) * gf2 + k0 * mag_r;
                e = kW * kW *
                    ((0.5 * k0rm2 - 3 * emin) * gf2 * gf2 + (4 * emin - k0rm2) * gf3 + 0.5 * k0 * mag_r_2 - emin);
            }
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

// ---- steric: the overlap of two tetrahedra -------------------------------
// The overlap of tetrahedra A and B is clipped out of A by B's four
// half-spaces: each face polygon clipped in turn (Sutherland-Hodgman) and each
// cut closed by a cap polygon, its points ordered by angle.  Two tetrahedra
// intersect in at most 8 half-spaces, so the polyhedron has at most 8 faces
// of at most 7 vertices.  Its volume is a fan of tetrahedra from the mean of
// its vertices; its "centre" is what FFEA's volumeIntersectionII returns
// (findCM, src/VolumeIntersection.cpp:95-104): the mean of its distinct
// vertices.  Points closer than 1e-9 of the tetrahedra's extent are one.
constexpr int kStV = 8, kStF = 8, kStC = 16, kStU = 32;

struct StPolyh {
    int nf;
    int n[kStF];
    double v[kStF][kStV][3];
};

__device__ __forceinline__ double st_dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

__device__ __forceinline__ double st_tet_volume(const double *a, const double *b, const double *c, const double *d)
{
    const double u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
    const double v0 = c[0] - a[0], v1 = c[1] - a[1], v2 = c[2] - a[2];
    const double w0 = d[0] - a[0], w1 = d[1] - a[1], w2 = d[2] - a[2];
    const double x0 = v1 * w2 - v2 * w1, x1 = v2 * w0 - v0 * w2, x2 = v0 * w1 - v1 * w0;
    return (u0 * x0 + u1 * x1 + u2 * x2) / 6.0;
}

__device__ __forceinline__ void st_add_unique(double (*pts)[3], int &n, int cap, const double *x, double tol2)
{
    for (int u = 0; u < n; u++) {
        const double e0 = x[0] - pts[u][0], e1 = x[1] - pts[u][1], e2 = x[2] - pts[u][2];
        if (e0 * e0 + e1 * e1 + e2 * e2 <= tol2) return;
    }
    if (n < cap) {
        pts[n][0] = x[0];
        pts[n][1] = x[1];
        pts[n][2] = x[2];
        n++;
    }
}

__constant__ int c_tri[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

// clip P by n . x <= off; false when nothing is left
__device__ bool st_clip(StPolyh &P, const double *nrm, double off, double tol2)
{
    double smin = 0.0, smax = 0.0;
    bool first = true;
    for (int f = 0; f < P.nf; f++)
        for (int k = 0; k < P.n[f]; k++) {
            const double sv = st_dot(nrm, P.v[f][k]) - off;
            if (first || sv < smin) smin = sv;
            if (first || sv > smax) smax = sv;
            first = false;
        }
    if (first || smin >= 0) {
        P.nf = 0;
        return false;
    }
    if (smax <= 0) return true;
    double cap[kStC][3];
    int nc = 0, nf = 0;
    for (int f = 0; f < P.nf; f++) {
        double out[kStV][3];
        int no = 0;
        const int m = P.n[f];
        for (int k = 0; k < m; k++) {
            const double *a = P.v[f][k], *b = P.v[f][k + 1 < m ? k + 1 : 0];
            const double sa = st_dot(nrm, a) - off, sb = st_dot(nrm, b) - off;
            if (sa <= 0) {
                if (no < kStV) {
                    out[no][0] = a[0];
                    out[no][1] = a[1];
                    out[no][2] = a[2];
                    no++;
                }
                if (sa == 0) st_add_unique(cap, nc, kStC, a, tol2);
            }
            if ((sa < 0 && sb > 0) || (sa > 0 && sb < 0)) {
                const double t = sa / (sa - sb);
                double x[3];
                for (int c = 0; c < 3; c++) x[c] = a[c] + t * (b[c] - a[c]);
                if (no < kStV) {
                    out[no][0] = x[0];
                    out[no][1] = x[1];
                    out[no][2] = x[2];
                    no++;
                }
                st_add_unique(cap, nc, kStC, x, tol2);
            }
        }
        if (no >= 3) {
            for (int k = 0; k < no; k++)
                for (int c = 0; c < 3; c++) P.v[nf][k][c] = out[k][c];
            P.n[nf++] = no;
        }
    }
    P.nf = nf;
    if (nf == 0) return false;
    if (nc >= 3 && nf < kStF) {
        double ctr[3] = {0, 0, 0};
        for (int k = 0; k < nc; k++)
            for (int d = 0; d < 3; d++) ctr[d] += cap[k][d];
        for (int d = 0; d < 3; d++) ctr[d] /= nc;
        int far = 0;
        double best = -1;
        for (int k = 0; k < nc; k++) {
            const double e0 = cap[k][0] - ctr[0], e1 = cap[k][1] - ctr[1], e2 = cap[k][2] - ctr[2];
            const double l = e0 * e0 + e1 * e1 + e2 * e2;
            if (l > best) {
                best = l;
                far = k;
            }
        }
        if (best > 0) {
            const double u[3] = {cap[far][0] - ctr[0], cap[far][1] - ctr[1], cap[far][2] - ctr[2]};
            const double w[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2],
                                 nrm[0] * u[1] - nrm[1] * u[0]};
            double ang[kStC];
            for (int k = 0; k < nc; k++) {
                const double e[3] = {cap[k][0] - ctr[0], cap[k][1] - ctr[1], cap[k][2] - ctr[2]};
                ang[k] = atan2(st_dot(e, w), st_dot(e, u));
            }
            for (int i = 1; i < nc; i++) {  // insertion sort by angle
                const double a = ang[i], v0 = cap[i][0], v1 = cap[i][1], v2 = cap[i][2];
                int j = i - 1;
                while (j >= 0 && ang[j] > a) {
                    ang[j + 1] = ang[j];
                    cap[j + 1][0] = cap[j][0];
                    cap[j + 1][1] = cap[j][1];
                    cap[j + 1][2] = cap[j][2];
                    j--;
                }
                ang[j + 1] = a;
                cap[j + 1][0] = v0;
                cap[j + 1][1] = v1;
                cap[j + 1][2] = v2;
            }
            const int nn = nc < kStV ? nc : kStV;
            for (int k = 0; k < nn; k++)
                for (int c = 0; c < 3; c++) P.v[P.nf][k][c] = cap[k][c];
            P.n[P.nf++] = nn;
        }
    }
    return true;
}

// overlap volume of tetrahedra A and B (4 x 3 each); with cm, FFEA's centre
__device__ double st_overlap(const double (*A)[3], const double (*B)[3], double *cm)
{
    double ext = 0.0;
    for (int i = 0; i < 4; i++)
        for (int d = 0; d < 3; d++) {
            ext = fmax(ext, fabs(A[i][d] - A[0][d]));
            ext = fmax(ext, fabs(B[i][d] - A[0][d]));
        }
    const double tol2 = (1e-9 * ext) * (1e-9 * ext);
    StPolyh P;
    P.nf = 4;
    for (int f = 0; f < 4; f++) {
        P.n[f] = 3;
        for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) P.v[f][k][c] = A[c_tri[f][k]][c];
    }
    for (int f = 0; f < 4; f++) {
        // the half-space of B's face f (opposite vertex f) that holds B
        const double *t0 = B[c_tri[f][0]], *t1 = B[c_tri[f][1]], *t2 = B[c_tri[f][2]];
        const double u[3] = {t1[0] - t0[0], t1[1] - t0[1], t1[2] - t0[2]};
        const double v[3] = {t2[0] - t0[0], t2[1] - t0[1], t2[2] - t0[2]};
        double nrm[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        double off = st_dot(nrm, t0);
        if (st_dot(nrm, B[f]) > off) {
            nrm[0] = -nrm[0];
            nrm[1] = -nrm[1];
            nrm[2] = -nrm[2];
            off = -off;
        }
        if (!st_clip(P, nrm, off, tol2)) {
            if (cm) cm[0] = cm[1] = cm[2] = 0.0;
            return 0.0;
        }
    }
    double o[3] = {0, 0, 0};
    int nv = 0;
    for (int f = 0; f < P.nf; f++)
        for (int k = 0; k < P.n[f]; k++) {
            for (int d = 0; d < 3; d++) o[d] += P.v[f][k][d];
            nv++;
        }
    for (int d = 0; d < 3; d++) o[d] /= nv;
    double vol = 0.0;
    for (int f = 0; f < P.nf; f++)
        for (int k = 1; k + 1 < P.n[f]; k++) vol += fabs(st_tet_volume(o, P.v[f][0], P.v[f][k], P.v[f][k + 1]));
    if (cm) {
        double uniq[kStU][3];
        int nu = 0;
        for (int f = 0; f < P.nf; f++)
            for (int k = 0; k < P.n[f]; k++) st_add_unique(uniq, nu, kStU, P.v[f][k], tol2);
        cm[0] = cm[1] = cm[2] = 0.0;
        for (int u = 0; u < nu; u++)
            for (int d = 0; d < 3; d++) cm[d] += uniq[u][d];
        for (int d = 0; d < 3; d++) cm[d] *= 1.0 / nu;
    }
    return vol;
}

// One steric pair, f1 = A, f2 = B (the tetrahedra of the faces' elements):
// Face::getTetraIntersectionVolumeTotalGradientAndShapeFunctions
// (src/Face.cpp:473-514) and do_steric_interaction's scaling
// (src/VdW_solver.cpp:470-483).  false when they do not overlap; else adds
// the A side's (phi1 k dV/dr) or the B side's (-phi2 k dV/dr) node forces to
// out and sets vol = k V.
__device__ bool steric_pair(const double (*A)[3], const double (*B)[3], double dr, double k, bool a_side,
                            double out[4][3], double &vol)
{
    double cm[3];
    const double V = st_overlap(A, B, cm);
    if (V == 0) return false;
    // getLocalCoordinatesForLinTet (src/mat_vec_fns_II.cpp:725-734) of the
    // side's own tetrahedron
    const double (*T)[3] = a_side ? A : B;
    double phi[4];
    phi[0] = st_tet_volume(cm, T[1], T[2], T[3]);
    phi[1] = -st_tet_volume(cm, T[0], T[2], T[3]);
    phi[2] = st_tet_volume(cm, T[0], T[1], T[3]);
    phi[3] = -st_tet_volume(cm, T[0], T[1], T[2]);
    const double tv = st_tet_volume(T[0], T[1], T[2], T[3]);
    for (int i = 0; i < 4; i++) phi[i] /= tv;
    double g[3];
    for (int dir = 0; dir < 3; dir++) {
        double S[4][3];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) S[i][j] = B[i][j] + (j == dir ? dr : 0.0);
        const double vb = st_overlap(A, S, nullptr);
        g[dir] = (vb - V) / dr;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) S[i][j] = A[i][j] + (j == dir ? dr : 0.0);
        const double va = st_overlap(B, S, nullptr);
        g[dir] -= (va - V) / dr;
    }
    vol = V * k;
    for (int d = 0; d < 3; d++) g[d] *= k;
    for (int i = 0; i < 4; i++)
        for (int d = 0; d < 3; d++) out[i][d] += a_side ? phi[i] * g[d] : -1.0 * phi[i] * g[d];
    return true;
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

// The faces of the 27 cells around face i's cell for one warp: s_beg / s_pre
// hold each cell's first sorted slot and the candidates before it; returns
// the number of candidates.
__device__ __forceinline__ int warp_cells(int ci, int nx, int ny, int nz, const int *__restrict__ start,
                                          const int *__restrict__ block, long long ncell, int nblocks, int lane,
                                          int *s_beg, int *s_pre)
{
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
        s_beg[lane] = beg;
        s_pre[lane] = incl - len;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 26);
    __syncwarp();
    return total;
}

// candidate k (< total) of the warp's cells
__device__ __forceinline__ int warp_candidate(int k, const int *s_beg, const int *s_pre, const int *__restrict__ sorted)
{
    int c = 0;
    while (c < 26 && s_pre[c + 1] <= k) c++;
    return sorted[s_beg[c] + (k - s_pre[c])];
}

// consider_interaction's checks for the types other than lennard-jones
// (src/VdW_solver.cpp:359-388): faces in front of each other, and within
// one blob (with self-interaction on) no shared node.  Symmetric in (i, j).
// With periodic corrections, cs = blob_corr[blob of A][blob of G] enters the
// separation (c_G - c_A - cs; FFEA's c2 - c1 - blob_corr[b1][b2] with its
// faces in either order, blob_corr being antisymmetric).
__device__ __forceinline__ bool steric_type_ok(const double *A, const double *G, bool same_blob, int inc_self,
                                               const int *ni, const int *nj, const double *cs)
{
    double sa = 0.0, sb = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double sep = (1.0 / 3.0) * (G[d] + G[3 + d] + G[6 + d]) - (1.0 / 3.0) * (A[d] + A[3 + d] + A[6 + d]);
        if (cs) sep -= cs[d];
        sa += sep * A[9 + d];
        sb += sep * G[9 + d];
    }
    if (sa < 0 && sb > 0) return false;
    if (inc_self && same_blob) {
        if (ni[3] == nj[3]) return false;
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int w = 0; w < 4; w++)
                if (ni[u] == nj[w]) return false;
    }
    return true;
}

// the element tetrahedron of face f: its corners, then the fourth node
__device__ __forceinline__ void face_tet(const double *__restrict__ geo, int f, double T[4][3])
{
    const double *g = geo + 16 * (long long)f;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int d = 0; d < 3; d++) T[k][d] = g[3 * k + d];
#pragma unroll
    for (int d = 0; d < 3; d++) T[3][d] = g[13 + d];
}

constexpr int kStericWarps = 4;  // warps (faces) per CTA of k_steric

// The steric part of the steric types, one warp per face i in cell order:
// every partner j of the 27 cells that consider_interaction admits and whose
// element tetrahedron's bounding box meets i's is queued; the queue is
// evaluated a lane per pair, each pair as (lower index, higher index) = FFEA's
// (f1, f2), so both sides compute the same overlap.  Face i's side of the
// forces goes to fforce (12 values, written here: this kernel runs first), the
// partners that overlapped to i's steric list (k_pairs skips them), the energy
// and the pair count from the side with the lower index.
__global__ void __launch_bounds__(32 * kStericWarps) k_steric(
    const double *__restrict__ geo, const int *__restrict__ sorted, const int *__restrict__ cell,
    const int *__restrict__ start, const int *__restrict__ block, long long ncell, int nblocks, int nx, int ny,
    int nz, const int *__restrict__ fblob, const int *__restrict__ corner, int num_blobs, int inc_self,
    double steric_factor, double steric_dr, const double *__restrict__ corr, double *__restrict__ fforce,
    int *__restrict__ stlist, int *__restrict__ stcnt, double *__restrict__ energy, unsigned long long *stats)
{
    __shared__ int s_pre[kStericWarps][28];
    __shared__ int s_beg[kStericWarps][27];
    __shared__ int s_q[kStericWarps][64];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long w = (long long)blockIdx.x * kStericWarps + wi;
    if (w >= block[nblocks]) return;  // warp-uniform
    if (stats[3]) return;             // the call fails (a cell too full to sort)
    const int i = sorted[w];
    const int total = warp_cells(cell[i], nx, ny, nz, start, block, ncell, nblocks, lane, s_beg[wi], s_pre[wi]);
    const double *A = geo + 16 * (long long)i;
    const int bi = fblob[i];
    int ni[4];
#pragma unroll
    for (int u = 0; u < 4; u++) ni[u] = corner[4 * i + u];
    double Ti[4][3];
    face_tet(geo, i, Ti);
    double lo_i[3], hi_i[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        lo_i[d] = fmin(fmin(Ti[0][d], Ti[1][d]), fmin(Ti[2][d], Ti[3][d]));
        hi_i[d] = fmax(fmax(Ti[0][d], Ti[1][d]), fmax(Ti[2][d], Ti[3][d]));
    }
    double out[4][3];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int d = 0; d < 3; d++) out[u][d] = 0.0;
    int listed = 0;
    unsigned long long npairs = 0;
    auto evaluate = [&](bool have, int j) {
        bool hit = false;
        if (have) {
            double Tj[4][3], vol;
            face_tet(geo, j, Tj);
            if (i < j) {
                // periodic: f2's tetrahedron minus blob_corr[b1][b2]
                // (Face::getTetraIntersectionVolumeTotalGradientAndShapeFunctions,
                // src/Face.cpp:517-531)
                if (corr) {
                    const double *c = corr + 3 * ((long long)bi * num_blobs + fblob[j]);
#pragma unroll
                    for (int u = 0; u < 4; u++)
#pragma unroll
                        for (int d = 0; d < 3; d++) Tj[u][d] -= c[d];
                }
                hit = steric_pair(Ti, Tj, steric_dr, steric_factor, true, out, vol);
            } else {
                double Tb[4][3];
                const double *c = corr ? corr + 3 * ((long long)fblob[j] * num_blobs + bi) : nullptr;
#pragma unroll
                for (int u = 0; u < 4; u++)
#pragma unroll
                    for (int d = 0; d < 3; d++) Tb[u][d] = c ? Ti[u][d] - c[d] : Ti[u][d];
                hit = steric_pair(Tj, Tb, steric_dr, steric_factor, false, out, vol);
            }
            if (hit && i < j) {
                atomicAdd(&energy[bi * num_blobs + fblob[j]], vol);
                npairs++;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int slot = listed + __popc(m & ((1u << lane) - 1u));
            if (slot < FFEA_GPU_SSINT_MAX_STERIC_PARTNERS) stlist[FFEA_GPU_SSINT_MAX_STERIC_PARTNERS * i + slot] = j;
        }
        listed += __popc(m);
    };
    int qn = 0;  // warp-uniform queue length, < 64
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        bool ok = false;
        int j = -1;
        if (k < total) {
            j = warp_candidate(k, s_beg[wi], s_pre[wi], sorted);
            const double *G = geo + 16 * (long long)j;
            const bool same = bi == fblob[j];
            ok = j != i && (inc_self || !same) && !(A[9] * G[9] + A[10] * G[10] + A[11] * G[11] > 0.0);
            // periodic: the partner as seen from face i, shifted by
            // -blob_corr[bi][bj]
            const double *cs = corr ? corr + 3 * ((long long)bi * num_blobs + fblob[j]) : nullptr;
            if (ok) {
                int nj[4];
#pragma unroll
                for (int u = 0; u < 4; u++) nj[u] = corner[4 * j + u];
                ok = steric_type_ok(A, G, same, inc_self, ni, nj, cs);
            }
            if (ok) {  // bounding boxes of the two tetrahedra
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const double sh = cs ? cs[d] : 0.0;
                    const double a0 = G[d] - sh, a1 = G[3 + d] - sh, a2 = G[6 + d] - sh, a3 = G[13 + d] - sh;
                    const double lo = fmin(fmin(a0, a1), fmin(a2, a3)), hi = fmax(fmax(a0, a1), fmax(a2, a3));
                    if (hi < lo_i[d] || lo > hi_i[d]) ok = false;
                }
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (ok) s_q[wi][qn + __popc(m & ((1u << lane) - 1u))] = j;
        qn += __popc(m);
        __syncwarp();
        if (qn >= 32) {
            evaluate(true, s_q[wi][lane]);
            const int rest = qn - 32;
            const int moved = lane < rest ? s_q[wi][32 + lane] : 0;
            __syncwarp();
            if (lane < rest) s_q[wi][lane] = moved;
            qn = rest;
            __syncwarp();
        }
    }
    if (qn > 0) evaluate(lane < qn, lane < qn ? s_q[wi][lane] : -1);
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
        for (int d = 0; d < 3; d++) out[u][d] = warp_sum_d(out[u][d]);
    unsigned long long np = npairs;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) np += __shfl_xor_sync(0xffffffffu, np, o);
    if (lane == 0) {
        if (np) atomicAdd(&stats[0], np);
        stcnt[i] = min(listed, FFEA_GPU_SSINT_MAX_STERIC_PARTNERS);
        if (listed > FFEA_GPU_SSINT_MAX_STERIC_PARTNERS) atomicAdd(&stats[4], 1ull);
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int d = 0; d < 3; d++) fforce[12 * (long long)i + 3 * u + d] = out[u][d];
    }
}

// One warp per face i (faces taken in cell order): the candidates of the 27
// cells around i's cell are numbered 0..total-1 through a prefix sum over the
// cells, lane l tests candidates l, l + 32, ..., and the partners that pass
// are evaluated from a per-warp queue.  Each lane keeps face i's side of its
// pairs; a fixed shuffle tree sums the lanes.  POT: Lennard-Jones or the soft
// potential; STERIC: the steric types' pair checks apply, the partners of i's
// steric list are skipped (k_steric gave them the steric force) and the
// forces add to what k_steric wrote.
template <int POT, bool STERIC>
__global__ void __launch_bounds__(32 * kPairWarps) k_pairs(
    const double *__restrict__ geo, const int *__restrict__ cell, const int *__restrict__ sorted,
    const int *__restrict__ start, const int *__restrict__ block, long long ncell, int nblocks, int nx, int ny,
    int nz, const int *__restrict__ fblob, const int *__restrict__ ftype, const double *__restrict__ emin,
    const double *__restrict__ rmin, const double *__restrict__ k0, const int *__restrict__ corner,
    const int *__restrict__ stlist, const int *__restrict__ stcnt, int num_types, int num_blobs, int inc_self,
    const double *__restrict__ corr, double *__restrict__ fforce, double *__restrict__ energy,
    unsigned long long *stats)
{
    __shared__ int s_pre[kPairWarps][28];
    __shared__ int s_beg[kPairWarps][27];
    __shared__ int s_q[kPairWarps][64];
    __shared__ int s_st[kPairWarps][FFEA_GPU_SSINT_MAX_STERIC_PARTNERS];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long w = (long long)blockIdx.x * kPairWarps + wi;
    if (w >= block[nblocks]) return;  // warp-uniform; faces outside the box are not binned
    if (stats[3]) return;             // a cell too full to sort: the call fails, nothing to evaluate
    const int i = sorted[w];
    const int total = warp_cells(cell[i], nx, ny, nz, start, block, ncell, nblocks, lane, s_beg[wi], s_pre[wi]);
    int nst = 0;
    int ni[4] = {0, 0, 0, 0};
    if constexpr (STERIC) {
        nst = stcnt[i];
        if (lane < nst) s_st[wi][lane] = stlist[FFEA_GPU_SSINT_MAX_STERIC_PARTNERS * i + lane];
#pragma unroll
        for (int u = 0; u < 4; u++) ni[u] = corner[4 * i + u];
        __syncwarp();
    }
    double A[13];
#pragma unroll
    for (int k = 0; k < 13; k++) A[k] = geo[16 * (long long)i + k];
    const int bi = fblob[i], ti = ftype[i];
    double out[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
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
            double en;
            if (corr) {
                // periodic: f1's corners minus blob_corr[b2][b1]
                // (Face::barycentric_calc_point_f2, src/Face.cpp:271-277)
                const double *c = corr + 3 * ((long long)fblob[j] * num_blobs + bi);
                double As[13];
#pragma unroll
                for (int q = 0; q < 13; q++) As[q] = q < 9 ? A[q] - c[q % 3] : A[q];
                en = pot_pair<POT, true>(As, B, emin[tt], rmin[tt], k0 ? k0[tt] : 0.0, out);
            } else {
                en = pot_pair<POT, true>(A, B, emin[tt], rmin[tt], k0 ? k0[tt] : 0.0, out);
            }
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
            if (corr) {
                const double *c = corr + 3 * ((long long)bi * num_blobs + fblob[j]);
#pragma unroll
                for (int q = 0; q < 9; q++) B[q] -= c[q % 3];
            }
            pot_pair<POT, false>(B, A, emin[tt], rmin[tt], k0 ? k0[tt] : 0.0, out);
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
            j = warp_candidate(k, s_beg[wi], s_pre[wi], sorted);
            const double *G = geo + 16 * (long long)j;
            ok = j != i && (inc_self || bi != fblob[j]) && !(A[9] * G[9] + A[10] * G[10] + A[11] * G[11] > 0.0);
            if constexpr (STERIC) {
                if (ok) {
                    int nj[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) nj[u] = corner[4 * j + u];
                    ok = steric_type_ok(A, G, bi == fblob[j], inc_self, ni, nj,
                                        corr ? corr + 3 * ((long long)bi * num_blobs + fblob[j]) : nullptr);
                }
                for (int t = 0; ok && t < nst; t++)
                    if (s_st[wi][t] == j) ok = false;  // the steric force applied instead
            }
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
        for (int k = 0; k < 4; k++)
#pragma unroll
            for (int d = 0; d < 3; d++) {
                double *f = &fforce[12 * (long long)i + 3 * k + d];
                *f = STERIC ? *f + out[k][d] : out[k][d];
            }
    }
}

// The sticky xz walls (VdW_solver::solve_sticky_wall / do_sticky_xz_interaction,
// src/VdW_solver.cpp:216-235, 396-456), after the pair pass: every face whose
// cell lies in the grid's bottom (y = 0) or top (y = ny - 1) row and faces
// that wall feels a y force from it, the Lennard-Jones factor of its own type
// at the height of its Gauss points, added to its corners (the energy is not
// recorded, as in FFEA).  One thread per face.
__global__ void k_sticky(const double *__restrict__ geo, const int *__restrict__ cell, int na,
                         const int *__restrict__ ftype, const double *__restrict__ emin,
                         const double *__restrict__ rmin, int num_types, int ny, int nz, double h,
                         double *__restrict__ fforce)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= na || cell[i] < 0) return;
    const int cy = (cell[i] / nz) % ny;
    if (cy != 0 && cy != ny - 1) return;
    const bool bottom = cy == 0;
    const double *g = geo + 16 * (long long)i;
    if ((bottom && g[10] > 0) || (!bottom && g[10] < 0)) return;
    const double y_wall = bottom ? 0.0 : h * ny;
    const int tt = ftype[i] * num_types + ftype[i];
    const double r6 = pow(rmin[tt], 6.0), em = emin[tt];
    double py[3], fm[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        py[k] = eta(k, 0) * g[1] + eta(k, 1) * g[4] + eta(k, 2) * g[7];
        const double r = py[k] - y_wall;
        fm[k] = -(12 * r6 * em * (pow(r, -7.0) - r6 * pow(r, -13.0)));
    }
    const double asq = g[12] * g[12];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        double fy = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int l = 0; l < 3; l++) fy += kW * kW * eta(l, j) * fm[k < l ? k : l];
        fforce[12 * (long long)i + 3 * j + 1] += fy * asq;
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
        if (cell[fc / 4] < 0) continue;
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
    const int stype = d->ssint_type;
    if (stype < FFEA_GPU_SSINT_LJ || stype > FFEA_GPU_SSINT_GENSOFT) return fail("unknown ssint_type %d", stype);
    const bool steric = stype != FFEA_GPU_SSINT_LJ;
    if (steric && d->num_faces && !d->face_apex) return fail("the steric types need face_apex (Face::n[3] per face)");
    if (steric && !(d->steric_dr > 0.0)) return fail("steric_dr must be positive");
    if (stype == FFEA_GPU_SSINT_GENSOFT && !d->k0) return fail("gensoft needs k0");
    std::vector<int> corner, blob, type;
    for (int f = 0; f < d->num_faces; f++) {
        if (d->face_type[f] < 0) continue;  // not ssint-active: not in the pool (src/Blob.cpp:1642-1648)
        if (d->face_type[f] >= d->num_types) return fail("face %d: interaction type %d >= num_types", f, d->face_type[f]);
        if (d->face_blob[f] < 0 || d->face_blob[f] >= d->num_blobs) return fail("face %d: blob %d out of range", f, d->face_blob[f]);
        for (int k = 0; k < 4; k++) {
            const int n = k < 3 ? d->faces[3 * f + k] : (steric ? d->face_apex[f] : -1);
            if (n < -1 || n >= d->num_nodes || (n < 0 && k < 3) || (n < 0 && steric))
                return fail("face %d: node %d out of range", f, n);
            corner.push_back(n);
        }
        blob.push_back(d->face_blob[f]);
        type.push_back(d->face_type[f]);
    }
    const int na = (int)blob.size();
    // node -> (active face, node of the face) entries in face order (the
    // fourth node only for the steric types)
    std::vector<int> ptr(d->num_nodes + 1, 0), ent;
    for (int i = 0; i < 4 * na; i++)
        if (corner[i] >= 0) ptr[corner[i] + 1]++;
    for (int n = 0; n < d->num_nodes; n++) ptr[n + 1] += ptr[n];
    ent.resize((size_t)ptr[d->num_nodes]);
    {
        std::vector<int> fill(ptr.begin(), ptr.end() - 1);
        for (int i = 0; i < 4 * na; i++)
            if (corner[i] >= 0) ent[fill[corner[i]]++] = i;
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
    s->type = stype;
    s->steric_factor = d->steric_factor;
    s->steric_dr = d->steric_dr;
    s->h = d->cell_size;
    s->ncell = ncell;
    s->nblocks = (int)((ncell + kScanBlock - 1) / kScanBlock);
    const int T2 = d->num_types * d->num_types;
    int rc = FFEA_GPU_OK;
    auto run = [&]() -> int {
        // blocking: its kernels must follow the uploads below, which run on
        // the legacy default stream and may still be in flight when
        // cudaMemcpy returns
        SSINT_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamDefault));
        if (dalloc(&s->d_corner, 4 * (size_t)na) || dalloc(&s->d_blob, na) || dalloc(&s->d_type, na) ||
            dalloc(&s->d_geo, 16 * (size_t)na) || dalloc(&s->d_cell, na) || dalloc(&s->d_fforce, 12 * (size_t)na) ||
            dalloc(&s->d_count, ncell) || dalloc(&s->d_start, ncell) || dalloc(&s->d_block, s->nblocks + 1) ||
            dalloc(&s->d_sorted, na) || dalloc(&s->d_node_ptr, d->num_nodes + 1) ||
            dalloc(&s->d_node_ent, ent.size()) || dalloc(&s->d_emin, T2) || dalloc(&s->d_rmin, T2) ||
            dalloc(&s->d_pos, 3 * (size_t)d->num_nodes) || dalloc(&s->d_force, 3 * (size_t)d->num_nodes) ||
            dalloc(&s->d_energy, (size_t)d->num_blobs * d->num_blobs) || dalloc(&s->d_stats, 5) ||
            dalloc(&s->d_large, (size_t)na / (kSortSmall + 1) + 1))
            return FFEA_GPU_ERROR;
        if (steric && (dalloc(&s->d_stlist, (size_t)FFEA_GPU_SSINT_MAX_STERIC_PARTNERS * na) ||
                       dalloc(&s->d_stcnt, na)))
            return FFEA_GPU_ERROR;
        if (stype == FFEA_GPU_SSINT_GENSOFT && dalloc(&s->d_k0, T2)) return FFEA_GPU_ERROR;
        if (na) {
            SSINT_CUDA(cudaMemcpy(s->d_corner, corner.data(), sizeof(int) * 4 * na, cudaMemcpyHostToDevice));
            SSINT_CUDA(cudaMemcpy(s->d_blob, blob.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
            SSINT_CUDA(cudaMemcpy(s->d_type, type.data(), sizeof(int) * na, cudaMemcpyHostToDevice));
        }
        if (!ent.empty())
            SSINT_CUDA(cudaMemcpy(s->d_node_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice));
        SSINT_CUDA(cudaMemcpy(s->d_node_ptr, ptr.data(), sizeof(int) * (d->num_nodes + 1), cudaMemcpyHostToDevice));
        SSINT_CUDA(cudaMemcpy(s->d_emin, d->emin, sizeof(double) * T2, cudaMemcpyHostToDevice));
        SSINT_CUDA(cudaMemcpy(s->d_rmin, d->rmin, sizeof(double) * T2, cudaMemcpyHostToDevice));
        if (s->d_k0) SSINT_CUDA(cudaMemcpy(s->d_k0, d->k0, sizeof(double) * T2, cudaMemcpyHostToDevice));
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
                    s->d_pos, s->d_force, s->d_energy, s->d_stats, s->d_large, s->d_stlist, s->d_stcnt, s->d_k0,
                    s->d_corr};
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
    SSINT_CUDA(cudaMemsetAsync(s->d_stats, 0, sizeof(unsigned long long) * 5, st));
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
    const int pw = (na + kPairWarps - 1) / kPairWarps;
    if (s->type != FFEA_GPU_SSINT_LJ)
        k_steric<<<(na + kStericWarps - 1) / kStericWarps, 32 * kStericWarps, 0, st>>>(
            s->d_geo, s->d_sorted, s->d_cell, s->d_start, s->d_block, s->ncell, s->nblocks, s->nx, s->ny, s->nz,
            s->d_blob, s->d_corner, s->num_blobs, s->inc_self, s->steric_factor, s->steric_dr,
            s->has_corr ? s->d_corr : nullptr, s->d_fforce, s->d_stlist, s->d_stcnt, energy, s->d_stats);
#define SSINT_PAIRS(POT, STERIC)                                                                                   \
    k_pairs<POT, STERIC><<<pw, 32 * kPairWarps, 0, st>>>(                                                           \
        s->d_geo, s->d_cell, s->d_sorted, s->d_start, s->d_block, s->ncell, s->nblocks, s->nx, s->ny, s->nz,        \
        s->d_blob, s->d_type, s->d_emin, s->d_rmin, s->d_k0, s->d_corner, s->d_stlist, s->d_stcnt, s->num_types,     \
        s->num_blobs, s->inc_self, s->has_corr ? s->d_corr : nullptr, s->d_fforce, energy, s->d_stats)
    if (s->type == FFEA_GPU_SSINT_LJ) SSINT_PAIRS(POT_LJ, false);
    else if (s->type == FFEA_GPU_SSINT_LJSTERIC) SSINT_PAIRS(POT_LJ, true);
    else if (s->type == FFEA_GPU_SSINT_GENSOFT) SSINT_PAIRS(POT_SOFT, true);
#undef SSINT_PAIRS
    if (s->sticky)
        k_sticky<<<fb, 128, 0, st>>>(s->d_geo, s->d_cell, na, s->d_type, s->d_emin, s->d_rmin, s->num_types, s->ny,
                                     s->nz, s->h, s->d_fforce);
    k_node_gather<<<(s->num_nodes + 255) / 256, 256, 0, st>>>(s->d_node_ptr, s->d_node_ent, s->num_nodes,
                                                              s->d_fforce, s->d_cell, force);
    SSINT_CUDA(cudaGetLastError());
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_ssint_set_pbc(ffea_gpu_ssint_t *s, const double *blob_corr)
{
    if (!s) return fail("ffea_gpu_ssint_set_pbc: null handle");
    if (!blob_corr) {
        s->has_corr = 0;
        return FFEA_GPU_OK;
    }
    const size_t n = 3 * (size_t)s->num_blobs * s->num_blobs;
    if (!s->d_corr) SSINT_CUDA(cudaMalloc(&s->d_corr, sizeof(double) * n));
    // ordered on the handle's stream before the next pass
    SSINT_CUDA(cudaMemcpyAsync(s->d_corr, blob_corr, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
    SSINT_CUDA(cudaStreamSynchronize(s->stream));
    s->has_corr = 1;
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_ssint_set_sticky_wall(ffea_gpu_ssint_t *s, int32_t enable)
{
    if (!s) return fail("ffea_gpu_ssint_set_sticky_wall: null handle");
    if (enable && s->ny < 2)
        return fail("the sticky wall needs at least two rows of cells in y (FFEA's row loop would not end)");
    s->sticky = enable ? 1 : 0;
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_ssint_blob_corr(int32_t num_blobs, const double *centroids, const double box[3],
                                        double *blob_corr)
{
    if (num_blobs < 0 || (num_blobs > 0 && (!centroids || !box || !blob_corr)))
        return fail("ffea_gpu_ssint_blob_corr: null argument");
    for (int i = 0; i < num_blobs; ++i) {
        for (int d = 0; d < 3; d++) blob_corr[3 * ((size_t)i * num_blobs + i) + d] = 0.0;
        for (int j = i + 1; j < num_blobs; ++j)
            for (int d = 0; d < 3; d++) {
                const double v = box[d] * floor((centroids[3 * j + d] - centroids[3 * i + d] + 0.5 * box[d]) / box[d]);
                blob_corr[3 * ((size_t)i * num_blobs + j) + d] = v;
                blob_corr[3 * ((size_t)j * num_blobs + i) + d] = -1 * v;
            }
    }
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_ssint_synchronize(ffea_gpu_ssint_t *s, int64_t *pairs)
{
    if (!s) return fail("ffea_gpu_ssint_synchronize: null handle");
    unsigned long long st[5] = {0, 0, 0, 0, 0};
    SSINT_CUDA(cudaMemcpyAsync(st, s->d_stats, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
    SSINT_CUDA(cudaStreamSynchronize(s->stream));
    if (pairs) *pairs = (int64_t)st[0];
    if (st[1]) return fail("%llu face centroids lie outside the interaction grid (FFEA reports this as an error)", st[1]);
    if (st[3])
        return fail("%llu grid cells hold more than %d faces each: the interaction grid is too coarse for this mesh "
                    "(use more, smaller cells)", st[3], kSortMax);
    if (st[4])
        return fail("%llu faces' tetrahedra overlap more than %d others (their steric partners beyond that are "
                    "not excluded from the Lennard-Jones or soft pairs)", st[4], FFEA_GPU_SSINT_MAX_STERIC_PARTNERS);
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
