// noalloc.cu -- strain / kinetic energy of one blob without any device allocation.
//
// Some callers cannot allocate device memory at the point where they want a
// measurement: a host code that calls this from inside its own time-step loop
// (where a cudaMalloc would implicitly synchronise the device and fragment a
// memory pool the host manages itself), or a caller whose device memory is
// owned by another allocator.  ffea_gpu_energies_noalloc serves them: the
// caller passes device buffers for inputs and output, and the scratch the
// reduction needs (one pair of partial sums per 128-element tile and a
// completion counter) lives in the file-scope array below, which every GPU
// that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"

namespace ffea {
void set_last_error(const char *msg);  // api.cu
}

namespace {

constexpr int kTile = 128;                 // elements per CTA
constexpr int kMaxTiles = 16384;           // => at most kTile * kMaxTiles = 2,097,152 elements per call

struct NoAllocScratch {
    double partials[2 * kMaxTiles];        // strain, kinetic per tile (256 KiB)
    unsigned int counter;                  // CTAs finished; must be 0 when a call starts
};

// Device-side scratch.  In host code `g_scratch` names a host-side stand-in,
// not a device address: the kernel is given the address returned by
// cudaGetSymbolAddress for the current device.
static __device__ __align__(256) NoAllocScratch g_scratch;

std::mutex g_mu;
std::vector<NoAllocScratch *> g_scratch_ptr;  // per device ordinal, set up on first use

// reported through ffea_gpu_last_error like every other entry point
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

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per element, FP64: rest state from rest_pos (mat3_invert, src/mat_vec_fns.cpp:148-175),
// F = (J_inv_0 J)^T, strain energy V0 [G (F:F - 3) + C/2 (J^2 - 1) - (C + 2G) ln J] and,
// for the mass path, v^T M_e v (src/Blob.cpp:1385-1427); halves applied at the end.
__global__ void __launch_bounds__(kTile) k_energies_noalloc(const double *pos, const double *vel, const int32_t *topo,
                                                            const double *rest_pos, const double *material, int32_t E,
                                                            int32_t mass_path, NoAllocScratch *scratch, double *out)
{
    __shared__ double red[2][kTile / 32];
    __shared__ int is_last;
    const int e = blockIdx.x * kTile + threadIdx.x;
    double se = 0.0, ke = 0.0;
    if (e < E) {
        const int32_t *t = topo + 10 * (size_t)e;
        double J[3][3], J0[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                J[r][c] = pos[3 * (size_t)t[r + 1] + c] - pos[3 * (size_t)t[0] + c];
                J0[r][c] = rest_pos[3 * (size_t)t[r + 1] + c] - rest_pos[3 * (size_t)t[0] + c];
            }
        double mi[3][3];
        mi[0][0] = J0[2][2] * J0[1][1] - J0[2][1] * J0[1][2];
        mi[0][1] = J0[2][1] * J0[0][2] - J0[2][2] * J0[0][1];
        mi[0][2] = J0[1][2] * J0[0][1] - J0[1][1] * J0[0][2];
        mi[1][0] = J0[2][0] * J0[1][2] - J0[2][2] * J0[1][0];
        mi[1][1] = J0[2][2] * J0[0][0] - J0[2][0] * J0[0][2];
        mi[1][2] = J0[1][0] * J0[0][2] - J0[1][2] * J0[0][0];
        mi[2][0] = J0[2][1] * J0[1][0] - J0[2][0] * J0[1][1];
        mi[2][1] = J0[2][0] * J0[0][1] - J0[2][1] * J0[0][0];
        mi[2][2] = J0[1][1] * J0[0][0] - J0[1][0] * J0[0][1];
        const double det0 = J0[0][0] * mi[0][0] + J0[1][0] * mi[0][1] + J0[2][0] * mi[0][2];
        const double inv0 = 1.0 / det0;
        const double vol0 = fabs(det0) / 6.0;
        const double det = J[0][0] * (J[2][2] * J[1][1] - J[2][1] * J[1][2]) +
                           J[1][0] * (J[2][1] * J[0][2] - J[2][2] * J[0][1]) +
                           J[2][0] * (J[1][2] * J[0][1] - J[1][1] * J[0][2]);
        const double vol = fabs(det) / 6.0;
        double ff = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                const double F = J[0][i] * mi[j][0] * inv0 + J[1][i] * mi[j][1] * inv0 + J[2][i] * mi[j][2] * inv0;
                ff += F * F;
            }
        const double rho = material[5 * (size_t)e], G = material[5 * (size_t)e + 3], Eb = material[5 * (size_t)e + 4];
        const double C = Eb - (2.0 / 3.0) * G;
        const double t1 = vol / vol0;
        se = vol0 * (G * (ff - 3) + 0.5 * C * (t1 * t1 - 1) - (C + 2 * G) * log(t1));
        if (mass_path && vel) {
            for (int i = 0; i < 3; i++)
                for (int a = 0; a < 4; a++) {
                    double mv = 0.0;
                    for (int b = 0; b < 4; b++) mv += (a == b ? .1 : .05) * vel[3 * (size_t)t[b] + i];
                    ke += vel[3 * (size_t)t[a] + i] * mv * (vol0 * rho);
                }
        }
    }
    // fixed-order CTA sum, one partial pair per tile
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    se = warp_sum(se);
    ke = warp_sum(ke);
    if (lane == 0) {
        red[0][warp] = se;
        red[1][warp] = ke;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < kTile / 32; w++) {
            s0 += red[0][w];
            s1 += red[1][w];
        }
        scratch->partials[2 * blockIdx.x] = s0;
        scratch->partials[2 * blockIdx.x + 1] = s1;
        __threadfence();
        const unsigned int prev = atomicAdd(&scratch->counter, 1u);
        is_last = prev == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    // the last CTA sums the tiles in a fixed order (lane-strided, then a butterfly)
    __threadfence();
    if (warp == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (unsigned int tl = lane; tl < gridDim.x; tl += 32) {
            s0 += __ldcg(&scratch->partials[2 * tl]);
            s1 += __ldcg(&scratch->partials[2 * tl + 1]);
        }
        s0 = warp_sum(s0);
        s1 = warp_sum(s1);
        if (lane == 0) {
            out[0] = 0.5 * s0;
            out[1] = 0.5 * s1;
            scratch->counter = 0;
        }
    }
}

}  // namespace

extern "C" int ffea_gpu_energies_noalloc(const double *pos, const double *vel, const int32_t *topology,
                                         const double *rest_pos, const double *material, int32_t num_elements,
                                         int32_t solver, double *out, void *stream)
{
    if (!pos || !topology || !rest_pos || !material || !out) return fail("null device pointer");
    if (num_elements <= 0) return fail("num_elements must be positive");
    if ((int64_t)num_elements > (int64_t)kTile * kMaxTiles)
        return fail("num_elements %d exceeds the maximum %d of the static scratch", num_elements, kTile * kMaxTiles);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail("cudaGetDevice: %s", cudaGetErrorString(e));
    NoAllocScratch *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if ((int)g_scratch_ptr.size() <= dev) g_scratch_ptr.resize(dev + 1, nullptr);
        if (!g_scratch_ptr[dev]) {
            // set-up, once per device, with that device current
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess) return fail("cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_scratch_ptr[dev] = static_cast<NoAllocScratch *>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the completion counter must start at zero
    e = cudaMemsetAsync(&scratch->counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return fail("cudaMemsetAsync: %s", cudaGetErrorString(e));
    const int tiles = (num_elements + kTile - 1) / kTile;
    k_energies_noalloc<<<tiles, kTile, 0, s>>>(pos, vel, topology, rest_pos, material, num_elements,
                                               solver != FFEA_GPU_SOLVER_NOMASS ? 1 : 0, scratch, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail("k_energies_noalloc launch: %s", cudaGetErrorString(e));
    return FFEA_GPU_OK;
}
