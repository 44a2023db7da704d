// api.cu -- the extern "C" boundary (include/ffea_gpu.h).
//
// A handle owns one packed batch of blobs in HBM, one CUDA stream and, in
// graph mode, one instantiated CUDA graph per step:
//   elements -> assemble -> nodes -> cg (persistent, cooperative) -> euler
// The whole CG solve of every blob runs inside one cooperative launch that
// iterates until each blob has converged, so a step (and a run of steps)
// needs no host synchronisation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ffea_gpu.h"
#include "host_build.h"
#include "kernels.h"

using namespace ffea;

namespace {

thread_local std::string g_last_error;

int fail(const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return FFEA_GPU_ERROR;
}

#define CK(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) return fail("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                  \
    } while (0)

struct DeviceArena {
    std::vector<void *> ptrs;
    ~DeviceArena()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T>
    cudaError_t alloc(T *&out, size_t count)
    {
        void *p = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) return e;
        ptrs.push_back(p);
        e = cudaMemset(p, 0, bytes);
        out = static_cast<T *>(p);
        return e;
    }
    cudaError_t alloc_bytes(void *&out, size_t bytes)
    {
        char *p = nullptr;
        cudaError_t e = alloc(p, bytes);
        out = p;
        return e;
    }
};

template <typename T>
cudaError_t upload(DeviceArena &A, T *&dst, const std::vector<T> &src)
{
    cudaError_t e = A.alloc(dst, src.size());
    if (e != cudaSuccess || src.empty()) return e;
    return cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// FP64 host values as T of the batch's precision (float in PREC_MIXED)
cudaError_t upload_t(DeviceArena &A, void *&dst, const std::vector<double> &src, int precision)
{
    if (precision == PREC_FP64) {
        double *p = nullptr;
        cudaError_t e = upload(A, p, src);
        dst = p;
        return e;
    }
    std::vector<float> f(src.begin(), src.end());
    float *p = nullptr;
    cudaError_t e = upload(A, p, f);
    dst = p;
    return e;
}

// process-wide jump table per device (for ffea_gpu_rng_draws)
std::mutex g_table_mu;
std::vector<mrg::JumpMat *> g_tables;

}  // namespace

namespace ffea {
// lets the other translation units of the library report through ffea_gpu_last_error
void set_last_error(const char *msg) { g_last_error = msg; }
}  // namespace ffea

struct ffea_gpu {
    HostBatch host;
    DeviceBatch dev;
    DeviceArena arena;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t step_exec = nullptr;
    cudaGraphExec_t step_exec_coarse = nullptr;  // the step with the coarse-space refresh
    int64_t fixed_per_step_coarse = 0;
    int coarse_every = 10;                       // steps between coarse-space refreshes
    int64_t steps_done = 0;
    int graph_mode = 1;
    int timing = 0;
    double phase_ms[5] = {0, 0, 0, 0, 0};
    double kernel_ms[FFEA_GPU_NUM_KERNEL_TIMES] = {};  // noise, elements, assembly, coarse, nodes, CG (+ update), 0
    cudaEvent_t ev[FFEA_GPU_NUM_KERNEL_TIMES + 1] = {};
    int64_t fixed_per_step = 0;  // kernels of a step graph outside the CG loop
    size_t tsize = 4;
    // node I/O in the reference's node order, reconstructed on the device:
    // per original node (row, -1) for a corner node, (row_a, row_b) for an
    // edge midpoint (its edge in the last element that lists it), (-1, -1)
    // for a node of no element; per blob the offset into these arrays
    std::vector<int64_t> io_off;
    int2 *io_src = nullptr;
    std::vector<int2> io_src_host;  // the same map on the host (external-force folding)
    std::vector<double> ext_host;   // external forces per row (3 per row, folded), mirror of dev.ext
    std::vector<uint32_t> stream_gen;  // per RNG stream: generation of its state (mirror of dev.stream_gen)
    double *io_secvel = nullptr;  // secondary-node velocities (mass blobs keep them; NoMass report 0)
    double *io_stage = nullptr;   // 9 doubles per node of the largest blob (pos, vel, force)
    int *io_moved = nullptr;      // set_nodes: 1 when a position changed
    int32_t io_max_nodes = 0;
    MeasView meas;                // measurements: node tiles in the reference's order, positions at creation
    int precond = FFEA_GPU_PRECOND_JACOBI;     // in use, after fall-backs
    MpnnBuffers mpnn;                          // learned smoother weights (allocated on first use)
    bool mpnn_ready = false;
    ~ffea_gpu()
    {
        if (step_exec) cudaGraphExecDestroy(step_exec);
        if (step_exec_coarse) cudaGraphExecDestroy(step_exec_coarse);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// One blob's nodes in the reference's order from the device state: corner
// nodes copy their row (velocity, and the solve's x as the force), edge
// midpoints average their edge's end rows (src/Blob.cpp:759-761), with the
// stored secondary velocity for the mass solver and zero for NoMass.
template <typename T>
__global__ void k_nodes_out(DeviceBatch d, const int2 *src, int n, const double *secvel, int nomass, double *pos,
                            double *vel, double *force)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 s = src[i];
    const T *x = static_cast<const T *>(d.x);
    for (int c = 0; c < 3; c++) {
        double p = 0.0, v = nomass ? 0.0 : secvel[3 * (size_t)i + c], f = 0.0;
        if (s.x >= 0 && s.y < 0) {
            p = d.pos[3 * (size_t)s.x + c];
            v = d.vel[3 * (size_t)s.x + c];
            f = (double)x[3 * (size_t)s.x + c];
        } else if (s.x >= 0) {
            p = .5 * (d.pos[3 * (size_t)s.x + c] + d.pos[3 * (size_t)s.y + c]);
        }
        pos[3 * (size_t)i + c] = p;
        vel[3 * (size_t)i + c] = v;
        force[3 * (size_t)i + c] = f;
    }
}

// The inverse for positions and velocities: corner nodes set their row;
// secondary velocities are kept for the mass solver.
__global__ void k_nodes_in(DeviceBatch d, const int2 *src, int n, const double *pos, const double *vel,
                           double *secvel, int mass, int *moved)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 s = src[i];
    for (int c = 0; c < 3; c++) {
        if (s.x >= 0 && s.y < 0) {
            if (pos) {
                double &dst = d.pos[3 * (size_t)s.x + c];
                const double v = pos[3 * (size_t)i + c];
                if (__double_as_longlong(dst) != __double_as_longlong(v)) *moved = 1;
                dst = v;
                if (d.pos_df) d.pos_df[3 * (size_t)s.x + c] = split_pos(v);
            }
            if (vel) d.vel[3 * (size_t)s.x + c] = vel[3 * (size_t)i + c];
        } else if (vel && mass) {
            secvel[3 * (size_t)i + c] = vel[3 * (size_t)i + c];
        }
    }
}

constexpr int kCoarseInitIterations = 40;      // Newton-Schulz from I / ||A_c||: log2(cond) + a few

// The coarse matrix of the current mesh and one Newton-Schulz update of its
// inverse (after the matrix assembly of every step or solve).
int refresh_coarse(ffea_gpu *h, cudaStream_t s, int iterations, bool init)
{
    if (!h->dev.coarse) return FFEA_GPU_OK;
    launch_coarse_assemble(h->dev, s);
    if (coarse_refresh(h->dev, h->host.bp, s, iterations, init) != 0)
        return fail("coarse-space refresh failed: %s", cudaGetErrorString(cudaGetLastError()));
    return FFEA_GPU_OK;
}

// Whether this step refreshes the coarse space (the first of every
// coarse_every steps; the matrix moves little from step to step and the
// refresh keeps X an inverse of a recent coarse matrix, which is what the
// preconditioner needs).
bool coarse_step(const ffea_gpu *h) { return h->dev.coarse && h->steps_done % h->coarse_every == 0; }

int capture_step_graph(ffea_gpu *h, bool with_coarse, cudaGraphExec_t *out, int64_t *fixed)
{
    DeviceBatch &d = h->dev;
    cudaStream_t s = h->stream;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    // every launcher counts its launches: the count across the capture is
    // the graph's kernels per replay (taken back out below, as nothing ran)
    const int64_t launches0 = kernel_launch_count();
    launch_noise(d, s);
    launch_elements(d, s, ELEM_STEP);
    if (d.any_nomass) launch_assemble(d, s);
    int rc = with_coarse ? refresh_coarse(h, s, 1, false) : FFEA_GPU_OK;
    launch_nodes(d, s, 0);
    cudaError_t le = launch_cg(d, s, true);  // the solve, then the Euler update and RNG advance
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    const int64_t captured = kernel_launch_count() - launches0;
    count_launches(-captured);
    if (rc != FFEA_GPU_OK || le != cudaSuccess || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return fail("capturing the step graph failed: %s / %s", cudaGetErrorString(le), cudaGetErrorString(ce));
    }
    *fixed = captured;
    cudaError_t e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail("cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
    return FFEA_GPU_OK;
}

int build_step_graph(ffea_gpu *h)
{
    if (capture_step_graph(h, false, &h->step_exec, &h->fixed_per_step)) return FFEA_GPU_ERROR;
    if (h->dev.coarse && capture_step_graph(h, true, &h->step_exec_coarse, &h->fixed_per_step_coarse))
        return FFEA_GPU_ERROR;
    return FFEA_GPU_OK;
}

int check_blob(ffea_gpu *h, int32_t blob)
{
    if (!h) return fail("null handle");
    if (blob < 0 || blob >= h->host.num_blobs) return fail("blob index %d out of range [0, %d)", blob, h->host.num_blobs);
    return FFEA_GPU_OK;
}

// device -> host copy of a T-typed array slice into doubles
int copy_typed_to_double(ffea_gpu *h, const void *src, size_t offset, size_t count, std::vector<double> &out)
{
    out.resize(count);
    if (h->dev.precision == PREC_FP64) {
        CK(cudaMemcpy(out.data(), static_cast<const double *>(src) + offset, count * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> tmp(count);
        CK(cudaMemcpy(tmp.data(), static_cast<const float *>(src) + offset, count * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < count; i++) out[i] = tmp[i];
    }
    return FFEA_GPU_OK;
}

}  // namespace

extern "C" {

int ffea_gpu_last_error(char *buf, size_t len)
{
    if (!buf || len == 0) return FFEA_GPU_ERROR;
    std::snprintf(buf, len, "%s", g_last_error.c_str());
    return FFEA_GPU_OK;
}

int64_t ffea_gpu_kernel_launches(void) { return kernel_launch_count(); }

int ffea_gpu_ffea_seed(int32_t rng_seed, uint64_t out[6])
{
    if (!out) return fail("null output");
    ffea_seed_words(rng_seed, out);
    return FFEA_GPU_OK;
}

namespace {
// The memory-resident solve of a batch of several blobs: every blob's
// segments dealt over the G CTAs, largest blob first, one segment per CTA in
// turn (CTA c keeps the count n_segs (c + 1) / G - n_segs c / G), then each
// CTA's segments sorted, which groups them by blob.  So each CTA holds a
// share of every large blob, and when the small blobs have converged every
// CTA still has rows to iterate instead of most of them waiting at the grid
// barriers.  Empty (the plain order) for one blob or one segment per CTA.
std::vector<int32_t> deal_segments(const HostBatch &H, int G)
{
    const int32_t n_segs = (int32_t)H.seg_row0.size();
    std::vector<int32_t> order;
    if (H.num_blobs <= 1 || n_segs <= G) return order;
    std::vector<int32_t> blobs(H.num_blobs);
    for (int b = 0; b < H.num_blobs; b++) blobs[b] = b;
    std::stable_sort(blobs.begin(), blobs.end(),
                     [&](int a, int b) { return H.bp[a].node_cnt > H.bp[b].node_cnt; });
    std::vector<int32_t> cap(G), start(G);
    for (int c = 0; c < G; c++) {
        start[c] = (int32_t)(((int64_t)n_segs * c) / G);
        cap[c] = (int32_t)(((int64_t)n_segs * (c + 1)) / G) - start[c];
    }
    std::vector<std::vector<int32_t>> per(G);
    int c = 0;
    for (int b : blobs)
        for (int32_t s = H.bp[b].seg_off; s < H.bp[b].seg_off + H.bp[b].seg_cnt; s++) {
            while ((int32_t)per[c].size() >= cap[c]) c = (c + 1) % G;
            per[c].push_back(s);
            c = (c + 1) % G;
        }
    order.resize(n_segs);
    for (int k = 0; k < G; k++) {
        std::sort(per[k].begin(), per[k].end());
        std::copy(per[k].begin(), per[k].end(), order.begin() + start[k]);
    }
    return order;
}
}  // namespace

int ffea_gpu_create_batch(int32_t num_blobs, const ffea_gpu_mesh *meshes, const ffea_gpu_params *params,
                          int32_t rng_mode, ffea_gpu_t **out)
{
    if (!out || !meshes || !params) return fail("null argument");
    *out = nullptr;
    if (rng_mode != FFEA_GPU_RNG_PER_BLOB && rng_mode != FFEA_GPU_RNG_SHARED) return fail("unknown rng_mode");
    std::unique_ptr<ffea_gpu> h(new ffea_gpu());
    std::string err;
    // persistent CG kernel: all CTAs co-resident (cooperative launch); the
    // register-resident variant when every CG segment gets a CTA of its own.
    // FFEA_GPU_CG_MAX_CTAS caps the grid, FFEA_GPU_CG_MEMORY_STATE=1 keeps the
    // segments but runs the memory-resident variant (both for tests).
    if (num_blobs <= 0) return fail("num_blobs must be >= 1");
    const int prec = params[0].precision;
    const int reg_grid0 = cg_max_grid(prec, 1, 0);
    const int max_grid = cg_max_grid(prec, 0, cg_mem_defer_bytes(prec));
    const bool sized = reg_grid0 > 0 && max_grid > 0;
    int cap = std::numeric_limits<int>::max();
    if (const char *e = std::getenv("FFEA_GPU_CG_MAX_CTAS")) cap = std::max(1, std::atoi(e));
    const int mem_cap = std::min(max_grid, cap);
    // the input is validated first, so that its errors are reported even
    // where no device is usable
    if (!build_batch(num_blobs, meshes, params, rng_mode, sized ? std::min(reg_grid0, cap) : 1, h->host, err))
        return fail("%s", err.c_str());
    if (!sized) return fail("cannot size the persistent CG kernel on this device");
    HostBatch &H = h->host;
    DeviceBatch &d = h->dev;
    DeviceArena &A = h->arena;
    // FFEA_GPU_CG_SMEM_SLOTS caps the matrix slots per row held in shared memory
    int max_slots = 64;
    if (const char *e = std::getenv("FFEA_GPU_CG_SMEM_SLOTS")) max_slots = std::max(0, std::atoi(e));
    int max_cols = 0;
    for (int32_t L : H.slice_len) max_cols = std::max(max_cols, (int)L);
    const int32_t n_segs = plan_cg_segments(H);
    // two-level preconditioner: NoMass blobs, mixed precision.  The
    // register-resident kernel carries it with one segment per CTA, local
    // reductions and at most CG_THREADS coarse dofs per blob; every other
    // batch runs it in the memory-resident kernel
    const int want = params[0].preconditioner;
    for (int b = 1; b < num_blobs; b++)
        if (params[b].preconditioner != want) return fail("all blobs of a batch must use the same preconditioner");
    if (want < FFEA_GPU_PRECOND_JACOBI || want > FFEA_GPU_PRECOND_LEARNED) return fail("unknown preconditioner");
    const int64_t coarse_total = build_coarse(H);
    int coarse_nmax = 0;
    // (the per-blob offsets of the dense coarse matrices are int32: a batch
    // whose matrices together pass that range runs Jacobi)
    bool coarse_ok = want != FFEA_GPU_PRECOND_JACOBI && H.precision == PREC_MIXED && !H.any_mass && !H.any_lumped &&
                     coarse_total <= INT32_MAX && H.coarse_htotal <= INT32_MAX;
    for (const BlobParams &bp : H.bp) coarse_nmax = std::max(coarse_nmax, (int)bp.coarse_n);
    const bool coarse_reg_ok = coarse_ok && coarse_nmax <= CG_THREADS;
    // phi per row, the CTA's six rows of X, c, 6 x 32 reduction floats and
    // the carried P^T s per coarse dof
    const size_t coarse_bytes =
        coarse_reg_ok ? 16 + 16 * (size_t)CG_THREADS +
                        sizeof(float) * (6 * (size_t)coarse_nmax + 8 + 6 * 32 + (size_t)CG_THREADS)
                  : 0;
    size_t dyn_bytes = 0;
    int cache_slots = 0, cache_cols = 0;
    if (cg_smem_plan(H.precision, max_slots, max_cols, coarse_bytes, &cache_slots, &cache_cols, &dyn_bytes) != 0)
        return fail("cannot size the shared memory of the CG kernel");
    const int reg_grid = cg_max_grid(H.precision, 1, dyn_bytes);
    if (reg_grid <= 0) return fail("cannot size the persistent CG kernel on this device");
    const int reg_cap = std::min(reg_grid, cap);
    const char *force_mem = std::getenv("FFEA_GPU_CG_MEMORY_STATE");
    d.n_segs = n_segs;
    d.cg_reg = n_segs <= reg_cap && !(force_mem && force_mem[0] == '1');
    d.cg_grid = n_segs <= reg_cap ? n_segs : std::min(mem_cap, n_segs);
    d.cg_cache_slots = d.cg_reg ? cache_slots : 0;
    d.cg_cache_cols = d.cg_reg ? cache_cols : 0;
    d.cg_dyn_smem = d.cg_reg ? (int32_t)dyn_bytes : (int32_t)cg_mem_defer_bytes(H.precision);
    if ((int64_t)d.cg_grid * CG_MAX_SEGS < n_segs)
        return fail("batch too large: %d CG segments need more than %d co-resident CTAs", n_segs, mem_cap);
    // local reduction (every CTA sums all partials, no serial last-arriver
    // step) while that read stays small
    const char *force_last = std::getenv("FFEA_GPU_CG_LAST_ARRIVER");
    d.cg_local = H.num_blobs <= CG_LOCAL_MAX_BLOBS && n_segs <= CG_LOCAL_MAX_SEGS &&
                 !(force_last && force_last[0] == '1');
    d.coarse = coarse_reg_ok && d.cg_reg && d.cg_local;
    if (coarse_ok && !d.coarse) {
        // the memory-resident kernel with the coarse space: its shared memory
        // holds g of one blob and P^T s of every blob a CTA touches
        const int G = std::min(mem_cap, n_segs);
        const std::vector<int32_t> order = deal_segments(H, G);
        int hmax = 0;
        for (int c = 0; c < G; c++) {
            const int S0 = (int)(((int64_t)n_segs * c) / G), S1 = (int)(((int64_t)n_segs * (c + 1)) / G);
            int sum = 0, last = -1;
            for (int k = S0; k < S1; k++) {
                const int sg = order.empty() ? k : order[k];
                if (H.seg_blob[sg] != last) {
                    last = H.seg_blob[sg];
                    sum += H.bp[last].coarse_n;
                }
            }
            hmax = std::max(hmax, sum);
        }
        const size_t mem_bytes = cg_mem_defer_bytes(H.precision) + cg_mem_coarse_bytes(hmax);
        if ((int64_t)G * CG_MAX_SEGS >= n_segs && cg_mem_smem_allow(H.precision, mem_bytes) == 0 &&
            cg_max_grid(H.precision, 0, mem_bytes) >= G) {
            d.coarse = 1;
            d.cg_reg = 0;
            d.cg_grid = G;
            d.cg_cache_slots = d.cg_cache_cols = 0;
            d.cg_dyn_smem = (int32_t)mem_bytes;
            d.coarse_hmax = hmax;
        }
    }
    d.coarse_nmax = d.coarse ? coarse_nmax : 0;
    d.part_stride = d.coarse ? 20 : 8;  // floats: DF dot terms 0..5; coarse P^T r 8..13, P^T w 14..19
    h->precond = d.coarse ? want : FFEA_GPU_PRECOND_JACOBI;
    d.num_blobs = H.num_blobs;
    d.nl_pad = H.nl_pad;
    d.ne_pad = H.ne_pad;
    d.n_edges = H.n_edges;
    d.n_tiles = H.n_tiles;
    d.n_etiles = H.n_etiles;
    d.num_streams = H.num_streams;
    d.precision = H.precision;
    d.any_mass = H.any_mass;
    d.any_nomass = H.any_nomass;
    d.any_lumped = H.any_lumped;
    const size_t ts = H.precision == PREC_FP64 ? sizeof(double) : sizeof(float);
    h->tsize = ts;
    CK(upload(A, d.bp, H.bp));
    CK(upload(A, d.mats, H.materials));
    CK(upload(A, d.tile_blob, H.tile_blob));
    CK(upload(A, d.seg_row0, H.seg_row0));
    CK(upload(A, d.seg_rows, H.seg_rows));
    CK(upload(A, d.seg_blob, H.seg_blob));
    if (!d.cg_reg) {
        const std::vector<int32_t> order = deal_segments(H, d.cg_grid);
        if (!order.empty()) CK(upload(A, d.seg_order, order));
    }
    CK(upload(A, d.etile_blob, H.etile_blob));
    std::vector<mrg::JumpMat> table(mrg::JUMP_TABLE_ENTRIES);
    mrg::build_jump_table(table.data());
    CK(upload(A, d.jump_table, table));
    CK(upload(A, d.stream_state, H.stream_state));
    CK(upload(A, d.stream_step, H.stream_step));
    CK(upload(A, d.noise_run_off, H.noise_run_off));
    d.noise_runs = H.noise_run_off.back();
    if (d.noise_runs > 0) {
        // no kept run state yet: every run jumps in the first step
        CK(upload(A, d.noise_run_state, std::vector<uint32_t>(6 * (size_t)d.noise_runs, 0u)));
        CK(upload(A, d.noise_run_gen, std::vector<uint32_t>((size_t)d.noise_runs, 0xffffffffu)));
    }
    h->stream_gen.assign((size_t)H.num_streams, 0u);
    CK(upload(A, d.stream_gen, h->stream_gen));
    CK(upload(A, d.pos, H.pos));
    if (H.precision == PREC_MIXED) {
        std::vector<float2> pdf(H.pos.size());
        for (size_t i = 0; i < H.pos.size(); i++) pdf[i] = split_pos(H.pos[i]);
        CK(upload(A, d.pos_df, pdf));
    }
    CK(upload(A, d.vel, H.vel));
    CK(upload(A, d.drag, H.drag));
    CK(upload(A, d.flags, H.flags));
    CK(upload(A, d.orig, H.orig));
    CK(upload(A, d.gather_ptr, H.gather_ptr));
    CK(upload(A, d.gather_idx, H.gather_idx));
    CK(upload(A, d.fold_ptr, H.fold_ptr));
    CK(upload(A, d.fold_sec, H.fold_sec));
    CK(upload_t(A, d.fold_amp, H.fold_amp, H.precision));
    CK(upload_t(A, d.node_amp, H.node_amp, H.precision));
    {
        std::vector<double> mt(MAT_T_STRIDE * std::max<size_t>(H.materials.size(), 1), 0.0);
        for (size_t i = 0; i < H.materials.size(); i++) {
            const Material &m = H.materials[i];
            double *o = &mt[MAT_T_STRIDE * i];
            o[MAT_T_RHO] = m.rho;
            o[MAT_T_A] = m.A;
            o[MAT_T_B] = m.B;
            o[MAT_T_G] = m.G;
            o[MAT_T_E] = m.E;
        }
        CK(upload_t(A, d.mat_t, mt, H.precision));
    }
    CK(upload(A, d.conn, H.conn));
    CK(upload(A, d.mat_id, H.mat_id));
    CK(upload(A, d.edge_p, H.edge_p));
    CK(upload(A, d.edge_q, H.edge_q));
    CK(upload(A, d.edge_cptr, H.edge_cptr));
    CK(upload(A, d.edge_cidx, H.edge_cidx));
    CK(upload(A, d.edge_pos_pq, H.edge_pos_pq));
    CK(upload(A, d.edge_pos_qp, H.edge_pos_qp));
    CK(upload(A, d.slice_ptr, H.slice_ptr));
    CK(upload(A, d.slice_len, H.slice_len));
    CK(upload(A, d.sell_col, H.sell_col));
    d.n_slices = (int32_t)H.slice_len.size();
    d.n_entries = (int32_t)H.sell_col.size();
    const size_t n3 = 3 * (size_t)H.nl_pad;
    CK(A.alloc(d.rhs, n3));
    for (void **v : {&d.x, &d.r, &d.u, &d.w, &d.p, &d.s, &d.dinv})
        CK(A.alloc_bytes(*v, n3 * ts));
    CK(A.alloc_bytes(d.u4, 4 * (size_t)H.nl_pad * ts));
    CK(A.alloc(d.det_sign, (size_t)H.ne_pad));
    CK(A.alloc_bytes(d.jinv0, 9 * (size_t)H.ne_pad * ts));
    CK(A.alloc_bytes(d.vol0, (size_t)H.ne_pad * ts));
    CK(A.alloc_bytes(d.efrc, 16 * (size_t)H.ne_pad * ts));  // a 4-vector per corner
    CK(A.alloc_bytes(d.elem_noise, 7 * (size_t)H.ne_pad * ts));
    CK(A.alloc_bytes(d.node_noise, std::max<size_t>(3 * (size_t)H.noise_nodes, 2) * ts));
    CK(A.alloc_bytes(d.g, H.any_nomass ? 12 * (size_t)H.ne_pad * ts : 16));
    CK(A.alloc_bytes(d.sell_val, H.any_nomass ? 9 * (size_t)d.n_entries * ts : 16));
    CK(A.alloc_bytes(d.sell_mval, H.any_mass ? (size_t)d.n_entries * ts : 16));
    CK(A.alloc_bytes(d.mass_diag, H.any_mass ? (size_t)H.nl_pad * ts : 16));
    if (H.any_lumped) CK(A.alloc(d.lumped_inv, (size_t)H.nl_pad));
    CK(A.alloc(d.partials, std::max(4 * (size_t)H.n_tiles, (size_t)d.part_stride * n_segs)));
    if (d.coarse) {
        CK(upload(A, d.seg_of_row, H.seg_of_row));
        CK(upload(A, d.seg_nbr_ptr, H.seg_nbr_ptr));
        CK(upload(A, d.seg_nbr, H.seg_nbr));
        CK(A.alloc(d.phi, (size_t)H.nl_pad));
        CK(cudaMemcpy(d.phi, H.phi.data(), H.phi.size() * sizeof(float), cudaMemcpyHostToDevice));
        CK(A.alloc(d.coarse_A, (size_t)coarse_total));
        CK(A.alloc(d.coarse_X, (size_t)coarse_total));
        if (!d.cg_reg) {
            // the memory-resident kernel reads X every iteration from global
            // memory: an FP16 copy, scaled to unit diagonal, halves that read
            size_t dofs = 0;
            for (const BlobParams &bp : H.bp) dofs += (size_t)bp.coarse_n;
            CK(A.alloc(d.coarse_Xh, (size_t)H.coarse_htotal));
            CK(A.alloc(d.coarse_s, dofs));
        }
        // Newton-Schulz scratch for a run of equal-size blobs at once
        CK(A.alloc(d.coarse_T, std::max((size_t)coarse_nmax * coarse_nmax, (size_t)coarse_total)));
        CK(A.alloc(d.coarse_Xn, std::max((size_t)coarse_nmax * coarse_nmax, (size_t)coarse_total)));
        if (const size_t np = coarse_part_floats(H.bp)) CK(A.alloc(d.coarse_part, np));
        CK(A.alloc(d.coarse_asm, 36 * (size_t)(CG_SEG_MAX_ROWS / 256) * std::max<size_t>(1, H.seg_nbr.size())));
    }
    CK(A.alloc(d.epartials, 2 * (size_t)H.n_etiles));
    CK(A.alloc(d.cg, (size_t)H.num_blobs));
    CK(A.alloc(d.last_sums, 3 * (size_t)H.num_blobs));
    CK(A.alloc(d.counters, (size_t)CNT_COUNT));
    CK(A.alloc(d.status, (size_t)H.num_blobs));
    CK(A.alloc(d.inverted, (size_t)H.num_blobs));
    CK(A.alloc(d.energy, 2 * (size_t)H.num_blobs));
    CK(A.alloc(d.bar, 8));
    CK(A.alloc(d.loop_count, 1));
    // a blocking stream: the zero fills (cudaMemset) and host-to-device
    // copies (cudaMemcpy) that set up and update the handle's buffers run on
    // the legacy default stream and can still be in flight when those calls
    // return; a non-blocking stream would not wait for them (seen as network
    // weights zeroed after their upload, so that every smoother weight came
    // out as 1, in some processes and not others)
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamDefault));
    for (auto &e : h->ev) CK(cudaEventCreate(&e));
    // secondary-node initial velocities (they never change: their rows are identity)
    {
        static const int mid[6][3] = {{4, 0, 1}, {5, 0, 2}, {6, 0, 3}, {7, 1, 2}, {8, 1, 3}, {9, 2, 3}};
        std::vector<int2> src;
        std::vector<double> secvel;
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_mesh &m = meshes[b];
            const BlobMap &map = H.maps[b];
            h->io_off.push_back((int64_t)src.size());
            h->io_max_nodes = std::max(h->io_max_nodes, m.num_nodes);
            const size_t base = src.size();
            src.resize(base + m.num_nodes, make_int2(-1, -1));
            secvel.resize(3 * src.size(), 0.0);
            for (int32_t n = 0; n < m.num_nodes; n++)
                if (map.lin_of_orig[n] >= 0) src[base + n] = make_int2(map.lin_of_orig[n], -1);
            for (int32_t e = 0; e < map.num_elements; e++) {  // last element wins (src/Blob.cpp:759-761)
                const int32_t *t = &map.topology[10 * (size_t)e];
                for (int k = 0; k < 6; k++)
                    src[base + t[mid[k][0]]] =
                        make_int2(map.lin_of_orig[t[mid[k][1]]], map.lin_of_orig[t[mid[k][2]]]);
            }
            if (m.vel && params[b].solver != SOLVER_NOMASS)
                for (int32_t n = 0; n < m.num_nodes; n++)
                    if (map.lin_of_orig[n] < 0)
                        for (int c = 0; c < 3; c++) secvel[3 * (base + n) + c] = m.vel[3 * (size_t)n + c];
        }
        CK(upload(A, h->io_src, src));
        h->io_src_host = src;
        CK(upload(A, h->io_secvel, secvel));
        CK(A.alloc(h->io_stage, 9 * (size_t)h->io_max_nodes));
        CK(A.alloc(h->io_moved, 1));
        // measurements: Blob::set_pos_0 (src/World.cpp:504) takes the
        // positions after Blob::init has put every edge midpoint between its
        // end nodes (linearise_elements, src/Blob.cpp:334-340), last element
        // first as above; node tiles of MEAS_TILE per blob
        std::vector<double> pos0(3 * src.size());
        std::vector<int64_t> off(h->io_off);
        off.push_back((int64_t)src.size());
        std::vector<int32_t> tile_blob, tile_first;
        for (int b = 0; b < num_blobs; b++) {
            const ffea_gpu_mesh &m = meshes[b];
            double *p0 = pos0.data() + 3 * off[b];
            std::copy(m.pos, m.pos + 3 * (size_t)m.num_nodes, p0);
            for (int32_t e = 0; e < m.num_elements; e++) {
                const int32_t *t = &m.topology[10 * (size_t)e];
                for (int k = 0; k < 6; k++)
                    for (int c = 0; c < 3; c++)
                        p0[3 * (size_t)t[mid[k][0]] + c] =
                            .5 * (p0[3 * (size_t)t[mid[k][1]] + c] + p0[3 * (size_t)t[mid[k][2]] + c]);
            }
            tile_first.push_back((int32_t)tile_blob.size());
            tile_blob.resize(tile_blob.size() + (meshes[b].num_nodes + MEAS_TILE - 1) / MEAS_TILE, b);
        }
        tile_first.push_back((int32_t)tile_blob.size());
        MeasView &mv = h->meas;
        double *p0 = nullptr;
        int64_t *po = nullptr;
        int32_t *tb = nullptr, *tf = nullptr;
        CK(upload(A, p0, pos0));
        CK(upload(A, po, off));
        CK(upload(A, tb, tile_blob));
        CK(upload(A, tf, tile_first));
        mv.io_src = h->io_src;
        mv.pos0 = p0;
        mv.io_off = po;
        mv.tile_blob = tb;
        mv.tile_first = tf;
        mv.n_tiles = (int32_t)tile_blob.size();
        CK(A.alloc(mv.partials, 4 * (size_t)(H.n_etiles + mv.n_tiles)));
        CK(A.alloc(mv.out, MEAS_VALUES * (size_t)num_blobs));
    }
    launch_rest_state(d, h->stream);
    if (d.any_mass) launch_mass_matrix(d, h->stream);
    if (d.any_lumped) launch_lumped_mass(d, h->stream);
    if (d.coarse) {
        // X ~ A_c^-1 of the rest mesh, Newton-Schulz from a scaled identity;
        // every step then refines it for the current mesh
        launch_elements(d, h->stream, ELEM_MATRIX_ONLY);
        launch_assemble(d, h->stream);
        if (refresh_coarse(h.get(), h->stream, kCoarseInitIterations, true)) return FFEA_GPU_ERROR;
        if (const char *e = std::getenv("FFEA_GPU_COARSE_REFRESH")) h->coarse_every = std::max(1, std::atoi(e));
    }
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    *out = h.release();
    return FFEA_GPU_OK;
}

int ffea_gpu_create(const ffea_gpu_mesh *mesh, const ffea_gpu_params *params, ffea_gpu_t **out)
{
    return ffea_gpu_create_batch(1, mesh, params, FFEA_GPU_RNG_PER_BLOB, out);
}

void ffea_gpu_destroy(ffea_gpu_t *h)
{
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
}

void *ffea_gpu_stream(ffea_gpu_t *h) { return h ? (void *)h->stream : nullptr; }

int ffea_gpu_set_graph_mode(ffea_gpu_t *h, int32_t enable)
{
    if (!h) return fail("null handle");
    h->graph_mode = enable ? 1 : 0;
    return FFEA_GPU_OK;
}

int ffea_gpu_set_timing(ffea_gpu_t *h, int32_t enable)
{
    if (!h) return fail("null handle");
    h->timing = enable ? 1 : 0;
    return FFEA_GPU_OK;
}

int ffea_gpu_phase_times(ffea_gpu_t *h, double out_ms[5])
{
    if (!h || !out_ms) return fail("null argument");
    for (int i = 0; i < 5; i++) out_ms[i] = h->phase_ms[i];
    return FFEA_GPU_OK;
}

int ffea_gpu_kernel_times(ffea_gpu_t *h, double out_ms[FFEA_GPU_NUM_KERNEL_TIMES])
{
    if (!h || !out_ms) return fail("null argument");
    for (int i = 0; i < FFEA_GPU_NUM_KERNEL_TIMES; i++) out_ms[i] = h->kernel_ms[i];
    return FFEA_GPU_OK;
}

int ffea_gpu_preconditioner(ffea_gpu_t *h) { return h ? h->precond : -1; }

int ffea_gpu_selftest_barrier_timeout(int32_t ctas, int32_t spin_limit, int32_t *timed_out)
{
    if (!timed_out) return fail("null result");
    if (ctas < 1 || ctas > 64 || spin_limit < 1 || spin_limit > (1 << 20))
        return fail("selftest: ctas must be in [1, 64] and spin_limit in [1, 2^20]");
    unsigned int *bar = nullptr;
    int *out = nullptr;
    CK(cudaMalloc(&bar, 8 * sizeof(unsigned int)));
    cudaError_t e = cudaMalloc(&out, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(bar, 0, 8 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(out, 0, sizeof(int));
    if (e == cudaSuccess) e = launch_barrier_timeout_selftest(bar, (unsigned)spin_limit, out, ctas, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int r = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&r, out, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(bar);
    cudaFree(out);
    if (e != cudaSuccess) return fail("selftest: %s", cudaGetErrorString(e));
    *timed_out = r;
    return FFEA_GPU_OK;
}

int ffea_gpu_set_smoother_weights(ffea_gpu_t *h, int32_t blob, const float *omega)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!omega) return fail("null weights");
    if (!h->dev.coarse) return fail("smoother weights need the two-level preconditioner, which this handle does not use");
    const BlobMap &map = h->host.maps[blob];
    std::vector<float> &phi = h->host.phi;
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        if (g < 0) continue;
        const float w = omega[n];
        if (!(w > 0.f && w <= 2.f)) return fail("smoother weight of node %d is %g, outside (0, 2]", n, (double)w);
        phi[4 * (size_t)g + 3] = w;
    }
    const BlobParams &bp = h->host.bp[blob];
    CK(cudaMemcpyAsync(h->dev.phi + bp.node_off, phi.data() + 4 * (size_t)bp.node_off,
                       4 * sizeof(float) * (size_t)bp.node_cnt, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FFEA_GPU_OK;
}

namespace {

int mpnn_alloc(ffea_gpu *h)
{
    if (h->mpnn_ready) return FFEA_GPU_OK;
    if (h->precond != FFEA_GPU_PRECOND_LEARNED) return fail("the network needs a handle with the LEARNED preconditioner");
    DeviceBatch &d = h->dev;
    DeviceArena &A = h->arena;
    MpnnBuffers &B = h->mpnn;
    const size_t n = d.nl_pad;
    int coarse_total = 0;
    for (const BlobParams &bp : h->host.bp) coarse_total += bp.coarse_n;
    CK(A.alloc(B.x0, n * MPNN_FEATURES));
    for (auto &hb : B.h) CK(A.alloc(hb, n * MPNN_HIDDEN));
    CK(A.alloc(B.omega, n));
    CK(A.alloc(B.v, n));
    CK(A.alloc(B.e, n));
    CK(A.alloc(B.gw, n));
    CK(A.alloc(B.gvec, (size_t)coarse_total));
    CK(A.alloc(B.cvec, (size_t)coarse_total));
    CK(A.alloc(B.cta_sums, 3 * ((n + 127) / 128)));
    CK(A.alloc(B.scal, 3));
    for (float **p : {&B.dh, &B.dh2, &B.dself, &B.tbuf}) CK(A.alloc(*p, n * MPNN_HIDDEN));
    CK(A.alloc(B.partial, ((n + 63) / 64) * (size_t)MPNN_NUM_PARAMS));
    CK(A.alloc(B.theta, (size_t)MPNN_NUM_PARAMS));
    CK(A.alloc(B.grad, (size_t)MPNN_NUM_PARAMS));
    h->mpnn_ready = true;
    return FFEA_GPU_OK;
}

int mpnn_upload(ffea_gpu *h, const float *theta)
{
    if (!theta) return fail("null network parameters");
    if (mpnn_alloc(h)) return FFEA_GPU_ERROR;
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpyAsync(h->mpnn.theta, theta, sizeof(float) * MPNN_NUM_PARAMS, cudaMemcpyHostToDevice, h->stream));
    return FFEA_GPU_OK;
}

}  // namespace

int ffea_gpu_mpnn_num_params(void) { return MPNN_NUM_PARAMS; }

int ffea_gpu_mpnn_apply(ffea_gpu_t *h, const float *theta)
{
    if (!h) return fail("null handle");
    if (mpnn_upload(h, theta)) return FFEA_GPU_ERROR;
    if (mpnn_forward(h->dev, h->mpnn, h->mpnn.theta, true, h->stream)) return fail("network forward pass failed");
    CK(cudaStreamSynchronize(h->stream));
    return FFEA_GPU_OK;
}

int ffea_gpu_mpnn_loss_grad(ffea_gpu_t *h, const float *theta, double *loss, float *grad)
{
    if (!h) return fail("null handle");
    if (mpnn_upload(h, theta)) return FFEA_GPU_ERROR;
    MpnnBuffers &B = h->mpnn;
    if (mpnn_forward(h->dev, B, B.theta, false, h->stream)) return fail("network forward pass failed");
    if (mpnn_loss(h->dev, B, h->stream)) return fail("network loss failed");
    if (grad && mpnn_backward(h->dev, B, B.theta, B.grad, h->stream)) return fail("network backward pass failed");
    double sc[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(sc, B.scal, sizeof(sc), cudaMemcpyDeviceToHost, h->stream));
    if (grad) CK(cudaMemcpyAsync(grad, B.grad, sizeof(float) * MPNN_NUM_PARAMS, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (loss) *loss = sc[0];
    return FFEA_GPU_OK;
}

int ffea_gpu_mpnn_probe(ffea_gpu_t *h, int32_t blob, const float *theta, const float *domega, float *features,
                        float *omega, float *grad)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (mpnn_upload(h, theta)) return FFEA_GPU_ERROR;
    DeviceBatch &d = h->dev;
    MpnnBuffers &B = h->mpnn;
    const BlobMap &map = h->host.maps[blob];
    if (mpnn_forward(d, B, B.theta, false, h->stream)) return fail("network forward pass failed");
    if (domega && grad) {
        // dL/d omega = k1 * gw.x - k2 * gw.y with k1 = 1, k2 = 0: gw.x = domega
        std::vector<float2> gw(d.nl_pad, make_float2(0.f, 0.f));
        for (int32_t n = 0; n < map.num_nodes_total; n++)
            if (map.lin_of_orig[n] >= 0) gw[map.lin_of_orig[n]].x = domega[n];
        const double sc[3] = {0.0, 1.0, 0.0};
        CK(cudaMemcpyAsync(B.gw, gw.data(), sizeof(float2) * gw.size(), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(B.scal, sc, sizeof(sc), cudaMemcpyHostToDevice, h->stream));
        if (mpnn_backward(d, B, B.theta, B.grad, h->stream)) return fail("network backward pass failed");
        CK(cudaMemcpyAsync(grad, B.grad, sizeof(float) * MPNN_NUM_PARAMS, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    std::vector<float> x0((size_t)d.nl_pad * MPNN_FEATURES), om(d.nl_pad);
    CK(cudaMemcpy(x0.data(), B.x0, sizeof(float) * x0.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(om.data(), B.omega, sizeof(float) * om.size(), cudaMemcpyDeviceToHost));
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        for (int k = 0; k < MPNN_FEATURES; k++)
            if (features) features[(size_t)n * MPNN_FEATURES + k] = g >= 0 ? x0[(size_t)g * MPNN_FEATURES + k] : 0.f;
        if (omega) omega[n] = g >= 0 ? om[g] : 1.f;
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_sizes(ffea_gpu_t *h, int64_t *linear_nodes, int64_t *elements, int64_t *edges)
{
    if (!h) return fail("null handle");
    int64_t nl = 0, ne = 0;
    for (auto &bp : h->host.bp) {
        nl += bp.node_cnt;
        ne += bp.elem_cnt;
    }
    if (linear_nodes) *linear_nodes = nl;
    if (elements) *elements = ne;
    if (edges) *edges = h->host.n_edges;
    return FFEA_GPU_OK;
}

namespace {
int enqueue_steps(ffea_gpu *h, int32_t nsteps, bool allow_direct)
{
    DeviceBatch &d = h->dev;
    for (int32_t s = 0; s < nsteps; s++) {
        if (h->graph_mode && !h->timing) {
            if (!h->step_exec && build_step_graph(h) != FFEA_GPU_OK) {
                // fall back to direct launches when the graph cannot be built
                h->graph_mode = 0;
            } else {
                const bool cs = coarse_step(h);
                CK(cudaGraphLaunch(cs ? h->step_exec_coarse : h->step_exec, h->stream));
                count_launches(cs ? h->fixed_per_step_coarse : h->fixed_per_step);
                h->steps_done++;
                continue;
            }
        }
        if (!allow_direct) return fail("asynchronous stepping needs graph mode without timing");
        // with timing on, an event after each kernel (or group) of the step
        auto mark = [&](int i) { return h->timing ? cudaEventRecord(h->ev[i], h->stream) : cudaSuccess; };
        CK(mark(0));
        launch_noise(d, h->stream);
        CK(mark(1));
        launch_elements(d, h->stream, ELEM_STEP);
        CK(mark(2));
        if (d.any_nomass) launch_assemble(d, h->stream);
        CK(mark(3));
        if (coarse_step(h) && refresh_coarse(h, h->stream, 1, false)) return FFEA_GPU_ERROR;
        h->steps_done++;
        CK(mark(4));
        launch_nodes(d, h->stream, 0);
        CK(mark(5));
        CK(launch_cg(d, h->stream, true));  // with the Euler update and RNG advance
        CK(mark(6));
        CK(mark(7));
        if (h->timing) {
            CK(cudaEventSynchronize(h->ev[FFEA_GPU_NUM_KERNEL_TIMES]));
            for (int i = 0; i < FFEA_GPU_NUM_KERNEL_TIMES; i++) {
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, h->ev[i], h->ev[i + 1]));
                h->kernel_ms[i] += ms;
            }
            // the coarser phases: elements (noise + elements), assembly (with
            // the coarse refresh), nodes, CG, update
            h->phase_ms[0] = h->kernel_ms[0] + h->kernel_ms[1];
            h->phase_ms[1] = h->kernel_ms[2] + h->kernel_ms[3];
            h->phase_ms[2] = h->kernel_ms[4];
            h->phase_ms[3] = h->kernel_ms[5];
            h->phase_ms[4] = h->kernel_ms[6];
        }
    }
    return FFEA_GPU_OK;
}

int sync_and_check(ffea_gpu *h)
{
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    std::vector<int32_t> st(h->host.num_blobs);
    CK(cudaMemcpy(st.data(), h->dev.status, st.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
    for (int b = 0; b < h->host.num_blobs; b++)
        if (st[b]) {
            const char *why = (st[b] & BLOB_FAIL_INVERSION) ? "an element inverted" : "the CG solve did not converge";
            return fail("blob %d: %s (status bits %d); the blob is frozen at the failing step", b, why, st[b]);
        }
    return FFEA_GPU_OK;
}
}  // namespace

int ffea_gpu_step(ffea_gpu_t *h, int32_t nsteps)
{
    if (!h) return fail("null handle");
    if (nsteps < 0) return fail("nsteps must be >= 0");
    for (int i = 0; i < 5; i++) h->phase_ms[i] = 0;
    for (int i = 0; i < FFEA_GPU_NUM_KERNEL_TIMES; i++) h->kernel_ms[i] = 0;
    if (enqueue_steps(h, nsteps, true) != FFEA_GPU_OK) return FFEA_GPU_ERROR;
    return sync_and_check(h);
}

int ffea_gpu_step_async(ffea_gpu_t *h, int32_t nsteps)
{
    if (!h) return fail("null handle");
    if (nsteps < 0) return fail("nsteps must be >= 0");
    return enqueue_steps(h, nsteps, false);
}

int ffea_gpu_synchronize(ffea_gpu_t *h)
{
    if (!h) return fail("null handle");
    return sync_and_check(h);
}

int64_t ffea_gpu_cg_loop_count(ffea_gpu_t *h)
{
    if (!h) return -1;
    unsigned long long c = 0;
    if (cudaMemcpy(&c, h->dev.loop_count, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return (int64_t)c;
}

// A caller's array in device memory of this device (used in place by the
// node kernels); NULL for host memory, which goes through staging and one
// copy-engine transfer per array: on GB300 that measured faster than the
// kernels reading or writing pinned host memory over the host link.
static void *device_view(const void *p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // not a pointer CUDA knows: clear the error
        return nullptr;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    if ((a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev)
        return const_cast<void *>(p);
    return nullptr;
}

int ffea_gpu_get_nodes(ffea_gpu_t *h, int32_t blob, double *pos, double *vel, double *force)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    const BlobParams &bp = h->host.bp[blob];
    const int32_t N = h->host.maps[blob].num_nodes_total;
    const int64_t o = h->io_off[blob];
    double *st = h->io_stage;
    if (N > 0) {
        // the kernel writes each array straight into the caller's device
        // memory, else into staging, copied to the host after
        double *const out[3] = {pos, vel, force};
        double *dst[3];
        for (int k = 0; k < 3; k++) {
            double *v = static_cast<double *>(device_view(out[k]));
            dst[k] = v ? v : st + 3 * (size_t)k * N;
        }
        const int blocks = (N + 255) / 256;
        if (h->dev.precision == PREC_FP64)
            k_nodes_out<double><<<blocks, 256, 0, h->stream>>>(h->dev, h->io_src + o, N, h->io_secvel + 3 * o,
                                                               bp.solver == SOLVER_NOMASS, dst[0], dst[1], dst[2]);
        else
            k_nodes_out<float><<<blocks, 256, 0, h->stream>>>(h->dev, h->io_src + o, N, h->io_secvel + 3 * o,
                                                              bp.solver == SOLVER_NOMASS, dst[0], dst[1], dst[2]);
        count_launches(1);
        const size_t bytes = 3 * sizeof(double) * (size_t)N;
        for (int k = 0; k < 3; k++)
            if (out[k] && dst[k] == st + 3 * (size_t)k * N)
                CK(cudaMemcpyAsync(out[k], dst[k], bytes, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    return FFEA_GPU_OK;
}

int ffea_gpu_set_nodes(ffea_gpu_t *h, int32_t blob, const double *pos, const double *vel)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    const BlobParams &bp = h->host.bp[blob];
    const int32_t N = h->host.maps[blob].num_nodes_total;
    const int64_t o = h->io_off[blob];
    double *st = h->io_stage;
    const size_t bytes = 3 * sizeof(double) * (size_t)N;
    if (N > 0 && (pos || vel)) {
        // read straight from the caller's device memory, else from staging
        const double *src_pos = static_cast<const double *>(device_view(pos));
        const double *src_vel = static_cast<const double *>(device_view(vel));
        if (pos && !src_pos) {
            CK(cudaMemcpyAsync(st, pos, bytes, cudaMemcpyHostToDevice, h->stream));
            src_pos = st;
        }
        if (vel && !src_vel) {
            CK(cudaMemcpyAsync(st + 3 * (size_t)N, vel, bytes, cudaMemcpyHostToDevice, h->stream));
            src_vel = st + 3 * (size_t)N;
        }
        if (pos) CK(cudaMemsetAsync(h->io_moved, 0, sizeof(int), h->stream));
        k_nodes_in<<<(N + 255) / 256, 256, 0, h->stream>>>(h->dev, h->io_src + o, N, src_pos, src_vel,
                                                          h->io_secvel + 3 * o, bp.solver != SOLVER_NOMASS,
                                                          h->io_moved);
        count_launches(1);
        if (pos) {
            // positions that differ from the current ones: refresh the
            // coarse space on the next step (the same positions need none)
            int moved = 0;
            CK(cudaMemcpyAsync(&moved, h->io_moved, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (moved) h->steps_done = 0;
        }
    }
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    return FFEA_GPU_OK;
}

int ffea_gpu_set_external_forces(ffea_gpu_t *h, int32_t blob, int32_t count, const int32_t *nodes,
                                 const double *forces)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    const int32_t N = h->host.maps[blob].num_nodes_total;
    if (count < 0) return fail("count must be >= 0");
    if (count > 0 && (!nodes || !forces)) return fail("null nodes or forces");
    for (int32_t i = 0; i < count; i++)
        if (nodes[i] < 0 || nodes[i] >= N) return fail("node index %d out of range [0, %d)", nodes[i], N);
    DeviceBatch &d = h->dev;
    if (!d.ext) {
        if (count == 0) return FFEA_GPU_OK;  // nothing set, nothing to clear
        CK(cudaStreamSynchronize(h->stream));
        CK(h->arena.alloc(d.ext, 3 * (size_t)h->host.nl_pad));  // zeroed
        h->ext_host.assign(3 * (size_t)h->host.nl_pad, 0.0);
        // the step graphs hold the batch by value: capture them again
        if (h->step_exec) cudaGraphExecDestroy(h->step_exec);
        if (h->step_exec_coarse) cudaGraphExecDestroy(h->step_exec_coarse);
        h->step_exec = h->step_exec_coarse = nullptr;
    }
    // fold onto the blob's corner rows in the given order: a corner node
    // keeps its force, an edge midpoint gives half to each end
    const BlobParams &bp = h->host.bp[blob];
    const int2 *src = h->io_src_host.data() + h->io_off[blob];
    double *e = h->ext_host.data() + 3 * (size_t)bp.node_off;
    std::fill(e, e + 3 * (size_t)bp.node_cnt, 0.0);
    for (int32_t i = 0; i < count; i++) {
        const int2 s = src[nodes[i]];
        const double *f = forces + 3 * (size_t)i;
        if (s.x >= 0 && s.y < 0) {
            for (int c = 0; c < 3; c++) e[3 * (size_t)(s.x - bp.node_off) + c] += f[c];
        } else if (s.x >= 0) {
            for (int c = 0; c < 3; c++) {
                e[3 * (size_t)(s.x - bp.node_off) + c] += 0.5 * f[c];
                e[3 * (size_t)(s.y - bp.node_off) + c] += 0.5 * f[c];
            }
        }  // a node of no element takes no part in the update
    }
    CK(cudaMemcpyAsync(d.ext + 3 * (size_t)bp.node_off, e, sizeof(double) * 3 * (size_t)bp.node_cnt,
                       cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FFEA_GPU_OK;
}

int ffea_gpu_get_rng_state(ffea_gpu_t *h, int32_t blob, uint64_t state[6])
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!state) return fail("null state");
    CK(cudaStreamSynchronize(h->stream));
    uint32_t st[6];
    CK(cudaMemcpy(st, h->dev.stream_state + 6 * h->host.bp[blob].stream, sizeof(st), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 6; i++) state[i] = st[i];
    return FFEA_GPU_OK;
}

int ffea_gpu_set_rng_state(ffea_gpu_t *h, int32_t blob, const uint64_t state[6])
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!state) return fail("null state");
    // RngStream::CheckSeed (src/RngStream.cpp:230-253): words below the moduli, not all zero per component
    for (int i = 0; i < 6; i++)
        if (state[i] >= (i < 3 ? mrg::M1 : mrg::M2)) return fail("seed word %d out of range", i);
    if ((state[0] | state[1] | state[2]) == 0 || (state[3] | state[4] | state[5]) == 0)
        return fail("seed component is all zero");
    CK(cudaStreamSynchronize(h->stream));
    uint32_t st[6];
    for (int i = 0; i < 6; i++) st[i] = (uint32_t)state[i];
    const int sm = h->host.bp[blob].stream;
    CK(cudaMemcpy(h->dev.stream_state + 6 * sm, st, sizeof(st), cudaMemcpyHostToDevice));
    // the noise kernel's kept run states belong to the old state: a new
    // generation makes every run of this stream jump again
    h->stream_gen[sm] += 1;
    CK(cudaMemcpy(h->dev.stream_gen + sm, &h->stream_gen[sm], sizeof(uint32_t), cudaMemcpyHostToDevice));
    return FFEA_GPU_OK;
}

int ffea_gpu_energies(ffea_gpu_t *h, int32_t blob, double *strain, double *kinetic)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    launch_energies(h->dev, h->stream);
    double e[2];
    CK(cudaMemcpyAsync(e, h->dev.energy + 2 * blob, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (strain) *strain = e[0];
    if (kinetic) *kinetic = e[1];
    return FFEA_GPU_OK;
}

int ffea_gpu_measurements(ffea_gpu_t *h, int32_t first_blob, int32_t count, double *out)
{
    if (!h || !out || count < 1 || first_blob < 0 || first_blob + (int64_t)count > h->dev.num_blobs)
        return FFEA_GPU_ERROR;
    launch_energies(h->dev, h->stream);
    launch_measurements(h->dev, h->meas, h->stream);
    std::vector<double> e(2 * (size_t)count), v(MEAS_VALUES * (size_t)count);
    CK(cudaMemcpyAsync(e.data(), h->dev.energy + 2 * (size_t)first_blob, sizeof(double) * e.size(),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(v.data(), h->meas.out + MEAS_VALUES * (size_t)first_blob, sizeof(double) * v.size(),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int32_t b = 0; b < count; b++) {
        double *o = out + FFEA_GPU_NUM_MEASUREMENTS * (size_t)b;
        const double *m = v.data() + MEAS_VALUES * (size_t)b;
        o[FFEA_GPU_MEAS_KINETIC] = e[2 * (size_t)b + 1];
        o[FFEA_GPU_MEAS_STRAIN] = e[2 * (size_t)b];
        for (int k = 0; k < 3; k++) {
            o[FFEA_GPU_MEAS_CENTROID + k] = m[k];
            o[FFEA_GPU_MEAS_COM + k] = m[4 + k];
            o[FFEA_GPU_MEAS_ANGMOM + k] = m[7 + k];
        }
        o[FFEA_GPU_MEAS_RMSD] = m[3];
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_status(ffea_gpu_t *h, int32_t blob, int32_t *inverted, int32_t *cg_iters, double *true_relres,
                    int32_t *fail_bits)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    CK(cudaStreamSynchronize(h->stream));
    CgScalars cg;
    int32_t inv = 0, st = 0;
    CK(cudaMemcpy(&cg, h->dev.cg + blob, sizeof(cg), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&inv, h->dev.inverted + blob, sizeof(inv), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&st, h->dev.status + blob, sizeof(st), cudaMemcpyDeviceToHost));
    if (inverted) *inverted = inv;
    if (cg_iters) *cg_iters = cg.iters;
    if (true_relres) *true_relres = cg.true_relres2 >= 0 ? std::sqrt(cg.true_relres2) : NAN;
    if (fail_bits) *fail_bits = st;
    return FFEA_GPU_OK;
}

int ffea_gpu_get_rhs(ffea_gpu_t *h, int32_t blob, double *rhs)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!rhs) return fail("null output");
    CK(cudaStreamSynchronize(h->stream));
    const BlobParams &bp = h->host.bp[blob];
    const BlobMap &map = h->host.maps[blob];
    const size_t n3 = 3 * (size_t)bp.node_cnt;
    std::vector<double> r(n3);
    CK(cudaMemcpy(r.data(), h->dev.rhs + 3 * (size_t)bp.node_off, n3 * sizeof(double), cudaMemcpyDeviceToHost));
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        for (int c = 0; c < 3; c++) rhs[3 * (size_t)n + c] = g < 0 ? 0.0 : r[3 * (size_t)(g - bp.node_off) + c];
    }
    return FFEA_GPU_OK;
}

int ffea_gpu_get_element_forces(ffea_gpu_t *h, int32_t blob, double *out)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!out) return fail("null output");
    CK(cudaStreamSynchronize(h->stream));
    const BlobParams &bp = h->host.bp[blob];
    std::vector<double> v;
    if (copy_typed_to_double(h, h->dev.efrc, 16 * (size_t)bp.elem_off, 16 * (size_t)bp.elem_cnt, v)) return FFEA_GPU_ERROR;
    // (x, y, z, 0) per corner on the device, 3 per corner out
    for (size_t c = 0; c < 4 * (size_t)bp.elem_cnt; c++)
        for (int i = 0; i < 3; i++) out[3 * c + i] = v[4 * c + i];
    return FFEA_GPU_OK;
}

int ffea_gpu_solver_solve(ffea_gpu_t *h, int32_t blob, const double *pos, double *x)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!x) return fail("null rhs/solution");
    if (pos && ffea_gpu_set_nodes(h, blob, pos, nullptr)) return FFEA_GPU_ERROR;
    DeviceBatch &d = h->dev;
    const BlobParams &bp = h->host.bp[blob];
    const BlobMap &map = h->host.maps[blob];
    std::vector<double> rhs(3 * (size_t)d.nl_pad, 0.0);
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        if (g < 0 || map.pinned_orig[n]) continue;
        for (int c = 0; c < 3; c++) rhs[3 * (size_t)g + c] = x[3 * (size_t)n + c];
    }
    CK(cudaMemcpyAsync(d.rhs, rhs.data(), rhs.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_elements(d, h->stream, ELEM_MATRIX_ONLY);
    if (d.any_nomass) launch_assemble(d, h->stream);
    if (refresh_coarse(h, h->stream, 1, false)) return FFEA_GPU_ERROR;
    launch_nodes(d, h->stream, 1);
    CK(launch_cg(d, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CgScalars cg;
    int32_t st = 0;
    CK(cudaMemcpy(&cg, d.cg + blob, sizeof(cg), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&st, d.status + blob, sizeof(st), cudaMemcpyDeviceToHost));
    std::vector<double> sol;
    if (copy_typed_to_double(h, d.x, 3 * (size_t)bp.node_off, 3 * (size_t)bp.node_cnt, sol)) return FFEA_GPU_ERROR;
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        for (int c = 0; c < 3; c++) {
            double &xv = x[3 * (size_t)n + c];
            if (map.pinned_orig[n] || (g < 0 && bp.solver == SOLVER_MASS)) continue;  // identity row: x = rhs
            if (g >= 0) xv = sol[3 * (size_t)(g - bp.node_off) + c];
            else xv = xv / (1.0 + (bp.calc_stokes == 1 ? map.drag_orig[n] : 0.0));
            // secondary rows of the viscosity matrix hold one (+ the Stokes drag)
            // on the diagonal only (src/NoMassCGSolver.cpp:109-139)
        }
    }
    if (st) return fail("blob %d: solve failed (status bits %d)", blob, st);
    return FFEA_GPU_OK;
}

int ffea_gpu_solver_apply(ffea_gpu_t *h, int32_t blob, const double *in, double *out)
{
    if (check_blob(h, blob)) return FFEA_GPU_ERROR;
    if (!in || !out) return fail("null argument");
    DeviceBatch &d = h->dev;
    const BlobParams &bp = h->host.bp[blob];
    const BlobMap &map = h->host.maps[blob];
    std::vector<double> v(3 * (size_t)d.nl_pad, 0.0);
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        if (g < 0 || map.pinned_orig[n]) continue;
        for (int c = 0; c < 3; c++) v[3 * (size_t)g + c] = in[3 * (size_t)n + c];
    }
    double *din = nullptr, *dout = nullptr;
    CK(cudaMallocAsync(&din, v.size() * sizeof(double), h->stream));
    CK(cudaMallocAsync(&dout, v.size() * sizeof(double), h->stream));
    CK(cudaMemcpyAsync(din, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_apply(d, h->stream, din, dout);
    CK(cudaMemcpyAsync(v.data(), dout, v.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaFreeAsync(din, h->stream));
    CK(cudaFreeAsync(dout, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int32_t n = 0; n < map.num_nodes_total; n++) {
        const int32_t g = map.lin_of_orig[n];
        for (int c = 0; c < 3; c++) {
            const size_t k = 3 * (size_t)n + c;
            if (g >= 0 && !map.pinned_orig[n]) out[k] = v[3 * (size_t)g + c];
            else out[k] = in[k];  // identity rows (pinned nodes; secondary nodes without drag)
        }
    }
    (void)bp;
    return FFEA_GPU_OK;
}

int ffea_gpu_rng_draws(const uint64_t state[6], uint64_t offset, int64_t count, double *out)
{
    if (!state || (!out && count > 0)) return fail("null argument");
    if (count <= 0) return FFEA_GPU_OK;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    mrg::JumpMat *table = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_table_mu);
        if ((int)g_tables.size() <= dev) g_tables.resize(dev + 1, nullptr);
        if (!g_tables[dev]) {
            std::vector<mrg::JumpMat> t(mrg::JUMP_TABLE_ENTRIES);
            mrg::build_jump_table(t.data());
            CK(cudaMalloc(&g_tables[dev], t.size() * sizeof(mrg::JumpMat)));
            CK(cudaMemcpy(g_tables[dev], t.data(), t.size() * sizeof(mrg::JumpMat), cudaMemcpyHostToDevice));
        }
        table = g_tables[dev];
    }
    uint32_t st[6];
    for (int i = 0; i < 6; i++) st[i] = (uint32_t)state[i];
    uint32_t *dst = nullptr;
    double *dout = nullptr;
    cudaStream_t s = nullptr;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaMallocAsync(&dst, sizeof(st), s));
    CK(cudaMallocAsync(&dout, (size_t)count * sizeof(double), s));
    CK(cudaMemcpyAsync(dst, st, sizeof(st), cudaMemcpyHostToDevice, s));
    launch_rng_draws(table, dst, offset, count, dout, s);
    CK(cudaMemcpyAsync(out, dout, (size_t)count * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaFreeAsync(dst, s));
    CK(cudaFreeAsync(dout, s));
    CK(cudaStreamSynchronize(s));
    CK(cudaStreamDestroy(s));
    return FFEA_GPU_OK;
}

}  // extern "C"

extern "C" int ffea_gpu_diag_spmv(ffea_gpu_t *h, int32_t variant, int32_t reps, double *us_per_spmv)
{
    if (!h || !us_per_spmv || reps <= 0) return fail("bad arguments");
    if (variant < 0 || variant > 3) return fail("SpMV variant must be 0..3");
    launch_spmv_variant(h->dev, h->stream, variant);  // warm-up
    CK(cudaEventRecord(h->ev[0], h->stream));
    for (int i = 0; i < reps; i++) launch_spmv_variant(h->dev, h->stream, variant);
    CK(cudaEventRecord(h->ev[1], h->stream));
    CK(cudaEventSynchronize(h->ev[1]));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
    CK(cudaGetLastError());
    *us_per_spmv = 1e3 * (double)ms / reps;
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_diag_coarse(ffea_gpu_t *h, int32_t blob, int32_t *n, float *coarse_matrix, float *inverse)
{
    if (!h || !n) return fail("bad arguments");
    if (blob < 0 || blob >= (int32_t)h->host.bp.size()) return fail("blob index %d out of range", blob);
    const BlobParams &bp = h->host.bp[blob];
    *n = h->dev.coarse ? bp.coarse_n : 0;
    if (*n == 0) return FFEA_GPU_OK;
    const size_t bytes = sizeof(float) * (size_t)bp.coarse_n * bp.coarse_n;
    CK(cudaStreamSynchronize(h->stream));
    if (coarse_matrix) CK(cudaMemcpy(coarse_matrix, h->dev.coarse_A + bp.coarse_xoff, bytes, cudaMemcpyDeviceToHost));
    if (inverse) CK(cudaMemcpy(inverse, h->dev.coarse_X + bp.coarse_xoff, bytes, cudaMemcpyDeviceToHost));
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_diag_coarse_half(ffea_gpu_t *h, int32_t blob, int32_t *n, int32_t *row_len,
                                         uint16_t *half_inverse, float *scale)
{
    if (!h || !n || !row_len) return fail("bad arguments");
    if (blob < 0 || blob >= (int32_t)h->host.bp.size()) return fail("blob index %d out of range", blob);
    const BlobParams &bp = h->host.bp[blob];
    *n = h->dev.coarse && h->dev.coarse_Xh ? bp.coarse_n : 0;
    *row_len = (*n + 7) / 8 * 8;
    if (*n == 0) return FFEA_GPU_OK;
    CK(cudaStreamSynchronize(h->stream));
    if (half_inverse)
        CK(cudaMemcpy(half_inverse, h->dev.coarse_Xh + bp.coarse_hxoff, sizeof(uint16_t) * (size_t)*n * *row_len,
                      cudaMemcpyDeviceToHost));
    if (scale)
        CK(cudaMemcpy(scale, h->dev.coarse_s + bp.coarse_off, sizeof(float) * (size_t)*n, cudaMemcpyDeviceToHost));
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_diag_sgemm(const float *a, const float *b, const float *d, float *c, int32_t n, int32_t batch,
                                   float alpha, float beta, void *stream)
{
    if (!a || !b || !c || n <= 0 || batch <= 0 || batch > 65535 || (beta != 0.f && !d)) return fail("bad arguments");
    if (n > 46340) return fail("n = %d: n^2 exceeds the int32 index range of a batch stride", n);
    // the split-K scratch of a large product (diagnostics may allocate)
    const int sp = sgemm_splits(n, batch);
    float *part = nullptr;
    if (sp > 1) CK(cudaMalloc(&part, sizeof(float) * (size_t)sp * batch * n * n));
    sgemm_batched(a, b, beta != 0.f ? d : nullptr, c, n, batch, alpha, beta, part, static_cast<cudaStream_t>(stream));
    cudaError_t e = cudaGetLastError();
    if (part) {
        if (e == cudaSuccess) e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
        cudaFree(part);
    }
    CK(e);
    return FFEA_GPU_OK;
}

extern "C" int ffea_gpu_diag_cg_vectors(ffea_gpu_t *h, int32_t blob, int32_t *rows, void *r, void *u, void *w,
                                        double *sums)
{
    if (!h || !rows) return fail("bad arguments");
    if (blob < 0 || blob >= (int32_t)h->host.bp.size()) return fail("blob index %d out of range", blob);
    const BlobParams &bp = h->host.bp[blob];
    *rows = bp.node_pad;  // the blob's rows with its padding rows (zero vectors)
    CK(cudaStreamSynchronize(h->stream));
    const size_t ts = h->dev.precision == PREC_FP64 ? sizeof(double) : sizeof(float);
    const size_t off = 3 * (size_t)bp.node_off * ts, bytes = 3 * (size_t)bp.node_pad * ts;
    if (r) CK(cudaMemcpy(r, static_cast<char *>(h->dev.r) + off, bytes, cudaMemcpyDeviceToHost));
    if (u) {
        // u from its published 16-byte copy (x, y, z, 0 per row), which the
        // memory-resident iteration keeps current
        std::vector<char> u4(4 * (size_t)bp.node_pad * ts);
        CK(cudaMemcpy(u4.data(), static_cast<char *>(h->dev.u4) + 4 * (size_t)bp.node_off * ts, u4.size(),
                      cudaMemcpyDeviceToHost));
        for (size_t r = 0; r < (size_t)bp.node_pad; r++)
            std::memcpy(static_cast<char *>(u) + 3 * r * ts, u4.data() + 4 * r * ts, 3 * ts);
    }
    if (w) CK(cudaMemcpy(w, static_cast<char *>(h->dev.w) + off, bytes, cudaMemcpyDeviceToHost));
    if (sums) CK(cudaMemcpy(sums, h->dev.last_sums + 3 * (size_t)blob, 3 * sizeof(double), cudaMemcpyDeviceToHost));
    return FFEA_GPU_OK;
}
