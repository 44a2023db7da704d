// GpuSolvers.cpp -- see GpuSolvers.h.
#include "GpuSolvers.h"

#include <cstdio>

#include "FFEA_return_codes.h"
#include "SimulationParams.h"
#include "mesh_node.h"
#include "tetra_element_linear.h"

GpuSolverBase::GpuSolverBase(int solver_kind, int precision, int preconditioner)
    : kind_(solver_kind), precision_(precision), preconditioner_(preconditioner), h_(NULL), num_nodes_(0), node_(NULL)
{
}

GpuSolverBase::~GpuSolverBase()
{
    if (h_) ffea_gpu_destroy(h_);
}

const char *GpuSolverBase::last_error()
{
    static thread_local char msg[512];
    ffea_gpu_last_error(msg, sizeof(msg));
    return msg;
}

// The arrays ffea_gpu_create copies: what Blob::init leaves in the nodes and
// elements (src/Blob.cpp:270-420), and the SimulationParams fields the
// update reads.  Binding-site pinned nodes join the pinned list, as in
// NoMassCGSolver::init (src/NoMassCGSolver.cpp:78-87).
int GpuSolverBase::init(int num_nodes, int num_elements, mesh_node *node, tetra_element_linear *elem,
                        SimulationParams *params, int num_pinned_nodes, int *pinned_nodes_list,
                        std::set<int> bsite_pinned_nodes_list)
{
    if (h_) {
        ffea_gpu_destroy(h_);
        h_ = NULL;
    }
    num_nodes_ = num_nodes;
    node_ = node;
    std::vector<double> pos(3 * (size_t)num_nodes), vel(3 * (size_t)num_nodes), drag(num_nodes);
    std::vector<double> mat(5 * (size_t)num_elements);
    std::vector<int32_t> topo(10 * (size_t)num_elements);
    for (int i = 0; i < num_nodes; i++) {
        for (int c = 0; c < 3; c++) {
            pos[3 * i + c] = node[i].pos[c];
            vel[3 * i + c] = node[i].vel[c];
        }
        drag[i] = node[i].stokes_drag;
    }
    for (int e = 0; e < num_elements; e++) {
        for (int j = 0; j < 10; j++) topo[10 * e + j] = elem[e].n[j]->index;
        mat[5 * e + 0] = elem[e].rho;
        mat[5 * e + 1] = elem[e].A;
        mat[5 * e + 2] = elem[e].B;
        mat[5 * e + 3] = elem[e].G;
        mat[5 * e + 4] = elem[e].E;
    }
    std::set<int> pins(bsite_pinned_nodes_list);
    for (int i = 0; i < num_pinned_nodes; i++) pins.insert(pinned_nodes_list[i]);
    std::vector<int32_t> pinned(pins.begin(), pins.end());
    ffea_gpu_mesh m;
    m.num_nodes = num_nodes;
    m.num_elements = num_elements;
    m.pos = pos.data();
    m.vel = vel.data();
    m.topology = topo.data();
    m.material = mat.data();
    m.stokes_drag = params->calc_stokes ? drag.data() : NULL;
    m.num_pinned = (int32_t)pinned.size();
    m.pinned = pinned.empty() ? NULL : pinned.data();
    ffea_gpu_params q;
    q.dt = params->dt;
    q.kT = params->kT;
    q.epsilon2 = params->epsilon2;
    q.max_iterations_cg = params->max_iterations_cg;
    q.calc_noise = params->calc_noise;
    q.calc_stokes = params->calc_stokes;
    q.solver = kind_;
    q.precision = precision_;
    q.rng_seed = params->rng_seed;
    q.true_residual = 1;
    q.preconditioner = preconditioner_;
    if (ffea_gpu_create(&m, &q, &h_) != FFEA_GPU_OK) {
        h_ = NULL;
        FFEA_ERROR_MESSG("GPU solver: %s\n", last_error());
    }
    pos_.resize(3 * (size_t)num_nodes);
    xs_.resize(3 * (size_t)num_nodes);
    return FFEA_OK;
}

int GpuSolverBase::solve(vector3 *x)
{
    if (!h_) FFEA_ERROR_MESSG("GPU solver: solve() before a successful init()\n");
    for (int i = 0; i < num_nodes_; i++)
        for (int c = 0; c < 3; c++) {
            pos_[3 * i + c] = node_[i].pos[c];
            xs_[3 * i + c] = x[i][c];
        }
    if (ffea_gpu_solver_solve(h_, 0, pos_.data(), xs_.data()) != FFEA_GPU_OK)
        FFEA_ERROR_MESSG("GPU solver: %s\n", last_error());
    for (int i = 0; i < num_nodes_; i++)
        for (int c = 0; c < 3; c++) x[i][c] = xs_[3 * i + c];
    return FFEA_OK;
}

void GpuSolverBase::apply_matrix(scalar *in, scalar *result)
{
    if (!h_ || ffea_gpu_solver_apply(h_, 0, in, result) != FFEA_GPU_OK)
        fprintf(stderr, "GPU solver: apply_matrix failed: %s\n", h_ ? last_error() : "no handle");
}
