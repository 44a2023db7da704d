// GpuSolvers.h -- FFEA's linear-solver plugin backed by libffea_gb300.
//
// Drop-in classes for FFEA's Solver interface (include/Solver.h:30-55):
//   GpuNoMassCGSolver           in place of NoMassCGSolver          (<solver = CG_nomass>)
//   GpuConjugateGradientSolver  in place of ConjugateGradientSolver (<solver = CG>)
// A maintainer adds this file and GpuSolvers.cpp to FFEA's src/ and has
// Blob::init's factory (src/Blob.cpp:359-375) construct them for a new
// solver keyword.  They compile against FFEA's own headers and link against
// libffea_gb300.so through include/ffea_gpu.h (plain C ABI).
//
// Contract, as FFEA's solvers: init() takes the blob's nodes and elements as
// Blob::init holds them (meso units); solve(x) takes the rhs in x and
// overwrites it with the solution, returning FFEA_OK or FFEA_ERROR (0 / -1,
// include/FFEA_return_codes.h:35-36); pinned and binding-site-pinned nodes
// and secondary nodes are identity rows.  The NoMass matrix is assembled on
// the GPU from the nodes' current positions at every solve, as
// NoMassCGSolver::solve rebuilds it from the elements' current viscosity
// matrices (src/NoMassCGSolver.cpp:165-171).  apply_matrix(in, result) is
// result = K in over 3 N_t scalars for the matrix of the last solve.
#ifndef GPU_SOLVERS_H_INCLUDED
#define GPU_SOLVERS_H_INCLUDED

#include <set>
#include <vector>

#include "Solver.h"
#include "ffea_gpu.h"

class GpuSolverBase : public Solver {
public:
    GpuSolverBase(int solver_kind, int precision, int preconditioner);
    virtual ~GpuSolverBase();

    int init(int num_nodes, int num_elements, mesh_node *node, tetra_element_linear *elem, SimulationParams *params,
             int num_pinned_nodes, int *pinned_nodes_list, std::set<int> bsite_pinned_nodes_list);
    int solve(vector3 *x);
    void apply_matrix(scalar *in, scalar *result);

    /** The library's message for the last failure of this thread. */
    static const char *last_error();

private:
    GpuSolverBase(const GpuSolverBase &);
    GpuSolverBase &operator=(const GpuSolverBase &);

    int kind_, precision_, preconditioner_;
    ffea_gpu_t *h_;
    int num_nodes_;
    mesh_node *node_;
    std::vector<double> pos_, xs_;
};

/** NoMassCGSolver on the GPU; mixed precision and the Jacobi preconditioner
 *  of FFEA unless asked otherwise (FFEA_GPU_PRECISION_FP64 reproduces FFEA's
 *  FP64 arithmetic to the solver tolerance). */
class GpuNoMassCGSolver : public GpuSolverBase {
public:
    explicit GpuNoMassCGSolver(int precision = FFEA_GPU_PRECISION_MIXED, int preconditioner = FFEA_GPU_PRECOND_JACOBI)
        : GpuSolverBase(FFEA_GPU_SOLVER_NOMASS, precision, preconditioner)
    {
    }
};

/** ConjugateGradientSolver (mass matrix) on the GPU. */
class GpuConjugateGradientSolver : public GpuSolverBase {
public:
    explicit GpuConjugateGradientSolver(int precision = FFEA_GPU_PRECISION_MIXED)
        : GpuSolverBase(FFEA_GPU_SOLVER_MASS, precision, FFEA_GPU_PRECOND_JACOBI)
    {
    }
};

#endif
