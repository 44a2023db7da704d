/*
 * ffea_gpu.h -- C ABI of the GB300 blob update for FFEA.
 *
 * This library replaces FFEA's per-timestep blob update -- the pair
 *   int Blob::update_internal_forces()   (include/Blob.h:130, src/Blob.cpp:638-735)
 *   int Blob::update_positions()         (include/Blob.h:140, src/Blob.cpp:737-764)
 * called for every blob by World::run (src/World.cpp:2024-2043) -- and the
 * linear-solver plugin behind it,
 *   class Solver { init(...); solve(vector3 *x); apply_matrix(scalar *in, scalar *result); }
 *                                          (include/Solver.h:30-55)
 * with its two CG implementations NoMassCGSolver (src/NoMassCGSolver.cpp)
 * and ConjugateGradientSolver (src/ConjugateGradientSolver.cpp).
 *
 * Conventions
 *  - Plain pointers and sizes only.  Host arrays are copied; nothing is kept
 *    from the caller's memory after a call returns.
 *  - All quantities are in FFEA meso units (include/dimensions.h:30-41), i.e.
 *    the values Blob and SimulationParams hold after loading.
 *  - Node arrays use the reference's own node numbering (linear and
 *    secondary nodes, N_t of them) and AoS x,y,z layout (vector3).
 *  - Every function returns FFEA_GPU_OK (0) or FFEA_GPU_ERROR (-1), the values
 *    of FFEA_OK / FFEA_ERROR (include/FFEA_return_codes.h:35-36).  The message
 *    of the last error on the calling thread is available from
 *    ffea_gpu_last_error().
 *  - Calls on one handle are not thread-safe; different handles may be used
 *    from different threads.  Each handle owns one CUDA stream.
 */
#ifndef FFEA_GPU_H
#define FFEA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFEA_GPU_OK 0
#define FFEA_GPU_ERROR (-1)

#define FFEA_GPU_SOLVER_NOMASS 0   /* <solver = CG_nomass>: NoMassCGSolver */
#define FFEA_GPU_SOLVER_MASS 1     /* <solver = CG>: ConjugateGradientSolver */
#define FFEA_GPU_SOLVER_LUMPED 2   /* <solver = masslumped>: MassLumpedSolver */

#define FFEA_GPU_PRECISION_FP64 0  /* every kernel in FP64 */
#define FFEA_GPU_PRECISION_MIXED 1 /* FP32 element forces, SpMV and CG vectors; FP64 positions and true
                                    * residual.  With true_residual on, the FP32 iterate bounds the
                                    * relative residual it can confirm at about 1e-7: tighter epsilons
                                    * need FP64 (a solve that cannot reach epsilon fails). */
/* Preconditioner of the NoMass CG solve.  JACOBI is NoMassCGSolver's
 * (src/NoMassCGSolver.cpp:278-291).  TWO_LEVEL adds a coarse correction
 * P A_c^-1 P^T r over six rigid modes per CG segment (a compact block of
 * about a thousand nodes), LEARNED also weights the Jacobi term per node by
 * ffea_gpu_set_smoother_weights.  Both stop on the same residual test; they
 * apply to NoMass blobs in mixed precision on the register-resident solve
 * path and fall back to JACOBI elsewhere (ffea_gpu_preconditioner reports
 * which). */
#define FFEA_GPU_PRECOND_JACOBI 0
#define FFEA_GPU_PRECOND_TWO_LEVEL 1
#define FFEA_GPU_PRECOND_LEARNED 2

#define FFEA_GPU_RNG_PER_BLOB 0    /* each blob draws from its own stream, seeded from its rng_seed */
#define FFEA_GPU_RNG_SHARED 1      /* all blobs share stream 0 in FFEA's single-thread draw order */

typedef struct ffea_gpu ffea_gpu_t;

/* One blob's mesh: what Blob holds after Blob::init (src/Blob.cpp:270-420). */
typedef struct {
    int32_t num_nodes;          /* N_t: linear + secondary nodes (Blob::num_nodes) */
    int32_t num_elements;       /* Blob::num_elements */
    const double *pos;          /* 3*num_nodes, mesh_node::pos */
    const double *vel;          /* 3*num_nodes, mesh_node::vel; NULL = at rest */
    const int32_t *topology;    /* 10*num_elements, tetra_element_linear::n[j]->index */
    const double *material;     /* 5*num_elements: rho, A, B, G, E (tetra_element_linear fields) */
    const double *stokes_drag;  /* num_nodes, mesh_node::stokes_drag; NULL = no drag */
    int32_t num_pinned;         /* Blob::num_pinned_nodes */
    const int32_t *pinned;      /* Blob::pinned_nodes_list */
} ffea_gpu_mesh;

/* The SimulationParams fields the update reads (include/SimulationParams.h:76-131). */
typedef struct {
    double dt;                  /* SimulationParams::dt */
    double kT;                  /* SimulationParams::kT */
    double epsilon2;            /* SimulationParams::epsilon2 (= epsilon^2) */
    int32_t max_iterations_cg;  /* SimulationParams::max_iterations_cg */
    int32_t calc_noise;         /* SimulationParams::calc_noise */
    int32_t calc_stokes;        /* SimulationParams::calc_stokes */
    int32_t solver;             /* FFEA_GPU_SOLVER_* (Blob::linear_solver) */
    int32_t precision;          /* FFEA_GPU_PRECISION_* */
    int32_t rng_seed;           /* SimulationParams::rng_seed, seeded as World::init does */
    int32_t true_residual;      /* 1: confirm every solve with an FP64 true residual */
    int32_t preconditioner;     /* FFEA_GPU_PRECOND_*; the same for every blob of a batch */
} ffea_gpu_params;

/* --- handle lifetime ----------------------------------------------------- */

/* One blob.  Replaces Blob::init's solver set-up (src/Blob.cpp:359-380) and
 * World::init's RNG seeding for a single OpenMP thread (src/World.cpp:299-317). */
int ffea_gpu_create(const ffea_gpu_mesh *mesh, const ffea_gpu_params *params, ffea_gpu_t **out);

/* Many blobs in one handle, stepped together by one launch sequence.  With
 * rng_mode FFEA_GPU_RNG_PER_BLOB blob b draws from its own stream seeded from
 * params[b].rng_seed; with FFEA_GPU_RNG_SHARED all blobs share the stream of
 * params[0].rng_seed in the order a one-thread World::run draws it
 * (src/World.cpp:2024-2043).  All blobs must use the same precision. */
int ffea_gpu_create_batch(int32_t num_blobs, const ffea_gpu_mesh *meshes, const ffea_gpu_params *params,
                          int32_t rng_mode, ffea_gpu_t **out);

void ffea_gpu_destroy(ffea_gpu_t *h);

/* --- stepping ------------------------------------------------------------ */

/* nsteps x (Blob::update_internal_forces + Blob::update_positions) for every
 * blob, with World::run's per-step force zeroing (src/World.cpp:1845,1907).
 * Returns FFEA_GPU_ERROR if an element inverted or a solve did not converge
 * in any blob; that blob stops at the failing step (see ffea_gpu_status). */
int ffea_gpu_step(ffea_gpu_t *h, int32_t nsteps);

/* --- state in / out (reference node numbering) --------------------------- */

/* pos/vel: mesh_node pos and vel; force: Blob::force after the last solve
 * (velocities for CG_nomass, accelerations for CG).  Any pointer may be NULL. */
int ffea_gpu_get_nodes(ffea_gpu_t *h, int32_t blob, double *pos, double *vel, double *force);
int ffea_gpu_set_nodes(ffea_gpu_t *h, int32_t blob, const double *pos, const double *vel);

/* External forces on a blob's nodes, added to the rhs of every following
 * step until replaced: count entries of (node index in the reference's
 * numbering, 3 force components in meso units); repeated nodes add up;
 * count 0 clears them.  They enter where FFEA's World interactions (springs,
 * src/World.cpp:3808-3846) and Blob::apply_ctforces (src/Blob.cpp:647,
 * 2094-2162) add to Blob::force before the element loop, after the per-step
 * zeroing (src/World.cpp:1907): a secondary node's force folds half onto
 * each end of its edge (Blob::linearise_force, src/Blob.cpp:1066-1085) and
 * pinned nodes keep none.  The first call on a handle allocates the buffer
 * and re-captures the step graphs. */
int ffea_gpu_set_external_forces(ffea_gpu_t *h, int32_t blob, int32_t count, const int32_t *nodes,
                                 const double *forces);

/* RngStream state words of a blob's stream (RngStream::GetState / SetSeed,
 * src/RngStream.cpp:381-399,439-443); the .fcp checkpoint holds these. */
int ffea_gpu_get_rng_state(ffea_gpu_t *h, int32_t blob, uint64_t state[6]);
int ffea_gpu_set_rng_state(ffea_gpu_t *h, int32_t blob, const uint64_t state[6]);

/* Strain and kinetic energy at the current state, as Blob::make_measurements
 * computes them (src/Blob.cpp:1363-1432); kinetic is 0 for CG_nomass. */
int ffea_gpu_energies(ffea_gpu_t *h, int32_t blob, double *strain, double *kinetic);

/* Blob::make_measurements (src/Blob.cpp:1363-1527) for blobs first_blob ..
 * first_blob + count - 1 at the current state: FFEA_GPU_NUM_MEASUREMENTS
 * values per blob into out, in meso units.  The centroid is the mean of all
 * N_t node positions; RMSD is taken against the positions given at creation
 * (Blob::set_pos_0, src/Blob.cpp:1035-1050) without removing the translation;
 * the centre of mass is Blob::get_CoM's sum (src/Blob.cpp:951-967), where the
 * element mass multiplies the first corner only and the sum is divided by
 * the element count; the angular momentum about that point is 0 for
 * CG_nomass.  Kinetic and strain energy are those of ffea_gpu_energies.  One
 * pass over the batch: the values of every blob are computed by each call. */
#define FFEA_GPU_MEAS_KINETIC 0
#define FFEA_GPU_MEAS_STRAIN 1
#define FFEA_GPU_MEAS_CENTROID 2  /* x, y, z: Blob::CoG */
#define FFEA_GPU_MEAS_RMSD 5      /* Blob::rmsd */
#define FFEA_GPU_MEAS_COM 6       /* x, y, z: Blob::CoM */
#define FFEA_GPU_MEAS_ANGMOM 9    /* x, y, z: Blob::L */
#define FFEA_GPU_NUM_MEASUREMENTS 12
int ffea_gpu_measurements(ffea_gpu_t *h, int32_t first_blob, int32_t count, double *out);

/* Status of the last step: inverted-element count, CG iterations of the last
 * solve, FP64 true relative residual ||b - A x|| / ||b|| of the last solve
 * (NaN when the check is off), and the failure bits (FFEA_GPU_FAIL_*). */
#define FFEA_GPU_FAIL_INVERSION 1  /* an element inverted (Blob::update_internal_forces' check) */
#define FFEA_GPU_FAIL_CG 2         /* the solve did not converge in max_iterations_cg */
#define FFEA_GPU_FAIL_NAN 4        /* non-finite values in the solve */
#define FFEA_GPU_FAIL_TIMEOUT 8    /* a grid barrier of the solve gave up waiting */
int ffea_gpu_status(ffea_gpu_t *h, int32_t blob, int32_t *inverted, int32_t *cg_iters, double *true_relres,
                    int32_t *fail_bits);

/* rhs of the last solve: Blob::force handed to Solver::solve after the
 * gather, Stokes terms, linearise_force and pinning (src/Blob.cpp:3826-3928). */
int ffea_gpu_get_rhs(ffea_gpu_t *h, int32_t blob, double *rhs);

/* Element nodal forces of the last step, 12 per element (corner 0..3 x,y,z):
 * tetra_element_linear::node_force[0..3] (src/tetra_element_linear.cpp:474-489). */
int ffea_gpu_get_element_forces(ffea_gpu_t *h, int32_t blob, double *out);

/* --- Solver plugin (include/Solver.h:30-55) ------------------------------- */

/* Solver::solve for the CURRENT node positions of `pos` (3*N_t): assembles
 * the viscosity (CG_nomass) or mass (CG) matrix and overwrites x (3*N_t) --
 * the rhs on entry -- with the solution.  Mirrors NoMassCGSolver::solve /
 * ConjugateGradientSolver::solve (src/NoMassCGSolver.cpp:165-197,
 * src/ConjugateGradientSolver.cpp:206-232). */
int ffea_gpu_solver_solve(ffea_gpu_t *h, int32_t blob, const double *pos, double *x);

/* Solver::apply_matrix: out = M in for the matrix of the last assembly,
 * in/out 3*N_t (NoMassCGSolver's V->apply, src/SparseMatrixFixedPattern.cpp:148-191). */
int ffea_gpu_solver_apply(ffea_gpu_t *h, int32_t blob, const double *in, double *out);

/* --- RNG ----------------------------------------------------------------- */

/* count draws of RngStream::RandU01 starting `offset` draws after `state`,
 * generated on the GPU with jump-ahead (for checks against RngStream). */
int ffea_gpu_rng_draws(const uint64_t state[6], uint64_t offset, int64_t count, double *out);

/* World::init's six seed words for an rng_seed (src/World.cpp:299-305). */
int ffea_gpu_ffea_seed(int32_t rng_seed, uint64_t out[6]);

/* --- FFEA script front end ----------------------------------------------- */

/* An FFEA input script (.ffea) read the way FFEA reads it
 * (SimulationParams::extract_params / assign, src/SimulationParams.cpp:184-550;
 * World::read_and_build_system, src/World.cpp:2205-2720) with its blob files
 * (.node, .top, .mat, .stokes, .pin: Blob::load_*, src/Blob.cpp:2415-2947,
 * 3691-3755), in meso units.  The subset is the blob update's: per blob one
 * DYNAMIC conformation, solver CG_nomass / CG / masslumped, scale, centroid,
 * velocity.  Parameters that switch on work outside the update (surface
 * interactions, electrostatics, kinetics, springs, constant forces, rods,
 * several conformations) are rejected with an error naming them;
 * calc_steric is accepted and not computed. */
#define FFEA_GPU_SCRIPT_PATH_MAX 1024

typedef struct ffea_gpu_script ffea_gpu_script_t;

/* The run settings of a script after SimulationParams::assign's unit
 * conversions (file names resolved against the script's directory; the
 * output names default to <script>.ftj, <script>.fm, <script>.fcp). */
typedef struct {
    double dt, kT, epsilon2, stokes_visc;   /* meso units */
    int64_t num_steps;
    int32_t check, rng_seed, max_iterations_cg, calc_noise, calc_stokes, restart, num_blobs, reserved;
    char trajectory_out_fname[FFEA_GPU_SCRIPT_PATH_MAX];
    char measurement_out_fname[FFEA_GPU_SCRIPT_PATH_MAX];
    char checkpoint_in[FFEA_GPU_SCRIPT_PATH_MAX];   /* empty if none */
    char checkpoint_out[FFEA_GPU_SCRIPT_PATH_MAX];
} ffea_gpu_script_params;

int ffea_gpu_script_load(const char *path, ffea_gpu_script_t **out);
void ffea_gpu_script_free(ffea_gpu_script_t *s);
int ffea_gpu_script_get_params(const ffea_gpu_script_t *s, ffea_gpu_script_params *out);

/* Blob `blob` of the script as ffea_gpu_create takes it.  The mesh arrays
 * belong to the script (valid until ffea_gpu_script_free); params carry the
 * script's values with precision MIXED, true_residual 1 and preconditioner
 * JACOBI, which the caller may change. */
int ffea_gpu_script_get_blob(const ffea_gpu_script_t *s, int32_t blob, ffea_gpu_mesh *mesh, ffea_gpu_params *params);

/* Every blob of the script in one batch handle, drawing from one RNG stream
 * in a one-thread FFEA run's order (FFEA_GPU_RNG_SHARED; for a single blob
 * the same as its own stream). */
int ffea_gpu_script_create(const ffea_gpu_script_t *s, int32_t precision, int32_t preconditioner,
                           int32_t true_residual, ffea_gpu_t **out);

/* --- surface-surface interactions ----------------------------------------- */

/* Replaces VdW_solver (include/VdW_solver.h:36-127; VdW_solver::init,
 * src/VdW_solver.cpp:124-157, and ::solve, :168-210) and its variants
 * Steric_solver, LJSteric_solver and GenSoftSSINT_solver
 * (src/Steric_solver.cpp, src/LJSteric_solver.cpp, src/GenSoftSSINT_solver.cpp)
 * for ssint_type lennard-jones, steric, ljsteric and gensoft, with the
 * nearest-neighbour grid they walk (NearestNeighbourLinkedListCube,
 * src/NearestNeighbourLinkedListCube.cpp:27-76) and the aggregation of face
 * forces onto nodes (src/Blob.cpp:3841-3851).  The resulting node forces
 * enter the blob update through ffea_gpu_set_external_forces. */
#define FFEA_GPU_SSINT_MAX_CELLS (1 << 26)

#define FFEA_GPU_SSINT_LJ 0        /* lennard-jones */
#define FFEA_GPU_SSINT_STERIC 1    /* steric: overlap volume of the faces' element tetrahedra */
#define FFEA_GPU_SSINT_LJSTERIC 2  /* steric where the tetrahedra overlap, else lennard-jones */
#define FFEA_GPU_SSINT_GENSOFT 3   /* steric where the tetrahedra overlap, else the soft polynomial */
/* a face's tetrahedron overlaps at most this many others in one call (more is an error) */
#define FFEA_GPU_SSINT_MAX_STERIC_PARTNERS 32

typedef struct ffea_gpu_ssint ffea_gpu_ssint_t;

typedef struct {
    int32_t num_nodes;        /* nodes of all blobs, one numbering (e.g. blobs concatenated) */
    int32_t num_faces;        /* surface faces of all blobs, in FFEA's pool order (blob, then face) */
    const int32_t *faces;     /* 3 corner node indices per face (Face::n[0..2]) */
    const int32_t *face_blob; /* blob index per face (Face::daddy_blob->blob_index) */
    const int32_t *face_type; /* interaction type per face; -1 = not active (Blob::get_face) */
    int32_t num_types;        /* SSINT_matrix::num_ssint_face_types */
    const double *emin;       /* num_types^2, meso energy / area^2 (src/LJ_matrix.cpp:141) */
    const double *rmin;       /* num_types^2, meso length (src/LJ_matrix.cpp:142) */
    int32_t num_blobs;
    double cell_size;         /* SimulationParams::ssint_cutoff */
    int32_t nx, ny, nz;       /* SimulationParams::es_N_x/y/z; nx*ny*nz <= FFEA_GPU_SSINT_MAX_CELLS */
    int32_t inc_self;         /* SimulationParams::inc_self_ssint */
    /* the steric types (ssint_type other than FFEA_GPU_SSINT_LJ; zero-initialise the
     * fields below for lennard-jones) */
    int32_t ssint_type;       /* FFEA_GPU_SSINT_*: SimulationParams::ssint_type */
    const int32_t *face_apex; /* per face, the fourth node of its element (Face::n[3]) */
    double steric_factor;     /* SimulationParams::steric_factor */
    double steric_dr;         /* SimulationParams::steric_dr (meso length) */
    const double *k0;         /* num_types^2, gensoft k0 in meso energy / area (src/LJ_matrix.cpp:245) */
} ffea_gpu_ssint_desc;

/* Copies the face lists and parameters to the device (VdW_solver::init and
 * World::init's pool set-up, src/World.cpp:925-960). */
int ffea_gpu_ssint_create(const ffea_gpu_ssint_desc *desc, ffea_gpu_ssint_t **out);
void ffea_gpu_ssint_destroy(ffea_gpu_ssint_t *s);

/* One VdW_solver::solve on HOST arrays: pos (3*num_nodes) in, force
 * (3*num_nodes, the surface forces alone, overwritten) and energy
 * (num_blobs^2, VdW_solver::fieldenergy[blob of f1][blob of f2]) out;
 * pairs (may be NULL) receives the number of interacting face pairs.  A
 * face centroid outside the grid after one periodic wrap is an error, as in
 * LinkedListCube::add_node_to_stack (src/LinkedListCube.tpp:217-235). */
int ffea_gpu_ssint_forces(ffea_gpu_ssint_t *s, const double *pos, double *force, double *energy, int64_t *pairs);

/* The same on DEVICE arrays, enqueued on the handle's stream without
 * waiting.  Its errors -- face centroids outside the grid, or a grid cell
 * holding more than 4096 faces (a grid far too coarse for the mesh) -- are
 * only known on the device: call ffea_gpu_ssint_synchronize after it to
 * wait, read the pair count and get that call's error; a caller that only
 * synchronises the stream itself does not see them.
 * Forces are summed in a fixed order (bit-reproducible run to run); the
 * per-blob-pair energies are summed with FP64 atomics, so their last bits
 * can vary from run to run. */
int ffea_gpu_ssint_forces_device(ffea_gpu_ssint_t *s, const double *pos, double *force, double *energy);
int ffea_gpu_ssint_synchronize(ffea_gpu_ssint_t *s, int64_t *pairs);

/* Periodic blob corrections for the following passes (force_pbc): blob_corr
 * is num_blobs x num_blobs x 3 doubles (host), as World::calc_blob_corr_matrix
 * fills it (src/World.cpp:4460-4483); NULL turns them off.  In a pair (f1 =
 * the lower pool index) the Lennard-Jones and soft potentials take f1's
 * corners minus blob_corr[b2][b1] (Face::barycentric_calc_point_f2,
 * src/Face.cpp:271-277), the steric overlap f2's tetrahedron minus
 * blob_corr[b1][b2] (src/Face.cpp:517-531), and the in-front test the
 * separation c2 - c1 - blob_corr[b1][b2] (src/VdW_solver.cpp:365-369).
 * Replaces the solve(blob_corr) argument of VdW_solver. */
int ffea_gpu_ssint_set_pbc(ffea_gpu_ssint_t *s, const double *blob_corr);

/* World::calc_blob_corr_matrix on the host: blob_corr[i][j] = box *
 * floor((c_j - c_i + box / 2) / box) per axis for i < j, its negation for
 * j < i, zero on the diagonal; centroids: 3 per blob; box: the grid's extent
 * (cell size x cells per axis). */
int ffea_gpu_ssint_blob_corr(int32_t num_blobs, const double *centroids, const double box[3], double *blob_corr);

/* The sticky xz walls (sticky_wall_xz = 1; VdW_solver::solve_sticky_wall,
 * src/VdW_solver.cpp:216-235, 396-456), applied after the pair pass of the
 * following calls: the faces of the grid's bottom and top rows of cells
 * that face the wall at y = 0 (y = cell_size x ny) feel the Lennard-Jones
 * force of their own type pair in y.  Needs ny >= 2 (FFEA's row loop does
 * not end for ny = 1).  The wall energy is not recorded, as in FFEA. */
int ffea_gpu_ssint_set_sticky_wall(ffea_gpu_ssint_t *s, int32_t enable);
void *ffea_gpu_ssint_stream(ffea_gpu_ssint_t *s);

/* --- allocation-free measurement ------------------------------------------ */

/* Strain and kinetic energy of one blob, like ffea_gpu_energies, for callers
 * that cannot allocate device memory where they measure (for instance a host
 * code's own time-step loop, where cudaMalloc would synchronise the device
 * and fragment a pool the host manages).  This entry point has no counterpart
 * in FFEA; it allocates nothing.
 *   Inputs and output are DEVICE pointers owned by the caller: pos, vel (may
 *   be NULL), rest_pos (positions the rest state is taken from) -- 3*N_t
 *   doubles each in the reference node numbering --, topology (10 int32 per
 *   element), material (rho, A, B, G, E per element), out (2 doubles: strain,
 *   kinetic).  solver selects whether the kinetic term is evaluated (the
 *   mass and lumped-mass paths).
 *   The topology is NOT checked: this entry point is not told the node count,
 *   so every index must be a valid node of pos, vel and rest_pos
 *   (0 <= index < N_t); an index outside reads past the caller's arrays.
 *   ffea_gpu_create checks the topology it is given; a caller that measures a
 *   handle's own mesh passes that same topology.
 *   Scratch is a static device array of the library sized for at most
 *   2,097,152 elements; larger meshes are rejected with an error.  Every GPU
 *   that loads the library holds that array (256 KiB) until the process exits.
 *   The first call on a device looks the array up on that device; make that
 *   first call before any stream capture.  All calls share the array: calls
 *   that overlap on the GPU (different streams, no ordering) race.
 *   Work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *   stream); the result is ready when the stream reaches that point. */
int ffea_gpu_energies_noalloc(const double *pos, const double *vel, const int32_t *topology, const double *rest_pos,
                              const double *material, int32_t num_elements, int32_t solver, double *out,
                              void *stream);

/* --- diagnostics --------------------------------------------------------- */

/* Copies the last error message of the calling thread (NUL-terminated). */
int ffea_gpu_last_error(char *buf, size_t len);

/* Average time (microseconds) of one standalone w = A u over every row of
 * the handle's last assembled viscosity matrix, for SpMV variant 0..3
 * (0: one thread per row with grouped loads, 1: one thread per row,
 * 2: two threads per row, 3: four threads per row).  Overwrites the solver's
 * scratch vector w. */
int ffea_gpu_diag_spmv(ffea_gpu_t *h, int32_t variant, int32_t reps, double *us_per_spmv);

/* The two-level preconditioner's dense coarse matrix A_c of one blob and
 * its current inverse X ~ A_c^-1 (Newton-Schulz), each n x n FP32 row-major,
 * copied to host arrays (either may be NULL; query n first with both NULL).
 * n = 0 when the handle has no coarse space.  No reference counterpart. */
int ffea_gpu_diag_coarse(ffea_gpu_t *h, int32_t blob, int32_t *n, float *coarse_matrix, float *inverse);

/* The FP16 copy of a blob's coarse inverse that the memory-resident CG
 * kernel reads: scale[i] = sqrt(X_ii) (1 where X_ii is not a positive finite
 * number) and half_inverse = X_ij / (scale[i] scale[j]) rounded to FP16 (IEEE
 * binary16 bit patterns), n rows of *row_len halves (n rounded up to 8, the
 * padding zero), copied to host arrays (either may be NULL; query n and
 * *row_len first with both NULL).  n = 0 when the handle keeps no such copy
 * (no coarse space, or the register-resident kernel).  No reference
 * counterpart. */
int ffea_gpu_diag_coarse_half(ffea_gpu_t *h, int32_t blob, int32_t *n, int32_t *row_len, uint16_t *half_inverse,
                              float *scale);

/* The coarse space's dense product on DEVICE arrays: c = alpha a b + beta d
 * for `batch` row-major n x n FP32 matrices n^2 apart (d may be NULL when
 * beta = 0; c may be d), enqueued on `stream` (cudaStream_t).  No reference
 * counterpart: a test point for the Newton-Schulz update. */
int ffea_gpu_diag_sgemm(const float *a, const float *b, const float *d, float *c, int32_t n, int32_t batch,
                        float alpha, float beta, void *stream);

/* The CG vectors r, u = M r and w = A u of one blob's rows as the solver
 * holds them in memory (the arithmetic type: float in mixed precision,
 * double in FP64; 3 per row, the handle's internal row order; `rows` rows,
 * the blob's rows and its padding rows, whose vectors are zero: query `rows`
 * first with NULL arrays),
 * and the sums r.u, w.u, r.r of the solver's last reduction for that blob.
 * The vectors are kept in memory by the memory-resident solve (environment
 * FFEA_GPU_CG_MEMORY_STATE=1 at creation forces it); after a converged solve
 * they and the sums belong to the same iteration.  Any pointer may be NULL.
 * No reference counterpart: a test point for the reductions' accuracy. */
int ffea_gpu_diag_cg_vectors(ffea_gpu_t *h, int32_t blob, int32_t *rows, void *r, void *u, void *w, double *sums);

/* Number of kernel launches the library issued so far (all handles). */
int64_t ffea_gpu_kernel_launches(void);

/* Sizes of a handle: total linear nodes, elements and edges across blobs. */
int ffea_gpu_sizes(ffea_gpu_t *h, int64_t *linear_nodes, int64_t *elements, int64_t *edges);

/* The preconditioner the handle's solves use (FFEA_GPU_PRECOND_*), after the
 * fall-back rules above; -1 on a null handle.  No reference counterpart. */
int ffea_gpu_preconditioner(ffea_gpu_t *h);

/* Failure-detection self-test of the solve's grid barrier: `ctas` CTAs wait
 * for one arrival more than there are, each gives up after `spin_limit`
 * sleeps of ~32 ns and raises the barrier's time-out flag, which the solve
 * reports as FFEA_GPU_FAIL_TIMEOUT.  *timed_out = number of CTAs that
 * reported it (ctas when the time-out works).  No reference counterpart. */
int ffea_gpu_selftest_barrier_timeout(int32_t ctas, int32_t spin_limit, int32_t *timed_out);

/* Per-node weights of the Jacobi term of the LEARNED preconditioner for one
 * blob: omega[num_nodes] in the blob's node order (secondary nodes ignored),
 * each in (0, 2].  Takes effect from the next solve.  No reference
 * counterpart. */
int ffea_gpu_set_smoother_weights(ffea_gpu_t *h, int32_t blob, const float *omega);

/* --- learned smoother weights (no reference counterpart) --------------------
 * A mesh message-passing network sets omega for every free node of every
 * NoMass blob: 8 features per node from the current matrix and coarse
 * layout, three layers h' = ReLU(Ws h + Wn mean(h over edge neighbours) + b)
 * of width 32 (BF16 activations, FP32 weights and sums), omega = 2
 * sigmoid(wo . h + bo).  theta holds ffea_gpu_mpnn_num_params() floats:
 * per layer Ws (32 x din, row-major), Wn (32 x din), b (32) with din = 8, 32,
 * 32; then wo (32), bo.  The handle must use the LEARNED preconditioner. */
int ffea_gpu_mpnn_num_params(void);

/* Evaluate the network on the current mesh and use its omega from the next
 * solve on. */
int ffea_gpu_mpnn_apply(ffea_gpu_t *h, const float *theta);

/* Training signal from the last solve's (rhs f, solution x) pair, on that
 * solve's matrix A and coarse inverse: loss = e^T A e / x^T f with
 * e = x - M f, M the preconditioner with the network's omega; grad (may be
 * NULL) = dloss/dtheta. */
int ffea_gpu_mpnn_loss_grad(ffea_gpu_t *h, const float *theta, double *loss, float *grad);

/* For testing the network against a CPU restatement: for blob `blob`, the
 * features (8 per node) and omega (1 per node) of theta, in the blob's node
 * order (zero / 1 on secondary and pinned nodes), and the gradient of
 * sum_n domega[n] omega[n] with respect to theta (domega per node). */
int ffea_gpu_mpnn_probe(ffea_gpu_t *h, int32_t blob, const float *theta, const float *domega, float *features,
                        float *omega, float *grad);

/* Per-phase timing of the last ffea_gpu_step call, measured with CUDA events
 * on the handle's stream (milliseconds): elements, assembly, node gather,
 * CG solve with the update, and 0 (the former separate update).  Only
 * filled when timing was enabled. */
int ffea_gpu_set_timing(ffea_gpu_t *h, int32_t enable);
int ffea_gpu_phase_times(ffea_gpu_t *h, double out_ms[5]);

/* The same timing per kernel (milliseconds, summed over the steps of the
 * last ffea_gpu_step call): random draws (k_noise), element forces
 * (k_elements), viscosity assembly (k_assemble), coarse-space refresh (every
 * tenth step with the two-level preconditioner, else 0), node gather
 * (k_nodes), CG solve with the Euler update at its end (k_cg), and a last
 * slot, now 0, that held the separate update kernel.  No reference
 * counterpart: it exists for the per-kernel roofline. */
#define FFEA_GPU_NUM_KERNEL_TIMES 7
int ffea_gpu_kernel_times(ffea_gpu_t *h, double out_ms[FFEA_GPU_NUM_KERNEL_TIMES]);

/* The handle's CUDA stream (cudaStream_t), for callers that order their own
 * work after a step. */
void *ffea_gpu_stream(ffea_gpu_t *h);

/* Execution mode: 1 = one CUDA graph per step (default); 0 = direct launches. */
int ffea_gpu_set_graph_mode(ffea_gpu_t *h, int32_t enable);

/* Enqueue nsteps steps on the handle's stream and return without waiting
 * (graph mode only); ffea_gpu_synchronize waits and reports failures the way
 * ffea_gpu_step does. */
int ffea_gpu_step_async(ffea_gpu_t *h, int32_t nsteps);
int ffea_gpu_synchronize(ffea_gpu_t *h);

/* Iterations of the CG loop (each one SpMV and one vector update over every
 * blob still iterating) that the handle's persistent solver kernel executed. */
int64_t ffea_gpu_cg_loop_count(ffea_gpu_t *h);

#ifdef __cplusplus
}
#endif

#endif /* FFEA_GPU_H */
