// ref_harness.cpp -- drives FFEA's OWN C++ objects for the blob update.
//
// TEST INFRASTRUCTURE ONLY (used to pin the C oracle and to generate the
// golden vectors under tests/golden/).  Built by oracle/Makefile from the
// reference sources in place into oracle/_ref/; never shipped, never on the
// product path.
//
// FFEA's Blob.cpp / World.cpp cannot be compiled here (include/Blob.h:39 and
// include/World.h need Eigen 3.3.7, which the reference downloads at configure
// time, cmake/GetEigen3.cmake:33).  This harness therefore restates the few
// lines of Blob / World orchestration around the reference's own classes:
// tetra_element_linear, NoMassCGSolver, ConjugateGradientSolver, RngStream,
// SimulationParams, mesh_node, mat_vec_fns.  Each block cites the lines it
// follows.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <set>

#include "ConjugateGradientSolver.h"
#include "NoMassCGSolver.h"
#include "MassLumpedSolver.h"
#include "RngStream.h"
#include "SimulationParams.h"
#include "mat_vec_fns.h"
#include "mesh_node.h"
#include "tetra_element_linear.h"

namespace {

struct RefBlob {
    int num_nodes = 0, num_elements = 0, solver_kind = 0, num_pinned = 0;
    mesh_node *node = nullptr;
    tetra_element_linear *elem = nullptr;
    vector3 *force = nullptr;
    int *pinned = nullptr;
    SimulationParams params;
    Solver *solver = nullptr;
    RngStream *rng = nullptr;
    int last_inversions = 0;
    std::set<int> bsite;
    double *rhs_copy = nullptr;
};

// RAND as defined in include/tetra_element_linear.h:118, thread 0.
#define REF_RAND(A, B) ((A) + ((B) - (A)) * (b->rng[0].RandU01()))

// Blob::update_internal_forces (src/Blob.cpp:638-735), one thread.
int ref_internal_forces(RefBlob *b)
{
    matrix3 J, stress;
    vector12 du;
    int num_inversions = 0;
    if (b->num_pinned == b->num_nodes) {  // src/Blob.cpp:643-645
        b->last_inversions = 0;
        return FFEA_OK;
    }
    for (int n = 0; n < b->num_elements; n++) {
        b->elem[n].calculate_jacobian(J);
        if (b->elem[n].calc_shape_function_derivatives_and_volume(J) == FFEA_ERROR) num_inversions++;
        b->elem[n].create_viscosity_matrix();
        mat3_set_zero(stress);
        b->elem[n].add_shear_elastic_stress(J, stress);
        b->elem[n].add_bulk_elastic_stress(stress);
        if (b->params.calc_noise == 1) b->elem[n].add_fluctuating_stress(&b->params, b->rng, stress, 0);
        b->elem[n].internal_stress_mag = sqrt(mat3_double_contraction_symmetric(stress));
        if (b->solver_kind != 0) {
            b->elem[n].get_element_velocity_vector(du);
            mat12_apply(b->elem[n].viscosity_matrix, du);
        } else {
            vec12_set_zero(du);
        }
        b->elem[n].apply_stress_tensor(stress, du);
        b->elem[n].add_element_force_vector(du);
    }
    b->last_inversions = num_inversions;
    return num_inversions ? FFEA_ERROR : FFEA_OK;
}

// Blob::linearise_force (src/Blob.cpp:1066-1085)
void ref_linearise_force(RefBlob *b)
{
    int nIdx[10];
    vector3 *force = b->force;
    for (int i = 0; i < b->num_elements; i++) {
        for (int j = 0; j < 10; j++) nIdx[j] = b->elem[i].n[j]->index;
        for (int j = 0; j < 3; j++) {
            force[nIdx[0]][j] += 0.5 * (force[nIdx[4]][j] + force[nIdx[5]][j] + force[nIdx[6]][j]);
            force[nIdx[1]][j] += 0.5 * (force[nIdx[4]][j] + force[nIdx[7]][j] + force[nIdx[8]][j]);
            force[nIdx[2]][j] += 0.5 * (force[nIdx[5]][j] + force[nIdx[7]][j] + force[nIdx[9]][j]);
            force[nIdx[3]][j] += 0.5 * (force[nIdx[6]][j] + force[nIdx[8]][j] + force[nIdx[9]][j]);
        }
        for (int j = 4; j < 10; j++) {
            force[nIdx[j]][0] = 0.;
            force[nIdx[j]][1] = 0.;
            force[nIdx[j]][2] = 0.;
        }
    }
}

// Blob::aggregate_forces_and_solve (src/Blob.cpp:3826-3931), no faces.
int ref_aggregate_and_solve(RefBlob *b)
{
    vector3 *force = b->force;
    for (int n = 0; n < b->num_nodes; n++)
        for (int m = 0; m < b->node[n].num_element_contributors; m++) {
            force[n][0] += b->node[n].force_contributions[m]->x;
            force[n][1] += b->node[n].force_contributions[m]->y;
            force[n][2] += b->node[n].force_contributions[m]->z;
        }
    SimulationParams *params = &b->params;
    if (params->calc_stokes == 1) {
        if (b->solver_kind != 0) {
            for (int i = 0; i < b->num_nodes; i++) {
                force[i].x -= b->node[i].vel.x * b->node[i].stokes_drag;
                force[i].y -= b->node[i].vel.y * b->node[i].stokes_drag;
                force[i].z -= b->node[i].vel.z * b->node[i].stokes_drag;
                if (params->calc_noise == 1) {
                    force[i].x -= REF_RAND(-.5, .5) * sqrt((24 * params->kT * b->node[i].stokes_drag) / (params->dt));
                    force[i].y -= REF_RAND(-.5, .5) * sqrt((24 * params->kT * b->node[i].stokes_drag) / (params->dt));
                    force[i].z -= REF_RAND(-.5, .5) * sqrt((24 * params->kT * b->node[i].stokes_drag) / (params->dt));
                }
            }
        } else if (params->calc_noise == 1) {
            for (int i = 0; i < b->num_nodes; i++) {
                force[i].x -= REF_RAND(-.5, .5) * sqrt((24 * params->kT * b->node[i].stokes_drag) / (params->dt));
                force[i].y -= REF_RAND(-.5, .5) * sqrt((24 * params->kT * b->node[i].stokes_drag) / (params->dt));
                force[i].z -= REF_RAND(-.5, .5) * sqrt((24 * params->kT * b->node[i].stokes_drag) / (params->dt));
            }
        }
    }
    ref_linearise_force(b);
    for (int n = 0; n < b->num_pinned; n++) {
        int pn = b->pinned[n];
        force[pn].x = 0;
        force[pn].y = 0;
        force[pn].z = 0;
    }
    for (int i = 0; i < b->num_nodes; i++)
        for (int c = 0; c < 3; c++) b->rhs_copy[3 * i + c] = force[i][c];
    return b->solver->solve(force);
}

// Blob::euler_integrate (src/Blob.cpp:3937-3969) + linearise_element loop (:759-761)
void ref_euler(RefBlob *b)
{
    const double dt = b->params.dt;
    vector3 *force = b->force;
    if (b->solver_kind == 0) {
        for (int i = 0; i < b->num_nodes; i++) {
            b->node[i].vel[0] = force[i][0];
            b->node[i].vel[1] = force[i][1];
            b->node[i].vel[2] = force[i][2];
            b->node[i].pos[0] += force[i][0] * dt;
            b->node[i].pos[1] += force[i][1] * dt;
            b->node[i].pos[2] += force[i][2] * dt;
        }
    } else {
        for (int i = 0; i < b->num_nodes; i++) {
            b->node[i].vel[0] += force[i][0] * dt;
            b->node[i].vel[1] += force[i][1] * dt;
            b->node[i].vel[2] += force[i][2] * dt;
            b->node[i].pos[0] += b->node[i].vel[0] * dt;
            b->node[i].pos[1] += b->node[i].vel[1] * dt;
            b->node[i].pos[2] += b->node[i].vel[2] * dt;
        }
    }
    for (int n = 0; n < b->num_elements; n++) b->elem[n].linearise_element();
}

}  // namespace

extern "C" {

// Same argument meaning as orc_blob_create in ffea_oracle.c.
void *ref_blob_create(int num_nodes, int num_elements, const double *pos, const int *topo, const double *material,
                      const double *stokes_drag, int num_pinned, const int *pinned, const double *fparams,
                      const int *iparams)
{
    RefBlob *b = new RefBlob();
    b->num_nodes = num_nodes;
    b->num_elements = num_elements;
    b->params.dt = fparams[0];
    b->params.kT = fparams[1];
    b->params.epsilon2 = fparams[2];
    b->params.max_iterations_cg = iparams[0];
    b->params.calc_noise = iparams[1];
    b->params.calc_stokes = iparams[2];
    b->params.calc_es = 0;
    b->params.calc_ctforces = 0;
    b->solver_kind = iparams[3];
    b->node = new mesh_node[num_nodes];
    b->force = new vector3[num_nodes];
    b->rhs_copy = new double[3 * num_nodes];
    // Blob::load_nodes (src/Blob.cpp:2487-2499)
    for (int i = 0; i < num_nodes; i++) {
        b->node[i].pos.x = pos[3 * i];
        b->node[i].pos.y = pos[3 * i + 1];
        b->node[i].pos.z = pos[3 * i + 2];
        b->node[i].vel.x = b->node[i].vel.y = b->node[i].vel.z = 0;
        b->node[i].index = i;
        b->node[i].stokes_drag = stokes_drag ? stokes_drag[i] : 0.0;
        b->force[i].x = b->force[i].y = b->force[i].z = 0;
    }
    // Blob::load_topology (src/Blob.cpp:2605-2625) + load_material_params (:2862-2868)
    b->elem = new tetra_element_linear[num_elements];
    for (int e = 0; e < num_elements; e++) {
        for (int j = 0; j < 10; j++) b->elem[e].n[j] = &b->node[topo[10 * e + j]];
        for (int j = 0; j < 4; j++) b->node[topo[10 * e + j]].set_linear();
        b->elem[e].index = e;
        b->elem[e].rho = material[5 * e + 0];
        b->elem[e].A = material[5 * e + 1];
        b->elem[e].B = material[5 * e + 2];
        b->elem[e].G = material[5 * e + 3];
        b->elem[e].E = material[5 * e + 4];
    }
    b->num_pinned = num_pinned;
    b->pinned = new int[num_pinned + 1];
    for (int i = 0; i < num_pinned; i++) b->pinned[i] = pinned[i];
    // Blob::init: linearise, rest state, connectivity, solver (src/Blob.cpp:334-380, :3760-3822, :3974-4019)
    for (int e = 0; e < num_elements; e++) b->elem[e].linearise_element();
    for (int e = 0; e < num_elements; e++) {
        matrix3 J;
        scalar temp;
        b->elem[e].calculate_jacobian(J);
        mat3_invert(J, b->elem[e].J_inv_0, &temp);
        b->elem[e].calc_shape_function_derivatives_and_volume(J);
        b->elem[e].vol_0 = b->elem[e].vol;
        b->elem[e].mass = b->elem[e].vol_0 * b->elem[e].rho;
    }
    for (int i = 0; i < num_nodes; i++) b->node[i].num_element_contributors = 0;
    for (int e = 0; e < num_elements; e++)
        for (int j = 0; j < 10; j++) b->node[b->elem[e].n[j]->index].num_element_contributors++;
    for (int i = 0; i < num_nodes; i++) b->node[i].force_contributions = new vector3 *[b->node[i].num_element_contributors];
    int *counter = new int[num_nodes]();
    for (int e = 0; e < num_elements; e++)
        for (int j = 0; j < 10; j++) {
            int ni = b->elem[e].n[j]->index;
            b->node[ni].force_contributions[counter[ni]++] = &b->elem[e].node_force[j];
        }
    delete[] counter;
    // the solver factory of Blob::init (src/Blob.cpp:359-375)
    if (b->solver_kind == 0) b->solver = new NoMassCGSolver();
    else if (b->solver_kind == 2) b->solver = new MassLumpedSolver();
    else b->solver = new ConjugateGradientSolver();
    if (b->solver->init(num_nodes, num_elements, b->node, b->elem, &b->params, num_pinned, b->pinned, b->bsite) ==
        FFEA_ERROR) {
        return nullptr;
    }
    b->rng = nullptr;
    return b;
}

// World::init seeding for one OpenMP thread (src/World.cpp:299-317), using
// the C library's srand/rand exactly as the reference does.
void ref_blob_seed(void *h, int rng_seed)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    unsigned long sixseed[6];
    unsigned long twoMax[2] = {4294967087UL, 4294944443UL};
    srand(rng_seed);
    for (int i = 0; i < 6; i++) sixseed[i] = (rand() + rand()) % twoMax[i / 3];
    RngStream::SetPackageSeed(sixseed);
    delete[] b->rng;
    b->rng = new RngStream[1];
}

void ref_ffea_seed(int rng_seed, uint64_t *out)
{
    unsigned long twoMax[2] = {4294967087UL, 4294944443UL};
    srand(rng_seed);
    for (int i = 0; i < 6; i++) out[i] = (rand() + rand()) % twoMax[i / 3];
}

void ref_blob_set_rng_state(void *h, const uint64_t *st)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    unsigned long s[6];
    for (int i = 0; i < 6; i++) s[i] = st[i];
    if (!b->rng) b->rng = new RngStream[1];
    b->rng[0].SetSeed(s);
}

void ref_blob_get_rng_state(void *h, uint64_t *st)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    unsigned long s[6];
    b->rng[0].GetState(s);
    for (int i = 0; i < 6; i++) st[i] = s[i];
}

// One World::run step (src/World.cpp:1845,1907,2024-2043).
int ref_blob_step(void *h, int nsteps)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    for (int s = 0; s < nsteps; s++) {
        for (int e = 0; e < b->num_elements; e++) b->elem[e].zero_force();
        for (int i = 0; i < b->num_nodes; i++) b->force[i].x = b->force[i].y = b->force[i].z = 0;
        if (ref_internal_forces(b) != FFEA_OK) return FFEA_ERROR;
        if (ref_aggregate_and_solve(b) != FFEA_OK) return FFEA_ERROR;
        ref_euler(b);
    }
    return FFEA_OK;
}

void ref_blob_get_nodes(void *h, double *pos, double *vel, double *force)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    for (int i = 0; i < b->num_nodes; i++)
        for (int c = 0; c < 3; c++) {
            if (pos) pos[3 * i + c] = b->node[i].pos[c];
            if (vel) vel[3 * i + c] = b->node[i].vel[c];
            if (force) force[3 * i + c] = b->force[i][c];
        }
}

void ref_blob_get_rhs(void *h, double *out)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    std::memcpy(out, b->rhs_copy, sizeof(double) * 3 * b->num_nodes);
}

void ref_blob_get_element_forces(void *h, double *out)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    for (int e = 0; e < b->num_elements; e++)
        for (int a = 0; a < 4; a++)
            for (int c = 0; c < 3; c++) out[12 * e + 3 * a + c] = b->elem[e].node_force[a][c];
}

int ref_blob_last_inversions(void *h) { return static_cast<RefBlob *>(h)->last_inversions; }

void ref_blob_destroy(void *h)
{
    RefBlob *b = static_cast<RefBlob *>(h);
    if (!b) return;
    delete b->solver;
    delete[] b->elem;
    delete[] b->node;
    delete[] b->force;
    delete[] b->pinned;
    delete[] b->rng;
    delete[] b->rhs_copy;
    delete b;
}

// The package's own known-answer test value (tests/consistency/rngstream/testRngStream.cpp:48-133)
// is produced by the test binary oracle/_ref/test_rngstream; this draws from a stream for
// cross-checks of the oracle's MRG32k3a.
void ref_rng_draws(const uint64_t *state, int64_t n, double *out)
{
    unsigned long s[6];
    for (int i = 0; i < 6; i++) s[i] = state[i];
    RngStream g;
    g.SetSeed(s);
    for (int64_t i = 0; i < n; i++) out[i] = g.RandU01();
}

void ref_rng_advance(const uint64_t *state, long e, long c, uint64_t *out)
{
    unsigned long s[6];
    for (int i = 0; i < 6; i++) s[i] = state[i];
    RngStream g;
    g.SetSeed(s);
    g.AdvanceState(e, c);
    g.GetState(s);
    for (int i = 0; i < 6; i++) out[i] = s[i];
}

}  // extern "C"

// FFEA's own reading of a script's <param> block: FFEA_input_reader::
// file_to_lines, SimulationParams::extract_params (src/SimulationParams.cpp:
// 184-550) and validate (:580-720, which fills in the default output names).
// out: dt, kT, epsilon2, stokes_visc, num_steps, check, rng_seed,
// max_iterations_cg, calc_noise, calc_stokes, restart, num_blobs.
// Returns 0, or -1 where FFEA's reading fails.
#include "FFEA_input_reader.h"
extern "C" int ref_script_params(const char *path, double *out)
{
    FFEA_input_reader reader;
    std::vector<std::string> lines;
    if (reader.file_to_lines(path, &lines) != FFEA_OK) return -1;
    SimulationParams p;
    p.FFEA_script_filename = path;
    if (p.extract_params(lines) != FFEA_OK) return -1;
    const double v[12] = {p.dt, p.kT, p.epsilon2, p.stokes_visc, (double)p.num_steps, (double)p.check,
                          (double)p.rng_seed, (double)p.max_iterations_cg, (double)p.calc_noise,
                          (double)p.calc_stokes, (double)p.restart, (double)p.num_blobs};
    for (int i = 0; i < 12; i++) out[i] = v[i];
    return 0;
}

// FFEA's own overlap of two tetrahedra (volumeIntersectionII,
// src/VolumeIntersection.cpp:951-1190) and its steric pair evaluation through
// Face (Face::checkTetraIntersection and getTetraIntersectionVolumeTotal-
// GradientAndShapeFunctions, src/Face.cpp:399-403, 473-514), for pinning the
// steric restatement.  A and B: 4 x 3 corner positions each.
#include "Face.h"
#include "VolumeIntersection.h"
extern "C" double ref_overlap_volume(const double *A, const double *B, int calc_cm, double *cm)
{
    arr3 a[4], b[4], c = {0, 0, 0};
    for (int i = 0; i < 4; i++)
        for (int d = 0; d < 3; d++) {
            a[i][d] = A[3 * i + d];
            b[i][d] = B[3 * i + d];
        }
    const double v = volumeIntersectionII<scalar, arr3>(a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], calc_cm != 0, c);
    if (cm)
        for (int d = 0; d < 3; d++) cm[d] = c[d];
    return v;
}

// out: [0] overlap test, [1] returned flag, [2] volume, [3..5] dV/dr,
// [6..9] phi1, [10..13] phi2 (dr the finite-difference step)
extern "C" void ref_steric_pair(const double *A, const double *B, double dr, double *out)
{
    static mesh_node na[4], nb[4];
    Face f1, f2;
    for (int i = 0; i < 4; i++) {
        na[i].pos.assign(A[3 * i], A[3 * i + 1], A[3 * i + 2]);
        nb[i].pos.assign(B[3 * i], B[3 * i + 1], B[3 * i + 2]);
        f1.n[i] = &na[i];
        f2.n[i] = &nb[i];
    }
    grr3 g = {0, 0, 0};
    grr4 p1 = {0, 0, 0, 0}, p2 = {0, 0, 0, 0};
    geoscalar vol = 0;
    out[0] = f1.checkTetraIntersection(&f2) ? 1.0 : 0.0;
    out[1] = f1.getTetraIntersectionVolumeTotalGradientAndShapeFunctions(&f2, dr, g, vol, p1, p2) ? 1.0 : 0.0;
    out[2] = vol;
    for (int d = 0; d < 3; d++) out[3 + d] = g[d];
    for (int i = 0; i < 4; i++) {
        out[6 + i] = p1[i];
        out[10 + i] = p2[i];
    }
    for (int i = 0; i < 4; i++) {
        f1.n[i] = nullptr;
        f2.n[i] = nullptr;
    }
}
