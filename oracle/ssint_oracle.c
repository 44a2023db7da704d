/* ssint_oracle.c -- CPU restatement of FFEA's surface-surface Lennard-Jones
 * interaction ("vdw_type = lennard-jones"), for tests only.
 *
 * This is test infrastructure: the tests and the bench's CPU leg compare the
 * GPU kernels in ffea_gb300/csrc/ssint.cu against it.  Nothing in the
 * product links it.
 *
 * It follows one single-threaded pass of VdW_solver::solve
 * (src/VdW_solver.cpp:168-210) over the nearest-neighbour grid that
 * NearestNeighbourLinkedListCube::build_nearest_neighbour_lookup builds
 * (src/NearestNeighbourLinkedListCube.cpp:27-76), in FFEA's own order:
 *   - faces of interaction type -1 are not in the pool (Blob::get_face,
 *     src/Blob.cpp:1642-1648; World::init adds the rest in blob / face order,
 *     src/World.cpp:940-958);
 *   - a face's cell is floor(centroid / h) per axis, wrapped once into the box
 *     (LinkedListCube::pbc, src/LinkedListCube.tpp:284-301); a centroid still
 *     outside after the wrap is an error (add_node_to_stack, :217-235);
 *   - each cell is a stack: the face added last is visited first (:228-233);
 *   - face i visits the 27 cells around its own (adjacent_cell_lookup_table,
 *     src/VdW_solver.cpp:31-59) and interacts with face j when i < j in pool
 *     order, the blobs differ unless self-interaction is on, and the unit
 *     normals do not face the same way (consider_interaction, :338-394; the
 *     in-front and shared-node checks apply to the other ssint types only);
 *   - do_lj_interaction (:237-330) integrates the LJ force over both
 *     triangles with the 3-point Gauss rule (:61-71), calc_lj_force_pair_matrix
 *     and calc_lj_factors (:664-699, :736-752);
 *   - face geometry is Face::calc_area_normal_centroid (src/Face.cpp:197-219)
 *     and barycentric_calc_point (:265-269);
 *   - face forces go onto nodes in face order (Blob::aggregate_forces_and_solve,
 *     src/Blob.cpp:3841-3851).
 * Periodic blob corrections (force_pbc, World::calc_blob_corr_matrix,
 * src/World.cpp:4460-4483; blob_corr[b1][b2] = box * floor((c2 - c1 + box/2) /
 * box) per axis, antisymmetric): the in-front test uses c2 - c1 -
 * blob_corr[b1][b2] (:365-369), the LJ and soft potentials take f1's points
 * as sum eta (x - blob_corr[b2][b1]) (Face::barycentric_calc_point_f2,
 * src/Face.cpp:271-277), the steric overlap f2's tetrahedron minus
 * blob_corr[b1][b2] (src/Face.cpp:517-531).  The sticky wall
 * (VdW_solver::solve_sticky_wall / do_sticky_xz_interaction, :216-235,
 * :396-456) runs after the pair pass over the faces of the grid's bottom and
 * top rows of cells.
 * The reference's VdW_solver cannot be compiled here (its header includes
 * Blob.h, which needs Eigen, absent from the image); the restatement is pinned
 * to the reference's own known answer instead: the LJ energy of two parallel
 * unit-cube faces 1 nm apart (tests/physics/cubes_lj/checkE.py, -1.7870e-19 J
 * within 1 %).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* 3-point rule on a triangle, the constants of src/VdW_solver.cpp:61-71 */
static const double kW = 0.333333333333333;
static const double kEta[3][3] = {{0.666666666666667, 0.166666666666667, 0.166666666666667},
                                  {0.166666666666667, 0.666666666666667, 0.166666666666667},
                                  {0.166666666666667, 0.166666666666667, 0.666666666666667}};

typedef struct {
    int face;              /* index into the caller's face list */
    double v[4][3];        /* corner positions, then the element's fourth node (steric types) */
    int node[4];           /* their node indices (node[3] = -1 without the fourth node) */
    double normal[3], area, centroid[3];
    int x, y, z;           /* cell */
} pool_face;

/* interaction types (SimulationParams::ssint_type; Steric_solver,
 * LJSteric_solver, GenSoftSSINT_solver) */
enum { SS_LJ = 0, SS_STERIC = 1, SS_LJSTERIC = 2, SS_GENSOFT = 3 };

/* steric_oracle.c */
int steric_pair(const double A[4][3], const double B[4][3], double dr, double k, double *vol, double f1[4][3],
                double f2[4][3]);

static void lj_factors(double mag_r, double emin, double rmin6, double *force_mag, double *e)
{
    double ri = 1. / mag_r;
    double ri2 = ri * ri;
    double ri4 = ri2 * ri2;
    double ri6 = ri4 * ri2;
    double ri7 = ri6 * ri;
    double f6 = rmin6 * ri6;
    *force_mag = 12 * ri7 * rmin6 * emin * (f6 - 1);
    *e = kW * kW * emin * f6 * (f6 - 2);
}

/* do_lj_interaction for faces a (f1) and b (f2); adds to fa[3][3], fb[3][3]
 * and returns the pair energy (already multiplied by the areas). */
/* f1's Gauss points: barycentric_calc_point (src/Face.cpp:265-269), or with a
 * periodic correction c = blob_corr[b2][b1] barycentric_calc_point_f2
 * (:271-277), sum eta (x - c) */
static void f1_points(const pool_face *a, const double *c, double p[3][3])
{
    for (int k = 0; k < 3; k++)
        for (int d = 0; d < 3; d++) {
            if (c)
                p[k][d] = kEta[k][0] * (a->v[0][d] - c[d]) + kEta[k][1] * (a->v[1][d] - c[d]) +
                          kEta[k][2] * (a->v[2][d] - c[d]);
            else
                p[k][d] = kEta[k][0] * a->v[0][d] + kEta[k][1] * a->v[1][d] + kEta[k][2] * a->v[2][d];
        }
}

static double lj_pair(const pool_face *a, const pool_face *b, const double *corr21, double emin, double rmin,
                      double fa[4][3], double fb[4][3])
{
    double p[3][3], q[3][3], fpm[3][3][3];
    f1_points(a, corr21, p);
    for (int k = 0; k < 3; k++)
        for (int d = 0; d < 3; d++)
            q[k][d] = kEta[k][0] * b->v[0][d] + kEta[k][1] * b->v[1][d] + kEta[k][2] * b->v[2][d];
    double r2 = rmin * rmin;
    double r4 = r2 * r2;
    double r6 = r4 * r2;
    double energy = 0.0, fm, e;
    for (int k = 0; k < 3; k++) {
        double dx = p[k][0] - q[k][0], dy = p[k][1] - q[k][1], dz = p[k][2] - q[k][2];
        double mag_r = sqrt(dx * dx + dy * dy + dz * dz);
        lj_factors(mag_r, emin, r6, &fm, &e);
        energy += e;
        for (int d = 0; d < 3; d++) fpm[k][k][d] = fm * ((p[k][d] - q[k][d]) / mag_r);
        for (int l = k + 1; l < 3; l++) {
            dx = p[k][0] - q[l][0];
            dy = p[k][1] - q[l][1];
            dz = p[k][2] - q[l][2];
            mag_r = sqrt(dx * dx + dy * dy + dz * dz);
            lj_factors(mag_r, emin, r6, &fm, &e);
            energy += 2 * e;
            for (int d = 0; d < 3; d++) {
                fpm[k][l][d] = fm * ((p[k][d] - q[l][d]) / mag_r);
                fpm[l][k][d] = fpm[k][l][d];
            }
        }
    }
    double apaq = a->area * b->area;
    energy *= apaq;
    for (int j = 0; j < 3; j++) {
        double f1[3] = {0, 0, 0}, f2[3] = {0, 0, 0};
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) {
                double c = kW * kW * kEta[l][j];
                double dd = kW * kW * kEta[k][j];
                for (int d = 0; d < 3; d++) {
                    f1[d] += c * fpm[k][l][d];
                    f2[d] -= dd * fpm[l][k][d];
                }
            }
        for (int d = 0; d < 3; d++) {
            fa[j][d] += f1[d] * apaq;
            fb[j][d] += f2[d] * apaq;
        }
    }
    return energy;
}

/* calc_gensoft_factors (src/VdW_solver.cpp:754-771) */
static void gensoft_factors(double mag_r, double emin, double rmin, double k0, double *force_mag, double *e)
{
    const double mag_r_2 = mag_r * mag_r;
    const double rmin_2 = rmin * rmin;
    const double gf2 = mag_r_2 / rmin_2;
    const double gf3 = gf2 * mag_r / rmin;
    const double k0rm = k0 * rmin;
    const double k0rm2 = k0rm * rmin;
    const double epsonrm = emin / rmin;
    *force_mag = 2 * (k0rm - 6 * epsonrm) * gf3 + 3 * (4 * epsonrm - k0rm) * gf2 + k0 * mag_r;
    const double emag = (0.5 * k0rm2 - 3 * emin) * gf2 * gf2 + (4 * emin - k0rm2) * gf3 + 0.5 * k0 * mag_r_2 - emin;
    *e = kW * kW * emag;
}

/* do_gensoft_interaction for faces a (f1) and b (f2) with
 * calc_gensoft_force_pair_matrix (src/VdW_solver.cpp:488-563, 701-734); adds
 * to fa[3][3], fb[3][3] and returns the pair energy. */
static double gensoft_pair(const pool_face *a, const pool_face *b, const double *corr21, double emin, double rmin,
                           double k0, double fa[4][3], double fb[4][3])
{
    double p[3][3], q[3][3], fpm[3][3][3];
    f1_points(a, corr21, p);
    for (int k = 0; k < 3; k++)
        for (int d = 0; d < 3; d++)
            q[k][d] = kEta[k][0] * b->v[0][d] + kEta[k][1] * b->v[1][d] + kEta[k][2] * b->v[2][d];
    double energy = 0.0, fm, e;
    for (int k = 0; k < 3; k++) {
        double dx = p[k][0] - q[k][0], dy = p[k][1] - q[k][1], dz = p[k][2] - q[k][2];
        double mag_r = sqrt(dx * dx + dy * dy + dz * dz);
        gensoft_factors(mag_r, emin, rmin, k0, &fm, &e);
        energy += e;
        for (int d = 0; d < 3; d++) fpm[k][k][d] = fm * ((p[k][d] - q[k][d]) / mag_r);
        for (int l = k + 1; l < 3; l++) {
            dx = p[k][0] - q[l][0];
            dy = p[k][1] - q[l][1];
            dz = p[k][2] - q[l][2];
            mag_r = sqrt(dx * dx + dy * dy + dz * dz);
            gensoft_factors(mag_r, emin, rmin, k0, &fm, &e);
            energy += 2 * e;
            for (int d = 0; d < 3; d++) {
                fpm[k][l][d] = fm * ((p[k][d] - q[l][d]) / mag_r);
                fpm[l][k][d] = fpm[k][l][d];
            }
        }
    }
    const double apaq = a->area * b->area;
    energy *= apaq;
    for (int j = 0; j < 3; j++) {
        double f1[3] = {0, 0, 0}, f2[3] = {0, 0, 0};
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) {
                const double c = kW * kW * kEta[l][j];
                const double dd = kW * kW * kEta[k][j];
                for (int d = 0; d < 3; d++) {
                    f1[d] += c * fpm[k][l][d];
                    f2[d] -= dd * fpm[l][k][d];
                }
            }
        for (int d = 0; d < 3; d++) {
            fa[j][d] += f1[d] * apaq;
            fb[j][d] += f2[d] * apaq;
        }
    }
    return energy;
}

/* Returns 0, or -1 when a face centroid lies outside the box after the
 * single wrap (FFEA reports the same as an error). node_force: num_nodes x 3,
 * overwritten with the surface forces alone; energy: num_blobs x num_blobs,
 * overwritten (VdW_solver::fieldenergy, [blob of f1][blob of f2]).
 * pairs_out (may be NULL): the number of face pairs that interacted. */
/* do_sticky_xz_interaction (src/VdW_solver.cpp:396-456) of one face against
 * the wall y = y_wall: the y force on its corners (the energy is not kept,
 * as in FFEA) */
static void sticky_face(const pool_face *f, int bottom, double y_wall, double emin, double rmin, double ff[4][3])
{
    if ((bottom && f->normal[1] > 0) || (!bottom && f->normal[1] < 0)) return;
    double py[3], fpm[3][3];
    for (int k = 0; k < 3; k++) py[k] = kEta[k][0] * f->v[0][1] + kEta[k][1] * f->v[1][1] + kEta[k][2] * f->v[2][1];
    const double r6 = pow(rmin, 6);
    for (int k = 0; k < 3; k++)
        for (int l = k; l < 3; l++) {
            const double mag_r = py[k] - y_wall;
            double force_mag = 12 * r6 * emin * (pow(mag_r, -7) - r6 * pow(mag_r, -13));
            force_mag *= -1;
            fpm[k][l] = force_mag;
            fpm[l][k] = force_mag;
        }
    const double asq = f->area * f->area;
    for (int j = 0; j < 3; j++) {
        double fy = 0.0;
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) fy += kW * kW * kEta[l][j] * fpm[k][l];
        ff[j][1] += fy * asq;
    }
}

int oracle_ssint(int num_nodes, const double *pos, int num_faces, const int *faces, const int *face_apex,
                 const int *face_blob, const int *face_type, int num_types, const double *emin, const double *rmin,
                 const double *k0, int num_blobs, double h, int nx, int ny, int nz, int inc_self, int ssint_type,
                 double steric_factor, double steric_dr, const double *blob_corr, int sticky_wall, double *node_force,
                 double *energy, long long *pairs_out)
{
    if (sticky_wall && ny < 2) return -2; /* FFEA's row loop (y += Ny - 1) would not end */
    static const int adj[27][3] = {{-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {-1, 0, 1},
                                   {-1, 1, -1},  {-1, 1, 0},  {-1, 1, 1},  {0, -1, -1}, {0, -1, 0}, {0, -1, 1},
                                   {0, 0, -1},   {0, 0, 0},   {0, 0, 1},   {0, 1, -1},  {0, 1, 0},  {0, 1, 1},
                                   {1, -1, -1},  {1, -1, 0},  {1, -1, 1},  {1, 0, -1},  {1, 0, 0},  {1, 0, 1},
                                   {1, 1, -1},   {1, 1, 0},   {1, 1, 1}};
    int np = 0;
    pool_face *pool = (pool_face *)malloc(sizeof(pool_face) * (size_t)(num_faces > 0 ? num_faces : 1));
    double (*fforce)[4][3] = calloc((size_t)(num_faces > 0 ? num_faces : 1), sizeof(double[4][3]));
    long ncell = (long)nx * ny * nz;
    int *root = (int *)malloc(sizeof(int) * (size_t)ncell);
    int *next = (int *)malloc(sizeof(int) * (size_t)(num_faces > 0 ? num_faces : 1));
    int rc = 0;
    for (long c = 0; c < ncell; c++) root[c] = -1;
    memset(energy, 0, sizeof(double) * (size_t)num_blobs * num_blobs);
    memset(node_force, 0, sizeof(double) * 3 * (size_t)num_nodes);
    for (int f = 0; f < num_faces; f++) {
        if (face_type[f] < 0) continue;
        pool_face *P = &pool[np];
        P->face = f;
        for (int i = 0; i < 3; i++) {
            P->node[i] = faces[3 * f + i];
            for (int d = 0; d < 3; d++) P->v[i][d] = pos[3 * faces[3 * f + i] + d];
        }
        P->node[3] = face_apex ? face_apex[f] : -1;
        for (int d = 0; d < 3; d++) P->v[3][d] = face_apex ? pos[3 * face_apex[f] + d] : 0.0;
        double a[3], b[3], n[3];
        for (int d = 0; d < 3; d++) {
            a[d] = P->v[1][d] - P->v[0][d];
            b[d] = P->v[2][d] - P->v[0][d];
        }
        n[0] = a[1] * b[2] - a[2] * b[1];
        n[1] = a[2] * b[0] - a[0] * b[2];
        n[2] = a[0] * b[1] - a[1] * b[0];
        double mag = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        P->area = .5 * mag;
        for (int d = 0; d < 3; d++) P->normal[d] = n[d] / mag;
        double *cen = P->centroid;
        for (int d = 0; d < 3; d++) cen[d] = (1.0 / 3.0) * (P->v[0][d] + P->v[1][d] + P->v[2][d]);
        int cx = (int)floor(cen[0] / h), cy = (int)floor(cen[1] / h), cz = (int)floor(cen[2] / h);
        if (cx < 0) cx += nx; else if (cx >= nx) cx -= nx;
        if (cy < 0) cy += ny; else if (cy >= ny) cy -= ny;
        if (cz < 0) cz += nz; else if (cz >= nz) cz -= nz;
        if (cx < 0 || cx >= nx || cy < 0 || cy >= ny || cz < 0 || cz >= nz) {
            rc = -1;
            goto done;
        }
        P->x = cx;
        P->y = cy;
        P->z = cz;
        long cell = ((long)cx * ny + cy) * nz + cz;
        next[np] = root[cell];
        root[cell] = np;
        np++;
    }
    long long pairs = 0;
    for (int i = 0; i < np; i++) {
        const pool_face *A = &pool[i];
        for (int c = 0; c < 27; c++) {
            int x = A->x + adj[c][0], y = A->y + adj[c][1], z = A->z + adj[c][2];
            if (x < 0) x += nx; else if (x >= nx) x -= nx;
            if (y < 0) y += ny; else if (y >= ny) y -= ny;
            if (z < 0) z += nz; else if (z >= nz) z -= nz;
            for (int j = root[((long)x * ny + y) * nz + z]; j >= 0; j = next[j]) {
                if (!(i < j)) continue;
                const pool_face *B = &pool[j];
                int ba = face_blob[A->face], bb = face_blob[B->face];
                if (!inc_self && ba == bb) continue;
                if (A->normal[0] * B->normal[0] + A->normal[1] * B->normal[1] + A->normal[2] * B->normal[2] > 0.0)
                    continue;
                /* periodic corrections of the pair: [b1][b2] and [b2][b1] */
                const double *c12 = blob_corr ? blob_corr + 3 * ((long)ba * num_blobs + bb) : NULL;
                const double *c21 = blob_corr ? blob_corr + 3 * ((long)bb * num_blobs + ba) : NULL;
                if (ssint_type != SS_LJ) {
                    /* faces in front of each other; no shared node within a blob */
                    double sep[3];
                    for (int d = 0; d < 3; d++)
                        sep[d] = c12 ? B->centroid[d] - A->centroid[d] - c12[d] : B->centroid[d] - A->centroid[d];
                    if (sep[0] * A->normal[0] + sep[1] * A->normal[1] + sep[2] * A->normal[2] < 0 &&
                        sep[0] * B->normal[0] + sep[1] * B->normal[1] + sep[2] * B->normal[2] > 0)
                        continue;
                    if (inc_self && ba == bb) {
                        if (A->node[3] == B->node[3]) continue;
                        int shared = 0;
                        for (int u = 0; u < 4; u++)
                            for (int w = 0; w < 4; w++) shared |= A->node[u] == B->node[w];
                        if (shared) continue;
                    }
                }
                int t = face_type[A->face] * num_types + face_type[B->face];
                int done = 0;
                if (ssint_type != SS_LJ) {
                    /* steric where the element tetrahedra overlap */
                    double vol, f1[4][3], f2[4][3], Bv[4][3];
                    for (int u = 0; u < 4; u++)
                        for (int d = 0; d < 3; d++) Bv[u][d] = c12 ? B->v[u][d] - c12[d] : B->v[u][d];
                    if (steric_pair((const double (*)[3])A->v, (const double (*)[3])Bv, steric_dr, steric_factor,
                                    &vol, f1, f2)) {
                        for (int u = 0; u < 4; u++)
                            for (int d = 0; d < 3; d++) {
                                fforce[i][u][d] += f1[u][d];
                                fforce[j][u][d] += f2[u][d];
                            }
                        energy[ba * num_blobs + bb] += vol;
                        done = 1;
                    }
                }
                if (!done && (ssint_type == SS_LJ || ssint_type == SS_LJSTERIC)) {
                    energy[ba * num_blobs + bb] += lj_pair(A, B, c21, emin[t], rmin[t], fforce[i], fforce[j]);
                    done = 1;
                } else if (!done && ssint_type == SS_GENSOFT) {
                    energy[ba * num_blobs + bb] +=
                        gensoft_pair(A, B, c21, emin[t], rmin[t], k0[t], fforce[i], fforce[j]);
                    done = 1;
                }
                pairs += done;
            }
        }
    }
    if (sticky_wall) {
        /* the bottom row of cells, then the top one, each cell's stack in turn */
        for (int y = 0; y < ny; y += ny - 1)
            for (int z = 0; z < nz; z++)
                for (int x = 0; x < nx; x++)
                    for (int f = root[((long)x * ny + y) * nz + z]; f >= 0; f = next[f]) {
                        const int t = face_type[pool[f].face] * num_types + face_type[pool[f].face];
                        sticky_face(&pool[f], y == 0, y == 0 ? 0.0 : h * ny, emin[t], rmin[t], fforce[f]);
                    }
    }
    for (int i = 0; i < np; i++)
        for (int k = 0; k < 4; k++) {
            const int nd = pool[i].node[k];
            if (nd < 0) continue;
            for (int d = 0; d < 3; d++) node_force[3 * nd + d] += fforce[i][k][d];
        }
    if (pairs_out) *pairs_out = pairs;
done:
    free(pool);
    free(fforce);
    free(root);
    free(next);
    return rc;
}

/* The Lennard-Jones pass alone (vdw_type = lennard-jones). */
int oracle_ssint_lj(int num_nodes, const double *pos, int num_faces, const int *faces, const int *face_blob,
                    const int *face_type, int num_types, const double *emin, const double *rmin, int num_blobs,
                    double h, int nx, int ny, int nz, int inc_self, double *node_force, double *energy,
                    long long *pairs_out)
{
    return oracle_ssint(num_nodes, pos, num_faces, faces, NULL, face_blob, face_type, num_types, emin, rmin, NULL,
                        num_blobs, h, nx, ny, nz, inc_self, SS_LJ, 0.0, 0.0, NULL, 0, node_force, energy, pairs_out);
}

/* World::calc_blob_corr_matrix (src/World.cpp:4460-4483): for blob centroids
 * c (3 per blob) and the box, blob_corr[i][j] = box * floor((c_j - c_i +
 * box / 2) / box) per axis for i < j, its negation for j < i, 0 on the
 * diagonal. */
void oracle_blob_corr(int num_blobs, const double *c, const double box[3], double *blob_corr)
{
    for (int i = 0; i < num_blobs; ++i) {
        for (int d = 0; d < 3; d++) blob_corr[3 * ((long)i * num_blobs + i) + d] = 0.0;
        for (int j = i + 1; j < num_blobs; ++j)
            for (int d = 0; d < 3; d++) {
                const double v = box[d] * floor((c[3 * j + d] - c[3 * i + d] + 0.5 * box[d]) / box[d]);
                blob_corr[3 * ((long)i * num_blobs + j) + d] = v;
                blob_corr[3 * ((long)j * num_blobs + i) + d] = -1 * v;
            }
    }
}
