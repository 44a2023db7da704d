/* steric_oracle.c -- CPU restatement of FFEA's steric, LJ-steric and
 * soft-potential ("gensoft") surface interactions, for tests only.
 *
 * This is test infrastructure: the tests compare the GPU kernels in
 * ffea_gb300/csrc/ssint.cu against it.  Nothing in the product links it.
 *
 * The three interaction types share VdW_solver::solve's pass over the
 * nearest-neighbour grid (src/VdW_solver.cpp:168-210, restated in
 * ssint_oracle.c) and consider_interaction's checks for the types other than
 * Lennard-Jones (:338-394): faces facing each other, faces in front of each
 * other, and, within one blob, no shared node.  Each face carries the
 * tetrahedron of its element (Face::n[0..3]: the three corners and the
 * element's fourth node).  Per pair:
 *   steric  (Steric_solver::do_interaction, src/Steric_solver.cpp:29-42;
 *            VdW_solver::do_steric_interaction, src/VdW_solver.cpp:458-486):
 *            the overlap volume V of the two tetrahedra and the centre of
 *            mass of the overlap (Face::getTetraIntersectionVolumeTotal-
 *            GradientAndShapeFunctions, src/Face.cpp:473-514), the gradient
 *            dV/dr by forward differences of size steric_dr moving each
 *            tetrahedron against the other along x, y, z, and the barycentric
 *            coordinates phi of the centre of mass in each tetrahedron
 *            (getLocalCoordinatesForLinTet, src/mat_vec_fns_II.cpp:725-734);
 *            node j of face 1 gets phi1[j] k dV/dr, of face 2 -phi2[j] k dV/dr,
 *            the blob-pair energy k V (k = steric_factor);
 *   ljsteric (LJSteric_solver::do_interaction, src/LJSteric_solver.cpp:29-45):
 *            steric where the tetrahedra overlap, else Lennard-Jones;
 *   gensoft (GenSoftSSINT_solver::do_interaction, src/GenSoftSSINT_solver.cpp:
 *            29-45): steric where they overlap, else the polynomial soft
 *            attraction of VdW_solver::do_gensoft_interaction (:488-563) with
 *            calc_gensoft_force_pair_matrix / calc_gensoft_factors
 *            (:701-734, :754-771).
 *
 * The overlap volume and centre of mass are computed by clipping one
 * tetrahedron with the four half-spaces of the other (each face polygon
 * clipped in turn, the cut closed by a cap polygon) and summing the
 * tetrahedra of a fan from an interior point: the same geometric quantities
 * FFEA's volumeIntersectionII (src/VolumeIntersection.cpp) returns, computed
 * by a different construction.  The tests pin this restatement against the
 * reference's own compiled volumeIntersectionII and Face code.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* The overlap of two tetrahedra is an intersection of 8 half-spaces: at most
 * 8 faces, each a polygon bounded by the 7 others. */
#define ST_MAXV 8  /* vertices of one face polygon */
#define ST_MAXF 8  /* faces of the clipped polyhedron */
#define ST_MAXC 16 /* distinct points of one cut */
#define ST_MAXU 32 /* distinct vertices of the overlap */

typedef struct {
    int n;
    double v[ST_MAXV][3];
} st_poly;

typedef struct {
    int nf;
    st_poly f[ST_MAXF];
} st_polyh;

static double st_dot(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void st_cross(const double a[3], const double b[3], double c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static void st_sub(const double a[3], const double b[3], double c[3])
{
    c[0] = a[0] - b[0];
    c[1] = a[1] - b[1];
    c[2] = a[2] - b[2];
}

/* signed volume of (a, b, c, d): det[b - a, c - a, d - a] / 6 */
static double st_tet_volume(const double a[3], const double b[3], const double c[3], const double d[3])
{
    double u[3], v[3], w[3], x[3];
    st_sub(b, a, u);
    st_sub(c, a, v);
    st_sub(d, a, w);
    st_cross(v, w, x);
    return st_dot(u, x) / 6.0;
}

/* the four faces of tetrahedron T as triangles */
static void st_tet_faces(const double T[4][3], st_polyh *P)
{
    static const int tri[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    P->nf = 4;
    for (int f = 0; f < 4; f++) {
        P->f[f].n = 3;
        for (int k = 0; k < 3; k++) memcpy(P->f[f].v[k], T[tri[f][k]], sizeof(double) * 3);
    }
}

/* The half-space of face f of T (opposite vertex f) that holds T:
 * n . x <= off. */
static void st_halfspace(const double T[4][3], int f, double n[3], double *off)
{
    static const int tri[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
    double u[3], v[3];
    st_sub(T[tri[f][1]], T[tri[f][0]], u);
    st_sub(T[tri[f][2]], T[tri[f][0]], v);
    st_cross(u, v, n);
    *off = st_dot(n, T[tri[f][0]]);
    if (st_dot(n, T[f]) > *off) {
        n[0] = -n[0];
        n[1] = -n[1];
        n[2] = -n[2];
        *off = -*off;
    }
}

/* Clip polyhedron P by n . x <= off; returns 0 when nothing is left.  A
 * plane with no vertex strictly outside leaves P as it is; one with no
 * vertex strictly inside leaves nothing (a convex polyhedron with a face on
 * the plane lies on one side of it, so a cutting plane never holds a face). */
/* adds x to pts (n of them, at most cap) unless a point within tol2 (squared
 * distance) is there already */
static void st_add_unique(double (*pts)[3], int *n, int cap, const double x[3], double tol2)
{
    for (int u = 0; u < *n; u++) {
        double e[3];
        st_sub(x, pts[u], e);
        if (st_dot(e, e) <= tol2) return;
    }
    if (*n < cap) memcpy(pts[(*n)++], x, sizeof(double) * 3);
}

static int st_clip(st_polyh *P, const double n[3], double off, double tol2)
{
    double smin = 0.0, smax = 0.0;
    int first = 1;
    for (int f = 0; f < P->nf; f++)
        for (int k = 0; k < P->f[f].n; k++) {
            const double s = st_dot(n, P->f[f].v[k]) - off;
            if (first || s < smin) smin = s;
            if (first || s > smax) smax = s;
            first = 0;
        }
    if (first || smin >= 0) {
        P->nf = 0;
        return 0;
    }
    if (smax <= 0) return 1;
    double cap[ST_MAXC][3];
    int nc = 0, nf = 0;
    for (int f = 0; f < P->nf; f++) {
        const st_poly *in = &P->f[f];
        st_poly out;
        out.n = 0;
        for (int k = 0; k < in->n; k++) {
            const double *a = in->v[k], *b = in->v[(k + 1) % in->n];
            const double sa = st_dot(n, a) - off, sb = st_dot(n, b) - off;
            if (sa <= 0) {
                if (out.n < ST_MAXV) memcpy(out.v[out.n++], a, sizeof(double) * 3);
                if (sa == 0) st_add_unique(cap, &nc, ST_MAXC, a, tol2);
            }
            if ((sa < 0 && sb > 0) || (sa > 0 && sb < 0)) {
                const double t = sa / (sa - sb);
                double x[3];
                for (int c = 0; c < 3; c++) x[c] = a[c] + t * (b[c] - a[c]);
                if (out.n < ST_MAXV) memcpy(out.v[out.n++], x, sizeof(double) * 3);
                st_add_unique(cap, &nc, ST_MAXC, x, tol2);
            }
        }
        if (out.n >= 3) P->f[nf++] = out;
    }
    P->nf = nf;
    if (nf == 0) return 0;
    if (nc >= 3 && nf < ST_MAXF) {
        /* the cap: the cut points ordered by angle around their mean */
        double c[3] = {0, 0, 0}, u[3], w[3];
        for (int k = 0; k < nc; k++)
            for (int d = 0; d < 3; d++) c[d] += cap[k][d];
        for (int d = 0; d < 3; d++) c[d] /= nc;
        int far = 0;
        double best = -1;
        for (int k = 0; k < nc; k++) {
            double e[3];
            st_sub(cap[k], c, e);
            const double l = st_dot(e, e);
            if (l > best) {
                best = l;
                far = k;
            }
        }
        if (best > 0) {
            st_sub(cap[far], c, u);
            st_cross(n, u, w);
            double ang[ST_MAXC];
            for (int k = 0; k < nc; k++) {
                double e[3];
                st_sub(cap[k], c, e);
                ang[k] = atan2(st_dot(e, w), st_dot(e, u));
            }
            for (int i = 1; i < nc; i++) { /* insertion sort by angle */
                double a = ang[i], v[3];
                memcpy(v, cap[i], sizeof(v));
                int j = i - 1;
                while (j >= 0 && ang[j] > a) {
                    ang[j + 1] = ang[j];
                    memcpy(cap[j + 1], cap[j], sizeof(v));
                    j--;
                }
                ang[j + 1] = a;
                memcpy(cap[j + 1], v, sizeof(v));
            }
            st_poly *cp = &P->f[P->nf++];
            cp->n = 0;
            for (int k = 0; k < nc && cp->n < ST_MAXV; k++) memcpy(cp->v[cp->n++], cap[k], sizeof(double) * 3);
        }
    }
    return 1;
}

/* Overlap volume of tetrahedra A and B and, with cm != NULL, the point
 * volumeIntersectionII returns as its centre (findCM,
 * src/VolumeIntersection.cpp:95-104): the mean of the overlap polyhedron's
 * distinct vertices (A's corners inside B, B's inside A, and the points where
 * an edge of one crosses a face of the other).  The clipping reaches a vertex
 * through several faces with rounding-level differences; points closer than
 * 1e-9 of the tetrahedra's extent are one vertex. */
double steric_overlap(const double A[4][3], const double B[4][3], double *cm)
{
    double ext = 0.0;
    for (int i = 0; i < 4; i++)
        for (int d = 0; d < 3; d++) {
            ext = fmax(ext, fabs(A[i][d] - A[0][d]));
            ext = fmax(ext, fabs(B[i][d] - A[0][d]));
        }
    const double tol2 = (1e-9 * ext) * (1e-9 * ext);
    st_polyh P;
    st_tet_faces(A, &P);
    for (int f = 0; f < 4; f++) {
        double n[3], off;
        st_halfspace(B, f, n, &off);
        if (!st_clip(&P, n, off, tol2)) {
            if (cm) cm[0] = cm[1] = cm[2] = 0.0;
            return 0.0;
        }
    }
    double o[3] = {0, 0, 0};
    int nv = 0;
    for (int f = 0; f < P.nf; f++)
        for (int k = 0; k < P.f[f].n; k++) {
            for (int d = 0; d < 3; d++) o[d] += P.f[f].v[k][d];
            nv++;
        }
    for (int d = 0; d < 3; d++) o[d] /= nv;
    double vol = 0.0, m[3] = {0, 0, 0};
    for (int f = 0; f < P.nf; f++) {
        const st_poly *p = &P.f[f];
        for (int k = 1; k + 1 < p->n; k++) {
            const double v = fabs(st_tet_volume(o, p->v[0], p->v[k], p->v[k + 1]));
            vol += v;
            for (int d = 0; d < 3; d++) m[d] += v * 0.25 * (o[d] + p->v[0][d] + p->v[k][d] + p->v[k + 1][d]);
        }
    }
    if (cm) {
        double uniq[ST_MAXU][3];
        int nu = 0;
        for (int f = 0; f < P.nf; f++)
            for (int k = 0; k < P.f[f].n; k++) st_add_unique(uniq, &nu, ST_MAXU, P.f[f].v[k], tol2);
        cm[0] = cm[1] = cm[2] = 0.0;
        for (int u = 0; u < nu; u++)
            for (int d = 0; d < 3; d++) cm[d] += uniq[u][d];
        for (int d = 0; d < 3; d++) cm[d] *= 1.0 / nu;
        (void)m;
    }
    return vol;
}

/* getLocalCoordinatesForLinTet (src/mat_vec_fns_II.cpp:725-734) */
static void st_local_coordinates(const double T[4][3], const double p[3], double phi[4])
{
    phi[0] = st_tet_volume(p, T[1], T[2], T[3]);
    phi[1] = -st_tet_volume(p, T[0], T[2], T[3]);
    phi[2] = st_tet_volume(p, T[0], T[1], T[3]);
    phi[3] = -st_tet_volume(p, T[0], T[1], T[2]);
    const double v = st_tet_volume(T[0], T[1], T[2], T[3]);
    for (int i = 0; i < 4; i++) phi[i] /= v;
}

/* One steric pair (Face::getTetraIntersectionVolumeTotalGradientAndShape-
 * Functions, src/Face.cpp:473-514, then do_steric_interaction's scaling,
 * src/VdW_solver.cpp:470-483): returns 0 when the tetrahedra do not overlap;
 * else 1 with vol = k V, the forces f1[4][3] on A's nodes and f2[4][3] on
 * B's. */
int steric_pair(const double A[4][3], const double B[4][3], double dr, double k, double *vol, double f1[4][3],
                double f2[4][3])
{
    double cm[3], phi1[4], phi2[4], g[3];
    const double V = steric_overlap(A, B, cm);
    if (V == 0) return 0;
    st_local_coordinates(A, cm, phi1);
    st_local_coordinates(B, cm, phi2);
    for (int dir = 0; dir < 3; dir++) {
        double As[4][3], Bs[4][3];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) {
                As[i][j] = A[i][j] + (j == dir ? dr : 0.0);
                Bs[i][j] = B[i][j] + (j == dir ? dr : 0.0);
            }
        const double vb = steric_overlap(A, Bs, NULL);
        g[dir] = (vb - V) / dr;
        const double va = steric_overlap(B, As, NULL);
        g[dir] -= (va - V) / dr;
    }
    *vol = V * k;
    for (int d = 0; d < 3; d++) g[d] *= k;
    for (int j = 0; j < 4; j++)
        for (int d = 0; d < 3; d++) {
            f1[j][d] = phi1[j] * g[d];
            f2[j][d] = -1.0 * phi2[j] * g[d];
        }
    return 1;
}
