/*
 * ffea_oracle.c -- CPU ORACLE for the FFEA per-timestep blob update.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C and FP64, the
 * reference algorithm of FFEA's Blob::update_internal_forces +
 * Blob::update_positions path so that the CUDA implementation in ffea_gb300/
 * can be checked against it.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.  It is never
 * part of the product path.
 *
 * Every function cites the reference file:line it follows (paths are relative
 * to the FFEA source tree).  Operation order inside each function follows the
 * reference statement by statement so that, compiled with -ffp-contract=off,
 * the FP64 results match the reference objects bit for bit (pinned by
 * tests/test_oracle.py and the committed golden vectors).
 *
 * Units: everything is in FFEA meso units (include/dimensions.h:30-41); the
 * caller converts SI inputs (see ffea_gb300/params.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERROR -1

enum { ORC_SOLVER_NOMASS = 0, ORC_SOLVER_MASS = 1, ORC_SOLVER_LUMPED = 2 };

/* ------------------------------------------------------------------------ */
/* MRG32k3a (L'Ecuyer 1999; L'Ecuyer, Simard, Chen, Kelton 2002).          */
/* Restated from the published algorithm; semantics follow                  */
/* src/RngStream.cpp:266-289 (U01), :293-306 (U01d), :327-345 (stream       */
/* spacing 2^127), :371-377 (substream 2^76), :408-435 (AdvanceState).      */
/* ------------------------------------------------------------------------ */
static const double orc_m1 = 4294967087.0;
static const double orc_m2 = 4294944443.0;
static const double orc_a12 = 1403580.0;
static const double orc_a13n = 810728.0;
static const double orc_a21 = 527612.0;
static const double orc_a23n = 1370589.0;
static const uint64_t orc_m1u = 4294967087ULL;
static const uint64_t orc_m2u = 4294944443ULL;

/* One draw; exact-integer double arithmetic (src/RngStream.cpp:266-289). */
static double orc_u01(double *Cg)
{
    long k;
    double p1, p2, u;
    const double norm = 1.0 / (orc_m1 + 1.0);
    p1 = orc_a12 * Cg[1] - orc_a13n * Cg[0];
    k = (long)(p1 / orc_m1);
    p1 -= k * orc_m1;
    if (p1 < 0.0) p1 += orc_m1;
    Cg[0] = Cg[1]; Cg[1] = Cg[2]; Cg[2] = p1;
    p2 = orc_a21 * Cg[5] - orc_a23n * Cg[3];
    k = (long)(p2 / orc_m2);
    p2 -= k * orc_m2;
    if (p2 < 0.0) p2 += orc_m2;
    Cg[3] = Cg[4]; Cg[4] = Cg[5]; Cg[5] = p2;
    u = ((p1 > p2) ? (p1 - p2) * norm : (p1 - p2 + orc_m1) * norm);
    return u;
}

/* 3x3 matrices mod m in exact uint64 arithmetic (each product < 2^64). */
typedef struct { uint64_t a[3][3]; } orc_mat;

static void orc_matmul(const orc_mat *A, const orc_mat *B, orc_mat *C, uint64_t m)
{
    orc_mat t;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            uint64_t s = 0;
            for (int k = 0; k < 3; k++) s = (s + (A->a[i][k] * B->a[k][j]) % m) % m;
            t.a[i][j] = s;
        }
    *C = t;
}

static void orc_matvec(const orc_mat *A, const uint64_t *v, uint64_t *out, uint64_t m)
{
    uint64_t t[3];
    for (int i = 0; i < 3; i++) {
        uint64_t s = 0;
        for (int k = 0; k < 3; k++) s = (s + (A->a[i][k] * v[k]) % m) % m;
        t[i] = s;
    }
    out[0] = t[0]; out[1] = t[1]; out[2] = t[2];
}

static void orc_identity(orc_mat *A)
{
    memset(A, 0, sizeof(*A));
    A->a[0][0] = A->a[1][1] = A->a[2][2] = 1;
}

/* One-step transition matrices of the two components (the recurrences of
 * src/RngStream.cpp:271-283 written as matrices). */
static void orc_step_matrices(orc_mat *A1, orc_mat *A2)
{
    memset(A1, 0, sizeof(*A1));
    memset(A2, 0, sizeof(*A2));
    A1->a[0][1] = 1; A1->a[1][2] = 1;
    A1->a[2][0] = orc_m1u - 810728ULL; A1->a[2][1] = 1403580ULL;
    A2->a[0][1] = 1; A2->a[1][2] = 1;
    A2->a[2][0] = orc_m2u - 1370589ULL; A2->a[2][2] = 527612ULL;
}

static void orc_matpow(const orc_mat *A, uint64_t n, orc_mat *out, uint64_t m)
{
    orc_mat r, b = *A;
    orc_identity(&r);
    while (n) {
        if (n & 1) orc_matmul(&r, &b, &r, m);
        orc_matmul(&b, &b, &b, m);
        n >>= 1;
    }
    *out = r;
}

/* A^(2^e) by e squarings. */
static void orc_mat2pow(const orc_mat *A, int e, orc_mat *out, uint64_t m)
{
    orc_mat b = *A;
    for (int i = 0; i < e; i++) orc_matmul(&b, &b, &b, m);
    *out = b;
}

static uint64_t orc_powmod(uint64_t b, uint64_t e, uint64_t m)
{
    uint64_t r = 1;
    b %= m;
    while (e) {
        if (e & 1) r = (r * b) % m;
        b = (b * b) % m;
        e >>= 1;
    }
    return r;
}

/* Inverse of a 3x3 matrix mod a prime m (adjugate / determinant). */
static void orc_matinv(const orc_mat *A, orc_mat *out, uint64_t m)
{
#define MM(x, y) (((x) * (y)) % m)
#define SUBM(x, y) (((x) + m - (y)) % m)
    const uint64_t (*a)[3] = A->a;
    orc_mat adj;
    adj.a[0][0] = SUBM(MM(a[1][1], a[2][2]), MM(a[1][2], a[2][1]));
    adj.a[0][1] = SUBM(MM(a[0][2], a[2][1]), MM(a[0][1], a[2][2]));
    adj.a[0][2] = SUBM(MM(a[0][1], a[1][2]), MM(a[0][2], a[1][1]));
    adj.a[1][0] = SUBM(MM(a[1][2], a[2][0]), MM(a[1][0], a[2][2]));
    adj.a[1][1] = SUBM(MM(a[0][0], a[2][2]), MM(a[0][2], a[2][0]));
    adj.a[1][2] = SUBM(MM(a[0][2], a[1][0]), MM(a[0][0], a[1][2]));
    adj.a[2][0] = SUBM(MM(a[1][0], a[2][1]), MM(a[1][1], a[2][0]));
    adj.a[2][1] = SUBM(MM(a[0][1], a[2][0]), MM(a[0][0], a[2][1]));
    adj.a[2][2] = SUBM(MM(a[0][0], a[1][1]), MM(a[0][1], a[1][0]));
    uint64_t det = (MM(a[0][0], adj.a[0][0]) + MM(a[0][1], adj.a[1][0]) + MM(a[0][2], adj.a[2][0])) % m;
    uint64_t inv = orc_powmod(det, m - 2, m);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) out->a[i][j] = MM(adj.a[i][j], inv);
#undef MM
#undef SUBM
}

/* Apply A^n (per component) to a 6-word state held as exact doubles. */
static void orc_apply(const orc_mat *B1, const orc_mat *B2, double *Cg)
{
    uint64_t v1[3] = {(uint64_t)Cg[0], (uint64_t)Cg[1], (uint64_t)Cg[2]};
    uint64_t v2[3] = {(uint64_t)Cg[3], (uint64_t)Cg[4], (uint64_t)Cg[5]};
    orc_matvec(B1, v1, v1, orc_m1u);
    orc_matvec(B2, v2, v2, orc_m2u);
    for (int i = 0; i < 3; i++) { Cg[i] = (double)v1[i]; Cg[3 + i] = (double)v2[i]; }
}

/* Jump a state forward by n draws (n >= 0). */
void orc_rng_advance(double *Cg, uint64_t n)
{
    orc_mat A1, A2, B1, B2;
    orc_step_matrices(&A1, &A2);
    orc_matpow(&A1, n, &B1, orc_m1u);
    orc_matpow(&A2, n, &B2, orc_m2u);
    orc_apply(&B1, &B2, Cg);
}

/* Draw n uniforms from a 6-word uint64 state (updates the state). */
void orc_rng_draws(uint64_t *state, int64_t n, double *out)
{
    double Cg[6];
    for (int i = 0; i < 6; i++) Cg[i] = (double)state[i];
    for (int64_t i = 0; i < n; i++) out[i] = orc_u01(Cg);
    for (int i = 0; i < 6; i++) state[i] = (uint64_t)Cg[i];
}

/* Sequential sum and FNV-style hash (h = (h ^ bits) * 0x100000001b3 from
 * 0xcbf29ce484222325) of n draws: a fingerprint of a whole stream. */
void orc_rng_fingerprint(const uint64_t *state, int64_t n, double *sum, uint64_t *hash)
{
    double Cg[6], s = 0.0;
    uint64_t h = 0xcbf29ce484222325ULL;
    for (int i = 0; i < 6; i++) Cg[i] = (double)state[i];
    for (int64_t i = 0; i < n; i++) {
        double u = orc_u01(Cg);
        uint64_t bits;
        memcpy(&bits, &u, sizeof(bits));
        h = (h ^ bits) * 0x100000001b3ULL;
        s += u;
    }
    *sum = s;
    *hash = h;
}

void orc_rng_jump(uint64_t *state, uint64_t n)
{
    double Cg[6];
    for (int i = 0; i < 6; i++) Cg[i] = (double)state[i];
    orc_rng_advance(Cg, n);
    for (int i = 0; i < 6; i++) state[i] = (uint64_t)Cg[i];
}

/* --- a minimal RngStream object, enough for the package's own KAT ------- */
/* (tests/consistency/rngstream/testRngStream.cpp).                          */
typedef struct { double Cg[6], Bg[6], Ig[6]; int anti, incPrec; } orc_stream;
static double orc_next_seed[6] = {12345.0, 12345.0, 12345.0, 12345.0, 12345.0, 12345.0};

static void orc_stream_init(orc_stream *s)
{
    /* src/RngStream.cpp:327-345: take the package seed, then advance it by 2^127. */
    orc_mat A1, A2, B1, B2;
    s->anti = 0; s->incPrec = 0;
    for (int i = 0; i < 6; i++) s->Bg[i] = s->Cg[i] = s->Ig[i] = orc_next_seed[i];
    orc_step_matrices(&A1, &A2);
    orc_mat2pow(&A1, 127, &B1, orc_m1u);
    orc_mat2pow(&A2, 127, &B2, orc_m2u);
    orc_apply(&B1, &B2, orc_next_seed);
}

static double orc_stream_u01(orc_stream *s)
{
    double u = orc_u01(s->Cg);
    return s->anti ? (1 - u) : u;
}

static double orc_stream_rand(orc_stream *s)
{
    /* src/RngStream.cpp:293-306 (U01d) and :509-515 (RandU01). */
    const double fact = 5.9604644775390625e-8;
    if (!s->incPrec) return orc_stream_u01(s);
    double u = orc_stream_u01(s);
    if (s->anti) {
        u += (orc_stream_u01(s) - 1.0) * fact;
        return (u < 0.0) ? u + 1.0 : u;
    }
    u += orc_stream_u01(s) * fact;
    return (u < 1.0) ? u : (u - 1.0);
}

static void orc_stream_advance(orc_stream *s, long e, long c)
{
    /* src/RngStream.cpp:408-435: n = +-2^|e| + c. */
    orc_mat A1, A2, B1, B2, C1, C2;
    orc_step_matrices(&A1, &A2);
    orc_identity(&B1); orc_identity(&B2);
    if (e > 0) { orc_mat2pow(&A1, (int)e, &B1, orc_m1u); orc_mat2pow(&A2, (int)e, &B2, orc_m2u); }
    else if (e < 0) {
        orc_mat I1, I2;
        orc_matinv(&A1, &I1, orc_m1u); orc_matinv(&A2, &I2, orc_m2u);
        orc_mat2pow(&I1, (int)-e, &B1, orc_m1u); orc_mat2pow(&I2, (int)-e, &B2, orc_m2u);
    }
    if (c >= 0) { orc_matpow(&A1, (uint64_t)c, &C1, orc_m1u); orc_matpow(&A2, (uint64_t)c, &C2, orc_m2u); }
    else {
        orc_mat I1, I2;
        orc_matinv(&A1, &I1, orc_m1u); orc_matinv(&A2, &I2, orc_m2u);
        orc_matpow(&I1, (uint64_t)-c, &C1, orc_m1u); orc_matpow(&I2, (uint64_t)-c, &C2, orc_m2u);
    }
    if (e) { orc_matmul(&B1, &C1, &C1, orc_m1u); orc_matmul(&B2, &C2, &C2, orc_m2u); }
    orc_apply(&C1, &C2, s->Cg);
}

static void orc_stream_next_substream(orc_stream *s)
{
    /* src/RngStream.cpp:371-377: Bg <- A^(2^76) Bg; Cg <- Bg. */
    orc_mat A1, A2, B1, B2;
    orc_step_matrices(&A1, &A2);
    orc_mat2pow(&A1, 76, &B1, orc_m1u);
    orc_mat2pow(&A2, 76, &B2, orc_m2u);
    orc_apply(&B1, &B2, s->Bg);
    for (int i = 0; i < 6; i++) s->Cg[i] = s->Bg[i];
}

static void orc_stream_reset_start(orc_stream *s) { for (int i = 0; i < 6; i++) s->Cg[i] = s->Bg[i] = s->Ig[i]; }
static void orc_stream_reset_substream(orc_stream *s) { for (int i = 0; i < 6; i++) s->Cg[i] = s->Bg[i]; }
static int orc_stream_randint(orc_stream *s, int lo, int hi) { return lo + (int)((hi - lo + 1.0) * orc_stream_rand(s)); }

/* The package's known-answer computation (testRngStream.cpp:48-133); the
 * reference prints it at precision 14 and expects "39.697547445251". */
double orc_rng_package_kat(void)
{
    double sum, sum3;
    int i;
    for (i = 0; i < 6; i++) orc_next_seed[i] = 12345.0;
    orc_stream g1, g2, g3;
    orc_stream_init(&g1); orc_stream_init(&g2); orc_stream_init(&g3);
    sum = orc_stream_rand(&g2) + orc_stream_rand(&g3);
    orc_stream_advance(&g1, 5, 3);
    sum += orc_stream_rand(&g1);
    orc_stream_reset_start(&g1);
    for (i = 0; i < 35; i++) orc_stream_advance(&g1, 0, 1);
    sum += orc_stream_rand(&g1);
    orc_stream_reset_start(&g1);
    long sumi = 0;
    for (i = 0; i < 35; i++) sumi += orc_stream_randint(&g1, 1, 10);
    sum += sumi / 100.0;
    sum3 = 0.0;
    for (i = 0; i < 100; i++) sum3 += orc_stream_rand(&g3);
    sum += sum3 / 10.0;
    orc_stream_reset_start(&g3);
    for (i = 1; i <= 5; i++) sum += orc_stream_rand(&g3);
    for (i = 0; i < 4; i++) orc_stream_next_substream(&g3);
    for (i = 0; i < 5; i++) sum += orc_stream_rand(&g3);
    orc_stream_reset_substream(&g3);
    for (i = 0; i < 5; i++) sum += orc_stream_rand(&g3);
    orc_stream_next_substream(&g2);
    sum3 = 0.0;
    for (i = 1; i <= 100000; i++) sum3 += orc_stream_rand(&g2);
    sum += sum3 / 10000.0;
    g3.anti = 1;
    sum3 = 0.0;
    for (i = 1; i <= 100000; i++) sum3 += orc_stream_rand(&g3);
    sum += sum3 / 10000.0;
    for (i = 0; i < 6; i++) orc_next_seed[i] = 1.0;
    orc_stream gar[4];
    for (i = 0; i < 4; i++) orc_stream_init(&gar[i]);
    for (i = 0; i < 4; i++) sum += orc_stream_rand(&gar[i]);
    orc_stream_advance(&gar[2], -127, 0);
    sum += orc_stream_rand(&gar[2]);
    orc_stream_next_substream(&gar[2]);
    gar[2].incPrec = 1;
    sum3 = 0.0;
    for (i = 0; i < 100000; i++) sum3 += orc_stream_rand(&gar[2]);
    sum += sum3 / 10000.0;
    gar[2].anti = 1;
    sum3 = 0.0;
    for (i = 0; i < 100000; i++) sum3 += orc_stream_rand(&gar[2]);
    sum += sum3 / 10000.0;
    gar[2].anti = 0;
    gar[2].incPrec = 0;
    for (i = 0; i < 4; i++) sum += orc_stream_rand(&gar[i]);
    for (i = 0; i < 6; i++) orc_next_seed[i] = 12345.0;
    return sum;
}

/* glibc rand() (TYPE_3 additive feedback generator, degree 31, separation
 * 3), restated from its published description so that seeding does not
 * depend on the host libc's global state.  FFEA calls libc srand/rand in
 * src/World.cpp:301-305. */
typedef struct { int32_t r[34 + 310 + 8]; int32_t ring[31]; int f, b; } orc_glibc_rand;

static void orc_glibc_srand(orc_glibc_rand *g, unsigned int seed)
{
    int32_t r[34];
    if (seed == 0) seed = 1;
    r[0] = (int32_t)seed;
    for (int i = 1; i < 31; i++) {
        /* 16807 * r[i-1] mod (2^31 - 1) via Schrage's method */
        int32_t hi = r[i - 1] / 127773;
        int32_t lo = r[i - 1] % 127773;
        int32_t word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        r[i] = word;
    }
    for (int i = 0; i < 31; i++) g->ring[i] = r[i];
    g->f = 3; g->b = 0;
    /* discard the first 310 outputs */
    for (int i = 0; i < 310; i++) {
        g->ring[g->f] = (int32_t)((uint32_t)g->ring[g->f] + (uint32_t)g->ring[g->b]);
        g->f = (g->f + 1) % 31; g->b = (g->b + 1) % 31;
    }
}

static int orc_glibc_next(orc_glibc_rand *g)
{
    uint32_t v = (uint32_t)g->ring[g->f] + (uint32_t)g->ring[g->b];
    g->ring[g->f] = (int32_t)v;
    g->f = (g->f + 1) % 31; g->b = (g->b + 1) % 31;
    return (int)(v >> 1);
}

/* FFEA's six-word seed from rng_seed (src/World.cpp:299-305):
 *   srand(seed); sixseed[i] = (rand() + rand()) % twoMax[i/3]
 * with the int sum wrapping and then converted to unsigned long. */
void orc_ffea_seed(int rng_seed, uint64_t out[6])
{
    orc_glibc_rand g;
    const uint64_t twoMax[2] = {4294967087ULL, 4294944443ULL};
    orc_glibc_srand(&g, (unsigned int)rng_seed);
    for (int i = 0; i < 6; i++) {
        int a = orc_glibc_next(&g);
        int b = orc_glibc_next(&g);
        int32_t s = (int32_t)((uint32_t)a + (uint32_t)b);
        uint64_t su = (uint64_t)(int64_t)s;
        out[i] = su % twoMax[i / 3];
    }
}

/* Stream k of the package after SetPackageSeed(six) (src/World.cpp:308-317):
 * stream k's state is A^(k * 2^127) six. */
void orc_ffea_thread_stream(const uint64_t six[6], int k, uint64_t out[6])
{
    double Cg[6];
    orc_mat A1, A2, B1, B2;
    for (int i = 0; i < 6; i++) Cg[i] = (double)six[i];
    orc_step_matrices(&A1, &A2);
    orc_mat2pow(&A1, 127, &B1, orc_m1u);
    orc_mat2pow(&A2, 127, &B2, orc_m2u);
    for (int j = 0; j < k; j++) orc_apply(&B1, &B2, Cg);
    for (int i = 0; i < 6; i++) out[i] = (uint64_t)Cg[i];
}

/* ------------------------------------------------------------------------ */
/* Blob state                                                                */
/* ------------------------------------------------------------------------ */
typedef struct {
    int num_nodes, num_elements;
    double *pos, *vel, *force;          /* 3 * num_nodes, AoS (x,y,z) */
    int *topo;                          /* 10 * num_elements */
    double *rho, *A, *B, *G, *E;        /* per element, meso units */
    double *stokes_drag;                /* per node: 6 pi eta r */
    int *is_pinned;                     /* per node */
    int num_pinned; int *pinned;
    /* element state (include/tetra_element_linear.h:135-190) */
    double *J_inv_0, *vol_0, *vol, *last_det, *dpsi, *visc, *node_force, *F_ij;
    /* params */
    double dt, kT, epsilon2;
    int max_iter, calc_noise, calc_stokes, solver, num_threads;
    int par_threads;                    /* > 1: parallel single-stream mode (orc_blob_set_parallel) */
    double *rng;                        /* 6 * num_threads exact-integer doubles */
    /* NoMass viscosity-matrix pattern: 3*num_nodes scalar rows */
    int nm_rows; int *nm_key; int *nm_col; double *nm_val;
    int *nm_src_ptr;                    /* nnz + 1 */
    int64_t *nm_src;                    /* >= 0: index into visc; -1: one; -2 - node: stokes drag */
    double *pre;                        /* preconditioner */
    double *r, *p, *z, *q, *f, *work_in, *work_out;
    /* mass matrix (scalar, num_nodes rows) */
    int *m_key; int *m_col; double *m_val;
    double *d, *s;
    int last_iters;
    int last_inversions;
    double *rhs_copy;                   /* rhs handed to the solver in the last step */
    double *ext;                        /* external forces per node (NULL: none), added every step */
    double *inv_m;                      /* lumped solver: inverse lumped mass per node */
    double *pos_0;                      /* positions after Blob::init (Blob::set_pos_0) */
} orc_blob;

static void *orc_alloc(size_t n) { void *p = calloc(n ? n : 1, 1); return p; }

/* Threads of the row-parallel loops (matrix build, SpMV): every row's sum
 * runs in the same order whatever the count, so the count changes no bit. */
static int orc_threads(const orc_blob *b) { return b->par_threads > b->num_threads ? b->par_threads : b->num_threads; }

/* calculate_jacobian (src/tetra_element_linear.cpp:193-205) */
static void orc_jacobian(const orc_blob *b, int e, double J[3][3])
{
    const int *n = &b->topo[10 * e];
    const double *p0 = &b->pos[3 * n[0]];
    for (int r = 0; r < 3; r++) {
        const double *pr = &b->pos[3 * n[r + 1]];
        J[r][0] = pr[0] - p0[0];
        J[r][1] = pr[1] - p0[1];
        J[r][2] = pr[2] - p0[2];
    }
}

/* calc_shape_function_derivatives_and_volume
 * (src/tetra_element_linear.cpp:223-293).  Returns ORC_ERROR on inversion
 * (last_det * det < 0) without touching last_det / vol, like the reference. */
static int orc_shape(orc_blob *b, int e, double J[3][3])
{
    double *dpsi = &b->dpsi[12 * e];
    double det;
    dpsi[1] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
    dpsi[2] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
    dpsi[3] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
    dpsi[5] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
    dpsi[6] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
    dpsi[7] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
    dpsi[9] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
    dpsi[10] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
    dpsi[11] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
    det = J[0][0] * dpsi[1] + J[1][0] * dpsi[2] + J[2][0] * dpsi[3];
    if (b->last_det[e] * det < 0) return ORC_ERROR;
    b->last_det[e] = det;
    b->vol[e] = (1.0 / 6.0) * fabs(det);
    det = 1.0 / det;
    dpsi[1] *= det; dpsi[2] *= det; dpsi[3] *= det;
    dpsi[5] *= det; dpsi[6] *= det; dpsi[7] *= det;
    dpsi[9] *= det; dpsi[10] *= det; dpsi[11] *= det;
    dpsi[0] = -(dpsi[1] + dpsi[2] + dpsi[3]);
    dpsi[4] = -(dpsi[5] + dpsi[6] + dpsi[7]);
    dpsi[8] = -(dpsi[9] + dpsi[10] + dpsi[11]);
    return ORC_OK;
}

/* create_viscosity_matrix (src/tetra_element_linear.cpp:299-328) with the
 * block formulas of include/tetra_element_linear.h:55-116 and
 * calc_del2_matrix / add_diffusion_matrix (:599-638). */
static void orc_viscosity(orc_blob *b, int e)
{
    const double *dpsi = &b->dpsi[12 * e];
    double (*V)[12] = (double (*)[12])&b->visc[144 * e];
    const double A = b->A[e], B = b->B[e];
    double K[4][4];
    for (int I = 0; I < 12; I += 4) {
        V[I + 0][I + 0] = dpsi[I + 0] * dpsi[I + 0] * (A + B);
        V[I + 1][I + 1] = dpsi[I + 1] * dpsi[I + 1] * (A + B);
        V[I + 2][I + 2] = dpsi[I + 2] * dpsi[I + 2] * (A + B);
        V[I + 3][I + 3] = dpsi[I + 3] * dpsi[I + 3] * (A + B);
        V[I + 0][I + 1] = dpsi[I + 1] * dpsi[I + 0] * (A + B);
        V[I + 0][I + 2] = dpsi[I + 2] * dpsi[I + 0] * (A + B);
        V[I + 0][I + 3] = dpsi[I + 3] * dpsi[I + 0] * (A + B);
        V[I + 1][I + 2] = dpsi[I + 1] * dpsi[I + 2] * (A + B);
        V[I + 1][I + 3] = dpsi[I + 1] * dpsi[I + 3] * (A + B);
        V[I + 2][I + 3] = dpsi[I + 2] * dpsi[I + 3] * (A + B);
    }
    static const int IJ[3][2] = {{0, 4}, {0, 8}, {4, 8}};
    for (int t = 0; t < 3; t++) {
        const int I = IJ[t][0], J = IJ[t][1];
        K[0][0] = dpsi[I] * dpsi[J];
        K[0][1] = dpsi[J + 1] * dpsi[I];
        K[0][2] = dpsi[J + 2] * dpsi[I];
        K[0][3] = dpsi[J + 3] * dpsi[I];
        for (int a = 1; a < 4; a++)
            for (int c = 0; c < 4; c++) K[a][c] = dpsi[I + a] * dpsi[J + c];
        for (int a = 0; a < 4; a++)
            for (int c = 0; c < 4; c++) {
                if (a == c) V[I + a][J + c] = (B + A) * K[a][a];
                else V[I + a][J + c] = B * K[a][c] + A * K[c][a];
            }
    }
    /* del2 (upper triangle) and the diffusion part on the diagonal blocks */
    double d2[4][4];
    for (int a = 0; a < 4; a++)
        for (int c = a; c < 4; c++)
            d2[a][c] = (dpsi[a] * dpsi[c] + dpsi[4 + a] * dpsi[4 + c] + dpsi[8 + a] * dpsi[8 + c]);
    for (int i = 0; i < 3; i++)
        for (int a = 0; a < 4; a++)
            for (int c = a; c < 4; c++) V[i * 4 + a][i * 4 + c] += d2[a][c] * A;
    const double vol = b->vol[e];
    for (int i = 0; i < 12; i++)
        for (int j = 0; j <= i; j++) V[j][i] *= vol;
    for (int i = 1; i < 12; i++)
        for (int j = 0; j < i; j++) V[i][j] = V[j][i];
}

/* mat3_mult_both_transposed / mat3_mult_transpose (src/mat_vec_fns.cpp:93-111)
 * and add_shear_elastic_stress (src/tetra_element_linear.cpp:378-396). */
static void orc_shear(orc_blob *b, int e, double J[3][3], double stress[3][3])
{
    double (*F)[3] = (double (*)[3])&b->F_ij[9 * e];
    const double (*Ji)[3] = (const double (*)[3])&b->J_inv_0[9 * e];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) F[i][j] = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) F[i][j] += J[k][i] * Ji[j][k];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) stress[i][j] += F[i][k] * F[j][k];
    const double s = (b->G[e] * b->vol_0[e] / b->vol[e]);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) stress[i][j] *= s;
    stress[0][0] -= b->G[e];
    stress[1][1] -= b->G[e];
    stress[2][2] -= b->G[e];
}

/* add_bulk_elastic_stress (src/tetra_element_linear.cpp:401-408) */
static void orc_bulk(const orc_blob *b, int e, double stress[3][3])
{
    const double G = b->G[e], E = b->E[e], v0 = b->vol_0[e], v = b->vol[e];
    double c_2 = E - G * 2.0 / 3.0;
    double c = G * (1.0 - (v0 / v)) + 0.5 * c_2 * ((v / v0) - (v0 / v));
    stress[0][0] += c;
    stress[1][1] += c;
    stress[2][2] += c;
}

#define ORC_RAND(rng) ((-.5) + ((.5) - (-.5)) * orc_u01(rng))

/* add_fluctuating_stress (src/tetra_element_linear.cpp:417-436): 7 draws. */
static void orc_fluct(const orc_blob *b, int e, double *rng, double stress[3][3])
{
    const double A = b->A[e], B = b->B[e];
    double c = sqrt((24 * b->kT) / (b->vol[e] * b->dt));
    double bf = sqrt(B) * ORC_RAND(rng);
    stress[0][0] += c * (sqrt(2 * A) * ORC_RAND(rng) + bf);
    stress[1][1] += c * (sqrt(2 * A) * ORC_RAND(rng) + bf);
    stress[2][2] += c * (sqrt(2 * A) * ORC_RAND(rng) + bf);
    stress[0][1] += c * sqrt(A) * ORC_RAND(rng);
    stress[0][2] += c * sqrt(A) * ORC_RAND(rng);
    stress[1][2] += c * sqrt(A) * ORC_RAND(rng);
    stress[1][0] = stress[0][1];
    stress[2][0] = stress[0][2];
    stress[2][1] = stress[1][2];
}

/* One element of Blob::update_internal_forces (src/Blob.cpp:650-733): the
 * element's nodal forces; returns 1 if the element inverted. */
static int orc_element(orc_blob *b, int n, double *rng)
{
    double J[3][3], stress[3][3], du[12];
    int inverted = 0;
    orc_jacobian(b, n, J);
    if (orc_shape(b, n, J) == ORC_ERROR) inverted = 1;
    orc_viscosity(b, n);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) stress[i][j] = 0;
    orc_shear(b, n, J, stress);
    orc_bulk(b, n, stress);
    if (b->calc_noise == 1) orc_fluct(b, n, rng, stress);
    if (b->solver != ORC_SOLVER_NOMASS) {
        /* get_element_velocity_vector + mat12_apply (src/tetra_element_linear.cpp:454-469, src/mat_vec_fns.cpp:26-34) */
        const int *nd = &b->topo[10 * n];
        double v[12], t[12];
        for (int a = 0; a < 4; a++) {
            v[a] = b->vel[3 * nd[a] + 0];
            v[4 + a] = b->vel[3 * nd[a] + 1];
            v[8 + a] = b->vel[3 * nd[a] + 2];
        }
        const double (*Vm)[12] = (const double (*)[12])&b->visc[144 * n];
        for (int i = 0; i < 12; i++) t[i] = 0;
        for (int i = 0; i < 12; i++)
            for (int j = 0; j < 12; j++) t[i] += Vm[i][j] * v[j];
        for (int i = 0; i < 12; i++) du[i] = t[i];
    } else {
        for (int i = 0; i < 12; i++) du[i] = 0;
    }
    /* apply_stress_tensor (src/tetra_element_linear.cpp:441-449) */
    const double *dpsi = &b->dpsi[12 * n];
    const double vol = b->vol[n];
    for (int i = 0; i < 3; i++) {
        du[4 * i] += vol * (dpsi[0] * stress[i][0] + dpsi[4] * stress[i][1] + dpsi[8] * stress[i][2]);
        du[4 * i + 1] += vol * (dpsi[1] * stress[i][0] + dpsi[5] * stress[i][1] + dpsi[9] * stress[i][2]);
        du[4 * i + 2] += vol * (dpsi[2] * stress[i][0] + dpsi[6] * stress[i][1] + dpsi[10] * stress[i][2]);
        du[4 * i + 3] += vol * (dpsi[3] * stress[i][0] + dpsi[7] * stress[i][1] + dpsi[11] * stress[i][2]);
    }
    /* add_element_force_vector (src/tetra_element_linear.cpp:474-489) */
    double *nf = &b->node_force[30 * n];
    for (int a = 0; a < 4; a++) {
        nf[3 * a + 0] -= du[a];
        nf[3 * a + 1] -= du[4 + a];
        nf[3 * a + 2] -= du[8 + a];
    }
    return inverted;
}

/* Blob::update_internal_forces (src/Blob.cpp:638-735). */
static int orc_internal_forces(orc_blob *b)
{
    int num_inversions = 0;
    const int E = b->num_elements;
    /* a blob with every node pinned takes no element step, so it draws no
     * element noise (src/Blob.cpp:643-645) */
    if (b->num_pinned == b->num_nodes) {
        b->last_inversions = 0;
        return ORC_OK;
    }
    if (b->par_threads > 1 && b->num_threads == 1) {
        /* Parallel evaluation with the single-stream draw order of a
         * one-thread run: element n takes draws 7n .. 7n+6 of the blob's
         * stream, so each thread starts from a copy of the stream jumped to
         * its first element.  Every element's arithmetic is unchanged, so
         * the results are those of the serial loop, bit for bit. */
        double start[6];
        memcpy(start, b->rng, sizeof(start));
#pragma omp parallel num_threads(b->par_threads) reduction(+ : num_inversions)
        {
            int nt = 1, t = 0;
#ifdef _OPENMP
            nt = omp_get_num_threads();
            t = omp_get_thread_num();
#endif
            const int e0 = (int)((int64_t)E * t / nt), e1 = (int)((int64_t)E * (t + 1) / nt);
            double rng[6];
            memcpy(rng, start, sizeof(rng));
            if (b->calc_noise == 1) orc_rng_advance(rng, 7ull * (uint64_t)e0);
            for (int n = e0; n < e1; n++) num_inversions += orc_element(b, n, rng);
        }
        if (b->calc_noise == 1) orc_rng_advance(b->rng, 7ull * (uint64_t)E);
        b->last_inversions = num_inversions;
        return num_inversions ? ORC_ERROR : ORC_OK;
    }
#pragma omp parallel num_threads(b->num_threads) reduction(+ : num_inversions)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *rng = &b->rng[6 * tid];
#pragma omp for schedule(guided)
        for (int n = 0; n < E; n++) num_inversions += orc_element(b, n, rng);
    }
    b->last_inversions = num_inversions;
    return num_inversions ? ORC_ERROR : ORC_OK;
}

/* Blob::linearise_force (src/Blob.cpp:1066-1085) */
static void orc_linearise_force(orc_blob *b)
{
    double *force = b->force;
    for (int i = 0; i < b->num_elements; i++) {
        const int *n = &b->topo[10 * i];
        for (int j = 0; j < 3; j++) {
            force[3 * n[0] + j] += 0.5 * (force[3 * n[4] + j] + force[3 * n[5] + j] + force[3 * n[6] + j]);
            force[3 * n[1] + j] += 0.5 * (force[3 * n[4] + j] + force[3 * n[7] + j] + force[3 * n[8] + j]);
            force[3 * n[2] + j] += 0.5 * (force[3 * n[5] + j] + force[3 * n[7] + j] + force[3 * n[9] + j]);
            force[3 * n[3] + j] += 0.5 * (force[3 * n[6] + j] + force[3 * n[8] + j] + force[3 * n[9] + j]);
        }
        for (int j = 4; j < 10; j++) {
            force[3 * n[j] + 0] = 0.;
            force[3 * n[j] + 1] = 0.;
            force[3 * n[j] + 2] = 0.;
        }
    }
}

/* ---- NoMassCGSolver ---------------------------------------------------- */

/* Sparsity pattern with source lists, equivalent to NoMassCGSolver::init
 * (src/NoMassCGSolver.cpp:63-162) + SparsityPattern (src/SparsityPattern.cpp:57-143).
 * Columns of a row are kept sorted; sources of an entry keep registration
 * order (element order, then the Stokes drag).  Built with counting passes
 * instead of linked lists; the resulting entries and source order are the
 * same. */
static int orc_nomass_init(orc_blob *b)
{
    const int Nn = b->num_nodes, E = b->num_elements;
    const int rows = 3 * Nn;
    b->nm_rows = rows;
    /* node -> sorted list of linear-pair neighbour nodes (incl. itself) */
    int *deg = orc_alloc(sizeof(int) * (Nn + 1));
    int *is_lin = orc_alloc(sizeof(int) * Nn);
    for (int e = 0; e < E; e++)
        for (int a = 0; a < 4; a++) is_lin[b->topo[10 * e + a]] = 1;
    /* count candidate neighbours with duplicates, then unique per node */
    for (int e = 0; e < E; e++)
        for (int a = 0; a < 4; a++) deg[b->topo[10 * e + a]] += 4;
    int *ptr = orc_alloc(sizeof(int) * (Nn + 1));
    for (int i = 0; i < Nn; i++) ptr[i + 1] = ptr[i] + deg[i];
    int *nb = orc_alloc(sizeof(int) * (ptr[Nn] + 1));
    int *fill = orc_alloc(sizeof(int) * (Nn + 1));
    for (int e = 0; e < E; e++)
        for (int a = 0; a < 4; a++) {
            int ni = b->topo[10 * e + a];
            for (int c = 0; c < 4; c++) nb[ptr[ni] + fill[ni]++] = b->topo[10 * e + c];
        }
    /* sort + unique per node (insertion sort: lists are short) */
    int *ucnt = orc_alloc(sizeof(int) * (Nn + 1));
    for (int i = 0; i < Nn; i++) {
        int *L = &nb[ptr[i]];
        int n = fill[i];
        for (int x = 1; x < n; x++) {
            int v = L[x], y = x - 1;
            while (y >= 0 && L[y] > v) { L[y + 1] = L[y]; y--; }
            L[y + 1] = v;
        }
        int u = 0;
        for (int x = 0; x < n; x++) if (u == 0 || L[u - 1] != L[x]) L[u++] = L[x];
        ucnt[i] = u;
    }
    /* rows: for node i unpinned & linear: 3 rows each with 3*ucnt entries (only
     * unpinned neighbours);  secondary or pinned node: only the diagonal. */
    b->nm_key = orc_alloc(sizeof(int) * (rows + 1));
    for (int i = 0; i < Nn; i++) {
        int cnt;
        if (is_lin[i] && !b->is_pinned[i]) {
            cnt = 0;
            for (int x = 0; x < ucnt[i]; x++) if (!b->is_pinned[nb[ptr[i] + x]]) cnt += 3;
        } else {
            cnt = 1;
        }
        for (int c = 0; c < 3; c++) b->nm_key[3 * i + c + 1] = cnt;
    }
    for (int r = 0; r < rows; r++) b->nm_key[r + 1] += b->nm_key[r];
    const int nnz = b->nm_key[rows];
    b->nm_col = orc_alloc(sizeof(int) * nnz);
    b->nm_val = orc_alloc(sizeof(double) * nnz);
    for (int i = 0; i < Nn; i++)
        for (int c = 0; c < 3; c++) {
            int r = 3 * i + c, k = b->nm_key[r];
            if (is_lin[i] && !b->is_pinned[i]) {
                for (int x = 0; x < ucnt[i]; x++) {
                    int j = nb[ptr[i] + x];
                    if (b->is_pinned[j]) continue;
                    for (int cc = 0; cc < 3; cc++) b->nm_col[k++] = 3 * j + cc;
                }
            } else {
                b->nm_col[k++] = r;
            }
        }
    /* sources: count, then fill in registration order */
    b->nm_src_ptr = orc_alloc(sizeof(int) * (nnz + 1));
    int *scount = orc_alloc(sizeof(int) * (nnz + 1));
#define ORC_FIND(row, col, out)                                                   \
    do {                                                                          \
        int lo_ = b->nm_key[row], hi_ = b->nm_key[(row) + 1] - 1, f_ = -1;        \
        while (lo_ <= hi_) {                                                      \
            int mid_ = (lo_ + hi_) / 2;                                           \
            if (b->nm_col[mid_] == (col)) { f_ = mid_; break; }                   \
            if (b->nm_col[mid_] < (col)) lo_ = mid_ + 1; else hi_ = mid_ - 1;     \
        }                                                                         \
        (out) = f_;                                                               \
    } while (0)
    /* element contributions: linear pairs, unpinned both */
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            for (int x = 0; x < nnz; x++) b->nm_src_ptr[x + 1] = b->nm_src_ptr[x] + scount[x];
            b->nm_src = orc_alloc(sizeof(int64_t) * (b->nm_src_ptr[nnz] + 1));
            memset(scount, 0, sizeof(int) * (nnz + 1));
        }
        for (int e = 0; e < E; e++)
            for (int ni = 0; ni < 4; ni++)
                for (int nj = 0; nj < 4; nj++) {
                    int a = b->topo[10 * e + ni], c = b->topo[10 * e + nj];
                    if (b->is_pinned[a] || b->is_pinned[c]) continue;
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++) {
                            int k;
                            ORC_FIND(3 * a + i, 3 * c + j, k);
                            if (pass == 1) b->nm_src[b->nm_src_ptr[k] + scount[k]] = (int64_t)144 * e + (ni + 4 * i) * 12 + (nj + 4 * j);
                            scount[k]++;
                        }
                }
        /* "one" on secondary / pinned diagonals (registered once) */
        for (int i = 0; i < Nn; i++) {
            if (is_lin[i] && !b->is_pinned[i]) continue;
            for (int c = 0; c < 3; c++) {
                int k = b->nm_key[3 * i + c];
                if (pass == 1) b->nm_src[b->nm_src_ptr[k] + scount[k]] = -1;
                scount[k]++;
            }
        }
        /* Stokes drag on every unpinned diagonal, registered last */
        if (b->calc_stokes == 1) {
            for (int i = 0; i < Nn; i++) {
                if (b->is_pinned[i]) continue;
                for (int c = 0; c < 3; c++) {
                    int k;
                    ORC_FIND(3 * i + c, 3 * i + c, k);
                    if (pass == 1) b->nm_src[b->nm_src_ptr[k] + scount[k]] = -2 - (int64_t)i;
                    scount[k]++;
                }
            }
        }
    }
#undef ORC_FIND
    b->pre = orc_alloc(sizeof(double) * rows);
    b->r = orc_alloc(sizeof(double) * rows);
    b->p = orc_alloc(sizeof(double) * rows);
    b->z = orc_alloc(sizeof(double) * rows);
    b->q = orc_alloc(sizeof(double) * rows);
    b->f = orc_alloc(sizeof(double) * rows);
    b->work_in = orc_alloc(sizeof(double) * rows);
    b->work_out = orc_alloc(sizeof(double) * rows);
    free(deg); free(ptr); free(nb); free(fill); free(ucnt); free(scount); free(is_lin);
    return ORC_OK;
}

/* SparseMatrixFixedPattern::build (src/SparseMatrixFixedPattern.cpp:85-93,
 * src/SparseMatrixTypes.cpp:52-58) */
static void orc_nomass_build(orc_blob *b)
{
    const int nnz = b->nm_key[b->nm_rows];
#pragma omp parallel for num_threads(orc_threads(b))
    for (int x = 0; x < nnz; x++) {
        double sum = 0.0;
        for (int s = b->nm_src_ptr[x]; s < b->nm_src_ptr[x + 1]; s++) {
            int64_t src = b->nm_src[s];
            if (src >= 0) sum += b->visc[src];
            else if (src == -1) sum += 1.0;
            else sum += b->stokes_drag[-2 - src];
        }
        b->nm_val[x] = sum;
    }
}

/* SparseMatrixFixedPattern::apply(vector3*, vector3*) (src/SparseMatrixFixedPattern.cpp:148-191) */
static void orc_nomass_apply(orc_blob *b, const double *in, double *out)
{
    const int rows = b->nm_rows;
#pragma omp parallel for num_threads(orc_threads(b))
    for (int i = 0; i < rows; i++) {
        double acc = 0.0;
        for (int j = b->nm_key[i]; j < b->nm_key[i + 1]; j++) acc += b->nm_val[j] * in[b->nm_col[j]];
        out[i] = acc;
    }
}

/* NoMassCGSolver::solve with more than one thread: the same iteration as
 * orc_nomass_solve below, with the vector updates and the dot products
 * spread over the threads as FFEA's OpenMP loops spread them
 * (src/NoMassCGSolver.cpp:209, 236, 253, 268, 281; src/mat_vec_fns.cpp:253,
 * 268).  The reductions round in a different order than the serial sums. */
static int orc_nomass_solve_par(orc_blob *b, double *x)
{
    const int rows = b->nm_rows, T = orc_threads(b);
    double *r = b->r, *p = b->p, *z = b->z, *q = b->q, *f = b->f, *pre = b->pre;
    double delta_new = 0, delta_old, pTq, alpha, f2 = 0;
#pragma omp parallel for num_threads(T) reduction(+ : delta_new, f2)
    for (int i = 0; i < rows; i++) {
        r[i] = x[i];
        f[i] = x[i];
        x[i] = 0;
        z[i] = pre[i] * r[i];
        p[i] = z[i];
        delta_new += r[i] * z[i];
        f2 += f[i] * f[i];
    }
    for (int it = 0; it < b->max_iter; it++) {
        orc_nomass_apply(b, p, q);
        pTq = 0;
#pragma omp parallel for num_threads(T) reduction(+ : pTq)
        for (int i = 0; i < rows; i++) pTq += p[i] * q[i];
        alpha = delta_new / pTq;
        double r2 = 0;
#pragma omp parallel for num_threads(T) reduction(+ : r2)
        for (int i = 0; i < rows; i++) {
            x[i] += alpha * p[i];
            r[i] += -alpha * q[i];
            r2 += r[i] * r[i];
        }
        const double res = (f2 == 0.0) ? 0.0 : r2 / f2;
        if (res < b->epsilon2) { b->last_iters = it + 1; return ORC_OK; }
        delta_old = delta_new;
        delta_new = 0;
#pragma omp parallel for num_threads(T) reduction(+ : delta_new)
        for (int i = 0; i < rows; i++) {
            z[i] = pre[i] * r[i];
            delta_new += r[i] * z[i];
        }
        const double beta = (delta_new / delta_old);
#pragma omp parallel for num_threads(T)
        for (int i = 0; i < rows; i++) p[i] = beta * p[i] + z[i];
    }
    b->last_iters = b->max_iter;
    return ORC_ERROR;
}

/* NoMassCGSolver::solve (src/NoMassCGSolver.cpp:165-197) with its helpers
 * (:205-291) and vec3_add_to_scaled / vec3_scale_and_add (src/mat_vec_fns.cpp:250-275). */
static int orc_nomass_solve(orc_blob *b, double *x)
{
    const int Nn = b->num_nodes;
    const int rows = b->nm_rows;
    orc_nomass_build(b);
    /* calc_inverse_diagonal (src/SparseMatrixFixedPattern.cpp:325-333) */
#pragma omp parallel for num_threads(orc_threads(b))
    for (int i = 0; i < rows; i++) {
        double dg = 0;
        for (int j = b->nm_key[i]; j < b->nm_key[i + 1]; j++) if (b->nm_col[j] == i) dg = b->nm_val[j];
        b->pre[i] = 1.0 / dg;
    }
    if (orc_threads(b) > 1) return orc_nomass_solve_par(b, x);
    double *r = b->r, *p = b->p, *z = b->z, *q = b->q, *f = b->f, *pre = b->pre;
    double delta_new = 0, delta_old, pTq, alpha;
    /* conjugate_gradient_residual_assume_x_zero (:205-230) */
    for (int i = 0; i < Nn; i++) {
        for (int c = 0; c < 3; c++) {
            r[3 * i + c] = x[3 * i + c];
            f[3 * i + c] = x[3 * i + c];
            x[3 * i + c] = 0;
            z[3 * i + c] = pre[3 * i + c] * r[3 * i + c];
            p[3 * i + c] = z[3 * i + c];
        }
        delta_new += r[3 * i] * z[3 * i] + r[3 * i + 1] * z[3 * i + 1] + r[3 * i + 2] * z[3 * i + 2];
    }
    for (int it = 0; it < b->max_iter; it++) {
        /* get_alpha_denominator (:261-275) */
        orc_nomass_apply(b, p, q);
        pTq = 0;
        for (int i = 0; i < Nn; i++)
            pTq += p[3 * i] * q[3 * i] + p[3 * i + 1] * q[3 * i + 1] + p[3 * i + 2] * q[3 * i + 2];
        alpha = delta_new / pTq;
        for (int i = 0; i < rows; i++) x[i] += alpha * p[i];
        for (int i = 0; i < rows; i++) r[i] += -alpha * q[i];
        /* residual2 (:233-247) */
        double r2 = 0, f2 = 0, res;
        for (int i = 0; i < Nn; i++) {
            r2 += r[3 * i] * r[3 * i] + r[3 * i + 1] * r[3 * i + 1] + r[3 * i + 2] * r[3 * i + 2];
            f2 += f[3 * i] * f[3 * i] + f[3 * i + 1] * f[3 * i + 1] + f[3 * i + 2] * f[3 * i + 2];
        }
        res = (f2 == 0.0) ? 0.0 : r2 / f2;
        if (res < b->epsilon2) { b->last_iters = it + 1; return ORC_OK; }
        delta_old = delta_new;
        /* parallel_apply_preconditioner (:278-291) */
        delta_new = 0;
        for (int i = 0; i < Nn; i++) {
            for (int c = 0; c < 3; c++) z[3 * i + c] = pre[3 * i + c] * r[3 * i + c];
            delta_new += r[3 * i] * z[3 * i] + r[3 * i + 1] * z[3 * i + 1] + r[3 * i + 2] * z[3 * i + 2];
        }
        const double beta = (delta_new / delta_old);
        for (int i = 0; i < rows; i++) p[i] = beta * p[i] + z[i];
    }
    b->last_iters = b->max_iter;
    return ORC_ERROR;
}

/* ---- ConjugateGradientSolver (mass matrix) ----------------------------- */

/* ConjugateGradientSolver::init (src/ConjugateGradientSolver.cpp:62-204),
 * without the dense N^2 scratch: entries accumulate per (row, col) in element
 * order, so every value is the same sum in the same order. */
static int orc_mass_init(orc_blob *b)
{
    const int Nn = b->num_nodes, E = b->num_elements;
    /* neighbour lists over all 10 nodes (diagonal only for secondary) */
    int *cnt = orc_alloc(sizeof(int) * (Nn + 1));
    for (int e = 0; e < E; e++)
        for (int i = 0; i < 10; i++) {
            int ni = b->topo[10 * e + i];
            cnt[ni] += (i < 4) ? 4 : 1;
        }
    int *ptr = orc_alloc(sizeof(int) * (Nn + 1));
    for (int i = 0; i < Nn; i++) ptr[i + 1] = ptr[i] + cnt[i];
    int *nb = orc_alloc(sizeof(int) * (ptr[Nn] + 1));
    int *fill = orc_alloc(sizeof(int) * (Nn + 1));
    for (int e = 0; e < E; e++)
        for (int i = 0; i < 10; i++) {
            int ni = b->topo[10 * e + i];
            if (i < 4) {
                for (int j = 0; j < 4; j++) {
                    int nj = b->topo[10 * e + j];
                    /* pinned pairs other than the diagonal never get a value */
                    if ((b->is_pinned[ni] || b->is_pinned[nj]) && ni != nj) continue;
                    nb[ptr[ni] + fill[ni]++] = nj;
                }
            } else {
                nb[ptr[ni] + fill[ni]++] = ni;
            }
        }
    b->m_key = orc_alloc(sizeof(int) * (Nn + 1));
    for (int i = 0; i < Nn; i++) {
        int *L = &nb[ptr[i]];
        int n = fill[i];
        for (int x = 1; x < n; x++) {
            int v = L[x], y = x - 1;
            while (y >= 0 && L[y] > v) { L[y + 1] = L[y]; y--; }
            L[y + 1] = v;
        }
        int u = 0;
        for (int x = 0; x < n; x++) if (u == 0 || L[u - 1] != L[x]) L[u++] = L[x];
        fill[i] = u;
        b->m_key[i + 1] = b->m_key[i] + u;
    }
    const int nnz = b->m_key[Nn];
    b->m_col = orc_alloc(sizeof(int) * nnz);
    b->m_val = orc_alloc(sizeof(double) * nnz);
    for (int i = 0; i < Nn; i++)
        for (int x = 0; x < fill[i]; x++) b->m_col[b->m_key[i] + x] = nb[ptr[i] + x];
    for (int e = 0; e < E; e++)
        for (int i = 0; i < 10; i++)
            for (int j = 0; j < 10; j++) {
                int ni = b->topo[10 * e + i], nj = b->topo[10 * e + j];
                int k = -1;
                for (int x = b->m_key[ni]; x < b->m_key[ni + 1]; x++) if (b->m_col[x] == nj) { k = x; break; }
                if (i < 4 && j < 4) {
                    if (b->is_pinned[ni] == 0 && b->is_pinned[nj] == 0) {
                        if (i == j) b->m_val[k] += .1 * b->rho[e] * b->vol_0[e];
                        else b->m_val[k] += .05 * b->rho[e] * b->vol_0[e];
                    } else if (i == j) {
                        b->m_val[k] = 1;
                    }
                } else if (i == j) {
                    b->m_val[k] = 1;
                }
            }
    b->pre = orc_alloc(sizeof(double) * Nn);
    for (int i = 0; i < Nn; i++)
        for (int x = b->m_key[i]; x < b->m_key[i + 1]; x++) if (b->m_col[x] == i) b->pre[i] = 1.0 / b->m_val[x];
    b->d = orc_alloc(sizeof(double) * 3 * Nn);
    b->r = orc_alloc(sizeof(double) * 3 * Nn);
    b->q = orc_alloc(sizeof(double) * 3 * Nn);
    b->s = orc_alloc(sizeof(double) * 3 * Nn);
    b->f = orc_alloc(sizeof(double) * 3 * Nn);
    free(cnt); free(ptr); free(nb); free(fill);
    return ORC_OK;
}

/* MassLumpedSolver::init (src/MassLumpedSolver.cpp:40-78): a quarter of each
 * element's mass rho vol_0 on each corner, 1 on secondary and pinned nodes,
 * inverted. */
static int orc_lumped_init(orc_blob *b)
{
    const int Nn = b->num_nodes;
    b->inv_m = orc_alloc(sizeof(double) * Nn);
    for (int n = 0; n < b->num_elements; n++)
        for (int i = 0; i < 10; i++) {
            const int ni = b->topo[10 * n + i];
            if (i < 4) b->inv_m[ni] += .25 * b->rho[n] * b->vol_0[n];
            else b->inv_m[ni] = 1;
        }
    for (int i = 0; i < b->num_pinned; i++) b->inv_m[b->pinned[i]] = 1.0;
    for (int i = 0; i < Nn; i++) b->inv_m[i] = 1.0 / b->inv_m[i];
    return ORC_OK;
}

/* MassLumpedSolver::solve (src/MassLumpedSolver.cpp:81-89) */
static int orc_lumped_solve(orc_blob *b, double *x)
{
    for (int i = 0; i < b->num_nodes; i++) {
        x[3 * i] = x[3 * i] * b->inv_m[i];
        x[3 * i + 1] = x[3 * i + 1] * b->inv_m[i];
        x[3 * i + 2] = x[3 * i + 2] * b->inv_m[i];
    }
    b->last_iters = 0;
    return ORC_OK;
}

/* ConjugateGradientSolver::solve (src/ConjugateGradientSolver.cpp:206-232,
 * helpers :249-349). */
static int orc_mass_solve(orc_blob *b, double *x)
{
    const int Nn = b->num_nodes;
    double *r = b->r, *d = b->d, *q = b->q, *s = b->s, *f = b->f, *pre = b->pre;
    double delta_new = 0, delta_old, dTq, alpha;
    for (int i = 0; i < Nn; i++) {
        for (int c = 0; c < 3; c++) {
            r[3 * i + c] = x[3 * i + c];
            f[3 * i + c] = x[3 * i + c];
            x[3 * i + c] = 0;
            d[3 * i + c] = pre[i] * r[3 * i + c];
        }
        delta_new += r[3 * i] * d[3 * i] + r[3 * i + 1] * d[3 * i + 1] + r[3 * i + 2] * d[3 * i + 2];
    }
    for (int it = 0; it < b->max_iter; it++) {
        double r2 = 0, f2 = 0, res;
        for (int i = 0; i < Nn; i++) {
            r2 += r[3 * i] * r[3 * i] + r[3 * i + 1] * r[3 * i + 1] + r[3 * i + 2] * r[3 * i + 2];
            f2 += f[3 * i] * f[3 * i] + f[3 * i + 1] * f[3 * i + 1] + f[3 * i + 2] * f[3 * i + 2];
        }
        res = (f2 == 0.0) ? 0.0 : r2 / f2;
        if (res < b->epsilon2) { b->last_iters = it; return ORC_OK; }
        dTq = 0;
        for (int i = 0; i < Nn; i++) {
            double qx = 0, qy = 0, qz = 0;
            for (int j = b->m_key[i]; j < b->m_key[i + 1]; j++) {
                const int cidx = b->m_col[j];
                qx += b->m_val[j] * d[3 * cidx];
                qy += b->m_val[j] * d[3 * cidx + 1];
                qz += b->m_val[j] * d[3 * cidx + 2];
            }
            q[3 * i] = qx; q[3 * i + 1] = qy; q[3 * i + 2] = qz;
            dTq += d[3 * i] * q[3 * i] + d[3 * i + 1] * q[3 * i + 1] + d[3 * i + 2] * q[3 * i + 2];
        }
        alpha = delta_new / dTq;
        for (int i = 0; i < 3 * Nn; i++) x[i] += alpha * d[i];
        for (int i = 0; i < 3 * Nn; i++) r[i] += -alpha * q[i];
        delta_old = delta_new;
        delta_new = 0;
        for (int i = 0; i < Nn; i++) {
            for (int c = 0; c < 3; c++) s[3 * i + c] = pre[i] * r[3 * i + c];
            delta_new += r[3 * i] * s[3 * i] + r[3 * i + 1] * s[3 * i + 1] + r[3 * i + 2] * s[3 * i + 2];
        }
        const double beta = (delta_new / delta_old);
        for (int i = 0; i < 3 * Nn; i++) d[i] = s[i] + beta * d[i];
    }
    b->last_iters = b->max_iter;
    return ORC_ERROR;
}

/* Blob::aggregate_forces_and_solve (src/Blob.cpp:3826-3931) */
static int orc_aggregate_and_solve(orc_blob *b)
{
    const int Nn = b->num_nodes, E = b->num_elements;
    double *force = b->force;
    /* node gather in node order, contributions in element order (the order
     * calculate_node_element_connectivity builds, src/Blob.cpp:3974-4019) */
    for (int e = 0; e < E; e++)
        for (int j = 0; j < 10; j++) {
            int nd = b->topo[10 * e + j];
            force[3 * nd + 0] += b->node_force[30 * e + 3 * j + 0];
            force[3 * nd + 1] += b->node_force[30 * e + 3 * j + 1];
            force[3 * nd + 2] += b->node_force[30 * e + 3 * j + 2];
        }
    if (b->calc_stokes == 1) {
        double *rng = &b->rng[0];
        if (b->solver != ORC_SOLVER_NOMASS) {
            for (int i = 0; i < Nn; i++) {
                force[3 * i + 0] -= b->vel[3 * i + 0] * b->stokes_drag[i];
                force[3 * i + 1] -= b->vel[3 * i + 1] * b->stokes_drag[i];
                force[3 * i + 2] -= b->vel[3 * i + 2] * b->stokes_drag[i];
                if (b->calc_noise == 1) {
                    force[3 * i + 0] -= ORC_RAND(rng) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                    force[3 * i + 1] -= ORC_RAND(rng) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                    force[3 * i + 2] -= ORC_RAND(rng) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                }
            }
        } else if (b->calc_noise == 1) {
            for (int i = 0; i < Nn; i++) {
                force[3 * i + 0] -= ORC_RAND(rng) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                force[3 * i + 1] -= ORC_RAND(rng) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
                force[3 * i + 2] -= ORC_RAND(rng) * sqrt((24 * b->kT * b->stokes_drag[i]) / (b->dt));
            }
        }
    }
    orc_linearise_force(b);
    for (int n = 0; n < b->num_pinned; n++) {
        int pn = b->pinned[n];
        force[3 * pn + 0] = 0;
        force[3 * pn + 1] = 0;
        force[3 * pn + 2] = 0;
    }
    memcpy(b->rhs_copy, force, sizeof(double) * 3 * Nn);
    if (b->solver == ORC_SOLVER_NOMASS) return orc_nomass_solve(b, force);
    if (b->solver == ORC_SOLVER_LUMPED) return orc_lumped_solve(b, force);
    return orc_mass_solve(b, force);
}

/* Blob::euler_integrate (src/Blob.cpp:3937-3969) and linearise_element for
 * every element (src/Blob.cpp:759-761, src/tetra_element_linear.cpp:567-591). */
static void orc_euler_and_linearise(orc_blob *b)
{
    const int Nn = b->num_nodes;
    double *pos = b->pos, *vel = b->vel, *force = b->force;
    if (b->solver == ORC_SOLVER_NOMASS) {
        for (int i = 0; i < Nn; i++)
            for (int c = 0; c < 3; c++) {
                vel[3 * i + c] = force[3 * i + c];
                pos[3 * i + c] += force[3 * i + c] * b->dt;
            }
    } else {
        for (int i = 0; i < Nn; i++) {
            for (int c = 0; c < 3; c++) vel[3 * i + c] += force[3 * i + c] * b->dt;
            for (int c = 0; c < 3; c++) pos[3 * i + c] += vel[3 * i + c] * b->dt;
        }
    }
    static const int mid[6][3] = {{4, 0, 1}, {5, 0, 2}, {6, 0, 3}, {7, 1, 2}, {8, 1, 3}, {9, 2, 3}};
    for (int e = 0; e < b->num_elements; e++) {
        const int *n = &b->topo[10 * e];
        for (int m = 0; m < 6; m++)
            for (int c = 0; c < 3; c++)
                pos[3 * n[mid[m][0]] + c] = .5 * (pos[3 * n[mid[m][1]] + c] + pos[3 * n[mid[m][2]] + c]);
    }
}

/* ------------------------------------------------------------------------ */
/* Public oracle API (ctypes)                                                */
/* ------------------------------------------------------------------------ */

/* Create a blob.  material: 5 doubles per element (rho, A, B, G, E; meso
 * units, as Blob::load_material_params leaves them, src/Blob.cpp:2864-2867).
 * stokes_drag: per node (6 pi eta r, src/Blob.cpp:408-412).
 * fparams: dt, kT, epsilon2.  iparams: max_iterations_cg, calc_noise,
 * calc_stokes, solver (0 = CG_nomass, 1 = CG, 2 = masslumped), num_threads. */
orc_blob *orc_blob_create(int num_nodes, int num_elements, const double *pos, const int *topo,
                          const double *material, const double *stokes_drag, int num_pinned,
                          const int *pinned, const double *fparams, const int *iparams)
{
    orc_blob *b = orc_alloc(sizeof(orc_blob));
    b->num_nodes = num_nodes;
    b->num_elements = num_elements;
    b->dt = fparams[0]; b->kT = fparams[1]; b->epsilon2 = fparams[2];
    b->max_iter = iparams[0]; b->calc_noise = iparams[1]; b->calc_stokes = iparams[2];
    b->solver = iparams[3]; b->num_threads = iparams[4] > 0 ? iparams[4] : 1;
    b->pos = orc_alloc(sizeof(double) * 3 * num_nodes);
    b->vel = orc_alloc(sizeof(double) * 3 * num_nodes);
    b->force = orc_alloc(sizeof(double) * 3 * num_nodes);
    b->rhs_copy = orc_alloc(sizeof(double) * 3 * num_nodes);
    memcpy(b->pos, pos, sizeof(double) * 3 * num_nodes);
    b->topo = orc_alloc(sizeof(int) * 10 * num_elements);
    memcpy(b->topo, topo, sizeof(int) * 10 * num_elements);
    for (int x = 0; x < 10 * num_elements; x++)
        if (topo[x] < 0 || topo[x] >= num_nodes) { free(b); return NULL; }
    b->rho = orc_alloc(sizeof(double) * num_elements);
    b->A = orc_alloc(sizeof(double) * num_elements);
    b->B = orc_alloc(sizeof(double) * num_elements);
    b->G = orc_alloc(sizeof(double) * num_elements);
    b->E = orc_alloc(sizeof(double) * num_elements);
    for (int e = 0; e < num_elements; e++) {
        b->rho[e] = material[5 * e + 0]; b->A[e] = material[5 * e + 1]; b->B[e] = material[5 * e + 2];
        b->G[e] = material[5 * e + 3]; b->E[e] = material[5 * e + 4];
    }
    b->stokes_drag = orc_alloc(sizeof(double) * num_nodes);
    if (stokes_drag) memcpy(b->stokes_drag, stokes_drag, sizeof(double) * num_nodes);
    b->is_pinned = orc_alloc(sizeof(int) * num_nodes);
    b->num_pinned = num_pinned;
    b->pinned = orc_alloc(sizeof(int) * (num_pinned + 1));
    for (int i = 0; i < num_pinned; i++) { b->pinned[i] = pinned[i]; b->is_pinned[pinned[i]] = 1; }
    b->J_inv_0 = orc_alloc(sizeof(double) * 9 * num_elements);
    b->vol_0 = orc_alloc(sizeof(double) * num_elements);
    b->vol = orc_alloc(sizeof(double) * num_elements);
    b->last_det = orc_alloc(sizeof(double) * num_elements);
    b->dpsi = orc_alloc(sizeof(double) * 12 * num_elements);
    b->visc = orc_alloc(sizeof(double) * 144 * num_elements);
    b->node_force = orc_alloc(sizeof(double) * 30 * num_elements);
    b->F_ij = orc_alloc(sizeof(double) * 9 * num_elements);
    b->rng = orc_alloc(sizeof(double) * 6 * b->num_threads);
    for (int t = 0; t < b->num_threads; t++)
        for (int i = 0; i < 6; i++) b->rng[6 * t + i] = 12345.0;
    /* Blob::init: linearise_element for all, calc_rest_state_info
     * (src/Blob.cpp:334-340, :3760-3822 with mat3_invert src/mat_vec_fns.cpp:148-175) */
    static const int mid[6][3] = {{4, 0, 1}, {5, 0, 2}, {6, 0, 3}, {7, 1, 2}, {8, 1, 3}, {9, 2, 3}};
    for (int e = 0; e < num_elements; e++) {
        const int *n = &b->topo[10 * e];
        for (int m = 0; m < 6; m++)
            for (int c = 0; c < 3; c++)
                b->pos[3 * n[mid[m][0]] + c] = .5 * (b->pos[3 * n[mid[m][1]] + c] + b->pos[3 * n[mid[m][2]] + c]);
    }
    /* World::init then records these positions (src/World.cpp:504, Blob::set_pos_0) */
    b->pos_0 = orc_alloc(sizeof(double) * 3 * num_nodes);
    memcpy(b->pos_0, b->pos, sizeof(double) * 3 * num_nodes);
    for (int e = 0; e < num_elements; e++) {
        double J[3][3], (*mi)[3] = (double (*)[3])&b->J_inv_0[9 * e], det;
        orc_jacobian(b, e, J);
        mi[0][0] = J[2][2] * J[1][1] - J[2][1] * J[1][2];
        mi[0][1] = J[2][1] * J[0][2] - J[2][2] * J[0][1];
        mi[0][2] = J[1][2] * J[0][1] - J[1][1] * J[0][2];
        mi[1][0] = J[2][0] * J[1][2] - J[2][2] * J[1][0];
        mi[1][1] = J[2][2] * J[0][0] - J[2][0] * J[0][2];
        mi[1][2] = J[1][0] * J[0][2] - J[1][2] * J[0][0];
        mi[2][0] = J[2][1] * J[1][0] - J[2][0] * J[1][1];
        mi[2][1] = J[2][0] * J[0][1] - J[2][1] * J[0][0];
        mi[2][2] = J[1][1] * J[0][0] - J[1][0] * J[0][1];
        det = J[0][0] * mi[0][0] + J[1][0] * mi[0][1] + J[2][0] * mi[0][2];
        det = 1.0 / det;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) mi[i][j] *= det;
        orc_shape(b, e, J);
        b->vol_0[e] = b->vol[e];
    }
    /* the solver init (src/Blob.cpp:359-380) */
    if (b->solver == ORC_SOLVER_NOMASS) orc_nomass_init(b);
    else if (b->solver == ORC_SOLVER_LUMPED) orc_lumped_init(b);
    else orc_mass_init(b);
    return b;
}

void orc_blob_destroy(orc_blob *b)
{
    if (!b) return;
    void *ptrs[] = {b->pos, b->vel, b->force, b->topo, b->rho, b->A, b->B, b->G, b->E, b->stokes_drag,
                    b->is_pinned, b->pinned, b->J_inv_0, b->vol_0, b->vol, b->last_det, b->dpsi, b->visc,
                    b->node_force, b->F_ij, b->rng, b->nm_key, b->nm_col, b->nm_val, b->nm_src_ptr,
                    b->nm_src, b->pre, b->r, b->p, b->z, b->q, b->f, b->work_in, b->work_out, b->m_key,
                    b->m_col, b->m_val, b->d, b->s, b->rhs_copy, b->ext, b->inv_m, b->pos_0};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    free(b);
}

/* World::init seeding with 1..num_threads streams (src/World.cpp:299-317). */
void orc_blob_seed(orc_blob *b, int rng_seed)
{
    uint64_t six[6], st[6];
    orc_ffea_seed(rng_seed, six);
    for (int t = 0; t < b->num_threads; t++) {
        orc_ffea_thread_stream(six, t, st);
        for (int i = 0; i < 6; i++) b->rng[6 * t + i] = (double)st[i];
    }
}

void orc_blob_set_rng_state(orc_blob *b, int thread, const uint64_t *st)
{
    for (int i = 0; i < 6; i++) b->rng[6 * thread + i] = (double)st[i];
}

void orc_blob_get_rng_state(const orc_blob *b, int thread, uint64_t *st)
{
    for (int i = 0; i < 6; i++) st[i] = (uint64_t)b->rng[6 * thread + i];
}

/* One World::run step for this blob: zero_force + set_forces_to_zero
 * (src/World.cpp:1845,1907), update_internal_forces, update_positions
 * (src/World.cpp:2024-2043).  Returns ORC_ERROR on inversion or
 * non-convergence, like the reference. */
int orc_blob_step(orc_blob *b, int nsteps)
{
    for (int s = 0; s < nsteps; s++) {
        memset(b->node_force, 0, sizeof(double) * 30 * b->num_elements);
        memset(b->force, 0, sizeof(double) * 3 * b->num_nodes);
        /* interactions and constant forces add to Blob::force before the
         * element loop (src/World.cpp:1907 zeroes it; springs
         * src/World.cpp:3808-3846; Blob::apply_ctforces src/Blob.cpp:647,
         * 2094-2162 through add_force_to_node-style sums, :2195-2199) */
        if (b->ext)
            for (int i = 0; i < 3 * b->num_nodes; i++) b->force[i] += b->ext[i];
        if (orc_internal_forces(b) != ORC_OK) return ORC_ERROR;
        if (orc_aggregate_and_solve(b) != ORC_OK) return ORC_ERROR;
        orc_euler_and_linearise(b);
    }
    return ORC_OK;
}

/* External forces: count (node, 3 components) entries, summed per node in
 * the given order, applied at every following step; count 0 clears them. */
void orc_blob_set_external_forces(orc_blob *b, int count, const int *nodes, const double *forces)
{
    if (!b->ext) b->ext = (double *)orc_alloc(sizeof(double) * 3 * b->num_nodes);
    memset(b->ext, 0, sizeof(double) * 3 * b->num_nodes);
    for (int i = 0; i < count; i++)
        for (int c = 0; c < 3; c++) b->ext[3 * nodes[i] + c] += forces[3 * i + c];
}

void orc_blob_get_nodes(const orc_blob *b, double *pos, double *vel, double *force)
{
    const size_t n = sizeof(double) * 3 * b->num_nodes;
    if (pos) memcpy(pos, b->pos, n);
    if (vel) memcpy(vel, b->vel, n);
    if (force) memcpy(force, b->force, n);
}

void orc_blob_set_nodes(orc_blob *b, const double *pos, const double *vel)
{
    const size_t n = sizeof(double) * 3 * b->num_nodes;
    if (pos) memcpy(b->pos, pos, n);
    if (vel) memcpy(b->vel, vel, n);
}

/* rhs handed to the solver in the last step (after gather, Stokes terms,
 * linearise_force and pinning) */
void orc_blob_get_rhs(const orc_blob *b, double *out) { memcpy(out, b->rhs_copy, sizeof(double) * 3 * b->num_nodes); }

/* element nodal forces of the last step: 12 per element (node 0..3, x,y,z) */
void orc_blob_get_element_forces(const orc_blob *b, double *out)
{
    for (int e = 0; e < b->num_elements; e++)
        for (int a = 0; a < 4; a++)
            for (int c = 0; c < 3; c++) out[12 * e + 3 * a + c] = b->node_force[30 * e + 3 * a + c];
}

/* Parallel single-stream mode (test infrastructure for large meshes): with
 * one RNG stream (num_threads 1), spread the element loop, the matrix build,
 * the SpMV and the NoMass CG vector work over `threads` threads while every
 * draw keeps its serial position in the stream.  Element forces, the matrix
 * and each SpMV are then bit-identical to a one-thread run; the NoMass CG dot
 * products sum in another order (FP64 round-off only).  threads <= 1 turns
 * the mode off.  Returns 0, or -1 if the blob has several streams. */
int orc_blob_set_parallel(orc_blob *b, int threads)
{
    if (b->num_threads != 1 && threads > 1) return -1;
    b->par_threads = threads > 1 ? threads : 0;
    return 0;
}

int orc_blob_last_cg_iters(const orc_blob *b) { return b->last_iters; }
int orc_blob_last_inversions(const orc_blob *b) { return b->last_inversions; }

/* Apply the current NoMass matrix (built from the current viscosity
 * matrices) to a 3*num_nodes vector: NoMassCGSolver's V->apply. */
void orc_blob_apply_nomass(orc_blob *b, const double *in, double *out)
{
    orc_nomass_build(b);
    orc_nomass_apply(b, in, out);
}

/* Blob::make_measurements strain / kinetic energy (src/Blob.cpp:1363-1432)
 * evaluated at the current positions and velocities (no noise): the values
 * the reference prints at the next step's measurement. */
void orc_blob_energies(orc_blob *b, double *strain, double *kinetic)
{
    double se = 0, ke = 0;
    for (int n = 0; n < b->num_elements; n++) {
        double J[3][3], stress[3][3] = {{0}};
        double save_det = b->last_det[n];
        orc_jacobian(b, n, J);
        orc_shape(b, n, J);
        b->last_det[n] = save_det;
        orc_shear(b, n, J, stress);
        if (b->solver != ORC_SOLVER_NOMASS) {
            const int *nd = &b->topo[10 * n];
            double v[12], t[12] = {0};
            for (int a = 0; a < 4; a++) {
                v[a] = b->vel[3 * nd[a]]; v[4 + a] = b->vel[3 * nd[a] + 1]; v[8 + a] = b->vel[3 * nd[a] + 2];
            }
            static const double M[4][4] = {{.1, .05, .05, .05}, {.05, .1, .05, .05}, {.05, .05, .1, .05}, {.05, .05, .05, .1}};
            for (int k = 0; k < 12; k += 4)
                for (int i = 0; i < 4; i++)
                    for (int j = 0; j < 4; j++) t[i + k] += M[i][j] * v[j + k];
            for (int i = 0; i < 12; i++) t[i] = t[i] * (b->vol_0[n] * b->rho[n]);
            for (int i = 0; i < 12; i++) ke += v[i] * t[i];
        }
        const double *F = &b->F_ij[9 * n];
        double C = b->E[n] - (2.0 / 3.0) * b->G[n];
        double t1 = b->vol[n] / b->vol_0[n];
        double ff = F[0] * F[0] + F[4] * F[4] + F[8] * F[8] + F[1] * F[1] + F[3] * F[3] + F[2] * F[2] + F[6] * F[6] + F[5] * F[5] + F[7] * F[7];
        se += b->vol_0[n] * (b->G[n] * (ff - 3) + 0.5 * C * (t1 * t1 - 1) - (C + 2 * b->G[n]) * log(t1));
    }
    *strain = se * 0.5;
    *kinetic = ke * 0.5;
}

/* The rest of Blob::make_measurements (src/Blob.cpp:1433-1527) at the
 * current state: out[0..2] the centroid of all nodes, out[3] the RMSD from
 * pos_0 (remTrans off), out[4..6] the centre of mass as Blob::get_CoM sums it
 * (src/Blob.cpp:951-967: the element mass multiplies the first corner only,
 * the sum is divided by the element count), out[7..9] the angular momentum
 * about that point, left at 0 for CG_nomass. */
void orc_blob_measurements(const orc_blob *b, double *out)
{
    static const double MM[4][4] = {{.1, .05, .05, .05}, {.05, .1, .05, .05}, {.05, .05, .1, .05}, {.05, .05, .05, .1}};
    double com[3] = {0, 0, 0}, cog[3] = {0, 0, 0}, l[3] = {0, 0, 0}, msd = 0;
    for (int n = 0; n < b->num_elements; n++) {
        const int *nd = &b->topo[10 * n];
        const double mass = b->vol_0[n] * b->rho[n];
        for (int c = 0; c < 3; c++)
            com[c] += (mass * b->pos[3 * nd[0] + c] + b->pos[3 * nd[1] + c] + b->pos[3 * nd[2] + c] +
                       b->pos[3 * nd[3] + c]) / 4;
    }
    if (b->num_elements)
        for (int c = 0; c < 3; c++) com[c] /= b->num_elements;
    if (b->solver != ORC_SOLVER_NOMASS) {
        for (int n = 0; n < b->num_elements; n++) {
            const int *nd = &b->topo[10 * n];
            double r[4][3], t[3] = {0, 0, 0};
            for (int i = 0; i < 4; i++)
                for (int c = 0; c < 3; c++) r[i][c] = b->pos[3 * nd[i] + c] - com[c];
            for (int i = 0; i < 4; i++) {
                const double *v = &b->vel[3 * nd[i]];
                for (int j = 0; j < 4; j++) {
                    t[0] += MM[i][j] * (r[j][1] * v[2] - r[j][2] * v[1]);
                    t[1] += MM[i][j] * (r[j][2] * v[0] - r[j][0] * v[2]);
                    t[2] += MM[i][j] * (r[j][0] * v[1] - r[j][1] * v[0]);
                }
            }
            const double mass = b->vol_0[n] * b->rho[n];
            for (int c = 0; c < 3; c++) l[c] += mass * t[c];
        }
    }
    for (int i = 0; i < b->num_nodes; i++) {
        double d[3];
        for (int c = 0; c < 3; c++) {
            cog[c] += b->pos[3 * i + c];
            d[c] = b->pos[3 * i + c] - b->pos_0[3 * i + c];
        }
        msd += d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    }
    for (int c = 0; c < 3; c++) {
        out[c] = cog[c] / b->num_nodes;
        out[4 + c] = com[c];
        out[7 + c] = l[c];
    }
    out[3] = sqrt(msd / b->num_nodes);
}

int orc_num_threads_available(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
