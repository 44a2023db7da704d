// mrg32k3a.cuh -- MRG32k3a in exact integer arithmetic, host and device.
//
// The generator is L'Ecuyer's combined multiple-recursive generator
// (Operations Research 47(1), 1999) as packaged in RngStreams (L'Ecuyer,
// Simard, Chen, Kelton 2002) and used by FFEA (src/RngStream.cpp:266-289):
//   component 1: x_n = (1403580 x_{n-2} - 810728 x_{n-3}) mod m1
//   component 2: y_n = (527612 y_{n-1} - 1370589 y_{n-3}) mod m2
//   u = ((x - y) mod m1) / (m1 + 1)          (x == y gives m1 / (m1 + 1))
// The reference stores the state in doubles but every value is an exact
// integer, so evaluating the recurrences in int64 gives the same words, and
// the final multiply by 1/(m1+1) is the same single double rounding: draws
// are bit-identical.
//
// Jump-ahead: A^n applied to a state advances it by n draws.  A GPU thread
// that needs draw number `off` of a step multiplies the step's base state by
// A^off = T3[d3] T2[d2] T1[d1] T0[d0] (base-256 digits of off), four 3x3
// matrix-vector products per component from a 1024-entry table.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define MRG_HD __host__ __device__ __forceinline__
#else
#define MRG_HD inline
#endif

namespace mrg {

constexpr uint32_t M1 = 4294967087u;  // 2^32 - 209
constexpr uint32_t M2 = 4294944443u;  // 2^32 - 22853
constexpr uint32_t C1 = 209u;
constexpr uint32_t C2 = 22853u;
constexpr int JUMP_DIGIT_BITS = 8;
constexpr int JUMP_LEVELS = 4;                     // offsets < 2^32
constexpr int JUMP_TABLE_ENTRIES = JUMP_LEVELS << JUMP_DIGIT_BITS;

// A pair of 3x3 matrices (component 1 mod M1, component 2 mod M2), row major.
struct JumpMat {
    uint32_t a[18];
};

// x mod M = 2^32 - C for any 64-bit x, C < 2^15: fold the high word twice
// (2^32 = C mod M).  After the first fold t < 2^32 (C + 1), after the second
// t < 2^32 + C (C + 1) = M + C (C + 2) < 2 M, so one conditional subtraction
// leaves the residue in [0, M).
template <uint32_t M, uint32_t C>
MRG_HD uint32_t reduce64(uint64_t x)
{
    static_assert(C < (1u << 15), "the bound below needs C (C + 2) < M");
    uint64_t t = (x >> 32) * C + (x & 0xffffffffull);  // < 2^32 (C + 1)
    t = (t >> 32) * C + (t & 0xffffffffull);           // < M + C (C + 2)
    if (t >= M) t -= M;
    return (uint32_t)t;
}

template <uint32_t M, uint32_t C>
MRG_HD uint32_t mulmod(uint32_t a, uint32_t b)
{
    return reduce64<M, C>((uint64_t)a * b);
}

template <uint32_t M, uint32_t C>
MRG_HD void matvec3(const uint32_t *A, uint32_t *v)
{
    uint32_t t[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        uint64_t s = (uint64_t)mulmod<M, C>(A[3 * i + 0], v[0]) + mulmod<M, C>(A[3 * i + 1], v[1]) +
                     mulmod<M, C>(A[3 * i + 2], v[2]);
        t[i] = reduce64<M, C>(s);
    }
    v[0] = t[0]; v[1] = t[1]; v[2] = t[2];
}

MRG_HD void apply(const JumpMat &J, uint32_t *s)
{
    matvec3<M1, C1>(J.a, s);
    matvec3<M2, C2>(J.a + 9, s + 3);
}

// Advance `s` by `off` draws using the 4-level base-256 table.
MRG_HD void jump(const JumpMat *table, uint32_t off, uint32_t *s)
{
#pragma unroll
    for (int l = 0; l < JUMP_LEVELS; l++) {
        uint32_t d = (off >> (JUMP_DIGIT_BITS * l)) & ((1u << JUMP_DIGIT_BITS) - 1u);
        if (d) apply(table[(l << JUMP_DIGIT_BITS) + d], s);
    }
}

// One step of both components (the recurrences of src/RngStream.cpp:270-283
// on int64); returns n = (p1 - p2) mod m1 in [1, m1] (m1 when p1 == p2),
// the integer that :286 scales by 1 / (m1 + 1).
// Each difference a s_i - b s_j is taken as a s_i + b (m - s_j), the same
// residue, with both products below 2^53 (a, b < 2^21; states below m), and
// reduced by folding (reduce64) rather than by a 64-bit division, which the
// GPU runs as a long instruction sequence.
MRG_HD int64_t next_n(uint32_t *s)
{
    const uint32_t p1 = reduce64<M1, C1>(1403580ull * s[1] + 810728ull * (uint64_t)(M1 - s[0]));
    s[0] = s[1]; s[1] = s[2]; s[2] = p1;
    const uint32_t p2 = reduce64<M2, C2>(527612ull * s[5] + 1370589ull * (uint64_t)(M2 - s[3]));
    s[3] = s[4]; s[4] = s[5]; s[5] = p2;
    return (p1 > p2) ? (int64_t)p1 - (int64_t)p2 : (int64_t)p1 - (int64_t)p2 + (int64_t)M1;
}

// One draw: the combination of src/RngStream.cpp:286 in double.  Returns u
// in (0, 1).
MRG_HD double u01(uint32_t *s)
{
    const double norm = 1.0 / (4294967087.0 + 1.0);
    return (double)next_n(s) * norm;
}

// RAND(-.5, .5) of include/tetra_element_linear.h:118: -0.5 + 1.0 * u.
MRG_HD double centred(uint32_t *s)
{
    return -0.5 + u01(s);
}

// The same draw in FP32 with no FP64 arithmetic: -0.5 + n / (m1 + 1) is
// (n - (m1 + 1) / 2) / (m1 + 1) exactly, an int32 numerator times one
// constant; two FP32 roundings (numerator, product) put it within 2 ulp of
// the FP64 value rounded to FP32.  The stream's integer state is the same.
MRG_HD float centred_f(uint32_t *s)
{
    constexpr float norm = (float)(1.0 / (4294967087.0 + 1.0));
    const int32_t q = (int32_t)(next_n(s) - 2147483544ll);  // (m1 + 1) / 2
    return (float)q * norm;
}

// ---- host-side helpers (table construction) --------------------------------
inline void mat_identity(uint32_t *A)
{
    for (int i = 0; i < 9; i++) A[i] = (i % 4 == 0) ? 1u : 0u;
}

template <uint32_t M, uint32_t C>
inline void matmul3(const uint32_t *A, const uint32_t *B, uint32_t *out)
{
    uint32_t t[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            uint64_t s = (uint64_t)mulmod<M, C>(A[3 * i], B[j]) + mulmod<M, C>(A[3 * i + 1], B[3 + j]) +
                         mulmod<M, C>(A[3 * i + 2], B[6 + j]);
            t[3 * i + j] = reduce64<M, C>(s);
        }
    for (int i = 0; i < 9; i++) out[i] = t[i];
}

inline void jm_mul(const JumpMat &A, const JumpMat &B, JumpMat &out)
{
    JumpMat t;
    matmul3<M1, C1>(A.a, B.a, t.a);
    matmul3<M2, C2>(A.a + 9, B.a + 9, t.a + 9);
    out = t;
}

inline JumpMat jm_identity()
{
    JumpMat J;
    mat_identity(J.a);
    mat_identity(J.a + 9);
    return J;
}

// One-draw transition (the recurrences above as companion matrices).
inline JumpMat jm_step()
{
    JumpMat J;
    for (int i = 0; i < 18; i++) J.a[i] = 0;
    J.a[1] = 1; J.a[5] = 1; J.a[6] = M1 - 810728u; J.a[7] = 1403580u;
    J.a[9 + 1] = 1; J.a[9 + 5] = 1; J.a[9 + 6] = M2 - 1370589u; J.a[9 + 8] = 527612u;
    return J;
}

inline JumpMat jm_pow(JumpMat base, uint64_t n)
{
    JumpMat r = jm_identity();
    while (n) {
        if (n & 1) jm_mul(r, base, r);
        jm_mul(base, base, base);
        n >>= 1;
    }
    return r;
}

// table[l*256 + d] = A^(d * 256^l)
inline void build_jump_table(JumpMat *table)
{
    JumpMat unit = jm_step();
    for (int l = 0; l < JUMP_LEVELS; l++) {
        JumpMat acc = jm_identity();
        for (int d = 0; d < (1 << JUMP_DIGIT_BITS); d++) {
            table[(l << JUMP_DIGIT_BITS) + d] = acc;
            jm_mul(acc, unit, acc);
        }
        unit = acc;  // A^(256^(l+1))
    }
}

}  // namespace mrg
