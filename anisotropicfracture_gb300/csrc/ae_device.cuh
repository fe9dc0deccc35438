// Device-side building blocks of the nodal elastic operator: geometry, field views,
// finite-difference stencils, stiffness contractions, boundary rows and the per-node
// operator.  Templated on the arithmetic type R (double or float) and on the stiffness
// kind M.
//
// Reference formulas restated here:
//   stencils          src/Numeric/Stencil.H:16-176
//   MajorMinor C:grad src/Set/Matrix4_MajorMinor.H:253-269, C:gradgrad :287-345
//   Isotropic         src/Set/Matrix4_Isotropic.H:60-91
//   Diagonal          src/Set/Matrix4_Diagonal.H:48-74
//   Major (45 slots)  src/Set/Matrix4_Major.H:198-300, 399-428
//   boundary rows     src/BC/Operator/Elastic.H:218-303
//   Fapply            src/Operator/Elastic.cpp:174-258
#pragma once
#include <cstdint>

namespace ae {

enum Model { ISO = 0, MM = 1, DIAG = 2, MAJOR = 3 };
template <int M> struct NCoef;
template <> struct NCoef<ISO> { static constexpr int value = 2; };
template <> struct NCoef<MM> { static constexpr int value = 21; };
template <> struct NCoef<DIAG> { static constexpr int value = 9; };
template <> struct NCoef<MAJOR> { static constexpr int value = 45; };

// Set::Matrix4<3, Sym::Major>: the 9 x 9 matrix A(3i+j, 3k+l) = C_ijkl is symmetric; its upper
// triangle is stored row by row in 45 slots.  Slot of entry (I, K).
__host__ __device__ constexpr int major_slot(int I, int K) {
    return I <= K ? I * 9 - I * (I - 1) / 2 + (K - I) : K * 9 - K * (K - 1) / 2 + (I - K);
}

// FP32 rows in one fixed rounding order.  The compiler fuses a product into a neighbouring
// addition at its own discretion, and the choice can differ between kernels that inline the same
// expression in different surroundings.  The FP32 operator's sums of products therefore go through
// explicitly rounded operations -- additions rounded, the first product of a sum rounded and each
// further one fused into the running sum -- so that every FP32 kernel computes a node's row to the
// same bits.  FP64 keeps the written expressions.
__device__ __forceinline__ float fx_sop_acc(float r) { return r; }
template <class... T>
__device__ __forceinline__ float fx_sop_acc(float r, float a, float x, T... rest) {
    return fx_sop_acc(__fmaf_rn(a, x, r), rest...);
}
// a0 x0 + a1 x1 + ... in that order
template <class... T>
__device__ __forceinline__ float fx_sop(float a, float x, T... rest) {
    return fx_sop_acc(__fmul_rn(a, x), rest...);
}
template <class R>
__device__ __forceinline__ R add2(R x, R y) {
    if constexpr (sizeof(R) == 4) return __fadd_rn(x, y);
    else return x + y;
}
// a0 x0 + ... + a5 x5 (one row of a MajorMinor contraction)
template <class R>
__device__ __forceinline__ R sop6(R a0, R x0, R a1, R x1, R a2, R x2, R a3, R x3, R a4, R x4, R a5, R x5) {
    if constexpr (sizeof(R) == 4) return fx_sop(a0, x0, a1, x1, a2, x2, a3, x3, a4, x4, a5, x5);
    else return a0 * x0 + a1 * x1 + a2 * x2 + a3 * x3 + a4 * x4 + a5 * x5;
}
// (c0 h0 + c1 h1) + c2 h2: the grad C columns of a row scaled by the central-difference factors
template <class R>
__device__ __forceinline__ R gradc_sum(R c0, R c1, R c2, const R h[3]) {
    if constexpr (sizeof(R) == 4) return fx_sop(c0, h[0], c1, h[1], c2, h[2]);
    else return (c0 * h[0] + c1 * h[1]) + c2 * h[2];
}
// f + the grad C term of the row
template <class R>
__device__ __forceinline__ R gradc_add(R f, R c0, R c1, R c2, const R h[3]) {
    if constexpr (sizeof(R) == 4) return __fadd_rn(f, gradc_sum(c0, c1, c2, h));
    else return f + ((c0 * h[0] + c1 * h[1]) + c2 * h[2]);
}

enum BCType { DISP = 0, TRAC = 1, PERIODIC = 2, NEUMANN = 3 };

struct Box3 {
    int lo[3], hi[3];
};

// One level (one nodal patch): domain, valid box, ghost layers stored around it.
struct Geo {
    int dlo[3], dhi[3];  // nodal problem domain (inclusive)
    int vlo[3], vhi[3];  // nodal valid box
    int ng;              // ghost layers stored: storage box = grow(valid, ng)
    int px = 0;          // row pitch of the level's internal arrays in nodes (0: the storage box's
                         // x-extent); padded to a multiple of 4 so rows start on 16-byte boundaries
    double dx[3];
};

// Field view in AMReX Array4 order: p points at (lo, comp 0).
template <class T>
struct View {
    T* p;
    int lo[3];
    long long sy, sz, sc;
    int wx = 0;  // nodes per row when the row pitch sy is padded past them (0: sy)
    __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
        return (long long)(i - lo[0]) + (long long)(j - lo[1]) * sy + (long long)(k - lo[2]) * sz;
    }
};

// Stencil constants, computed on the host in double precision.
template <class R>
struct SCoef {
    R h[3];        // 0.5 / dx   (central first derivative)
    R id[3];       // 1 / dx     (one-sided first derivative)
    R i2[3];       // 1 / dx^2   (second derivative)
    R m01, m02, m12;  // 0.25 / (dx_a dx_b)  (mixed derivative)
    R bb[3];       // -2 / dx / dx  (diagonal of the second derivative)
};

// BC types per face (26) and direction (3).
struct BCP {
    unsigned char t[26][3];
};

// Truncated normals of src/BC/Operator/Elastic.H:218-219
#define AE_SQRT3INV 0.57735026919
#define AE_SQRT2INV 0.70710678118

// Face index of a domain-boundary node, -1 for interior nodes; numbering and
// precedence (corner, edge, face) of src/BC/Operator/Elastic.H:236-278.
template <class R>
__device__ __forceinline__ int classify(const Geo& g, int i, int j, int k, R n[3]) {
    const int s0 = (i == g.dlo[0]) ? -1 : (i == g.dhi[0]) ? 1 : 0;
    const int s1 = (j == g.dlo[1]) ? -1 : (j == g.dhi[1]) ? 1 : 0;
    const int s2 = (k == g.dlo[2]) ? -1 : (k == g.dhi[2]) ? 1 : 0;
    const int cnt = (s0 != 0) + (s1 != 0) + (s2 != 0);
    if (cnt == 0) return -1;
    const R w = cnt == 3 ? R(AE_SQRT3INV) : cnt == 2 ? R(AE_SQRT2INV) : R(1.0);
    n[0] = s0 == 0 ? R(0) : (s0 > 0 ? w : -w);
    n[1] = s1 == 0 ? R(0) : (s1 > 0 ? w : -w);
    n[2] = s2 == 0 ? R(0) : (s2 > 0 ? w : -w);
    if (cnt == 3) return 18 + 4 * (s0 > 0) + 2 * (s1 > 0) + (s2 > 0);
    if (cnt == 2) {
        if (s0 == 0) return 6 + 2 * (s1 > 0) + (s2 > 0);
        if (s1 == 0) return 10 + 2 * (s2 > 0) + (s0 > 0);
        return 14 + 2 * (s0 > 0) + (s1 > 0);
    }
    if (s0) return s0 < 0 ? 0 : 3;
    if (s1) return s1 < 0 ? 1 : 4;
    return s2 < 0 ? 2 : 5;
}

// ------------------------------------------------------------------ contractions
template <class R>
__device__ __forceinline__ void stress_mm(const R* a, const R g[3][3], R s[3][3]) {
    const R e01 = g[0][1] + g[1][0], e02 = g[0][2] + g[2][0], e12 = g[1][2] + g[2][1];
    const R r00 = a[0] * g[0][0] + a[1] * e01 + a[2] * e02 + a[3] * g[1][1] + a[4] * e12 + a[5] * g[2][2];
    const R r11 = a[3] * g[0][0] + a[8] * e01 + a[12] * e02 + a[15] * g[1][1] + a[16] * e12 + a[17] * g[2][2];
    const R r22 = a[5] * g[0][0] + a[10] * e01 + a[14] * e02 + a[17] * g[1][1] + a[19] * e12 + a[20] * g[2][2];
    const R r12 = a[4] * g[0][0] + a[9] * e01 + a[13] * e02 + a[16] * g[1][1] + a[18] * e12 + a[19] * g[2][2];
    const R r20 = a[2] * g[0][0] + a[7] * e01 + a[11] * e02 + a[12] * g[1][1] + a[13] * e12 + a[14] * g[2][2];
    const R r01 = a[1] * g[0][0] + a[6] * e01 + a[7] * e02 + a[8] * g[1][1] + a[9] * e12 + a[10] * g[2][2];
    s[0][0] = r00; s[1][1] = r11; s[2][2] = r22;
    s[1][2] = r12; s[2][1] = r12;
    s[2][0] = r20; s[0][2] = r20;
    s[0][1] = r01; s[1][0] = r01;
}
template <class R>
__device__ __forceinline__ void stress_iso(const R* a, const R g[3][3], R s[3][3]) {
    const R lambda = a[0], mu = a[1];
    s[0][0] = (lambda + R(2) * mu) * g[0][0] + lambda * g[1][1] + lambda * g[2][2];
    s[1][1] = lambda * g[0][0] + (lambda + R(2) * mu) * g[1][1] + lambda * g[2][2];
    s[2][2] = lambda * g[0][0] + lambda * g[1][1] + (lambda + R(2) * mu) * g[2][2];
    s[1][2] = mu * (g[1][2] + g[2][1]); s[2][1] = s[1][2];
    s[2][0] = mu * (g[2][0] + g[0][2]); s[0][2] = s[2][0];
    s[0][1] = mu * (g[0][1] + g[1][0]); s[1][0] = s[0][1];
}
template <class R>
__device__ __forceinline__ void stress_diag(const R* a, const R g[3][3], R s[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) s[i][j] = a[3 * i + j] * g[i][j];
}
// Matrix4_Major.H:399-413: sigma_ij = sum_kl C_ijkl g_kl, summed in (k, l) order
template <class R>
__device__ __forceinline__ void stress_major(const R* a, const R g[3][3], R s[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            R r = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int l = 0; l < 3; ++l) r += a[major_slot(3 * i + j, 3 * k + l)] * g[k][l];
            s[i][j] = r;
        }
}
template <int M, class R>
__device__ __forceinline__ void stress_of(const R* a, const R g[3][3], R s[3][3]) {
    if (M == ISO) stress_iso(a, g, s);
    else if (M == MM) stress_mm(a, g, s);
    else if (M == MAJOR) stress_major(a, g, s);
    else stress_diag(a, g, s);
}

// C_ijkl u_{k,lj} with b[k][l][j] = u_{k,lj}
template <class R>
__device__ __forceinline__ void div_mm(const R* a, const R b[3][3][3], R f[3]) {
#define B(p, q, r) b[p][q][r]
    if constexpr (sizeof(R) == 4) {
        // the same terms in the same order, explicitly rounded
#define S2(x, y) __fadd_rn(x, y)
#define S3(x, y, z) __fadd_rn(__fadd_rn(x, y), z)
#define S4(x, y, z, w) __fadd_rn(__fadd_rn(__fadd_rn(x, y), z), w)
        f[0] = fx_sop(a[0], B(0, 0, 0), a[1], S3(B(0, 1, 0), B(1, 0, 0), B(0, 0, 1)),
                      a[2], S3(B(0, 2, 0), B(2, 0, 0), B(0, 0, 2)), a[3], B(1, 1, 0), a[4], S2(B(1, 2, 0), B(2, 1, 0)),
                      a[5], B(2, 2, 0), a[6], S2(B(0, 1, 1), B(1, 0, 1)),
                      a[7], S4(B(0, 2, 1), B(2, 0, 1), B(0, 1, 2), B(1, 0, 2)), a[8], B(1, 1, 1),
                      a[9], S2(B(1, 2, 1), B(2, 1, 1)), a[10], B(2, 2, 1), a[11], S2(B(0, 2, 2), B(2, 0, 2)),
                      a[12], B(1, 1, 2), a[13], S2(B(1, 2, 2), B(2, 1, 2)), a[14], B(2, 2, 2));
        f[1] = fx_sop(a[1], B(0, 0, 0), a[4], B(0, 0, 2), a[3], B(0, 0, 1), a[6], S2(B(0, 1, 0), B(1, 0, 0)),
                      a[7], S2(B(0, 2, 0), B(2, 0, 0)), a[8], S3(B(1, 1, 0), B(0, 1, 1), B(1, 0, 1)),
                      a[9], S4(B(1, 2, 0), B(2, 1, 0), B(0, 1, 2), B(1, 0, 2)), a[10], B(2, 2, 0),
                      a[12], S2(B(0, 2, 1), B(2, 0, 1)), a[13], S2(B(0, 2, 2), B(2, 0, 2)), a[15], B(1, 1, 1),
                      a[16], S3(B(1, 2, 1), B(2, 1, 1), B(1, 1, 2)), a[17], B(2, 2, 1), a[18], S2(B(1, 2, 2), B(2, 1, 2)),
                      a[19], B(2, 2, 2));
        f[2] = fx_sop(a[2], B(0, 0, 0), a[4], B(0, 0, 1), a[5], B(0, 0, 2), a[7], S2(B(0, 1, 0), B(1, 0, 0)),
                      a[9], S2(B(0, 1, 1), B(1, 0, 1)), a[10], S2(B(0, 1, 2), B(1, 0, 2)),
                      a[11], S2(B(0, 2, 0), B(2, 0, 0)), a[12], B(1, 1, 0),
                      a[13], S4(B(1, 2, 0), B(2, 1, 0), B(0, 2, 1), B(2, 0, 1)),
                      a[14], S3(B(2, 2, 0), B(0, 2, 2), B(2, 0, 2)), a[16], B(1, 1, 1), a[17], B(1, 1, 2),
                      a[18], S2(B(1, 2, 1), B(2, 1, 1)), a[19], S3(B(2, 2, 1), B(1, 2, 2), B(2, 1, 2)), a[20], B(2, 2, 2));
#undef S2
#undef S3
#undef S4
        return;
    }
    f[0] = a[0] * B(0, 0, 0) + a[1] * (B(0, 1, 0) + B(1, 0, 0) + B(0, 0, 1)) +
           a[2] * (B(0, 2, 0) + B(2, 0, 0) + B(0, 0, 2)) + a[3] * B(1, 1, 0) + a[4] * (B(1, 2, 0) + B(2, 1, 0)) +
           a[5] * B(2, 2, 0) + a[6] * (B(0, 1, 1) + B(1, 0, 1)) +
           a[7] * (B(0, 2, 1) + B(2, 0, 1) + B(0, 1, 2) + B(1, 0, 2)) + a[8] * B(1, 1, 1) +
           a[9] * (B(1, 2, 1) + B(2, 1, 1)) + a[10] * B(2, 2, 1) + a[11] * (B(0, 2, 2) + B(2, 0, 2)) +
           a[12] * B(1, 1, 2) + a[13] * (B(1, 2, 2) + B(2, 1, 2)) + a[14] * B(2, 2, 2);
    f[1] = a[1] * B(0, 0, 0) + a[4] * B(0, 0, 2) + a[3] * B(0, 0, 1) + a[6] * (B(0, 1, 0) + B(1, 0, 0)) +
           a[7] * (B(0, 2, 0) + B(2, 0, 0)) + a[8] * (B(1, 1, 0) + B(0, 1, 1) + B(1, 0, 1)) +
           a[9] * (B(1, 2, 0) + B(2, 1, 0) + B(0, 1, 2) + B(1, 0, 2)) + a[10] * B(2, 2, 0) +
           a[12] * (B(0, 2, 1) + B(2, 0, 1)) + a[13] * (B(0, 2, 2) + B(2, 0, 2)) + a[15] * B(1, 1, 1) +
           a[16] * (B(1, 2, 1) + B(2, 1, 1) + B(1, 1, 2)) + a[17] * B(2, 2, 1) + a[18] * (B(1, 2, 2) + B(2, 1, 2)) +
           a[19] * B(2, 2, 2);
    f[2] = a[2] * B(0, 0, 0) + a[4] * B(0, 0, 1) + a[5] * B(0, 0, 2) + a[7] * (B(0, 1, 0) + B(1, 0, 0)) +
           a[9] * (B(0, 1, 1) + B(1, 0, 1)) + a[10] * (B(0, 1, 2) + B(1, 0, 2)) +
           a[11] * (B(0, 2, 0) + B(2, 0, 0)) + a[12] * B(1, 1, 0) +
           a[13] * (B(1, 2, 0) + B(2, 1, 0) + B(0, 2, 1) + B(2, 0, 1)) +
           a[14] * (B(2, 2, 0) + B(0, 2, 2) + B(2, 0, 2)) + a[16] * B(1, 1, 1) + a[17] * B(1, 1, 2) +
           a[18] * (B(1, 2, 1) + B(2, 1, 1)) + a[19] * (B(2, 2, 1) + B(1, 2, 2) + B(2, 1, 2)) + a[20] * B(2, 2, 2);
#undef B
}
template <class R>
__device__ __forceinline__ void div_iso(const R* a, const R b[3][3][3], R f[3]) {
    const R lambda = a[0], mu = a[1];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        R r = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) r += mu * (b[i][j][j] + b[j][i][j]) + lambda * b[j][j][i];
        f[i] = r;
    }
}
template <class R>
__device__ __forceinline__ void div_diag(const R* a, const R b[3][3][3], R f[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        R r = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) r += a[3 * i + j] * b[i][j][j];
        f[i] = r;
    }
}
// Matrix4_Major.H:415-428: f_i = sum_{j,k,l} C_ijkl b[k][l][j], b[k][l][j] = u_{k,lj}
template <class R>
__device__ __forceinline__ void div_major(const R* a, const R b[3][3][3], R f[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        R r = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int l = 0; l < 3; ++l) r += a[major_slot(3 * i + j, 3 * k + l)] * b[k][l][j];
        f[i] = r;
    }
}
template <int M, class R>
__device__ __forceinline__ void div_of(const R* a, const R b[3][3][3], R f[3]) {
    if (M == ISO) div_iso(a, b, f);
    else if (M == MM) div_mm(a, b, f);
    else if (M == MAJOR) div_major(a, b, f);
    else div_diag(a, b, f);
}

// read-only load: through the non-coherent cache for global memory (LDG), plain otherwise
// (stiffness staged in shared memory)
// A Voronoi stiffness on one level: a grain id per node (laid out like the level's stiffness
// view) and a per-grain coefficient table tab[g * ncoef + q].  gid == nullptr: not used.
template <class R>
struct Grains {
    const unsigned short* gid = nullptr;
    const R* tab = nullptr;
};

template <bool LDG, class T>
__device__ __forceinline__ T ldv(const T* p) {
    if constexpr (LDG) return __ldg(p);
    else return *p;
}

// Column d of (dC : grad u), dC the (unscaled) central difference of the stiffness in
// direction d.  Only the slots that feed column d are read: 15 of 21 for MajorMinor.
template <int M, class R, bool LDG = true>
__device__ __forceinline__ void gradC_col(const R* __restrict__ C, long long cs, long long c, long long o,
                                          const R g[3][3], int d, R col[3]) {
#define DC(q) (ldv<LDG>(C + (q) * cs + c + o) - ldv<LDG>(C + (q) * cs + c - o))
    if (M == MM) {
        const R e00 = g[0][0], e11 = g[1][1], e22 = g[2][2];
        const R e01 = add2(g[0][1], g[1][0]), e02 = add2(g[0][2], g[2][0]), e12 = add2(g[1][2], g[2][1]);
        if (d == 0) {  // (s00, s01, s20)
            const R a0 = DC(0), a1 = DC(1), a2 = DC(2), a3 = DC(3), a4 = DC(4), a5 = DC(5), a6 = DC(6), a7 = DC(7);
            const R a8 = DC(8), a9 = DC(9), a10 = DC(10), a11 = DC(11), a12 = DC(12), a13 = DC(13), a14 = DC(14);
            col[0] = sop6(a0, e00, a1, e01, a2, e02, a3, e11, a4, e12, a5, e22);
            col[1] = sop6(a1, e00, a6, e01, a7, e02, a8, e11, a9, e12, a10, e22);
            col[2] = sop6(a2, e00, a7, e01, a11, e02, a12, e11, a13, e12, a14, e22);
        } else if (d == 1) {  // (s01, s11, s12)
            const R a1 = DC(1), a3 = DC(3), a4 = DC(4), a6 = DC(6), a7 = DC(7), a8 = DC(8), a9 = DC(9), a10 = DC(10);
            const R a12 = DC(12), a13 = DC(13), a15 = DC(15), a16 = DC(16), a17 = DC(17), a18 = DC(18), a19 = DC(19);
            col[0] = sop6(a1, e00, a6, e01, a7, e02, a8, e11, a9, e12, a10, e22);
            col[1] = sop6(a3, e00, a8, e01, a12, e02, a15, e11, a16, e12, a17, e22);
            col[2] = sop6(a4, e00, a9, e01, a13, e02, a16, e11, a18, e12, a19, e22);
        } else {  // (s20, s12, s22)
            const R a2 = DC(2), a4 = DC(4), a5 = DC(5), a7 = DC(7), a9 = DC(9), a10 = DC(10), a11 = DC(11), a12 = DC(12);
            const R a13 = DC(13), a14 = DC(14), a16 = DC(16), a17 = DC(17), a18 = DC(18), a19 = DC(19), a20 = DC(20);
            col[0] = sop6(a2, e00, a7, e01, a11, e02, a12, e11, a13, e12, a14, e22);
            col[1] = sop6(a4, e00, a9, e01, a13, e02, a16, e11, a18, e12, a19, e22);
            col[2] = sop6(a5, e00, a10, e01, a14, e02, a17, e11, a19, e12, a20, e22);
        }
    } else if (M == MAJOR) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            R v = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int l = 0; l < 3; ++l) v += DC(major_slot(3 * r + d, 3 * k + l)) * g[k][l];
            col[r] = v;
        }
    } else if (M == ISO) {
        const R dl = DC(0), dm = DC(1);
        const R tr = dl * (g[0][0] + g[1][1] + g[2][2]);
        if (d == 0) {
            col[0] = tr + R(2) * dm * g[0][0];
            col[1] = dm * (g[0][1] + g[1][0]);
            col[2] = dm * (g[2][0] + g[0][2]);
        } else if (d == 1) {
            col[0] = dm * (g[0][1] + g[1][0]);
            col[1] = tr + R(2) * dm * g[1][1];
            col[2] = dm * (g[1][2] + g[2][1]);
        } else {
            col[0] = dm * (g[2][0] + g[0][2]);
            col[1] = dm * (g[1][2] + g[2][1]);
            col[2] = tr + R(2) * dm * g[2][2];
        }
    } else {
#pragma unroll
        for (int r = 0; r < 3; ++r) col[r] = DC(3 * r + d) * g[r][d];
    }
#undef DC
}

// Column d of (dC : grad u) with the slot differences supplied by a callable dC(q); the same
// 15-of-21 slot selection as gradC_col.
template <int M, class R, class F>
__device__ __forceinline__ void gradC_col_f(F&& dC, const R g[3][3], int d, R col[3]) {
    if (M == MM) {
        const R e00 = g[0][0], e11 = g[1][1], e22 = g[2][2];
        const R e01 = add2(g[0][1], g[1][0]), e02 = add2(g[0][2], g[2][0]), e12 = add2(g[1][2], g[2][1]);
        if (d == 0) {
            const R a0 = dC(0), a1 = dC(1), a2 = dC(2), a3 = dC(3), a4 = dC(4), a5 = dC(5), a6 = dC(6), a7 = dC(7);
            const R a8 = dC(8), a9 = dC(9), a10 = dC(10), a11 = dC(11), a12 = dC(12), a13 = dC(13), a14 = dC(14);
            col[0] = sop6(a0, e00, a1, e01, a2, e02, a3, e11, a4, e12, a5, e22);
            col[1] = sop6(a1, e00, a6, e01, a7, e02, a8, e11, a9, e12, a10, e22);
            col[2] = sop6(a2, e00, a7, e01, a11, e02, a12, e11, a13, e12, a14, e22);
        } else if (d == 1) {
            const R a1 = dC(1), a3 = dC(3), a4 = dC(4), a6 = dC(6), a7 = dC(7), a8 = dC(8), a9 = dC(9), a10 = dC(10);
            const R a12 = dC(12), a13 = dC(13), a15 = dC(15), a16 = dC(16), a17 = dC(17), a18 = dC(18), a19 = dC(19);
            col[0] = sop6(a1, e00, a6, e01, a7, e02, a8, e11, a9, e12, a10, e22);
            col[1] = sop6(a3, e00, a8, e01, a12, e02, a15, e11, a16, e12, a17, e22);
            col[2] = sop6(a4, e00, a9, e01, a13, e02, a16, e11, a18, e12, a19, e22);
        } else {
            const R a2 = dC(2), a4 = dC(4), a5 = dC(5), a7 = dC(7), a9 = dC(9), a10 = dC(10), a11 = dC(11), a12 = dC(12);
            const R a13 = dC(13), a14 = dC(14), a16 = dC(16), a17 = dC(17), a18 = dC(18), a19 = dC(19), a20 = dC(20);
            col[0] = sop6(a2, e00, a7, e01, a11, e02, a12, e11, a13, e12, a14, e22);
            col[1] = sop6(a4, e00, a9, e01, a13, e02, a16, e11, a18, e12, a19, e22);
            col[2] = sop6(a5, e00, a10, e01, a14, e02, a17, e11, a19, e12, a20, e22);
        }
    } else if (M == MAJOR) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            R v = R(0);
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int l = 0; l < 3; ++l) v += dC(major_slot(3 * r + d, 3 * k + l)) * g[k][l];
            col[r] = v;
        }
    } else if (M == ISO) {
        const R dl = dC(0), dm = dC(1);
        const R tr = dl * (g[0][0] + g[1][1] + g[2][2]);
        if (d == 0) {
            col[0] = tr + R(2) * dm * g[0][0];
            col[1] = dm * (g[0][1] + g[1][0]);
            col[2] = dm * (g[2][0] + g[0][2]);
        } else if (d == 1) {
            col[0] = dm * (g[0][1] + g[1][0]);
            col[1] = tr + R(2) * dm * g[1][1];
            col[2] = dm * (g[1][2] + g[2][1]);
        } else {
            col[0] = dm * (g[2][0] + g[0][2]);
            col[1] = dm * (g[1][2] + g[2][1]);
            col[2] = tr + R(2) * dm * g[2][2];
        }
    } else {
#pragma unroll
        for (int r = 0; r < 3; ++r) col[r] = dC(3 * r + d) * g[r][d];
    }
}

// Slots that the z column of the grad C term reads (gradC_col, d = 2), in order.
template <int M> struct ZSlots;
template <> struct ZSlots<MM> {
    static constexpr int n = 15;
    __device__ static constexpr int at(int s) {
        return s < 1 ? 2 : s < 2 ? 4 : s < 3 ? 5 : s < 4 ? 7 : s < 5 ? 9 : s < 6 ? 10 : s < 7 ? 11 : s < 8 ? 12
             : s < 9 ? 13 : s < 10 ? 14 : s < 11 ? 16 : s < 12 ? 17 : s < 13 ? 18 : s < 14 ? 19 : 20;
    }
};
template <> struct ZSlots<ISO> {
    static constexpr int n = 2;
    __device__ static constexpr int at(int s) { return s; }
};
template <> struct ZSlots<DIAG> {
    static constexpr int n = 3;
    __device__ static constexpr int at(int s) { return 3 * s + 2; }
};

// position of slot q in the ZSlots list (-1 if absent)
template <int M>
__device__ __forceinline__ constexpr int zslot_index(int q) {
    for (int s = 0; s < ZSlots<M>::n; ++s)
        if (ZSlots<M>::at(s) == q) return s;
    return -1;
}

// ------------------------------------------------------------------ the operator at one node
// f = A u at node (i,j,k): boundary rows through the BC table, interior rows
// C : grad grad u + sum_d (d_d C : grad u) e_d  (src/Operator/Elastic.cpp:174-258).
// u and C are read through views whose strides may differ.  LDG = false when C lives in
// shared memory.
template <int M, class R, bool LDG = true>
__device__ __forceinline__ void apply_node(const Geo& g, const SCoef<R>& K, const BCP& bc, bool uniform,
                                           const R* __restrict__ C, long long cs, long long cc,
                                           long long csy, long long csz, const R* __restrict__ U,
                                           long long usc, long long uc, long long usy, long long usz, int i, int j,
                                           int k, R f[3]) {
    constexpr int NC = NCoef<M>::value;
    R nrm[3];
    const int face = classify<R>(g, i, j, k, nrm);
    if (face >= 0) {
        // one-sided first derivatives: Hi stencil on the lo face, Lo on the hi face
        const int ci[3] = {i, j, k};
        const long long os[3] = {1, usy, usz};
        R gu[3][3], u[3];
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const R* up = U + p * usc + uc;
            u[p] = up[0];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const long long o = os[d];
                if (ci[d] == g.dlo[d]) gu[p][d] = (up[o] - up[0]) * K.id[d];
                else if (ci[d] == g.dhi[d]) gu[p][d] = (up[0] - up[-o]) * K.id[d];
                else gu[p][d] = (up[o] - up[-o]) * K.h[d];
            }
        }
        const unsigned char* t = bc.t[face];
        R s[3][3];
        bool need_s = (t[0] == TRAC) || (t[1] == TRAC) || (t[2] == TRAC);
        if (need_s) {
            R a[NC];
#pragma unroll
            for (int q = 0; q < NC; ++q) a[q] = ldv<LDG>(C + q * cs + cc);
            stress_of<M, R>(a, gu, s);
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            R v = R(0);
            if (t[r] == DISP) v = u[r];
            else if (t[r] == TRAC) v = s[r][0] * nrm[0] + s[r][1] * nrm[1] + s[r][2] * nrm[2];
            else if (t[r] == NEUMANN) v = gu[r][0] * nrm[0] + gu[r][1] * nrm[1] + gu[r][2] * nrm[2];
            f[r] = v;
        }
        return;
    }
    R gu[3][3], b[3][3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const R* up = U + p * usc + uc;
        const R c0 = up[0];
        const R xm = up[-1], xp = up[1], ym = up[-usy], yp = up[usy], zm = up[-usz], zp = up[usz];
        gu[p][0] = (xp - xm) * K.h[0];
        gu[p][1] = (yp - ym) * K.h[1];
        gu[p][2] = (zp - zm) * K.h[2];
        b[p][0][0] = (xp - R(2) * c0 + xm) * K.i2[0];
        b[p][1][1] = (yp - R(2) * c0 + ym) * K.i2[1];
        b[p][2][2] = (zp - R(2) * c0 + zm) * K.i2[2];
        b[p][0][1] = (up[1 + usy] + up[-1 - usy] - up[1 - usy] - up[-1 + usy]) * K.m01;
        b[p][0][2] = (up[1 + usz] + up[-1 - usz] - up[1 - usz] - up[-1 + usz]) * K.m02;
        b[p][1][2] = (up[usy + usz] + up[-usy - usz] - up[usy - usz] - up[-usy + usz]) * K.m12;
        b[p][1][0] = b[p][0][1];
        b[p][2][0] = b[p][0][2];
        b[p][2][1] = b[p][1][2];
    }
    {
        R a[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) a[q] = ldv<LDG>(C + q * cs + cc);
        div_of<M, R>(a, b, f);
    }
    if (!uniform) {
        R c0[3], c1[3], c2[3];
        gradC_col<M, R, LDG>(C, cs, cc, 1, gu, 0, c0);
        gradC_col<M, R, LDG>(C, cs, cc, csy, gu, 1, c1);
        gradC_col<M, R, LDG>(C, cs, cc, csz, gu, 2, c2);
#pragma unroll
        for (int r = 0; r < 3; ++r) f[r] = gradc_add(f[r], c0[r], c1[r], c2[r], K.h);
    }
}

// apply_node for a stiffness given as a grain id per node (gid, strides gsy, gsz, node index gc)
// and a per-grain coefficient table (tab[g * ncoef + q]): the same arithmetic on the same values.
// A direction whose two neighbours lie in one grain has an exactly zero stiffness difference; its
// grad C column is zero and its table reads are skipped.
template <int M, class R>
__device__ __forceinline__ void apply_node_grains(const Geo& g, const SCoef<R>& K, const BCP& bc, bool uniform,
                                                  const unsigned short* __restrict__ gid, long long gc,
                                                  long long gsy, long long gsz, const R* __restrict__ tab,
                                                  const R* __restrict__ U, long long usc, long long uc, long long usy,
                                                  long long usz, int i, int j, int k, R f[3]) {
    constexpr int NC = NCoef<M>::value;
    const R* a0 = tab + (int)__ldg(gid + gc) * NC;
    R nrm[3];
    const int face = classify<R>(g, i, j, k, nrm);
    if (face >= 0) {
        const int ci[3] = {i, j, k};
        const long long os[3] = {1, usy, usz};
        R gu[3][3], u[3];
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const R* up = U + p * usc + uc;
            u[p] = up[0];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const long long o = os[d];
                if (ci[d] == g.dlo[d]) gu[p][d] = (up[o] - up[0]) * K.id[d];
                else if (ci[d] == g.dhi[d]) gu[p][d] = (up[0] - up[-o]) * K.id[d];
                else gu[p][d] = (up[o] - up[-o]) * K.h[d];
            }
        }
        const unsigned char* t = bc.t[face];
        R s[3][3];
        bool need_s = (t[0] == TRAC) || (t[1] == TRAC) || (t[2] == TRAC);
        if (need_s) {
            R a[NC];
#pragma unroll
            for (int q = 0; q < NC; ++q) a[q] = __ldg(a0 + q);
            stress_of<M, R>(a, gu, s);
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            R v = R(0);
            if (t[r] == DISP) v = u[r];
            else if (t[r] == TRAC) v = s[r][0] * nrm[0] + s[r][1] * nrm[1] + s[r][2] * nrm[2];
            else if (t[r] == NEUMANN) v = gu[r][0] * nrm[0] + gu[r][1] * nrm[1] + gu[r][2] * nrm[2];
            f[r] = v;
        }
        return;
    }
    R gu[3][3], b[3][3][3];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const R* up = U + p * usc + uc;
        const R c0 = up[0];
        const R xm = up[-1], xp = up[1], ym = up[-usy], yp = up[usy], zm = up[-usz], zp = up[usz];
        gu[p][0] = (xp - xm) * K.h[0];
        gu[p][1] = (yp - ym) * K.h[1];
        gu[p][2] = (zp - zm) * K.h[2];
        b[p][0][0] = (xp - R(2) * c0 + xm) * K.i2[0];
        b[p][1][1] = (yp - R(2) * c0 + ym) * K.i2[1];
        b[p][2][2] = (zp - R(2) * c0 + zm) * K.i2[2];
        b[p][0][1] = (up[1 + usy] + up[-1 - usy] - up[1 - usy] - up[-1 + usy]) * K.m01;
        b[p][0][2] = (up[1 + usz] + up[-1 - usz] - up[1 - usz] - up[-1 + usz]) * K.m02;
        b[p][1][2] = (up[usy + usz] + up[-usy - usz] - up[usy - usz] - up[-usy + usz]) * K.m12;
        b[p][1][0] = b[p][0][1];
        b[p][2][0] = b[p][0][2];
        b[p][2][1] = b[p][1][2];
    }
    {
        R a[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) a[q] = __ldg(a0 + q);
        div_of<M, R>(a, b, f);
    }
    if (!uniform) {
        const long long go[3] = {1, gsy, gsz};
        R col[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int gp = __ldg(gid + gc + go[d]), gm = __ldg(gid + gc - go[d]);
            if (gp == gm) {
                col[d][0] = col[d][1] = col[d][2] = R(0);
            } else {
                const R* cp = tab + gp * NC;
                const R* cm = tab + gm * NC;
                gradC_col_f<M, R>([&](int q) { return __ldg(cp + q) - __ldg(cm + q); }, gu, d, col[d]);
            }
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) f[r] = gradc_add(f[r], col[0][r], col[1][r], col[2][r], K.h);
    }
}

}  // namespace ae
