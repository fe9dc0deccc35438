// CPU FP64 restatement of the reference's nodal elastic operator path and of the
// AMReX MLMG cycle around it.  TEST INFRASTRUCTURE ONLY: the parity reference for the
// CUDA library, loaded by tests/, the smoke check and bench.py's cpu_baseline leg.
//
// Every function cites the reference lines it restates.  Arithmetic follows the
// reference's expression order; the build uses -ffp-contract=off so that no
// multiply-add is fused behind the source's back.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- boxes and fields
struct Box {
    int lo[3], hi[3];
};
inline Box grow(Box b, int g) {
    for (int d = 0; d < 3; ++d) { b.lo[d] -= g; b.hi[d] += g; }
    return b;
}
inline Box isect(const Box& a, const Box& b) {
    Box r;
    for (int d = 0; d < 3; ++d) { r.lo[d] = std::max(a.lo[d], b.lo[d]); r.hi[d] = std::min(a.hi[d], b.hi[d]); }
    return r;
}
inline bool empty(const Box& b) {
    return b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1] || b.hi[2] < b.lo[2];
}

struct Lev {
    Box dom, valid, store;
    double dx[3];
    long sx, sy, sz;  // strides of i, j, k
    long nn;          // nodes stored (component stride)
    explicit Lev(const orc_level& L) {
        for (int d = 0; d < 3; ++d) {
            dom.lo[d] = L.dom_lo[d]; dom.hi[d] = L.dom_hi[d];
            valid.lo[d] = L.lo[d]; valid.hi[d] = L.hi[d];
            dx[d] = L.dx[d];
        }
        store = grow(valid, L.ng);
        sx = 1;
        sy = store.hi[0] - store.lo[0] + 1;
        sz = sy * (store.hi[1] - store.lo[1] + 1);
        nn = sz * (store.hi[2] - store.lo[2] + 1);
    }
    long at(int i, int j, int k) const {
        return (long)(i - store.lo[0]) + (long)(j - store.lo[1]) * sy + (long)(k - store.lo[2]) * sz;
    }
    long stride(int d) const { return d == 0 ? sx : (d == 1 ? sy : sz); }
};

template <class F>
void for_box(const Box& b, F&& fn) {
    if (empty(b)) return;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = b.lo[2]; k <= b.hi[2]; ++k)
        for (int j = b.lo[1]; j <= b.hi[1]; ++j)
            for (int i = b.lo[0]; i <= b.hi[0]; ++i) fn(i, j, k);
}

// ---------------------------------------------------------------- Numeric::Stencil
// src/Numeric/Stencil.H:12-34 (GetStencil: Hi at the lo face, Lo at the hi face)
enum { ST_LO = 0, ST_HI = 1, ST_CEN = 2 };
inline void get_stencil(const Lev& L, int i, int j, int k, int st[3]) {
    const int c[3] = {i, j, k};
    for (int d = 0; d < 3; ++d)
        st[d] = (c[d] == L.dom.lo[d]) ? ST_HI : (c[d] == L.dom.hi[d]) ? ST_LO : ST_CEN;
}
// src/Numeric/Stencil.H:44-102 (first derivative, one-sided first order on the boundary)
inline double D1(const double* f, long o, double dx, int st) {
    if (st == ST_LO) return (f[0] - f[-o]) / dx;
    if (st == ST_HI) return (f[o] - f[0]) / dx;
    return (f[o] - f[-o]) * 0.5 / dx;
}
// src/Numeric/Stencil.H:108-142
inline double D2(const double* f, long o, double dx) { return (f[o] - 2.0 * f[0] + f[-o]) / dx / dx; }
// src/Numeric/Stencil.H:144-176
inline double Dmix(const double* f, long oa, long ob, double dxa, double dxb) {
    return 0.25 * (f[oa + ob] + f[-oa - ob] - f[oa - ob] - f[-oa + ob]) / (dxa * dxb);
}

// max(m, |v|) for residual max-norms; a NaN makes the norm infinite (std::max alone would drop
// it and report a diverged solve as converged)
inline double amax(double m, double v) {
    const double a = std::fabs(v);
    return (a != a) ? INFINITY : std::max(m, a);
}

// ---------------------------------------------------------------- Set::Matrix4 contractions
constexpr int kMaxCoef = 45;  // the largest kind: the Sym::Major tangent of a finite-kinematics model
int ncoef_of(int model) {
    return model == ORC_ISOTROPIC ? 2 : model == ORC_MAJORMINOR ? 21 : model == ORC_MAJOR ? 45 : 9;
}

// src/Set/Matrix4_MajorMinor.H:253-269 (stress of a 21-coefficient tensor)
inline void stress_mm(const double* a, const double g[3][3], double s[3][3]) {
    const double e01 = g[0][1] + g[1][0], e02 = g[0][2] + g[2][0], e12 = g[1][2] + g[2][1];
    double r00 = 0, r11 = 0, r22 = 0, r12 = 0, r20 = 0, r01 = 0;
    r00 += a[0] * g[0][0] + a[1] * e01 + a[2] * e02 + a[3] * g[1][1] + a[4] * e12 + a[5] * g[2][2];
    r11 += a[3] * g[0][0] + a[8] * e01 + a[12] * e02 + a[15] * g[1][1] + a[16] * e12 + a[17] * g[2][2];
    r22 += a[5] * g[0][0] + a[10] * e01 + a[14] * e02 + a[17] * g[1][1] + a[19] * e12 + a[20] * g[2][2];
    r12 += a[4] * g[0][0] + a[9] * e01 + a[13] * e02 + a[16] * g[1][1] + a[18] * e12 + a[19] * g[2][2];
    r20 += a[2] * g[0][0] + a[7] * e01 + a[11] * e02 + a[12] * g[1][1] + a[13] * e12 + a[14] * g[2][2];
    r01 += a[1] * g[0][0] + a[6] * e01 + a[7] * e02 + a[8] * g[1][1] + a[9] * e12 + a[10] * g[2][2];
    s[0][0] = r00; s[1][1] = r11; s[2][2] = r22;
    s[1][2] = r12; s[2][1] = r12;
    s[2][0] = r20; s[0][2] = r20;
    s[0][1] = r01; s[1][0] = r01;
}
// src/Set/Matrix4_MajorMinor.H:287-345 (divergence term C_ijkl u_{k,lj}); b[k][l][j] = u_{k,lj}
inline void div_mm(const double* a, const double b[3][3][3], double f[3]) {
#define B(p, q, r) b[p][q][r]
    double r0 = 0, r1 = 0, r2 = 0;
    r0 += a[0] * B(0, 0, 0) + a[1] * (B(0, 1, 0) + B(1, 0, 0) + B(0, 0, 1)) +
          a[2] * (B(0, 2, 0) + B(2, 0, 0) + B(0, 0, 2)) + a[3] * B(1, 1, 0) + a[4] * (B(1, 2, 0) + B(2, 1, 0)) +
          a[5] * B(2, 2, 0) + a[6] * (B(0, 1, 1) + B(1, 0, 1)) +
          a[7] * (B(0, 2, 1) + B(2, 0, 1) + B(0, 1, 2) + B(1, 0, 2)) + a[8] * B(1, 1, 1) +
          a[9] * (B(1, 2, 1) + B(2, 1, 1)) + a[10] * B(2, 2, 1) + a[11] * (B(0, 2, 2) + B(2, 0, 2)) +
          a[12] * B(1, 1, 2) + a[13] * (B(1, 2, 2) + B(2, 1, 2)) + a[14] * B(2, 2, 2);
    r1 += a[1] * B(0, 0, 0) + a[4] * B(0, 0, 2) + a[3] * B(0, 0, 1) + a[6] * (B(0, 1, 0) + B(1, 0, 0)) +
          a[7] * (B(0, 2, 0) + B(2, 0, 0)) + a[8] * (B(1, 1, 0) + B(0, 1, 1) + B(1, 0, 1)) +
          a[9] * (B(1, 2, 0) + B(2, 1, 0) + B(0, 1, 2) + B(1, 0, 2)) + a[10] * B(2, 2, 0) +
          a[12] * (B(0, 2, 1) + B(2, 0, 1)) + a[13] * (B(0, 2, 2) + B(2, 0, 2)) + a[15] * B(1, 1, 1) +
          a[16] * (B(1, 2, 1) + B(2, 1, 1) + B(1, 1, 2)) + a[17] * B(2, 2, 1) + a[18] * (B(1, 2, 2) + B(2, 1, 2)) +
          a[19] * B(2, 2, 2);
    r2 += a[2] * B(0, 0, 0) + a[4] * B(0, 0, 1) + a[5] * B(0, 0, 2) + a[7] * (B(0, 1, 0) + B(1, 0, 0)) +
          a[9] * (B(0, 1, 1) + B(1, 0, 1)) + a[10] * (B(0, 1, 2) + B(1, 0, 2)) +
          a[11] * (B(0, 2, 0) + B(2, 0, 0)) + a[12] * B(1, 1, 0) +
          a[13] * (B(1, 2, 0) + B(2, 1, 0) + B(0, 2, 1) + B(2, 0, 1)) +
          a[14] * (B(2, 2, 0) + B(0, 2, 2) + B(2, 0, 2)) + a[16] * B(1, 1, 1) + a[17] * B(1, 1, 2) +
          a[18] * (B(1, 2, 1) + B(2, 1, 1)) + a[19] * (B(2, 2, 1) + B(1, 2, 2) + B(2, 1, 2)) + a[20] * B(2, 2, 2);
#undef B
    f[0] = r0; f[1] = r1; f[2] = r2;
}
// src/Set/Matrix4_Isotropic.H:71-76; coefficients (lambda, mu)
inline void stress_iso(const double* a, const double g[3][3], double s[3][3]) {
    const double lambda = a[0], mu = a[1];
    s[0][0] = (lambda + 2. * mu) * g[0][0] + lambda * g[1][1] + lambda * g[2][2];
    s[1][1] = lambda * g[0][0] + (lambda + 2. * mu) * g[1][1] + lambda * g[2][2];
    s[2][2] = lambda * g[0][0] + lambda * g[1][1] + (lambda + 2. * mu) * g[2][2];
    s[1][2] = mu * (g[1][2] + g[2][1]); s[2][1] = s[1][2];
    s[2][0] = mu * (g[2][0] + g[0][2]); s[0][2] = s[2][0];
    s[0][1] = mu * (g[0][1] + g[1][0]); s[1][0] = s[0][1];
}
// src/Set/Matrix4_Isotropic.H:82-91
inline void div_iso(const double* a, const double b[3][3][3], double f[3]) {
    const double lambda = a[0], mu = a[1];
    for (int i = 0; i < 3; ++i) {
        double r = 0;
        for (int j = 0; j < 3; ++j) r += mu * (b[i][j][j] + b[j][i][j]) + lambda * b[j][j][i];
        f[i] = r;
    }
}
// src/Set/Matrix4_Diagonal.H:48-74; coefficients A(i,j) row-major
inline void stress_diag(const double* a, const double g[3][3], double s[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) s[i][j] = a[3 * i + j] * g[i][j];
}
inline void div_diag(const double* a, const double b[3][3][3], double f[3]) {
    for (int i = 0; i < 3; ++i) {
        double r = 0;
        for (int j = 0; j < 3; ++j) r += a[3 * i + j] * b[i][j][j];
        f[i] = r;
    }
}
// Set::Matrix4<3, Sym::Major> (src/Set/Matrix4_Major.H:198-300): the 9 x 9 matrix
// A(3i+j, 3k+l) = C_ijkl is symmetric; its upper triangle is stored row by row (45 slots).
inline int major_slot(int I, int K) {
    if (I > K) { const int t = I; I = K; K = t; }
    return I * 9 - I * (I - 1) / 2 + (K - I);
}
// src/Set/Matrix4_Major.H:399-413: sigma_ij = sum_kl C_ijkl g_kl, summed in (k, l) order
inline void stress_major(const double* a, const double g[3][3], double s[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double r = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) r += a[major_slot(3 * i + j, 3 * k + l)] * g[k][l];
            s[i][j] = r;
        }
}
// src/Set/Matrix4_Major.H:415-428: f_i = sum_{j,k,l} C_ijkl b[k][l][j], b[k][l][j] = u_{k,lj}
inline void div_major(const double* a, const double b[3][3][3], double f[3]) {
    for (int i = 0; i < 3; ++i) {
        double r = 0.0;
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) r += a[major_slot(3 * i + j, 3 * k + l)] * b[k][l][j];
        f[i] = r;
    }
}
inline void stress_of(int model, const double* a, const double g[3][3], double s[3][3]) {
    if (model == ORC_ISOTROPIC) stress_iso(a, g, s);
    else if (model == ORC_MAJORMINOR) stress_mm(a, g, s);
    else if (model == ORC_MAJOR) stress_major(a, g, s);
    else stress_diag(a, g, s);
}
inline void div_of(int model, const double* a, const double b[3][3][3], double f[3]) {
    if (model == ORC_ISOTROPIC) div_iso(a, b, f);
    else if (model == ORC_MAJORMINOR) div_mm(a, b, f);
    else if (model == ORC_MAJOR) div_major(a, b, f);
    else div_diag(a, b, f);
}

// ---------------------------------------------------------------- BC::Operator::Elastic
// src/BC/Operator/Elastic.H:33-41 face numbering; :218-219 truncated normals; :222-284 classification
const double SQRT3INV = 0.57735026919;
const double SQRT2INV = 0.70710678118;
inline int classify(const Box& dom, int i, int j, int k, double n[3]) {
    const int c[3] = {i, j, k};
    int s[3], cnt = 0;
    for (int d = 0; d < 3; ++d) {
        s[d] = (c[d] == dom.lo[d]) ? -1 : (c[d] == dom.hi[d]) ? 1 : 0;
        cnt += s[d] != 0;
    }
    if (cnt == 0) return -1;
    const double w = cnt == 3 ? SQRT3INV : cnt == 2 ? SQRT2INV : 1.0;
    for (int d = 0; d < 3; ++d) n[d] = s[d] == 0 ? 0.0 : (s[d] > 0 ? w : -w);
    if (cnt == 3) return 18 + 4 * (s[0] > 0) + 2 * (s[1] > 0) + (s[2] > 0);
    if (cnt == 2) {
        if (s[0] == 0) return 6 + 2 * (s[1] > 0) + (s[2] > 0);
        if (s[1] == 0) return 10 + 2 * (s[2] > 0) + (s[0] > 0);
        return 14 + 2 * (s[0] > 0) + (s[1] > 0);
    }
    if (s[0]) return s[0] < 0 ? 0 : 3;
    if (s[1]) return s[1] < 0 ? 1 : 4;
    return s[2] < 0 ? 2 : 5;
}
// src/BC/Operator/Elastic.H:286-303
inline void bc_set(const int* type3, const double u[3], const double g[3][3], const double s[3][3],
                   const double n[3], double f[3]) {
    for (int i = 0; i < 3; ++i) {
        f[i] = 0.0;
        if (type3[i] == ORC_DISP) f[i] = u[i];
        else if (type3[i] == ORC_TRAC) f[i] = s[i][0] * n[0] + s[i][1] * n[1] + s[i][2] * n[2];
        else if (type3[i] == ORC_NEUMANN) f[i] = g[i][0] * n[0] + g[i][1] * n[1] + g[i][2] * n[2];
    }
}

// ---------------------------------------------------------------- Elastic<T>::Fapply (per node)
// src/Operator/Elastic.cpp:174-258
inline void fapply_node(const Lev& L, int model, const double* C, const int* bctype, int uniform,
                        const double* U, int i, int j, int k, double f[3]) {
    const long c = L.at(i, j, k), nn = L.nn;
    const int nc = ncoef_of(model);
    int st[3];
    get_stencil(L, i, j, k, st);
    double a[kMaxCoef];
    for (int q = 0; q < nc; ++q) a[q] = C[q * nn + c];
    double u[3], g[3][3];
    for (int p = 0; p < 3; ++p) {
        const double* up = U + p * nn + c;
        u[p] = up[0];
        for (int d = 0; d < 3; ++d) g[p][d] = D1(up, L.stride(d), L.dx[d], st[d]);
    }
    double s[3][3];
    stress_of(model, a, g, s);  // computed at every node, used on the boundary (Elastic.cpp:201)
    double nrm[3];
    const int face = classify(L.dom, i, j, k, nrm);
    if (face >= 0) {
        bc_set(bctype + 3 * face, u, g, s, nrm, f);
        return;
    }
    double b[3][3][3];
    for (int p = 0; p < 3; ++p) {
        const double* up = U + p * nn + c;
        b[p][0][0] = D2(up, L.sx, L.dx[0]);
        b[p][1][1] = D2(up, L.sy, L.dx[1]);
        b[p][2][2] = D2(up, L.sz, L.dx[2]);
        b[p][0][1] = Dmix(up, L.sx, L.sy, L.dx[0], L.dx[1]);
        b[p][1][0] = b[p][0][1];
        b[p][0][2] = Dmix(up, L.sx, L.sz, L.dx[0], L.dx[2]);
        b[p][1][2] = Dmix(up, L.sy, L.sz, L.dx[1], L.dx[2]);
        b[p][2][0] = b[p][0][2];
        b[p][2][1] = b[p][1][2];
    }
    div_of(model, a, b, f);
    if (!uniform) {
        // (Stencil<T,..>::D(C)) (gradu) .col(d), Elastic.cpp:249-254
        double col[3][3];
        for (int d = 0; d < 3; ++d) {
            const long o = L.stride(d);
            double cg[kMaxCoef];
            for (int q = 0; q < nc; ++q) {
                const double* cq = C + q * nn + c;
                if (st[d] == ST_LO) cg[q] = (cq[0] - cq[-o]) / L.dx[d];
                else if (st[d] == ST_HI) cg[q] = (cq[o] - cq[0]) / L.dx[d];
                else cg[q] = (cq[o] - cq[-o]) * 0.5 / L.dx[d];
            }
            double sd[3][3];
            stress_of(model, cg, g, sd);
            for (int r = 0; r < 3; ++r) col[d][r] = sd[r][d];
        }
        for (int r = 0; r < 3; ++r) f[r] += (col[0][r] + col[1][r]) + col[2][r];
    }
}

Box apply_region(const Lev& L) { return isect(grow(L.valid, 1), isect(L.dom, L.store)); }

void fapply(const Lev& L, int model, const double* C, const int* bctype, int uniform, const double* U, double* F) {
    const Box r = apply_region(L);
    for_box(r, [&](int i, int j, int k) {
        double f[3];
        fapply_node(L, model, C, bctype, uniform, U, i, j, k, f);
        const long c = L.at(i, j, k);
        for (int p = 0; p < 3; ++p) F[p * L.nn + c] = f[p];
    });
}

// ---------------------------------------------------------------- Elastic<T>::Diagonal
// src/Operator/Elastic.cpp:264-352 (analytic self-coefficient, over valid grown 1 ∩ domain)
void diagonal(const Lev& L, int model, const double* C, const int* bctype, double* D) {
    const Box r = apply_region(L);
    const int nc = ncoef_of(model);
    for_box(r, [&](int i, int j, int k) {
        const long c = L.at(i, j, k), nn = L.nn;
        int st[3];
        get_stencil(L, i, j, k, st);
        const bool xmin = i == L.dom.lo[0], ymin = j == L.dom.lo[1], zmin = k == L.dom.lo[2];
        const bool xmax = i == L.dom.hi[0], ymax = j == L.dom.hi[1], zmax = k == L.dom.hi[2];
        const bool mn[3] = {xmin, ymin, zmin}, mx[3] = {xmax, ymax, zmax};
        double a[kMaxCoef];
        for (int q = 0; q < nc; ++q) a[q] = C[q * nn + c];
        double nrm[3];
        const int face = classify(L.dom, i, j, k, nrm);
        for (int p = 0; p < 3; ++p) {
            double g[3][3], b[3][3][3];
            for (int q = 0; q < 3; ++q) {
                for (int d = 0; d < 3; ++d)
                    g[q][d] = ((!mx[d] ? 0.0 : (p == q ? 1.0 : 0.0)) - (!mn[d] ? 0.0 : (p == q ? 1.0 : 0.0))) /
                              ((mn[d] || mx[d] ? 1.0 : 2.0) * L.dx[d]);
                for (int l = 0; l < 3; ++l)
                    for (int jj = 0; jj < 3; ++jj) b[q][l][jj] = 0.0;
                for (int d = 0; d < 3; ++d) b[q][d][d] = (p == q ? -2.0 : 0.0) / L.dx[d] / L.dx[d];
            }
            double s[3][3];
            stress_of(model, a, g, s);
            double val = 0.0;
            if (face >= 0) {
                double u[3] = {0, 0, 0}, f[3];
                u[p] = 1.0;
                bc_set(bctype + 3 * face, u, g, s, nrm, f);
                val = f[p];
            } else {
                double f[3], col[3][3];
                div_of(model, a, b, f);
                for (int d = 0; d < 3; ++d) {
                    const long o = L.stride(d);
                    double cg[kMaxCoef];
                    for (int q = 0; q < nc; ++q) {
                        const double* cq = C + q * nn + c;
                        cg[q] = (cq[o] - cq[-o]) * 0.5 / L.dx[d];
                    }
                    double sd[3][3];
                    stress_of(model, cg, g, sd);
                    for (int rr = 0; rr < 3; ++rr) col[d][rr] = sd[rr][d];
                }
                val += f[p] + ((col[0][p] + col[1][p]) + col[2][p]);
            }
            D[p * nn + c] = val;
        }
    });
}

// ---------------------------------------------------------------- Operator<Node>::Fsmooth
// src/Operator/Operator.cpp:90-162: damped Jacobi, x = (1-w) x + w (b - (Ax - D x)) / D,
// over the valid box grown by 2 clipped to the domain, outermost ring set to zero.
void fsmooth(const Lev& L, int model, const double* C, const int* bctype, int uniform, const double* D,
             double* X, const double* B, int nsweeps, double omega) {
    std::vector<double> Ax(3 * L.nn, 0.0);
    const Box g2 = isect(grow(L.valid, 2), L.store);
    for (int s = 0; s < nsweeps; ++s) {
        fapply(L, model, C, bctype, uniform, X, Ax.data());
        for (int n = 0; n < 3; ++n) {
            for_box(g2, [&](int i, int j, int k) {
                const int m[3] = {i, j, k};
                for (int d = 0; d < 3; ++d)
                    if (m[d] < L.dom.lo[d] || m[d] > L.dom.hi[d]) return;
                const long c = n * L.nn + L.at(i, j, k);
                for (int d = 0; d < 3; ++d)
                    if (m[d] == L.valid.lo[d] - 2 || m[d] == L.valid.hi[d] + 2) { X[c] = 0.0; return; }
                const double Dx = X[c] * D[c];
                const double Rx = Ax[c] - Dx;
                X[c] = (1. - omega) * X[c] + omega * (B[c] - Rx) / D[c];
            });
        }
    }
}

// ---------------------------------------------------------------- residuals
// src/Operator/Operator.cpp:841-863: r = b - A x (Xpay), inf norm over the valid box
double residual(const Lev& L, int model, const double* C, const int* bctype, int uniform, const double* X,
                const double* B, double* R) {
    fapply(L, model, C, bctype, uniform, X, R);
    const Box r = apply_region(L);
    double mx = 0.0;
    for (int n = 0; n < 3; ++n) {
        for_box(r, [&](int i, int j, int k) {
            const long c = n * L.nn + L.at(i, j, k);
            R[c] = B[c] + (-1.0) * R[c];
        });
    }
    const Box v = isect(L.valid, L.dom);
    for (int n = 0; n < 3; ++n)
        for (int k = v.lo[2]; k <= v.hi[2]; ++k)
            for (int j = v.lo[1]; j <= v.hi[1]; ++j)
                for (int i = v.lo[0]; i <= v.hi[0]; ++i) mx = amax(mx, R[n * L.nn + L.at(i, j, k)]);
    return mx;
}

// ---------------------------------------------------------------- restriction / interpolation
// src/Operator/Operator.cpp:486-543 (nodal full weighting, reduced on the domain boundary).
// The same weights restrict the stiffness field, src/Operator/Elastic.cpp:759-803, and the
// fine residual onto covered coarse nodes in reflux, src/Operator/Operator.cpp:776-824.
void restrict_box(const Lev& Lc, const Lev& Lf, int ncomp, double* crse, const double* fine, const Box& bx);
void restrict_(const Lev& Lc, const Lev& Lf, int ncomp, double* crse, const double* fine) {
    restrict_box(Lc, Lf, ncomp, crse, fine, isect(Lc.valid, Lc.dom));
}
void restrict_box(const Lev& Lc, const Lev& Lf, int ncomp, double* crse, const double* fine, const Box& bx) {
    const Box& cd = Lc.dom;
    for (int n = 0; n < ncomp; ++n) {
        for_box(bx, [&](int I, int J, int K) {
            const int i = 2 * I, j = 2 * J, k = 2 * K;
            const double* F0 = fine + n * Lf.nn;
            auto f = [&](int a, int b, int c) { return F0[Lf.at(a, b, c)]; };
            const bool xe = I == cd.lo[0] || I == cd.hi[0];
            const bool ye = J == cd.lo[1] || J == cd.hi[1];
            const bool ze = K == cd.lo[2] || K == cd.hi[2];
            double v;
            if (xe && ye && ze) v = f(i, j, k);
            else if (ye && ze) v = 0.25 * f(i - 1, j, k) + 0.5 * f(i, j, k) + 0.25 * f(i + 1, j, k);
            else if (ze && xe) v = 0.25 * f(i, j - 1, k) + 0.5 * f(i, j, k) + 0.25 * f(i, j + 1, k);
            else if (xe && ye) v = 0.25 * f(i, j, k - 1) + 0.5 * f(i, j, k) + 0.25 * f(i, j, k + 1);
            else if (xe)
                v = (+f(i, j - 1, k - 1) + 2.0 * f(i, j, k - 1) + f(i, j + 1, k - 1) + 2.0 * f(i, j - 1, k) +
                     4.0 * f(i, j, k) + 2.0 * f(i, j + 1, k) + f(i, j - 1, k + 1) + 2.0 * f(i, j, k + 1) +
                     f(i, j + 1, k + 1)) / 16.0;
            else if (ye)
                v = (+f(i - 1, j, k - 1) + 2.0 * f(i - 1, j, k) + f(i - 1, j, k + 1) + 2.0 * f(i, j, k - 1) +
                     4.0 * f(i, j, k) + 2.0 * f(i, j, k + 1) + f(i + 1, j, k - 1) + 2.0 * f(i + 1, j, k) +
                     f(i + 1, j, k + 1)) / 16.0;
            else if (ze)
                v = (+f(i - 1, j - 1, k) + 2.0 * f(i, j - 1, k) + f(i + 1, j - 1, k) + 2.0 * f(i - 1, j, k) +
                     4.0 * f(i, j, k) + 2.0 * f(i + 1, j, k) + f(i - 1, j + 1, k) + 2.0 * f(i, j + 1, k) +
                     f(i + 1, j + 1, k)) / 16.0;
            else
                v = (f(i - 1, j - 1, k - 1) + f(i - 1, j - 1, k + 1) + f(i - 1, j + 1, k - 1) + f(i - 1, j + 1, k + 1) +
                     f(i + 1, j - 1, k - 1) + f(i + 1, j - 1, k + 1) + f(i + 1, j + 1, k - 1) + f(i + 1, j + 1, k + 1)) /
                        64.0 +
                    (f(i, j - 1, k - 1) + f(i, j - 1, k + 1) + f(i, j + 1, k - 1) + f(i, j + 1, k + 1) +
                     f(i - 1, j, k - 1) + f(i + 1, j, k - 1) + f(i - 1, j, k + 1) + f(i + 1, j, k + 1) +
                     f(i - 1, j - 1, k) + f(i - 1, j + 1, k) + f(i + 1, j - 1, k) + f(i + 1, j + 1, k)) /
                        32.0 +
                    (f(i - 1, j, k) + f(i, j - 1, k) + f(i, j, k - 1) + f(i + 1, j, k) + f(i, j + 1, k) +
                     f(i, j, k + 1)) / 16.0 +
                    f(i, j, k) / 8.0;
            crse[n * Lc.nn + Lc.at(I, J, K)] = v;
        });
    }
}

// src/Operator/Operator.cpp:556-624 (trilinear nodal prolongation, added into fine)
void interp_add_box(const Lev& Lf, const Lev& Lc, int ncomp, double* fine, const double* crse, const Box& bx);
void interp_add(const Lev& Lf, const Lev& Lc, int ncomp, double* fine, const double* crse) {
    interp_add_box(Lf, Lc, ncomp, fine, crse, isect(Lf.valid, Lf.dom));
}
void interp_add_box(const Lev& Lf, const Lev& Lc, int ncomp, double* fine, const double* crse, const Box& bx) {
    for (int n = 0; n < ncomp; ++n) {
        for_box(bx, [&](int i, int j, int k) {
            const double* C0 = crse + n * Lc.nn;
            auto c = [&](int a, int b, int d) { return C0[Lc.at(a, b, d)]; };
            const int I = i / 2, J = j / 2, K = k / 2;
            const bool ie = i % 2 == 0, je = j % 2 == 0, ke = k % 2 == 0;
            double v;
            if (ie && je && ke) v = c(I, J, K);
            else if (je && ke) v = 0.5 * (c(I, J, K) + c(I + 1, J, K));
            else if (ke && ie) v = 0.5 * (c(I, J, K) + c(I, J + 1, K));
            else if (ie && je) v = 0.5 * (c(I, J, K) + c(I, J, K + 1));
            else if (ie) v = 0.25 * (c(I, J, K) + c(I, J + 1, K) + c(I, J, K + 1) + c(I, J + 1, K + 1));
            else if (je) v = 0.25 * (c(I, J, K) + c(I, J, K + 1) + c(I + 1, J, K) + c(I + 1, J, K + 1));
            else if (ke) v = 0.25 * (c(I, J, K) + c(I + 1, J, K) + c(I, J + 1, K) + c(I + 1, J + 1, K));
            else
                v = 0.125 * (c(I, J, K) + c(I + 1, J, K) + c(I, J + 1, K) + c(I, J, K + 1) + c(I, J + 1, K + 1) +
                             c(I + 1, J, K + 1) + c(I + 1, J + 1, K) + c(I + 1, J + 1, K + 1));
            fine[n * Lf.nn + Lf.at(i, j, k)] += v;
        });
    }
}

// ---------------------------------------------------------------- MLMG restatement
// AMReX MLMG (tag 20.05) is not part of the reference tree; its cycle is restated from
// the reference's call sites (src/Solver/Nonlocal/Linear.H:23-29,102-112;
// src/Operator/Operator.cpp:90-162,454-624,841-863) and from AMReX's published
// MLMG/MLCGSolver algorithm.  Single AMR level, single box per level.
struct MGLevel {
    orc_level ol;
    Lev* L = nullptr;
    std::vector<double> C, D, res, cor, rescor, corhold;
};

struct Solver {
    int model, nc, uniform;
    const int* bctype;
    orc_opts o;
    std::vector<MGLevel> lv;
    int bottom_fail = 0;

    ~Solver() { for (auto& l : lv) delete l.L; }

    void apply(int m, const double* x, double* out) { fapply(*lv[m].L, model, lv[m].C.data(), bctype, o.uniform, x, out); }
    void smooth(int m, double* x, const double* b) {
        fsmooth(*lv[m].L, model, lv[m].C.data(), bctype, o.uniform, lv[m].D.data(), x, b, o.sweeps, o.omega);
    }
    // rescor = res - A cor
    void res_of_cor(int m) {
        residual(*lv[m].L, model, lv[m].C.data(), bctype, o.uniform, lv[m].cor.data(), lv[m].res.data(),
                 lv[m].rescor.data());
    }
    double dot(int m, const double* a, const double* b) {
        const Lev& L = *lv[m].L;
        double s = 0;
        for (long i = 0; i < 3 * L.nn; ++i) s += a[i] * b[i];
        return s;
    }
    double ninf(int m, const double* a) {
        const Lev& L = *lv[m].L;
        double s = 0;
        for (long i = 0; i < 3 * L.nn; ++i) s = std::max(s, std::fabs(a[i]));
        return s;
    }
    // MLCGSolver::solve_cg / solve_bicgstab restated; returns AMReX status code
    int bottom_krylov(int m, double* sol, const double* rhs) {
        const Lev& L = *lv[m].L;
        const long N = 3 * L.nn;
        const double eps_rel = o.bottom_reltol, eps_abs = -1.0;
        std::vector<double> sorig(sol, sol + N), r(N), tmp(N);
        residual(L, model, lv[m].C.data(), bctype, o.uniform, sol, rhs, r.data());
        std::fill(sol, sol + N, 0.0);
        double rnorm = ninf(m, r.data());
        const double rnorm0 = rnorm;
        int ret = 0;
        if (rnorm0 == 0 || rnorm0 < eps_abs) {
            for (long i = 0; i < N; ++i) sol[i] += sorig[i];
            return 0;
        }
        if (o.bottom == 0) {
            std::vector<double> p(N, 0.0), z(N), q(N);
            double rho_1 = 0;
            for (int iter = 1; iter <= o.bottom_max_iter; ++iter) {
                z = r;
                const double rho = dot(m, z.data(), r.data());
                if (rho == 0) { ret = 1; break; }
                if (iter == 1) p = z;
                else {
                    const double beta = rho / rho_1;
                    for (long i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
                }
                apply(m, p.data(), q.data());
                const double pw = dot(m, p.data(), q.data());
                double alpha;
                if (pw != 0) alpha = rho / pw;
                else { ret = 1; break; }
                for (long i = 0; i < N; ++i) { sol[i] += alpha * p[i]; r[i] += -alpha * q[i]; }
                rnorm = ninf(m, r.data());
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                rho_1 = rho;
            }
        } else {
            std::vector<double> p(N, 0.0), rh(r), v(N, 0.0), t(N);
            double rho_1 = 0, alpha = 0, omega = 0;
            for (int iter = 1; iter <= o.bottom_max_iter; ++iter) {
                const double rho = dot(m, rh.data(), r.data());
                if (rho == 0) { ret = 1; break; }
                if (iter == 1) p = r;
                else {
                    const double beta = (rho / rho_1) * (alpha / omega);
                    for (long i = 0; i < N; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
                }
                apply(m, p.data(), v.data());
                const double rhTv = dot(m, rh.data(), v.data());
                if (rhTv != 0) alpha = rho / rhTv;
                else { ret = 2; break; }
                for (long i = 0; i < N; ++i) { sol[i] += alpha * p[i]; r[i] += -alpha * v[i]; }
                rnorm = ninf(m, r.data());
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                apply(m, r.data(), t.data());
                const double tt = dot(m, t.data(), t.data()), tr = dot(m, t.data(), r.data());
                if (tt != 0) omega = tr / tt;
                else { ret = 3; break; }
                for (long i = 0; i < N; ++i) { sol[i] += omega * r[i]; r[i] += -omega * t[i]; }
                rnorm = ninf(m, r.data());
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                if (omega == 0) { ret = 4; break; }
                rho_1 = rho;
            }
        }
        if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
        if ((ret == 0 || ret == 8) && rnorm < rnorm0) {
            for (long i = 0; i < N; ++i) sol[i] += sorig[i];
        } else {
            for (long i = 0; i < N; ++i) sol[i] = sorig[i];
        }
        return ret;
    }
    // MLMG::actualBottomSolve: x = 0, Krylov, zero on failure, then nub (0) / nuf smooths
    void bottom_solve() {
        const int m = (int)lv.size() - 1;
        double* x = lv[m].cor.data();
        const double* b = lv[m].res.data();
        std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
        const int ret = bottom_krylov(m, x, b);
        if (ret != 0 && ret != 9) {
            std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
            ++bottom_fail;
        }
        const int n = (ret == 0) ? 0 : o.nuf;
        for (int i = 0; i < n; ++i) smooth(m, x, b);
    }
    // MLMG::mgVcycle(0, top)
    void vcycle(int top) {
        const int bot = (int)lv.size() - 1;
        for (int m = top; m < bot; ++m) {
            std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
            for (int i = 0; i < o.nu1; ++i) smooth(m, lv[m].cor.data(), lv[m].res.data());
            res_of_cor(m);
            restrict_(*lv[m + 1].L, *lv[m].L, 3, lv[m + 1].res.data(), lv[m].rescor.data());
        }
        bottom_solve();
        for (int m = bot - 1; m >= top; --m) {
            interp_add(*lv[m].L, *lv[m + 1].L, 3, lv[m].cor.data(), lv[m + 1].cor.data());
            for (int i = 0; i < o.nu2; ++i) smooth(m, lv[m].cor.data(), lv[m].res.data());
        }
    }
    // MLMG::mgFcycle
    void fcycle() {
        const int bot = (int)lv.size() - 1;
        for (int m = 1; m <= bot; ++m) restrict_(*lv[m].L, *lv[m - 1].L, 3, lv[m].res.data(), lv[m - 1].res.data());
        bottom_solve();
        for (int m = bot - 1; m >= 0; --m) {
            std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
            interp_add(*lv[m].L, *lv[m + 1].L, 3, lv[m].cor.data(), lv[m + 1].cor.data());
            res_of_cor(m);
            lv[m].res = lv[m].rescor;
            std::swap(lv[m].cor, lv[m].corhold);
            vcycle(m);
            for (size_t i = 0; i < lv[m].cor.size(); ++i) lv[m].cor[i] += lv[m].corhold[i];
        }
    }
};

// ---------------------------------------------------------------- composite multi-level solve
// MLMG::oneIter over AMR levels with the reference's nodal pieces: per fine level a
// smoother-only cycle (miniCycle), fine correction residuals, reflux of the fine residual
// onto covered coarse nodes (src/Operator/Operator.cpp:728-839), trilinear interpolation of
// the coarse correction into the fine patch and its ghost nodes, and injection of the fine
// solution onto covered coarse nodes (averageDownSolutionRHS, src/Operator/Operator.cpp:626-641).
struct FineLevel {
    orc_level ol;
    Lev* L = nullptr;
    std::vector<double> C, D, res, cor, rescor, corhold;
    double* sol = nullptr;
    const double* rhs = nullptr;
};

Box covered_by(const Lev& Lf) {
    Box b;
    for (int d = 0; d < 3; ++d) { b.lo[d] = Lf.valid.lo[d] / 2; b.hi[d] = Lf.valid.hi[d] / 2; }
    return b;
}

// The AMR hierarchy as a list of patches: entry 0 covers the level-0 domain; the entries of a
// finer level follow, with twice the domain of the level before.  Several entries with one
// domain are the patches of one level (an AMReX BoxArray of separated boxes: their storage boxes
// grow(valid, 2) are disjoint, so no ghost node of one patch lies in another, and AMReX's
// FillBoundary between them has nothing to copy).  Each patch nests in one patch of the level
// below, its parent.  Returns false when the list does not describe such a hierarchy.
struct Hier {
    std::vector<int> rl, parent;     // refinement level and parent entry of every entry
    std::vector<std::vector<int>> at;  // the entries of each level
    int R = 0;                         // finest level
    bool build(const orc_level* Ls, int n) {
        rl.assign(n, 0);
        parent.assign(n, -1);
        at.assign(1, std::vector<int>{0});
        for (int a = 1; a < n; ++a) {
            bool same = true, twice = true;
            for (int d = 0; d < 3; ++d) {
                same = same && Ls[a].dom_hi[d] == Ls[a - 1].dom_hi[d];
                twice = twice && Ls[a].dom_hi[d] == 2 * Ls[a - 1].dom_hi[d];
            }
            if (same && a > 1 && rl[a - 1] >= 1) {
                rl[a] = rl[a - 1];
            } else if (twice) {
                rl[a] = rl[a - 1] + 1;
                at.emplace_back();
            } else {
                return false;
            }
            at[rl[a]].push_back(a);
            for (int q : at[rl[a] - 1]) {
                bool in = true;
                for (int d = 0; d < 3; ++d)
                    in = in && Ls[a].lo[d] / 2 >= Ls[q].lo[d] && Ls[a].hi[d] / 2 <= Ls[q].hi[d];
                if (in) { parent[a] = q; break; }
            }
            if (parent[a] < 0) return false;
            for (int q : at[rl[a]]) {  // separated from the level's other patches
                if (q == a) continue;
                bool apart = false;
                for (int d = 0; d < 3; ++d)
                    apart = apart || Ls[a].lo[d] - 2 > Ls[q].hi[d] + 2 || Ls[q].lo[d] - 2 > Ls[a].hi[d] + 2;
                if (!apart) return false;
            }
        }
        R = (int)at.size() - 1;
        return true;
    }
};

struct Amr {
    Solver* S = nullptr;
    std::vector<FineLevel> F;
    Hier H;
    double* sol0 = nullptr;
    const double* rhs0 = nullptr;
    int finest() const { return (int)F.size(); }
    Lev& L(int a) { return a == 0 ? *S->lv[0].L : *F[a - 1].L; }
    double* res(int a) { return a == 0 ? S->lv[0].res.data() : F[a - 1].res.data(); }
    double* cor(int a) { return a == 0 ? S->lv[0].cor.data() : F[a - 1].cor.data(); }
    double* sol(int a) { return a == 0 ? sol0 : F[a - 1].sol; }
    const double* rhs(int a) { return a == 0 ? rhs0 : F[a - 1].rhs; }
    const double* C(int a) { return a == 0 ? S->lv[0].C.data() : F[a - 1].C.data(); }
    long N(int a) { return 3 * L(a).nn; }

    void mini_cycle(int a) {
        FineLevel& f = F[a - 1];
        std::fill(f.cor.begin(), f.cor.end(), 0.0);
        for (int i = 0; i < S->o.nu1 + S->o.nu2; ++i)
            fsmooth(*f.L, S->model, f.C.data(), S->bctype, S->uniform, f.D.data(), f.cor.data(), f.res.data(),
                    S->o.sweeps, S->o.omega);
    }
    void sol_residual(int a) { residual(L(a), S->model, C(a), S->bctype, S->uniform, sol(a), rhs(a), res(a)); }
    void cor_residual(int a) {
        FineLevel& f = F[a - 1];
        residual(*f.L, S->model, f.C.data(), S->bctype, S->uniform, f.cor.data(), f.res.data(), f.rescor.data());
        const Box r = isect(grow(f.L->valid, 1), isect(f.L->dom, f.L->store));
        for (int n = 0; n < 3; ++n)
            for_box(r, [&](int i, int j, int k) {
                const long c = n * f.L->nn + f.L->at(i, j, k);
                f.res[c] = f.rescor[c];
            });
    }
    // the fine residual of patch e restricted onto the coarse nodes of its parent it covers
    void reflux(int e) {
        const int c = H.parent[e];
        restrict_box(L(c), L(e), 3, res(c), res(e), isect(covered_by(L(e)), L(c).dom));
    }
    void add(int a, const double* x) {
        double* s = sol(a);
        for (long i = 0; i < N(a); ++i) s[i] += x[i];
    }
    void interp_cor(int a) {
        FineLevel& f = F[a - 1];
        std::fill(f.cor.begin(), f.cor.end(), 0.0);
        interp_add_box(*f.L, L(H.parent[a]), 3, f.cor.data(), cor(H.parent[a]), isect(f.L->store, f.L->dom));
    }
    void average_down(int a) {
        Lev& Lc = L(H.parent[a]);
        Lev& Lf = L(a);
        const Box r = isect(covered_by(Lf), Lc.dom);
        double* sc = sol(H.parent[a]);
        const double* sf = sol(a);
        for (int n = 0; n < 3; ++n)
            for_box(r, [&](int I, int J, int K) {
                sc[n * Lc.nn + Lc.at(I, J, K)] = sf[n * Lf.nn + Lf.at(2 * I, 2 * J, 2 * K)];
            });
    }
    double norm(int a, const double* v) {
        Lev& l = L(a);
        const Box r = isect(l.valid, l.dom);
        double m = 0;
        for (int n = 0; n < 3; ++n)
            for (int k = r.lo[2]; k <= r.hi[2]; ++k)
                for (int j = r.lo[1]; j <= r.hi[1]; ++j)
                    for (int i = r.lo[0]; i <= r.hi[0]; ++i) m = amax(m, v[n * l.nn + l.at(i, j, k)]);
        return m;
    }
    // MLMG::computeMLResidual + composite max-norm (level by level, finest first; the patches of
    // a level are independent)
    double ml_residual() {
        double m = 0;
        for (int r = H.R; r >= 0; --r) {
            for (int e : H.at[r]) sol_residual(e);
            if (r < H.R)
                for (int e : H.at[r + 1]) reflux(e);
        }
        for (int a = 0; a <= finest(); ++a) m = std::max(m, norm(a, res(a)));
        return m;
    }
    void one_iter(int it) {
        for (int r = H.R; r >= 1; --r) {
            for (int e : H.at[r]) {
                mini_cycle(e);
                add(e, cor(e));
            }
            for (int c : H.at[r - 1]) sol_residual(c);  // computeResWithCrseSolFineCor
            for (int e : H.at[r]) {
                cor_residual(e);
                reflux(e);
                if (r != H.R) F[e - 1].corhold = F[e - 1].cor;
            }
        }
        if (it < S->o.max_fmg_iter) S->fcycle();
        else S->vcycle(0);
        add(0, cor(0));
        for (int r = 1; r <= H.R; ++r)
            for (int a : H.at[r]) {
                FineLevel& f = F[a - 1];
                interp_cor(a);
                add(a, cor(a));
                if (r != H.R)
                    for (size_t i = 0; i < f.cor.size(); ++i) f.corhold[i] += f.cor[i];
                cor_residual(a);  // computeResWithCrseCorFineCor
                mini_cycle(a);
                add(a, cor(a));
                if (r != H.R)
                    for (size_t i = 0; i < f.cor.size(); ++i) f.cor[i] += f.corhold[i];
            }
        for (int r = H.R; r >= 1; --r)
            for (int a : H.at[r]) average_down(a);
    }
};

bool coarsenable(const orc_level& L) {
    for (int d = 0; d < 3; ++d) {
        const int nc = L.dom_hi[d] - L.dom_lo[d];
        if (nc % 2 != 0 || nc / 2 < 2 || L.dom_lo[d] % 2 != 0) return false;
    }
    return true;
}

}  // namespace

extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_fapply(const orc_level* L, int model, const double* C, const int* bctype, int uniform, const double* u,
               double* f) {
    Lev l(*L);
    fapply(l, model, C, bctype, uniform, u, f);
    return 0;
}
int orc_diagonal(const orc_level* L, int model, const double* C, const int* bctype, double* diag) {
    Lev l(*L);
    diagonal(l, model, C, bctype, diag);
    return 0;
}
int orc_fsmooth(const orc_level* L, int model, const double* C, const int* bctype, int uniform, const double* diag,
                double* x, const double* b, int nsweeps, double omega) {
    Lev l(*L);
    fsmooth(l, model, C, bctype, uniform, diag, x, b, nsweeps, omega);
    return 0;
}
int orc_residual(const orc_level* L, int model, const double* C, const int* bctype, int uniform, const double* x,
                 const double* b, double* r, double* norm_inf) {
    Lev l(*L);
    const double n = residual(l, model, C, bctype, uniform, x, b, r);
    if (norm_inf) *norm_inf = n;
    return 0;
}
int orc_restrict(const orc_level* Lc, const orc_level* Lf, int ncomp, double* crse, const double* fine) {
    Lev c(*Lc), f(*Lf);
    restrict_(c, f, ncomp, crse, fine);
    return 0;
}
int orc_interp_add(const orc_level* Lf, const orc_level* Lc, int ncomp, double* fine, const double* crse) {
    Lev f(*Lf), c(*Lc);
    interp_add(f, c, ncomp, fine, crse);
    return 0;
}

// src/BC/Operator/Elastic.H:106-181 (BC values into the rhs on boundary nodes, tilebox grown 2 ∩ domain)
int orc_bc_init(const orc_level* L, const int* bctype, const double* bcval, int homogeneous, double* rhs) {
    Lev l(*L);
    const Box r = isect(grow(l.valid, 2), isect(l.dom, l.store));
    for_box(r, [&](int i, int j, int k) {
        double n[3];
        const int face = classify(l.dom, i, j, k, n);
        if (face < 0) return;
        for (int dir = 0; dir < 3; ++dir) {
            const long c = dir * l.nn + l.at(i, j, k);
            if (homogeneous && bctype[3 * face + dir] == ORC_DISP) rhs[c] = 0.0;
            else rhs[c] = bcval[3 * face + dir];
        }
    });
    return 0;
}

// src/Operator/Elastic.cpp:399-457 (valid box)
int orc_strain(const orc_level* L, const double* U, int voigt, double* E) {
    Lev l(*L);
    const Box r = isect(l.valid, l.dom);
    for_box(r, [&](int i, int j, int k) {
        int st[3];
        get_stencil(l, i, j, k, st);
        const long c = l.at(i, j, k);
        double g[3][3], e[3][3];
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) g[p][d] = D1(U + p * l.nn + c, l.stride(d), l.dx[d], st[d]);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) e[a][b] = 0.5 * (g[a][b] + g[b][a]);
        if (voigt) {
            const double v[6] = {e[0][0], e[1][1], e[2][2], e[1][2], e[2][0], e[0][1]};
            for (int q = 0; q < 6; ++q) E[q * l.nn + c] = v[q];
        } else {
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) E[(3 * a + b) * l.nn + c] = e[a][b];
        }
    });
    return 0;
}
// src/Operator/Elastic.cpp:460-519
int orc_stress(const orc_level* L, int model, const double* C, const double* U, int voigt, double* S) {
    Lev l(*L);
    const int nc = ncoef_of(model);
    const Box r = isect(l.valid, l.dom);
    for_box(r, [&](int i, int j, int k) {
        int st[3];
        get_stencil(l, i, j, k, st);
        const long c = l.at(i, j, k);
        double g[3][3], s[3][3], a[kMaxCoef];
        for (int q = 0; q < nc; ++q) a[q] = C[q * l.nn + c];
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) g[p][d] = D1(U + p * l.nn + c, l.stride(d), l.dx[d], st[d]);
        stress_of(model, a, g, s);
        if (voigt) {
            const double v[6] = {s[0][0], s[1][1], s[2][2], s[1][2], s[2][0], s[0][1]};
            for (int q = 0; q < 6; ++q) S[q * l.nn + c] = v[q];
        } else {
            for (int a2 = 0; a2 < 3; ++a2)
                for (int b = 0; b < 3; ++b) S[(3 * a2 + b) * l.nn + c] = s[a2][b];
        }
    });
    return 0;
}
// src/Operator/Elastic.cpp:522-572: energy = W(gradu) + sum 0.5 sig:eps, with
// W = trace(0.5 gradu^T (C gradu)) (src/Model/Solid/Linear/Isotropic.H:31-34, Cubic.H:60-63)
int orc_energy(const orc_level* L, int model, const double* C, const double* U, double* W) {
    Lev l(*L);
    const int nc = ncoef_of(model);
    const Box r = isect(l.valid, l.dom);
    for_box(r, [&](int i, int j, int k) {
        int st[3];
        get_stencil(l, i, j, k, st);
        const long c = l.at(i, j, k);
        double g[3][3], s[3][3], a[kMaxCoef], e[3][3];
        for (int q = 0; q < nc; ++q) a[q] = C[q * l.nn + c];
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) g[p][d] = D1(U + p * l.nn + c, l.stride(d), l.dx[d], st[d]);
        for (int a2 = 0; a2 < 3; ++a2)
            for (int b = 0; b < 3; ++b) e[a2][b] = .5 * (g[a2][b] + g[b][a2]);
        stress_of(model, a, g, s);
        double w = 0;  // trace(0.5 * g^T * s) = 0.5 * sum_{ij} g_ji s_ji
        for (int ii = 0; ii < 3; ++ii) {
            double t = 0;
            for (int jj = 0; jj < 3; ++jj) t += g[jj][ii] * s[jj][ii];
            w += 0.5 * t;
        }
        for (int m = 0; m < 3; ++m)
            for (int n = 0; n < 3; ++n) w += .5 * s[m][n] * e[m][n];
        W[c] = w;
    });
    return 0;
}

// Generic 81-term tensors from the 21-slot MajorMinor storage, index map of
// src/Set/Matrix4_MajorMinor.H:145-192 rewritten as a table.
void orc_mm_full(const double* c21, double* c81) {
    // slot of (i,j,k,l) via the sorted Voigt pair (ij),(kl): 21 = upper triangle of 6x6
    static const int voigt[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}};
    // reference slot for each upper-triangle (V1<=V2) pair in its ordering
    // Voigt index v: 0=00 1=11 2=22 3=12 4=20 5=01
    // Reference slots by (pair of index pairs), derived from Matrix4_MajorMinor.H:148-189.
    static int slot[6][6];
    static bool init = false;
    if (!init) {
        // pairs (ij) in reference component order; each entry lists (i,j,k,l) representative and slot
        const int rep[21][5] = {{0, 0, 0, 0, 0},  {0, 0, 0, 1, 1},  {0, 0, 0, 2, 2},  {0, 0, 1, 1, 3},
                                {0, 0, 1, 2, 4},  {0, 0, 2, 2, 5},  {0, 1, 0, 1, 6},  {0, 1, 0, 2, 7},
                                {0, 1, 1, 1, 8},  {0, 1, 1, 2, 9},  {0, 1, 2, 2, 10}, {0, 2, 0, 2, 11},
                                {0, 2, 1, 1, 12}, {0, 2, 1, 2, 13}, {0, 2, 2, 2, 14}, {1, 1, 1, 1, 15},
                                {1, 1, 1, 2, 16}, {1, 1, 2, 2, 17}, {1, 2, 1, 2, 18}, {1, 2, 2, 2, 19},
                                {2, 2, 2, 2, 20}};
        for (int t = 0; t < 21; ++t) {
            const int v1 = voigt[rep[t][0]][rep[t][1]], v2 = voigt[rep[t][2]][rep[t][3]];
            slot[v1][v2] = rep[t][4];
            slot[v2][v1] = rep[t][4];
        }
        init = true;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) c81[((i * 3 + j) * 3 + k) * 3 + l] = c21[slot[voigt[i][j]][voigt[k][l]]];
}
void orc_mm_stress(const double* c21, const double* g9, double* s9) {
    double g[3][3], s[3][3];
    for (int a = 0; a < 9; ++a) g[a / 3][a % 3] = g9[a];
    stress_mm(c21, g, s);
    for (int a = 0; a < 9; ++a) s9[a] = s[a / 3][a % 3];
}
void orc_mm_div(const double* c21, const double* b27, double* f3) {
    double b[3][3][3];
    for (int a = 0; a < 27; ++a) b[a / 9][(a / 3) % 3][a % 3] = b27[a];
    div_mm(c21, b, f3);
}

int orc_num_mg_levels(const orc_level* L, int max_mg_levels) {
    orc_level cur = *L;
    int n = 1;
    while (coarsenable(cur) && (max_mg_levels <= 0 || n < max_mg_levels)) {
        for (int d = 0; d < 3; ++d) {
            cur.dom_lo[d] /= 2; cur.dom_hi[d] /= 2; cur.lo[d] /= 2; cur.hi[d] /= 2;
        }
        ++n;
    }
    return n;
}

// MLMG::computeMLResidual restated on its own (the composite residual Amr::ml_residual takes, with
// no multigrid set-up): r_a = b_a - A_a u_a on every AMR level, finest first, and on each coarser
// level the fine residual restricted onto the nodes the finer patch covers (reflux,
// src/Operator/Operator.cpp:728-839).  rs may be NULL (scratch is allocated); norm_inf gets the
// max-norm over the valid nodes of every level.
int orc_residual_amr(const orc_level* Ls, int namr, int model, const double* const* Cs, const int* bctype,
                     int uniform, const double* const* us, const double* const* bs, double* const* rs,
                     double* norm_inf) {
    if (namr < 1 || Ls[0].ng != 0) return -1;
    Hier H;
    if (!H.build(Ls, namr)) return -1;
    std::vector<std::unique_ptr<Lev>> L;
    std::vector<std::vector<double>> own(namr);
    std::vector<double*> r(namr);
    for (int a = 0; a < namr; ++a) {
        L.emplace_back(new Lev(Ls[a]));
        if (rs && rs[a]) {
            r[a] = rs[a];
        } else {
            own[a].assign(3 * L[a]->nn, 0.0);
            r[a] = own[a].data();
        }
    }
    for (int lv = H.R; lv >= 0; --lv) {
        for (int a : H.at[lv]) residual(*L[a], model, Cs[a], bctype, uniform, us[a], bs[a], r[a]);
        if (lv < H.R)
            for (int e : H.at[lv + 1]) {
                const int c = H.parent[e];
                restrict_box(*L[c], *L[e], 3, r[c], r[e], isect(covered_by(*L[e]), L[c]->dom));
            }
    }
    double m = 0.0;
    for (int a = 0; a < namr; ++a) {
        const Box v = isect(L[a]->valid, L[a]->dom);
        for (int n = 0; n < 3; ++n)
            for (int k = v.lo[2]; k <= v.hi[2]; ++k)
                for (int j = v.lo[1]; j <= v.hi[1]; ++j)
                    for (int i = v.lo[0]; i <= v.hi[0]; ++i) m = amax(m, r[a][n * L[a]->nn + L[a]->at(i, j, k)]);
    }
    if (norm_inf) *norm_inf = m;
    return 0;
}

// MLMG::solve restated: convergence when the composite ||r||_inf <= max(tol_abs, tol_rel * max_norm),
// max_norm = ||b||_inf if ||b||_inf >= ||r0||_inf else ||r0||_inf.  Ls[0] covers its domain
// (ng = 0); Ls[l >= 1] are patches of finer levels refined by 2 with ng = 2, several per level
// when they share a domain (Hier).
int orc_solve_amr(const orc_level* Ls, int namr, int model, const double* const* Cs, const int* bctype,
                  double* const* us, const double* const* bs, double tol_rel, double tol_abs, const orc_opts* opts,
                  orc_stats* stats) {
    const orc_level* L0 = &Ls[0];
    if (L0->ng != 0 || namr < 1) return -1;
    for (int a = 1; a < namr; ++a)
        if (Ls[a].ng != 2) return -1;
    const double* C = Cs[0];
    double* u = us[0];
    const double* b = bs[0];
    Solver S;
    S.model = model;
    S.nc = ncoef_of(model);
    S.bctype = bctype;
    S.o = *opts;
    S.uniform = opts->uniform;
    const int nlev = orc_num_mg_levels(L0, opts->max_mg_levels);
    S.lv.resize(nlev);
    orc_level cur = *L0;
    for (int m = 0; m < nlev; ++m) {
        if (m > 0)
            for (int d = 0; d < 3; ++d) {
                cur.dom_lo[d] /= 2; cur.dom_hi[d] /= 2; cur.lo[d] /= 2; cur.hi[d] /= 2; cur.dx[d] *= 2.0;
            }
        S.lv[m].ol = cur;
        S.lv[m].L = new Lev(S.lv[m].ol);
        const long nn = S.lv[m].L->nn;
        S.lv[m].C.assign(S.nc * nn, 0.0);
        S.lv[m].D.assign(3 * nn, 0.0);
        S.lv[m].res.assign(3 * nn, 0.0);
        S.lv[m].cor.assign(3 * nn, 0.0);
        S.lv[m].rescor.assign(3 * nn, 0.0);
        S.lv[m].corhold.assign(3 * nn, 0.0);
    }
    // Operator<Node>::prepareForSolve: averageDownCoeffs, then Diagonal (Operator.cpp:445-452)
    std::memcpy(S.lv[0].C.data(), C, sizeof(double) * S.nc * S.lv[0].L->nn);
    for (int m = 1; m < nlev; ++m) restrict_(*S.lv[m].L, *S.lv[m - 1].L, S.nc, S.lv[m].C.data(), S.lv[m - 1].C.data());
    for (int m = 0; m < nlev; ++m) diagonal(*S.lv[m].L, model, S.lv[m].C.data(), bctype, S.lv[m].D.data());

    Amr A;
    if (!A.H.build(Ls, namr)) return -1;
    A.S = &S;
    A.sol0 = u;
    A.rhs0 = b;
    A.F.resize(namr - 1);
    for (int a = 1; a < namr; ++a) {
        FineLevel& f = A.F[a - 1];
        f.ol = Ls[a];
        f.L = new Lev(f.ol);
        const long nn = f.L->nn;
        f.C.assign(Cs[a], Cs[a] + S.nc * nn);
        f.D.assign(3 * nn, 0.0);
        f.res.assign(3 * nn, 0.0);
        f.cor.assign(3 * nn, 0.0);
        f.rescor.assign(3 * nn, 0.0);
        f.corhold.assign(3 * nn, 0.0);
        f.sol = us[a];
        f.rhs = bs[a];
        diagonal(*f.L, model, f.C.data(), bctype, f.D.data());
    }
    struct Cleanup {
        Amr& A;
        ~Cleanup() { for (auto& f : A.F) delete f.L; }
    } cleanup{A};

    double bnorm = 0;
    for (int a = 0; a < namr; ++a) bnorm = std::max(bnorm, A.norm(a, A.rhs(a)));
    const double res0 = A.ml_residual();
    const double max_norm = (bnorm >= res0) ? bnorm : res0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm);
    int iters = 0, conv = 0;
    double rn = res0;
    if (res0 <= target) conv = 1;
    for (int it = 0; !conv && it < opts->max_iter; ++it) {
        A.one_iter(it);
        rn = A.ml_residual();
        if (stats && it < 256) stats->hist[it] = rn;
        iters = it + 1;
        if (!std::isfinite(rn)) break;
        if (rn <= target) conv = 1;
    }
    if (stats) {
        stats->iters = iters;
        stats->converged = conv;
        stats->nlevels = nlev;
        stats->bottom_fail = S.bottom_fail;
        stats->res0 = res0;
        stats->resfinal = rn;
        stats->target = target;
    }
    return conv ? 0 : 1;
}

int orc_solve(const orc_level* L0, int model, const double* C, const int* bctype, double* u, const double* b,
              double tol_rel, double tol_abs, const orc_opts* opts, orc_stats* stats) {
    const double* Cs[1] = {C};
    double* us[1] = {u};
    const double* bs[1] = {b};
    return orc_solve_amr(L0, 1, model, Cs, bctype, us, bs, tol_rel, tol_abs, opts, stats);
}

}  // extern "C"

// ================================================================ periodic RVE cells
// Homogenisation of a periodic cell under a macroscopic displacement gradient E:
// u = E x + w with w periodic.  The operator is the interior row of Elastic<T>::Fapply
// (src/Operator/Elastic.cpp:216-255) at every node, neighbours taken modulo the cell, since a
// periodic cell has no domain boundary.  (The reference's BC::Operator::Elastic marks a periodic
// face with Type::Periodic, src/BC/Operator/Elastic.H:299-300, and leaves the node coupling to
// AMReX's periodic ghost fill.)  Because the stencils are exact on affine fields,
// A(E x) = sum_d (d_d C) : E e_d, so w solves A w = b with b = -sum_d (d_d C) : E e_d.
//
// A annihilates constants but the non-divergence form is not conservative on the grid: its
// left null vectors are not constant, so b is in general not in the range of A.  The cell
// problem is therefore posed with a uniform body force c (the Lagrange multiplier of mean(w) = 0):
//     A w + c = b,   mean(w) = 0,
// which is consistent and has a unique solution.  Each MLMG-style iteration removes the mean of
// the residual (that mean is the current c), the convergence test is on the mean-free residual,
// and the coarsest level solves the same bordered problem with the Krylov iteration run on the
// mean-projected operator.  Every node stores n[0] n[1] n[2] unique nodes, no ghosts, index order
// [comp][k][j][i].
namespace {

struct PLev {
    int n[3];
    double dx[3];
    long nn;
    explicit PLev(const orc_rve_level& L) {
        for (int d = 0; d < 3; ++d) { n[d] = L.n[d]; dx[d] = L.dx[d]; }
        nn = (long)n[0] * n[1] * n[2];
    }
    long at(int i, int j, int k) const {
        i = (i % n[0] + n[0]) % n[0];
        j = (j % n[1] + n[1]) % n[1];
        k = (k % n[2] + n[2]) % n[2];
        return (long)i + (long)n[0] * (j + (long)n[1] * k);
    }
};

template <class F>
void for_cell(const PLev& L, F&& fn) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < L.n[2]; ++k)
        for (int j = 0; j < L.n[1]; ++j)
            for (int i = 0; i < L.n[0]; ++i) fn(i, j, k);
}

// value of component array f at (i,j,k) + offsets, periodic
struct PAt {
    const PLev& L;
    const double* f;
    int i, j, k;
    double operator()(int a, int b, int c) const { return f[L.at(i + a, j + b, k + c)]; }
};

// gradient (central) and second derivatives of component p at a node, the Numeric::Stencil
// interior formulas (src/Numeric/Stencil.H:44-176) on periodic neighbours
inline void pgrad(const PLev& L, const double* U, int i, int j, int k, double g[3][3], double b[3][3][3]) {
    for (int p = 0; p < 3; ++p) {
        const PAt f{L, U + p * L.nn, i, j, k};
        const double c0 = f(0, 0, 0);
        g[p][0] = (f(1, 0, 0) - f(-1, 0, 0)) * 0.5 / L.dx[0];
        g[p][1] = (f(0, 1, 0) - f(0, -1, 0)) * 0.5 / L.dx[1];
        g[p][2] = (f(0, 0, 1) - f(0, 0, -1)) * 0.5 / L.dx[2];
        if (!b) continue;
        b[p][0][0] = (f(1, 0, 0) - 2.0 * c0 + f(-1, 0, 0)) / L.dx[0] / L.dx[0];
        b[p][1][1] = (f(0, 1, 0) - 2.0 * c0 + f(0, -1, 0)) / L.dx[1] / L.dx[1];
        b[p][2][2] = (f(0, 0, 1) - 2.0 * c0 + f(0, 0, -1)) / L.dx[2] / L.dx[2];
        b[p][0][1] = 0.25 * (f(1, 1, 0) + f(-1, -1, 0) - f(1, -1, 0) - f(-1, 1, 0)) / (L.dx[0] * L.dx[1]);
        b[p][0][2] = 0.25 * (f(1, 0, 1) + f(-1, 0, -1) - f(1, 0, -1) - f(-1, 0, 1)) / (L.dx[0] * L.dx[2]);
        b[p][1][2] = 0.25 * (f(0, 1, 1) + f(0, -1, -1) - f(0, 1, -1) - f(0, -1, 1)) / (L.dx[1] * L.dx[2]);
        b[p][1][0] = b[p][0][1];
        b[p][2][0] = b[p][0][2];
        b[p][2][1] = b[p][1][2];
    }
}

// sum_d column d of (d_d C) : g  (Elastic.cpp:249-254 with central differences)
inline void pgradC(const PLev& L, int model, const double* C, int i, int j, int k, const double g[3][3],
                   double out[3]) {
    const int nc = ncoef_of(model);
    double col[3][3];
    for (int d = 0; d < 3; ++d) {
        const int o[3] = {d == 0, d == 1, d == 2};
        double cg[kMaxCoef];
        for (int q = 0; q < nc; ++q) {
            const PAt c{L, C + q * L.nn, i, j, k};
            cg[q] = (c(o[0], o[1], o[2]) - c(-o[0], -o[1], -o[2])) * 0.5 / L.dx[d];
        }
        double sd[3][3];
        stress_of(model, cg, g, sd);
        for (int r = 0; r < 3; ++r) col[d][r] = sd[r][d];
    }
    for (int r = 0; r < 3; ++r) out[r] = (col[0][r] + col[1][r]) + col[2][r];
}

inline void pfapply_node(const PLev& L, int model, const double* C, int uniform, const double* U, int i, int j,
                         int k, double f[3]) {
    const long c = L.at(i, j, k);
    const int nc = ncoef_of(model);
    double a[kMaxCoef];
    for (int q = 0; q < nc; ++q) a[q] = C[q * L.nn + c];
    double g[3][3], b[3][3][3];
    pgrad(L, U, i, j, k, g, b);
    div_of(model, a, b, f);
    if (!uniform) {
        double gc[3];
        pgradC(L, model, C, i, j, k, g, gc);
        for (int r = 0; r < 3; ++r) f[r] += gc[r];
    }
}

void pfapply(const PLev& L, int model, const double* C, int uniform, const double* U, double* F) {
    for_cell(L, [&](int i, int j, int k) {
        double f[3];
        pfapply_node(L, model, C, uniform, U, i, j, k, f);
        const long c = L.at(i, j, k);
        for (int p = 0; p < 3; ++p) F[p * L.nn + c] = f[p];
    });
}

// Elastic<T>::Diagonal interior row (src/Operator/Elastic.cpp:320-341): the central gradient
// of a unit spike vanishes at its own node, leaving C_{pjpj} (-2 / dx_j^2)
void pdiagonal(const PLev& L, int model, const double* C, double* D) {
    const int nc = ncoef_of(model);
    for_cell(L, [&](int i, int j, int k) {
        const long c = L.at(i, j, k);
        double a[kMaxCoef];
        for (int q = 0; q < nc; ++q) a[q] = C[q * L.nn + c];
        for (int p = 0; p < 3; ++p) {
            double b[3][3][3] = {};
            for (int d = 0; d < 3; ++d) b[p][d][d] = -2.0 / L.dx[d] / L.dx[d];
            double f[3];
            div_of(model, a, b, f);
            D[p * L.nn + c] = f[p];
        }
    });
}

// Operator<Node>::Fsmooth update (src/Operator/Operator.cpp:128-150) at every node of the cell
void pfsmooth(const PLev& L, int model, const double* C, int uniform, const double* D, double* X, const double* B,
              int nsweeps, double omega) {
    std::vector<double> Ax(3 * L.nn);
    for (int s = 0; s < nsweeps; ++s) {
        pfapply(L, model, C, uniform, X, Ax.data());
#pragma omp parallel for schedule(static)
        for (long c = 0; c < 3 * L.nn; ++c) {
            const double Dx = X[c] * D[c];
            const double Rx = Ax[c] - Dx;
            X[c] = (1. - omega) * X[c] + omega * (B[c] - Rx) / D[c];
        }
    }
}

// per-component mean, summed in node order
void pmean(const PLev& L, const double* v, double m[3]) {
    for (int p = 0; p < 3; ++p) {
        double s = 0.0;
        for (long c = 0; c < L.nn; ++c) s += v[p * L.nn + c];
        m[p] = s / (double)L.nn;
    }
}
void psubtract(const PLev& L, double* v, const double m[3]) {
    for (int p = 0; p < 3; ++p)
        for (long c = 0; c < L.nn; ++c) v[p * L.nn + c] -= m[p];
}
double pninf(const PLev& L, const double* v) {
    double m = 0.0;
    for (long c = 0; c < 3 * L.nn; ++c) m = amax(m, v[c]);
    return m;
}

// r = b - A x; with project, the per-component mean of r is removed (returned in mean)
double presidual(const PLev& L, int model, const double* C, int uniform, const double* X, const double* B, double* R,
                 int project, double mean[3]) {
    pfapply(L, model, C, uniform, X, R);
    for (long c = 0; c < 3 * L.nn; ++c) R[c] = B[c] + (-1.0) * R[c];
    double m[3] = {0, 0, 0};
    if (project) {
        pmean(L, R, m);
        psubtract(L, R, m);
    }
    if (mean)
        for (int p = 0; p < 3; ++p) mean[p] = m[p];
    return pninf(L, R);
}

// nodal full weighting (the interior weights of Operator<Node>::restriction,
// src/Operator/Operator.cpp:527-541), neighbours modulo the fine cell; coarse I <- fine 2I
void prestrict(const PLev& Lc, const PLev& Lf, int ncomp, double* crse, const double* fine) {
    for (int n = 0; n < ncomp; ++n) {
        for_cell(Lc, [&](int I, int J, int K) {
            const PAt f{Lf, fine + n * Lf.nn, 2 * I, 2 * J, 2 * K};
            const double v =
                (f(-1, -1, -1) + f(-1, -1, +1) + f(-1, +1, -1) + f(-1, +1, +1) + f(+1, -1, -1) + f(+1, -1, +1) +
                 f(+1, +1, -1) + f(+1, +1, +1)) / 64.0 +
                (f(0, -1, -1) + f(0, -1, +1) + f(0, +1, -1) + f(0, +1, +1) + f(-1, 0, -1) + f(+1, 0, -1) +
                 f(-1, 0, +1) + f(+1, 0, +1) + f(-1, -1, 0) + f(-1, +1, 0) + f(+1, -1, 0) + f(+1, +1, 0)) / 32.0 +
                (f(-1, 0, 0) + f(0, -1, 0) + f(0, 0, -1) + f(+1, 0, 0) + f(0, +1, 0) + f(0, 0, +1)) / 16.0 +
                f(0, 0, 0) / 8.0;
            crse[n * Lc.nn + Lc.at(I, J, K)] = v;
        });
    }
}

// trilinear nodal prolongation added into fine (src/Operator/Operator.cpp:586-614), coarse
// neighbours modulo the coarse cell
void pinterp_add(const PLev& Lf, const PLev& Lc, int ncomp, double* fine, const double* crse) {
    for (int n = 0; n < ncomp; ++n) {
        for_cell(Lf, [&](int i, int j, int k) {
            const PAt c{Lc, crse + n * Lc.nn, i / 2, j / 2, k / 2};
            const bool ie = i % 2 == 0, je = j % 2 == 0, ke = k % 2 == 0;
            double v;
            if (ie && je && ke) v = c(0, 0, 0);
            else if (je && ke) v = 0.5 * (c(0, 0, 0) + c(1, 0, 0));
            else if (ke && ie) v = 0.5 * (c(0, 0, 0) + c(0, 1, 0));
            else if (ie && je) v = 0.5 * (c(0, 0, 0) + c(0, 0, 1));
            else if (ie) v = 0.25 * (c(0, 0, 0) + c(0, 1, 0) + c(0, 0, 1) + c(0, 1, 1));
            else if (je) v = 0.25 * (c(0, 0, 0) + c(0, 0, 1) + c(1, 0, 0) + c(1, 0, 1));
            else if (ke) v = 0.25 * (c(0, 0, 0) + c(1, 0, 0) + c(0, 1, 0) + c(1, 1, 0));
            else
                v = 0.125 * (c(0, 0, 0) + c(1, 0, 0) + c(0, 1, 0) + c(0, 0, 1) + c(0, 1, 1) + c(1, 0, 1) + c(1, 1, 0) +
                             c(1, 1, 1));
            fine[n * Lf.nn + Lf.at(i, j, k)] += v;
        });
    }
}

bool pcoarsenable(const orc_rve_level& L) {
    for (int d = 0; d < 3; ++d)
        if (L.n[d] % 2 != 0 || L.n[d] / 2 < 2) return false;
    return true;
}

struct PMG {
    orc_rve_level ol;
    PLev* L = nullptr;
    std::vector<double> C, D, res, cor, rescor, corhold;
};

// The MLMG cycle of Solver above on a periodic cell; the bottom solve works on the
// mean-projected operator.
struct PSolver {
    int model, nc, uniform;
    orc_opts o;
    std::vector<PMG> lv;
    int bottom_fail = 0;
    ~PSolver() { for (auto& l : lv) delete l.L; }

    void apply(int m, const double* x, double* out) { pfapply(*lv[m].L, model, lv[m].C.data(), uniform, x, out); }
    void smooth(int m, double* x, const double* b) {
        pfsmooth(*lv[m].L, model, lv[m].C.data(), uniform, lv[m].D.data(), x, b, o.sweeps, o.omega);
    }
    void res_of_cor(int m) {
        presidual(*lv[m].L, model, lv[m].C.data(), uniform, lv[m].cor.data(), lv[m].res.data(), lv[m].rescor.data(), 0,
                  nullptr);
    }
    double dot(int m, const double* a, const double* b) {
        double s = 0;
        for (long i = 0; i < 3 * lv[m].L->nn; ++i) s += a[i] * b[i];
        return s;
    }
    // A x with its per-component mean removed
    void papply(int m, const double* x, double* out) {
        apply(m, x, out);
        double mu[3];
        pmean(*lv[m].L, out, mu);
        psubtract(*lv[m].L, out, mu);
    }
    // MLCGSolver CG / BiCGStab (as Solver::bottom_krylov) on P A, P the mean projection
    int bottom_krylov(int m, double* sol, const double* rhs) {
        const PLev& L = *lv[m].L;
        const long N = 3 * L.nn;
        const double eps_rel = o.bottom_reltol, eps_abs = -1.0;
        std::vector<double> sorig(sol, sol + N), r(N);
        double mu[3];
        presidual(L, model, lv[m].C.data(), uniform, sol, rhs, r.data(), 1, mu);
        std::fill(sol, sol + N, 0.0);
        double rnorm = pninf(L, r.data());
        const double rnorm0 = rnorm;
        int ret = 0;
        if (rnorm0 == 0 || rnorm0 < eps_abs) {
            for (long i = 0; i < N; ++i) sol[i] += sorig[i];
            return 0;
        }
        if (o.bottom == 0) {
            std::vector<double> p(N, 0.0), q(N);
            double rho_1 = 0;
            for (int iter = 1; iter <= o.bottom_max_iter; ++iter) {
                const double rho = dot(m, r.data(), r.data());
                if (rho == 0) { ret = 1; break; }
                if (iter == 1) p = r;
                else {
                    const double beta = rho / rho_1;
                    for (long i = 0; i < N; ++i) p[i] = r[i] + beta * p[i];
                }
                papply(m, p.data(), q.data());
                const double pw = dot(m, p.data(), q.data());
                if (pw == 0) { ret = 1; break; }
                const double alpha = rho / pw;
                for (long i = 0; i < N; ++i) { sol[i] += alpha * p[i]; r[i] += -alpha * q[i]; }
                rnorm = pninf(L, r.data());
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                rho_1 = rho;
            }
        } else {
            std::vector<double> p(N, 0.0), rh(r), v(N, 0.0), t(N);
            double rho_1 = 0, alpha = 0, omega = 0;
            for (int iter = 1; iter <= o.bottom_max_iter; ++iter) {
                const double rho = dot(m, rh.data(), r.data());
                if (rho == 0) { ret = 1; break; }
                if (iter == 1) p = r;
                else {
                    const double beta = (rho / rho_1) * (alpha / omega);
                    for (long i = 0; i < N; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
                }
                papply(m, p.data(), v.data());
                const double rhTv = dot(m, rh.data(), v.data());
                if (rhTv != 0) alpha = rho / rhTv;
                else { ret = 2; break; }
                for (long i = 0; i < N; ++i) { sol[i] += alpha * p[i]; r[i] += -alpha * v[i]; }
                rnorm = pninf(L, r.data());
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                papply(m, r.data(), t.data());
                const double tt = dot(m, t.data(), t.data()), tr = dot(m, t.data(), r.data());
                if (tt != 0) omega = tr / tt;
                else { ret = 3; break; }
                for (long i = 0; i < N; ++i) { sol[i] += omega * r[i]; r[i] += -omega * t[i]; }
                rnorm = pninf(L, r.data());
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                if (omega == 0) { ret = 4; break; }
                rho_1 = rho;
            }
        }
        if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
        if ((ret == 0 || ret == 8) && rnorm < rnorm0) {
            for (long i = 0; i < N; ++i) sol[i] += sorig[i];
        } else {
            for (long i = 0; i < N; ++i) sol[i] = sorig[i];
        }
        return ret;
    }
    void bottom_solve() {
        const int m = (int)lv.size() - 1;
        double* x = lv[m].cor.data();
        const double* b = lv[m].res.data();
        std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
        const int ret = bottom_krylov(m, x, b);
        if (ret != 0 && ret != 9) {
            std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
            ++bottom_fail;
        }
        const int n = (ret == 0) ? 0 : o.nuf;
        for (int i = 0; i < n; ++i) smooth(m, x, b);
    }
    void vcycle(int top) {
        const int bot = (int)lv.size() - 1;
        for (int m = top; m < bot; ++m) {
            std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
            for (int i = 0; i < o.nu1; ++i) smooth(m, lv[m].cor.data(), lv[m].res.data());
            res_of_cor(m);
            prestrict(*lv[m + 1].L, *lv[m].L, 3, lv[m + 1].res.data(), lv[m].rescor.data());
        }
        bottom_solve();
        for (int m = bot - 1; m >= top; --m) {
            pinterp_add(*lv[m].L, *lv[m + 1].L, 3, lv[m].cor.data(), lv[m + 1].cor.data());
            for (int i = 0; i < o.nu2; ++i) smooth(m, lv[m].cor.data(), lv[m].res.data());
        }
    }
    void fcycle() {
        const int bot = (int)lv.size() - 1;
        for (int m = 1; m <= bot; ++m) prestrict(*lv[m].L, *lv[m - 1].L, 3, lv[m].res.data(), lv[m - 1].res.data());
        bottom_solve();
        for (int m = bot - 1; m >= 0; --m) {
            std::fill(lv[m].cor.begin(), lv[m].cor.end(), 0.0);
            pinterp_add(*lv[m].L, *lv[m + 1].L, 3, lv[m].cor.data(), lv[m + 1].cor.data());
            res_of_cor(m);
            lv[m].res = lv[m].rescor;
            std::swap(lv[m].cor, lv[m].corhold);
            vcycle(m);
            for (size_t i = 0; i < lv[m].cor.size(); ++i) lv[m].cor[i] += lv[m].corhold[i];
        }
    }
};

// b = -sum_d (d_d C) : E e_d
void prhs(const PLev& L, int model, const double* C, int uniform, const double E[9], double* B) {
    double g[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) g[a][b] = E[3 * a + b];
    for_cell(L, [&](int i, int j, int k) {
        const long c = L.at(i, j, k);
        double gc[3] = {0, 0, 0};
        if (!uniform) pgradC(L, model, C, i, j, k, g, gc);
        for (int p = 0; p < 3; ++p) B[p * L.nn + c] = -gc[p];
    });
}

}  // namespace

extern "C" {

int orc_rve_num_mg_levels(const orc_rve_level* L, int max_mg_levels) {
    orc_rve_level cur = *L;
    int n = 1;
    while (pcoarsenable(cur) && (max_mg_levels <= 0 || n < max_mg_levels)) {
        for (int d = 0; d < 3; ++d) cur.n[d] /= 2;
        ++n;
    }
    return n;
}
int orc_rve_fapply(const orc_rve_level* L, int model, const double* C, int uniform, const double* u, double* f) {
    pfapply(PLev(*L), model, C, uniform, u, f);
    return 0;
}
int orc_rve_diagonal(const orc_rve_level* L, int model, const double* C, double* diag) {
    pdiagonal(PLev(*L), model, C, diag);
    return 0;
}
int orc_rve_fsmooth(const orc_rve_level* L, int model, const double* C, int uniform, const double* diag, double* x,
                    const double* b, int nsweeps, double omega) {
    pfsmooth(PLev(*L), model, C, uniform, diag, x, b, nsweeps, omega);
    return 0;
}
int orc_rve_residual(const orc_rve_level* L, int model, const double* C, int uniform, const double* x,
                     const double* b, double* r, int project, double* mean, double* norm_inf) {
    const double n = presidual(PLev(*L), model, C, uniform, x, b, r, project, mean);
    if (norm_inf) *norm_inf = n;
    return 0;
}
int orc_rve_restrict(const orc_rve_level* Lc, const orc_rve_level* Lf, int ncomp, double* crse, const double* fine) {
    for (int d = 0; d < 3; ++d)
        if (Lf->n[d] != 2 * Lc->n[d]) return -1;
    prestrict(PLev(*Lc), PLev(*Lf), ncomp, crse, fine);
    return 0;
}
int orc_rve_interp_add(const orc_rve_level* Lf, const orc_rve_level* Lc, int ncomp, double* fine,
                       const double* crse) {
    for (int d = 0; d < 3; ++d)
        if (Lf->n[d] != 2 * Lc->n[d]) return -1;
    pinterp_add(PLev(*Lf), PLev(*Lc), ncomp, fine, crse);
    return 0;
}
int orc_rve_rhs(const orc_rve_level* L, int model, const double* C, int uniform, const double* E, double* b) {
    prhs(PLev(*L), model, C, uniform, E, b);
    return 0;
}
// cell average of the stress C : (E + grad w), grad w by central differences
int orc_rve_mean_stress(const orc_rve_level* L0, int model, const double* C, const double* E, const double* w,
                        double* sig) {
    const PLev L(*L0);
    const int nc = ncoef_of(model);
    double acc[9] = {0};
    for (int k = 0; k < L.n[2]; ++k)
        for (int j = 0; j < L.n[1]; ++j)
            for (int i = 0; i < L.n[0]; ++i) {
                const long c = L.at(i, j, k);
                double a[kMaxCoef], g[3][3], s[3][3];
                for (int q = 0; q < nc; ++q) a[q] = C[q * L.nn + c];
                pgrad(L, w, i, j, k, g, nullptr);
                for (int p = 0; p < 3; ++p)
                    for (int d = 0; d < 3; ++d) g[p][d] += E[3 * p + d];
                stress_of(model, a, g, s);
                for (int p = 0; p < 3; ++p)
                    for (int d = 0; d < 3; ++d) acc[3 * p + d] += s[p][d];
            }
    for (int q = 0; q < 9; ++q) sig[q] = acc[q] / (double)L.nn;
    return 0;
}
// Cell solve: w (initial guess in, solution out, mean removed) for the macroscopic gradient E.
// Convergence as MLMG (orc_solve_amr) on the mean-free residual; stats->res0/resfinal are those
// norms.  body_force (3) receives the mean of the last residual.
int orc_rve_solve(const orc_rve_level* L0, int model, const double* C, const double* E, double* w,
                  double tol_rel, double tol_abs, const orc_opts* opts, orc_stats* stats, double* body_force) {
    PSolver S;
    S.model = model;
    S.nc = ncoef_of(model);
    S.o = *opts;
    S.uniform = opts->uniform;
    const int nlev = orc_rve_num_mg_levels(L0, opts->max_mg_levels);
    S.lv.resize(nlev);
    orc_rve_level cur = *L0;
    for (int m = 0; m < nlev; ++m) {
        if (m > 0)
            for (int d = 0; d < 3; ++d) { cur.n[d] /= 2; cur.dx[d] *= 2.0; }
        S.lv[m].ol = cur;
        S.lv[m].L = new PLev(cur);
        const long nn = S.lv[m].L->nn;
        S.lv[m].C.assign(S.nc * nn, 0.0);
        S.lv[m].D.assign(3 * nn, 0.0);
        S.lv[m].res.assign(3 * nn, 0.0);
        S.lv[m].cor.assign(3 * nn, 0.0);
        S.lv[m].rescor.assign(3 * nn, 0.0);
        S.lv[m].corhold.assign(3 * nn, 0.0);
    }
    const PLev& L = *S.lv[0].L;
    std::memcpy(S.lv[0].C.data(), C, sizeof(double) * S.nc * L.nn);
    for (int m = 1; m < nlev; ++m) prestrict(*S.lv[m].L, *S.lv[m - 1].L, S.nc, S.lv[m].C.data(), S.lv[m - 1].C.data());
    for (int m = 0; m < nlev; ++m) pdiagonal(*S.lv[m].L, model, S.lv[m].C.data(), S.lv[m].D.data());

    std::vector<double> b(3 * L.nn);
    prhs(L, model, S.lv[0].C.data(), S.uniform, E, b.data());
    double bm[3];
    pmean(L, b.data(), bm);
    psubtract(L, b.data(), bm);
    const double bnorm = pninf(L, b.data());
    double mu[3] = {0, 0, 0};
    double* res0v = S.lv[0].res.data();
    const double res0 = presidual(L, model, S.lv[0].C.data(), S.uniform, w, b.data(), res0v, 1, mu);
    const double max_norm = (bnorm >= res0) ? bnorm : res0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm);
    int iters = 0, conv = 0;
    double rn = res0;
    if (res0 <= target) conv = 1;
    for (int it = 0; !conv && it < opts->max_iter; ++it) {
        if (it < opts->max_fmg_iter) S.fcycle();
        else S.vcycle(0);
        for (long i = 0; i < 3 * L.nn; ++i) w[i] += S.lv[0].cor[i];
        rn = presidual(L, model, S.lv[0].C.data(), S.uniform, w, b.data(), res0v, 1, mu);
        if (stats && it < 256) stats->hist[it] = rn;
        iters = it + 1;
        if (!std::isfinite(rn)) break;
        if (rn <= target) conv = 1;
    }
    double wm[3];
    pmean(L, w, wm);
    psubtract(L, w, wm);
    if (body_force)
        for (int p = 0; p < 3; ++p) body_force[p] = mu[p];
    if (stats) {
        stats->iters = iters;
        stats->converged = conv;
        stats->nlevels = nlev;
        stats->bottom_fail = S.bottom_fail;
        stats->res0 = res0;
        stats->resfinal = rn;
        stats->target = target;
    }
    return conv ? 0 : 1;
}

}  // extern "C"

// ================================================================ Solver::Nonlocal::Newton<T>
// For the linear and affine models the kinematic variable is grad u and DW(grad u) =
// C : (grad u - F0) (src/Model/Solid/Linear/Cubic.H:64-67, src/Model/Solid/Affine/Cubic.H:38-41,
// src/Model/Solid/Affine/Isotropic.H:35-38); F0 = 0 for the Linear models.
namespace {

// GetStencil relative to an arbitrary box (src/Numeric/Stencil.H:12-34)
inline void box_stencil(const Box& b, int i, int j, int k, int st[3]) {
    const int c[3] = {i, j, k};
    for (int d = 0; d < 3; ++d) st[d] = (c[d] == b.lo[d]) ? ST_HI : (c[d] == b.hi[d]) ? ST_LO : ST_CEN;
}

inline void newton_grad(const Lev& L, const double* U, const int st[3], long c, double g[3][3]) {
    for (int p = 0; p < 3; ++p)
        for (int d = 0; d < 3; ++d) g[p][d] = D1(U + p * L.nn + c, L.stride(d), L.dx[d], st[d]);
}

// sig = DW(grad u) at node c
inline void newton_dw_node(const Lev& L, int model, const double* C, const double* F0, const double g[3][3], long c,
                           double sig[3][3]) {
    const int nc = ncoef_of(model);
    double a[kMaxCoef], e[3][3];
    for (int q = 0; q < nc; ++q) a[q] = C[q * L.nn + c];
    for (int p = 0; p < 3; ++p)
        for (int d = 0; d < 3; ++d) e[p][d] = g[p][d] - (F0 ? F0[(3 * p + d) * L.nn + c] : 0.0);
    stress_of(model, a, e, sig);
}

// Second half of Newton::prepareForSolve (src/Solver/Nonlocal/Newton.H:84-136): on
// grow(valid, 1) ∩ domain, rhs = b - BC(u, grad u, dw) on the domain boundary (BC faces
// classified against that box) and rhs = b - div(dw) by central differences inside.
void newton_rhs_from_dw(const Lev& L, const int* bctype, const double* u, const double* b, const double* dw,
                        double* rhs) {
    const Box bx1 = isect(isect(grow(L.valid, 1), L.dom), L.store);
    for_box(bx1, [&](int i, int j, int k) {
        const long c = L.at(i, j, k);
        const int m[3] = {i, j, k};
        bool bnd = false;
        for (int d = 0; d < 3; ++d) bnd = bnd || m[d] == L.dom.lo[d] || m[d] == L.dom.hi[d];
        if (bnd) {
            int st[3];
            box_stencil(bx1, i, j, k, st);
            double g[3][3], s[3][3], uu[3], nrm[3], f[3] = {0, 0, 0};
            newton_grad(L, u, st, c, g);
            for (int p = 0; p < 3; ++p) {
                uu[p] = u[p * L.nn + c];
                for (int d = 0; d < 3; ++d) s[p][d] = dw[(3 * p + d) * L.nn + c];
            }
            const int face = classify(bx1, i, j, k, nrm);
            if (face >= 0) bc_set(bctype + 3 * face, uu, g, s, nrm, f);
            for (int p = 0; p < 3; ++p) rhs[p * L.nn + c] = b[p * L.nn + c] - f[p];
        } else {
            for (int p = 0; p < 3; ++p) {
                const double* w0 = &dw[(3 * p + 0) * L.nn + c];
                const double* w1 = &dw[(3 * p + 1) * L.nn + c];
                const double* w2 = &dw[(3 * p + 2) * L.nn + c];
                rhs[p * L.nn + c] = b[p * L.nn + c] - ((w0[L.sx] - w0[-L.sx]) / 2. / L.dx[0] +
                                                       (w1[L.sy] - w1[-L.sy]) / 2. / L.dx[1] +
                                                       (w2[L.sz] - w2[-L.sz]) / 2. / L.dx[2]);
            }
        }
    });
}

}  // namespace

extern "C" {

// Newton::prepareForSolve (src/Solver/Nonlocal/Newton.H:30-139) on one box: dw = DW(grad u) on
// grow(valid, 2) ∩ domain, stencils one-sided at that box's faces; then rhs from dw as in
// newton_rhs_from_dw.  Nodes outside grow(valid, 1) ∩ domain keep rhs.
int orc_newton_residual(const orc_level* L0, int model, const double* C, const int* bctype, const double* u,
                        const double* b, const double* F0, double* rhs) {
    const Lev L(*L0);
    const Box bx2 = isect(isect(grow(L.valid, 2), L.dom), L.store);
    std::vector<double> dw(9 * L.nn, 0.0);
    for_box(bx2, [&](int i, int j, int k) {
        int st[3];
        box_stencil(bx2, i, j, k, st);
        const long c = L.at(i, j, k);
        double g[3][3], s[3][3];
        newton_grad(L, u, st, c, g);
        newton_dw_node(L, model, C, F0, g, c, s);
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) dw[(3 * p + d) * L.nn + c] = s[p][d];
    });
    newton_rhs_from_dw(L, bctype, u, b, dw.data(), rhs);
    return 0;
}

// The kinematic input of Newton::prepareForSolve for any model: grad u on grow(valid, 2) ∩ domain
// with the stencils one-sided at that box's faces (Newton.H:52-58), 9 components row-major
// (gradu(3 p + d) = du_p / dx_d).  Other nodes are not written.
int orc_newton_grad(const orc_level* L0, const double* u, double* gradu) {
    const Lev L(*L0);
    const Box bx2 = isect(isect(grow(L.valid, 2), L.dom), L.store);
    for_box(bx2, [&](int i, int j, int k) {
        int st[3];
        box_stencil(bx2, i, j, k, st);
        const long c = L.at(i, j, k);
        double g[3][3];
        newton_grad(L, u, st, c, g);
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) gradu[(3 * p + d) * L.nn + c] = g[p][d];
    });
    return 0;
}

// rhs = b - N(u) for a model whose DW the caller evaluated (e.g. a finite-kinematics model at
// F = I + grad u, Newton.H:70-75): dw holds 9 components over the storage box, set on
// grow(valid, 2) ∩ domain.
int orc_newton_residual_dw(const orc_level* L0, const int* bctype, const double* u, const double* b,
                           const double* dw, double* rhs) {
    const Lev L(*L0);
    newton_rhs_from_dw(L, bctype, u, b, dw, rhs);
    return 0;
}

// Newton::DW / Newton::W (src/Solver/Nonlocal/Newton.H:233-333) on the valid box, stencils
// relative to the domain.  dw: 9 components, row-major (dw(0) = sig(0,0), dw(1) = sig(0,1), ...).
// W(grad u) = 0.5 tr((G)^T C G), G = grad u - F0 (src/Model/Solid/Linear/Cubic.H:60-63,
// Affine/Cubic.H:34-37); Affine::Isotropic has no factor 0.5 (src/Model/Solid/Affine/Isotropic.H:31-34),
// applied when model is isotropic and F0 is given.
int orc_newton_dw(const orc_level* L0, int model, const double* C, const double* u, const double* F0, double* dw,
                  double* w) {
    const Lev L(*L0);
    const Box v = isect(L.valid, L.dom);
    const double half = (model == ORC_ISOTROPIC && F0) ? 1.0 : 0.5;
    for_box(v, [&](int i, int j, int k) {
        int st[3];
        get_stencil(L, i, j, k, st);
        const long c = L.at(i, j, k);
        double g[3][3], s[3][3];
        newton_grad(L, u, st, c, g);
        newton_dw_node(L, model, C, F0, g, c, s);
        if (dw)
            for (int p = 0; p < 3; ++p)
                for (int d = 0; d < 3; ++d) dw[(3 * p + d) * L.nn + c] = s[p][d];
        if (w) {
            double tr = 0.0;
            for (int p = 0; p < 3; ++p)
                for (int d = 0; d < 3; ++d) tr += (g[p][d] - (F0 ? F0[(3 * p + d) * L.nn + c] : 0.0)) * s[p][d];
            w[c] = half * tr;
        }
    });
    return 0;
}

}  // extern "C"
