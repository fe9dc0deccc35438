// Device functions of the periodic cell (homogenisation RVE): the interior row of
// Elastic<T>::Fapply (src/Operator/Elastic.cpp:216-255) at every node, neighbours taken
// modulo the cell, and the interior weights of the nodal transfers
// (src/Operator/Operator.cpp:527-541 restriction, :586-614 interpolation) with the same wrap.
// A cell stores n[0] n[1] n[2] unique nodes, no ghosts, index t = i + n0 (j + n1 k), components
// (and stiffness slots) nn apart.
#pragma once
#include "ae_device.cuh"

namespace ae {

// offsets from node t to its six face neighbours, wrapped into the cell
struct POff {
    int xp, xm, yp, ym, zp, zm;
};
__device__ __forceinline__ POff cell_offsets(const int n[3], int i, int j, int k) {
    const int sy = n[0], sz = n[0] * n[1];
    POff o;
    o.xp = (i == n[0] - 1) ? -(n[0] - 1) : 1;
    o.xm = (i == 0) ? (n[0] - 1) : -1;
    o.yp = (j == n[1] - 1) ? -(n[1] - 1) * sy : sy;
    o.ym = (j == 0) ? (n[1] - 1) * sy : -sy;
    o.zp = (k == n[2] - 1) ? -(n[2] - 1) * sz : sz;
    o.zm = (k == 0) ? (n[2] - 1) * sz : -sz;
    return o;
}
__device__ __forceinline__ void cell_ijk(const int n[3], int t, int& i, int& j, int& k) {
    const int sz = n[0] * n[1];
    k = t / sz;
    const int r = t - k * sz;
    j = r / n[0];
    i = r - j * n[0];
}

// central gradient and second derivatives of the three components of U at node t
template <class R>
__device__ __forceinline__ void cell_derivs(const SCoef<R>& K, const R* __restrict__ U, int us, int t, const POff& o,
                                            R gu[3][3], R b[3][3][3]) {
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const R* up = U + p * us + t;
        const R c0 = up[0];
        const R xm = up[o.xm], xp = up[o.xp], ym = up[o.ym], yp = up[o.yp], zm = up[o.zm], zp = up[o.zp];
        gu[p][0] = (xp - xm) * K.h[0];
        gu[p][1] = (yp - ym) * K.h[1];
        gu[p][2] = (zp - zm) * K.h[2];
        b[p][0][0] = (xp - R(2) * c0 + xm) * K.i2[0];
        b[p][1][1] = (yp - R(2) * c0 + ym) * K.i2[1];
        b[p][2][2] = (zp - R(2) * c0 + zm) * K.i2[2];
        b[p][0][1] = (up[o.xp + o.yp] + up[o.xm + o.ym] - up[o.xp + o.ym] - up[o.xm + o.yp]) * K.m01;
        b[p][0][2] = (up[o.xp + o.zp] + up[o.xm + o.zm] - up[o.xp + o.zm] - up[o.xm + o.zp]) * K.m02;
        b[p][1][2] = (up[o.yp + o.zp] + up[o.ym + o.zm] - up[o.yp + o.zm] - up[o.ym + o.zp]) * K.m12;
        b[p][1][0] = b[p][0][1];
        b[p][2][0] = b[p][0][2];
        b[p][2][1] = b[p][1][2];
    }
}

// sum_d column d of (d_d C) : g, central differences of C over the wrapped neighbours
template <int M, class R, bool LDG = true>
__device__ __forceinline__ void cell_gradC(const SCoef<R>& K, const R* __restrict__ C, int cs, int t, const POff& o,
                                           const R g[3][3], R out[3]) {
    const R* c0 = C + t;
    R c_x[3], c_y[3], c_z[3];
    gradC_col_f<M, R>([&](int q) { return ldv<LDG>(c0 + q * cs + o.xp) - ldv<LDG>(c0 + q * cs + o.xm); }, g, 0, c_x);
    gradC_col_f<M, R>([&](int q) { return ldv<LDG>(c0 + q * cs + o.yp) - ldv<LDG>(c0 + q * cs + o.ym); }, g, 1, c_y);
    gradC_col_f<M, R>([&](int q) { return ldv<LDG>(c0 + q * cs + o.zp) - ldv<LDG>(c0 + q * cs + o.zm); }, g, 2, c_z);
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r] = gradc_sum(c_x[r], c_y[r], c_z[r], K.h);
}

// f = A u at node t of a periodic cell
template <int M, class R, bool LDG = true>
__device__ __forceinline__ void cell_apply(const SCoef<R>& K, bool uniform, const R* __restrict__ C, int cs,
                                           const R* __restrict__ U, int us, int t, const POff& o, R f[3]) {
    constexpr int NC = NCoef<M>::value;
    R gu[3][3], b[3][3][3];
    cell_derivs<R>(K, U, us, t, o, gu, b);
    {
        R a[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) a[q] = ldv<LDG>(C + q * cs + t);
        div_of<M, R>(a, b, f);
    }
    if (!uniform) {
        R gc[3];
        cell_gradC<M, R, LDG>(K, C, cs, t, o, gu, gc);
#pragma unroll
        for (int r = 0; r < 3; ++r) f[r] += gc[r];
    }
}

// f = A u at node t of a Voronoi cell stored as a grain id per node and a per-grain coefficient
// table (tab[g * ncoef + q]).  The arithmetic is that of cell_apply on the equivalent per-node
// field; a direction whose two neighbours lie in the same grain has an exactly zero stiffness
// difference, so its column of the grad C term is zero and its loads are skipped.
template <int M, class R>
__device__ __forceinline__ void cell_apply_grains(const SCoef<R>& K, bool uniform,
                                                  const unsigned short* __restrict__ gid,
                                                  const R* __restrict__ tab, const R* __restrict__ U, int us, int t,
                                                  const POff& o, R f[3]) {
    constexpr int NC = NCoef<M>::value;
    R gu[3][3], b[3][3][3];
    cell_derivs<R>(K, U, us, t, o, gu, b);
    {
        const R* a0 = tab + (int)__ldg(gid + t) * NC;
        R a[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) a[q] = __ldg(a0 + q);
        div_of<M, R>(a, b, f);
    }
    if (!uniform) {
        const int gp[3] = {__ldg(gid + t + o.xp), __ldg(gid + t + o.yp), __ldg(gid + t + o.zp)};
        const int gm[3] = {__ldg(gid + t + o.xm), __ldg(gid + t + o.ym), __ldg(gid + t + o.zm)};
        R col[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (gp[d] == gm[d]) {
                col[d][0] = col[d][1] = col[d][2] = R(0);
            } else {
                const R* cp = tab + gp[d] * NC;
                const R* cm = tab + gm[d] * NC;
                gradC_col_f<M, R>([&](int q) { return __ldg(cp + q) - __ldg(cm + q); }, gu, d, col[d]);
            }
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) f[r] = gradc_add(f[r], col[0][r], col[1][r], col[2][r], K.h);
    }
}

// interior diagonal (src/Operator/Elastic.cpp:320-341): C_{pjpj} (-2 / dx_j^2)
template <int M, class R>
__device__ __forceinline__ void cell_diag(const SCoef<R>& K, const R* __restrict__ C, int cs, int t, R d[3]) {
    constexpr int NC = NCoef<M>::value;
    R a[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) a[q] = C[q * cs + t];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        R bb[3][3][3];
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
            for (int l = 0; l < 3; ++l)
#pragma unroll
                for (int jj = 0; jj < 3; ++jj) bb[q][l][jj] = (q == p && l == jj) ? K.bb[l] : R(0);
        R f[3];
        div_of<M, R>(a, bb, f);
        d[p] = f[p];
    }
}

// full weighting of fine component array F (fine cell nf) at coarse node (I,J,K)
template <class R>
__device__ __forceinline__ R cell_restrict(const R* __restrict__ F, const int nf[3], int I, int J, int K) {
    const int i = 2 * I, j = 2 * J, k = 2 * K;
    const int t = i + nf[0] * (j + nf[1] * k);
    const POff o = cell_offsets(nf, i, j, k);
    const int ox[3] = {o.xm, 0, o.xp}, oy[3] = {o.ym, 0, o.yp}, oz[3] = {o.zm, 0, o.zp};
    const R* f0 = F + t;
    auto f = [&](int a, int b, int c) { return f0[ox[a + 1] + oy[b + 1] + oz[c + 1]]; };
    return (f(-1, -1, -1) + f(-1, -1, +1) + f(-1, +1, -1) + f(-1, +1, +1) + f(+1, -1, -1) + f(+1, -1, +1) +
            f(+1, +1, -1) + f(+1, +1, +1)) / R(64) +
           (f(0, -1, -1) + f(0, -1, +1) + f(0, +1, -1) + f(0, +1, +1) + f(-1, 0, -1) + f(+1, 0, -1) + f(-1, 0, +1) +
            f(+1, 0, +1) + f(-1, -1, 0) + f(-1, +1, 0) + f(+1, -1, 0) + f(+1, +1, 0)) / R(32) +
           (f(-1, 0, 0) + f(0, -1, 0) + f(0, 0, -1) + f(+1, 0, 0) + f(0, +1, 0) + f(0, 0, +1)) / R(16) +
           f(0, 0, 0) / R(8);
}

// trilinear prolongation of coarse component array Cc (coarse cell nc) at fine node (i,j,k)
template <class R>
__device__ __forceinline__ R cell_interp(const R* __restrict__ Cc, const int nc[3], int i, int j, int k) {
    const int I = i >> 1, J = j >> 1, K = k >> 1;
    const int t = I + nc[0] * (J + nc[1] * K);
    const POff o = cell_offsets(nc, I, J, K);
    const R* c0 = Cc + t;
    auto c = [&](int a, int b, int d) { return c0[(a ? o.xp : 0) + (b ? o.yp : 0) + (d ? o.zp : 0)]; };
    const bool ie = (i & 1) == 0, je = (j & 1) == 0, ke = (k & 1) == 0;
    if (ie && je && ke) return c(0, 0, 0);
    if (je && ke) return R(0.5) * (c(0, 0, 0) + c(1, 0, 0));
    if (ke && ie) return R(0.5) * (c(0, 0, 0) + c(0, 1, 0));
    if (ie && je) return R(0.5) * (c(0, 0, 0) + c(0, 0, 1));
    if (ie) return R(0.25) * (c(0, 0, 0) + c(0, 1, 0) + c(0, 0, 1) + c(0, 1, 1));
    if (je) return R(0.25) * (c(0, 0, 0) + c(0, 0, 1) + c(1, 0, 0) + c(1, 0, 1));
    if (ke) return R(0.25) * (c(0, 0, 0) + c(1, 0, 0) + c(0, 1, 0) + c(1, 1, 0));
    return R(0.125) * (c(0, 0, 0) + c(1, 0, 0) + c(0, 1, 0) + c(0, 0, 1) + c(0, 1, 1) + c(1, 0, 1) + c(1, 1, 0) +
                       c(1, 1, 1));
}

}  // namespace ae
