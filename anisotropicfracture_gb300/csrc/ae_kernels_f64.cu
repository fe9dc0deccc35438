// FP64 instantiation of the operator kernels, plus the FP64-only kernels: boundary
// values, post-processing fields and the single-CTA bottom solver.
#include <type_traits>

#include "ae_kernels.cuh"
#include "ae_krylov.cuh"

#define AE_REAL double
#include "ae_kernels_common.inc"
#undef AE_REAL

namespace ae {

std::atomic<long long> g_kernel_launches{0};

AE_INST_COPY(double, double)
AE_INST_COPY(double, float)

// ------------------------------------------------------------------ BC::Operator::Elastic::Init
// src/BC/Operator/Elastic.H:106-181: boundary values into the rhs on every domain-boundary node.
struct BCVal {
    double v[26][3];
};
__global__ void __launch_bounds__(kBlock) k_bc_init(Geo g, BCP bc, BCVal val, int homogeneous, Reg reg,
                                                    View<double> rhs) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double n[3];
    const int face = classify<double>(g, i, j, k, n);
    if (face < 0) return;
    const long long o = rhs.at(i, j, k);
    for (int dir = 0; dir < 3; ++dir)
        rhs.p[o + dir * rhs.sc] = (homogeneous && bc.t[face][dir] == DISP) ? 0.0 : val.v[face][dir];
}
void launch_bc_init(const Geo& g, const BCP& bc, const double* val, int homogeneous, View<double> rhs,
                    cudaStream_t st) {
    const Box3 region = box_isect(box_grow(geo_valid(g), g.ng < 2 ? g.ng : 2), geo_domain(g));
    const Reg reg = make_reg(region);
    if (reg.n == 0) return;
    BCVal v;
    for (int f = 0; f < 26; ++f)
        for (int d = 0; d < 3; ++d) v.v[f][d] = val[3 * f + d];
    k_bc_init<<<nblocks(reg.n), kBlock, 0, st>>>(g, bc, v, homogeneous, reg, rhs);
    launched();
}

// ------------------------------------------------------------------ Voronoi stiffness
__global__ void __launch_bounds__(kBlock) k_grains_box(Reg reg, View<const int> ids, View<unsigned short> gid,
                                                       View<double> C, const double* __restrict__ tab, int ng, int nc,
                                                       int* bad) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const int id = ids.p[ids.at(i, j, k)];
    if (id < 0 || id >= ng) {
        atomicExch(bad, 1);
        return;
    }
    gid.p[gid.at(i, j, k)] = (unsigned short)id;
    const long long o = C.at(i, j, k);
    for (int q = 0; q < nc; ++q) C.p[o + q * C.sc] = tab[id * nc + q];
}
__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (float)a[t];
}
void launch_grains_box(const Box3& region, View<const int> ids, View<unsigned short> gid, View<double> C,
                       const double* tab, int ng, int nc, float* tab32, int* bad, cudaStream_t st) {
    const Reg reg = make_reg(region);
    if (reg.n > 0) {
        k_grains_box<<<nblocks(reg.n), kBlock, 0, st>>>(reg, ids, gid, C, tab, ng, nc, bad);
        launched();
    }
    k_to_float<<<(ng * nc + 255) / 256, 256, 0, st>>>(tab, tab32, ng * nc);
    launched();
}

// ------------------------------------------------------------------ stiffness from order parameters
// Phase-field mixture, src/Integrator/PhaseFieldMicrostructure.cpp:531-539 with
// Affine::Cubic::Combine (src/Model/Solid/Affine/Cubic.H:70-82): the weight of phase n at a node
// is its mean over the four cells (i-1..i, j-1..j) of cell layer k, divided by the sum of those
// means; stiffness slots and eigenstrain are the weighted sums of the per-phase tables.
template <int NC>
__global__ void __launch_bounds__(kBlock) k_model_mixture(Reg reg, View<const double> eta, int np,
                                                          const double* __restrict__ tab,
                                                          const double* __restrict__ f0tab, View<double> C,
                                                          View<double> F0, int* bad) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const long long o00 = eta.at(i, j, k), o01 = eta.at(i, j - 1, k);
    const long long o10 = eta.at(i - 1, j, k), o11 = eta.at(i - 1, j - 1, k);
    double sum = 0.0;
    for (int n = 0; n < np; ++n) {
        const double* e = eta.p + n * eta.sc;
        sum += 0.25 * (e[o00] + e[o01] + e[o10] + e[o11]);
    }
    if (sum == 0.0 || isnan(sum)) {
        atomicExch(bad, 1);
        return;
    }
    double acc[NC], f[9];
    for (int q = 0; q < NC; ++q) acc[q] = 0.0;
    for (int r = 0; r < 9; ++r) f[r] = 0.0;
    for (int n = 0; n < np; ++n) {
        const double* e = eta.p + n * eta.sc;
        const double w = 0.25 * (e[o00] + e[o01] + e[o10] + e[o11]) / sum;
        for (int q = 0; q < NC; ++q) acc[q] += tab[n * NC + q] * w;
        if (F0.p)
            for (int r = 0; r < 9; ++r) f[r] += f0tab[n * 9 + r] * w;
    }
    const long long o = C.at(i, j, k);
    for (int q = 0; q < NC; ++q) C.p[o + q * C.sc] = acc[q];
    if (F0.p) {
        const long long of = F0.at(i, j, k);
        for (int r = 0; r < 9; ++r) F0.p[of + r * F0.sc] = f[r];
    }
}
void launch_model_mixture(const Box3& region, int nc, View<const double> eta, int np, const double* tab,
                          const double* f0tab, View<double> C, View<double> F0, int* bad, cudaStream_t st) {
    const Reg reg = make_reg(region);
    if (reg.n == 0) return;
    if (nc == 2)
        k_model_mixture<2><<<nblocks(reg.n), kBlock, 0, st>>>(reg, eta, np, tab, f0tab, C, F0, bad);
    else if (nc == 9)
        k_model_mixture<9><<<nblocks(reg.n), kBlock, 0, st>>>(reg, eta, np, tab, f0tab, C, F0, bad);
    else
        k_model_mixture<21><<<nblocks(reg.n), kBlock, 0, st>>>(reg, eta, np, tab, f0tab, C, F0, bad);
    launched();
}

// Isotropic degradation, src/Integrator/PolymerDegradation.cpp:794-833 with
// Degradable::Isotropic::DegradeModulus (src/Model/Solid/LinearElastic/Degradable/Isotropic.H:74-81):
// every node starts undamaged; each valid node takes (lambda0 (1 - e), mu0 (1 - e)) with e the
// mean of an order parameter over the 8 cells around the node.  Each component is averaged and
// range-checked in turn and the last one is kept, as the reference's loop over components does.
__global__ void __launch_bounds__(kBlock) k_model_degraded(Reg reg, Box3 valid, View<const double> eta, int neta,
                                                           double lam0, double mu0, View<double> C, int* bad) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double lam = lam0, mu = mu0;
    const bool in_valid = i >= valid.lo[0] && i <= valid.hi[0] && j >= valid.lo[1] && j <= valid.hi[1] &&
                          k >= valid.lo[2] && k <= valid.hi[2];
    if (in_valid && neta > 0) {
        const long long c000 = eta.at(i, j, k), c100 = eta.at(i - 1, j, k);
        const long long c010 = eta.at(i, j - 1, k), c110 = eta.at(i - 1, j - 1, k);
        const long long c001 = eta.at(i, j, k - 1), c101 = eta.at(i - 1, j, k - 1);
        const long long c011 = eta.at(i, j - 1, k - 1), c111 = eta.at(i - 1, j - 1, k - 1);
        double e = 0.0;
        for (int n = 0; n < neta; ++n) {
            const double* p = eta.p + n * eta.sc;
            e = 0.125 * (p[c000] + p[c100] + p[c010] + p[c110] + p[c001] + p[c101] + p[c011] + p[c111]);
            if (!(e >= 0.0 && e <= 1.0)) {
                atomicExch(bad, 1);
                return;
            }
        }
        lam = lam0 * (1.0 - e);
        mu = mu0 * (1.0 - e);
    }
    const long long o = C.at(i, j, k);
    C.p[o] = lam;
    C.p[o + C.sc] = mu;
}
void launch_model_degraded(const Box3& region, const Box3& valid, View<const double> eta, int neta, double lam0,
                           double mu0, View<double> C, int* bad, cudaStream_t st) {
    const Reg reg = make_reg(region);
    if (reg.n == 0) return;
    k_model_degraded<<<nblocks(reg.n), kBlock, 0, st>>>(reg, valid, eta, neta, lam0, mu0, C, bad);
    launched();
}

// ------------------------------------------------------------------ Strain / Stress / Energy
// src/Operator/Elastic.cpp:399-572 (valid box, boundary-aware first derivatives)
__device__ __forceinline__ void grad_at(const Geo& g, const SCoef<double>& K, const View<const double>& u, int i,
                                        int j, int k, double gu[3][3]) {
    const int ci[3] = {i, j, k};
    const long long os[3] = {1, u.sy, u.sz};
    const long long o = u.at(i, j, k);
    for (int p = 0; p < 3; ++p) {
        const double* up = u.p + o + p * u.sc;
        for (int d = 0; d < 3; ++d) {
            const long long s = os[d];
            if (ci[d] == g.dlo[d]) gu[p][d] = (up[s] - up[0]) * K.id[d];
            else if (ci[d] == g.dhi[d]) gu[p][d] = (up[0] - up[-s]) * K.id[d];
            else gu[p][d] = (up[s] - up[-s]) * K.h[d];
        }
    }
}
__global__ void __launch_bounds__(kBlock) k_strain(Geo g, SCoef<double> K, Reg reg, View<const double> u,
                                                   View<double> e, int voigt) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double gu[3][3];
    grad_at(g, K, u, i, j, k, gu);
    double s[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) s[a][b] = 0.5 * (gu[a][b] + gu[b][a]);
    const long long o = e.at(i, j, k);
    if (voigt) {
        const double v[6] = {s[0][0], s[1][1], s[2][2], s[1][2], s[2][0], s[0][1]};
        for (int q = 0; q < 6; ++q) e.p[o + q * e.sc] = v[q];
    } else {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) e.p[o + (3 * a + b) * e.sc] = s[a][b];
    }
}
template <int M>
__global__ void __launch_bounds__(kBlock) k_stress(Geo g, SCoef<double> K, Reg reg, View<const double> C,
                                                   View<const double> u, View<double> sg, int voigt, int energy) {
    constexpr int NC = NCoef<M>::value;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double gu[3][3], s[3][3], a[NC];
    grad_at(g, K, u, i, j, k, gu);
    const long long cc = C.at(i, j, k);
    for (int q = 0; q < NC; ++q) a[q] = C.p[cc + q * C.sc];
    stress_of<M, double>(a, gu, s);
    const long long o = sg.at(i, j, k);
    if (energy) {
        // W(gradu) = trace(0.5 gradu^T (C gradu)), then += sum 0.5 sig:eps (Elastic.cpp:557-569)
        double w = 0.0;
        for (int ii = 0; ii < 3; ++ii) {
            double tt = 0.0;
            for (int jj = 0; jj < 3; ++jj) tt += gu[jj][ii] * s[jj][ii];
            w += 0.5 * tt;
        }
        for (int m = 0; m < 3; ++m)
            for (int n = 0; n < 3; ++n) w += .5 * s[m][n] * (.5 * (gu[m][n] + gu[n][m]));
        sg.p[o] = w;
    } else if (voigt) {
        const double v[6] = {s[0][0], s[1][1], s[2][2], s[1][2], s[2][0], s[0][1]};
        for (int q = 0; q < 6; ++q) sg.p[o + q * sg.sc] = v[q];
    } else {
        for (int a2 = 0; a2 < 3; ++a2)
            for (int b = 0; b < 3; ++b) sg.p[o + (3 * a2 + b) * sg.sc] = s[a2][b];
    }
}
void launch_strain(const Geo& g, View<const double> u, View<double> e, int voigt, cudaStream_t st) {
    const Reg reg = make_reg(box_isect(geo_valid(g), geo_domain(g)));
    if (reg.n == 0) return;
    k_strain<<<nblocks(reg.n), kBlock, 0, st>>>(g, make_scoef<double>(g), reg, u, e, voigt);
    launched();
}
void launch_stress(const OpParams& P, View<const double> C, View<const double> u, View<double> s, int voigt,
                   cudaStream_t st) {
    const Reg reg = make_reg(box_isect(geo_valid(P.g), geo_domain(P.g)));
    if (reg.n == 0) return;
    dispatch_model<double>(P.model, [&](auto m) {
        k_stress<decltype(m)::value><<<nblocks(reg.n), kBlock, 0, st>>>(P.g, make_scoef<double>(P.g), reg, C, u, s,
                                                                        voigt, 0);
    });
    launched();
}
void launch_energy(const OpParams& P, View<const double> C, View<const double> u, View<double> w, cudaStream_t st) {
    const Reg reg = make_reg(box_isect(geo_valid(P.g), geo_domain(P.g)));
    if (reg.n == 0) return;
    dispatch_model<double>(P.model, [&](auto m) {
        k_stress<decltype(m)::value><<<nblocks(reg.n), kBlock, 0, st>>>(P.g, make_scoef<double>(P.g), reg, C, u, w,
                                                                        0, 1);
    });
    launched();
}

// ------------------------------------------------------------------ Solver::Nonlocal::Newton<T>
// DW(grad u) = C : (grad u - F0) for the linear and affine models (kinematic variable grad u:
// src/Model/Solid/Linear/Cubic.H:64-67, src/Model/Solid/Affine/Cubic.H:38-41).
// grad u with Numeric::GetStencil relative to the box bx (one-sided on its faces).
__device__ __forceinline__ void grad_box(const Box3& bx, const SCoef<double>& K, const View<const double>& u, int i,
                                         int j, int k, double gu[3][3]) {
    const int ci[3] = {i, j, k};
    const long long os[3] = {1, u.sy, u.sz};
    const long long o = u.at(i, j, k);
    for (int p = 0; p < 3; ++p) {
        const double* up = u.p + o + p * u.sc;
        for (int d = 0; d < 3; ++d) {
            const long long s = os[d];
            if (ci[d] == bx.lo[d]) gu[p][d] = (up[s] - up[0]) * K.id[d];
            else if (ci[d] == bx.hi[d]) gu[p][d] = (up[0] - up[-s]) * K.id[d];
            else gu[p][d] = (up[s] - up[-s]) * K.h[d];
        }
    }
}
template <int M>
__device__ __forceinline__ void newton_sigma(const View<const double>& C, const View<const double>& F0, int i, int j,
                                             int k, double gu[3][3], double s[3][3]) {
    constexpr int NC = NCoef<M>::value;
    double a[NC];
    const long long cc = C.at(i, j, k);
    for (int q = 0; q < NC; ++q) a[q] = C.p[cc + q * C.sc];
    if (F0.p) {
        const long long of = F0.at(i, j, k);
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) gu[p][d] -= F0.p[of + (3 * p + d) * F0.sc];
    }
    stress_of<M, double>(a, gu, s);
}
// dw on bx2 = grow(valid, 2) ∩ domain (src/Solver/Nonlocal/Newton.H:45-76)
template <int M>
__global__ void __launch_bounds__(kBlock) k_newton_dw(SCoef<double> K, Reg reg, Box3 bx2, View<const double> C,
                                                      View<const double> u, View<const double> F0, View<double> dw) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double gu[3][3], s[3][3];
    grad_box(bx2, K, u, i, j, k, gu);
    newton_sigma<M>(C, F0, i, j, k, gu, s);
    const long long o = dw.at(i, j, k);
    for (int p = 0; p < 3; ++p)
        for (int d = 0; d < 3; ++d) dw.p[o + (3 * p + d) * dw.sc] = s[p][d];
}
// rhs on bx1 = grow(valid, 1) ∩ domain (src/Solver/Nonlocal/Newton.H:80-135): BC rows with
// sigma = dw on the domain boundary (faces classified against bx1), b - div(dw) inside
__global__ void __launch_bounds__(kBlock) k_newton_rhs(Geo g, BCP bc, SCoef<double> K, Reg reg, Box3 bx1,
                                                       View<const double> u, View<const double> b,
                                                       View<const double> dw, View<double> rhs) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const long long ob = b.at(i, j, k), orr = rhs.at(i, j, k), ow = dw.at(i, j, k);
    const bool bnd = i == g.dlo[0] || i == g.dhi[0] || j == g.dlo[1] || j == g.dhi[1] || k == g.dlo[2] ||
                     k == g.dhi[2];
    if (bnd) {
        double gu[3][3], s[3][3], n[3];
        grad_box(bx1, K, u, i, j, k, gu);
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) s[p][d] = dw.p[ow + (3 * p + d) * dw.sc];
        Geo gb = g;
        for (int d = 0; d < 3; ++d) { gb.dlo[d] = bx1.lo[d]; gb.dhi[d] = bx1.hi[d]; }
        const int face = classify<double>(gb, i, j, k, n);
        const long long ou = u.at(i, j, k);
        for (int r = 0; r < 3; ++r) {
            double v = 0.0;
            if (face >= 0) {
                const unsigned char tp = bc.t[face][r];
                if (tp == DISP) v = u.p[ou + r * u.sc];
                else if (tp == TRAC) v = s[r][0] * n[0] + s[r][1] * n[1] + s[r][2] * n[2];
                else if (tp == NEUMANN) v = gu[r][0] * n[0] + gu[r][1] * n[1] + gu[r][2] * n[2];
            }
            rhs.p[orr + r * rhs.sc] = b.p[ob + r * b.sc] - v;
        }
        return;
    }
    const long long os[3] = {1, dw.sy, dw.sz};
    for (int p = 0; p < 3; ++p) {
        double div = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double* w = dw.p + ow + (3 * p + d) * dw.sc;
            div += (w[os[d]] - w[-os[d]]) / 2. / g.dx[d];
        }
        rhs.p[orr + p * rhs.sc] = b.p[ob + p * b.sc] - div;
    }
}
// Newton::DW and Newton::W on valid ∩ domain, stencils relative to the domain
// (src/Solver/Nonlocal/Newton.H:233-333); half = 0.5, or 1 for Affine::Isotropic
// (src/Model/Solid/Affine/Isotropic.H:31-34)
template <int M>
__global__ void __launch_bounds__(kBlock) k_newton_post(Geo g, SCoef<double> K, Reg reg, View<const double> C,
                                                        View<const double> u, View<const double> F0, View<double> dw,
                                                        View<double> w, double half) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double gu[3][3], s[3][3];
    grad_at(g, K, u, i, j, k, gu);
    newton_sigma<M>(C, F0, i, j, k, gu, s);  // gu now holds grad u - F0
    if (dw.p) {
        const long long o = dw.at(i, j, k);
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) dw.p[o + (3 * p + d) * dw.sc] = s[p][d];
    }
    if (w.p) {
        double tr = 0.0;
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) tr += gu[p][d] * s[p][d];
        w.p[w.at(i, j, k)] = half * tr;
    }
}
void launch_newton_residual(const OpParams& P, View<const double> C, View<const double> u, View<const double> b,
                            View<const double> F0, View<double> dw, View<double> rhs, cudaStream_t st) {
    const Box3 bx2 = box_isect(box_isect(box_grow(geo_valid(P.g), 2), geo_domain(P.g)), geo_store(P.g));
    const Box3 bx1 = box_isect(box_isect(box_grow(geo_valid(P.g), 1), geo_domain(P.g)), geo_store(P.g));
    const SCoef<double> K = make_scoef<double>(P.g);
    const Reg r2 = make_reg(bx2), r1 = make_reg(bx1);
    if (r2.n == 0) return;
    dispatch_model<double>(P.model, [&](auto m) {
        k_newton_dw<decltype(m)::value><<<nblocks(r2.n), kBlock, 0, st>>>(K, r2, bx2, C, u, F0, dw);
    });
    launched();
    k_newton_rhs<<<nblocks(r1.n), kBlock, 0, st>>>(P.g, P.bc, K, r1, bx1, u, b, cview(dw), rhs);
    launched();
}
void launch_newton_post(const OpParams& P, View<const double> C, View<const double> u, View<const double> F0,
                        View<double> dw, View<double> w, double half, cudaStream_t st) {
    const Reg reg = make_reg(box_isect(geo_valid(P.g), geo_domain(P.g)));
    if (reg.n == 0) return;
    dispatch_model<double>(P.model, [&](auto m) {
        k_newton_post<decltype(m)::value><<<nblocks(reg.n), kBlock, 0, st>>>(P.g, make_scoef<double>(P.g), reg, C, u,
                                                                              F0, dw, w, half);
    });
    launched();
}

// ------------------------------------------------------------------ NeoHookean (finite kinematics)
// Model::Solid::Elastic::NeoHookean (src/Model/Solid/Elastic/NeoHookean.H:19-66) at F = I + grad u.
// G = F^-T is the signed cofactor matrix of F times 1 / det F; J23 = |det F|^(2/3); tr = F : F.
struct NeoKin {
    double F[3][3], G[3][3], J, J23, tr;
};
__device__ __forceinline__ void neo_kin(const double gu[3][3], NeoKin& n) {
    for (int p = 0; p < 3; ++p)
        for (int d = 0; d < 3; ++d) n.F[p][d] = gu[p][d] + (p == d ? 1.0 : 0.0);
    const auto& F = n.F;
    double cof[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            cof[i][j] = F[i1][j1] * F[i2][j2] - F[i1][j2] * F[i2][j1];
        }
    n.J = F[0][0] * cof[0][0] + F[1][0] * cof[1][0] + F[2][0] * cof[2][0];
    const double inv = 1.0 / n.J;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) n.G[i][j] = cof[i][j] * inv;
    n.J23 = pow(fabs(n.J), 2. / 3.);
    double tr = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tr += F[i][j] * F[i][j];
    n.tr = tr;
}
// NeoHookean::DW (NeoHookean.H:28-39): mu (F / J23 - tr G / (3 J23)) + kappa (J - 1) J G
__device__ __forceinline__ void neo_dw(const NeoKin& n, double mu, double kappa, double dw[3][3]) {
    const double a = kappa * (n.J - 1) * n.J;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            dw[i][j] = mu * (n.F[i][j] / n.J23 - n.tr * n.G[i][j] / (3. * n.J23)) + a * n.G[i][j];
}
// NeoHookean::DDW (NeoHookean.H:40-66) entry (i, j, k, l)
__device__ __forceinline__ double neo_ddw(const NeoKin& n, double mu, double kappa, int i, int j, int k, int l) {
    const auto& F = n.F;
    const auto& G = n.G;
    double t1 = 0.0, t2 = 0.0;
    if (i == k && j == l) t1 += 1.0;
    t1 -= (2. / 3.) * F[i][j] * G[k][l];
    t1 -= (2. / 3.) * G[i][j] * F[k][l];
    t1 += (2. / 9.) * n.tr * G[i][j] * G[k][l];
    t1 += (1. / 3.) * n.tr * G[i][l] * G[k][j];
    t2 += (2. * n.J - 1.) * G[i][j] * G[k][l];
    t2 += (1. - n.J) * G[i][l] * G[k][j];
    return (mu / n.J23) * t1 + kappa * n.J * t2;
}
// Newton::prepareForSolve with kinematic variable F (src/Solver/Nonlocal/Newton.H:45-76) on
// bx2 = grow(valid, 2) ∩ domain: dw = DW(F), and the level's stiffness C = DDW(F) in the 45
// Sym::Major slots.  The reference assigns ddw(i,j,k,l) in (i, j, k, l) order through the shared
// slot of A(3i+j, 3k+l) and A(3k+l, 3i+j), so each slot ends up holding the value evaluated with
// (i, j) the larger row index of the pair: that is the evaluation made here.
__global__ void __launch_bounds__(kBlock) k_neohookean(SCoef<double> K, Reg reg, Box3 bx2, View<const double> u,
                                                       double mu, double kappa, View<double> dw, View<double> C) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double gu[3][3], w[3][3];
    grad_box(bx2, K, u, i, j, k, gu);
    NeoKin n;
    neo_kin(gu, n);
    neo_dw(n, mu, kappa, w);
    const long long o = dw.at(i, j, k);
    for (int p = 0; p < 3; ++p)
        for (int d = 0; d < 3; ++d) dw.p[o + (3 * p + d) * dw.sc] = w[p][d];
    const long long oc = C.at(i, j, k);
#pragma unroll
    for (int I = 0; I < 9; ++I)
#pragma unroll
        for (int Kk = I; Kk < 9; ++Kk)
            C.p[oc + major_slot(I, Kk) * C.sc] = neo_ddw(n, mu, kappa, Kk / 3, Kk % 3, I / 3, I % 3);
}
// Newton::W and Newton::DW with kinematic variable F on valid ∩ domain, stencils relative to
// the domain (src/Solver/Nonlocal/Newton.H:233-333)
__global__ void __launch_bounds__(kBlock) k_neohookean_post(Geo g, SCoef<double> K, Reg reg, View<const double> u,
                                                            double mu, double kappa, View<double> dw,
                                                            View<double> w) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    double gu[3][3];
    grad_at(g, K, u, i, j, k, gu);
    NeoKin n;
    neo_kin(gu, n);
    if (dw.p) {
        double s[3][3];
        neo_dw(n, mu, kappa, s);
        const long long o = dw.at(i, j, k);
        for (int p = 0; p < 3; ++p)
            for (int d = 0; d < 3; ++d) dw.p[o + (3 * p + d) * dw.sc] = s[p][d];
    }
    // NeoHookean::W (NeoHookean.H:19-27)
    if (w.p) {
        double e = 0.0;
        e += 0.5 * mu * (n.tr / n.J23 - 3.);
        e += 0.5 * kappa * (n.J - 1.0) * (n.J - 1.0);
        w.p[w.at(i, j, k)] = e;
    }
}
void launch_neohookean_residual(const OpParams& P, View<const double> u, View<const double> b, double mu,
                                double kappa, View<double> C, View<double> dw, View<double> rhs, cudaStream_t st) {
    const Box3 bx2 = box_isect(box_isect(box_grow(geo_valid(P.g), 2), geo_domain(P.g)), geo_store(P.g));
    const Box3 bx1 = box_isect(box_isect(box_grow(geo_valid(P.g), 1), geo_domain(P.g)), geo_store(P.g));
    const SCoef<double> K = make_scoef<double>(P.g);
    const Reg r2 = make_reg(bx2), r1 = make_reg(bx1);
    if (r2.n == 0) return;
    k_neohookean<<<nblocks(r2.n), kBlock, 0, st>>>(K, r2, bx2, u, mu, kappa, dw, C);
    launched();
    k_newton_rhs<<<nblocks(r1.n), kBlock, 0, st>>>(P.g, P.bc, K, r1, bx1, u, b, cview(dw), rhs);
    launched();
}
void launch_neohookean_post(const Geo& g, View<const double> u, double mu, double kappa, View<double> dw,
                            View<double> w, cudaStream_t st) {
    const Reg reg = make_reg(box_isect(geo_valid(g), geo_domain(g)));
    if (reg.n == 0) return;
    k_neohookean_post<<<nblocks(reg.n), kBlock, 0, st>>>(g, make_scoef<double>(g), reg, u, mu, kappa, dw, w);
    launched();
}

// ------------------------------------------------------------------ bottom solve (one CTA)
// MLMG::actualBottomSolve + MLCGSolver::solve_cg / solve_bicgstab (krylov_bottom); the whole
// Krylov loop runs inside one thread block on the coarsest level (ng = 0, storage = domain).
// C, D and invD are either the level's global arrays or their copies in shared memory
// (SMEM = true: plain loads instead of __ldg).
template <int M, bool SMEM>
struct BottomOps {
    const BottomArgs& a;
    SCoef<double> K;
    View<const double> Cv;
    const double* D;
    const double* invD;
    int sy, sz, nn;  // the coarsest level is small: 32-bit index arithmetic
    int nx, ny, nz;
    __device__ BottomOps(const BottomArgs& aa, const double* C, const double* D_, const double* invD_)
        : a(aa), D(D_), invD(invD_) {
        K = aa.K;
        const Geo& g = aa.P.g;
        nx = g.vhi[0] - g.vlo[0] + 1;
        ny = g.vhi[1] - g.vlo[1] + 1;
        nz = g.vhi[2] - g.vlo[2] + 1;
        sy = nx;
        sz = nx * ny;
        nn = sz * nz;
        Cv.p = C;
        Cv.lo[0] = g.vlo[0]; Cv.lo[1] = g.vlo[1]; Cv.lo[2] = g.vlo[2];
        Cv.sy = sy; Cv.sz = sz; Cv.sc = nn;
    }
    // out = A x over every node
    __device__ void apply(const double* x, double* out, BlkRed&) const {
        const Geo& g = a.P.g;
        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
            const int k = t / sz, rem = t - k * sz;
            const int j = rem / nx, i = rem - j * nx;
            double v[3];
            apply_node<M, double, !SMEM>(g, K, a.P.bc, a.P.uniform, Cv.p, nn, t, sy, sz, x, nn, t, sy, sz,
                                         i + g.vlo[0], j + g.vlo[1], k + g.vlo[2], v);
            out[t] = v[0];
            out[t + nn] = v[1];
            out[t + 2 * nn] = v[2];
        }
        __syncthreads();
    }
    __device__ void residual(const double* x, const double* b, double* r, BlkRed& sh) const {
        apply(x, r, sh);
        for (int t = threadIdx.x; t < 3 * nn; t += blockDim.x) r[t] = b[t] - r[t];
        __syncthreads();
    }
    __device__ double dot(const double* x, const double* y, BlkRed& sh) const {
        double s = 0.0;
        for (int t = threadIdx.x; t < 3 * nn; t += blockDim.x) s += x[t] * y[t];
        return blk_sum(s, sh);
    }
    __device__ double ninf(const double* x, BlkRed& sh) const {
        double s = 0.0;
        for (int t = threadIdx.x; t < 3 * nn; t += blockDim.x) s = fmax(s, fabs(x[t]));
        return blk_max(s, sh);
    }
    // one Fsmooth call: a.sweeps damped-Jacobi sweeps (ng = 0: every node is updated)
    __device__ void smooth(double* x, const double* b, double* tmp, BlkRed& sh) const {
        for (int s = 0; s < a.sweeps; ++s) {
            apply(x, tmp, sh);
            for (int t = threadIdx.x; t < 3 * nn; t += blockDim.x) {
                const double xv = x[t];
                const double rx = tmp[t] - xv * D[t];
                x[t] = (1.0 - a.omega) * xv + a.omega * (b[t] - rx) * invD[t];
            }
            __syncthreads();
        }
    }
};

// SMEM = true: the whole level (C, D, invD, b, x and the 8 work vectors, bottom_smem_doubles)
// lives in dynamic shared memory; x is copied back at the end.
template <int M, bool SMEM>
__global__ void __launch_bounds__(kBottomThreads) k_bottom(BottomArgs a) {
    __shared__ BlkRed sh;
    extern __shared__ double smem[];
    constexpr int NC = NCoef<M>::value;
    const int N = (int)(3 * a.nn);
    const double* Cp = a.C;
    const double* Dp = a.D;
    const double* invDp = a.invD;
    double* x = a.x;
    const double* b = a.b;
    double* work = a.work;
    if (SMEM) {
        double* sC = smem;
        double* sD = sC + NC * a.nn;
        double* sI = sD + N;
        double* sb = sI + N;
        double* sx = sb + N;
        for (long long t = threadIdx.x; t < NC * a.nn; t += blockDim.x) sC[t] = a.C[t];
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            sD[t] = a.D[t];
            sI[t] = a.invD[t];
            sb[t] = a.b[t];
            sx[t] = a.x[t];
        }
        __syncthreads();
        Cp = sC; Dp = sD; invDp = sI; b = sb; x = sx;
        work = sx + N;
    }
    const BottomOps<M, SMEM> ops(a, Cp, Dp, invDp);
    const KrylovParams kp{a.bottom, a.maxiter, a.reltol, a.nuf};
    const int ret = krylov_bottom(ops, kp, N, x, b, work, sh);
    if (ret != 0 && ret != 9 && threadIdx.x == 0 && a.fail_count) atomicAdd(a.fail_count, 1);
    if (SMEM) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) a.x[t] = x[t];
    }
}

// doubles of dynamic shared memory the SMEM variant needs for nn nodes
__host__ __device__ constexpr long long bottom_smem_doubles(int nc, long long nn) { return (nc + 36) * nn; }

// Levels whose arrays fit the default 48 KB of dynamic shared memory (no function attribute,
// so the launch is legal inside stream capture) run from shared memory; larger ones from global.
void launch_bottom(const BottomArgs& a, cudaStream_t st) {
    dispatch_model4<double>(a.P.model, [&](auto m) {
        constexpr int Mv = decltype(m)::value;
        const size_t bytes = (size_t)bottom_smem_doubles(NCoef<Mv>::value, a.nn) * sizeof(double);
        if (bytes <= kBottomSmemBytes) k_bottom<Mv, true><<<1, kBottomThreads, bytes, st>>>(a);
        else k_bottom<Mv, false><<<1, kBottomThreads, 0, st>>>(a);
    });
    launched();
}

// Mixed precision on a refined patch: the FP32 correction e was just added to the FP64 solution
// x.  The outermost ghost ring of the patch (grow(valid, 2)) has no equation of its own; in the
// FP64 solve it only ever receives coarse corrections interpolated to it, so there it equals the
// interpolation of the coarse solution.  The FP32 cycle interpolates in FP32, and its rounding
// would stay in the ring (nothing corrects it) and bias the interface rows.  Here the ring's
// increment is replaced by the coarse FP32 correction interpolated in FP64:
//   x_ring += interp(e_coarse) - e_ring.
__global__ void __launch_bounds__(kBlock) k_ring_interp_fix(Reg reg, Geo gf, View<double> x, View<const float> ecrse,
                                                            View<const float> efine) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const bool ring = i == gf.vlo[0] - 2 || i == gf.vhi[0] + 2 || j == gf.vlo[1] - 2 || j == gf.vhi[1] + 2 ||
                      k == gf.vlo[2] - 2 || k == gf.vhi[2] + 2;
    if (!ring) return;
    for (int n = 0; n < 3; ++n) {
        const double v = interp_at<double, float>(ecrse, i, j, k, n);
        x.p[x.at(i, j, k) + n * x.sc] += v - (double)efine.p[efine.at(i, j, k) + n * efine.sc];
    }
}

void launch_ring_interp_fix(const Geo& gf, View<double> x, View<const float> ecrse, View<const float> efine,
                            cudaStream_t st) {
    if (gf.ng < 2) return;
    const Reg reg = make_reg(box_isect(geo_store(gf), geo_domain(gf)));
    if (reg.n == 0) return;
    k_ring_interp_fix<<<nblocks(reg.n), kBlock, 0, st>>>(reg, gf, x, ecrse, efine);
    launched();
}

// ------------------------------------------------------------------ assembled bottom operator
// The coarsest level's operator as an explicit FP64 matrix, for the bottom solve of the FP32
// cycle.  GB300 issues FP64 at a small fraction of its FP32 rate, and the stencil form of the
// level operator costs a few hundred FP64 instructions per node on one SM; the assembled rows
// cost one FMA per nonzero.  Column j is the operator applied to the unit vector e_j (so every
// entry is the stencil's own coefficient sum for that pair of unknowns); the host compresses
// the columns to CSR.  The FP64 solve keeps the stencil form (its bottom follows the reference
// operation for operation).

// block j: column j of the dense N x N matrix A (row-major); E holds one unit vector per block
template <int M>
__global__ void __launch_bounds__(128) k_bottom_assemble(BottomArgs a, double* A, double* E) {
    const long long nn = a.nn, N = 3 * nn;
    const long long j = blockIdx.x;
    double* e = E + j * N;
    for (int t = threadIdx.x; t < N; t += blockDim.x) e[t] = (t == j) ? 1.0 : 0.0;
    __syncthreads();
    const Geo& g = a.P.g;
    const int nx = g.vhi[0] - g.vlo[0] + 1, ny = g.vhi[1] - g.vlo[1] + 1;
    const long long sy = nx, sz = (long long)nx * ny;
    for (long long t = threadIdx.x; t < nn; t += blockDim.x) {
        const int k = (int)(t / sz), rem = (int)(t - (long long)k * sz);
        const int jj = rem / nx, i = rem - jj * nx;
        double v[3];
        apply_node<M, double, true>(g, a.K, a.P.bc, a.P.uniform, a.C, nn, t, sy, sz, e, nn, t, sy, sz, i + g.vlo[0],
                                    jj + g.vlo[1], k + g.vlo[2], v);
        A[t * N + j] = v[0];
        A[(t + nn) * N + j] = v[1];
        A[(t + 2 * nn) * N + j] = v[2];
    }
}
void launch_bottom_assemble(const BottomArgs& a, double* A, double* E, cudaStream_t st) {
    dispatch_model4<double>(a.P.model, [&](auto m) {
        k_bottom_assemble<decltype(m)::value><<<(unsigned)(3 * a.nn), 128, 0, st>>>(a, A, E);
    });
    launched();
}

// Krylov operations over the CSR rows (fixed order: deterministic).  With chunks (part != null)
// a thread sums the products of a chunk into part[], then a thread per row adds its chunks in
// order; else one thread per row.
struct CsrOps {
    const BottomArgs& a;
    const int* rowptr;
    const int* col;
    const double* val;
    int N;
    const int* cptr = nullptr;
    const int* rch = nullptr;
    double* part = nullptr;
    int nchunk = 0;
    __device__ void apply(const double* x, double* out, BlkRed&) const {
        if (part) {
            for (int c = threadIdx.x; c < nchunk; c += blockDim.x) {
                double s = 0.0;
                for (int q = cptr[c]; q < cptr[c + 1]; ++q) s += val[q] * x[col[q]];
                part[c] = s;
            }
            __syncthreads();
            for (int r = threadIdx.x; r < N; r += blockDim.x) {
                double s = part[rch[r]];
                for (int c = rch[r] + 1; c < rch[r + 1]; ++c) s += part[c];
                out[r] = s;
            }
        } else {
            for (int r = threadIdx.x; r < N; r += blockDim.x) {
                double s = 0.0;
                for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) s += val[q] * x[col[q]];
                out[r] = s;
            }
        }
        __syncthreads();
    }
    __device__ void residual(const double* x, const double* b, double* r, BlkRed& sh) const {
        apply(x, r, sh);
        for (int t = threadIdx.x; t < N; t += blockDim.x) r[t] = b[t] - r[t];
        __syncthreads();
    }
    __device__ double dot(const double* x, const double* y, BlkRed& sh) const {
        double s = 0.0;
        for (int t = threadIdx.x; t < N; t += blockDim.x) s += x[t] * y[t];
        return blk_sum(s, sh);
    }
    __device__ double ninf(const double* x, BlkRed& sh) const {
        double s = 0.0;
        for (int t = threadIdx.x; t < N; t += blockDim.x) s = fmax(s, fabs(x[t]));
        return blk_max(s, sh);
    }
    // one Fsmooth call with the level's FP64 diagonal (the same update as the stencil form)
    __device__ void smooth(double* x, const double* b, double* tmp, BlkRed& sh) const {
        for (int s = 0; s < a.sweeps; ++s) {
            apply(x, tmp, sh);
            for (int t = threadIdx.x; t < N; t += blockDim.x) {
                const double xv = x[t];
                const double rx = tmp[t] - xv * a.D[t];
                x[t] = (1.0 - a.omega) * xv + a.omega * (b[t] - rx) * a.invD[t];
            }
            __syncthreads();
        }
    }
};

// the matrix and the vectors in dynamic shared memory when they fit (SMEM), else from global
template <bool SMEM>
__global__ void __launch_bounds__(kBottomThreads) k_bottom_csr(BottomArgs a, BottomCsr m) {
    __shared__ BlkRed sh;
    extern __shared__ double smem[];
    const int N = (int)(3 * a.nn);
    double* x = a.x;
    const double* b = a.b;
    double* work = a.work;
    const int* rowptr = m.rowptr;
    const int* col = m.col;
    const double* val = m.val;
    if (SMEM) {
        double* sval = smem;
        double* sb = sval + m.nnz;
        double* sx = sb + N;
        double* sw = sx + N;
        double* spart = sw + 8 * N;
        int* srow = reinterpret_cast<int*>(spart + (m.cptr ? m.nchunk : 0));
        int* scol = srow + N + 1;
        int* scp = scol + m.nnz;
        int* src = scp + m.nchunk + 1;
        for (long long t = threadIdx.x; t < m.nnz; t += blockDim.x) { sval[t] = m.val[t]; scol[t] = m.col[t]; }
        for (long long t = threadIdx.x; t <= N; t += blockDim.x) srow[t] = m.rowptr[t];
        for (int t = threadIdx.x; t < N; t += blockDim.x) { sb[t] = a.b[t]; sx[t] = a.x[t]; }
        if (m.cptr) {
            for (int t = threadIdx.x; t <= m.nchunk; t += blockDim.x) scp[t] = m.cptr[t];
            for (int t = threadIdx.x; t <= N; t += blockDim.x) src[t] = m.rch[t];
        }
        __syncthreads();
        rowptr = srow; col = scol; val = sval; b = sb; x = sx; work = sw;
        if (m.cptr) {
            const CsrOps ops{a, rowptr, col, val, N, scp, src, spart, m.nchunk};
            const KrylovParams kp{a.bottom, a.maxiter, a.reltol, a.nuf};
            const int ret = krylov_bottom(ops, kp, N, x, b, work, sh);
            if (ret != 0 && ret != 9 && threadIdx.x == 0 && a.fail_count) atomicAdd(a.fail_count, 1);
            for (int t = threadIdx.x; t < N; t += blockDim.x) a.x[t] = x[t];
            return;
        }
    }
    const CsrOps ops{a, rowptr, col, val, N};
    const KrylovParams kp{a.bottom, a.maxiter, a.reltol, a.nuf};
    const int ret = krylov_bottom(ops, kp, N, x, b, work, sh);
    if (ret != 0 && ret != 9 && threadIdx.x == 0 && a.fail_count) atomicAdd(a.fail_count, 1);
    if (SMEM) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) a.x[t] = x[t];
    }
}

size_t bottom_csr_smem_bytes(long long N, long long nnz, long long nchunk) {
    return (size_t)(nnz + 10 * N + nchunk) * sizeof(double) + (size_t)(N + 1 + nnz + nchunk + 1 + N + 1) * sizeof(int);
}

// one thread per row or chunk, rounded up to whole warps
void launch_bottom_csr(const BottomArgs& a, const BottomCsr& m, cudaStream_t st) {
    const int N = (int)(3 * a.nn);
    const int threads = (int)std::min<long long>(kBottomThreads, (std::max(N, m.nchunk) + 31) / 32 * 32);
    const size_t bytes = bottom_csr_smem_bytes(N, m.nnz, m.cptr ? m.nchunk : 0);
    if (bytes <= kBottomSmemBytes) k_bottom_csr<true><<<1, threads, bytes, st>>>(a, m);
    else k_bottom_csr<false><<<1, threads, 0, st>>>(a, m);
    launched();
}

// Linear::solveaffine's right-hand side (src/Solver/Nonlocal/Linear.H:62-89): with r = 0 - A 0,
// the negated apply of zero, rhs += r on nodes inside the domain, nothing on its boundary.
__global__ void __launch_bounds__(kBlock) k_affine_rhs(Geo g, Reg reg, View<double> rhs, View<const double> r) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    if (i == g.dlo[0] || i == g.dhi[0] || j == g.dlo[1] || j == g.dhi[1] || k == g.dlo[2] || k == g.dhi[2]) return;
    const long long o = rhs.at(i, j, k), q = r.at(i, j, k);
#pragma unroll
    for (int n = 0; n < 3; ++n) rhs.p[o + n * rhs.sc] += r.p[q + n * r.sc];
}
void launch_affine_rhs(const Geo& g, const Box3& region, View<double> rhs, View<const double> r, cudaStream_t st) {
    const Reg reg = make_reg(region);
    if (reg.n == 0) return;
    k_affine_rhs<<<nblocks(reg.n), kBlock, 0, st>>>(g, reg, rhs, r);
    launched();
}

}  // namespace ae
