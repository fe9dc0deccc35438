// Host-side declarations of the kernel launchers shared by the translation units of
// libaefast.so.  Each launcher is instantiated for R = double and R = float.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "ae_device.cuh"

namespace ae {

// kernels launched by this library (eager launches; graph replays are added by the solver)
extern std::atomic<long long> g_kernel_launches;
// message returned by ae_last_error() on the calling thread
void set_last_error(const std::string& msg);

inline Box3 box_grow(Box3 b, int n) {
    for (int d = 0; d < 3; ++d) { b.lo[d] -= n; b.hi[d] += n; }
    return b;
}
inline Box3 box_isect(const Box3& a, const Box3& b) {
    Box3 r;
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = a.lo[d] > b.lo[d] ? a.lo[d] : b.lo[d];
        r.hi[d] = a.hi[d] < b.hi[d] ? a.hi[d] : b.hi[d];
    }
    return r;
}
inline bool box_empty(const Box3& b) { return b.hi[0] < b.lo[0] || b.hi[1] < b.lo[1] || b.hi[2] < b.lo[2]; }
inline long long box_npts(const Box3& b) {
    if (box_empty(b)) return 0;
    return (long long)(b.hi[0] - b.lo[0] + 1) * (b.hi[1] - b.lo[1] + 1) * (b.hi[2] - b.lo[2] + 1);
}
inline bool box_contains(const Box3& outer, const Box3& inner) {
    for (int d = 0; d < 3; ++d)
        if (inner.lo[d] < outer.lo[d] || inner.hi[d] > outer.hi[d]) return false;
    return true;
}
inline Box3 geo_domain(const Geo& g) {
    Box3 b;
    for (int d = 0; d < 3; ++d) { b.lo[d] = g.dlo[d]; b.hi[d] = g.dhi[d]; }
    return b;
}
inline Box3 geo_valid(const Geo& g) {
    Box3 b;
    for (int d = 0; d < 3; ++d) { b.lo[d] = g.vlo[d]; b.hi[d] = g.vhi[d]; }
    return b;
}
inline Box3 geo_store(const Geo& g) { return box_grow(geo_valid(g), g.ng); }
// Fapply / Diagonal region: valid box grown by 1, clipped to the domain (Elastic.cpp:164-166)
inline Box3 geo_apply_region(const Geo& g) {
    return box_isect(box_isect(box_grow(geo_valid(g), 1), geo_domain(g)), geo_store(g));
}

template <class R>
SCoef<R> make_scoef(const Geo& g) {
    SCoef<R> K;
    for (int d = 0; d < 3; ++d) {
        K.h[d] = (R)(0.5 / g.dx[d]);
        K.id[d] = (R)(1.0 / g.dx[d]);
        K.i2[d] = (R)(1.0 / (g.dx[d] * g.dx[d]));
        K.bb[d] = (R)(-2.0 / g.dx[d] / g.dx[d]);
    }
    K.m01 = (R)(0.25 / (g.dx[0] * g.dx[1]));
    K.m02 = (R)(0.25 / (g.dx[0] * g.dx[2]));
    K.m12 = (R)(0.25 / (g.dx[1] * g.dx[2]));
    return K;
}

// View over a level's storage box (the layout of every internal array).
template <class T>
View<T> level_view(const Geo& g, T* p) {
    const Box3 s = geo_store(g);
    View<T> v;
    v.p = p;
    for (int d = 0; d < 3; ++d) v.lo[d] = s.lo[d];
    v.sy = g.px > 0 ? g.px : s.hi[0] - s.lo[0] + 1;
    v.sz = v.sy * (s.hi[1] - s.lo[1] + 1);
    v.sc = v.sz * (s.hi[2] - s.lo[2] + 1);
    v.wx = s.hi[0] - s.lo[0] + 1;
    return v;
}
// elements per component of a level's internal arrays (padding included)
inline long long geo_nn(const Geo& g) {
    const Box3 s = geo_store(g);
    if (box_empty(s)) return 0;
    const long long nx = g.px > 0 ? g.px : s.hi[0] - s.lo[0] + 1;
    return nx * (s.hi[1] - s.lo[1] + 1) * (s.hi[2] - s.lo[2] + 1);
}
template <class T>
View<const T> cview(const View<T>& v) {
    View<const T> c;
    c.p = v.p;
    for (int d = 0; d < 3; ++d) c.lo[d] = v.lo[d];
    c.sy = v.sy; c.sz = v.sz; c.sc = v.sc;
    c.wx = v.wx;
    return c;
}

struct OpParams {
    Geo g;
    BCP bc;
    int model;
    int uniform;
};

// ------------------------------------------------------------------ launchers
// G: the level's grain ids (laid out like C) and per-grain table, when the stiffness was given
// as a Voronoi map; the kernels then read those instead of C (same values).
template <class R>
void launch_fapply(const OpParams& P, View<const R> C, View<const R> u, View<R> f, cudaStream_t st,
                   Grains<R> G = Grains<R>{});
// r = b - A x over the apply region; if norm != nullptr, atomically max-reduce |r| over
// valid ∩ domain into *norm (bit pattern of a non-negative double, zero it first);
// if r32 != nullptr also store (float) r there.
template <class R>
void launch_residual(const OpParams& P, View<const R> C, View<const R> x, View<const R> b, View<R> r,
                     unsigned long long* norm, View<float>* r32, cudaStream_t st, Grains<R> G = Grains<R>{});
// One damped-Jacobi sweep: xo = (1-w) xi + w (b - (A xi - D xi)) / D on grow(valid,1)∩dom,
// zero on the ring grow(valid,2) \ grow(valid,1), copy elsewhere.
template <class R>
void launch_jacobi(const OpParams& P, View<const R> C, View<const R> invD, View<const R> D, View<const R> xi,
                   View<const R> b, View<R> xo, R omega, cudaStream_t st, Grains<R> G = Grains<R>{});
// Fapply (op 0), damped-Jacobi sweep (op 1) or residual (op 2) with the z-marching tiled
// kernel, on the level's internal storage views only.  tiled_init must have run once.
template <class R>
void launch_tiled(int op, const OpParams& P, View<const R> C, View<const R> x, View<const R> b, View<const R> invD,
                  View<const R> D, View<R> out, R omega, cudaStream_t st);
template <class R>
void tiled_init();
template <class R>
void launch_diagonal(const OpParams& P, View<const R> C, View<R> D, View<R> invD, int* nan_flag, cudaStream_t st);
// crse = R fine on `region` of coarse nodes (default: coarse valid ∩ domain); the weights
// depend on where a coarse node sits relative to the coarse domain boundary.
template <class R>
void launch_restrict(const Geo& gc, int ncomp, View<R> crse, View<const R> fine, cudaStream_t st,
                     const Box3* region = nullptr);
// fine += I crse on `region` of fine nodes (default: fine valid ∩ domain)
template <class R>
void launch_interp_add(const Geo& gf, int ncomp, View<R> fine, View<const R> crse, cudaStream_t st,
                       const Box3* region = nullptr);
// crse(I) = fine(2 I) on `region` of coarse nodes (nodal average_down)
template <class R>
void launch_inject(const Box3& region, int ncomp, View<R> crse, View<const R> fine, cudaStream_t st);
// region-wise copy/convert: dst(region) = src(region), component by component
template <class Ro, class Ri>
void launch_copy(const Box3& region, int ncomp, View<Ro> dst, View<const Ri> src, cudaStream_t st);
// dst += alpha * src over region
template <class Ro, class Ri>
void launch_axpy(const Box3& region, int ncomp, View<Ro> dst, double alpha, View<const Ri> src, cudaStream_t st);
template <class R>
void launch_fill(const Box3& region, int ncomp, View<R> dst, R value, cudaStream_t st);
// The first damped-Jacobi sweep from x = 0 over the level's storage box: every node as the full
// sweep leaves it for x = 0 (x_new = w b / D where the sweep updates, 0 elsewhere), no stencil.
template <class R>
void launch_jacobi_zero(const Geo& g, View<const R> invD, View<const R> D, View<const R> b, View<R> xo, R omega,
                        cudaStream_t st);
// max |v| over region into *norm (bit pattern)
template <class R>
void launch_norminf(const Box3& region, int ncomp, View<const R> v, unsigned long long* norm, cudaStream_t st);
void launch_bc_init(const Geo& g, const BCP& bc, const double* val, int homogeneous, View<double> rhs,
                    cudaStream_t st);
void launch_strain(const Geo& g, View<const double> u, View<double> e, int voigt, cudaStream_t st);
// rhs += r on the nodes of region not on the domain boundary (Linear::solveaffine)
void launch_affine_rhs(const Geo& g, const Box3& region, View<double> rhs, View<const double> r, cudaStream_t st);
void launch_stress(const OpParams& P, View<const double> C, View<const double> u, View<double> s, int voigt,
                   cudaStream_t st);
void launch_energy(const OpParams& P, View<const double> C, View<const double> u, View<double> w, cudaStream_t st);

// Newton<T>: rhs = b - N(u) (dw: 9-component scratch over the level's storage; F0.p may be null)
void launch_newton_residual(const OpParams& P, View<const double> C, View<const double> u, View<const double> b,
                            View<const double> F0, View<double> dw, View<double> rhs, cudaStream_t st);
// Newton::DW (dw.p may be null) and Newton::W (w.p may be null) on valid ∩ domain
void launch_newton_post(const OpParams& P, View<const double> C, View<const double> u, View<const double> F0,
                        View<double> dw, View<double> w, double half, cudaStream_t st);
// Newton<NeoHookean>: dw = DW(I + grad u) and C = DDW(I + grad u) (45 Sym::Major slots) on
// grow(valid, 2) ∩ domain, then rhs = b - N(u) on grow(valid, 1) ∩ domain
void launch_neohookean_residual(const OpParams& P, View<const double> u, View<const double> b, double mu,
                                double kappa, View<double> C, View<double> dw, View<double> rhs, cudaStream_t st);
// NeoHookean DW (dw.p may be null) and W (w.p may be null) on valid ∩ domain
void launch_neohookean_post(const Geo& g, View<const double> u, double mu, double kappa, View<double> dw,
                            View<double> w, cudaStream_t st);
// Voronoi stiffness over `region`: ids (int32 per node) -> gid (uint16) and the per-node FP64
// stiffness C = tab[id]; tab32 = (float) tab.  *bad is set if an id is outside [0, ng).
void launch_grains_box(const Box3& region, View<const int> ids, View<unsigned short> gid, View<double> C,
                       const double* tab, int ng, int nc, float* tab32, int* bad, cudaStream_t st);
// Phase-field mixture over `region` (nodes): eta is cell-centred with np components, tab np x nc,
// f0tab np x 9 (read only when F0.p is set).  *bad is set where the order parameters sum to zero.
void launch_model_mixture(const Box3& region, int nc, View<const double> eta, int np, const double* tab,
                          const double* f0tab, View<double> C, View<double> F0, int* bad, cudaStream_t st);
// Degraded isotropic stiffness over `region` (nodes); only nodes in `valid` read eta (cell-centred,
// neta components).  *bad is set where a cell mean lies outside [0, 1].
void launch_model_degraded(const Box3& region, const Box3& valid, View<const double> eta, int neta, double lam0,
                           double mu0, View<double> C, int* bad, cudaStream_t st);

struct BottomArgs {
    OpParams P;
    SCoef<double> K;
    const double* C;
    const double* D;
    const double* invD;
    double* x;
    const double* b;
    double* work;  // 8 vectors of 3 * nn doubles
    long long nn;
    int bottom;    // 0 CG, 1 BiCGStab
    int maxiter;
    double reltol;
    int nuf;
    int sweeps;
    double omega;
    int* fail_count;  // incremented when the Krylov solve fails
};
void launch_bottom(const BottomArgs& a, cudaStream_t st);
// mixed precision, refined patch gf (ghost layers >= 2): on the outermost ghost ring replace the
// FP32 correction just added to x by the coarse correction interpolated in FP64
void launch_ring_interp_fix(const Geo& gf, View<double> x, View<const float> ecrse, View<const float> efine,
                            cudaStream_t st);
// Coarsest-level operator assembled as an FP64 CSR matrix (rows = unknowns t + c nn), used by the
// bottom solve of the FP32 cycle.  The dense form comes first: column j of the row-major N x N
// matrix A is the operator applied to e_j (E: N x N scratch for the unit vectors).
struct BottomCsr {
    const int* rowptr;
    const int* col;
    const double* val;
    int nnz;
    // the nonzeros cut into chunks of at most kCsrChunk consecutive entries of one row: chunk c is
    // [cptr[c], cptr[c + 1]), the chunks of row r are [rch[r], rch[r + 1]) (null: none)
    const int* cptr = nullptr;
    const int* rch = nullptr;
    int nchunk = 0;
};
// nonzeros per chunk of the bottom's sparse product: one thread sums a chunk, then each row adds
// its chunks' sums, so a long row's dependent FP64 chain is a few chunks long, not the whole row
constexpr int kCsrChunk = 8;
void launch_bottom_assemble(const BottomArgs& a, double* A, double* E, cudaStream_t st);
void launch_bottom_csr(const BottomArgs& a, const BottomCsr& m, cudaStream_t st);
// unknowns up to which the coarsest level is assembled (dense scratch 2 N^2 doubles at set-up)
constexpr long long kBottomCsrMaxN = 1536;

}  // namespace ae
