// Kernel templates of the nodal elastic operator.  Included by ae_kernels_f64.cu and
// ae_kernels_f32.cu, each of which instantiates the launchers for one precision.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "ae_device.cuh"
#include "ae_launch.h"

namespace ae {

#define AE_CUDA_CHECK(x)                                                                         \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess)                                                                   \
            throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " \
                                     + __FILE__ + ":" + std::to_string(__LINE__));               \
    } while (0)

constexpr int kBlock = 256;

// Flattened iteration over a box: thread t -> (i, j, k), i fastest.
struct Reg {
    int lo[3];
    unsigned nx, nxy;
    unsigned n;
};
inline Reg make_reg(const Box3& b) {
    Reg r;
    for (int d = 0; d < 3; ++d) r.lo[d] = b.lo[d];
    if (box_empty(b)) { r.nx = r.nxy = 1; r.n = 0; return r; }
    r.nx = (unsigned)(b.hi[0] - b.lo[0] + 1);
    r.nxy = r.nx * (unsigned)(b.hi[1] - b.lo[1] + 1);
    r.n = r.nxy * (unsigned)(b.hi[2] - b.lo[2] + 1);
    return r;
}
__device__ __forceinline__ void reg_ijk(const Reg& r, unsigned t, int& i, int& j, int& k) {
    const unsigned kk = t / r.nxy;
    const unsigned rem = t - kk * r.nxy;
    const unsigned jj = rem / r.nx;
    i = r.lo[0] + (int)(rem - jj * r.nx);
    j = r.lo[1] + (int)jj;
    k = r.lo[2] + (int)kk;
}
inline unsigned nblocks(unsigned n) { return (n + kBlock - 1) / kBlock; }

// after every kernel launch: surface launch errors and count the launch
inline void launched() {
    AE_CUDA_CHECK(cudaGetLastError());
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);
}

__device__ __forceinline__ bool in_box(const int lo[3], const int hi[3], int i, int j, int k) {
    return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
}

// warp + block max of a non-negative double, then one atomicMax on its bit pattern
__device__ __forceinline__ void block_max_atomic(double v, unsigned long long* out) {
    __shared__ double sm[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (lane < (int)(blockDim.x >> 5)) ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
    }
}

// f = A u at one node: through the grain tables when the level has them (G.gid laid out like C),
// otherwise through the per-node stiffness C
// (GR: compiled for the grain tables, so each variant keeps its own register budget)
template <int M, class R, bool GR>
__device__ __forceinline__ void apply_any(const OpParams& P, const SCoef<R>& K, const View<const R>& C,
                                          const Grains<R>& G, const View<const R>& u, int i, int j, int k, R v[3]) {
    if constexpr (GR)
        apply_node_grains<M, R>(P.g, K, P.bc, P.uniform, G.gid, C.at(i, j, k), C.sy, C.sz, G.tab, u.p, u.sc,
                                u.at(i, j, k), u.sy, u.sz, i, j, k, v);
    else
        apply_node<M, R>(P.g, K, P.bc, P.uniform, C.p, C.sc, C.at(i, j, k), C.sy, C.sz, u.p, u.sc, u.at(i, j, k),
                         u.sy, u.sz, i, j, k, v);
}

// The same with the node's offsets given: oc into C (and the grain ids), ou into u
template <int M, class R, bool GR>
__device__ __forceinline__ void apply_at(const OpParams& P, const SCoef<R>& K, const View<const R>& C,
                                         const Grains<R>& G, const View<const R>& u, int i, int j, int k,
                                         long long oc, long long ou, R v[3]) {
    if constexpr (GR)
        apply_node_grains<M, R>(P.g, K, P.bc, P.uniform, G.gid, oc, C.sy, C.sz, G.tab, u.p, u.sc, ou, u.sy, u.sz, i,
                                j, k, v);
    else
        apply_node<M, R>(P.g, K, P.bc, P.uniform, C.p, C.sc, oc, C.sy, C.sz, u.p, u.sc, ou, u.sy, u.sz, i, j, k, v);
}

// true when two views index the same storage layout (same box origin and strides): the
// solver's level arrays all do, so one offset serves every array of a sweep
template <class A, class B>
inline bool same_layout(const View<A>& a, const View<B>& b) {
    return a.lo[0] == b.lo[0] && a.lo[1] == b.lo[1] && a.lo[2] == b.lo[2] && a.sy == b.sy && a.sz == b.sz &&
           a.sc == b.sc;
}

// Resident blocks per SM requested for the per-node sweeps.  The FP32 grain-map sweeps are
// bound by load latency: 5 blocks of 256 threads (48 registers) hide more of it than the 4
// (64 registers) the compiler picks by itself (257^3 Jacobi sweep 0.53 ms against 0.59 ms).
// 0: no request (the compiler's choice).
#ifndef AE_GRAIN_SWEEP_BLOCKS
#define AE_GRAIN_SWEEP_BLOCKS 5
#endif
#ifndef AE_PERNODE_SWEEP_BLOCKS
#define AE_PERNODE_SWEEP_BLOCKS 0
#endif
template <class R, bool GR>
constexpr int sweep_min_blocks() {
    return sizeof(R) != 4 ? 0 : GR ? AE_GRAIN_SWEEP_BLOCKS : AE_PERNODE_SWEEP_BLOCKS;
}

// ------------------------------------------------------------------ Fapply
template <int M, class R, bool GR>
__global__ void __launch_bounds__(kBlock) k_fapply(OpParams P, SCoef<R> K, Reg reg, View<const R> C, Grains<R> G,
                                                   View<const R> u, View<R> f) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    R v[3];
    apply_any<M, R, GR>(P, K, C, G, u, i, j, k, v);
    const long long o = f.at(i, j, k);
    f.p[o] = v[0];
    f.p[o + f.sc] = v[1];
    f.p[o + 2 * f.sc] = v[2];
}

// ------------------------------------------------------------------ residual (+ norm, + FP32 copy)
template <int M, class R, bool NORM, bool R32, bool GR, bool SAME>
__global__ void __launch_bounds__(kBlock, sweep_min_blocks<R, GR>()) k_residual(OpParams P, SCoef<R> K, Reg reg,
                                                                                 View<const R> C, Grains<R> G,
                                                                                 View<const R> x, View<const R> b,
                                                                                 View<R> r, unsigned long long* norm,
                                                                                 View<float> r32) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    double mx = 0.0;
    if (t < reg.n) {
        int i, j, k;
        reg_ijk(reg, t, i, j, k);
        R v[3];
        // SAME: every view has the layout of x (checked by the launcher)
        const long long ox = x.at(i, j, k);
        const long long oc = SAME ? ox : C.at(i, j, k);
        apply_at<M, R, GR>(P, K, C, G, x, i, j, k, oc, ox, v);
        const long long ob = SAME ? ox : b.at(i, j, k), orr = SAME ? ox : r.at(i, j, k);
        const long long o32 = SAME ? ox : (R32 ? r32.at(i, j, k) : 0);
        const long long bsc = SAME ? x.sc : b.sc, rsc = SAME ? x.sc : r.sc, r32sc = SAME ? x.sc : r32.sc;
        const bool inv = in_box(P.g.vlo, P.g.vhi, i, j, k);
#pragma unroll
        for (int n = 0; n < 3; ++n) {
            const R rv = b.p[ob + n * bsc] - v[n];
            r.p[orr + n * rsc] = rv;
            if (R32) r32.p[o32 + n * r32sc] = (float)rv;
            // a NaN residual reports an infinite norm (fmax alone would drop it)
            if (NORM && inv) mx = (rv != rv) ? (double)INFINITY : fmax(mx, (double)fabs(rv));
        }
    }
    if (NORM) block_max_atomic(mx, norm);
}

// ------------------------------------------------------------------ damped Jacobi sweep
// src/Operator/Operator.cpp:109-157 with the per-node Fapply fused in: one node (i, j, k).
// The damped-Jacobi update of one component: x_new from x, (A x), b, D and 1/D.
__device__ __forceinline__ double jacobi_update_impl(double xv, double ax, double b, double d, double invd,
                                                     double omega) {
    // the reference's update, (1-w) x + w (b - (Ax - D x)) / D (Operator.cpp:154)
    const double dx = xv * d;
    const double rx = ax - dx;
    return (1.0 - omega) * xv + omega * (b - rx) * invd;
}
__device__ __forceinline__ float jacobi_update_impl(float xv, float ax, float b, float, float invd, float omega) {
    // FP32 cycle: the same update written x + w (b - Ax) / D, which reads no D (rounded in one
    // fixed order, as the FP32 rows are)
    return __fmaf_rn(__fmul_rn(omega, __fsub_rn(b, ax)), invd, xv);
}
template <class R>
__device__ __forceinline__ R jacobi_update(R xv, R ax, R b, R d, R invd, R omega) {
    return jacobi_update_impl(xv, ax, b, d, invd, omega);
}

template <int M, class R, bool GR, bool SAME>
__device__ __forceinline__ void jacobi_node(const OpParams& P, const SCoef<R>& K, const View<const R>& C,
                                            const Grains<R>& G, const View<const R>& invD, const View<const R>& D,
                                            const View<const R>& xi, const View<const R>& b, const View<R>& xo,
                                            R omega, int i, int j, int k) {
    const Geo& g = P.g;
    // SAME: every view has the layout of xi (checked by the launcher)
    const long long ox = xi.at(i, j, k), oo = SAME ? ox : xo.at(i, j, k);
    const long long xsc = xi.sc, osc = SAME ? xsc : xo.sc;
    // outside the domain: untouched
    if (!in_box(g.dlo, g.dhi, i, j, k)) {
#pragma unroll
        for (int n = 0; n < 3; ++n) xo.p[oo + n * osc] = xi.p[ox + n * xsc];
        return;
    }
    // outermost ring of grow(valid, 2): zero
    if (g.ng >= 2 && (i == g.vlo[0] - 2 || i == g.vhi[0] + 2 || j == g.vlo[1] - 2 || j == g.vhi[1] + 2 ||
                      k == g.vlo[2] - 2 || k == g.vhi[2] + 2)) {
#pragma unroll
        for (int n = 0; n < 3; ++n) xo.p[oo + n * osc] = R(0);
        return;
    }
    R v[3];
    apply_at<M, R, GR>(P, K, C, G, xi, i, j, k, SAME ? ox : C.at(i, j, k), ox, v);
    const long long od = SAME ? ox : invD.at(i, j, k), ob = SAME ? ox : b.at(i, j, k);
    const long long dsc = SAME ? xsc : D.sc, isc = SAME ? xsc : invD.sc, bsc = SAME ? xsc : b.sc;
#pragma unroll
    for (int n = 0; n < 3; ++n)
        xo.p[oo + n * osc] = jacobi_update<R>(xi.p[ox + n * xsc], v[n], b.p[ob + n * bsc],
                                              sizeof(R) == 8 ? D.p[od + n * dsc] : R(0), invD.p[od + n * isc], omega);
}

// The first sweep of a smoother call whose correction starts at zero (the pre-smoothing of a
// V-cycle level, a patch's mini-cycle): A 0 = 0 on every row, interior and boundary, so the
// sweep needs no stencil.  Every node gets what jacobi_node gives it for x = 0 and A x = 0,
// through the same update with the zeros passed in at run time (zero == 0), so the arithmetic
// and its rounding are the full sweep's.
template <class R>
__global__ void __launch_bounds__(kBlock) k_jacobi_zero(Geo g, Reg reg, View<const R> invD, View<const R> D,
                                                        View<const R> b, View<R> xo, R omega, R zero) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const long long oo = xo.at(i, j, k);
    const bool ring = g.ng >= 2 && (i == g.vlo[0] - 2 || i == g.vhi[0] + 2 || j == g.vlo[1] - 2 || j == g.vhi[1] + 2 ||
                                    k == g.vlo[2] - 2 || k == g.vhi[2] + 2);
    if (!in_box(g.dlo, g.dhi, i, j, k) || ring) {
#pragma unroll
        for (int n = 0; n < 3; ++n) xo.p[oo + n * xo.sc] = zero;
        return;
    }
    const long long od = invD.at(i, j, k), ob = b.at(i, j, k);
#pragma unroll
    for (int n = 0; n < 3; ++n)
        xo.p[oo + n * xo.sc] = jacobi_update<R>(zero, zero, b.p[ob + n * b.sc], sizeof(R) == 8 ? D.p[od + n * D.sc] : R(0),
                                                invD.p[od + n * invD.sc], omega);
}

template <int M, class R, bool GR, bool SAME>
__global__ void __launch_bounds__(kBlock, sweep_min_blocks<R, GR>()) k_jacobi(OpParams P, SCoef<R> K, Reg reg,
                                                                               View<const R> C, Grains<R> G,
                                                                               View<const R> invD, View<const R> D,
                                                                               View<const R> xi, View<const R> b,
                                                                               View<R> xo, R omega) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    jacobi_node<M, R, GR, SAME>(P, K, C, G, invD, D, xi, b, xo, omega, i, j, k);
}

// ------------------------------------------------------------------ z-marching tiled stencil sweeps
// A block owns a TX x TY column of nodes and marches KZ planes in z.  Displacement planes and
// stiffness planes sit in shared-memory rings with a one-node halo in x and y, filled by
// asynchronous global->shared copies (cp.async) one plane ahead of the plane being computed,
// so HBM streams while the block computes.  The stiffness slots the z column of the grad C
// term needs at k-1 are kept in registers.  Every array element is read from global memory
// once per block (plus the halo), all reads coalesced along i.  Domain-boundary nodes (a thin
// shell) take the per-node path.  The views must be the level's internal storage views (halo
// copies are guarded by the storage box).
enum SweepOp { OP_FAPPLY = 0, OP_JACOBI = 1, OP_RESIDUAL = 2 };
constexpr int TX = 32, TY = 8, KZ = 32;
constexpr int HX = TX + 2, HY = TY + 2, HP = HX * HY;
constexpr int NU_SLOTS = 4, NC_SLOTS = 3;  // displacement planes k-1..k+2, stiffness planes k..k+2

template <int M, class R>
constexpr size_t tiled_smem_bytes() {
    return sizeof(R) * (size_t)(NU_SLOTS * 3 + NC_SLOTS * NCoef<M>::value) * HP;
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gsrc), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int M, class R, int OP>
__global__ void __launch_bounds__(TX* TY, 2) k_tiled(OpParams P, SCoef<R> K, Box3 box, View<const R> C,
                                                     View<const R> x, View<const R> b, View<const R> invD,
                                                     View<const R> D, View<R> out, R omega) {
    constexpr int NC = NCoef<M>::value;
    constexpr int NZ = ZSlots<M>::n;
    constexpr int NT = TX * TY;
    static_assert(NT < HP && HP <= 2 * NT, "each thread stages two halo positions per plane");
    extern __shared__ __align__(16) unsigned char smraw[];
    R* su = reinterpret_cast<R*>(smraw);  // [NU_SLOTS][3 comps][HP]
    R* sC = su + NU_SLOTS * 3 * HP;        // [NC_SLOTS][NC][HP]
    const Geo& g = P.g;
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int i0 = box.lo[0] + blockIdx.x * TX, j0 = box.lo[1] + blockIdx.y * TY;
    const int kbeg = box.lo[2] + blockIdx.z * KZ;
    const int kend = min(kbeg + KZ, box.hi[2] + 1);
    const int i = i0 + tx, j = j0 + ty;
    const bool active = i <= box.hi[0] && j <= box.hi[1];
    int slo[3], shi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) { slo[d] = g.vlo[d] - g.ng; shi[d] = g.vhi[d] + g.ng; }

    // the two halo positions this thread stages in every plane, their in-plane offsets and validity
    const int r0 = threadIdx.x, r1 = threadIdx.x + NT;
    const bool has1 = r1 < HP;
    auto xy_of = [&](int r, long long& ou, long long& oc, bool& ok) {
        const int hy = r / HX, hx = r - hy * HX;
        const int gi = i0 - 1 + hx, gj = j0 - 1 + hy;
        ok = gi >= slo[0] && gi <= shi[0] && gj >= slo[1] && gj <= shi[1];
        ou = (long long)(gi - x.lo[0]) + (long long)(gj - x.lo[1]) * x.sy;
        oc = (long long)(gi - C.lo[0]) + (long long)(gj - C.lo[1]) * C.sy;
    };
    long long ou0, oc0, ou1 = 0, oc1 = 0;
    bool ok0, ok1 = false;
    xy_of(r0, ou0, oc0, ok0);
    if (has1) xy_of(r1, ou1, oc1, ok1);
    // asynchronous copy of plane kk of a field into a ring slot (zeros where the halo leaves storage)
    auto stage = [&](const View<const R>& v, long long o0, long long o1, int ncomp, int kk, R* dst) {
        const bool kok = kk >= slo[2] && kk <= shi[2];
        const R* base = v.p + (long long)(kk - v.lo[2]) * v.sz;
        for (int c = 0; c < ncomp; ++c) {
            const R* src = base + (long long)c * v.sc;
            if (kok && ok0) cp_async<sizeof(R)>(dst + c * HP + r0, src + o0);
            else dst[c * HP + r0] = R(0);
            if (has1) {
                if (kok && ok1) cp_async<sizeof(R)>(dst + c * HP + r1, src + o1);
                else dst[c * HP + r1] = R(0);
            }
        }
    };
    auto uslot = [&](int kk) { return su + ((kk - kbeg + 1) & 3) * 3 * HP; };
    auto cslot = [&](int kk) { return sC + ((kk - kbeg) % NC_SLOTS) * NC * HP; };

    // prologue: planes k-1..k+1 (displacement) and k, k+1 (stiffness); then the lookahead plane
    stage(x, ou0, ou1, 3, kbeg - 1, uslot(kbeg - 1));
    stage(x, ou0, ou1, 3, kbeg, uslot(kbeg));
    stage(x, ou0, ou1, 3, kbeg + 1, uslot(kbeg + 1));
    stage(C, oc0, oc1, NC, kbeg, cslot(kbeg));
    stage(C, oc0, oc1, NC, kbeg + 1, cslot(kbeg + 1));
    cp_async_commit();
    stage(x, ou0, ou1, 3, kbeg + 2, uslot(kbeg + 2));
    stage(C, oc0, oc1, NC, kbeg + 2, cslot(kbeg + 2));
    cp_async_commit();
    R Cm[NZ];
    const bool km_ok = active && kbeg - 1 >= slo[2];
#pragma unroll
    for (int s = 0; s < NZ; ++s)
        Cm[s] = km_ok ? __ldg(C.p + C.at(i, j, kbeg - 1) + ZSlots<M>::at(s) * C.sc) : R(0);
    cp_async_wait<1>();
    __syncthreads();

    const int idx = (ty + 1) * HX + (tx + 1);
    for (int k = kbeg; k < kend; ++k) {
        const R* Uc = uslot(k);
        const R* Um = uslot(k - 1);
        const R* Up = uslot(k + 1);
        const R* Cc = cslot(k);
        const R* Cn = cslot(k + 1);
        if (active) {
            const long long oo = out.at(i, j, k);
            bool done = false;
            if (OP == OP_JACOBI) {
                if (!in_box(g.dlo, g.dhi, i, j, k)) {
#pragma unroll
                    for (int n = 0; n < 3; ++n) out.p[oo + n * out.sc] = Uc[n * HP + idx];
                    done = true;
                } else if (g.ng >= 2 && (i == g.vlo[0] - 2 || i == g.vhi[0] + 2 || j == g.vlo[1] - 2 ||
                                         j == g.vhi[1] + 2 || k == g.vlo[2] - 2 || k == g.vhi[2] + 2)) {
#pragma unroll
                    for (int n = 0; n < 3; ++n) out.p[oo + n * out.sc] = R(0);
                    done = true;
                }
            }
            if (!done) {
                R f[3];
                const bool interior = i > g.dlo[0] && i < g.dhi[0] && j > g.dlo[1] && j < g.dhi[1] &&
                                      k > g.dlo[2] && k < g.dhi[2];
                if (!interior) {
                    apply_node<M, R>(g, K, P.bc, P.uniform, C.p, C.sc, C.at(i, j, k), C.sy, C.sz, x.p, x.sc,
                                     x.at(i, j, k), x.sy, x.sz, i, j, k, f);
                } else {
                    R gu[3][3], bb[3][3][3];
#pragma unroll
                    for (int p = 0; p < 3; ++p) {
                        const R* u0 = Uc + p * HP + idx;
                        const R* um = Um + p * HP + idx;
                        const R* up = Up + p * HP + idx;
                        const R c0 = u0[0];
                        const R xm = u0[-1], xp = u0[1], ym = u0[-HX], yp = u0[HX], zm = um[0], zp = up[0];
                        gu[p][0] = (xp - xm) * K.h[0];
                        gu[p][1] = (yp - ym) * K.h[1];
                        gu[p][2] = (zp - zm) * K.h[2];
                        bb[p][0][0] = (xp - R(2) * c0 + xm) * K.i2[0];
                        bb[p][1][1] = (yp - R(2) * c0 + ym) * K.i2[1];
                        bb[p][2][2] = (zp - R(2) * c0 + zm) * K.i2[2];
                        bb[p][0][1] = (u0[1 + HX] + u0[-1 - HX] - u0[1 - HX] - u0[-1 + HX]) * K.m01;
                        bb[p][0][2] = (up[1] + um[-1] - um[1] - up[-1]) * K.m02;
                        bb[p][1][2] = (up[HX] + um[-HX] - um[HX] - up[-HX]) * K.m12;
                        bb[p][1][0] = bb[p][0][1];
                        bb[p][2][0] = bb[p][0][2];
                        bb[p][2][1] = bb[p][1][2];
                    }
                    R a[NC];
#pragma unroll
                    for (int q = 0; q < NC; ++q) a[q] = Cc[q * HP + idx];
                    div_of<M, R>(a, bb, f);
                    if (!P.uniform) {
                        R c0v[3], c1v[3], c2v[3];
                        gradC_col_f<M, R>([&](int q) { return Cc[q * HP + idx + 1] - Cc[q * HP + idx - 1]; }, gu, 0,
                                          c0v);
                        gradC_col_f<M, R>([&](int q) { return Cc[q * HP + idx + HX] - Cc[q * HP + idx - HX]; }, gu, 1,
                                          c1v);
                        gradC_col_f<M, R>([&](int q) { return Cn[q * HP + idx] - Cm[zslot_index<M>(q)]; }, gu, 2,
                                          c2v);
#pragma unroll
                        for (int r = 0; r < 3; ++r) f[r] = gradc_add(f[r], c0v[r], c1v[r], c2v[r], K.h);
                    }
                }
                if (OP == OP_FAPPLY) {
#pragma unroll
                    for (int n = 0; n < 3; ++n) out.p[oo + n * out.sc] = f[n];
                } else if (OP == OP_RESIDUAL) {
                    const long long ob = b.at(i, j, k);
#pragma unroll
                    for (int n = 0; n < 3; ++n) out.p[oo + n * out.sc] = b.p[ob + n * b.sc] - f[n];
                } else {
                    const long long ob = b.at(i, j, k), od = invD.at(i, j, k);
#pragma unroll
                    for (int n = 0; n < 3; ++n)
                        out.p[oo + n * out.sc] = jacobi_update<R>(Uc[n * HP + idx], f[n], b.p[ob + n * b.sc],
                                                                  sizeof(R) == 8 ? D.p[od + n * D.sc] : R(0),
                                                                  invD.p[od + n * invD.sc], omega);
                }
            }
        }
        // the stiffness of plane k becomes the k-1 plane of the next step
#pragma unroll
        for (int s = 0; s < NZ; ++s) Cm[s] = Cc[ZSlots<M>::at(s) * HP + idx];
        __syncthreads();  // every thread is done with the slots of planes k-1 (displacement) and k (stiffness)
        if (k + 1 < kend) {
            if (k + 3 <= kend) {  // the next lookahead plane reuses those slots
                stage(x, ou0, ou1, 3, k + 3, uslot(k + 3));
                stage(C, oc0, oc1, NC, k + 3, cslot(k + 3));
            }
            cp_async_commit();
            cp_async_wait<1>();  // plane k+2 has landed
            __syncthreads();
        }
    }
    cp_async_wait<0>();
}

// ------------------------------------------------------------------ Diagonal
// src/Operator/Elastic.cpp:285-350: the operator applied to a unit spike, component by component.
template <int M, class R>
__global__ void __launch_bounds__(kBlock) k_diagonal(OpParams P, SCoef<R> K, Reg reg, View<const R> C, View<R> D,
                                                     View<R> invD, int* nan_flag) {
    constexpr int NC = NCoef<M>::value;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const Geo& g = P.g;
    const long long cc = C.at(i, j, k), od = D.at(i, j, k);
    const int ci[3] = {i, j, k};
    bool mn[3], mx[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) { mn[d] = ci[d] == g.dlo[d]; mx[d] = ci[d] == g.dhi[d]; }
    R a[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) a[q] = C.p[cc + q * C.sc];
    R nrm[3];
    const int face = classify<R>(g, i, j, k, nrm);
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        R gu[3][3], bb[3][3][3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const R hi = (mx[d] && p == q) ? R(1) : R(0);
                const R lo = (mn[d] && p == q) ? R(1) : R(0);
                gu[q][d] = (hi - lo) / ((mn[d] || mx[d] ? R(1) : R(2)) * (R)g.dx[d]);
            }
#pragma unroll
            for (int l = 0; l < 3; ++l)
#pragma unroll
                for (int jj = 0; jj < 3; ++jj) bb[q][l][jj] = R(0);
#pragma unroll
            for (int d = 0; d < 3; ++d) bb[q][d][d] = (p == q) ? K.bb[d] : R(0);
        }
        R val;
        if (face >= 0) {
            const unsigned char tp = P.bc.t[face][p];
            if (tp == DISP) val = R(1);
            else if (tp == TRAC) {
                R s[3][3];
                stress_of<M, R>(a, gu, s);
                val = s[p][0] * nrm[0] + s[p][1] * nrm[1] + s[p][2] * nrm[2];
            } else if (tp == NEUMANN) val = gu[p][0] * nrm[0] + gu[p][1] * nrm[1] + gu[p][2] * nrm[2];
            else val = R(0);
        } else {
            R f[3];
            div_of<M, R>(a, bb, f);
            val = f[p];  // the grad C term multiplies grad u = 0 at interior nodes
        }
        D.p[od + p * D.sc] = val;
        invD.p[invD.at(i, j, k) + p * invD.sc] = R(1) / val;
        if (!(fabs((double)val) <= 1.0e300) || val == R(0)) atomicExch(nan_flag, 1);
    }
}

// ------------------------------------------------------------------ restriction / interpolation
// src/Operator/Operator.cpp:486-543 (coarse node I, fine node 2I)
template <class R>
__global__ void __launch_bounds__(kBlock) k_restrict(Geo gc, Reg reg, int ncomp, View<R> crse, View<const R> fine) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int I, J, Kc;
    reg_ijk(reg, t, I, J, Kc);
    const bool xe = I == gc.dlo[0] || I == gc.dhi[0];
    const bool ye = J == gc.dlo[1] || J == gc.dhi[1];
    const bool ze = Kc == gc.dlo[2] || Kc == gc.dhi[2];
    const long long sy = fine.sy, sz = fine.sz;
    for (int n = 0; n < ncomp; ++n) {
        const R* f = fine.p + fine.at(2 * I, 2 * J, 2 * Kc) + n * fine.sc;
        R v;
        if (xe && ye && ze) v = f[0];
        else if (ye && ze) v = R(0.25) * f[-1] + R(0.5) * f[0] + R(0.25) * f[1];
        else if (ze && xe) v = R(0.25) * f[-sy] + R(0.5) * f[0] + R(0.25) * f[sy];
        else if (xe && ye) v = R(0.25) * f[-sz] + R(0.5) * f[0] + R(0.25) * f[sz];
        else if (xe)
            v = (f[-sy - sz] + R(2) * f[-sz] + f[sy - sz] + R(2) * f[-sy] + R(4) * f[0] + R(2) * f[sy] + f[-sy + sz] +
                 R(2) * f[sz] + f[sy + sz]) * R(1.0 / 16.0);
        else if (ye)
            v = (f[-1 - sz] + R(2) * f[-1] + f[-1 + sz] + R(2) * f[-sz] + R(4) * f[0] + R(2) * f[sz] + f[1 - sz] +
                 R(2) * f[1] + f[1 + sz]) * R(1.0 / 16.0);
        else if (ze)
            v = (f[-1 - sy] + R(2) * f[-sy] + f[1 - sy] + R(2) * f[-1] + R(4) * f[0] + R(2) * f[1] + f[-1 + sy] +
                 R(2) * f[sy] + f[1 + sy]) * R(1.0 / 16.0);
        else
            v = (f[-1 - sy - sz] + f[-1 - sy + sz] + f[-1 + sy - sz] + f[-1 + sy + sz] + f[1 - sy - sz] +
                 f[1 - sy + sz] + f[1 + sy - sz] + f[1 + sy + sz]) * R(1.0 / 64.0) +
                (f[-sy - sz] + f[-sy + sz] + f[sy - sz] + f[sy + sz] + f[-1 - sz] + f[1 - sz] + f[-1 + sz] +
                 f[1 + sz] + f[-1 - sy] + f[-1 + sy] + f[1 - sy] + f[1 + sy]) * R(1.0 / 32.0) +
                (f[-1] + f[-sy] + f[-sz] + f[1] + f[sy] + f[sz]) * R(1.0 / 16.0) + f[0] * R(1.0 / 8.0);
        crse.p[crse.at(I, J, Kc) + n * crse.sc] = v;
    }
}

// src/Operator/Operator.cpp:589-618 (fine node (i,j,k), coarse node (i/2, j/2, k/2)): the
// coarse field interpolated to fine node (i, j, k), component n, in the arithmetic type T
template <class T, class R>
__device__ __forceinline__ T interp_at(const View<const R>& crse, int i, int j, int k, int n) {
    const int I = i >> 1, J = j >> 1, Kc = k >> 1;  // non-negative indices
    const bool ie = !(i & 1), je = !(j & 1), ke = !(k & 1);
    const long long sy = crse.sy, sz = crse.sz;
    const R* c = crse.p + crse.at(I, J, Kc) + n * crse.sc;
    const auto C = [&](long long o) { return (T)c[o]; };
    if (ie && je && ke) return C(0);
    if (je && ke) return T(0.5) * (C(0) + C(1));
    if (ke && ie) return T(0.5) * (C(0) + C(sy));
    if (ie && je) return T(0.5) * (C(0) + C(sz));
    if (ie) return T(0.25) * (C(0) + C(sy) + C(sz) + C(sy + sz));
    if (je) return T(0.25) * (C(0) + C(sz) + C(1) + C(1 + sz));
    if (ke) return T(0.25) * (C(0) + C(1) + C(sy) + C(1 + sy));
    return T(0.125) * (C(0) + C(1) + C(sy) + C(sz) + C(sy + sz) + C(1 + sz) + C(1 + sy) + C(1 + sy + sz));
}

// Interpolation added into the fine level (the same weights), one thread per coarse node
// (I, J, K) of the coarse box cb: it adds into the up to 8 fine nodes (2I + a, 2J + b, 2K + c),
// a, b, c in {0, 1}, that lie in the fine region fr.  The parity of each of those nodes is known
// at compile time, so a warp runs no divergent branches and the coarse values are loaded once
// for the 8 nodes.  Each node's value is the expression of interp_at for its parity.
template <class R>
__global__ void __launch_bounds__(kBlock) k_interp_add8(Reg cb, Box3 fr, int ncomp, View<R> fine,
                                                        View<const R> crse) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cb.n) return;
    int I, J, Kc;
    reg_ijk(cb, t, I, J, Kc);
    const long long sy = crse.sy, sz = crse.sz;
    const bool x1 = 2 * I + 1 <= fr.hi[0], y1 = 2 * J + 1 <= fr.hi[1], z1 = 2 * Kc + 1 <= fr.hi[2];
    const bool x0 = 2 * I >= fr.lo[0], y0 = 2 * J >= fr.lo[1], z0 = 2 * Kc >= fr.lo[2];
    for (int n = 0; n < ncomp; ++n) {
        const R* __restrict__ c = crse.p + crse.at(I, J, Kc) + n * crse.sc;
        R* __restrict__ f = fine.p + fine.at(2 * I, 2 * J, 2 * Kc) + n * fine.sc;
        const long long fy = fine.sy, fz = fine.sz;
        // (a, b, c) = (0, 0, 0): the coincident node
        if (x0 && y0 && z0) f[0] += c[0];
        if (x1 && y0 && z0) f[1] += R(0.5) * (c[0] + c[1]);
        if (x0 && y1 && z0) f[fy] += R(0.5) * (c[0] + c[sy]);
        if (x0 && y0 && z1) f[fz] += R(0.5) * (c[0] + c[sz]);
        if (x0 && y1 && z1) f[fy + fz] += R(0.25) * (c[0] + c[sy] + c[sz] + c[sy + sz]);
        if (x1 && y0 && z1) f[1 + fz] += R(0.25) * (c[0] + c[sz] + c[1] + c[1 + sz]);
        if (x1 && y1 && z0) f[1 + fy] += R(0.25) * (c[0] + c[1] + c[sy] + c[1 + sy]);
        if (x1 && y1 && z1)
            f[1 + fy + fz] +=
                R(0.125) * (c[0] + c[1] + c[sy] + c[sz] + c[sy + sz] + c[1 + sz] + c[1 + sy] + c[1 + sy + sz]);
    }
}

// nodal average_down (src/Operator/Operator.cpp:631): coarse node I takes fine node 2I
template <class R>
__global__ void __launch_bounds__(kBlock) k_inject(Reg reg, int ncomp, View<R> crse, View<const R> fine) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int I, J, Kc;
    reg_ijk(reg, t, I, J, Kc);
    const long long oc = crse.at(I, J, Kc), of = fine.at(2 * I, 2 * J, 2 * Kc);
    for (int n = 0; n < ncomp; ++n) crse.p[oc + n * crse.sc] = fine.p[of + n * fine.sc];
}

// ------------------------------------------------------------------ elementwise
template <class Ro, class Ri>
__global__ void __launch_bounds__(kBlock) k_copy(Reg reg, int ncomp, View<Ro> dst, View<const Ri> src) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const long long od = dst.at(i, j, k), os = src.at(i, j, k);
    for (int n = 0; n < ncomp; ++n) dst.p[od + n * dst.sc] = (Ro)src.p[os + n * src.sc];
}
template <class Ro, class Ri>
__global__ void __launch_bounds__(kBlock) k_axpy(Reg reg, int ncomp, View<Ro> dst, double alpha, View<const Ri> src) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const long long od = dst.at(i, j, k), os = src.at(i, j, k);
    for (int n = 0; n < ncomp; ++n) dst.p[od + n * dst.sc] += (Ro)(alpha * (double)src.p[os + n * src.sc]);
}
template <class R>
__global__ void __launch_bounds__(kBlock) k_fill(Reg reg, int ncomp, View<R> dst, R value) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= reg.n) return;
    int i, j, k;
    reg_ijk(reg, t, i, j, k);
    const long long od = dst.at(i, j, k);
    for (int n = 0; n < ncomp; ++n) dst.p[od + n * dst.sc] = value;
}
// Flat forms of copy / fill / axpy for a region that is the whole storage of its views (the
// common case: level-wide vectors): the components are one contiguous run of n values, so a
// grid-stride loop streams it with no index arithmetic.  ADD: alpha == 1, where the general form
// dst + (Ro)(1.0 * (double)src) is exactly dst + (Ro)src (no FP64 multiply).
template <class Ro, class Ri>
__global__ void __launch_bounds__(kBlock) k_flat_copy(long long n, Ro* __restrict__ dst, const Ri* __restrict__ src) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = (Ro)src[t];
}
template <class R>
__global__ void __launch_bounds__(kBlock) k_flat_fill(long long n, R* __restrict__ dst, R value) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[t] = value;
}
template <class Ro, class Ri, bool ADD>
__global__ void __launch_bounds__(kBlock) k_flat_axpy(long long n, Ro* __restrict__ dst, double alpha,
                                                      const Ri* __restrict__ src) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        if (ADD) dst[t] += (Ro)src[t];
        else dst[t] += (Ro)(alpha * (double)src[t]);
    }
}
// true when region, taken over ncomp components, covers whole rows and planes of v's storage
// from its first node, so that the elements from there on form one contiguous run (row padding
// included: padding is never read by the stencil kernels, and the level arrays hold it)
template <class T>
inline bool flat_view(const Reg& reg, int ncomp, const View<T>& v) {
    const long long w = v.wx > 0 ? v.wx : v.sy;
    const long long ny = reg.nxy / reg.nx, nz = reg.n / reg.nxy;
    return reg.n > 0 && reg.lo[0] == v.lo[0] && reg.lo[1] == v.lo[1] && reg.lo[2] == v.lo[2] &&
           (long long)reg.nx == w && ny * v.sy == v.sz && (ncomp == 1 || nz * v.sz == v.sc);
}
// elements of that contiguous run
template <class T>
inline long long flat_count(const Reg& reg, int ncomp, const View<T>& v) {
    const long long nz = reg.n / reg.nxy;
    return ncomp == 1 ? nz * v.sz : v.sc * ncomp;
}
// the same run in two views: same pitches
template <class A, class B>
inline bool same_pitch(const View<A>& a, const View<B>& b) {
    return a.sy == b.sy && a.sz == b.sz && a.sc == b.sc;
}
// grid of a flat loop: enough blocks to cover n, capped at 8 resident blocks per SM of 152
inline unsigned flat_blocks(long long n) {
    const long long b = (n + kBlock - 1) / kBlock;
    return (unsigned)(b < 152 * 8 ? b : 152 * 8);
}

// max-norm of a region: grid-stride over the nodes with a capped grid (kNormBlocks), so that a
// few thousand blocks, not one per 256 nodes, end in a barrier and an atomic
constexpr unsigned kNormBlocks = 152 * 8;
template <class R>
__global__ void __launch_bounds__(kBlock) k_norminf(Reg reg, int ncomp, View<const R> v, unsigned long long* out) {
    double mx = 0.0;
    for (unsigned long long t = blockIdx.x * blockDim.x + threadIdx.x; t < reg.n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        reg_ijk(reg, (unsigned)t, i, j, k);
        const long long o = v.at(i, j, k);
        for (int n = 0; n < ncomp; ++n) {
            const R a = v.p[o + n * v.sc];
            mx = (a != a) ? (double)INFINITY : fmax(mx, (double)fabs(a));
        }
    }
    block_max_atomic(mx, out);
}

// ------------------------------------------------------------------ launcher bodies
template <class R, class F>
inline void dispatch_model(int model, F&& f) {
    if (model == ISO) f(std::integral_constant<int, ISO>());
    else if (model == MM) f(std::integral_constant<int, MM>());
    else f(std::integral_constant<int, DIAG>());
}
// the box operator's kinds: the three above and the 45-slot Sym::Major tangent of a
// finite-kinematics model
template <class R, class F>
inline void dispatch_model4(int model, F&& f) {
    if (model == MAJOR) f(std::integral_constant<int, MAJOR>());
    else dispatch_model<R>(model, f);
}

}  // namespace ae
