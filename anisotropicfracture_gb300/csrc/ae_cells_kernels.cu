// Kernels of the batched periodic-cell solve.  Every stencil kernel walks a work table with a
// grid-stride loop (a persistent grid sized by the tuner); each entry is a run of `chunk`
// consecutive nodes of one solve's level, one node per thread.  Entries of solves that are not
// active (converged, failed, or without that level) are skipped by the whole block.
#include <type_traits>

#include "ae_cell.cuh"
#include "ae_cells.h"
#include "ae_kernels.cuh"

namespace ae {

namespace {

template <class R>
__device__ __forceinline__ const CellVec<R>& vec_of(const SolveDev& S, int m) {
    if constexpr (sizeof(R) == 8) return S.v64[m];
    else return S.v32[m];
}
template <class R>
__device__ __forceinline__ const R* cfield(const CellLevelDev& L) {
    if constexpr (sizeof(R) == 8) return L.C64;
    else return L.C32;
}
template <class R>
__device__ __forceinline__ const R* ifield(const CellLevelDev& L) {
    if constexpr (sizeof(R) == 8) return L.I64;
    else return L.I32;
}
template <class R>
__device__ __forceinline__ const SCoef<R>& kfield(const CellLevelDev& L) {
    if constexpr (sizeof(R) == 8) return L.K64;
    else return L.K32;
}
template <class R>
__device__ __forceinline__ const R* tabfield(const CellLevelDev& L) {
    if constexpr (sizeof(R) == 8) return L.tab64;
    else return L.tab32;
}
template <class R>
__device__ __forceinline__ const R* itabfield(const CellLevelDev& L) {
    if constexpr (sizeof(R) == 8) return L.itab64;
    else return L.itab32;
}

// Which finest-level representation a launch serves: GR = true the grain tables (entries of
// cells without them are skipped), GR = false the per-node arrays (on the finest level, entries
// of cells with grain tables are skipped).  Coarser levels always use the per-node arrays.
__device__ __forceinline__ bool rep_skips(bool GR, int m, const CellLevelDev& L) {
    return GR ? (m != 0 || L.gid == nullptr) : (m == 0 && L.gid != nullptr);
}

// f = A u at node t of level m
template <int M, class R, bool GR>
__device__ __forceinline__ void level_apply(const CellLevelDev& L, int uniform, const R* U, int t, const POff& o,
                                            R f[3]) {
    if constexpr (GR) cell_apply_grains<M, R>(kfield<R>(L), uniform, L.gid, tabfield<R>(L), U, L.nn, t, o, f);
    else cell_apply<M, R>(kfield<R>(L), uniform, cfield<R>(L), L.nn, U, L.nn, t, o, f);
}

constexpr int kCellThreads = 256;
// Resident blocks per SM requested for the FP32 cell sweeps (smoother, correction residual);
// 0: the compiler's choice.  On a 512-cell mixed batch:
//   finest level on a grain map: 4 blocks (64 registers), 482 solves/s, against 444 with the
//     compiler's 80 registers;
//   per-node levels: 3 blocks (80 registers, about 100 B of spills), 507 solves/s, against 482
//     with the compiler's 118 registers.
#ifndef AE_CELL_SMOOTH_BLOCKS
#define AE_CELL_SMOOTH_BLOCKS 4
#endif
#ifndef AE_CELL_SMOOTH_BLOCKS_PERNODE
#define AE_CELL_SMOOTH_BLOCKS_PERNODE 3
#endif
template <class R, bool GR>
constexpr int cell_min_blocks() {
    return sizeof(R) != 4 ? 0 : GR ? AE_CELL_SMOOTH_BLOCKS : AE_CELL_SMOOTH_BLOCKS_PERNODE;
}

// one damped-Jacobi sweep of the correction at level m: from2 = 0 reads cor and writes cor2,
// from2 = 1 the reverse.  ZERO: the input is the zero vector (the first sweep of a V-cycle).
template <int M, class R, bool ZERO, bool GR>
__global__ void __launch_bounds__(kCellThreads, cell_min_blocks<R, GR>()) kb_smooth(CellArgs A, const Work* __restrict__ tab, int ntab, int m,
                                                          int from2) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (m >= S.nlev - 1 || !S.st->active) continue;
        const CellLevelDev& L = A.cells[S.cell].lv[m];
        if (rep_skips(GR, m, L)) continue;
        const int t = w.start + threadIdx.x;
        const int nn = L.nn;
        if (t >= nn) continue;
        const CellVec<R>& V = vec_of<R>(S, m);
        const R* __restrict__ xin = from2 ? V.cor2 : V.cor;
        R* __restrict__ xout = from2 ? V.cor : V.cor2;
        const R* __restrict__ b = V.res;
        const R omega = (R)A.omega;
        // grain tables on the finest level of a Voronoi cell, per-node arrays otherwise
        constexpr bool grains = GR;
        const int g3 = grains ? 3 * (int)__ldg(L.gid + t) : 0;
        const R* __restrict__ invD = grains ? itabfield<R>(L) + g3 : ifield<R>(L) + t;
        const int ds = grains ? 1 : nn;  // component stride of invD / D
        if (ZERO) {
#pragma unroll
            for (int p = 0; p < 3; ++p) xout[p * nn + t] = (omega * b[p * nn + t]) * invD[p * ds];
            continue;
        }
        int i, j, k;
        cell_ijk(L.n, t, i, j, k);
        const POff o = cell_offsets(L.n, i, j, k);
        R f[3];
        level_apply<M, R, GR>(L, A.uniform, xin, t, o, f);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const R xv = xin[p * nn + t];
            if constexpr (sizeof(R) == 8) {
                // the reference's update, (1-w) x + w (b - (Ax - D x)) / D (Operator.cpp:154)
                const R Dv = grains ? L.dtab64[g3 + p] : L.D64[p * nn + t];
                const R rx = f[p] - xv * Dv;
                xout[p * nn + t] = (R(1) - omega) * xv + omega * (b[p * nn + t] - rx) * invD[p * ds];
            } else {
                xout[p * nn + t] = xv + omega * (b[p * nn + t] - f[p]) * invD[p * ds];
            }
        }
    }
}

template <class R>
__global__ void __launch_bounds__(kCellThreads) kb_copy2(CellArgs A, const Work* __restrict__ tab, int ntab, int m,
                                                         int fill0) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (m >= S.nlev - 1 || !S.st->active) continue;
        const int nn = A.cells[S.cell].lv[m].nn;
        const int t = w.start + threadIdx.x;
        if (t >= nn) continue;
        const CellVec<R>& V = vec_of<R>(S, m);
#pragma unroll
        for (int p = 0; p < 3; ++p) V.cor[p * nn + t] = fill0 ? R(0) : V.cor2[p * nn + t];
    }
}

// rescor = res - A cor at level m (inplace: into res)
template <int M, class R, bool GR>
__global__ void __launch_bounds__(kCellThreads, cell_min_blocks<R, GR>()) kb_rescor(CellArgs A, const Work* __restrict__ tab, int ntab, int m,
                                                          int inplace) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        // the cycle's residual skips the bottom level; the in-place update between inner cycles
        // (top level) also runs on single-level cells
        if ((!inplace && m >= S.nlev - 1) || !S.st->active) continue;
        const CellLevelDev& L = A.cells[S.cell].lv[m];
        if (rep_skips(GR, m, L)) continue;
        const int t = w.start + threadIdx.x;
        const int nn = L.nn;
        if (t >= nn) continue;
        const CellVec<R>& V = vec_of<R>(S, m);
        int i, j, k;
        cell_ijk(L.n, t, i, j, k);
        const POff o = cell_offsets(L.n, i, j, k);
        R f[3];
        level_apply<M, R, GR>(L, A.uniform, V.cor, t, o, f);
        R* out = inplace ? V.res : V.rescor;
#pragma unroll
        for (int p = 0; p < 3; ++p) out[p * nn + t] = V.res[p * nn + t] - f[p];
    }
}

// res_{m+1} = R rescor_m over the level m+1 nodes of solves that have level m+1
template <class R>
__global__ void __launch_bounds__(kCellThreads) kb_restrict(CellArgs A, const Work* __restrict__ tab, int ntab,
                                                            int m) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (m + 1 > S.nlev - 1 || !S.st->active) continue;
        const CellLevelDev& Lf = A.cells[S.cell].lv[m];
        const CellLevelDev& Lc = A.cells[S.cell].lv[m + 1];
        const int t = w.start + threadIdx.x;
        if (t >= Lc.nn) continue;
        int I, J, K;
        cell_ijk(Lc.n, t, I, J, K);
        const R* fine = vec_of<R>(S, m).rescor;
        R* crse = vec_of<R>(S, m + 1).res;
#pragma unroll
        for (int p = 0; p < 3; ++p) crse[p * Lc.nn + t] = cell_restrict<R>(fine + p * Lf.nn, Lf.n, I, J, K);
    }
}

// cor_m += I cor_{m+1} over the level m nodes
template <class R>
__global__ void __launch_bounds__(kCellThreads) kb_interp(CellArgs A, const Work* __restrict__ tab, int ntab, int m) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (m >= S.nlev - 1 || !S.st->active) continue;
        const CellLevelDev& Lf = A.cells[S.cell].lv[m];
        const CellLevelDev& Lc = A.cells[S.cell].lv[m + 1];
        const int t = w.start + threadIdx.x;
        if (t >= Lf.nn) continue;
        int i, j, k;
        cell_ijk(Lf.n, t, i, j, k);
        R* fine = vec_of<R>(S, m).cor;
        const R* crse = vec_of<R>(S, m + 1).cor;
#pragma unroll
        for (int p = 0; p < 3; ++p) fine[p * Lf.nn + t] += cell_interp<R>(crse + p * Lc.nn, Lc.n, i, j, k);
    }
}

// ------------------------------------------------------------------ bottom (one CTA per solve)
// The bordered cell problem on the coarsest level: Krylov on the mean-projected operator.
template <int M, bool LDG>
struct CellBottomOps {
    int n[3];
    int nn;
    SCoef<double> K;
    const double* C;
    const double* D;
    const double* I;
    int uniform;
    int sweeps;
    double omega;
    __device__ void apply_raw(const double* x, double* out) const {
        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
            int i, j, k;
            cell_ijk(n, t, i, j, k);
            const POff o = cell_offsets(n, i, j, k);
            double f[3];
            cell_apply<M, double, LDG>(K, uniform, C, nn, x, nn, t, o, f);
            out[t] = f[0];
            out[t + nn] = f[1];
            out[t + 2 * nn] = f[2];
        }
        __syncthreads();
    }
    __device__ void project(double* v, BlkRed& sh) const {
#pragma unroll 1
        for (int p = 0; p < 3; ++p) {
            double s = 0.0;
            for (int t = threadIdx.x; t < nn; t += blockDim.x) s += v[p * nn + t];
            const double mean = blk_sum(s, sh) / (double)nn;
            for (int t = threadIdx.x; t < nn; t += blockDim.x) v[p * nn + t] -= mean;
        }
        __syncthreads();
    }
    __device__ void apply(const double* x, double* out, BlkRed& sh) const {
        apply_raw(x, out);
        project(out, sh);
    }
    __device__ void residual(const double* x, const double* b, double* r, BlkRed& sh) const {
        apply_raw(x, r);
        for (int t = threadIdx.x; t < 3 * nn; t += blockDim.x) r[t] = b[t] - r[t];
        __syncthreads();
        project(r, sh);
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
    __device__ void smooth(double* x, const double* b, double* tmp, BlkRed&) const {
        for (int s = 0; s < sweeps; ++s) {
            apply_raw(x, tmp);
            for (int t = threadIdx.x; t < 3 * nn; t += blockDim.x) {
                const double xv = x[t];
                const double rx = tmp[t] - xv * D[t];
                x[t] = (1.0 - omega) * xv + omega * (b[t] - rx) * I[t];
            }
            __syncthreads();
        }
    }
};

__host__ __device__ constexpr long long cell_bottom_smem_doubles(int nc, long long nn) { return (nc + 36) * nn; }

template <int M, class R>
__global__ void __launch_bounds__(kBottomThreads) kb_bottom(CellArgs A, KrylovParams kp, int dyn_bytes) {
    __shared__ BlkRed sh;
    extern __shared__ double smem[];
    constexpr int NC = NCoef<M>::value;
    const SolveDev& S = A.solves[blockIdx.x];
    if (!S.st->active) return;
    const int m = S.nlev - 1;
    const CellLevelDev& L = A.cells[S.cell].lv[m];
    const int nn = L.nn;
    const long long N = 3LL * nn;
    const bool fits = cell_bottom_smem_doubles(NC, nn) * (long long)sizeof(double) <= dyn_bytes;
    const double* Cp = L.C64;
    const double* Dp = L.D64;
    const double* Ip = L.I64;
    double* b = S.bwork + 8 * N;
    double* x = b + N;
    double* work = S.bwork;
    if (fits) {
        double* sC = smem;
        double* sD = sC + NC * nn;
        double* sI = sD + N;
        b = sI + N;
        x = b + N;
        work = x + N;
        for (int t = threadIdx.x; t < NC * nn; t += blockDim.x) sC[t] = L.C64[t];
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            sD[t] = L.D64[t];
            sI[t] = L.I64[t];
        }
        Cp = sC; Dp = sD; Ip = sI;
    }
    const CellVec<R>& V = vec_of<R>(S, m);
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        b[t] = (double)V.res[t];
        x[t] = 0.0;
    }
    __syncthreads();
    int ret;
    if (fits) {
        const CellBottomOps<M, false> ops{{L.n[0], L.n[1], L.n[2]}, nn, L.K64, Cp, Dp, Ip, A.uniform, A.sweeps,
                                          A.omega};
        ret = krylov_bottom(ops, kp, N, x, b, work, sh);
    } else {
        const CellBottomOps<M, true> ops{{L.n[0], L.n[1], L.n[2]}, nn, L.K64, Cp, Dp, Ip, A.uniform, A.sweeps,
                                         A.omega};
        ret = krylov_bottom(ops, kp, N, x, b, work, sh);
    }
    if (ret != 0 && ret != 9 && threadIdx.x == 0) S.st->bfail += 1;
    for (int t = threadIdx.x; t < N; t += blockDim.x) V.cor[t] = (R)x[t];
}

// ------------------------------------------------------------------ FP64 top level
// block sums of up to kPartStride values per thread, in a fixed tree, into S.part[chunk]
template <int NQ>
__device__ __forceinline__ void block_partials(double (&v)[NQ], double* dst) {
    __shared__ double red[kCellThreads / 32][NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        double s = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = s;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
        double s = 0.0;
        for (int wq = 0; wq < (int)(blockDim.x >> 5); ++wq) s += red[wq][threadIdx.x];
        dst[threadIdx.x] = s;
    }
    __syncthreads();
}

// r = b - A x at level 0 with per-chunk sums of r (tab: one kRedChunk run per entry)
template <int M, bool GR>
__global__ void __launch_bounds__(kCellThreads) kb_resid_top(CellArgs A, const Work* __restrict__ tab, int ntab) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (!S.st->active) continue;
        const CellLevelDev& L = A.cells[S.cell].lv[0];
        if (rep_skips(GR, 0, L)) continue;
        const int t = w.start + threadIdx.x;
        const int nn = L.nn;
        double v[3] = {0.0, 0.0, 0.0};
        if (t < nn) {
            int i, j, k;
            cell_ijk(L.n, t, i, j, k);
            const POff o = cell_offsets(L.n, i, j, k);
            double f[3];
            level_apply<M, double, GR>(L, A.uniform, S.x, t, o, f);
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                v[p] = S.b[p * nn + t] - f[p];
                S.r[p * nn + t] = v[p];
            }
        }
        block_partials<3>(v, S.part + (size_t)(w.start / kRedChunk) * kPartStride);
    }
}

// b = -sum_d (d_d C) : E e_d, with per-chunk sums
template <int M>
__global__ void __launch_bounds__(kCellThreads) kb_rhs(CellArgs A, const Work* __restrict__ tab, int ntab) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        const CellLevelDev& L = A.cells[S.cell].lv[0];
        const int t = w.start + threadIdx.x;
        const int nn = L.nn;
        double v[3] = {0.0, 0.0, 0.0};
        if (t < nn) {
            double g[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int c = 0; c < 3; ++c) g[a][c] = S.E[3 * a + c];
            if (!A.uniform) {
                int i, j, k;
                cell_ijk(L.n, t, i, j, k);
                const POff o = cell_offsets(L.n, i, j, k);
                double gc[3];
                cell_gradC<M, double>(L.K64, L.C64, nn, t, o, g, gc);
#pragma unroll
                for (int p = 0; p < 3; ++p) v[p] = -gc[p];
            }
#pragma unroll
            for (int p = 0; p < 3; ++p) S.b[p * nn + t] = v[p];
        }
        block_partials<3>(v, S.part + (size_t)(w.start / kRedChunk) * kPartStride);
    }
}

// per-chunk sums of x
__global__ void __launch_bounds__(kCellThreads) kb_xpart(CellArgs A, const Work* __restrict__ tab, int ntab) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        const int nn = A.cells[S.cell].lv[0].nn;
        const int t = w.start + threadIdx.x;
        double v[3] = {0.0, 0.0, 0.0};
        if (t < nn)
#pragma unroll
            for (int p = 0; p < 3; ++p) v[p] = S.x[p * nn + t];
        block_partials<3>(v, S.part + (size_t)(w.start / kRedChunk) * kPartStride);
    }
}

// per-chunk sums of the stress C : (E + grad w)
template <int M>
__global__ void __launch_bounds__(kCellThreads) kb_stress(CellArgs A, const Work* __restrict__ tab, int ntab) {
    constexpr int NC = NCoef<M>::value;
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        const CellLevelDev& L = A.cells[S.cell].lv[0];
        const int nn = L.nn;
        const int t = w.start + threadIdx.x;
        double v[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) v[q] = 0.0;
        if (t < nn) {
            int i, j, k;
            cell_ijk(L.n, t, i, j, k);
            const POff o = cell_offsets(L.n, i, j, k);
            const int ox[3] = {o.xp, o.yp, o.zp}, om[3] = {o.xm, o.ym, o.zm};
            double g[3][3], a[NC], s[3][3];
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    g[p][d] = S.E[3 * p + d] + (S.x[p * nn + t + ox[d]] - S.x[p * nn + t + om[d]]) * L.K64.h[d];
#pragma unroll
            for (int q = 0; q < NC; ++q) a[q] = L.C64[q * nn + t];
            stress_of<M, double>(a, g, s);
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int d = 0; d < 3; ++d) v[3 * p + d] = s[p][d];
        }
        block_partials<9>(v, S.part + (size_t)(w.start / kRedChunk) * kPartStride);
    }
}

// per-solve mean over its partials (one block per solve, fixed order)
__global__ void __launch_bounds__(kBottomThreads) kb_mean(CellArgs A, const int* slots, int which, int all) {
    __shared__ BlkRed sh;
    const SolveDev& S = A.solves[slots ? slots[blockIdx.x] : blockIdx.x];
    if (!all && !S.st->active) return;
    const int nn = A.cells[S.cell].lv[0].nn;
    const int nch = (nn + kRedChunk - 1) / kRedChunk;
    const int nq = which == 2 ? 9 : 3;
    double* dst = which == 0 ? S.st->mean : which == 1 ? S.st->wmean : S.st->sig;
    for (int q = 0; q < nq; ++q) {
        double s = 0.0;
        for (int c = threadIdx.x; c < nch; c += blockDim.x) s += S.part[(size_t)c * kPartStride + q];
        s = blk_sum(s, sh);
        if (threadIdx.x == 0) dst[q] = s / (double)nn;
    }
}

__device__ __forceinline__ double nan_to_inf(double a) { return a != a ? INFINITY : a; }

__device__ __forceinline__ void block_max_to(double v, unsigned long long* dst) {
    __shared__ double red[kCellThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s = fmax(s, red[q]);
        atomicMax(dst, (unsigned long long)__double_as_longlong(s));
    }
    __syncthreads();
}

template <class R>
__global__ void __launch_bounds__(kCellThreads) kb_project(CellArgs A, const Work* __restrict__ tab, int ntab, int vec) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (vec == 0 && !S.st->active) continue;
        const int nn = A.cells[S.cell].lv[0].nn;
        const int t = w.start + threadIdx.x;
        double mx = 0.0;
        if (t < nn) {
            if (vec == 0) {
                const CellVec<R>& V = vec_of<R>(S, 0);
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    const double v = S.r[p * nn + t] - S.st->mean[p];
                    S.r[p * nn + t] = v;
                    V.res[p * nn + t] = (R)v;
                    mx = fmax(mx, nan_to_inf(fabs(v)));
                }
            } else if (vec == 1) {
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    const double v = S.b[p * nn + t] - S.st->mean[p];
                    S.b[p * nn + t] = v;
                    mx = fmax(mx, nan_to_inf(fabs(v)));
                }
            } else {
#pragma unroll
                for (int p = 0; p < 3; ++p) S.x[p * nn + t] -= S.st->wmean[p];
            }
        }
        if (vec != 2) block_max_to(mx, vec == 0 ? &S.st->norm_bits : &S.st->bnorm_bits);
    }
}

template <class R>
__global__ void __launch_bounds__(kCellThreads) kb_update(CellArgs A, const Work* __restrict__ tab, int ntab) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        if (!S.st->active) continue;
        const int nn = A.cells[S.cell].lv[0].nn;
        const int t = w.start + threadIdx.x;
        if (t >= nn) continue;
        const R* cor = vec_of<R>(S, 0).cor;
#pragma unroll
        for (int p = 0; p < 3; ++p) S.x[p * nn + t] += (double)cor[p * nn + t];
    }
}

__global__ void __launch_bounds__(kCellThreads) kb_zero_x(CellArgs A, const Work* __restrict__ tab, int ntab) {
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const SolveDev& S = A.solves[w.id];
        const int nn = A.cells[S.cell].lv[0].nn;
        const int t = w.start + threadIdx.x;
        if (t >= nn) continue;
#pragma unroll
        for (int p = 0; p < 3; ++p) S.x[p * nn + t] = 0.0;
    }
}

__global__ void kb_begin(CellArgs A, const int* slots, int nsolves) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsolves; s += gridDim.x * blockDim.x) {
        CellStatus* st = A.solves[slots ? slots[s] : s].st;
        st->active = 1;
        st->iters = 0;
        st->conv = 0;
        st->bfail = 0;
        st->norm_bits = 0ull;
        st->bnorm_bits = 0ull;
    }
}

// convergence test of every active solve (MLMG: ||r|| <= max(tol_abs, tol_rel max(||b||, ||r0||)))
__global__ void __launch_bounds__(1024) kb_status(CellArgs A, const int* slots, int nsolves, int first,
                                                  double tol_rel, double tol_abs, int max_iter, int* count,
                                                  int* active_out) {
    __shared__ int total;
    if (threadIdx.x == 0) total = 0;
    __syncthreads();
    int mine = 0;
    for (int s = threadIdx.x; s < nsolves; s += blockDim.x) {
        CellStatus* st = A.solves[slots ? slots[s] : s].st;
        if (active_out) active_out[s] = 0;
        if (!st->active) continue;
        const double norm = __longlong_as_double((long long)st->norm_bits);
        st->norm_bits = 0ull;
        st->resn = norm;
        if (first) {
            const double bn = __longlong_as_double((long long)st->bnorm_bits);
            st->bnorm = bn;
            st->res0 = norm;
            const double maxn = bn >= norm ? bn : norm;
            st->target = fmax(tol_abs, fmax(tol_rel, 1.e-16) * maxn);
        }
        if (!isfinite(norm)) {
            st->active = 0;
            st->conv = 0;
        } else if (norm <= st->target) {
            st->active = 0;
            st->conv = 1;
        } else if (st->iters >= max_iter) {
            st->active = 0;
            st->conv = 0;
        } else {
            st->iters += 1;
            ++mine;
            if (active_out) active_out[s] = 1;
        }
    }
    atomicAdd(&total, mine);
    __syncthreads();
    if (threadIdx.x == 0) *count = total;
}

// Loop condition of the batch's device-side iteration (the body of a conditional WHILE graph
// node): continue while some solve is active and fewer than `limit` iterations have run.  The
// counter bounds the loop whatever the status says.
__global__ void kb_loop_cond(cudaGraphConditionalHandle h, const int* count, int* iter, int limit) {
    const int it = *iter + 1;
    *iter = it;
    cudaGraphSetConditional(h, (*count > 0 && it < limit) ? 1u : 0u);
}
// ------------------------------------------------------------------ cell set-up
template <int M>
__global__ void __launch_bounds__(kCellThreads) kb_coarsen_C(CellArgs A, const Work* __restrict__ tab, int ntab,
                                                             int m) {
    constexpr int NC = NCoef<M>::value;
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const CellDev& Cd = A.cells[w.id];
        const CellLevelDev& Lf = Cd.lv[m - 1];
        const CellLevelDev& Lc = Cd.lv[m];
        const int t = w.start + threadIdx.x;
        if (t >= Lc.nn) continue;
        int I, J, K;
        cell_ijk(Lc.n, t, I, J, K);
        for (int q = 0; q < NC; ++q) Lc.C64[q * Lc.nn + t] = cell_restrict<double>(Lf.C64 + q * Lf.nn, Lf.n, I, J, K);
    }
}

template <int M>
__global__ void __launch_bounds__(kCellThreads) kb_diag(CellArgs A, const Work* __restrict__ tab, int ntab, int m,
                                                        int* nan_flag) {
    constexpr int NC = NCoef<M>::value;
    for (int e = blockIdx.x; e < ntab; e += gridDim.x) {
        const Work w = tab[e];
        const CellLevelDev& L = A.cells[w.id].lv[m];
        const int t = w.start + threadIdx.x;
        const int nn = L.nn;
        if (t >= nn) continue;
        double d[3];
        cell_diag<M, double>(L.K64, L.C64, nn, t, d);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            if (!(d[p] == d[p]) || d[p] == 0.0) atomicExch(nan_flag, 1);
            L.D64[p * nn + t] = d[p];
            L.I64[p * nn + t] = 1.0 / d[p];
            L.I32[p * nn + t] = (float)(1.0 / d[p]);
        }
        for (int q = 0; q < NC; ++q) L.C32[q * nn + t] = (float)L.C64[q * nn + t];
    }
}

// Voronoi cell model: node stiffness = table row of the nearest seed (minimum-image distance in
// the periodic cell; ties go to the lower seed index), the semantics of IC::Voronoi
// (src/IC/Voronoi.H:47-101) on a periodic cell.
template <int M>
__global__ void __launch_bounds__(kCellThreads) kb_grains(CellLevelDev L, double lx, double ly, double lz,
                                                          const double* __restrict__ seeds, int ng,
                                                          const double* __restrict__ table) {
    constexpr int NC = NCoef<M>::value;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.nn) return;
    int i, j, k;
    cell_ijk(L.n, t, i, j, k);
    const double x = i * (lx / L.n[0]), y = j * (ly / L.n[1]), z = k * (lz / L.n[2]);
    int best = 0;
    double bd = 0.0;
    for (int g = 0; g < ng; ++g) {
        double dx = x - seeds[3 * g], dy = y - seeds[3 * g + 1], dz = z - seeds[3 * g + 2];
        dx -= lx * rint(dx / lx);
        dy -= ly * rint(dy / ly);
        dz -= lz * rint(dz / lz);
        const double d = dx * dx + dy * dy + dz * dz;
        if (g == 0 || d < bd) { bd = d; best = g; }
    }
    if (L.gid) L.gid[t] = (unsigned short)best;
    for (int q = 0; q < NC; ++q) L.C64[q * L.nn + t] = table[best * NC + q];
}

// per-grain FP32 stiffness, diagonal and 1/diagonal (the values kb_diag gives the grain's nodes)
template <int M>
__global__ void kb_grain_tables(CellLevelDev L) {
    constexpr int NC = NCoef<M>::value;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= L.ngrains) return;
    double d[3];
    cell_diag<M, double>(L.K64, L.tab64 + g * NC, 1, 0, d);
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        L.dtab64[3 * g + p] = d[p];
        L.itab64[3 * g + p] = 1.0 / d[p];
        L.itab32[3 * g + p] = (float)(1.0 / d[p]);
    }
    for (int q = 0; q < NC; ++q) L.tab32[g * NC + q] = (float)L.tab64[g * NC + q];
}

inline int grid_of(int ntab, Shape sh) { return ntab < sh.grid ? ntab : sh.grid; }

template <class F>
void by_prec(int prec, F&& f) {
    if (prec == 1) f(float());
    else f(double());
}

}  // namespace

// ------------------------------------------------------------------ launchers
// reps: bit 0 launch the per-node variant, bit 1 the grain-table variant (finest level)
template <class F>
void by_rep(int reps, F&& f) {
    if (reps & 1) f(std::false_type());
    if (reps & 2) f(std::true_type());
}

void cells_launch_smooth(int model, int prec, bool zero, const CellArgs& A, const Work* tab, int ntab, Shape sh,
                         int m, int from2, int reps, cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        constexpr int M = decltype(mm)::value;
        by_prec(prec, [&](auto r) {
            using R = decltype(r);
            by_rep(reps, [&](auto gr) {
                constexpr bool GR = decltype(gr)::value;
                if (zero) kb_smooth<M, R, true, GR><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m, from2);
                else kb_smooth<M, R, false, GR><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m, from2);
                launched();
            });
        });
    });
}
void cells_launch_copy2(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st) {
    if (ntab == 0) return;
    by_prec(prec, [&](auto r) { kb_copy2<decltype(r)><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m, 0); });
    launched();
}
void cells_launch_fill0(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st) {
    if (ntab == 0) return;
    by_prec(prec, [&](auto r) { kb_copy2<decltype(r)><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m, 1); });
    launched();
}
void cells_launch_rescor(int model, int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m,
                         int inplace, int reps, cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        constexpr int M = decltype(mm)::value;
        by_prec(prec, [&](auto r) {
            by_rep(reps, [&](auto gr) {
                kb_rescor<M, decltype(r), decltype(gr)::value><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m,
                                                                                                       inplace);
                launched();
            });
        });
    });
}
void cells_launch_restrict(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st) {
    if (ntab == 0) return;
    by_prec(prec, [&](auto r) { kb_restrict<decltype(r)><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m); });
    launched();
}
void cells_launch_interp(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st) {
    if (ntab == 0) return;
    by_prec(prec, [&](auto r) { kb_interp<decltype(r)><<<grid_of(ntab, sh), sh.chunk, 0, st>>>(A, tab, ntab, m); });
    launched();
}
void cells_launch_bottom(int model, int prec, const CellArgs& A, int nsolves, const KrylovParams& kp,
                         cudaStream_t st) {
    if (nsolves == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        constexpr int M = decltype(mm)::value;
        by_prec(prec, [&](auto r) {
            kb_bottom<M, decltype(r)><<<nsolves, kBottomThreads, kBottomSmemBytes, st>>>(A, kp, (int)kBottomSmemBytes);
        });
    });
    launched();
}
void cells_launch_resid_top(int model, const CellArgs& A, const Work* tab, int ntab, int reps, cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        by_rep(reps, [&](auto gr) {
            kb_resid_top<decltype(mm)::value, decltype(gr)::value><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab);
            launched();
        });
    });
}
void cells_launch_rhs(int model, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) { kb_rhs<decltype(mm)::value><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab); });
    launched();
}
void cells_launch_mean(const CellArgs& A, const int* slots, int nsolves, int which, int all, cudaStream_t st) {
    if (nsolves == 0) return;
    kb_mean<<<nsolves, kBottomThreads, 0, st>>>(A, slots, which, all);
    launched();
}
void cells_launch_project(int prec, int vec, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st) {
    if (ntab == 0) return;
    by_prec(prec, [&](auto r) { kb_project<decltype(r)><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab, vec); });
    launched();
}
void cells_launch_update(int prec, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st) {
    if (ntab == 0) return;
    by_prec(prec, [&](auto r) { kb_update<decltype(r)><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab); });
    launched();
}
void cells_launch_xpart(const CellArgs& A, const Work* tab, int ntab, cudaStream_t st) {
    if (ntab == 0) return;
    kb_xpart<<<ntab, kRedChunk, 0, st>>>(A, tab, ntab);
    launched();
}
void cells_launch_stress(int model, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        kb_stress<decltype(mm)::value><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab);
    });
    launched();
}
void cells_launch_status(const CellArgs& A, const int* slots, int nsolves, int first, double tol_rel, double tol_abs,
                         int max_iter, int* count, int* active_out, cudaStream_t st) {
    kb_status<<<1, 1024, 0, st>>>(A, slots, nsolves, first, tol_rel, tol_abs, max_iter, count, active_out);
    launched();
}
void cells_launch_begin(const CellArgs& A, const int* slots, int nsolves, cudaStream_t st) {
    if (nsolves == 0) return;
    kb_begin<<<(nsolves + 255) / 256, 256, 0, st>>>(A, slots, nsolves);
    launched();
}
void cells_launch_zero_x(const CellArgs& A, const Work* tab, int ntab, cudaStream_t st) {
    if (ntab == 0) return;
    kb_zero_x<<<ntab, kRedChunk, 0, st>>>(A, tab, ntab);
    launched();
}
void cells_launch_coarsen_C(int model, const CellArgs& A, const Work* tab, int ntab, int m, cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        kb_coarsen_C<decltype(mm)::value><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab, m);
    });
    launched();
}
void cells_launch_grains(int model, const CellLevelDev& L, const double len[3], const double* seeds, int ng,
                         const double* table, cudaStream_t st) {
    if (L.nn == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        kb_grains<decltype(mm)::value><<<(L.nn + kCellThreads - 1) / kCellThreads, kCellThreads, 0, st>>>(
            L, len[0], len[1], len[2], seeds, ng, table);
    });
    launched();
    if (L.gid && L.ngrains > 0) {
        dispatch_model<double>(model, [&](auto mm) {
            kb_grain_tables<decltype(mm)::value><<<(L.ngrains + 127) / 128, 128, 0, st>>>(L);
        });
        launched();
    }
}
void cells_launch_diag(int model, const CellArgs& A, const Work* tab, int ntab, int m, int* nan_flag,
                       cudaStream_t st) {
    if (ntab == 0) return;
    dispatch_model<double>(model, [&](auto mm) {
        kb_diag<decltype(mm)::value><<<ntab, kRedChunk, 0, st>>>(A, tab, ntab, m, nan_flag);
    });
    launched();
}

void cells_launch_loop_cond(cudaGraphConditionalHandle h, const int* count, int* iter, int limit, cudaStream_t st) {
    kb_loop_cond<<<1, 1, 0, st>>>(h, count, iter, limit);
    launched();
}

}  // namespace ae
