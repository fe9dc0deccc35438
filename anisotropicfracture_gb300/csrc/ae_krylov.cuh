// Single-CTA Krylov bottom solve: MLMG::actualBottomSolve with MLCGSolver::solve_cg /
// solve_bicgstab (AMReX tag 20.05, called from src/Solver/Nonlocal/Linear.H:23-29,106) restated
// for one thread block.  The operator is supplied by an Ops class:
//   residual(x, b, r, sh)  r = b - A x (the periodic cell also removes the mean of r)
//   apply(x, out, sh)      out = A x (the periodic cell also removes the mean of out)
//   dot(x, y, sh), ninf(x, sh) block reductions in a fixed order
//   smooth(x, b, tmp, sh)  one Fsmooth call (the configured Jacobi sweeps)
// Every reduction has a fixed thread-to-element map and tree, so the result depends only on the
// level, not on what else runs on the device.
#pragma once
#include "ae_device.cuh"

namespace ae {

constexpr int kBottomThreads = 256;
// dynamic shared memory of the shared-memory bottom variants: 48 KB less room for the static BlkRed
constexpr size_t kBottomSmemBytes = 47 * 1024;

struct BlkRed {
    double part[kBottomThreads / 32];
    double res[2];
};
__device__ __forceinline__ double blk_sum(double v, BlkRed& sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh.part[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += sh.part[q];
        sh.res[0] = s;
    }
    __syncthreads();
    const double r = sh.res[0];
    __syncthreads();
    return r;
}
__device__ __forceinline__ double blk_max(double v, BlkRed& sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh.part[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s = fmax(s, sh.part[q]);
        sh.res[0] = s;
    }
    __syncthreads();
    const double r = sh.res[0];
    __syncthreads();
    return r;
}

struct KrylovParams {
    int bottom;    // 0 CG, 1 BiCGStab
    int maxiter;
    double reltol;
    int nuf;       // smoother calls after a failed solve
};

// x: the correction (in: initial guess, out: solution); work: 8 vectors of N doubles.
// Returns the MLCGSolver status (0 converged; nonzero failed, then x = 0 + nuf smooths).
template <class Ops>
__device__ int krylov_bottom(const Ops& ops, const KrylovParams& kp, int N, double* x, const double* b,
                             double* work, BlkRed& sh) {
    double* r = work;
    double* p = r + N;
    double* q = p + N;
    double* rh = q + N;
    double* v = rh + N;
    double* tt = v + N;
    double* sorig = tt + N;
    double* tmp = sorig + N;
    const double eps_rel = kp.reltol, eps_abs = -1.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) sorig[t] = x[t];
    __syncthreads();
    ops.residual(x, b, r, sh);
    for (int t = threadIdx.x; t < N; t += blockDim.x) x[t] = 0.0;
    __syncthreads();
    double rnorm = ops.ninf(r, sh);
    const double rnorm0 = rnorm;
    int ret = 0;
    if (!(rnorm0 == 0.0 || rnorm0 < eps_abs)) {
        if (kp.bottom == 0) {
            double rho_1 = 0.0;
            for (int iter = 1; iter <= kp.maxiter; ++iter) {
                const double rho = ops.dot(r, r, sh);  // z = r (no preconditioner)
                if (rho == 0.0) { ret = 1; break; }
                const double beta = iter == 1 ? 0.0 : rho / rho_1;
                for (int t = threadIdx.x; t < N; t += blockDim.x) p[t] = iter == 1 ? r[t] : r[t] + beta * p[t];
                __syncthreads();
                ops.apply(p, q, sh);
                const double pw = ops.dot(p, q, sh);
                if (pw == 0.0) { ret = 1; break; }
                const double alpha = rho / pw;
                for (int t = threadIdx.x; t < N; t += blockDim.x) { x[t] += alpha * p[t]; r[t] += -alpha * q[t]; }
                __syncthreads();
                rnorm = ops.ninf(r, sh);
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                rho_1 = rho;
            }
        } else {
            double rho_1 = 0.0, alpha = 0.0, omega = 0.0;
            for (int t = threadIdx.x; t < N; t += blockDim.x) { rh[t] = r[t]; p[t] = 0.0; v[t] = 0.0; }
            __syncthreads();
            for (int iter = 1; iter <= kp.maxiter; ++iter) {
                const double rho = ops.dot(rh, r, sh);
                if (rho == 0.0) { ret = 1; break; }
                if (iter == 1) {
                    for (int t = threadIdx.x; t < N; t += blockDim.x) p[t] = r[t];
                } else {
                    const double beta = (rho / rho_1) * (alpha / omega);
                    for (int t = threadIdx.x; t < N; t += blockDim.x) p[t] = r[t] + beta * (p[t] - omega * v[t]);
                }
                __syncthreads();
                ops.apply(p, v, sh);
                const double rhTv = ops.dot(rh, v, sh);
                if (rhTv != 0.0) alpha = rho / rhTv;
                else { ret = 2; break; }
                for (int t = threadIdx.x; t < N; t += blockDim.x) { x[t] += alpha * p[t]; r[t] += -alpha * v[t]; }
                __syncthreads();
                rnorm = ops.ninf(r, sh);
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                ops.apply(r, tt, sh);
                const double t_t = ops.dot(tt, tt, sh), t_r = ops.dot(tt, r, sh);
                if (t_t != 0.0) omega = t_r / t_t;
                else { ret = 3; break; }
                for (int t = threadIdx.x; t < N; t += blockDim.x) { x[t] += omega * r[t]; r[t] += -omega * tt[t]; }
                __syncthreads();
                rnorm = ops.ninf(r, sh);
                if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
                if (omega == 0.0) { ret = 4; break; }
                rho_1 = rho;
            }
        }
        if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
    }
    const bool keep = (ret == 0 || ret == 8) && rnorm < rnorm0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) x[t] = keep ? x[t] + sorig[t] : sorig[t];
    __syncthreads();
    // MLMG: on failure the correction is zeroed and nuf smoother calls follow
    if (ret != 0 && ret != 9) {
        for (int t = threadIdx.x; t < N; t += blockDim.x) x[t] = 0.0;
        __syncthreads();
        for (int s = 0; s < kp.nuf; ++s) ops.smooth(x, b, tmp, sh);
    }
    return ret;
}

}  // namespace ae
