// Batched periodic cells: device descriptors shared by the kernels (ae_cells_kernels.cu) and the
// host engine (ae_cells.cu).
//
// A cell is one periodic RVE with its own multigrid hierarchy (stiffness, diagonal, FP32 copies
// per level); a solve is one macroscopic displacement gradient E on a cell, with its own vectors.
// Kernels run over work tables whose entries name a solve (or a cell) and a run of consecutive
// nodes of one level, so one launch covers every live solve whatever its size.  Every per-solve
// reduction uses a chunking and tree fixed by the solve's own size, so a solve's arithmetic does
// not depend on which other solves share the launch.
#pragma once
#include <cuda_runtime.h>

#include "ae_device.cuh"
#include "ae_krylov.cuh"

namespace ae {

constexpr int kMaxCellLevels = 8;
constexpr int kRedChunk = 256;  // nodes per reduction partial (fixed: results must not depend on tuning)
constexpr int kPartStride = 9;  // doubles per partial slot

struct CellLevelDev {
    int n[3];
    int nn;
    double* C64;
    double* D64;
    double* I64;  // 1 / D
    float* C32;
    float* I32;
    SCoef<double> K64;
    SCoef<float> K32;
    // Voronoi cells, finest level only: grain id per node and per-grain tables of the stiffness
    // (ncoef), diagonal and 1/diagonal (3).  gid == nullptr: per-node arrays only.  The kernels of
    // the finest level read these instead of the per-node arrays (same values, far fewer bytes).
    unsigned short* gid;
    int ngrains;
    double* tab64;
    float* tab32;
    double* dtab64;
    double* itab64;
    float* itab32;
};
struct CellDev {
    int nlev;
    int pad_;
    CellLevelDev lv[kMaxCellLevels];
};

template <class R>
struct CellVec {
    R* cor;
    R* cor2;    // second Jacobi buffer
    R* res;
    R* rescor;
};

// device-resident status of one solve
struct CellStatus {
    int active;
    int iters;
    int conv;
    int bfail;
    unsigned long long norm_bits;  // max |r| of the current residual (bit pattern, atomicMax)
    unsigned long long bnorm_bits;
    double res0, target, resn, bnorm;
    double mean[3];   // mean of the last residual: the body force
    double wmean[3];
    double sig[9];    // cell-averaged stress
};

struct SolveDev {
    int cell;       // slot of its cell in the live cell table
    int nlev;
    double* x;      // w, level 0, FP64
    double* b;
    double* r;
    double* part;   // ceil(nn0 / kRedChunk) * kPartStride doubles
    double* bwork;  // bottom: 10 vectors of 3 nn_bottom doubles (8 work, b, x)
    CellStatus* st;
    double E[9];
    CellVec<float> v32[kMaxCellLevels];
    CellVec<double> v64[kMaxCellLevels];
};

struct Work {
    int id;     // solve (or cell) slot
    int start;  // first node of the run
};

struct CellArgs {
    const CellDev* cells;
    const SolveDev* solves;
    int uniform;
    int sweeps;
    double omega;
};

// launch shape of one table: nodes per entry (= threads per block) and grid size
struct Shape {
    int chunk;
    int grid;
};

// ---- launchers (ae_cells_kernels.cu); model 0 ISO, 1 MM, 2 DIAG
// reps (stencil launchers): bit 0 runs the per-node variant, bit 1 the grain-table variant; on
// the finest level each entry is served by the variant that matches its cell, coarser levels
// always take the per-node variant (reps = 1).
void cells_launch_smooth(int model, int prec, bool zero, const CellArgs& A, const Work* tab, int ntab, Shape sh,
                         int m, int from2, int reps, cudaStream_t st);
void cells_launch_copy2(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st);
void cells_launch_fill0(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st);
// rescor_m = res_m - A cor_m (inplace: res_m -= A cor_m)
void cells_launch_rescor(int model, int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m,
                         int inplace, int reps, cudaStream_t st);
// res_{m+1} = R rescor_m, tab over level m+1 nodes
void cells_launch_restrict(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st);
// cor_m += I cor_{m+1}, tab over level m nodes
void cells_launch_interp(int prec, const CellArgs& A, const Work* tab, int ntab, Shape sh, int m, cudaStream_t st);
void cells_launch_bottom(int model, int prec, const CellArgs& A, int nsolves, const KrylovParams& kp,
                         cudaStream_t st);
// FP64 top level (tab: level-0 runs of kRedChunk nodes, one block each)
void cells_launch_resid_top(int model, const CellArgs& A, const Work* tab, int ntab, int reps, cudaStream_t st);
void cells_launch_rhs(int model, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st);
// per-solve mean of the partials: which 0 residual/rhs -> mean, 1 w -> wmean, 2 stress -> sig
// (slots: the solve slots to visit, nullptr = 0 .. nsolves-1)
void cells_launch_mean(const CellArgs& A, const int* slots, int nsolves, int which, int all, cudaStream_t st);
// vec 0: r (active solves): r -= mean, norm, res_0 = r in the cycle precision
// vec 1: b (setup, every solve): b -= mean, bnorm
// vec 2: x (final, every solve): x -= wmean
void cells_launch_project(int prec, int vec, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st);
void cells_launch_update(int prec, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st);
void cells_launch_xpart(const CellArgs& A, const Work* tab, int ntab, cudaStream_t st);
void cells_launch_stress(int model, const CellArgs& A, const Work* tab, int ntab, cudaStream_t st);
// status: first = 1 for the initial residual; count receives the number of solves still active,
// active_out (optional, one int per visited solve) their flags
void cells_launch_status(const CellArgs& A, const int* slots, int nsolves, int first, double tol_rel, double tol_abs,
                         int max_iter, int* count, int* active_out, cudaStream_t st);
// *iter += 1; the WHILE node's condition = (*count > 0 && *iter < limit)
void cells_launch_loop_cond(cudaGraphConditionalHandle h, const int* count, int* iter, int limit, cudaStream_t st);
void cells_launch_begin(const CellArgs& A, const int* slots, int nsolves, cudaStream_t st);
void cells_launch_zero_x(const CellArgs& A, const Work* tab, int ntab, cudaStream_t st);
// cell set-up (tab over cell ids): C_{m} = R C_{m-1}; D, 1/D, FP32 copies; NaN flag
void cells_launch_coarsen_C(int model, const CellArgs& A, const Work* tab, int ntab, int m, cudaStream_t st);
// level-0 stiffness of a Voronoi cell from seeds (ng x 3, in the cell's length units) and a
// per-grain coefficient table (ng x ncoef); device pointers.  When L.gid is set, also the grain
// ids and L's grain tables (L.tab64 must hold the table, L.ngrains = ng).
void cells_launch_grains(int model, const CellLevelDev& L, const double len[3], const double* seeds, int ng,
                         const double* table, cudaStream_t st);
void cells_launch_diag(int model, const CellArgs& A, const Work* tab, int ntab, int m, int* nan_flag, cudaStream_t st);

}  // namespace ae
