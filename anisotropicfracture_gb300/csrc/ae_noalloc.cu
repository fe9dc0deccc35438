// ae_bottom_solve_noalloc: the coarsest-level (bottom) solve of the multigrid cycle for callers
// that cannot allocate device memory.
//
// Who needs it: a host application that already owns the GPU's memory and hands none of it to
// libraries. Examples: an AMReX code whose arena has reserved the device, or a real-time loop
// that must not enter the CUDA allocator. Such an application can still run its own multigrid
// hierarchy and call this for the coarse-grid correction. ae_op_create allocates the whole
// hierarchy, so that path is closed to it. This entry point calls no cudaMalloc, no cudaFree and
// no allocating library routine. Its work space is a file-scope __device__ array of a fixed size;
// every GPU that loads the library holds that array until the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/aefast.h"
#include "ae_launch.h"

namespace {

using namespace ae;

// D (3 nn) + 1/D (3 nn) + the eight Krylov vectors of the bottom solve (8 x 3 nn), in doubles
constexpr long long kNoallocDoubles = 10LL * 3 * AE_NOALLOC_MAX_NODES;
static __device__ __align__(256) double g_noalloc_work[kNoallocDoubles];
// [0] NaN/zero-diagonal flag, [1] failed Krylov solves
static __device__ __align__(256) int g_noalloc_flags[2];

// device address of the arrays, looked up once per device with that device current
constexpr int kMaxDevices = 64;
double* g_work_addr[kMaxDevices] = {nullptr};
int* g_flag_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

int fail(int code, const std::string& msg) {
    ae::set_last_error(msg);  // read back with ae_last_error()
    return code;
}

}  // namespace

extern "C" int ae_bottom_solve_noalloc(const ae_level_desc* level, int model, const double* C, const int* bctype,
                                       int uniform, const double* b, double* x, int bottom, int max_iter,
                                       double reltol, int nuf, int* krylov_failed, void* stream) {
    if (!level || !C || !bctype || !b || !x) return fail(AE_ERR_ARG, "null argument");
    if (model < 0 || model > 2) return fail(AE_ERR_ARG, "unknown model kind");
    if (bottom != 0 && bottom != 1) return fail(AE_ERR_ARG, "bottom must be 0 (CG) or 1 (BiCGStab)");
    if (max_iter < 0 || nuf < 0) return fail(AE_ERR_ARG, "max_iter and nuf must be non-negative");
    Geo g;
    long long nn = 1;
    for (int d = 0; d < 3; ++d) {
        if (level->domain_cells[d] < 1 || level->dx[d] <= 0.0) return fail(AE_ERR_ARG, "bad level");
        if (level->lo[d] != 0 || level->hi[d] != level->domain_cells[d])
            return fail(AE_ERR_ARG, "the level must cover its whole domain");
        g.dlo[d] = 0;
        g.dhi[d] = level->domain_cells[d];
        g.vlo[d] = 0;
        g.vhi[d] = level->domain_cells[d];
        g.dx[d] = level->dx[d];
        // checked after every factor, so the product cannot overflow before the test
        nn *= (long long)level->domain_cells[d] + 1;
        if (level->domain_cells[d] >= AE_NOALLOC_MAX_NODES || nn > AE_NOALLOC_MAX_NODES)
            return fail(AE_ERR_ARG, "level too large: ae_bottom_solve_noalloc handles at most " +
                                        std::to_string(AE_NOALLOC_MAX_NODES) + " nodes (its fixed work space)");
    }
    g.ng = 0;
    OpParams P;
    P.g = g;
    P.model = model;
    P.uniform = uniform ? 1 : 0;
    for (int f = 0; f < 26; ++f)
        for (int d = 0; d < 3; ++d) {
            const int t = bctype[3 * f + d];
            if (t < 0 || t > 3) return fail(AE_ERR_ARG, "unknown BC type");
            P.bc.t[f][d] = (unsigned char)t;
        }
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // set-up: the device address of the scratch arrays, once per device, with that device current
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(AE_ERR_CUDA, "no usable current device");
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_work_addr[dev]) {
            void* w = nullptr;
            void* f = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&w, g_noalloc_work);
            if (e != cudaSuccess) return fail(AE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            e = cudaGetSymbolAddress(&f, g_noalloc_flags);
            if (e != cudaSuccess) return fail(AE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_work_addr[dev] = static_cast<double*>(w);
            g_flag_addr[dev] = static_cast<int*>(f);
        }
    }
    double* work = g_work_addr[dev];
    int* flags = g_flag_addr[dev];
    double* D = work;
    double* invD = work + 3 * nn;
    double* krylov = work + 6 * nn;
    try {
        // the solve starts from zero (MLMG::actualBottomSolve); flags start cleared
        cudaError_t e = cudaMemsetAsync(x, 0, sizeof(double) * 3 * nn, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 2 * sizeof(int), st);
        if (e != cudaSuccess) return fail(AE_ERR_CUDA, cudaGetErrorString(e));
        View<const double> Cv = cview(level_view(g, const_cast<double*>(C)));
        launch_diagonal<double>(P, Cv, level_view(g, D), level_view(g, invD), flags, st);
        BottomArgs a;
        a.P = P;
        a.K = make_scoef<double>(g);
        a.C = C;
        a.D = D;
        a.invD = invD;
        a.x = x;
        a.b = b;
        a.work = krylov;
        a.nn = nn;
        a.bottom = bottom;
        a.maxiter = max_iter;
        a.reltol = reltol;
        a.nuf = nuf;
        a.sweeps = 2;
        a.omega = 2.0 / 3.0;
        a.fail_count = flags + 1;
        launch_bottom(a, st);
        int h[2] = {0, 0};
        e = cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail(AE_ERR_CUDA, cudaGetErrorString(e));
        if (krylov_failed) *krylov_failed = h[1];
        if (h[0]) return fail(AE_ERR_NAN, "diagonal is NaN, infinite or zero on some node");
    } catch (const std::exception& ex) {
        return fail(AE_ERR_CUDA, ex.what());
    }
    return AE_OK;
}
