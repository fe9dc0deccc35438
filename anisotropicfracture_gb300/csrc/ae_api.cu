// C ABI of libaefast.so (include/aefast.h): operator handle, multigrid hierarchy and
// the MLMG-style solve driver.  Host C++; every field operation is a kernel launch on
// the operator's stream.
//
// The cycle restates AMReX MLMG (tag 20.05, not part of the reference tree) as driven
// by Solver::Nonlocal::Linear (src/Solver/Nonlocal/Linear.H:23-29,102-112):
//   solve   : res0 = b - A x; target = max(tol_abs, tol_rel * max(|b|, |res0|)); repeat
//             { cycle; x += cor; r = b - A x } until |r| <= target
//   V-cycle : per level: cor = 0, nu1 smoother calls, rescor = res - A cor,
//             res_{m+1} = R rescor; bottom solve; back up: cor += I cor_{m+1}, nu2 calls
//   F-cycle : restrict res to every level, bottom solve, then for each level upwards:
//             cor = I cor_{m+1}, res = res - A cor, V-cycle from that level, cor += saved
//   bottom  : CG or BiCGStab to bottom_reltol, correction zeroed + nuf smoother calls on failure
// Mixed precision: the cycle runs in FP32 (stiffness, diagonal, smoother, transfers)
// inside an FP64 refinement loop whose residual, update, norms and bottom solve are FP64.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/aefast.h"
#include "ae_csr_chunks.h"
#include "ae_launch.h"
#include "ae_split.h"

#define AE_CHECK(x)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) throw CudaErr(std::string(cudaGetErrorString(e_)) + " at " + \
                                             __FILE__ + ":" + std::to_string(__LINE__), e_);     \
    } while (0)

namespace {

using namespace ae;

thread_local std::string g_last_error;

}  // namespace

void ae::set_last_error(const std::string& msg) { g_last_error = msg; }

namespace {
using namespace ae;

struct ApiErr : std::runtime_error {
    int code;
    ApiErr(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
struct CudaErr : std::runtime_error {
    cudaError_t err;
    CudaErr(const std::string& m, cudaError_t e) : std::runtime_error(m), err(e) {}
};

template <class F>
int guarded(F&& f) {
    try {
        f();
        return AE_OK;
    } catch (const ApiErr& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const CudaErr& e) {
        g_last_error = e.what();
        return e.err == cudaErrorMemoryAllocation ? AE_ERR_OOM : AE_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return AE_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return (std::string(e.what()).find("out of memory") != std::string::npos) ? AE_ERR_OOM : AE_ERR_CUDA;
    }
}

void require(bool ok, const std::string& msg, int code = AE_ERR_ARG) {
    if (!ok) throw ApiErr(code, msg);
}

struct MGLevel {
    Geo g;
    long long nn = 0;
    double *C = nullptr, *D = nullptr, *invD = nullptr;
    double *res = nullptr, *cor = nullptr, *rescor = nullptr, *corhold = nullptr, *tmp = nullptr;
    float *C32 = nullptr, *D32 = nullptr, *invD32 = nullptr;
    float *res32 = nullptr, *cor32 = nullptr, *rescor32 = nullptr, *corhold32 = nullptr, *tmp32 = nullptr;
    // Voronoi stiffness (finest MG level of an AMR level, ae_op_set_model_grains): grain id per
    // node laid out like C, per-grain tables; the sweeps read these instead of C / C32
    unsigned short* gid = nullptr;
    double* gtab64 = nullptr;
    float* gtab32 = nullptr;
    int ngrains = 0, gcap = 0;
    bool grains = false;
    // FP32 sweeps of a grain-map level split into a tiled interior kernel and a node list
    // (ae_split.cu); built by prepare32, rebuilt after the model changes
    SplitList split;
    bool split_built = false;
    // coarsest MG level of AMR level 0: its operator as an FP64 CSR matrix, for the bottom solve
    // of the FP32 cycle (assembled by prepare32)
    int* csr_rowptr = nullptr;
    int* csr_col = nullptr;
    double* csr_val = nullptr;
    int csr_nnz = 0, csr_cap = 0;
    int* csr_cptr = nullptr;  // chunks of the rows (BottomCsr)
    int* csr_rch = nullptr;
    int csr_nchunk = 0, csr_ccap = 0;
    bool csr_ok = false;
};

struct AmrLevel {
    ae_level_desc desc;
    int rl = 0;       // refinement level (0: the base level)
    int parent = -1;  // the patch of level rl - 1 this patch nests in
    std::vector<MGLevel> mg;
    double *sol = nullptr, *rhs = nullptr;
    float *sol32 = nullptr, *rhs32 = nullptr;  // mixed precision: correction and its right-hand side
    bool model_set = false;
};

}  // namespace

struct ae_op_s {
    int model = 0, ncoef = 0;
    BCP bc;
    double bcval[26 * 3];
    bool bc_set = false;
    int uniform = 0, homogeneous = 0;
    std::vector<AmrLevel> amr;               // the patches, level by level (entry 0: the base level)
    std::vector<std::vector<int>> rlev;      // the patches of each refinement level
    cudaStream_t st = nullptr;
    cudaStream_t own_st = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    unsigned long long* dnorm = nullptr;  // device scratch: 8 norm slots
    unsigned long long* hnorm = nullptr;  // pinned mirror
    int* dflag = nullptr;                 // [0] NaN/zero-diagonal flags, [1] bottom failures
    double* bottom_work = nullptr;
    double* newton_dw = nullptr;  // Newton<T> scratch: 9 components over the largest level store
    long long newton_dw_n = 0;
    long long bottom_work_n = 0;
    bool prepared = false;
    bool have32 = false;
    bool prepared32 = false;
    bool tiled32 = false, tiled64 = false;  // z-marching tiled sweeps per precision (opt-in)
    bool split32 = true;                    // split FP32 sweeps on grain-map levels (AE_SPLIT=0: off)
    bool zero_sweep = true;                 // stencil-free first sweep from a zero correction (AE_ZERO_SWEEP=0: off)
    long long bytes = 0;
    std::vector<void*> allocs;
    void* stage = nullptr;  // device staging for host fabs
    size_t stage_bytes = 0;
    void* stage2 = nullptr;
    size_t stage2_bytes = 0;
    void* mixtab = nullptr;  // device copy of the per-phase tables of ae_op_set_model_mixture
    size_t mixtab_bytes = 0;

    template <class T>
    T* alloc(long long n) {
        void* p = nullptr;
        AE_CHECK(cudaMalloc(&p, sizeof(T) * (size_t)(n > 0 ? n : 1)));
        allocs.push_back(p);
        bytes += sizeof(T) * n;
        AE_CHECK(cudaMemsetAsync(p, 0, sizeof(T) * (size_t)(n > 0 ? n : 1), st));
        return static_cast<T*>(p);
    }
    ~ae_op_s() {
        for (auto& A : amr)
            for (auto& L : A.mg) {
                if (L.split.list) cudaFree(L.split.list);
                if (L.split.list_r) cudaFree(L.split.list_r);
                if (L.split.gidm) cudaFree(L.split.gidm);
            }
        for (void* p : allocs) cudaFree(p);
        if (stage) cudaFree(stage);
        if (stage2) cudaFree(stage2);
        if (mixtab) cudaFree(mixtab);
        if (hnorm) cudaFreeHost(hnorm);
        if (own_st) cudaStreamDestroy(own_st);
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
    }
    OpParams params(const Geo& g) const {
        OpParams P;
        P.g = g;
        P.bc = bc;
        P.model = model;
        P.uniform = uniform;
        return P;
    }
    // the grain-map level whose stiffness (FP32 copy or FP64) is C, when its sweeps are split;
    // else nullptr
    template <class R>
    const MGLevel* split_for(const R* C) const {
        if (!split32) return nullptr;
        for (const AmrLevel& A : amr) {
            const MGLevel& L = A.mg[0];
            const void* mine = sizeof(R) == 4 ? static_cast<const void*>(L.C32) : static_cast<const void*>(L.C);
            if (L.grains && L.split_built && static_cast<const void*>(C) == mine) return &L;
        }
        return nullptr;
    }
    // the grain tables of the level whose stiffness array is C, if it has them
    template <class R>
    Grains<R> grains_for(const R* C) const {
        Grains<R> G;
        for (const AmrLevel& A : amr) {
            const MGLevel& L = A.mg[0];
            if (!L.grains) continue;
            if constexpr (sizeof(R) == 8) {
                if (C == L.C) { G.gid = L.gid; G.tab = L.gtab64; }
            } else {
                if (C == L.C32) { G.gid = L.gid; G.tab = L.gtab32; }
            }
        }
        return G;
    }
};

namespace {

int ncoef_of(int model) {
    return model == AE_MODEL_ISOTROPIC ? 2 : model == AE_MODEL_MAJORMINOR ? 21 : model == AE_MODEL_MAJOR ? 45 : 9;
}

// Orders the operator's own stream after earlier work on the legacy default stream and the
// legacy stream after the work an entry point enqueued, so that callers that produce and
// consume device fields on the default stream (e.g. PyTorch) need no extra synchronisation.
// A caller-provided stream (ae_op_set_stream) is left to the caller.
struct StreamScope {
    ae_op* op;
    explicit StreamScope(ae_op* o) : op(o) {
        if (op->st == op->own_st) {
            AE_CHECK(cudaEventRecord(op->ev_in, cudaStreamLegacy));
            AE_CHECK(cudaStreamWaitEvent(op->st, op->ev_in, 0));
        }
    }
    ~StreamScope() {
        if (op->st == op->own_st) {
            cudaEventRecord(op->ev_out, op->st);
            cudaStreamWaitEvent(cudaStreamLegacy, op->ev_out, 0);
        }
    }
};

// multigrid coarsening of AMR level 0: every cell count even, coarse count >= 2
// (AMReX mg_domain_min_width = 2)
bool coarsenable(const Geo& g) {
    for (int d = 0; d < 3; ++d) {
        const int nc = g.dhi[d] - g.dlo[d];
        if (nc % 2 != 0 || nc / 2 < 2) return false;
    }
    return true;
}

Geo coarsen_geo(const Geo& g) {
    Geo c = g;
    for (int d = 0; d < 3; ++d) {
        c.dlo[d] = g.dlo[d] / 2; c.dhi[d] = g.dhi[d] / 2;
        c.vlo[d] = g.vlo[d] / 2; c.vhi[d] = g.vhi[d] / 2;
        c.dx[d] = g.dx[d] * 2.0;
    }
    c.ng = 0;
    c.px = 0;
    return c;
}

template <class T>
View<T> fab_view(const ae_fab& f) {
    View<T> v;
    v.p = static_cast<T*>(f.data);
    for (int d = 0; d < 3; ++d) v.lo[d] = f.lo[d];
    v.sy = f.hi[0] - f.lo[0] + 1;
    v.sz = v.sy * (f.hi[1] - f.lo[1] + 1);
    v.sc = v.sz * (f.hi[2] - f.lo[2] + 1);
    return v;
}
Box3 fab_box(const ae_fab& f) {
    Box3 b;
    for (int d = 0; d < 3; ++d) { b.lo[d] = f.lo[d]; b.hi[d] = f.hi[d]; }
    return b;
}
long long fab_elems(const ae_fab& f) { return box_npts(fab_box(f)) * f.ncomp; }

bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void check_fab(const ae_fab* f, const Box3& need, int ncomp, const char* what) {
    require(f != nullptr && f->data != nullptr, std::string(what) + ": null fab");
    require(f->ncomp >= ncomp, std::string(what) + ": needs " + std::to_string(ncomp) + " components");
    require(box_contains(fab_box(*f), need), std::string(what) + ": fab box does not cover the required region");
}

MGLevel& level_at(ae_op* op, int amrlev, int mglev) {
    require(amrlev >= 0 && amrlev < (int)op->amr.size(), "amrlev out of range");
    require(mglev >= 0 && mglev < (int)op->amr[amrlev].mg.size(), "mglev out of range");
    return op->amr[amrlev].mg[mglev];
}

void ensure_stage(void*& buf, size_t& have, size_t need) {
    if (have >= need) return;
    if (buf) AE_CHECK(cudaFree(buf));
    buf = nullptr;
    AE_CHECK(cudaMalloc(&buf, need));
    have = need;
}

// A device view of a fab of doubles: the fab itself if it is device memory, otherwise
// an asynchronous copy into a staging buffer.
View<const double> device_view_in(ae_op* op, const ae_fab& f, int slot) {
    if (is_device_ptr(f.data)) return cview(fab_view<double>(f));
    const size_t bytes = sizeof(double) * (size_t)fab_elems(f);
    void*& buf = slot == 0 ? op->stage : op->stage2;
    size_t& have = slot == 0 ? op->stage_bytes : op->stage2_bytes;
    ensure_stage(buf, have, bytes);
    AE_CHECK(cudaMemcpyAsync(buf, f.data, bytes, cudaMemcpyHostToDevice, op->st));
    ae_fab d = f;
    d.data = buf;
    return cview(fab_view<double>(d));
}

void alloc_level_fp32(ae_op* op) {
    if (op->have32) return;
    for (auto& A : op->amr)
        for (auto& L : A.mg) {
            L.C32 = op->alloc<float>(op->ncoef * L.nn);
            L.D32 = op->alloc<float>(3 * L.nn);
            L.invD32 = op->alloc<float>(3 * L.nn);
            L.res32 = op->alloc<float>(3 * L.nn);
            L.cor32 = op->alloc<float>(3 * L.nn);
            L.rescor32 = op->alloc<float>(3 * L.nn);
            L.corhold32 = op->alloc<float>(3 * L.nn);
            L.tmp32 = op->alloc<float>(3 * L.nn);
        }
    for (auto& A : op->amr) {
        A.sol32 = op->alloc<float>(3 * A.mg[0].nn);
        A.rhs32 = op->alloc<float>(3 * A.mg[0].nn);
    }
    op->have32 = true;
}

// The coarsest level of AMR level 0 as an FP64 CSR matrix (levels of up to kBottomCsrMaxN
// unknowns): dense columns A e_j on the device, compressed here, uploaded once per preparation.
void assemble_bottom(ae_op* op) {
    MGLevel& L = op->amr[0].mg.back();
    L.csr_ok = false;
    const long long N = 3 * L.nn;
    if (N > kBottomCsrMaxN) return;
    cudaStream_t st = op->st;
    BottomArgs a{};
    a.P = op->params(L.g);
    a.K = make_scoef<double>(L.g);
    a.C = L.C;
    a.nn = L.nn;
    // the dense matrix and the unit vectors live only for the assembly (freed on every path)
    struct Scratch {
        double* p = nullptr;
        ~Scratch() {
            if (p) cudaFree(p);
        }
    } A, E;
    AE_CHECK(cudaMalloc(&A.p, sizeof(double) * N * N));
    AE_CHECK(cudaMalloc(&E.p, sizeof(double) * N * N));
    std::vector<double> h((size_t)(N * N));
    launch_bottom_assemble(a, A.p, E.p, st);
    AE_CHECK(cudaMemcpyAsync(h.data(), A.p, sizeof(double) * N * N, cudaMemcpyDeviceToHost, st));
    AE_CHECK(cudaStreamSynchronize(st));
    std::vector<int> rp((size_t)N + 1, 0), cl;
    std::vector<double> vl;
    for (long long r = 0; r < N; ++r) {
        for (long long c = 0; c < N; ++c) {
            const double v = h[(size_t)(r * N + c)];
            if (v != 0.0) {
                cl.push_back((int)c);
                vl.push_back(v);
            }
        }
        rp[(size_t)r + 1] = (int)cl.size();
    }
    const int nnz = (int)cl.size();
    if (!L.csr_rowptr) L.csr_rowptr = op->alloc<int>(N + 1);
    if (nnz > L.csr_cap) {
        L.csr_col = op->alloc<int>(nnz);
        L.csr_val = op->alloc<double>(nnz);
        L.csr_cap = nnz;
    }
    AE_CHECK(cudaMemcpyAsync(L.csr_rowptr, rp.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, st));
    if (nnz) {
        AE_CHECK(cudaMemcpyAsync(L.csr_col, cl.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, st));
        AE_CHECK(cudaMemcpyAsync(L.csr_val, vl.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice, st));
    }
    // chunks of at most kCsrChunk nonzeros, row by row
    std::vector<int> cp, rc;
    csr_chunks(rp, kCsrChunk, cp, rc);
    const int nchunk = (int)cp.size() - 1;
    if (!L.csr_rch) L.csr_rch = op->alloc<int>(N + 1);
    if (nchunk + 1 > L.csr_ccap) {
        L.csr_cptr = op->alloc<int>(nchunk + 1);
        L.csr_ccap = nchunk + 1;
    }
    AE_CHECK(cudaMemcpyAsync(L.csr_cptr, cp.data(), sizeof(int) * (nchunk + 1), cudaMemcpyHostToDevice, st));
    AE_CHECK(cudaMemcpyAsync(L.csr_rch, rc.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice, st));
    AE_CHECK(cudaStreamSynchronize(st));
    L.csr_nnz = nnz;
    L.csr_nchunk = nchunk;
    L.csr_ok = true;
}

// FP32 copies of the stiffness and diagonal on every level (mixed-precision cycle)
void prepare32(ae_op* op) {
    alloc_level_fp32(op);
    if (op->prepared32) return;
    for (auto& A : op->amr)
        for (auto& L : A.mg) {
            const Box3 s = geo_store(L.g);
            launch_copy<float, double>(s, op->ncoef, level_view(L.g, L.C32), cview(level_view(L.g, L.C)), op->st);
            launch_copy<float, double>(s, 3, level_view(L.g, L.D32), cview(level_view(L.g, L.D)), op->st);
            launch_copy<float, double>(s, 3, level_view(L.g, L.invD32), cview(level_view(L.g, L.invD)), op->st);
        }
    AE_CHECK(cudaStreamSynchronize(op->st));
    assemble_bottom(op);
    op->prepared32 = true;
}

// node lists and id/mask arrays of the split sweeps (FP32 and FP64) on grain-map levels
void build_splits(ae_op* op) {
    if (!op->split32) return;
    for (auto& A : op->amr) {
        MGLevel& L = A.mg[0];
        if (!L.grains || L.split_built || (L.g.ng != 0 && L.g.ng < 2) || L.ngrains > kSplitMaxGrains ||
            !split_supported(L.g))
            continue;
        split_build(L.g, cview(level_view(L.g, L.gid)), L.split, op->st, op->dnorm + 7);
        if (const char* e = std::getenv("AE_SPLIT_KZ")) L.split.kz = std::atoi(e);
        L.split_built = true;
    }
}

// dflag[2] is set by the split sweep's tiled kernel when a TMA load did not complete within its
// wait limit; the sweep's output is then incomplete
void check_tma_flag(ae_op* op) {
    int f = 0;
    AE_CHECK(cudaMemcpyAsync(&f, op->dflag + 2, sizeof(int), cudaMemcpyDeviceToHost, op->st));
    AE_CHECK(cudaStreamSynchronize(op->st));
    if (f) {
        AE_CHECK(cudaMemsetAsync(op->dflag + 2, 0, sizeof(int), op->st));
        throw ApiErr(AE_ERR_CUDA, "a shared-memory tile load of the split FP32 sweep did not complete");
    }
}

double read_norm(ae_op* op, int slot) {
    AE_CHECK(cudaMemcpyAsync(op->hnorm + slot, op->dnorm + slot, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             op->st));
    AE_CHECK(cudaStreamSynchronize(op->st));
    double v;
    std::memcpy(&v, op->hnorm + slot, sizeof(double));
    return v;
}

// ------------------------------------------------------------------ prepare
void prepare(ae_op* op) {
    for (size_t a = 0; a < op->amr.size(); ++a)
        require(op->amr[a].model_set, "SetModel has not been called on every AMR level", AE_ERR_STATE);
    cudaStream_t st = op->st;
    // Elastic<T>::averageDownCoeffs: restrict the stiffness down the MG levels of every AMR level
    for (auto& A : op->amr)
        for (size_t m = 1; m < A.mg.size(); ++m)
            launch_restrict<double>(A.mg[m].g, op->ncoef, level_view(A.mg[m].g, A.mg[m].C),
                                    cview(level_view(A.mg[m - 1].g, A.mg[m - 1].C)), st);
    AE_CHECK(cudaMemsetAsync(op->dflag, 0, sizeof(int), st));
    for (auto& A : op->amr)
        for (auto& L : A.mg)
            launch_diagonal<double>(op->params(L.g), cview(level_view(L.g, L.C)), level_view(L.g, L.D),
                                    level_view(L.g, L.invD), op->dflag, st);
    op->prepared32 = false;
    for (auto& A : op->amr)
        for (auto& L : A.mg) {
            if (L.split.list) AE_CHECK(cudaFree(L.split.list));
            if (L.split.list_r) AE_CHECK(cudaFree(L.split.list_r));
            if (L.split.gidm) AE_CHECK(cudaFree(L.split.gidm));
            L.split = SplitList{};
            L.split_built = false;
        }
    int flag = 0;
    AE_CHECK(cudaMemcpyAsync(&flag, op->dflag, sizeof(int), cudaMemcpyDeviceToHost, st));
    AE_CHECK(cudaStreamSynchronize(st));
    build_splits(op);
    op->prepared = true;
    if (flag) {
        op->prepared = false;
        throw ApiErr(AE_ERR_NAN, "diagonal is NaN, infinite or zero on some node (Elastic<T>::Diagonal)");
    }
}

// ------------------------------------------------------------------ sweep dispatch
// The z-marching tiled kernels serve internal level buffers on request (AE_TILED32=1,
// AE_TILED64=1); the per-node kernels are the default, measured faster on GB300 (FP32 Jacobi
// sweep at 257^3: 1.04 ms per-node, 1.53 ms tiled with 4-byte cp.async staging).
template <class R>
bool use_tiled(const ae_op* op) {
    return sizeof(R) == 4 ? op->tiled32 : op->tiled64;
}
template <class R>
void sweep_jacobi(ae_op* op, const Geo& g, const R* C, const R* invD, const R* D, const R* xi, const R* b, R* xo,
                  R omega, cudaStream_t st) {
    const OpParams P = op->params(g);
    if (use_tiled<R>(op))
        launch_tiled<R>(1, P, cview(level_view(g, const_cast<R*>(C))), cview(level_view(g, const_cast<R*>(xi))),
                        cview(level_view(g, const_cast<R*>(b))), cview(level_view(g, const_cast<R*>(invD))),
                        cview(level_view(g, const_cast<R*>(D))), level_view(g, xo), omega, st);
    else if (const MGLevel* sl = op->split_for<R>(C))
        launch_jacobi_split<R>(P, sl->split, cview(level_view(g, const_cast<R*>(C))),
                               cview(level_view(g, const_cast<R*>(invD))), cview(level_view(g, const_cast<R*>(D))),
                               cview(level_view(g, const_cast<R*>(xi))), cview(level_view(g, const_cast<R*>(b))),
                               level_view(g, xo), omega, st, op->grains_for<R>(C), sl->ngrains, op->dflag + 2);
    else
        launch_jacobi<R>(P, cview(level_view(g, const_cast<R*>(C))), cview(level_view(g, const_cast<R*>(invD))),
                         cview(level_view(g, const_cast<R*>(D))), cview(level_view(g, const_cast<R*>(xi))),
                         cview(level_view(g, const_cast<R*>(b))), level_view(g, xo), omega, st,
                         op->grains_for<R>(C));
}
// r = b - A x on internal buffers (no norm); r may alias b
template <class R>
void sweep_residual(ae_op* op, const Geo& g, const R* C, const R* x, const R* b, R* r, cudaStream_t st) {
    const OpParams P = op->params(g);
    if (use_tiled<R>(op))
        launch_tiled<R>(2, P, cview(level_view(g, const_cast<R*>(C))), cview(level_view(g, const_cast<R*>(x))),
                        cview(level_view(g, const_cast<R*>(b))), cview(level_view(g, const_cast<R*>(b))),
                        cview(level_view(g, const_cast<R*>(b))), level_view(g, r), R(0), st);
    else if (const MGLevel* sl = op->split_for<R>(C))
        launch_residual_split<R>(P, sl->split, cview(level_view(g, const_cast<R*>(C))),
                                 cview(level_view(g, const_cast<R*>(x))), cview(level_view(g, const_cast<R*>(b))),
                                 level_view(g, r), st, op->grains_for<R>(C), sl->ngrains, op->dflag + 2);
    else
        launch_residual<R>(P, cview(level_view(g, const_cast<R*>(C))), cview(level_view(g, const_cast<R*>(x))),
                           cview(level_view(g, const_cast<R*>(b))), level_view(g, r), nullptr, nullptr, st,
                           op->grains_for<R>(C));
}
template <class R>
void sweep_fapply(ae_op* op, const Geo& g, const R* C, const R* x, R* f, cudaStream_t st) {
    const OpParams P = op->params(g);
    if (use_tiled<R>(op))
        launch_tiled<R>(0, P, cview(level_view(g, const_cast<R*>(C))), cview(level_view(g, const_cast<R*>(x))),
                        cview(level_view(g, const_cast<R*>(x))), cview(level_view(g, const_cast<R*>(x))),
                        cview(level_view(g, const_cast<R*>(x))), level_view(g, f), R(0), st);
    else if (const MGLevel* sl = op->split_for<R>(C))
        launch_fapply_split<R>(P, sl->split, cview(level_view(g, const_cast<R*>(C))),
                               cview(level_view(g, const_cast<R*>(x))), level_view(g, f), st, op->grains_for<R>(C),
                               sl->ngrains, op->dflag + 2);
    else
        launch_fapply<R>(P, cview(level_view(g, const_cast<R*>(C))), cview(level_view(g, const_cast<R*>(x))),
                         level_view(g, f), st, op->grains_for<R>(C));
}

// ------------------------------------------------------------------ the multigrid cycle
template <class R>
struct LevelPtrs {
    R *C, *D, *invD, *res, *cor, *rescor, *corhold, *tmp;
};
template <class R>
LevelPtrs<R> ptrs(MGLevel& L);
template <>
LevelPtrs<double> ptrs<double>(MGLevel& L) {
    return {L.C, L.D, L.invD, L.res, L.cor, L.rescor, L.corhold, L.tmp};
}
template <>
LevelPtrs<float> ptrs<float>(MGLevel& L) {
    return {L.C32, L.D32, L.invD32, L.res32, L.cor32, L.rescor32, L.corhold32, L.tmp32};
}

template <class R>
struct Cycle {
    ae_op* op;
    const ae_solver_opts& o;
    std::vector<MGLevel>& lv;
    cudaStream_t st;

    // one smoother call (Fsmooth): o.sweeps Jacobi sweeps, x ping-pongs through tmp.  from_zero:
    // x is known to be zero (and need not hold it): the first sweep is the stencil-free one.
    void smooth(int m, R* x, const R* b, bool from_zero = false) {
        MGLevel& L = lv[m];
        LevelPtrs<R> p = ptrs<R>(L);
        R* a = x;
        R* t = p.tmp;
        for (int s = 0; s < o.sweeps; ++s) {
            if (s == 0 && from_zero)
                launch_jacobi_zero<R>(L.g, cview(level_view(L.g, const_cast<R*>(p.invD))),
                                      cview(level_view(L.g, const_cast<R*>(p.D))), cview(level_view(L.g, const_cast<R*>(b))),
                                      level_view(L.g, t), (R)o.omega, st);
            else
                sweep_jacobi<R>(op, L.g, p.C, p.invD, p.D, a, b, t, (R)o.omega, st);
            std::swap(a, t);
        }
        if (a != x) launch_copy<R, R>(geo_store(L.g), 3, level_view(L.g, x), cview(level_view(L.g, a)), st);
    }
    // rescor = res - A cor
    void res_of_cor(int m) {
        MGLevel& L = lv[m];
        LevelPtrs<R> p = ptrs<R>(L);
        sweep_residual<R>(op, L.g, p.C, p.cor, p.res, p.rescor, st);
    }
    void zero(int m, R* x) { launch_fill<R>(geo_store(lv[m].g), 3, level_view(lv[m].g, x), R(0), st); }
    void restrict_res(int m, R* src) {  // res_{m+1} = R src_m
        launch_restrict<R>(lv[m + 1].g, 3, level_view(lv[m + 1].g, ptrs<R>(lv[m + 1]).res),
                           cview(level_view(lv[m].g, src)), st);
    }
    void interp_add(int m) {  // cor_m += I cor_{m+1}
        launch_interp_add<R>(lv[m].g, 3, level_view(lv[m].g, ptrs<R>(lv[m]).cor),
                             cview(level_view(lv[m + 1].g, ptrs<R>(lv[m + 1]).cor)), st);
    }
    void bottom() {
        const int m = (int)lv.size() - 1;
        MGLevel& L = lv[m];
        const Box3 s = geo_store(L.g);
        if (sizeof(R) == 4) launch_copy<double, R>(s, 3, level_view(L.g, L.res), cview(level_view(L.g, ptrs<R>(L).res)), st);
        launch_fill<double>(s, 3, level_view(L.g, L.cor), 0.0, st);
        BottomArgs a;
        a.P = op->params(L.g);
        a.K = make_scoef<double>(L.g);
        a.C = L.C;
        a.D = L.D;
        a.invD = L.invD;
        a.x = L.cor;
        a.b = L.res;
        a.work = op->bottom_work;
        a.nn = L.nn;
        a.bottom = o.bottom;
        a.maxiter = o.bottom_max_iter;
        a.reltol = o.bottom_reltol;
        a.nuf = o.nuf;
        a.sweeps = o.sweeps;
        a.omega = o.omega;
        a.fail_count = op->dflag + 1;
        // the FP32 cycle's bottom: the same FP64 Krylov loop over the assembled level operator
        if (sizeof(R) == 4 && L.csr_ok)
            launch_bottom_csr(a, BottomCsr{L.csr_rowptr, L.csr_col, L.csr_val, L.csr_nnz, L.csr_cptr, L.csr_rch,
                                           L.csr_nchunk},
                              st);
        else launch_bottom(a, st);
        if (sizeof(R) == 4) launch_copy<R, double>(s, 3, level_view(L.g, ptrs<R>(L).cor), cview(level_view(L.g, L.cor)), st);
    }
    void vcycle(int top) {
        const int bot = (int)lv.size() - 1;
        for (int m = top; m < bot; ++m) {
            LevelPtrs<R> p = ptrs<R>(lv[m]);
            const bool z = op->zero_sweep && o.nu1 > 0 && o.sweeps > 0;
            if (!z) zero(m, p.cor);
            for (int i = 0; i < o.nu1; ++i) smooth(m, p.cor, p.res, z && i == 0);
            res_of_cor(m);
            restrict_res(m, p.rescor);
        }
        bottom();
        for (int m = bot - 1; m >= top; --m) {
            LevelPtrs<R> p = ptrs<R>(lv[m]);
            interp_add(m);
            for (int i = 0; i < o.nu2; ++i) smooth(m, p.cor, p.res);
        }
    }
    void fcycle() {
        const int bot = (int)lv.size() - 1;
        for (int m = 0; m < bot; ++m) restrict_res(m, ptrs<R>(lv[m]).res);
        bottom();
        for (int m = bot - 1; m >= 0; --m) {
            MGLevel& L = lv[m];
            LevelPtrs<R> p = ptrs<R>(L);
            const Box3 s = geo_store(L.g);
            zero(m, p.cor);
            interp_add(m);
            res_of_cor(m);
            launch_copy<R, R>(s, 3, level_view(L.g, p.res), cview(level_view(L.g, p.rescor)), st);
            launch_copy<R, R>(s, 3, level_view(L.g, p.corhold), cview(level_view(L.g, p.cor)), st);
            vcycle(m);
            launch_axpy<R, R>(s, 3, level_view(L.g, p.cor), 1.0, cview(level_view(L.g, p.corhold)), st);
        }
    }
    void run(bool f) {
        if (f) fcycle();
        else vcycle(0);
    }
};

// ------------------------------------------------------------------ composite multi-level iteration
// MLMG::oneIter over the AMR levels in precision R (see the file header): fine levels are
// smoothed only (their single multigrid level is the bottom of their cycle), the fine
// residual is refluxed onto covered coarse nodes (src/Operator/Operator.cpp:728-839), the
// coarse correction is interpolated into the fine patch and its ghost nodes, and the fine
// solution is injected onto covered coarse nodes (src/Operator/Operator.cpp:626-641).
template <class R>
struct AmrIter {
    ae_op* op;
    const ae_solver_opts& o;
    cudaStream_t st;
    std::vector<R*> sol, rhs;  // per AMR level, level storage layout

    int finest() const { return (int)op->amr.size() - 1; }  // last patch
    int top() const { return (int)op->rlev.size() - 1; }    // finest refinement level
    const std::vector<int>& lev(int r) const { return op->rlev[r]; }
    int up(int a) const { return op->amr[a].parent; }
    MGLevel& T(int a) { return op->amr[a].mg[0]; }
    const Geo& G(int a) { return T(a).g; }
    LevelPtrs<R> P(int a) { return ptrs<R>(T(a)); }
    View<R> V(int a, R* p) { return level_view(G(a), p); }
    View<const R> CV(int a, R* p) { return cview(level_view(G(a), p)); }
    Box3 store_dom(int a) { return box_isect(geo_store(G(a)), geo_domain(G(a))); }
    Box3 covered(int a) {  // nodes of the parent patch under patch a
        Box3 b;
        for (int d = 0; d < 3; ++d) { b.lo[d] = G(a).vlo[d] / 2; b.hi[d] = G(a).vhi[d] / 2; }
        return box_isect(b, geo_domain(G(up(a))));
    }
    void sol_residual(int a) { sweep_residual<R>(op, G(a), P(a).C, sol[a], rhs[a], P(a).res, st); }
    void cor_residual(int a) { sweep_residual<R>(op, G(a), P(a).C, P(a).cor, P(a).res, P(a).res, st); }  // in place
    // the residual of patch e restricted onto the nodes of its parent it covers
    void reflux(int e) {
        const int c = up(e);
        const Box3 r = covered(e);
        launch_restrict<R>(G(c), 3, V(c, P(c).res), CV(e, P(e).res), st, &r);
    }
    void add_cor(int a) { launch_axpy<R, R>(store_dom(a), 3, V(a, sol[a]), 1.0, CV(a, P(a).cor), st); }
    void mini_cycle(int a) {
        const bool z = op->zero_sweep && o.nu1 + o.nu2 > 0 && o.sweeps > 0;
        if (!z) launch_fill<R>(geo_store(G(a)), 3, V(a, P(a).cor), R(0), st);
        Cycle<R> cy{op, o, op->amr[a].mg, st};
        for (int i = 0; i < o.nu1 + o.nu2; ++i) cy.smooth(0, P(a).cor, P(a).res, z && i == 0);
    }
    void interp_cor(int a) {
        launch_fill<R>(geo_store(G(a)), 3, V(a, P(a).cor), R(0), st);
        const Box3 r = store_dom(a);
        launch_interp_add<R>(G(a), 3, V(a, P(a).cor), CV(up(a), P(up(a)).cor), st, &r);
    }
    void average_down(int a) { launch_inject<R>(covered(a), 3, V(up(a), sol[up(a)]), CV(a, sol[a]), st); }
    // residual of every level, fine residuals refluxed onto covered coarse nodes (level by level,
    // finest first; the patches of a level are independent)
    void ml_residual() {
        for (int r = top(); r >= 0; --r) {
            for (int a : lev(r)) sol_residual(a);
            if (r < top())
                for (int e : lev(r + 1)) reflux(e);
        }
    }
    void one_iter(bool fcyc) {
        const int F = top();
        for (int r = F; r >= 1; --r) {
            for (int a : lev(r)) {
                mini_cycle(a);
                add_cor(a);
            }
            for (int c : lev(r - 1)) sol_residual(c);  // computeResWithCrseSolFineCor
            for (int a : lev(r)) {
                cor_residual(a);
                reflux(a);
                if (r != F) launch_copy<R, R>(geo_store(G(a)), 3, V(a, P(a).corhold), CV(a, P(a).cor), st);
            }
        }
        Cycle<R> cy{op, o, op->amr[0].mg, st};
        cy.run(fcyc);
        add_cor(0);
        for (int r = 1; r <= F; ++r)
            for (int a : lev(r)) {
                interp_cor(a);
                add_cor(a);
                if (r != F) launch_axpy<R, R>(geo_store(G(a)), 3, V(a, P(a).corhold), 1.0, CV(a, P(a).cor), st);
                cor_residual(a);  // computeResWithCrseCorFineCor
                mini_cycle(a);
                add_cor(a);
                if (r != F) launch_axpy<R, R>(geo_store(G(a)), 3, V(a, P(a).cor), 1.0, CV(a, P(a).corhold), st);
            }
        for (int a = finest(); a >= 1; --a) average_down(a);  // entries run level by level
    }
};

std::vector<double*> sol64(ae_op* op) {
    std::vector<double*> v;
    for (auto& A : op->amr) v.push_back(A.sol);
    return v;
}
std::vector<double*> rhs64(ae_op* op) {
    std::vector<double*> v;
    for (auto& A : op->amr) v.push_back(A.rhs);
    return v;
}

// FP64 composite residual of the current solution and its max-norm (into dnorm[0]); in mixed
// precision also the FP32 copy that drives the next correction cycle.
void ml_residual64(ae_op* op, const ae_solver_opts& o) {
    cudaStream_t st = op->st;
    AmrIter<double> it{op, o, st, sol64(op), rhs64(op)};
    AE_CHECK(cudaMemsetAsync(op->dnorm, 0, sizeof(unsigned long long), st));
    if (it.finest() == 0) {  // fused residual + norm (+ FP32 copy)
        MGLevel& L = it.T(0);
        View<float> r32 = o.precision ? level_view(L.g, L.res32) : View<float>{};
        launch_residual<double>(op->params(L.g), cview(level_view(L.g, L.C)), it.CV(0, it.sol[0]),
                                it.CV(0, it.rhs[0]), level_view(L.g, L.res), op->dnorm, o.precision ? &r32 : nullptr,
                                st, op->grains_for<double>(L.C));
        return;
    }
    it.ml_residual();
    for (int a = 0; a <= it.finest(); ++a) {
        MGLevel& L = it.T(a);
        launch_norminf<double>(box_isect(geo_valid(L.g), geo_domain(L.g)), 3, cview(level_view(L.g, L.res)),
                               op->dnorm, st);
        if (o.precision) {
            launch_copy<float, double>(geo_store(L.g), 3, level_view(L.g, L.res32), cview(level_view(L.g, L.res)), st);
            launch_copy<float, float>(geo_store(L.g), 3, level_view(L.g, op->amr[a].rhs32),
                                      cview(level_view(L.g, L.res32)), st);
        }
    }
}

// One step of the solve on the stream: a composite cycle (FP64), or an FP32 correction cycle
// added to the FP64 solution (mixed), then the FP64 composite residual and norm.  Everything
// is stream-ordered so it can be captured in a CUDA graph.
void iteration_body(ae_op* op, const ae_solver_opts& o, bool fcyc) {
    cudaStream_t st = op->st;
    if (o.precision == 0) {
        AmrIter<double> it{op, o, st, sol64(op), rhs64(op)};
        it.one_iter(fcyc);
    } else {
        std::vector<float*> e, r;
        for (auto& A : op->amr) { e.push_back(A.sol32); r.push_back(A.rhs32); }
        AmrIter<float> it{op, o, st, e, r};
        const int inner = o.inner_cycles > 0 ? o.inner_cycles : 1;
        if (it.finest() == 0) {
            MGLevel& L = it.T(0);
            const OpParams P = op->params(L.g);
            Cycle<float> cy{op, o, op->amr[0].mg, st};
            for (int c = 0; c < inner; ++c) {
                cy.run(fcyc);
                launch_axpy<double, float>(geo_store(L.g), 3, level_view(L.g, op->amr[0].sol), 1.0,
                                           cview(level_view(L.g, L.cor32)), st);
                if (c + 1 < inner)  // FP32 residual of the correction equation, in place
                    sweep_residual<float>(op, L.g, L.C32, L.cor32, L.res32, L.res32, st);
            }
        } else {
            for (int a = 0; a <= it.finest(); ++a) launch_fill<float>(geo_store(it.G(a)), 3, it.V(a, e[a]), 0.f, st);
            for (int c = 0; c < inner; ++c) {
                it.one_iter(fcyc);
                if (c + 1 < inner) it.ml_residual();
            }
            for (int a = 0; a <= it.finest(); ++a)
                launch_axpy<double, float>(it.store_dom(a), 3, level_view(it.G(a), op->amr[a].sol), 1.0,
                                           it.CV(a, e[a]), st);
            // the patches' outermost ghost rings: the coarse correction interpolated in FP64, as
            // the FP64 solve's rings hold (see k_ring_interp_fix)
            for (int a = 1; a <= it.finest(); ++a)
                launch_ring_interp_fix(it.G(a), level_view(it.G(a), op->amr[a].sol), it.CV(it.up(a), e[it.up(a)]),
                                       it.CV(a, e[a]), st);
            AmrIter<double> it64{op, o, st, sol64(op), rhs64(op)};
            for (int a = it.finest(); a >= 1; --a) it64.average_down(a);
        }
    }
    ml_residual64(op, o);
}

void solve_ml(ae_op* op, const ae_solver_opts& o, double tol_rel, double tol_abs, ae_solve_stats* stats) {
    AmrLevel& A = op->amr[0];
    cudaStream_t st = op->st;
    AE_CHECK(cudaMemsetAsync(op->dnorm, 0, 2 * sizeof(unsigned long long), st));
    AE_CHECK(cudaMemsetAsync(op->dflag + 1, 0, sizeof(int), st));
    for (auto& Al : op->amr) {
        const Geo& g = Al.mg[0].g;
        launch_norminf<double>(box_isect(geo_valid(g), geo_domain(g)), 3, cview(level_view(g, Al.rhs)), op->dnorm + 1,
                               st);
    }
    ml_residual64(op, o);
    const double res0 = read_norm(op, 0);
    const double bnorm = read_norm(op, 1);
    require(std::isfinite(res0) && std::isfinite(bnorm), "initial residual is NaN or infinite", AE_ERR_NAN);
    const double max_norm = bnorm >= res0 ? bnorm : res0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm);
    double rn = res0;
    int iters = 0, conv = res0 <= target;
    // one CUDA graph per cycle kind (F, V), captured on first use
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaGraph_t graph[2] = {nullptr, nullptr};
    long long kernels_per_graph[2] = {0, 0};
    auto cleanup = [&] {
        for (int q = 0; q < 2; ++q) {
            if (exec[q]) cudaGraphExecDestroy(exec[q]);
            if (graph[q]) cudaGraphDestroy(graph[q]);
        }
    };
    try {
        // MLMG with fixed_iter: exactly that many iterations, whatever the residual
        const bool fixed = o.fixed_iter > 0;
        while (fixed ? iters < o.fixed_iter : (!conv && iters < o.max_iter)) {
            const bool fcyc = iters < o.max_fmg_iter;
            const int q = fcyc ? 0 : 1;
            if (o.use_graph && !exec[q]) {
                const long long c0 = g_kernel_launches.load();
                AE_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                try {
                    iteration_body(op, o, fcyc);
                } catch (...) {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(st, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                AE_CHECK(cudaStreamEndCapture(st, &graph[q]));
                AE_CHECK(cudaGraphInstantiate(&exec[q], graph[q], 0));
                // captured launches execute only when the graph is replayed
                kernels_per_graph[q] = g_kernel_launches.load() - c0;
                g_kernel_launches.fetch_sub(kernels_per_graph[q]);
            }
            if (exec[q]) {
                AE_CHECK(cudaGraphLaunch(exec[q], st));
                g_kernel_launches.fetch_add(kernels_per_graph[q]);
            } else {
                iteration_body(op, o, fcyc);
            }
            rn = read_norm(op, 0);
            ++iters;
            if (o.verbose) fprintf(stderr, "aefast: iter %d |r|_inf = %.6e (target %.3e)\n", iters, rn, target);
            require(std::isfinite(rn), "residual became NaN or infinite", AE_ERR_NAN);
            if (rn <= target) conv = 1;
        }
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
    check_tma_flag(op);
    int fails = 0;
    AE_CHECK(cudaMemcpyAsync(&fails, op->dflag + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    AE_CHECK(cudaStreamSynchronize(st));
    if (stats) {
        stats->iters = iters;
        stats->cycles = iters * (o.precision ? std::max(1, o.inner_cycles) : 1);
        stats->converged = conv;
        stats->nlevels = (int)A.mg.size();
        stats->bottom_fail = fails;
        stats->res0 = res0;
        stats->resfinal = rn;
        stats->target = target;
    }
    if (!conv && o.fixed_iter <= 0) throw ApiErr(AE_ERR_NOT_CONVERGED, "MLMG failed to converge within max_iter");
}

// Host fabs handed to an entry point are staged through temporary device copies; out() copies
// a result back, finish() waits for the copies when there were any, the destructor frees them.
struct HostStage {
    cudaStream_t st;
    std::vector<void*> tmp;
    explicit HostStage(cudaStream_t s) : st(s) {}
    HostStage(const HostStage&) = delete;
    HostStage& operator=(const HostStage&) = delete;
    ~HostStage() {
        for (void* p : tmp) cudaFree(p);
    }
    ae_fab in(const ae_fab& f) {
        ae_fab d = f;
        if (is_device_ptr(f.data)) return d;
        const size_t bytes = sizeof(double) * (size_t)fab_elems(f);
        void* p = nullptr;
        AE_CHECK(cudaMalloc(&p, bytes));
        tmp.push_back(p);
        AE_CHECK(cudaMemcpyAsync(p, f.data, bytes, cudaMemcpyHostToDevice, st));
        d.data = p;
        return d;
    }
    void out(const ae_fab& host, const ae_fab& dev) {
        if (dev.data != host.data)
            AE_CHECK(cudaMemcpyAsync(host.data, dev.data, sizeof(double) * (size_t)fab_elems(host),
                                     cudaMemcpyDeviceToHost, st));
    }
    void finish() {
        if (!tmp.empty()) AE_CHECK(cudaStreamSynchronize(st));
    }
};

}  // namespace

// ===================================================================== C ABI
extern "C" {

const char* ae_last_error(void) { return g_last_error.c_str(); }
const char* ae_version(void) { return "aefast 0.1 (sm_103a)"; }

void ae_default_solver_opts(ae_solver_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->max_fmg_iter = 0;
    o->nu1 = 1;
    o->nu2 = 1;
    o->sweeps = 2;
    o->bottom = 0;
    o->max_iter = 200;
    o->bottom_max_iter = 200;
    o->bottom_reltol = 1.0e-4;
    o->nuf = 8;
    o->max_mg_levels = 0;
    o->omega = 2.0 / 3.0;
    o->precision = 0;
    o->inner_cycles = 1;
    o->verbose = 0;
    o->use_graph = 1;
    o->fixed_iter = 0;
}

int ae_op_create(const ae_level_desc* levels, int nlev, int model, ae_op** out) {
    return guarded([&] {
        require(out != nullptr, "out is null");
        *out = nullptr;
        require(levels != nullptr && nlev >= 1, "need at least one level");
        require(model >= 0 && model <= 3, "unknown model kind");
        std::unique_ptr<ae_op> op(new ae_op());
        op->model = model;
        op->ncoef = ncoef_of(model);
        for (int f = 0; f < 26; ++f)
            for (int d = 0; d < 3; ++d) { op->bc.t[f][d] = DISP; op->bcval[3 * f + d] = 0.0; }
        op->amr.resize(nlev);
        for (int a = 0; a < nlev; ++a) {
            const ae_level_desc& L = levels[a];
            AmrLevel& A = op->amr[a];
            A.desc = L;
            Geo g;
            for (int d = 0; d < 3; ++d) {
                require(L.domain_cells[d] >= 1, "domain needs at least one cell per direction");
                require(L.dx[d] > 0.0, "dx must be positive");
                require(L.lo[d] >= 0 && L.hi[d] <= L.domain_cells[d] && L.lo[d] < L.hi[d], "patch outside domain");
                g.dlo[d] = 0;
                g.dhi[d] = L.domain_cells[d];
                g.vlo[d] = L.lo[d];
                g.vhi[d] = L.hi[d];
                g.dx[d] = L.dx[d];
                if (a > 0) require(L.lo[d] % 2 == 0 && L.hi[d] % 2 == 0, "fine patch must align with coarse nodes");
            }
            // the hierarchy: consecutive entries with one domain are the patches of one level; a
            // new level refines the previous one by 2 and each patch nests in one patch below it
            if (a == 0) {
                op->rlev.assign(1, std::vector<int>{0});
            } else {
                const ae_level_desc& Pv = levels[a - 1];
                bool same = true, twice = true;
                for (int d = 0; d < 3; ++d) {
                    same = same && L.domain_cells[d] == Pv.domain_cells[d];
                    twice = twice && L.domain_cells[d] == 2 * Pv.domain_cells[d];
                }
                require((same && op->amr[a - 1].rl >= 1) || twice, "AMR levels must refine by 2");
                A.rl = same && op->amr[a - 1].rl >= 1 ? op->amr[a - 1].rl : op->amr[a - 1].rl + 1;
                if (A.rl == (int)op->rlev.size()) op->rlev.emplace_back();
                for (int q : op->rlev[A.rl - 1]) {
                    const ae_level_desc& Pc = levels[q];
                    bool in = true;
                    for (int d = 0; d < 3; ++d) in = in && L.lo[d] / 2 >= Pc.lo[d] && L.hi[d] / 2 <= Pc.hi[d];
                    if (in) { A.parent = q; break; }
                }
                require(A.parent >= 0, "fine patch must nest in a patch of the coarser level");
                for (int q : op->rlev[A.rl]) {  // storage boxes grow(valid, 2) of one level disjoint
                    const ae_level_desc& Pq = levels[q];
                    bool apart = false;
                    for (int d = 0; d < 3; ++d)
                        apart = apart || L.lo[d] - 2 > Pq.hi[d] + 2 || Pq.lo[d] - 2 > L.hi[d] + 2;
                    require(apart, "patches of one level must be separated (their ghost layers may not meet)");
                }
                op->rlev[A.rl].push_back(a);
            }
            if (a == 0) {
                for (int d = 0; d < 3; ++d)
                    require(L.lo[d] == 0 && L.hi[d] == L.domain_cells[d], "AMR level 0 must cover its whole domain");
                g.ng = 0;
            } else {
                g.ng = 2;
            }
            A.mg.push_back(MGLevel());
            A.mg.back().g = g;
            if (a == 0)
                while (coarsenable(A.mg.back().g)) {
                    MGLevel c;
                    c.g = coarsen_geo(A.mg.back().g);
                    A.mg.push_back(c);
                }
        }
        // a non-blocking (capturable) stream; StreamScope orders it with the legacy stream
        AE_CHECK(cudaStreamCreateWithFlags(&op->own_st, cudaStreamNonBlocking));
        AE_CHECK(cudaEventCreateWithFlags(&op->ev_in, cudaEventDisableTiming));
        AE_CHECK(cudaEventCreateWithFlags(&op->ev_out, cudaEventDisableTiming));
        op->st = op->own_st;
        if (const char* e = std::getenv("AE_TILED32")) op->tiled32 = std::atoi(e) != 0;
        if (const char* e = std::getenv("AE_TILED64")) op->tiled64 = std::atoi(e) != 0;
        if (const char* e = std::getenv("AE_SPLIT")) op->split32 = std::atoi(e) != 0;
        if (const char* e = std::getenv("AE_ZERO_SWEEP")) op->zero_sweep = std::atoi(e) != 0;
        if (model == AE_MODEL_MAJOR) op->tiled32 = op->tiled64 = false;  // per-node kernels only
        tiled_init<float>();
        tiled_init<double>();
        AE_CHECK(cudaMallocHost(&op->hnorm, 8 * sizeof(unsigned long long)));
        op->dnorm = op->alloc<unsigned long long>(8);
        op->dflag = op->alloc<int>(4);
        AE_CHECK(cudaMemsetAsync(op->dflag, 0, 4 * sizeof(int), op->st));
        // row pitch: a multiple of 4 nodes on every level but AMR level 0's coarsest, whose
        // bottom solve works on its dense layout (AE_PAD=0: dense everywhere)
        bool pad = true;
        if (const char* e = std::getenv("AE_PAD")) pad = std::atoi(e) != 0;
        for (size_t a = 0; a < op->amr.size(); ++a)
            for (size_t m = 0; m < op->amr[a].mg.size(); ++m) {
                Geo& g = op->amr[a].mg[m].g;
                const int nx = g.vhi[0] - g.vlo[0] + 1 + 2 * g.ng;
                const bool bottom = a == 0 && m + 1 == op->amr[a].mg.size();
                g.px = (pad && !bottom && nx >= 16) ? (nx + 3) / 4 * 4 : 0;
            }
        for (auto& A : op->amr) {
            for (auto& L : A.mg) {
                L.nn = geo_nn(L.g);
                L.C = op->alloc<double>(op->ncoef * L.nn);
                L.D = op->alloc<double>(3 * L.nn);
                L.invD = op->alloc<double>(3 * L.nn);
                L.res = op->alloc<double>(3 * L.nn);
                L.cor = op->alloc<double>(3 * L.nn);
                L.rescor = op->alloc<double>(3 * L.nn);
                L.corhold = op->alloc<double>(3 * L.nn);
                L.tmp = op->alloc<double>(3 * L.nn);
            }
            A.sol = op->alloc<double>(3 * A.mg[0].nn);
            A.rhs = op->alloc<double>(3 * A.mg[0].nn);
        }
        const MGLevel& B = op->amr[0].mg.back();
        op->bottom_work_n = 8 * 3 * B.nn;
        op->bottom_work = op->alloc<double>(op->bottom_work_n);
        AE_CHECK(cudaStreamSynchronize(op->st));
        *out = op.release();
    });
}

int ae_op_destroy(ae_op* op) {
    return guarded([&] {
        if (!op) return;
        cudaStreamSynchronize(op->st);
        delete op;
    });
}

int ae_op_set_stream(ae_op* op, void* stream) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        AE_CHECK(cudaStreamSynchronize(op->st));
        op->st = stream ? static_cast<cudaStream_t>(stream) : op->own_st;
    });
}

int ae_op_set_model(ae_op* op, int amrlev, const ae_fab* coeffs) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        // Elastic<T>::SetModel copies the tilebox grown by the model's 2 ghosts ∩ domain
        const Box3 need = box_isect(box_isect(box_grow(geo_valid(L.g), 2), geo_domain(L.g)), geo_store(L.g));
        check_fab(coeffs, need, op->ncoef, "SetModel");
        require(!coeffs->is_float, "SetModel: coefficients must be double");
        View<const double> src = device_view_in(op, *coeffs, 0);
        launch_copy<double, double>(need, op->ncoef, level_view(L.g, L.C), src, op->st);
        AE_CHECK(cudaStreamSynchronize(op->st));
        L.grains = false;
        op->amr[amrlev].model_set = true;
        op->prepared = false;
    });
}

int ae_op_set_model_grains(ae_op* op, int amrlev, const ae_fab* grain_id, int ngrains, const double* table) {
    return guarded([&] {
        require(op != nullptr && table != nullptr, "null argument");
        require(ngrains >= 1 && ngrains <= 65535, "SetModelGrains: 1 to 65535 grains");
        require(op->model != AE_MODEL_MAJOR, "SetModelGrains: not for the Sym::Major kind");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 need = box_isect(box_isect(box_grow(geo_valid(L.g), 2), geo_domain(L.g)), geo_store(L.g));
        check_fab(grain_id, need, 1, "SetModelGrains");
        View<const int> ids;
        if (is_device_ptr(grain_id->data)) {
            ids = cview(fab_view<int>(*grain_id));
        } else {
            const size_t bytes = sizeof(int) * (size_t)box_npts(fab_box(*grain_id));
            ensure_stage(op->stage, op->stage_bytes, bytes);
            AE_CHECK(cudaMemcpyAsync(op->stage, grain_id->data, bytes, cudaMemcpyHostToDevice, op->st));
            ae_fab d = *grain_id;
            d.data = op->stage;
            ids = cview(fab_view<int>(d));
        }
        const int nc = op->ncoef;
        if (!L.gid) L.gid = op->alloc<unsigned short>(L.nn);
        if (L.gcap < ngrains) {
            L.gtab64 = op->alloc<double>((long long)ngrains * nc);
            L.gtab32 = op->alloc<float>((long long)ngrains * nc);
            L.gcap = ngrains;
        }
        AE_CHECK(cudaMemcpyAsync(L.gtab64, table, sizeof(double) * ngrains * nc, cudaMemcpyDefault, op->st));
        AE_CHECK(cudaMemsetAsync(op->dflag, 0, sizeof(int), op->st));
        launch_grains_box(need, ids, level_view(L.g, L.gid), level_view(L.g, L.C), L.gtab64, ngrains, nc, L.gtab32,
                          op->dflag, op->st);
        int bad = 0;
        AE_CHECK(cudaMemcpyAsync(&bad, op->dflag, sizeof(int), cudaMemcpyDeviceToHost, op->st));
        AE_CHECK(cudaStreamSynchronize(op->st));
        require(bad == 0, "SetModelGrains: a grain id is outside [0, ngrains)");
        L.ngrains = ngrains;
        L.grains = true;
        op->amr[amrlev].model_set = true;
        op->prepared = false;
    });
}

int ae_op_set_model_mixture(ae_op* op, int amrlev, const ae_fab* eta, int nphase, const double* table,
                            const double* F0table, const ae_fab* F0) {
    return guarded([&] {
        require(op != nullptr && table != nullptr, "null argument");
        require(nphase >= 1, "SetModelMixture: at least one phase");
        require((F0table == nullptr) == (F0 == nullptr), "SetModelMixture: F0table and F0 go together");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 need = box_isect(box_isect(box_grow(geo_valid(L.g), 2), geo_domain(L.g)), geo_store(L.g));
        // node (i, j, k) reads cells (i-1..i, j-1..j, k)
        Box3 cells = need;
        cells.lo[0] -= 1;
        cells.lo[1] -= 1;
        check_fab(eta, cells, nphase, "SetModelMixture eta");
        require(!eta->is_float, "SetModelMixture: eta must be double");
        View<double> f0v{};
        if (F0) {
            check_fab(F0, need, 9, "SetModelMixture F0");
            require(!F0->is_float, "SetModelMixture: F0 must be double");
        }
        const int nc = op->ncoef;
        const size_t tab_n = (size_t)nphase * nc, f0_n = F0table ? (size_t)nphase * 9 : 0;
        ensure_stage(op->mixtab, op->mixtab_bytes, sizeof(double) * (tab_n + f0_n));
        double* dtab = static_cast<double*>(op->mixtab);
        AE_CHECK(cudaMemcpyAsync(dtab, table, sizeof(double) * tab_n, cudaMemcpyDefault, op->st));
        if (F0table)
            AE_CHECK(cudaMemcpyAsync(dtab + tab_n, F0table, sizeof(double) * f0_n, cudaMemcpyDefault, op->st));
        View<const double> ev = device_view_in(op, *eta, 0);
        const bool f0_host = F0 && !is_device_ptr(F0->data);
        if (F0) {
            if (f0_host) {
                // stage the whole host fab so that the nodes outside the region come back unchanged
                const size_t bytes = sizeof(double) * (size_t)fab_elems(*F0);
                ensure_stage(op->stage2, op->stage2_bytes, bytes);
                AE_CHECK(cudaMemcpyAsync(op->stage2, F0->data, bytes, cudaMemcpyHostToDevice, op->st));
                ae_fab d = *F0;
                d.data = op->stage2;
                f0v = fab_view<double>(d);
            } else {
                f0v = fab_view<double>(*F0);
            }
        }
        op->amr[amrlev].model_set = false;
        AE_CHECK(cudaMemsetAsync(op->dflag, 0, sizeof(int), op->st));
        launch_model_mixture(need, nc, ev, nphase, dtab, F0table ? dtab + tab_n : nullptr, level_view(L.g, L.C), f0v,
                             op->dflag, op->st);
        int bad = 0;
        AE_CHECK(cudaMemcpyAsync(&bad, op->dflag, sizeof(int), cudaMemcpyDeviceToHost, op->st));
        if (f0_host)
            AE_CHECK(cudaMemcpyAsync(F0->data, op->stage2, sizeof(double) * (size_t)fab_elems(*F0),
                                     cudaMemcpyDeviceToHost, op->st));
        AE_CHECK(cudaStreamSynchronize(op->st));
        require(bad == 0, "SetModelMixture: the order parameters sum to zero at a node");
        L.grains = false;
        op->amr[amrlev].model_set = true;
        op->prepared = false;
    });
}

int ae_op_set_model_degraded(ae_op* op, int amrlev, const ae_fab* eta, int neta, double lambda0, double mu0) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        require(op->ncoef == 2, "SetModelDegraded: isotropic operators only");
        require(neta >= 0, "SetModelDegraded: negative component count");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 need = box_isect(box_isect(box_grow(geo_valid(L.g), 2), geo_domain(L.g)), geo_store(L.g));
        const Box3 valid = box_isect(geo_valid(L.g), geo_domain(L.g));
        View<const double> ev{};
        if (neta > 0) {
            // node (i, j, k) reads cells (i-1..i, j-1..j, k-1..k)
            Box3 cells = valid;
            for (int d = 0; d < 3; ++d) cells.lo[d] -= 1;
            check_fab(eta, cells, neta, "SetModelDegraded eta");
            require(!eta->is_float, "SetModelDegraded: eta must be double");
            ev = device_view_in(op, *eta, 0);
        }
        op->amr[amrlev].model_set = false;
        AE_CHECK(cudaMemsetAsync(op->dflag, 0, sizeof(int), op->st));
        launch_model_degraded(need, valid, ev, neta, lambda0, mu0, level_view(L.g, L.C), op->dflag, op->st);
        int bad = 0;
        AE_CHECK(cudaMemcpyAsync(&bad, op->dflag, sizeof(int), cudaMemcpyDeviceToHost, op->st));
        AE_CHECK(cudaStreamSynchronize(op->st));
        require(bad == 0, "SetModelDegraded: an order parameter's cell mean is outside [0, 1]");
        L.grains = false;
        op->amr[amrlev].model_set = true;
        op->prepared = false;
    });
}

int ae_op_set_model_uniform(ae_op* op, const double* coeffs, int ncoef) {
    return guarded([&] {
        require(op != nullptr && coeffs != nullptr, "null argument");
        require(ncoef == op->ncoef, "coefficient count does not match the model kind");
        StreamScope scope_(op);
        for (size_t a = 0; a < op->amr.size(); ++a) {
            MGLevel& L = op->amr[a].mg[0];
            std::vector<double> host((size_t)op->ncoef * L.nn);
            for (int q = 0; q < op->ncoef; ++q)
                for (long long n = 0; n < L.nn; ++n) host[(size_t)q * L.nn + n] = coeffs[q];
            AE_CHECK(cudaMemcpyAsync(L.C, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, op->st));
            AE_CHECK(cudaStreamSynchronize(op->st));
            L.grains = false;
            op->amr[a].model_set = true;
        }
        op->prepared = false;
    });
}

int ae_op_set_bc(ae_op* op, const int* type, const double* val) {
    return guarded([&] {
        require(op != nullptr && type != nullptr, "null argument");
        for (int f = 0; f < 26; ++f)
            for (int d = 0; d < 3; ++d) {
                const int t = type[3 * f + d];
                require(t >= 0 && t <= 3, "unknown BC type");
                op->bc.t[f][d] = (unsigned char)t;
                op->bcval[3 * f + d] = val ? val[3 * f + d] : 0.0;
            }
        op->bc_set = true;
        op->prepared = false;
    });
}

int ae_op_set_flags(ae_op* op, int uniform, int homogeneous) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        op->uniform = uniform ? 1 : 0;
        op->homogeneous = homogeneous ? 1 : 0;
    });
}

int ae_op_prepare(ae_op* op) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        prepare(op);
    });
}

int ae_op_num_amr_levels(const ae_op* op) { return op ? (int)op->amr.size() : 0; }
int ae_op_num_mg_levels(const ae_op* op, int amrlev) {
    if (!op || amrlev < 0 || amrlev >= (int)op->amr.size()) return 0;
    return (int)op->amr[amrlev].mg.size();
}
int ae_op_level_info(const ae_op* op, int amrlev, int mglev, int lo[3], int hi[3], int dom_hi[3], double dx[3]) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        const MGLevel& L = level_at(const_cast<ae_op*>(op), amrlev, mglev);
        for (int d = 0; d < 3; ++d) {
            if (lo) lo[d] = L.g.vlo[d];
            if (hi) hi[d] = L.g.vhi[d];
            if (dom_hi) dom_hi[d] = L.g.dhi[d];
            if (dx) dx[d] = L.g.dx[d];
        }
    });
}
long long ae_op_device_bytes(const ae_op* op) { return op ? op->bytes : 0; }

int ae_fapply(ae_op* op, int amrlev, int mglev, const ae_fab* out, const ae_fab* in) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, mglev);
        require(op->amr[amrlev].model_set, "Fapply before SetModel", AE_ERR_STATE);
        const Box3 reg = geo_apply_region(L.g);
        const Box3 rd = box_isect(box_grow(reg, 1), geo_domain(L.g));
        check_fab(in, rd, 3, "Fapply in");
        check_fab(out, reg, 3, "Fapply out");
        require(in->is_float == out->is_float, "Fapply: in and out must share a precision");
        require(is_device_ptr(in->data) && is_device_ptr(out->data), "Fapply: fabs must be device memory");
        const OpParams P = op->params(L.g);
        // the tiled and split kernels work on internal buffers: stage in -> tmp, apply into rescor,
        // copy out
        auto tiled = [&](auto zero) {
            using R = decltype(zero);
            LevelPtrs<R> p = ptrs<R>(L);
            launch_copy<R, R>(rd, 3, level_view(L.g, p.tmp), cview(fab_view<R>(*in)), op->st);
            sweep_fapply<R>(op, L.g, p.C, p.tmp, p.rescor, op->st);
            launch_copy<R, R>(reg, 3, fab_view<R>(*out), cview(level_view(L.g, p.rescor)), op->st);
        };
        if (in->is_float) {
            require(op->prepared, "FP32 Fapply needs a prepared operator", AE_ERR_STATE);
            prepare32(op);
            if (op->tiled32 || op->split_for<float>(L.C32)) tiled(0.0f);
            else
                launch_fapply<float>(P, cview(level_view(L.g, L.C32)), cview(fab_view<float>(*in)),
                                     fab_view<float>(*out), op->st, op->grains_for<float>(L.C32));
        } else {
            if (op->tiled64 || op->split_for<double>(L.C)) tiled(0.0);
            else
                launch_fapply<double>(P, cview(level_view(L.g, L.C)), cview(fab_view<double>(*in)),
                                      fab_view<double>(*out), op->st, op->grains_for<double>(L.C));
        }
    });
}

int ae_diagonal(ae_op* op, int amrlev, int mglev, const ae_fab* diag) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, mglev);
        require(op->prepared, "Diagonal before prepare", AE_ERR_STATE);
        const Box3 reg = geo_apply_region(L.g);
        check_fab(diag, reg, 3, "Diagonal");
        require(is_device_ptr(diag->data) && !diag->is_float, "Diagonal: device double fab required");
        launch_copy<double, double>(reg, 3, fab_view<double>(*diag), cview(level_view(L.g, L.D)), op->st);
    });
}

int ae_fsmooth(ae_op* op, int amrlev, int mglev, const ae_fab* x, const ae_fab* b, int nsweeps, double omega) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, mglev);
        require(op->prepared, "Operator::Diagonal() must be called before using Fsmooth", AE_ERR_STATE);
        require(nsweeps >= 0, "nsweeps must be non-negative");
        const Box3 s = geo_store(L.g);
        const Box3 need = box_isect(s, geo_domain(L.g));
        check_fab(x, need, 3, "Fsmooth x");
        check_fab(b, need, 3, "Fsmooth b");
        require(x->is_float == b->is_float, "Fsmooth: x and b must share a precision");
        require(is_device_ptr(x->data) && is_device_ptr(b->data), "Fsmooth: fabs must be device memory");
        // x and b -> internal buffers (tmp, corhold), sweeps ping-pong tmp <-> rescor, copy back
        auto run = [&](auto zero) {
            using R = decltype(zero);
            LevelPtrs<R> p = ptrs<R>(L);
            launch_copy<R, R>(need, 3, level_view(L.g, p.tmp), cview(fab_view<R>(*x)), op->st);
            launch_copy<R, R>(need, 3, level_view(L.g, p.corhold), cview(fab_view<R>(*b)), op->st);
            R *a = p.tmp, *t = p.rescor;
            launch_copy<R, R>(s, 3, level_view(L.g, t), cview(level_view(L.g, a)), op->st);
            for (int sw = 0; sw < nsweeps; ++sw) {
                sweep_jacobi<R>(op, L.g, p.C, p.invD, p.D, a, p.corhold, t, (R)omega, op->st);
                std::swap(a, t);
            }
            launch_copy<R, R>(need, 3, fab_view<R>(*x), cview(level_view(L.g, a)), op->st);
            check_tma_flag(op);
        };
        if (!x->is_float) {
            run(0.0);
        } else {
            prepare32(op);
            run(0.0f);
        }
    });
}

int ae_residual(ae_op* op, int amrlev, int mglev, const ae_fab* r, const ae_fab* x, const ae_fab* b,
                double* norm_inf) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, mglev);
        const Box3 reg = geo_apply_region(L.g);
        check_fab(x, box_isect(box_grow(reg, 1), geo_domain(L.g)), 3, "residual x");
        check_fab(b, reg, 3, "residual b");
        check_fab(r, reg, 3, "residual r");
        require(!x->is_float && !b->is_float && !r->is_float, "residual: double fabs required");
        require(is_device_ptr(x->data) && is_device_ptr(b->data) && is_device_ptr(r->data),
                "residual: fabs must be device memory");
        AE_CHECK(cudaMemsetAsync(op->dnorm, 0, sizeof(unsigned long long), op->st));
        launch_residual<double>(op->params(L.g), cview(level_view(L.g, L.C)), cview(fab_view<double>(*x)),
                                cview(fab_view<double>(*b)), fab_view<double>(*r), op->dnorm, nullptr, op->st,
                                op->grains_for<double>(L.C));
        const double n = read_norm(op, 0);
        if (norm_inf) *norm_inf = n;
    });
}

int ae_restrict(ae_op* op, int amrlev, int cmglev, const ae_fab* crse, const ae_fab* fine) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        require(cmglev >= 1, "cmglev must be >= 1");
        StreamScope scope_(op);
        MGLevel& Lc = level_at(op, amrlev, cmglev);
        MGLevel& Lf = level_at(op, amrlev, cmglev - 1);
        check_fab(crse, geo_valid(Lc.g), 3, "restriction crse");
        check_fab(fine, box_isect(geo_valid(Lf.g), geo_domain(Lf.g)), 3, "restriction fine");
        require(crse->is_float == fine->is_float, "restriction: precision mismatch");
        require(is_device_ptr(crse->data) && is_device_ptr(fine->data), "restriction: fabs must be device memory");
        if (crse->is_float)
            launch_restrict<float>(Lc.g, 3, fab_view<float>(*crse), cview(fab_view<float>(*fine)), op->st);
        else
            launch_restrict<double>(Lc.g, 3, fab_view<double>(*crse), cview(fab_view<double>(*fine)), op->st);
    });
}

int ae_interp_add(ae_op* op, int amrlev, int fmglev, const ae_fab* fine, const ae_fab* crse) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& Lf = level_at(op, amrlev, fmglev);
        MGLevel& Lc = level_at(op, amrlev, fmglev + 1);
        check_fab(fine, box_isect(geo_valid(Lf.g), geo_domain(Lf.g)), 3, "interpolation fine");
        check_fab(crse, geo_valid(Lc.g), 3, "interpolation crse");
        require(crse->is_float == fine->is_float, "interpolation: precision mismatch");
        require(is_device_ptr(crse->data) && is_device_ptr(fine->data), "interpolation: fabs must be device memory");
        if (fine->is_float)
            launch_interp_add<float>(Lf.g, 3, fab_view<float>(*fine), cview(fab_view<float>(*crse)), op->st);
        else
            launch_interp_add<double>(Lf.g, 3, fab_view<double>(*fine), cview(fab_view<double>(*crse)), op->st);
    });
}

int ae_bc_init(ae_op* op, int amrlev, const ae_fab* rhs, int homogeneous) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 need = box_isect(box_grow(geo_valid(L.g), L.g.ng < 2 ? L.g.ng : 2), geo_domain(L.g));
        check_fab(rhs, need, 3, "BC Init rhs");
        require(!rhs->is_float && is_device_ptr(rhs->data), "BC Init: device double fab required");
        launch_bc_init(L.g, op->bc, op->bcval, homogeneous, fab_view<double>(*rhs), op->st);
    });
}

int ae_strain(ae_op* op, int amrlev, const ae_fab* eps, const ae_fab* u, int voigt) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 v = box_isect(geo_valid(L.g), geo_domain(L.g));
        check_fab(u, box_isect(box_grow(v, 1), geo_domain(L.g)), 3, "Strain u");
        check_fab(eps, v, voigt ? 6 : 9, "Strain eps");
        require(is_device_ptr(u->data) && is_device_ptr(eps->data), "Strain: fabs must be device memory");
        launch_strain(L.g, cview(fab_view<double>(*u)), fab_view<double>(*eps), voigt, op->st);
    });
}

int ae_stress(ae_op* op, int amrlev, const ae_fab* sig, const ae_fab* u, int voigt) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 v = box_isect(geo_valid(L.g), geo_domain(L.g));
        check_fab(u, box_isect(box_grow(v, 1), geo_domain(L.g)), 3, "Stress u");
        check_fab(sig, v, voigt ? 6 : 9, "Stress sigma");
        require(op->model != AE_MODEL_MAJOR, "Stress: the Sym::Major kind is a tangent (use NeoHookeanDW)");
        require(is_device_ptr(u->data) && is_device_ptr(sig->data), "Stress: fabs must be device memory");
        launch_stress(op->params(L.g), cview(level_view(L.g, L.C)), cview(fab_view<double>(*u)),
                      fab_view<double>(*sig), voigt, op->st);
    });
}

int ae_newton_residual(ae_op* op, int amrlev, const ae_fab* u, const ae_fab* b, const ae_fab* F0, ae_fab* rhs) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        require(op->bc_set, "SetBC has not been called", AE_ERR_STATE);
        require(op->model != AE_MODEL_MAJOR, "NewtonResidual: linear models only (use NewtonNeoHookean)");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        require(op->amr[amrlev].model_set, "SetModel has not been called on this level", AE_ERR_STATE);
        const Box3 bx2 = box_isect(box_isect(box_grow(geo_valid(L.g), 2), geo_domain(L.g)), geo_store(L.g));
        const Box3 bx1 = box_isect(box_isect(box_grow(geo_valid(L.g), 1), geo_domain(L.g)), geo_store(L.g));
        check_fab(u, bx2, 3, "NewtonResidual u");
        check_fab(b, bx1, 3, "NewtonResidual b");
        check_fab(rhs, bx1, 3, "NewtonResidual rhs");
        if (F0) check_fab(F0, bx2, 9, "NewtonResidual F0");
        require(!u->is_float && !b->is_float && !rhs->is_float && (!F0 || !F0->is_float),
                "NewtonResidual: FP64 fields required");
        if (op->newton_dw_n < 9 * L.nn) {
            op->newton_dw = op->alloc<double>(9 * L.nn);
            op->newton_dw_n = 9 * L.nn;
        }
        // host fabs are staged through temporary device copies (rhs is copied back)
        HostStage hs(op->st);
        const ae_fab ud = hs.in(*u), bd = hs.in(*b), rd = hs.in(*rhs);
        ae_fab fd{};
        if (F0) fd = hs.in(*F0);
        launch_newton_residual(op->params(L.g), cview(level_view(L.g, L.C)), cview(fab_view<double>(ud)),
                               cview(fab_view<double>(bd)), F0 ? cview(fab_view<double>(fd)) : View<const double>{},
                               level_view(L.g, op->newton_dw), fab_view<double>(rd), op->st);
        hs.out(*rhs, rd);
        hs.finish();
    });
}

int ae_newton_neohookean(ae_op* op, int amrlev, const ae_fab* u, const ae_fab* b, double mu, double kappa,
                         ae_fab* rhs) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        require(op->bc_set, "SetBC has not been called", AE_ERR_STATE);
        require(op->model == AE_MODEL_MAJOR, "NewtonNeoHookean: needs an operator of the Sym::Major kind");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 bx2 = box_isect(box_isect(box_grow(geo_valid(L.g), 2), geo_domain(L.g)), geo_store(L.g));
        const Box3 bx1 = box_isect(box_isect(box_grow(geo_valid(L.g), 1), geo_domain(L.g)), geo_store(L.g));
        check_fab(u, bx2, 3, "NewtonNeoHookean u");
        check_fab(b, bx1, 3, "NewtonNeoHookean b");
        check_fab(rhs, bx1, 3, "NewtonNeoHookean rhs");
        require(!u->is_float && !b->is_float && !rhs->is_float, "NewtonNeoHookean: FP64 fields required");
        if (op->newton_dw_n < 9 * L.nn) {
            op->newton_dw = op->alloc<double>(9 * L.nn);
            op->newton_dw_n = 9 * L.nn;
        }
        HostStage hs(op->st);
        const ae_fab ud = hs.in(*u), bd = hs.in(*b), rd = hs.in(*rhs);
        launch_neohookean_residual(op->params(L.g), cview(fab_view<double>(ud)), cview(fab_view<double>(bd)), mu,
                                   kappa, level_view(L.g, L.C), level_view(L.g, op->newton_dw), fab_view<double>(rd),
                                   op->st);
        hs.out(*rhs, rd);
        hs.finish();
        L.grains = false;
        op->amr[amrlev].model_set = true;
        op->prepared = false;
    });
}

int ae_neohookean_dw(ae_op* op, int amrlev, const ae_fab* u, double mu, double kappa, ae_fab* dw, ae_fab* w) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        require(dw || w, "NeoHookeanDW: nothing to compute");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 v = box_isect(geo_valid(L.g), geo_domain(L.g));
        check_fab(u, box_isect(box_grow(v, 1), geo_domain(L.g)), 3, "NeoHookeanDW u");
        if (dw) check_fab(dw, v, 9, "NeoHookeanDW dw");
        if (w) check_fab(w, v, 1, "NeoHookeanDW w");
        require(is_device_ptr(u->data) && (!dw || is_device_ptr(dw->data)) && (!w || is_device_ptr(w->data)),
                "NeoHookeanDW: fabs must be device memory");
        launch_neohookean_post(L.g, cview(fab_view<double>(*u)), mu, kappa, dw ? fab_view<double>(*dw) : View<double>{},
                               w ? fab_view<double>(*w) : View<double>{}, op->st);
    });
}

int ae_newton_dw(ae_op* op, int amrlev, const ae_fab* u, const ae_fab* F0, ae_fab* dw, ae_fab* w) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        require(dw || w, "NewtonDW: nothing to compute");
        require(op->model != AE_MODEL_MAJOR, "NewtonDW: linear models only (use NeoHookeanDW)");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        require(op->amr[amrlev].model_set, "SetModel has not been called on this level", AE_ERR_STATE);
        const Box3 v = box_isect(geo_valid(L.g), geo_domain(L.g));
        check_fab(u, box_isect(box_grow(v, 1), geo_domain(L.g)), 3, "NewtonDW u");
        if (F0) check_fab(F0, v, 9, "NewtonDW F0");
        if (dw) check_fab(dw, v, 9, "NewtonDW dw");
        if (w) check_fab(w, v, 1, "NewtonDW w");
        require(op->model != AE_MODEL_DIAGONAL || !F0, "NewtonDW: no affine form of the diagonal model");
        require(is_device_ptr(u->data) && (!F0 || is_device_ptr(F0->data)) && (!dw || is_device_ptr(dw->data)) &&
                    (!w || is_device_ptr(w->data)),
                "NewtonDW: fabs must be device memory");
        const double half = (op->model == AE_MODEL_ISOTROPIC && F0) ? 1.0 : 0.5;
        launch_newton_post(op->params(L.g), cview(level_view(L.g, L.C)), cview(fab_view<double>(*u)),
                           F0 ? cview(fab_view<double>(*F0)) : View<const double>{},
                           dw ? fab_view<double>(*dw) : View<double>{}, w ? fab_view<double>(*w) : View<double>{}, half,
                           op->st);
    });
}

int ae_energy(ae_op* op, int amrlev, const ae_fab* w, const ae_fab* u) {
    return guarded([&] {
        require(op != nullptr, "null operator");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, 0);
        const Box3 v = box_isect(geo_valid(L.g), geo_domain(L.g));
        check_fab(u, box_isect(box_grow(v, 1), geo_domain(L.g)), 3, "Energy u");
        check_fab(w, v, 1, "Energy w");
        require(op->model != AE_MODEL_MAJOR, "Energy: linear models only (use NeoHookeanDW)");
        require(is_device_ptr(u->data) && is_device_ptr(w->data), "Energy: fabs must be device memory");
        launch_energy(op->params(L.g), cview(level_view(L.g, L.C)), cview(fab_view<double>(*u)),
                      fab_view<double>(*w), op->st);
    });
}

// ae_solve and ae_solveaffine: affine < 0 plain solve; 0 / 1 solveaffine without / with copyrhs
static int solve_entry(ae_op* op, const ae_fab* sol, const ae_fab* rhs, double tol_rel, double tol_abs,
                const ae_solver_opts* opts, ae_solve_stats* stats, int affine) {
    return guarded([&] {
        const auto t0 = std::chrono::steady_clock::now();
        require(op != nullptr && sol != nullptr && rhs != nullptr, "null argument");
        StreamScope scope_(op);
        ae_solver_opts o;
        if (opts) o = *opts;
        else ae_default_solver_opts(&o);
        require(o.sweeps >= 1 && o.nu1 >= 0 && o.nu2 >= 0 && o.max_iter >= 0, "bad solver options");
        require(o.bottom == 0 || o.bottom == 1, "bottom must be 0 (CG) or 1 (BiCGStab)");
        if (!op->prepared) prepare(op);
        if (o.precision) prepare32(op);
        const int namr = (int)op->amr.size();
        // fields: level 0 over its domain, finer levels over the patch and its 2 ghost layers
        std::vector<Box3> region(namr);
        for (int a = 0; a < namr; ++a) {
            const Geo& g = op->amr[a].mg[0].g;
            region[a] = box_isect(geo_store(g), geo_domain(g));
            check_fab(&sol[a], region[a], 3, "solve sol");
            check_fab(&rhs[a], region[a], 3, "solve rhs");
            require(!sol[a].is_float && !rhs[a].is_float, "solve: double fabs required");
        }
        for (int a = 0; a < namr; ++a) {
            AmrLevel& A = op->amr[a];
            const Geo& g = A.mg[0].g;
            launch_copy<double, double>(region[a], 3, level_view(g, A.rhs), device_view_in(op, rhs[a], 0), op->st);
            launch_copy<double, double>(region[a], 3, level_view(g, A.sol), device_view_in(op, sol[a], 1), op->st);
        }
        if (affine >= 0) {
            // Solver::Nonlocal::Linear::solveaffine (src/Solver/Nonlocal/Linear.H:41-100):
            // rhs_tmp = MLMG::apply(0) with the inhomogeneous operator (composite: each level's
            // apply, the finer level's restricted onto the coarse nodes it covers), then -rhs_tmp
            // inside the domain and 0 on its boundary, added to rhs; the solve is homogeneous.
            // AmrIter::ml_residual with x = b = 0 gives r = -rhs_tmp.
            op->homogeneous = 0;
            std::vector<double*> zx, zb;
            for (int a = 0; a < namr; ++a) {
                MGLevel& L = op->amr[a].mg[0];
                launch_fill<double>(geo_store(L.g), 3, level_view(L.g, L.tmp), 0.0, op->st);
                launch_fill<double>(geo_store(L.g), 3, level_view(L.g, L.corhold), 0.0, op->st);
                zx.push_back(L.tmp);
                zb.push_back(L.corhold);
            }
            AmrIter<double> it{op, o, op->st, zx, zb};
            it.ml_residual();
            for (int a = 0; a < namr; ++a) {
                AmrLevel& A = op->amr[a];
                const Geo& g = A.mg[0].g;
                launch_affine_rhs(g, region[a], level_view(g, A.rhs), cview(level_view(g, A.mg[0].res)), op->st);
                if (affine == 1) {  // copyrhs: the caller's rhs receives the modified right-hand side
                    if (is_device_ptr(rhs[a].data)) {
                        launch_copy<double, double>(region[a], 3, fab_view<double>(rhs[a]), cview(level_view(g, A.rhs)),
                                                    op->st);
                    } else {
                        const size_t bytes = sizeof(double) * (size_t)fab_elems(rhs[a]);
                        ensure_stage(op->stage2, op->stage2_bytes, bytes);
                        ae_fab d = rhs[a];
                        d.data = op->stage2;
                        AE_CHECK(cudaMemcpyAsync(op->stage2, rhs[a].data, bytes, cudaMemcpyHostToDevice, op->st));
                        launch_copy<double, double>(region[a], 3, fab_view<double>(d), cview(level_view(g, A.rhs)),
                                                    op->st);
                        AE_CHECK(cudaMemcpyAsync(rhs[a].data, op->stage2, bytes, cudaMemcpyDeviceToHost, op->st));
                        AE_CHECK(cudaStreamSynchronize(op->st));
                    }
                }
            }
            op->homogeneous = 1;
        }
        int status = AE_OK;
        std::string msg;
        try {
            solve_ml(op, o, tol_rel, tol_abs, stats);
        } catch (const ApiErr& e) {
            if (e.code != AE_ERR_NOT_CONVERGED) throw;
            status = e.code;
            msg = e.what();
        }
        // copy the solution out (also when not converged, as MLMG leaves its iterate in sol)
        for (int a = 0; a < namr; ++a) {
            AmrLevel& A = op->amr[a];
            const Geo& g = A.mg[0].g;
            if (is_device_ptr(sol[a].data)) {
                launch_copy<double, double>(region[a], 3, fab_view<double>(sol[a]), cview(level_view(g, A.sol)),
                                            op->st);
            } else {
                const size_t bytes = sizeof(double) * (size_t)fab_elems(sol[a]);
                ensure_stage(op->stage2, op->stage2_bytes, bytes);
                ae_fab d = sol[a];
                d.data = op->stage2;
                // keep the caller's values outside the written region (ghosts beyond the domain)
                const Box3 fb = fab_box(sol[a]);
                if (!(box_contains(region[a], fb) && sol[a].ncomp == 3))
                    AE_CHECK(cudaMemcpyAsync(op->stage2, sol[a].data, bytes, cudaMemcpyHostToDevice, op->st));
                launch_copy<double, double>(region[a], 3, fab_view<double>(d), cview(level_view(g, A.sol)), op->st);
                AE_CHECK(cudaMemcpyAsync(sol[a].data, op->stage2, bytes, cudaMemcpyDeviceToHost, op->st));
            }
        }
        AE_CHECK(cudaStreamSynchronize(op->st));
        if (stats) stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (status != AE_OK) throw ApiErr(status, msg);
    });
}

int ae_solve(ae_op* op, const ae_fab* sol, const ae_fab* rhs, double tol_rel, double tol_abs,
             const ae_solver_opts* opts, ae_solve_stats* stats) {
    return solve_entry(op, sol, rhs, tol_rel, tol_abs, opts, stats, -1);
}

int ae_solveaffine(ae_op* op, const ae_fab* sol, const ae_fab* rhs, double tol_rel, double tol_abs, int copyrhs,
                   const ae_solver_opts* opts, ae_solve_stats* stats) {
    return solve_entry(op, sol, rhs, tol_rel, tol_abs, opts, stats, copyrhs ? 1 : 0);
}

long long ae_kernel_launches(void) { return g_kernel_launches.load(); }

int ae_profile_kernel(ae_op* op, int which, int amrlev, int mglev, int precision, int reps, double* avg_ms) {
    return guarded([&] {
        require(op != nullptr && avg_ms != nullptr && reps >= 1, "bad argument");
        StreamScope scope_(op);
        MGLevel& L = level_at(op, amrlev, mglev);
        require(op->prepared, "profile needs a prepared operator", AE_ERR_STATE);
        if (precision) prepare32(op);
        require(which >= 0 && which <= 4, "which must be 0..4");
        require(which < 3 || mglev + 1 < (int)op->amr[amrlev].mg.size(), "transfer needs a coarser level");
        const OpParams P = op->params(L.g);
        cudaStream_t st = op->st;
        (void)P;
        auto body = [&](auto zero) {
            using R = decltype(zero);
            LevelPtrs<R> p = ptrs<R>(L);
            if (which == 0) sweep_fapply<R>(op, L.g, p.C, p.cor, p.tmp, st);
            else if (which == 1) sweep_jacobi<R>(op, L.g, p.C, p.invD, p.D, p.cor, p.res, p.tmp, R(2.0 / 3.0), st);
            else if (which == 2) sweep_residual<R>(op, L.g, p.C, p.cor, p.res, p.rescor, st);
            else {
                MGLevel& Lc = op->amr[amrlev].mg[mglev + 1];
                LevelPtrs<R> pc = ptrs<R>(Lc);
                if (which == 3)
                    launch_restrict<R>(Lc.g, 3, level_view(Lc.g, pc.rescor), cview(level_view(L.g, p.rescor)), st);
                else
                    launch_interp_add<R>(L.g, 3, level_view(L.g, p.tmp), cview(level_view(Lc.g, pc.cor)), st);
            }
        };
        auto once = [&]() {
            if (precision) body(0.0f);
            else body(0.0);
        };
        once();  // warm-up
        cudaEvent_t e0, e1;
        AE_CHECK(cudaEventCreate(&e0));
        AE_CHECK(cudaEventCreate(&e1));
        AE_CHECK(cudaEventRecord(e0, st));
        for (int r = 0; r < reps; ++r) once();
        AE_CHECK(cudaEventRecord(e1, st));
        AE_CHECK(cudaEventSynchronize(e1));
        float ms = 0.f;
        AE_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check_tma_flag(op);
        *avg_ms = (double)ms / reps;
    });
}

}  // extern "C"
