// Batched periodic-cell solve: engine and the ae_batch_* C ABI (include/aefast.h).
//
// Each cell is a periodic RVE under a macroscopic displacement gradient E per solve.  The solve
// restates the MLMG iteration of the single-box driver on the bordered cell problem
//   A w + c = b,  mean(w) = 0,  b = -sum_d (d_d C) : E e_d
// (A: the interior row of Elastic<T>::Fapply, src/Operator/Elastic.cpp:216-255, with periodic
// neighbours).  Per iteration: r = b - A w, c = mean(r), r -= c, test ||r|| against
// max(tol_abs, tol_rel max(||b||, ||r0||)); then a V-cycle on the correction (FP32 in the mixed
// mode, with inner_cycles FP32 cycles per FP64 residual), w += correction.  The coarsest level
// runs BiCGStab/CG on the mean-projected operator, one thread block per solve.
//
// All live solves advance together: every kernel covers every live solve through a work table,
// converged solves drop out through their status flag, and each iteration is captured once as
// a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ae_cells_engine.h"
#include "ae_host.h"

using namespace ae;
using ae::hx::require;

namespace ae {

namespace {

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

template <class R>
SCoef<R> scoef_dx(const double dx[3]) {
    SCoef<R> K;
    for (int d = 0; d < 3; ++d) {
        K.h[d] = (R)(0.5 / dx[d]);
        K.id[d] = (R)(1.0 / dx[d]);
        K.i2[d] = (R)(1.0 / (dx[d] * dx[d]));
        K.bb[d] = (R)(-2.0 / dx[d] / dx[d]);
    }
    K.m01 = (R)(0.25 / (dx[0] * dx[1]));
    K.m02 = (R)(0.25 / (dx[0] * dx[2]));
    K.m12 = (R)(0.25 / (dx[1] * dx[2]));
    return K;
}

int ncoef_of(int model) { return model == AE_MODEL_ISOTROPIC ? 2 : model == AE_MODEL_MAJORMINOR ? 21 : 9; }

// Lays out one cell in `base` (nullptr: dry run).  Returns the bytes used.
size_t cell_layout(CellRes& c, char* base) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        off = align256(off);
        char* p = base ? base + off : nullptr;
        off += bytes;
        return p;
    };
    const int nc = c.nc;
    int n[3] = {c.n[0], c.n[1], c.n[2]};
    double dx[3];
    for (int d = 0; d < 3; ++d) dx[d] = c.len[d] / c.n[d];
    for (int m = 0; m < c.nlev; ++m) {
        CellLevelDev& L = c.lv[m];
        for (int d = 0; d < 3; ++d) L.n[d] = n[d];
        L.nn = n[0] * n[1] * n[2];
        const size_t nn = (size_t)L.nn;
        L.C64 = (double*)take(sizeof(double) * nc * nn);
        L.D64 = (double*)take(sizeof(double) * 3 * nn);
        L.I64 = (double*)take(sizeof(double) * 3 * nn);
        L.C32 = (float*)take(sizeof(float) * nc * nn);
        L.I32 = (float*)take(sizeof(float) * 3 * nn);
        L.K64 = scoef_dx<double>(dx);
        L.K32 = scoef_dx<float>(dx);
        L.gid = nullptr;
        L.ngrains = 0;
        L.tab64 = nullptr;
        L.tab32 = nullptr;
        L.dtab64 = nullptr;
        L.itab64 = nullptr;
        L.itab32 = nullptr;
        for (int d = 0; d < 3; ++d) { n[d] /= 2; dx[d] *= 2.0; }
    }
    const size_t nn0 = (size_t)c.lv[0].nn, nnb = (size_t)c.lv[c.nlev - 1].nn;
    c.gid_mem = (unsigned short*)take(sizeof(unsigned short) * nn0);
    const size_t nch = (nn0 + kRedChunk - 1) / kRedChunk;
    c.sol.assign(c.nrhs, SolveDev{});
    for (int r = 0; r < c.nrhs; ++r) {
        SolveDev& s = c.sol[r];
        s.nlev = c.nlev;
        s.x = (double*)take(sizeof(double) * 3 * nn0);
        s.b = (double*)take(sizeof(double) * 3 * nn0);
        s.r = (double*)take(sizeof(double) * 3 * nn0);
        s.part = (double*)take(sizeof(double) * kPartStride * nch);
        s.bwork = (double*)take(sizeof(double) * 10 * 3 * nnb);
        s.st = (CellStatus*)take(sizeof(CellStatus));
        for (int m = 0; m < c.nlev; ++m) {
            const size_t nn = (size_t)c.lv[m].nn;
            s.v32[m].cor = (float*)take(sizeof(float) * 3 * nn);
            s.v32[m].cor2 = (float*)take(sizeof(float) * 3 * nn);
            s.v32[m].res = (float*)take(sizeof(float) * 3 * nn);
            s.v32[m].rescor = (float*)take(sizeof(float) * 3 * nn);
            s.v64[m].cor = (double*)take(sizeof(double) * 3 * nn);
            s.v64[m].cor2 = (double*)take(sizeof(double) * 3 * nn);
            s.v64[m].res = (double*)take(sizeof(double) * 3 * nn);
            s.v64[m].rescor = (double*)take(sizeof(double) * 3 * nn);
        }
    }
    return align256(off);
}

}  // namespace

int cell_num_levels(const int n[3]) {
    int cur[3] = {n[0], n[1], n[2]};
    int L = 1;
    while (L < kMaxCellLevels) {
        bool ok = true;
        for (int d = 0; d < 3; ++d)
            if (cur[d] % 2 != 0 || cur[d] / 2 < 2) ok = false;
        if (!ok) break;
        for (int d = 0; d < 3; ++d) cur[d] /= 2;
        ++L;
    }
    return L;
}

size_t cell_plan_bytes(const int n[3], int nrhs, int model) {
    CellRes c;
    for (int d = 0; d < 3; ++d) c.n[d] = n[d];
    c.nrhs = nrhs;
    c.model = model;
    c.nc = ncoef_of(model);
    c.nlev = cell_num_levels(n);
    return cell_layout(c, nullptr);
}

void Table::upload(cudaStream_t st) {
    n = (int)h.size();
    if ((size_t)n > cap) {
        if (d) AEH_CHECK(cudaFree(d));
        d = nullptr;
        cap = std::max<size_t>((size_t)n, 2 * cap);
        AEH_CHECK(cudaMalloc(&d, sizeof(Work) * cap));
    }
    if (n) AEH_CHECK(cudaMemcpyAsync(d, h.data(), sizeof(Work) * n, cudaMemcpyHostToDevice, st));
}
void Table::release() {
    if (d) cudaFree(d);
    d = nullptr;
    cap = 0;
    n = 0;
}

CellEngine::CellEngine(int model_) : model(model_), nc(ncoef_of(model_)) {
    int dev = 0;
    AEH_CHECK(cudaGetDevice(&dev));
    AEH_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    AEH_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    AEH_CHECK(cudaMalloc(&dcount, sizeof(int) * 2));
    AEH_CHECK(cudaMemset(dcount, 0, sizeof(int) * 2));
    dnan = dcount + 1;
    AEH_CHECK(cudaMallocHost(&hcount, sizeof(int) * 2));
    for (int m = 0; m < kMaxCellLevels; ++m) {
        chunk_idx[m] = 1;
        grid[m] = 0;
        forced[m] = false;
    }
}

CellEngine::~CellEngine() {
    if (st) cudaStreamSynchronize(st);
    invalidate_graphs();
    for (CellRes* c : live) free_cell(c);
    live.clear();
    for (auto& a : tall)
        for (auto& t : a) t.release();
    tred.release();
    tsub.release();
    for (auto& t : tcell) t.release();
    if (dcells) cudaFree(dcells);
    if (dsolves) cudaFree(dsolves);
    if (dslots) cudaFree(dslots);
    if (dactive) cudaFree(dactive);
    if (hactive) cudaFreeHost(hactive);
    if (dcount) cudaFree(dcount);
    if (hcount) cudaFreeHost(hcount);
    if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
}

void CellEngine::invalidate_graphs() {
    for (int p = 0; p < 2; ++p) {
        if (gexec[p]) cudaGraphExecDestroy(gexec[p]);
        gexec[p] = nullptr;
        gvalid[p] = false;
        if (wexec[p]) cudaGraphExecDestroy(wexec[p]);
        wexec[p] = nullptr;
        wvalid[p] = false;
    }
}

CellArgs CellEngine::args(const ae_solver_opts& o) const {
    CellArgs A;
    A.cells = dcells;
    A.solves = dsolves;
    A.uniform = 0;
    A.sweeps = o.sweeps;
    A.omega = o.omega;
    return A;
}

Shape CellEngine::shape(int m) const {
    const int chunk = chunk_idx[m] == 0 ? 128 : 256;
    const int ntab = tall[chunk_idx[m]][m].n;
    Shape s;
    s.chunk = chunk;
    s.grid = grid[m] > 0 ? grid[m] : std::max(1, ntab);
    return s;
}

CellRes* CellEngine::new_cell(const int n[3], const double len[3], int nrhs) {
    CellRes* c = new CellRes();
    for (int d = 0; d < 3; ++d) {
        c->n[d] = n[d];
        c->len[d] = len[d];
    }
    c->nrhs = nrhs;
    c->model = model;
    c->nc = nc;
    c->nlev = cell_num_levels(n);
    c->bytes = cell_layout(*c, nullptr);
    c->E.assign(nrhs, std::array<double, 9>{});
    void* mem = nullptr;
    const cudaError_t e = cudaMallocAsync(&mem, c->bytes, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete c;
        throw hx::CudaErr(std::string("cell allocation: ") + cudaGetErrorString(e), e);
    }
    c->mem = (char*)mem;
    AEH_CHECK(cudaMemsetAsync(c->mem, 0, c->bytes, st));
    cell_layout(*c, c->mem);
    return c;
}

void CellEngine::free_cell(CellRes* c) {
    if (!c) return;
    if (c->mem) cudaFreeAsync(c->mem, st);
    if (c->gtab) cudaFreeAsync(c->gtab, st);
    delete c;
}

void CellEngine::set_grains(CellRes* c, int ng, const double* seeds, const double* table) {
    require(ng >= 1 && ng <= 65535, "grains: 1 to 65535 grains");
    require(seeds && table, "grains: seeds and table required");
    CellLevelDev& L = c->lv[0];
    if (c->gtab) AEH_CHECK(cudaFreeAsync(c->gtab, st));
    c->gtab = nullptr;
    // tables: stiffness FP64 and FP32, diagonal FP64, 1/diagonal FP64 and FP32
    const size_t n64 = (size_t)ng * nc, n32 = n64;
    const size_t bytes = align256(8 * n64) + align256(4 * n32) + 3 * align256(8 * 3 * (size_t)ng);
    void* mem = nullptr;
    AEH_CHECK(cudaMallocAsync(&mem, bytes, st));
    c->gtab = mem;
    char* p = (char*)mem;
    L.tab64 = (double*)p;
    p += align256(8 * n64);
    L.tab32 = (float*)p;
    p += align256(4 * n32);
    L.dtab64 = (double*)p;
    p += align256(8 * 3 * (size_t)ng);
    L.itab64 = (double*)p;
    p += align256(8 * 3 * (size_t)ng);
    L.itab32 = (float*)p;
    L.ngrains = ng;
    L.gid = c->gid_mem;
    void* sbuf = nullptr;
    AEH_CHECK(cudaMallocAsync(&sbuf, sizeof(double) * 3 * ng, st));
    AEH_CHECK(cudaMemcpyAsync(sbuf, seeds, sizeof(double) * 3 * ng, cudaMemcpyDefault, st));
    AEH_CHECK(cudaMemcpyAsync(L.tab64, table, sizeof(double) * n64, cudaMemcpyDefault, st));
    cells_launch_grains(model, L, c->len, (const double*)sbuf, ng, L.tab64, st);
    AEH_CHECK(cudaFreeAsync(sbuf, st));
    AEH_CHECK(cudaStreamSynchronize(st));
    c->model_set = true;
    c->prepared = false;
}

void CellEngine::set_field(CellRes* c, const void* C) {
    CellLevelDev& L = c->lv[0];
    L.gid = nullptr;
    L.ngrains = 0;
    L.tab64 = nullptr;
    L.tab32 = nullptr;
    L.dtab64 = nullptr;
    L.itab64 = nullptr;
    L.itab32 = nullptr;
    if (c->gtab) AEH_CHECK(cudaFreeAsync(c->gtab, st));
    c->gtab = nullptr;
    AEH_CHECK(cudaMemcpyAsync(L.C64, C, sizeof(double) * nc * (size_t)L.nn, cudaMemcpyDefault, st));
    AEH_CHECK(cudaStreamSynchronize(st));
    c->model_set = true;
    c->prepared = false;
}

void CellEngine::rebuild() {
    invalidate_graphs();
    const int ncell = (int)live.size();
    hcells.assign(ncell, CellDev{});
    hsolves.clear();
    solve_base.assign(ncell, 0);
    maxL = 0;
    reps0 = 0;
    for (int c = 0; c < ncell; ++c) {
        CellRes* r = live[c];
        CellDev& d = hcells[c];
        d.nlev = r->nlev;
        for (int m = 0; m < r->nlev; ++m) d.lv[m] = r->lv[m];
        solve_base[c] = (int)hsolves.size();
        for (int k = 0; k < r->nrhs; ++k) {
            SolveDev s = r->sol[k];
            s.cell = c;
            s.nlev = r->nlev;
            for (int q = 0; q < 9; ++q) s.E[q] = r->E[k][q];
            hsolves.push_back(s);
        }
        maxL = std::max(maxL, r->nlev);
        reps0 |= r->lv[0].gid ? 2 : 1;
    }
    nsolves = (int)hsolves.size();
    if ((size_t)ncell > cap_cells || !dcells) {
        if (dcells) AEH_CHECK(cudaFree(dcells));
        cap_cells = std::max<size_t>(std::max(ncell, 1), 2 * cap_cells);
        AEH_CHECK(cudaMalloc(&dcells, sizeof(CellDev) * cap_cells));
    }
    if ((size_t)nsolves > cap_solves || !dsolves) {
        if (dsolves) AEH_CHECK(cudaFree(dsolves));
        cap_solves = std::max<size_t>(std::max(nsolves, 1), 2 * cap_solves);
        AEH_CHECK(cudaMalloc(&dsolves, sizeof(SolveDev) * cap_solves));
    }
    if ((size_t)nsolves > cap_active || !dactive) {
        if (dactive) AEH_CHECK(cudaFree(dactive));
        if (hactive) AEH_CHECK(cudaFreeHost(hactive));
        cap_active = std::max<size_t>(std::max(nsolves, 1), 2 * cap_active);
        AEH_CHECK(cudaMalloc(&dactive, sizeof(int) * cap_active));
        AEH_CHECK(cudaMallocHost(&hactive, sizeof(int) * cap_active));
    }
    AEH_CHECK(cudaMemsetAsync(dactive, 0, sizeof(int) * cap_active, st));
    if (ncell) AEH_CHECK(cudaMemcpyAsync(dcells, hcells.data(), sizeof(CellDev) * ncell, cudaMemcpyHostToDevice, st));
    if (nsolves)
        AEH_CHECK(cudaMemcpyAsync(dsolves, hsolves.data(), sizeof(SolveDev) * nsolves, cudaMemcpyHostToDevice, st));
    // work tables: runs ordered cell, run, load case, so that the load cases of a cell read the
    // same stiffness run back to back (one HBM read, the rest from L2)
    for (int ci = 0; ci < 2; ++ci) {
        const int chunk = ci == 0 ? 128 : 256;
        for (int m = 0; m < kMaxCellLevels; ++m) {
            Table& T = tall[ci][m];
            T.h.clear();
            for (int c = 0; c < ncell; ++c) {
                const CellRes* r = live[c];
                if (m >= r->nlev) continue;
                for (int t0 = 0; t0 < r->lv[m].nn; t0 += chunk)
                    for (int k = 0; k < r->nrhs; ++k) T.h.push_back(Work{solve_base[c] + k, t0});
            }
            T.upload(st);
        }
    }
    tred.h.clear();
    for (int s = 0; s < nsolves; ++s) {
        const CellRes* r = live[hsolves[s].cell];
        for (int t0 = 0; t0 < r->lv[0].nn; t0 += kRedChunk) tred.h.push_back(Work{s, t0});
    }
    tred.upload(st);
    for (int m = 0; m < kMaxCellLevels; ++m) {
        Table& T = tcell[m];
        T.h.clear();
        for (int c = 0; c < ncell; ++c) {
            if (m >= live[c]->nlev) continue;
            for (int t0 = 0; t0 < live[c]->lv[m].nn; t0 += kRedChunk) T.h.push_back(Work{c, t0});
        }
        T.upload(st);
    }
    tuned[0] = tuned[1] = false;
    AEH_CHECK(cudaStreamSynchronize(st));
}

void CellEngine::upload_loads() {
    int s = 0;
    for (CellRes* r : live)
        for (int k = 0; k < r->nrhs; ++k, ++s)
            for (int q = 0; q < 9; ++q) hsolves[s].E[q] = r->E[k][q];
    if (nsolves)
        AEH_CHECK(cudaMemcpyAsync(dsolves, hsolves.data(), sizeof(SolveDev) * nsolves, cudaMemcpyHostToDevice, st));
    AEH_CHECK(cudaStreamSynchronize(st));
}

void CellEngine::prepare_cell(CellRes* c) {
    // a one-cell descriptor set for the set-up kernels
    const int slot = (int)(std::find(live.begin(), live.end(), c) - live.begin());
    require(slot < (int)live.size(), "cell is not live", AE_ERR_STATE);
    ae_solver_opts o;
    ae_default_solver_opts(&o);
    const CellArgs A = args(o);
    AEH_CHECK(cudaMemsetAsync(dnan, 0, sizeof(int), st));
    for (int m = 0; m < c->nlev; ++m) {
        tsub.h.clear();
        for (int t0 = 0; t0 < c->lv[m].nn; t0 += kRedChunk) tsub.h.push_back(Work{slot, t0});
        tsub.upload(st);
        if (m > 0) cells_launch_coarsen_C(model, A, tsub.d, tsub.n, m, st);
        cells_launch_diag(model, A, tsub.d, tsub.n, m, dnan, st);
    }
    AEH_CHECK(cudaMemcpyAsync(hcount + 1, dnan, sizeof(int), cudaMemcpyDeviceToHost, st));
    AEH_CHECK(cudaStreamSynchronize(st));
    require(hcount[1] == 0, "stiffness gives a NaN or zero diagonal", AE_ERR_NAN);
    c->prepared = true;
}

void CellEngine::subset(const std::vector<int>& cell_slots, std::vector<int>& slots) {
    slots.clear();
    tsub.h.clear();
    for (int c : cell_slots) {
        const CellRes* r = live[c];
        for (int k = 0; k < r->nrhs; ++k) {
            const int s = solve_base[c] + k;
            slots.push_back(s);
            for (int t0 = 0; t0 < r->lv[0].nn; t0 += kRedChunk) tsub.h.push_back(Work{s, t0});
        }
    }
    tsub.upload(st);
    if (slots.size() > cap_slots || !dslots) {
        if (dslots) AEH_CHECK(cudaFree(dslots));
        cap_slots = std::max<size_t>(std::max<size_t>(slots.size(), 1), 2 * cap_slots);
        AEH_CHECK(cudaMalloc(&dslots, sizeof(int) * cap_slots));
    }
    if (!slots.empty())
        AEH_CHECK(cudaMemcpyAsync(dslots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice, st));
}

// zero guess, b, its mean removed, the first residual and status of the given cells' solves
void CellEngine::begin(const std::vector<int>& cell_slots, const ae_solver_opts& o, double tol_rel, double tol_abs) {
    std::vector<int> slots;
    subset(cell_slots, slots);
    const int ns = (int)slots.size();
    const CellArgs A = args(o);
    const int prec = o.precision ? 1 : 0;
    cells_launch_begin(A, dslots, ns, st);
    cells_launch_zero_x(A, tsub.d, tsub.n, st);
    cells_launch_rhs(model, A, tsub.d, tsub.n, st);
    cells_launch_mean(A, dslots, ns, 0, 1, st);
    cells_launch_project(prec, 1, A, tsub.d, tsub.n, st);
    cells_launch_resid_top(model, A, tsub.d, tsub.n, reps0, st);
    cells_launch_mean(A, dslots, ns, 0, 0, st);
    cells_launch_project(prec, 0, A, tsub.d, tsub.n, st);
    cells_launch_status(A, dslots, ns, 1, tol_rel, tol_abs, o.max_iter, dcount, nullptr, st);
    // the subset scratch is reused by the next call: finish the host-side work first
    AEH_CHECK(cudaStreamSynchronize(st));
}

void CellEngine::smooth_phase(int prec, int m, int calls, bool zero, const ae_solver_opts& o, const CellArgs& A) {
    const Table& T = table(m);
    const Shape sh = shape(m);
    const int total = calls * o.sweeps;
    if (total <= 0) {
        if (zero) cells_launch_fill0(prec, A, T.d, T.n, sh, m, st);
        return;
    }
    int from2 = 0;
    for (int s = 0; s < total; ++s) {
        cells_launch_smooth(model, prec, zero && s == 0, A, T.d, T.n, sh, m, from2, reps(m), st);
        from2 ^= 1;
    }
    if (from2) cells_launch_copy2(prec, A, T.d, T.n, sh, m, st);
}

void CellEngine::vcycle(int prec, const ae_solver_opts& o) {
    const CellArgs A = args(o);
    for (int m = 0; m + 1 < maxL; ++m) {
        smooth_phase(prec, m, o.nu1, true, o, A);
        cells_launch_rescor(model, prec, A, table(m).d, table(m).n, shape(m), m, 0, reps(m), st);
        cells_launch_restrict(prec, A, table(m + 1).d, table(m + 1).n, shape(m + 1), m, st);
    }
    const KrylovParams kp{o.bottom, o.bottom_max_iter, o.bottom_reltol, o.nuf};
    cells_launch_bottom(model, prec, A, nsolves, kp, st);
    for (int m = maxL - 2; m >= 0; --m) {
        cells_launch_interp(prec, A, table(m).d, table(m).n, shape(m), m, st);
        smooth_phase(prec, m, o.nu2, false, o, A);
    }
}

// cycles + update + FP64 residual, mean, norm and status, all stream-ordered
void CellEngine::iteration_body(int prec, const ae_solver_opts& o, double tol_rel, double tol_abs) {
    const CellArgs A = args(o);
    const int inner = prec ? std::max(1, o.inner_cycles) : 1;
    for (int c = 0; c < inner; ++c) {
        vcycle(prec, o);
        cells_launch_update(prec, A, tred.d, tred.n, st);
        if (c + 1 < inner) cells_launch_rescor(model, prec, A, table(0).d, table(0).n, shape(0), 0, 1, reps0, st);
    }
    cells_launch_resid_top(model, A, tred.d, tred.n, reps0, st);
    cells_launch_mean(A, nullptr, nsolves, 0, 0, st);
    cells_launch_project(prec, 0, A, tred.d, tred.n, st);
    cells_launch_status(A, nullptr, nsolves, 0, tol_rel, tol_abs, o.max_iter, dcount, dactive, st);
}

static bool same_opts(const ae_solver_opts& a, const ae_solver_opts& b) {
    return a.nu1 == b.nu1 && a.nu2 == b.nu2 && a.sweeps == b.sweeps && a.bottom == b.bottom &&
           a.max_iter == b.max_iter && a.bottom_max_iter == b.bottom_max_iter && a.bottom_reltol == b.bottom_reltol &&
           a.nuf == b.nuf && a.omega == b.omega && a.precision == b.precision && a.inner_cycles == b.inner_cycles;
}

void CellEngine::iterate(int prec, const ae_solver_opts& o, double tol_rel, double tol_abs) {
    if (!o.use_graph) {
        iteration_body(prec, o, tol_rel, tol_abs);
        return;
    }
    // tolerances live in the captured status launch: key the graph on them through gopts
    ae_solver_opts key = o;
    key.max_fmg_iter = 0;
    if (gvalid[prec] && (!same_opts(gopts[prec], key) || gtol[prec][0] != tol_rel || gtol[prec][1] != tol_abs)) {
        cudaGraphExecDestroy(gexec[prec]);
        gexec[prec] = nullptr;
        gvalid[prec] = false;
    }
    if (!gvalid[prec]) {
        const long long before = g_kernel_launches.load();
        cudaGraph_t g = nullptr;
        AEH_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            iteration_body(prec, o, tol_rel, tol_abs);
        } catch (...) {
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        AEH_CHECK(cudaStreamEndCapture(st, &g));
        const cudaError_t e = cudaGraphInstantiate(&gexec[prec], g, 0);
        cudaGraphDestroy(g);
        AEH_CHECK(e);
        glaunches[prec] = g_kernel_launches.load() - before;
        g_kernel_launches.fetch_sub(glaunches[prec]);
        gopts[prec] = key;
        gtol[prec][0] = tol_rel;
        gtol[prec][1] = tol_abs;
        gvalid[prec] = true;
    }
    AEH_CHECK(cudaGraphLaunch(gexec[prec], st));
    g_kernel_launches.fetch_add(glaunches[prec]);
}

bool CellEngine::iterate_all(int prec, const ae_solver_opts& o, double tol_rel, double tol_abs) {
    if (!o.use_graph || !while_ok) return false;
    ae_solver_opts key = o;
    key.max_fmg_iter = 0;
    if (wvalid[prec] && (!same_opts(wopts[prec], key) || wtol[prec][0] != tol_rel || wtol[prec][1] != tol_abs)) {
        cudaGraphExecDestroy(wexec[prec]);
        wexec[prec] = nullptr;
        wvalid[prec] = false;
    }
    if (!wvalid[prec]) {
        cudaGraph_t g = nullptr;
        AEH_CHECK(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle h;
        cudaGraphNodeParams np = {};
        cudaGraphNode_t node;
        if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphDestroy(g);
            while_ok = false;
            return false;
        }
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphDestroy(g);
            while_ok = false;
            return false;
        }
        cudaGraph_t body = np.conditional.phGraph_out[0];
        const long long before = g_kernel_launches.load();
        AEH_CHECK(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        try {
            iteration_body(prec, o, tol_rel, tol_abs);
            cells_launch_loop_cond(h, dcount, dcount + 1, o.max_iter + 2, st);
        } catch (...) {
            cudaGraph_t tmp = nullptr;
            cudaStreamEndCapture(st, &tmp);
            cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t captured = nullptr;
        AEH_CHECK(cudaStreamEndCapture(st, &captured));
        const cudaError_t e = cudaGraphInstantiate(&wexec[prec], g, 0);
        cudaGraphDestroy(g);
        AEH_CHECK(e);
        wlaunches[prec] = g_kernel_launches.load() - before;
        g_kernel_launches.fetch_sub(wlaunches[prec]);
        wopts[prec] = key;
        wtol[prec][0] = tol_rel;
        wtol[prec][1] = tol_abs;
        wvalid[prec] = true;
    }
    AEH_CHECK(cudaMemsetAsync(dcount + 1, 0, sizeof(int), st));
    AEH_CHECK(cudaGraphLaunch(wexec[prec], st));
    AEH_CHECK(cudaMemcpyAsync(hcount + 1, dcount + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    AEH_CHECK(cudaStreamSynchronize(st));
    g_kernel_launches.fetch_add(wlaunches[prec] * hcount[1]);
    return true;
}

int CellEngine::read_count() {
    AEH_CHECK(cudaMemcpyAsync(hcount, dcount, sizeof(int), cudaMemcpyDeviceToHost, st));
    AEH_CHECK(cudaStreamSynchronize(st));
    return hcount[0];
}

const int* CellEngine::read_active() {
    if (nsolves) AEH_CHECK(cudaMemcpyAsync(hactive, dactive, sizeof(int) * nsolves, cudaMemcpyDeviceToHost, st));
    AEH_CHECK(cudaStreamSynchronize(st));
    return hactive;
}

// w with its mean removed and the cell-averaged stress of the given cells' solves
void CellEngine::finish(const std::vector<int>& cell_slots) {
    std::vector<int> slots;
    subset(cell_slots, slots);
    const int ns = (int)slots.size();
    ae_solver_opts o;
    ae_default_solver_opts(&o);
    const CellArgs A = args(o);
    cells_launch_xpart(A, tsub.d, tsub.n, st);
    cells_launch_mean(A, dslots, ns, 1, 1, st);
    cells_launch_project(0, 2, A, tsub.d, tsub.n, st);
    cells_launch_stress(model, A, tsub.d, tsub.n, st);
    cells_launch_mean(A, dslots, ns, 2, 1, st);
    AEH_CHECK(cudaStreamSynchronize(st));
}

// Launch shape per level: nodes per block (128 or 256) and the persistent grid size, timed on
// the smoother sweep of that level over the live set (the solves must be active: call after
// begin).  The per-node arithmetic does not depend on the shape, so results are unchanged.
void CellEngine::tune(int prec, const ae_solver_opts& o) {
    const CellArgs A = args(o);
    cudaEvent_t e0, e1;
    AEH_CHECK(cudaEventCreate(&e0));
    AEH_CHECK(cudaEventCreate(&e1));
    const int mults[] = {0, 2, 4, 8, 16, 32};
    for (int m = 0; m + 1 < maxL; ++m) {
        if (forced[m]) continue;
        float best = 1e30f;
        int bc = 1, bg = 0;
        for (int ci = 0; ci < 2; ++ci) {
            const Table& T = tall[ci][m];
            if (T.n == 0) continue;
            for (int mu : mults) {
                Shape sh;
                sh.chunk = ci == 0 ? 128 : 256;
                sh.grid = mu == 0 ? T.n : std::min(T.n, nsm * mu);
                if (mu != 0 && sh.grid == T.n) continue;
                cells_launch_smooth(model, prec, false, A, T.d, T.n, sh, m, 0, reps(m), st);  // warm
                AEH_CHECK(cudaEventRecord(e0, st));
                for (int r = 0; r < 3; ++r)
                    cells_launch_smooth(model, prec, false, A, T.d, T.n, sh, m, 0, reps(m), st);
                AEH_CHECK(cudaEventRecord(e1, st));
                AEH_CHECK(cudaEventSynchronize(e1));
                float ms = 0.f;
                AEH_CHECK(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    bc = ci;
                    bg = mu == 0 ? 0 : sh.grid;
                }
            }
        }
        chunk_idx[m] = bc;
        grid[m] = bg;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    invalidate_graphs();
    tuned[prec] = true;
}

}  // namespace ae

// ==================================================================== C ABI: ae_batch_*
struct ae_batch_s {
    CellEngine eng;
    std::vector<CellRes*> cells;  // in creation order (= live order)
    bool prepared = false;
    explicit ae_batch_s(int model) : eng(model) {}
};

namespace {

void check_desc(const ae_cell_desc& d) {
    for (int k = 0; k < 3; ++k) {
        require(d.n[k] >= 2, "cell: every node count must be >= 2");
        require(d.length[k] > 0.0, "cell: every length must be positive");
    }
    require(d.nrhs >= 1, "cell: nrhs must be >= 1");
    require((long long)d.n[0] * d.n[1] * d.n[2] < (1ll << 31) / 4, "cell too large");
}

CellRes* cell_of(ae_batch b, int cell) {
    require(b != nullptr, "null batch");
    require(cell >= 0 && cell < (int)b->cells.size(), "cell index out of range");
    return b->cells[cell];
}

std::pair<CellRes*, int> solve_of(ae_batch b, int solve) {
    require(b != nullptr, "null batch");
    int s = solve;
    require(s >= 0, "solve index out of range");
    for (CellRes* c : b->cells) {
        if (s < c->nrhs) return {c, s};
        s -= c->nrhs;
    }
    throw hx::ApiErr(AE_ERR_ARG, "solve index out of range");
}

// copy a cell-shaped fab [0, n-1]^3 (ncomp components) to/from device memory dst/src
void fab_cell_check(const ae_fab* f, const CellRes* c, int ncomp, const char* what) {
    require(f != nullptr && f->data != nullptr, std::string(what) + ": null fab");
    require(!f->is_float, std::string(what) + ": FP64 data required");
    require(f->ncomp >= ncomp, std::string(what) + ": needs " + std::to_string(ncomp) + " components");
    for (int d = 0; d < 3; ++d)
        require(f->lo[d] == 0 && f->hi[d] == c->n[d] - 1,
                std::string(what) + ": fab box must be [0, n-1] in every direction (the cell's unique nodes)");
}

}  // namespace

extern "C" {

long long ae_batch_plan_bytes(const ae_cell_desc* cell, int model) {
    if (!cell || model < 0 || model > 2) return -1;
    for (int d = 0; d < 3; ++d)
        if (cell->n[d] < 2) return -1;
    if (cell->nrhs < 1) return -1;
    return (long long)cell_plan_bytes(cell->n, cell->nrhs, model);
}

int ae_batch_create(const ae_cell_desc* cells, int ncells, int model, ae_batch* out) {
    return hx::guarded([&] {
        require(out != nullptr, "null output handle");
        *out = nullptr;
        require(cells != nullptr && ncells >= 1, "no cells");
        require(model >= 0 && model <= 2, "unknown model kind");
        for (int i = 0; i < ncells; ++i) check_desc(cells[i]);
        auto b = std::make_unique<ae_batch_s>(model);
        for (int i = 0; i < ncells; ++i) {
            CellRes* c = b->eng.new_cell(cells[i].n, cells[i].length, cells[i].nrhs);
            b->cells.push_back(c);
            b->eng.live.push_back(c);
        }
        b->eng.rebuild();
        *out = b.release();
    });
}

int ae_batch_destroy(ae_batch b) {
    return hx::guarded([&] { delete b; });
}

int ae_batch_num_solves(ae_batch b) { return b ? b->eng.nsolves : 0; }

int ae_batch_num_levels(ae_batch b, int cell) {
    if (!b || cell < 0 || cell >= (int)b->cells.size()) return 0;
    return b->cells[cell]->nlev;
}

long long ae_batch_device_bytes(ae_batch b) {
    if (!b) return 0;
    long long s = 0;
    for (CellRes* c : b->cells) s += (long long)c->bytes;
    return s;
}

int ae_batch_set_model(ae_batch b, int cell, const ae_fab* C) {
    return hx::guarded([&] {
        CellRes* c = cell_of(b, cell);
        fab_cell_check(C, c, c->nc, "ae_batch_set_model");
        b->eng.set_field(c, C->data);
        b->prepared = false;
    });
}

int ae_batch_set_model_grains(ae_batch b, int cell, int ngrains, const double* seeds, const double* table) {
    return hx::guarded([&] {
        CellRes* c = cell_of(b, cell);
        b->eng.set_grains(c, ngrains, seeds, table);
        b->prepared = false;
    });
}

int ae_batch_set_load(ae_batch b, int solve, const double* E) {
    return hx::guarded([&] {
        require(E != nullptr, "null displacement gradient");
        auto cs = solve_of(b, solve);
        for (int q = 0; q < 9; ++q) {
            require(std::isfinite(E[q]), "displacement gradient must be finite");
            cs.first->E[cs.second][q] = E[q];
        }
    });
}

int ae_batch_prepare(ae_batch b) {
    return hx::guarded([&] {
        require(b != nullptr, "null batch");
        for (CellRes* c : b->cells) require(c->model_set, "the model of every cell must be set", AE_ERR_STATE);
        b->eng.rebuild();  // descriptors carry each cell's finest-level representation
        for (CellRes* c : b->cells)
            if (!c->prepared) b->eng.prepare_cell(c);
        b->prepared = true;
    });
}

int ae_batch_set_shape(ae_batch b, int level, int chunk, int grid) {
    return hx::guarded([&] {
        require(b != nullptr, "null batch");
        require(level >= 0 && level < kMaxCellLevels, "level out of range");
        if (chunk == 0 && grid == 0) {
            b->eng.forced[level] = false;
            b->eng.tuned[0] = b->eng.tuned[1] = false;
        } else {
            require(chunk == 128 || chunk == 256, "chunk must be 128 or 256");
            require(grid >= 0, "grid must be >= 0 (0: one block per table entry)");
            b->eng.forced[level] = true;
            b->eng.chunk_idx[level] = chunk == 128 ? 0 : 1;
            b->eng.grid[level] = grid;
        }
        b->eng.invalidate_graphs();
    });
}

int ae_batch_get_shape(ae_batch b, int level, int* chunk, int* grid) {
    return hx::guarded([&] {
        require(b != nullptr && chunk && grid, "null argument");
        require(level >= 0 && level < kMaxCellLevels, "level out of range");
        const Shape s = b->eng.shape(level);
        *chunk = s.chunk;
        *grid = b->eng.grid[level];
    });
}

int ae_batch_solve(ae_batch b, double tol_rel, double tol_abs, const ae_solver_opts* opts, ae_cell_stats* stats) {
    return hx::guarded([&] {
        require(b != nullptr, "null batch");
        require(b->prepared, "ae_batch_prepare has not been called", AE_ERR_STATE);
        ae_solver_opts o;
        if (opts) o = *opts;
        else ae_default_solver_opts(&o);
        require(o.sweeps >= 1 && o.nu1 >= 0 && o.nu2 >= 0 && o.max_iter >= 0 && o.bottom_max_iter >= 0,
                "bad cycle counts");
        require(o.omega > 0.0 && o.omega < 2.0, "omega out of range");
        const auto t0 = std::chrono::steady_clock::now();
        CellEngine& E = b->eng;
        const int prec = o.precision ? 1 : 0;
        E.upload_loads();
        std::vector<int> all(E.live.size());
        for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
        E.begin(all, o, tol_rel, tol_abs);
        int count = E.read_count();
        // the tuner times smoother sweeps that write only the second correction buffers, which
        // the first sweep of every V-cycle overwrites
        if (!E.tuned[prec] && count > 0) E.tune(prec, o);
        // the whole iteration sequence as one graph launch (a device-side WHILE loop); the
        // host-polled replay where the runtime has no conditional nodes or graphs are off
        const bool whole = count > 0 && E.iterate_all(prec, o, tol_rel, tol_abs);
        if (whole) count = E.read_count();
        for (int it = 0; !whole && count > 0 && it <= o.max_iter + 1; ++it) {
            E.iterate(prec, o, tol_rel, tol_abs);
            count = E.read_count();
        }
        E.finish(all);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        bool all_conv = true, nan = false;
        std::vector<CellStatus> hs(E.nsolves);
        for (int s = 0; s < E.nsolves; ++s)
            AEH_CHECK(cudaMemcpyAsync(&hs[s], E.hsolves[s].st, sizeof(CellStatus), cudaMemcpyDeviceToHost, E.st));
        AEH_CHECK(cudaStreamSynchronize(E.st));
        for (int s = 0; s < E.nsolves; ++s) {
            const CellStatus& c = hs[s];
            if (!c.conv) all_conv = false;
            if (!std::isfinite(c.resn)) nan = true;
            if (stats) {
                ae_cell_stats& o2 = stats[s];
                o2.iters = c.iters;
                o2.converged = c.conv;
                o2.nlevels = E.hsolves[s].nlev;
                o2.bottom_fail = c.bfail;
                o2.res0 = c.res0;
                o2.resfinal = c.resn;
                o2.target = c.target;
                o2.seconds = secs;
                for (int q = 0; q < 3; ++q) o2.body_force[q] = c.mean[q];
                for (int q = 0; q < 9; ++q) o2.mean_stress[q] = c.sig[q];
            }
        }
        if (nan) throw hx::ApiErr(AE_ERR_NAN, "a cell residual became NaN or infinite");
        if (!all_conv) throw hx::ApiErr(AE_ERR_NOT_CONVERGED, "not every cell solve converged within max_iter");
    });
}

int ae_batch_solution(ae_batch b, int solve, ae_fab* w) {
    return hx::guarded([&] {
        auto cs = solve_of(b, solve);
        CellRes* c = cs.first;
        fab_cell_check(w, c, 3, "ae_batch_solution");
        const size_t bytes = sizeof(double) * 3 * (size_t)c->lv[0].nn;
        AEH_CHECK(cudaMemcpyAsync(w->data, c->sol[cs.second].x, bytes, cudaMemcpyDefault, b->eng.st));
        AEH_CHECK(cudaStreamSynchronize(b->eng.st));
    });
}

}  // extern "C"
