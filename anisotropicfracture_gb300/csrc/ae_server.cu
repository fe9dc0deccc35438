// Serving loop for periodic-cell homogenisation requests: the ae_server_* C ABI.
//
// A request is one periodic cell (its stiffness as a Voronoi description or a full field) with
// nrhs load cases.  A worker thread owns a CellEngine and runs continuous batching: between
// iterations it admits queued requests whose device memory fits the budget (FIFO), builds their
// stiffness and hierarchy on the device and starts their solves; every iteration advances all
// live solves together; a request whose solves have all finished is completed (w mean-free,
// cell-averaged stresses), its results copied to the host and its memory returned.  A request's
// arithmetic does not depend on the requests it shares the device with.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ae_cells_engine.h"
#include "ae_host.h"

using namespace ae;
using ae::hx::require;

namespace {

struct Request {
    long long ticket = 0;
    ae_cell_desc desc{};
    int ngrains = 0;
    std::vector<double> seeds, table;  // Voronoi description, or
    std::vector<double> field;         // a full stiffness field (ncoef x nn)
    std::vector<std::array<double, 9>> E;
    int state = 1;  // 1 queued, 2 running, 0 done, < 0 failed (ae_status)
    std::string error;
    double t_submit = 0, t_admit = 0, t_done = 0;
    size_t bytes = 0;
    CellRes* cell = nullptr;
    std::vector<ae_cell_stats> stats;
    std::vector<double> w;  // nrhs x 3 x nn (keep_solution)
};

}  // namespace

struct ae_server_s {
    int model = 0;
    int dev = 0;
    ae_server_opts opts{};
    std::unique_ptr<CellEngine> eng;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    bool fatal = false;
    std::string fatal_msg;
    std::deque<Request*> queue;
    std::map<long long, std::unique_ptr<Request>> reqs;
    long long next_ticket = 1;
    size_t budget = 0, used = 0;
    long long completed = 0, failed = 0, iterations = 0;
    double busy = 0.0;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
    void run();
    void fail_live(const std::string& msg);
};

namespace {

ae_cell_stats stats_of(const CellStatus& c, int nlev) {
    ae_cell_stats o{};
    o.iters = c.iters;
    o.converged = c.conv;
    o.nlevels = nlev;
    o.bottom_fail = c.bfail;
    o.res0 = c.res0;
    o.resfinal = c.resn;
    o.target = c.target;
    for (int q = 0; q < 3; ++q) o.body_force[q] = c.mean[q];
    for (int q = 0; q < 9; ++q) o.mean_stress[q] = c.sig[q];
    return o;
}

}  // namespace

void ae_server_s::fail_live(const std::string& msg) {
    std::lock_guard<std::mutex> lk(mu);
    for (CellRes* c : eng->live) {
        auto it = reqs.find(c->tag);
        if (it != reqs.end() && it->second->state == 2) {
            it->second->state = AE_ERR_CUDA;
            it->second->error = msg;
            it->second->t_done = now();
            ++failed;
        }
    }
    fatal = true;
    fatal_msg = msg;
    cv_done.notify_all();
}

void ae_server_s::run() {
    cudaSetDevice(dev);
    CellEngine& E = *eng;
    const ae_solver_opts& o = opts.solver;
    const int prec = o.precision ? 1 : 0;
    try {
        for (;;) {
            // ---- admission: FIFO while the head fits the memory budget and the solve limit
            std::vector<Request*> admit;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (E.live.empty())
                    cv_work.wait(lk, [&] { return stop || !queue.empty(); });
                if (stop) break;
                int live_solves = E.nsolves;
                while (!queue.empty()) {
                    Request* r = queue.front();
                    if (used + r->bytes > budget) break;
                    if (opts.max_live_solves > 0 && live_solves + r->desc.nrhs > opts.max_live_solves &&
                        live_solves > 0)
                        break;
                    queue.pop_front();
                    used += r->bytes;
                    live_solves += r->desc.nrhs;
                    r->state = 2;
                    r->t_admit = now();
                    admit.push_back(r);
                }
            }
            const auto tb = std::chrono::steady_clock::now();
            if (!admit.empty()) {
                std::vector<Request*> ok;
                for (Request* r : admit) {
                    try {
                        CellRes* c = E.new_cell(r->desc.n, r->desc.length, r->desc.nrhs);
                        c->tag = r->ticket;
                        r->cell = c;
                        for (int k = 0; k < r->desc.nrhs; ++k) c->E[k] = r->E[k];
                        // both synchronise the stream: the host inputs may be released afterwards
                        if (r->ngrains > 0) E.set_grains(c, r->ngrains, r->seeds.data(), r->table.data());
                        else E.set_field(c, r->field.data());
                        r->field.clear();
                        r->field.shrink_to_fit();
                        E.live.push_back(c);
                        ok.push_back(r);
                    } catch (const hx::CudaErr& e) {
                        if (e.err != cudaErrorMemoryAllocation) throw;
                        std::lock_guard<std::mutex> lk(mu);
                        r->state = AE_ERR_OOM;
                        r->error = e.what();
                        r->t_done = now();
                        used -= r->bytes;
                        if (r->cell) {
                            E.free_cell(r->cell);
                            r->cell = nullptr;
                        }
                        ++failed;
                        cv_done.notify_all();
                    }
                }
                E.rebuild();
                std::vector<int> slots;
                for (Request* r : ok) {
                    bool good = true;
                    try {
                        E.prepare_cell(r->cell);
                    } catch (const hx::ApiErr& e) {
                        good = false;
                        std::lock_guard<std::mutex> lk(mu);
                        r->state = e.code;
                        r->error = e.what();
                    }
                    if (good) {
                        const int slot = (int)(std::find(E.live.begin(), E.live.end(), r->cell) - E.live.begin());
                        slots.push_back(slot);
                    }
                }
                // drop requests whose stiffness was rejected
                bool dropped = false;
                for (Request* r : ok)
                    if (r->state < 0) {
                        E.live.erase(std::find(E.live.begin(), E.live.end(), r->cell));
                        E.free_cell(r->cell);
                        r->cell = nullptr;
                        std::lock_guard<std::mutex> lk(mu);
                        used -= r->bytes;
                        r->t_done = now();
                        ++failed;
                        dropped = true;
                    }
                if (dropped) {
                    E.rebuild();
                    slots.clear();
                    for (Request* r : ok)
                        if (r->state == 2)
                            slots.push_back((int)(std::find(E.live.begin(), E.live.end(), r->cell) - E.live.begin()));
                    cv_done.notify_all();
                }
                if (!slots.empty()) E.begin(slots, o, opts.tol_rel, opts.tol_abs);
            }
            if (E.live.empty()) continue;
            // ---- one iteration of every live solve
            E.iterate(prec, o, opts.tol_rel, opts.tol_abs);
            const int* act = E.read_active();
            ++iterations;
            // ---- retire requests with no active solve
            std::vector<int> done_slots;
            for (int c = 0; c < (int)E.live.size(); ++c) {
                const CellRes* cr = E.live[c];
                bool any = false;
                for (int k = 0; k < cr->nrhs; ++k) any = any || act[E.solve_base[c] + k];
                if (!any) done_slots.push_back(c);
            }
            if (!done_slots.empty()) {
                E.finish(done_slots);
                std::vector<CellRes*> gone;
                for (int c : done_slots) {
                    CellRes* cr = E.live[c];
                    std::vector<CellStatus> hs(cr->nrhs);
                    for (int k = 0; k < cr->nrhs; ++k)
                        AEH_CHECK(cudaMemcpyAsync(&hs[k], cr->sol[k].st, sizeof(CellStatus), cudaMemcpyDeviceToHost,
                                                  E.st));
                    Request* r = nullptr;
                    {
                        std::lock_guard<std::mutex> lk(mu);
                        r = reqs[cr->tag].get();
                    }
                    const size_t nn = (size_t)cr->lv[0].nn;
                    if (opts.keep_solution) {
                        r->w.assign((size_t)cr->nrhs * 3 * nn, 0.0);
                        for (int k = 0; k < cr->nrhs; ++k)
                            AEH_CHECK(cudaMemcpyAsync(r->w.data() + (size_t)k * 3 * nn, cr->sol[k].x,
                                                      sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, E.st));
                    }
                    AEH_CHECK(cudaStreamSynchronize(E.st));
                    bool conv = true;
                    r->stats.resize(cr->nrhs);
                    for (int k = 0; k < cr->nrhs; ++k) {
                        r->stats[k] = stats_of(hs[k], cr->nlev);
                        conv = conv && hs[k].conv;
                    }
                    gone.push_back(cr);
                    std::lock_guard<std::mutex> lk(mu);
                    r->t_done = now();
                    for (auto& s : r->stats) s.seconds = r->t_done - r->t_submit;
                    r->state = conv ? AE_OK : AE_ERR_NOT_CONVERGED;
                    used -= r->bytes;
                    r->cell = nullptr;
                    if (conv) ++completed;
                    else ++failed;
                }
                for (CellRes* cr : gone) {
                    E.live.erase(std::find(E.live.begin(), E.live.end(), cr));
                    E.free_cell(cr);
                }
                E.rebuild();
                cv_done.notify_all();
            }
            busy += std::chrono::duration<double>(std::chrono::steady_clock::now() - tb).count();
        }
    } catch (const std::exception& e) {
        fail_live(e.what());
    }
}

extern "C" {

void ae_server_default_opts(ae_server_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->hbm_budget_bytes = 0;
    o->max_live_solves = 0;
    o->keep_solution = 0;
    o->tol_rel = 1e-8;
    o->tol_abs = 0.0;
    ae_default_solver_opts(&o->solver);
    o->solver.max_fmg_iter = 0;
    o->solver.bottom = 1;
    o->solver.precision = 1;
    // FP32 cycles per FP64 residual: the FP64 residual of a cell batch costs about a third of
    // an FP32 V-cycle on GB300, so 4 (512-cell batch: 443 solves/s, against 396 with 2;
    // displacement error 4.6e-8 against FP64)
    o->solver.inner_cycles = 4;
    o->solver.use_graph = 1;
}

int ae_server_create(int model, const ae_server_opts* opts, ae_server* out) {
    return hx::guarded([&] {
        require(out != nullptr, "null output handle");
        *out = nullptr;
        require(model >= 0 && model <= 2, "unknown model kind");
        auto s = std::make_unique<ae_server_s>();
        s->model = model;
        if (opts) s->opts = *opts;
        else ae_server_default_opts(&s->opts);
        const ae_solver_opts& o = s->opts.solver;
        require(o.sweeps >= 1 && o.nu1 >= 0 && o.nu2 >= 0 && o.max_iter >= 0 && o.omega > 0.0 && o.omega < 2.0,
                "bad solver options");
        AEH_CHECK(cudaGetDevice(&s->dev));
        size_t fr = 0, tot = 0;
        AEH_CHECK(cudaMemGetInfo(&fr, &tot));
        s->budget = s->opts.hbm_budget_bytes > 0 ? (size_t)s->opts.hbm_budget_bytes : (size_t)(0.8 * (double)fr);
        s->eng = std::make_unique<CellEngine>(model);
        ae_server_s* raw = s.get();
        s->worker = std::thread([raw] { raw->run(); });
        *out = s.release();
    });
}

int ae_server_destroy(ae_server s) {
    return hx::guarded([&] {
        if (!s) return;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        if (s->worker.joinable()) s->worker.join();
        delete s;
    });
}

int ae_server_submit(ae_server s, const ae_cell_desc* desc, int ngrains, const double* seeds, const double* table,
                     const ae_fab* C, const double* E, long long* ticket) {
    return hx::guarded([&] {
        require(s != nullptr && desc != nullptr && E != nullptr && ticket != nullptr, "null argument");
        for (int k = 0; k < 3; ++k) {
            require(desc->n[k] >= 2, "cell: every node count must be >= 2");
            require(desc->length[k] > 0.0, "cell: every length must be positive");
        }
        require(desc->nrhs >= 1, "cell: nrhs must be >= 1");
        const int nc = s->model == AE_MODEL_ISOTROPIC ? 2 : s->model == AE_MODEL_MAJORMINOR ? 21 : 9;
        auto r = std::make_unique<Request>();
        r->desc = *desc;
        const size_t nn = (size_t)desc->n[0] * desc->n[1] * desc->n[2];
        if (ngrains > 0) {
            require(seeds && table, "grains: seeds and table required");
            r->ngrains = ngrains;
            r->seeds.assign(seeds, seeds + 3 * (size_t)ngrains);
            r->table.assign(table, table + (size_t)nc * ngrains);
        } else {
            require(C && C->data && !C->is_float && C->ncomp >= nc, "need a grain description or an FP64 field");
            for (int d = 0; d < 3; ++d)
                require(C->lo[d] == 0 && C->hi[d] == desc->n[d] - 1, "field box must be [0, n-1] per direction");
            require(!hx::is_device_ptr(C->data), "the field must be host memory");
            const double* p = static_cast<const double*>(C->data);
            r->field.assign(p, p + nc * nn);
        }
        r->E.resize(desc->nrhs);
        for (int k = 0; k < desc->nrhs; ++k)
            for (int q = 0; q < 9; ++q) {
                require(std::isfinite(E[9 * k + q]), "displacement gradient must be finite");
                r->E[k][q] = E[9 * k + q];
            }
        r->bytes = cell_plan_bytes(desc->n, desc->nrhs, s->model);
        std::lock_guard<std::mutex> lk(s->mu);
        require(!s->fatal, "server stopped after a device error: " + s->fatal_msg, AE_ERR_CUDA);
        require(r->bytes <= s->budget, "request needs more device memory than the server's budget", AE_ERR_OOM);
        r->ticket = s->next_ticket++;
        r->t_submit = s->now();
        *ticket = r->ticket;
        s->queue.push_back(r.get());
        s->reqs[r->ticket] = std::move(r);
        s->cv_work.notify_all();
    });
}

static void fill_info(ae_server s, Request* r, ae_request_info* info, ae_cell_stats* stats, double* w) {
    if (info) {
        info->status = r->state;
        info->nrhs = r->desc.nrhs;
        info->t_submit = r->t_submit;
        info->t_admit = r->t_admit;
        info->t_done = r->t_done;
        info->latency = r->state <= 0 ? r->t_done - r->t_submit : -1.0;
    }
    if (r->state <= 0) {
        if (stats)
            for (size_t k = 0; k < r->stats.size(); ++k) stats[k] = r->stats[k];
        if (w && !r->w.empty()) std::memcpy(w, r->w.data(), sizeof(double) * r->w.size());
    }
    (void)s;
}

int ae_server_poll(ae_server s, long long ticket, ae_request_info* info, ae_cell_stats* stats, double* w) {
    return hx::guarded([&] {
        require(s != nullptr, "null server");
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        require(it != s->reqs.end(), "unknown ticket");
        fill_info(s, it->second.get(), info, stats, w);
    });
}

int ae_server_wait(ae_server s, long long ticket, double timeout_s, ae_request_info* info, ae_cell_stats* stats,
                   double* w) {
    return hx::guarded([&] {
        require(s != nullptr, "null server");
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        require(it != s->reqs.end(), "unknown ticket");
        Request* r = it->second.get();
        const auto pred = [&] { return r->state <= 0 || s->fatal; };
        if (timeout_s < 0) s->cv_done.wait(lk, pred);
        else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
        fill_info(s, r, info, stats, w);
    });
}

int ae_server_release(ae_server s, long long ticket) {
    return hx::guarded([&] {
        require(s != nullptr, "null server");
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        require(it != s->reqs.end(), "unknown ticket");
        require(it->second->state <= 0, "request still in flight", AE_ERR_STATE);
        s->reqs.erase(it);
    });
}

int ae_server_get_stats(ae_server s, ae_server_stats* out) {
    return hx::guarded([&] {
        require(s != nullptr && out != nullptr, "null argument");
        std::lock_guard<std::mutex> lk(s->mu);
        out->submitted = s->next_ticket - 1;
        out->completed = s->completed;
        out->failed = s->failed;
        out->queued = (long long)s->queue.size();
        out->iterations = s->iterations;
        out->hbm_used = (long long)s->used;
        out->hbm_budget = (long long)s->budget;
        out->busy_seconds = s->busy;
        out->uptime_seconds = s->now();
    });
}

}  // extern "C"
