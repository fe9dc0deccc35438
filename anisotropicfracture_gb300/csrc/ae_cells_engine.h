// Host engine of the batched periodic-cell solve (ae_cells.cu): device resources of a cell and
// its solves, the live set with its work tables, and the stream-ordered steps of the solve.
// The batch ABI (ae_batch_*) drives one engine over a fixed set of cells; the server
// (ae_server_*) admits and retires cells between iterations of its engine.
#pragma once
#include <array>
#include <cstddef>
#include <vector>

#include "../../include/aefast.h"
#include "ae_cells.h"

namespace ae {

// one periodic cell: its hierarchy and its solves, in one device allocation
struct CellRes {
    int n[3] = {0, 0, 0};
    double len[3] = {1, 1, 1};
    int nlev = 0;
    int nrhs = 0;
    int model = 0;
    int nc = 0;
    char* mem = nullptr;
    size_t bytes = 0;
    unsigned short* gid_mem = nullptr;  // grain ids of the finest level (inside mem)
    void* gtab = nullptr;               // grain tables of a Voronoi cell (own allocation)
    CellLevelDev lv[kMaxCellLevels];
    std::vector<SolveDev> sol;
    std::vector<std::array<double, 9>> E;
    bool model_set = false;
    bool prepared = false;
    long long tag = 0;  // owner's id (the server's ticket)
};

// multigrid levels of a periodic cell: halve while every count is even and stays >= 2
int cell_num_levels(const int n[3]);
// device bytes one cell with nrhs solves needs (both cycle precisions)
size_t cell_plan_bytes(const int n[3], int nrhs, int model);

struct Table {
    Work* d = nullptr;
    size_t cap = 0;
    int n = 0;
    std::vector<Work> h;
    void upload(cudaStream_t st);
    void release();
};

struct CellEngine {
    int model = 0, nc = 0;
    cudaStream_t st = nullptr;
    int nsm = 0;
    std::vector<CellRes*> live;  // cell slots
    // descriptors of the live set
    std::vector<CellDev> hcells;
    std::vector<SolveDev> hsolves;
    CellDev* dcells = nullptr;
    size_t cap_cells = 0;
    SolveDev* dsolves = nullptr;
    size_t cap_solves = 0;
    int nsolves = 0, maxL = 0;
    int reps0 = 1;  // finest-level representations present (bit 0 per-node, bit 1 grain tables)
    int reps(int m) const { return m == 0 ? reps0 : 1; }
    std::vector<int> solve_base;  // first solve slot of each cell slot
    // tables: per chunk option (128, 256) and level, solves; level-0 reduction runs; cells
    Table tall[2][kMaxCellLevels];
    Table tred;
    Table tcell[kMaxCellLevels];
    // launch shapes per level (chunk option index and grid); forced[m] set by the caller
    int chunk_idx[kMaxCellLevels];
    int grid[kMaxCellLevels];
    bool forced[kMaxCellLevels];
    bool tuned[2] = {false, false};
    int* dcount = nullptr;
    int* hcount = nullptr;  // pinned
    int* dnan = nullptr;
    int* dactive = nullptr;  // per solve slot: still active after the last status (device, pinned mirror)
    int* hactive = nullptr;
    size_t cap_active = 0;
    // subset scratch (begin/finish of some cells)
    Table tsub;
    int* dslots = nullptr;
    size_t cap_slots = 0;
    // one graph per cycle precision of the iteration body
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    long long glaunches[2] = {0, 0};
    ae_solver_opts gopts[2];
    double gtol[2][2] = {{0, 0}, {0, 0}};
    bool gvalid[2] = {false, false};
    // one graph per precision that runs the whole iteration sequence: a conditional WHILE node
    // whose body is the iteration and the loop condition (dcount[1] counts the iterations)
    cudaGraphExec_t wexec[2] = {nullptr, nullptr};
    long long wlaunches[2] = {0, 0};
    ae_solver_opts wopts[2];
    double wtol[2][2] = {{0, 0}, {0, 0}};
    bool wvalid[2] = {false, false};
    bool while_ok = true;  // false once the runtime refused a conditional node

    explicit CellEngine(int model);
    ~CellEngine();
    CellArgs args(const ae_solver_opts& o) const;
    Shape shape(int m) const;
    const Table& table(int m) const { return tall[chunk_idx[m]][m]; }

    // allocate a cell's device memory (stream-ordered) and lay it out
    CellRes* new_cell(const int n[3], const double len[3], int nrhs);
    void free_cell(CellRes* c);
    // descriptors and tables from `live`
    void rebuild();
    void upload_loads();  // E of every solve
    // coarsen the stiffness, diagonals, FP32 copies of a cell; NaN/zero-diagonal check
    void prepare_cell(CellRes* c);
    // finest-level stiffness of a Voronoi cell (host seeds ng x 3 and table ng x ncoef): the
    // per-node field, the grain ids and the grain tables the finest-level kernels read
    void set_grains(CellRes* c, int ng, const double* seeds, const double* table);
    // finest-level stiffness as a per-node field (host or device, ncoef x nn)
    void set_field(CellRes* c, const void* C);

    // solve steps on the stream
    void begin(const std::vector<int>& cell_slots, const ae_solver_opts& o, double tol_rel, double tol_abs);
    void vcycle(int prec, const ae_solver_opts& o);
    void iteration_body(int prec, const ae_solver_opts& o, double tol_rel, double tol_abs);
    void iterate(int prec, const ae_solver_opts& o, double tol_rel, double tol_abs);  // graph or direct
    // every iteration until no solve is active (or max_iter + 2 of them) in one graph launch;
    // false (nothing run) when graphs are off or the runtime has no conditional nodes
    bool iterate_all(int prec, const ae_solver_opts& o, double tol_rel, double tol_abs);
    int read_count();
    // per-slot active flags of the last iteration (host copy, valid after read_active)
    const int* read_active();
    void finish(const std::vector<int>& cell_slots);
    void tune(int prec, const ae_solver_opts& o);
    void invalidate_graphs();

   private:
    void smooth_phase(int prec, int m, int calls, bool zero, const ae_solver_opts& o, const CellArgs& A);
    void subset(const std::vector<int>& cell_slots, std::vector<int>& slots);
};

}  // namespace ae
