/*
 * aefast.h -- C ABI of the GB300 elastic-operator library (libaefast.so).
 *
 * This is the drop-in boundary for the reference's nodal linear-elastic solve path:
 * Operator::Elastic<T> (src/Operator/Elastic.H:20-171), its base
 * Operator::Operator<Grid::Node> (src/Operator/Operator.H:30-128), the operator
 * boundary conditions BC::Operator::Elastic<T> (src/BC/Operator/Elastic.H:12-406)
 * and the Solver::Nonlocal::Linear / Newton<T> drivers
 * (src/Solver/Nonlocal/Linear.H:19-143, src/Solver/Nonlocal/Newton.H:15-349).
 * The reference exposes these as C++ virtuals on AMReX types; this header gives the
 * same operations as plain C entry points over plain pointers and sizes.
 * include/alamo_elastic.H wraps it back into the reference's class and method names.
 *
 * Conventions
 *  - Every function returns an ae_status (0 = success, negative = error);
 *    ae_last_error() gives a message for the calling thread.
 *  - Fields are described by ae_fab, which is the memory layout of an AMReX
 *    FArrayBox/Array4: index box [lo, hi] (ghost nodes included), i fastest, then j,
 *    then k, then the component.  Nodal indices; the problem domain starts at 0.
 *  - Kernel-level entry points (ae_fapply ... ae_interp_add) take DEVICE pointers and
 *    are ordered on the operator's stream (ae_op_set_stream).  ae_op_set_model and
 *    ae_solve accept host or device pointers.
 *  - One operator handle may be used by one host thread at a time; distinct handles
 *    are independent.
 */
#ifndef AEFAST_H
#define AEFAST_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ae_op_s ae_op;

typedef enum {
    AE_OK = 0,
    AE_ERR_ARG = -1,           /* bad argument (sizes, layout, index out of range)         */
    AE_ERR_NAN = -2,           /* NaN/Inf found (diagonal, residual)                        */
    AE_ERR_NOT_CONVERGED = -3, /* solver reached max_iter (reference: MLMG aborts)          */
    AE_ERR_OOM = -4,           /* device allocation failed                                  */
    AE_ERR_CUDA = -5,          /* CUDA runtime error                                        */
    AE_ERR_STATE = -6          /* call order violated (e.g. solve before set_model)         */
} ae_status;

/* Per-node stiffness kinds (Model::Solid::Solid<Sym>::ddw storage).
 *  ISOTROPIC : 2 coefficients (lambda, mu)        Set::Matrix4<3,Sym::Isotropic>
 *  MAJORMINOR: 21 coefficients (reference slots)   Set::Matrix4<3,Sym::MajorMinor>
 *  DIAGONAL  : 9 coefficients A(i,j), row-major    Set::Matrix4<3,Sym::Diagonal>
 *  MAJOR     : 45 coefficients, the upper triangle of the 9 x 9 matrix A(3i+j, 3k+l) row by row
 *              (src/Set/Matrix4_Major.H:203-258)  Set::Matrix4<3,Sym::Major>: the tangent
 *              DDW of a finite-kinematics model (Model::Solid::Elastic::NeoHookean).  No grain
 *              maps (ae_op_set_model_grains), no Stress / Energy / NewtonResidual / NewtonDW
 *              (those evaluate a linear model); ae_newton_neohookean sets it.            */
typedef enum {
    AE_MODEL_ISOTROPIC = 0,
    AE_MODEL_MAJORMINOR = 1,
    AE_MODEL_DIAGONAL = 2,
    AE_MODEL_MAJOR = 3
} ae_model_kind;

/* BC::Operator::Elastic<T>::Type, same numbering (src/BC/Operator/Elastic.H:24) */
typedef enum { AE_BC_DISPLACEMENT = 0, AE_BC_TRACTION = 1, AE_BC_PERIODIC = 2, AE_BC_NEUMANN = 3 } ae_bc_type;

/* Face/edge/corner numbering of BC::Operator::Elastic<T>::Face (src/BC/Operator/Elastic.H:33-41) */
enum {
    AE_XLO, AE_YLO, AE_ZLO, AE_XHI, AE_YHI, AE_ZHI,
    AE_YLO_ZLO, AE_YLO_ZHI, AE_YHI_ZLO, AE_YHI_ZHI,
    AE_ZLO_XLO, AE_ZLO_XHI, AE_ZHI_XLO, AE_ZHI_XHI,
    AE_XLO_YLO, AE_XLO_YHI, AE_XHI_YLO, AE_XHI_YHI,
    AE_XLO_YLO_ZLO, AE_XLO_YLO_ZHI, AE_XLO_YHI_ZLO, AE_XLO_YHI_ZHI,
    AE_XHI_YLO_ZLO, AE_XHI_YLO_ZHI, AE_XHI_YHI_ZLO, AE_XHI_YHI_ZHI,
    AE_NFACES
};

/* One AMR level: a single nodal patch inside the level's problem domain.
 * Replaces the Geometry/BoxArray pair passed to Operator::Elastic<T>::define
 * (src/Operator/Elastic.cpp:30-55).  Level l+1 refines level l by 2. */
typedef struct {
    int domain_cells[3]; /* cells of the level's problem domain (nodal domain = [0, cells]) */
    int lo[3], hi[3];    /* nodal valid box of the level's patch (inclusive)                */
    double dx[3];        /* cell size                                                        */
} ae_level_desc;

/* Field view in AMReX Array4 layout (see conventions above). */
typedef struct {
    void* data;        /* element (lo, comp 0)                                              */
    int lo[3], hi[3];  /* index box spanned by data (inclusive, ghosts included)            */
    int ncomp;
    int is_float;      /* 0: double, 1: float                                               */
} ae_fab;

/* Solver options: AMReX MLMG knobs set by Solver::Nonlocal::Linear
 * (src/Solver/Nonlocal/Linear.H:23-29, Parse :121-140). */
typedef struct {
    int max_fmg_iter;     /* iterations run as F-cycles before V-cycles (MLMG max_fmg_iter;    
                             reference default 1e8: always F; 0: always V)                     */
    int nu1, nu2;         /* smoother calls before/after the coarse correction (MLMG nu1/nu2) */
    int sweeps;           /* damped-Jacobi sweeps per smoother call (reference Fsmooth: 2)    */
    int bottom;           /* 0: CG, 1: BiCGStab (reference default)                           */
    int max_iter;         /* MLMG max_iter                                                    */
    int bottom_max_iter;  /* MLMG bottom_max_iter                                             */
    double bottom_reltol; /* MLMG bottom relative tolerance                                   */
    int nuf;              /* smoother calls after a failed bottom solve                       */
    int max_mg_levels;    /* cap on multigrid levels (<= 0: coarsen while possible)           */
    double omega;         /* Jacobi damping (reference: 2/3)                                  */
    int precision;        /* 0: FP64 throughout; 1: FP32 cycle inside FP64 refinement         */
    int inner_cycles;     /* precision 1: FP32 cycles per FP64 residual                       */
    int verbose;
    int use_graph;        /* capture each iteration in a CUDA graph                           */
    int fixed_iter;       /* > 0: run exactly this many iterations, converged or not (MLMG     
                             fixed_iter, Solver::Nonlocal::Linear::Parse "fixed_iter",
                             src/Solver/Nonlocal/Linear.H:132-133); 0: iterate to the tolerance */
} ae_solver_opts;

typedef struct {
    int iters;            /* outer iterations (MLMG iterations, or refinement steps)          */
    int cycles;           /* multigrid cycles executed                                        */
    int converged;
    int nlevels;          /* multigrid levels on AMR level 0                                  */
    int bottom_fail;      /* bottom solves that did not converge (smoother fallback used)     */
    int pad_;
    double res0, resfinal, target;
    double seconds;       /* wall time of the solve call                                      */
} ae_solve_stats;

const char* ae_last_error(void);
const char* ae_version(void);
void ae_default_solver_opts(ae_solver_opts* o);

/* Operator::Elastic<T>::define + Operator<Grid::Node>::define (Elastic.cpp:30-55,
 * Operator.cpp:215-258): allocates the multigrid hierarchy and the operator diagonal.
 * levels: the patches of the AMR hierarchy, level by level.  Entry 0 covers the level-0 domain.
 * Each finer level refines the one before by 2 (domain_cells doubled); consecutive entries with
 * the same domain_cells are the patches of one level (an AMReX BoxArray), each nested in one
 * patch of the level below and separated from the level's other patches: their storage boxes,
 * the nodal patch grown by 2, may not meet.  Touching boxes whose union is a box are passed as
 * that one box.  Every other call's amrlev is an index into this list, and solves take one fab
 * per entry. */
int ae_op_create(const ae_level_desc* levels, int nlev, int model, ae_op** out);
int ae_op_destroy(ae_op* op);
/* cudaStream_t passed as void*; NULL selects the operator's own stream, a blocking
 * stream that is ordered with the legacy default stream. */
int ae_op_set_stream(ae_op* op, void* stream);
/* Operator::Elastic<T>::SetModel(amrlev, FabArray) (Elastic.cpp:84-118): ncomp = coefficient count;
 * the fab must cover the level's valid box grown by 2 clipped to the domain. */
int ae_op_set_model(ae_op* op, int amrlev, const ae_fab* coeffs);
/* Operator::Elastic<T>::SetModel(T&) (Elastic.cpp:57-82): one stiffness on every node. */
int ae_op_set_model_uniform(ae_op* op, const double* coeffs, int ncoef);
/* SetModel for a stiffness that takes one of `ngrains` values per node, as a Voronoi
 * polycrystal does (IC::Voronoi, src/IC/Voronoi.H:47-101, one Linear::Cubic per grain): grain_id
 * is an int32 fab (ncomp 1) over the same region as ae_op_set_model's, table is ngrains x ncoef
 * (host or device).  Equivalent to ae_op_set_model with C(x) = table[grain_id(x)]; the sweeps on
 * the level then read 2-byte grain ids and the table instead of 84/168 bytes per node, with the
 * same arithmetic on the same values. */
int ae_op_set_model_grains(ae_op* op, int amrlev, const ae_fab* grain_id, int ngrains, const double* table);
/* SetModel from cell-centred phase-field order parameters, built on the device.  Replaces the
 * model field PhaseFieldMicrostructure::TimeStepBegin fills before its elastic solve
 * (src/Integrator/PhaseFieldMicrostructure.cpp:516-541), node by node, with
 * Affine::Cubic::Combine (src/Model/Solid/Affine/Cubic.H:70-82).
 *  - eta: nphase components, FP64, cell-centred (cell (i,j,k) spans nodes i..i+1, ...), covering
 *    cells [lo-1, hi] in x and y and [lo, hi] in z of the SetModel region (ae_op_set_model).
 *  - At node (i,j,k): e_n = (eta_n(i,j,k) + eta_n(i,j-1,k) + eta_n(i-1,j,k) + eta_n(i-1,j-1,k)) / 4
 *    (the reference averages over the four cells of the x-y plane at cell layer k, in 3-D too)
 *    and C = sum_n table[n] e_n / sum_m e_m.  table: nphase x ncoef.
 *  - F0table (nphase x 9, row-major) and F0 (9 components over the SetModel region) are optional
 *    together: F0 receives the eigenstrain mixed with the same weights, as ae_newton_residual and
 *    ae_newton_dw take it.
 *  - Host or device memory.  AE_ERR_ARG where the order parameters sum to zero at a node (the
 *    reference divides by zero there). */
int ae_op_set_model_mixture(ae_op* op, int amrlev, const ae_fab* eta, int nphase, const double* table,
                            const double* F0table, const ae_fab* F0);
/* SetModel for the isotropic degradable model, built on the device: PolymerDegradation::
 * DegradeMaterial (src/Integrator/PolymerDegradation.cpp:794-833) with
 * Degradable::Isotropic::DegradeModulus (src/Model/Solid/LinearElastic/Degradable/Isotropic.H:74-81).
 *  - Every node of the SetModel region gets (lambda0, mu0).  Each valid node then gets
 *    (lambda0 (1 - e), mu0 (1 - e)), e the mean of eta over the 8 cells around the node.  With
 *    several components each is averaged and range-checked in turn and the last one is kept, as
 *    the reference's loop does.
 *  - eta: neta components, FP64, cell-centred, covering cells [lo-1, hi] of the valid box; host
 *    or device memory; may be NULL when neta = 0.
 *  - Isotropic operators only.  AE_ERR_ARG where a mean lies outside [0, 1] (the reference
 *    aborts) or is NaN. */
int ae_op_set_model_degraded(ae_op* op, int amrlev, const ae_fab* eta, int neta, double lambda0, double mu0);
/* BC::Operator::Elastic<T>::Set for all 26 faces (Elastic.H:61-69); val used by ae_bc_init. */
int ae_op_set_bc(ae_op* op, const int* type /*[26][3]*/, const double* val /*[26][3]*/);
/* Operator::Elastic<T>::SetUniform / SetHomogeneous (Elastic.H:48,111). */
int ae_op_set_flags(ae_op* op, int uniform, int homogeneous);
/* Operator<Grid::Node>::prepareForSolve (Operator.cpp:445-452): stiffness average-down
 * (Elastic.cpp:620-652,722-809) and Diagonal on every level (Elastic.cpp:264-352). */
int ae_op_prepare(ae_op* op);
int ae_op_num_amr_levels(const ae_op* op);
int ae_op_num_mg_levels(const ae_op* op, int amrlev);
/* nodal valid box and domain of (amrlev, mglev) */
int ae_op_level_info(const ae_op* op, int amrlev, int mglev, int lo[3], int hi[3], int dom_hi[3], double dx[3]);

/* Elastic<T>::Fapply (Elastic.cpp:151-260): out = A in over the valid box grown by 1
 * clipped to the domain.  Device fabs, 3 components. */
int ae_fapply(ae_op* op, int amrlev, int mglev, const ae_fab* out, const ae_fab* in);
/* Elastic<T>::Diagonal (Elastic.cpp:264-352) copied out of the operator. */
int ae_diagonal(ae_op* op, int amrlev, int mglev, const ae_fab* diag);
/* Operator<Grid::Node>::Fsmooth (Operator.cpp:90-162): nsweeps damped-Jacobi sweeps in place. */
int ae_fsmooth(ae_op* op, int amrlev, int mglev, const ae_fab* x, const ae_fab* b, int nsweeps, double omega);
/* Operator<Grid::Node>::correctionResidual / solutionResidual (Operator.cpp:841-863):
 * r = b - A x; *norm_inf (host) receives the max-norm over the valid box. */
int ae_residual(ae_op* op, int amrlev, int mglev, const ae_fab* r, const ae_fab* x, const ae_fab* b,
                double* norm_inf);
/* Operator<Grid::Node>::restriction (Operator.cpp:454-554): crse on mglev cmglev from fine on cmglev-1. */
int ae_restrict(ae_op* op, int amrlev, int cmglev, const ae_fab* crse, const ae_fab* fine);
/* Operator<Grid::Node>::interpolation (Operator.cpp:556-624): fine (mglev fmglev) += I(crse). */
int ae_interp_add(ae_op* op, int amrlev, int fmglev, const ae_fab* fine, const ae_fab* crse);
/* BC::Operator::Elastic<T>::Init (BC/Operator/Elastic.H:106-181): BC values into rhs. */
int ae_bc_init(ae_op* op, int amrlev, const ae_fab* rhs, int homogeneous);
/* Elastic<T>::Strain / Stress / Energy (Elastic.cpp:399-572), valid box, device fabs. */
int ae_strain(ae_op* op, int amrlev, const ae_fab* eps, const ae_fab* u, int voigt);
int ae_stress(ae_op* op, int amrlev, const ae_fab* sig, const ae_fab* u, int voigt);
int ae_energy(ae_op* op, int amrlev, const ae_fab* w, const ae_fab* u);
/* Solver::Nonlocal::Newton<T>::prepareForSolve (src/Solver/Nonlocal/Newton.H:30-139) for the
 * linear and affine models (DW = C : (grad u - F0), src/Model/Solid/Affine/Cubic.H:38-41):
 * rhs = b - N(u) on grow(valid, 1) ∩ domain, N(u) = BC rows with sigma = DW on the domain
 * boundary (faces classified against that box) and the central divergence of DW inside, DW from
 * one-sided gradients at the faces of grow(valid, 2) ∩ domain.  F0: 9 components (row-major
 * eigenstrain, an Affine model) or NULL.  u and F0 cover grow(valid, 2) ∩ domain, b and rhs
 * grow(valid, 1) ∩ domain; FP64, host or device memory (host fabs are staged and the call then
 * synchronises).  Other nodes of rhs are not written. */
int ae_newton_residual(ae_op* op, int amrlev, const ae_fab* u, const ae_fab* b, const ae_fab* F0, ae_fab* rhs);
/* Newton<T>::DW (9 components, row-major) and Newton<T>::W on valid ∩ domain
 * (src/Solver/Nonlocal/Newton.H:233-333); either output may be NULL.  W = 1/2 G : C G,
 * G = grad u - F0, except Affine::Isotropic (isotropic model with F0) whose W has no 1/2
 * (src/Model/Solid/Affine/Isotropic.H:31-34). */
int ae_newton_dw(ae_op* op, int amrlev, const ae_fab* u, const ae_fab* F0, ae_fab* dw, ae_fab* w);
/* Newton<Model::Solid::Elastic::NeoHookean>::prepareForSolve (src/Solver/Nonlocal/Newton.H:30-139
 * with kinematic variable F; src/Model/Solid/Elastic/NeoHookean.H:28-66): at F = I + grad u,
 * node by node over grow(valid, 2) ∩ domain, the level's stiffness becomes DDW(F) (what
 * Elastic<Sym::Major>::SetModel then copies) and DW(F) feeds rhs = b - N(u) on
 * grow(valid, 1) ∩ domain as in ae_newton_residual.  The operator must be of kind
 * AE_MODEL_MAJOR; fab extents, types and memory as ae_newton_residual.  Marks the operator
 * unprepared (ae_solve prepares it again). */
int ae_newton_neohookean(ae_op* op, int amrlev, const ae_fab* u, const ae_fab* b, double mu, double kappa,
                         ae_fab* rhs);
/* Newton<NeoHookean>::DW (9 components, row-major) and ::W on valid ∩ domain with F = I + grad u,
 * stencils as ae_newton_dw; device fabs, either output may be NULL. */
int ae_neohookean_dw(ae_op* op, int amrlev, const ae_fab* u, double mu, double kappa, ae_fab* dw, ae_fab* w);

/* Solver::Nonlocal::Linear::solve (Linear.H:102-112) -> MLMG::solve.
 * sol and rhs: one fab per AMR level, host or device; sol holds the initial guess.
 * Returns AE_ERR_NOT_CONVERGED if max_iter is reached. */
int ae_solve(ae_op* op, const ae_fab* sol, const ae_fab* rhs, double tol_rel, double tol_abs,
             const ae_solver_opts* opts, ae_solve_stats* stats);
/* Solver::Nonlocal::Linear::solveaffine (src/Solver/Nonlocal/Linear.H:41-100): the operator with
 * its inhomogeneous rows is applied to zero (MLMG::apply), the result is negated inside the domain
 * and zeroed on its boundary and added to rhs (written back to rhs when copyrhs != 0), and the
 * homogeneous operator solves for that right-hand side.  Arguments and returns as ae_solve.  For
 * the linear stiffness kinds the apply of zero is exactly zero, so the solve sees rhs itself. */
int ae_solveaffine(ae_op* op, const ae_fab* sol, const ae_fab* rhs, double tol_rel, double tol_abs, int copyrhs,
                   const ae_solver_opts* opts, ae_solve_stats* stats);

/* The nodal plotfile of Integrator::WritePlotFile (src/Integrator/Integrator.cpp:582-681, the
 * "node" half, written by amrex::WriteMultiLevelPlotfile): an AMReX plotfile directory
 * (HyperCLaw-V1.1 Header; Level_<l>/Cell_H and Cell_D_00000) holding ncomp nodal components on
 * each level's valid box, one patch per level.  fabs: one FP64 HOST fab per level covering its
 * valid box (ghost nodes are not written); names: ncomp component names without whitespace (the
 * reference names a vector field's components name001, name002, ...); steps: per-level step
 * numbers or NULL.  AE_ERR_NAN if a written value is NaN or infinite. */
int ae_write_plotfile(const char* dir, int nlevels, const ae_level_desc* levels, const ae_fab* fabs, int ncomp,
                      const char* const* names, double time, const int* steps);

/* Device memory of the operator (bytes), for admission control. */
long long ae_op_device_bytes(const ae_op* op);

/* Bottom solve without allocation.  No counterpart in the reference.
 * For callers that cannot allocate device memory: an application whose memory arena already
 * owns the GPU (an AMReX code that reserved it, say), or a loop that must not enter the CUDA
 * allocator, but that runs its own multigrid hierarchy.  It solves the coarsest level exactly
 * as the cycle inside ae_solve does: CG or BiCGStab in one thread block; on failure the
 * correction is zeroed and `nuf` smoother calls (2 damped-Jacobi sweeps, w = 2/3) follow.
 * No cudaMalloc, cudaFree or allocating library call: the work space is a fixed device array
 * inside libaefast.so, sized for AE_NOALLOC_MAX_NODES nodes (10 x 3 doubles per node, 1.2 MB),
 * which every GPU that loads the library holds until the process exits.  Larger levels are
 * rejected with AE_ERR_ARG.
 *  - level: one nodal box covering its domain (lo = 0, hi = domain_cells).
 *  - C (ncoef per node), b and x (3 per node): DEVICE arrays in the level's nodal layout
 *    without ghosts, [comp][k][j][i].  x receives the solution; the solve starts from zero.
 *  - bctype: host array [26][3] of ae_bc_type.  *krylov_failed (may be NULL) receives the
 *    number of failed Krylov solves (0 or 1).
 *  - The first call on a device looks up the work space's device address with that device
 *    current; make that first call before any stream capture.  With CUDA's lazy module loading
 *    that first call also loads the library's device code, which can itself need device memory
 *    from the driver: make it (or run with CUDA_MODULE_LOADING=EAGER) before the application's
 *    arena reserves the device.
 *  - The address is kept per device for the life of the process; after a cudaDeviceReset the
 *    kept address is stale, so the entry point must not be called again in that process.
 *  - Every call shares the one work space: calls that overlap on the GPU (other streams, other
 *    host threads) race.  The call synchronizes `stream` (a cudaStream_t) before returning. */
#define AE_NOALLOC_MAX_NODES 4913 /* 17^3 */
int ae_bottom_solve_noalloc(const ae_level_desc* level, int model, const double* C, const int* bctype, int uniform,
                            const double* b, double* x, int bottom, int max_iter, double reltol, int nuf,
                            int* krylov_failed, void* stream);

/* Instrumentation (no counterpart in the reference, which times with BL_PROFILE scopes).
 * ae_kernel_launches: kernels this library has launched in the process (graph replays
 * count every kernel in the graph).  ae_profile_kernel: average CUDA-event duration of
 * `reps` back-to-back launches of one kernel on the operator's own buffers at
 * (amrlev, mglev): which = 0 Fapply, 1 Jacobi sweep, 2 residual, 3 restriction to
 * mglev+1, 4 interpolation from mglev+1; precision 0 = FP64, 1 = FP32. */
long long ae_kernel_launches(void);
int ae_profile_kernel(ae_op* op, int which, int amrlev, int mglev, int precision, int reps, double* avg_ms);

/* ---------------------------------------------------------------- periodic cells (RVEs)
 * Homogenisation of periodic cells under a macroscopic displacement gradient E (3x3,
 * row-major, E[3*i+j] = du_i/dx_j): u = E x + w, w periodic.  The operator is the interior row
 * of Operator::Elastic<T>::Fapply (src/Operator/Elastic.cpp:216-255) at every node with
 * neighbours taken modulo the cell: a periodic cell has no domain boundary, so the reference's
 * BC::Operator::Elastic Type::Periodic rows (src/BC/Operator/Elastic.H:299-300) never occur.
 * Because the non-divergence form is not conservative on the grid, each cell problem carries a
 * uniform body force c: A w + c = b, mean(w) = 0, b = -sum_d (d_d C) : E e_d.  The solve is the
 * MLMG iteration of ae_solve on the mean-free residual (V-cycles; max_fmg_iter is not used),
 * bottom Krylov on the mean-projected operator.  No counterpart in the reference: the batched
 * RVE solve and the serving loop below are built on its operator and cycle.
 *
 * A cell stores n[0] n[1] n[2] unique nodes (x = i length/n), fields [comp][k][j][i]; fabs
 * passed for a cell have lo = 0, hi = n-1.  A batch advances every solve of every cell together:
 * each kernel launch covers all of them and each iteration is one CUDA graph launch.  The
 * arithmetic of one solve does not depend on the other solves of the batch. */
typedef struct {
    int n[3];          /* nodes (= cells) per direction */
    int nrhs;          /* solves (load cases) on this cell */
    double length[3];  /* cell edge lengths */
} ae_cell_desc;

typedef struct {
    int iters, converged, nlevels, bottom_fail;
    double res0, resfinal, target;
    double seconds;            /* wall time of the ae_batch_solve call */
    double body_force[3];      /* c of the last residual */
    double mean_stress[9];     /* cell average of C : (E + grad w), central differences */
} ae_cell_stats;

typedef struct ae_batch_s* ae_batch;

/* device bytes one cell needs (its hierarchy and nrhs solves), or -1 for a bad descriptor */
long long ae_batch_plan_bytes(const ae_cell_desc* cell, int model);
int ae_batch_create(const ae_cell_desc* cells, int ncells, int model, ae_batch* out);
int ae_batch_destroy(ae_batch b);
int ae_batch_num_solves(ae_batch b);  /* solves are numbered cell by cell, nrhs each */
int ae_batch_num_levels(ae_batch b, int cell);
long long ae_batch_device_bytes(ae_batch b);
/* stiffness per node: a fab of ncoef FP64 components over [0, n-1]^3, host or device */
int ae_batch_set_model(ae_batch b, int cell, const ae_fab* C);
/* stiffness from a Voronoi cell (IC::Voronoi semantics, src/IC/Voronoi.H:47-101, with the
 * minimum-image distance of the periodic cell; ties to the lower seed): seeds ngrains x 3 in
 * length units, table ngrains x ncoef; host or device pointers.  Built on the device. */
int ae_batch_set_model_grains(ae_batch b, int cell, int ngrains, const double* seeds, const double* table);
int ae_batch_set_load(ae_batch b, int solve, const double* E);
/* coarsened stiffness, diagonals and FP32 copies of every cell (Operator::prepareForSolve) */
int ae_batch_prepare(ae_batch b);
/* Solve every load case to ||r|| <= max(tol_abs, tol_rel max(||b||, ||r0||)).  opts->precision
 * 0: FP64 cycles; 1: FP32 cycles (inner_cycles per FP64 residual) inside FP64 refinement.
 * stats: NULL or ae_batch_num_solves entries.  AE_ERR_NOT_CONVERGED if any solve stopped at
 * max_iter (the stats say which). */
int ae_batch_solve(ae_batch b, double tol_rel, double tol_abs, const ae_solver_opts* opts, ae_cell_stats* stats);
/* w (mean removed) of one solve into a 3-component fab over [0, n-1]^3, host or device */
int ae_batch_solution(ae_batch b, int solve, ae_fab* w);
/* Launch shape of the stencil kernels on multigrid level `level`: nodes per block (128 or 256)
 * and persistent grid size (0: one block per 128/256-node run).  chunk = grid = 0 returns the
 * level to the autotuner, which times the candidates on the first solve of each precision. */
int ae_batch_set_shape(ae_batch b, int level, int chunk, int grid);
int ae_batch_get_shape(ae_batch b, int level, int* chunk, int* grid);

/* ---------------------------------------------------------------- serving
 * A request loop for cell homogenisation.  A worker thread owns the device work and runs
 * continuous batching: between iterations it admits queued requests (FIFO) whose device memory
 * fits the budget, builds their stiffness and multigrid hierarchy on the device and starts their
 * solves; every iteration advances all live solves in the same launches; a request whose load
 * cases have all finished is completed and its memory returned.  A request's result does not
 * depend on the other requests on the device.  Times are seconds since ae_server_create. */
typedef struct {
    long long hbm_budget_bytes;  /* device memory for live requests; 0 = 80 % of free memory at creation */
    int max_live_solves;         /* admission cap on live load cases; 0 = none */
    int keep_solution;           /* copy every load case's w back with the result */
    double tol_rel, tol_abs;
    ae_solver_opts solver;       /* precision, inner_cycles, cycle counts, bottom solver, use_graph */
} ae_server_opts;

typedef struct {
    int status;      /* AE_OK done, < 0 failed (ae_status), 1 queued, 2 running */
    int nrhs;
    double t_submit, t_admit, t_done;
    double latency;  /* t_done - t_submit once finished, else -1 */
} ae_request_info;

typedef struct {
    long long submitted, completed, failed, queued, iterations;
    long long hbm_used, hbm_budget;
    double busy_seconds;    /* worker time spent admitting, iterating and retiring */
    double uptime_seconds;
} ae_server_stats;

typedef struct ae_server_s* ae_server;

void ae_server_default_opts(ae_server_opts* opts);  /* mixed precision, 4 inner cycles, 1e-8, graphs */
int ae_server_create(int model, const ae_server_opts* opts, ae_server* out);
/* Stop the worker (finishing its current iteration) and free everything; queued and running
 * requests are dropped. */
int ae_server_destroy(ae_server s);
/* Queue one cell with desc->nrhs load cases (E: nrhs x 9).  The stiffness is either a Voronoi
 * description (ngrains > 0: seeds ngrains x 3, table ngrains x ncoef, host memory; built on the
 * device as ae_batch_set_model_grains) or a host FP64 field C (ngrains = 0).  Inputs are copied;
 * *ticket identifies the request. */
int ae_server_submit(ae_server s, const ae_cell_desc* desc, int ngrains, const double* seeds, const double* table,
                     const ae_fab* C, const double* E, long long* ticket);
/* Current state of a request; once finished, stats (nrhs entries) and w (nrhs x 3 x nn, if
 * keep_solution) are filled when non-NULL. */
int ae_server_poll(ae_server s, long long ticket, ae_request_info* info, ae_cell_stats* stats, double* w);
/* As poll, after waiting until the request finishes (timeout_s < 0: no limit). */
int ae_server_wait(ae_server s, long long ticket, double timeout_s, ae_request_info* info, ae_cell_stats* stats,
                   double* w);
/* Forget a finished request. */
int ae_server_release(ae_server s, long long ticket);
int ae_server_get_stats(ae_server s, ae_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif
