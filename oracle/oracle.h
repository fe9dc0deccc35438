/*
 * CPU FP64 restatement of the reference's nodal linear-elastic operator path
 * (Operator::Elastic<T>, Operator::Operator<Grid::Node>, BC::Operator::Elastic<T>,
 * Numeric::Stencil, Set::Matrix4 contractions) and of the AMReX MLMG cycle that
 * drives it.
 *
 * TEST INFRASTRUCTURE ONLY: the parity reference for the CUDA library. tests/, the
 * smoke check and bench.py's cpu_baseline leg may load it; the product (the CUDA
 * library under anisotropicfracture_gb300/csrc) never links or calls it.
 *
 * Pinning: the reference ships no golden vectors and cannot be built here
 * (AMReX, Eigen and MPI are absent). The restatement is pinned against the
 * reference's own known-answer tests, restated in tests/test_oracle_known_answers.py:
 *   - src/Test/Numeric/Stencil.H:58-106   (stencil derivatives of cos*cos*cos, 1 %)
 *   - src/Test/Set/Matrix4.H:9-30          (MajorMinor symmetry)
 *   - src/Test/Operator/Elastic_TrigTest.cpp:17-140    (Laplacian solve vs sine series, 2 %)
 *   - src/Test/Operator/Elastic_UniaxialTest.cpp:13-203 (isotropic affine solution, 1 %)
 *   - src/Test/Operator/Elastic_RefluxTest.cpp:12-107   (Fapply of affine fields)
 * and against a generic 81-term tensor contraction.
 *
 * Layout of every field: one nodal box per level, stored over
 * grow(valid, ng); index order [comp][k][j][i], i fastest (AMReX Array4 order).
 */
#ifndef AE_ORACLE_H
#define AE_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int dom_lo[3], dom_hi[3]; /* nodal problem domain of this level (inclusive) */
    int lo[3], hi[3];         /* nodal valid box of this level (inclusive)      */
    int ng;                   /* ghost layers stored around the valid box       */
    int pad_;
    double dx[3];             /* cell size                                      */
} orc_level;

/* model kinds: per-node coefficient count in parentheses */
enum {
    ORC_ISOTROPIC = 0 /* (lambda, mu) */, ORC_MAJORMINOR = 1 /* 21 */, ORC_DIAGONAL = 2 /* 9, A(i,j) row-major */,
    ORC_MAJOR = 3 /* 45: upper triangle of the symmetric 9 x 9 matrix C(3i+j, 3k+l), row by row */
};

/* BC types, same numbering as BC::Operator::Elastic<T>::Type (src/BC/Operator/Elastic.H:24) */
enum { ORC_DISP = 0, ORC_TRAC = 1, ORC_PERIODIC = 2, ORC_NEUMANN = 3 };

typedef struct {
    int max_fmg_iter;     /* iterations run as F-cycles before V-cycles (MLMG max_fmg_iter)  */
    int nu1, nu2;         /* smoother calls before/after coarse-grid correction              */
    int sweeps;           /* Jacobi sweeps per smoother call (reference Fsmooth: 2)          */
    int bottom;           /* 0 = CG, 1 = BiCGStab                                            */
    int max_iter;         /* MLMG max iterations                                             */
    int bottom_max_iter;  /* MLCGSolver max iterations                                       */
    double bottom_reltol; /* MLMG bottom relative tolerance (AMReX default 1e-4)             */
    int nuf;              /* smoother calls after a failed bottom solve (AMReX default 8)    */
    int max_mg_levels;    /* cap on multigrid levels (<=0: coarsen while possible)           */
    double omega;         /* Jacobi damping (reference: 2/3)                                 */
    int uniform;          /* Operator::Elastic m_uniform                                     */
    int pad_;
} orc_opts;

typedef struct {
    int iters;            /* MLMG iterations performed                                        */
    int converged;
    int nlevels;          /* multigrid levels used                                            */
    int bottom_fail;      /* number of bottom solves that returned nonzero                   */
    double res0, resfinal, target;
    double hist[256];     /* residual inf-norm after each iteration                          */
} orc_stats;

void orc_set_threads(int n);
int orc_num_threads(void);

int orc_fapply(const orc_level* L, int model, const double* C, const int* bctype,
               int uniform, const double* u, double* f);
int orc_diagonal(const orc_level* L, int model, const double* C, const int* bctype, double* diag);
int orc_fsmooth(const orc_level* L, int model, const double* C, const int* bctype, int uniform,
                const double* diag, double* x, const double* b, int nsweeps, double omega);
int orc_residual(const orc_level* L, int model, const double* C, const int* bctype, int uniform,
                 const double* x, const double* b, double* r, double* norm_inf);
int orc_restrict(const orc_level* Lc, const orc_level* Lf, int ncomp, double* crse, const double* fine);
int orc_interp_add(const orc_level* Lf, const orc_level* Lc, int ncomp, double* fine, const double* crse);
int orc_bc_init(const orc_level* L, const int* bctype, const double* bcval, int homogeneous, double* rhs);
int orc_strain(const orc_level* L, const double* u, int voigt, double* eps);
int orc_stress(const orc_level* L, int model, const double* C, const double* u, int voigt, double* sig);
int orc_energy(const orc_level* L, int model, const double* C, const double* u, double* w);
/* generic 81-term contractions from a 21-coefficient MajorMinor tensor (cross-check) */
void orc_mm_full(const double* c21, double* c81);
void orc_mm_stress(const double* c21, const double* g9, double* s9);
void orc_mm_div(const double* c21, const double* b27, double* f3);
/* single-level MLMG solve; u holds the initial guess and receives the solution */
int orc_solve(const orc_level* L, int model, const double* C, const int* bctype,
              double* u, const double* b, double tol_rel, double tol_abs,
              const orc_opts* opts, orc_stats* stats);
/* composite multi-level solve: Ls[0] covers its domain (ng = 0); Ls[l >= 1] are patches of finer
 * levels refined by 2 with ng = 2, listed level by level; consecutive entries with one domain are
 * the patches of one level (storage boxes grow(valid, 2) disjoint), each nested in one patch of
 * the level below.  Cs, us, bs hold one stored field per entry.  -1 for a malformed list. */
int orc_solve_amr(const orc_level* Ls, int namr, int model, const double* const* Cs, const int* bctype,
                  double* const* us, const double* const* bs, double tol_rel, double tol_abs,
                  const orc_opts* opts, orc_stats* stats);
/* composite residual of given solutions (MLMG::computeMLResidual: per-level b - A u, the fine
 * residual restricted onto covered coarse nodes); rs (one field per level) may be NULL */
int orc_residual_amr(const orc_level* Ls, int namr, int model, const double* const* Cs, const int* bctype,
                     int uniform, const double* const* us, const double* const* bs, double* const* rs,
                     double* norm_inf);
/* number of multigrid levels the solver builds for this level */
int orc_num_mg_levels(const orc_level* L, int max_mg_levels);

/* Solver::Nonlocal::Newton<T> pieces for the linear / affine models: the Newton right-hand side
 * rhs = b - N(u) (DW = C : (grad u - F0); F0: 9 components row-major, or NULL) and the DW / W
 * post-processing fields (dw: 9 components, w: 1; either may be NULL). */
int orc_newton_residual(const orc_level* L, int model, const double* C, const int* bctype, const double* u,
                        const double* b, const double* F0, double* rhs);
int orc_newton_dw(const orc_level* L, int model, const double* C, const double* u, const double* F0, double* dw,
                  double* w);

/* ---- periodic cells (homogenisation): n[0] n[1] n[2] unique nodes, no ghosts ----
 * w periodic, u = E x + w; A w + c = b with b = -sum_d (d_d C) : E e_d, mean(w) = 0 and c a
 * uniform body force (the multiplier of the mean constraint; see oracle.cpp). */
typedef struct {
    int n[3];
    int pad_;
    double dx[3];
} orc_rve_level;

int orc_rve_num_mg_levels(const orc_rve_level* L, int max_mg_levels);
int orc_rve_fapply(const orc_rve_level* L, int model, const double* C, int uniform, const double* u, double* f);
int orc_rve_diagonal(const orc_rve_level* L, int model, const double* C, double* diag);
int orc_rve_fsmooth(const orc_rve_level* L, int model, const double* C, int uniform, const double* diag, double* x,
                    const double* b, int nsweeps, double omega);
/* r = b - A x; project != 0 removes the per-component mean (returned in mean[3]) */
int orc_rve_residual(const orc_rve_level* L, int model, const double* C, int uniform, const double* x,
                     const double* b, double* r, int project, double* mean, double* norm_inf);
int orc_rve_restrict(const orc_rve_level* Lc, const orc_rve_level* Lf, int ncomp, double* crse, const double* fine);
int orc_rve_interp_add(const orc_rve_level* Lf, const orc_rve_level* Lc, int ncomp, double* fine,
                       const double* crse);
/* E: 3x3 row-major displacement gradient */
int orc_rve_rhs(const orc_rve_level* L, int model, const double* C, int uniform, const double* E, double* b);
int orc_rve_mean_stress(const orc_rve_level* L, int model, const double* C, const double* E, const double* w,
                        double* sig);
int orc_rve_solve(const orc_rve_level* L, int model, const double* C, const double* E, double* w,
                  double tol_rel, double tol_abs, const orc_opts* opts, orc_stats* stats, double* body_force);

#ifdef __cplusplus
}
#endif
#endif
