// alamo_elastic.H -- header-only C++ shim with the reference's class and method names over
// the C ABI of libaefast.so (aefast.h).  An integrator that used
//   Operator::Elastic<T>            (src/Operator/Elastic.H:20-171)
//   BC::Operator::Elastic<T>        (src/BC/Operator/Elastic.H:12-406)
//   Solver::Nonlocal::Linear        (src/Solver/Nonlocal/Linear.H:19-143)
//   Solver::Nonlocal::Newton<T>     (src/Solver/Nonlocal/Newton.H:15-349)
// swaps its includes for this header.  AMReX MultiFabs become alamo::Fab views (one patch per
// level, Array4 layout, host or device memory); Util::Abort becomes a thrown alamo::Error, as
// the reference throws with amrex.throw_exception = 1 (src/Util/Util.cpp:93-99).
#ifndef ALAMO_ELASTIC_H
#define ALAMO_ELASTIC_H

#include <array>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "aefast.h"

namespace alamo {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
inline void check(int rc) {
    if (rc != AE_OK) throw Error(rc, ae_last_error());
}

// A field over the index box [lo, hi] (ghosts included), i fastest, then j, k, component.
struct Fab {
    double* data = nullptr;
    std::array<int, 3> lo{{0, 0, 0}}, hi{{0, 0, 0}};
    int ncomp = 0;
    Fab() = default;
    Fab(double* d, std::array<int, 3> l, std::array<int, 3> h, int n) : data(d), lo(l), hi(h), ncomp(n) {}
    long long npts() const { return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1); }
    double& operator()(int i, int j, int k, int n) {
        const long long sy = hi[0] - lo[0] + 1, sz = sy * (hi[1] - lo[1] + 1);
        return data[(i - lo[0]) + (j - lo[1]) * sy + (k - lo[2]) * sz + n * npts()];
    }
    ae_fab c() const {
        ae_fab f;
        f.data = data;
        for (int d = 0; d < 3; ++d) { f.lo[d] = lo[d]; f.hi[d] = hi[d]; }
        f.ncomp = ncomp;
        f.is_float = 0;
        return f;
    }
};

// Geometry of one AMR level: cells of the level's domain, nodal patch, cell size.
struct Level {
    std::array<int, 3> cells, lo, hi;
    std::array<double, 3> dx;
    ae_level_desc c() const {
        ae_level_desc L;
        for (int d = 0; d < 3; ++d) {
            L.domain_cells[d] = cells[d];
            L.lo[d] = lo[d];
            L.hi[d] = hi[d];
            L.dx[d] = dx[d];
        }
        return L;
    }
};

// Integrator::WritePlotFile, node half (src/Integrator/Integrator.cpp:582-681): writes
// <plot_file>/<step:05d>[init]node as an AMReX plotfile (one host fab per level, the named
// components on its valid box) and appends its Header to <plot_file>/nodeoutput.visit, which
// step 0 creates.  Returns the plotfile directory.
inline std::string WritePlotFile(const std::string& plot_file, int step, const std::vector<Level>& levels,
                                 const std::vector<Fab>& fabs, const std::vector<std::string>& names,
                                 double time, bool initial = false) {
    std::vector<ae_level_desc> d;
    std::vector<ae_fab> f;
    for (const auto& L : levels) d.push_back(L.c());
    for (const auto& x : fabs) f.push_back(x.c());
    std::vector<const char*> cn;
    for (const auto& n : names) cn.push_back(n.c_str());
    char num[16];
    std::snprintf(num, sizeof(num), "%05d", step);
    const std::string name = std::string(num) + (initial ? "init" : "") + "node";
    const std::string dir = plot_file + "/" + name;
    check(ae_write_plotfile(dir.c_str(), (int)d.size(), d.data(), f.data(), (int)cn.size(), cn.data(), time, nullptr));
    std::FILE* visit = std::fopen((plot_file + "/nodeoutput.visit").c_str(), step == 0 ? "w" : "a");
    if (!visit) throw Error(AE_ERR_STATE, "cannot write " + plot_file + "/nodeoutput.visit");
    std::fprintf(visit, "%s/Header\n", name.c_str());
    std::fclose(visit);
    return dir;
}

}  // namespace alamo

namespace Model {
namespace Solid {
namespace Linear {
// Linear::Isotropic(mu, lambda) (src/Model/Solid/Linear/Isotropic.H:19-29)
struct Isotropic {
    static constexpr int kind = AE_MODEL_ISOTROPIC;
    static constexpr int ncoef = 2;
    double lambda = 0, mu = 0;
    Isotropic() = default;
    Isotropic(double a_mu, double a_lambda) { Define(a_mu, a_lambda); }
    void Define(double a_mu, double a_lambda) { mu = a_mu; lambda = a_lambda; }
    void coeffs(double* c) const { c[0] = lambda; c[1] = mu; }
};
// Linear::Laplacian: Diagonal tensor, A = ones (src/Model/Solid/Linear/Laplacian.H:31-34)
struct Laplacian {
    static constexpr int kind = AE_MODEL_DIAGONAL;
    static constexpr int ncoef = 9;
    void coeffs(double* c) const { for (int q = 0; q < 9; ++q) c[q] = 1.0; }
};
// Linear::Cubic::Define(C11, C12, C44, R) (src/Model/Solid/Linear/Cubic.H:20-59): the rotated
// tensor in the 21 MajorMinor slots; each slot keeps the value of the last (p,q,s,t) in loop order.
struct Cubic {
    static constexpr int kind = AE_MODEL_MAJORMINOR;
    static constexpr int ncoef = 21;
    double ddw[21] = {0};
    static int slot(int i, int j, int k, int l) {
        static const int voigt[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}};
        static const int table[6][6] = {{0, 3, 5, 4, 2, 1},      {3, 15, 17, 16, 12, 8},  {5, 17, 20, 19, 14, 10},
                                        {4, 16, 19, 18, 13, 9},  {2, 12, 14, 13, 11, 7},  {1, 8, 10, 9, 7, 6}};
        return table[voigt[i][j]][voigt[k][l]];
    }
    void Define(double C11, double C12, double C44, const double R[3][3]) {
        double Ct[3][3][3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k)
                    for (int l = 0; l < 3; ++l) {
                        if (i == j && j == k && k == l) Ct[i][j][k][l] = C11;
                        else if (i == k && j == l) Ct[i][j][k][l] = C44;
                        else if (i == j && k == l) Ct[i][j][k][l] = C12;
                        else Ct[i][j][k][l] = 0.0;
                    }
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q)
                for (int s = 0; s < 3; ++s)
                    for (int t = 0; t < 3; ++t) {
                        double acc = 0.0;
                        for (int i = 0; i < 3; ++i)
                            for (int j = 0; j < 3; ++j)
                                for (int k = 0; k < 3; ++k)
                                    for (int l = 0; l < 3; ++l) acc += R[p][i] * R[s][k] * Ct[i][j][k][l] * R[q][j] * R[t][l];
                        ddw[slot(p, q, s, t)] = acc;
                    }
    }
    // Bunge-like X-Z-X Euler angles: R = Rx(phi2) Rz(Phi) Rx(phi1) (Cubic.H:22-29)
    void Define(double C11, double C12, double C44, double phi1, double Phi, double phi2) {
        auto rx = [](double a, double m[3][3]) {
            const double c = std::cos(a), s = std::sin(a);
            const double r[3][3] = {{1, 0, 0}, {0, c, -s}, {0, s, c}};
            for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m[i][j] = r[i][j];
        };
        auto rz = [](double a, double m[3][3]) {
            const double c = std::cos(a), s = std::sin(a);
            const double r[3][3] = {{c, -s, 0}, {s, c, 0}, {0, 0, 1}};
            for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) m[i][j] = r[i][j];
        };
        auto mul = [](const double a[3][3], const double b[3][3], double o[3][3]) {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    o[i][j] = 0;
                    for (int k = 0; k < 3; ++k) o[i][j] += a[i][k] * b[k][j];
                }
        };
        double A[3][3], B[3][3], Cm[3][3], T[3][3], R[3][3];
        rx(phi2, A); rz(Phi, B); rx(phi1, Cm);
        mul(A, B, T);
        mul(T, Cm, R);
        Define(C11, C12, C44, R);
    }
    void coeffs(double* c) const { for (int q = 0; q < 21; ++q) c[q] = ddw[q]; }
};
}  // namespace Linear
namespace Elastic {
// Elastic::NeoHookean (src/Model/Solid/Elastic/NeoHookean.H:11-81), kinematic variable
// F = I + grad u.  Its per-node tangent DDW(F) is a Sym::Major field (45 slots), which
// Newton<NeoHookean> evaluates on the device (ae_newton_neohookean); coeffs() gives DDW(I),
// the small-strain tangent, for a uniform SetModel.
struct NeoHookean {
    static constexpr int kind = AE_MODEL_MAJOR;
    static constexpr int ncoef = 45;
    double mu = 0, kappa = 0;
    NeoHookean() = default;
    NeoHookean(double a_mu, double a_kappa) : mu(a_mu), kappa(a_kappa) {}
    // NeoHookean::DDW (NeoHookean.H:40-66) at F = I: G = F^-T = I, J = 1, F:F = 3
    void coeffs(double* c) const {
        const double d[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int I = 0; I < 9; ++I)
            for (int K = I; K < 9; ++K) {
                const int i = K / 3, j = K % 3, k = I / 3, l = I % 3;
                double t1 = 0.0, t2 = 0.0;
                if (i == k && j == l) t1 += 1.0;
                t1 -= (2. / 3.) * d[i][j] * d[k][l];
                t1 -= (2. / 3.) * d[i][j] * d[k][l];
                t1 += (2. / 9.) * 3.0 * d[i][j] * d[k][l];
                t1 += (1. / 3.) * 3.0 * d[i][l] * d[k][j];
                t2 += (2. * 1.0 - 1.) * d[i][j] * d[k][l];
                t2 += (1. - 1.0) * d[i][l] * d[k][j];
                c[I * 9 - I * (I - 1) / 2 + (K - I)] = mu * t1 + kappa * t2;
            }
    }
};
}  // namespace Elastic
}  // namespace Solid
}  // namespace Model

namespace BC {
namespace Operator {
template <class T>
class Elastic {
public:
    enum Type { Displacement = AE_BC_DISPLACEMENT, Traction = AE_BC_TRACTION, Periodic = AE_BC_PERIODIC,
                Neumann = AE_BC_NEUMANN };
    enum Face {
        XLO, YLO, ZLO, XHI, YHI, ZHI, YLO_ZLO, YLO_ZHI, YHI_ZLO, YHI_ZHI, ZLO_XLO, ZLO_XHI, ZHI_XLO, ZHI_XHI,
        XLO_YLO, XLO_YHI, XHI_YLO, XHI_YHI, XLO_YLO_ZLO, XLO_YLO_ZHI, XLO_YHI_ZLO, XLO_YHI_ZHI, XHI_YLO_ZLO,
        XHI_YLO_ZHI, XHI_YHI_ZLO, XHI_YHI_ZHI, INT
    };
    enum Direction { X = 0, Y = 1, Z = 2 };
    Elastic() {
        for (int f = 0; f < 26; ++f)
            for (int d = 0; d < 3; ++d) { m_type[3 * f + d] = Displacement; m_val[3 * f + d] = 0.0; }
    }
    void Set(Face face, Direction direction, Type type, double value) {
        m_type[3 * face + direction] = type;
        m_val[3 * face + direction] = value;
    }
    const int* types() const { return m_type; }
    const double* values() const { return m_val; }

private:
    int m_type[26 * 3];
    double m_val[26 * 3];
};
}  // namespace Operator
}  // namespace BC

namespace Operator {
// Operator::Operator<Grid::Node> (src/Operator/Operator.H:30-128): owns the library handle.
class NodeOperator {
public:
    NodeOperator() = default;
    NodeOperator(const NodeOperator&) = delete;
    NodeOperator& operator=(const NodeOperator&) = delete;
    virtual ~NodeOperator() { if (m_op) ae_op_destroy(m_op); }
    ae_op* handle() const { return m_op; }
    int NMGLevels(int amrlev) const { return ae_op_num_mg_levels(m_op, amrlev); }

protected:
    ae_op* m_op = nullptr;
};

template <class T>
class Elastic : public NodeOperator {
public:
    Elastic() = default;
    explicit Elastic(const std::vector<alamo::Level>& levels) { define(levels); }
    // Elastic<T>::define (Elastic.cpp:30-55)
    void define(const std::vector<alamo::Level>& levels) {
        std::vector<ae_level_desc> d;
        for (const auto& L : levels) d.push_back(L.c());
        alamo::check(ae_op_create(d.data(), (int)d.size(), T::kind, &m_op));
    }
    // SetModel(T&): one stiffness everywhere (Elastic.cpp:57-82)
    void SetModel(const T& model) {
        double c[T::ncoef];
        model.coeffs(c);
        alamo::check(ae_op_set_model_uniform(m_op, c, T::ncoef));
    }
    // SetModel(amrlev, FabArray<BaseFab<T>>) with the coefficients in a fab (ncomp = T::ncoef)
    void SetModel(int amrlev, const alamo::Fab& coeffs) {
        const ae_fab f = coeffs.c();
        alamo::check(ae_op_set_model(m_op, amrlev, &f));
    }
    // The model field PhaseFieldMicrostructure::TimeStepBegin mixes from its order parameters
    // (PhaseFieldMicrostructure.cpp:516-541, Affine::Cubic::Combine), built on the device: eta is
    // the cell-centred order-parameter fab, one model per phase; F0 (9 components) receives the
    // mixed eigenstrain when the phases carry one (F0tab: nphase x 9, row-major).
    void SetModelMixture(int amrlev, const alamo::Fab& eta, const std::vector<T>& phases,
                         const std::vector<double>* F0tab = nullptr, alamo::Fab* F0 = nullptr) {
        std::vector<double> tab(phases.size() * T::ncoef);
        for (size_t n = 0; n < phases.size(); ++n) {
            double c[T::ncoef];
            phases[n].coeffs(c);
            for (int q = 0; q < T::ncoef; ++q) tab[n * T::ncoef + q] = c[q];
        }
        const ae_fab fe = eta.c();
        ae_fab ff{};
        if (F0) ff = F0->c();
        alamo::check(ae_op_set_model_mixture(m_op, amrlev, &fe, (int)phases.size(), tab.data(),
                                             F0tab ? F0tab->data() : nullptr, F0 ? &ff : nullptr));
    }
    // PolymerDegradation::DegradeMaterial (PolymerDegradation.cpp:794-833) for the isotropic
    // degradable model, built on the device from the cell-centred damage fab eta.
    void SetModelDegraded(int amrlev, const alamo::Fab& eta, double lambda0, double mu0) {
        const ae_fab fe = eta.c();
        alamo::check(ae_op_set_model_degraded(m_op, amrlev, &fe, fe.ncomp, lambda0, mu0));
    }
    // SetBC stores the table; the reference keeps a non-owning pointer (Elastic.H:58-66)
    void SetBC(BC::Operator::Elastic<T>* bc) {
        m_bc = bc;
        alamo::check(ae_op_set_bc(m_op, bc->types(), bc->values()));
    }
    BC::Operator::Elastic<T>& GetBC() { return *m_bc; }
    void SetUniform(bool a) { m_uniform = a; alamo::check(ae_op_set_flags(m_op, m_uniform, m_homogeneous)); }
    void SetHomogeneous(bool a) { m_homogeneous = a; alamo::check(ae_op_set_flags(m_op, m_uniform, m_homogeneous)); }
    void prepareForSolve() { alamo::check(ae_op_prepare(m_op)); }
    // kernel-level pieces on DEVICE fabs
    void Fapply(int amrlev, int mglev, alamo::Fab& out, const alamo::Fab& in) {
        const ae_fab o = out.c(), i = in.c();
        alamo::check(ae_fapply(m_op, amrlev, mglev, &o, &i));
    }
    void Fsmooth(int amrlev, int mglev, alamo::Fab& x, const alamo::Fab& b) {
        const ae_fab fx = x.c(), fb = b.c();
        alamo::check(ae_fsmooth(m_op, amrlev, mglev, &fx, &fb, 2, 2.0 / 3.0));
    }
    void Stress(int amrlev, alamo::Fab& sigma, const alamo::Fab& u, bool voigt = false) {
        const ae_fab s = sigma.c(), fu = u.c();
        alamo::check(ae_stress(m_op, amrlev, &s, &fu, voigt));
    }
    void Strain(int amrlev, alamo::Fab& eps, const alamo::Fab& u, bool voigt = false) {
        const ae_fab e = eps.c(), fu = u.c();
        alamo::check(ae_strain(m_op, amrlev, &e, &fu, voigt));
    }

private:
    BC::Operator::Elastic<T>* m_bc = nullptr;
    bool m_uniform = false, m_homogeneous = false;
};
}  // namespace Operator

namespace Solver {
namespace Nonlocal {
// Solver::Nonlocal::Linear with the reference's MLMG defaults (Linear.H:23-29)
class Linear {
public:
    explicit Linear(Operator::NodeOperator& op) : linop(op) {
        ae_default_solver_opts(&m_opts);
        m_opts.bottom = 1;                  // bicgstab
        m_opts.max_fmg_iter = 100000000;    // F-cycles
        m_opts.nu1 = m_opts.nu2 = 2;        // AMReX MLMG nu1 / nu2
    }
    virtual ~Linear() = default;
    void setMaxIter(int n) { m_opts.max_iter = n; }
    void setBottomMaxIter(int n) { m_opts.bottom_max_iter = n; }
    void setMaxFmgIter(int n) { m_opts.max_fmg_iter = n; }
    void setFixedIter(int n) { m_opts.fixed_iter = n; }
    void setVerbose(int v) { m_opts.verbose = v; }
    void setBottomSolverCG(bool cg) { m_opts.bottom = cg ? 0 : 1; }
    void setPreSmooth(int n) { m_opts.nu1 = n; }
    void setPostSmooth(int n) { m_opts.nu2 = n; }
    void setMixedPrecision(bool on) { m_opts.precision = on ? 1 : 0; }
    // Linear::solve(sol, rhs, tol_rel, tol_abs) (Linear.H:102-107): one fab per AMR level
    double solve(std::vector<alamo::Fab>& sol, std::vector<alamo::Fab>& rhs, double tol_rel, double tol_abs) {
        std::vector<ae_fab> s, r;
        for (auto& f : sol) s.push_back(f.c());
        for (auto& f : rhs) r.push_back(f.c());
        alamo::check(ae_solve(linop.handle(), s.data(), r.data(), tol_rel, tol_abs, &m_opts, &m_stats));
        return m_stats.resfinal;
    }
    double solve(std::vector<alamo::Fab>& sol, std::vector<alamo::Fab>& rhs) { return solve(sol, rhs, m_tol_rel, m_tol_abs); }
    // Linear::solveaffine(sol, rhs, tol_rel, tol_abs, copyrhs) (Linear.H:41-100)
    double solveaffine(std::vector<alamo::Fab>& sol, std::vector<alamo::Fab>& rhs, double tol_rel, double tol_abs,
                       bool copyrhs = false) {
        std::vector<ae_fab> s, r;
        for (auto& f : sol) s.push_back(f.c());
        for (auto& f : rhs) r.push_back(f.c());
        alamo::check(ae_solveaffine(linop.handle(), s.data(), r.data(), tol_rel, tol_abs, copyrhs ? 1 : 0, &m_opts,
                                    &m_stats));
        return m_stats.resfinal;
    }
    const ae_solve_stats& stats() const { return m_stats; }

protected:
    Operator::NodeOperator& linop;
    ae_solver_opts m_opts;
    ae_solve_stats m_stats{};
    double m_tol_rel = 1e-8, m_tol_abs = 1e-8;
};

// Newton<T>::solve (src/Solver/Nonlocal/Newton.H:141-205): m_nriters times, rhs = b - N(u), one
// Linear::solve of the correction (starting from the previous correction, as the reference
// keeps dsol), u += dsol.  Linear and affine models: rhs from ae_newton_residual (F0: one
// 9-component eigenstrain fab per level for an Affine model, or none).  NeoHookean: pass the
// model; every iteration sets the operator's stiffness to DDW(I + grad u) and forms rhs with
// DW(I + grad u) (ae_newton_neohookean).
template <class T>
class Newton : public Linear {
public:
    explicit Newton(Operator::Elastic<T>& op) : Linear(op), m_op(op) {}
    void setNRIters(int n) { m_nriters = n; }
    double solve(std::vector<alamo::Fab>& u, std::vector<alamo::Fab>& b, double tol_rel, double tol_abs,
                 const std::vector<alamo::Fab>* F0 = nullptr) {
        return run(u, b, tol_rel, tol_abs, F0, nullptr);
    }
    double solve(std::vector<alamo::Fab>& u, std::vector<alamo::Fab>& b, const T& model, double tol_rel,
                 double tol_abs) {
        return run(u, b, tol_rel, tol_abs, nullptr, &model);
    }

private:
    double run(std::vector<alamo::Fab>& u, std::vector<alamo::Fab>& b, double tol_rel, double tol_abs,
               const std::vector<alamo::Fab>* F0, const T* model) {
        const size_t nl = u.size();
        std::vector<std::vector<double>> dbuf(nl), rbuf(nl);
        std::vector<alamo::Fab> dsol(nl), rhs(nl);
        for (size_t l = 0; l < nl; ++l) {
            const size_t n = (size_t)b[l].npts() * b[l].ncomp;
            dbuf[l].assign((size_t)u[l].npts() * u[l].ncomp, 0.0);
            rbuf[l].assign(b[l].data, b[l].data + n);
            dsol[l] = alamo::Fab(dbuf[l].data(), u[l].lo, u[l].hi, u[l].ncomp);
            rhs[l] = alamo::Fab(rbuf[l].data(), b[l].lo, b[l].hi, b[l].ncomp);
        }
        double res = 0.0;
        for (int it = 0; it < m_nriters; ++it) {
            for (size_t l = 0; l < nl; ++l) {
                const ae_fab fu = u[l].c(), fb = b[l].c();
                ae_fab fr = rhs[l].c();
                if (model && T::kind == AE_MODEL_MAJOR) {
                    alamo::check(ae_newton_neohookean(m_op.handle(), (int)l, &fu, &fb, model_mu(*model),
                                                      model_kappa(*model), &fr));
                    continue;
                }
                ae_fab f0{};
                if (F0) f0 = (*F0)[l].c();
                alamo::check(ae_newton_residual(m_op.handle(), (int)l, &fu, &fb, F0 ? &f0 : nullptr, &fr));
            }
            res = Linear::solve(dsol, rhs, tol_rel, tol_abs);
            for (size_t l = 0; l < nl; ++l)
                for (size_t q = 0; q < dbuf[l].size(); ++q) u[l].data[q] += dbuf[l][q];
        }
        return res;
    }
    template <class M>
    static double model_mu(const M& m) {
        if constexpr (M::kind == AE_MODEL_MAJOR) return m.mu;
        else return 0.0;
    }
    template <class M>
    static double model_kappa(const M& m) {
        if constexpr (M::kind == AE_MODEL_MAJOR) return m.kappa;
        else return 0.0;
    }

    Operator::Elastic<T>& m_op;
    int m_nriters = 1;
};
}  // namespace Nonlocal
}  // namespace Solver

#endif
