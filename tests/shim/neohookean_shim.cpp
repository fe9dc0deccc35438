// Newton<Model::Solid::Elastic::NeoHookean> through the C++ shim include/alamo_elastic.H, the way
// src/Integrator/FiniteKinematics.H:79-117 calls it: a block stretched 10 % along x with symmetry
// rollers on the low faces and traction-free elsewhere.  The exact solution is homogeneous,
// F = diag(s, t, t) with the lateral stress DW_yy(F) = 0, and the nodal operator reproduces affine
// fields exactly, so Newton lands on it.  Host fabs; prints the error and exits 0 below 1e-9.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "alamo_elastic.H"

// DW_yy of NeoHookean.H:28-39 at F = diag(s, t, t)
static double dw_yy(double mu, double kappa, double s, double t) {
    const double J = s * t * t, J23 = std::pow(std::fabs(J), 2.0 / 3.0), tr = s * s + 2 * t * t;
    return mu * (t / J23 - tr * (1.0 / t) / (3.0 * J23)) + kappa * (J - 1.0) * J * (1.0 / t);
}

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 8;
    const double mu = 1.3, kappa = 2.7, d = 0.1, s = 1.0 + d;
    double lo = 0.5, hi = 1.5;  // lateral stretch t: dw_yy changes sign once on [0.5, 1.5]
    for (int it = 0; it < 200; ++it) {
        const double m = 0.5 * (lo + hi);
        if ((dw_yy(mu, kappa, s, lo) < 0) == (dw_yy(mu, kappa, s, m) < 0)) lo = m;
        else hi = m;
    }
    const double t = 0.5 * (lo + hi);
    using model_type = Model::Solid::Elastic::NeoHookean;
    alamo::Level L0{{n, n, n}, {0, 0, 0}, {n, n, n}, {1.0 / n, 1.0 / n, 1.0 / n}};
    Operator::Elastic<model_type> op({L0});
    op.SetUniform(false);
    using B = BC::Operator::Elastic<model_type>;
    B bc;
    static const char* names[26] = {"XLO", "YLO", "ZLO", "XHI", "YHI", "ZHI", "YLO_ZLO", "YLO_ZHI", "YHI_ZLO",
                                    "YHI_ZHI", "ZLO_XLO", "ZLO_XHI", "ZHI_XLO", "ZHI_XHI", "XLO_YLO", "XLO_YHI",
                                    "XHI_YLO", "XHI_YHI", "XLO_YLO_ZLO", "XLO_YLO_ZHI", "XLO_YHI_ZLO", "XLO_YHI_ZHI",
                                    "XHI_YLO_ZLO", "XHI_YLO_ZHI", "XHI_YHI_ZLO", "XHI_YHI_ZHI"};
    static const char* lo_of[3] = {"XLO", "YLO", "ZLO"};
    for (int f = 0; f < 26; ++f)
        for (int p = 0; p < 3; ++p) {
            const auto face = static_cast<B::Face>(f);
            const auto dir = static_cast<B::Direction>(p);
            if (std::strstr(names[f], lo_of[p])) bc.Set(face, dir, B::Displacement, 0.0);
            else if (p == 0 && std::strstr(names[f], "XHI")) bc.Set(face, dir, B::Displacement, d);
            else bc.Set(face, dir, B::Traction, 0.0);
        }
    op.SetBC(&bc);
    const long long npts = (long long)(n + 1) * (n + 1) * (n + 1);
    std::vector<double> u(3 * npts, 0.0), rhs(3 * npts, 0.0);
    alamo::Fab U(u.data(), {0, 0, 0}, {n, n, n}, 3), R(rhs.data(), {0, 0, 0}, {n, n, n}, 3);
    for (int k = 0; k <= n; ++k)  // BC::Operator::Elastic::Init: the pulled face's x values
        for (int j = 0; j <= n; ++j) R(n, j, k, 0) = d;
    std::vector<alamo::Fab> sol{U}, b{R};
    Solver::Nonlocal::Newton<model_type> nr(op);
    nr.setNRIters(7);
    nr.setMaxIter(400);
    nr.solve(sol, b, model_type(mu, kappa), 1e-12, 0.0);
    double err = 0.0;
    for (int k = 0; k <= n; ++k)
        for (int j = 0; j <= n; ++j)
            for (int i = 0; i <= n; ++i) {
                const double x = (double)i / n, y = (double)j / n, z = (double)k / n;
                err = std::fmax(err, std::fabs(U(i, j, k, 0) - (s - 1) * x));
                err = std::fmax(err, std::fabs(U(i, j, k, 1) - (t - 1) * y));
                err = std::fmax(err, std::fabs(U(i, j, k, 2) - (t - 1) * z));
            }
    std::printf("{\"t\": %.12f, \"max_err\": %.3e}\n", t, err);
    return err < 1e-9 ? 0 : 1;
}
