// The reference's UniaxialTest (src/Test/Operator/Elastic_UniaxialTest.cpp:13-203) written against
// the C++ shim include/alamo_elastic.H, exactly as an Alamo integrator would call the operator:
// Operator::Elastic<Linear::Isotropic>, BC::Operator::Elastic, Solver::Nonlocal::Newton.
// Host fabs; prints the relative error of u_x = 0.1 x and exits 0 when it is below 1 %.
#include <cmath>
#include <cstdio>
#include <vector>

#include "alamo_elastic.H"

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 32;
    using model_type = Model::Solid::Linear::Isotropic;
    model_type model(2.6, 6.0);  // (mu, lambda), Elastic_UniaxialTest.cpp:164-165
    alamo::Level L0{{n, n, n}, {0, 0, 0}, {n, n, n}, {1.0 / n, 1.0 / n, 1.0 / n}};
    Operator::Elastic<model_type> elastic({L0});
    elastic.SetUniform(false);
    elastic.SetModel(model);
    BC::Operator::Elastic<model_type> bc;
    using B = BC::Operator::Elastic<model_type>;
    bc.Set(B::XHI, B::X, B::Displacement, 0.1);
    bc.Set(B::XHI, B::Y, B::Neumann, 0.0);
    bc.Set(B::YLO, B::X, B::Neumann, 0.0);
    bc.Set(B::YHI, B::X, B::Neumann, 0.0);
    bc.Set(B::XHI_YHI, B::X, B::Displacement, 0.1);
    bc.Set(B::XHI_YLO, B::X, B::Displacement, 0.1);
    bc.Set(B::XHI, B::Z, B::Neumann, 0.0);
    bc.Set(B::ZLO, B::X, B::Neumann, 0.0);
    bc.Set(B::ZHI, B::X, B::Neumann, 0.0);
    bc.Set(B::ZHI_XHI, B::X, B::Displacement, 0.1);
    bc.Set(B::ZLO_XHI, B::X, B::Displacement, 0.1);
    for (auto c : {B::XHI_YLO_ZLO, B::XHI_YLO_ZHI, B::XHI_YHI_ZLO, B::XHI_YHI_ZHI}) bc.Set(c, B::X, B::Displacement, 0.1);
    for (auto e : {B::YLO_ZLO, B::YLO_ZHI, B::YHI_ZLO, B::YHI_ZHI}) {
        bc.Set(e, B::X, B::Neumann, 0.0);
        bc.Set(e, B::Y, B::Neumann, 0.0);
    }
    elastic.SetBC(&bc);
    const long long npts = (long long)(n + 1) * (n + 1) * (n + 1);
    std::vector<double> u(3 * npts, 0.0), rhs(3 * npts, 0.0);
    alamo::Fab U(u.data(), {0, 0, 0}, {n, n, n}, 3), R(rhs.data(), {0, 0, 0}, {n, n, n}, 3);
    // BC::Operator::Elastic::Init: boundary values into the rhs (only XHI-side x values are nonzero)
    for (int k = 0; k <= n; ++k)
        for (int j = 0; j <= n; ++j) R(n, j, k, 0) = 0.1;
    std::vector<alamo::Fab> sol{U}, b{R};
    Solver::Nonlocal::Newton<model_type> solver(elastic);
    solver.setMaxIter(400);
    solver.solve(sol, b, 1e-8, 1e-8);
    double err = 0.0;
    for (int k = 0; k <= n; ++k)
        for (int j = 0; j <= n; ++j)
            for (int i = 0; i <= n; ++i) {
                err = std::fmax(err, std::fabs(U(i, j, k, 0) - 0.1 * i / n));
                err = std::fmax(err, std::fabs(U(i, j, k, 1)) + std::fabs(U(i, j, k, 2)));
            }
    std::printf("{\"iters\": %d, \"rel_err\": %.3e, \"converged\": %d}\n", solver.stats().iters, err / 0.1,
                solver.stats().converged);
    return err / 0.1 < 0.01 ? 0 : 1;
}
