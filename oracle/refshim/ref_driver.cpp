// Driver that runs the reference's OWN per-node code on single-box levels, to produce golden
// vectors for the oracle.  TEST INFRASTRUCTURE ONLY: tests/golden/make_ref_golden.py loads the
// library built from this file (oracle/_ref/libref.so); nothing in the product links it.
//
// What is the reference's code here, compiled unmodified from the reference tree:
//   - the headers src/Set/{Base,Set,Matrix3,Matrix4*}.H, src/Numeric/Stencil.H,
//     src/Model/Solid/Solid.H, src/Model/Solid/Linear/{Isotropic,Cubic,Laplacian}.H,
//     src/BC/Operator/Elastic.H, src/Numeric/Interpolator/{Interpolator,Linear}.H;
//   - the member-function definitions that oracle/refshim/build_ref.py extracts verbatim into
//     oracle/_ref/extracted.inc: Elastic<T>::Fapply, Diagonal, Strain, Stress, Energy and
//     averageDownCoeffsSameAmrLevel (src/Operator/Elastic.cpp:151-352, 399-569, 722-809) and
//     Operator<Grid::Node>::Fsmooth, restriction and interpolation
//     (src/Operator/Operator.cpp:90-162, 454-624).
// What is ours: the AMReX / Eigen / Util / ParmParse stand-ins under oracle/refshim/include, the
// two stand-in class declarations below (the members those definitions use, with the reference's
// names and signatures), and the extern "C" entry points at the end.
//
// One box per level.  AMReX's FillBoundary, ParallelCopy and nodalSync exchange data between the
// boxes of a level; with one box covering the level they copy nothing, so realFillBoundary,
// nodalSync, applyBC and FillBoundaryCoeff are no-ops here.
#include <cstring>
#include <string>

#include "Set/Set.H"
#include "Numeric/Stencil.H"
#include "Model/Solid/Linear/Isotropic.H"
#include "Model/Solid/Linear/Cubic.H"
#include "Model/Solid/Linear/Laplacian.H"
#include "Model/Solid/Elastic/NeoHookean.H"
#include "BC/Operator/Elastic.H"

using namespace amrex;

enum Grid { Cell, Node };

namespace Operator {

template <Grid G>
class Operator;

// Stand-in for src/Operator/Operator.H:30-128 (an amrex::MLNodeLinOp subclass there).
template <>
class Operator<Grid::Node> {
public:
    enum class BCMode { Homogeneous, Inhomogeneous };  // amrex::MLLinOp::BCMode
    enum class StateMode { Solution, Correction };     // amrex::MLLinOp::StateMode
    virtual ~Operator() {}
    virtual void Fapply(int amrlev, int mglev, MultiFab& out, const MultiFab& in) const = 0;
    void Fsmooth(int amrlev, int mglev, amrex::MultiFab& x, const amrex::MultiFab& b) const;
    void restriction(int amrlev, int cmglev, MultiFab& crse, MultiFab& fine) const;
    void interpolation(int amrlev, int fmglev, MultiFab& fine, const MultiFab& crse) const;
    static void realFillBoundary(MultiFab&, const Geometry&) {}
    void nodalSync(int, int, MultiFab&) const {}
    void applyBC(int, int, MultiFab&, BCMode, StateMode, bool = false) const {}

    Vector<Vector<Geometry>> m_geom;
    Vector<int> m_num_mg_levels;
    int m_num_amr_levels = 1;
    bool m_diagonal_computed = false;
    Vector<Vector<std::unique_ptr<MultiFab>>> m_diag;
};

// Stand-in for src/Operator/Elastic.H:20-171.
template <class T>
class Elastic : public Operator<Grid::Node> {
public:
    using TArrayBox = amrex::BaseFab<T>;
    using MultiTab = amrex::FabArray<TArrayBox>;
    void Fapply(int amrlev, int mglev, MultiFab& a_f, const MultiFab& a_u) const override;
    void Diagonal(int amrlev, int mglev, MultiFab& a_diag);
    void Strain(int amrlev, amrex::MultiFab& a_eps, const amrex::MultiFab& a_u, bool voigt) const;
    void Stress(int amrlev, amrex::MultiFab& a_sigma, const amrex::MultiFab& a_u, bool voigt, bool a_homogeneous);
    void Energy(int amrlev, amrex::MultiFab& a_energy, const amrex::MultiFab& a_u, bool a_homogeneous);
    void averageDownCoeffsSameAmrLevel(int amrlev);
    void FillBoundaryCoeff(MultiTab&, const Geometry&) {}
    void SetHomogeneous(bool a_homogeneous) { m_homogeneous = a_homogeneous; }

    amrex::Vector<amrex::Vector<std::unique_ptr<amrex::FabArray<amrex::BaseFab<T>>>>> model;
    bool m_uniform = false;
    bool m_homogeneous = false;
    ::BC::Operator::Elastic<T>* m_bc = nullptr;
};

#include "extracted.inc"

}  // namespace Operator

// ===================================================================== extern "C" driver
namespace {

// Same layout as the oracle's orc_level: nodal domain, nodal valid box, ghost layers, cell size.
struct RefLevel {
    int dom_lo[3], dom_hi[3];
    int lo[3], hi[3];
    int ng;
    int pad_;
    double dx[3];
};

std::string g_err;

Box valid_box(const RefLevel& L) {
    return Box(IntVect(L.lo[0], L.lo[1], L.lo[2]), IntVect(L.hi[0], L.hi[1], L.hi[2]), IntVect::TheNodeVector());
}
Box store_box(const RefLevel& L) { return grow(valid_box(L), L.ng); }
// cell-centred domain: nodes [dom_lo, dom_hi] are cells [dom_lo, dom_hi - 1]
Geometry geometry(const RefLevel& L) {
    Box cells(IntVect(L.dom_lo[0], L.dom_lo[1], L.dom_lo[2]), IntVect(L.dom_hi[0] - 1, L.dom_hi[1] - 1, L.dom_hi[2] - 1));
    return Geometry(cells, L.dx);
}
long npts(const RefLevel& L) { return store_box(L).numPts(); }

// A MultiFab over the level's storage that reads/writes the caller's array [comp][k][j][i].
std::unique_ptr<MultiFab> wrap(const RefLevel& L, int ncomp, const double* data) {
    std::unique_ptr<MultiFab> mf(new MultiFab());
    mf->define_borrowed(valid_box(L), ncomp, L.ng, const_cast<double*>(data));
    return mf;
}

template <class T>
using Op = ::Operator::Elastic<T>;
using Iso = Model::Solid::Linear::Isotropic;
using Cub = Model::Solid::Linear::Cubic;
using Lap = Model::Solid::Linear::Laplacian;
using Neo = Model::Solid::Elastic::NeoHookean;

// One model per node from the oracle's coefficient layout [slot][k][j][i].
Iso make_model(const Iso*, const double* C, long n, long p, const int*) { return Iso(C[p + n], C[p]); }  // (mu, lambda)
Cub make_model(const Cub*, const double* C, long n, long p, const int* slot81) {
    Cub m;
    m.ddw = Set::Matrix4<3, Set::Sym::MajorMinor>::Zero();
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) m.ddw(i, j, k, l) = C[p + n * slot81[((i * 3 + j) * 3 + k) * 3 + l]];
    return m;
}
Lap make_model(const Lap*, const double* C, long n, long p, const int*) {
    Set::Matrix A;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A(i, j) = C[p + n * (3 * i + j)];
    Model::Solid::Solid<Set::Sym::Diagonal> base;
    base.ddw = Set::Matrix4<3, Set::Sym::Diagonal>(A);
    return Lap(base);
}

// Elastic<NeoHookean> reads only the tangent ddw (a Sym::Major tensor): the 45 slots in
// upper-triangle order, written through the tensor's (i, j, k, l) accessor
Neo make_model(const Neo*, const double* C, long n, long p, const int*) {
    Neo m;
    int s = 0;
    for (int I = 0; I < 9; I++)
        for (int K = I; K < 9; K++, s++) m.ddw(I / 3, I % 3, K / 3, K % 3) = C[p + n * s];
    return m;
}

template <class T>
std::unique_ptr<amrex::FabArray<amrex::BaseFab<T>>> model_fab(const RefLevel& L, const double* C, const int* slot81) {
    std::unique_ptr<amrex::FabArray<amrex::BaseFab<T>>> fa(new amrex::FabArray<amrex::BaseFab<T>>());
    fa->define(BoxArray(valid_box(L)), DistributionMapping(), 1, L.ng);
    T* d = fa->fabs[0].dataPtr();
    const long n = npts(L);
    for (long p = 0; p < n; p++) d[p] = make_model((const T*)nullptr, C, n, p, slot81);
    return fa;
}

template <class T>
struct Setup {
    Op<T> op;
    ::BC::Operator::Elastic<T> bc;
    Setup(const RefLevel& L, const double* C, const int* slot81, const int* bctype, const double* bcval, int uniform,
          int homogeneous) {
        op.m_geom = {{geometry(L)}};
        op.m_num_mg_levels = {1};
        op.model.resize(1);
        op.model[0].push_back(model_fab<T>(L, C, slot81));
        for (int f = 0; f < 26; f++)
            for (int d = 0; d < 3; d++)
                bc.Set((typename ::BC::Operator::Elastic<T>::Face)f, (typename ::BC::Operator::Elastic<T>::Direction)d,
                       (typename ::BC::Operator::Elastic<T>::Type)(bctype ? bctype[3 * f + d] : 0),
                       bcval ? bcval[3 * f + d] : 0.0);
        op.m_bc = &bc;
        op.m_uniform = uniform != 0;
        op.m_homogeneous = homogeneous != 0;
    }
};

template <class F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

template <template <class> class Fn, class... A>
int dispatch(int model, A... a) {
    switch (model) {
        case 0: return guarded([&] { Fn<Iso>::run(a...); });
        case 1: return guarded([&] { Fn<Cub>::run(a...); });
        case 2: return guarded([&] { Fn<Lap>::run(a...); });
        case 3: return guarded([&] { Fn<Neo>::run(a...); });
    }
    g_err = "unknown model kind";
    return -2;
}

template <class T>
struct FapplyFn {
    static void run(const RefLevel* L, const double* C, const int* slot81, const int* bctype, const double* bcval,
                    int uniform, int homogeneous, const double* u, double* f) {
        Setup<T> s(*L, C, slot81, bctype, bcval, uniform, homogeneous);
        auto U = wrap(*L, 3, u), F = wrap(*L, 3, f);
        s.op.Fapply(0, 0, *F, *U);
    }
};
template <class T>
struct DiagonalFn {
    static void run(const RefLevel* L, const double* C, const int* slot81, const int* bctype, const double* bcval,
                    double* diag) {
        Setup<T> s(*L, C, slot81, bctype, bcval, 0, 0);
        auto D = wrap(*L, 3, diag);
        s.op.Diagonal(0, 0, *D);
    }
};
template <class T>
struct FsmoothFn {  // one Operator<Node>::Fsmooth call: two damped-Jacobi sweeps
    static void run(const RefLevel* L, const double* C, const int* slot81, const int* bctype, const double* bcval,
                    int uniform, const double* diag, double* x, const double* b) {
        Setup<T> s(*L, C, slot81, bctype, bcval, uniform, 0);
        s.op.m_diag.resize(1);
        s.op.m_diag[0].push_back(wrap(*L, 3, diag));
        s.op.m_diagonal_computed = true;
        auto X = wrap(*L, 3, x), B = wrap(*L, 3, b);
        s.op.Fsmooth(0, 0, *X, *B);
    }
};
template <class T>
struct FieldsFn {  // which: 0 strain (voigt?), 1 stress (voigt?), 2 energy
    static void run(const RefLevel* L, const double* C, const int* slot81, int which, int voigt, const double* u,
                    double* out) {
        Setup<T> s(*L, C, slot81, nullptr, nullptr, 0, 0);
        auto U = wrap(*L, 3, u);
        const int nc = which == 2 ? 1 : (voigt ? 6 : 9);
        auto O = wrap(*L, nc, out);
        if (which == 0) s.op.Strain(0, *O, *U, voigt != 0);
        else if (which == 1) s.op.Stress(0, *O, *U, voigt != 0, false);
        else s.op.Energy(0, *O, *U, false);
    }
};
template <class T>
struct AvgDownFn {  // stiffness of the level below (coarsened by 2): averageDownCoeffsSameAmrLevel
    static void run(const RefLevel* Lf, const RefLevel* Lc, const double* Cf, const int* slot81, double* Cc,
                    int ncoef) {
        Setup<T> s(*Lf, Cf, slot81, nullptr, nullptr, 0, 0);
        s.op.m_geom[0].push_back(geometry(*Lc));
        s.op.m_num_mg_levels = {2};
        std::vector<double> zero(size_t(npts(*Lc)) * ncoef, 0.0);
        s.op.model[0].push_back(model_fab<T>(*Lc, zero.data(), slot81));
        s.op.averageDownCoeffsSameAmrLevel(0);
        // read back the coarse models in the oracle's layout
        const long n = npts(*Lc);
        const T* d = s.op.model[0][1]->fabs[0].dataPtr();
        for (long p = 0; p < n; p++) {
            T m = d[p];
            for (int c = 0; c < ncoef; c++) Cc[p + n * c] = 0.0;
            read_coeffs(m, Cc, n, p, slot81);
        }
    }
    static void read_coeffs(Iso& m, double* Cc, long n, long p, const int*) {
        Cc[p] = m.ddw(0, 0, 1, 1);      // lambda
        Cc[p + n] = m.ddw(0, 1, 0, 1);  // mu
    }
    static void read_coeffs(Cub& m, double* Cc, long n, long p, const int* slot81) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) Cc[p + n * slot81[((i * 3 + j) * 3 + k) * 3 + l]] = m.ddw(i, j, k, l);
    }
    static void read_coeffs(Lap& m, double* Cc, long n, long p, const int*) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Cc[p + n * (3 * i + j)] = m.ddw(i, j, i, j);
    }
    static void read_coeffs(Neo& m, double* Cc, long n, long p, const int*) {
        int s = 0;
        for (int I = 0; I < 9; I++)
            for (int K = I; K < 9; K++, s++) Cc[p + n * s] = m.ddw(I / 3, I % 3, K / 3, K % 3);
    }
};
template <class T>
struct BcInitFn {
    static void run(const RefLevel* L, const int* bctype, const double* bcval, int homogeneous, double* rhs) {
        ::BC::Operator::Elastic<T> bc;
        for (int f = 0; f < 26; f++)
            for (int d = 0; d < 3; d++)
                bc.Set((typename ::BC::Operator::Elastic<T>::Face)f, (typename ::BC::Operator::Elastic<T>::Direction)d,
                       (typename ::BC::Operator::Elastic<T>::Type)bctype[3 * f + d], bcval[3 * f + d]);
        auto R = wrap(*L, 3, rhs);
        bc.Init(R.get(), geometry(*L), homogeneous != 0);
    }
};

}  // namespace

extern "C" {

const char* ref_error(void) { return g_err.c_str(); }

int ref_fapply(const RefLevel* L, int model, const double* C, const int* slot81, const int* bctype,
               const double* bcval, int uniform, int homogeneous, const double* u, double* f) {
    return dispatch<FapplyFn>(model, L, C, slot81, bctype, bcval, uniform, homogeneous, u, f);
}

int ref_diagonal(const RefLevel* L, int model, const double* C, const int* slot81, const int* bctype,
                 const double* bcval, double* diag) {
    return dispatch<DiagonalFn>(model, L, C, slot81, bctype, bcval, diag);
}

int ref_fsmooth(const RefLevel* L, int model, const double* C, const int* slot81, const int* bctype,
                const double* bcval, int uniform, const double* diag, double* x, const double* b) {
    return dispatch<FsmoothFn>(model, L, C, slot81, bctype, bcval, uniform, diag, x, b);
}

int ref_fields(const RefLevel* L, int model, const double* C, const int* slot81, int which, int voigt,
               const double* u, double* out) {
    return dispatch<FieldsFn>(model, L, C, slot81, which, voigt, u, out);
}

int ref_average_down_coeffs(const RefLevel* Lf, const RefLevel* Lc, int model, const double* Cf, const int* slot81,
                            double* Cc) {
    const int ncoef = model == 0 ? 2 : (model == 1 ? 21 : 9);
    return dispatch<AvgDownFn>(model, Lf, Lc, Cf, slot81, Cc, ncoef);
}

int ref_bc_init(const RefLevel* L, const int* bctype, const double* bcval, int homogeneous, double* rhs) {
    return guarded([&] { BcInitFn<Iso>::run(L, bctype, bcval, homogeneous, rhs); });
}

// Operator<Node>::restriction from level Lf (fine, MG level 0) to Lc (MG level 1), ncomp components
int ref_restrict(const RefLevel* Lc, const RefLevel* Lf, int ncomp, double* crse, const double* fine) {
    return guarded([&] {
        Op<Iso> op;
        op.m_geom = {{geometry(*Lf), geometry(*Lc)}};
        auto Cr = wrap(*Lc, ncomp, crse), Fi = wrap(*Lf, ncomp, fine);
        op.restriction(0, 1, *Cr, *Fi);
    });
}

// Operator<Node>::interpolation: fine += interpolated coarse
int ref_interp_add(const RefLevel* Lf, const RefLevel* Lc, int ncomp, double* fine, const double* crse) {
    return guarded([&] {
        Op<Iso> op;
        op.m_geom = {{geometry(*Lf), geometry(*Lc)}};
        auto Cr = wrap(*Lc, ncomp, crse), Fi = wrap(*Lf, ncomp, fine);
        op.interpolation(0, 0, *Fi, *Cr);
    });
}

// Model::Solid::Linear::Cubic::Define(C11, C12, C44, R) (src/Model/Solid/Linear/Cubic.H:31-59);
// R row-major; out21 in the oracle's slot order
int ref_cubic_define(double C11, double C12, double C44, const double* R, const int* slot81, double* out21) {
    return guarded([&] {
        Eigen::Matrix3d m;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) m(i, j) = R[3 * i + j];
        Cub c;
        c.Define(C11, C12, C44, m);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) out21[slot81[((i * 3 + j) * 3 + k) * 3 + l]] = c.ddw(i, j, k, l);
    });
}

// Model::Solid::Elastic::NeoHookean::W / DW / DDW (src/Model/Solid/Elastic/NeoHookean.H:19-66) at
// n deformation gradients F (row-major 3 x 3 each): w[n], dw[n][9] row-major, ddw[n][45] the
// Sym::Major slots, each read through the tensor's own (i, j, k, l) accessor at its
// upper-triangle index (3i+j <= 3k+l)
int ref_neohookean(double mu, double kappa, int n, const double* F, double* w, double* dw, double* ddw) {
    return guarded([&] {
        Model::Solid::Elastic::NeoHookean m;
        m.mu = mu;
        m.kappa = kappa;
        for (int p = 0; p < n; p++) {
            Set::Matrix Fm;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) Fm(i, j) = F[9 * p + 3 * i + j];
            w[p] = m.W(Fm);
            const Set::Matrix d = m.DW(Fm);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) dw[9 * p + 3 * i + j] = d(i, j);
            const Set::Matrix4<3, Set::Sym::Major> t = m.DDW(Fm);
            int s = 0;
            for (int I = 0; I < 9; I++)
                for (int K = I; K < 9; K++, s++) ddw[45 * p + s] = t(I / 3, I % 3, K / 3, K % 3);
        }
    });
}

}  // extern "C"
