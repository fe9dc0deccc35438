// Minimal stand-in for the part of AMReX 20.05 that the reference's per-node operator code uses,
// for levels made of ONE box: Box / IntVect / Dim3 / Array4 / BaseFab / FabArray / MultiFab /
// MFIter / Geometry / BoxArray, ParallelFor, and the AMREX_* macros.  TEST INFRASTRUCTURE ONLY:
// it lets the reference's own Fapply / Diagonal / Fsmooth / restriction / interpolation bodies
// (src/Operator/Elastic.cpp, src/Operator/Operator.cpp) and its model, stencil, tensor and BC
// headers compile unmodified, so that their outputs can pin the oracle.  AMReX itself is not in
// this image.
//
// Semantics kept from AMReX (public documentation of AMReX_Box.H / AMReX_Array4.H /
// AMReX_FabArray.H): inclusive index boxes with a cell/node type per direction; convert() turns a
// cell box into its node box (big end + 1); coarsen/refine of node boxes; Array4 indexing
// (i, j, k, n) with i fastest over a box that includes ghosts; MultiFab::Copy / Multiply /
// Subtract over the valid box grown by nghost; one MFIter tile per box (tiling only changes the
// traversal, not the values written).
#ifndef REFSHIM_AMREX_H
#define REFSHIM_AMREX_H

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <complex>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#define AMREX_SPACEDIM 3
#define BL_SPACEDIM 3
#define AMREX_FORCE_INLINE inline
#define AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST
#define AMREX_D_TERM(a, b, c) a b c
#define AMREX_D_DECL(a, b, c) a, b, c
#define AMREX_D_PICK(a, b, c) c
#define BL_PROFILE(x)
#define BL_PROFILE_VAR(x, y)
#define BL_PROFILE_VAR_STOP(y)
#define AMREX_ASSERT(x)
#define AMREX_ALWAYS_ASSERT(x)                                           \
    do {                                                                 \
        if (!(x)) throw std::runtime_error("amrex assertion: " #x);      \
    } while (0)
#define BL_ASSERT(x)

namespace amrex {

using Real = double;
template <class T>
using Vector = std::vector<T>;
template <class T, std::size_t N>
using Array = std::array<T, N>;

inline void Abort(const std::string& msg = "") { throw std::runtime_error("amrex::Abort " + msg); }

struct Dim3 {
    int x, y, z;
};

class IntVect {
public:
    int v[3];
    IntVect() : v{0, 0, 0} {}
    IntVect(int a, int b, int c) : v{a, b, c} {}
    explicit IntVect(int a) : v{a, a, a} {}
    int& operator[](int d) { return v[d]; }
    const int& operator[](int d) const { return v[d]; }
    const int* getVect() const { return v; }
    static IntVect TheNodeVector() { return IntVect(1, 1, 1); }
    static IntVect TheCellVector() { return IntVect(0, 0, 0); }
    static IntVect TheZeroVector() { return IntVect(0, 0, 0); }
    static IntVect TheUnitVector() { return IntVect(1, 1, 1); }
    bool operator==(const IntVect& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
    bool operator!=(const IntVect& o) const { return !(*this == o); }
    IntVect operator+(const IntVect& o) const { return IntVect(v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]); }
    IntVect operator-(const IntVect& o) const { return IntVect(v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]); }
};

// floor division, as AMReX's coarsen of an index
inline int coarsen_index(int i, int r) { return (i < 0) ? -((-i - 1) / r) - 1 : i / r; }

class Box {
public:
    IntVect smallend, bigend;
    IntVect btype;  // 1 = node-centred in that direction
    Box() : smallend(0), bigend(-1), btype(0) {}
    Box(const IntVect& lo, const IntVect& hi, const IntVect& t = IntVect(0)) : smallend(lo), bigend(hi), btype(t) {}
    const int* loVect() const { return smallend.v; }
    const int* hiVect() const { return bigend.v; }
    const IntVect& smallEnd() const { return smallend; }
    const IntVect& bigEnd() const { return bigend; }
    int smallEnd(int d) const { return smallend[d]; }
    int bigEnd(int d) const { return bigend[d]; }
    IntVect type() const { return btype; }
    bool ok() const { return bigend[0] >= smallend[0] && bigend[1] >= smallend[1] && bigend[2] >= smallend[2]; }
    long numPts() const {
        return ok() ? long(bigend[0] - smallend[0] + 1) * (bigend[1] - smallend[1] + 1) * (bigend[2] - smallend[2] + 1)
                    : 0;
    }
    int length(int d) const { return bigend[d] - smallend[d] + 1; }
    bool contains(const IntVect& p) const {
        for (int d = 0; d < 3; d++)
            if (p[d] < smallend[d] || p[d] > bigend[d]) return false;
        return true;
    }
    Box& convert(const IntVect& t) {
        for (int d = 0; d < 3; d++) {
            if (t[d] == btype[d]) continue;
            if (t[d] == 1) bigend[d] += 1; else bigend[d] -= 1;
            btype[d] = t[d];
        }
        return *this;
    }
    Box& grow(int n) {
        for (int d = 0; d < 3; d++) { smallend[d] -= n; bigend[d] += n; }
        return *this;
    }
    Box& grow(int d, int n) { smallend[d] -= n; bigend[d] += n; return *this; }
    Box& coarsen(int r) {
        for (int d = 0; d < 3; d++) {
            int off = (btype[d] && (bigend[d] % r)) ? 1 : 0;
            smallend[d] = coarsen_index(smallend[d], r);
            bigend[d] = coarsen_index(bigend[d], r) + off;
        }
        return *this;
    }
    Box& refine(int r) {
        for (int d = 0; d < 3; d++) {
            smallend[d] *= r;
            bigend[d] = btype[d] ? bigend[d] * r : (bigend[d] + 1) * r - 1;
        }
        return *this;
    }
    Box operator&(const Box& o) const {
        Box b(*this);
        for (int d = 0; d < 3; d++) {
            b.smallend[d] = std::max(smallend[d], o.smallend[d]);
            b.bigend[d] = std::min(bigend[d], o.bigend[d]);
        }
        return b;
    }
    Box& operator&=(const Box& o) { *this = *this & o; return *this; }
    bool operator==(const Box& o) const { return smallend == o.smallend && bigend == o.bigend && btype == o.btype; }
};

inline Box grow(const Box& b, int n) { Box r(b); return r.grow(n); }
inline Box coarsen(const Box& b, int r) { Box x(b); return x.coarsen(r); }
inline Box refine(const Box& b, int r) { Box x(b); return x.refine(r); }
inline Box convert(const Box& b, const IntVect& t) { Box x(b); return x.convert(t); }
inline Dim3 lbound(const Box& b) { return Dim3{b.smallend[0], b.smallend[1], b.smallend[2]}; }
inline Dim3 ubound(const Box& b) { return Dim3{b.bigend[0], b.bigend[1], b.bigend[2]}; }
inline Dim3 length(const Box& b) { return Dim3{b.length(0), b.length(1), b.length(2)}; }

template <class T>
struct Array4 {
    T* p = nullptr;
    long jstride = 0, kstride = 0, nstride = 0;
    Dim3 begin{0, 0, 0}, end{0, 0, 0};  // end is exclusive
    int ncomp = 0;
    Array4() {}
    Array4(T* a_p, const Box& b, int nc) : p(a_p), ncomp(nc) {
        begin = lbound(b);
        Dim3 h = ubound(b);
        end = Dim3{h.x + 1, h.y + 1, h.z + 1};
        jstride = end.x - begin.x;
        kstride = jstride * (end.y - begin.y);
        nstride = kstride * (end.z - begin.z);
    }
    template <class U>
    Array4(const Array4<U>& o)
        : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), begin(o.begin), end(o.end),
          ncomp(o.ncomp) {}
    long index(int i, int j, int k) const {
        if (i < begin.x || i >= end.x || j < begin.y || j >= end.y || k < begin.z || k >= end.z) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "Array4 index (%d,%d,%d) outside [%d..%d]x[%d..%d]x[%d..%d]", i, j, k,
                          begin.x, end.x - 1, begin.y, end.y - 1, begin.z, end.z - 1);
            throw std::runtime_error(msg);
        }
        return (i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride;
    }
    T& operator()(int i, int j, int k) const { return p[index(i, j, k)]; }
    T& operator()(int i, int j, int k, int n) const {
        if (n < 0 || n >= ncomp) throw std::runtime_error("Array4 component out of range");
        return p[index(i, j, k) + n * nstride];
    }
    T& operator()(const IntVect& m, int n = 0) const { return (*this)(m[0], m[1], m[2], n); }
    int nComp() const { return ncomp; }
};

// A fab over `box` (ghosts included) with `nc` components; data owned, or borrowed from a caller.
template <class T>
class BaseFab {
public:
    Box domain;
    int nvar = 0;
    std::vector<T> own;
    T* dptr = nullptr;
    BaseFab() {}
    BaseFab(const Box& b, int nc) { resize(b, nc); }
    BaseFab(const Box& b, int nc, T* borrowed) : domain(b), nvar(nc), dptr(borrowed) {}
    void resize(const Box& b, int nc) {
        domain = b;
        nvar = nc;
        own.assign(size_t(b.numPts()) * nc, T());
        dptr = own.data();
    }
    const Box& box() const { return domain; }
    int nComp() const { return nvar; }
    T* dataPtr() { return dptr; }
    Array4<T> array() { return Array4<T>(dptr, domain, nvar); }
    Array4<const T> array() const { return Array4<const T>(dptr, domain, nvar); }
    Array4<const T> const_array() const { return Array4<const T>(dptr, domain, nvar); }
    T& operator()(const IntVect& m, int n = 0) { return array()(m, n); }
    const T& operator()(const IntVect& m, int n = 0) const { return const_array()(m, n); }
    void setVal(const T& v) { for (long i = 0; i < domain.numPts() * nvar; i++) dptr[i] = v; }
    // this(dst region) += src(src region) over components [scomp, scomp + nc)
    BaseFab& plus(const BaseFab& src, const Box& srcbox, const Box& destbox, int scomp, int dcomp, int nc) {
        if (!(srcbox.numPts() == destbox.numPts())) throw std::runtime_error("plus: box mismatch");
        Array4<T> d = array();
        Array4<const T> s = src.const_array();
        for (int n = 0; n < nc; n++)
            for (int k = 0; k < destbox.length(2); k++)
                for (int j = 0; j < destbox.length(1); j++)
                    for (int i = 0; i < destbox.length(0); i++)
                        d(destbox.smallend[0] + i, destbox.smallend[1] + j, destbox.smallend[2] + k, dcomp + n) +=
                            s(srcbox.smallend[0] + i, srcbox.smallend[1] + j, srcbox.smallend[2] + k, scomp + n);
        return *this;
    }
};
using FArrayBox = BaseFab<Real>;

class BoxArray {
public:
    std::vector<Box> boxes;
    BoxArray() {}
    explicit BoxArray(const Box& b) : boxes{b} {}
    int size() const { return int(boxes.size()); }
    const Box& operator[](int i) const { return boxes[i]; }
    BoxArray& refine(int r) { for (auto& b : boxes) b.refine(r); return *this; }
    BoxArray& coarsen(int r) { for (auto& b : boxes) b.coarsen(r); return *this; }
    BoxArray& convert(const IntVect& t) { for (auto& b : boxes) b.convert(t); return *this; }
};
inline BoxArray coarsen(const BoxArray& ba, int r) { BoxArray x(ba); return x.coarsen(r); }

class DistributionMapping {
public:
    DistributionMapping() {}
    explicit DistributionMapping(const BoxArray&) {}
};

struct Periodicity {
    static Periodicity NonPeriodic() { return Periodicity(); }
};

class Geometry {
public:
    Box dom;       // cell-centred problem domain
    Real dx[3];
    Geometry() : dx{1, 1, 1} {}
    Geometry(const Box& cell_domain, const Real* a_dx) : dom(cell_domain), dx{a_dx[0], a_dx[1], a_dx[2]} {}
    const Box& Domain() const { return dom; }
    const Real* CellSize() const { return dx; }
    Real CellSize(int d) const { return dx[d]; }
    Periodicity periodicity() const { return Periodicity(); }
    bool isAnyPeriodic() const { return false; }
    bool isPeriodic(int) const { return false; }
};

class MFIter;

// A FabArray of exactly one fab: the valid box of the level plus nghost layers.
template <class FAB>
class FabArray {
public:
    BoxArray ba;
    DistributionMapping dm;
    int ncomp = 0, ngrow = 0;
    std::vector<FAB> fabs;
    FabArray() {}
    FabArray(const BoxArray& a_ba, const DistributionMapping& a_dm, int nc, int ng) { define(a_ba, a_dm, nc, ng); }
    void define(const BoxArray& a_ba, const DistributionMapping& a_dm, int nc, int ng) {
        ba = a_ba; dm = a_dm; ncomp = nc; ngrow = ng;
        fabs.clear();
        for (const Box& b : ba.boxes) fabs.emplace_back(grow(b, ng), nc);
    }
    // wrap caller memory (one box)
    template <class T>
    void define_borrowed(const Box& valid, int nc, int ng, T* data) {
        ba = BoxArray(valid); ncomp = nc; ngrow = ng;
        fabs.clear();
        fabs.emplace_back(grow(valid, ng), nc, data);
    }
    const BoxArray& boxArray() const { return ba; }
    const DistributionMapping& DistributionMap() const { return dm; }
    int nComp() const { return ncomp; }
    int nGrow() const { return ngrow; }
    int size() const { return int(fabs.size()); }
    FAB& operator[](const MFIter& mfi);
    const FAB& operator[](const MFIter& mfi) const;
    auto array(const MFIter& mfi) -> decltype(fabs[0].array());
    auto array(const MFIter& mfi) const -> decltype(static_cast<const FAB&>(fabs[0]).array());
    auto const_array(const MFIter& mfi) const -> decltype(fabs[0].const_array());
    template <class T>
    void setVal(const T& v) { for (auto& f : fabs) f.setVal(v); }
    // same-box copies (one box per level: FillBoundary / ParallelCopy have no other box to read)
    void FillBoundary(const Periodicity& = Periodicity()) {}
    template <class... A>
    void ParallelCopy(const FabArray& src, A...) { copy_region(src, 0, 0, std::min(ncomp, src.ncomp), src.ngrow, ngrow); }
    template <class... A>
    void copy(const FabArray& src, A...) { copy_region(src, 0, 0, std::min(ncomp, src.ncomp), src.ngrow, ngrow); }
    // copy src's valid box grown by src_ng into this fab where both are defined
    void copy_region(const FabArray& src, int scomp, int dcomp, int nc, int src_ng, int dst_ng) {
        for (size_t f = 0; f < fabs.size(); f++) {
            Box region = grow(src.ba[f], src_ng) & grow(ba[f], dst_ng);
            region &= src.fabs[f].box();
            region &= fabs[f].box();
            auto d = fabs[f].array();
            auto s = src.fabs[f].const_array();
            for (int n = 0; n < nc; n++)
                for (int k = region.smallend[2]; k <= region.bigend[2]; k++)
                    for (int j = region.smallend[1]; j <= region.bigend[1]; j++)
                        for (int i = region.smallend[0]; i <= region.bigend[0]; i++)
                            d(i, j, k, dcomp + n) = s(i, j, k, scomp + n);
        }
    }
};

class MultiFab : public FabArray<FArrayBox> {
public:
    MultiFab() {}
    MultiFab(const BoxArray& a_ba, const DistributionMapping& a_dm, int nc, int ng) : FabArray(a_ba, a_dm, nc, ng) {}
    Real norminf(int comp = 0, int ng = 0) const;
    template <class OP>
    static void binary(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int nc, int ng, OP op) {
        for (size_t f = 0; f < dst.fabs.size(); f++) {
            Box region = grow(dst.ba[f], ng) & dst.fabs[f].box() & src.fabs[f].box();
            auto d = dst.fabs[f].array();
            auto s = src.fabs[f].const_array();
            for (int n = 0; n < nc; n++)
                for (int k = region.smallend[2]; k <= region.bigend[2]; k++)
                    for (int j = region.smallend[1]; j <= region.bigend[1]; j++)
                        for (int i = region.smallend[0]; i <= region.bigend[0]; i++)
                            op(d(i, j, k, dcomp + n), s(i, j, k, scomp + n));
        }
    }
    static void Copy(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int nc, int ng) {
        binary(dst, src, scomp, dcomp, nc, ng, [](Real& a, Real b) { a = b; });
    }
    static void Multiply(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int nc, int ng) {
        binary(dst, src, scomp, dcomp, nc, ng, [](Real& a, Real b) { a *= b; });
    }
    static void Subtract(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int nc, int ng) {
        binary(dst, src, scomp, dcomp, nc, ng, [](Real& a, Real b) { a -= b; });
    }
    static void Add(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int nc, int ng) {
        binary(dst, src, scomp, dcomp, nc, ng, [](Real& a, Real b) { a += b; });
    }
};

class MFIter {
public:
    int idx = 0, n = 0;
    Box vbox;
    template <class FAB>
    MFIter(const FabArray<FAB>& fa, bool = false) : n(fa.size()), fa_ba(&fa.ba) { if (n) vbox = fa.ba[0]; }
    bool isValid() const { return idx < n; }
    MFIter& operator++() { idx++; if (idx < n) vbox = (*fa_ba)[idx]; return *this; }
    int index() const { return idx; }
    Box tilebox() const { return vbox; }
    Box validbox() const { return vbox; }
    Box growntilebox(int ng = 0) const { return grow(vbox, ng); }
    Box fabbox() const { return vbox; }
private:
    const BoxArray* fa_ba;
};

template <class FAB>
FAB& FabArray<FAB>::operator[](const MFIter& mfi) { return fabs[mfi.index()]; }
template <class FAB>
const FAB& FabArray<FAB>::operator[](const MFIter& mfi) const { return fabs[mfi.index()]; }
template <class FAB>
auto FabArray<FAB>::array(const MFIter& mfi) -> decltype(fabs[0].array()) { return fabs[mfi.index()].array(); }
template <class FAB>
auto FabArray<FAB>::array(const MFIter& mfi) const -> decltype(static_cast<const FAB&>(fabs[0]).array()) {
    return static_cast<const FAB&>(fabs[mfi.index()]).array();
}
template <class FAB>
auto FabArray<FAB>::const_array(const MFIter& mfi) const -> decltype(fabs[0].const_array()) {
    return fabs[mfi.index()].const_array();
}

inline Real MultiFab::norminf(int comp, int ng) const {
    Real m = 0;
    for (size_t f = 0; f < fabs.size(); f++) {
        Box region = grow(ba[f], ng);
        auto a = fabs[f].const_array();
        for (int k = region.smallend[2]; k <= region.bigend[2]; k++)
            for (int j = region.smallend[1]; j <= region.bigend[1]; j++)
                for (int i = region.smallend[0]; i <= region.bigend[0]; i++) m = std::max(m, std::fabs(a(i, j, k, comp)));
    }
    return m;
}

inline bool TilingIfNotGPU() { return true; }

template <class F>
void ParallelFor(const Box& bx, F&& f) {
    for (int k = bx.smallend[2]; k <= bx.bigend[2]; k++)
        for (int j = bx.smallend[1]; j <= bx.bigend[1]; j++)
            for (int i = bx.smallend[0]; i <= bx.bigend[0]; i++) f(i, j, k);
}

template <class FAB>
bool isMFIterSafe(const FabArray<FAB>&, const FabArray<FAB>&) { return true; }

template <class T>
Vector<T*> GetVecOfPtrs(Vector<T>& a) {
    Vector<T*> r;
    for (auto& x : a) r.push_back(&x);
    return r;
}
template <class T>
Vector<T*> GetVecOfPtrs(const Vector<std::unique_ptr<T>>& a) {
    Vector<T*> r;
    for (auto& x : a) r.push_back(x.get());
    return r;
}

inline std::ostream& Print() { return std::cout; }

}  // namespace amrex

#endif
