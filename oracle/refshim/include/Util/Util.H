// Stand-in for the reference's src/Util/Util.H with the names its operator, model and BC
// headers use: INFO / TEST, Util::Abort (throws, as amrex.throw_exception = 1 makes the
// reference's do), Util::Message / Warning / Assert, Util::Random and Util::String helpers.
// Test infrastructure only: it takes the place of the real header, which pulls in AMReX's
// I/O and parallel layers.
#ifndef UTIL_UTIL_H
#define UTIL_UTIL_H

#include <cstdlib>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "AMReX.H"

#define INFO __FILE__, __func__, __LINE__
#define TEST(x) #x, x

namespace Util {

namespace detail {
inline void put(std::ostringstream&) {}
template <class A, class... R>
void put(std::ostringstream& os, const A& a, const R&... r) {
    os << a;
    put(os, r...);
}
}  // namespace detail

template <typename... Args>
void Abort(std::string file, std::string func, int line, Args const&... args) {
    std::ostringstream os;
    os << file << ":" << line << " (" << func << ") ";
    detail::put(os, args...);
    throw std::runtime_error(os.str());
}
inline void Abort(const char* msg) { throw std::runtime_error(msg); }
template <typename... Args>
void Message(std::string, std::string, int, Args const&...) {}
template <typename... Args>
void Warning(std::string, std::string, int, Args const&...) {}
template <typename... Args>
void ParallelMessage(std::string, std::string, int, Args const&...) {}
inline void Assert(std::string file, std::string func, int line, std::string smt, bool pass) {
    if (!pass) Abort(file, func, line, "assertion failed: ", smt);
}
inline double Random() { return double(std::rand()) / double(RAND_MAX); }

namespace String {
inline int ReplaceAll(std::string& str, const std::string before, const std::string after) {
    int n = 0;
    size_t p = 0;
    while (!before.empty() && (p = str.find(before, p)) != std::string::npos) {
        str.replace(p, before.size(), after);
        p += after.size();
        n++;
    }
    return n;
}
inline int ReplaceAll(std::string& str, const char before, const std::string after) {
    return ReplaceAll(str, std::string(1, before), after);
}
inline std::vector<std::string> Split(std::string& str, const char token = ' ') {
    std::vector<std::string> out;
    std::string cur;
    for (char c : str) {
        if (c == token) { if (!cur.empty()) out.push_back(cur); cur.clear(); }
        else cur += c;
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}
inline bool Contains(std::string& str, const std::string find) { return str.find(find) != std::string::npos; }
}  // namespace String

namespace Test {
inline int Message(std::string) { return 0; }
inline int Message(std::string, int passed) { return passed; }
}  // namespace Test

template <class T>
void RealFillBoundary(amrex::FabArray<amrex::BaseFab<T>>&, const amrex::Geometry&) {}
inline void RealFillBoundary(amrex::MultiFab&, const amrex::Geometry&) {}

}  // namespace Util

#endif
