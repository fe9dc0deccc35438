// Stand-in for the reference's src/IO/ParmParse.H (a wrapper of amrex::ParmParse): an input
// reader with no entries, so every query leaves its default in place.  Test infrastructure
// only; the golden-vector driver sets models and BCs through their C++ setters instead.
#ifndef IO_PARMPARSE
#define IO_PARMPARSE

#include <string>
#include <vector>

#include "AMReX.H"

namespace IO {
class ParmParse {
public:
    ParmParse() {}
    explicit ParmParse(const std::string&) {}
    template <class T>
    int query(const char*, T&) const { return 0; }
    template <class T>
    int query(const std::string&, T&) const { return 0; }
    template <class T>
    int queryarr(const char*, T&) const { return 0; }
    template <class T>
    int queryarr(const std::string&, T&) const { return 0; }
    int contains(const char*) const { return 0; }
    int contains(const std::string&) const { return 0; }
    std::string getPrefix() const { return ""; }
    template <class T>
    void queryclass(std::string, T*) {}
    template <class T>
    void queryclass(std::string, T&) {}
    template <class T>
    void queryclass(T*) {}
    template <class T>
    void queryclass(T&) {}
};
}  // namespace IO

#endif
