// AMReX plotfile writer for nodal fields: the "node" plotfile Integrator::WritePlotFile emits
// (src/Integrator/Integrator.cpp:582-681) through amrex::WriteMultiLevelPlotfile, one patch per
// AMR level.  Host code only (no CUDA calls), so it runs where the fields already are on the host.
//
// Directory layout, as AMReX writes it and as the reference's scripts/analyze.py reads it:
//   <dir>/Header               HyperCLaw-V1.1 plotfile header
//   <dir>/Level_<l>/Cell_H     VisMF header: box array, FAB file and offset, per-component min/max
//   <dir>/Level_<l>/Cell_D_00000  "FAB <real descriptor><box> <ncomp>\n" then the raw doubles,
//                              i fastest, then j, k, component (the Array4 order of the fab)
#include <cmath>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "aefast.h"

namespace ae {
void set_last_error(const std::string& msg);  // ae_api.cu: the message ae_last_error() returns
}

namespace {

struct PlotError {
    ae_status code;
    std::string msg;
};

void need(bool ok, const std::string& msg, ae_status code = AE_ERR_ARG) {
    if (!ok) throw PlotError{code, msg};
}

// an AMReX Box as text: ((lo) (hi) (type))
std::string box_text(const int lo[3], const int hi[3], int type) {
    std::ostringstream s;
    s << "((" << lo[0] << ',' << lo[1] << ',' << lo[2] << ") (" << hi[0] << ',' << hi[1] << ',' << hi[2] << ") ("
      << type << ',' << type << ',' << type << "))";
    return s.str();
}

bool little_endian() {
    const unsigned one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// IEEE double, byte order of this machine, in AMReX's RealDescriptor notation
std::string real_descriptor() {
    return little_endian() ? "((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))"
                           : "((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))";
}

struct LevelOut {
    int lo[3], hi[3];  // nodal valid box
    std::vector<double> mn, mx;
};

}  // namespace

extern "C" {

int ae_write_plotfile(const char* dir, int nlevels, const ae_level_desc* levels, const ae_fab* fabs, int ncomp,
                      const char* const* names, double time, const int* steps) {
    try {
        need(dir != nullptr && levels != nullptr && fabs != nullptr && names != nullptr, "null argument");
        need(nlevels >= 1, "at least one level");
        need(ncomp >= 1, "at least one component");
        for (int c = 0; c < ncomp; ++c) {
            need(names[c] != nullptr && names[c][0] != '\0', "empty component name");
            need(std::strpbrk(names[c], " \t\n") == nullptr, "component names may not contain whitespace");
        }
        std::vector<LevelOut> out(nlevels);
        for (int l = 0; l < nlevels; ++l) {
            const ae_level_desc& L = levels[l];
            const ae_fab& f = fabs[l];
            need(f.data != nullptr && !f.is_float, "fabs must be FP64 host data");
            need(f.ncomp >= ncomp, "a fab has fewer components than names");
            for (int d = 0; d < 3; ++d) {
                need(L.lo[d] >= 0 && L.hi[d] <= L.domain_cells[d] && L.lo[d] < L.hi[d], "patch outside domain");
                need(f.lo[d] <= L.lo[d] && f.hi[d] >= L.hi[d], "fab does not cover the level's valid box");
                need(L.dx[d] > 0.0, "dx must be positive");
                if (l > 0) need(L.domain_cells[d] == 2 * levels[l - 1].domain_cells[d], "AMR levels must refine by 2");
                out[l].lo[d] = L.lo[d];
                out[l].hi[d] = L.hi[d];
            }
        }
        namespace fs = std::filesystem;
        std::error_code ec;
        fs::create_directories(dir, ec);
        need(!ec, std::string("cannot create ") + dir + ": " + ec.message(), AE_ERR_STATE);

        // Level_<l>/Cell_D_00000 and Cell_H
        for (int l = 0; l < nlevels; ++l) {
            const ae_fab& f = fabs[l];
            LevelOut& o = out[l];
            const std::string ldir = std::string(dir) + "/Level_" + std::to_string(l);
            fs::create_directories(ldir, ec);
            need(!ec, "cannot create " + ldir + ": " + ec.message(), AE_ERR_STATE);
            const long long fx = f.hi[0] - f.lo[0] + 1, fy = f.hi[1] - f.lo[1] + 1, fz = f.hi[2] - f.lo[2] + 1;
            const long long nx = o.hi[0] - o.lo[0] + 1, ny = o.hi[1] - o.lo[1] + 1, nz = o.hi[2] - o.lo[2] + 1;
            const double* base = static_cast<const double*>(f.data);
            std::vector<double> row(nx);
            std::ofstream data(ldir + "/Cell_D_00000", std::ios::binary);
            need(data.good(), "cannot write " + ldir + "/Cell_D_00000", AE_ERR_STATE);
            data << "FAB " << real_descriptor() << box_text(o.lo, o.hi, 1) << ' ' << ncomp << '\n';
            o.mn.assign(ncomp, 0.0);
            o.mx.assign(ncomp, 0.0);
            for (int c = 0; c < ncomp; ++c) {
                double mn = INFINITY, mx = -INFINITY;
                for (long long k = 0; k < nz; ++k)
                    for (long long j = 0; j < ny; ++j) {
                        const long long off = c * fx * fy * fz + (k + o.lo[2] - f.lo[2]) * fx * fy +
                                              (j + o.lo[1] - f.lo[1]) * fx + (o.lo[0] - f.lo[0]);
                        for (long long i = 0; i < nx; ++i) {
                            const double v = base[off + i];
                            if (!std::isfinite(v))
                                need(false, std::string("component ") + names[c] + " is not finite", AE_ERR_NAN);
                            mn = v < mn ? v : mn;
                            mx = v > mx ? v : mx;
                            row[i] = v;
                        }
                        data.write(reinterpret_cast<const char*>(row.data()), sizeof(double) * nx);
                    }
                o.mn[c] = mn;
                o.mx[c] = mx;
            }
            need(data.good(), "write failed: " + ldir + "/Cell_D_00000", AE_ERR_STATE);
            data.close();

            std::ofstream h(ldir + "/Cell_H");
            need(h.good(), "cannot write " + ldir + "/Cell_H", AE_ERR_STATE);
            h << 1 << '\n' << 1 << '\n' << ncomp << '\n' << 0 << '\n';
            h << "(1 0\n" << box_text(o.lo, o.hi, 1) << "\n)\n";
            h << 1 << '\n' << "FabOnDisk: Cell_D_00000 0" << '\n' << '\n';
            h.setf(std::ios::scientific, std::ios::floatfield);
            h.precision(15);
            for (const std::vector<double>* v : {&o.mn, &o.mx}) {
                h << 1 << ',' << ncomp << '\n';
                for (int c = 0; c < ncomp; ++c) h << (*v)[c] << ',';
                h << '\n' << '\n';
            }
            need(h.good(), "write failed: " + ldir + "/Cell_H", AE_ERR_STATE);
        }

        // Header
        std::ofstream h(std::string(dir) + "/Header");
        need(h.good(), std::string("cannot write ") + dir + "/Header", AE_ERR_STATE);
        h.precision(17);
        h << "HyperCLaw-V1.1\n" << ncomp << '\n';
        for (int c = 0; c < ncomp; ++c) h << names[c] << '\n';
        h << 3 << '\n' << time << '\n' << nlevels - 1 << '\n';
        const ae_level_desc& L0 = levels[0];
        for (int d = 0; d < 3; ++d) h << 0.0 << ' ';
        h << '\n';
        for (int d = 0; d < 3; ++d) h << L0.domain_cells[d] * L0.dx[d] << ' ';
        h << '\n';
        for (int l = 0; l + 1 < nlevels; ++l) h << 2 << ' ';
        h << '\n';
        for (int l = 0; l < nlevels; ++l) {
            const int lo[3] = {0, 0, 0};
            const int hi[3] = {levels[l].domain_cells[0] - 1, levels[l].domain_cells[1] - 1,
                               levels[l].domain_cells[2] - 1};
            h << box_text(lo, hi, 0) << ' ';
        }
        h << '\n';
        for (int l = 0; l < nlevels; ++l) h << (steps ? steps[l] : 0) << ' ';
        h << '\n';
        for (int l = 0; l < nlevels; ++l) {
            for (int d = 0; d < 3; ++d) h << levels[l].dx[d] << ' ';
            h << '\n';
        }
        h << 0 << '\n' << "0\n";
        for (int l = 0; l < nlevels; ++l) {
            h << l << ' ' << 1 << ' ' << time << '\n';
            h << (steps ? steps[l] : 0) << '\n';
            // physical extent of the nodal patch: lo * dx .. hi * dx
            for (int d = 0; d < 3; ++d) h << out[l].lo[d] * levels[l].dx[d] << ' ' << out[l].hi[d] * levels[l].dx[d] << '\n';
            h << "Level_" << l << "/Cell" << '\n';
        }
        need(h.good(), std::string("write failed: ") + dir + "/Header", AE_ERR_STATE);
        return AE_OK;
    } catch (const PlotError& e) {
        ae::set_last_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {
        ae::set_last_error(e.what());
        return AE_ERR_STATE;
    }
}

}  // extern "C"
