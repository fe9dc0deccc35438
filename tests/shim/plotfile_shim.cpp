// Writes a two-level nodal plotfile through alamo::WritePlotFile (host data only, no GPU) for
// tests/test_shim.py: level 0 is 8^3 cells, level 1 refines the central half; the fields are
// u_p(i, j, k) = 100 p + i + 10 j + 0.5 k on each level's nodes, ghosts included.
#include <cstdio>
#include <vector>

#include "alamo_elastic.H"

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::vector<alamo::Level> levels = {{{8, 8, 8}, {0, 0, 0}, {8, 8, 8}, {0.125, 0.125, 0.125}},
                                        {{16, 16, 16}, {4, 4, 4}, {12, 12, 12}, {0.0625, 0.0625, 0.0625}}};
    const int ng[2] = {0, 2};
    std::vector<std::vector<double>> store(2);
    std::vector<alamo::Fab> fabs;
    for (int l = 0; l < 2; ++l) {
        std::array<int, 3> lo, hi;
        for (int d = 0; d < 3; ++d) { lo[d] = levels[l].lo[d] - ng[l]; hi[d] = levels[l].hi[d] + ng[l]; }
        alamo::Fab f(nullptr, lo, hi, 3);
        store[l].resize(3 * f.npts());
        f.data = store[l].data();
        for (int p = 0; p < 3; ++p)
            for (int k = lo[2]; k <= hi[2]; ++k)
                for (int j = lo[1]; j <= hi[1]; ++j)
                    for (int i = lo[0]; i <= hi[0]; ++i) f(i, j, k, p) = 100.0 * p + i + 10.0 * j + 0.5 * k;
        fabs.push_back(f);
    }
    try {
        alamo::WritePlotFile(argv[1], 0, levels, fabs, {"disp001", "disp002", "disp003"}, 0.0);
        std::printf("%s\n", alamo::WritePlotFile(argv[1], 3, levels, fabs, {"disp001", "disp002", "disp003"}, 1.5).c_str());
    } catch (const alamo::Error& e) {
        std::printf("error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
