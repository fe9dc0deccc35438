// Prints Linear::Cubic::Define of the C++ shim for a few Euler angles (no GPU calls).
#include <cstdio>

#include "alamo_elastic.H"

int main() {
    const double ang[3][3] = {{0.3, 0.2, 0.1}, {1.0, 2.0, 0.5}, {0.0, 1.5707963267948966, 0.0}};
    for (auto& a : ang) {
        Model::Solid::Linear::Cubic c;
        c.Define(1.68, 1.21, 0.75, a[0], a[1], a[2]);
        for (int q = 0; q < 21; ++q) std::printf("%.17g%c", c.ddw[q], q == 20 ? '\n' : ' ');
    }
    return 0;
}
