// csr_chunks (the bottom solve's row chunks) on random row lengths: every chunk holds at most the
// chunk size, a row's chunks cover its nonzeros in order and nothing else, every row has at least
// one chunk.  Exit status 0 when every case holds.
#include <cstdio>
#include <random>
#include <vector>

#include "ae_csr_chunks.h"

int main() {
    std::mt19937 rng(7);
    const int lens[] = {0, 1, 2, 7, 8, 9, 15, 16, 17, 57, 81};
    for (int trial = 0; trial < 4000; ++trial) {
        const int nrows = 1 + (int)(rng() % 60), chunk = 1 + (int)(rng() % 12);
        std::vector<int> rp(1, 0);
        for (int r = 0; r < nrows; ++r) rp.push_back(rp.back() + lens[rng() % 11]);
        std::vector<int> cp, rc;
        ae::csr_chunks(rp, chunk, cp, rc);
        if ((int)rc.size() != nrows + 1 || cp.back() != rp.back() || rc[nrows] + 1 != (int)cp.size()) {
            std::printf("trial %d: bad sizes\n", trial);
            return 1;
        }
        for (int r = 0; r < nrows; ++r) {
            if (rc[r + 1] <= rc[r]) {
                std::printf("trial %d row %d: no chunk\n", trial, r);
                return 1;
            }
            int next = rp[r];
            for (int c = rc[r]; c < rc[r + 1]; ++c) {
                if (cp[c] != next || cp[c + 1] - cp[c] > chunk || cp[c + 1] < cp[c]) {
                    std::printf("trial %d row %d chunk %d: bad bounds\n", trial, r, c);
                    return 1;
                }
                next = cp[c + 1];
            }
            if (next != rp[r + 1]) {
                std::printf("trial %d row %d: nonzeros not covered\n", trial, r);
                return 1;
            }
        }
    }
    std::printf("ok\n");
    return 0;
}
