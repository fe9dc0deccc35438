// Row chunks of an assembled sparse matrix, for the bottom solve's sparse product (host code).
#pragma once
#include <algorithm>
#include <vector>

namespace ae {

// Cut every row of a CSR matrix into chunks of at most `chunk` consecutive nonzeros; a row without
// nonzeros gets one empty chunk.  Chunk c covers the nonzeros [cptr[c], cptr[c + 1]) (cptr has one
// entry per chunk plus the end, nnz); the chunks of row r are [rch[r], rch[r + 1]).
inline void csr_chunks(const std::vector<int>& rowptr, int chunk, std::vector<int>& cptr, std::vector<int>& rch) {
    const size_t nrows = rowptr.empty() ? 0 : rowptr.size() - 1;
    cptr.clear();
    rch.assign(nrows + 1, 0);
    for (size_t r = 0; r < nrows; ++r) {
        rch[r] = (int)cptr.size();
        int q = rowptr[r];
        do {
            cptr.push_back(q);
            q = std::min(q + chunk, rowptr[r + 1]);
        } while (q < rowptr[r + 1]);
    }
    rch[nrows] = (int)cptr.size();
    cptr.push_back(nrows ? rowptr[nrows] : 0);
}

}  // namespace ae
