// Split FP32 sweeps on Voronoi (grain-map) levels: a tiled kernel over the interior box plus
// the per-node code over a list of the nodes that need it (see ae_split.cu).
#pragma once
#include <cuda_runtime.h>

#include "ae_launch.h"

namespace ae {

struct SplitList {
    unsigned long long* list = nullptr;  // nodes outside the interior box: packed offsets from the
                                         // storage box's low corner
    long long n = 0;
    unsigned long long* list_r = nullptr;  // the same for the residual's region grow(valid,1) ∩ domain
    long long n_r = 0;
    unsigned* gidm = nullptr;            // per stored node: grain id | grad C directions << 16
    int kz = 0;                          // planes per block of the tiled kernel (0: default 8)
};
// grain ids the split sweep can carry next to its 3-bit direction mask
constexpr int kSplitMaxGrains = 1 << 16;

// Interior box of the tiled kernel: grow(valid, 1) without the domain's boundary nodes, with a
// one-node halo inside the storage box.
Box3 split_interior(const Geo& g);
// whether a level's layout allows the split sweep (row pitch a multiple of 4 nodes)
bool split_supported(const Geo& g);
// Build the node list and the id/mask array of a grain-map level (gid laid out like the level's
// storage, at most kSplitMaxGrains grains); allocates sl.list and sl.gidm with cudaMalloc and
// returns the list's length.  scratch_count: one device counter.  Synchronises the stream.
long long split_build(const Geo& g, View<const unsigned short> gid, SplitList& sl, cudaStream_t st,
                      unsigned long long* scratch_count);
// One damped-Jacobi sweep (FP32 or FP64) of a grain-map level: the tiled interior kernel, then the
// list.  *err is set (device) when a TMA load of the tiled kernel did not complete.
template <class R>
void launch_jacobi_split(const OpParams& P, const SplitList& sl, View<const R> C, View<const R> invD, View<const R> D,
                         View<const R> xi, View<const R> b, View<R> xo, R omega, cudaStream_t st, Grains<R> G,
                         int ngrains, int* err);
// f = A x on the apply region of a grain-map level, the same split (f other than x).
template <class R>
void launch_fapply_split(const OpParams& P, const SplitList& sl, View<const R> C, View<const R> x, View<R> f,
                         cudaStream_t st, Grains<R> G, int ngrains, int* err);
// r = b - A x on the apply region of a grain-map level, the same split; r may alias b.
template <class R>
void launch_residual_split(const OpParams& P, const SplitList& sl, View<const R> C, View<const R> x, View<const R> b,
                           View<R> r, cudaStream_t st, Grains<R> G, int ngrains, int* err);

}  // namespace ae
