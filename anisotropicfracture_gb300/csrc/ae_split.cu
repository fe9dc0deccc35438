// Split sweeps on Voronoi (grain-map) levels, FP32 and FP64.
//
// On a grain-map level the per-node sweep spends most of its issue slots on work that few nodes
// need -- the domain-boundary classification, six neighbour grain ids, the grad C branch that
// only the nodes whose stencil straddles a grain boundary take -- and waits on scattered loads.
// A sweep there is split by node:
//
//   k_sweep_tile   every node of the interior box I (not on the domain boundary, inside
//                  grow(valid, 1)).  A block owns a 32 x 8 column of (i, j) and marches in k.
//                  Per plane one elected thread loads, with TMA (cp.async.bulk.tensor) onto an
//                  mbarrier, the x halo tile (three components), b, 1/D and the grain id/mask
//                  tile of the next plane, so every read of the stencil and the update is a
//                  shared-memory load at a fixed offset.  The grain table sits in shared memory.
//                  In FP32 a thread computes the nodes of two neighbouring rows, which share the
//                  loads of the rows between them.  The grad C term is computed only where the
//                  node's mask says a direction's two neighbours lie in different grains.
//   k_*_list       every node of the sweep region outside I (domain-boundary rows, the ghost
//                  ring, nodes outside the domain), through the per-node code.
//
// Three operations are split this way: the damped-Jacobi smoother, the residual r = b - A x and
// Fapply.
//
// Every node is computed by the per-node sweep's own arithmetic: where a direction's neighbours
// share a grain the grad C column is exactly zero, and the interior and grad C expressions are
// written operation for operation as apply_node_grains writes them (the FP32 sums of products in
// the explicitly rounded order of ae_device.cuh), so the split sweep equals the one-pass sweep
// bit for bit.  The list and the id/mask array are built once per level (k_split_mark), when the
// operator is prepared.  TMA needs 16-byte aligned rows: the level arrays' row pitch is a
// multiple of 4 nodes (Geo::px).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <type_traits>

#include "ae_kernels.cuh"
#include "ae_split.h"

namespace ae {

namespace {

constexpr int STX = 32, STY = 8, SNT = STX * STY;
constexpr int SBW = 36;                    // box width: 32 nodes + halo + alignment shift (<= 2)
constexpr int SXR = STY + 2;               // x tile rows (one-node halo in j)
constexpr int SXP = SBW * SXR;             // elements per x component plane tile
constexpr int SVP = SBW * STY;             // elements per b / 1/D / D component tile (no halo)
constexpr int SXRING = 4, SVRING = 2;      // x planes k-1, k, k+1 + the one in flight; b, 1/D, ids
constexpr int kWaitLimit = 1 << 20;        // try_wait polls before a wait is declared failed
#ifndef AE_SPLIT_MIN_BLOCKS
#define AE_SPLIT_MIN_BLOCKS 4
#endif
// FP32: each thread computes the nodes of NPT consecutive rows j .. j + NPT - 1, which share the
// loads of the rows between them in every plane: for two rows, 28 instead of 38 shared-memory
// loads per component
#ifndef AE_SPLIT_NPT32
#define AE_SPLIT_NPT32 2
#endif
#ifndef AE_SPLIT_PAIR_BLOCKS
#define AE_SPLIT_PAIR_BLOCKS 5
#endif

__host__ __device__ constexpr int up128(int b) { return (b + 127) / 128 * 128; }
__host__ __device__ constexpr int up16(int b) { return (b + 15) / 16 * 16; }

// Shared memory of the tiled kernel, in bytes, for elements R: the x ring, the b, 1/D and (FP64
// Jacobi: the reference's update reads D) D rings, the id ring -- every TMA destination on a
// 128-byte boundary -- two mbarriers, the queue of the plane's nodes with a non-zero grad C
// column (count, thread index, main-term f) and the grain table.
template <class R>
struct TL {
    static constexpr int E = (int)sizeof(R);
    static constexpr int XS = up128(3 * SXP * E);  // bytes per x ring slot
    static constexpr int VS = 3 * SVP * E;         // bytes per b / 1/D / D ring slot
    static constexpr int GS = SVP * 4;             // bytes per id ring slot
    static constexpr int oB = SXRING * XS;
    static constexpr int oI = oB + SVRING * VS;
    static constexpr int oD = oI + SVRING * VS;
    static constexpr int oG = oD + (E == 8 ? SVRING * VS : 0);
    static constexpr int oBar = oG + SVRING * GS;
    static constexpr int oQ = oBar + 16;
    static constexpr int oQt = oQ + 16;
    static constexpr int oQf = up16(oQt + 4 * SNT);
    static constexpr int oT = up16(oQf + 3 * SNT * E);
    static constexpr unsigned kX = 3 * SXP * E, kV = 3 * SVP * E, kG = SVP * 4;
    static_assert(VS % 128 == 0 && GS % 128 == 0 && oB % 128 == 0 && oI % 128 == 0 && oD % 128 == 0 &&
                      oG % 128 == 0,
                  "TMA slot alignment");
};
constexpr int kTabSmemMax = 24 * 1024;  // bytes of grain table kept in shared memory

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for a phase of the barrier: false when it did not complete within kWaitLimit polls
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    for (int it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// 4-D tiled TMA load (x, y, z, component) into shared memory, completing on an mbarrier
__device__ __forceinline__ void tma_load4(unsigned dst, const CUtensorMap* map, int x, int y, int z, int c,
                                          unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(c), "r"(bar)
        : "memory");
}

// packed node of a list: offsets from the storage box's low corner, 21 bits each
__device__ __forceinline__ unsigned long long pack_node(int di, int dj, int dk) {
    return (unsigned long long)di | ((unsigned long long)dj << 21) | ((unsigned long long)dk << 42);
}
__device__ __forceinline__ void unpack_node(unsigned long long c, const int lo[3], int& i, int& j, int& k) {
    i = lo[0] + (int)(c & 0x1fffffull);
    j = lo[1] + (int)((c >> 21) & 0x1fffffull);
    k = lo[2] + (int)((c >> 42) & 0x1fffffull);
}

// Mark the nodes of region R (inside the storage box) outside the interior box I, which a list
// kernel computes, and compact them (FILL = false: count only; order within a block follows the
// node order).  With FILL and gidm, also write gidm = gid | mask << 16 for every stored node, mask
// bit d set (nodes of I only) when the two neighbours in direction d lie in different grains: a
// non-zero grad C column.
template <bool FILL>
__global__ void __launch_bounds__(kBlock) k_split_mark(Reg reg, Box3 R, Box3 I, View<const unsigned short> gid,
                                                       unsigned* gidm, unsigned long long* list,
                                                       unsigned long long* count) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    bool f = false;
    unsigned long long code = 0;
    if (t < reg.n) {
        int i, j, k;
        reg_ijk(reg, t, i, j, k);
        const long long o = gid.at(i, j, k);
        if (!in_box(I.lo, I.hi, i, j, k)) {
            f = in_box(R.lo, R.hi, i, j, k);
            if (FILL && gidm) gidm[o] = gid.p[o];
        } else if (FILL && gidm) {
            const long long off[3] = {1, gid.sy, gid.sz};
            unsigned mask = 0;
#pragma unroll
            for (int d = 0; d < 3; ++d) mask |= (gid.p[o + off[d]] != gid.p[o - off[d]]) ? (1u << d) : 0u;
            gidm[o] = (unsigned)gid.p[o] | (mask << 16);
        }
        code = pack_node(i - reg.lo[0], j - reg.lo[1], k - reg.lo[2]);
    }
    __shared__ unsigned wcnt[kBlock / 32];
    __shared__ unsigned long long base;
    const unsigned ball = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) wcnt[w] = __popc(ball);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (int q = 0; q < kBlock / 32; ++q) {
            const unsigned c = wcnt[q];
            wcnt[q] = tot;
            tot += c;
        }
        base = tot ? atomicAdd(count, (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    if (FILL && f) list[base + wcnt[w] + __popc(ball & ((1u << lane) - 1u))] = code;
}

// Tile geometry shared by the host and the kernel: tensor coordinates are offsets from the
// storage box's low corner; the boxes of a tile start at column xa (a multiple of 4, as TMA
// requires), and node i of the tile sits at column sh + 1 + (i - i0).
struct TileGeo {
    Box3 I;        // interior box (absolute node indices)
    int slo[3];    // storage box low corner
    int tiles_x;   // tiles per row of I
    int kz;        // planes per block
    int sh;        // column shift of the tile's first halo column inside the box
};

// One sweep over the interior box I of a grain-map level, A the interior row of
// Elastic<T>::Fapply: OP = SPLIT_JACOBI, the damped-Jacobi update (jacobi_update: the reference's
// form in FP64, x + w (b - A x) / D in the FP32 cycle; Operator.cpp:109-157); OP = SPLIT_RESIDUAL,
// out = b - A x (out may alias b: every node reads only its own b); OP = SPLIT_FAPPLY, out = A x.  The grain table is staged
// in shared memory (TABS, rows padded to 16 bytes) or read through L1.  err: set when a TMA load
// did not complete.  NPT: rows of the tile per thread (1, 2 or 4: the thread's nodes (i, j) ..
// (i, j + NPT - 1) take the x values of rows j - 1 .. j + NPT from one set of loads; each node's
// arithmetic is unchanged).
enum SplitOp { SPLIT_JACOBI = 0, SPLIT_RESIDUAL = 1, SPLIT_FAPPLY = 2 };
template <int M, class R, bool TABS, int OP, int NPT>
__global__ void __launch_bounds__(SNT / NPT, NPT > 1 ? AE_SPLIT_PAIR_BLOCKS : sizeof(R) == 4 ? AE_SPLIT_MIN_BLOCKS : 2)
    k_sweep_tile(const __grid_constant__ CUtensorMap tm_x, const __grid_constant__ CUtensorMap tm_b,
                 const __grid_constant__ CUtensorMap tm_i, const __grid_constant__ CUtensorMap tm_d,
                 const __grid_constant__ CUtensorMap tm_g, SCoef<R> K, TileGeo T, int uniform, long long sy,
                 long long sz, long long sc, const unsigned* __restrict__ gidm_g, const R* __restrict__ tab, int tab_n,
                 R* __restrict__ xo, R omega, int* err) {
    static_assert(NPT == 1 || NPT == 2 || NPT == 4, "one, two or four rows per thread");
    static_assert(STY % NPT == 0, "whole row groups per tile");
    constexpr int NT = SNT / NPT;  // threads per block
    using L = TL<R>;
    constexpr int NC = NCoef<M>::value;
    // grain rows in shared memory padded to whole 16-byte vectors (four coefficients)
    constexpr int NCP = (NC + 3) / 4 * 4;
    constexpr int TS = TABS ? NCP : NC;  // row stride of the table the kernel reads
    constexpr bool D64 = sizeof(R) == 8 && OP == SPLIT_JACOBI;
    extern __shared__ __align__(128) unsigned char smem[];
    auto xslot = [&](int k) { return reinterpret_cast<const R*>(smem + (k & 3) * L::XS); };
    const unsigned* gring = reinterpret_cast<const unsigned*>(smem + L::oG);
    int* qn = reinterpret_cast<int*>(smem + L::oQ);
    int* qtid = reinterpret_cast<int*>(smem + L::oQt);
    R* qf = reinterpret_cast<R*>(smem + L::oQf);
    const R* tb = tab;
    if (TABS) {
        R* ts = reinterpret_cast<R*>(smem + L::oT);
        const int rows = tab_n / NC;
        for (int q = threadIdx.x; q < rows * NCP; q += NT) {
            const int g = q / NCP, c = q - g * NCP;
            ts[q] = c < NC ? __ldg(tab + g * NC + c) : R(0);
        }
        tb = ts;
    }
    const int tx = threadIdx.x % STX, ty = NPT * (threadIdx.x / STX);  // the thread's first row
    const int i0 = T.I.lo[0] + (int)(blockIdx.x % T.tiles_x) * STX, j0 = T.I.lo[1] + (int)(blockIdx.x / T.tiles_x) * STY;
    const int k0 = T.I.lo[2] + (int)blockIdx.y * T.kz;
    const int k1 = min(k0 + T.kz - 1, T.I.hi[2]);
    const int i = i0 + tx, j = j0 + ty;
    const bool act = i <= T.I.hi[0] && j <= T.I.hi[1];
    auto act_n = [&](int n) { return i <= T.I.hi[0] && j + n <= T.I.hi[1]; };  // node n of the thread
    // tensor coordinates of the boxes
    const int xa = i0 - 1 - T.slo[0] - T.sh;
    const int yx = j0 - 1 - T.slo[1], yv = j0 - T.slo[1];
    const unsigned sb = smem_u32(smem);
    const unsigned bar0 = sb + (unsigned)L::oBar;
    const bool leader = threadIdx.x == 0;
    if (leader) {
        *qn = 0;
        mbar_init(bar0, 1);
        mbar_init(bar0 + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto load_x = [&](int k, unsigned bar) {
        tma_load4(sb + (unsigned)((k & 3) * L::XS), &tm_x, xa, yx, k - T.slo[2], 0, bar);
    };
    auto load_v = [&](int k, unsigned bar) {
        const unsigned s = (unsigned)(k & 1);
        if (OP != SPLIT_FAPPLY) tma_load4(sb + (unsigned)L::oB + s * L::VS, &tm_b, xa, yv, k - T.slo[2], 0, bar);
        if (OP == SPLIT_JACOBI) tma_load4(sb + (unsigned)L::oI + s * L::VS, &tm_i, xa, yv, k - T.slo[2], 0, bar);
        if (D64) tma_load4(sb + (unsigned)L::oD + s * L::VS, &tm_d, xa, yv, k - T.slo[2], 0, bar);
        tma_load4(sb + (unsigned)L::oG + s * L::GS, &tm_g, xa, yv, k - T.slo[2], 0, bar);
    };
    constexpr unsigned kVTile = (OP == SPLIT_JACOBI ? (D64 ? 3 : 2) : OP == SPLIT_RESIDUAL ? 1 : 0) * L::kV + L::kG;
    // stage 0: planes k0-1, k0, k0+1 of x and the b, 1/D (D), id tiles of plane k0
    if (leader) {
        mbar_expect_tx(bar0, 3 * L::kX + kVTile);
        load_x(k0 - 1, bar0);
        load_x(k0, bar0);
        load_x(k0 + 1, bar0);
        load_v(k0, bar0);
    }
    const int col = T.sh + 1 + tx;
    const int cx = (ty + 1) * SBW + col;  // this node inside an x component tile
    const int cv = ty * SBW + col;        // ... inside a b / 1/D / id component tile
    long long o = (long long)(i - T.slo[0]) + (long long)(j - T.slo[1]) * sy + (long long)(k0 - T.slo[2]) * sz;
    bool failed = false;
    int last = 0;  // last stage issued
    for (int k = k0; k <= k1; ++k, o += sz) {
        const int s = k - k0;
        // stage s + 1: plane k + 2 of x and the tiles of plane k + 1; their ring slots were last
        // read in iteration k - 1, which the barrier at its end closed
        if (k + 1 <= k1) {
            last = s + 1;
            if (leader) {
                const unsigned bn = bar0 + 8u * (unsigned)((s + 1) & 1);
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                mbar_expect_tx(bn, L::kX + kVTile);
                load_x(k + 2, bn);
                load_v(k + 1, bn);
            }
        }
        const bool ok = mbar_wait(bar0 + 8u * (unsigned)(s & 1), (unsigned)((s >> 1) & 1));
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        const unsigned vs = (unsigned)(k & 1);
        const R* pm = xslot(k - 1) + cx;
        const R* pc = xslot(k) + cx;
        const R* pp = xslot(k + 1) + cx;
        const R* bv = reinterpret_cast<const R*>(smem + L::oB + vs * L::VS) + cv;
        const R* iv = reinterpret_cast<const R*>(smem + L::oI + vs * L::VS) + cv;
        const R* dv = reinterpret_cast<const R*>(smem + L::oD + vs * L::VS) + cv;
        bool queued[NPT];
        R f[NPT][3], xv[NPT][3];
        // the 21 (9, 2, 45) coefficients of a node's grain, then its interior term div(C : grad grad x)
        auto interior = [&](unsigned gw, const R (&bb)[3][3][3], R (&fo)[3]) {
            R a[NCP];
            const R* a0 = tb + (int)(gw & 0xffffu) * TS;
            if (TABS) {
                if (sizeof(R) == 4) {
#pragma unroll
                    for (int q = 0; q < NCP; q += 4) {
                        const float4 v = *reinterpret_cast<const float4*>(a0 + q);
                        a[q] = (R)v.x;
                        a[q + 1] = (R)v.y;
                        a[q + 2] = (R)v.z;
                        a[q + 3] = (R)v.w;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < NCP; q += 2) {
                        const double2 v = *reinterpret_cast<const double2*>(a0 + q);
                        a[q] = (R)v.x;
                        a[q + 1] = (R)v.y;
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < NC; ++q) a[q] = a0[q];
            }
            div_of<M, R>(a, bb, fo);
        };
        if constexpr (NPT == 1) {
            queued[0] = false;
            if (act) {
                const unsigned gw = gring[vs * SVP + cv];
                R bb[3][3][3];
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    const R* um = pm + p * SXP;
                    const R* uc = pc + p * SXP;
                    const R* up = pp + p * SXP;
                    const R c0 = uc[0];
                    xv[0][p] = c0;
                    const R xm = uc[-1], xp = uc[1], ym = uc[-SBW], yp = uc[SBW], zm = um[0], zp = up[0];
                    bb[p][0][0] = (xp - R(2) * c0 + xm) * K.i2[0];
                    bb[p][1][1] = (yp - R(2) * c0 + ym) * K.i2[1];
                    bb[p][2][2] = (zp - R(2) * c0 + zm) * K.i2[2];
                    bb[p][0][1] = (uc[1 + SBW] + uc[-1 - SBW] - uc[1 - SBW] - uc[-1 + SBW]) * K.m01;
                    bb[p][0][2] = (up[1] + um[-1] - um[1] - up[-1]) * K.m02;
                    bb[p][1][2] = (up[SBW] + um[-SBW] - um[SBW] - up[-SBW]) * K.m12;
                    bb[p][1][0] = bb[p][0][1];
                    bb[p][2][0] = bb[p][0][2];
                    bb[p][2][1] = bb[p][1][2];
                }
                interior(gw, bb, f[0]);
                queued[0] = !uniform && (gw >> 16) != 0;
            }
        } else {
#pragma unroll
            for (int n = 0; n < NPT; ++n) queued[n] = false;
            if (act) {
                // per component: plane k at rows j - 1 .. j + NPT and columns i - 1 .. i + 1;
                // planes k -+ 1 at rows j .. j + NPT - 1 (three columns) and rows j - 1, j + NPT
                // (column i).  Row r of these arrays is row j - 1 + r.
                constexpr int NR = NPT + 2;
                R h[NPT][3][6];
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    const R* um = pm + p * SXP;
                    const R* uc = pc + p * SXP;
                    const R* up = pp + p * SXP;
                    R ac[NR][3], am[NR][3], ap[NR][3];
#pragma unroll
                    for (int r = 0; r < NR; ++r)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            ac[r][c] = uc[(r - 1) * SBW + c - 1];
                            const bool need = (r >= 1 && r <= NPT) || c == 1;
                            am[r][c] = need ? um[(r - 1) * SBW + c - 1] : R(0);
                            ap[r][c] = need ? up[(r - 1) * SBW + c - 1] : R(0);
                        }
#pragma unroll
                    for (int n = 0; n < NPT; ++n) {
                        const R c0 = ac[n + 1][1];
                        xv[n][p] = c0;
                        const R xm = ac[n + 1][0], xp = ac[n + 1][2], ym = ac[n][1], yp = ac[n + 2][1];
                        const R zm = am[n + 1][1], zp = ap[n + 1][1];
                        h[n][p][0] = (xp - R(2) * c0 + xm) * K.i2[0];
                        h[n][p][1] = (yp - R(2) * c0 + ym) * K.i2[1];
                        h[n][p][2] = (zp - R(2) * c0 + zm) * K.i2[2];
                        h[n][p][3] = (ac[n + 2][2] + ac[n][0] - ac[n][2] - ac[n + 2][0]) * K.m01;
                        h[n][p][4] = (ap[n + 1][2] + am[n + 1][0] - am[n + 1][2] - ap[n + 1][0]) * K.m02;
                        h[n][p][5] = (ap[n + 2][1] + am[n][1] - am[n + 2][1] - ap[n][1]) * K.m12;
                    }
                }
#pragma unroll
                for (int n = 0; n < NPT; ++n) {
                    if (n > 0 && !act_n(n)) break;
                    const unsigned gw = gring[vs * SVP + cv + n * SBW];
                    R bb[3][3][3];
#pragma unroll
                    for (int p = 0; p < 3; ++p) {
                        bb[p][0][0] = h[n][p][0];
                        bb[p][1][1] = h[n][p][1];
                        bb[p][2][2] = h[n][p][2];
                        bb[p][0][1] = bb[p][1][0] = h[n][p][3];
                        bb[p][0][2] = bb[p][2][0] = h[n][p][4];
                        bb[p][1][2] = bb[p][2][1] = h[n][p][5];
                    }
                    interior(gw, bb, f[n]);
                    queued[n] = !uniform && (gw >> 16) != 0;
                }
            }
        }
        // nodes with a grad C column go to the plane's queue (one shared-memory atomic per warp
        // and row); the others are finished here
#pragma unroll
        for (int n = 0; n < NPT; ++n) {
            const bool an = n == 0 ? act : act && act_n(n);
            const unsigned ball = __ballot_sync(0xffffffffu, queued[n]);
            if (ball) {
                const int lane = threadIdx.x & 31;
                int base = 0;
                if (lane == __ffs(ball) - 1) base = atomicAdd(qn, __popc(ball));
                base = __shfl_sync(0xffffffffu, base, __ffs(ball) - 1);
                if (queued[n]) {
                    const int e = base + __popc(ball & ((1u << lane) - 1u));
                    qtid[e] = (ty + n) * STX + tx;  // the node's place in the tile
                    qf[3 * e] = f[n][0];
                    qf[3 * e + 1] = f[n][1];
                    qf[3 * e + 2] = f[n][2];
                }
            }
            if (an && !queued[n]) {
                const long long on = o + n * sy;
                const int vn = n * SBW;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    if (OP == SPLIT_JACOBI)
                        xo[on + r * sc] = jacobi_update<R>(xv[n][r], f[n][r], bv[vn + r * SVP],
                                                           D64 ? dv[vn + r * SVP] : R(0), iv[vn + r * SVP], omega);
                    else if (OP == SPLIT_RESIDUAL)
                        xo[on + r * sc] = bv[vn + r * SVP] - f[n][r];
                    else
                        xo[on + r * sc] = f[n][r];
                }
            }
        }
        __syncthreads();
        // the queued nodes, one per thread: grad C columns of the directions whose neighbours lie in
        // different grains, then the update
        for (int e = threadIdx.x; e < *qn; e += NT) {
            const int t = qtid[e];
            const int qx = t % STX, qy = t / STX;
            const int qcx = (qy + 1) * SBW + T.sh + 1 + qx, qcv = qy * SBW + T.sh + 1 + qx;
            const long long qo = o + (long long)(qx - tx) + (long long)(qy - ty) * sy;
            const R* qm = xslot(k - 1) + qcx;
            const R* qc = xslot(k) + qcx;
            const R* qp = xslot(k + 1) + qcx;
            R gu[3][3];
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                gu[p][0] = (qc[p * SXP + 1] - qc[p * SXP - 1]) * K.h[0];
                gu[p][1] = (qc[p * SXP + SBW] - qc[p * SXP - SBW]) * K.h[1];
                gu[p][2] = (qp[p * SXP] - qm[p * SXP]) * K.h[2];
            }
            // neighbour ids: x from the tile, y from the tile inside it, the rest from global
            const unsigned* gv = gring + vs * SVP + qcv;
            const unsigned mask = gv[0] >> 16;
            const int gid_n[3][2] = {
                {(int)(gv[1] & 0xffffu), (int)(gv[-1] & 0xffffu)},
                {(int)((qy + 1 < STY ? gv[SBW] : __ldg(gidm_g + qo + sy)) & 0xffffu),
                 (int)((qy > 0 ? gv[-SBW] : __ldg(gidm_g + qo - sy)) & 0xffffu)},
                {(int)(__ldg(gidm_g + qo + sz) & 0xffffu), (int)(__ldg(gidm_g + qo - sz) & 0xffffu)}};
            R colv[3][3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (mask & (1u << d)) {
                    const R* cp = tb + gid_n[d][0] * TS;
                    const R* cm = tb + gid_n[d][1] * TS;
                    gradC_col_f<M, R>([&](int q) { return cp[q] - cm[q]; }, gu, d, colv[d]);
                } else {
                    colv[d][0] = colv[d][1] = colv[d][2] = R(0);
                }
            }
            const R* qb = reinterpret_cast<const R*>(smem + L::oB + vs * L::VS) + qcv;
            const R* qi = reinterpret_cast<const R*>(smem + L::oI + vs * L::VS) + qcv;
            const R* qd = reinterpret_cast<const R*>(smem + L::oD + vs * L::VS) + qcv;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                R fr = qf[3 * e + r];
                fr = gradc_add(fr, colv[0][r], colv[1][r], colv[2][r], K.h);
                if (OP == SPLIT_JACOBI)
                    xo[qo + r * sc] = jacobi_update<R>(qc[r * SXP], fr, qb[r * SVP], D64 ? qd[r * SVP] : R(0),
                                                       qi[r * SVP], omega);
                else if (OP == SPLIT_RESIDUAL)
                    xo[qo + r * sc] = qb[r * SVP] - fr;
                else
                    xo[qo + r * sc] = fr;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) *qn = 0;
    }
    if (failed) {
        if (leader) atomicExch(err, 1);
        // loads still in flight may land: wait (bounded) for the stages issued before leaving
        for (int s = max(last - 1, 0); s <= last; ++s) mbar_wait(bar0 + 8u * (unsigned)(s & 1), (unsigned)((s >> 1) & 1));
    }
}

// FP32: 4 resident blocks (64 registers): at 48 the cubic variant spills
template <int M, class R, bool SAME>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? 4 : 2)
    k_jacobi_list(OpParams P, SCoef<R> K, const unsigned long long* __restrict__ list, long long n, Box3 S,
                  View<const R> C, Grains<R> G, View<const R> invD, View<const R> D, View<const R> xi,
                  View<const R> b, View<R> xo, R omega) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_node(list[t], S.lo, i, j, k);
    jacobi_node<M, R, true, SAME>(P, K, C, G, invD, D, xi, b, xo, omega, i, j, k);
}

// r = b - A x at the listed nodes (the per-node residual, k_residual's arithmetic); r may alias b
template <int M, class R>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? 4 : 2)
    k_residual_list(OpParams P, SCoef<R> K, const unsigned long long* __restrict__ list, long long n, Box3 S,
                    View<const R> C, Grains<R> G, View<const R> x, View<const R> b, View<R> r) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_node(list[t], S.lo, i, j, k);
    R v[3];
    const long long ox = x.at(i, j, k);
    apply_at<M, R, true>(P, K, C, G, x, i, j, k, ox, ox, v);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const R rv = b.p[ox + q * x.sc] - v[q];
        r.p[ox + q * x.sc] = rv;
    }
}

// f = A x at the listed nodes (k_fapply's arithmetic)
template <int M, class R>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? 4 : 2)
    k_fapply_list(OpParams P, SCoef<R> K, const unsigned long long* __restrict__ list, long long n, Box3 S,
                  View<const R> C, Grains<R> G, View<const R> x, View<R> f) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i, j, k;
    unpack_node(list[t], S.lo, i, j, k);
    R v[3];
    const long long ox = x.at(i, j, k);
    apply_at<M, R, true>(P, K, C, G, x, i, j, k, ox, ox, v);
#pragma unroll
    for (int q = 0; q < 3; ++q) f.p[ox + q * x.sc] = v[q];
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is not available");
    return fn;
}

// Tensor map over a level array [comp][k][j][i] (storage box, row pitch px), boxes of
// SBW x rows x 1 x ncomp elements of esize bytes.
CUtensorMap level_tmap(const void* base, const Geo& g, int ncomp, int rows, CUtensorMapDataType type, int esize) {
    const Box3 s = geo_store(g);
    const cuuint64_t nx = (cuuint64_t)(s.hi[0] - s.lo[0] + 1), ny = (cuuint64_t)(s.hi[1] - s.lo[1] + 1),
                     nz = (cuuint64_t)(s.hi[2] - s.lo[2] + 1);
    const cuuint64_t px = (cuuint64_t)g.px;
    const cuuint64_t dims[4] = {nx, ny, nz, (cuuint64_t)ncomp};
    const cuuint64_t e = (cuuint64_t)esize;
    const cuuint64_t strides[3] = {px * e, px * ny * e, px * ny * nz * e};
    const cuuint32_t box[4] = {(cuuint32_t)SBW, (cuuint32_t)rows, 1, (cuuint32_t)ncomp};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUtensorMap m;
    const CUresult r = encode_fn()(&m, type, 4, const_cast<void*>(base), dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return m;
}

template <int M, class R, bool TABS, int OP, int NPT>
void tile_smem_attr(size_t bytes) {
    static size_t set = 0;
    if (bytes > set) {
        AE_CUDA_CHECK(cudaFuncSetAttribute(k_sweep_tile<M, R, TABS, OP, NPT>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        set = bytes;
    }
}

// the tiled kernel of one operation over I; b: the right-hand side, invD: 1/D and D (Jacobi only;
// D read in FP64)
template <class R, int OP>
void launch_tile(const OpParams& P, const SplitList& sl, const Box3& I, const Box3& S, View<const R> x, const R* b,
                 const R* invD, const R* D, R* out, R omega, cudaStream_t st, Grains<R> G, int ngrains, int* err) {
    const SCoef<R> K = make_scoef<R>(P.g);
    const CUtensorMapDataType dt = sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    constexpr int E = (int)sizeof(R);
    dispatch_model<R>(P.model, [&](auto m) {
        constexpr int Mv = decltype(m)::value;
        TileGeo T;
        T.I = I;
        for (int q = 0; q < 3; ++q) T.slo[q] = S.lo[q];
        const int nx = I.hi[0] - I.lo[0] + 1, ny = I.hi[1] - I.lo[1] + 1, nz = I.hi[2] - I.lo[2] + 1;
        T.tiles_x = (nx + STX - 1) / STX;
        const int tiles_y = (ny + STY - 1) / STY;
        T.kz = sl.kz > 0 ? sl.kz : 8;
        // every tile starts 32 nodes after the previous one, so one shift serves all of them: the
        // boxes' first column is then 16-byte aligned (x * E a multiple of 16)
        T.sh = (I.lo[0] - 1 - S.lo[0]) & (16 / E - 1);
        const CUtensorMap tx = level_tmap(x.p, P.g, 3, SXR, dt, E);
        const CUtensorMap tb = level_tmap(b, P.g, 3, STY, dt, E);
        const CUtensorMap ti = level_tmap(invD ? invD : b, P.g, 3, STY, dt, E);
        const CUtensorMap td = level_tmap(D ? D : b, P.g, 3, STY, dt, E);
        const CUtensorMap tg = level_tmap(sl.gidm, P.g, 1, STY, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4);
        const dim3 grid((unsigned)(T.tiles_x * tiles_y), (unsigned)((nz + T.kz - 1) / T.kz));
        const int tab_n = ngrains * NCoef<Mv>::value;
        const int tab_pad = ngrains * ((NCoef<Mv>::value + 3) / 4 * 4);
        const bool tabs = tab_pad * E <= kTabSmemMax;
        const size_t smem = (size_t)TL<R>::oT + (tabs ? (size_t)tab_pad * E : 0);
        constexpr int NPT = E == 4 ? AE_SPLIT_NPT32 : 1;
        if (tabs) {
            tile_smem_attr<Mv, R, true, OP, NPT>(smem);
            k_sweep_tile<Mv, R, true, OP, NPT><<<grid, SNT / NPT, smem, st>>>(
                tx, tb, ti, td, tg, K, T, P.uniform, x.sy, x.sz, x.sc, sl.gidm, G.tab, tab_n, out, omega, err);
        } else {
            tile_smem_attr<Mv, R, false, OP, NPT>(smem);
            k_sweep_tile<Mv, R, false, OP, NPT><<<grid, SNT / NPT, smem, st>>>(
                tx, tb, ti, td, tg, K, T, P.uniform, x.sy, x.sz, x.sc, sl.gidm, G.tab, tab_n, out, omega, err);
        }
        launched();
    });
}

}  // namespace

Box3 split_interior(const Geo& g) {
    Box3 d = geo_domain(g);
    for (int q = 0; q < 3; ++q) { d.lo[q] += 1; d.hi[q] -= 1; }
    return box_isect(box_isect(box_grow(geo_valid(g), 1), d), box_grow(geo_store(g), -1));
}

bool split_supported(const Geo& g) {
    if (g.px <= 0 || g.px % 4 != 0) return false;
    const Box3 S = geo_store(g);
    for (int q = 0; q < 3; ++q)
        if (S.hi[q] - S.lo[q] >= (1 << 21)) return false;
    // the tiles' column shift (TileGeo::sh) must leave the 34 columns of a tile inside the box:
    // 0 on level 0 and on refined patches with 2 ghost layers, 1 or 2 where one touches the domain's
    // low face
    const Box3 I = split_interior(g);
    return ((I.lo[0] - 1 - S.lo[0]) & 3) <= SBW - 34;
}

// count and fill the list of region R \ I (and, with gidm, the id/mask array)
long long build_list(const Reg& reg, const Box3& R, const Box3& I, View<const unsigned short> gid, unsigned* gidm,
                     unsigned long long** list, cudaStream_t st, unsigned long long* scratch_count) {
    AE_CUDA_CHECK(cudaMemsetAsync(scratch_count, 0, sizeof(unsigned long long), st));
    k_split_mark<false><<<nblocks(reg.n), kBlock, 0, st>>>(reg, R, I, gid, nullptr, nullptr, scratch_count);
    launched();
    unsigned long long n = 0;
    AE_CUDA_CHECK(cudaMemcpyAsync(&n, scratch_count, sizeof(n), cudaMemcpyDeviceToHost, st));
    AE_CUDA_CHECK(cudaStreamSynchronize(st));
    *list = nullptr;
    if (n > 0) AE_CUDA_CHECK(cudaMalloc(list, sizeof(unsigned long long) * n));
    if (n > 0 || gidm) {
        AE_CUDA_CHECK(cudaMemsetAsync(scratch_count, 0, sizeof(unsigned long long), st));
        k_split_mark<true><<<nblocks(reg.n), kBlock, 0, st>>>(reg, R, I, gid, gidm, *list, scratch_count);
        launched();
        AE_CUDA_CHECK(cudaStreamSynchronize(st));
    }
    return (long long)n;
}

long long split_build(const Geo& g, View<const unsigned short> gid, SplitList& sl, cudaStream_t st,
                      unsigned long long* scratch_count) {
    if (!split_supported(g)) throw std::runtime_error("split sweep: level layout not supported");
    const Box3 S = geo_store(g);
    const Reg reg = make_reg(S);
    const Box3 I = split_interior(g);
    AE_CUDA_CHECK(cudaMalloc(&sl.gidm, sizeof(unsigned) * (size_t)geo_nn(g)));
    AE_CUDA_CHECK(cudaMemsetAsync(sl.gidm, 0, sizeof(unsigned) * (size_t)geo_nn(g), st));
    // the Jacobi sweep writes the whole storage box, the residual the apply region
    sl.n = build_list(reg, S, I, gid, sl.gidm, &sl.list, st, scratch_count);
    sl.n_r = build_list(reg, geo_apply_region(g), I, gid, nullptr, &sl.list_r, st, scratch_count);
    return sl.n;
}

template <class R>
void launch_jacobi_split(const OpParams& P, const SplitList& sl, View<const R> C, View<const R> invD, View<const R> D,
                         View<const R> xi, View<const R> b, View<R> xo, R omega, cudaStream_t st, Grains<R> G,
                         int ngrains, int* err) {
    const Box3 S = geo_store(P.g);
    const Box3 I = split_interior(P.g);
    const bool same = same_layout(xi, C) && same_layout(xi, invD) && same_layout(xi, D) && same_layout(xi, b) &&
                      same_layout(xi, xo);
    if (!same || !split_supported(P.g)) throw std::runtime_error("split sweep needs the level's internal arrays");
    if (!box_empty(I))
        launch_tile<R, SPLIT_JACOBI>(P, sl, I, S, xi, b.p, invD.p, sizeof(R) == 8 ? D.p : nullptr, xo.p, omega, st, G,
                                     ngrains, err);
    if (sl.n > 0) {
        const SCoef<R> K = make_scoef<R>(P.g);
        dispatch_model<R>(P.model, [&](auto m) {
            k_jacobi_list<decltype(m)::value, R, true><<<(unsigned)((sl.n + kBlock - 1) / kBlock), kBlock, 0, st>>>(
                P, K, sl.list, sl.n, S, C, G, invD, D, xi, b, xo, omega);
        });
        launched();
    }
}

template <class R>
void launch_residual_split(const OpParams& P, const SplitList& sl, View<const R> C, View<const R> x, View<const R> b,
                           View<R> r, cudaStream_t st, Grains<R> G, int ngrains, int* err) {
    const Box3 S = geo_store(P.g);
    const Box3 I = split_interior(P.g);
    const bool same = same_layout(x, C) && same_layout(x, b) && same_layout(x, r);
    if (!same || !split_supported(P.g)) throw std::runtime_error("split sweep needs the level's internal arrays");
    if (!box_empty(I))
        launch_tile<R, SPLIT_RESIDUAL>(P, sl, I, S, x, b.p, nullptr, nullptr, r.p, R(0), st, G, ngrains, err);
    if (sl.n_r > 0) {
        const SCoef<R> K = make_scoef<R>(P.g);
        dispatch_model<R>(P.model, [&](auto m) {
            k_residual_list<decltype(m)::value, R><<<(unsigned)((sl.n_r + kBlock - 1) / kBlock), kBlock, 0, st>>>(
                P, K, sl.list_r, sl.n_r, S, C, G, x, b, r);
        });
        launched();
    }
}

template <class R>
void launch_fapply_split(const OpParams& P, const SplitList& sl, View<const R> C, View<const R> x, View<R> f,
                         cudaStream_t st, Grains<R> G, int ngrains, int* err) {
    const Box3 S = geo_store(P.g);
    const Box3 I = split_interior(P.g);
    const bool same = same_layout(x, C) && same_layout(x, f);
    if (!same || !split_supported(P.g)) throw std::runtime_error("split sweep needs the level's internal arrays");
    if (!box_empty(I)) launch_tile<R, SPLIT_FAPPLY>(P, sl, I, S, x, x.p, nullptr, nullptr, f.p, R(0), st, G, ngrains, err);
    if (sl.n_r > 0) {
        const SCoef<R> K = make_scoef<R>(P.g);
        dispatch_model<R>(P.model, [&](auto m) {
            k_fapply_list<decltype(m)::value, R><<<(unsigned)((sl.n_r + kBlock - 1) / kBlock), kBlock, 0, st>>>(
                P, K, sl.list_r, sl.n_r, S, C, G, x, f);
        });
        launched();
    }
}

template void launch_fapply_split<float>(const OpParams&, const SplitList&, View<const float>, View<const float>,
                                         View<float>, cudaStream_t, Grains<float>, int, int*);
template void launch_fapply_split<double>(const OpParams&, const SplitList&, View<const double>, View<const double>,
                                          View<double>, cudaStream_t, Grains<double>, int, int*);
template void launch_jacobi_split<float>(const OpParams&, const SplitList&, View<const float>, View<const float>,
                                         View<const float>, View<const float>, View<const float>, View<float>, float,
                                         cudaStream_t, Grains<float>, int, int*);
template void launch_jacobi_split<double>(const OpParams&, const SplitList&, View<const double>, View<const double>,
                                          View<const double>, View<const double>, View<const double>, View<double>,
                                          double, cudaStream_t, Grains<double>, int, int*);
template void launch_residual_split<float>(const OpParams&, const SplitList&, View<const float>, View<const float>,
                                           View<const float>, View<float>, cudaStream_t, Grains<float>, int, int*);
template void launch_residual_split<double>(const OpParams&, const SplitList&, View<const double>, View<const double>,
                                            View<const double>, View<double>, cudaStream_t, Grains<double>, int, int*);

}  // namespace ae
