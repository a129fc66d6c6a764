// contact.cu -- self-contact broad and narrow phase (the reference's MC/src/sim.cpp:144-165
// hash grid and closest-shape penalty), rebuilt as a Morton-ordered uniform grid.
//
// This translation unit is compiled with -fmad=false: the closest-point arithmetic must
// round exactly like the reference so that the set of pairs with dist < target is the
// reference's set bit for bit (positions are bit-identical, see k_state).
//
// Broad phase.  Every shape (N joint spheres, then B beam capsules, as sim.cpp:148-150)
// enters every grid cell its margin-inflated AABB touches (sim.cpp:153-157; same cell size
// and the same floor() cell coordinates).  Cells are numbered by the Morton code of their
// coordinates relative to the grid origin (row-major when the Morton range does not fit),
// and entries are counting-sorted into those bins: one atomic count per entry, a scan over
// bins, one scatter.  The pair pass gives each occupied bin to one warp, which stages the
// bin's shapes in shared memory in ascending shape order, so every result is independent
// of the order the atomics handed out.  A pair is examined only in the cell that is the
// minimum corner of the intersection of the two shapes' cell ranges: every pair that
// shares a cell is examined exactly once -- the reference's `tested` set without a set.
// A conservative FP32 AABB test and the local-shape exclusion (sim.cpp:24-39) run before
// the FP64 narrow phase.
//
// Output order.  Candidate pairs are counted per bin, scanned and written in (bin, pair)
// order; the narrow phase flags the candidates in contact, a scan places them, and the
// contact list keeps the candidate order: the list and every sum over it are
// deterministic.  Per-node force lists are built with counters and sorted by the gather.
//
// No host synchronisation: sizes that can overflow a buffer (entries, bins, contacts, a
// shape spanning too many cells) raise a flag instead of writing out of bounds, and the
// host repeats the evaluation with larger buffers (or coarser cells) when it sees one.
#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

constexpr long long kMaxCellsPerShape = 1 << 12;
constexpr int kWarpCap = 64;            // bins up to this size are staged in shared memory
constexpr int kPairWarps = kBlock / 32;
constexpr int kStreamBlocks = 8 * 152;

__device__ __forceinline__ uint32_t spread3_10(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t compact3_10(uint32_t v) {
    v &= 0x09249249u;
    v = (v ^ (v >> 2)) & 0x030c30c3u;
    v = (v ^ (v >> 4)) & 0x0300f00fu;
    v = (v ^ (v >> 8)) & 0x030000ffu;
    v = (v ^ (v >> 16)) & 0x000003ffu;
    return v;
}

// grid[]: 0-2 origin cell, 3-5 dims, 6 mode (0 Morton, 1 row-major), 7 valid,
//         8 number of bins
__device__ __forceinline__ uint32_t bin_of(const int* g, int i, int j, int k) {
    if (g[6] == 0) return spread3_10(uint32_t(i)) | (spread3_10(uint32_t(j)) << 1) | (spread3_10(uint32_t(k)) << 2);
    return uint32_t((k * g[4] + j) * g[3] + i);
}
__device__ __forceinline__ int3 cell_of(const int* g, uint32_t b) {
    if (g[6] == 0) return make_int3(int(compact3_10(b)), int(compact3_10(b >> 1)), int(compact3_10(b >> 2)));
    const int i = int(b % uint32_t(g[3]));
    const int j = int((b / uint32_t(g[3])) % uint32_t(g[4]));
    const int k = int(b / (uint32_t(g[3]) * uint32_t(g[4])));
    return make_int3(i, j, k);
}

// ---- geometry (sim.cpp:9-22), rounding as the reference --------------------------------
__device__ __forceinline__ double sat(double x) { return clampd(x, 0.0, 1.0); }

struct Closest { double s, t; d3 pa, pb; };

__device__ Closest seg_seg(d3 p1, d3 q1, d3 p2, d3 q2) {
    const d3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
    const double a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    double s = 0, t = 0;
    if (a <= 1e-20 && e <= 1e-20) return {0, 0, p1, p2};
    if (a <= 1e-20) {
        s = 0;
        t = sat(f / e);
    } else {
        const double c = dot(d1, r);
        if (e <= 1e-20) {
            t = 0;
            s = sat(-c / a);
        } else {
            const double b = dot(d1, d2), den = a * e - b * b;
            s = fabs(den) > 1e-20 ? sat((b * f - c * e) / den) : 0;
            t = (b * s + f) / e;
            if (t < 0) {
                t = 0;
                s = sat(-c / a);
            } else if (t > 1) {
                t = 1;
                s = sat((b - c) / a);
            }
        }
    }
    return {s, t, p1 + d1 * s, p2 + d2 * t};
}

struct ShapeRef {
    d3 a, b;
    double r;
    bool capsule;
};

__device__ __forceinline__ int2 shape_nodes(const DevTopo& t, uint32_t s) {
    if (s < uint32_t(t.N)) return make_int2(int(s), -1);
    return t.ab[s - uint32_t(t.N)];
}

__device__ __forceinline__ ShapeRef load_shape(const DevTopo& t, const double4_32a* x, double jr, uint32_t s) {
    ShapeRef sh;
    if (s < uint32_t(t.N)) {
        const double4_32a v = x[s];
        sh.a = sh.b = d3{v.x, v.y, v.z};
        sh.r = jr;
        sh.capsule = false;
    } else {
        const int bi = int(s) - t.N;
        const int2 ab = t.ab[bi];
        const double4_32a va = x[ab.x], vb = x[ab.y];
        sh.a = d3{va.x, va.y, va.z};
        sh.b = d3{vb.x, vb.y, vb.z};
        sh.r = t.radius[bi];
        sh.capsule = true;
    }
    return sh;
}

__device__ Closest shape_closest(const ShapeRef& a, const ShapeRef& b) {
    if (a.capsule && b.capsule) return seg_seg(a.a, a.b, b.a, b.b);
    if (a.capsule && !b.capsule) {
        const d3 d = a.b - a.a;
        const double s = sat(dot(b.a - a.a, d) / fmax(1e-30, len2(d)));
        return {s, 0, a.a + d * s, b.a};
    }
    if (!a.capsule && b.capsule) {
        const d3 d = b.b - b.a;
        const double t = sat(dot(a.a - b.a, d) / fmax(1e-30, len2(d)));
        return {0, t, a.a, b.a + d * t};
    }
    return {0, 0, a.a, b.a};
}

__device__ __forceinline__ bool is_connected(const DevTopo& t, int u, int v) {
    const int k1 = t.conn_start[u + 1];
    for (int k = t.conn_start[u]; k < k1; k++) {
        const int w = t.conn_nbr[k];
        if (w == v) return true;
        if (w > v) return false;
    }
    return false;
}

// Local shapes (sim.cpp:24-39): a shared node, or a connected node pair.  Shapes are
// distinct here, so "same beam" cannot occur.  The shared-node half is cheap and decides
// most broad-phase candidates in a lattice; the connected half scans adjacency lists.
__device__ __forceinline__ bool share_node(int2 a, int2 b) {
    return a.x == b.x || (b.y >= 0 && a.x == b.y) || (a.y >= 0 && (a.y == b.x || (b.y >= 0 && a.y == b.y)));
}
__device__ __forceinline__ bool any_connected(const DevTopo& t, int2 a, int2 b) {
    const int an[2] = {a.x, a.y}, bn[2] = {b.x, b.y};
    const int na = a.y >= 0 ? 2 : 1, nb = b.y >= 0 ? 2 : 1;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j)
            if (is_connected(t, an[i], bn[j])) return true;
    return false;
}

// Rest of the test of a candidate pair (sa < sb) that shares no node: connected-pair
// exclusion, FP64 closest points, dist < target.  Out of line: few candidates get here,
// and keeping its registers out of the pair loop keeps that loop's occupancy up.
struct PairHit {
    bool hit;
    double s, t, pen;
    d3 n;
};
__device__ __noinline__ PairHit narrow_phase(const DevTopo& t, const PhysParams& p, const double4_32a* x, uint32_t sa,
                                             uint32_t sb, int2 na, int2 nb) {
    PairHit h;
    h.hit = false;
    if (any_connected(t, na, nb)) return h;
    const ShapeRef A = load_shape(t, x, p.joint_radius, sa);
    const ShapeRef B = load_shape(t, x, p.joint_radius, sb);
    const Closest cp = shape_closest(A, B);
    const d3 delta = cp.pb - cp.pa;
    const double dist = len(delta), target = A.r + B.r + p.contact_margin;
    if (!(dist < target)) return h;
    h.hit = true;
    h.s = cp.s;
    h.t = cp.t;
    h.pen = target - dist;
    h.n = dist > 1e-12 ? delta * (1.0 / dist) : unit(d3{.37 + .001 * double(int(sa)), .73, -.41 + .001 * double(int(sb))});
    return h;
}

// ---- kernels -------------------------------------------------------------------------------
// Grid origin, extent and bin numbering from the node bounding box (e.cen[3..8]).
__global__ void k_grid_params(const double* __restrict__ cen, double pad, double cell, long long bin_cap, int* grid,
                              uint32_t* flags) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    bool ok = true;
    long long lo[3], dim[3];
    for (int d = 0; d < 3; d++) {
        const double a = floor((cen[3 + d] - pad) / cell) - 1.0;
        const double b = floor((cen[6 + d] + pad) / cell) + 1.0;
        if (!isfinite(a) || !isfinite(b) || fabs(a) > 1e9 || fabs(b) > 1e9) {
            ok = false;
            lo[d] = 0;
            dim[d] = 1;
            continue;
        }
        lo[d] = (long long)a;
        dim[d] = (long long)b - lo[d] + 1;
    }
    int bits = 0;
    for (int d = 0; d < 3; d++)
        while ((1LL << bits) < dim[d]) bits++;
    long long nb;
    int mode;
    if (bits <= 10 && (1LL << (3 * bits)) <= bin_cap) {
        mode = 0;
        nb = 1LL << (3 * bits);
    } else {
        mode = 1;
        nb = dim[0] * dim[1] * dim[2];
    }
    grid[9] = int(nb < (1LL << 30) ? nb : (1LL << 30));
    if (ok && nb > bin_cap) {  // the host enlarges the bins or coarsens the cells
        atomicOr(flags, uint32_t(kOverBins));
        ok = false;
    }
    for (int d = 0; d < 3; d++) {
        grid[d] = int(lo[d]);
        grid[3 + d] = int(dim[d]);
    }
    grid[6] = mode;
    grid[7] = ok ? 1 : 0;
    grid[8] = ok ? int(nb) : 0;
}

// Per-shape bounding box and cell range, in single precision rounded outward: the box
// contains the reference's double-precision box (sim.cpp:154), and cell indices are a
// monotone function of it, so two shapes whose reference boxes overlap share a cell.
__global__ void __launch_bounds__(kBlock) k_shape_prep(DevTopo t, PhysParams p, const float4* __restrict__ xf_lo,
                                                       const float4* __restrict__ xf_hi, const int* __restrict__ grid,
                                                       int4* __restrict__ cell_lo, int4* __restrict__ cell_hi,
                                                       float4* __restrict__ bb_lo, float4* __restrict__ bb_hi,
                                                       uint32_t* __restrict__ count, uint32_t* __restrict__ flags) {
    const int S = t.N + t.B;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int2 nd = shape_nodes(t, uint32_t(s));
    const int n1 = nd.y >= 0 ? nd.y : nd.x;
    const float4 al = xf_lo[nd.x], ah = xf_hi[nd.x], bl = xf_lo[n1], bh = xf_hi[n1];
    const float pad = s < t.N ? p.joint_padf : t.padf[s - t.N];
    const float lo[3] = {__fsub_rd(fminf(al.x, bl.x), pad), __fsub_rd(fminf(al.y, bl.y), pad),
                         __fsub_rd(fminf(al.z, bl.z), pad)};
    const float hi[3] = {__fadd_ru(fmaxf(ah.x, bh.x), pad), __fadd_ru(fmaxf(ah.y, bh.y), pad),
                         __fadd_ru(fmaxf(ah.z, bh.z), pad)};
    bb_lo[s] = make_float4(lo[0], lo[1], lo[2], 0.f);
    bb_hi[s] = make_float4(hi[0], hi[1], hi[2], 0.f);
    const bool finite_box = isfinite(lo[0]) && isfinite(lo[1]) && isfinite(lo[2]) && isfinite(hi[0]) &&
                            isfinite(hi[1]) && isfinite(hi[2]);
    if (!grid[7] || !finite_box) {
        count[s] = 0;
        cell_lo[s] = make_int4(0, 0, 0, 0);
        cell_hi[s] = make_int4(-1, -1, -1, 0);
        if (!finite_box) atomicOr(flags, uint32_t(kNonFinite));
        return;
    }
    int c0[3], c1[3];
    long long n = 1;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float dim = float(grid[3 + d] - 1);
        const float org = float(grid[d]);
        c0[d] = int(fminf(fmaxf(floorf(lo[d] * p.inv_cell_f) - org, 0.f), dim));
        c1[d] = int(fminf(fmaxf(floorf(hi[d] * p.inv_cell_f) - org, 0.f), dim));
        n *= (long long)(c1[d] - c0[d] + 1);
    }
    if (n > kMaxCellsPerShape) {  // the host coarsens the grid and evaluates again
        atomicOr(flags, uint32_t(kOverSpan));
        n = 0;
        c1[0] = c0[0] - 1;
    }
    count[s] = uint32_t(n);
    cell_lo[s] = make_int4(c0[0], c0[1], c0[2], 0);
    cell_hi[s] = make_int4(c1[0], c1[1], c1[2], 0);
}

// Entries of shape s: bin key and rank inside the bin (bin_count counts them).
__global__ void __launch_bounds__(kBlock) k_emit(int S, const int* __restrict__ grid, const int4* __restrict__ cell_lo,
                                                 const int4* __restrict__ cell_hi, const uint32_t* __restrict__ offset,
                                                 long long cap, uint32_t* __restrict__ ekey,
                                                 uint32_t* __restrict__ erank, uint32_t* __restrict__ bin_count,
                                                 uint32_t* __restrict__ flags) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    if ((long long)offset[S] > cap) {
        if (s == 0) atomicOr(flags, uint32_t(kOverEntries));
        return;
    }
    const int4 lo = cell_lo[s], hi = cell_hi[s];
    uint32_t o = offset[s];
    for (int j = lo.y; j <= hi.y; j++)
        for (int k = lo.z; k <= hi.z; k++)
            for (int i = lo.x; i <= hi.x; i++) {
                const uint32_t b = bin_of(grid, i, j, k);
                ekey[o] = b;
                erank[o] = atomicAdd(&bin_count[b], 1u);
                o++;
            }
}

__global__ void __launch_bounds__(kBlock) k_scatter(int S, const uint32_t* __restrict__ offset, long long cap,
                                                    const uint32_t* __restrict__ ekey,
                                                    const uint32_t* __restrict__ erank,
                                                    const uint32_t* __restrict__ bin_start,
                                                    uint32_t* __restrict__ sorted) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S || (long long)offset[S] > cap) return;
    for (uint32_t o = offset[s]; o < offset[s + 1]; o++) sorted[bin_start[ekey[o]] + erank[o]] = uint32_t(s);
}

// Row and column of pair p in the strict upper triangle of an n x n matrix, pairs (i, j),
// i < j, numbered row by row.
__device__ __forceinline__ void pair_index(int n, int p, int& i, int& j) {
    const float fn = float(2 * n - 1);
    int r = int((fn - sqrtf(fmaxf(fn * fn - 8.f * float(p), 0.f))) * 0.5f);
    r = max(0, min(r, n - 2));
    while (r > 0 && r * (2 * n - r - 1) / 2 > p) r--;
    while (r < n - 2 && (r + 1) * (2 * n - r - 2) / 2 <= p) r++;
    i = r;
    j = p - r * (2 * n - r - 1) / 2 + r + 1;
}

struct BinShape {
    uint32_t s;
    int lx, ly, lz;
    float bx0, by0, bz0, bx1, by1, bz1;
    int n0, n1;
};

__device__ __forceinline__ BinShape load_bin_shape(const DevTopo& t, uint32_t v, const int4* __restrict__ cell_lo,
                                                   const float4* __restrict__ bb_lo, const float4* __restrict__ bb_hi) {
    const int4 l = cell_lo[v];
    const float4 a = bb_lo[v], z = bb_hi[v];
    const int2 nd = shape_nodes(t, v);
    return BinShape{v, l.x, l.y, l.z, a.x, a.y, a.z, z.x, z.y, z.z, nd.x, nd.y};
}

// Broad-phase filter of one pair in cell cc: first common cell, AABB overlap, no shared
// node.  Survivors become narrow-phase candidates.
__device__ __forceinline__ bool candidate(const BinShape& A, const BinShape& B, int3 cc) {
    return max(A.lx, B.lx) == cc.x && max(A.ly, B.ly) == cc.y && max(A.lz, B.lz) == cc.z &&
           !(A.bx0 > B.bx1 || B.bx0 > A.bx1 || A.by0 > B.by1 || B.by0 > A.by1 || A.bz0 > B.bz1 || B.bz0 > A.bz1) &&
           !share_node(make_int2(A.n0, A.n1), make_int2(B.n0, B.n1));
}

__device__ __forceinline__ BinShape shfl_shape(const BinShape& v, int src) {
    BinShape o;
    o.s = __shfl_sync(0xffffffffu, v.s, src);
    o.lx = __shfl_sync(0xffffffffu, v.lx, src);
    o.ly = __shfl_sync(0xffffffffu, v.ly, src);
    o.lz = __shfl_sync(0xffffffffu, v.lz, src);
    o.bx0 = __shfl_sync(0xffffffffu, v.bx0, src);
    o.by0 = __shfl_sync(0xffffffffu, v.by0, src);
    o.bz0 = __shfl_sync(0xffffffffu, v.bz0, src);
    o.bx1 = __shfl_sync(0xffffffffu, v.bx1, src);
    o.by1 = __shfl_sync(0xffffffffu, v.by1, src);
    o.bz1 = __shfl_sync(0xffffffffu, v.bz1, src);
    o.n0 = __shfl_sync(0xffffffffu, v.n0, src);
    o.n1 = __shfl_sync(0xffffffffu, v.n1, src);
    return o;
}

// Candidate pairs of every occupied bin.  Warp w of the fixed grid takes the occupied bins
// occ[w], occ[w + W], ... in order and appends their candidate pairs (lower shape, higher
// shape) to its own region cand[w R .. (w + 1) R), so the candidate list -- regions in warp
// order, each in bin and enumeration order -- is deterministic without a second counting
// pass.  A region that fills up flags kOverCandidates; wcount[w] keeps the full count so the
// host can size R.  Enumeration inside a bin:
//   n <= 32  the bin's shapes are sorted across the warp's lanes (bitonic, by shape id)
//            and every unordered pair is visited by rotation: in round k lane i meets
//            lane (i + k) mod n, k = 1 .. n/2 (the last round of an even n only from the
//            lower half), the partner's data arriving by register shuffles;
//   n <= 64  the sorted shapes are staged in shared memory and the pairs enumerated by
//            index;
//   larger   sorted through a scratch copy, pairs read from global memory.
__global__ void __launch_bounds__(kBlock) k_bin_pairs(DevTopo t, const int* __restrict__ grid,
                                                      const uint32_t* __restrict__ bin_count,
                                                      const uint32_t* __restrict__ bin_start,
                                                      const uint32_t* __restrict__ occ, const uint32_t* __restrict__ nocc_p,
                                                      const uint32_t* __restrict__ sorted, uint32_t* __restrict__ sorted2,
                                                      const int4* __restrict__ cell_lo, const float4* __restrict__ bb_lo,
                                                      const float4* __restrict__ bb_hi, int region,
                                                      uint2* __restrict__ cand, uint32_t* __restrict__ wcount,
                                                      uint32_t* __restrict__ flags) {
    __shared__ BinShape sh[kPairWarps][kWarpCap];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    const long long nocc = *nocc_p;
    const long long gw = (long long)blockIdx.x * kPairWarps + w;
    const long long warps = (long long)gridDim.x * kPairWarps;
    uint2* mine = cand + gw * region;
    uint32_t out = 0;
    auto emit = [&](bool hit, uint32_t sa, uint32_t sb) {
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const uint32_t pos = out + __popc(m & below);
            if (pos < uint32_t(region)) mine[pos] = make_uint2(sa, sb);
        }
        out += __popc(m);
    };
    for (long long j = gw; j < nocc; j += warps) {
        const uint32_t b = occ[j];
        const int n = int(bin_count[b]);
        const uint32_t start = bin_start[b];
        const int3 cc = cell_of(grid, b);
        if (n <= 32) {
            uint32_t v = lane < n ? sorted[start + lane] : 0xffffffffu;
            for (int k = 2; k <= 32; k <<= 1)  // bitonic sort, ascending
                for (int j = k >> 1; j > 0; j >>= 1) {
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, v, j);
                    const bool up = (lane & k) == 0, lower = (lane & j) == 0;
                    v = (lower == up) ? min(v, o) : max(v, o);
                }
            BinShape me{};
            if (lane < n) me = load_bin_shape(t, v, cell_lo, bb_lo, bb_hi);
            const int half = n >> 1;
            for (int k = 1; k <= half; k++) {
                const int src = lane < n ? (lane + k < n ? lane + k : lane + k - n) : lane;
                const BinShape o = shfl_shape(me, src);
                const bool active = lane < n && !((n & 1) == 0 && k == half && lane >= half);
                const bool hit = active && candidate(me, o, cc);
                emit(hit, min(me.s, o.s), max(me.s, o.s));
            }
        } else if (n <= kWarpCap) {
            const uint32_t v0 = sorted[start + lane];
            const uint32_t v1 = lane + 32 < n ? sorted[start + 32 + lane] : 0xffffffffu;
            int r0 = 0, r1 = 0;
            for (int q = 0; q < 32; q++) {
                const uint32_t u0 = __shfl_sync(0xffffffffu, v0, q), u1 = __shfl_sync(0xffffffffu, v1, q);
                r0 += (u0 < v0) + (u1 < v0);
                r1 += (u0 < v1) + (u1 < v1);
            }
            __syncwarp();
            sh[w][r0] = load_bin_shape(t, v0, cell_lo, bb_lo, bb_hi);
            if (v1 != 0xffffffffu) sh[w][r1] = load_bin_shape(t, v1, cell_lo, bb_lo, bb_hi);
            __syncwarp();
            const int P = n * (n - 1) / 2;
            for (int base = 0; base < P; base += 32) {
                const int pidx = base + lane;
                bool hit = false;
                uint32_t sa = 0, sb = 0;
                if (pidx < P) {
                    int i, j;
                    pair_index(n, pidx, i, j);
                    hit = candidate(sh[w][i], sh[w][j], cc);
                    sa = sh[w][i].s;
                    sb = sh[w][j].s;
                }
                emit(hit, sa, sb);
            }
            __syncwarp();
        } else {
            // large bin: ascending order through a scratch copy, pairs from global memory
            for (int e = lane; e < n; e += 32) {
                const uint32_t v = sorted[start + e];
                int r = 0;
                for (int q = 0; q < n; q++) r += sorted[start + q] < v;
                sorted2[start + r] = v;
            }
            __syncwarp();
            const long long P = (long long)n * (n - 1) / 2;
            int i = 0;
            long long row_end = n - 1;  // pairs of rows 0..i end here
            for (long long base = 0; base < P; base += 32) {
                const long long pidx = base + lane;
                bool hit = false;
                uint32_t sa = 0, sb = 0;
                if (pidx < P) {
                    while (pidx >= row_end) {  // rows advance monotonically with base
                        i++;
                        row_end += n - 1 - i;
                    }
                    const int j = int(pidx - (row_end - (n - 1 - i))) + i + 1;
                    const BinShape A = load_bin_shape(t, sorted2[start + i], cell_lo, bb_lo, bb_hi);
                    const BinShape B = load_bin_shape(t, sorted2[start + j], cell_lo, bb_lo, bb_hi);
                    hit = candidate(A, B, cc);
                    sa = A.s;
                    sb = B.s;
                }
                emit(hit, sa, sb);
            }
            __syncwarp();
        }
    }
    if (lane == 0) {
        wcount[gw] = out;
        if (out > uint32_t(region)) atomicOr(flags, uint32_t(kOverCandidates));
    }
}

// Occupied bins (two or more entries), in bin order: flags, then a scan, then this.
__global__ void __launch_bounds__(kBlock) k_occ_flags(long long nb_cap, const int* __restrict__ grid,
                                                      const uint32_t* __restrict__ bin_count, uint32_t* __restrict__ f) {
    const long long nb = grid[8];
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < nb_cap; b += (long long)gridDim.x * blockDim.x)
        f[b] = (b < nb && bin_count[b] >= 2) ? 1u : 0u;
}
__global__ void __launch_bounds__(kBlock) k_occ_write(long long nb_cap, const uint32_t* __restrict__ f,
                                                      const uint32_t* __restrict__ off, uint32_t* __restrict__ occ) {
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < nb_cap; b += (long long)gridDim.x * blockDim.x)
        if (f[b]) occ[off[b]] = uint32_t(b);
}

constexpr int kContactPartBlocks = 128;

// Narrow phase over the candidate regions, one warp per region (the region's owner in
// k_bin_pairs).  Pass 0: test every candidate, keep one hit bit per candidate and the hit
// count per region.  Pass 1 (after a scan of the counts): test the hits again and write
// them as contacts, in region and candidate order.
__global__ void __launch_bounds__(kBlock) k_narrow(DevTopo t, PhysParams p, const double4_32a* __restrict__ x,
                                                   int region, const uint2* __restrict__ cand,
                                                   const uint32_t* __restrict__ wcount, int pass,
                                                   uint32_t* __restrict__ hitbits, uint32_t* __restrict__ hcount,
                                                   const uint32_t* __restrict__ hoff, ContactBufs c) {
    const int lane = threadIdx.x & 31;
    const long long gw = (long long)blockIdx.x * kPairWarps + (threadIdx.x >> 5);
    const uint32_t nc = min(wcount[gw], uint32_t(region));
    const uint2* mine = cand + gw * region;
    uint32_t* bits = hitbits + gw * (region / 32);
    const unsigned below = (1u << lane) - 1u;
    uint32_t pos = pass ? hoff[gw] : 0;
    for (uint32_t base = 0; base < nc; base += 32) {
        const uint32_t i = base + lane;
        if (pass) {
            const unsigned m = bits[base / 32];
            if (m & (1u << lane)) {
                const uint2 q = mine[i];
                const PairHit h = narrow_phase(t, p, x, q.x, q.y, shape_nodes(t, q.x), shape_nodes(t, q.y));
                const uint32_t o = pos + __popc(m & below);
                if (o < uint32_t(c.contact_cap)) {
                    c.c_a[o] = q.x;
                    c.c_b[o] = q.y;
                    c.c_s[o] = h.s;
                    c.c_t[o] = h.t;
                    c.c_n[3 * size_t(o)] = h.n.x;
                    c.c_n[3 * size_t(o) + 1] = h.n.y;
                    c.c_n[3 * size_t(o) + 2] = h.n.z;
                    c.c_pen[o] = h.pen;
                }
            }
            pos += __popc(m);
        } else {
            bool hit = false;
            if (i < nc) {
                const uint2 q = mine[i];
                hit = narrow_phase(t, p, x, q.x, q.y, shape_nodes(t, q.x), shape_nodes(t, q.y)).hit;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) bits[base / 32] = m;
            pos += __popc(m);
        }
    }
    if (!pass && lane == 0) hcount[gw] = pos;
}

// Fixed-partition reduction over the contact list: energy, max penetration, count.
__global__ void __launch_bounds__(kBlock) k_contact_reduce(const uint32_t* __restrict__ total, long long cap, double k,
                                                           const double* __restrict__ pen, double* __restrict__ part,
                                                           uint32_t* flags) {
    __shared__ double sm[2 * (kBlock / 32)];
    __shared__ double smx[kBlock / 32];
    const long long nc_all = *total;
    if (nc_all > cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(flags, uint32_t(kOverContacts));
    const long long nc = nc_all > cap ? cap : nc_all;
    double acc[2] = {0, 0};
    double m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x) {
        const double pp = pen[i];
        acc[0] += .5 * k * pp * pp;
        acc[1] += 1;
        m = fmax(m, pp);
    }
    block_sum<2>(acc, sm);
    m = block_max(m, smx);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = acc[0];
        part[3 * blockIdx.x + 1] = m;
        part[3 * blockIdx.x + 2] = acc[1];
    }
}

__device__ __forceinline__ int slot_node(const DevTopo& t, uint32_t shape, int slot) {
    if (shape < uint32_t(t.N)) return slot == 0 ? int(shape) : -1;
    const int2 ab = t.ab[shape - uint32_t(t.N)];
    return slot == 0 ? ab.x : ab.y;
}

__global__ void __launch_bounds__(kBlock) k_node_count(DevTopo t, const uint32_t* __restrict__ total, ContactBufs c) {
    const long long nc = min((long long)*total, c.contact_cap);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x)
        for (int slot = 0; slot < 4; slot++) {
            const int node = slot_node(t, slot < 2 ? c.c_a[i] : c.c_b[i], slot & 1);
            if (node >= 0) atomicAdd(&c.n_count[node], 1u);
        }
}

__global__ void __launch_bounds__(kBlock) k_node_fill(DevTopo t, const uint32_t* __restrict__ total, ContactBufs c) {
    const long long nc = min((long long)*total, c.contact_cap);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long long)gridDim.x * blockDim.x)
        for (int slot = 0; slot < 4; slot++) {
            const int node = slot_node(t, slot < 2 ? c.c_a[i] : c.c_b[i], slot & 1);
            if (node < 0) continue;
            const uint32_t pos = atomicAdd(&c.n_cursor[node], 1u);
            c.n_items[c.n_start[node] + pos] = (uint32_t(i) << 2) | uint32_t(slot);
        }
}

}  // namespace

int contact_part_blocks(long long) { return kContactPartBlocks; }

int contact_pair_blocks(long long shapes) {
    const long long b = shapes / 256;
    return int(b < 1 ? 1 : (b > 8 * 152 ? 8 * 152 : b));
}

void launch_contacts(const DevTopo& t, const PhysParams& p, const EvalBufs& e, ContactBufs& c, double pad,
                     cudaStream_t s) {
    const int S = t.N + t.B;
    cudaMemsetAsync(c.flags, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(c.bin_count, 0, size_t(c.bin_cap + 1) * sizeof(uint32_t), s);
    (k_grid_params<<<1, 32, 0, s>>>(e.cen, pad, p.broad_cell, c.bin_cap, c.grid, c.flags), note_launches(1));
    (k_shape_prep<<<grid_for(S), kBlock, 0, s>>>(t, p, e.xf_lo, e.xf_hi, c.grid, c.cell_lo, c.cell_hi, c.bb_lo,
                                                 c.bb_hi, c.count, c.flags), note_launches(1));
    exclusive_scan_u32(c.count, c.offset, S, c.scan_tmp, s);
    (k_emit<<<grid_for(S), kBlock, 0, s>>>(S, c.grid, c.cell_lo, c.cell_hi, c.offset, c.entry_cap, c.ekey, c.erank,
                                           c.bin_count, c.flags), note_launches(1));
    exclusive_scan_u32(c.bin_count, c.bin_start, c.bin_cap, c.scan_tmp, s);
    (k_scatter<<<grid_for(S), kBlock, 0, s>>>(S, c.offset, c.entry_cap, c.ekey, c.erank, c.bin_start, c.sorted),
     note_launches(1));
    // occupied bins, then candidates into per-warp regions
    (k_occ_flags<<<kStreamBlocks, kBlock, 0, s>>>(c.bin_cap, c.grid, c.bin_count, c.bcount), note_launches(1));
    exclusive_scan_u32(c.bcount, c.boffset, c.bin_cap, c.scan_tmp, s);
    (k_occ_write<<<kStreamBlocks, kBlock, 0, s>>>(c.bin_cap, c.bcount, c.boffset, c.occ), note_launches(1));
    const uint32_t* nocc = c.boffset + c.bin_cap;
    const int W = c.pair_blocks * kPairWarps;
    (k_bin_pairs<<<c.pair_blocks, kBlock, 0, s>>>(t, c.grid, c.bin_count, c.bin_start, c.occ, nocc, c.sorted, c.sorted2,
                                                c.cell_lo, c.bb_lo, c.bb_hi, c.region, c.cand, c.wcount, c.flags),
     note_launches(1));
    // narrow phase: hit bits and counts per region, scan, contacts
    (k_narrow<<<c.pair_blocks, kBlock, 0, s>>>(t, p, e.x, c.region, c.cand, c.wcount, 0, c.hitbits, c.hcount,
                                               c.hoff, c), note_launches(1));
    exclusive_scan_u32(c.hcount, c.hoff, W, c.scan_tmp, s);
    (k_narrow<<<c.pair_blocks, kBlock, 0, s>>>(t, p, e.x, c.region, c.cand, c.wcount, 1, c.hitbits, c.hcount,
                                               c.hoff, c), note_launches(1));
    const uint32_t* total = c.hoff + W;
    (k_contact_reduce<<<kContactPartBlocks, kBlock, 0, s>>>(total, c.contact_cap, p.contact_k, c.c_pen, c.part, c.flags),
     note_launches(1));
    cudaMemsetAsync(c.n_count, 0, size_t(t.N + 1) * sizeof(uint32_t), s);
    cudaMemsetAsync(c.n_cursor, 0, size_t(t.N) * sizeof(uint32_t), s);
    (k_node_count<<<kStreamBlocks, kBlock, 0, s>>>(t, total, c), note_launches(1));
    exclusive_scan_u32(c.n_count, c.n_start, t.N, c.scan_tmp, s);
    (k_node_fill<<<kStreamBlocks, kBlock, 0, s>>>(t, total, c), note_launches(1));
}

}  // namespace mcg
