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
// and each entry goes straight into a slot of its bin (bins of fixed capacity, the slot
// handed out by the bin's atomic counter).  The pair pass gives each occupied bin to one
// warp, which enumerates the bin's pairs in the order the atomics handed out: the candidate
// list's order can vary from run to run, its content cannot, and nothing computed from it
// depends on the order (contact forces and energies are summed per node in shape-pair
// order, and pair sets are reported sorted).  A pair is examined only in the cell that is the
// minimum corner of the intersection of the two shapes' cell ranges: every pair that
// shares a cell is examined exactly once -- the reference's `tested` set without a set.
// A conservative FP32 AABB test and the local-shape exclusion (sim.cpp:24-39) run before
// the FP64 narrow phase.
//
// Output order.  Candidate pairs are appended to one flat list in chunks staged per warp;
// the narrow phase flags the candidates in contact, a scan places them, and the contact
// list keeps the candidate order.  Per-node force lists are built with counters and sorted by contact
// key (lower shape, higher shape, slot), so every sum is independent of the list order.
//
// No host synchronisation: sizes that can overflow a buffer (a bin's slots, bins,
// candidates, contacts, a shape spanning too many cells) raise a flag instead of writing out of bounds, and the
// host repeats the evaluation with larger buffers (or coarser cells) when it sees one.
#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

constexpr long long kMaxCellsPerShape = 1 << 12;
constexpr float kBoxQuanta = 32000.f;   // quantization steps across the grid extent
constexpr uint32_t kBoxMax = 32767u;    // 15-bit box coordinates
constexpr uint32_t kGuard2 = 0x80008000u;
constexpr uint32_t kShapeBits = 29;     // shape id below, first-cell flags above
constexpr int kPairWarps = kBlock / 32;
constexpr int kPairGrab = 2;             // bins a warp claims at a time (<= 32)
constexpr int kPairRanks = 128;          // bins up to this size are enumerated from registers
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

// First cell of a shape packed for the pair test (10 bits per axis, relative to the grid
// origin).
__device__ __forceinline__ uint32_t pack_cell(int i, int j, int k) {
    return (uint32_t(i) & 1023u) | ((uint32_t(j) & 1023u) << 10) | ((uint32_t(k) & 1023u) << 20);
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

// Membership of the node pair (u, v) in the connected set (sim.cpp:24-39 reads
// connected_.count(pairKey(u, v))): multiplicative hash, linear probing.
__device__ __forceinline__ bool is_connected(const DevTopo& t, int u, int v) {
    const unsigned long long key = u <= v ? ((unsigned long long)u << 32) | uint32_t(v)
                                          : ((unsigned long long)v << 32) | uint32_t(u);
    unsigned long long h = (key * 0x9E3779B97F4A7C15ull) >> t.conn_shift;
    for (unsigned long long probe = 0; probe <= t.conn_mask; probe++) {
        const unsigned long long k = t.conn_hash[h];
        if (k == key) return true;
        if (k == ~0ull) return false;
        h = (h + 1) & t.conn_mask;
    }
    return false;
}

// Local shapes (sim.cpp:24-39): a shared node, or a connected node pair.  Shapes are
// distinct here, so "same beam" cannot occur.  The shared-node half is cheap and decides
// most broad-phase candidates in a lattice; the connected half scans adjacency lists.
__device__ __forceinline__ bool any_connected(const DevTopo& t, int2 a, int2 b) {
    const int an[2] = {a.x, a.y}, bn[2] = {b.x, b.y};
    const int na = a.y >= 0 ? 2 : 1, nb = b.y >= 0 ? 2 : 1;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j)
            if (is_connected(t, an[i], bn[j])) return true;
    return false;
}

// Rest of the test of a candidate pair (sa < sb) that is not a local pair (shared or
// connected nodes, excluded by the pair pass and the filter): FP64 closest points,
// dist < target.  Out of line: few candidates get here, and keeping its registers out of the
// calling loops keeps their occupancy up.
struct PairHit {
    bool hit;
    double s, t, pen;
    d3 n;
};
__device__ __noinline__ PairHit narrow_phase(const DevTopo& t, const PhysParams& p, const double4_32a* x, uint32_t sa,
                                             uint32_t sb) {
    PairHit h;
    h.hit = false;
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

// ---- candidate-list reuse -------------------------------------------------------------------
// The list built with boxes inflated by `skin` holds every pair whose boxes overlap at any
// state where no node has moved farther than skin (Euclidean, so no farther on any axis)
// from its position at the build: each current box lies inside the inflated box of the
// build.  flags[1] = rebuild now.
// A node's displacement is bounded from its FP32 interval [lo, hi] and the stored lower end
// of its interval at the build (one FP32 ulp wide at most), rounding upward.
__global__ void __launch_bounds__(kBlock) k_skin_check(DevTopo t, int N, const float4* __restrict__ xf_lo,
                                                       const float4* __restrict__ xf_hi,
                                                       const float4* __restrict__ xref, float skin,
                                                       uint32_t* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!(skin > 0.f)) {  // no reuse: every evaluation builds, no position to compare
        if (i == 0) atomicOr(flags + 1, 1u);
        return;
    }
    bool moved = false;
    if (i == 0 && flags[2]) moved = true;
    if (i < N && !moved && t.active[t.node_inst[i]]) {
        const float4 l = xf_lo[i], h = xf_hi[i], r = xref[i];
        // per-axis bounds of the move, then its Euclidean length, all rounded upward
        const float ulp = 1.2e-7f * fmaxf(fmaxf(fabsf(r.x), fabsf(r.y)), fabsf(r.z)) + 1e-30f;
        const float dx = __fadd_ru(fmaxf(__fsub_ru(h.x, r.x), __fsub_ru(r.x, l.x)), ulp);
        const float dy = __fadd_ru(fmaxf(__fsub_ru(h.y, r.y), __fsub_ru(r.y, l.y)), ulp);
        const float dz = __fadd_ru(fmaxf(__fsub_ru(h.z, r.z), __fsub_ru(r.z, l.z)), ulp);
        const float d2 = __fadd_ru(__fadd_ru(__fmul_ru(dx, dx), __fmul_ru(dy, dy)), __fmul_ru(dz, dz));
        moved = !(__fsqrt_ru(d2) <= skin);  // also when not finite
    }
    if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(flags + 1, 1u);
}

// After a rebuild: the build positions and the end of a forced rebuild.  A build that
// overflowed a buffer (bins, bin slots, cell span, candidates) left an incomplete list:
// the next evaluation must build again, whatever the skin says, so that the overflow is
// raised again there (the overflow bits are per evaluation; a caller that enqueues several
// evaluations before reading sees only the last one's).
__global__ void __launch_bounds__(kBlock) k_skin_commit(int N, const float4* __restrict__ xf_lo,
                                                        float4* __restrict__ xref, uint32_t* __restrict__ flags) {
    if (!flags[1]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) xref[i] = xf_lo[i];
    if (i == 0)
        flags[2] = (flags[0] & uint32_t(kOverEntries | kOverBins | kOverSpan | kOverCandidates)) ? 1u : 0u;
}

__global__ void __launch_bounds__(kBlock) k_zero_gated(long long n, uint32_t* __restrict__ a,
                                                       const uint32_t* __restrict__ gate) {
    if (!*gate) return;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        a[k] = 0;
}

// ---- kernels -------------------------------------------------------------------------------
// Grid origin, extent and bin numbering from the node bounding box (e.cen[3..8]).
__global__ void k_grid_params(const double* __restrict__ cen, double pad, double cell, long long bin_cap, int* grid,
                              uint32_t* flags, uint32_t* ncand, uint32_t* nentries) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || !flags[1]) return;
    flags[4]++;  // builds since the buffers were allocated
    *ncand = 0;  // the candidate list and entry counts of this build
    nentries[0] = 0;
    nentries[1] = 0;
    nentries[2] = 0;
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
    if (bits <= 10 && (1LL << (3 * bits)) <= bin_cap && (1LL << (3 * bits)) <= 4 * dim[0] * dim[1] * dim[2]) {
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
        // box quantization: kBoxQuanta steps across the grid's extent on each axis
        grid[10 + d] = __float_as_int(float(double(kBoxQuanta) / (double(dim[d]) * cell)));
        grid[13 + d] = __float_as_int(float(double(lo[d]) * cell));
    }
    grid[6] = mode;
    grid[7] = ok ? 1 : 0;
    grid[8] = ok ? int(nb) : 0;
}

// Per-shape bounding box and cell range, in single precision rounded outward: the box
// contains the reference's double-precision box (sim.cpp:154), and cell indices are a
// monotone function of it, so two shapes whose reference boxes overlap share a cell.
// The pair-test record holds the box quantized to 15 bits per axis (floor minus one
// quantum for the low side, ceil plus one for the high side, so the quantized box contains
// the FP32 box whatever the rounding of the scaling) with a guard bit over each high
// value, and the first cell packed as three 10-bit fields.
__global__ void __launch_bounds__(kBlock) k_shape_prep(DevTopo t, PhysParams p, const float4* __restrict__ xf_lo,
                                                       const float4* __restrict__ xf_hi, const int* __restrict__ grid,
                                                       int4* __restrict__ cell_lo, int4* __restrict__ cell_hi,
                                                       uint4* __restrict__ rec, float skin,
                                                       uint32_t* __restrict__ flags) {
    const int S = t.N + t.B;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S || !flags[1]) return;
    const int2 nd = shape_nodes(t, uint32_t(s));
    const int n1 = nd.y >= 0 ? nd.y : nd.x;
    const float4 al = xf_lo[nd.x], ah = xf_hi[nd.x], bl = xf_lo[n1], bh = xf_hi[n1];
    const float pad = __fadd_ru(s < t.N ? p.joint_padf : t.padf[s - t.N], skin);
    const float lo[3] = {__fsub_rd(fminf(al.x, bl.x), pad), __fsub_rd(fminf(al.y, bl.y), pad),
                         __fsub_rd(fminf(al.z, bl.z), pad)};
    const float hi[3] = {__fadd_ru(fmaxf(ah.x, bh.x), pad), __fadd_ru(fmaxf(ah.y, bh.y), pad),
                         __fadd_ru(fmaxf(ah.z, bh.z), pad)};
    const bool finite_box = isfinite(lo[0]) && isfinite(lo[1]) && isfinite(lo[2]) && isfinite(hi[0]) &&
                            isfinite(hi[1]) && isfinite(hi[2]);
    if (!grid[7] || !finite_box || !t.active[t.node_inst[nd.x]]) {  // inactive instances take no part
        cell_lo[s] = make_int4(0, 0, 0, 0);
        cell_hi[s] = make_int4(-1, -1, -1, 0);
        rec[s] = make_uint4(0, 0, 0, 0);
        if (!finite_box) atomicOr(flags, uint32_t(kNonFinite));
        return;
    }
    int c0[3], c1[3];
    uint32_t q0[3], q1[3];
    long long n = 1;
    bool wide = false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float dim = float(grid[3 + d] - 1);
        const float org = float(grid[d]);
        c0[d] = int(fminf(fmaxf(floorf(lo[d] * p.inv_cell_f) - org, 0.f), dim));
        c1[d] = int(fminf(fmaxf(floorf(hi[d] * p.inv_cell_f) - org, 0.f), dim));
        n *= (long long)(c1[d] - c0[d] + 1);
        wide |= c1[d] - c0[d] >= 1024;
        const float qs = __int_as_float(grid[10 + d]), qo = __int_as_float(grid[13 + d]);
        q0[d] = uint32_t(fminf(fmaxf(floorf((lo[d] - qo) * qs) - 1.f, 0.f), float(kBoxMax)));
        q1[d] = uint32_t(fminf(fmaxf(ceilf((hi[d] - qo) * qs) + 1.f, 0.f), float(kBoxMax)));
    }
    if (n > kMaxCellsPerShape || wide) {  // the host coarsens the grid and evaluates again
        atomicOr(flags, uint32_t(kOverSpan));
        n = 0;
        c1[0] = c0[0] - 1;
    }
    cell_lo[s] = make_int4(c0[0], c0[1], c0[2], 0);
    cell_hi[s] = make_int4(c1[0], c1[1], c1[2], 0);
    rec[s] = make_uint4(q0[0] | (q0[1] << 16), (q1[0] | (q1[1] << 16)) | kGuard2, q0[2] | ((q1[2] | 0x8000u) << 16),
                        pack_cell(c0[0], c0[1], c0[2]));
}

// Entries of shape s: one per cell of its range, written straight into the bin's slot that
// the bin counter hands out.  A bin that fills up keeps counting (kOverEntries, and the
// largest count in nentries[1] so the host can size bin_slots).
__global__ void __launch_bounds__(kBlock) k_emit(int S, const int* __restrict__ grid, const int4* __restrict__ cell_lo,
                                                 const int4* __restrict__ cell_hi, int bin_slots,
                                                 uint32_t* __restrict__ bin_count, uint32_t* __restrict__ bin_items,
                                                 uint32_t* __restrict__ nentries, uint32_t* __restrict__ flags) {
    if (!flags[1]) return;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < S) {
        const int4 lo = cell_lo[s], hi = cell_hi[s];
        for (int j = lo.y; j <= hi.y; j++)
            for (int k = lo.z; k <= hi.z; k++)
                for (int i = lo.x; i <= hi.x; i++) {
                    const uint32_t b = bin_of(grid, i, j, k);
                    const uint32_t slot = atomicAdd(&bin_count[b], 1u);
                    if (slot < uint32_t(bin_slots)) {
                        bin_items[size_t(b) * size_t(bin_slots) + slot] = uint32_t(s);
                    } else {
                        atomicOr(flags, uint32_t(kOverEntries));
                        atomicMax(nentries + 1, slot + 1);
                    }
                }
    }
}

// One shape as the pair test sees it inside one bin: id with the first-cell flags in the
// top three bits (bit d set when the shape's first cell on axis d is the bin's cell), the
// quantized box words and the shape's nodes (a joint's node twice).
struct PairRec {
    uint32_t id, w0, w1, w2;
    int n0, n1;
};

__device__ __forceinline__ PairRec load_rec(const DevTopo& t, uint32_t s, const uint4* __restrict__ rec, uint32_t ccp) {
    const uint4 r = rec[s];
    const int2 nd = s < uint32_t(t.N) ? make_int2(int(s), int(s)) : t.ab[s - uint32_t(t.N)];
    // cell spans are below 1024 per axis, so the 10-bit fields compare exactly
    const uint32_t e = ~(r.w ^ ccp);
    const uint32_t f = ((e & 0x3ffu) == 0x3ffu) | (((e & 0xffc00u) == 0xffc00u) << 1) |
                       (((e & 0x3ff00000u) == 0x3ff00000u) << 2);
    return PairRec{s | (f << kShapeBits), r.x, r.y, r.z, nd.x, nd.y};
}

// Broad-phase filter of one pair in its bin: the bin is the first common cell (the OR of
// the flags has all three bits), the quantized boxes overlap, and no node is shared.
// Box overlap by guarded subtraction: with a guard bit over each 15-bit high value,
// (hi | guard) - lo keeps the guard exactly when hi >= lo, two axes per word.
__device__ __forceinline__ bool pair_test(const PairRec& A, const PairRec& B) {
    const bool first = (A.id | B.id) >= 0xe0000000u;
    const uint32_t d1 = B.w1 - A.w0, d2 = A.w1 - B.w0;
    const uint32_t d3 = __byte_perm(B.w2, A.w2, 0x7632) - __byte_perm(A.w2, B.w2, 0x5410);
    const bool box = (d1 & d2 & d3 & kGuard2) == kGuard2;
    const bool share = A.n0 == B.n0 || A.n0 == B.n1 || A.n1 == B.n0 || A.n1 == B.n1;
    return first && box && !share;
}


constexpr uint32_t kIdMask = (1u << kShapeBits) - 1u;

// Appends every lane's hits to the flat candidate list: lane l's hits are the set bits of
// `bits`, bit k standing for its pair with the record partner(k) returns; the lanes' counts
// are placed by a warp scan behind one atomic on ncand.  Past cand_cap the pairs are counted
// but not stored and kOverCandidates is raised.  All lanes of the warp call it.
template <typename Partner>
__device__ __forceinline__ void append_bits(uint32_t bits, uint32_t me, Partner partner, int lane,
                                            long long cand_cap, uint2* __restrict__ cand,
                                            uint32_t* __restrict__ ncand, uint32_t* __restrict__ flags) {
    const uint32_t cnt = uint32_t(__popc(bits));
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) return;  // warp-uniform
    uint32_t base = 0;
    if (lane == 0) {
        base = atomicAdd(ncand, total);
        if ((long long)base + total > cand_cap) atomicOr(flags, uint32_t(kOverCandidates));
    }
    long long at = (long long)__shfl_sync(0xffffffffu, base, 0) + (incl - cnt);
    while (bits) {
        const int k = __ffs(bits) - 1;
        bits &= bits - 1;
        const uint32_t o = partner(k);
        if (at < cand_cap) cand[at] = make_uint2(min(me, o), max(me, o));
        at++;
    }
}

// Every unordered pair of the records at ranks base .. base + m - 1 (m <= 32; lane i holds
// rank base + i in `me`, and all of them are staged in shared memory), by rotation: in
// round k lane i meets rank base + (i + k) mod m, k = 1 .. m/2 (the last round of an even m
// only from the lower half), the partner's record read from shared memory.  Hits are kept as
// one bit per round and appended at the end.
__device__ __forceinline__ void rotate_pairs(const PairRec& me, const uint4* __restrict__ srec,
                                             const int2* __restrict__ snd, int base, int m, int lane,
                                             long long cand_cap, uint2* __restrict__ cand,
                                             uint32_t* __restrict__ ncand, uint32_t* __restrict__ flags) {
    const int half = m >> 1;
    uint32_t bits = 0;
    if (m == 32) {
        // a full group (the common case): partners (lane + k) & 31, every lane active but in
        // the last round, fully unrolled so that the hit bits' shifts are constants
#pragma unroll
        for (int k = 1; k <= 16; k++) {
            const int src = base + ((lane + k) & 31);
            const uint4 r = srec[src];
            const int2 q = snd[src];
            const PairRec o{r.x, r.y, r.z, r.w, q.x, q.y};
            const bool hit = pair_test(me, o) && (k < 16 || lane < 16);
            bits |= uint32_t(hit) << (k - 1);
        }
    } else {
        int src = lane;
        for (int k = 1; k <= half; k++) {
            src = src + 1 < m ? src + 1 : 0;  // (lane + k) mod m for lanes below m
            const uint4 r = srec[base + src];
            const int2 q = snd[base + src];
            const PairRec o{r.x, r.y, r.z, r.w, q.x, q.y};
            const bool active = lane < m && !((m & 1) == 0 && k == half && lane >= half);
            bits |= uint32_t(active && pair_test(me, o)) << (k - 1);
        }
    }
    append_bits(bits, me.id & kIdMask,
                [&](int k) {
                    int j = lane + k + 1;
                    j = j >= m ? j - m : j;
                    return srec[base + j].x & kIdMask;
                },
                lane, cand_cap, cand, ncand, flags);
}

// Candidate pairs of every bin holding two or more shapes.  Warps claim the grid's bins
// kPairGrab at a time (single bins near the end) from a cursor (flags[3]) and skip the empty
// ones (one ballot), so bins of uneven size balance over the grid; they count the build's
// cell entries and occupied bins into nentries[0] and [2] on the way, and append their
// candidate pairs (lower shape, higher shape) to the flat list in warp-sized batches, one
// atomic on ncand per batch, without a counting pass.  The list's length is the number of
// pairs, whatever the order.
// Enumeration inside a bin, entries in bin order:
//   n <= 128  the entries in groups of 32, lane i holding entry 32 g + i of group g and every
//             record staged in shared memory: the pairs inside each group by rotation
//             (rotate_pairs), then each full group against every record of the later groups
//             (one record read by all lanes per round), hits kept as bits over windows of 32
//             partners;
//   larger    the same by groups of 32: each group is staged in turn and then meets every
//             later group, staged 32 records at a time.
__global__ void __launch_bounds__(kBlock, 6) k_bin_pairs(DevTopo t, const int* __restrict__ grid,
                                                      const uint32_t* __restrict__ bin_count, int bin_slots,
                                                      uint32_t* __restrict__ nentries,
                                                      const uint32_t* __restrict__ bin_items,
                                                      const uint4* __restrict__ rec, long long cand_cap,
                                                      uint2* __restrict__ cand, uint32_t* __restrict__ ncand,
                                                      uint32_t* __restrict__ flags) {
    __shared__ uint4 rec_all[kPairWarps][kPairRanks];  // the bin's records, staged for the partner reads
    __shared__ int2 nd_all[kPairWarps][kPairRanks];
    if (!flags[1]) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t nbins = uint32_t(grid[8]);
    uint4* srec = rec_all[w];
    int2* snd = nd_all[w];
    uint32_t* cursor = flags + 3;
    auto stage_rec = [&](const PairRec& r, int rank) {
        srec[rank] = make_uint4(r.id, r.w0, r.w1, r.w2);
        snd[rank] = make_int2(r.n0, r.n1);
    };
    uint32_t entries = 0, occupied = 0;  // this lane's share of the build's counts
    // kPairGrab bins per claim, then single bins for the last 4 per warp of the grid, so that
    // a few heavy bins do not end up queued behind one warp
    const uint32_t tail = 4u * gridDim.x * kPairWarps;
    const uint32_t single_from = nbins > tail ? nbins - tail : 0u;
    uint32_t grab = kPairGrab;  // warp-uniform
    for (;;) {
        uint32_t b0 = 0;
        if (lane == 0) b0 = atomicAdd(cursor, grab);
        b0 = __shfl_sync(0xffffffffu, b0, 0);
        if (b0 >= nbins) break;
        const uint32_t cnt = lane < int(grab) && b0 + lane < nbins ? bin_count[b0 + lane] : 0u;
        if (b0 + grab >= single_from) grab = 1;
        entries += cnt;
        unsigned todo = __ballot_sync(0xffffffffu, cnt >= 2);  // the claimed bins holding pairs
        occupied += lane == 0 ? uint32_t(__popc(todo)) : 0u;
        while (todo) {
            const int j = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t b = b0 + uint32_t(j);
            // a full bin repeats the build (kOverEntries), so clamping only keeps reads in bounds
            const int n = int(min(__shfl_sync(0xffffffffu, cnt, j), uint32_t(bin_slots)));
            const uint32_t* items = bin_items + size_t(b) * size_t(bin_slots);
            const int3 cc = cell_of(grid, b);
            const uint32_t ccp = pack_cell(cc.x, cc.y, cc.z);
            __syncwarp();  // the previous bin's partner reads are done
            if (n <= kPairRanks) {
                // ranks 32 g + lane in group g = 0 .. G-1, all staged in shared memory
                const int G = (n + 31) >> 5;
                for (int g = 0; g < G; g++)
                    if (32 * g + lane < n) stage_rec(load_rec(t, items[32 * g + lane], rec, ccp), 32 * g + lane);
                __syncwarp();
                for (int g = 0; g < G; g++) {
                    const int mg = min(32, n - 32 * g);
                    PairRec me{};
                    if (lane < mg) {
                        const uint4 q = srec[32 * g + lane];
                        const int2 nq = snd[32 * g + lane];
                        me = PairRec{q.x, q.y, q.z, q.w, nq.x, nq.y};
                    }
                    rotate_pairs(me, srec, snd, 32 * g, mg, lane, cand_cap, cand, ncand, flags);  // within group g
                    // group g (full: a later group exists) against the records of the later
                    // groups, 32 partners per window of hit bits
                    for (int r0 = 32 * (g + 1); r0 < n; r0 += 32) {
                        const int rn = min(32, n - r0);
                        uint32_t bits = 0;
                        if (rn == 32) {  // a full window: constant shifts
#pragma unroll
                            for (int k = 0; k < 32; k++) {
                                const uint4 q = srec[r0 + k];
                                const int2 nq = snd[r0 + k];
                                const PairRec o{q.x, q.y, q.z, q.w, nq.x, nq.y};
                                bits |= uint32_t(pair_test(me, o)) << k;
                            }
                        } else {
#pragma unroll 4
                            for (int k = 0; k < rn; k++) {
                                const uint4 q = srec[r0 + k];
                                const int2 nq = snd[r0 + k];
                                const PairRec o{q.x, q.y, q.z, q.w, nq.x, nq.y};
                                bits |= uint32_t(pair_test(me, o)) << k;
                            }
                        }
                        append_bits(bits, me.id & kIdMask, [&](int k) { return srec[r0 + k].x & kIdMask; }, lane,
                                    cand_cap, cand, ncand, flags);
                    }
                }
            } else {
                // large bin: its groups of 32 entries in turn.  Group g is staged in shared
                // ranks 0..31 (lane i holding entry 32 g + i) and its pairs found by
                // rotation; each later group is then staged in ranks 32..63 and met 32
                // partners per window of hit bits.  A group with a later group is full, so
                // every lane holds an entry there.
                const int G = (n + 31) >> 5;
                for (int g = 0; g < G; g++) {
                    const int mg = min(32, n - 32 * g);
                    __syncwarp();  // the previous group's partner reads are done
                    if (lane < mg) stage_rec(load_rec(t, items[32 * g + lane], rec, ccp), lane);
                    __syncwarp();
                    PairRec me{};
                    if (lane < mg) {
                        const uint4 q = srec[lane];
                        const int2 nq = snd[lane];
                        me = PairRec{q.x, q.y, q.z, q.w, nq.x, nq.y};
                    }
                    rotate_pairs(me, srec, snd, 0, mg, lane, cand_cap, cand, ncand, flags);
                    for (int h = g + 1; h < G; h++) {
                        const int rn = min(32, n - 32 * h);
                        __syncwarp();
                        if (lane < rn) stage_rec(load_rec(t, items[32 * h + lane], rec, ccp), 32 + lane);
                        __syncwarp();
                        uint32_t bits = 0;
#pragma unroll 4
                        for (int k = 0; k < rn; k++) {
                            const uint4 q = srec[32 + k];
                            const int2 nq = snd[32 + k];
                            const PairRec o{q.x, q.y, q.z, q.w, nq.x, nq.y};
                            bits |= uint32_t(pair_test(me, o)) << k;
                        }
                        append_bits(bits, me.id & kIdMask, [&](int k) { return srec[32 + k].x & kIdMask; }, lane,
                                    cand_cap, cand, ncand, flags);
                    }
                }
                __syncwarp();
            }
        }
    }
    entries = __reduce_add_sync(0xffffffffu, entries);
    if (lane == 0) {
        if (entries) atomicAdd(nentries, entries);
        if (occupied) atomicAdd(nentries + 2, occupied);
    }
}



// Certified single-precision distance bounds of a candidate pair.  A pair certainly farther
// apart than pad_a + pad_b (>= the reference's target ra + rb + margin) fails the reference's
// test dist < target; a pair certainly closer than the target passes it.
//
// For any unit vector n, the distance between segments p1 + s d1 and p2 + t d2 (s, t in
// [0, 1]) is at least  L(n) = n.(p1 - p2) + min(0, n.d1) - max(0, n.d2):  n.(P - Q) <= |P - Q|
// and the minimum of the linear form over the parameter square is at a corner.  n is the
// unit direction between approximate closest points (FP32, the clamped solution of
// sim.cpp:9-18), which makes the bound nearly tight.  L is evaluated from FP32 endpoints
// rounded down (|error| <= 2^-23 X per coordinate, X the largest endpoint coordinate); the
// rounding of the differences, the three dot products and the sums adds at most about
// 4e-6 X in total, bounded here by 3e-5 X + 1e-9 m, and |n| = 1 up to 1e-6.  A pair that
// cannot be certified (touching segments, non-finite data) goes to the exact test.
struct DistBounds {
    bool far_ok;      // far is a valid lower bound (the closest points are not within 1e-7 m)
    float far;        // certified lower bound on the distance, already less its error
    float near;       // certified upper bound on the distance between points at (s, tt)
    float pad_sum;    // pad_a + pad_b >= the reference's target
    float target_lo;  // <= the reference's target ra + rb + margin
};
__device__ __forceinline__ DistBounds dist_bounds(const DevTopo& t, const PhysParams& p, const float4* __restrict__ xf,
                                                  uint32_t sa, uint32_t sb) {
    const int2 na = sa < uint32_t(t.N) ? make_int2(int(sa), int(sa)) : t.ab[sa - uint32_t(t.N)];
    const int2 nb = sb < uint32_t(t.N) ? make_int2(int(sb), int(sb)) : t.ab[sb - uint32_t(t.N)];
    const float pa = sa < uint32_t(t.N) ? p.joint_padf : t.padf[sa - uint32_t(t.N)];
    const float pb = sb < uint32_t(t.N) ? p.joint_padf : t.padf[sb - uint32_t(t.N)];
    const float4 a0 = xf[na.x], a1 = xf[na.y], b0 = xf[nb.x], b1 = xf[nb.y];
    const float X = fmaxf(fmaxf(fmaxf(fabsf(a0.x), fabsf(a0.y)), fmaxf(fabsf(a0.z), fabsf(a1.x))),
                          fmaxf(fmaxf(fabsf(a1.y), fabsf(a1.z)), fmaxf(fmaxf(fabsf(b0.x), fabsf(b0.y)),
                                                                     fmaxf(fmaxf(fabsf(b0.z), fabsf(b1.x)),
                                                                           fmaxf(fabsf(b1.y), fabsf(b1.z))))));
    const float wx = a0.x - b0.x, wy = a0.y - b0.y, wz = a0.z - b0.z;
    const float ux = a1.x - a0.x, uy = a1.y - a0.y, uz = a1.z - a0.z;
    const float vx = b1.x - b0.x, vy = b1.y - b0.y, vz = b1.z - b0.z;
    // dot products by explicit FMAs (this unit is compiled without contraction, which only
    // the FP64 closest-point arithmetic needs; one rounding per FMA only tightens the bound)
    const float a = fmaf(ux, ux, fmaf(uy, uy, uz * uz)), e = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    const float f = fmaf(vx, wx, fmaf(vy, wy, vz * wz)), c = fmaf(ux, wx, fmaf(uy, wy, uz * wz));
    float s = 0.f, tt = 0.f;
    if (a > 1e-20f && e > 1e-20f) {
        const float b = fmaf(ux, vx, fmaf(uy, vy, uz * vz)), den = fmaf(a, e, -b * b);
        s = den > 1e-12f * a * e ? __saturatef(__fdividef(b * f - c * e, den)) : 0.f;
        tt = __fdividef(b * s + f, e);
        if (tt < 0.f) {
            tt = 0.f;
            s = __saturatef(__fdividef(-c, a));
        } else if (tt > 1.f) {
            tt = 1.f;
            s = __saturatef(__fdividef(b - c, a));
        }
    } else if (a > 1e-20f) {
        s = __saturatef(__fdividef(-c, a));
    } else if (e > 1e-20f) {
        tt = __saturatef(__fdividef(f, e));
    }
    const float nx = fmaf(-vx, tt, fmaf(ux, s, wx)), ny = fmaf(-vy, tt, fmaf(uy, s, wy)),
                nz = fmaf(-vz, tt, fmaf(uz, s, wz));
    const float nn = fmaf(nx, nx, fmaf(ny, ny, nz * nz));
    const float err = 3e-5f * X + 1e-9f;
    DistBounds r;
    r.pad_sum = (pa + pb) * 1.000001f;
    // the pads less one margin exceed the target by at most two FP32 roundings
    r.target_lo = (pa + pb - float(p.contact_margin)) * 0.999999f;
    r.near = isfinite(nn) ? sqrtf(nn) * 1.000001f + err : __int_as_float(0x7f800000);
    r.far_ok = nn > 1e-14f;  // false also when not finite
    r.far = 0.f;
    if (r.far_ok) {
        const float inv = rsqrtf(nn);
        const float mx = nx * inv, my = ny * inv, mz = nz * inv;
        const float nu = fmaf(mx, ux, fmaf(my, uy, mz * uz)), nv = fmaf(mx, vx, fmaf(my, vy, mz * vz));
        const float L = fmaf(mx, wx, fmaf(my, wy, mz * wz)) + fminf(0.f, nu) - fmaxf(0.f, nv);
        r.far = L * 0.999999f - err;
    }
    return r;
}

// -1: certainly no contact; +1: certainly within the target (if not a local pair); 0: only
// the exact test can tell.
__device__ __forceinline__ int distance_class(const DevTopo& t, const PhysParams& p, const float4* __restrict__ xf,
                                              uint32_t sa, uint32_t sb) {
    const DistBounds d = dist_bounds(t, p, xf, sa, sb);
    if (d.near < d.target_lo) return 1;
    return d.far_ok && d.far > d.pad_sum ? -1 : 0;
}

// Candidate filter, once per list build: keeps, in order, the candidates of one
// instance whose certified distance lower bound at the build does not exceed the pads plus
// `reach` (2 skin: every point of a segment whose endpoints move at most skin moves at most
// skin, so two segments close a gap by at most 2 skin) and whose nodes are not connected (sim.cpp:24-39).  Pass 0: keep bits and counts per chunk of 32; pass 1 (after a scan of the
// counts): the kept candidates, compacted.
template <int pass>
__global__ void __launch_bounds__(kBlock) k_filter(DevTopo t, PhysParams p, const float4* __restrict__ xf,
                                                   long long cand_cap, const uint2* __restrict__ cand,
                                                   const uint32_t* __restrict__ ncand, float reach,
                                                   uint32_t* __restrict__ fbits, uint32_t* __restrict__ fcount,
                                                   const uint32_t* __restrict__ foff, uint2* __restrict__ cand2,
                                                   const uint32_t* __restrict__ gate) {
    if (!*gate) return;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t total = uint32_t(min((long long)*ncand, cand_cap));
    const long long nchunk = (total + 31) / 32;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < nchunk; ch += warps) {
        const uint32_t g = uint32_t(ch * 32 + lane);
        if constexpr (pass == 1) {
            if (!fbits[ch]) continue;  // warp-uniform
        }
        if constexpr (pass == 0) {
            bool keep = false;
            if (g < total) {
                const uint2 q = cand[g];
                const int2 na = shape_nodes(t, q.x), nb = shape_nodes(t, q.y);
                if (t.node_inst[na.x] == t.node_inst[nb.x]) {
                    const DistBounds d = dist_bounds(t, p, xf, q.x, q.y);
                    keep = !(d.far_ok && d.far > d.pad_sum + reach);
                    // local pairs (sim.cpp:24-39) never make contact: dropped here, once per
                    // build, so the narrow phase of every evaluation needs no hash lookups
                    if (keep) keep = !any_connected(t, na, nb);
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (lane == 0) {
                fbits[ch] = m;
                fcount[ch] = __popc(m);
            }
        } else {
            const unsigned m = fbits[ch];
            if (m & (1u << lane)) cand2[foff[ch] + __popc(m & below)] = cand[g];
        }
    }
}

// Narrow phase over the filtered list (flat, in order), one candidate per thread.
// Pass 0: test every candidate; one hit bit per candidate and the hit count per chunk of
// 32.  Pass 1 (after a scan of the chunk counts of the list's length): the hits' candidate
// indices, compacted in candidate order (into c_a, overwritten by k_contacts).
template <int pass>
__global__ void __launch_bounds__(kBlock) k_narrow(DevTopo t, PhysParams p, const double4_32a* __restrict__ x,
                                                   const float4* __restrict__ xf, const uint2* __restrict__ cand2,
                                                   const uint32_t* __restrict__ ntotal,
                                                   uint32_t* __restrict__ hitbits, uint32_t* __restrict__ hcount,
                                                   const uint32_t* __restrict__ hoff, ContactBufs c) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t total = *ntotal;
    const long long nchunk = (total + 31) / 32;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < nchunk; ch += warps) {
        const uint32_t g = uint32_t(ch * 32 + lane);
        if constexpr (pass == 1) {
            // the hits' candidates, compacted in order: contact o is candidate hits[o]
            const unsigned m = hitbits[ch];
            if (m & (1u << lane)) {
                const uint32_t o = hoff[ch] + __popc(m & below);
                if (o < uint32_t(c.contact_cap)) c.c_a[o] = g;
            }
        } else {
            bool hit = false;
            if (g < total) {
                const uint2 q = cand2[g];  // not a local pair (k_filter)
                const int cls = distance_class(t, p, xf, q.x, q.y);
                if (cls > 0) hit = true;  // certainly within the target
                else if (cls == 0) hit = narrow_phase(t, p, x, q.x, q.y).hit;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) {
                hitbits[ch] = m;
                hcount[ch] = __popc(m);
            }
        }
    }
}

// The contacts, one hit per thread (dense: the FP64 closest points run with full warps):
// contact o is candidate c_a[o] of the filtered list, written in candidate order.
__global__ void __launch_bounds__(kBlock) k_contacts(DevTopo t, PhysParams p, const double4_32a* __restrict__ x,
                                                     const uint2* __restrict__ cand2,
                                                     const uint32_t* __restrict__ total, ContactBufs c) {
    const long long nc = min((long long)*total, c.contact_cap);
    for (long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x; o < nc; o += (long long)gridDim.x * blockDim.x) {
        const uint2 q = cand2[c.c_a[o]];
        const PairHit h = narrow_phase(t, p, x, q.x, q.y);
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

__device__ __forceinline__ int slot_node(const DevTopo& t, uint32_t shape, int slot) {
    if (shape < uint32_t(t.N)) return slot == 0 ? int(shape) : -1;
    const int2 ab = t.ab[shape - uint32_t(t.N)];
    return slot == 0 ? ab.x : ab.y;
}

// Per-node item counts; a contact list longer than its capacity flags kOverContacts.
__global__ void __launch_bounds__(kBlock) k_node_count(DevTopo t, const uint32_t* __restrict__ total, ContactBufs c) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && (long long)*total > c.contact_cap)
        atomicOr(c.flags, uint32_t(kOverContacts));
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

// Per-node contact lists in canonical order: by the contact's (lower shape, higher shape)
// and the slot, which no two items of one node share.  The gather sums each list in this
// order, so forces do not depend on the order of the contact list.
__device__ __forceinline__ unsigned long long item_key(const ContactBufs& c, uint32_t item) {
    const uint32_t ci = item >> 2;
    return ((unsigned long long)c.c_a[ci] << 31) | ((unsigned long long)c.c_b[ci] << 2) | (item & 3u);
}

// One warp per node with contacts: lists of up to 32 items ranked by shuffles; longer lists
// are queued.
__global__ void __launch_bounds__(kBlock) k_node_sort(int N, ContactBufs c) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long groups = (N + 31) / 32;
    // warp w takes the groups of 32 consecutive nodes w, w + warps, ...; one ballot finds the
    // group's nodes that have contacts (most have none)
    for (long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < groups; g += warps) {
        const long long i0 = g * 32;
        const uint32_t mine = i0 + lane < N ? c.n_count[i0 + lane] : 0u;
        unsigned todo = __ballot_sync(0xffffffffu, mine != 0);
        while (todo) {
            const int b = __ffs(todo) - 1;
            todo &= todo - 1;
            const long long i = i0 + b;
            const uint32_t cnt = __shfl_sync(0xffffffffu, mine, b), s0 = c.n_start[i];
            if (cnt > 32) {
                if (lane == 0) {
                    const uint32_t at = atomicAdd(c.n_long, 1u);
                    c.n_long[1 + at] = uint32_t(i);
                    c.n_cursor[i] = at;  // the fill is done with it
                }
                continue;
            }
            uint32_t item = 0;
            unsigned long long key = ~0ull;
            if (lane < int(cnt)) {
                item = c.n_items[s0 + lane];
                key = item_key(c, item);
            }
            uint32_t rank = 0;
            for (uint32_t q = 0; q < cnt; q++) rank += __shfl_sync(0xffffffffu, key, int(q)) < key;
            if (lane < int(cnt)) c.n_sorted[s0 + rank] = item;
        }
    }
}

constexpr int kLongCap = 2048;  // keys staged in shared memory per long list

// One block per queued node (longer lists): each item's rank is the number of smaller keys.
__global__ void __launch_bounds__(kBlock) k_node_sort_long(ContactBufs c) {
    __shared__ unsigned long long keys[kLongCap];
    const uint32_t nl = c.n_long[0];
    for (uint32_t j = blockIdx.x; j < nl; j += gridDim.x) {
        const uint32_t i = c.n_long[1 + j];
        const uint32_t cnt = c.n_count[i], s0 = c.n_start[i];
        const bool staged = cnt <= uint32_t(kLongCap);
        if (staged)
            for (uint32_t e = threadIdx.x; e < cnt; e += blockDim.x) keys[e] = item_key(c, c.n_items[s0 + e]);
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < cnt; e += blockDim.x) {
            const uint32_t item = c.n_items[s0 + e];
            const unsigned long long k = staged ? keys[e] : item_key(c, item);
            uint32_t r = 0;
            for (uint32_t q = 0; q < cnt; q++) r += (staged ? keys[q] : item_key(c, c.n_items[s0 + q])) < k;
            c.n_sorted[s0 + r] = item;
        }
        __syncthreads();
    }
}

}  // namespace


int contact_pair_blocks(long long shapes) {
    const long long b = shapes / 256;
    return int(b < 1 ? 1 : (b > 8 * 152 ? 8 * 152 : b));
}

void launch_contacts(const DevTopo& t, const PhysParams& p, const EvalBufs& e, ContactBufs& c, double pad,
                     float skin, cudaStream_t s, cudaEvent_t pairs_begin, cudaEvent_t pairs_end) {
    const int S = t.N + t.B;
    const uint32_t* gate = c.flags + 1;
    cudaMemsetAsync(c.flags, 0, 2 * sizeof(uint32_t), s);
    cudaMemsetAsync(c.flags + 3, 0, sizeof(uint32_t), s);  // the pair pass's bin cursor
    (k_skin_check<<<grid_for(t.N), kBlock, 0, s>>>(t, t.N, e.xf_lo, e.xf_hi, c.xref, skin, c.flags), note_launches(1));
    // candidate list (only when rebuilding)
    (k_zero_gated<<<kStreamBlocks, kBlock, 0, s>>>(c.bin_cap + 1, c.bin_count, gate), note_launches(1));
    (k_grid_params<<<1, 32, 0, s>>>(e.cen + 9 * size_t(t.I), pad + double(skin > 0.f ? skin : 0.f), p.broad_cell,
                                    c.bin_cap, c.grid, c.flags, c.ncand, c.nentries),
     note_launches(1));
    (k_shape_prep<<<grid_for(S), kBlock, 0, s>>>(t, p, e.xf_lo, e.xf_hi, c.grid, c.cell_lo, c.cell_hi, c.rec,
                                                 skin > 0.f ? skin : 0.f, c.flags), note_launches(1));
    (k_emit<<<grid_for(S), kBlock, 0, s>>>(S, c.grid, c.cell_lo, c.cell_hi, c.bin_slots, c.bin_count, c.bin_items,
                                           c.nentries, c.flags), note_launches(1));
    // occupied bins, then the candidate list
    if (pairs_begin) cudaEventRecord(pairs_begin, s);
    (k_bin_pairs<<<c.pair_blocks, kBlock, 0, s>>>(t, c.grid, c.bin_count, c.bin_slots, c.nentries, c.bin_items,
                                                c.rec, c.cand_cap, c.cand, c.ncand, c.flags),
     note_launches(1));
    if (pairs_end) cudaEventRecord(pairs_end, s);
    // filtered list (only when rebuilding)
    const long long chunks = c.cand_cap / 32;
    const float reach = skin > 0.f ? 2.0001f * skin : 0.f;  // >= 2 skin
    (k_filter<0><<<kStreamBlocks, kBlock, 0, s>>>(t, p, e.xf_lo, c.cand_cap, c.cand, c.ncand, reach, c.fbits,
                                                c.fcount, c.foff, c.cand2, gate), note_launches(1));
    exclusive_scan_u32(c.fcount, c.foff, chunks, c.scan_tmp, s, gate, c.ncand, 31, 5);
    (k_filter<1><<<kStreamBlocks, kBlock, 0, s>>>(t, p, e.xf_lo, c.cand_cap, c.cand, c.ncand, reach, c.fbits,
                                                c.fcount, c.foff, c.cand2, gate), note_launches(1));
    (k_skin_commit<<<grid_for(t.N), kBlock, 0, s>>>(t.N, e.xf_lo, c.xref, c.flags), note_launches(1));
    // narrow phase over the filtered list: hit bits and counts per chunk, scan, contacts
    const uint32_t* nkept = c.foff + chunks;
    (k_narrow<0><<<kStreamBlocks, kBlock, 0, s>>>(t, p, e.x, e.xf_lo, c.cand2, nkept, c.hitbits, c.hcount, c.hoff, c),
     note_launches(1));
    exclusive_scan_u32(c.hcount, c.hoff, chunks, c.scan_tmp, s, nullptr, nkept, 31, 5);
    (k_narrow<1><<<kStreamBlocks, kBlock, 0, s>>>(t, p, e.x, e.xf_lo, c.cand2, nkept, c.hitbits, c.hcount, c.hoff, c),
     note_launches(1));
    // one warp per block: the few thousand contacts spread over every SM's FP64 pipe
    (k_contacts<<<8 * kStreamBlocks, 32, 0, s>>>(t, p, e.x, c.cand2, c.hoff + chunks, c), note_launches(1));
    const uint32_t* total = c.hoff + chunks;
    cudaMemsetAsync(c.n_count, 0, size_t(t.N + 1) * sizeof(uint32_t), s);
    cudaMemsetAsync(c.n_cursor, 0, size_t(t.N) * sizeof(uint32_t), s);
    (k_node_count<<<kStreamBlocks, kBlock, 0, s>>>(t, total, c), note_launches(1));
    exclusive_scan_u32(c.n_count, c.n_start, t.N, c.scan_tmp, s);
    (k_node_fill<<<kStreamBlocks, kBlock, 0, s>>>(t, total, c), note_launches(1));
    cudaMemsetAsync(c.n_long, 0, sizeof(uint32_t), s);
    (k_node_sort<<<kStreamBlocks, kBlock, 0, s>>>(t.N, c), note_launches(1));
    (k_node_sort_long<<<kStreamBlocks, kBlock, 0, s>>>(c), note_launches(1));
}

}  // namespace mcg
