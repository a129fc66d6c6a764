// contact.cu -- self-contact broad and narrow phase (the reference's
// MC/src/sim.cpp:144-165 hash grid + closest-shape penalty), rebuilt as a Morton-ordered
// uniform grid over sorted (cell, shape) entries.
//
// This translation unit is compiled with -fmad=false: the closest-point arithmetic must
// round exactly like the reference so that the set of pairs with dist < target is the
// reference's set bit for bit (positions are bit-identical, see k_state).
//
// Broad phase.  Every shape (N joint spheres, then B beam capsules, as sim.cpp:148-150)
// enters every grid cell its margin-inflated AABB touches (sim.cpp:153-157, same cell size
// and the same floor() cell coordinates).  Entries are keyed by the Morton code of the
// cell relative to the grid origin and radix-sorted (stable, so a cell's entries stay in
// ascending shape order).  A pair is examined only in the cell that is the minimum corner
// of the intersection of the two shapes' cell ranges: every pair that shares a cell is
// examined exactly once, which is the reference's `tested` set without a hash set.
// A conservative FP32 AABB test and the local-shape exclusion (sim.cpp:24-39) run before
// the FP64 narrow phase.
//
// Output order.  Contacts are written in (cell, first shape, second shape) order through
// a count/scan/emit pass pair, so the contact list -- and every sum over it -- is
// deterministic.  Per-node force lists are built with counters and sorted by the gather.
#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

constexpr long long kMaxCellsPerShape = 1 << 16;

__device__ __forceinline__ uint64_t spread3(uint32_t v) {  // 21 bits -> every third bit
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffULL;
    x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    x = (x | (x << 2)) & 0x1249249249249249ULL;
    return x;
}
__device__ __forceinline__ uint32_t compact3(uint64_t x) {
    x &= 0x1249249249249249ULL;
    x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ULL;
    x = (x ^ (x >> 4)) & 0x100f00f00f00f00fULL;
    x = (x ^ (x >> 8)) & 0x1f0000ff0000ffULL;
    x = (x ^ (x >> 16)) & 0x1f00000000ffffULL;
    x = (x ^ (x >> 32)) & 0x1fffffULL;
    return uint32_t(x);
}
__device__ __forceinline__ uint64_t morton(uint32_t i, uint32_t j, uint32_t k) {
    return spread3(i) | (spread3(j) << 1) | (spread3(k) << 2);
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
    int n0, n1;
    bool capsule;
};

__device__ __forceinline__ ShapeRef load_shape(const DevTopo& t, const double4_32a* x, double jr, uint32_t s) {
    ShapeRef sh;
    if (s < uint32_t(t.N)) {
        const double4_32a v = x[s];
        sh.a = sh.b = d3{v.x, v.y, v.z};
        sh.r = jr;
        sh.n0 = int(s);
        sh.n1 = -1;
        sh.capsule = false;
    } else {
        const int bi = int(s) - t.N;
        const int2 ab = t.ab[bi];
        const double4_32a va = x[ab.x], vb = x[ab.y];
        sh.a = d3{va.x, va.y, va.z};
        sh.b = d3{vb.x, vb.y, vb.z};
        sh.r = t.radius[bi];
        sh.n0 = ab.x;
        sh.n1 = ab.y;
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

// Same beam, a shared node, or a connected node pair (sim.cpp:24-39).
__device__ __forceinline__ bool excluded(const DevTopo& t, const ShapeRef& a, const ShapeRef& b) {
    const int an[2] = {a.n0, a.n1}, bn[2] = {b.n0, b.n1};
    const int na = a.capsule ? 2 : 1, nb = b.capsule ? 2 : 1;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            if (an[i] == bn[j]) return true;
            if (is_connected(t, an[i], bn[j])) return true;
        }
    return false;
}

// ---- kernels -------------------------------------------------------------------------------
// Grid origin, extent and Morton width from the node bounding box (e.cen[3..8]).
__global__ void k_grid_params(const double* __restrict__ cen, double pad, double cell, int* grid) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    bool ok = true;
    long long lo[3], dim[3];
    int bits = 1;
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
        if (dim[d] > (1LL << 21)) dim[d] = 1LL << 21;
        while ((1LL << bits) < dim[d]) bits++;
    }
    for (int d = 0; d < 3; d++) {
        grid[d] = int(lo[d]);
        grid[3 + d] = int(dim[d]);
    }
    grid[6] = bits;
    grid[7] = ok ? 1 : 0;
}

__global__ void __launch_bounds__(kBlock) k_shape_prep(DevTopo t, PhysParams p, const double4_32a* __restrict__ x,
                                                       const int* __restrict__ grid, int4* __restrict__ cell_lo,
                                                       int4* __restrict__ cell_hi, float4* __restrict__ bb_lo,
                                                       float4* __restrict__ bb_hi, uint32_t* __restrict__ count,
                                                       uint32_t* __restrict__ flags) {
    const int S = t.N + t.B;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const ShapeRef sh = load_shape(t, x, p.joint_radius, uint32_t(s));
    const double pad = sh.r + p.contact_margin;
    const d3 lo{fmin(sh.a.x, sh.b.x) - pad, fmin(sh.a.y, sh.b.y) - pad, fmin(sh.a.z, sh.b.z) - pad};
    const d3 hi{fmax(sh.a.x, sh.b.x) + pad, fmax(sh.a.y, sh.b.y) + pad, fmax(sh.a.z, sh.b.z) + pad};
    bb_lo[s] = make_float4(__double2float_rd(lo.x), __double2float_rd(lo.y), __double2float_rd(lo.z), 0.f);
    bb_hi[s] = make_float4(__double2float_ru(hi.x), __double2float_ru(hi.y), __double2float_ru(hi.z), 0.f);
    const bool finite_box = isfinite(lo.x) && isfinite(lo.y) && isfinite(lo.z) && isfinite(hi.x) &&
                            isfinite(hi.y) && isfinite(hi.z);
    if (!grid[7] || !finite_box) {
        count[s] = 0;
        cell_lo[s] = make_int4(0, 0, 0, 0);
        cell_hi[s] = make_int4(-1, -1, -1, 0);
        if (!finite_box) atomicOr(flags, 2u);
        return;
    }
    const double cl[3] = {lo.x, lo.y, lo.z}, ch[3] = {hi.x, hi.y, hi.z};
    int c0[3], c1[3];
    long long n = 1;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double dim = double(grid[3 + d]) - 1.0;
        const double a = clampd(floor(cl[d] / p.broad_cell) - double(grid[d]), 0.0, dim);
        const double b = clampd(floor(ch[d] / p.broad_cell) - double(grid[d]), 0.0, dim);
        c0[d] = int(a);
        c1[d] = int(b);
        n *= (long long)(c1[d] - c0[d] + 1);
    }
    if (n > kMaxCellsPerShape) {  // the host coarsens the grid and runs this again
        atomicOr(flags, 1u);
        n = 0;
    }
    count[s] = uint32_t(n);
    cell_lo[s] = make_int4(c0[0], c0[1], c0[2], 0);
    cell_hi[s] = make_int4(c1[0], c1[1], c1[2], 0);
}

__global__ void __launch_bounds__(kBlock) k_emit(int S, const int4* __restrict__ cell_lo,
                                                 const int4* __restrict__ cell_hi,
                                                 const uint32_t* __restrict__ offset, uint64_t* __restrict__ keys,
                                                 uint32_t* __restrict__ vals) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int4 lo = cell_lo[s], hi = cell_hi[s];
    uint32_t o = offset[s];
    const uint32_t end = offset[s + 1];
    for (int j = lo.y; j <= hi.y; j++)
        for (int k = lo.z; k <= hi.z; k++)
            for (int i = lo.x; i <= hi.x; i++) {
                if (o >= end) return;
                keys[o] = morton(uint32_t(i), uint32_t(j), uint32_t(k));
                vals[o] = uint32_t(s);
                o++;
            }
}

// Pass 1 (emit == 0): contacts per entry into ccount.  Pass 2 (emit != 0): contacts written
// at coffset[e] in partner order.
__global__ void __launch_bounds__(kBlock) k_pairs(DevTopo t, PhysParams p, const double4_32a* __restrict__ x,
                                                  long long n, const uint64_t* __restrict__ keys,
                                                  const uint32_t* __restrict__ vals,
                                                  const int4* __restrict__ cell_lo, const float4* __restrict__ bb_lo,
                                                  const float4* __restrict__ bb_hi, int emit,
                                                  uint32_t* __restrict__ ccount, const uint32_t* __restrict__ coffset,
                                                  ContactBufs c) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    if (emit && ccount[e] == 0) return;
    const uint64_t key = keys[e];
    if (e + 1 >= n || keys[e + 1] != key) {
        if (!emit) ccount[e] = 0;
        return;
    }
    const uint32_t sa = vals[e];
    const int ci = int(compact3(key)), cj = int(compact3(key >> 1)), ck = int(compact3(key >> 2));
    const int4 la = cell_lo[sa];
    const float4 alo = bb_lo[sa], ahi = bb_hi[sa];
    const ShapeRef A = load_shape(t, x, p.joint_radius, sa);
    uint32_t found = 0;
    uint32_t out = emit ? coffset[e] : 0;
    for (long long f = e + 1; f < n && keys[f] == key; f++) {
        const uint32_t sb = vals[f];
        const int4 lb = cell_lo[sb];
        if (max(la.x, lb.x) != ci || max(la.y, lb.y) != cj || max(la.z, lb.z) != ck) continue;
        const float4 blo = bb_lo[sb], bhi = bb_hi[sb];
        if (alo.x > bhi.x || blo.x > ahi.x || alo.y > bhi.y || blo.y > ahi.y || alo.z > bhi.z || blo.z > ahi.z)
            continue;
        const ShapeRef Bs = load_shape(t, x, p.joint_radius, sb);
        if (excluded(t, A, Bs)) continue;
        const Closest cp = shape_closest(A, Bs);
        const d3 delta = cp.pb - cp.pa;
        const double dist = len(delta), target = A.r + Bs.r + p.contact_margin;
        if (!(dist < target)) continue;
        if (emit) {
            const d3 nn = dist > 1e-12 ? delta * (1.0 / dist)
                                       : unit(d3{.37 + .001 * double(int(sa)), .73, -.41 + .001 * double(int(sb))});
            c.c_a[out] = sa;
            c.c_b[out] = sb;
            c.c_s[out] = cp.s;
            c.c_t[out] = cp.t;
            c.c_n[3 * size_t(out)] = nn.x;
            c.c_n[3 * size_t(out) + 1] = nn.y;
            c.c_n[3 * size_t(out) + 2] = nn.z;
            c.c_pen[out] = target - dist;
            out++;
        }
        found++;
    }
    if (!emit) ccount[e] = found;
}

constexpr int kContactPartBlocks = 128;

// Fixed-partition reduction over the contact list: energy, max penetration, count.
__global__ void __launch_bounds__(kBlock) k_contact_reduce(long long nc, double k, const double* __restrict__ pen,
                                                           double* __restrict__ part) {
    __shared__ double sm[2 * (kBlock / 32)];
    __shared__ double smx[kBlock / 32];
    double acc[2] = {0, 0};
    double m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc;
         i += (long long)gridDim.x * blockDim.x) {
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

__global__ void __launch_bounds__(kBlock) k_node_count(DevTopo t, long long nc, ContactBufs c) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    for (int slot = 0; slot < 4; slot++) {
        const int node = slot_node(t, slot < 2 ? c.c_a[i] : c.c_b[i], slot & 1);
        if (node >= 0) atomicAdd(&c.n_count[node], 1u);
    }
}

__global__ void __launch_bounds__(kBlock) k_node_fill(DevTopo t, long long nc, ContactBufs c) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    for (int slot = 0; slot < 4; slot++) {
        const int node = slot_node(t, slot < 2 ? c.c_a[i] : c.c_b[i], slot & 1);
        if (node < 0) continue;
        const uint32_t pos = atomicAdd(&c.n_cursor[node], 1u);
        c.n_items[c.n_start[node] + pos] = (uint32_t(i) << 2) | uint32_t(slot);
    }
}

}  // namespace

int contact_part_blocks(long long) { return kContactPartBlocks; }

void contact_shapes(const DevTopo& t, const PhysParams& p, const EvalBufs& e, ContactBufs& c, double pad,
                    cudaStream_t s) {
    const int S = t.N + t.B;
    cudaMemsetAsync(c.dev_total, 0, 4 * sizeof(uint32_t), s);
    (k_grid_params<<<1, 32, 0, s>>>(e.cen, pad, p.broad_cell, c.grid), note_launches(1));
    (k_shape_prep<<<grid_for(S), kBlock, 0, s>>>(t, p, e.x, c.grid, c.cell_lo, c.cell_hi, c.bb_lo, c.bb_hi, c.count,
                                                c.dev_total + 2), note_launches(1));
    exclusive_scan_u32(c.count, c.offset, S, c.sort_tmp, s);
}

int contact_sort_and_count(const DevTopo& t, const PhysParams& p, const EvalBufs& e, ContactBufs& c,
                           long long entries, int key_bits, cudaStream_t s) {
    const int S = t.N + t.B;
    (k_emit<<<grid_for(S), kBlock, 0, s>>>(S, c.cell_lo, c.cell_hi, c.offset, c.keys[0], c.vals[0]), note_launches(1));
    const int res = radix_sort_u64(c.keys, c.vals, entries, key_bits, c.sort_tmp, nullptr, s);
    if (entries > 0) {
        (k_pairs<<<grid_for(entries), kBlock, 0, s>>>(t, p, e.x, entries, c.keys[res], c.vals[res], c.cell_lo, c.bb_lo,
                                                     c.bb_hi, 0, c.ccount, c.coffset, c), note_launches(1));
    }
    exclusive_scan_u32(c.ccount, c.coffset, entries, c.sort_tmp, s);
    return res;
}

void contact_emit(const DevTopo& t, const PhysParams& p, const EvalBufs& e, ContactBufs& c, long long entries,
                  int res, long long ncontacts, cudaStream_t s) {
    if (entries > 0 && ncontacts > 0)
        (k_pairs<<<grid_for(entries), kBlock, 0, s>>>(t, p, e.x, entries, c.keys[res], c.vals[res], c.cell_lo, c.bb_lo,
                                                     c.bb_hi, 1, c.ccount, c.coffset, c), note_launches(1));
    (k_contact_reduce<<<kContactPartBlocks, kBlock, 0, s>>>(ncontacts, p.contact_k, c.c_pen, c.part), note_launches(1));
    cudaMemsetAsync(c.n_count, 0, size_t(t.N + 1) * sizeof(uint32_t), s);
    cudaMemsetAsync(c.n_cursor, 0, size_t(t.N) * sizeof(uint32_t), s);
    if (ncontacts > 0) (k_node_count<<<grid_for(ncontacts), kBlock, 0, s>>>(t, ncontacts, c), note_launches(1));
    exclusive_scan_u32(c.n_count, c.n_start, t.N, c.sort_tmp, s);
    if (ncontacts > 0) (k_node_fill<<<grid_for(ncontacts), kBlock, 0, s>>>(t, ncontacts, c), note_launches(1));
}

}  // namespace mcg
