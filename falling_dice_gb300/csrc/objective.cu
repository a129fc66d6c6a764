// objective.cu -- FP64 kernels of the energy/gradient evaluation
// (the reference's Simulator::state + objective, MC/src/sim.cpp:136-172).
//
//   k_state    per node: z -> current position/orientation; block partial sums of x
//   k_center   one block: mean position for the centering term
//   k_beams    per beam: axial/shear/bending/torsion energy with return mapping,
//              the two end 6-vectors of its gradient, optional trial state
//   k_gather   per node: deterministic CSR sum of the incident beams' end vectors in
//              ascending beam order, gravity, centering, self-contact contributions
//              (sorted), platen contact; packs, scales and locks the 6-DOF gradient
//   k_finalize one block: fixed-order totals, diagnostics, non-finite guard
#include "common.cuh"
#include "kernels.h"

namespace mcg {

static_assert(kMapBlock == kBlock, "mapped blocks are launched with kBlock threads");

int nb_nodes(int N) { return int(grid_for(N)); }
int nb_beams(int B) { return int(grid_for(B)); }

// ---- node state: MC/src/sim.cpp:136 -------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_state(DevTopo t, PhysParams p, const double* __restrict__ z,
                                                  const double* __restrict__ bx, const double* __restrict__ br,
                                                  double4_32a* __restrict__ x4, double4_32a* __restrict__ R4,
                                                  double4_32a* __restrict__ M4, float4* __restrict__ xf_lo,
                                                  float4* __restrict__ xf_hi, double* __restrict__ part) {
    __shared__ double sm[3 * kBlock];
    __shared__ float smx[4 * (kBlock / 32)];
    const MapPos mp = map_pos(t.nblk);
    if (!t.active[mp.inst]) return;  // block-uniform
    const int i = mp.i;
    double acc[3] = {0, 0, 0};
    const float ninf = __int_as_float(0xff800000);
    float mx[4] = {ninf, ninf, ninf, ninf};  // -min x, -min z, max x, max z (grid frame, FP32)
    const double ninfd = __longlong_as_double(0xfff0000000000000LL);
    double my[2] = {ninfd, ninfd};  // -min y, max y (FP64: the permanent set reads them)
    if (mp.valid) {
        const double* zi = z + 6 * size_t(i);
        const uint8_t* li = t.locked + 6 * size_t(i);
        double tr[3], r[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            tr[d] = li[d] ? 0.0 : zi[d];
            r[d] = li[d + 3] ? 0.0 : zi[d + 3];
        }
        // x = base + s t, rounded exactly as the reference (no fused multiply-add), so that
        // positions -- and with them the contact pair set -- are bit-identical.
        const double ts = p.translation_scale;
        const double xx = __dadd_rn(bx[3 * size_t(i)], __dmul_rn(ts, tr[0]));
        const double xy = __dadd_rn(bx[3 * size_t(i) + 1], __dmul_rn(ts, tr[1]));
        const double xz = __dadd_rn(bx[3 * size_t(i) + 2], __dmul_rn(ts, tr[2]));
        const q4 b{br[4 * size_t(i)], br[4 * size_t(i) + 1], br[4 * size_t(i) + 2], br[4 * size_t(i) + 3]};
        const q4 R = qnorm(qmul(exp_map(d3{r[0], r[1], r[2]}), b));
        x4[i] = make_double4_32a(xx, xy, xz, 0.0);
        // single-precision bounds of the position in the contact grid's frame (the
        // instance's offset added with outward rounding)
        const float2 o = t.off[mp.inst];
        const float4 lo = make_float4(__fadd_rd(__double2float_rd(xx), o.x), __double2float_rd(xy),
                                      __fadd_rd(__double2float_rd(xz), o.y), 0.f);
        const float4 hi = make_float4(__fadd_ru(__double2float_ru(xx), o.x), __double2float_ru(xy),
                                      __fadd_ru(__double2float_ru(xz), o.y), 0.f);
        xf_lo[i] = lo;
        xf_hi[i] = hi;
        R4[i] = make_double4_32a(R.w, R.x, R.y, R.z);
        const m3 M = quat_matrix(R);
        M4[3 * size_t(i)] = make_double4_32a(M.r0.x, M.r0.y, M.r0.z, 0.0);
        M4[3 * size_t(i) + 1] = make_double4_32a(M.r1.x, M.r1.y, M.r1.z, 0.0);
        M4[3 * size_t(i) + 2] = make_double4_32a(M.r2.x, M.r2.y, M.r2.z, 0.0);
        acc[0] = xx; acc[1] = xy; acc[2] = xz;
        // bounding box in the grid's frame: x and z from the outward-rounded bounds (they
        // contain the FP64 positions), y exact; fmax/fmaxf skip NaN coordinates
        mx[0] = -lo.x; mx[1] = -lo.z; mx[2] = hi.x; mx[3] = hi.z;
        my[0] = -xy; my[1] = xy;
    }
    block_sum_t<3>(acc, sm);
    block_max_nf<4>(mx, smx);
    block_max_t<2>(my, sm);
    if (threadIdx.x == 0) {
        double* q = part + 9 * size_t(blockIdx.x);
        q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2];
        q[3] = double(mx[0]); q[4] = my[0]; q[5] = double(mx[1]);
        q[6] = double(mx[2]); q[7] = my[1]; q[8] = double(mx[3]);
    }
}

// Mean position of each instance's nodes (MC/src/sim.cpp:143) and bounding boxes from the
// k_state partials: block i < I writes instance i's cen[9i..9i+8] (mean, minimum, maximum);
// block I the minimum and maximum over all instances at cen[9I + 3..8].
__global__ void __launch_bounds__(kBlock) k_center(DevTopo t, const double* __restrict__ part,
                                                   double* __restrict__ cen) {
    __shared__ double sm[6 * kBlock];
    const int inst = blockIdx.x;
    int k0 = 0, k1 = t.n_nblk;
    if (inst < t.I) {
        const int4 r = t.irange[inst];
        k0 = r.x;
        k1 = r.y;
    }
    double acc[3] = {0, 0, 0};
    const double ninf = __longlong_as_double(0xfff0000000000000LL);
    double mx[6] = {ninf, ninf, ninf, ninf, ninf, ninf};
#pragma unroll 4
    for (int k = k0 + int(threadIdx.x); k < k1; k += blockDim.x) {
        const double* q = part + 9 * size_t(k);
        acc[0] += q[0]; acc[1] += q[1]; acc[2] += q[2];
#pragma unroll
        for (int j = 0; j < 6; j++) mx[j] = fmax(mx[j], q[3 + j]);
    }
    block_sum_t<3>(acc, sm);
    block_max_t<6>(mx, sm);
    if (threadIdx.x == 0) {
        double* c = cen + 9 * size_t(inst);
        if (inst < t.I) {
            const double inv = 1.0 / double(t.inst_n[inst]);
            c[0] = acc[0] * inv; c[1] = acc[1] * inv; c[2] = acc[2] * inv;
        }
        c[3] = -mx[0]; c[4] = -mx[1]; c[5] = -mx[2];
        c[6] = mx[3]; c[7] = mx[4]; c[8] = mx[5];
    }
}

// ---- constitutive return maps: MC/src/sim.cpp:5-8 ------------------------------------------
struct Ret1 { double force, p, a, dg, energy, hard; bool yielded; };
// inv_kH = 1 / max(1e-20, k + H), precomputed per beam (the reference divides).
__device__ __forceinline__ Ret1 return1(double total, double pc, double ac, double k, double y, double H,
                                        double inv_kH) {
    Ret1 r;
    const double trial = k * (total - pc);
    const double f = fabs(trial) - (y + H * ac);
    if (f > 0) {
        const double s = trial >= 0 ? 1.0 : -1.0;
        r.dg = f * inv_kH;
        r.p = pc + s * r.dg;
        r.a = ac + r.dg;
        r.yielded = true;
    } else {
        r.dg = 0; r.p = pc; r.a = ac; r.yielded = false;
    }
    r.force = k * (total - r.p);
    r.energy = .5 * k * sqr(total - r.p);
    r.hard = .5 * H * sqr(r.a);
    return r;
}
struct Ret3 { d3 force, p; double a, dg, energy, hard; bool yielded; };
__device__ __forceinline__ Ret3 return3(d3 t, d3 pc, double ac, double k, double y, double H, double inv_kH) {
    Ret3 r;
    const d3 trial = (t - pc) * k;
    const double n = len(trial);
    const double f = n - (y + H * ac);
    if (f > 0 && n > 1e-20) {
        const d3 d = trial * (1.0 / n);
        r.dg = f * inv_kH;
        r.p = pc + d * r.dg;
        r.a = ac + r.dg;
        r.yielded = true;
    } else {
        r.dg = 0; r.p = pc; r.a = ac; r.yielded = false;
    }
    r.force = (t - r.p) * k;
    r.energy = .5 * k * len2(t - r.p);
    r.hard = .5 * H * sqr(r.a);
    return r;
}

__device__ __forceinline__ q4 ldq(const double4_32a* R, int i) {
    const double4_32a v = R[i];
    return q4{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ d3 ldx(const double4_32a* x, int i) {
    const double4_32a v = x[i];
    return d3{v.x, v.y, v.z};
}
__device__ __forceinline__ m3 ldm(const double4_32a* M, int i) {
    const double4_32a a = M[3 * size_t(i)], b = M[3 * size_t(i) + 1], c = M[3 * size_t(i) + 2];
    return m3{d3{a.x, a.y, a.z}, d3{b.x, b.y, b.z}, d3{c.x, c.y, c.z}};
}
// Unit quaternion by one reciprocal square root (the reference divides by the norm).
__device__ __forceinline__ q4 qnorm_fast(q4 q) {
    const double n2 = q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z;
    if (n2 < 1e-60) return q4{1, 0, 0, 0};
    const double r = rsqrt(n2);
    return q4{q.w * r, q.x * r, q.y * r, q.z * r};
}
// normalize() of MC/include/core.hpp:39 with a reciprocal square root.
__device__ __forceinline__ d3 unit_fast(d3 v) {
    const double l2 = len2(v);
    return (isfinite(l2) && l2 > 1e-30) ? v * rsqrt(l2) : d3{0, 1, 0};
}

// ---- beam kernel: MC/src/sim.cpp:139-141 ---------------------------------------------------
// kMinBlocks: CTAs per SM the register allocation must allow (an occupancy variant picked by
// mcg_autotune; the arithmetic, and so the result, is the same in every variant).
template <int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_beams(DevTopo t, Material m, const double* __restrict__ plastic,
                                                              int trials, EvalBufs e) {
    __shared__ double sm[3 * (kBlock / 32)];
    const MapPos mp = map_pos(t.bblk);
    if (!t.active[mp.inst]) return;
    if (trials == 2) trials = t.trial_inst[mp.inst];  // per instance (device-resident solver)
    const int b = mp.i;
    const int B = t.B;
    double acc[3] = {0, 0, 0};  // energy, elastic, plastic
    if (mp.valid) {
        const int2 ab = t.ab[b];
        const d3 xa = ldx(e.x, ab.x), xb = ldx(e.x, ab.y);
        // chord, length and tangent rounded as the reference (no fused multiply-add), so
        // that a beam at its rest length has exactly zero strain here too
        const d3 d{__dsub_rn(xb.x, xa.x), __dsub_rn(xb.y, xa.y), __dsub_rn(xb.z, xa.z)};
        const double L = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d.x, d.x), __dmul_rn(d.y, d.y)), __dmul_rn(d.z, d.z)));
        double* sa = e.slotA + 6 * size_t(b);
        double* sb = e.slotB + 6 * size_t(b);
        if (L < 1e-10) {
            // Degenerate element: penalty energy only, no gradient and a default trial.
            acc[0] = 1e8 * sqr(1e-10 - L);
#pragma unroll
            for (int k = 0; k < 6; k++) { sa[k] = 0; sb[k] = 0; }
            if (trials) {
#pragma unroll
                for (int k = 0; k < 7; k++) { e.trial_next[k * size_t(B) + b] = 0; e.trial_aux[k * size_t(B) + b] = 0; }
#pragma unroll
                for (int k = 0; k < 3; k++) e.trial_flags[k * size_t(B) + b] = 0;
            }
        } else {
            const double pl_epsp = plastic[b], pl_alpha = plastic[size_t(B) + b];
            const d3 rotp{plastic[2 * size_t(B) + b], plastic[3 * size_t(B) + b], plastic[4 * size_t(B) + b]};
            const double pl_alphaB = plastic[5 * size_t(B) + b], pl_alphaT = plastic[6 * size_t(B) + b];
            const double invL = 1.0 / L;
            const d3 tt{__dmul_rn(d.x, invL), __dmul_rn(d.y, invL), __dmul_rn(d.z, invL)};
            // axial
            const double eps = (L - t.L0[b]) * t.invL0[b];
            const Ret1 ax = return1(eps, pl_epsp, pl_alpha, m.E, t.sy[b], m.H, m.inv_EH);
            const double aL = t.aL[b];
            const double uax = aL * (ax.energy + ax.hard);
            const double dax = t.aLsy[b] * ax.dg;
            const double Nf = t.area[b] * ax.force;
            d3 F = tt * Nf;
            // shear: the end directors against the chord (rotations by the nodes' matrices)
            const m3 Ma = ldm(e.M, ab.x), Mb = ldm(e.M, ab.y);
            const d3 e0{t.e0x[b], t.e0y[b], t.e0z[b]};
            const d3 da = mrot(Ma, e0), db = mrot(Mb, e0);
            const double cs = t.cs[b];
            const d3 ma = da - tt, mb = db - tt;
            const double us = .5 * cs * (len2(ma) + len2(mb));
            const d3 gt = ((tt * 2.0 - da) - db) * cs;
            const d3 trans = (gt - tt * dot(gt, tt)) * invL;
            F = F + trans;
            d3 Ga = -(cross(da, tt) * cs);
            d3 Gb = -(cross(db, tt) * cs);
            // bending and torsion from the relative rotation Q = Ra^* Rb
            const q4 Ra = ldq(e.R, ab.x), Rb = ldq(e.R, ab.y);
            q4 Q = qnorm_fast(qmul(conj(Ra), Rb));
            if (Q.w < 0) Q = q4{-Q.w, -Q.x, -Q.y, -Q.z};
            d3 phi;
            {  // log map (MC/include/core.hpp:52); Q is already unit
                const double s2 = Q.x * Q.x + Q.y * Q.y + Q.z * Q.z;
                const double sq = sqrt(s2);
                if (sq < 1e-12) {
                    phi = d3{2 * Q.x, 2 * Q.y, 2 * Q.z};
                } else {
                    const double ang = 2 * atan2(sq, clampd(Q.w, -1, 1));
                    phi = d3{Q.x, Q.y, Q.z} * (ang / sq);
                }
            }
            const d3 axis = unit_fast(mrot_t(Ma, tt));
            const double tw = dot(phi, axis), ptw = dot(rotp, axis);
            const d3 bend = phi - axis * tw, pb = rotp - axis * ptw;
            const double kb = t.kb[b], kt = t.kt[b], my = t.my[b], ty = t.ty[b];
            const Ret3 br = return3(bend, pb, pl_alphaB, kb, my, t.hb[b], t.inv_kbh[b]);
            const Ret1 tor = return1(tw, ptw, pl_alphaT, kt, ty, t.ht[b], t.inv_kth[b]);
            const d3 moment = br.force + axis * tor.force;
            const double ur = br.energy + br.hard + tor.energy + tor.hard;
            const double dr = my * br.dg + ty * tor.dg;
            const d3 world = mrot(Ma, jl_inv_t(phi, moment));
            Ga = Ga - world;
            Gb = Gb + world;
            acc[0] = (uax + dax) + us + (ur + dr);
            acc[1] = uax + us + ur;
            acc[2] = dax + dr;
            sa[0] = -F.x; sa[1] = -F.y; sa[2] = -F.z; sa[3] = Ga.x; sa[4] = Ga.y; sa[5] = Ga.z;
            sb[0] = F.x;  sb[1] = F.y;  sb[2] = F.z;  sb[3] = Gb.x; sb[4] = Gb.y; sb[5] = Gb.z;
            if (trials) {
                const size_t S = size_t(B);
                const d3 nrot = br.p + axis * tor.p;
                e.trial_next[b] = ax.p;
                e.trial_next[S + b] = ax.a;
                e.trial_next[2 * S + b] = nrot.x;
                e.trial_next[3 * S + b] = nrot.y;
                e.trial_next[4 * S + b] = nrot.z;
                e.trial_next[5 * S + b] = br.a;
                e.trial_next[6 * S + b] = tor.a;
                e.trial_aux[b] = eps;
                e.trial_aux[S + b] = ax.force;
                e.trial_aux[2 * S + b] = moment.x;
                e.trial_aux[3 * S + b] = moment.y;
                e.trial_aux[4 * S + b] = moment.z;
                e.trial_aux[5 * S + b] = uax + us + ur;
                e.trial_aux[6 * S + b] = dax + dr;
                e.trial_flags[b] = ax.yielded;
                e.trial_flags[S + b] = br.yielded;
                e.trial_flags[2 * S + b] = tor.yielded;
            }
        }
    }
    block_sum<3>(acc, sm);
    if (threadIdx.x == 0) {
        e.part_beam[3 * blockIdx.x] = acc[0];
        e.part_beam[3 * blockIdx.x + 1] = acc[1];
        e.part_beam[3 * blockIdx.x + 2] = acc[2];
    }
}

// Contribution of one contact slot to its node (MC/src/sim.cpp:23 addShapeGradient):
// slots 0/1 are shape a's ends, 2/3 shape b's; capsule ends split the force (1-u, u).
__device__ __forceinline__ d3 contact_slot_force(const ContactBufs& c, const PhysParams& p, int N,
                                                 uint32_t item) {
    const uint32_t ci = item >> 2, slot = item & 3u;
    const d3 n{c.c_n[3 * size_t(ci)], c.c_n[3 * size_t(ci) + 1], c.c_n[3 * size_t(ci) + 2]};
    const double mag = p.contact_k * c.c_pen[ci];
    const bool side_b = slot >= 2;
    const uint32_t shape = side_b ? c.c_b[ci] : c.c_a[ci];
    const bool capsule = shape >= uint32_t(N);
    const d3 v = n * (side_b ? -mag : mag);
    if (!capsule) return v;
    const double u = side_b ? c.c_t[ci] : c.c_s[ci];
    return (slot & 1u) ? v * u : v * (1 - u);
}

// One item of a node's contact list: its force, and for slot 0 (the first node of the
// lower shape, present for every contact) the contact's penalty energy, count and
// penetration (sim.cpp:163-164).
__device__ __forceinline__ void add_contact_item(const ContactBufs& c, const PhysParams& p, int N, uint32_t item,
                                                 d3& gx, double& energy, double& count, double& pen_max) {
    gx = gx + contact_slot_force(c, p, N, item);
    if ((item & 3u) == 0) {
        const double pen = c.c_pen[item >> 2];
        energy += .5 * p.contact_k * pen * pen;
        count += 1;
        pen_max = fmax(pen_max, pen);
    }
}

// The sums of each long list (n_long) for the gather, one warp per node: lane l takes items
// l, l + 32, ... in list order, then the lanes' partial sums meet in a fixed butterfly, so
// the sums do not depend on the order of the queue or of the contact list.  A node of a
// densely compressed lattice holds a few hundred items; walked by one thread in the gather,
// its dependent loads set the gather's time.
__global__ void __launch_bounds__(kBlock) k_node_contact_long(DevTopo t, PhysParams p, ContactBufs c) {
    const int lane = threadIdx.x & 31;
    const uint32_t nl = c.n_long[0];
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long j = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < nl; j += warps) {
        const uint32_t i = c.n_long[1 + j];
        const uint32_t s0 = c.n_start[i], cnt = c.n_count[i];
        d3 f{0, 0, 0};
        double energy = 0, count = 0, pen_max = 0;
        for (uint32_t k = uint32_t(lane); k < cnt; k += 32)
            add_contact_item(c, p, t.N, c.n_sorted[s0 + k], f, energy, count, pen_max);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            f.x += __shfl_xor_sync(0xffffffffu, f.x, o);
            f.y += __shfl_xor_sync(0xffffffffu, f.y, o);
            f.z += __shfl_xor_sync(0xffffffffu, f.z, o);
            energy += __shfl_xor_sync(0xffffffffu, energy, o);
            count += __shfl_xor_sync(0xffffffffu, count, o);
            pen_max = fmax(pen_max, __shfl_xor_sync(0xffffffffu, pen_max, o));
        }
        if (lane == 0) {
            double* q = c.long_sum + 6 * size_t(j);
            q[0] = f.x;
            q[1] = f.y;
            q[2] = f.z;
            q[3] = energy;
            q[4] = count;
            q[5] = pen_max;
        }
    }
}

// ---- per-node gather: the scatter of MC/src/sim.cpp:139-172, as a deterministic CSR sum ---
// Sums the incident beams' end vectors of node i in ascending beam order: FP64 slots
// directly, FP32 slots (mixed form) with compensated FP32 sums.
template <bool F32>
__device__ __forceinline__ void sum_slots(const DevTopo& t, const EvalBufs& e, int i, d3& gx, d3& gr) {
    const int k0 = t.inc_start[i], k1 = t.inc_start[i + 1];
    // unrolled so that the loads of several incident beams are in flight together; the
    // additions keep their order
    if (!F32) {
#pragma unroll 4
        for (int k = k0; k < k1; k++) {
            const int v = t.inc[k];
            const double* s = ((v & 1) ? e.slotB : e.slotA) + 6 * size_t(v >> 1);
            gx.x += s[0]; gx.y += s[1]; gx.z += s[2];
            gr.x += s[3]; gr.y += s[4]; gr.z += s[5];
        }
    } else {
        float hi[6] = {0, 0, 0, 0, 0, 0}, lo[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 4
        for (int k = k0; k < k1; k++) {
            const int v = t.inc[k];
            const float* s = ((v & 1) ? e.slotBf : e.slotAf) + 6 * size_t(v >> 1);
#pragma unroll
            for (int j = 0; j < 6; j++) {  // two-sum
                const float a = s[j], sum = hi[j] + a, bp = sum - hi[j];
                lo[j] += (hi[j] - (sum - bp)) + (a - bp);
                hi[j] = sum;
            }
        }
        gx = d3{double(hi[0]) + double(lo[0]), double(hi[1]) + double(lo[1]), double(hi[2]) + double(lo[2])};
        gr = d3{double(hi[3]) + double(lo[3]), double(hi[4]) + double(lo[4]), double(hi[5]) + double(lo[5])};
    }
}

template <bool F32, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_gather(DevTopo t, PhysParams p, ContactBufs c, int use_contacts,
                                                               EvalBufs e, double* __restrict__ grad) {
    __shared__ double sm[6 * kBlock];
    __shared__ double cforce[2];
    const MapPos mp = map_pos(t.nblk);
    if (!t.active[mp.inst]) return;  // block-uniform
    const int i = mp.i;
    const int N = t.N;
    // centering force of the block's instance (sim.cpp:143), the same for all its nodes:
    // one FP64 division per block (GB300's FP64 pipe is narrow)
    if (threadIdx.x == 0) {
        const double* cen = e.cen + 9 * size_t(mp.inst);
        const double Ni = double(t.inst_n[mp.inst]);
        cforce[0] = p.centering * cen[0] / Ni;
        cforce[1] = p.centering * cen[2] / Ni;
    }
    __syncthreads();
    double acc[6] = {0, 0, 0, 0, 0, 0};  // gravity E, platen E, reaction, contacts, self-contact E, |g|^2
    double pen_max = 0;
    unsigned long long gbits = 0;  // max |g| as the bits of a non-negative double (integer max)
    if (mp.valid) {
        d3 gx{0, 0, 0}, gr{0, 0, 0};
        sum_slots<F32>(t, e, i, gx, gr);
        const d3 xi = ldx(e.x, i);
        // gravity (sim.cpp:142)
        const double mg = t.mass[i] * p.gravity;
        acc[0] = mg * xi.y;
        gx.y += mg;
        // centering (sim.cpp:143)
        gx.x += cforce[0];
        gx.z += cforce[1];
        // self-contact forces on this node in ascending (lower shape, higher shape, slot)
        // order (the list is sorted by the contact pipeline), and the self-contact energy of
        // each contact on the first node of its lower shape: both independent of the order
        // of the contact list
        const uint32_t cnt = use_contacts ? c.n_count[i] : 0u;
        if (cnt > 32 && c.long_sum) {  // summed by k_node_contact_long
            const double* q = c.long_sum + 6 * size_t(c.n_cursor[i]);
            gx = gx + d3{q[0], q[1], q[2]};
            acc[4] += q[3];
            acc[3] += q[4];
            pen_max = fmax(pen_max, q[5]);
        } else if (use_contacts) {
            const uint32_t s0 = c.n_start[i];
            uint32_t k = 0;
            // four items at a time: their loads in flight together (a joint of a densely
            // compressed lattice can hold a few hundred items), the additions in list order
            for (; k + 4 <= cnt; k += 4) {
                d3 f[4];
                double pen[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const uint32_t item = c.n_sorted[s0 + k + j];
                    f[j] = contact_slot_force(c, p, N, item);
                    pen[j] = (item & 3u) == 0 ? c.c_pen[item >> 2] : -1.0;  // a contact's pen > 0
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    gx = gx + f[j];
                    if (pen[j] >= 0) {
                        acc[4] += .5 * p.contact_k * pen[j] * pen[j];
                        acc[3] += 1;
                        pen_max = fmax(pen_max, pen[j]);
                    }
                }
            }
            for (; k < cnt; k++) add_contact_item(c, p, N, c.n_sorted[s0 + k], gx, acc[4], acc[3], pen_max);
        }
        // platens (sim.cpp:168-171)
        const double jr = p.joint_radius, kc = p.contact_k;
        const double pb = jr - xi.y;
        if (pb > 0) {
            const double mm = kc * pb;
            acc[1] += .5 * kc * pb * pb;
            pen_max = fmax(pen_max, pb);
            acc[3] += 1;
            gx.y -= mm;
        }
        const double pt = xi.y + jr - e.tops[mp.inst];
        if (pt > 0) {
            const double mm = kc * pt;
            acc[1] += .5 * kc * pt * pt;
            acc[2] += mm;
            pen_max = fmax(pen_max, pt);
            acc[3] += 1;
            gx.y += mm;
        }
        // pack, scale and lock (sim.cpp:172)
        const double ts = p.translation_scale;
        const uint8_t* li = t.locked + 6 * size_t(i);
        double* g = grad + 6 * size_t(i);
        const double gv[6] = {ts * gx.x, ts * gx.y, ts * gx.z, gr.x, gr.y, gr.z};
#pragma unroll
        for (int k = 0; k < 6; k++) {
            g[k] = li[k] ? 0.0 : gv[k];
            // residual over free DOFs for the solver's convergence test (sim.cpp:44-45)
            if (!li[k]) {
                acc[5] += gv[k] * gv[k];
                // fmax(gmax, |g|) on the bit patterns; a NaN (above the infinity pattern) is
                // skipped as fmax skips it
                const unsigned long long b = (unsigned long long)__double_as_longlong(gv[k]) & 0x7fffffffffffffffULL;
                if (b <= 0x7ff0000000000000ULL && b > gbits) gbits = b;
            }
        }
    }
    block_sum_t<6>(acc, sm);
    double m2[2] = {pen_max, __longlong_as_double((long long)gbits)};
    block_max_t<2>(m2, sm);
    if (threadIdx.x == 0) {
        double* q = e.part_node + kNodeParts * size_t(blockIdx.x);
        q[0] = acc[0]; q[1] = acc[1]; q[2] = acc[2]; q[3] = m2[0]; q[4] = acc[3]; q[5] = acc[4];
        q[6] = acc[5]; q[7] = m2[1];
    }
}

// ---- totals and the non-finite guard ---------------------------------------------------------
// Two stages, so the FP64 additions spread over many SMs (GB300's FP64 pipe is narrow).
// Stage 1: block (f, inst) sums the instance's block partials k = first + f + kFinFan j.
constexpr int kFinFan = 32;
constexpr int kFinVals = 11;  // beamE, elastic, plastic, gravityE, platenE, reaction, contactE,
                              // contacts, |g|^2, max penetration, max |g|
static_assert(kFinPartDoubles == kFinFan * kFinVals, "first-stage totals buffer");
__global__ void __launch_bounds__(kBlock) k_finalize_parts(DevTopo t, const double* __restrict__ pbeam,
                                                           const double* __restrict__ pnode,
                                                           double* __restrict__ fpart) {
    __shared__ double sm[9 * kBlock];
    const int inst = blockIdx.y, f = blockIdx.x;
    if (!t.active[inst]) return;
    const int4 r = t.irange[inst];
    double acc[6] = {0, 0, 0, 0, 0, 0};  // beamE, elastic, plastic, gravityE, platenE, reaction
    double cacc[3] = {0, 0, 0};          // self-contact E, contacts (platen and self), |g|^2
    double m2[2] = {0, 0};               // max penetration, max |g|
    for (int k = r.z + f + kFinFan * int(threadIdx.x); k < r.w; k += kFinFan * int(blockDim.x)) {
        acc[0] += pbeam[3 * k]; acc[1] += pbeam[3 * k + 1]; acc[2] += pbeam[3 * k + 2];
    }
    for (int k = r.x + f + kFinFan * int(threadIdx.x); k < r.y; k += kFinFan * int(blockDim.x)) {
        const double* q = pnode + kNodeParts * size_t(k);
        acc[3] += q[0]; acc[4] += q[1]; acc[5] += q[2];
        m2[0] = fmax(m2[0], q[3]);
        cacc[1] += q[4];
        cacc[0] += q[5];
        cacc[2] += q[6];
        m2[1] = fmax(m2[1], q[7]);
    }
    double all[9] = {acc[0], acc[1], acc[2], acc[3], acc[4], acc[5], cacc[0], cacc[1], cacc[2]};
    block_sum_t<9>(all, sm);
    block_max_t<2>(m2, sm);
    if (threadIdx.x == 0) {
        double* o = fpart + kFinVals * (size_t(inst) * kFinFan + f);
        for (int k = 0; k < 9; k++) o[k] = all[k];
        o[9] = m2[0]; o[10] = m2[1];
    }
}

// Stage 2, one block per instance: the kFinFan stage-1 results in order, the energy in the
// reference's group order, diagnostics, non-finite guard.
__global__ void __launch_bounds__(kBlock) k_finalize(DevTopo t, PhysParams p, const double* __restrict__ fpart,
                                                     const double* __restrict__ cen,
                                                     const uint32_t* __restrict__ flags, EvalOut* out_all) {
    static_assert(kFinFan == 32, "one stage-1 result per lane");
    const int inst = blockIdx.x;
    if (!t.active[inst]) return;
    const double* q = fpart + kFinVals * (size_t(inst) * kFinFan + threadIdx.x);
    double acc[6], cacc[3];  // beamE, elastic, plastic, gravityE, platenE, reaction; contactE,
                             // contacts, |g|^2
#pragma unroll
    for (int k = 0; k < 6; k++) acc[k] = warp_sum(q[k]);
#pragma unroll
    for (int k = 0; k < 3; k++) cacc[k] = warp_sum(q[6 + k]);
    const double pmax = warp_max(q[9]), gmax = warp_max(q[10]);
    if (threadIdx.x != 0) return;
    if (threadIdx.x == 0) {
        const double* c = cen + 9 * size_t(inst);
        const double center = .5 * p.centering * (sqr(c[0]) + sqr(c[2]));
        const double contactE = cacc[0];
        // Group order of the reference's accumulation: beams, gravity, centering,
        // self-contact, platens (sim.cpp:139-171).
        double energy = acc[0];
        energy += acc[3];
        energy += center;
        energy += contactE;
        energy += acc[4];
        const int nonfinite = isfinite(energy) ? 0 : 1;
        EvalOut* out = out_all + inst;
        out->energy = nonfinite ? __longlong_as_double(0x7ff0000000000000LL) : energy;
        out->elastic = acc[1];
        out->plastic = acc[2];
        out->contact = contactE + acc[4];
        out->reaction = acc[5];
        out->max_pen = pmax;
        out->contacts = int(cacc[1]);
        out->nonfinite = nonfinite;
        out->beam_energy = acc[0];
        out->node_energy = acc[3];
        out->center_energy = center;
        out->contact_energy = contactE;
        out->platen_energy = acc[4];
        out->overflow = flags ? int(flags[0] & ~uint32_t(kNonFinite)) : 0;
        // a non-finite evaluation has a zero gradient (k_zero_if_nonfinite)
        const long long nf = t.inst_free[inst];
        out->rms = nonfinite ? 0.0 : (nf ? sqrt(cacc[2] / double(nf)) : 0.0);
        out->gmax = nonfinite ? 0.0 : gmax;
    }
}

// Non-finite energy: the instance's whole gradient is zero (sim.cpp:172).
__global__ void __launch_bounds__(kBlock) k_zero_if_nonfinite(DevTopo t, const EvalOut* __restrict__ out,
                                                              double* __restrict__ grad) {
    const MapPos mp = map_pos(t.nblk);
    if (!mp.valid || !t.active[mp.inst] || !out[mp.inst].nonfinite) return;
#pragma unroll
    for (int k = 0; k < 6; k++) grad[6 * size_t(mp.i) + k] = 0;
}

// ---- commit (MC/src/sim.cpp:212): base state <- current state, plastic <- trial ----------
__global__ void __launch_bounds__(kBlock) k_commit_nodes(DevTopo t, const uint8_t* __restrict__ mask,
                                                         const double4_32a* __restrict__ x4,
                                                         const double4_32a* __restrict__ R4, double* __restrict__ bx,
                                                         double* __restrict__ br) {
    const MapPos mp = map_pos(t.nblk);
    if (!mp.valid || (mask && !mask[mp.inst])) return;
    const int i = mp.i;
    const double4_32a x = x4[i], r = R4[i];
    bx[3 * size_t(i)] = x.x; bx[3 * size_t(i) + 1] = x.y; bx[3 * size_t(i) + 2] = x.z;
    br[4 * size_t(i)] = r.x; br[4 * size_t(i) + 1] = r.y; br[4 * size_t(i) + 2] = r.z; br[4 * size_t(i) + 3] = r.w;
}

// plastic <- trial.next for the beams of the committed instances (7 SoA arrays)
__global__ void __launch_bounds__(kBlock) k_commit_plastic(DevTopo t, const uint8_t* __restrict__ mask,
                                                           const double* __restrict__ next, double* __restrict__ pl) {
    const MapPos mp = map_pos(t.bblk);
    if (!mp.valid || (mask && !mask[mp.inst])) return;
#pragma unroll
    for (int k = 0; k < 7; k++) pl[k * size_t(t.B) + mp.i] = next[k * size_t(t.B) + mp.i];
}

// Plastic statistics of the committed state (MC/src/sim.cpp:339-362), one partial per beam
// block: sum and max of |epsp|, sum and max of |rotp|, counts above 1e-5 and 1e-4.
__global__ void __launch_bounds__(kBlock) k_plastic_part(DevTopo t, const double* __restrict__ pl,
                                                         double* __restrict__ part) {
    __shared__ double sm[4 * (kBlock / 32)];
    __shared__ double smx[kBlock / 32];
    const MapPos mp = map_pos(t.bblk);
    const int B = t.B;
    double acc[4] = {0, 0, 0, 0};
    double m0 = 0, m1 = 0;
    if (mp.valid) {
        const int b = mp.i;
        const double pa = fabs(pl[b]);
        const d3 r{pl[2 * size_t(B) + b], pl[3 * size_t(B) + b], pl[4 * size_t(B) + b]};
        const double pr = len(r);
        acc[0] += pa; acc[1] += pr;
        acc[2] += pa > 1e-5 ? 1.0 : 0.0;
        acc[3] += pr > 1e-4 ? 1.0 : 0.0;
        m0 = fmax(m0, pa); m1 = fmax(m1, pr);
    }
    block_sum<4>(acc, sm);
    m0 = block_max(m0, smx);
    m1 = block_max(m1, smx);
    if (threadIdx.x == 0) {
        double* q = part + 6 * size_t(blockIdx.x);
        q[0] = acc[0]; q[1] = m0; q[2] = acc[1]; q[3] = m1; q[4] = acc[2]; q[5] = acc[3];
    }
}
// One block per instance over its beam blocks.
__global__ void __launch_bounds__(kBlock) k_plastic_final(DevTopo t, const double* __restrict__ part,
                                                          double* __restrict__ out) {
    __shared__ double sm[4 * (kBlock / 32)];
    __shared__ double smx[kBlock / 32];
    const int4 r = t.irange[blockIdx.x];
    double acc[4] = {0, 0, 0, 0};
    double m0 = 0, m1 = 0;
    for (int k = r.z + int(threadIdx.x); k < r.w; k += blockDim.x) {
        const double* q = part + 6 * size_t(k);
        acc[0] += q[0]; acc[1] += q[2]; acc[2] += q[4]; acc[3] += q[5];
        m0 = fmax(m0, q[1]); m1 = fmax(m1, q[3]);
    }
    block_sum<4>(acc, sm);
    m0 = block_max(m0, smx);
    m1 = block_max(m1, smx);
    if (threadIdx.x == 0) {
        double* o = out + 6 * size_t(blockIdx.x);
        o[0] = acc[0]; o[1] = m0; o[2] = acc[1]; o[3] = m1; o[4] = acc[2]; o[5] = acc[3];
    }
}

// ---- launchers ------------------------------------------------------------------------------
void launch_state(const DevTopo& t, const PhysParams& p, const double* z, const double* base_x,
                  const double* base_r, EvalBufs& e, cudaStream_t s) {
    k_state<<<t.n_nblk, kBlock, 0, s>>>(t, p, z, base_x, base_r, e.x, e.R, e.M, e.xf_lo, e.xf_hi, e.part_state);
    note_launches(1);
    launch_center(t, e, s);
}

void launch_center(const DevTopo& t, EvalBufs& e, cudaStream_t s) {
    k_center<<<t.I + 1, kBlock, 0, s>>>(t, e.part_state, e.cen);
    note_launches(1);
}

void launch_commit(const DevTopo& t, const uint8_t* mask, const EvalBufs& e, double* base_x, double* base_r,
                   double* plastic, cudaStream_t s) {
    k_commit_nodes<<<t.n_nblk, kBlock, 0, s>>>(t, mask, e.x, e.R, base_x, base_r);
    note_launches(1);
    if (t.B > 0 && plastic) {
        k_commit_plastic<<<t.n_bblk, kBlock, 0, s>>>(t, mask, e.trial_next, plastic);
        note_launches(1);
    }
}

void launch_plastic_stats(const DevTopo& t, const double* plastic, double* part, double* out6, cudaStream_t s) {
    if (t.B == 0) return;
    k_plastic_part<<<t.n_bblk, kBlock, 0, s>>>(t, plastic, part);
    k_plastic_final<<<t.I, kBlock, 0, s>>>(t, part, out6);
    note_launches(2);
}

// Occupancy variants (CTAs per SM) of the FP64 beam kernel and of the gather.
constexpr int kBeamBlocks[] = {1, 2, 3};
constexpr int kGatherBlocks[] = {1, 2, 4};

int shape_variants(ShapeKernel k) {
    switch (k) {
        case ShapeKernel::kBeams: return 3;
        case ShapeKernel::kGather: return 3;
        default: return beams_mixed_variants();
    }
}
int shape_blocks(ShapeKernel k, int v) {
    switch (k) {
        case ShapeKernel::kBeams: return kBeamBlocks[v];
        case ShapeKernel::kGather: return kGatherBlocks[v];
        default: return beams_mixed_blocks(v);
    }
}

void launch_beams(const DevTopo& t, const Material& m, const double* plastic, int trials, EvalBufs& e,
                  cudaStream_t s, int variant) {
    if (t.B == 0) return;
    const int tr = trials;  // 0, 1, or 2: per instance (t.trial_inst)
    switch (variant) {
        case 1: k_beams<kBeamBlocks[1]><<<t.n_bblk, kBlock, 0, s>>>(t, m, plastic, tr, e); break;
        case 2: k_beams<kBeamBlocks[2]><<<t.n_bblk, kBlock, 0, s>>>(t, m, plastic, tr, e); break;
        default: k_beams<kBeamBlocks[0]><<<t.n_bblk, kBlock, 0, s>>>(t, m, plastic, tr, e); break;
    }
    note_launches(1);
}

constexpr int kLongListBlocks = 4 * 152;  // eight long lists per block, grid-stride

template <bool F32>
void gather_variant(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad, EvalBufs& e,
                    cudaStream_t s, int variant) {
    ContactBufs cc{};
    if (c) cc = *c;
    const int uc = c ? 1 : 0;
    if (c && c->long_sum) {
        (k_node_contact_long<<<kLongListBlocks, kBlock, 0, s>>>(t, p, cc), note_launches(1));
    }
    switch (variant) {
        case 1: k_gather<F32, kGatherBlocks[1]><<<t.n_nblk, kBlock, 0, s>>>(t, p, cc, uc, e, grad); break;
        case 2: k_gather<F32, kGatherBlocks[2]><<<t.n_nblk, kBlock, 0, s>>>(t, p, cc, uc, e, grad); break;
        default: k_gather<F32, kGatherBlocks[0]><<<t.n_nblk, kBlock, 0, s>>>(t, p, cc, uc, e, grad); break;
    }
    note_launches(1);
}

void launch_gather(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad, EvalBufs& e,
                   cudaStream_t s, int variant) {
    gather_variant<false>(t, p, c, grad, e, s, variant);
}

void launch_gather_mixed(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad, EvalBufs& e,
                         cudaStream_t s, int variant) {
    gather_variant<true>(t, p, c, grad, e, s, variant);
}

void launch_finalize(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad, EvalBufs& e,
                     cudaStream_t s) {
    k_finalize_parts<<<dim3(kFinFan, t.I), kBlock, 0, s>>>(t, e.part_beam, e.part_node, e.part_fin);
    k_finalize<<<t.I, 32, 0, s>>>(t, p, e.part_fin, e.cen, c ? c->flags : nullptr, e.out);
    k_zero_if_nonfinite<<<t.n_nblk, kBlock, 0, s>>>(t, e.out, grad);
    note_launches(3);
}

}  // namespace mcg
