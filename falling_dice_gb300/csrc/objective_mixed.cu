// objective_mixed.cu -- the mixed-precision form of the energy/gradient evaluation.
//
// FP32 does the bulk arithmetic: every per-beam term of the reference's objective
// (MC/src/sim.cpp:139-141).  FP64 stays where stability needs it: the base configuration,
// the per-increment base terms below, node positions for contact and platen tests,
// energy totals (compensated FP32 block sums, FP64 across blocks), node gradient totals
// (compensated FP32 sums), and everything the L-BFGS solver does.
//
// Naively FP32 would lose the quantities the energy depends on by cancellation:
//   * the chord length change L - L0 (strain ~1e-3 of a 5 mm chord);
//   * the shear vectors d_a - t, d_b - t (directors nearly aligned with the chord);
//   * the relative rotation Ra^* Rb between two nearly aligned nodes.
// The configuration is therefore split into the base state of the increment (FP64; the
// reference re-bases it at every commit, MC/src/sim.cpp:212, and every increment starts
// from z = 0, sim.cpp:398) and the FP32 increment since it:
//   x = x_base + u,  R = e R_base with e = exp(r) kept as (w - 1, v),
// and the cancelling quantities are formed from small terms only:
//   |d|^2 - L0^2 = c0 + 2 d0.du + du.du              c0 = |d0|^2 - L0^2   (base, FP64)
//   d_a - t      = inc(e_a, d_a0) + s_a0 - (t - t0)   s_a0 = d_a0 - t0     (base, FP64)
//   t - t0       = (du |d0| - d0 (L - |d0|)) / (L |d0|)
//   Ra^* Rb      = (Ra0^* delta Ra0) Q0,  delta = e_a^* e_b              Q0 = Ra0^* Rb0
// with inc(e, v) = R(e) v - v evaluated as 2w (u x v) + 2 u x (u x v) and the near-identity
// quaternions held as (w - 1, v), so that every FP32 rounding is relative to an increment.
// d0 is the base chord rounded to FP32, while c0, |d0| and s_a0 are computed from the exact
// chord: the rounding of d0 then only enters multiplied by an increment, and a beam at its
// base state sees exactly the base strain and shear.  One case stays out of reach: the
// reference's degenerate-beam branch (chord below 1e-10 m, sim.cpp:139) lies below the
// FP32 resolution of a position increment, so the mixed form resolves chords only down to
// about 1e-9 m.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float fdot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 xyz(float4 v) { return {v.x, v.y, v.z}; }

// R(q) v - v for a unit quaternion q = (w, u).
__device__ __forceinline__ f3 rot_inc(float w, f3 u, f3 v) {
    const f3 t = fcross(u, v) * 2.f;
    return t * w + fcross(u, t);
}
__device__ __forceinline__ f3 rot(float w, f3 u, f3 v) { return v + rot_inc(w, u, v); }
__device__ __forceinline__ f3 rot_conj(float w, f3 u, f3 v) { return v + rot_inc(w, -u, v); }


// Warp sum of compensated pairs (hi, lo) into lane 0, in FP32.
__device__ __forceinline__ void warp_sum_comp(float& hi, float& lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
        const float s = hi + h2;
        const float bp = s - hi;
        lo += l2 + ((hi - (s - bp)) + (h2 - bp));
        hi = s;
    }
}

// Sums kBlock per-thread FP32 values (v[t] in smem, written by thread t before the
// caller's barrier) with one warp: lane l adds v[l], v[l + 32], ... in order with
// compensation, then the lanes' compensated pairs are summed by a fixed shuffle tree.  The
// result, one FP64 rounding of the compensated pair, is in lane 0.  The order is fixed, so
// the sum is reproducible; only one warp spends instructions on it.
__device__ __forceinline__ double warp_sum_smem(const float* v, int lane) {
    float hi = v[lane], lo = 0.f;
#pragma unroll
    for (int k = 1; k < kBlock / 32; k++) {
        const float a = v[lane + 32 * k], s = hi + a, bp = s - hi;
        lo += (hi - (s - bp)) + (a - bp);
        hi = s;
    }
    warp_sum_comp(hi, lo);
    return double(hi) + double(lo);
}

struct R1 { float force, p, a, dg, energy, hard; bool yielded; };
__device__ __forceinline__ R1 ret1(float total, float pc, float ac, float k, float y, float H) {
    R1 r;
    const float trial = k * (total - pc);
    const float f = fabsf(trial) - (y + H * ac);
    if (f > 0.f) {
        r.dg = __fdividef(f, fmaxf(1e-20f, k + H));
        r.p = pc + (trial >= 0.f ? r.dg : -r.dg);
        r.a = ac + r.dg;
        r.yielded = true;
    } else {
        r.dg = 0.f; r.p = pc; r.a = ac; r.yielded = false;
    }
    const float e = total - r.p;
    r.force = k * e;
    r.energy = .5f * k * e * e;
    r.hard = .5f * H * r.a * r.a;
    return r;
}
struct R3 { f3 force, p; float a, dg, energy, hard; bool yielded; };
__device__ __forceinline__ R3 ret3(f3 t, f3 pc, float ac, float k, float y, float H) {
    R3 r;
    const f3 e0 = t - pc;
    const f3 trial = e0 * k;
    const float n = sqrtf(fdot(trial, trial));
    const float f = n - (y + H * ac);
    if (f > 0.f && n > 1e-20f) {
        r.dg = __fdividef(f, fmaxf(1e-20f, k + H));
        r.p = pc + trial * __fdividef(r.dg, n);
        r.a = ac + r.dg;
        r.yielded = true;
    } else {
        r.dg = 0.f; r.p = pc; r.a = ac; r.yielded = false;
    }
    const f3 e = t - r.p;
    r.force = e * k;
    r.energy = .5f * k * fdot(e, e);
    r.hard = .5f * H * r.a * r.a;
    return r;
}

// J_l^{-T}(p) v in FP32 (MC/include/core.hpp:53): series coefficient below 0.5 rad (four
// terms reach FP32 precision there), closed form above.
__device__ __forceinline__ f3 jl_inv_t_f(f3 p, f3 v) {
    const float a2 = fdot(p, p);
    const f3 c1 = fcross(p, v);
    const f3 c2 = fcross(p, c1);
    float A;
    if (a2 < 0.25f) {
        A = fmaf(fmaf(fmaf(1.f / 1209600.f, a2, 1.f / 30240.f), a2, 1.f / 720.f), a2, 1.f / 12.f);
    } else {
        const float a = sqrtf(a2);
        float s, c;
        sincosf(a, &s, &c);
        A = 1.f / a2 - (1.f + c) / (2.f * a * s);
    }
    return (v + c1 * .5f) + c2 * A;
}

// Rotation vector of the unit quaternion (qw, qv), qw >= 0: qv 2 atan2(|qv|, qw) / |qv|
// (MC/include/core.hpp:52).  Up to |qv| = qw / 4 (angles up to 28 degrees: nearly every
// beam) the factor is (2 / qw) atan(x) / x, x^2 = |qv|^2 / qw^2, from the Gregory series
// atan(x) / x = 1 - x^2/3 + x^4/5 - ...; stopping after x^10/11 leaves less than
// x^12/13 < 5e-9.  Larger angles use atan2f.
__device__ __forceinline__ f3 rotvec_f(float qw, f3 qv) {
    const float s2 = fdot(qv, qv);
    if (s2 <= 0.0625f * qw * qw) {
        const float rq = __fdividef(1.f, qw);
        const float u = s2 * rq * rq;
        float P = fmaf(u, -1.f / 11.f, 1.f / 9.f);
        P = fmaf(u, P, -1.f / 7.f);
        P = fmaf(u, P, 1.f / 5.f);
        P = fmaf(u, P, -1.f / 3.f);
        P = fmaf(u, P, 1.f);
        return qv * (2.f * rq * P);
    }
    const float s = sqrtf(s2);
    return qv * __fdividef(2.f * atan2f(s, qw), s);
}

// ---- node state --------------------------------------------------------------------------
// u = s t (FP32), e = exp(r) as (w - 1, v) (FP32), x = x_base + u (FP64, for contact,
// platen and centering), FP32 position bounds; block partial sums and extrema of x.
__global__ void __launch_bounds__(kBlock) k_state_mixed(DevTopo t, double ts, const double* __restrict__ z,
                                                        const double* __restrict__ bx, float4* __restrict__ UE,
                                                        double4_32a* __restrict__ x4,
                                                        float4* __restrict__ xf_lo, float4* __restrict__ xf_hi,
                                                        double* __restrict__ part) {
    __shared__ double sm[3 * kBlock];
    __shared__ float smx[4 * (kBlock / 32)];
    const MapPos mp = map_pos(t.nblk);
    if (!t.active[mp.inst]) return;
    const int i = mp.i;
    double acc[3] = {0, 0, 0};
    const float ninf = __int_as_float(0xff800000);
    float mx[4] = {ninf, ninf, ninf, ninf};  // -min x, -min z, max x, max z (grid frame, FP32)
    const double ninfd = __longlong_as_double(0xfff0000000000000LL);
    double my[2] = {ninfd, ninfd};  // -min y, max y (FP64: the permanent set reads them)
    if (mp.valid) {
        const double* zi = z + 6 * size_t(i);
        const uint8_t* li = t.locked + 6 * size_t(i);
        float tr[3], r[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            tr[d] = li[d] ? 0.f : float(zi[d] * ts);
            r[d] = li[d + 3] ? 0.f : float(zi[d + 3]);
        }
        UE[2 * size_t(i)] = make_float4(tr[0], tr[1], tr[2], 0.f);
        const float th2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        float wm1, sv;  // cos(th/2) - 1 and sin(th/2)/th
        if (th2 < 1e-6f) {
            wm1 = th2 * (-0.125f + th2 * (1.f / 384.f));
            sv = 0.5f + th2 * (-1.f / 48.f + th2 * (1.f / 3840.f));
        } else {
            const float th = sqrtf(th2);
            float s4, c4;  // sin, cos of th/4: cos(th/2) - 1 = -2 s4^2, sin(th/2) = 2 s4 c4
            sincosf(0.25f * th, &s4, &c4);
            wm1 = -2.f * s4 * s4;
            sv = 2.f * s4 * c4 / th;
        }
        UE[2 * size_t(i) + 1] = make_float4(wm1, r[0] * sv, r[1] * sv, r[2] * sv);
        const double xx = bx[3 * size_t(i)] + double(tr[0]);
        const double xy = bx[3 * size_t(i) + 1] + double(tr[1]);
        const double xz = bx[3 * size_t(i) + 2] + double(tr[2]);
        x4[i] = make_double4_32a(xx, xy, xz, 0.0);
        const float2 o = t.off[mp.inst];
        const float4 lo = make_float4(__fadd_rd(__double2float_rd(xx), o.x), __double2float_rd(xy),
                                      __fadd_rd(__double2float_rd(xz), o.y), 0.f);
        const float4 hi = make_float4(__fadd_ru(__double2float_ru(xx), o.x), __double2float_ru(xy),
                                      __fadd_ru(__double2float_ru(xz), o.y), 0.f);
        xf_lo[i] = lo;
        xf_hi[i] = hi;
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

// ---- per-increment base terms (FP64, once per commit) ----------------------------------------
__global__ void __launch_bounds__(kBlock) k_rebase_nodes(int N, const double* __restrict__ br, float4* __restrict__ R0f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double* q = br + 4 * size_t(i);
    R0f[i] = make_float4(float(q[0]), float(q[1]), float(q[2]), float(q[3]));
}

__global__ void __launch_bounds__(kBlock) k_rebase_beams(DevTopo t, const double* __restrict__ bx,
                                                         const double* __restrict__ br, MixedBeams m) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= t.B) return;
    const int2 ab = t.ab[b];
    const d3 xa{bx[3 * size_t(ab.x)], bx[3 * size_t(ab.x) + 1], bx[3 * size_t(ab.x) + 2]};
    const d3 xb{bx[3 * size_t(ab.y)], bx[3 * size_t(ab.y) + 1], bx[3 * size_t(ab.y) + 2]};
    const q4 Ra{br[4 * size_t(ab.x)], br[4 * size_t(ab.x) + 1], br[4 * size_t(ab.x) + 2], br[4 * size_t(ab.x) + 3]};
    const q4 Rb{br[4 * size_t(ab.y)], br[4 * size_t(ab.y) + 1], br[4 * size_t(ab.y) + 2], br[4 * size_t(ab.y) + 3]};
    // The base chord is stored rounded to FP32; c0, |d0| and t0 come from the exact FP64
    // chord, so a beam at its base state carries no prestrain or shear from that rounding
    // (the rounding only enters multiplied by the increment).
    const d3 d0{xb.x - xa.x, xb.y - xa.y, xb.z - xa.z};
    const float4 d0f = make_float4(float(d0.x), float(d0.y), float(d0.z), 0.f);
    const double L0 = t.L0[b];
    const double Lb = sqrt(dot(d0, d0));
    const double c0 = dot(d0, d0) - L0 * L0;
    const d3 t0 = d0 * (1.0 / Lb);
    const d3 e0{t.e0x[b], t.e0y[b], t.e0z[b]};
    const d3 da0 = qrot(Ra, e0), db0 = qrot(Rb, e0);
    const d3 sa0 = da0 - t0, sb0 = db0 - t0;
    q4 Q0 = qmul(conj(Ra), Rb);
    if (Q0.w < 0) Q0 = q4{-Q0.w, -Q0.x, -Q0.y, -Q0.z};
    const double v2 = Q0.x * Q0.x + Q0.y * Q0.y + Q0.z * Q0.z;
    const double wm1 = -v2 / (1.0 + Q0.w);  // w - 1 without cancellation
    m.B0[b] = make_float4(d0f.x, d0f.y, d0f.z, float(c0));
    m.B1[b] = make_float4(float(sa0.x), float(sa0.y), float(sa0.z), float(L0));
    m.B2[b] = make_float4(float(sb0.x), float(sb0.y), float(sb0.z), float(Lb));
    m.B5[b] = make_float4(float(wm1), float(Q0.x), float(Q0.y), float(Q0.z));
}

// Streamed section constants in FP32 (the FP64 constants rounded), once per upload; only for
// sections that are not the circular section's (see MixedBeams).
__global__ void __launch_bounds__(kBlock) k_mixed_constants(DevTopo t, MixedBeams m) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= t.B) return;
    m.C0[b] = make_float4(float(t.kb[b]), float(t.kt[b]), float(t.my[b]), float(t.ty[b]));
    m.C1[b] = make_float4(float(t.cs[b]), float(t.aL[b]), float(t.area[b]), float(t.aLsy[b]));
}

// Section constants of beam b: (kb, kt, my, ty) and (cs, area L0, area, area L0 yield).  The
// circular-section form derives them from r and L0 (area = pi r^2, I = pi r^4 / 4, J = 2 I:
// kb = E I / L0, kt = G J / L0, my = yield I / r, ty = yield / sqrt 3 J / r,
// cs = shear G area L0 / 2, MC/src/sim.cpp:115, 139-141); each is a few FP32 roundings from
// the FP64 value, which the mixed form's tolerance covers.
template <bool kStreamed>
__device__ __forceinline__ void section_constants(const MixedBeams& m, int b, float r, float L0, const float4 ic,
                                                  float4& C0, float4& C1) {
    if (kStreamed) {
        C0 = m.C0[b];
        C1 = m.C1[b];
    } else {
        const float r2 = r * r, r3 = r2 * r, r4 = r2 * r2, inv = 1.f / L0, r2L = r2 * L0;
        C0 = make_float4(m.kg.x * r4 * inv, m.kg.y * r4 * inv, ic.y * r3, ic.z * r3);
        C1 = make_float4(m.kg.z * r2L, m.kg.w * r2L, m.kg.w * r2, ic.w * r2L);
    }
}

// ---- beam kernel (MC/src/sim.cpp:139-141, FP32 with the split above) ---------------------
// The per-beam records of beam b: base chord and c0, the two base shear vectors with L0 and
// |d0|, the base relative rotation, the plastic state and the radius.
struct BeamRec {
    float4 B0, B1, B2, B5, P0, P1;
};
// The node increments of its two ends and the base orientation of end a.
struct BeamNodes {
    float4 ua4, ub4, ea, eb, ra0;
};

// One beam: energies into ue (elastic) and up (plastic dissipation), its two end 6-vectors
// into the gradient slots, its trial state when `trials`.
template <bool kStreamed>
__device__ __forceinline__ void beam_mixed(const Material& mat, const MixedBeams& m, int trials, EvalBufs& e, int B, int b,
                                           const BeamRec& R, const BeamNodes& Nd, float4 ic, float& ue, float& up) {
    const float4 B0 = R.B0, B1 = R.B1, B2 = R.B2, B5 = R.B5, P0 = R.P0, P1 = R.P1;
    const float4 ua4 = Nd.ua4, ub4 = Nd.ub4, ea = Nd.ea, eb = Nd.eb, ra0 = Nd.ra0;
    const f3 d0 = xyz(B0), du = xyz(ub4) - xyz(ua4);
    const float c0 = B0.w, L0 = B1.w, Lb = B2.w;
    const float q = c0 + 2.f * fdot(d0, du) + fdot(du, du);  // |d|^2 - L0^2
    const f3 d = d0 + du;
    const float L = sqrtf(fmaxf(L0 * L0 + q, 0.f));
    float* sa = e.slotAf + 6 * size_t(b);
    float* sb = e.slotBf + 6 * size_t(b);
    if (L < 1e-10f) {
        ue = 1e8f * (1e-10f - L) * (1e-10f - L);
#pragma unroll
        for (int k = 0; k < 6; k++) { sa[k] = 0.f; sb[k] = 0.f; }
        if (trials) {
#pragma unroll
            for (int k = 0; k < 7; k++) { e.trial_nextf[k * size_t(B) + b] = 0.f; e.trial_auxf[k * size_t(B) + b] = 0.f; }
#pragma unroll
            for (int k = 0; k < 3; k++) e.trial_flags[k * size_t(B) + b] = 0;
        }
    } else {
        // Divisions are the approximate single-instruction form (__fdividef, relative
        // error ~2 ulp): every divisor is a length or a small positive sum, well inside
        // its range, and the form's error budget is set by FP32 itself.
        const float invL = __fdividef(1.f, L);
        const f3 tt = d * invL;
        const float eps = __fdividef(q, (L + L0) * L0);
        float4 C0, C1;  // (kb, kt, my, ty), (cs, aL, area, aLsy)
        section_constants<kStreamed>(m, b, P1.w, L0, ic, C0, C1);
        const float E = mat.Ef, H = mat.Hf, sy = ic.x;
        // axial
        const R1 ax = ret1(eps, P0.x, P0.y, E, sy, H);
        const float uax = C1.y * (ax.energy + ax.hard);
        const float dax = C1.w * ax.dg;
        f3 F = tt * (C1.z * ax.force);
        // shear from the split director/chord differences
        const f3 va = xyz(make_float4(ea.y, ea.z, ea.w, 0.f)), vb = xyz(make_float4(eb.y, eb.z, eb.w, 0.f));
        const float wa = 1.f + ea.x, wb = 1.f + eb.x;
        // base directors d_a0 = t0 + s_a0, d_b0 = t0 + s_b0: they only enter multiplied by
        // a small vector (the rotation increment, the shear vector), so the ~1e-7 of the
        // FP32 t0 is harmless; the small s_a0, s_b0 themselves come exact from FP64
        const f3 sa0 = xyz(B1), sb0 = xyz(B2);
        const float invLb = __fdividef(1.f, Lb);
        const f3 t0 = d0 * invLb;
        const f3 da0 = t0 + sa0, db0 = t0 + sb0;
        const f3 dda = rot_inc(wa, va, da0), ddb = rot_inc(wb, vb, db0);
        const f3 da = da0 + dda, db = db0 + ddb;
        const float dLb = __fdividef(2.f * fdot(d0, du) + fdot(du, du), L + Lb);
        const f3 tdiff = (du * Lb - d0 * dLb) * (invL * invLb);  // t - t0
        const f3 ma = dda + sa0 - tdiff, mb = ddb + sb0 - tdiff;
        const float cs = C1.x;
        const float us = .5f * cs * (fdot(ma, ma) + fdot(mb, mb));
        const f3 gt = (ma + mb) * (-cs);  // cs (2t - da - db)
        const f3 trans = (gt - tt * fdot(gt, tt)) * invL;
        F = F + trans;
        // -cs (d x t) = cs d x (d - t): the moment from the small shear vector, so the
        // independent FP32 roundings of d and t leave no residual moment at rest
        f3 Ga = fcross(da, ma) * cs;
        f3 Gb = fcross(db, mb) * cs;
        // relative rotation (Ra0^* delta Ra0) Q0, delta = e_a^* e_b, near-identity forms
        const float dw1 = ea.x + eb.x + ea.x * eb.x + fdot(va, vb);
        const f3 dv0 = (vb - va) + vb * ea.x - va * eb.x - fcross(va, vb);
        const f3 ra0v{ra0.y, ra0.z, ra0.w};
        const f3 dv = rot_conj(ra0.x, ra0v, dv0);
        const float a0 = B5.x;
        const f3 v0{B5.y, B5.z, B5.w};
        const float qw1 = dw1 + a0 + dw1 * a0 - fdot(dv, v0);
        f3 qv = dv + v0 + v0 * dw1 + dv * a0 + fcross(dv, v0);
        float qw = 1.f + qw1;
        if (qw < 0.f) { qw = -qw; qv = -qv; }
        const f3 phi = rotvec_f(qw, qv);
        // axis = unit(Ra^T t), Ra = e_a Ra0
        f3 ax_ = rot_conj(ra0.x, ra0v, rot_conj(wa, va, tt));
        const float al2 = fdot(ax_, ax_);
        const f3 axis = (isfinite(al2) && al2 > 1e-30f) ? ax_ * rsqrtf(al2) : f3{0.f, 1.f, 0.f};
        const f3 rotp{P1.x, P1.y, P1.z};
        const float tw = fdot(phi, axis), ptw = fdot(rotp, axis);
        const f3 bend = phi - axis * tw, pbv = rotp - axis * ptw;
        const float kb = C0.x, kt = C0.y, my = C0.z, ty = C0.w;
        const R3 br = ret3(bend, pbv, P0.z, kb, my, mat.bend_hf * kb);
        const R1 tor = ret1(tw, ptw, P0.w, kt, ty, mat.torsion_hf * kt);
        const f3 moment = br.force + axis * tor.force;
        const float ur = br.energy + br.hard + tor.energy + tor.hard;
        const float dr = my * br.dg + ty * tor.dg;
        const f3 world = rot(wa, va, rot(ra0.x, ra0v, jl_inv_t_f(phi, moment)));
        Ga = Ga - world;
        Gb = Gb + world;
        ue = uax + us + ur;
        up = dax + dr;
        sa[0] = -F.x; sa[1] = -F.y; sa[2] = -F.z; sa[3] = Ga.x; sa[4] = Ga.y; sa[5] = Ga.z;
        sb[0] = F.x;  sb[1] = F.y;  sb[2] = F.z;  sb[3] = Gb.x; sb[4] = Gb.y; sb[5] = Gb.z;
        if (trials) {
            const size_t S = size_t(B);
            const f3 nrot = br.p + axis * tor.p;
            e.trial_nextf[b] = ax.p;
            e.trial_nextf[S + b] = ax.a;
            e.trial_nextf[2 * S + b] = nrot.x;
            e.trial_nextf[3 * S + b] = nrot.y;
            e.trial_nextf[4 * S + b] = nrot.z;
            e.trial_nextf[5 * S + b] = br.a;
            e.trial_nextf[6 * S + b] = tor.a;
            e.trial_auxf[b] = eps;
            e.trial_auxf[S + b] = ax.force;
            e.trial_auxf[2 * S + b] = moment.x;
            e.trial_auxf[3 * S + b] = moment.y;
            e.trial_auxf[4 * S + b] = moment.z;
            e.trial_auxf[5 * S + b] = ue;
            e.trial_auxf[6 * S + b] = up;
            e.trial_flags[b] = ax.yielded;
            e.trial_flags[S + b] = br.yielded;
            e.trial_flags[2 * S + b] = tor.yielded;
        }
    }
}

// Both halves of a node's increment record share one 32-byte sector.
__device__ __forceinline__ BeamNodes load_nodes(int2 ab, const float4* __restrict__ UE, const float4* __restrict__ R0f) {
    const float4* a = UE + 2 * size_t(ab.x);
    const float4* b = UE + 2 * size_t(ab.y);
    return BeamNodes{a[0], b[0], a[1], b[1], R0f[ab.x]};
}

// Block totals: warp 0 sums the elastic and the plastic energies of the block (compensated,
// fixed order) while the other warps only store theirs; the beam energy total is the FP64
// sum of the two.  All threads call it; sm holds 2 kBlock floats.
__device__ __forceinline__ void beam_block_totals(float ue, float up, float* sm, double* out3) {
    sm[threadIdx.x] = ue;
    sm[kBlock + threadIdx.x] = up;
    __syncthreads();
    if (threadIdx.x < 32) {
        const double se = warp_sum_smem(sm, threadIdx.x);
        const double sp = warp_sum_smem(sm + kBlock, threadIdx.x);
        if (threadIdx.x == 0) {
            out3[0] = se + sp;
            out3[1] = se;
            out3[2] = sp;
        }
    }
}

// kMinBlocks: the occupancy variant (CTAs per SM), picked by mcg_autotune.
template <bool kStreamed, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_beams_mixed(DevTopo t, Material mat, MixedBeams m, int trials,
                                                        const float4* __restrict__ UE,
                                                        const float4* __restrict__ R0f, EvalBufs e) {
    __shared__ float sm[2 * kBlock];  // per-thread elastic and plastic energies
    const MapPos mp = map_pos(t.bblk);
    if (!t.active[mp.inst]) return;
    if (trials == 2) trials = t.trial_inst[mp.inst];  // per instance (device-resident solver)
    float ue = 0.f, up = 0.f;  // elastic energy, plastic dissipation of this beam
    if (mp.valid) {
        // Every load is issued here, before any arithmetic: the streamed beam records and,
        // one step behind the end indices, the node increments, so that each thread keeps
        // all of its memory requests in flight at once (the kernel is latency-bound).
        const int b = mp.i;
        const int2 ab = t.ab[b];
        const BeamRec R{m.B0[b], m.B1[b], m.B2[b], m.B5[b], m.P0[b], m.P1[b]};
        const BeamNodes Nd = load_nodes(ab, UE, R0f);
        beam_mixed<kStreamed>(mat, m, trials, e, t.B, b, R, Nd, m.ic[mp.inst], ue, up);
    }
    beam_block_totals(ue, up, sm, e.part_beam + 3 * size_t(blockIdx.x));
}

// ---- the same kernel with its records staged by bulk copies --------------------------------
// Persistent CTAs (kMinBlocks per SM) walk the beam blocks b = blockIdx.x, + gridDim.x, ...;
// the six float4 records of a block's beams (4 KB each, contiguous) arrive in shared memory
// by cp.async.bulk on an mbarrier, two blocks ahead of the arithmetic (double buffer), so
// the streamed bytes are in flight during a whole block's computation without holding
// registers; the threads still load the end indices and the node increments (mostly L2
// hits) themselves.  Arithmetic, block partials and their order are those of
// k_beams_mixed, bit for bit.  Every wait on a barrier is bounded: one that gives up sets
// e.err (the host reports it), waits (bounded) for the CTA's copies in flight and returns.
constexpr int kStageFields = 6;
constexpr unsigned kStageWaitPolls = 1u << 20;  // a normal wait ends within microseconds

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for the phase of `parity` to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    for (unsigned it = 0; it < kStageWaitPolls; it++)
        if (mbar_test(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

template <bool kStreamed, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_beams_mixed_staged(DevTopo t, Material mat, MixedBeams m,
                                                                           int trials, const float4* __restrict__ UE,
                                                                           const float4* __restrict__ R0f, EvalBufs e) {
    extern __shared__ __align__(128) float4 stage[];  // [2][kStageFields][kBlock]
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ float sm[2 * kBlock];
    const int nt = t.n_bblk, G = int(gridDim.x);
    const float4* src[kStageFields] = {m.B0, m.B1, m.B2, m.B5, m.P0, m.P1};
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // tile i of this CTA is beam block blockIdx.x + i G; thread 0 issues its copies (a
    // plain arrival for an inactive instance, whose block is skipped)
    auto issue = [&](int i) {
        const int vb = int(blockIdx.x) + i * G;
        if (vb >= nt) return;
        const int4 q = t.bblk[vb];
        uint64_t* br = &bar[i & 1];
        if (!t.active[q.z] || q.y <= 0) {
            mbar_arrive(br);
            return;
        }
        const unsigned bytes = unsigned(q.y) * 16u;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // after the generic reads
        mbar_arrive_tx(br, kStageFields * bytes);
        float4* dst = stage + size_t(i & 1) * kStageFields * kBlock;
        for (int f = 0; f < kStageFields; f++) bulk_to_smem(dst + f * kBlock, src[f] + q.x, bytes, br);
    };
    if (threadIdx.x == 0) {
        issue(0);
        issue(1);
    }
    for (int i = 0;; i++) {
        const int vb = int(blockIdx.x) + i * G;
        if (vb >= nt) break;
        const int4 q = t.bblk[vb];
        const bool ok = __syncthreads_and(mbar_wait(&bar[i & 1], unsigned(i >> 1) & 1u));
        if (!ok) {
            // give up: report, let the copies in flight land (bounded), return
            if (threadIdx.x == 0) {
                atomicOr(e.err, 1u);
                mbar_wait(&bar[i & 1], unsigned(i >> 1) & 1u);
                if (vb + G < nt) mbar_wait(&bar[(i + 1) & 1], unsigned((i + 1) >> 1) & 1u);
            }
            __syncthreads();
            return;
        }
        if (t.active[q.z]) {  // block-uniform
            const int tr = trials == 2 ? int(t.trial_inst[q.z]) : trials;
            float ue = 0.f, up = 0.f;
            if (int(threadIdx.x) < q.y) {
                const int b = q.x + int(threadIdx.x);
                const int2 ab = t.ab[b];
                const BeamNodes Nd = load_nodes(ab, UE, R0f);
                const float4* st = stage + size_t(i & 1) * kStageFields * kBlock + threadIdx.x;
                const BeamRec R{st[0], st[kBlock], st[2 * kBlock], st[3 * kBlock], st[4 * kBlock], st[5 * kBlock]};
                beam_mixed<kStreamed>(mat, m, tr, e, t.B, b, R, Nd, m.ic[q.z], ue, up);
            }
            beam_block_totals(ue, up, sm, e.part_beam + 3 * size_t(vb));
        }
        __syncthreads();  // every read of this buffer (and of sm) is done
        if (threadIdx.x == 0) issue(i + 2);
    }
}

// Plastic state of the mixed form: (epsp, alpha, alphaB, alphaT) and rotp as float4 pairs,
// from/to the 7-array SoA trial layout.
__global__ void __launch_bounds__(kBlock) k_plastic_pack(DevTopo t, const uint8_t* __restrict__ mask,
                                                         const float* __restrict__ soa7, float4* __restrict__ P0,
                                                         float4* __restrict__ P1) {
    const MapPos mp = map_pos(t.bblk);
    if (!mp.valid || (mask && !mask[mp.inst])) return;
    const int b = mp.i;
    const size_t S = size_t(t.B);
    P0[b] = make_float4(soa7[b], soa7[S + b], soa7[5 * S + b], soa7[6 * S + b]);
    P1[b] = make_float4(soa7[2 * S + b], soa7[3 * S + b], soa7[4 * S + b], float(t.radius[b]));
}
__global__ void __launch_bounds__(kBlock) k_plastic_from_f64(int B, const double* __restrict__ soa7,
                                                             const double* __restrict__ radius,
                                                             float4* __restrict__ P0, float4* __restrict__ P1) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const size_t S = size_t(B);
    P0[b] = make_float4(float(soa7[b]), float(soa7[S + b]), float(soa7[5 * S + b]), float(soa7[6 * S + b]));
    P1[b] = make_float4(float(soa7[2 * S + b]), float(soa7[3 * S + b]), float(soa7[4 * S + b]), float(radius[b]));
}
__global__ void __launch_bounds__(kBlock) k_plastic_to_f64(DevTopo t, const uint8_t* __restrict__ mask,
                                                           const float4* __restrict__ P0,
                                                           const float4* __restrict__ P1, double* __restrict__ soa7) {
    const MapPos mp = map_pos(t.bblk);
    if (!mp.valid || (mask && !mask[mp.inst])) return;
    const int b = mp.i;
    const size_t S = size_t(t.B);
    const float4 p = P0[b], r = P1[b];
    soa7[b] = p.x; soa7[S + b] = p.y; soa7[2 * S + b] = r.x; soa7[3 * S + b] = r.y; soa7[4 * S + b] = r.z;
    soa7[5 * S + b] = p.z; soa7[6 * S + b] = p.w;
}
__global__ void k_f32_to_f64(long long n, const float* __restrict__ a, double* __restrict__ o) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        o[i] = a[i];
}

}  // namespace

void launch_state_mixed(const DevTopo& t, const PhysParams& p, const double* z, const double* base_x,
                        const MixedNodes& mn, EvalBufs& e, cudaStream_t s) {
    k_state_mixed<<<t.n_nblk, kBlock, 0, s>>>(t, p.translation_scale, z, base_x, mn.UE, e.x, e.xf_lo, e.xf_hi,
                                              e.part_state);
    note_launches(1);
    launch_center(t, e, s);
}

// Variants of the mixed beam kernel: the plain kernel at 3, 4, 5 or 6 CTAs per SM, and the
// kernel with bulk-copy staged records at 3 or 4 (reported as -3, -4); the
// streamed-constants form (sections that are not circular) has the default one only.
constexpr int kMixedBlocks[] = {3, 4, 5, 6, -3, -4};
int beams_mixed_variants() { return 6; }
int beams_mixed_blocks(int v) { return kMixedBlocks[v]; }

namespace {
constexpr size_t kStageBytes = size_t(2) * kStageFields * kBlock * sizeof(float4);
int g_stage_sms = 0;  // SMs of the device (set by prepare_beams_mixed)
template <int kMin>
void launch_staged(const DevTopo& t, const Material& m, const MixedBeams& mb, const MixedNodes& mn, int tr, EvalBufs& e,
                   cudaStream_t s) {
    const int grid = std::min(t.n_bblk, kMin * std::max(g_stage_sms, 1));  // persistent: all resident
    k_beams_mixed_staged<false, kMin><<<grid, kBlock, kStageBytes, s>>>(t, m, mb, tr, mn.UE, mn.R0f, e);
}
}  // namespace

void prepare_beams_mixed(int device) {
    cudaDeviceGetAttribute(&g_stage_sms, cudaDevAttrMultiProcessorCount, device);
    cudaFuncSetAttribute(k_beams_mixed_staged<false, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStageBytes));
    cudaFuncSetAttribute(k_beams_mixed_staged<false, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStageBytes));
}

void launch_beams_mixed(const DevTopo& t, const Material& m, const MixedBeams& mb, const MixedNodes& mn, int trials,
                        EvalBufs& e, cudaStream_t s, int variant) {
    if (t.B == 0) return;
    const int tr = trials;  // 0, 1, or 2: per instance (t.trial_inst)
    if (mb.C0) {
        k_beams_mixed<true, kMixedBlocks[0]><<<t.n_bblk, kBlock, 0, s>>>(t, m, mb, tr, mn.UE, mn.R0f, e);
    } else {
        switch (variant) {
            case 1: k_beams_mixed<false, kMixedBlocks[1]><<<t.n_bblk, kBlock, 0, s>>>(t, m, mb, tr, mn.UE, mn.R0f, e); break;
            case 2: k_beams_mixed<false, kMixedBlocks[2]><<<t.n_bblk, kBlock, 0, s>>>(t, m, mb, tr, mn.UE, mn.R0f, e); break;
            case 3: k_beams_mixed<false, kMixedBlocks[3]><<<t.n_bblk, kBlock, 0, s>>>(t, m, mb, tr, mn.UE, mn.R0f, e); break;
            case 4: launch_staged<3>(t, m, mb, mn, tr, e, s); break;
            case 5: launch_staged<4>(t, m, mb, mn, tr, e, s); break;
            default: k_beams_mixed<false, kMixedBlocks[0]><<<t.n_bblk, kBlock, 0, s>>>(t, m, mb, tr, mn.UE, mn.R0f, e); break;
        }
    }
    note_launches(1);
}

void launch_rebase_mixed(const DevTopo& t, const double* base_x, const double* base_r, MixedBeams& mb,
                         MixedNodes& mn, cudaStream_t s) {
    k_rebase_nodes<<<grid_for(t.N), kBlock, 0, s>>>(t.N, base_r, mn.R0f);
    note_launches(1);
    if (t.B) {
        k_rebase_beams<<<grid_for(t.B), kBlock, 0, s>>>(t, base_x, base_r, mb);
        note_launches(1);
    }
}

void launch_mixed_constants(const DevTopo& t, MixedBeams& mb, cudaStream_t s) {
    if (!t.B || !mb.C0) return;
    k_mixed_constants<<<grid_for(t.B), kBlock, 0, s>>>(t, mb);
    note_launches(1);
}

void launch_plastic_mixed(const DevTopo& t, const uint8_t* mask, const double* plastic64, const float* trial32,
                          MixedBeams& mb, cudaStream_t s) {
    if (!t.B) return;
    if (trial32) k_plastic_pack<<<t.n_bblk, kBlock, 0, s>>>(t, mask, trial32, mb.P0, mb.P1);
    else k_plastic_from_f64<<<grid_for(t.B), kBlock, 0, s>>>(t.B, plastic64, t.radius, mb.P0, mb.P1);
    note_launches(1);
}

void launch_plastic_mixed_to_f64(const DevTopo& t, const uint8_t* mask, const MixedBeams& mb, double* plastic64,
                                 cudaStream_t s) {
    if (!t.B) return;
    k_plastic_to_f64<<<t.n_bblk, kBlock, 0, s>>>(t, mask, mb.P0, mb.P1, plastic64);
    note_launches(1);
}

void launch_f32_to_f64(long long n, const float* a, double* o, cudaStream_t s) {
    if (n <= 0) return;
    k_f32_to_f64<<<grid_for(n < 152 * 8 * kBlock ? n : 152 * 8 * kBlock), kBlock, 0, s>>>(n, a, o);
    note_launches(1);
}

}  // namespace mcg
