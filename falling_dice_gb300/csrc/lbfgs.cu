// lbfgs.cu -- device vector kernels of the L-BFGS minimizer
// (the reference's Simulator::minimize and helpers, MC/src/sim.cpp:42-46, 174-211), for every
// instance of a context at once.
//
// Vectors hold 6 entries per node in the ABI layout; all instances' nodes are stored one
// after another and every kernel runs over the node blocks of the context (a block never
// straddles two instances).  Each instance has its own solver state (history count, ring
// head, line-search step, which operations it takes part in), written by the host into a
// small control array before each step.  Dot products are per-block partial sums (each
// thread its node's six products in order, then a fixed tree) and one block per instance
// summing its blocks in order: the same partition whether an instance is solved alone or
// with others, so a batch reproduces the separate runs bit for bit.  The two-loop scalars
// (alpha_h, H0) never leave the device.
#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

__device__ __forceinline__ const double* hist_slot(const double* base, long long stride, int slot) {
    return base + stride * slot;
}

// Slot of the h-th oldest history pair of an instance.
__device__ __forceinline__ int ring_slot(const SolveCtl& c, int H, int h) { return (c.head + h) % H; }

// An instance's control record with its history state (pairs held, oldest slot), which
// lives on the device: the solver kernels update it themselves.
__device__ __forceinline__ SolveCtl load_ctl(const SolveCtl* __restrict__ ctl, const int2* __restrict__ hist, int inst) {
    SolveCtl c = ctl[inst];
    const int2 h = hist[inst];
    c.m = h.x;
    c.head = h.y;
    return c;
}

// One instance's sum of its block partials part[k * nblk + b], b in its node-block range,
// for k < K (one block per instance; fixed order).
template <int K>
__device__ __forceinline__ void instance_sum(const DevTopo& t, const double* __restrict__ part, int inst,
                                             double (&acc)[K], double* sm) {
    const int4 r = t.irange[inst];
#pragma unroll
    for (int k = 0; k < K; k++) acc[k] = 0;
    for (int b = r.x + int(threadIdx.x); b < r.y; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] += part[size_t(k) * t.n_nblk + b];
    block_sum<K>(acc, sm);
}

__device__ __forceinline__ double dot6(const double* a, const double* b) {
    double s = a[0] * b[0];
    s += a[1] * b[1];
    s += a[2] * b[2];
    s += a[3] * b[3];
    s += a[4] * b[4];
    s += a[5] * b[5];
    return s;
}

// ---- two-loop recursion (sim.cpp:184-187) -----------------------------------------------
// Step j of loop LOOP for the instances computing a direction with j < m.  Every block of
// an instance sums the instance's partials of step j's dot product (in `cur`, same order in
// each block) into the coefficient and updates its nodes of p; when j + 1 < m it then writes
// its partial of step j + 1's dot product with the updated p to `nxt`.
//   loop 1 (newest first, h = m - 1 - j): alpha = rho <s, p> (kept), p -= alpha y;
//   loop 2 (oldest first, h = j):         beta = rho <y, p>, p += s (alpha - beta).
template <int LOOP>
__global__ void __launch_bounds__(kBlock) k_tl_step(DevTopo t, const SolveCtl* __restrict__ ctl,
                                                    const int2* __restrict__ hist, int H, int j,
                                                    double* __restrict__ p, const double* __restrict__ S,
                                                    const double* __restrict__ Y, long long stride,
                                                    const double* __restrict__ rho, double* __restrict__ alpha,
                                                    const double* __restrict__ cur, double* __restrict__ nxt) {
    __shared__ double sm[kBlock / 32];
    __shared__ double coef;
    const MapPos mp = map_pos(t.nblk);
    const SolveCtl c = load_ctl(ctl, hist, mp.inst);
    if (!(c.flags & kOpDirection) || j >= c.m) return;  // block-uniform
    const int h = LOOP == 1 ? c.m - 1 - j : j;
    const int slot = ring_slot(c, H, h);
    double acc[1];
    instance_sum<1>(t, cur, mp.inst, acc, sm);
    if (threadIdx.x == 0) {
        const double r = rho[size_t(mp.inst) * H + slot] * acc[0];
        if (LOOP == 1) {
            coef = r;
            if (blockIdx.x == t.irange[mp.inst].x) alpha[size_t(mp.inst) * H + h] = r;
        } else {
            coef = alpha[size_t(mp.inst) * H + h] - r;
        }
    }
    __syncthreads();
    const double k = coef;
    double pn[6] = {0, 0, 0, 0, 0, 0};
    if (mp.valid) {
        double* pi = p + 6 * size_t(mp.i);
        if (LOOP == 1) {
            const double* y = hist_slot(Y, stride, slot) + 6 * size_t(mp.i);
#pragma unroll
            for (int d = 0; d < 6; d++) pn[d] = pi[d] - k * y[d];
        } else {
            const double* sv = hist_slot(S, stride, slot) + 6 * size_t(mp.i);
#pragma unroll
            for (int d = 0; d < 6; d++) pn[d] = pi[d] + sv[d] * k;
        }
#pragma unroll
        for (int d = 0; d < 6; d++) pi[d] = pn[d];
    }
    if (j + 1 >= c.m) return;  // block-uniform
    const int slot2 = ring_slot(c, H, LOOP == 1 ? c.m - 2 - j : j + 1);
    const double* v = hist_slot(LOOP == 1 ? S : Y, stride, slot2);
    double a2[1] = {0};
    if (mp.valid) a2[0] = dot6(v + 6 * size_t(mp.i), pn);
    block_sum<1>(a2, sm);
    if (threadIdx.x == 0) nxt[blockIdx.x] = a2[0];
}

// Partials of <s, y> and <y, y> of the newest pair (for H0, into h0part), the copy p = g
// that starts the recursion and the partial of loop 1's first dot product <s, g> (into
// part0).
__global__ void __launch_bounds__(kBlock) k_tl_start(DevTopo t, const SolveCtl* __restrict__ ctl, const int2* __restrict__ hist, int H,
                                                     double* __restrict__ p, const double* __restrict__ g,
                                                     const double* __restrict__ S, const double* __restrict__ Y,
                                                     long long stride, double* __restrict__ h0part,
                                                     double* __restrict__ part0) {
    __shared__ double sm[3 * (kBlock / 32)];
    const MapPos mp = map_pos(t.nblk);
    const SolveCtl c = load_ctl(ctl, hist, mp.inst);
    if (!(c.flags & kOpDirection)) return;
    if (mp.valid)
#pragma unroll
        for (int d = 0; d < 6; d++) p[6 * size_t(mp.i) + d] = g[6 * size_t(mp.i) + d];
    if (c.m == 0) return;
    const int slot = ring_slot(c, H, c.m - 1);
    double acc[3] = {0, 0, 0};
    if (mp.valid) {
        const double* s = hist_slot(S, stride, slot) + 6 * size_t(mp.i);
        const double* y = hist_slot(Y, stride, slot) + 6 * size_t(mp.i);
        acc[0] = dot6(s, y);
        acc[1] = dot6(y, y);
        acc[2] = dot6(s, g + 6 * size_t(mp.i));
    }
    block_sum<3>(acc, sm);
    if (threadIdx.x == 0) {
        h0part[blockIdx.x] = acc[0];
        h0part[size_t(t.n_nblk) + blockIdx.x] = acc[1];
        part0[blockIdx.x] = acc[2];
    }
}

// p *= H0, H0 = clamp(sy/yy, 1e-7, 1e4) when both are positive, else 0.1 (sim.cpp:186), and
// the partial of loop 2's first dot product <y, p> (into part0).
__global__ void __launch_bounds__(kBlock) k_tl_scale(DevTopo t, const SolveCtl* __restrict__ ctl, const int2* __restrict__ hist,
                                                     int H, double* __restrict__ p, const double* __restrict__ Y,
                                                     long long stride, const double* __restrict__ h0part,
                                                     double* __restrict__ part0) {
    __shared__ double sm[2 * (kBlock / 32)];
    __shared__ double h0;
    const MapPos mp = map_pos(t.nblk);
    const SolveCtl c = load_ctl(ctl, hist, mp.inst);
    if (!(c.flags & kOpDirection)) return;
    if (c.m > 0) {
        double acc[2];
        instance_sum<2>(t, h0part, mp.inst, acc, sm);
        if (threadIdx.x == 0) {
            double v = .10;
            if (acc[0] > 1e-20 && acc[1] > 1e-20) v = clampd(acc[0] / acc[1], 1e-7, 1e4);
            h0 = v;
        }
    } else if (threadIdx.x == 0) {
        h0 = .10;
    }
    __syncthreads();
    const double k = h0;
    double pn[6] = {0, 0, 0, 0, 0, 0};
    if (mp.valid)
#pragma unroll
        for (int d = 0; d < 6; d++) {
            pn[d] = p[6 * size_t(mp.i) + d] * k;
            p[6 * size_t(mp.i) + d] = pn[d];
        }
    if (c.m == 0) return;  // block-uniform
    const double* v = hist_slot(Y, stride, ring_slot(c, H, 0));
    double a2[1] = {0};
    if (mp.valid) a2[0] = dot6(v + 6 * size_t(mp.i), pn);
    block_sum<1>(a2, sm);
    if (threadIdx.x == 0) part0[blockIdx.x] = a2[0];
}

// Direction finish for the instances with `bit` set: p = clamp(lock(-src)) per node
// (sim.cpp:188-190, clampDirection sim.cpp:46), and the partial of <g, p>.
__global__ void __launch_bounds__(kBlock) k_finish(DevTopo t, const SolveCtl* __restrict__ ctl, int bit,
                                                   double* __restrict__ p, const double* __restrict__ src,
                                                   const double* __restrict__ g, double mt, double mr,
                                                   double* __restrict__ part) {
    __shared__ double sm[kBlock / 32];
    const MapPos mp = map_pos(t.nblk);
    if (!(ctl[mp.inst].flags & bit)) return;
    double acc[1] = {0};
    if (mp.valid) {
        const size_t b = 6 * size_t(mp.i);
        const uint8_t* lk = t.locked + b;
        double v[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            v[k] = -src[b + k];
            if (lk[k]) v[k] = 0;
        }
        const double lt = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (lt > mt) {
            const double f = mt / lt;
            v[0] *= f; v[1] *= f; v[2] *= f;
        }
        const double lr = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
        if (lr > mr) {
            const double f = mr / lr;
            v[3] *= f; v[4] *= f; v[5] *= f;
        }
#pragma unroll
        for (int k = 0; k < 6; k++) {
            v[k] = lk[k] ? 0.0 : v[k];
            p[b + k] = v[k];
        }
        acc[0] = dot6(g + b, v);
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
}

// One block per instance with `bit` set: out[K i + k] = sum of its partials.
template <int K>
__global__ void __launch_bounds__(kBlock) k_inst_final(DevTopo t, const SolveCtl* __restrict__ ctl, int bit,
                                                       const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sm[K * (kBlock / 32)];
    const int inst = blockIdx.x;
    if (!(ctl[inst].flags & bit)) return;
    double acc[K];
    instance_sum<K>(t, part, inst, acc, sm);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; k++) out[size_t(K) * inst + k] = acc[k];
}

// ---- vectors around an evaluation ------------------------------------------------------------
// Per node, in this order for each instance's flags: z = 0 (kOpZero), z = best (kOpRestore),
// best = z (kOpKeepBest), zeval = z + step p with locked entries 0 (kOpCandidate, sim.cpp:179)
// or zeval = z (kOpEvalAtZ), zfinal = z (kOpFinal).
__global__ void __launch_bounds__(kBlock) k_prepare(DevTopo t, const SolveCtl* __restrict__ ctl,
                                                    double* __restrict__ z, double* __restrict__ best,
                                                    double* __restrict__ zeval, const double* __restrict__ p,
                                                    double* __restrict__ zfinal) {
    const MapPos mp = map_pos(t.nblk);
    const SolveCtl c = ctl[mp.inst];
    if (!mp.valid || !(c.flags & (kOpZero | kOpRestore | kOpKeepBest | kOpCandidate | kOpEvalAtZ | kOpFinal))) return;
    const size_t b = 6 * size_t(mp.i);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        double v = z[b + k];
        if (c.flags & kOpZero) v = 0;
        if (c.flags & kOpRestore) v = best[b + k];
        z[b + k] = v;
        if (c.flags & kOpKeepBest) best[b + k] = v;
        if (c.flags & kOpCandidate) zeval[b + k] = t.locked[b + k] ? 0.0 : v + c.step * p[b + k];
        if (c.flags & kOpEvalAtZ) zeval[b + k] = v;
        if (c.flags & kOpFinal) zfinal[b + k] = v;
    }
}

// After an evaluation: g = geval for the instances that evaluated at z (kOpTakeGrad), and
// for accepted trials (kOpAccept, sim.cpp:205-206) s = zeval - z, y = geval - g into the
// history slot `target` (kOpPair), the partials of <s, y>, <s, s>, <y, y>, then z = zeval,
// g = geval; best = z afterwards when kOpKeepBestAfter.
__global__ void __launch_bounds__(kBlock) k_accept(DevTopo t, const SolveCtl* __restrict__ ctl, const int2* __restrict__ hist,
                                                   int H, double* __restrict__ z, double* __restrict__ g,
                                                   const double* __restrict__ zeval, const double* __restrict__ geval,
                                                   double* __restrict__ S, double* __restrict__ Y, long long stride,
                                                   double* __restrict__ best, double* __restrict__ part) {
    __shared__ double sm[3 * (kBlock / 32)];
    const MapPos mp = map_pos(t.nblk);
    const SolveCtl c = load_ctl(ctl, hist, mp.inst);
    if (!(c.flags & (kOpTakeGrad | kOpAccept))) return;
    const size_t b = 6 * size_t(mp.i);
    if (c.flags & kOpTakeGrad) {
        if (mp.valid)
#pragma unroll
            for (int k = 0; k < 6; k++) g[b + k] = geval[b + k];
        return;
    }
    double acc[3] = {0, 0, 0};
    if (mp.valid) {
        double sv[6], yv[6];
#pragma unroll
        for (int k = 0; k < 6; k++) {
            sv[k] = zeval[b + k] - z[b + k];
            yv[k] = geval[b + k] - g[b + k];
        }
        if (c.flags & kOpPair) {
            const int target = c.m < H ? (c.head + c.m) % H : c.head;
            double* s = S + stride * target + b;
            double* y = Y + stride * target + b;
#pragma unroll
            for (int k = 0; k < 6; k++) {
                s[k] = sv[k];
                y[k] = yv[k];
            }
        }
        acc[0] = dot6(sv, yv);
        acc[1] = dot6(sv, sv);
        acc[2] = dot6(yv, yv);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            z[b + k] = zeval[b + k];
            g[b + k] = geval[b + k];
        }
        if (c.flags & kOpKeepBestAfter)
#pragma unroll
            for (int k = 0; k < 6; k++) best[b + k] = zeval[b + k];
    }
    block_sum<3>(acc, sm);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = acc[0];
        part[size_t(t.n_nblk) + blockIdx.x] = acc[1];
        part[2 * size_t(t.n_nblk) + blockIdx.x] = acc[2];
    }
}

// ---- the whole direction in one CTA per instance ---------------------------------------------
// For instances of at most kFuseChunks node blocks: the same steps as k_tl_start ...
// k_finish + k_inst_final (each block partial here is one chunk of kBlock nodes reduced by the
// same tree, each instance sum the same strided tree), so the result is bit for bit that of
// the multi-launch path; one launch instead of 2 H + 4.
constexpr int kFuseChunks = 64;

// Partial of one chunk: thread t the node first + t (if valid), then the block tree.
__device__ __forceinline__ double chunk_dot(const double* a, const double* b, int first, int count, double* sm) {
    double acc[1] = {0};
    if (int(threadIdx.x) < count) acc[0] = dot6(a + 6 * size_t(first + threadIdx.x), b + 6 * size_t(first + threadIdx.x));
    block_sum<1>(acc, sm);
    return acc[0];
}

// Sum of nchunk partials held in shared memory, strided as instance_sum.
template <int K>
__device__ __forceinline__ void chunk_sum(const double (*part)[kFuseChunks], int nchunk, double (&acc)[K], double* sm) {
#pragma unroll
    for (int k = 0; k < K; k++) acc[k] = 0;
    for (int b = int(threadIdx.x); b < nchunk; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] += part[k][b];
    block_sum<K>(acc, sm);
}

__global__ void __launch_bounds__(kBlock) k_direction_fused(DevTopo t, const SolveCtl* __restrict__ ctl, const int2* __restrict__ hist, int H,
                                                            double* __restrict__ p, const double* __restrict__ g,
                                                            const double* __restrict__ S, const double* __restrict__ Y,
                                                            long long stride, const double* __restrict__ rho,
                                                            double* __restrict__ dg, double mt, double mr) {
    __shared__ double sm[2 * (kBlock / 32)];
    __shared__ double part[2][kFuseChunks];
    __shared__ double alpha[64];
    __shared__ double coef;
    const int inst = blockIdx.x;
    const SolveCtl c = load_ctl(ctl, hist, inst);
    if (!(c.flags & kOpDirFused)) return;
    const int4 r = t.irange[inst];
    const int nchunk = r.y - r.x;
    // p = g; partials of <s, y>, <y, y> of the newest pair
    for (int b = 0; b < nchunk; b++) {
        const int4 q = t.nblk[r.x + b];
        if (int(threadIdx.x) < q.y)
#pragma unroll
            for (int d = 0; d < 6; d++) p[6 * size_t(q.x + threadIdx.x) + d] = g[6 * size_t(q.x + threadIdx.x) + d];
        if (c.m > 0) {
            const int slot = ring_slot(c, H, c.m - 1);
            double acc[2] = {0, 0};
            if (int(threadIdx.x) < q.y) {
                const double* sv = hist_slot(S, stride, slot) + 6 * size_t(q.x + threadIdx.x);
                const double* yv = hist_slot(Y, stride, slot) + 6 * size_t(q.x + threadIdx.x);
                acc[0] = dot6(sv, yv);
                acc[1] = dot6(yv, yv);
            }
            block_sum<2>(acc, sm);
            if (threadIdx.x == 0) {
                part[0][b] = acc[0];
                part[1][b] = acc[1];
            }
        }
    }
    __syncthreads();
    double h0acc[2] = {0, 0};
    if (c.m > 0) chunk_sum<2>(part, nchunk, h0acc, sm);
    __syncthreads();
    // loop 1, newest first
    for (int j = 0; j < c.m; j++) {
        const int h = c.m - 1 - j, slot = ring_slot(c, H, h);
        for (int b = 0; b < nchunk; b++) {
            const int4 q = t.nblk[r.x + b];
            const double v = chunk_dot(hist_slot(S, stride, slot), p, q.x, q.y, sm);
            if (threadIdx.x == 0) part[0][b] = v;
        }
        __syncthreads();
        double acc[1];
        chunk_sum<1>(part, nchunk, acc, sm);
        if (threadIdx.x == 0) {
            coef = rho[size_t(inst) * H + slot] * acc[0];
            alpha[h] = coef;
        }
        __syncthreads();
        const double k = coef;
        const double* yv = hist_slot(Y, stride, slot);
        for (int b = 0; b < nchunk; b++) {
            const int4 q = t.nblk[r.x + b];
            if (int(threadIdx.x) < q.y)
#pragma unroll
                for (int d = 0; d < 6; d++) p[6 * size_t(q.x + threadIdx.x) + d] -= k * yv[6 * size_t(q.x + threadIdx.x) + d];
        }
        __syncthreads();
    }
    // H0 (sim.cpp:186); the block sums are complete in thread 0 only
    if (threadIdx.x == 0) {
        double v = .10;
        if (c.m > 0 && h0acc[0] > 1e-20 && h0acc[1] > 1e-20) v = clampd(h0acc[0] / h0acc[1], 1e-7, 1e4);
        coef = v;
    }
    __syncthreads();
    {
        const double v = coef;
        for (int b = 0; b < nchunk; b++) {
            const int4 q = t.nblk[r.x + b];
            if (int(threadIdx.x) < q.y)
#pragma unroll
                for (int d = 0; d < 6; d++) p[6 * size_t(q.x + threadIdx.x) + d] *= v;
        }
        __syncthreads();
    }
    // loop 2, oldest first
    for (int j = 0; j < c.m; j++) {
        const int slot = ring_slot(c, H, j);
        for (int b = 0; b < nchunk; b++) {
            const int4 q = t.nblk[r.x + b];
            const double v = chunk_dot(hist_slot(Y, stride, slot), p, q.x, q.y, sm);
            if (threadIdx.x == 0) part[0][b] = v;
        }
        __syncthreads();
        double acc[1];
        chunk_sum<1>(part, nchunk, acc, sm);
        if (threadIdx.x == 0) coef = alpha[j] - rho[size_t(inst) * H + slot] * acc[0];
        __syncthreads();
        const double k = coef;
        const double* sv = hist_slot(S, stride, slot);
        for (int b = 0; b < nchunk; b++) {
            const int4 q = t.nblk[r.x + b];
            if (int(threadIdx.x) < q.y)
#pragma unroll
                for (int d = 0; d < 6; d++) p[6 * size_t(q.x + threadIdx.x) + d] += sv[6 * size_t(q.x + threadIdx.x) + d] * k;
        }
        __syncthreads();
    }
    // finish: clamp (sim.cpp:188-190, 46) and <g, p>
    for (int b = 0; b < nchunk; b++) {
        const int4 q = t.nblk[r.x + b];
        double acc[1] = {0};
        if (int(threadIdx.x) < q.y) {
            const size_t o = 6 * size_t(q.x + threadIdx.x);
            const uint8_t* lk = t.locked + o;
            double v[6];
#pragma unroll
            for (int k = 0; k < 6; k++) {
                v[k] = -p[o + k];
                if (lk[k]) v[k] = 0;
            }
            const double lt = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (lt > mt) {
                const double f = mt / lt;
                v[0] *= f; v[1] *= f; v[2] *= f;
            }
            const double lr = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
            if (lr > mr) {
                const double f = mr / lr;
                v[3] *= f; v[4] *= f; v[5] *= f;
            }
#pragma unroll
            for (int k = 0; k < 6; k++) {
                v[k] = lk[k] ? 0.0 : v[k];
                p[o + k] = v[k];
            }
            acc[0] = dot6(g + o, v);
        }
        block_sum<1>(acc, sm);
        if (threadIdx.x == 0) part[0][b] = acc[0];
    }
    __syncthreads();
    double acc[1];
    chunk_sum<1>(part, nchunk, acc, sm);
    if (threadIdx.x == 0) dg[inst] = acc[0];
}

// ---- decisions the device takes itself ------------------------------------------------------
// Not a descent direction (sim.cpp:191): steepest descent instead.  For the instances that
// computed a direction and found dg >= 0: p = clamp(lock(-g)) and the partial of <g, p>.
__global__ void __launch_bounds__(kBlock) k_descent_fix(DevTopo t, const SolveCtl* __restrict__ ctl,
                                                        const double* __restrict__ dg, double* __restrict__ p,
                                                        const double* __restrict__ g, double mt, double mr,
                                                        double* __restrict__ part) {
    __shared__ double sm[kBlock / 32];
    const MapPos mp = map_pos(t.nblk);
    if (!(ctl[mp.inst].flags & (kOpDirection | kOpDirFused)) || dg[mp.inst] < 0) return;  // block-uniform
    double acc[1] = {0};
    if (mp.valid) {
        const size_t b = 6 * size_t(mp.i);
        const uint8_t* lk = t.locked + b;
        double v[6];
#pragma unroll
        for (int k = 0; k < 6; k++) v[k] = lk[k] ? 0.0 : -g[b + k];
        const double lt = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (lt > mt) {
            const double f = mt / lt;
            v[0] *= f; v[1] *= f; v[2] *= f;
        }
        const double lr = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
        if (lr > mr) {
            const double f = mr / lr;
            v[3] *= f; v[4] *= f; v[5] *= f;
        }
#pragma unroll
        for (int k = 0; k < 6; k++) {
            v[k] = lk[k] ? 0.0 : v[k];
            p[b + k] = v[k];
        }
        acc[0] = dot6(g + b, v);
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = acc[0];
}
// ... and per instance: the new dg and the history cleared (m = 0).
__global__ void __launch_bounds__(kBlock) k_descent_final(DevTopo t, const SolveCtl* __restrict__ ctl,
                                                          const double* __restrict__ part, double* __restrict__ dg,
                                                          int2* __restrict__ hist) {
    __shared__ double sm[kBlock / 32];
    const int inst = blockIdx.x;
    if (!(ctl[inst].flags & (kOpDirection | kOpDirFused))) return;
    if (dg[inst] < 0) return;
    double acc[1];
    instance_sum<1>(t, part, inst, acc, sm);
    if (threadIdx.x == 0) {
        dg[inst] = acc[0];
        hist[inst].x = 0;
    }
}
// The steepest-descent retry (sim.cpp:193-196) starts with an empty history.
__global__ void k_clear_history(int I, const SolveCtl* __restrict__ ctl, int bits, int2* __restrict__ hist) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < I && (ctl[i].flags & bits)) hist[i] = make_int2(0, 0);
}
__global__ void k_clear_history_m(int I, const SolveCtl* __restrict__ ctl, int bits, int2* __restrict__ hist) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < I && (ctl[i].flags & bits)) hist[i].x = 0;
}
// History after an accepted step (sim.cpp:205-206): keep the pair when
// s.y > 1e-12 sqrt(max(1e-30, s.s y.y)) (rho = 1 / s.y in its slot), else clear the history.
__global__ void k_history_update(int I, int H, const SolveCtl* __restrict__ ctl, const double* __restrict__ dots3,
                                 int2* __restrict__ hist, double* __restrict__ rho) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= I || !(ctl[i].flags & kOpAccept) || H <= 0) return;
    const double sy = dots3[3 * i], ss = dots3[3 * i + 1], yy = dots3[3 * i + 2];
    int2 h = hist[i];
    if (sy > 1e-12 * sqrt(fmax(1e-30, ss * yy))) {
        const int target = h.x < H ? (h.y + h.x) % H : h.y;
        rho[size_t(i) * H + target] = 1 / sy;
        if (h.x == H) h.y = (h.y + 1) % H;
        else h.x++;
    } else {
        h.x = 0;
    }
    hist[i] = h;
}

}  // namespace

size_t lbfgs_part_doubles(int n_nblk) { return 4 * size_t(n_nblk) + 8; }

int fused_direction_limit() { return kFuseChunks; }

void bl_direction_fused(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, double* p, const double* g,
                        const double* S, const double* Y, long long stride, const double* rho, double* dg, double mt,
                        double mr, cudaStream_t s) {
    (k_direction_fused<<<t.I, kBlock, 0, s>>>(t, ctl, hist, H, p, g, S, Y, stride, rho, dg, mt, mr), note_launches(1));
}

void bl_direction_multi(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, double* p, const double* g,
                        const double* S, const double* Y, long long stride, const double* rho, double* alpha,
                        double* part, double* dg, double mt, double mr, cudaStream_t s) {
    const int nb = t.n_nblk;
    // partials: step dot products ping-pong between part and part + nb; H0's in part + 2 nb
    double* pp[2] = {part, part + size_t(nb)};
    double* h0part = part + 2 * size_t(nb);
    (k_tl_start<<<nb, kBlock, 0, s>>>(t, ctl, hist, H, p, g, S, Y, stride, h0part, pp[0]), note_launches(1));
    for (int j = 0; j < H; j++)
        (k_tl_step<1><<<nb, kBlock, 0, s>>>(t, ctl, hist, H, j, p, S, Y, stride, rho, alpha, pp[j & 1],
                                            pp[(j + 1) & 1]),
         note_launches(1));
    (k_tl_scale<<<nb, kBlock, 0, s>>>(t, ctl, hist, H, p, Y, stride, h0part, pp[0]), note_launches(1));
    for (int j = 0; j < H; j++)
        (k_tl_step<2><<<nb, kBlock, 0, s>>>(t, ctl, hist, H, j, p, S, Y, stride, rho, alpha, pp[j & 1],
                                            pp[(j + 1) & 1]),
         note_launches(1));
    (k_finish<<<nb, kBlock, 0, s>>>(t, ctl, kOpDirection, p, p, g, mt, mr, part), note_launches(1));
    (k_inst_final<1><<<t.I, kBlock, 0, s>>>(t, ctl, kOpDirection, part, dg), note_launches(1));
}

void bl_descent_fix(const DevTopo& t, const SolveCtl* ctl, int2* hist, double* p, const double* g, double* part,
                    double* dg, double mt, double mr, cudaStream_t s) {
    // not a descent direction: steepest descent, history cleared (sim.cpp:191)
    (k_descent_fix<<<t.n_nblk, kBlock, 0, s>>>(t, ctl, dg, p, g, mt, mr, part), note_launches(1));
    (k_descent_final<<<t.I, kBlock, 0, s>>>(t, ctl, part, dg, hist), note_launches(1));
}

void bl_direction(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, bool multi, double* p, const double* g,
                  const double* S, const double* Y, long long stride, const double* rho, double* alpha, double* part,
                  double* dg, double mt, double mr, cudaStream_t s) {
    bl_direction_fused(t, ctl, hist, H, p, g, S, Y, stride, rho, dg, mt, mr, s);
    if (multi) bl_direction_multi(t, ctl, hist, H, p, g, S, Y, stride, rho, alpha, part, dg, mt, mr, s);
    bl_descent_fix(t, ctl, hist, p, g, part, dg, mt, mr, s);
}

void bl_steepest(const DevTopo& t, const SolveCtl* ctl, int2* hist, double* p, const double* g, double* part,
                 double* dg, double mt, double mr, cudaStream_t s) {
    (k_clear_history_m<<<(t.I + kBlock - 1) / kBlock, kBlock, 0, s>>>(t.I, ctl, kOpSteepest, hist), note_launches(1));
    (k_finish<<<t.n_nblk, kBlock, 0, s>>>(t, ctl, kOpSteepest, p, g, g, mt, mr, part), note_launches(1));
    (k_inst_final<1><<<t.I, kBlock, 0, s>>>(t, ctl, kOpSteepest, part, dg), note_launches(1));
}

void bl_prepare(const DevTopo& t, const SolveCtl* ctl, int2* hist, double* z, double* best, double* zeval,
                const double* p, double* zfinal, cudaStream_t s) {
    (k_clear_history<<<(t.I + kBlock - 1) / kBlock, kBlock, 0, s>>>(t.I, ctl, kOpResetHistory, hist),
     note_launches(1));
    (k_prepare<<<t.n_nblk, kBlock, 0, s>>>(t, ctl, z, best, zeval, p, zfinal), note_launches(1));
}

void bl_accept(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, double* z, double* g, const double* zeval,
               const double* geval, double* S, double* Y, long long stride, double* best, double* rho, double* part,
               double* out3, cudaStream_t s) {
    (k_accept<<<t.n_nblk, kBlock, 0, s>>>(t, ctl, hist, H, z, g, zeval, geval, S, Y, stride, best, part),
     note_launches(1));
    (k_inst_final<3><<<t.I, kBlock, 0, s>>>(t, ctl, kOpAccept, part, out3), note_launches(1));
    (k_history_update<<<(t.I + kBlock - 1) / kBlock, kBlock, 0, s>>>(t.I, H, ctl, out3, hist, rho), note_launches(1));
}

}  // namespace mcg

