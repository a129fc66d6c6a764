// common.cuh -- shared device helpers: FP64 vector/quaternion algebra, deterministic
// block reductions, launch geometry.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mcg {

constexpr int kBlock = 256;          // threads per CTA for the streaming kernels
constexpr double kPiD = 3.1415926535897932384626433832795;

// ---- FP64 3-vectors and quaternions ----------------------------------------------------
// Same algebra as the reference's Vec3/Quat (MC/include/core.hpp:37-41): a vector divided
// by s is a multiplication with 1/s, and rotation is v + w t + q x t with t = 2 q x v.
struct d3 { double x, y, z; };
struct q4 { double w, x, y, z; };

__device__ __forceinline__ d3 mk3(double x, double y, double z) { return d3{x, y, z}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator-(d3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double len2(d3 v) { return dot(v, v); }
__device__ __forceinline__ double len(d3 v) { return sqrt(len2(v)); }
__device__ __forceinline__ d3 unit(d3 v) {
    const double l2 = len2(v);
    return (isfinite(l2) && l2 > 1e-30) ? v * (1.0 / sqrt(l2)) : d3{0, 1, 0};
}
__device__ __forceinline__ double clampd(double x, double lo, double hi) { return fmax(lo, fmin(hi, x)); }
__device__ __forceinline__ double sqr(double x) { return x * x; }

__device__ __forceinline__ q4 conj(q4 q) { return {q.w, -q.x, -q.y, -q.z}; }
__device__ __forceinline__ q4 qnorm(q4 q) {
    const double n = sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
    if (n < 1e-30) return q4{1, 0, 0, 0};
    return {q.w / n, q.x / n, q.y / n, q.z / n};
}
__device__ __forceinline__ q4 qmul(q4 a, q4 b) {
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
            a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}
__device__ __forceinline__ d3 qrot(q4 q, d3 v) {
    const d3 u{q.x, q.y, q.z};
    const d3 t = cross(u, v) * 2.0;
    return (v + t * q.w) + cross(u, t);
}
__device__ __forceinline__ d3 qrot_inv(q4 q, d3 v) { return qrot(conj(q), v); }

// Unit quaternion of the rotation vector v (MC/include/core.hpp:51 quatExp, :42 quatAxisAngle).
__device__ __forceinline__ q4 exp_map(d3 v) {
    const double a = len(v);
    if (a < 1e-12) return qnorm(q4{1 - .125 * a * a, .5 * v.x, .5 * v.y, .5 * v.z});
    const d3 axis = unit(v * (1.0 / a));
    double s, c;
    sincos(.5 * a, &s, &c);
    return qnorm(q4{c, axis.x * s, axis.y * s, axis.z * s});
}
// Rotation vector of a unit quaternion (MC/include/core.hpp:52 quatLog).
__device__ __forceinline__ d3 log_map(q4 q) {
    q = qnorm(q);
    if (q.w < 0) q = q4{-q.w, -q.x, -q.y, -q.z};
    const double s = sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
    if (s < 1e-12) return {2 * q.x, 2 * q.y, 2 * q.z};
    const double a = 2 * atan2(s, clampd(q.w, -1, 1));
    return d3{q.x, q.y, q.z} * (a / s);
}
// J_l^{-T}(p) v, the SO(3) left-Jacobian inverse transpose applied to v
// (MC/include/core.hpp:53): v + p x v / 2 + A p x (p x v) with
// A(a) = 1/a^2 - (1 + cos a) / (2 a sin a) = 1/a^2 - cot(a/2) / (2a).
// Below a = 0.5 A is evaluated from its Taylor series (the Laurent series of cot, whose
// coefficients are Bernoulli numbers): 1/12 + a^2/720 + a^4/30240 + ...; eight terms leave
// a truncation error below 2e-18 relative there, and avoid both the sine/cosine and the
// cancellation of the closed form, which loses about log10(12/a^2) digits at small a.
// Above it the closed form is used as the reference writes it.
__device__ __forceinline__ double jl_coef(double a2) {
    double A = 3617.0 / 10670622842880000.0;
    A = fma(A, a2, 1.0 / 74724249600.0);
    A = fma(A, a2, 691.0 / 1307674368000.0);
    A = fma(A, a2, 1.0 / 47900160.0);
    A = fma(A, a2, 1.0 / 1209600.0);
    A = fma(A, a2, 1.0 / 30240.0);
    A = fma(A, a2, 1.0 / 720.0);
    return fma(A, a2, 1.0 / 12.0);
}
__device__ __forceinline__ d3 jl_inv_t(d3 p, d3 v) {
    const double a2 = len2(p);
    const d3 c1 = cross(p, v);
    const d3 c2 = cross(p, c1);
    double A;
    if (a2 < 0.25) {
        A = jl_coef(a2);
    } else {
        const double a = sqrt(a2);
        double s, c;
        sincos(a, &s, &c);
        A = 1 / (a * a) - (1 + c) / (2 * a * s);
    }
    return (v + c1 * .5) + c2 * A;
}

// Rotation matrix of a unit quaternion, rows as 32-byte records (x, y, z, pad).
struct m3 { d3 r0, r1, r2; };
__device__ __forceinline__ m3 quat_matrix(q4 q) {
    const double xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    const double xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    const double wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    return m3{d3{1 - 2 * (yy + zz), 2 * (xy - wz), 2 * (xz + wy)},
              d3{2 * (xy + wz), 1 - 2 * (xx + zz), 2 * (yz - wx)},
              d3{2 * (xz - wy), 2 * (yz + wx), 1 - 2 * (xx + yy)}};
}
__device__ __forceinline__ d3 mrot(const m3& m, d3 v) { return d3{dot(m.r0, v), dot(m.r1, v), dot(m.r2, v)}; }
__device__ __forceinline__ d3 mrot_t(const m3& m, d3 v) {
    return d3{m.r0.x * v.x + m.r1.x * v.y + m.r2.x * v.z, m.r0.y * v.x + m.r1.y * v.y + m.r2.y * v.z,
              m.r0.z * v.x + m.r1.z * v.y + m.r2.z * v.z};
}

// ---- deterministic reductions ------------------------------------------------------------
// Fixed shuffle tree inside a warp, fixed order across warps: the same inputs in the same
// threads always give the same bits.  The warp results are complete in lane 0 only; at
// each level only the lanes whose sums lane 0 still needs add (the FP64 pipe is narrow).
__device__ __forceinline__ double warp_sum(double v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, v, o);
        if (lane < o) v += y;
    }
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, v, o);
        if (lane < o) v = fmax(v, y);
    }
    return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sums NV values per thread over the block; thread 0 receives the totals.  `smem` needs
// NV * (blockDim.x / 32) doubles.  blockDim.x must be a multiple of 32.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) smem[k * nw + warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0;
            for (int w = 0; w < nw; w++) s += smem[k * nw + w];
            v[k] = s;
        }
    __syncthreads();
}

// Sums NV values per thread over the block into thread 0 with few FP64 warp instructions
// (GB300's FP64 pipe is narrow): the values go through shared memory, warp w reduces values
// w, w + 8, ...: lane l adds entries l, l + 32, ... in order, then the warp's shuffle tree.
// `smem` needs NV * blockDim.x doubles.  blockDim.x must be a multiple of 32.
template <int NV>
__device__ __forceinline__ void block_sum_t(double (&v)[NV], double* smem) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) smem[k * nt + tid] = v[k];
    __syncthreads();
    for (int k = warp; k < NV; k += nw) {
        const double* a = smem + k * nt;
        double s = a[lane];
        for (int j = lane + 32; j < nt; j += 32) s += a[j];
        s = warp_sum(s);
        __syncwarp();
        if (lane == 0) smem[k * nt] = s;
    }
    __syncthreads();
    if (tid == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = smem[k * nt];
    __syncthreads();
}

// The same for maxima (fmax skips NaN); `smem` needs NV * blockDim.x doubles.
template <int NV>
__device__ __forceinline__ void block_max_t(double (&v)[NV], double* smem) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) smem[k * nt + tid] = v[k];
    __syncthreads();
    for (int k = warp; k < NV; k += nw) {
        const double* a = smem + k * nt;
        double m = a[lane];
        for (int j = lane + 32; j < nt; j += 32) m = fmax(m, a[j]);
        m = warp_max(m);
        __syncwarp();
        if (lane == 0) smem[k * nt] = m;
    }
    __syncthreads();
    if (tid == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = smem[k * nt];
    __syncthreads();
}

// NV maxima over the block into thread 0, one barrier pair for all of them; smem holds
// NV * (blockDim.x / 32) doubles.
template <int NV>
__device__ __forceinline__ void block_max_n(double (&v)[NV], double* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_max(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) smem[k * nw + warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double m = smem[k * nw];
            for (int w = 1; w < nw; w++) m = fmax(m, smem[k * nw + w]);
            v[k] = m;
        }
    __syncthreads();
}

// The same in single precision (fmaxf skips NaN like fmax); smem holds NV * (blockDim.x / 32)
// floats.
template <int NV>
__device__ __forceinline__ void block_max_nf(float (&v)[NV], float* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_max_f(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) smem[k * nw + warp] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) {
            float m = smem[k * nw];
            for (int w = 1; w < nw; w++) m = fmaxf(m, smem[k * nw + w]);
            v[k] = m;
        }
    __syncthreads();
}

__device__ __forceinline__ double block_max(double v, double* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max(v);
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = smem[0];
        for (int w = 1; w < nw; w++) m = fmax(m, smem[w]);
        v = m;
    }
    __syncthreads();
    return v;
}

inline unsigned grid_for(long long n, int block = kBlock) {
    long long g = (n + block - 1) / block;
    return unsigned(g < 1 ? 1 : g);
}

}  // namespace mcg
