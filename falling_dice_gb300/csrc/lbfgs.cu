// lbfgs.cu -- device vector kernels of the L-BFGS minimizer
// (the reference's Simulator::minimize and helpers, MC/src/sim.cpp:42-46, 174-211).
//
// The two-loop recursion, direction clamp, candidate steps and curvature products all run
// on the device; scalars the recursion needs (alpha_h, beta_h, H0) never leave it.  Dot
// products use a fixed two-level partition (a fixed grid of partial sums, then one block)
// so that every value is reproducible bit for bit.
#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

constexpr int kDotBlocks = 296;  // 2 x 148: fixed partition of every reduction

// Up to three dot products over the same index range: out[k] = sum a_k[i] * b_k[i].
template <int K>
__global__ void __launch_bounds__(kBlock) k_dots_part(const double* __restrict__ a0, const double* __restrict__ b0,
                                                      const double* __restrict__ a1, const double* __restrict__ b1,
                                                      const double* __restrict__ a2, const double* __restrict__ b2,
                                                      long long n, double* __restrict__ part) {
    __shared__ double sm[K * (kBlock / 32)];
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; k++) acc[k] = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        acc[0] += a0[i] * b0[i];
        if (K > 1) acc[1 % K] += a1[i] * b1[i];
        if (K > 2) acc[2 % K] += a2[i] * b2[i];
    }
    block_sum<K>(acc, sm);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; k++) part[k * kDotBlocks + blockIdx.x] = acc[k];
}

template <int K>
__global__ void __launch_bounds__(kBlock) k_dots_final(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sm[K * (kBlock / 32)];
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        acc[k] = 0;
        for (int j = threadIdx.x; j < kDotBlocks; j += blockDim.x) acc[k] += part[k * kDotBlocks + j];
    }
    block_sum<K>(acc, sm);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; k++) out[k] = acc[k];
}

// Sum of squares and max |g| over unlocked DOFs (sim.cpp:44-45).
__global__ void __launch_bounds__(kBlock) k_rms_max_part(const double* __restrict__ g, const uint8_t* __restrict__ locked,
                                                         long long n, double* __restrict__ part) {
    __shared__ double sm[kBlock / 32];
    __shared__ double smx[kBlock / 32];
    double acc[1] = {0};
    double m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (!locked[i]) {
            const double v = g[i];
            acc[0] += v * v;
            m = fmax(m, fabs(v));
        }
    }
    block_sum<1>(acc, sm);
    m = block_max(m, smx);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = acc[0];
        part[kDotBlocks + blockIdx.x] = m;
    }
}

__global__ void __launch_bounds__(kBlock) k_rms_max_final(const double* __restrict__ part, long long n_free,
                                                          double* __restrict__ out) {
    __shared__ double sm[kBlock / 32];
    __shared__ double smx[kBlock / 32];
    double acc[1] = {0};
    double m = 0;
    for (int j = threadIdx.x; j < kDotBlocks; j += blockDim.x) {
        acc[0] += part[j];
        m = fmax(m, part[kDotBlocks + j]);
    }
    block_sum<1>(acc, sm);
    m = block_max(m, smx);
    if (threadIdx.x == 0) {
        out[0] = n_free ? sqrt(acc[0] / double(n_free)) : 0.0;
        out[1] = m;
    }
}

__global__ void k_copy(double* __restrict__ dst, const double* __restrict__ src, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// p -= (rho * <s, p>) y, with alpha = rho * dot stored for the second loop.
__global__ void k_loop1_update(double* __restrict__ p, const double* __restrict__ y, long long n,
                               const double* __restrict__ rho, const double* __restrict__ dotv,
                               double* __restrict__ alpha_out) {
    const double alpha = (*rho) * (*dotv);
    if (blockIdx.x == 0 && threadIdx.x == 0) *alpha_out = alpha;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] -= alpha * y[i];
}

// p *= H0 with H0 = clamp(sy/yy, 1e-7, 1e4) when both are positive, else 0.1 (sim.cpp:186).
__global__ void k_scale_h0(double* __restrict__ p, long long n, const double* __restrict__ syyy, int have) {
    double H0 = .10;
    if (have) {
        const double sy = syyy[0], yy = syyy[1];
        if (sy > 1e-20 && yy > 1e-20) H0 = clampd(sy / yy, 1e-7, 1e4);
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] *= H0;
}

// p += s (alpha - rho <y, p>).
__global__ void k_loop2_update(double* __restrict__ p, const double* __restrict__ s, long long n,
                               const double* __restrict__ rho, const double* __restrict__ dotv,
                               const double* __restrict__ alpha) {
    const double beta = (*rho) * (*dotv);
    const double c = *alpha - beta;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] += s[i] * c;
}

// Direction finish: optional negation of src into p, lock, per-node step clamp, lock
// (sim.cpp:188-190 and clampDirection, sim.cpp:46).
__global__ void __launch_bounds__(kBlock) k_finish_dir(double* p, const double* src,
                                                       const uint8_t* __restrict__ locked, int N, double mt,
                                                       double mr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const size_t b = 6 * size_t(i);
    double v[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        v[k] = -src[b + k];
        if (locked[b + k]) v[k] = 0;
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
    for (int k = 0; k < 6; k++) p[b + k] = locked[b + k] ? 0.0 : v[k];
}

// zc = z + step p, locked entries zero (sim.cpp:179).
__global__ void k_candidate(double* __restrict__ zc, const double* __restrict__ z, const double* __restrict__ p,
                            double step, const uint8_t* __restrict__ locked, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        zc[i] = locked[i] ? 0.0 : z[i] + step * p[i];
}

// s = zc - z, y = gc - g (sim.cpp:205).
__global__ void k_sy(double* __restrict__ s, double* __restrict__ y, const double* __restrict__ zc,
                     const double* __restrict__ z, const double* __restrict__ gc, const double* __restrict__ g,
                     long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        s[i] = zc[i] - z[i];
        y[i] = gc[i] - g[i];
    }
}

__global__ void k_rho(double* __restrict__ rho, const double* __restrict__ sy) { *rho = 1 / *sy; }

inline unsigned vgrid(long long n) {
    const unsigned g = grid_for(n);
    return g < 4 * 152 ? g : 4 * 152;
}

}  // namespace

size_t lbfgs_part_doubles() { return 3 * kDotBlocks + 8; }

void dots(int k, const double* a0, const double* b0, const double* a1, const double* b1, const double* a2,
          const double* b2, long long n, double* part, double* out, cudaStream_t s) {
    if (k == 1) {
        (k_dots_part<1><<<kDotBlocks, kBlock, 0, s>>>(a0, b0, a1, b1, a2, b2, n, part), note_launches(1));
        (k_dots_final<1><<<1, kBlock, 0, s>>>(part, out), note_launches(1));
    } else if (k == 2) {
        (k_dots_part<2><<<kDotBlocks, kBlock, 0, s>>>(a0, b0, a1, b1, a2, b2, n, part), note_launches(1));
        (k_dots_final<2><<<1, kBlock, 0, s>>>(part, out), note_launches(1));
    } else {
        (k_dots_part<3><<<kDotBlocks, kBlock, 0, s>>>(a0, b0, a1, b1, a2, b2, n, part), note_launches(1));
        (k_dots_final<3><<<1, kBlock, 0, s>>>(part, out), note_launches(1));
    }
}

void rms_max(const double* g, const uint8_t* locked, long long n, long long n_free, double* part, double* out2,
             cudaStream_t s) {
    (k_rms_max_part<<<kDotBlocks, kBlock, 0, s>>>(g, locked, n, part), note_launches(1));
    (k_rms_max_final<<<1, kBlock, 0, s>>>(part, n_free, out2), note_launches(1));
}

void vcopy(double* dst, const double* src, long long n, cudaStream_t s) {
    (k_copy<<<vgrid(n), kBlock, 0, s>>>(dst, src, n), note_launches(1));
}

void two_loop(double* p, const double* g, const double* const* S, const double* const* Y, const double* const* rho,
              int m, double* alpha, double* scal, double* part, long long n, cudaStream_t s) {
    (k_copy<<<vgrid(n), kBlock, 0, s>>>(p, g, n), note_launches(1));
    for (int h = m - 1; h >= 0; h--) {
        dots(1, S[h], p, nullptr, nullptr, nullptr, nullptr, n, part, scal, s);
        (k_loop1_update<<<vgrid(n), kBlock, 0, s>>>(p, Y[h], n, rho[h], scal, alpha + h), note_launches(1));
    }
    if (m > 0) dots(2, S[m - 1], Y[m - 1], Y[m - 1], Y[m - 1], nullptr, nullptr, n, part, scal + 1, s);
    (k_scale_h0<<<vgrid(n), kBlock, 0, s>>>(p, n, scal + 1, m > 0 ? 1 : 0), note_launches(1));
    for (int h = 0; h < m; h++) {
        dots(1, Y[h], p, nullptr, nullptr, nullptr, nullptr, n, part, scal, s);
        (k_loop2_update<<<vgrid(n), kBlock, 0, s>>>(p, S[h], n, rho[h], scal, alpha + h), note_launches(1));
    }
}

void finish_direction(double* p, const double* src, const uint8_t* locked, int N, double mt, double mr,
                      cudaStream_t s) {
    (k_finish_dir<<<grid_for(N), kBlock, 0, s>>>(p, src, locked, N, mt, mr), note_launches(1));
}

void candidate(double* zc, const double* z, const double* p, double step, const uint8_t* locked, long long n,
               cudaStream_t s) {
    (k_candidate<<<vgrid(n), kBlock, 0, s>>>(zc, z, p, step, locked, n), note_launches(1));
}

void make_sy(double* sv, double* yv, const double* zc, const double* z, const double* gc, const double* g,
             long long n, cudaStream_t s) {
    (k_sy<<<vgrid(n), kBlock, 0, s>>>(sv, yv, zc, z, gc, g, n), note_launches(1));
}

void set_rho(double* rho, const double* sy, cudaStream_t s) { (k_rho<<<1, 1, 0, s>>>(rho, sy), note_launches(1)); }

}  // namespace mcg
