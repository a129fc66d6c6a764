// sort.cu -- deterministic exclusive scan of uint32 counts: reduce-then-scan over tiles of
// 2048 items (256 threads x 8 consecutive items).  Up to 1024 tiles each block of the second
// pass sums the tile totals before it itself (two launches); beyond, one block scans the
// tile totals between the two passes.
#include "common.cuh"
#include "kernels.h"

namespace mcg {

namespace {

constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;  // 2048

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) smem[lane] = w;
    }
    __syncthreads();
    const uint32_t warp_base = warp ? smem[warp - 1] : 0;
    if (total) *total = smem[nw - 1];
    __syncthreads();
    return warp_base + x - v;
}

// Element count: n, or min(n, (*dn + add) >> shift) when the count is on the device.
__device__ __forceinline__ long long scan_len(long long n, const uint32_t* dn, int add, int shift) {
    if (!dn) return n;
    const long long m = ((long long)*dn + add) >> shift;
    return m < n ? m : n;
}

__global__ void __launch_bounds__(kBlock) k_scan_reduce(const uint32_t* __restrict__ in, long long cap,
                                                        uint32_t* __restrict__ part, const uint32_t* __restrict__ gate,
                                                        const uint32_t* __restrict__ dn, int add, int shift) {
    if (gate && !*gate) return;
    const long long n = scan_len(cap, dn, add, shift);
    if ((long long)blockIdx.x * kTile >= n && blockIdx.x > 0) return;
    __shared__ uint32_t sm[kBlock / 32];
    const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_exclusive_scan(s, sm, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// One block scans the tile partials in chunks, carrying the running total.
__global__ void __launch_bounds__(kBlock) k_scan_partials(uint32_t* part, long long np_cap, uint32_t* total_out,
                                                          const uint32_t* __restrict__ gate,
                                                          const uint32_t* __restrict__ dn, int add, int shift) {
    if (gate && !*gate) return;
    const long long n = scan_len(np_cap * kTile, dn, add, shift);
    const long long np = dn ? (n + kTile - 1) / kTile : np_cap;
    __shared__ uint32_t sm[kBlock / 32];
    uint32_t carry = 0;
    for (long long c = 0; c < np; c += kTile) {
        const long long base = c + (long long)threadIdx.x * kItems;
        uint32_t v[kItems], s = 0;
#pragma unroll
        for (int k = 0; k < kItems; k++) {
            v[k] = base + k < np ? part[base + k] : 0;
            s += v[k];
        }
        uint32_t tot;
        uint32_t run = carry + block_exclusive_scan(s, sm, &tot);
#pragma unroll
        for (int k = 0; k < kItems; k++)
            if (base + k < np) { part[base + k] = run; run += v[k]; }
        carry += tot;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

// DIRECT: the tile partials are not scanned; each block sums those before it (and block 0
// all of them), for at most kDirectTiles tiles.
constexpr long long kDirectTiles = 1024;

__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v, uint32_t* smem) {
    uint32_t tot;
    block_exclusive_scan(v, smem, &tot);
    return tot;
}

template <bool DIRECT>
__global__ void __launch_bounds__(kBlock) k_scan_down(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                      long long cap, const uint32_t* __restrict__ part,
                                                      const uint32_t* __restrict__ total_p,
                                                      const uint32_t* __restrict__ gate,
                                                      const uint32_t* __restrict__ dn, int add, int shift) {
    if (gate && !*gate) return;
    const long long n = scan_len(cap, dn, add, shift);
    __shared__ uint32_t sm[kBlock / 32];
    uint32_t prefix, total = 0;
    if (DIRECT) {
        const long long np = (n + kTile - 1) / kTile;
        if (blockIdx.x > 0 && (long long)blockIdx.x * kTile >= n) return;
        const long long upto = blockIdx.x == 0 ? np : (long long)blockIdx.x;
        uint32_t a = 0, b = 0;  // partials before this block; all partials (block 0)
        for (long long i = threadIdx.x; i < upto; i += kBlock) {
            const uint32_t v = part[i];
            if (i < (long long)blockIdx.x) a += v;
            b += v;
        }
        prefix = block_sum_u32(a, sm);
        if (blockIdx.x == 0) total = block_sum_u32(b, sm);
    } else {
        if (blockIdx.x == 0) total = *total_p;
        if ((long long)blockIdx.x * kTile >= n && blockIdx.x > 0) return;
        prefix = part[blockIdx.x];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[cap] = total;  // the total at a fixed place
    if ((long long)blockIdx.x * kTile >= n) return;
    const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    uint32_t v[kItems], s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t run = prefix + block_exclusive_scan(s, sm, nullptr);
#pragma unroll
    for (int k = 0; k < kItems; k++)
        if (base + k < n) { out[base + k] = run; run += v[k]; }
    if (blockIdx.x == 0 && threadIdx.x == 0 && n < cap) out[n] = total;
}

}  // namespace

size_t scan_tmp_bytes(long long n) {
    const long long np = (n + kTile - 1) / kTile + 1;
    return size_t(np + 4) * sizeof(uint32_t);
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, long long n, void* tmp, cudaStream_t s,
                        const uint32_t* gate, const uint32_t* dn, int add, int shift) {
    uint32_t* part = static_cast<uint32_t*>(tmp);
    const long long np = (n + kTile - 1) / kTile;
    uint32_t* total = part + np + 1;
    if (n <= 0) {
        if (!gate) cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
        return;
    }
    (k_scan_reduce<<<unsigned(np), kBlock, 0, s>>>(in, n, part, gate, dn, add, shift), note_launches(1));
    if (np <= kDirectTiles) {
        (k_scan_down<true><<<unsigned(np), kBlock, 0, s>>>(in, out, n, part, total, gate, dn, add, shift),
         note_launches(1));
        return;
    }
    (k_scan_partials<<<1, kBlock, 0, s>>>(part, np, total, gate, dn, add, shift), note_launches(1));
    (k_scan_down<false><<<unsigned(np), kBlock, 0, s>>>(in, out, n, part, total, gate, dn, add, shift),
     note_launches(1));
}

}  // namespace mcg
