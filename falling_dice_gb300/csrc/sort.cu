// sort.cu -- exclusive scan and stable LSD radix sort (8-bit digits), both deterministic.
//
// Scan: reduce-then-scan over tiles of 2048 items (256 threads x 8 consecutive items).
// Radix sort: per pass, tile histograms -> digit-major exclusive scan -> stable scatter in
// which each tile ranks its items in input order (warp match + per-warp digit counters),
// so equal keys keep their input order and the result does not depend on scheduling.
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

__global__ void __launch_bounds__(kBlock) k_scan_reduce(const uint32_t* __restrict__ in, long long n,
                                                        uint32_t* __restrict__ part) {
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
__global__ void __launch_bounds__(kBlock) k_scan_partials(uint32_t* part, long long np, uint32_t* total_out) {
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

__global__ void __launch_bounds__(kBlock) k_scan_down(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                      long long n, const uint32_t* __restrict__ part,
                                                      const uint32_t* __restrict__ total) {
    __shared__ uint32_t sm[kBlock / 32];
    const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    uint32_t v[kItems], s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t run = part[blockIdx.x] + block_exclusive_scan(s, sm, nullptr);
#pragma unroll
    for (int k = 0; k < kItems; k++)
        if (base + k < n) { out[base + k] = run; run += v[k]; }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = *total;
}

// ---- radix sort -----------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_radix_hist(const uint64_t* __restrict__ keys, long long n, int shift,
                                                       int ntiles, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kTile;
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        const long long i = base + (long long)r * kBlock + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kBlock) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                          const uint32_t* __restrict__ vin,
                                                          uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                          long long n, int shift, int ntiles,
                                                          const uint32_t* __restrict__ offs) {
    constexpr int NW = kBlock / 32;
    __shared__ uint32_t cnt[NW][256];
    __shared__ uint32_t base[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    base[threadIdx.x] = offs[(long long)threadIdx.x * ntiles + blockIdx.x];
    const unsigned lt_mask = (1u << lane) - 1u;
    const long long tile = (long long)blockIdx.x * kTile;
    for (int r = 0; r < kItems; r++) {
#pragma unroll
        for (int w = 0; w < NW; w++) cnt[w][threadIdx.x] = 0;
        __syncthreads();
        const long long i = tile + (long long)r * kBlock + threadIdx.x;
        const bool valid = i < n;
        uint64_t key = 0;
        uint32_t val = 0, d = 256;
        if (valid) {
            key = kin[i];
            val = vin[i];
            d = uint32_t((key >> shift) & 255u);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) cnt[warp][d] = __popc(peers);
        __syncthreads();
        {  // thread t owns digit t: exclusive prefix over warps, then advance its base
            const int dd = threadIdx.x;
            uint32_t run = base[dd];
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const uint32_t c = cnt[w][dd];
                cnt[w][dd] = run;
                run += c;
            }
            base[dd] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = cnt[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

}  // namespace

size_t scan_tmp_bytes(long long n) {
    const long long np = (n + kTile - 1) / kTile + 1;
    return size_t(np + 4) * sizeof(uint32_t);
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, long long n, void* tmp, cudaStream_t s) {
    uint32_t* part = static_cast<uint32_t*>(tmp);
    const long long np = (n + kTile - 1) / kTile;
    uint32_t* total = part + np + 1;
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
        return;
    }
    (k_scan_reduce<<<unsigned(np), kBlock, 0, s>>>(in, n, part), note_launches(1));
    (k_scan_partials<<<1, kBlock, 0, s>>>(part, np, total), note_launches(1));
    (k_scan_down<<<unsigned(np), kBlock, 0, s>>>(in, out, n, part, total), note_launches(1));
}

size_t radix_tmp_bytes(long long n) {
    const long long nt = (n + kTile - 1) / kTile;
    const long long nh = 256 * (nt > 0 ? nt : 1);
    return size_t(2 * nh + 16) * sizeof(uint32_t) + scan_tmp_bytes(nh);
}

int radix_sort_u64(uint64_t* keys[2], uint32_t* vals[2], long long n, int end_bit, void* tmp,
                   const uint32_t* /*n_dev*/, cudaStream_t s) {
    if (n <= 1 || end_bit <= 0) return 0;
    const long long nt = (n + kTile - 1) / kTile;
    const long long nh = 256 * nt;
    uint32_t* hist = static_cast<uint32_t*>(tmp);
    uint32_t* offs = hist + nh + 8;
    void* stmp = offs + nh + 8;
    int cur = 0;
    for (int shift = 0; shift < end_bit; shift += 8) {
        (k_radix_hist<<<unsigned(nt), kBlock, 0, s>>>(keys[cur], n, shift, int(nt), hist), note_launches(1));
        exclusive_scan_u32(hist, offs, nh, stmp, s);
        (k_radix_scatter<<<unsigned(nt), kBlock, 0, s>>>(keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, shift,
                                                        int(nt), offs), note_launches(1));
        cur ^= 1;
    }
    return cur;
}

}  // namespace mcg
