// noalloc.cu -- mcg_objective_noalloc: the energy/gradient evaluation for callers that
// cannot allocate device memory at the time they evaluate.
//
// mcg_objective sizes its self-contact buffers on demand: when an evaluation needs more
// cell entries, bins, candidate pairs or contacts than the context holds, it frees and
// re-allocates them and evaluates again.  Some callers cannot let that happen: real-time
// loops that run against a fixed device-memory budget, hosts whose device memory is owned
// by another allocator (a framework's caching pool that has reserved it), and schedulers
// that must not stall, since cudaFree waits for all work on the device.  This entry point
// evaluates with the self-contact scratch placed in one file-scope __device__ array of
// fixed size instead, and never calls cudaMalloc, cudaFree or any allocating routine.
// Everything else it uses (the lattice, the base state, the per-node and per-beam buffers)
// was allocated when the context was set up.
//
// The array is kNoAllocScratchBytes (4 MiB) and exists once on every GPU that loads the
// library, for the life of the process.  It bounds the lattice: at most
// kNoAllocMaxNodes nodes and kNoAllocMaxShapes nodes + beams, and per evaluation at most
// the entry/bin/candidate/contact counts below; a larger lattice or state is rejected with
// MCG_ERR_CAPACITY and a message naming what overflowed.  The bins cover the grid box of the
// deformed specimen at the grid cell (the reference's max(2.8 joint radius, 0.72 cell)):
// about 9 cells per axis of a cube-shaped specimen.
//
// Host code cannot use the array's name as an address: the first call on each context
// looks the device address up with cudaGetSymbolAddress, with the context's device current,
// and keeps it in the context (a context created after a cudaDeviceReset looks it up again).
//
// All calls on a device share the one array, which keeps the previous call's contents;
// every buffer that must start at zero is cleared by the evaluation itself.  Two calls whose
// work overlaps on the GPU (two contexts on two host threads, or two streams) race on the
// array: callers must order them.
#include <cuda_runtime.h>

#include "../../include/mcg.h"
#include "common.cuh"
#include "kernels.h"

namespace mcg {

int objective_with_fixed_contacts(mcg_ctx* c, ContactBufs& fixed, const double* z, double top, double* energy,
                                  double* grad, mcg_diag* diag);
int ctx_counts(const mcg_ctx* c, int* n_nodes, int* n_beams, int* device);
void** ctx_noalloc_scratch(mcg_ctx* c);
void ctx_set_error(mcg_ctx* c, const char* msg);

namespace {

constexpr long long kNoAllocMaxNodes = 4096;
constexpr long long kNoAllocMaxShapes = 8192;       // nodes + beams
constexpr int kNoAllocBinSlots = 128;                // entries one grid bin holds
constexpr long long kNoAllocBins = 4096;
constexpr long long kNoAllocCandidates = 4 * kNoAllocMaxShapes;
constexpr long long kNoAllocContacts = 8192;
constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;

// The self-contact scratch of mcg_objective_noalloc.  In host code this name is a
// host-side stand-in, not a device address: host code must use the address obtained by
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the array on the context's device (which is current), looked up by the
// first call on the context and kept in it.
cudaError_t scratch_address(mcg_ctx* ctx, unsigned char** out) {
    void** slot = ctx_noalloc_scratch(ctx);
    if (!*slot) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        *slot = p;
    }
    *out = static_cast<unsigned char*>(*slot);
    return cudaSuccess;
}

// Carves the contact buffers out of the array; false if they do not fit.
bool carve(unsigned char* base, long long N, long long S, ContactBufs& c) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += (bytes + 255) & ~size_t(255);
        return p;
    };
    c = ContactBufs{};
    c.cell_lo = reinterpret_cast<int4*>(take(size_t(S) * sizeof(int4)));
    c.cell_hi = reinterpret_cast<int4*>(take(size_t(S) * sizeof(int4)));
    c.rec = reinterpret_cast<uint4*>(take(size_t(S) * sizeof(uint4)));
    c.grid = reinterpret_cast<int*>(take(16 * sizeof(int)));
    c.flags = reinterpret_cast<uint32_t*>(take(5 * 4));
    c.xref = reinterpret_cast<float4*>(take(size_t(N > 0 ? N : 1) * sizeof(float4)));
    c.bin_cap = kNoAllocBins;
    c.bin_slots = kNoAllocBinSlots;
    c.bin_count = reinterpret_cast<uint32_t*>(take(size_t(kNoAllocBins + 1) * 4));
    c.bin_items = reinterpret_cast<uint32_t*>(take(size_t(kNoAllocBins) * kNoAllocBinSlots * 4));
    c.nentries = reinterpret_cast<uint32_t*>(take(3 * 4));
    c.pair_blocks = contact_pair_blocks(S);
    c.cand_cap = kNoAllocCandidates;
    c.cand = reinterpret_cast<uint2*>(take(size_t(kNoAllocCandidates) * sizeof(uint2)));
    c.ncand = reinterpret_cast<uint32_t*>(take(4));
    const long long chunks = kNoAllocCandidates / 32;
    c.cand2 = reinterpret_cast<uint2*>(take(size_t(kNoAllocCandidates) * sizeof(uint2)));
    c.fbits = reinterpret_cast<uint32_t*>(take(size_t(chunks) * 4));
    c.fcount = reinterpret_cast<uint32_t*>(take(size_t(chunks + 1) * 4));
    c.foff = reinterpret_cast<uint32_t*>(take(size_t(chunks + 1) * 4));
    c.hitbits = reinterpret_cast<uint32_t*>(take(size_t(chunks) * 4));
    c.hcount = reinterpret_cast<uint32_t*>(take(size_t(chunks + 1) * 4));
    c.hoff = reinterpret_cast<uint32_t*>(take(size_t(chunks + 1) * 4));
    c.contact_cap = kNoAllocContacts;
    c.c_a = reinterpret_cast<uint32_t*>(take(size_t(kNoAllocContacts) * 4));
    c.c_b = reinterpret_cast<uint32_t*>(take(size_t(kNoAllocContacts) * 4));
    c.c_s = reinterpret_cast<double*>(take(size_t(kNoAllocContacts) * 8));
    c.c_t = reinterpret_cast<double*>(take(size_t(kNoAllocContacts) * 8));
    c.c_n = reinterpret_cast<double*>(take(size_t(3 * kNoAllocContacts) * 8));
    c.c_pen = reinterpret_cast<double*>(take(size_t(kNoAllocContacts) * 8));
    c.n_count = reinterpret_cast<uint32_t*>(take(size_t(N + 1) * 4));
    c.n_start = reinterpret_cast<uint32_t*>(take(size_t(N + 1) * 4));
    c.n_cursor = reinterpret_cast<uint32_t*>(take(size_t(N) * 4));
    c.n_items = reinterpret_cast<uint32_t*>(take(size_t(4 * kNoAllocContacts) * 4));
    c.n_sorted = reinterpret_cast<uint32_t*>(take(size_t(4 * kNoAllocContacts) * 4));
    c.n_long = reinterpret_cast<uint32_t*>(take(size_t(N + 1) * 4));
    c.long_sum = nullptr;  // the gather walks every list (no room for the long lists' sums)
    long long scan_n = N + 1;
    if (chunks + 1 > scan_n) scan_n = chunks + 1;
    c.scan_tmp_bytes = scan_tmp_bytes(scan_n);
    c.scan_tmp = take(c.scan_tmp_bytes);
    return off <= kNoAllocScratchBytes;
}

}  // namespace
}  // namespace mcg

extern "C" int mcg_objective_noalloc(mcg_ctx* ctx, const double* z, double top, double* energy, double* grad,
                                     mcg_diag* diag) {
    using namespace mcg;
    int N = 0, B = 0, device = 0;
    const int rc = ctx_counts(ctx, &N, &B, &device);
    if (rc != MCG_OK) return ctx ? rc : MCG_ERR_INVALID;
    if (N > kNoAllocMaxNodes || (long long)N + B > kNoAllocMaxShapes) {
        ctx_set_error(ctx, "mcg_objective_noalloc: the lattice exceeds the fixed scratch (at most 4096 nodes and "
                           "8192 nodes + beams)");
        return MCG_ERR_CAPACITY;
    }
    // like every entry point, this one makes the context's device current on the calling thread
    if (cudaSetDevice(device) != cudaSuccess) {
        ctx_set_error(ctx, "mcg_objective_noalloc: cudaSetDevice failed");
        return MCG_ERR_CUDA;
    }
    unsigned char* base = nullptr;
    const cudaError_t e = scratch_address(ctx, &base);
    if (e != cudaSuccess) {
        ctx_set_error(ctx, cudaGetErrorString(e));
        return MCG_ERR_CUDA;
    }
    ContactBufs fixed;
    if (!carve(base, N, (long long)N + B, fixed)) {
        ctx_set_error(ctx, "mcg_objective_noalloc: internal scratch layout exceeds the array");
        return MCG_ERR_CAPACITY;
    }
    return objective_with_fixed_contacts(ctx, fixed, z, top, energy, grad, diag);
}
