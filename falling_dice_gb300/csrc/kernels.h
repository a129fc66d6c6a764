// kernels.h -- device data layout and the host-side launchers of the CUDA kernels.
//
// HBM layout (one context = one lattice):
//   per beam (SoA, FP64): L0, area, radius, e0[3 arrays], and the section constants the
//     reference recomputes on every call (E I/L0, G J/L0, yield moments, hardening
//     moduli, shear and axial energy scales), precomputed once with the reference's own
//     expressions so they are bit-identical; plastic state as 7 SoA arrays.
//   per node: base position (3 FP64, AoS), base orientation (4 FP64, AoS), current
//     position/orientation as 32-byte double4_32a records so each beam-end gather is one
//     sector; the 6-DOF z/grad vectors in the ABI layout.
//   incidence CSR: for every node the beams touching it in ascending beam order, as
//     (beam << 1 | role) -- the order the reference's scatter adds them in.
//   per-beam gradient slots: the beam kernel writes, for each end, the 6-vector it adds to
//     that end's node, and the gather sums them per node; no atomics anywhere on the
//     gradient path, so every evaluation is bitwise reproducible.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace mcg {

struct Material {
    double E, G, sy, H, bend_h, torsion_h;
    double inv_EH;  // 1 / max(1e-20, E + H)
    float Ef, Hf, bend_hf, torsion_hf;  // the same in single precision (mixed form)
};

struct DevTopo {
    int N, B;
    const int2* ab;
    const double *L0, *area, *radius;
    const double *e0x, *e0y, *e0z;
    const double *kb, *kt, *my, *ty, *hb, *ht, *cs, *aL, *aLsy;
    const double *invL0, *inv_kbh, *inv_kth;  // 1/L0, 1/max(1e-20, kb+hb), 1/max(1e-20, kt+ht)
    const double* mass;
    const uint8_t* locked;    // [6N]
    const int* inc_start;     // [N+1]
    const int* inc;           // [2B]
    // connected node pairs (the reference's connected_ set) as an open-addressing hash set
    // of keys u << 32 | v, u <= v; empty slots hold ~0; at most half full
    const unsigned long long* conn_hash;
    unsigned long long conn_mask;  // slots - 1 (a power of two)
    int conn_shift;                // 64 - log2(slots)
    const float* padf;        // [B] radius + contact margin, rounded up to single precision
    const double* sy;         // [B] yield stress (the beam's instance)
    // Instances: a context holds I lattices stored one after another (I = 1 for a plain
    // context).  Node and beam kernels run over blocks that never straddle two instances,
    // so every block partial belongs to one instance and per-instance totals are sums over
    // an instance's own blocks, in the same order as for that lattice alone.
    int I;
    int n_nblk, n_bblk;       // node blocks, beam blocks
    const int4* nblk;         // [n_nblk] first node, node count, instance, 0
    const int4* bblk;         // [n_bblk] first beam, beam count, instance, 0
    const int4* irange;       // [I] node blocks [x, y), beam blocks [z, w) of the instance
    const int* inst_n;        // [I] nodes of the instance
    const long long* inst_free;  // [I] unlocked DOFs of the instance
    const float2* off;        // [I] (x, z) offset of the instance in the contact grid
    const int* node_inst;     // [N] instance of each node
    const uint8_t* active;    // [I] 0: the instance is not evaluated (its outputs keep old values)
    const uint8_t* trial_inst;  // [I] with trials == 2: 1 where the instance writes its trial states
};

// Elements per mapped block (the launch block size of the mapped kernels).
constexpr int kMapBlock = 256;

#if defined(__CUDACC__)
// Position of a thread of a mapped block: element index, instance; valid == false past the
// block's element count.
struct MapPos {
    int i, inst;
    bool valid;
};
__device__ __forceinline__ MapPos map_pos(const int4* __restrict__ blk) {
    const int4 q = blk[blockIdx.x];
    return MapPos{q.x + int(threadIdx.x), q.z, int(threadIdx.x) < q.y};
}
#endif

struct PhysParams {
    double translation_scale, gravity, centering, contact_k, contact_margin, joint_radius;
    double broad_cell, top;
    float joint_padf;        // joint radius + margin, rounded up to single precision
    float inv_cell_f;        // 1 / broad_cell in single precision (broad-phase cell index)
    int self_contact;
};

// Totals of one evaluation, written by the finalize kernel.
struct EvalOut {
    double energy, elastic, plastic, contact, reaction, max_pen;
    int contacts, nonfinite;
    double beam_energy, node_energy, center_energy, contact_energy, platen_energy;
    int overflow;                    // ContactFlag bits that invalidate this evaluation
    int pad_;
    double rms, gmax;                // residual over free DOFs: sqrt(mean g^2), max |g| (sim.cpp:44-45)
};

// Device scratch of the contact pipeline (contact.cu).  Capacities are host-chosen and
// grown on demand: a kernel that would exceed one sets a bit in flags[0] instead.
enum ContactFlag : uint32_t {
    kOverEntries = 1,    // a bin holds more (cell, shape) entries than bin_slots
    kOverContacts = 2,   // more contacts than contact_cap
    kOverBins = 4,       // the grid needs more bins than bin_cap
    kNonFinite = 8,      // a shape has a non-finite bounding box (informational)
    kOverSpan = 16,      // a shape spans more cells than allowed: coarsen the grid
    kOverCandidates = 32 // more narrow-phase candidates than cand_cap
};

struct ContactBufs {
    // per shape (S = N + B)
    int4* cell_lo;          // [S] first cell (i, j, k) relative to the grid origin
    int4* cell_hi;          // [S] last cell
    uint4* rec;             // [S] pair-test record: quantized AABB (3 words), packed first cell
    int* grid;              // [16]: origin i,j,k; dims i,j,k; mode; valid; bins; bins needed;
                            //       box quantization scale x,y,z and origin x,y,z (float bits)
    uint32_t* flags;        // [5]: [0] ContactFlag bits of this evaluation, [1] candidate list
                            //      rebuilt by this evaluation, [2] rebuild forced (by the host,
                            //      or by a build that overflowed), [3] the pair pass's
                            //      occupied-bin cursor, [4] builds since allocation
    float4* xref;           // [N] node positions (FP32, rounded down) when the list was built
    // bins of fixed capacity: the shapes of bin b at bin_items[b * bin_slots ...]
    long long bin_cap;
    int bin_slots;          // entries a bin holds, a power of two
    uint32_t* bin_count;    // [bin_cap+1] entries counted per bin (may exceed bin_slots)
    uint32_t* bin_items;    // [bin_cap * bin_slots]
    uint32_t* nentries;     // [3]: [0] cell entries of the last build, [1] the largest bin count
                            //      above bin_slots (0 when every bin fitted), [2] bins holding
                            //      two or more entries
    // narrow-phase candidates: one flat list, appended by the pair grid's warps in chunks
    int pair_blocks;        // blocks of the pair grid (8 warps each)
    long long cand_cap;     // candidate slots, a multiple of 32
    uint2* cand;            // [cand_cap] (lower shape, higher shape)
    uint32_t* ncand;        // [1] candidates found by the last build (may exceed cand_cap)
    // filtered candidates (the ones that can reach contact before the next build), in order
    uint2* cand2;           // [cand_cap]
    uint32_t* fbits;        // [chunks] keep bit per candidate (chunks = cand_cap / 32)
    uint32_t* fcount;       // [chunks + 1] kept per chunk
    uint32_t* foff;         // [chunks + 1] scan of fcount; foff[chunks] = filtered list length
    // narrow phase, per chunk of 32 consecutive filtered candidates
    uint32_t* hitbits;      // [chunks] contact bit per candidate
    uint32_t* hcount;       // [chunks + 1] contacts per chunk
    uint32_t* hoff;         // [chunks + 1] scan of hcount; hoff[chunks] = contact count
    long long contact_cap;
    uint32_t* c_a;          // lower shape index
    uint32_t* c_b;          // higher shape index
    double* c_s;            // closest-point parameters on a and b
    double* c_t;
    double* c_n;            // [3 * cap] unit normal from a to b
    double* c_pen;          // penetration
    // per-node contact force lists (CSR built per evaluation)
    uint32_t* n_count;      // [N+1]
    uint32_t* n_start;      // [N+1]
    uint32_t* n_cursor;     // [N] fill cursor; then, for a node in n_long, its place there
    uint32_t* n_items;      // [4 * contact_cap]  (contact << 2 | slot), in arrival order
    uint32_t* n_sorted;     // [4 * contact_cap]  the same per node, by (lower shape, higher shape, slot)
    uint32_t* n_long;       // [N + 1] count, then the nodes whose lists exceed one warp
    // [6 * N] or null: per node of n_long (by its place there), the sums of its list --
    // force (3), self-contact energy, contacts, largest penetration -- taken by the gather
    // instead of walking the list (null: the gather walks every list)
    double* long_sum;
    void* scan_tmp;
    size_t scan_tmp_bytes;
};

// per node block: gravity E, platen E, reaction, max penetration, contacts, self-contact E,
// sum of squared free gradient entries, max |free gradient entry|
constexpr int kNodeParts = 8;
constexpr int kFinPartDoubles = 32 * 11;  // per instance: 32 first-stage blocks x 11 totals

struct EvalBufs {
    double4_32a* x;             // [N]
    double4_32a* R;             // [N]
    double4_32a* M;             // [3N] rotation matrix rows of R (x, y, z, pad)
    float4* xf_lo;              // [N] position rounded down to single precision
    float4* xf_hi;              // [N] position rounded up
    double* slotA;          // [6B] (-F, Ga) per beam, added to node a
    double* slotB;          // [6B] (+F, Gb) per beam, added to node b
    double* part_state;     // [9 * nb_nodes] sum, -min, max of x per block
    double* part_beam;      // [3 * nb_beams]
    unsigned* err;          // [1] a kernel's bounded wait gave up (the host reports it)
    double* part_node;      // [kNodeParts * nb_nodes]
    double* part_fin;       // [I * kFinPartDoubles] first-stage totals of the finalize
    double* cen;            // [9 (I + 1)] per instance mean, min, max of the node positions (min/max
                            //   in the contact grid's frame); then min/max over all instances
    double* tops;           // [I] platen height per instance
    EvalOut* out;           // [I]
    double* trial_next;     // [7B] SoA
    double* trial_aux;      // [7B] SoA
    uint8_t* trial_flags;   // [3B] SoA
    // mixed-precision form
    float* slotAf;          // [6B]
    float* slotBf;          // [6B]
    float* trial_nextf;     // [7B] SoA
    float* trial_auxf;      // [7B] SoA
};

// Per-beam data of the mixed-precision form (objective_mixed.cu), float4 SoA.
struct MixedBeams {
    float4* B0;  // base chord d0 (FP32-rounded), c0 = |d0|^2 - L0^2
    float4* B1;  // base shear vector d_a0 - t0, L0
    float4* B2;  // base shear vector d_b0 - t0, |d0|
    float4* B5;  // base relative rotation Q0 as (w - 1, v)
    float4* P0;  // plastic: epsp, alpha, alphaB, alphaT
    float4* P1;  // plastic: rotp; radius
    // Section constants.  When every beam's area, I and J are the circular section's
    // (pi r^2, pi r^4 / 4, 2 I, MC/src/sim.cpp:115) they are formed in the kernel from r and
    // L0 with the factors below and C0/C1 stay null; otherwise they are streamed.
    float4* C0;  // kb, kt, my, ty (streamed form only)
    float4* C1;  // cs, area L0, area, area L0 yield (streamed form only)
    float4* ic;  // [I] per instance: yield, yield pi/4, yield pi/(2 sqrt 3), yield pi
    float4 kg;   // E pi/4, G pi/2, shear G pi/2, pi
};
// Per-node data of the mixed-precision form.
struct MixedNodes {
    float4* UE;   // [2 N] per node, one 32-byte sector: the increment displacement s t since
                  // the base state, then the increment rotation exp(r) as (w - 1, v)
    float4* R0f;  // base orientation (w, x, y, z)
};

// ---- launch accounting -------------------------------------------------------------------
extern std::atomic<long long> g_launch_count;
inline void note_launches(int k) { g_launch_count += k; }

// ---- launchers (objective.cu) ----------------------------------------------------------
int nb_nodes(int N);
int nb_beams(int B);
void launch_state(const DevTopo& t, const PhysParams& p, const double* z, const double* base_x,
                  const double* base_r, EvalBufs& e, cudaStream_t s);
// Occupancy variants of the beam kernels and the gather (CTAs per SM the register allocation
// allows; the arithmetic is the same in every variant).  Variant 0 is the default.
enum class ShapeKernel { kBeams, kBeamsMixed, kGather };
int shape_variants(ShapeKernel k);
int shape_blocks(ShapeKernel k, int variant);
int beams_mixed_variants();
// Once per context, outside any stream capture: the staged variants' shared-memory limit and
// the SM count that sizes their persistent grid.
void prepare_beams_mixed(int device);
int beams_mixed_blocks(int variant);
void launch_beams(const DevTopo& t, const Material& m, const double* plastic, int trials,
                  EvalBufs& e, cudaStream_t s, int variant = 0);
void launch_gather(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad,
                   EvalBufs& e, cudaStream_t s, int variant = 0);
void launch_finalize(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad,
                     EvalBufs& e, cudaStream_t s);
// base state <- current state, plastic <- trial (plastic == nullptr skips it) for the
// instances with mask[i] != 0 (mask == nullptr: all)
void launch_commit(const DevTopo& t, const uint8_t* mask, const EvalBufs& e, double* base_x, double* base_r,
                   double* plastic, cudaStream_t s);
void launch_center(const DevTopo& t, EvalBufs& e, cudaStream_t s);
void launch_gather_mixed(const DevTopo& t, const PhysParams& p, const ContactBufs* c, double* grad, EvalBufs& e,
                         cudaStream_t s, int variant = 0);

// ---- mixed-precision form (objective_mixed.cu) ------------------------------------------
void launch_state_mixed(const DevTopo& t, const PhysParams& p, const double* z, const double* base_x,
                        const MixedNodes& mn, EvalBufs& e, cudaStream_t s);
void launch_beams_mixed(const DevTopo& t, const Material& m, const MixedBeams& mb, const MixedNodes& mn, int trials,
                        EvalBufs& e, cudaStream_t s, int variant = 0);
void launch_rebase_mixed(const DevTopo& t, const double* base_x, const double* base_r, MixedBeams& mb,
                         MixedNodes& mn, cudaStream_t s);
// The streamed section constants (mb.C0/C1, when allocated), once per upload.
void launch_mixed_constants(const DevTopo& t, MixedBeams& mb, cudaStream_t s);
// plastic state of the mixed form from the FP64 SoA array (trial32 == nullptr, all beams) or
// from an FP32 trial (the beams of the instances with mask[i] != 0; mask == nullptr: all)
void launch_plastic_mixed(const DevTopo& t, const uint8_t* mask, const double* plastic64, const float* trial32,
                          MixedBeams& mb, cudaStream_t s);
void launch_plastic_mixed_to_f64(const DevTopo& t, const uint8_t* mask, const MixedBeams& mb, double* plastic64,
                                 cudaStream_t s);
void launch_f32_to_f64(long long n, const float* a, double* o, cudaStream_t s);
// out6[6 i..]: per instance sum|epsp|, max|epsp|, sum|rotp|, max|rotp|, #|epsp|>1e-5, #|rotp|>1e-4
// (part: 6 doubles per beam block)
void launch_plastic_stats(const DevTopo& t, const double* plastic, double* part, double* out6, cudaStream_t s);

// ---- contact pipeline (contact.cu) ------------------------------------------------------
// Blocks of the pair / narrow-phase grid for a model of `shapes` shapes (8 warps each).
int contact_pair_blocks(long long shapes);
// The whole broad/narrow phase: grid, entries, bins, pairs, contact list, node lists.
// The candidate list is rebuilt only when a node has moved more than skin (m, per axis)
// since the last build, or the host forced it (flags[2]); skin <= 0 rebuilds every time.
// pairs_begin / pairs_end (may be null) are recorded around the pair enumeration.
void launch_contacts(const DevTopo& t, const PhysParams& p, const EvalBufs& e, ContactBufs& c, double pad,
                     float skin, cudaStream_t s, cudaEvent_t pairs_begin = nullptr, cudaEvent_t pairs_end = nullptr);

// ---- scan (sort.cu) -----------------------------------------------------------------------
size_t scan_tmp_bytes(long long n);
// Exclusive scan of n uint32 values; out[n] receives the total.
// Exclusive scan of n counts into out[0..n] (out[n] = total).  With a gate, every kernel
// returns at once when *gate is 0 (the output keeps its previous contents).  With dn, only
// the first min(n, (*dn + add) >> shift) counts are scanned (a count known on the device;
// the total also goes to out[n]).
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, long long n, void* tmp, cudaStream_t s,
                        const uint32_t* gate = nullptr, const uint32_t* dn = nullptr, int add = 0, int shift = 0);

// ---- L-BFGS vector kernels (lbfgs.cu), all instances of a context per launch --------------
// Operations an instance takes part in during one solver step (SolveCtl::flags).
enum SolveOp : int {
    kOpDirection = 1,      // two-loop direction from g, clamp, <g, p>
    kOpSteepest = 2,       // p = clamp(-g), <g, p>
    kOpZero = 4,           // z = 0
    kOpRestore = 8,        // z = best
    kOpKeepBest = 16,      // best = z
    kOpCandidate = 32,     // zeval = z + step p
    kOpEvalAtZ = 64,       // zeval = z
    kOpFinal = 128,        // zfinal = z
    kOpTakeGrad = 256,     // g = geval
    kOpAccept = 512,       // s, y, curvature dots, z = zeval, g = geval
    kOpPair = 1024,        // with kOpAccept: store (s, y) in history slot `target`
    kOpKeepBestAfter = 2048, // with kOpAccept: best = the accepted z
    kOpDirFused = 4096,      // as kOpDirection, by one CTA for the instance (small instances)
    kOpResetHistory = 8192   // the history starts empty (a new minimization)
};
// Per-instance solver control, written by the host before each step.  The history state
// (pairs held m, oldest slot head) lives on the device (int2 per instance) and is filled in
// by the kernels.
struct SolveCtl {
    double step;       // line-search step of the candidate
    int flags;         // SolveOp bits
    int m, head;       // (device history, loaded by the kernels)
    int pad_;
};
size_t lbfgs_part_doubles(int n_nblk);
// Largest instance (in node blocks) whose direction one CTA computes (kOpDirFused).
int fused_direction_limit();
// Two-loop recursion (sim.cpp:184-187) into p for the kOpDirFused (one CTA each) and, with
// multi, the kOpDirection instances; then p = clamp(lock(-p)) and dg[i] = <g, p>; where
// not dg < 0, steepest descent with the history cleared (sim.cpp:191).
// History: H slots of `stride` doubles, state hist[I], rho and alpha [I * H].
void bl_direction(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, bool multi, double* p, const double* g,
                  const double* S, const double* Y, long long stride, const double* rho, double* alpha, double* part,
                  double* dg, double mt, double mr, cudaStream_t s);
// The pieces of bl_direction, for callers that launch them under separate conditions: the
// one-CTA directions (kOpDirFused), the multi-block two-loop (kOpDirection), and the
// steepest-descent fallback of either kind where <g, p> >= 0.
void bl_direction_fused(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, double* p, const double* g,
                        const double* S, const double* Y, long long stride, const double* rho, double* dg, double mt,
                        double mr, cudaStream_t s);
void bl_direction_multi(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, double* p, const double* g,
                        const double* S, const double* Y, long long stride, const double* rho, double* alpha,
                        double* part, double* dg, double mt, double mr, cudaStream_t s);
void bl_descent_fix(const DevTopo& t, const SolveCtl* ctl, int2* hist, double* p, const double* g, double* part,
                    double* dg, double mt, double mr, cudaStream_t s);
// The steepest-descent retry for the kOpSteepest instances: history cleared,
// p = clamp(lock(-g)), dg[i] = <g, p> (sim.cpp:193-196).
void bl_steepest(const DevTopo& t, const SolveCtl* ctl, int2* hist, double* p, const double* g, double* part,
                 double* dg, double mt, double mr, cudaStream_t s);
// kOpResetHistory / kOpZero / kOpRestore / kOpKeepBest / kOpCandidate / kOpEvalAtZ / kOpFinal
void bl_prepare(const DevTopo& t, const SolveCtl* ctl, int2* hist, double* z, double* best, double* zeval,
                const double* p, double* zfinal, cudaStream_t s);
// kOpTakeGrad / kOpAccept (+kOpPair, kOpKeepBestAfter); out3[3 i..] = <s, y>, <s, s>, <y, y>;
// then the history update of the accepted instances (sim.cpp:205-206).
void bl_accept(const DevTopo& t, const SolveCtl* ctl, int2* hist, int H, double* z, double* g, const double* zeval,
               const double* geval, double* S, double* Y, long long stride, double* best, double* rho, double* part,
               double* out3, cudaStream_t s);

}  // namespace mcg
