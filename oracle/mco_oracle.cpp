// mco_oracle.cpp -- TEST INFRASTRUCTURE ONLY: the CPU restatement of the reference's
// beam-lattice energy/gradient and L-BFGS path, used as the parity checker for the GPU
// library and as the timed CPU baseline.  It is never linked by, or called from, the
// product library.
//
// Reference: projects/metamaterial-compression/industry-grade ("MC/"), files
// MC/include/core.hpp, MC/include/sim.hpp, MC/src/sim.cpp.  Each function below names the
// lines it follows.  The floating-point expressions keep the reference's operation order
// (including its habit of dividing vectors by multiplying with a reciprocal) and its
// hash-grid container and iteration order, so that this file rounds exactly like the
// reference on the same compiler and architecture; oracle/ref_harness.cpp compiles the
// reference itself and tests/test_oracle.py checks the two bit for bit.
//
// Parity of this restatement is pinned by (a) bitwise comparison with the reference
// solver built from its sources (objective, pair sets, minimize, full runs) and (b) the
// reference's published step-refinement results (MC/docs/VALIDATION.md:45-49).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <stdexcept>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "oracle.h"
#include "specimens.h"

namespace {

constexpr double kPi = 3.1415926535897932384626433832795;  // core.hpp:28
constexpr double kInf = std::numeric_limits<double>::infinity();

// ---- scalar helpers (core.hpp:30-33) -------------------------------------------------
inline double clampd(double x, double lo, double hi) { return std::max(lo, std::min(hi, x)); }
inline double sat(double x) { return clampd(x, 0.0, 1.0); }
inline double sqr(double x) { return x * x; }
inline double mix1(double a, double b, double t) { return a * (1.0 - t) + b * t; }

// ---- 3-vectors (core.hpp:37-39) ------------------------------------------------------
struct V3 {
    double x = 0, y = 0, z = 0;
    V3() = default;
    V3(double X, double Y, double Z) : x(X), y(Y), z(Z) {}
    static V3 all(double s) { return {s, s, s}; }
    double& at(int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(const V3& a) { return {-a.x, -a.y, -a.z}; }
inline V3 scale(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
// The reference divides a vector by s as a multiplication with 1/s (core.hpp:37).
inline V3 divide(const V3& a, double s) { return scale(a, 1.0 / s); }
inline void addTo(V3& a, const V3& b) { a.x += b.x; a.y += b.y; a.z += b.z; }
inline void subFrom(V3& a, const V3& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
inline double dot3(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross3(const V3& a, const V3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double len2(const V3& v) { return dot3(v, v); }
inline double len(const V3& v) { return std::sqrt(len2(v)); }
inline V3 unit(const V3& v) {
    const double l2 = len2(v);
    return std::isfinite(l2) && l2 > 1e-30 ? divide(v, std::sqrt(l2)) : V3{0, 1, 0};
}
inline V3 vmin3(const V3& a, const V3& b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
inline V3 vmax3(const V3& a, const V3& b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
inline V3 perpendicular(const V3& n) {  // core.hpp:47 orthogonal
    V3 h = std::abs(n.z) < .8 ? V3{0, 0, 1} : V3{0, 1, 0};
    return unit(cross3(h, n));
}

// ---- quaternions (core.hpp:40-42, 51-53) ----------------------------------------------
struct Q4 {
    double w = 1, x = 0, y = 0, z = 0;
    Q4() = default;
    Q4(double W, double X, double Y, double Z) : w(W), x(X), y(Y), z(Z) {}
};
inline Q4 conj(const Q4& q) { return {q.w, -q.x, -q.y, -q.z}; }
inline Q4 qnorm(Q4 q) {
    const double n = std::sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
    if (n < 1e-30) return Q4{};
    return {q.w / n, q.x / n, q.y / n, q.z / n};
}
inline Q4 qmul(const Q4& a, const Q4& b) {
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
            a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}
// v' = v + w t + q x t with t = 2 q x v (core.hpp:40 Quat::rotate).
inline V3 qrot(const Q4& q, const V3& v) {
    const V3 u{q.x, q.y, q.z};
    const V3 t = scale(cross3(u, v), 2.0);
    return (v + scale(t, q.w)) + cross3(u, t);
}
inline V3 qrotInv(const Q4& q, const V3& v) { return qrot(conj(q), v); }
inline Q4 fromAxisAngle(V3 axis, double angle) {  // core.hpp:42
    axis = unit(axis);
    const double s = std::sin(.5 * angle);
    return qnorm({std::cos(.5 * angle), axis.x * s, axis.y * s, axis.z * s});
}
inline Q4 expMap(const V3& v) {  // core.hpp:51
    const double a = len(v);
    if (a < 1e-12) return qnorm({1 - .125 * a * a, .5 * v.x, .5 * v.y, .5 * v.z});
    return fromAxisAngle(divide(v, a), a);
}
inline V3 logMap(Q4 q) {  // core.hpp:52
    q = qnorm(q);
    if (q.w < 0) q = {-q.w, -q.x, -q.y, -q.z};
    const double s = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z);
    if (s < 1e-12) return {2 * q.x, 2 * q.y, 2 * q.z};
    const double a = 2 * std::atan2(s, clampd(q.w, -1, 1));
    return scale(V3{q.x, q.y, q.z}, a / s);
}
// J_l^{-T}(p) v for the SO(3) left Jacobian (core.hpp:53), with its series branch.
inline V3 jlInvT(const V3& p, const V3& v) {
    const double a = len(p);
    const V3 c1 = cross3(p, v);
    const V3 c2 = cross3(p, c1);
    if (a < 1e-7) return (v + scale(c1, .5)) + scale(c2, 1.0 / 12.0);
    const double A = 1 / (a * a) - (1 + std::cos(a)) / (2 * a * std::sin(a));
    return (v + scale(c1, .5)) + scale(c2, A);
}

inline uint64_t mix64(uint64_t x) {  // core.hpp:46 splitmix64
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}
struct Rng {  // core.hpp:46 RNG
    uint64_t state;
    explicit Rng(uint64_t seed) : state(mix64(seed)) {}
    uint32_t next32() { state = mix64(state); return uint32_t(state >> 32); }
    double uniform() { return (double(next32()) + .5) / 4294967296.0; }
    double signedUniform() { return 2 * uniform() - 1; }
};
struct CellHash {  // core.hpp:47 Int3Hash
    size_t operator()(int64_t k) const noexcept { return size_t(mix64(uint64_t(k))); }
};
inline int64_t gridKey(int x, int y, int z) {  // core.hpp:47 cellKey
    constexpr int64_t B = 1LL << 20, M = (1LL << 21) - 1;
    return ((int64_t(x) + B) & M) | (((int64_t(y) + B) & M) << 21) | (((int64_t(z) + B) & M) << 42);
}
inline uint64_t keyOf(int a, int b) {  // core.hpp:47 pairKey
    if (a > b) std::swap(a, b);
    return (uint64_t(uint32_t(a)) << 32) | uint32_t(b);
}

// ---- constitutive return maps (sim.cpp:5-8) -------------------------------------------
struct Ret1 { double force = 0, p = 0, a = 0, dg = 0, energy = 0, hard = 0; bool yielded = false; };
// 1-D elastoplastic return with linear isotropic hardening.
Ret1 return1(double total, double pc, double ac, double k, double y, double H) {
    Ret1 r;
    const double trial = k * (total - pc);
    const double f = std::abs(trial) - (y + H * ac);
    if (f > 0) {
        const double s = trial >= 0 ? 1 : -1;
        r.dg = f / std::max(1e-20, k + H);
        r.p = pc + s * r.dg;
        r.a = ac + r.dg;
        r.yielded = true;
    } else {
        r.p = pc;
        r.a = ac;
    }
    r.force = k * (total - r.p);
    r.energy = .5 * k * sqr(total - r.p);
    r.hard = .5 * H * sqr(r.a);
    return r;
}
struct Ret3 { V3 force, p; double a = 0, dg = 0, energy = 0, hard = 0; bool yielded = false; };
// Radial return of a 3-vector (bending).
Ret3 return3(const V3& t, const V3& pc, double ac, double k, double y, double H) {
    Ret3 r;
    const V3 trial = scale(t - pc, k);
    const double n = len(trial);
    const double f = n - (y + H * ac);
    if (f > 0 && n > 1e-20) {
        const V3 d = divide(trial, n);
        r.dg = f / std::max(1e-20, k + H);
        r.p = pc + scale(d, r.dg);
        r.a = ac + r.dg;
        r.yielded = true;
    } else {
        r.p = pc;
        r.a = ac;
    }
    r.force = scale(t - r.p, k);
    r.energy = .5 * k * len2(t - r.p);
    r.hard = .5 * H * sqr(r.a);
    return r;
}

// ---- contact geometry (sim.cpp:9-39) ---------------------------------------------------
struct Shape { V3 a, b; double r = 0; int n0 = -1, n1 = -1, beam = -1; bool capsule = false; };
struct Closest { double s = 0, t = 0; V3 pa, pb; };
Closest segSeg(const V3& p1, const V3& q1, const V3& p2, const V3& q2) {  // sim.cpp:11-16
    const V3 d1 = q1 - p1, d2 = q2 - p2, r = p1 - p2;
    const double a = dot3(d1, d1), e = dot3(d2, d2), f = dot3(d2, r);
    double s = 0, t = 0;
    if (a <= 1e-20 && e <= 1e-20) return {0, 0, p1, p2};
    if (a <= 1e-20) {
        s = 0;
        t = sat(f / e);
    } else {
        const double c = dot3(d1, r);
        if (e <= 1e-20) {
            t = 0;
            s = sat(-c / a);
        } else {
            const double b = dot3(d1, d2), den = a * e - b * b;
            s = std::abs(den) > 1e-20 ? sat((b * f - c * e) / den) : 0;
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
    return {s, t, p1 + scale(d1, s), p2 + scale(d2, t)};
}
Closest shapeClosest(const Shape& a, const Shape& b) {  // sim.cpp:17-22
    if (a.capsule && b.capsule) return segSeg(a.a, a.b, b.a, b.b);
    if (a.capsule && !b.capsule) {
        const V3 d = a.b - a.a;
        const double s = sat(dot3(b.a - a.a, d) / std::max(1e-30, len2(d)));
        return {s, 0, a.a + scale(d, s), b.a};
    }
    if (!a.capsule && b.capsule) {
        const V3 d = b.b - b.a;
        const double t = sat(dot3(a.a - b.a, d) / std::max(1e-30, len2(d)));
        return {0, t, a.a, b.a + scale(d, t)};
    }
    return {0, 0, a.a, b.a};
}
void spreadForce(std::vector<V3>& g, const Shape& s, double u, const V3& v) {  // sim.cpp:23
    if (s.capsule) {
        addTo(g[size_t(s.n0)], scale(v, 1 - u));
        addTo(g[size_t(s.n1)], scale(v, u));
    } else {
        addTo(g[size_t(s.n0)], v);
    }
}
// Same beam, a shared node, or a `connected` node pair (sim.cpp:24-39).
bool excluded(const Shape& a, const Shape& b, const std::unordered_set<uint64_t>& connected) {
    if (a.beam >= 0 && a.beam == b.beam) return true;
    const int an[2] = {a.n0, a.n1}, bn[2] = {b.n0, b.n1};
    const int na = a.capsule ? 2 : 1, nb = b.capsule ? 2 : 1;
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            if (an[i] == bn[j]) return true;
            if (connected.count(keyOf(an[i], bn[j]))) return true;
        }
    return false;
}

// ---- model ---------------------------------------------------------------------------
struct Plastic { double epsp = 0, alpha = 0; V3 rotp; double alphaB = 0, alphaT = 0; };
struct NodeRec { V3 x0, x; Q4 R; double mass = 0; int layer = 0; };
struct BeamRec {
    int a = -1, b = -1, layer = 0, family = 0;
    double L0 = 0, radius = .001, area = 0, I = 0, J = 0;
    V3 e0{1, 0, 0};
    Plastic plastic;
};
struct Trial {
    Plastic next;
    double strain = 0, stress = 0;
    V3 moment;
    double elastic = 0, dissipation = 0;
    bool axialPlastic = false, bendPlastic = false, torsionPlastic = false;
};
struct Diag { double elastic = 0, plastic = 0, contact = 0, reaction = 0, maxPen = 0; int contacts = 0; };
struct Eval { double energy = 0; std::vector<double> grad; Diag d; std::vector<Trial> trial; };
struct Stats { int iterations = 0, backtracks = 0; double rms = kInf, max = kInf, energy = kInf; bool converged = false; };

}  // namespace

struct orc_model {
    mcg_config cfg{};
    std::vector<NodeRec> nodes;
    std::vector<BeamRec> beams;
    std::unordered_set<uint64_t> connected;
    std::vector<uint8_t> locked;
    std::vector<V3> baseX;
    std::vector<Q4> baseR;
    double width = 0, height = 0, depth = 0, area = 0, mass = 0, top0 = 0;
    // run() bookkeeping (sim.hpp:47)
    double loadingWork = 0, recoveredWork = 0, prevDisp = 0, prevForce = 0, reactionOffset = 0;
    // Rounding-order variant (0 = the reference's order).  Bits: 1 adds gravity to the node
    // forces before the beam loop, 2 scatters the beams in descending order, 4 adds the
    // centering force before the beam loop, 8 adds the platen forces before the
    // self-contact forces, 16 scatters the odd-numbered beams before the even-numbered
    // ones.  Each is the same sum in another order; runs under these variants measure how
    // far rounding alone moves a load/unload trajectory.
    int variant = 0;
    // last minimize, for commit
    std::vector<double> lastZ;
    Eval lastFinal;
    bool haveFinal = false;
    // Objective hook: when set, objective() forwards to this energy/gradient implementation
    // (whose signature is mcg_objective's) instead of evaluating here, and commit() hands the
    // re-based state to stateHook (mcg_set_state's signature).  minimize, run and the
    // verification checks stay exactly as they are: this is the reference driver calling an
    // external objective through its unchanged interface.  A non-zero hook status is kept in
    // hookStatus and the evaluation reads as non-finite, which the driver rejects.
    orc_objective_fn objHook = nullptr;
    orc_state_fn stateHook = nullptr;
    void* hookCtx = nullptr;
    mutable int hookStatus = 0;
    mutable long long hookCalls = 0;
    // When on, each evaluation keeps its sorted self-contact pair set here.
    bool recordPairs = false;
    mutable std::vector<uint64_t> lastPairs;

    double jointRadius() const { return cfg.joint_scale * cfg.max_radius; }

    // -- lattice builder: Simulator::build, sim.cpp:51-132 -------------------------------
    void build() {
        const int nx = cfg.cells_x, ny = cfg.cells_y, nz = cfg.cells_z;
        const int corners = (nx + 1) * (ny + 1) * (nz + 1);
        auto corner = [&](int i, int j, int k) { return (j * (nz + 1) + k) * (nx + 1) + i; };
        auto center = [&](int i, int j, int k) { return corners + (j * nz + k) * nx + i; };
        const double cs = cfg.cell_size;
        width = nx * cs; height = ny * cs; depth = nz * cs; area = width * depth;
        const double jr = jointRadius();
        const V3 origin{-.5 * width, jr, -.5 * depth};
        Rng rng(cfg.seed);
        nodes.clear(); beams.clear(); connected.clear();
        for (int j = 0; j <= ny; j++)
            for (int k = 0; k <= nz; k++)
                for (int i = 0; i <= nx; i++) {  // corner nodes, sim.cpp:63-69
                    NodeRec n;
                    n.x0 = origin + V3{i * cs, j * cs, k * cs};
                    const double yf = double(j) / ny, env = std::sin(kPi * yf);
                    const double sg = ((i + 2 * k + 3 * j) & 1) ? 1.0 : -1.0;
                    n.x0.x += cfg.imperfection * env * (.55 * sg + .45 * rng.signedUniform());
                    n.x0.z += cfg.imperfection * env * (.35 * sg + .65 * rng.signedUniform());
                    n.x = n.x0; n.layer = j;
                    nodes.push_back(n);
                }
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                for (int i = 0; i < nx; i++) {  // BCC centres, sim.cpp:70-82
                    NodeRec n;
                    n.x0 = origin + V3{(i + .5) * cs, (j + .5) * cs, (k + .5) * cs};
                    const double yf = (j + .5) / double(ny), env = std::sin(kPi * yf);
                    const double sg = ((i + k + j) & 1) ? 1.0 : -1.0;
                    const double sx = (j & 1) ? -1.0 : 1.0, sz = ((j / 2) & 1) ? -1.0 : 1.0;
                    n.x0.x += cs * (.082 * (1 - .32 * yf) * sx + .018 * env * sg)
                              + 1.2 * cfg.imperfection * env * rng.signedUniform();
                    n.x0.z += cs * (.032 * (.65 + .35 * (1 - yf)) * sz - .012 * env * sg)
                              + 1.2 * cfg.imperfection * env * rng.signedUniform();
                    n.x = n.x0; n.layer = j;
                    nodes.push_back(n);
                }
        std::unordered_set<uint64_t> physical;
        auto strutRadius = [&](int a, int b, int layer, double s) {  // sim.cpp:84-93
            const V3 m = scale(nodes[size_t(a)].x0 + nodes[size_t(b)].x0, .5);
            const double y = sat((m.y - jr) / height);
            const double radial = sat(std::sqrt(m.x * m.x + m.z * m.z) / (.72 * std::max(width, depth)));
            double grade = .58 + .42 * std::pow(1 - y, .72);
            grade *= .94 + .12 * radial;
            if (layer == 0) grade *= cfg.trigger_scale;
            else if (layer == 1) grade *= std::sqrt(cfg.trigger_scale);
            else if (layer == 2) grade *= .88;
            return s * mix1(cfg.min_radius, cfg.max_radius, sat(grade));
        };
        auto strut = [&](int a, int b, int layer, int family, double s) {  // sim.cpp:94-118
            const uint64_t key = keyOf(a, b);
            if (a == b || !physical.insert(key).second) return;
            const V3 pa = nodes[size_t(a)].x0, pb = nodes[size_t(b)].x0, d = pb - pa;
            const V3 tangent = unit(d);
            const uint64_t h = mix64(cfg.seed ^ key ^ uint64_t(family + 31) * 0x9e3779b97f4a7c15ULL);
            const V3 helper{double(int((h >> 0) & 1023) - 511), double(int((h >> 10) & 1023) - 511),
                            double(int((h >> 20) & 1023) - 511)};
            V3 axis = cross3(tangent, helper);
            axis = len2(axis) < 1e-12 ? perpendicular(tangent) : unit(axis);
            const V3 axis2 = unit(cross3(tangent, axis));
            const double layerFactor = layer == 0 ? 2.60 : (layer == 1 ? 1.60 : 1.0);
            const double amplitude = cfg.member_imperfection * layerFactor *
                                     (.55 + .90 * double((h >> 32) & 65535) / 65535.0);
            const int segments = std::clamp(cfg.elements_per_strut, 2, 5);
            std::vector<int> chain{a};
            for (int sg = 1; sg < segments; sg++) {
                const double t = double(sg) / segments;
                NodeRec mid;
                mid.x0 = ((scale(pa, 1 - t) + scale(pb, t)) + scale(axis, std::sin(kPi * t) * amplitude)) +
                         scale(axis2, .22 * std::sin(2 * kPi * t) * amplitude);
                mid.x = mid.x0; mid.layer = layer;
                chain.push_back(int(nodes.size()));
                nodes.push_back(mid);
            }
            chain.push_back(b);
            const double r = strutRadius(a, b, layer, s);
            for (size_t q = 0; q + 1 < chain.size(); q++) {
                const int u = chain[q], v = chain[q + 1];
                BeamRec e;
                e.a = u; e.b = v; e.layer = layer; e.family = family;
                const V3 ed = nodes[size_t(v)].x0 - nodes[size_t(u)].x0;
                e.L0 = len(ed); e.e0 = unit(ed); e.radius = r;
                e.area = kPi * r * r; e.I = .25 * kPi * std::pow(r, 4); e.J = 2 * e.I;
                beams.push_back(e);
                connected.insert(keyOf(u, v));
            }
            connected.insert(key);
        };
        static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                for (int i = 0; i < nx; i++) {
                    const int c = center(i, j, k);
                    for (int q = 0; q < 8; q++)
                        strut(c, corner(i + off[q][0], j + off[q][1], k + off[q][2]), j, q, 1.0);
                }
        for (int face : {0, ny}) {  // face grids, sim.cpp:127-130
            for (int k = 0; k <= nz; k++)
                for (int i = 0; i < nx; i++)
                    strut(corner(i, face, k), corner(i + 1, face, k), std::clamp(face, 0, ny - 1), 30, .62);
            for (int i = 0; i <= nx; i++)
                for (int k = 0; k < nz; k++)
                    strut(corner(i, face, k), corner(i, face, k + 1), std::clamp(face, 0, ny - 1), 31, .62);
        }
        top0 = jr + height + jr;
    }

    // -- Simulator::distributeMass, sim.cpp:134 -----------------------------------------
    void distributeMass() {
        mass = 0;
        for (NodeRec& n : nodes) n.mass = 0;
        for (const BeamRec& e : beams) {
            const double m = cfg.material.density * e.area * e.L0;
            nodes[size_t(e.a)].mass += .5 * m;
            nodes[size_t(e.b)].mass += .5 * m;
            mass += m;
        }
        const double jr = jointRadius();
        const double jm = cfg.material.density * (4.0 / 3.0) * kPi * std::pow(jr, 3) * .28;
        for (NodeRec& n : nodes) { n.mass += jm; mass += jm; }
        locked.assign(nodes.size() * 6, 0);
        int a = -1, b = -1;
        double da = kInf, db = kInf;
        for (int i = 0; i < int(nodes.size()); i++)
            if (nodes[size_t(i)].layer == 0) {
                const V3 p = nodes[size_t(i)].x0;
                const double qa = sqr(p.x + .5 * width) + sqr(p.z + .5 * depth);
                const double qb = sqr(p.x - .5 * width) + sqr(p.z + .5 * depth);
                if (qa < da) { da = qa; a = i; }
                if (qb < db) { db = qb; b = i; }
            }
        if (a < 0 || b < 0) throw std::runtime_error("failed to create anti-drift constraints");
        locked[size_t(6 * a)] = 1; locked[size_t(6 * a + 2)] = 1; locked[size_t(6 * b + 2)] = 1;
    }

    void resetBase() {
        baseX.resize(nodes.size()); baseR.resize(nodes.size());
        for (size_t i = 0; i < nodes.size(); i++) { baseX[i] = nodes[i].x; baseR[i] = nodes[i].R; }
    }

    // -- Simulator::state, sim.cpp:136 --------------------------------------------------
    void state(const std::vector<double>& z, std::vector<V3>& x, std::vector<Q4>& R) const {
        x.resize(nodes.size()); R.resize(nodes.size());
        for (size_t i = 0; i < nodes.size(); i++) {
            const size_t b = 6 * i;
            V3 t{z[b], z[b + 1], z[b + 2]}, r{z[b + 3], z[b + 4], z[b + 5]};
            for (int d = 0; d < 3; d++) {
                if (locked[b + size_t(d)]) t.at(d) = 0;
                if (locked[b + size_t(d + 3)]) r.at(d) = 0;
            }
            x[i] = baseX[i] + scale(t, cfg.translation_scale);
            R[i] = qnorm(qmul(expMap(r), baseR[i]));
        }
    }

    // -- shapes of the self-contact pass (sim.cpp:148-150) --------------------------------
    std::vector<Shape> shapesOf(const std::vector<V3>& x) const {
        const double jr = jointRadius();
        std::vector<Shape> shapes;
        shapes.reserve(nodes.size() + beams.size());
        for (int i = 0; i < int(nodes.size()); i++) shapes.push_back({x[size_t(i)], x[size_t(i)], jr, i, -1, -1, false});
        for (int bi = 0; bi < int(beams.size()); bi++) {
            const BeamRec& e = beams[size_t(bi)];
            shapes.push_back({x[size_t(e.a)], x[size_t(e.b)], e.radius, e.a, e.b, bi, true});
        }
        return shapes;
    }

    // Hash-grid broad phase and narrow phase (sim.cpp:151-165).  `visit` receives every
    // contacting pair in the reference's accumulation order.
    template <class F>
    void selfContact(const std::vector<Shape>& shapes, F&& visit) const {
        const double jr = jointRadius();
        const double cell = std::max(2.8 * jr, .72 * cfg.cell_size);
        std::unordered_map<int64_t, std::vector<int>, CellHash> grid;
        grid.reserve(shapes.size() * 3);
        for (int si = 0; si < int(shapes.size()); si++) {
            const Shape& s = shapes[size_t(si)];
            const V3 lo = vmin3(s.a, s.b) - V3::all(s.r + cfg.contact_margin);
            const V3 hi = vmax3(s.a, s.b) + V3::all(s.r + cfg.contact_margin);
            const int i0 = int(std::floor(lo.x / cell)), j0 = int(std::floor(lo.y / cell)), k0 = int(std::floor(lo.z / cell));
            const int i1 = int(std::floor(hi.x / cell)), j1 = int(std::floor(hi.y / cell)), k1 = int(std::floor(hi.z / cell));
            for (int j = j0; j <= j1; j++)
                for (int k = k0; k <= k1; k++)
                    for (int i = i0; i <= i1; i++) grid[gridKey(i, j, k)].push_back(si);
        }
        std::unordered_set<uint64_t> seen;
        seen.reserve(shapes.size() * 8);
        for (const auto& cellEntry : grid) {
            const std::vector<int>& list = cellEntry.second;
            for (size_t ia = 0; ia < list.size(); ia++)
                for (size_t ib = ia + 1; ib < list.size(); ib++) {
                    const int ai = list[ia], bi = list[ib];
                    if (!seen.insert(keyOf(ai, bi)).second) continue;
                    const Shape &a = shapes[size_t(ai)], &b = shapes[size_t(bi)];
                    if (excluded(a, b, connected)) continue;
                    const Closest cp = shapeClosest(a, b);
                    const V3 delta = cp.pb - cp.pa;
                    const double dist = len(delta), target = a.r + b.r + cfg.contact_margin;
                    if (dist >= target) continue;
                    visit(ai, bi, a, b, cp, delta, dist, target);
                }
        }
    }

    // -- Simulator::objective, sim.cpp:138-172 -----------------------------------------
    Eval objective(const std::vector<double>& z, double top, bool trials) const {
        if (objHook) return hookedObjective(z, top, trials);
        Eval o;
        o.grad.assign(nodes.size() * 6, 0);
        if (trials) o.trial.resize(beams.size());
        if (recordPairs) lastPairs.clear();
        std::vector<V3> x, gx(nodes.size()), gr(nodes.size());
        std::vector<Q4> R;
        state(z, x, R);
        const double E = cfg.material.young, G = E / (2 * (1 + cfg.material.nu));
        const double sy = cfg.material.yield, H = cfg.material.hardening;
        V3 cen;  // centering, sim.cpp:143
        for (const V3& p : x) addTo(cen, p);
        cen = divide(cen, double(x.size()));
        if (variant & 1)
            for (size_t i = 0; i < nodes.size(); i++) gx[i].y += nodes[i].mass * cfg.gravity;
        if (variant & 4)
            for (V3& g : gx) {
                g.x += cfg.centering_stiffness * cen.x / x.size();
                g.z += cfg.centering_stiffness * cen.z / x.size();
            }
        const size_t nbeams = beams.size(), nodd = nbeams / 2;
        for (size_t bk = 0; bk < nbeams; bk++) {  // sim.cpp:139-141
            size_t bj = (variant & 2) ? nbeams - 1 - bk : bk;
            if (variant & 16) bj = bj < nodd ? 2 * bj + 1 : 2 * (bj - nodd);
            const size_t bi = bj;
            const BeamRec& e = beams[bi];
            const V3 d = x[size_t(e.b)] - x[size_t(e.a)];
            const double L = len(d);
            if (L < 1e-10) { o.energy += 1e8 * sqr(1e-10 - L); continue; }
            const V3 t = divide(d, L);
            Trial tr;
            // axial
            const double eps = (L - e.L0) / e.L0;
            const Ret1 ax = return1(eps, e.plastic.epsp, e.plastic.alpha, E, sy, H);
            tr.strain = eps; tr.stress = ax.force;
            tr.next = e.plastic; tr.next.epsp = ax.p; tr.next.alpha = ax.a;
            tr.axialPlastic = ax.yielded;
            const double uax = e.area * e.L0 * (ax.energy + ax.hard);
            const double dax = e.area * e.L0 * sy * ax.dg;
            o.energy += uax + dax; o.d.elastic += uax; o.d.plastic += dax;
            const double Nf = e.area * ax.force;
            subFrom(gx[size_t(e.a)], scale(t, Nf));
            addTo(gx[size_t(e.b)], scale(t, Nf));
            // shear: directors against the chord
            const V3 da = qrot(R[size_t(e.a)], e.e0), db = qrot(R[size_t(e.b)], e.e0);
            const double cs = .5 * cfg.shear_correction * G * e.area * e.L0;
            const V3 ma = da - t, mb = db - t;
            const double us = .5 * cs * (len2(ma) + len2(mb));
            o.energy += us; o.d.elastic += us;
            const V3 gt = scale((scale(t, 2) - da) - db, cs);
            const V3 trans = divide(gt - scale(t, dot3(gt, t)), L);
            subFrom(gx[size_t(e.a)], trans);
            addTo(gx[size_t(e.b)], trans);
            subFrom(gr[size_t(e.a)], scale(cross3(da, t), cs));
            subFrom(gr[size_t(e.b)], scale(cross3(db, t), cs));
            // bending and torsion from the relative rotation
            const Q4 Q = qnorm(qmul(conj(R[size_t(e.a)]), R[size_t(e.b)]));
            const V3 phi = logMap(Q), axis = unit(qrotInv(R[size_t(e.a)], t));
            const double tw = dot3(phi, axis), ptw = dot3(e.plastic.rotp, axis);
            const V3 bend = phi - scale(axis, tw), pb = e.plastic.rotp - scale(axis, ptw);
            const double kb = E * e.I / e.L0, kt = G * e.J / e.L0, my = sy * e.I / e.radius;
            const double ty = (sy / std::sqrt(3.0)) * e.J / e.radius;
            const double hb = cfg.material.bend_hardening * kb, ht = cfg.material.torsion_hardening * kt;
            const Ret3 br = return3(bend, pb, e.plastic.alphaB, kb, my, hb);
            const Ret1 tor = return1(tw, ptw, e.plastic.alphaT, kt, ty, ht);
            tr.next.rotp = br.p + scale(axis, tor.p);
            tr.next.alphaB = br.a; tr.next.alphaT = tor.a;
            tr.moment = br.force + scale(axis, tor.force);
            tr.bendPlastic = br.yielded; tr.torsionPlastic = tor.yielded;
            const double ur = br.energy + br.hard + tor.energy + tor.hard;
            const double dr = my * br.dg + ty * tor.dg;
            o.energy += ur + dr; o.d.elastic += ur; o.d.plastic += dr;
            tr.elastic = uax + us + ur; tr.dissipation = dax + dr;
            const V3 world = qrot(R[size_t(e.a)], jlInvT(phi, tr.moment));
            subFrom(gr[size_t(e.a)], world);
            addTo(gr[size_t(e.b)], world);
            if (trials) o.trial[bi] = tr;
        }
        for (size_t i = 0; i < nodes.size(); i++) {  // gravity, sim.cpp:142
            const double u = nodes[i].mass * cfg.gravity * x[i].y;
            o.energy += u;
            if (!(variant & 1)) gx[i].y += nodes[i].mass * cfg.gravity;
        }
        o.energy += .5 * cfg.centering_stiffness * (sqr(cen.x) + sqr(cen.z));
        if (!(variant & 4))
            for (V3& g : gx) {
                g.x += cfg.centering_stiffness * cen.x / x.size();
                g.z += cfg.centering_stiffness * cen.z / x.size();
            }
        const double jr = jointRadius();
        auto platens = [&]() {  // platens, sim.cpp:168-171
            for (size_t i = 0; i < nodes.size(); i++) {
                const double pb = jr - x[i].y;
                if (pb > 0) {
                    const double m = cfg.contact_stiffness * pb, en = .5 * cfg.contact_stiffness * pb * pb;
                    o.energy += en; o.d.contact += en; o.d.maxPen = std::max(o.d.maxPen, pb); o.d.contacts++;
                    gx[i].y -= m;
                }
                const double pt = x[i].y + jr - top;
                if (pt > 0) {
                    const double m = cfg.contact_stiffness * pt, en = .5 * cfg.contact_stiffness * pt * pt;
                    o.energy += en; o.d.contact += en; o.d.reaction += m;
                    o.d.maxPen = std::max(o.d.maxPen, pt); o.d.contacts++;
                    gx[i].y += m;
                }
            }
        };
        if (variant & 8) platens();
        if (cfg.self_contact) {
            const std::vector<Shape> shapes = shapesOf(x);
            selfContact(shapes, [&](int ai, int bi, const Shape& a, const Shape& b, const Closest& cp,
                                    const V3& delta, double dist, double target) {
                const V3 n = dist > 1e-12 ? divide(delta, dist) : unit(V3{.37 + .001 * ai, .73, -.41 + .001 * bi});
                const double pen = target - dist, mag = cfg.contact_stiffness * pen;
                const double en = .5 * cfg.contact_stiffness * pen * pen;
                o.energy += en; o.d.contact += en; o.d.maxPen = std::max(o.d.maxPen, pen); o.d.contacts++;
                spreadForce(gx, a, cp.s, scale(n, mag));
                spreadForce(gx, b, cp.t, scale(n, -mag));
                if (recordPairs) lastPairs.push_back(keyOf(ai, bi));
            });
            if (recordPairs) std::sort(lastPairs.begin(), lastPairs.end());
        }
        if (!(variant & 8)) platens();
        for (size_t i = 0; i < nodes.size(); i++) {  // pack, lock, guard: sim.cpp:172
            const size_t b = 6 * i;
            o.grad[b] = cfg.translation_scale * gx[i].x;
            o.grad[b + 1] = cfg.translation_scale * gx[i].y;
            o.grad[b + 2] = cfg.translation_scale * gx[i].z;
            o.grad[b + 3] = gr[i].x; o.grad[b + 4] = gr[i].y; o.grad[b + 5] = gr[i].z;
        }
        for (size_t i = 0; i < o.grad.size(); i++)
            if (locked[i]) o.grad[i] = 0;
        if (!std::isfinite(o.energy)) {
            o.energy = kInf;
            std::fill(o.grad.begin(), o.grad.end(), 0);
        }
        return o;
    }

    // The evaluation through the objective hook, in the layouts of include/mcg.h.
    Eval hookedObjective(const std::vector<double>& z, double top, bool trials) const {
        const size_t N = nodes.size(), B = beams.size();
        Eval o;
        o.grad.assign(6 * N, 0);
        std::vector<double> nxt, aux;
        std::vector<uint8_t> fl;
        if (trials) {
            nxt.assign(7 * B, 0);
            aux.assign(7 * B, 0);
            fl.assign(3 * B, 0);
        }
        mcg_diag dg{};
        double e = kInf;
        hookCalls++;
        const int rc = objHook(hookCtx, z.data(), top, trials ? 1 : 0, &e, o.grad.data(), &dg,
                               trials ? nxt.data() : nullptr, trials ? aux.data() : nullptr,
                               trials ? fl.data() : nullptr);
        if (rc != 0) {
            if (!hookStatus) hookStatus = rc;
            o.energy = kInf;
            std::fill(o.grad.begin(), o.grad.end(), 0);
            return o;
        }
        o.energy = e;
        o.d.elastic = dg.elastic; o.d.plastic = dg.plastic; o.d.contact = dg.contact;
        o.d.reaction = dg.reaction; o.d.maxPen = dg.max_pen; o.d.contacts = dg.contacts;
        if (trials) {
            o.trial.resize(B);
            for (size_t b = 0; b < B; b++) {
                Trial& t = o.trial[b];
                const double* q = &nxt[7 * b];
                t.next.epsp = q[0]; t.next.alpha = q[1]; t.next.rotp = {q[2], q[3], q[4]};
                t.next.alphaB = q[5]; t.next.alphaT = q[6];
                const double* w = &aux[7 * b];
                t.strain = w[0]; t.stress = w[1]; t.moment = {w[2], w[3], w[4]};
                t.elastic = w[5]; t.dissipation = w[6];
                t.axialPlastic = fl[3 * b] != 0; t.bendPlastic = fl[3 * b + 1] != 0;
                t.torsionPlastic = fl[3 * b + 2] != 0;
            }
        }
        return o;
    }

    // Hands the current base state and plastic state to the hook's implementation.
    void pushStateToHook() const {
        if (!stateHook) return;
        const size_t N = nodes.size(), B = beams.size();
        std::vector<double> bx(3 * N), br(4 * N), pl(7 * B);
        for (size_t i = 0; i < N; i++) {
            bx[3 * i] = baseX[i].x; bx[3 * i + 1] = baseX[i].y; bx[3 * i + 2] = baseX[i].z;
            br[4 * i] = baseR[i].w; br[4 * i + 1] = baseR[i].x; br[4 * i + 2] = baseR[i].y; br[4 * i + 3] = baseR[i].z;
        }
        for (size_t b = 0; b < B; b++) {
            const Plastic& p = beams[b].plastic;
            double* q = &pl[7 * b];
            q[0] = p.epsp; q[1] = p.alpha; q[2] = p.rotp.x; q[3] = p.rotp.y; q[4] = p.rotp.z;
            q[5] = p.alphaB; q[6] = p.alphaT;
        }
        const int rc = stateHook(hookCtx, bx.data(), br.data(), pl.data());
        if (rc != 0 && !hookStatus) hookStatus = rc;
    }

    // -- solver vector helpers, sim.cpp:42-46 --------------------------------------------
    static double vdot(const std::vector<double>& a, const std::vector<double>& b) {
        double r = 0;
        for (size_t i = 0; i < a.size(); i++) r += a[i] * b[i];
        return r;
    }
    double vrms(const std::vector<double>& a) const {
        double s = 0;
        size_t n = 0;
        for (size_t i = 0; i < a.size(); i++)
            if (!locked[i]) { s += a[i] * a[i]; n++; }
        return n ? std::sqrt(s / n) : 0;
    }
    double vmax(const std::vector<double>& a) const {
        double m = 0;
        for (size_t i = 0; i < a.size(); i++)
            if (!locked[i]) m = std::max(m, std::abs(a[i]));
        return m;
    }
    void limitStep(std::vector<double>& p) const {  // clampDirection
        const double mt = cfg.max_translation_step / cfg.translation_scale;
        for (size_t i = 0; i < p.size() / 6; i++) {
            const size_t b = 6 * i;
            V3 t{p[b], p[b + 1], p[b + 2]};
            const double lt = len(t);
            if (lt > mt) { t = scale(t, mt / lt); p[b] = t.x; p[b + 1] = t.y; p[b + 2] = t.z; }
            V3 r{p[b + 3], p[b + 4], p[b + 5]};
            const double lr = len(r);
            if (lr > cfg.max_rotation_step) {
                r = scale(r, cfg.max_rotation_step / lr);
                p[b + 3] = r.x; p[b + 4] = r.y; p[b + 5] = r.z;
            }
        }
        for (size_t i = 0; i < p.size(); i++)
            if (locked[i]) p[i] = 0;
    }
    void zeroLocked(std::vector<double>& p) const {
        for (size_t i = 0; i < p.size(); ++i)
            if (locked[i]) p[i] = 0;
    }

    // -- Simulator::minimize, sim.cpp:174-211 ---------------------------------------------
    Stats minimize(double top, std::vector<double>& z, Eval& final) const {
        struct Pair { std::vector<double> s, y; double rho = 0; };
        Stats st;
        std::vector<Pair> hist;
        hist.reserve(size_t(cfg.history));
        Eval cur = objective(z, top, false), best = cur;
        std::vector<double> bestZ = z;
        // Extension (no reference counterpart): with relative_gradient_tolerance > 0 an
        // iterate has converged when rms(g) <= tol * rms(g at the start point), in place of
        // the reference's absolute and reaction-relative tests; the penetration bar stays.
        const double rms0 = vrms(cur.grad);
        auto converged = [&](const Eval& o, double rms, double mx) {
            if (cfg.relative_gradient_tolerance > 0)
                return rms <= cfg.relative_gradient_tolerance * rms0 && o.d.maxPen <= cfg.penetration_tolerance;
            const double rel = rms / std::max(1e-6, cfg.translation_scale * std::max(1.0, o.d.reaction));
            // extension: reaction_relative_tolerance (0: the reference's 1.5e-3; < 0: off)
            const double rrt = cfg.reaction_relative_tolerance == 0 ? 1.5e-3 : cfg.reaction_relative_tolerance;
            const bool forceOK = (rms <= cfg.gradient_rms_tolerance && mx <= cfg.gradient_max_tolerance) || rel < rrt;
            return forceOK && o.d.maxPen <= cfg.penetration_tolerance;
        };
        auto lineSearch = [&](const std::vector<double>& p, double dg, std::vector<double>& zc, Eval& cand) {
            double step = 1.0;
            for (int bt = 0; bt < cfg.max_line_search; bt++) {
                for (size_t i = 0; i < z.size(); i++) {
                    zc[i] = z[i] + step * p[i];
                    if (locked[i]) zc[i] = 0;
                }
                cand = objective(zc, top, false);
                st.backtracks++;
                if (std::isfinite(cand.energy) && cand.energy <= cur.energy + cfg.armijo * step * dg) return true;
                step *= .5;
                if (step < cfg.min_line_step) break;
            }
            return false;
        };
        auto steepest = [&](std::vector<double>& p) {
            p = cur.grad;
            for (double& v : p) v = -v;
            zeroLocked(p);
            limitStep(p);
        };
        for (int it = 0; it < cfg.max_iterations; it++) {
            st.iterations = it + 1;
            st.rms = vrms(cur.grad); st.max = vmax(cur.grad); st.energy = cur.energy;
            if (converged(cur, st.rms, st.max)) { st.converged = true; break; }
            // two-loop recursion (sim.cpp:184-188)
            std::vector<double> p = cur.grad, alpha(hist.size());
            for (int h = int(hist.size()) - 1; h >= 0; h--) {
                alpha[size_t(h)] = hist[size_t(h)].rho * vdot(hist[size_t(h)].s, p);
                for (size_t i = 0; i < p.size(); i++) p[i] -= alpha[size_t(h)] * hist[size_t(h)].y[i];
            }
            double H0 = .10;
            if (!hist.empty()) {
                const Pair& h = hist.back();
                const double sy = vdot(h.s, h.y), yy = vdot(h.y, h.y);
                if (sy > 1e-20 && yy > 1e-20) H0 = clampd(sy / yy, 1e-7, 1e4);
            }
            for (double& v : p) v *= H0;
            for (size_t h = 0; h < hist.size(); h++) {
                const double beta = hist[h].rho * vdot(hist[h].y, p);
                for (size_t i = 0; i < p.size(); i++) p[i] += hist[h].s[i] * (alpha[h] - beta);
            }
            for (double& v : p) v = -v;
            zeroLocked(p);
            limitStep(p);
            double dg = vdot(cur.grad, p);
            if (!(dg < 0)) {  // not a descent direction (sim.cpp:191)
                hist.clear();
                steepest(p);
                dg = vdot(cur.grad, p);
            }
            std::vector<double> zc(z.size());
            Eval cand;
            bool ok = lineSearch(p, dg, zc, cand);
            if (!ok) {  // steepest-descent retry (sim.cpp:193-203)
                hist.clear();
                steepest(p);
                dg = vdot(cur.grad, p);
                ok = lineSearch(p, dg, zc, cand);
            }
            if (!ok) break;
            std::vector<double> sv(z.size()), yv(z.size());
            for (size_t i = 0; i < z.size(); i++) { sv[i] = zc[i] - z[i]; yv[i] = cand.grad[i] - cur.grad[i]; }
            const double sy = vdot(sv, yv), ss = vdot(sv, sv), yy = vdot(yv, yv);
            if (sy > 1e-12 * std::sqrt(std::max(1e-30, ss * yy))) {  // curvature guard (sim.cpp:206)
                if (int(hist.size()) == cfg.history) hist.erase(hist.begin());
                hist.push_back({std::move(sv), std::move(yv), 1 / sy});
            } else {
                hist.clear();
            }
            z = std::move(zc);
            cur = std::move(cand);
            if (cur.energy < best.energy) { best = cur; bestZ = z; }
        }
        if (!st.converged && best.energy < cur.energy) { z = bestZ; cur = best; }
        final = objective(z, top, true);
        st.rms = vrms(final.grad); st.max = vmax(final.grad); st.energy = final.energy;
        st.converged = converged(final, st.rms, st.max);
        return st;
    }

    // -- Simulator::commit and topY, sim.cpp:212-213 --------------------------------------
    void commit(const std::vector<double>& z, const Eval& o) {
        std::vector<V3> x;
        std::vector<Q4> R;
        state(z, x, R);
        if (o.trial.size() != beams.size()) throw std::runtime_error("missing constitutive trial states");
        for (size_t i = 0; i < nodes.size(); i++) { nodes[i].x = x[i]; nodes[i].R = R[i]; baseX[i] = x[i]; baseR[i] = R[i]; }
        for (size_t i = 0; i < beams.size(); i++) beams[i].plastic = o.trial[i].next;
        pushStateToHook();
    }
    double topY(double s, bool loading) const {
        const double compressed = top0 - cfg.max_strain * height;
        return loading ? mix1(top0, compressed, sat(s)) : mix1(compressed, top0, sat(s));
    }

    // -- Simulator::diagnostics, sim.cpp:312-372 ------------------------------------------
    mcg_frame diagnostics(double time, double top, bool loading, const Eval& o, const Stats& s) const {
        mcg_frame d;
        std::memset(&d, 0, sizeof(d));
        d.time = time; d.platen_y = top; d.displacement = top0 - top;
        d.engineering_strain = d.displacement / std::max(1e-12, height);
        d.reaction_force = std::max(0.0, o.d.reaction - reactionOffset);
        d.engineering_stress = d.reaction_force / std::max(1e-12, area);
        d.loading_work = loadingWork; d.recovered_work = recoveredWork;
        d.dissipated_work = std::max(0.0, loadingWork - recoveredWork);
        d.specific_energy_absorption = d.dissipated_work / std::max(1e-12, mass);
        d.elastic_energy = o.d.elastic; d.plastic_dissipation = o.d.plastic; d.contact_energy = o.d.contact;
        d.residual_rms = s.rms; d.residual_max = s.max; d.max_penetration = o.d.maxPen;
        d.active_contacts = o.d.contacts; d.iterations = s.iterations;
        d.converged = s.converged; d.loading = loading;
        double sumAxial = 0, maxAxial = 0, sumRot = 0, maxRot = 0;
        int plasticBeams = 0, plasticHinges = 0;
        for (const BeamRec& e : beams) {
            const double pa = std::abs(e.plastic.epsp), pr = len(e.plastic.rotp);
            sumAxial += pa; maxAxial = std::max(maxAxial, pa);
            sumRot += pr; maxRot = std::max(maxRot, pr);
            if (pa > 1e-5) ++plasticBeams;
            if (pr > 1e-4) ++plasticHinges;
        }
        if (!beams.empty()) {
            d.mean_plastic_strain = sumAxial / beams.size(); d.max_plastic_strain = maxAxial;
            d.mean_plastic_rotation = sumRot / beams.size(); d.max_plastic_rotation = maxRot;
        }
        d.plastic_beams = plasticBeams; d.plastic_hinges = plasticHinges;
        double ymin = kInf, ymax = -kInf;
        for (const NodeRec& n : nodes) { ymin = std::min(ymin, n.x.y); ymax = std::max(ymax, n.x.y); }
        const double currentHeight = std::max(0.0, ymax - ymin);
        d.permanent_set = std::max(0.0, 1.0 - currentHeight / std::max(1e-12, height));
        return d;
    }

    // -- Simulator::run, sim.cpp:374-467 (snapshot capture omitted: visualisation only) -----
    int run(std::vector<mcg_frame>& frames, bool verbose) {
        loadingWork = recoveredWork = prevDisp = prevForce = reactionOffset = 0;
        double time = 0, currentTop = top0;
        bool first = true;
        int accepted = 0;
        std::function<void(double, bool, int)> advanceTo = [&](double targetTop, bool loading, int refinement) {
            std::vector<double> z(nodes.size() * 6, 0);
            Eval fin;
            const Stats stats = minimize(targetTop, z, fin);
            const bool acceptable = stats.converged && fin.d.maxPen <= cfg.penetration_tolerance && std::isfinite(fin.energy);
            if (!acceptable && refinement < cfg.max_adaptive_refinements && std::abs(targetTop - currentTop) > 2.5e-5) {
                const double midpoint = 0.5 * (currentTop + targetTop);
                advanceTo(midpoint, loading, refinement + 1);
                advanceTo(targetTop, loading, refinement + 1);
                return;
            }
            if (!acceptable) throw std::runtime_error("quasi-static equilibrium failed");
            commit(z, fin);
            if (first) reactionOffset = fin.d.reaction;
            const double force = std::max(0.0, fin.d.reaction - reactionOffset);
            const double displacement = top0 - targetTop;
            if (!first) {
                const double dd = displacement - prevDisp;
                const double work = 0.5 * (prevForce + force) * dd;
                if (dd >= 0.0) loadingWork += std::max(0.0, work);
                else recoveredWork += std::max(0.0, -work);
            }
            prevDisp = displacement; prevForce = force; currentTop = targetTop;
            mcg_frame d = diagnostics(time, targetTop, loading, fin, stats);
            d.refinement = refinement;
            frames.push_back(d);
            if (verbose)
                std::printf("[equilibrium] %3d %s strain=%.4f force=%.3f N residual=%.2e pen=%.3f mm iter=%d %s\n",
                            accepted, loading ? "load  " : "unload", d.engineering_strain, d.reaction_force,
                            d.residual_rms, d.max_penetration * 1000.0, d.iterations, refinement ? "[REFINED]" : "[OK]");
            accepted++;
            first = false;
            time += cfg.step_time;
        };
        try {
            advanceTo(top0, true, 0);
            for (int step = 1; step <= cfg.load_steps; ++step)
                advanceTo(topY(double(step) / std::max(1, cfg.load_steps), true), true, 0);
            for (int step = 1; step <= cfg.unload_steps; ++step)
                advanceTo(topY(double(step) / std::max(1, cfg.unload_steps), false), false, 0);
        } catch (const std::runtime_error&) {
            return MCG_ERR_EQUILIBRIUM;
        }
        return 0;
    }

    // -- verification (sim.cpp:468-577) --------------------------------------------------
    double beamPotential(const std::vector<V3>& x, const std::vector<Q4>& R) const {
        const double E = cfg.material.young, G = E / (2.0 * (1.0 + cfg.material.nu));
        const double sy = cfg.material.yield, H = cfg.material.hardening;
        double total = 0.0;
        for (const BeamRec& e : beams) {
            const V3 d = x[size_t(e.b)] - x[size_t(e.a)];
            const double L = std::max(1e-12, len(d));
            const V3 t = divide(d, L);
            const double eps = (L - e.L0) / e.L0;
            const Ret1 ax = return1(eps, e.plastic.epsp, e.plastic.alpha, E, sy, H);
            total += e.area * e.L0 * (ax.energy + ax.hard);
            const V3 da = qrot(R[size_t(e.a)], e.e0), db = qrot(R[size_t(e.b)], e.e0);
            const double cs = 0.5 * cfg.shear_correction * G * e.area * e.L0;
            total += 0.5 * cs * (len2(da - t) + len2(db - t));
            const Q4 Q = qnorm(qmul(conj(R[size_t(e.a)]), R[size_t(e.b)]));
            const V3 phi = logMap(Q), axis = unit(qrotInv(R[size_t(e.a)], t));
            const double tw = dot3(phi, axis), ptw = dot3(e.plastic.rotp, axis);
            const V3 bend = phi - scale(axis, tw), pb = e.plastic.rotp - scale(axis, ptw);
            const double kb = E * e.I / e.L0, kt = G * e.J / e.L0, my = sy * e.I / e.radius;
            const double ty = (sy / std::sqrt(3.0)) * e.J / e.radius;
            const Ret3 br = return3(bend, pb, e.plastic.alphaB, kb, my, cfg.material.bend_hardening * kb);
            const Ret1 tor = return1(tw, ptw, e.plastic.alphaT, kt, ty, cfg.material.torsion_hardening * kt);
            total += br.energy + br.hard + tor.energy + tor.hard;
        }
        return total;
    }
    double rigidRotationError() const {
        std::vector<V3> x(nodes.size());
        std::vector<Q4> R(nodes.size());
        for (size_t i = 0; i < nodes.size(); ++i) {
            const NodeRec& n = nodes[i];
            const double yf = sat((n.x0.y - cfg.joint_scale * cfg.max_radius) / std::max(1e-12, height));
            x[i] = n.x0;
            x[i].y -= 0.018 * height * yf;
            x[i].x += 0.00018 * std::sin(2.0 * kPi * yf + 0.17 * i);
            R[i] = fromAxisAngle({0, 0, 1}, 0.035 * yf);
        }
        const double e0 = beamPotential(x, R);
        const Q4 Q = fromAxisAngle(unit(V3{0.37, 0.81, -0.44}), 1.137);
        const V3 shift{0.081, -0.024, 0.053};
        std::vector<V3> xr(x.size());
        std::vector<Q4> Rr(R.size());
        for (size_t i = 0; i < x.size(); ++i) { xr[i] = qrot(Q, x[i]) + shift; Rr[i] = qnorm(qmul(Q, R[i])); }
        const double e1 = beamPotential(xr, Rr);
        return std::abs(e1 - e0) / std::max({1e-12, std::abs(e0), std::abs(e1)});
    }
    double gradientCheckError() const {
        std::vector<double> z(nodes.size() * 6, 0);
        Rng rng(cfg.seed ^ 0x475241444348454bULL);
        for (size_t i = 0; i < nodes.size(); ++i) {
            const size_t b = 6 * i;
            z[b + 0] = 0.003 * rng.signedUniform();
            z[b + 1] = 0.100 + 0.003 * rng.signedUniform();
            z[b + 2] = 0.003 * rng.signedUniform();
            z[b + 3] = 0.004 * rng.signedUniform();
            z[b + 4] = 0.004 * rng.signedUniform();
            z[b + 5] = 0.004 * rng.signedUniform();
            for (int d = 0; d < 6; ++d)
                if (locked[b + size_t(d)]) z[b + size_t(d)] = 0.0;
        }
        const double top = top0 + 0.020;
        const Eval a = objective(z, top, false);
        double num = 0.0, den = 0.0;
        int checked = 0;
        for (size_t k = 0; k < z.size() && checked < 42; ++k) {
            if (locked[k]) continue;
            if ((mix64(k * 0x9e3779b97f4a7c15ULL + cfg.seed) & 15ULL) > 1ULL) continue;
            const double h = (k % 6 < 3) ? 2e-6 : 1e-6;
            std::vector<double> zp = z, zm = z;
            zp[k] += h; zm[k] -= h;
            const double fp = objective(zp, top, false).energy, fm = objective(zm, top, false).energy;
            const double numeric = (fp - fm) / (2.0 * h), analytic = a.grad[k];
            num += sqr(numeric - analytic);
            den += sqr(numeric) + sqr(analytic);
            ++checked;
        }
        return std::sqrt(num / std::max(1e-30, den));
    }
};

namespace {
std::vector<double> vecOf(const double* p, size_t n) { return std::vector<double>(p, p + n); }
void putDiag(const Diag& d, mcg_diag* out) {
    if (!out) return;
    out->elastic = d.elastic; out->plastic = d.plastic; out->contact = d.contact;
    out->reaction = d.reaction; out->max_pen = d.maxPen; out->contacts = d.contacts; out->pad_ = 0;
}
}  // namespace

extern "C" {

int orc_is_reference(void) { return 0; }

orc_model* orc_create_builder(const mcg_config* cfg) {
    auto m = new orc_model;
    m->cfg = *cfg;
    m->cfg.translation_scale = m->cfg.cell_size;  // sim.cpp:49
    try {
        m->build();
        m->distributeMass();
    } catch (...) {
        delete m;
        return nullptr;
    }
    m->resetBase();
    return m;
}

orc_model* orc_create_injected(const mcg_config* cfg, const mcg_topology* t, const mcg_geometry* g,
                               const double* x0, const double* r0, const int32_t* layer) {
    auto m = new orc_model;
    m->cfg = *cfg;
    const size_t N = size_t(t->n_nodes), B = size_t(t->n_beams);
    m->nodes.assign(N, NodeRec{});
    for (size_t i = 0; i < N; i++) {
        NodeRec& n = m->nodes[i];
        n.x0 = {x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]};
        n.x = n.x0;
        if (r0) n.R = {r0[4 * i], r0[4 * i + 1], r0[4 * i + 2], r0[4 * i + 3]};
        n.mass = t->mass[i];
        n.layer = layer ? layer[i] : 0;
    }
    m->beams.assign(B, BeamRec{});
    for (size_t b = 0; b < B; b++) {
        BeamRec& e = m->beams[b];
        e.a = t->beam_a[b]; e.b = t->beam_b[b]; e.L0 = t->L0[b]; e.radius = t->radius[b];
        e.area = t->area[b]; e.I = t->I[b]; e.J = t->J[b];
        e.e0 = {t->e0[3 * b], t->e0[3 * b + 1], t->e0[3 * b + 2]};
    }
    for (int64_t k = 0; k < t->n_connected; k++) m->connected.insert(t->connected[k]);
    m->locked.assign(t->locked, t->locked + 6 * N);
    m->width = g->width; m->height = g->height; m->depth = g->depth;
    m->area = g->area; m->mass = g->mass; m->top0 = g->top0;
    m->resetBase();
    return m;
}

void orc_free(orc_model* m) { delete m; }

void orc_counts(const orc_model* m, int32_t* n, int32_t* b, int64_t* nc) {
    if (n) *n = int32_t(m->nodes.size());
    if (b) *b = int32_t(m->beams.size());
    if (nc) *nc = int64_t(m->connected.size());
}

void orc_export(const orc_model* m, double* x0, double* r0, int32_t* layer, double* mass, uint8_t* locked,
                int32_t* beam_a, int32_t* beam_b, double* L0, double* radius, double* area, double* I,
                double* J, double* e0, uint64_t* connected, mcg_geometry* geom, double* ts) {
    for (size_t i = 0; i < m->nodes.size(); i++) {
        const NodeRec& n = m->nodes[i];
        if (x0) { x0[3 * i] = n.x0.x; x0[3 * i + 1] = n.x0.y; x0[3 * i + 2] = n.x0.z; }
        if (r0) { r0[4 * i] = n.R.w; r0[4 * i + 1] = n.R.x; r0[4 * i + 2] = n.R.y; r0[4 * i + 3] = n.R.z; }
        if (layer) layer[i] = n.layer;
        if (mass) mass[i] = n.mass;
    }
    if (locked) std::copy(m->locked.begin(), m->locked.end(), locked);
    for (size_t b = 0; b < m->beams.size(); b++) {
        const BeamRec& e = m->beams[b];
        if (beam_a) beam_a[b] = e.a;
        if (beam_b) beam_b[b] = e.b;
        if (L0) L0[b] = e.L0;
        if (radius) radius[b] = e.radius;
        if (area) area[b] = e.area;
        if (I) I[b] = e.I;
        if (J) J[b] = e.J;
        if (e0) { e0[3 * b] = e.e0.x; e0[3 * b + 1] = e.e0.y; e0[3 * b + 2] = e.e0.z; }
    }
    if (connected) {
        std::vector<uint64_t> keys(m->connected.begin(), m->connected.end());
        std::sort(keys.begin(), keys.end());
        std::copy(keys.begin(), keys.end(), connected);
    }
    if (geom) {
        geom->width = m->width; geom->height = m->height; geom->depth = m->depth;
        geom->area = m->area; geom->mass = m->mass; geom->top0 = m->top0;
    }
    if (ts) *ts = m->cfg.translation_scale;
}

void orc_set_state(orc_model* m, const double* bx, const double* br, const double* pl) {
    for (size_t i = 0; i < m->nodes.size(); i++) {
        if (bx) { m->baseX[i] = {bx[3 * i], bx[3 * i + 1], bx[3 * i + 2]}; m->nodes[i].x = m->baseX[i]; }
        if (br) { m->baseR[i] = {br[4 * i], br[4 * i + 1], br[4 * i + 2], br[4 * i + 3]}; m->nodes[i].R = m->baseR[i]; }
    }
    if (pl)
        for (size_t b = 0; b < m->beams.size(); b++) {
            Plastic& p = m->beams[b].plastic;
            const double* q = pl + 7 * b;
            p.epsp = q[0]; p.alpha = q[1]; p.rotp = {q[2], q[3], q[4]}; p.alphaB = q[5]; p.alphaT = q[6];
        }
    if (bx || br || pl) m->pushStateToHook();
}

void orc_set_objective_hook(orc_model* m, orc_objective_fn objective, orc_state_fn state, void* ctx) {
    m->objHook = objective;
    m->stateHook = objective ? state : nullptr;
    m->hookCtx = objective ? ctx : nullptr;
    m->hookStatus = 0;
    m->hookCalls = 0;
    m->pushStateToHook();
}

int orc_hook_status(const orc_model* m, int64_t* calls) {
    if (calls) *calls = m->hookCalls;
    return m->hookStatus;
}

void orc_record_pairs(orc_model* m, int on) {
    m->recordPairs = on != 0;
    m->lastPairs.clear();
}

int64_t orc_last_pairs(const orc_model* m, uint64_t* keys, int64_t cap) {
    for (int64_t k = 0; k < int64_t(m->lastPairs.size()) && k < cap; k++) keys[k] = m->lastPairs[size_t(k)];
    return int64_t(m->lastPairs.size());
}

orc_model* orc_create_specimen(const mcg_config* cfg, const mcg_lattice_spec* spec) {
    orcspec::Specimen s;
    if (!cfg || !spec || !orcspec::build(*spec, *cfg, s)) return nullptr;
    mcg_topology t{};
    t.n_nodes = int32_t(s.mass.size());
    t.n_beams = int32_t(s.L0.size());
    t.beam_a = s.beam_a.data(); t.beam_b = s.beam_b.data(); t.L0 = s.L0.data(); t.radius = s.radius.data();
    t.area = s.area.data(); t.I = s.I.data(); t.J = s.J.data(); t.e0 = s.e0.data(); t.mass = s.mass.data();
    t.locked = s.locked.data(); t.n_connected = int64_t(s.connected.size()); t.connected = s.connected.data();
    return orc_create_injected(cfg, &t, &s.geometry, s.x0.data(), s.r0.data(), s.layer.data());
}

void orc_random_state(int32_t n_nodes, int32_t n_beams, const uint8_t* locked, double sigma_t, double sigma_r,
                      double epsp_max, uint64_t seed, double* z, double* plastic) {
    orcspec::random_state(n_nodes, n_beams, locked, sigma_t, sigma_r, epsp_max, seed, z, plastic);
}

void orc_get_state(const orc_model* m, double* bx, double* br, double* pl) {
    for (size_t i = 0; i < m->nodes.size(); i++) {
        if (bx) { bx[3 * i] = m->baseX[i].x; bx[3 * i + 1] = m->baseX[i].y; bx[3 * i + 2] = m->baseX[i].z; }
        if (br) { br[4 * i] = m->baseR[i].w; br[4 * i + 1] = m->baseR[i].x; br[4 * i + 2] = m->baseR[i].y; br[4 * i + 3] = m->baseR[i].z; }
    }
    if (pl)
        for (size_t b = 0; b < m->beams.size(); b++) {
            const Plastic& p = m->beams[b].plastic;
            double* q = pl + 7 * b;
            q[0] = p.epsp; q[1] = p.alpha; q[2] = p.rotp.x; q[3] = p.rotp.y; q[4] = p.rotp.z;
            q[5] = p.alphaB; q[6] = p.alphaT;
        }
}

double orc_objective(const orc_model* m, const double* z, double top, int trials, double* grad,
                     mcg_diag* diag, double* next, double* aux, uint8_t* flags) {
    const Eval o = m->objective(vecOf(z, 6 * m->nodes.size()), top, trials != 0);
    if (grad) std::copy(o.grad.begin(), o.grad.end(), grad);
    putDiag(o.d, diag);
    if (trials)
        for (size_t b = 0; b < o.trial.size(); b++) {
            const Trial& t = o.trial[b];
            if (next) {
                double* q = next + 7 * b;
                q[0] = t.next.epsp; q[1] = t.next.alpha; q[2] = t.next.rotp.x; q[3] = t.next.rotp.y;
                q[4] = t.next.rotp.z; q[5] = t.next.alphaB; q[6] = t.next.alphaT;
            }
            if (aux) {
                double* q = aux + 7 * b;
                q[0] = t.strain; q[1] = t.stress; q[2] = t.moment.x; q[3] = t.moment.y; q[4] = t.moment.z;
                q[5] = t.elastic; q[6] = t.dissipation;
            }
            if (flags) { flags[3 * b] = t.axialPlastic; flags[3 * b + 1] = t.bendPlastic; flags[3 * b + 2] = t.torsionPlastic; }
        }
    return o.energy;
}

int64_t orc_contact_pairs(const orc_model* m, const double* z, uint64_t* keys, int64_t cap) {
    std::vector<V3> x;
    std::vector<Q4> R;
    m->state(vecOf(z, 6 * m->nodes.size()), x, R);
    std::vector<uint64_t> out;
    m->selfContact(m->shapesOf(x), [&](int ai, int bi, const Shape&, const Shape&, const Closest&, const V3&,
                                       double, double) { out.push_back(keyOf(ai, bi)); });
    std::sort(out.begin(), out.end());
    for (int64_t k = 0; k < int64_t(out.size()) && k < cap; k++) keys[k] = out[size_t(k)];
    return int64_t(out.size());
}

int orc_minimize(orc_model* m, double top, double* z, mcg_optstats* stats, double* fe, mcg_diag* fd) {
    std::vector<double> zz = vecOf(z, 6 * m->nodes.size());
    Eval fin;
    const Stats st = m->minimize(top, zz, fin);
    std::copy(zz.begin(), zz.end(), z);
    if (stats) {
        stats->iterations = st.iterations; stats->backtracks = st.backtracks; stats->rms = st.rms;
        stats->max = st.max; stats->energy = st.energy; stats->converged = st.converged; stats->pad_ = 0;
    }
    if (fe) *fe = fin.energy;
    putDiag(fin.d, fd);
    m->lastZ = zz;
    m->lastFinal = std::move(fin);
    m->haveFinal = true;
    return 0;
}

int orc_commit(orc_model* m) {
    if (!m->haveFinal) return MCG_ERR_STATE;
    m->commit(m->lastZ, m->lastFinal);
    m->haveFinal = false;
    return 0;
}

int orc_run(orc_model* m, mcg_frame* frames, int32_t cap, int32_t* count, int verbose) {
    std::vector<mcg_frame> out;
    const int rc = m->run(out, verbose != 0);
    for (size_t f = 0; f < out.size() && int32_t(f) < cap; f++) frames[f] = out[f];
    *count = int32_t(out.size());
    return rc;
}

double orc_rigid_rotation_error(const orc_model* m) { return m->rigidRotationError(); }
double orc_gradient_check_error(const orc_model* m) { return m->gradientCheckError(); }

double orc_beam_potential(const orc_model* m, const double* x, const double* r) {
    std::vector<V3> xv(m->nodes.size());
    std::vector<Q4> rv(m->nodes.size());
    for (size_t i = 0; i < xv.size(); i++) {
        xv[i] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
        rv[i] = {r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]};
    }
    return m->beamPotential(xv, rv);
}

double orc_top_y(const orc_model* m, double s, int loading) { return m->topY(s, loading != 0); }

int orc_set_variant(orc_model* m, int variant) {
    m->variant = variant;
    return 0;
}

}  // extern "C"
