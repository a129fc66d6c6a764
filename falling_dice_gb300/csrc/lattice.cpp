// lattice.cpp -- beam lattices and seeded deformed states.
//
// Two families.  The reference's own specimen (MCG_LATTICE_REFERENCE_BCC): the graded BCC
// lattice with face grids, imperfections and 2-5 elements per strut that Simulator::build
// makes (MC/src/sim.cpp:51-132), reproduced bit for bit from the same configuration.  And the
// cubic and cubic+BCC specimens the throughput workloads are defined on, with one element
// per strut, which apply the reference's own rules for what they share with it:
// node numbering of the corner grid (sim.cpp:54), section properties (sim.cpp:115),
// element-endpoint exclusion pairs (sim.cpp:115-117), lumped mass and the two anti-drift
// locks (sim.cpp:134), platen height (sim.cpp:131) and the splitmix64 generator
// (MC/include/core.hpp:46).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <new>
#include <unordered_set>
#include <vector>

#include "../../include/mcg.h"

namespace {

constexpr double kPi = 3.1415926535897932384626433832795;

uint64_t mix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

struct Rng {
    uint64_t state;
    explicit Rng(uint64_t seed) : state(mix64(seed)) {}
    uint32_t next32() { state = mix64(state); return uint32_t(state >> 32); }
    double uniform() { return (double(next32()) + .5) / 4294967296.0; }
    double signedUniform() { return 2 * uniform() - 1; }
    double normal() {  // Box-Muller on two uniforms
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

uint64_t pair_key(int a, int b) {
    if (a > b) std::swap(a, b);
    return (uint64_t(uint32_t(a)) << 32) | uint32_t(b);
}

// 3-vectors with the reference's rounding (MC/include/core.hpp:37-39, 47): a vector divided
// by s is multiplied by 1 / s; a unit vector of a (near-)zero or non-finite vector is +y.
struct V {
    double x, y, z;
};
V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V operator*(double s, V a) { return {s * a.x, s * a.y, s * a.z}; }
double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V cross(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V unit(V v) {
    const double l2 = dot(v, v);
    return std::isfinite(l2) && l2 > 1e-30 ? (1.0 / std::sqrt(l2)) * v : V{0, 1, 0};
}
V perpendicular(V n) { return unit(cross(std::abs(n.z) < .8 ? V{0, 0, 1} : V{0, 1, 0}, n)); }
double sat(double v) { return std::max(0.0, std::min(1.0, v)); }

}  // namespace

struct mcg_lattice {
    std::vector<double> x0, r0, mass, L0, radius, area, I, J, e0;
    std::vector<int32_t> layer, beam_a, beam_b;
    std::vector<uint8_t> locked;
    std::vector<uint64_t> connected;
    mcg_geometry geometry{};
};

namespace {

// Lumped mass (half of each element to either end, plus a joint mass per node), the specimen
// mass and the two anti-drift locks on the bottom layer (Simulator::distributeMass,
// MC/src/sim.cpp:134); the geometry and platen height (sim.cpp:56, 131).
bool finish(mcg_lattice* L, const mcg_config& cfg, double width, double height, double depth) {
    const size_t N = L->layer.size(), B = L->L0.size();
    const double jr = cfg.joint_scale * cfg.max_radius;
    double total = 0;
    L->mass.assign(N, 0.0);
    for (size_t b = 0; b < B; b++) {
        const double m = cfg.material.density * L->area[b] * L->L0[b];
        L->mass[size_t(L->beam_a[b])] += .5 * m;
        L->mass[size_t(L->beam_b[b])] += .5 * m;
        total += m;
    }
    const double jm = cfg.material.density * (4.0 / 3.0) * kPi * std::pow(jr, 3) * .28;
    for (size_t n = 0; n < N; n++) { L->mass[n] += jm; total += jm; }
    L->locked.assign(6 * N, 0);
    int la = -1, lb = -1;
    double da = std::numeric_limits<double>::infinity(), db = da;
    for (size_t n = 0; n < N; n++)
        if (L->layer[n] == 0) {
            const double px = L->x0[3 * n], pz = L->x0[3 * n + 2];
            const double qa = (px + .5 * width) * (px + .5 * width) + (pz + .5 * depth) * (pz + .5 * depth);
            const double qb = (px - .5 * width) * (px - .5 * width) + (pz + .5 * depth) * (pz + .5 * depth);
            if (qa < da) { da = qa; la = int(n); }
            if (qb < db) { db = qb; lb = int(n); }
        }
    if (la < 0 || lb < 0) return false;
    L->locked[size_t(6 * la)] = 1; L->locked[size_t(6 * la + 2)] = 1; L->locked[size_t(6 * lb + 2)] = 1;
    L->geometry.width = width; L->geometry.height = height; L->geometry.depth = depth;
    L->geometry.area = width * depth; L->geometry.mass = total; L->geometry.top0 = jr + height + jr;
    return true;
}

// The reference's specimen (Simulator::build, MC/src/sim.cpp:51-132) from cfg: corner and
// BCC-centre nodes with seeded imperfections and the alternating accordion offsets of the
// centres, struts from every centre to its cell's eight corners and face grids at the bottom
// and top layers, each strut split into elements_per_strut (clamped to 2..5) elements along a
// seeded bow, radii graded with height and distance from the axis (with the trigger layers
// slenderer), excluded node pairs for every element and every strut's end pair.  Every
// expression keeps the reference's operation order, so the arrays are the reference's bit
// for bit on the same compiler flags (no FMA contraction).
bool build_reference(const mcg_config& cfg, mcg_lattice* L) {
    const int nx = cfg.cells_x, ny = cfg.cells_y, nz = cfg.cells_z;
    const long long corners = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    const double cs = cfg.cell_size;
    const double width = nx * cs, height = ny * cs, depth = nz * cs;
    const double jr = cfg.joint_scale * cfg.max_radius;
    const V origin{-.5 * width, jr, -.5 * depth};
    auto corner = [&](int i, int j, int k) { return int((j * (nz + 1) + k) * (nx + 1) + i); };
    auto centre = [&](int i, int j, int k) { return int(corners + (j * nz + k) * nx + i); };
    std::vector<V> x;
    Rng rng(cfg.seed);
    for (int j = 0; j <= ny; j++)
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                V p = origin + V{i * cs, j * cs, k * cs};
                const double yf = double(j) / ny, env = std::sin(kPi * yf), sg = ((i + 2 * k + 3 * j) & 1) ? 1.0 : -1.0;
                p.x += cfg.imperfection * env * (.55 * sg + .45 * rng.signedUniform());
                p.z += cfg.imperfection * env * (.35 * sg + .65 * rng.signedUniform());
                x.push_back(p);
                L->layer.push_back(j);
            }
    for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz; k++)
            for (int i = 0; i < nx; i++) {
                V p = origin + V{(i + .5) * cs, (j + .5) * cs, (k + .5) * cs};
                const double yf = (j + .5) / double(ny), env = std::sin(kPi * yf), sg = ((i + k + j) & 1) ? 1.0 : -1.0;
                const double sx = (j & 1) ? -1.0 : 1.0, sz = ((j / 2) & 1) ? -1.0 : 1.0;
                p.x += cs * (.082 * (1 - .32 * yf) * sx + .018 * env * sg) + 1.2 * cfg.imperfection * env * rng.signedUniform();
                p.z += cs * (.032 * (.65 + .35 * (1 - yf)) * sz - .012 * env * sg) +
                       1.2 * cfg.imperfection * env * rng.signedUniform();
                x.push_back(p);
                L->layer.push_back(j);
            }
    std::unordered_set<uint64_t> struts;  // end pairs of the struts made so far
    std::vector<uint64_t> excluded;
    auto strut_radius = [&](int a, int b, int layer, double scale) {
        const V m = .5 * (x[size_t(a)] + x[size_t(b)]);
        const double y = sat((m.y - jr) / height);
        const double radial = sat(std::sqrt(m.x * m.x + m.z * m.z) / (.72 * std::max(width, depth)));
        double grade = .58 + .42 * std::pow(1 - y, .72);
        grade *= .94 + .12 * radial;
        if (layer == 0) grade *= cfg.trigger_scale;
        else if (layer == 1) grade *= std::sqrt(cfg.trigger_scale);
        else if (layer == 2) grade *= .88;
        const double g = sat(grade);
        return scale * (cfg.min_radius * (1.0 - g) + cfg.max_radius * g);
    };
    auto strut = [&](int a, int b, int layer, int family, double scale) {
        const uint64_t key = pair_key(a, b);
        if (a == b || !struts.insert(key).second) return;
        const V pa = x[size_t(a)], pb = x[size_t(b)];
        const V tangent = unit(pb - pa);
        const uint64_t h = mix64(cfg.seed ^ key ^ uint64_t(family + 31) * 0x9e3779b97f4a7c15ULL);
        const V helper{double(int((h >> 0) & 1023) - 511), double(int((h >> 10) & 1023) - 511),
                       double(int((h >> 20) & 1023) - 511)};
        V axis = cross(tangent, helper);
        axis = dot(axis, axis) < 1e-12 ? perpendicular(tangent) : unit(axis);
        const V axis2 = unit(cross(tangent, axis));
        const double layer_factor = layer == 0 ? 2.60 : (layer == 1 ? 1.60 : 1.0);
        const double amplitude = cfg.member_imperfection * layer_factor * (.55 + .90 * double((h >> 32) & 65535) / 65535.0);
        const int segments = std::clamp(cfg.elements_per_strut, 2, 5);
        std::vector<int> chain{a};
        for (int sgm = 1; sgm < segments; sgm++) {
            const double t = double(sgm) / segments;
            x.push_back((1 - t) * pa + t * pb + std::sin(kPi * t) * amplitude * axis +
                        .22 * std::sin(2 * kPi * t) * amplitude * axis2);
            L->layer.push_back(layer);
            chain.push_back(int(x.size()) - 1);
        }
        chain.push_back(b);
        const double r = strut_radius(a, b, layer, scale);
        for (size_t q = 0; q + 1 < chain.size(); q++) {
            const int u = chain[q], v = chain[q + 1];
            const V ed = x[size_t(v)] - x[size_t(u)];
            const V e0 = unit(ed);
            L->beam_a.push_back(u);
            L->beam_b.push_back(v);
            L->L0.push_back(std::sqrt(dot(ed, ed)));
            L->e0.insert(L->e0.end(), {e0.x, e0.y, e0.z});
            L->radius.push_back(r);
            L->area.push_back(kPi * r * r);
            L->I.push_back(.25 * kPi * std::pow(r, 4));
            L->J.push_back(2 * L->I.back());
            excluded.push_back(pair_key(u, v));
        }
        excluded.push_back(key);  // no self-contact across one physical strut
    };
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    for (int j = 0; j < ny; j++)
        for (int k = 0; k < nz; k++)
            for (int i = 0; i < nx; i++)
                for (int q = 0; q < 8; q++) strut(centre(i, j, k), corner(i + off[q][0], j + off[q][1], k + off[q][2]), j, q, 1.0);
    for (int face : {0, ny}) {
        const int layer = std::clamp(face, 0, ny - 1);
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i < nx; i++) strut(corner(i, face, k), corner(i + 1, face, k), layer, 30, .62);
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k < nz; k++) strut(corner(i, face, k), corner(i, face, k + 1), layer, 31, .62);
    }
    L->x0.resize(3 * x.size());
    L->r0.assign(4 * x.size(), 0.0);
    for (size_t n = 0; n < x.size(); n++) {
        L->x0[3 * n] = x[n].x; L->x0[3 * n + 1] = x[n].y; L->x0[3 * n + 2] = x[n].z;
        L->r0[4 * n] = 1.0;
    }
    std::sort(excluded.begin(), excluded.end());
    excluded.erase(std::unique(excluded.begin(), excluded.end()), excluded.end());
    L->connected = std::move(excluded);
    return finish(L, cfg, width, height, depth);
}

}  // namespace

extern "C" {

int mcg_lattice_generate(const mcg_lattice_spec* spec, const mcg_config* cfg, mcg_lattice** out) {
    if (!spec || !cfg || !out) return MCG_ERR_INVALID;
    *out = nullptr;
    if (spec->kind == MCG_LATTICE_REFERENCE_BCC) {
        const mcg_config& c = *cfg;
        if (c.cells_x < 1 || c.cells_y < 1 || c.cells_z < 1 || !(c.cell_size > 0) || !(c.min_radius > 0) ||
            !(c.max_radius > 0) || (long long)c.cells_x * c.cells_y * c.cells_z > (1LL << 22))
            return MCG_ERR_INVALID;
        mcg_lattice* R = new (std::nothrow) mcg_lattice;
        if (!R) return MCG_ERR_INVALID;
        if (!build_reference(c, R)) {
            delete R;
            return MCG_ERR_INVALID;
        }
        *out = R;
        return MCG_OK;
    }
    const int nx = spec->cells_x, ny = spec->cells_y, nz = spec->cells_z;
    if (nx < 1 || ny < 1 || nz < 1 || !(spec->cell_size > 0) || !(spec->r0 > 0) || !(spec->r1 > 0) ||
        spec->jitter < 0 || spec->jitter >= 0.5 ||
        (spec->kind != MCG_LATTICE_CUBIC && spec->kind != MCG_LATTICE_CUBIC_BCC) ||
        (spec->radius_mode != MCG_RADIUS_GRADED_Y && spec->radius_mode != MCG_RADIUS_UNIFORM))
        return MCG_ERR_INVALID;
    const long long corners = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    const long long centres = spec->kind == MCG_LATTICE_CUBIC_BCC ? (long long)nx * ny * nz : 0;
    if (corners + centres > std::numeric_limits<int32_t>::max() / 8) return MCG_ERR_INVALID;
    mcg_lattice* L = new (std::nothrow) mcg_lattice;
    if (!L) return MCG_ERR_INVALID;
    const double cs = spec->cell_size;
    const double width = nx * cs, height = ny * cs, depth = nz * cs;
    const double jr = cfg->joint_scale * cfg->max_radius;
    const double ox = -.5 * width, oy = jr, oz = -.5 * depth;  // as sim.cpp:57
    auto corner = [&](int i, int j, int k) { return int((j * (nz + 1) + k) * (nx + 1) + i); };
    auto centre = [&](int i, int j, int k) { return int(corners + (j * nz + k) * nx + i); };
    const size_t N = size_t(corners + centres);
    L->x0.resize(3 * N);
    L->r0.assign(4 * N, 0.0);
    L->layer.resize(N);
    Rng rng(spec->seed);
    const double jit = spec->jitter * cs;
    for (int j = 0; j <= ny; j++)
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                const size_t n = size_t(corner(i, j, k));
                const double jx = jit * rng.signedUniform();
                const double jy = jit * rng.signedUniform();
                const double jz = jit * rng.signedUniform();
                L->x0[3 * n] = ox + i * cs + jx;
                // the top and bottom faces stay planar so that the platens seat evenly
                L->x0[3 * n + 1] = oy + j * cs + ((j == 0 || j == ny) ? 0.0 : jy);
                L->x0[3 * n + 2] = oz + k * cs + jz;
                L->layer[n] = j;
            }
    for (long long c = 0; c < centres; c++) {
        const int i = int(c % nx), k = int((c / nx) % nz), j = int(c / ((long long)nx * nz));
        const size_t n = size_t(centre(i, j, k));
        L->x0[3 * n] = ox + (i + .5) * cs + jit * rng.signedUniform();
        L->x0[3 * n + 1] = oy + (j + .5) * cs + jit * rng.signedUniform();
        L->x0[3 * n + 2] = oz + (k + .5) * cs + jit * rng.signedUniform();
        L->layer[n] = j;
    }
    for (size_t n = 0; n < N; n++) L->r0[4 * n] = 1.0;
    auto add_beam = [&](int a, int b) { L->beam_a.push_back(a); L->beam_b.push_back(b); };
    for (int j = 0; j <= ny; j++)
        for (int k = 0; k <= nz; k++)
            for (int i = 0; i <= nx; i++) {
                const int a = corner(i, j, k);
                if (i < nx) add_beam(a, corner(i + 1, j, k));
                if (j < ny) add_beam(a, corner(i, j + 1, k));
                if (k < nz) add_beam(a, corner(i, j, k + 1));
            }
    if (centres) {
        static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                      {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                for (int i = 0; i < nx; i++)
                    for (int q = 0; q < 8; q++)
                        add_beam(centre(i, j, k), corner(i + off[q][0], j + off[q][1], k + off[q][2]));
    }
    const size_t B = L->beam_a.size();
    L->L0.resize(B); L->radius.resize(B); L->area.resize(B); L->I.resize(B); L->J.resize(B);
    L->e0.resize(3 * B);
    L->connected.resize(B);
    Rng rrng(mix64(spec->seed ^ 0x5241444949ULL));
    for (size_t b = 0; b < B; b++) {
        const int a = L->beam_a[b], c = L->beam_b[b];
        const double dx = L->x0[3 * size_t(c)] - L->x0[3 * size_t(a)];
        const double dy = L->x0[3 * size_t(c) + 1] - L->x0[3 * size_t(a) + 1];
        const double dz = L->x0[3 * size_t(c) + 2] - L->x0[3 * size_t(a) + 2];
        const double l = std::sqrt(dx * dx + dy * dy + dz * dz);
        const double inv = 1.0 / l;
        L->L0[b] = l;
        L->e0[3 * b] = dx * inv; L->e0[3 * b + 1] = dy * inv; L->e0[3 * b + 2] = dz * inv;
        double r;
        if (spec->radius_mode == MCG_RADIUS_GRADED_Y) {
            const double my = .5 * (L->x0[3 * size_t(a) + 1] + L->x0[3 * size_t(c) + 1]);
            const double yf = std::clamp((my - jr) / height, 0.0, 1.0);
            r = spec->r0 + (spec->r1 - spec->r0) * yf;
        } else {
            r = spec->r0 + (spec->r1 - spec->r0) * rrng.uniform();
        }
        L->radius[b] = r;
        L->area[b] = kPi * r * r;
        L->I[b] = .25 * kPi * std::pow(r, 4);
        L->J[b] = 2 * L->I[b];
        L->connected[b] = pair_key(a, c);
    }
    std::sort(L->connected.begin(), L->connected.end());
    L->connected.erase(std::unique(L->connected.begin(), L->connected.end()), L->connected.end());
    // lumped mass, joint mass and the two anti-drift locks (sim.cpp:134)
    double total = 0;
    L->mass.assign(N, 0.0);
    for (size_t b = 0; b < B; b++) {
        const double m = cfg->material.density * L->area[b] * L->L0[b];
        L->mass[size_t(L->beam_a[b])] += .5 * m;
        L->mass[size_t(L->beam_b[b])] += .5 * m;
        total += m;
    }
    const double jm = cfg->material.density * (4.0 / 3.0) * kPi * std::pow(jr, 3) * .28;
    for (size_t n = 0; n < N; n++) { L->mass[n] += jm; total += jm; }
    L->locked.assign(6 * N, 0);
    int la = -1, lb = -1;
    double da = std::numeric_limits<double>::infinity(), db = da;
    for (size_t n = 0; n < N; n++)
        if (L->layer[n] == 0) {
            const double px = L->x0[3 * n], pz = L->x0[3 * n + 2];
            const double qa = (px + .5 * width) * (px + .5 * width) + (pz + .5 * depth) * (pz + .5 * depth);
            const double qb = (px - .5 * width) * (px - .5 * width) + (pz + .5 * depth) * (pz + .5 * depth);
            if (qa < da) { da = qa; la = int(n); }
            if (qb < db) { db = qb; lb = int(n); }
        }
    if (la < 0 || lb < 0) { delete L; return MCG_ERR_INVALID; }
    L->locked[size_t(6 * la)] = 1; L->locked[size_t(6 * la + 2)] = 1; L->locked[size_t(6 * lb + 2)] = 1;
    L->geometry.width = width; L->geometry.height = height; L->geometry.depth = depth;
    L->geometry.area = width * depth; L->geometry.mass = total; L->geometry.top0 = jr + height + jr;
    *out = L;
    return MCG_OK;
}

int mcg_lattice_view_of(const mcg_lattice* L, mcg_lattice_view* v) {
    if (!L || !v) return MCG_ERR_INVALID;
    v->n_nodes = int32_t(L->mass.size());
    v->n_beams = int32_t(L->L0.size());
    v->n_connected = int64_t(L->connected.size());
    v->x0 = L->x0.data(); v->r0 = L->r0.data(); v->layer = L->layer.data(); v->mass = L->mass.data();
    v->locked = L->locked.data(); v->beam_a = L->beam_a.data(); v->beam_b = L->beam_b.data();
    v->L0 = L->L0.data(); v->radius = L->radius.data(); v->area = L->area.data(); v->I = L->I.data();
    v->J = L->J.data(); v->e0 = L->e0.data(); v->connected = L->connected.data();
    v->geometry = L->geometry;
    return MCG_OK;
}

int mcg_lattice_topology(const mcg_lattice* L, mcg_topology* t) {
    if (!L || !t) return MCG_ERR_INVALID;
    t->n_nodes = int32_t(L->mass.size());
    t->n_beams = int32_t(L->L0.size());
    t->beam_a = L->beam_a.data(); t->beam_b = L->beam_b.data();
    t->L0 = L->L0.data(); t->radius = L->radius.data(); t->area = L->area.data();
    t->I = L->I.data(); t->J = L->J.data(); t->e0 = L->e0.data(); t->mass = L->mass.data();
    t->locked = L->locked.data();
    t->n_connected = int64_t(L->connected.size());
    t->connected = L->connected.data();
    return MCG_OK;
}

void mcg_lattice_free(mcg_lattice* L) { delete L; }

int mcg_random_state(int32_t n_nodes, int32_t n_beams, const uint8_t* locked, double sigma_t, double sigma_r,
                     double epsp_max, uint64_t seed, double* z, double* plastic) {
    if (n_nodes < 0 || n_beams < 0) return MCG_ERR_INVALID;
    Rng rng(seed);
    if (z) {
        for (int32_t i = 0; i < n_nodes; i++) {
            double* zi = z + 6 * size_t(i);
            for (int d = 0; d < 3; d++) zi[d] = sigma_t * rng.normal();
            double ax = rng.normal(), ay = rng.normal(), az = rng.normal();
            double l = std::sqrt(ax * ax + ay * ay + az * az);
            if (!(l > 1e-12)) { ax = 0; ay = 0; az = 1; l = 1; }
            const double th = sigma_r * rng.normal();
            zi[3] = ax / l * th; zi[4] = ay / l * th; zi[5] = az / l * th;
            if (locked)
                for (int d = 0; d < 6; d++)
                    if (locked[6 * size_t(i) + d]) zi[d] = 0;
        }
    }
    if (plastic) {
        Rng prng(mix64(seed ^ 0x504c4153ULL));
        for (int32_t b = 0; b < n_beams; b++) {
            double* q = plastic + 7 * size_t(b);
            const double e = epsp_max * prng.uniform();
            q[0] = e; q[1] = e;
            for (int k = 2; k < 7; k++) q[k] = 0;
        }
    }
    return MCG_OK;
}

}  // extern "C"
