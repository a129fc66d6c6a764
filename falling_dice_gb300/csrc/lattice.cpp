// lattice.cpp -- synthetic cubic and cubic+BCC beam lattices and seeded deformed states.
//
// The reference builds one graded-BCC specimen (MC/src/sim.cpp:51-135).  These generators
// make the cubic and cubic+BCC specimens the throughput workloads are defined on, with one
// element per strut, and apply the reference's own rules for what they share with it:
// node numbering of the corner grid (sim.cpp:54), section properties (sim.cpp:115),
// element-endpoint exclusion pairs (sim.cpp:115-117), lumped mass and the two anti-drift
// locks (sim.cpp:134), platen height (sim.cpp:131) and the splitmix64 generator
// (MC/include/core.hpp:46).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <new>
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

}  // namespace

struct mcg_lattice {
    std::vector<double> x0, r0, mass, L0, radius, area, I, J, e0;
    std::vector<int32_t> layer, beam_a, beam_b;
    std::vector<uint8_t> locked;
    std::vector<uint64_t> connected;
    mcg_geometry geometry{};
};

extern "C" {

int mcg_lattice_generate(const mcg_lattice_spec* spec, const mcg_config* cfg, mcg_lattice** out) {
    if (!spec || !cfg || !out) return MCG_ERR_INVALID;
    *out = nullptr;
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
