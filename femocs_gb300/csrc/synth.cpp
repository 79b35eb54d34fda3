#include "synth.h"

#include <algorithm>
#include <cmath>

namespace fgb {

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // approximately standard normal: Irwin-Hall sum of 12 uniforms minus 6
    double normal() {
        double acc = 0.0;
        for (int i = 0; i < 12; ++i) acc += uniform();
        return acc - 6.0;
    }
};

// 1-D graded coordinates: uniform spacing inside [c0, c1], geometrically growing spacing
// outside, ending exactly at lo and hi.
std::vector<double> graded_axis(double lo, double c0, double c1, double hi, double h, double g) {
    FGB_REQUIRE(h > 0 && g >= 1.0 && hi > lo, "invalid grid grading");
    if (c1 - c0 < h) {  // degenerate core (e.g. no tip): one cell of size h around its middle
        const double mid = 0.5 * (c0 + c1);
        c0 = std::max(lo, mid - 0.5 * h);
        c1 = std::min(hi, mid + 0.5 * h);
    }
    std::vector<double> core;
    int n = std::max(1, (int)std::ceil((c1 - c0) / h - 1e-9));
    double step = (c1 - c0) / n;
    for (int i = 0; i <= n; ++i) core.push_back(i == n ? c1 : c0 + step * i);
    auto grow = [&](double start, double end, double dir) {
        std::vector<double> out;
        double x = start, s = step;
        while (true) {
            s *= g;
            double nx = x + dir * s;
            double rem = dir * (end - nx);
            if (rem <= 0.5 * s * g) { out.push_back(end); break; }
            out.push_back(nx);
            x = nx;
        }
        return out;
    };
    std::vector<double> axis;
    if (lo < c0) {
        std::vector<double> d = grow(c0, lo, -1.0);
        std::reverse(d.begin(), d.end());
        axis.insert(axis.end(), d.begin(), d.end());
    }
    axis.insert(axis.end(), core.begin(), core.end());
    if (hi > c1) {
        std::vector<double> u = grow(c1, hi, +1.0);
        axis.insert(axis.end(), u.begin(), u.end());
    }
    return axis;
}

}  // namespace

bool inside_metal(const NanotipSpec& s, double x, double y, double z) {
    if (z <= 0.0) return true;
    const double zc = s.height - s.radius;
    const double r2 = x * x + y * y;
    const double R2 = s.radius * s.radius;
    if (z <= zc) return r2 <= R2;
    const double dz = z - zc;
    return r2 + dz * dz <= R2;
}

namespace {
void nanotip_axes(const NanotipSpec& s, std::vector<double>& ax, std::vector<double>& az) {
    const double cx = s.radius + s.margin;
    ax = graded_axis(-s.box_half, -cx, cx, s.box_half, s.h, s.growth);
    az.clear();
    std::vector<double> up = graded_axis(0.0, 0.0, s.height + s.margin, s.top, s.h, s.growth);
    std::vector<double> down = graded_axis(-s.slab, 0.0, 0.0 + s.h, s.h, s.h, s.growth);
    for (double z : down)
        if (z < 0.0) az.push_back(z);
    az.insert(az.end(), up.begin(), up.end());
}
const int kKuhn[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
}  // namespace

long long nanotip_vacuum_hexes(const NanotipSpec& s) {
    std::vector<double> ax, az;
    nanotip_axes(s, ax, az);
    const int nx = (int)ax.size(), nz = (int)az.size();
    long long n = 0;
    for (int k = 0; k + 1 < nz; ++k)
        for (int j = 0; j + 1 < nx; ++j)
            for (int i = 0; i + 1 < nx; ++i)
                for (int p = 0; p < 6; ++p) {
                    // centroid of the Kuhn tet: corner 000, +e_p0, +e_p0+e_p1, corner 111
                    int c[3] = {0, 0, 0};
                    double sx = ax[i] + ax[i + 1], sy = ax[j] + ax[j + 1], sz = az[k] + az[k + 1];
                    for (int s2 = 0; s2 < 2; ++s2) {
                        c[kKuhn[p][s2]] = 1;
                        sx += ax[i + c[0]];
                        sy += ax[j + c[1]];
                        sz += az[k + c[2]];
                    }
                    if (!inside_metal(s, sx * 0.25, sy * 0.25, sz * 0.25)) n += 4;
                }
    return n;
}

double fit_nanotip_spacing(NanotipSpec s, long long target_hexes) {
    FGB_REQUIRE(target_hexes > 0, "target hex count must be positive");
    double lo = 0.05 * std::max(1.0, s.radius), hi = std::max(s.box_half, s.top);
    for (int it = 0; it < 50; ++it) {
        const double mid = std::sqrt(lo * hi);
        s.h = mid;
        if (nanotip_vacuum_hexes(s) > target_hexes) lo = mid;
        else hi = mid;
        if (hi / lo < 1.002) break;
    }
    return std::sqrt(lo * hi);
}

TetMesh make_nanotip_mesh(const NanotipSpec& s) {
    const double cx = s.radius + s.margin;
    std::vector<double> ax = graded_axis(-s.box_half, -cx, cx, s.box_half, s.h, s.growth);
    std::vector<double> az;
    {
        // below the slab surface: graded downward from z=0; above: core up to the apex + margin
        std::vector<double> up = graded_axis(0.0, 0.0, s.height + s.margin, s.top, s.h, s.growth);
        std::vector<double> down = graded_axis(-s.slab, 0.0, 0.0 + s.h, s.h, s.h, s.growth);
        // `down` spans [-slab, h]; keep its part below zero
        for (double z : down)
            if (z < 0.0) az.push_back(z);
        az.insert(az.end(), up.begin(), up.end());
    }
    const int nx = (int)ax.size(), ny = nx, nz = (int)az.size();
    TetMesh tm;
    tm.xyz.resize(3 * (size_t)nx * ny * nz);
    auto nid = [&](int i, int j, int k) { return (int32_t)(((size_t)k * ny + j) * nx + i); };
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t o = 3 * (size_t)nid(i, j, k);
                tm.xyz[o] = ax[i];
                tm.xyz[o + 1] = ax[j];
                tm.xyz[o + 2] = az[k];
            }
    // Kuhn split: tet = corner 000, +e_p0, +e_p0+e_p1, corner 111 for each axis order p
    static const int perms[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
    const size_t n_cells = (size_t)(nx - 1) * (ny - 1) * (nz - 1);
    tm.tets.reserve(24 * n_cells);
    tm.marker.reserve(6 * n_cells);
    for (int k = 0; k < nz - 1; ++k)
        for (int j = 0; j < ny - 1; ++j)
            for (int i = 0; i < nx - 1; ++i)
                for (int p = 0; p < 6; ++p) {
                    int c[3] = {0, 0, 0};
                    int32_t v[4];
                    v[0] = nid(i, j, k);
                    for (int s2 = 0; s2 < 2; ++s2) {
                        c[perms[p][s2]] = 1;
                        v[1 + s2] = nid(i + c[0], j + c[1], k + c[2]);
                    }
                    v[3] = nid(i + 1, j + 1, k + 1);
                    if (p >= 3) std::swap(v[2], v[3]);  // odd permutations: restore positive orientation
                    double cxx = 0, cyy = 0, czz = 0;
                    for (int q = 0; q < 4; ++q) {
                        cxx += tm.xyz[3 * (size_t)v[q]];
                        cyy += tm.xyz[3 * (size_t)v[q] + 1];
                        czz += tm.xyz[3 * (size_t)v[q] + 2];
                    }
                    const bool metal = inside_metal(s, cxx * 0.25, cyy * 0.25, czz * 0.25);
                    for (int q = 0; q < 4; ++q) tm.tets.push_back(v[q]);
                    tm.marker.push_back(metal ? kBulk : kVacuum);
                }
    return tm;
}

AtomSet make_nanotip_atoms(const NanotipSpec& s, double a, double sigma, double cutoff, uint64_t seed) {
    static const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    AtomSet at;
    std::vector<double> pos;
    const int imax = (int)std::ceil(s.box_half / a) + 1;
    const int kmin = -(int)std::ceil(s.slab / a) - 1;
    const int kmax = (int)std::ceil(s.height / a) + 1;
    const double lim = s.box_half - 0.25 * a;
    for (int k = kmin; k <= kmax; ++k)
        for (int j = -imax; j <= imax; ++j)
            for (int i = -imax; i <= imax; ++i)
                for (int b = 0; b < 4; ++b) {
                    double x = a * (i + basis[b][0]);
                    double y = a * (j + basis[b][1]);
                    double z = a * (k + basis[b][2]) - 0.5 * a;  // top layer just below z=0
                    if (z < -s.slab || std::fabs(x) > lim || std::fabs(y) > lim) continue;
                    if (!inside_metal(s, x, y, z)) continue;
                    pos.push_back(x);
                    pos.push_back(y);
                    pos.push_back(z);
                }
    const size_t n = pos.size() / 3;
    Rng rng(seed);
    for (size_t i = 0; i < 3 * n; ++i) pos[i] += sigma * rng.normal();

    // coordination by cell list
    const double cs = cutoff;
    double bmin[3] = {1e300, 1e300, 1e300}, bmax[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            bmin[c] = std::min(bmin[c], pos[3 * i + c]);
            bmax[c] = std::max(bmax[c], pos[3 * i + c]);
        }
    int nc[3];
    for (int c = 0; c < 3; ++c) nc[c] = std::max(1, (int)((bmax[c] - bmin[c]) / cs) + 1);
    auto cell_of = [&](size_t i, int* ci) {
        for (int c = 0; c < 3; ++c) ci[c] = std::min(nc[c] - 1, (int)((pos[3 * i + c] - bmin[c]) / cs));
    };
    const size_t ncell = (size_t)nc[0] * nc[1] * nc[2];
    std::vector<int32_t> head(ncell + 1, 0), items(n);
    std::vector<int32_t> cid(n);
    for (size_t i = 0; i < n; ++i) {
        int ci[3];
        cell_of(i, ci);
        cid[i] = (int32_t)(((size_t)ci[2] * nc[1] + ci[1]) * nc[0] + ci[0]);
        head[cid[i] + 1]++;
    }
    for (size_t c = 0; c < ncell; ++c) head[c + 1] += head[c];
    {
        std::vector<int32_t> p(head.begin(), head.end() - 1);
        for (size_t i = 0; i < n; ++i) items[p[cid[i]]++] = (int32_t)i;
    }
    const double c2 = cutoff * cutoff;
    at.xyz = pos;
    at.type.assign(n, kBulk);
    for (size_t i = 0; i < n; ++i) {
        int ci[3];
        cell_of(i, ci);
        int coord = 0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    int x = ci[0] + dx, y = ci[1] + dy, z = ci[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) continue;
                    size_t c = ((size_t)z * nc[1] + y) * nc[0] + x;
                    for (int p = head[c]; p < head[c + 1]; ++p) {
                        int32_t jj = items[p];
                        if ((size_t)jj == i) continue;
                        double ddx = pos[3 * i] - pos[3 * (size_t)jj];
                        double ddy = pos[3 * i + 1] - pos[3 * (size_t)jj + 1];
                        double ddz = pos[3 * i + 2] - pos[3 * (size_t)jj + 2];
                        if (ddx * ddx + ddy * ddy + ddz * ddz <= c2) ++coord;
                    }
                }
        const bool rim = std::fabs(pos[3 * i]) > s.box_half - cutoff - a ||
                         std::fabs(pos[3 * i + 1]) > s.box_half - cutoff - a ||
                         pos[3 * i + 2] < -s.slab + cutoff + a;
        if (coord < 12 && !rim) at.type[i] = kSurface;
    }
    return at;
}

std::vector<double> make_vacuum_probes(const NanotipSpec& s, int n, uint64_t seed) {
    Rng rng(seed ^ 0xA5A5A5A5ull);
    std::vector<double> p;
    p.reserve(3 * (size_t)n);
    while ((int)(p.size() / 3) < n) {
        double x = -s.box_half + 2.0 * s.box_half * rng.uniform();
        double y = -s.box_half + 2.0 * s.box_half * rng.uniform();
        double z = s.top * rng.uniform();
        if (inside_metal(s, x, y, z)) continue;
        p.push_back(x);
        p.push_back(y);
        p.push_back(z);
    }
    return p;
}

void jitter_points(std::vector<double>& xyz, double sigma, uint64_t seed) {
    Rng rng(seed);
    for (double& v : xyz) v += sigma * rng.normal();
}

}  // namespace fgb
