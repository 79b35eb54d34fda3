// Seeded synthetic nanotip workloads: a graded tetrahedral mesh of the box around a
// cylinder+hemisphere tip on a slab, FCC atoms of the metal with thermal jitter, their
// surface subset (coordination analysis) and random probe points in the vacuum.
//
// Stands in for the reference's atom import + TetGen meshing (out of scope for the GPU
// path); all arithmetic is IEEE +,-,*,/ and sqrt only, so x86 and Arm produce identical
// meshes and points.
#pragma once

#include "mesh.h"

namespace fgb {

struct NanotipSpec {
    double radius = 20.0;       // tip radius [A]
    double height = 80.0;       // apex height above the slab surface z=0 [A]
    double box_half = 100.0;    // half width of the box in x and y [A]
    double slab = 20.0;         // slab thickness below z=0 [A]
    double top = 600.0;         // z of the vacuum box top [A]
    double h = 8.0;             // grid spacing in the refined core [A]
    double growth = 1.3;        // spacing growth factor outside the core
    double margin = 10.0;       // core extends this far beyond the tip [A]
};

bool inside_metal(const NanotipSpec& s, double x, double y, double z);

// Graded tensor grid, each cell split into six tets along the main diagonal; tet marker
// kVacuum if its centroid lies outside the metal, kBulk otherwise.
TetMesh make_nanotip_mesh(const NanotipSpec& s);
// vacuum hexahedra of the mesh make_nanotip_mesh would build (4 per vacuum tet)
long long nanotip_vacuum_hexes(const NanotipSpec& s);
// core spacing h for which the mesh has about target_hexes vacuum hexahedra
double fit_nanotip_spacing(NanotipSpec s, long long target_hexes);

struct AtomSet {
    std::vector<double> xyz;        // 3 * n
    std::vector<int32_t> type;      // kBulk or kSurface
};
// FCC lattice (lattice constant a) filling the metal, jitter ~N(0, sigma^2) per coordinate
// (Irwin-Hall sum of 12 uniforms), surface = coordination < 12 within `cutoff`.
AtomSet make_nanotip_atoms(const NanotipSpec& s, double a, double sigma, double cutoff, uint64_t seed);

// Uniform random points in the vacuum part of the box (rejection sampling).
std::vector<double> make_vacuum_probes(const NanotipSpec& s, int n, uint64_t seed);

// Gaussian displacement of every coordinate (MD step stand-in).
void jitter_points(std::vector<double>& xyz, double sigma, uint64_t seed);

}  // namespace fgb
