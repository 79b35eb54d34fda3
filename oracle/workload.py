"""The seeded synthetic nanotip workload, restated in numpy -- TEST INFRASTRUCTURE ONLY.

The product's generator (femocs_gb300/csrc/synth.cpp) stands in for the reference's atom
import and TetGen meshing, which are outside the measured path. This module produces the same
arrays bit for bit (tests/test_oracle_workload.py checks it) so that the CPU reference arm of
the benchmark can build its inputs without loading the product's library:

* a graded tensor grid (uniform core of spacing h around the tip, geometric growth outside)
  split into six Kuhn tetrahedra per cell, marked vacuum (3) or bulk (1) by the centroid;
* FCC atoms (lattice constant a) filling the metal with Gaussian-like jitter (Irwin-Hall sum
  of 12 uniforms from a SplitMix64 stream), surface atoms = coordination < 12 within a
  cutoff, away from the box rim;
* uniform random vacuum probes by rejection sampling.

Only IEEE +, -, *, / and comparisons are used, in the generator's order, so results are
identical on x86 and Arm.
"""
from __future__ import annotations

import math

import numpy as np

VACUUM, BULK, SURFACE = 3, 1, 2

# the benchmarked nanotips [Angstrom]: R = 2 nm, H = 8 nm on a 20 x 20 x 2 nm slab, vacuum to
# 60 nm (configuration 1); R = 5 nm, H = 40 nm on 80 x 80 x 4 nm, vacuum to 250 nm
# (configuration 2); the grid spacing and growth give ~2.8e5 and ~2.3e6 vacuum hexahedra
CONFIG1 = dict(radius=20.0, height=80.0, box_half=100.0, slab=20.0, top=600.0, h=7.0, growth=1.25, margin=12.0)
CONFIG2 = dict(radius=50.0, height=400.0, box_half=400.0, slab=40.0, top=2500.0, h=9.5, growth=1.18, margin=20.0)
GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

__all__ = ["CONFIG1", "CONFIG2", "graded_axis", "nanotip_axes", "inside_metal", "tet_mesh", "atoms", "probes", "jitter", "VACUUM", "BULK",
           "SURFACE"]


def _rng_state(seed):
    with np.errstate(over="ignore"):
        return np.uint64(seed) * GOLDEN + np.uint64(0x632BE59BD9B4E019)


def _uniforms(state, first, count):
    """uniforms number first..first+count-1 of a SplitMix64 stream in state `state`"""
    with np.errstate(over="ignore"):
        z = state + (np.arange(first + 1, first + count + 1, dtype=np.uint64) * GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _normals(state, count, chunk=1 << 20):
    """`count` approximately standard normal deviates: sum of 12 uniforms (in order) minus 6"""
    out = np.empty(count)
    for o in range(0, count, chunk):
        m = min(chunk, count - o)
        u = _uniforms(state, 12 * o, 12 * m).reshape(m, 12)
        acc = u[:, 0].copy()
        for k in range(1, 12):
            acc += u[:, k]
        out[o:o + m] = acc - 6.0
    return out


def graded_axis(lo, c0, c1, hi, h, g):
    """uniform spacing inside [c0, c1], geometrically growing spacing outside, ending at lo, hi"""
    if c1 - c0 < h:
        mid = 0.5 * (c0 + c1)
        c0 = max(lo, mid - 0.5 * h)
        c1 = min(hi, mid + 0.5 * h)
    n = max(1, int(math.ceil((c1 - c0) / h - 1e-9)))
    step = (c1 - c0) / n
    core = [c1 if i == n else c0 + step * i for i in range(n + 1)]

    def grow(start, end, direction):
        out, x, s = [], start, step
        while True:
            s *= g
            nx = x + direction * s
            rem = direction * (end - nx)
            if rem <= 0.5 * s * g:
                out.append(end)
                break
            out.append(nx)
            x = nx
        return out

    axis = []
    if lo < c0:
        axis.extend(reversed(grow(c0, lo, -1.0)))
    axis.extend(core)
    if hi > c1:
        axis.extend(grow(c1, hi, 1.0))
    return np.array(axis)


def nanotip_axes(spec):
    cx = spec["radius"] + spec["margin"]
    ax = graded_axis(-spec["box_half"], -cx, cx, spec["box_half"], spec["h"], spec["growth"])
    up = graded_axis(0.0, 0.0, spec["height"] + spec["margin"], spec["top"], spec["h"], spec["growth"])
    down = graded_axis(-spec["slab"], 0.0, 0.0 + spec["h"], spec["h"], spec["h"], spec["growth"])
    az = np.r_[down[down < 0.0], up]
    return ax, az


def inside_metal(spec, x, y, z):
    """cylinder of radius R up to height - R, capped by a hemisphere, on the slab z <= 0"""
    R = spec["radius"]
    zc = spec["height"] - R
    r2 = x * x + y * y
    R2 = R * R
    dz = z - zc
    return (z <= 0.0) | np.where(z <= zc, r2 <= R2, r2 + dz * dz <= R2)


_KUHN = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (2, 1, 0), (1, 0, 2))


def tet_mesh(spec):
    """(xyz (n, 3), tets (m, 4) int32, markers (m,) int32) of the graded Kuhn-split grid"""
    ax, az = nanotip_axes(spec)
    nx = ny = len(ax)
    nz = len(az)
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    xyz = np.stack([ax[I.ravel()], ax[J.ravel()], az[K.ravel()]], axis=1)
    K, J, I = (a.ravel() for a in np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij"))

    def nid(i, j, k):
        return ((k * ny + j) * nx + i).astype(np.int32)

    tets = np.empty((len(I), 6, 4), dtype=np.int32)
    for p, perm in enumerate(_KUHN):
        c = [0, 0, 0]
        v = [nid(I, J, K)]
        for s2 in range(2):
            c[perm[s2]] = 1
            v.append(nid(I + c[0], J + c[1], K + c[2]))
        v.append(nid(I + 1, J + 1, K + 1))
        if p >= 3:
            v[2], v[3] = v[3], v[2]
        tets[:, p, :] = np.stack(v, axis=1)
    tets = tets.reshape(-1, 4)
    P = xyz[tets]  # (m, 4, 3)
    ctr = ((P[:, 0] + P[:, 1]) + P[:, 2]) + P[:, 3]
    metal = inside_metal(spec, ctr[:, 0] * 0.25, ctr[:, 1] * 0.25, ctr[:, 2] * 0.25)
    return xyz, tets, np.where(metal, BULK, VACUUM).astype(np.int32)


def atoms(spec, a=3.615, sigma=0.05, cutoff=3.1, seed=12345):
    """(xyz (n, 3), types (n,)) of the jittered FCC metal; types 2 = surface, 1 = bulk"""
    from scipy.spatial import cKDTree
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    imax = int(math.ceil(spec["box_half"] / a)) + 1
    kmin = -int(math.ceil(spec["slab"] / a)) - 1
    kmax = int(math.ceil(spec["height"] / a)) + 1
    lim = spec["box_half"] - 0.25 * a
    K, J, I, B = (v.ravel() for v in np.meshgrid(np.arange(kmin, kmax + 1), np.arange(-imax, imax + 1),
                                                np.arange(-imax, imax + 1), np.arange(4), indexing="ij"))
    x = a * (I + basis[B, 0])
    y = a * (J + basis[B, 1])
    z = a * (K + basis[B, 2]) - 0.5 * a
    keep = ~((z < -spec["slab"]) | (np.abs(x) > lim) | (np.abs(y) > lim))
    x, y, z = x[keep], y[keep], z[keep]
    keep = inside_metal(spec, x, y, z)
    pos = np.stack([x[keep], y[keep], z[keep]], axis=1).reshape(-1)
    n = len(pos) // 3
    pos = pos + sigma * _normals(_rng_state(seed), 3 * n)
    pos = pos.reshape(n, 3)
    # coordination: neighbours with squared distance (dx*dx + dy*dy) + dz*dz <= cutoff^2
    pairs = cKDTree(pos).query_pairs(cutoff * (1.0 + 1e-9), output_type="ndarray")
    d = pos[pairs[:, 0]] - pos[pairs[:, 1]]
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    pairs = pairs[d2 <= cutoff * cutoff]
    coord = np.bincount(pairs.ravel(), minlength=n)
    rim = ((np.abs(pos[:, 0]) > spec["box_half"] - cutoff - a) | (np.abs(pos[:, 1]) > spec["box_half"] - cutoff - a)
           | (pos[:, 2] < -spec["slab"] + cutoff + a))
    types = np.where((coord < 12) & ~rim, SURFACE, BULK).astype(np.int32)
    return pos, types


def probes(spec, n, seed=777):
    """n uniform random points of the vacuum part of the box (rejection sampling)"""
    state = _rng_state(np.uint64(seed) ^ np.uint64(0xA5A5A5A5))
    out, drawn = [], 0
    b, top = spec["box_half"], spec["top"]
    while sum(len(o) for o in out) < n:
        m = max(1024, 2 * (n - sum(len(o) for o in out)))
        u = _uniforms(state, drawn, 3 * m).reshape(m, 3)
        drawn += 3 * m
        x = -b + 2.0 * b * u[:, 0]
        y = -b + 2.0 * b * u[:, 1]
        z = top * u[:, 2]
        ok = ~inside_metal(spec, x, y, z)
        out.append(np.stack([x[ok], y[ok], z[ok]], axis=1))
    return np.concatenate(out)[:n]


def jitter(xyz, sigma, seed):
    """Gaussian-like displacement of every coordinate (the MD step stand-in)"""
    p = np.asarray(xyz, dtype=np.float64).reshape(-1)
    return (p + sigma * _normals(_rng_state(seed), len(p))).reshape(np.shape(xyz))
