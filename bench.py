#!/usr/bin/env python
"""Benchmark of the FEMOCS field-solve path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config2|config1|probe|batch|serve] [--order 1|2]

Workload (default `config2`): synthetic FCC-Cu nanotip, tip radius 5 nm, height 40 nm, on an
80x80x4 nm slab, vacuum box up to 250 nm, graded tet mesh split into ~2.1e6 vacuum hexahedra
with Q2 (27-node) elements (~1.7e7 DoFs; `--order 1` gives the reference's Q1 elements,
2.3e6 DoFs); applied field 1 GV/m (Neumann), phi = 0 on the metal; 1e6 query points = all
surface atoms (coordination < 12) + uniform random vacuum probes. `config1` is the R = 2 nm
tip with Q1 elements.

One step = the reference's Femocs::run field path on resident data: full assembly (element
matrices, CSR scatter, Neumann rhs, Dirichlet elimination), CG solve to a 1e-9 relative
FP64 residual (FP64 CG preconditioned by an FP32 multigrid V-cycle; the hierarchy is built
once per mesh, in the warm-up, and its setup time is reported), nodal field recovery +
smoothing, location + interpolation (rank 1) of all query points. Metric: solved DOF/s =
DoFs / step time. The plain FP64 Jacobi-PCG and the FP32-Jacobi/FP64-refinement solvers are
timed on the same system for comparison.
`e2e` runs the same step through the reference-facing C ABI (femocs_run +
femocs_interpolate_elfield) with host arrays in and out.

N > 1 (torchrun): independent replicas, one per GPU (the solve does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

E0 = -0.1          # V/A, i.e. 1 GV/m; the Neumann value on the top is -E0
REL_TOL = 1e-9
RANK = 1           # interpolation_rank default of the reference (src/Config.cpp:29)
N_POINTS = {"config2": 1_000_000, "config1": 100_000, "probe": 200_000}
# DRAM bytes (read + write) per row of one launch of the hot multigrid kernels, from ncu
# captures of the Q2 probe workload (the SELL level-0 Chebyshev step at 61.9 nonzeros per row,
# as the R = 5 nm nanotip's Q2 rows; the cell-block step, k_cb_apply + k_cb_finish, from the element
# matrices and matrix-free from the FP16 geometric factors); a launch's traffic scales with
# its rows
KERNEL_TRAFFIC_PER_ROW = {("smoother", 2): 551.6, ("smoother_ebe", 2): 261.8, ("smoother_mf16", 2): 114.3}
FALLBACK_HBM_GBS = 6800.0


def element_order(args):
    """the R = 5 nm nanotip (`config2`) is quoted with Q2 elements, the R = 2 nm one (`config1`)
    with Q1 (the reference's element)"""
    if args.order:
        return args.order
    return 2 if args.workload in ("config2", "probe") else 1


def spec_of(workload):
    import femocs_gb300 as fg
    if workload == "probe":  # the R = 5 nm geometry on a coarser grid, small enough for full ncu captures
        return dict(fg.CONFIG2, h=22.0, growth=1.3)
    return dict(fg.CONFIG2 if workload == "config2" else fg.CONFIG1)


def make_points(spec, n_points):
    import numpy as np
    import femocs_gb300 as fg
    atoms, types = fg.synth_atoms(spec, seed=12345)
    surf = atoms[types == 2]
    n_probe = max(0, n_points - len(surf))
    probes = fg.synth_probes(spec, n_probe, seed=777) if n_probe else np.zeros((0, 3))
    return np.ascontiguousarray(np.r_[surf, probes][:n_points]), len(surf)


def write_conf(path, spec, precision="amg", order=1):
    with open(path, "w") as f:
        f.write(f"""mesh_file synthetic
radius {spec['radius']}
tip_height {spec['height']}
gpu_box_half {spec['box_half']}
gpu_slab {spec['slab']}
gpu_top {spec['top']}
gpu_h {spec['h']}
gpu_growth {spec['growth']}
gpu_margin {spec['margin']}
elfield {E0}
anode_bc neumann
interpolation_rank {RANK}
smoothen_field true
gpu_precision {precision}
gpu_rel_tol {REL_TOL}
gpu_element_order {order}
field_ncg 100000
""")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,uuid")

    def __init__(self):
        self.lines = []
        self.proc = None
        # nvidia-smi numbers GPUs physically and ignores CUDA_VISIBLE_DEVICES: rows are kept by
        # the UUID of the device this process computes on
        try:
            import femocs_gb300 as fg
            self.uuid = fg.device_info()[2]
        except Exception:  # noqa: BLE001 -- no device: the sampler reports itself unavailable
            self.uuid = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # nvidia-smi's start-up (driver/NVML initialisation) stalls this process's CUDA calls:
        # the timed region starts after its first sample
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 5.0:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10 or not f[0].isdigit():
                continue
            if (f[9] != self.uuid) if self.uuid else int(f[0]) != 0:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "uuid": self.uuid}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(world, v):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return v


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


# ----------------------------------------------------------------------------------------
def cpu_baseline(field, workload, order, sysm=None, budget_s=12.0):
    """The reference's solver on the host cores for this arm's line: SSOR(1.2)-PCG iterations
    (deal.II SolverCG + PreconditionSSOR restated, src/DealSolver.cpp:443-459) on the system the
    GPU solved, timed live with one thread and with all cores for the SpMV and vector operations
    (the SSOR sweeps are sequential, as in deal.II), times the iteration count of a full oracle
    solve of the same workload (oracle/ssor_iterations.json). Solve only; the CPU reference arm
    (--impl reference) times the whole step on inputs the oracle builds itself."""
    import oracle as orc
    if sysm is None:
        rowptr, col, val, rhs, d2n = field.system()
        sysm = orc.System(csr=(rowptr, col, val, rhs))
    rec = ssor_iterations(workload, order, field.n_dofs)
    cores, model = host_cpu()
    t1 = sysm.ssor_cg_fixed(1)
    k = max(1, min(200, int(0.4 * budget_s / max(t1, 1e-6))))
    t_one = sysm.ssor_cg_fixed(k, threads=1) / k
    t_all = sysm.ssor_cg_fixed(k, threads=cores) / k
    t_it, threads = (t_all, cores) if t_all < t_one else (t_one, 1)
    solve_s = t_it * rec["iterations"]
    return dict(value=field.n_dofs / solve_s, unit="DOF/s", cores=threads, kind="port",
                sample=f"2 x {k} SSOR(1.2)-PCG iterations of the oracle on the full {field.n_dofs}-DoF Q{order} system "
                       f"the GPU solved ({t_one * 1e3:.1f} ms/iteration on 1 thread, {t_all * 1e3:.1f} ms on {cores}) x "
                       f"{rec['iterations']} iterations of a full oracle solve to 1e-9; solve only",
                host={"nproc": cores, "cpu_model": model})


MESH_TABLES = ["tet_nodes", "tet_marker", "tet_nbor", "node_xyz", "node_marker", "hex_nodes", "hex_marker", "tet_det",
               "tet_centroid", "hex_coeffs", "nbr_ptr", "nbr_idx", "quad_nodes", "voro_ptr", "voro_idx",
               "vac_node2vertex", "vac_cells", "tet_search", "edgemax", "node_parents"]


def mesh_prep_timing(spec, order=1):
    """Tet -> hex split, grouping and interpolation tables of the workload's mesh: host builder
    against the kernels (second device run; the first warms the allocator), tables compared
    byte for byte. Outside the timed steps (the bench mesh is prepared once)."""
    import numpy as np
    import femocs_gb300 as fg
    mh = fg.Mesh.synthetic(**spec)
    fg.Mesh.synthetic(device=True, **spec)
    md = fg.Mesh.synthetic(device=True, **spec)
    equal = mh.sizes() == md.sizes() and all(
        np.array_equal(np.ascontiguousarray(mh.export(t)).view(np.uint8), np.ascontiguousarray(md.export(t)).view(np.uint8))
        for t in MESH_TABLES)
    th, td = mh.prep_timing(), md.prep_timing()
    s = md.sizes()
    out = {"tets": s["n_tets"], "hexes": s["n_hexs"], "nodes": s["n_nodes"], "host_ms": th["total_ms"],
           "device_ms": td["total_ms"], "device_kernel_ms": td["kernel_ms"], "tables_equal": bool(equal),
           "note": "device_ms includes the tet upload and the download of every table into host memory"}
    del mh
    # the rest of a re-mesh step on the device-prepared mesh: FEM structure + device system,
    # multigrid hierarchy (built by the first solve), the first solve itself
    t0 = time.perf_counter()
    f = fg.Field(md, order=order)
    field_ms = (time.perf_counter() - t0) * 1e3
    f.setup(E0, 0.0)
    f.assemble(True, False)
    rc, st = f.solve(precision=2, rel_tol=REL_TOL, max_iter=100000)
    out["remesh"] = {"order": order, "field_create_ms": field_ms, "multigrid_setup_ms": st["setup_ms"],
                     "first_solve_ms": st["ms"] - st["setup_ms"],
                     "note": "after the mesh preparation: host FEM structure (device SELL columns for Q2), "
                             "uploads, host multigrid hierarchy"}
    return out


def surface_cpu_timing(spec, surf_pts, sample=2000):
    """The oracle's sequential restatement of the reference's surface interpolation (1 thread)
    on a sample of the surface atoms (the nodal values do not change the work)."""
    import numpy as np
    import femocs_gb300 as fg
    import oracle as orc
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from util import oracle_tables
    m = fg.Mesh.synthetic(**spec)
    tables = oracle_tables(m, np.zeros((m.sizes()["n_nodes"], 5)))
    tris, t2t, _ = m.surface()
    pts = np.ascontiguousarray(surf_pts[:sample])
    t0 = time.perf_counter()
    orc.surface_interpolate(tables, tris, t2t, m.export("node_xyz"), 1, pts)
    dt = time.perf_counter() - t0
    return {"cpu_points_per_s": len(pts) / dt, "cpu_sample": len(pts), "cpu_kind": "port", "cpu_cores": 1}


PARITY_PREFIX = 20000   # points of the timed list checked against the oracle's chain
PARITY_PROBES = 300     # vacuum probes checked as a chain of their own (full scans in the oracle)


def parity_snapshot(fem, spec, field, n_points, d_cells, d_out):
    """What the last timed step produced: the solution (DoF order), the nodal solution and the
    first PARITY_PREFIX located cells and interpolated values."""
    import numpy as np
    import femocs_gb300 as fg
    m = fg.Mesh.synthetic(**spec)
    n_pre = min(PARITY_PREFIX, n_points)
    return {"mesh": m, "x": field.solution(), "nodal": fem.field(m.sizes()).nodal(),
            "cells": d_cells.download(np.zeros(n_points, dtype=np.int32))[:n_pre].copy(),
            "out": d_out.download(np.zeros((n_points, 5)))[:n_pre].copy()}


def interp_parity(fem, snap, pts, n_surf):
    """Location and interpolation of the timed step against the oracle's sequential chain
    (src/SolutionReader.cpp:136-165) with the GPU's own nodal solution: the first
    PARITY_PREFIX points of the timed list (a prefix replays the same chain) and a sample of
    the random vacuum probes as a chain of their own. Cells and values must be bit-exact."""
    import numpy as np
    import oracle as orc
    from oracle import pipeline
    m = snap["mesh"]
    tab = pipeline.tables(m, snap["nodal"])
    cells, out = snap["cells"], snap["out"]
    n_pre = len(cells)
    out_parity = {}
    t0 = time.perf_counter()
    rc, ro = orc.locate_interpolate(tab, RANK, pts[:n_pre])
    out_parity["prefix"] = {"points": int(n_pre), "cells_bit_exact": bool(np.array_equal(cells, rc)),
                            "values_bit_exact": bool(np.array_equal(out.view(np.int64), ro.view(np.int64))),
                            "oracle_s": time.perf_counter() - t0,
                            "note": "first points of the timed step's output (surface atoms first)"}
    n_probe = len(pts) - n_surf
    if n_probe > 0:
        rng = np.random.default_rng(31)
        probes = np.ascontiguousarray(pts[n_surf:][np.sort(rng.choice(n_probe, size=min(PARITY_PROBES, n_probe),
                                                                      replace=False))])
        f = fem.field(m.sizes())
        f.set_nodal(snap["nodal"])
        c, o = f.interpolate(probes, rank=RANK)
        t0 = time.perf_counter()
        rc, ro = orc.locate_interpolate(tab, RANK, probes)
        out_parity["probes"] = {"points": int(len(probes)), "cells_bit_exact": bool(np.array_equal(c, rc)),
                                "values_bit_exact": bool(np.array_equal(o.view(np.int64), ro.view(np.int64))),
                                "oracle_s": time.perf_counter() - t0,
                                "note": "random vacuum probes as their own chain (the oracle scans the mesh)"}
    return out_parity


def config1_parity():
    """Per-result parity at the R = 2 nm configuration (Q1, 2.8e5 DoFs) against the oracle's
    FP64 SSOR(1.2)-CG solve to 1e-13 (src/DealSolver.cpp:443-459), nodal field and smoothing
    (src/Interpolator.cpp:125-170) and the sequential location of the surface atoms: the
    default solver at 1e-9 and FP32-Jacobi with FP64 refinement at 1e-9 and 1e-12."""
    import numpy as np
    import femocs_gb300 as fg
    import oracle as orc
    from oracle import pipeline
    m = fg.Mesh.synthetic(**fg.CONFIG1)
    atoms, types = fg.synth_atoms(fg.CONFIG1, seed=12345)
    surf = np.ascontiguousarray(atoms[types == 2])
    t0 = time.perf_counter()
    sol, info = pipeline.reference_solution(m, -E0, rel_tol=1e-13)
    ref_cells, ref_out = orc.locate_interpolate(pipeline.tables(m, sol), RANK, surf)
    res = {"workload": "config1: nanotip R=2 nm H=8 nm, box 20 nm, top 60 nm, Q1", "n_dofs": info["n_dofs"],
           "surface_atoms": int(len(surf)), "rank": RANK, "oracle_ssor_iterations": info["ssor_iterations"],
           "oracle_rel_residual": info["rel_residual"], "oracle_rel_floor": info["rel_floor"],
           "oracle_s": time.perf_counter() - t0,
           "note": "residuals in the oracle's system, compensated (Dot2); rel_floor = 2^-53 ||(|b|+|A||x|)||/||b||, "
                   "the FP64 rounding floor (two assemblies differ by about that much)",
           "max_abs_phi": float(np.abs(sol[:, 4]).max()), "runs": []}
    system, v2n = info["system"], info["vertex2node"]
    f = fg.Field(m)
    for precision, tol in ((2, 1e-9), (1, 1e-9), (1, 1e-12)):
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=precision, rel_tol=tol, max_iter=100000)
        x = f.phi_nodes()[v2n]
        bnorm = float(np.linalg.norm(system.rhs))
        r_abs, floor_abs = system.residual(x)
        f.extract(True)
        c, o = f.interpolate(surf, rank=RANK)
        p = pipeline.point_parity(c, o, ref_cells, ref_out)
        p.update(solver={2: "FP64 CG + FP32 multigrid", 1: "FP32 Jacobi-PCG + FP64 refinement"}[precision],
                 rel_tol=tol, status={1: "converged", 2: "at the FP64 floor"}.get(st["status"], st["status"]),
                 iterations=st["iterations"], rel_residual_gpu=st["rel_residual"],
                 rel_residual_oracle=r_abs / bnorm, rel_floor=floor_abs / bnorm)
        res["runs"].append(p)
    return res


def run_ours(args, world, rank):
    import numpy as np
    import femocs_gb300 as fg
    from femocs_gb300._lib import load

    spec = spec_of(args.workload)
    order = element_order(args)
    n_points = args.points or N_POINTS[args.workload]
    pts, n_surf = make_points(spec, n_points)
    tmp = tempfile.mkdtemp(prefix="fgb_bench_")
    conf = os.path.join(tmp, "bench.in")
    write_conf(conf, spec, order=order)
    fem = fg.Femocs(conf)
    if fem.run() != 0:
        raise RuntimeError("femocs_run failed: " + fg.last_error())
    # borrowed handle of the device field femocs_run solved on (only DoF-indexed exports used)
    field = fem.field({"n_nodes": 0})
    n = field.n_dofs
    d_pts = fg.DeviceBuffer(24 * n_points)
    d_pts.upload(pts)
    d_cells = fg.DeviceBuffer(4 * n_points)
    d_out = fg.DeviceBuffer(40 * n_points)

    solve_stats = []
    # Q2 level 0: the matrix-free smoother from FP16 geometric factors is the default; stated
    # here so that the line names the kind in use (FP32 when a factor exceeds the FP16 range)
    l0_kind = field.set_level0_operator(2) if order == 2 else 0

    def step(precision):
        field.setup(-E0, 0.0)
        field.assemble(True, False)
        rc, st = field.solve(precision=precision, rel_tol=REL_TOL, max_iter=100000)
        if rc <= 0:
            raise RuntimeError(f"solve did not converge: {st}")
        field.extract(True)
        field.interpolate_device(n_points, d_pts.ptr, RANK, d_cells.ptr, d_out.ptr)
        return st

    # femocs_run above already built the multigrid hierarchy of this mesh (its setup time)
    setup_ms = fem.last_stats()["setup_ms"]
    for _ in range(args.warmup):
        step(2)
    lib = load()
    field.set_profiling(True)
    sampler = ClockSampler()
    sampler.start()
    barrier(world)
    launches0 = lib.fgb_kernel_launches()
    field.mark(0)
    for _ in range(args.steps):
        solve_stats.append(step(2))
    field.mark(1)
    dev_ms = field.elapsed(0, 1)
    launches = lib.fgb_kernel_launches() - launches0
    clocks = sampler.stop()
    field.set_profiling(False)
    snap = (parity_snapshot(fem, spec, field, n_points, d_cells, d_out)
            if rank == 0 and world == 1 and not args.no_parity else None)
    dev_ms = reduce_max(world, dev_ms)
    ms_per_step = dev_ms / args.steps
    value = n * args.steps * world / (dev_ms * 1e-3)
    solve_ms = [s["ms"] for s in solve_stats]
    last = solve_stats[-1]
    levels = field.amg_levels().split()
    # the same solve with the level-0 smoother reading the element matrices (the memory-bound
    # kernel the matrix-free default replaced), for the roofline comparison
    ke_cmp = None
    if order == 2 and l0_kind != 0:
        field.set_level0_operator(0)
        field.set_profiling(True)
        st0 = step(2)
        field.set_profiling(False)
        field.set_level0_operator(l0_kind)
        ms0 = st0["smoother_ms"] / max(st0["smoother_launches"], 1)
        ke_cmp = {"kernel": "k_cb_apply + k_cb_finish, element matrices (FP32 K_e, 1512 B per hex)",
                  "launch_ms": ms0, "bytes_per_launch": st0["smoother_bytes"],
                  "gbs": st0["smoother_bytes"] / (ms0 * 1e-3) / 1e9, "iterations": st0["iterations"],
                  "solve_ms": st0["ms"]}

    # the same step with the plain FP64 Jacobi-PCG, and with FP32 Jacobi-PCG + FP64 refinement
    plain = [step(0) for _ in range(min(2, args.steps))]
    plain_ms = [s["ms"] for s in plain]
    # the FP32-Jacobi/FP64-refinement solver needs ~1e4 iterations (80+ s) on the Q2 system:
    # timed on Q1 workloads only
    mixed = [step(1) for _ in range(min(2, args.steps))] if order == 1 else []
    mixed_ms = [s["ms"] for s in mixed]

    # end to end through the reference-facing C ABI with host buffers
    x, y, z = (np.ascontiguousarray(pts[:, k]) for k in range(3))
    e2e_t = []
    for _ in range(min(3, args.steps)):
        t0 = time.perf_counter()
        if fem.run() != 0:
            raise RuntimeError(fg.last_error())
        rv, Ex, Ey, Ez, En, flag = fem.interpolate_elfield(x, y, z)
        e2e_t.append(time.perf_counter() - t0)
        if rv != 0:
            raise RuntimeError(fg.last_error())
    e2e_s = reduce_max(world, statistics.median(e2e_t))

    # surface (2-D) interpolation of the surface atoms (rank 1, LinearTriangles), points resident
    surf_reps = 5
    lib.fgb_field_interpolate_surface_device(field.h, n_surf, d_pts.ptr, 1, d_cells.ptr, d_out.ptr)
    field.mark(2)
    for _ in range(surf_reps):
        lib.fgb_field_interpolate_surface_device(field.h, n_surf, d_pts.ptr, 1, d_cells.ptr, d_out.ptr)
    field.mark(3)
    surf_ms = field.elapsed(2, 3) / surf_reps

    # roofline of the dominant kernel of the solve, timed live by event pairs around each of
    # its launches in the timed steps. Algorithmic bytes per launch:
    #   level-0 Chebyshev step (k_cheb_step): FP32 SELL matrix, 4 B value + 4 B column per
    #     nonzero, and 24 B per row (b, x gathered once, D^-1 read; d read + written; x written);
    #     Q2 element by element: the solver's own count (AmgDevice::smoother_bytes)
    #   outer SpMV (k_cg_spmv_pq_df, FP64-accurate from FP32 hi/lo pairs): 4 + 4 B value + 4 B
    #     column per nonzero, 24 B per row (p pair gathered once, p read, q written); Q2 over
    #     cell blocks: the solver's own count (FemDevice::outer_spmv_bytes)
    nnz = field.nnz
    ebe = order == 2 and last["smoother_bytes"] != nnz * 8 + 24 * n
    l0_name, l0_key = {
        0: ("k_cb_apply + k_cb_finish (level-0 Chebyshev smoothing, Q2 cell blocks, FP32 element matrices)",
            "smoother_ebe"),
        1: ("k_cb_apply + k_cb_finish (level-0 Chebyshev smoothing, Q2 cell blocks, matrix-free from FP32 "
            "geometric factors by sum factorisation)", "smoother_mf32"),
        2: ("k_cb_apply + k_cb_finish (level-0 Chebyshev smoothing, Q2 cell blocks, matrix-free from FP16 "
            "geometric factors by sum factorisation)", "smoother_mf16")}[l0_kind] if ebe else (
        "k_cheb_step (level-0 Chebyshev smoothing, FP32)", "smoother")
    kern = {
        l0_name: (
            sum(s["smoother_ms"] for s in solve_stats), sum(s["smoother_launches"] for s in solve_stats),
            last["smoother_bytes"], l0_key),
        ("k_cb_spmv_df + k_cb_spmv_finish (outer FP64-accurate SpMV + p.q, Q2 cell blocks, FP32 pairs)"
         if order == 2 else "k_cg_spmv_pq_df (outer FP64-accurate SpMV from FP32 pairs + p.q)"): (
            sum(s["spmv_ms"] for s in solve_stats), sum(s["spmv_launches"] for s in solve_stats),
            field.outer_spmv_bytes(), "spmv_cb" if order == 2 else "spmv_df"),
    }
    name, (tot_ms, cnt, bytes_per_launch, key) = max(kern.items(), key=lambda kv: kv[1][0])
    launch_ms = tot_ms / max(cnt, 1)
    peak, peak_kind = measured_hbm_peak()
    achieved = bytes_per_launch / (launch_ms * 1e-3) / 1e9
    traffic = KERNEL_TRAFFIC_PER_ROW[(key, order)] * n if (key, order) in KERNEL_TRAFFIC_PER_ROW else None
    spmv32_ms = field.time_spmv(1, 50)
    spmv64_ms = field.time_spmv(0, 20)

    line = {
        "metric": "solved DOF/s and p50/p99 solve latency at 1e-9 rel. residual vs plain FP64 CG",
        "value": value,
        "unit": "DOF/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 CG / f32 multigrid preconditioner",
        "data": "synthetic (seeded nanotip mesh, FCC surface atoms, random vacuum probes)",
        "config": workload_config(args.workload, spec, order, n, nnz, n_points, n_surf, world),
        "precision": "FP64 CG (true residual, search directions, dot products, boundary values and the solution "
                     "update in FP64) preconditioned by one FP32 multigrid V-cycle; the FP32-Jacobi / FP64-"
                     "refinement solver is timed on Q1 workloads (mixed_jacobi_cg)",
        "solve": {"p50_ms": statistics.median(solve_ms), "p99_ms": float(np.percentile(solve_ms, 99)),
                  "iterations": last["iterations"], "rel_residual": last["rel_residual"],
                  "solved_dof_per_s": n / (statistics.median(solve_ms) * 1e-3),
                  "multigrid_levels": levels, "multigrid_setup_ms": setup_ms},
        "plain_fp64_cg": {"p50_ms": statistics.median(plain_ms), "iterations": plain[-1]["iterations"],
                          "rel_residual": plain[-1]["rel_residual"],
                          "solved_dof_per_s": n / (statistics.median(plain_ms) * 1e-3),
                          "speedup_vs_plain": statistics.median(plain_ms) / statistics.median(solve_ms)},
        "mixed_jacobi_cg": ({"p50_ms": statistics.median(mixed_ms), "iterations": mixed[-1]["iterations"],
                             "refinements": mixed[-1]["outer"], "kernel_ms": mixed[-1]["kernel_ms"],
                             "rel_residual": mixed[-1]["rel_residual"]} if mixed else
                            "not timed on Q2 (~1e4 iterations, 83 s per solve on the 1.7e7-DoF nanotip)"),
        "e2e": {"value": n * world / e2e_s, "unit": "DOF/s", "h2d_bytes_per_step": 24 * n_points,
                "d2h_bytes_per_step": 36 * n_points,
                "note": "femocs_run + femocs_interpolate_elfield through the C ABI, host arrays"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "traffic_note": "ncu dram bytes per row of the Q2 probe capture x rows (Q2 only)",
                     "kernel": name, "bytes_per_launch": bytes_per_launch, "launch_ms": launch_ms,
                     "launches": cnt, "share_of_solve": tot_ms / sum(solve_ms),
                     "other": {k: {"ms": v[0], "launches": v[1], "gbs": v[2] / (v[0] / max(v[1], 1) * 1e-3) / 1e9}
                               for k, v in kern.items() if k != name},
                     "peak_kind": peak_kind, "spmv_fp32_launch_ms": spmv32_ms, "spmv_fp64_launch_ms": spmv64_ms,
                     "spmv_fp32_gbs": (nnz * 8 + 12 * n) / (spmv32_ms * 1e-3) / 1e9,
                     "element_matrix_smoother": (dict(ke_cmp, frac=ke_cmp["gbs"] / peak) if ke_cmp else None)},
        "clocks": clocks,
        "gpu_launches": launches,
        # index of the first timed launch among all of this process's kernel launches, and the
        # count (ncu -s/-c for a launch list of exactly the timed region)
        "timed_launch_range": [launches0, launches],
    }
    sysm = None
    if snap is not None:
        # parity of the timed step's results: the FP64 true residual recomputed by the oracle's
        # SpMV on the system the GPU solved, and location/interpolation against the oracle
        import oracle as orc
        t0 = time.perf_counter()
        rowptr, col, val, rhs, d2n = field.system()
        sysm = orc.System(csr=(rowptr, col, val, rhs))
        r_abs, floor_abs = sysm.residual(snap["x"])
        r_orc = r_abs / float(np.linalg.norm(rhs))
        del rowptr, col, val
        line["parity"] = {"rel_residual_oracle": r_orc, "rel_residual_gpu": last["rel_residual"],
                          "rel_floor": floor_abs / float(np.linalg.norm(rhs)),
                          "residual_note": "||b - A x|| / ||b|| of the last timed solve, recomputed by the "
                                           "oracle (compensated) on the exported system",
                          "export_and_spmv_s": time.perf_counter() - t0}
        line["parity"].update(interp_parity(fem, snap, pts, n_surf))
        if args.workload != "config1":
            line["parity"]["config1"] = config1_parity()
    if rank == 0 and world == 1 and not args.no_cpu and args.workload in ("config1", "config2"):
        try:
            line["cpu_baseline"] = cpu_baseline(field, args.workload, order, sysm=sysm)
        except RuntimeError as e:  # no full-solve iteration count recorded for this system
            line["cpu_baseline"] = {"unavailable": str(e)}
    del sysm, snap
    line["surface_interp"] = {"points": n_surf, "gpu_ms": surf_ms, "gpu_points_per_s": n_surf / (surf_ms * 1e-3),
                              "rank": 1, "note": "femocs_interpolate_surface_elfield path, device-resident points"}
    if rank == 0 and world == 1 and not args.no_cpu:
        line["mesh_prep"] = mesh_prep_timing(spec, order)
        line["surface_interp"].update(surface_cpu_timing(spec, pts[:n_surf]))
    if rank == 0 and world == 1 and args.workload == "config2" and not args.no_extra:
        del field, fem
        line.update(batch_and_serve_summaries(args, world, rank))
    if rank == 0:
        print(json.dumps(line), flush=True)


def host_cpu():
    """(logical cores, CPU model) of this host"""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return os.cpu_count() or 1, model or platform.processor() or platform.machine()


def ssor_iterations(workload, order, n_dofs):
    """SSOR(1.2)-CG iterations to 1e-9 of a full oracle solve of this workload's system
    (oracle/ssor_iterations.json, written by `python -m oracle.ssor_iterations`)"""
    from oracle.ssor_iterations import load_fixture
    rec = load_fixture().get(f"{workload}_q{order}")
    if not rec or rec["n_dofs"] != n_dofs:
        raise RuntimeError(f"no SSOR iteration count for {workload} Q{order} with {n_dofs} DoFs in "
                           "oracle/ssor_iterations.json: run python -m oracle.ssor_iterations")
    return rec


def reference_setup(args):
    """The reference's path on the CPU, built entirely by the oracle (no product library):
    the workload (oracle/workload.py, identical to the product's generator), the tet -> hex
    split and interpolator tables (oracle/mesh_prep.py), the FEM system of the workload's
    element order (Q1: oracle/femocs_oracle.c, Q2: oracle/q2_oracle.c) with its assembly
    timed, and one timed nodal-field recovery + smoothing."""
    import numpy as np
    import oracle as orc
    from oracle import mesh_prep, pipeline, workload
    spec = {"config1": workload.CONFIG1, "config2": workload.CONFIG2,
            "probe": dict(workload.CONFIG2, h=22.0, growth=1.3)}[args.workload]
    order = element_order(args)
    n_points = args.points or N_POINTS[args.workload]
    atoms, types = workload.atoms(spec, seed=12345)
    surf = atoms[types == 2]
    n_probe = max(0, n_points - len(surf))
    probes = workload.probes(spec, n_probe, seed=777) if n_probe else np.zeros((0, 3))
    pts = np.ascontiguousarray(np.r_[surf, probes][:n_points])
    om = mesh_prep.OracleMesh(*workload.tet_mesh(spec))
    t0 = time.perf_counter()
    if order == 2:
        cells = om.export("hex_nodes").reshape(-1, 8)[om.export("vac_cells")]
        sysm = orc.Q2CSystem(om.export("node_xyz"), cells, -E0)
    else:
        vx, vc, _ = pipeline.vacuum_inputs(om)
        sysm = orc.System(vx, vc, -E0)
    t_assembly = time.perf_counter() - t0
    n = om.sizes()
    phi = np.zeros(n["n_nodes"])
    n2v = om.export("vac_node2vertex")
    t0 = time.perf_counter()
    E = orc.nodal_field(om.export("node_xyz"), om.export("hex_nodes"), om.export("hex_marker"),
                        (n2v >= 0).astype(np.int8), phi)
    t_nodal = time.perf_counter() - t0
    t0 = time.perf_counter()
    orc.smooth_field(n["n_tetnodes"], om.export("node_xyz"), om.export("voro_ptr"), om.export("voro_idx"),
                     -1.0 / om.export("edgemax")[0], E)
    t_smooth = time.perf_counter() - t0
    tables = pipeline.tables(om, np.zeros((n["n_nodes"], 5)))
    return dict(spec=spec, order=order, pts=pts, n_surf=int(min(len(surf), n_points)), mesh=om, system=sysm,
                tables=tables, t_assembly=t_assembly, t_nodal=t_nodal, t_smooth=t_smooth)


def workload_config(workload, spec, order, n_dofs, nnz, n_points, n_surf, world):
    """The `config` object both arms print: the workload, not the implementation."""
    return {"workload": f"{workload}: nanotip R={spec['radius'] / 10:g} nm H={spec['height'] / 10:g} nm, "
                        f"box {2 * spec['box_half'] / 10:g} nm, top {spec['top'] / 10:g} nm, Q{order}",
            "elements": f"Q{order}", "n_dofs": int(n_dofs), "nnz": int(nnz), "n_points": int(n_points),
            "n_surface_atoms": int(n_surf), "interpolation_rank": RANK, "rel_tol": REL_TOL,
            "l2": "inputs larger than L2 (FP64 matrix %.0f MB)" % (nnz * 12 / 1e6),
            "parallelism": f"replicas x{world} (independent solves, no exchange)"}


def batch_and_serve_summaries(args, world, rank):
    """Compact results of the batched (256 meshes) and served (64 MD runs, Poisson arrivals)
    workloads for the default line; `--workload batch` / `--workload serve` give the full lines."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup, a.meshes, a.sample = 2, 1, 256, 8
    bl = run_batch(a, world, rank, quiet=True)
    sp = bl["sample_vs_plain_fp64_cg"]
    out = {"batch": {"workload": bl["config"]["workload"], "meshes": bl["config"]["n_meshes"],
                     "total_dofs": bl["config"]["total_dofs"], "dof_per_s": bl["value"],
                     "ms_per_step": bl["ms_per_step"], "solves_per_s": bl["batch"]["solves_per_s"],
                     "converged": bl["batch"]["converged"], "iterations_p50": bl["batch"]["iterations_p50"],
                     "kernels_per_iteration": bl["batch"]["kernels_per_iteration"], "build_s": bl["batch"]["build_s"],
                     "steps": a.steps, "clocks": bl["clocks"],
                     "sample_vs_plain_fp64_cg": {k: sp[k] for k in ("meshes", "dofs", "batched_ms", "plain_sequential_ms",
                                                                    "solves_per_s_batched", "solves_per_s_plain",
                                                                    "speedup")}}}
    a = copy.copy(args)
    a.rates, a.duration, a.runs = [50.0, 200.0, 1000.0], 2.0, 64
    sl = run_serve(a, world, rank, quiet=True)
    out["serve"] = {"workload": sl["config"]["workload"], "total_dofs": sl["config"]["total_dofs"],
                    "saturation_solves_per_s": sl["value"],
                    "rates": [{k: d[k] for k in ("rate", "requests", "completed", "converged", "solves_per_s", "p50_ms",
                                                 "p99_ms", "p50_queue_ms", "p50_solve_ms", "p50_post_ms", "p99_queue_ms",
                                                 "p99_solve_ms", "p99_post_ms", "iterations_mean")}
                              for d in sl["sweep"]],
                    "plain_fp64_cg_served_one_at_a_time": sl["plain_fp64_cg_served_one_at_a_time"],
                    "speedup_vs_plain": sl["speedup_vs_plain"], "iters_per_launch": a.iters_per_launch,
                    "idle_iters": a.idle_iters, "stop_at_first": bool(a.stop_at_first),
                    "build_s": sl["build_s"], "clocks": sl["clocks"]}
    return out


def run_reference(args, world, rank):
    """The reference's CPU path for the same workload, built and timed without the product's
    library: per step a bounded sample -- SSOR(1.2)-PCG iterations of deal.II's solver restated
    (src/DealSolver.cpp:443-459) on the full system, and the reference's sequential location +
    interpolation (src/SolutionReader.cpp:136-165) of a run of surface atoms and of a few
    random vacuum probes; the step's DOF/s is the workload's DoFs over the modelled full step:
    assembly (timed once) + per-iteration time x the iterations of a full oracle solve
    (oracle/ssor_iterations.json) + nodal field + smoothing (timed once) + per-point location
    times x the point counts."""
    if args.workload in ("batch", "serve"):
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference solves one mesh per process; "
                              "its CPU arm is timed on the single-mesh workloads (config1, config2)"}), flush=True)
        return
    if rank != 0:
        return
    import numpy as np
    import oracle as orc
    t_setup = time.perf_counter()
    R = reference_setup(args)
    sysm, pts, n_surf = R["system"], R["pts"], R["n_surf"]
    n_points = len(pts)
    n_dofs, nnz = int(sysm.n), int(len(sysm.col))
    rec = ssor_iterations(args.workload, R["order"], n_dofs)
    cores, model = host_cpu()
    t_setup = time.perf_counter() - t_setup
    # iterations per step: about a second of SSOR work
    t1 = sysm.ssor_cg_fixed(1) if n_dofs > 2e6 else sysm.ssor_cg_fixed(5) / 5
    k_it = max(1, int(1.0 / max(t1, 1e-6)))
    # the SpMV and vector operations may use every core (the SSOR sweeps stay sequential, as
    # deal.II's PreconditionSSOR): keep the faster of one thread and all threads
    t_all = sysm.ssor_cg_fixed(k_it, threads=cores) / k_it
    t_one = sysm.ssor_cg_fixed(k_it, threads=1) / k_it
    threads = cores if t_all < t_one else 1
    n_probe = n_points - n_surf
    rng = np.random.default_rng(3)
    surf_run, probe_run = min(2000, n_surf), min(30, n_probe)
    steps = []

    def one_step(k):
        t0 = time.perf_counter()
        t_it = sysm.ssor_cg_fixed(k_it, threads=threads) / k_it
        # a run of consecutive surface atoms (the chain finds them by neighbours) and random
        # vacuum probes (each a scan of the searchable tets in the reference's order)
        o = (k * surf_run) % max(1, n_surf - surf_run + 1)
        ti = time.perf_counter()
        orc.locate_interpolate(R["tables"], RANK, pts[o:o + surf_run])
        t_s = (time.perf_counter() - ti) / max(surf_run, 1)
        t_p = 0.0
        if probe_run:
            sel = n_surf + rng.choice(n_probe, size=probe_run, replace=False)
            ti = time.perf_counter()
            orc.locate_interpolate(R["tables"], RANK, pts[np.sort(sel)])
            t_p = (time.perf_counter() - ti) / probe_run
        wall = time.perf_counter() - t0
        full = (R["t_assembly"] + t_it * rec["iterations"] + R["t_nodal"] + R["t_smooth"] + t_s * n_surf + t_p * n_probe)
        return wall, full, t_it, t_s, t_p

    for k in range(args.warmup):
        one_step(k)
    for k in range(args.steps):
        steps.append(one_step(args.warmup + k))
    wall = statistics.median(s[0] for s in steps)
    full = statistics.median(s[1] for s in steps)
    t_it = statistics.median(s[2] for s in steps)
    t_s = statistics.median(s[3] for s in steps)
    t_p = statistics.median(s[4] for s in steps)
    v = n_dofs / full
    sample = (f"per step {k_it} SSOR(1.2)-PCG iteration(s) on the full {n_dofs}-DoF Q{R['order']} system "
              f"({threads} thread(s) for SpMV/vectors, sequential SSOR sweeps) and the sequential location + "
              f"interpolation of {surf_run} consecutive surface atoms and {probe_run} random vacuum probes; DOF/s from "
              f"the modelled full step: assembly {R['t_assembly']:.1f} s (timed once) + {t_it:.3f} s/iteration x "
              f"{rec['iterations']} iterations (full oracle solve to 1e-9) + nodal field and smoothing "
              f"{R['t_nodal'] + R['t_smooth']:.2f} s (timed once) + {t_s * 1e6:.1f} us x {n_surf} surface atoms + "
              f"{t_p * 1e3:.2f} ms x {n_probe} probes")
    line = {
        "metric": "solved DOF/s and p50/p99 solve latency at 1e-9 rel. residual vs plain FP64 CG",
        "value": v, "unit": "DOF/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded nanotip mesh, FCC surface atoms, random vacuum probes)",
        "impl": "reference",
        "config": workload_config(args.workload, R["spec"], R["order"], n_dofs, nnz, n_points, n_surf, world),
        "cpu_baseline": {"value": v, "unit": "DOF/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_model": {
            "step_s": full, "assembly_s": R["t_assembly"], "ssor_iterations": rec["iterations"],
            "s_per_iteration": t_it, "s_per_iteration_1_thread": t_one, "s_per_iteration_all_threads": t_all,
            "solve_s": t_it * rec["iterations"], "nodal_field_s": R["t_nodal"], "smoothing_s": R["t_smooth"],
            "locate_interpolate_s": t_s * n_surf + t_p * n_probe, "us_per_surface_atom": t_s * 1e6,
            "ms_per_probe": t_p * 1e3, "setup_s": t_setup,
            "measured": "assembly, nodal field, smoothing once; SSOR iterations and location per step",
            "extrapolated": "the solve (per-iteration time x iteration count of a full oracle solve) and the "
                            "location of all points (per-point times x point counts)",
            "iteration_count_source": rec["how"] + f"; {rec['host']}, true residual {rec['true_rel_residual']:.2e}"},
        "host": {"nproc": cores, "cpu_model": model},
    }
    print(json.dumps(line), flush=True)


def run_batch(args, world, rank, quiet=False):
    """256 independent nanotip meshes (tip radius 1-6 nm, aspect 2-8, field 0.5-3 GV/m, Q1
    meshes of 2e4-8e5 vacuum hexes, log-uniform) resident in one batch. One step = a cold
    (zero start) solve of every mesh to 1e-9, all meshes in one graph-captured WHILE loop.
    Plain FP64 Jacobi-CG single-mesh solves of a size-stratified sample give the baseline;
    the batch solves the same sample alone for the like-for-like ratio."""
    import numpy as np
    import femocs_gb300 as fg
    from femocs_gb300._lib import load

    n_mesh = args.meshes or 256
    specs, fields = fg.batch_specs(n_mesh, seed=2024)
    b = fg.Batch(persistent=args.persistent)
    t0 = time.perf_counter()
    slots = [int(v) for v in b.add_synthetic(specs)]
    build_s = time.perf_counter() - t0
    if min(slots) < 0:
        raise RuntimeError("device memory did not admit every mesh")
    dofs = np.array([b.info(s)["n_dofs"] for s in slots])
    total = int(dofs.sum())
    req = {s: float(e) for s, e in zip(slots, fields)}

    def step(sel):
        for s_ in sel:
            b.reset_solution(s_)
        return b.solve_all({s_: req[s_] for s_ in sel}, rel_tol=REL_TOL, max_iter=1000)

    for _ in range(args.warmup):
        step(slots)
    lib = load()
    sampler = ClockSampler()
    sampler.start()
    launches0 = lib.fgb_kernel_launches()
    b.mark(0)
    results = [step(slots) for _ in range(args.steps)]
    b.mark(1)
    dev_ms = reduce_max(world, b.elapsed(0, 1))
    launches = lib.fgb_kernel_launches() - launches0
    clocks = sampler.stop()
    res = results[-1]
    its = np.array([res[s_]["iterations"] for s_ in slots])
    conv = sum(res[s_]["status"] == 1 for s_ in slots)
    ms_per_step = dev_ms / args.steps

    # like-for-like: a size-stratified sample, plain FP64 Jacobi-CG one mesh at a time vs
    # the same sample solved as one batch
    order = np.argsort(dofs)
    sample = [slots[k] for k in order[np.linspace(0, n_mesh - 1, min(args.sample, n_mesh)).astype(int)]]
    b.mark(2)
    step(sample)
    b.mark(3)
    batch_sample_ms = b.elapsed(2, 3)
    plain_ms, plain_its = [], []
    for s_ in sample:
        m = fg.Mesh.synthetic(**specs[slots.index(s_)])
        f = fg.Field(m)
        f.setup(-req[s_])
        f.assemble(True, False)
        rc, st = f.solve(precision=0, rel_tol=REL_TOL, max_iter=100000)
        plain_ms.append(st["ms"])
        plain_its.append(st["iterations"])
        del f, m
    sample_dofs = int(sum(dofs[slots.index(s_)] for s_ in sample))
    line = {
        "metric": "solved DOF/s and p50/p99 solve latency at 1e-9 rel. residual vs plain FP64 CG",
        "value": world * total * args.steps / (dev_ms * 1e-3), "unit": "DOF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 CG / f32 multigrid preconditioner",
        "data": "synthetic (seeded random nanotips)",
        "config": {"workload": f"batch: {n_mesh} nanotips, radius 1-6 nm, aspect 2-8, field 0.5-3 GV/m, "
                               "Q1 2e4-8e5 vacuum hexes log-uniform, "
                               + ("one persistent cooperative kernel per step" if args.persistent
                                  else "one graph-captured launch per step"),
                   "n_meshes": n_mesh, "total_dofs": total, "rel_tol": REL_TOL,
                   "l2": "inputs larger than L2 (level-0 matrices %.1f GB)" % (total * 25 * 12 / 1e9)},
        "batch": {"solves_per_s": world * n_mesh * args.steps / (dev_ms * 1e-3), "converged": int(conv),
                  "iterations_p50": float(np.median(its)), "iterations_max": int(its.max()),
                  "dofs_min": int(dofs.min()), "dofs_max": int(dofs.max()), "build_s": build_s,
                  "device_bytes": b.stats()["device_bytes"], "tuning": b.tuning(),
                  "kernels_per_iteration": b.stats()["kernels_per_iteration"]},
        "sample_vs_plain_fp64_cg": {"meshes": len(sample), "dofs": sample_dofs,
                                    "batched_ms": batch_sample_ms, "plain_sequential_ms": float(sum(plain_ms)),
                                    "plain_iterations_p50": float(np.median(plain_its)),
                                    "solves_per_s_batched": len(sample) / (batch_sample_ms * 1e-3),
                                    "solves_per_s_plain": len(sample) / (sum(plain_ms) * 1e-3),
                                    "speedup": float(sum(plain_ms)) / batch_sample_ms},
        "clocks": clocks, "gpu_launches": launches,
    }
    if rank == 0 and not quiet:
        print(json.dumps(line), flush=True)
    return line


def serve_plain_baseline(specs, base, n_atoms, runs, steps=3, seed=5):
    """Like-for-like baseline of the serving loop: the same MD-step requests (atoms displaced by
    N(0, 0.02 A), applied field within 1 % of the run's base field, solve warm-started from the
    run's previous phi to 1e-9, nodal field + smoothing, location + interpolation at the run's
    atoms, results copied to the host) served one at a time with the plain FP64 Jacobi-PCG.
    Each run is first solved cold, as the serving loop's warm-up does."""
    import numpy as np
    import femocs_gb300 as fg
    rng = np.random.default_rng(17)
    times, iters = [], []
    for r in runs:
        spec = specs[r]
        m = fg.Mesh.synthetic(**spec)
        f = fg.Field(m)
        atoms, types = fg.synth_atoms(spec, seed=seed + 7919 * r)
        surf = atoms[types == 2]
        if len(surf) >= n_atoms:
            pts = surf[(np.arange(n_atoms) * len(surf)) // n_atoms]
        else:
            pts = np.r_[surf, fg.synth_probes(spec, n_atoms - len(surf), seed=seed + 104729 * r)]
        d_pts = fg.DeviceBuffer(24 * len(pts))
        d_cells = fg.DeviceBuffer(4 * len(pts))
        d_out = fg.DeviceBuffer(40 * len(pts))
        out = np.zeros((len(pts), 5))
        f.setup(base[r])
        f.assemble(True, False)
        f.solve(precision=0, rel_tol=REL_TOL, max_iter=100000)
        for _ in range(steps):
            pts = pts + rng.normal(0.0, 0.02, pts.shape)
            t0 = time.perf_counter()
            phi = f.phi_nodes()
            f.setup(base[r] * (1.0 + 0.01 * rng.standard_normal()))
            f.set_phi_nodes(phi)
            f.assemble(False, False)
            rc, st = f.solve(precision=0, rel_tol=REL_TOL, max_iter=100000)
            f.extract(True)
            d_pts.upload(np.ascontiguousarray(pts))
            f.interpolate_device(len(pts), d_pts.ptr, RANK, d_cells.ptr, d_out.ptr)
            d_out.download(out)
            times.append(time.perf_counter() - t0)
            iters.append(st["iterations"])
        del f, m
    return {"runs": [int(r) for r in runs], "requests": len(times), "p50_ms": float(np.median(times) * 1e3),
            "mean_ms": float(np.mean(times) * 1e3), "iterations_mean": float(np.mean(iters)),
            "solves_per_s": float(len(times) / np.sum(times)),
            "note": "the serving loop's request (atom step, warm start, nodal field, interpolation, host copy) "
                    "one at a time with plain FP64 Jacobi-PCG"}


def run_serve(args, world, rank, quiet=False):
    """64 concurrent MD runs (half the R = 2 nm, H = 8 nm tip, half random batch-style tips), ~5e4
    atoms each, resident; Poisson arrivals swept over rates; each request displaces its run's
    atoms by N(0, 0.02 A), re-solves warm-started with an applied field within 1% of the
    run's base field, recovers the nodal field and interpolates E and phi at the atoms, and
    copies the result to the host. Latency = submit to result on the host."""
    import numpy as np
    import femocs_gb300 as fg
    from femocs_gb300._lib import load

    n_runs = args.runs or 64
    rng = np.random.default_rng(99)
    half = n_runs // 2
    spec0 = dict(fg.CONFIG1)
    rspecs, rfields = fg.batch_specs(n_runs - half, seed=4242)
    specs = [spec0] * half + rspecs
    base = np.r_[np.full(half, 0.1), rfields]
    b = fg.Batch(persistent=args.persistent)
    srv = fg.Server(b, rel_tol=REL_TOL, max_iter=1000, iters_per_launch=args.iters_per_launch, rank=RANK)
    srv.set_launch_policy(args.idle_iters, args.stop_at_first)
    t0 = time.perf_counter()
    srv.add_synthetic_runs(specs, n_atoms=args.atoms, seed=5)
    build_s = time.perf_counter() - t0
    dofs = np.array([b.info(srv.run_info(r)["slot"])["n_dofs"] for r in range(n_runs)])
    srv.start()
    # warm-up: every run solved once (cold), so the sweep sees warm-started MD steps
    for r in range(n_runs):
        srv.submit(r, float(base[r]), 0.02)
    srv.drain(600)
    lib = load()
    sampler = ClockSampler()
    sampler.start()
    launches0 = lib.fgb_kernel_launches()
    sweep = []
    for rate in args.rates:
        srv.clear_records()
        n_req = int(max(20, rate * args.duration))
        t_start = time.perf_counter()
        srv.run_poisson(rate=rate, n=n_req, base_fields=base, sigma=0.02, seed=int(rate))
        wall = time.perf_counter() - t_start
        rec = srv.records()
        lat = (rec["t_done"] - rec["t_submit"]) * 1e3
        sweep.append({"rate": rate, "requests": n_req, "completed": int(len(lat)),
                      "converged": int((rec["status"] == 1).sum()),
                      "solves_per_s": len(lat) / (rec["t_done"].max() - rec["t_submit"].min()),
                      "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                      # where a request's time goes (medians): waiting for its run / the
                      # scheduler, solving in the batch, nodal field + interpolation + copy
                      "p50_queue_ms": float(np.median(rec["t_admit"] - rec["t_submit"]) * 1e3),
                      "p50_solve_ms": float(np.median(rec["t_solved"] - rec["t_admit"]) * 1e3),
                      "p50_post_ms": float(np.median(rec["t_done"] - rec["t_solved"]) * 1e3),
                      "p99_queue_ms": float(np.percentile(rec["t_admit"] - rec["t_submit"], 99) * 1e3),
                      "p99_solve_ms": float(np.percentile(rec["t_solved"] - rec["t_admit"], 99) * 1e3),
                      "p99_post_ms": float(np.percentile(rec["t_done"] - rec["t_solved"], 99) * 1e3),
                      "iterations_mean": float(rec["iterations"].mean()), "wall_s": wall})
    launches = lib.fgb_kernel_launches() - launches0
    clocks = sampler.stop()
    srv.stop()
    info = srv.info()
    # like-for-like: the same requests one at a time with the plain FP64 Jacobi-PCG, on runs of
    # both halves (R = 2 nm tips and random batch tips)
    sample_runs = sorted(set([0, 1, half, half + 1, n_runs - 1]))
    plain = serve_plain_baseline(specs, base, args.atoms, sample_runs)
    best = max(sweep, key=lambda d: d["solves_per_s"])
    line = {
        "metric": "solves/s and p50/p99 latency at 1e-9 rel. residual (serving, Poisson arrivals)",
        "value": best["solves_per_s"], "unit": "solves/s", "n_gpus": world, "steps": len(args.rates),
        "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 CG / f32 multigrid preconditioner", "data": "synthetic (seeded nanotips, FCC surface atoms)",
        "config": {"workload": f"serve: {n_runs} MD runs ({half} R=2 nm H=8 nm tips, {n_runs - half} random tips), "
                               f"{args.atoms} atoms each, sigma 0.02 A per step, Poisson arrivals",
                   "total_dofs": int(dofs.sum()), "rates": args.rates, "iters_per_launch": args.iters_per_launch,
                   "solver_launch": "persistent cooperative kernel" if args.persistent else "graph (WHILE node)",
                   "idle_iters": args.idle_iters, "stop_at_first": bool(args.stop_at_first)},
        "sweep": sweep, "build_s": build_s, "max_requests_in_flight": info["max_in_flight"],
        "solver_launches": info["solver_launches"], "plain_fp64_cg_served_one_at_a_time": plain,
        "speedup_vs_plain": best["solves_per_s"] / plain["solves_per_s"],
        "clocks": clocks, "gpu_launches": launches,
    }
    if rank == 0 and not quiet:
        print(json.dumps(line), flush=True)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=["config2", "config1", "probe", "batch", "serve"])
    ap.add_argument("--meshes", type=int, default=0, help="batch: number of meshes (default 256)")
    ap.add_argument("--sample", type=int, default=16, help="batch: meshes solved by plain CG for the ratio")
    ap.add_argument("--runs", type=int, default=0, help="serve: MD runs (default 64)")
    ap.add_argument("--atoms", type=int, default=50000, help="serve: atoms per run")
    ap.add_argument("--rates", type=float, nargs="+", default=[50, 200, 500, 1000, 2000])
    ap.add_argument("--duration", type=float, default=2.0, help="serve: seconds of arrivals per rate")
    ap.add_argument("--iters-per-launch", type=int, default=4)
    ap.add_argument("--idle-iters", type=int, default=0,
                    help="serve: solver iterations per launch while no request waits (0: --iters-per-launch)")
    ap.add_argument("--persistent", action="store_true",
                    help="batch/serve: one persistent cooperative kernel per solver step instead of the graph")
    ap.add_argument("--stop-at-first", action="store_true",
                    help="serve: end a launch after the iteration in which a solve finished")
    ap.add_argument("--points", type=int, default=0)
    ap.add_argument("--order", type=int, default=0, choices=[0, 1, 2],
                    help="element order (default: 2 for config2/probe, 1 for config1)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity checks against the oracle")
    ap.add_argument("--no-extra", action="store_true", help="config2: skip the batch and serving summaries")
    args = ap.parse_args()
    world, rank, _ = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        from femocs_gb300.build import build
        build()
        if args.workload == "batch":
            run_batch(args, world, rank)
        elif args.workload == "serve":
            run_serve(args, world, rank)
        else:
            run_ours(args, world, rank)


if __name__ == "__main__":
    main()
