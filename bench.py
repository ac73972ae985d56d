#!/usr/bin/env python
"""Benchmark: mixed Darcy RT1 x P0 assembly on 64^3 x 6 tetrahedra (4.74 M DoF).

One step = one assembly pass of the whole mesh: element integrals of every
cell, scattered into the CSR matrix (nnz 36,200,448) and the residual.  The
headline is FP64 values (the reference's precision, within 1e-12 of the FP64
oracle at this size; element arithmetic in double-float on the FP32 pipes),
with the FP32 assembly (the inner solver's matrix, within 1e-5) timed beside
it in `precision_legs`.  Inputs are resident in
HBM; the L2 is flushed (256 MB write) before every timed step and each step
is timed with CUDA events on the launching stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm on the host cores: the
oracle's per-cell loop (the reference's own structure: per-cell mapping,
tabulation, Piola, orientation, element matrix, entry-by-entry scatter),
parallel over all host cores, on a bounded sample of cells per step; DoF/s
is extrapolated to the full mesh.  Under torchrun, N ranks run independent
replicas (the path is one problem on one GPU; "replicas only").
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "DoF/s assembled (3D mixed Darcy RT1xP0, 64^3x6 tets, lognormal K)"
UNIT = "DoF/s"
N_SIDE = 64


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest per-rank value (the job's step time); every rank gets it.
    One rank, or no process group, returns the value itself."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms):
    """Whole-job throughput: every rank processes its own units (replicas,
    weak scaling) in at most `ms` milliseconds."""
    return world * units_per_rank / (ms * 1e-3)


# ------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        import statistics
        sm = [r[0] for r in rows]
        mx = max(r[1] for r in rows)
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[2]) if v.lower().startswith("active")})
        top = sorted(sm)[len(sm) // 2:]
        return {"sm_mhz": statistics.median(top), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def measured_bf16_peak():
    """Dense bf16 TFLOP/s of the GB300s (burst), else the fallback."""
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def profiled_traffic(name):
    """Per-launch DRAM bytes of the timed kernel from the committed ncu summary."""
    path = os.path.join(HERE, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        pass
    return None


def algorithmic_bytes(T, V, nnz, n_dof, vbytes, verts_per_cell=4):
    """Compulsory bytes of one assembly with `vbytes`-wide values: cell->vertex
    ids (4 B per vertex of a cell), point coordinates (24 B/point), kappa and
    f (one value per cell), RT1 orientation mask (1 B/cell), CSR values
    written once, the residual written once.  The CSR index structures are
    setup data and are not counted (they are counted in the measured DRAM
    traffic)."""
    return T * 4 * verts_per_cell + V * 24 + 2 * T * vbytes + T + nnz * vbytes + n_dof * vbytes


# ------------------------------------------------------------------ CPU (oracle) path
def _cpu_worker(args):
    """Per-cell loop of the reference's structure over a chunk of cells."""
    import numpy as np
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import forms, quadrature
    X, signs, kappa, f, dest = args
    quad = quadrature.make_quadrature(3, 3)
    rows, cols, vals = [], [], []
    rhs = {}
    t0 = time.perf_counter()
    for c in range(X.shape[0]):
        r_el, j_el = forms.darcy_element(X[c], signs[c], 3, quad, float(kappa[c]), float(f[c]))
        d = dest[c]
        n = len(d)
        rows.append(np.repeat(d, n))
        cols.append(np.tile(d, n))
        vals.append(j_el.ravel())
        for k, g in enumerate(d):
            rhs[int(g)] = rhs.get(int(g), 0.0) + r_el[k]
    import scipy.sparse as sp
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols)))).tocsr()
    return time.perf_counter() - t0, A.nnz


_CPU_MESH = {}


def cpu_problem(n_side, sample):
    import numpy as np
    from oracle import mesh_gen, topology
    from nfempy_gb300.workloads import darcy3d_coefficients
    if n_side not in _CPU_MESH:  # the oracle's numbering of the mesh, built once
        m = mesh_gen.cube(n_side)
        topo = topology.Topology(m)
        cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "RT", 1),
                                           topology.FieldSpec("p", "P", 0, 1, True)])
        _CPU_MESH[n_side] = (m, topo, cd, nd, darcy3d_coefficients(m))
    m, topo, cd, nd, (kappa, f) = _CPU_MESH[n_side]
    idx = np.linspace(0, topo.n_cells - 1, sample).astype(np.int64)
    X = m["points"][topo.cells[idx]]
    return dict(X=X, signs=topo.rt1_signs()[idx], kappa=kappa[idx], f=f[idx], dest=cd[idx], T=topo.n_cells, n_dof=nd)


def cpu_rate(prob, workers, pool=None):
    """(DoF/s extrapolated, seconds) for one pass over the sample."""
    import numpy as np
    S = prob["X"].shape[0]
    chunks = np.array_split(np.arange(S), workers)
    jobs = [(prob["X"][c], prob["signs"][c], prob["kappa"][c], prob["f"][c], prob["dest"][c]) for c in chunks]
    t0 = time.perf_counter()
    if pool is None:
        for j in jobs:
            _cpu_worker(j)
    else:
        list(pool.map(_cpu_worker, jobs))
    dt = time.perf_counter() - t0
    t_full = dt * prob["T"] / S
    return prob["n_dof"] / t_full, dt


def _cpu_vec_worker(job):
    """Vectorised numpy assembly of a chunk of cells: element matrices of all
    cells at once (oracle.forms.darcy_batch) scattered into a CSR matrix."""
    import numpy as np
    from oracle import assembly, forms, quadrature
    X, signs, kappa, f, dest, n_dof = job
    quad = quadrature.make_quadrature(3, 3)
    Q = len(quad[1])
    t0 = time.perf_counter()
    r, j = forms.darcy_batch(X, signs, 3, quad, np.repeat(kappa[:, None], Q, 1), np.repeat(f[:, None], Q, 1))
    assembly.assemble_csr(dest, j, r, n_dof)
    return time.perf_counter() - t0


def cpu_vectorised(n_side, sample, workers):
    """Vectorised numpy assembly (oracle.forms.darcy_batch + a COO -> CSR
    scatter) over `sample` evenly spaced cells, split over `workers` spawn
    processes; DoF/s extrapolated linearly to the full mesh."""
    import multiprocessing as mp
    import numpy as np
    prob = cpu_problem(n_side, sample)
    chunks = np.array_split(np.arange(prob["X"].shape[0]), workers)
    jobs = [(prob["X"][c], prob["signs"][c], prob["kappa"][c], prob["f"][c], prob["dest"][c], prob["n_dof"])
            for c in chunks]
    with mp.get_context("spawn").Pool(workers) as pool:
        pool.map(_cpu_vec_worker, jobs[:workers])  # warm the workers (imports)
        t0 = time.perf_counter()
        pool.map(_cpu_vec_worker, jobs)
        wall = time.perf_counter() - t0
    rate = prob["n_dof"] / (wall * prob["T"] / prob["X"].shape[0])
    return {"value": rate, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": (f"vectorised numpy (oracle.forms.darcy_batch + COO -> CSR scatter) over {prob['X'].shape[0]} "
                       f"of {prob['T']} cells in {workers} spawn workers, {wall:.2f} s; DoF/s extrapolated")}


def cpu_solve_baselines(n_side=16):
    """Host solves (scipy, FP64): SuperLU on the 2-D 32x32 manufactured Darcy
    problem, and GMRES(50) with the cell-block Jacobi preconditioner (the plain
    method) to 1e-8 on 3-D mixed Darcy at n_side^3 x 6 with the bench's field
    statistics.  Returns the record and the 3-D system for the GPU to solve."""
    import numpy as np
    import scipy.sparse.linalg as spla
    from nfempy_gb300 import meshes
    from oracle import assembly, forms, mesh_gen, quadrature, solve, topology
    out = {}
    m = mesh_gen.square(32)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "RT", 1), topology.FieldSpec("p", "P", 0, 1, True)])
    X = m["points"][topo.cells]
    quad = quadrature.make_quadrature(2, 3)
    from oracle.elements import create_element
    lam = create_element("P", 2, 1).tabulate(0, quad[0])[0, :, :, 0]
    xq = np.einsum("qv,tvg->tqg", lam, X)
    fq = 2 * np.pi ** 2 * np.sin(np.pi * xq[..., 0]) * np.sin(np.pi * xq[..., 1])
    r, j = forms.darcy_batch(X, topo.rt1_signs(), 2, quad, np.ones_like(fq), fq)
    A, res = assembly.assemble_csr(cd, j, r, nd)
    t0 = time.perf_counter()
    x = spla.spsolve(A.tocsc(), -res)
    out["superlu_darcy2d_32x32"] = {"n_dof": nd, "seconds": time.perf_counter() - t0,
                                    "relres": solve.relative_residual(A, x, -res)}
    m = mesh_gen.cube(n_side)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "RT", 1), topology.FieldSpec("p", "P", 0, 1, True)])
    X = m["points"][topo.cells]
    quad = quadrature.make_quadrature(3, 3)
    kappa = np.exp(meshes.grf_log_field(X.mean(axis=1), 0.05, 2.0, 20261208, device="cpu"))
    T = topo.n_cells
    r, j = forms.darcy_batch(X, topo.rt1_signs(), 3, quad, np.repeat(kappa[:, None], 8, 1), np.ones((T, 8)))
    A, res = assembly.assemble_csr(cd, j, r, nd)
    t0 = time.perf_counter()
    x, its, rel = solve.gmres_block_jacobi(A, -res, cd, rtol=1e-8, restart=50)
    out[f"gmres_block_jacobi_darcy3d_{n_side}x6"] = {"n_dof": nd, "seconds": time.perf_counter() - t0,
                                                     "iterations": its, "relres": rel, "restart": 50}
    out["cores"] = "scipy (SuperLU and the GMRES loop single-threaded; numpy kernels may use BLAS threads)"
    return out, (kappa, n_side)


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    per_core = 600
    prob = cpu_problem(N_SIDE, per_core * cores)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            cpu_rate(prob, cores, pool)
        rates, secs = [], []
        for _ in range(args.steps):
            r, s = cpu_rate(prob, cores, pool)
            rates.append(r)
            secs.append(s)
    import statistics
    value = statistics.median(rates)
    sample = (f"oracle per-cell loop (reference structure) over {prob['X'].shape[0]} of {prob['T']} cells per step, "
              f"{cores} spawn workers; DoF/s extrapolated linearly to the full mesh")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * prob["n_dof"] / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": f"darcy3d_rt1p0_cube{N_SIDE}x6", "n_cells": prob["T"],
                                            "n_dof": prob["n_dof"], "extrapolated": True},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)



def _timed_solve(ksp, b, args, stream, two_level=False):
    """Setup + solve to 1e-8 (FP64 residual); the FP32 inner solves stop at
    the preconditioner's inner tolerance (--inner-rtol / --tl-inner-rtol)."""
    import torch
    from nfempy_gb300.solvers import INNER_RTOL
    inner_rtol = args.tl_inner_rtol if two_level else args.inner_rtol
    ev0, ev1, ev2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    ev0.record(stream)
    ksp.setup()
    ev1.record(stream)
    x, info = ksp.solve(b, rtol=1e-8, inner_rtol=inner_rtol, max_inner=args.max_iters, raise_on_failure=False)
    ksp.last_x = x
    ev2.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    relres = float(ksp.residual(x, b).norm() / b.norm())
    return {"setup_ms": ev0.elapsed_time(ev1), "solve_ms": ev1.elapsed_time(ev2),
            "time_to_solve_ms": ev0.elapsed_time(ev2), "wall_s": wall,
            "inner_iterations": info.inner_iterations, "outer_iterations": info.outer_iterations,
            "final_relres_fp64": relres, "status": info.status,
            "ms_per_inner_iteration": ev1.elapsed_time(ev2) / max(1, info.inner_iterations),
            "restart": ksp.restart, "inner_rtol": inner_rtol if inner_rtol is not None else INNER_RTOL[ksp.pc_kind]}


def solve_bench(args, A, wf, coefs, res, stream):
    """Time to ||b - A x|| / ||b|| <= 1e-8 (FP64) on the benchmark system:
    plain block-Jacobi FGMRES, the two-level preconditioner with classical
    flux weights, and with the network's weights (the learned preconditioner)."""
    import torch
    from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
    A64 = A.with_dtype(torch.float64)
    res64 = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
    wf.assemble(A64, res64, coefficients=wf.coefficients(torch.float64))
    # the FP32 operator of the inner iterations, assembled in FP32
    A = A.with_dtype(torch.float32)
    res32 = torch.empty(A.n_rows, dtype=torch.float32, device="cuda")
    wf.assemble(A, res32, coefficients=wf.coefficients(torch.float32))
    b = -res64
    out = {"rtol": 1e-8, "krylov": (f"FGMRES FP32 inside FP64 iterative refinement; restart {args.restart} "
                                    f"(plain), {args.tl_restart} (two-level)"),
           "field": "log K GRF, correlation length 0.05, sigma 2.0, seed 20261208 (not a training seed)"}
    ksp = KrylovSolver(A64, pc="cell_block", A32_values=A.values, restart=args.restart)
    out["plain_block_jacobi"] = _timed_solve(ksp, b, args, stream)
    nc = N_SIDE // 4
    # the structure is built on the device from the mesh; the first build of
    # a process also pays the one-time loading of the torch kernels it uses
    # (sort, bincount, nonzero, ...), timed apart
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tl = TwoLevelCoarse(A64, nc)
    torch.cuda.synchronize()
    t_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    tl = TwoLevelCoarse(A64, nc)
    torch.cuda.synchronize()
    t_struct = time.perf_counter() - t0
    ksp = KrylovSolver(A64, pc="two_level", A32_values=A.values, restart=args.tl_restart, two_level=tl)
    out["two_level_classical"] = _timed_solve(ksp, b, args, stream, two_level=True)
    out["two_level_classical"]["host_structure_s"] = t_struct
    out["two_level_classical"]["host_structure_first_call_s"] = t_first
    out["two_level_classical"]["aggregates"] = tl.n_agg
    out["two_level_classical"]["cycle"] = "symmetric (pre- and post-smoothing), omega 0.9"
    try:
        from nfempy_gb300 import learned, train_learned
        model, ck = train_learned.load()
        alpha = ck["alphas_by_side_fraction"][4]["alpha"]
        kappa = wf.functions["kappa"]
        tl2 = TwoLevelCoarse(A64, nc)
        tl2.set_weights(learned.learned_weights(tl2, model, kappa, alpha))
        try:
            inference = mlp_inference_timing(model, learned.FaceData(tl2).features(kappa))
        except Exception as e:  # the timing is a report, not part of the solve
            inference = {"error": f"{type(e).__name__}: {e}"}
        ksp = KrylovSolver(A64, pc="two_level", A32_values=A.values, restart=args.tl_restart, two_level=tl2)
        out["learned"] = _timed_solve(ksp, b, args, stream, two_level=True)
        out["learned"]["alpha"] = alpha
        out["learned"]["network_inference"] = inference
        out["learned"]["training"] = {k: ck["record"][k] for k in ("n", "fields", "solves_used", "pairs",
                                                                   "data_seconds", "train_seconds")}
        plain = out["plain_block_jacobi"]["time_to_solve_ms"]
        out["learned"]["network_active"] = bool(alpha > 0)
        out["learned"]["speedup_vs_classical_two_level"] = (out["two_level_classical"]["time_to_solve_ms"]
                                                            / out["learned"]["time_to_solve_ms"])
        if alpha > 0:
            out["learned"]["speedup_vs_plain"] = plain / out["learned"]["time_to_solve_ms"]
        else:
            out["learned"]["note"] = ("alpha = 0 on validation: the network's correction is switched off and this "
                                      "arm equals the classical two-level preconditioner")
    except (OSError, FileNotFoundError, KeyError) as e:
        out["learned"] = {"unavailable": f"no trained network checkpoint ({type(e).__name__})"}
    tl = out["two_level_classical"]
    tl["speedup_vs_plain"] = out["plain_block_jacobi"]["time_to_solve_ms"] / tl["time_to_solve_ms"]
    tl["time_to_solve_incl_host_structure_ms"] = tl["time_to_solve_ms"] + 1e3 * tl["host_structure_s"]
    tl["speedup_vs_plain_incl_host_structure"] = (out["plain_block_jacobi"]["time_to_solve_ms"]
                                                  / tl["time_to_solve_incl_host_structure_ms"])
    return out


def mlp_inference_timing(model, x, reps=20, warmup=3):
    """The network's inference over the faces of the benchmark mesh: the
    fused tcgen05 kernel against the tiled CUDA-core GEMMs (same BF16
    weights), CUDA events on the current stream, inputs resident."""
    import torch
    rows = int(x.shape[0])
    flops_row = 2 * (int(model.dims[0]) * int(model.dims[1]) + int(model.dims[1]) * int(model.dims[2])
                     + int(model.dims[2]) * int(model.dims[3]))
    out = {"rows": rows, "flops_per_row": flops_row,
           "network": "x[8] -> 256 -> 256 -> 1, BF16 weights, FP32 accumulation"}

    def timeit(fn):
        for _ in range(warmup):
            fn()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s.record()
        for _ in range(reps):
            fn()
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / reps
    if model.tensor_core_shape():
        y_tc = model.infer_tc(x)
        ms = timeit(lambda: model.infer_tc(x))
        pk, kind = measured_bf16_peak()
        ach = rows * flops_row / (ms * 1e-3) / 1e12
        out["tensor_core"] = {"kernel": "mlp_infer_tc_kernel (tcgen05.mma kind::f16, M128 N256 K16, TMEM accumulators)",
                              "ms": ms, "tflops": ach, "bf16_peak_tflops": pk, "peak_source": kind,
                              "frac_of_bf16_peak": ach / pk}
    chunk = 1 << 16

    def cuda_core():
        for s0 in range(0, rows, chunk):
            model.forward(x[s0:s0 + chunk])
    ms_cc = timeit(cuda_core)
    out["cuda_core"] = {"kernel": "gemm_kernel x3 (64x64 tiles, FP32 FMA)", "ms": ms_cc,
                        "tflops": rows * flops_row / (ms_cc * 1e-3) / 1e12}
    if "tensor_core" in out:
        y_cc = torch.cat([model.forward(x[s0:s0 + chunk])[2] for s0 in range(0, rows, chunk)])
        out["tensor_core"]["speedup_vs_cuda_core"] = ms_cc / out["tensor_core"]["ms"]
        out["tensor_core"]["max_abs_diff_vs_cuda_core"] = float((y_tc - y_cc).abs().max().item())
        out["tensor_core"]["max_abs_output"] = float(y_cc.abs().max().item())
    return out


def mlp_only(args):
    """The learned network's inference alone on --mlp-rows synthetic feature
    rows (seeded normal features, the shipped checkpoint's weights, or a
    seeded network of the same shape when no checkpoint is present)."""
    import torch
    from nfempy_gb300 import learned
    try:
        from nfempy_gb300 import train_learned
        model, _ = train_learned.load()
        src = "checkpoint"
    except (OSError, FileNotFoundError, KeyError):
        model = learned.MLP(learned.N_FEAT, width=256, n_out=1, seed=0)
        src = "seeded"
    g = torch.Generator(device="cuda").manual_seed(20261204)
    x = torch.randn((args.mlp_rows, int(model.dims[0])), device="cuda", generator=g)
    out = mlp_inference_timing(model, x, reps=args.steps, warmup=args.warmup)
    out["weights"] = src
    return out


def small_system_gpu(args, kappa, n_side):
    """GPU time to 1e-8 on the host baseline's 16^3 x 6 Darcy system: plain
    block-Jacobi FGMRES and the two-level preconditioner (setup included;
    the two-level host structure reported apart)."""
    import torch
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
    from nfempy_gb300 import meshes
    sp = wl.darcy_space(meshes.cube(n_side))
    A32 = nf.CSRMatrix(sp, dtype=torch.float32)
    A64 = A32.with_dtype(torch.float64)
    r32 = torch.empty(A32.n_rows, dtype=torch.float32, device="cuda")
    r64 = torch.empty(A32.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": 1.0}
    wf.assemble(A32, r32)
    wf.assemble(A64, r64)
    b = -r64
    stream = torch.cuda.current_stream()
    out = {"n_dof": sp.n_dof}
    out["plain_block_jacobi"] = _timed_solve(KrylovSolver(A64, pc="cell_block", A32_values=A32.values,
                                                          restart=args.restart), b, args, stream)
    t0 = time.perf_counter()
    tl = TwoLevelCoarse(A64, max(2, n_side // 4))
    t_struct = time.perf_counter() - t0
    out["two_level"] = _timed_solve(KrylovSolver(A64, pc="two_level", A32_values=A32.values,
                                                 restart=args.tl_restart, two_level=tl), b, args, stream,
                                    two_level=True)
    out["two_level"]["host_structure_s"] = t_struct
    return out


def assembly_only(args):
    """The headline assembly alone (64^3 x 6 tets, --precision, --kernel),
    timed like the main run: the profiling runs capture it."""
    import torch
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    dtype = torch.float32 if args.precision == "f32" else torch.float64
    m, sp, kappa, f = wl.darcy3d(N_SIDE)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.use_chunks = args.kernel == "chunks"
    wf.use_records = args.kernel == "records"
    wf.use_slices = args.slices
    wf.use_streams = args.streams
    wf.use_fused = args.fused
    if args.slice_shift:
        wf.min_slice_shift = args.slice_shift
    if args.record_quarters:
        wf.record_quarters = args.record_quarters
    wf.functions = {"kappa": kappa, "rhs": f}
    coefs = wf.coefficients(dtype)
    ms = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    A.check_status("assembly")
    vb = 4 if dtype == torch.float32 else 8
    alg = algorithmic_bytes(sp.n_cells, m["points"].shape[0], A.nnz, sp.n_dof, vb)
    peak, kind = measured_peaks()
    ach = alg / (ms * 1e-3) / 1e9
    out = {"precision": args.precision, "kernel": args.kernel, "ms_per_step": ms, "value": sp.n_dof / (ms * 1e-3),
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "frac": ach / peak, "algorithmic_bytes": alg,
                        "peak_source": kind}}
    if dtype == torch.float64 and args.kernel == "records":
        from nfempy_gb300 import autotune
        autotune.set_knobs({"darcy_f64_records": 1})  # double-float records for every cell
        try:
            out["double_float_records_ms"] = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs),
                                                            args.steps, args.warmup)
        finally:
            autotune.set_knobs({"darcy_f64_records": 0})
        A.check_status("assembly, double-float records")
    return out


def solve_only(args):
    """The benchmark system's solves alone (profiling runs): plain block-Jacobi
    and two-level FGMRES on 64^3 x 6 tets, to 1e-8 or --max-iters inner
    iterations."""
    import torch
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
    m, sp, kappa, f = wl.darcy3d(N_SIDE)
    A32 = nf.CSRMatrix(sp, dtype=torch.float32)
    A64 = A32.with_dtype(torch.float64)
    r32 = torch.empty(A32.n_rows, dtype=torch.float32, device="cuda")
    r64 = torch.empty(A32.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": f}
    wf.assemble(A32, r32)
    wf.assemble(A64, r64)
    b = -r64
    stream = torch.cuda.current_stream()
    out = {"workload": "solve", "n_dof": sp.n_dof, "restart": args.restart, "max_inner": args.max_iters}
    if args.solver in ("both", "plain"):
        out["plain_block_jacobi"] = _timed_solve(KrylovSolver(A64, pc="cell_block", A32_values=A32.values,
                                                              restart=args.restart), b, args, stream)
    if args.solver in ("both", "two_level"):
        tl = TwoLevelCoarse(A64, N_SIDE // 4)
        out["two_level"] = _timed_solve(KrylovSolver(A64, pc="two_level", A32_values=A32.values,
                                                     restart=args.tl_restart, two_level=tl), b, args, stream,
                                        two_level=True)
    return out


def _time_assembly(fn, steps, warmup):
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        flush.zero_()
        fn()
    ts = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        ts.append((e0, e1))
    torch.cuda.synchronize()
    import statistics
    return statistics.mean(a.elapsed_time(b) for a, b in ts)


def elasticity_bench(args):
    """Vector P2 elasticity assembly: 40^3 x 6 tets, per-cell lognormal
    lambda, mu (mean-log 0, sigma 0.5), body force (1, 1, 1), FP32."""
    import torch
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    from nfempy_gb300.assembly import LEPrimalWeakForm
    m, sp, functions = wl.elasticity3d(40)
    A = nf.CSRMatrix(sp, dtype=torch.float32)
    res = torch.empty(A.n_rows, dtype=torch.float32, device="cuda")
    T = sp.n_cells
    wf = LEPrimalWeakForm(sp)
    wf.functions = functions
    coefs = wf.coefficients(torch.float32)
    ms = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    A.check_status("elasticity bench")
    from nfempy_gb300 import autotune
    best, best_ms, tried = autotune.tune(f"elasticity_p2_f32_cells{sp.n_cells}",
                                         lambda: wf.assemble(A, res, coefficients=coefs),
                                         autotune.elasticity_candidates(), reps=max(3, args.steps // 4))
    tuned_ms = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    A.check_status("elasticity tuned")
    autotune.reset_knobs()
    V = m["points"].shape[0]
    alg = T * 16 + V * 24 + T * 4 * 2 + T * 12 + A.nnz * 4 + A.n_rows * 4
    peak, kind = measured_peaks()
    ach = alg / (ms * 1e-3) / 1e9
    out = {"metric": "DoF/s assembled", "value": sp.n_dof / (ms * 1e-3), "ms_per_step": ms, "dtype": "f32",
           "n_cells": T, "n_dof": sp.n_dof, "nnz": A.nnz, "kernel": "elasticity_rows_kernel",
           "autotuned": {"config": best, "ms_per_step": tuned_ms, "candidates": len(tried)},
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "algorithmic_bytes": alg, "peak_source": kind,
                        "traffic": profiled_traffic("elasticity_rows_f32_cube40.txt")}}
    if not args.no_solve:
        # the driver's step: FP64 system, boundary clamped by the beta = 1e12
        # penalty, solved to 1e-8 (point-Jacobi FGMRES, FP32 inner iterations)
        from nfempy_gb300.assembly import LEPrimalWeakFormBCDirichlet
        from nfempy_gb300.solvers import KrylovSolver
        A64 = A.with_dtype(torch.float64)
        r64 = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
        wf.assemble(A64, r64, coefficients=wf.coefficients(torch.float64))
        bc = LEPrimalWeakFormBCDirichlet(sp)
        bc.functions = {"u": None}
        bc.assemble(A64)
        A32v = A64.values.to(torch.float32)
        ksp = KrylovSolver(A64, pc="jacobi", A32_values=A32v, restart=args.restart)
        out["solve"] = _timed_solve(ksp, -r64, args, torch.cuda.current_stream())
        out["solve"]["preconditioner"] = "point Jacobi"
        # the cell cliques' 30 x 30 blocks (weighted additive Schwarz)
        ksp = KrylovSolver(A64, pc="cell_block", A32_values=A32v, restart=args.restart)
        out["solve_cell_block"] = _timed_solve(ksp, -r64, args, torch.cuda.current_stream())
        out["solve_cell_block"]["preconditioner"] = "cell-block Jacobi (30 x 30 cell blocks)"
        out["solve_cell_block"]["speedup_vs_point_jacobi"] = (out["solve"]["time_to_solve_ms"]
                                                              / out["solve_cell_block"]["time_to_solve_ms"])
        # the driver's own solver family: CG (ICC replaced by 3 x 3 node blocks)
        from nfempy_gb300.solvers import CGSolver
        for pc in ("node_block", "jacobi"):
            cg = CGSolver(A64, pc=pc, A32_values=A32v)
            torch.cuda.synchronize()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            cg.setup()
            e1.record()
            xcg, info = cg.solve(-r64, rtol=1e-8, raise_on_failure=False)
            e2.record()
            torch.cuda.synchronize()
            rel = float(cg.residual(xcg, -r64).norm() / r64.norm())
            out[f"solve_cg_{pc}"] = {"setup_ms": e0.elapsed_time(e1), "solve_ms": e1.elapsed_time(e2),
                                     "time_to_solve_ms": e0.elapsed_time(e2), "inner_iterations": info.inner_iterations,
                                     "outer_iterations": info.outer_iterations, "final_relres_fp64": rel,
                                     "status": info.status,
                                     "ms_per_inner_iteration": e1.elapsed_time(e2) / max(1, info.inner_iterations),
                                     "preconditioner": ("3 x 3 node-block Jacobi" if pc == "node_block"
                                                        else "point Jacobi"),
                                     "speedup_vs_fgmres_point_jacobi": out["solve"]["time_to_solve_ms"]
                                     / e0.elapsed_time(e2)}
    return out


def cosserat_bench(args):
    """Mixed Cosserat assembly: 24^3 x 6 tets, RT1^3 x RT1^3 x P0^3 x P0^3,
    Lame 1/1, Cosserat coupling 0.5, the manufactured solution's load and the
    material as callables (sampled once), FP32."""
    import torch
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    from nfempy_gb300.assembly import LCEDualWeakForm
    m, sp, functions, exact = wl.cosserat3d(24)
    A = nf.CSRMatrix(sp, dtype=torch.float32)
    res = torch.empty(A.n_rows, dtype=torch.float32, device="cuda")
    wf = LCEDualWeakForm(sp)
    wf.functions = functions
    coefs = wf.coefficients(torch.float32)
    from nfempy_gb300 import autotune
    autotune.set_knobs({"elas_rows": 2})  # register accumulation, for comparison
    ms_registers = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    autotune.reset_knobs()
    ms = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    A.check_status("cosserat bench")
    T = sp.n_cells
    V = m["points"].shape[0]
    alg = T * 16 + V * 24 + T + T * 24 + A.nnz * 4 + A.n_rows * 4
    peak, kind = measured_peaks()
    ach = alg / (ms * 1e-3) / 1e9
    out = {"metric": "DoF/s assembled", "value": sp.n_dof / (ms * 1e-3), "ms_per_step": ms, "dtype": "f32",
           "n_cells": T, "n_dof": sp.n_dof, "nnz": A.nnz,
           "kernel": "cosserat_rows_kernel (shared-memory row images)",
           "ms_per_step_register_accumulation": ms_registers,
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "algorithmic_bytes": alg, "peak_source": kind,
                        "traffic": profiled_traffic("cosserat_rows_f32_cube24.txt")}}
    if not args.no_solve:
        # the FP64 system solved to 1e-8: FGMRES (FP32 inner iterations, FP64
        # refinement) with the cell-block Jacobi preconditioner (30 x 30
        # blocks of the matrix itself), then the P0 errors against the
        # manufactured solution on the device
        import nfempy_gb300 as nf
        from nfempy_gb300.solvers import KrylovSolver
        A64 = A.with_dtype(torch.float64)
        r64 = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
        wf.assemble(A64, r64, coefficients=wf.coefficients(torch.float64))
        wf.assemble(A, res, coefficients=coefs)
        ksp = KrylovSolver(A64, pc="cell_block", A32_values=A.values, restart=args.cos_restart)
        out["solve"] = _timed_solve(ksp, -r64, args, torch.cuda.current_stream())
        out["solve"]["preconditioner"] = "cell-block Jacobi (30 x 30 blocks of A, weighted additive Schwarz)"
        out["solve"]["l2_error_u_t_vs_manufactured"] = nf.l2_error(3, sp, exact, ksp.last_x.cpu().numpy(),
                                                                   skip_fields=["s", "m"])
    return out


def batch2d_bench(args):
    """512 independent 2-D mixed Darcy problems (n_i ~ U{8..128} squares per
    side, 2 n_i^2 triangles, log K_i GRF with correlation length 0.1 and
    sigma 1, f = 1) assembled together over their disjoint union (one cell pass,
    one row pass), FP32."""
    import numpy as np
    import torch
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    m, sp, kappa, f, sides = wl.darcy2d_batch(512)
    A = nf.CSRMatrix(sp, dtype=torch.float32)
    res = torch.empty(A.n_rows, dtype=torch.float32, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": f}
    coefs = wf.coefficients(torch.float32)
    ms = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    A.check_status("batch2d bench")
    # the same assembly captured once in a CUDA graph and replayed (the entry
    # point allocates nothing, so it is capturable)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        wf.assemble(A, res, coefficients=coefs)
    graph_ms = _time_assembly(graph.replay, args.steps, args.warmup)
    A.check_status("batch2d graph")
    # autotuned form and launch shape (nfempy_gb300.autotune, cached per GPU)
    from nfempy_gb300 import autotune
    import tempfile as _tf
    os.environ.setdefault("NFEM_TUNING_CACHE", os.path.join(_tf.gettempdir(), "nfempy_gb300_tuning.json"))
    best, best_ms, tried = autotune.tune(autotune.darcy_key(sp, torch.float32),
                                         lambda: wf.assemble(A, res, coefficients=coefs),
                                         autotune.darcy_candidates(2), form=wf, reps=max(3, args.steps // 4))
    tuned_ms = _time_assembly(lambda: wf.assemble(A, res, coefficients=coefs), args.steps, args.warmup)
    A.check_status("batch2d tuned")
    T = sp.n_cells
    V = m["points"].shape[0]
    alg = algorithmic_bytes(T, V, A.nnz, sp.n_dof, 4, verts_per_cell=3)
    peak, kind = measured_peaks()
    ach = alg / (ms * 1e-3) / 1e9
    out = {"metric": "DoF/s assembled", "value": sp.n_dof / (ms * 1e-3), "ms_per_step": ms, "dtype": "f32",
           "problems": len(sides), "n_cells": T, "n_dof": sp.n_dof, "nnz": A.nnz,
           "kernel": "darcy_records_kernel + darcy_rows_kernel (two passes: triangles, FP32)",
           "graph_replay_ms_per_step": graph_ms,
           "autotuned": {"config": best, "ms_per_step": tuned_ms, "candidates": len(tried),
                         "value": sp.n_dof / (tuned_ms * 1e-3), "cache": autotune.cache_path()},
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "algorithmic_bytes": alg, "peak_source": kind,
                        "traffic": profiled_traffic("darcy_records_rows_f32_batch512.txt")}}
    if not args.no_solve:
        # every problem at once: two-level FGMRES on the block-diagonal union,
        # aggregates of about s x s squares inside each problem (none spans
        # two problems) and the coarse matrix stored per problem
        from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
        A64 = A.with_dtype(torch.float64)
        r64 = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
        wf.assemble(A64, r64, coefficients=wf.coefficients(torch.float64))
        t0 = time.perf_counter()
        agg, bp = wl.batch_aggregates(sides, size=args.batch_agg, blocks=True)
        tl = TwoLevelCoarse(A64, None, cell_agg=agg, blocks=bp)
        t_struct = time.perf_counter() - t0
        ksp = KrylovSolver(A64, pc="two_level", A32_values=A.values, restart=args.tl_restart, two_level=tl)
        out["solve"] = _timed_solve(ksp, -r64, args, torch.cuda.current_stream(), two_level=True)
        out["solve"].update({"preconditioner": f"two-level (symmetric cycle, omega 0.9), {args.batch_agg}x"
                                               f"{args.batch_agg}-square aggregates, coarse matrix block-diagonal "
                                               "per problem",
                             "aggregates": tl.n_agg, "largest_block": int(np.diff(bp).max()),
                             "host_structure_s": t_struct,
                             "time_to_solve_incl_host_structure_ms": out["solve"]["time_to_solve_ms"] + 1e3 * t_struct})
        # one CUDA graph per step: both assemblies, the preconditioner setup
        # and the solve replaying the schedule a first solve recorded (no host
        # synchronisation inside); the FP64 residual is checked on the device
        c32, c64 = coefs, wf.coefficients(torch.float64)
        b = torch.empty_like(r64)
        torch.neg(r64, out=b)
        _, info_rec = ksp.solve(b.clone(), record_schedule=True, inner_rtol=args.tl_inner_rtol)
        xg = torch.zeros_like(r64)
        rel = torch.zeros(1, dtype=torch.float64, device="cuda")

        def step():
            wf.assemble(A, res, coefficients=c32)
            wf.assemble(A64, r64, coefficients=c64)
            torch.neg(r64, out=b)
            xg.zero_()
            ksp.refresh()
            ksp.solve(b, xg, inner_rtol=args.tl_inner_rtol, replay=True, relres_out=rel)

        step()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g.replay()
        n_rep = max(3, args.steps // 4)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(n_rep):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        out["graph_step"] = {"ms_per_step": e0.elapsed_time(e1) / n_rep, "replays": n_rep,
                             "final_relres_fp64": float(rel.item()),
                             "contents": "FP32 + FP64 assembly, two-level setup, FGMRES replaying a recorded schedule "
                                         f"({info_rec.inner_iterations} inner iterations, {info_rec.outer_iterations} "
                                         "refinement steps)"}
    autotune.reset_knobs()
    return out


# ------------------------------------------------------------------ GPU path
def bind_host_near_gpu(dev):
    """Keeps this process's host threads, and so the pinned buffers they
    allocate for the end-to-end copies, on the NUMA node the GPU hangs off
    when sysfs names one (a buffer on the far socket's memory crosses the
    CPU-to-CPU link on every copy).  Returns what was done, or None."""
    import torch
    try:
        pr = torch.cuda.get_device_properties(dev)
        bdf = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{bdf}/numa_node") as fh:
            node = int(fh.read().strip())
        if node < 0:
            return None
        with open(f"/sys/devices/system/node/node{node}/cpulist") as fh:
            spec = fh.read().strip()
        cpus = set()
        for part in spec.split(","):
            if "-" in part:
                lo, hi = part.split("-")
                cpus.update(range(int(lo), int(hi) + 1))
            elif part:
                cpus.add(int(part))
        if not cpus:
            return None
        os.sched_setaffinity(0, cpus)
        return {"numa_node": node, "cpus": len(cpus)}
    except (OSError, ValueError, AttributeError):
        return None


def run_ours(args):
    rank, world, local = env_rank()
    cpu_prob = cpu_vec = cpu_solve = None
    if rank == 0 and not args.no_cpu:
        cpu_prob = cpu_problem(N_SIDE, args.cpu_sample)  # before any CUDA use
        cpu_vec = cpu_vectorised(N_SIDE, args.cpu_vec_sample, os.cpu_count() or 1)
        if not args.no_solve:
            # the host solves run in a spawned process of their own, so no BLAS
            # or intra-op thread pool of theirs stays in this process while the
            # GPU is timed
            import multiprocessing as mp
            with mp.get_context("spawn").Pool(1) as pool:
                cpu_solve, small = pool.apply(cpu_solve_baselines, (16,))
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    host_affinity = bind_host_near_gpu(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import nfempy_gb300 as nf
    from nfempy_gb300 import _lib, autotune, workloads

    dtype = torch.float32 if args.precision == "f32" else torch.float64
    vbytes = 4 if dtype == torch.float32 else 8
    m, sp, kappa, f = workloads.darcy3d(N_SIDE)
    A = nf.CSRMatrix(sp, dtype=dtype)
    wf = nf.LaplaceDualWeakForm(sp)
    wf.use_chunks = args.kernel == "chunks"
    wf.use_records = args.kernel == "records"
    wf.use_slices = args.slices
    wf.use_streams = args.streams
    wf.use_fused = args.fused
    if args.slice_shift:
        wf.min_slice_shift = args.slice_shift
    if args.record_quarters:
        wf.record_quarters = args.record_quarters
    wf.functions = {"kappa": kappa, "rhs": f}
    coefs = wf.coefficients(dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        wf.assemble(A, res, coefficients=coefs)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    A.check_status("warmup")
    clocks = Clocks(local)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_begin = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_begin.record(stream)
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = float(np.mean(step_ms))
    bracket_ms = t_begin.elapsed_time(t_end)
    ms = max_over_ranks(ms, dist, "cuda")

    # ---------------- e2e: host buffers in, host result out, through the same API.
    # (a) serial: every step uploads the mesh points, kappa and f from pinned
    #     host memory, splits the points, assembles and reads values + residual
    #     back, all on one stream;
    # (b) pipelined (the reported e2e): the mesh stays resident (uploaded once,
    #     as for a sequence of coefficient fields on one mesh), each step uploads
    #     kappa and f and reads values + residual back; two buffer sets and two
    #     streams let step i's read-back overlap step i+1's upload and assembly.
    T, V = sp.n_cells, m["points"].shape[0]
    pts_h = torch.as_tensor(m["points"], dtype=torch.float64).pin_memory()
    k_h = [torch.as_tensor(kappa).to(dtype).pin_memory() for _ in range(2)]
    f_h = [torch.as_tensor(f).to(dtype).pin_memory() for _ in range(2)]
    vals_h = [torch.empty(A.nnz, dtype=dtype).pin_memory() for _ in range(2)]
    res_h = [torch.empty(A.n_rows, dtype=dtype).pin_memory() for _ in range(2)]
    A2 = [A, A.with_dtype(dtype)]
    res2 = [res, torch.empty_like(res)]
    k_d = [coefs[0], coefs[0].clone()]
    f_d = [coefs[1], coefs[1].clone()]
    h2d_serial = pts_h.numel() * 8 + k_h[0].numel() * vbytes + f_h[0].numel() * vbytes
    h2d = k_h[0].numel() * vbytes + f_h[0].numel() * vbytes
    d2h = A.nnz * vbytes + A.n_rows * vbytes

    def e2e_serial_step():
        sp.points.copy_(pts_h, non_blocking=True)
        k_d[0].copy_(k_h[0], non_blocking=True)
        f_d[0].copy_(f_h[0], non_blocking=True)
        if dtype == torch.float32:
            _lib.call("nfem_points_split", _lib.ptr(sp.points), V, _lib.ptr(sp.points_split), _lib.stream_ptr())
        else:
            _lib.call("nfem_points_fixed64", _lib.ptr(sp.points), V, _lib.ptr(sp.points_fixed64), _lib.stream_ptr())
        wf.assemble(A, res, coefficients=(k_d[0], f_d[0], coefs[2]))
        vals_h[0].copy_(A.values[: A.nnz], non_blocking=True)
        res_h[0].copy_(res, non_blocking=True)

    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()
    ready = [torch.cuda.Event(), torch.cuda.Event()]
    freed = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_step(i):
        j = i % 2
        s_up.wait_event(freed[j])  # buffer set j: its previous read-back has finished
        with torch.cuda.stream(s_up):
            k_d[j].copy_(k_h[j], non_blocking=True)
            f_d[j].copy_(f_h[j], non_blocking=True)
            wf.assemble(A2[j], res2[j], coefficients=(k_d[j], f_d[j], coefs[2]), stream=s_up)
            ready[j].record(s_up)
        s_down.wait_event(ready[j])
        with torch.cuda.stream(s_down):
            vals_h[j].copy_(A2[j].values[: A.nnz], non_blocking=True)
            res_h[j].copy_(res2[j], non_blocking=True)
            freed[j].record(s_down)

    def timed(fn, n, pipelined):
        e_s = torch.cuda.Event(enable_timing=True)
        e_e = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e_s.record(stream)
        if pipelined:
            s_up.wait_stream(stream)
            s_down.wait_stream(stream)
        for i in range(n):
            fn(i)
        if pipelined:
            stream.wait_stream(s_down)
            stream.wait_stream(s_up)
        e_e.record(stream)
        torch.cuda.synchronize()
        return e_s.elapsed_time(e_e) / n

    n_e2e = max(3, args.steps // 2)
    timed(lambda i: e2e_serial_step(), max(1, args.warmup), False)
    e2e_serial_ms = max_over_ranks(timed(lambda i: e2e_serial_step(), n_e2e, False), dist, "cuda")
    timed(e2e_step, max(2, args.warmup), True)
    # three timed windows, the median reported (each window's time beside it)
    e2e_windows = [timed(e2e_step, n_e2e, True) for _ in range(3)]
    e2e_ms = max_over_ranks(float(np.median(e2e_windows)), dist, "cuda")
    e2e_ok = torch.equal(vals_h[0], vals_h[1]) and torch.equal(vals_h[0], A.values[: A.nnz].cpu())
    A.check_status("bench")

    # ---------------- the other precision, timed the same way (its own roofline)
    other = "f64" if args.precision == "f32" else "f32"
    odt = torch.float64 if other == "f64" else torch.float32
    ob = 8 if other == "f64" else 4
    A_o = A.with_dtype(odt)
    res_o = torch.empty(A.n_rows, dtype=odt, device="cuda")
    coefs_o = wf.coefficients(odt)
    ms_o = _time_assembly(lambda: wf.assemble(A_o, res_o, coefficients=coefs_o), args.steps, args.warmup)
    A_o.check_status("bench other precision")
    ms_o = max_over_ranks(ms_o, dist, "cuda")
    # ---------------- FP64 with double-float records for every cell (the
    # arithmetic of cells off a dyadic lattice), same mesh and buffers
    A64, res64, coefs64 = (A, res, coefs) if args.precision == "f64" else (A_o, res_o, coefs_o)
    autotune.set_knobs({"darcy_f64_records": 1})
    try:
        ms_df = _time_assembly(lambda: wf.assemble(A64, res64, coefficients=coefs64), args.steps, args.warmup)
    finally:
        autotune.set_knobs({"darcy_f64_records": 0})
    A64.check_status("bench double-float records")
    ms_df = max_over_ranks(ms_df, dist, "cuda")
    clk = clocks.stop()
    v32, v64 = (A.values, A_o.values) if other == "f64" else (A_o.values, A.values)
    r32, r64 = (res, res_o) if other == "f64" else (res_o, res)
    rp = A.row_ptr.long()
    rows_of = torch.repeat_interleave(torch.arange(A.n_rows, device=rp.device), rp[1:] - rp[:-1])
    a64 = v64[: A.nnz].abs()
    rowmax = torch.zeros(A.n_rows, dtype=torch.float64, device=rp.device).scatter_reduce(0, rows_of, a64, "amax")
    f32_vs_f64 = float(((v32[: A.nnz].double() - v64[: A.nnz]).abs() / rowmax[rows_of].clamp_min(1e-300)).max())
    f32_vs_f64_rhs = float((r32.double() - r64).abs().max() / r64.abs().max())
    del rows_of, a64

    # ---------------- time to solve: FP64 system, FP32 inner iterations
    solve = None
    if not args.no_solve:
        solve = solve_bench(args, A, wf, coefs, res, stream)
    if cpu_solve is not None:
        # the same 16^3 x 6 system solved on the GPU, for a same-size comparison
        cpu_solve["gpu_same_system"] = small_system_gpu(args, *small)
    workloads = {}
    if not args.no_extra:
        workloads["elasticity_p2_cube40x6"] = elasticity_bench(args)
        workloads["cosserat_cube24x6"] = cosserat_bench(args)
        workloads["darcy2d_batch512"] = batch2d_bench(args)

    if rank != 0:
        return
    n_dof = sp.n_dof
    value = job_rate(n_dof, world, ms)
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(T, V, A.nnz, n_dof, vbytes)
    achieved = alg / (ms * 1e-3) / 1e9
    kname = {"chunks": "darcy_cells", "rows": "darcy_rows", "records": "darcy_records_rows"}[args.kernel]
    kernels = {"chunks": "darcy_cells_kernel", "rows": "darcy_rows_kernel",
               "records": "darcy_records_kernel + darcy_rows_kernel (two passes)"}[args.kernel]
    launches_per_step = 2 if args.kernel == "records" else 1
    prof_name = f"{kname}_{args.precision}_cube64.txt"
    traffic = profiled_traffic(prof_name)
    cpu = None
    if cpu_prob is not None:
        rate, secs = cpu_rate(cpu_prob, 1)
        cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": (f"oracle per-cell loop (reference structure: mapping, tabulation, Piola, orientation, "
                          f"element matrix, entry-wise scatter) over {cpu_prob['X'].shape[0]} of {cpu_prob['T']} "
                          f"cells, 1 thread, {secs:.1f} s; DoF/s extrapolated to the full mesh")}
    alg_o = algorithmic_bytes(T, V, A.nnz, n_dof, ob)
    ach_o = alg_o / (ms_o * 1e-3) / 1e9
    legs = {args.precision: {"ms_per_step": ms, "value": value, "algorithmic_bytes": alg,
                             "roofline_frac": achieved / peak, "headline": True},
            other: {"ms_per_step": ms_o, "value": job_rate(n_dof, world, ms_o), "unit": UNIT,
                    "kernel": kernels, "algorithmic_bytes": alg_o,
                    "roofline": {"bound": "hbm", "achieved": ach_o, "peak": peak, "unit": "GB/s",
                                 "frac": ach_o / peak, "algorithmic_bytes": alg_o, "peak_source": peak_kind,
                                 "traffic": profiled_traffic(f"{kname}_{other}_cube64.txt")}}}
    legs["f32"]["max_row_scaled_diff_vs_f64"] = f32_vs_f64
    legs["f32"]["max_rhs_diff_vs_f64"] = f32_vs_f64_rhs
    legs["f64"]["parity"] = ("FP64 values within 1e-12 of the FP64 oracle, row-scaled, at this size "
                             "(tests/test_gpu_fullsize.py)")
    legs["f64"]["records"] = ("cell pass: exact integer records for lattice cells (every cell of this dyadic "
                              "cube), double-float for cells off the lattice")
    legs["f64"]["double_float_records"] = {
        "ms_per_step": ms_df, "value": job_rate(n_dof, world, ms_df),
        "roofline_frac": algorithmic_bytes(T, V, A.nnz, n_dof, 8) / (ms_df * 1e-3) / 1e9 / peak,
        "what": "the same FP64 assembly with double-float records for every cell (knob "
                "NFEM_KNOB_DARCY_F64_RECORDS = 1): the cost on meshes off a dyadic lattice"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.precision, "data": "synthetic (seeded GRF log-permeability)",
        "config": {"workload": f"darcy3d_rt1p0_cube{N_SIDE}x6", "n_cells": T, "n_points": V, "n_dof": n_dof,
                   "nnz": A.nnz, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "flushed before every timed step (256 MB write, outside the step events)",
                   "bracket_ms_incl_flush": bracket_ms, "kernel": kernels, "host_affinity": host_affinity},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes": alg, "peak_source": peak_kind},
        "cpu_baseline": cpu,
        "cpu_baseline_vectorised": cpu_vec,
        "cpu_solve_baseline": cpu_solve,
        "e2e": {"value": job_rate(n_dof, world, e2e_ms), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "mode": "pipelined: kappa, f up and values, residual down every step (two buffer sets, two "
                        "streams); mesh resident", "results_match_device": bool(e2e_ok),
                "windows_ms_per_step": e2e_windows, "window_steps": n_e2e,
                "serial": {"value": job_rate(n_dof, world, e2e_serial_ms), "ms_per_step": e2e_serial_ms,
                           "h2d_bytes_per_step": h2d_serial, "d2h_bytes_per_step": d2h,
                           "mode": "points, kappa, f up, split, assemble, values + residual down; one stream"}},
        "precision_legs": legs,
        "solve": solve,
        "workloads": workloads,
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["f32", "f64"], default="f64",
                    help="headline precision (f64: the reference's; the other precision is reported beside it)")
    ap.add_argument("--cpu-sample", type=int, default=3000)
    ap.add_argument("--cpu-vec-sample", type=int, default=262144,
                    help="cells of the vectorised all-core numpy assembly baseline")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--restart", type=int, default=50, help="FGMRES restart of the plain block-Jacobi solve")
    ap.add_argument("--tl-restart", type=int, default=15, help="FGMRES restart of the two-level solves")
    ap.add_argument("--max-iters", type=int, default=20000)
    ap.add_argument("--inner-rtol", type=float, default=None,
                    help="FP32 inner tolerance of the block-Jacobi and point-Jacobi solves (default: the solver's)")
    ap.add_argument("--tl-inner-rtol", type=float, default=None,
                    help="FP32 inner tolerance of the two-level solves (default: the solver's)")
    ap.add_argument("--cos-restart", type=int, default=30, help="FGMRES restart of the Cosserat solve")
    ap.add_argument("--batch-agg", type=int, default=4,
                    help="aggregate side in squares of the batched 2-D two-level solve")
    ap.add_argument("--solver", choices=["both", "plain", "two_level"], default="both",
                    help="with --only solve: which preconditioners to run")
    ap.add_argument("--kernel", choices=["records", "rows", "chunks"], default="records",
                    help="Darcy assembly: cell records then rows (default), rows alone, or cell chunks")
    ap.add_argument("--slices", action="store_true",
                    help="the overlapped Darcy assembly by cell slices (nfem_darcy_rt1p0_assemble_sliced)")
    ap.add_argument("--slice-shift", type=int, default=0, help="cells per slice = 2^shift (default: the library's)")
    ap.add_argument("--record-quarters", type=int, default=0,
                    help="quarters of the blocks forming records in the overlapped assembly (default: the library's)")
    ap.add_argument("--fused", type=int, default=0,
                    help="1: FP64 tetrahedra through the fused persistent launch (record and row tiles from a plan)")
    ap.add_argument("--streams", type=int, default=0,
                    help="K > 0: the headline's two passes over K cell slices on two streams")
    ap.add_argument("--mlp-rows", type=int, default=3_200_000,
                    help="rows (faces) of --only mlp: synthetic features through the learned network")
    ap.add_argument("--only", choices=["assembly", "elasticity", "cosserat", "batch2d", "solve", "mlp"], default=None,
                    help="time one secondary assembly workload alone and print its record (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.only:
        fn = {"assembly": assembly_only, "elasticity": elasticity_bench, "cosserat": cosserat_bench, "batch2d": batch2d_bench,
              "solve": solve_only, "mlp": mlp_only}[args.only]
        print(json.dumps({"workload": args.only, **fn(args)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
