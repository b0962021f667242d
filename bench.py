#!/usr/bin/env python3
"""Benchmark of the GB300-native LightFEM solve path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the 1000x1000 Q4 plane-strain cantilever (2,004,002 DOFs, 36,024,004
nonzeros, RCM ordering), solved to a 1e-8 relative residual.  A step is one pass of
the solve path on one GPU with the model resident in HBM: element stiffness +
colouring assembly + loads, Dirichlet elimination, the PCG solve, reactions.
`value` is the device time of a step (CUDA events on the library's stream) for the
FP32-inner PCG with FP64 refinement; the FP64 PCG of the same storage and
preconditioner is timed beside it.  Every input array (K alone is 324 MB in FP64
BSR) is larger than the 129 MB L2, so no flush is needed between steps.

`e2e` is the same step through the C ABI from pinned host buffers, as the
reference's host library would call it: mesh, loads and constraints are uploaded,
the pattern, element map and colouring are built by the library, and u and R are
downloaded, inside the timed region of every step.

`--impl reference` times the reference's algorithm on the host cores instead (the
CPU restatement in oracle/, which reproduces the reference's iterates bit for bit),
on a bounded sample of PCG iterations extrapolated to the reference's own
iteration count for this model.

Under torchrun each rank solves its own copy of the model on its own GPU (weak
scaling, no collective on the data path); rank 0 prints the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Solve ms to 1e-8 rel. residual, 2M-dof Q4: FP32+refine vs FP64 PCG; SpMV GB/s"
WORKLOAD = "1000x1000 Q4 plane-strain cantilever (2.0 m x 1.0 m), 2,004,002 DOFs, 36,024,004 nnz, RCM"
DATA = ("synthetic: seeded structured Q4 mesh of the 1000x1000 cantilever workload (E 70 GPa, nu 0.33, "
        "t 0.01 m, left edge clamped, -1000 N over the right-edge nodes)")
CONFIG_IDX = 2
STEP_DESC = "element stiffness + colouring assembly + loads, Dirichlet, PCG to 1e-8, reactions"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    """Host-side barrier and max-reduction across torchrun ranks (gloo)."""

    def __init__(self, world: int):
        self.world = world
        self.rank = int(os.environ.get("RANK", "0"))
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if not self.dist:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.index = gpu_index
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, power, reasons = [], [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or not f[0].isdigit() or int(f[0]) != self.index:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


def gpu_index_for(local_rank: int) -> int:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v for v in vis.split(",") if v.strip()]
    if ids and ids[min(local_rank, len(ids) - 1)].strip().isdigit():
        return int(ids[min(local_rank, len(ids) - 1)])
    return local_rank


# ---------------------------------------------------------------------- model
def build_model(scale: int = 1):
    from lightfem_gb300 import mesh
    m = mesh.workload(CONFIG_IDX, scale=scale)
    m.sort_and_index()
    return m


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profiled_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel:
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


def spmv_bytes(kind: str, n: int, nnz: int, nblocks: int) -> int:
    """Algorithmic bytes of one product (int32 columns and row pointers, x read once,
    y written once): CSR Z(s+4) + 4(n+1) + 2sn, BSR B(4s+4) + 4(n/2+1) + 2sn."""
    s = 8 if kind.endswith("64") else 4
    if kind.startswith("csr"):
        return nnz * (s + 4) + 4 * (n + 1) + 2 * s * n
    return nblocks * (4 * s + 4) + 4 * (n // 2 + 1) + 2 * s * n


def product_bytes(n: int, matrix_bytes: int, precond: str = "jacobi") -> int:
    """Algorithmic bytes of one inner-loop product launch (mx_product): the FP32
    matrix as the library streams it (2x2 blocks with int32 or 16-bit block-column
    offsets, for BSR storage and for the paired CSR patterns of these meshes; the
    solve report's matrix_bytes_per_matvec), the block-row offsets and the FP32
    diagonal pair (hi, lo) read once, q written once.  With the pointwise
    preconditioners (Jacobi, 2x2 blocks) the update has formed p: p is read once.
    With the others the product forms p from z and the previous p: both read
    once, p written once."""
    direct = precond in ("jacobi", "block")
    vectors = 4 * n * ((1 + 2 + 1) if direct else (2 + 2 + 2))
    return matrix_bytes + 4 * (n // 2 + 1) + vectors


# ---------------------------------------------------------------------- CPU leg
def reference_iterations(storage: str, precond: str) -> tuple[int, str]:
    """The reference's own PCG iteration count on this model (tests/golden/golden.json)."""
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as fh:
        g = json.load(fh).get("cfg2", {})
    key = {("bsr", "jacobi"): "bsr_jacobi", ("csr", "jacobi"): "jacobi", ("bsr", "block"): "block",
           ("csr", "ic0"): "ic0"}.get((storage, precond), "jacobi")
    if key in g:
        return int(g[key]["iterations"]), key
    return int(g["jacobi"]["iterations"]), "jacobi"


def cpu_solve_sample(model, storage: str, precond: str, sample_iters: int, threads: int = 0) -> dict:
    """Time the reference algorithm (oracle restatement, with the reference's
    threading: colour-parallel scatter, row-parallel products, serial level-1
    work) on the host: assembly, loads, elimination, preconditioner setup, PCG and
    the reactions product.  ``sample_iters`` > 0 caps the PCG at that many
    iterations and extrapolates its time to the reference's iteration count for
    this model; 0 runs the complete solve and measures it.  TEST/BASELINE
    INFRASTRUCTURE: this is the only place bench.py runs the oracle."""
    from oracle import lf_oracle as O
    if threads > 0:
        O.set_threads(threads)
    m = model.copy()
    t0 = time.perf_counter()
    out = O.solve_model(m, stop_after="dirichlet", assembly="coloring")
    setup_total = (time.perf_counter() - t0) * 1e3
    asm_ms = out["timing"]["assembly_ms"]
    loads_ms = out["timing"]["loads_ms"]
    bnd_ms = out["timing"]["boundary_ms"]
    t1 = time.perf_counter()
    u, rep = O.pcg(out["rowptr"], out["col"], out["Kc"], out["fc"], 1e-8, 10 ** 6, storage, precond, "chunk", 1,
                   m.xy, iteration_cap=sample_iters)
    pcg_total = (time.perf_counter() - t1) * 1e3
    t2 = time.perf_counter()
    O.spmv(out["rowptr"], out["col"], out["K"], u)
    react_ms = (time.perf_counter() - t2) * 1e3
    iters = max(1, rep["iterations"])
    per_iter = rep["solve_ms"] / iters
    outside_loop = pcg_total - rep["solve_ms"]  # BSR conversion + preconditioner setup
    full_iters, key = reference_iterations(storage, precond)
    if sample_iters > 0:
        value = asm_ms + loads_ms + bnd_ms + outside_loop + per_iter * full_iters + react_ms
    else:
        value = asm_ms + loads_ms + bnd_ms + pcg_total + react_ms
    return {"value": value, "per_iter_ms": per_iter, "sample_iters": iters, "full_iters": full_iters,
            "measured": sample_iters == 0, "iterations": rep["iterations"], "converged": bool(rep["converged"]),
            "iters_source": f"reference run on this model ({key})", "assembly_ms": asm_ms, "loads_ms": loads_ms,
            "boundary_ms": bnd_ms, "pcg_setup_ms": outside_loop, "pcg_ms": pcg_total, "reactions_ms": react_ms,
            "threads": O.num_threads(), "untimed_setup_ms": setup_total - asm_ms - loads_ms - bnd_ms}


def run_reference(args) -> int:
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    model = build_model(args.scale)
    storage, precond = args.storage, args.precond if args.precond != "block" else "block"
    # Warm-up steps: bounded samples.  Timed steps: the first is the complete solve
    # (every PCG iteration runs, nothing extrapolated) and gives the value; the
    # others are bounded samples whose extrapolation is reported beside it, with its
    # error against the complete solve.
    for k in range(args.warmup):
        r = cpu_solve_sample(model, storage, precond, args.ref_sample_iters)
        log(f"reference warm-up {k}: {r['value']:.1f} ms extrapolated (per-iteration {r['per_iter_ms']:.3f} ms)")
    t_timed = time.perf_counter()
    full = cpu_solve_sample(model, storage, precond, 0)
    log(f"reference complete solve: {full['value']:.1f} ms, {full['iterations']} iterations")
    samples = []
    for k in range(1, args.steps):
        r = cpu_solve_sample(model, storage, precond, args.ref_sample_iters)
        samples.append(r)
        log(f"reference step {k}: {r['value']:.1f} ms extrapolated (per-iteration {r['per_iter_ms']:.3f} ms)")
    timed_s = time.perf_counter() - t_timed
    value = full["value"]
    extrapolated = statistics.median(r["value"] for r in samples) if samples else None
    sample = (f"step 1: the complete solve ({full['iterations']} FP64 PCG iterations, {storage}/{precond}) with "
              f"assembly, loads, elimination, setup and reactions, measured; steps 2..{args.steps}: "
              f"{args.ref_sample_iters} PCG iterations each, loop time extrapolated to the reference's "
              f"{full['full_iters']} iterations")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "ms", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(timed_s * 1e3 / max(1, args.steps), 3),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": {"workload": WORKLOAD, "precision": "fp64", "storage": storage, "preconditioner": precond,
                   "tolerance": 1e-8, "step": STEP_DESC},
        "cpu_baseline": {"value": round(value, 3), "unit": "ms", "cores": full["threads"], "kind": "port",
                         "sample": sample, "full_solve_ms": round(full["value"], 3),
                         "full_solve_iterations": full["iterations"], "full_solve_converged": full["converged"],
                         "full_solve_parts_ms": {k: round(full[k], 1) for k in (
                             "assembly_ms", "loads_ms", "boundary_ms", "pcg_setup_ms", "pcg_ms", "reactions_ms")},
                         "extrapolated_median_ms": None if extrapolated is None else round(extrapolated, 3),
                         "extrapolation_error_pct": None if extrapolated is None else round(
                             100.0 * (extrapolated - full["value"]) / full["value"], 2),
                         "per_iter_ms": round(full["per_iter_ms"], 4)},
        "e2e": {"value": round(value, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------- GPU leg
_PINNED = []


def pinned(a: np.ndarray) -> np.ndarray:
    """A copy of `a` in page-locked host memory (torch only allocates it)."""
    try:
        import torch
        t = torch.empty(a.size, dtype={np.dtype(np.float64): torch.float64, np.dtype(np.int32): torch.int32,
                                       np.dtype(np.int64): torch.int64}[a.dtype], pin_memory=True)
        _PINNED.append(t)  # the numpy view below does not own the allocation
        out = t.numpy().reshape(a.shape)
        out[...] = a
        return out
    except Exception:
        return np.ascontiguousarray(a)


def cpu_adjoint(model, tip_dof: int, sample_iters: int = 0, iterations: tuple[int, int] | None = None) -> dict:
    """The CPU FP64 gradient of the tip-node y displacement with respect to every
    element modulus, on all host cores: the oracle's forward solve (assembly, loads,
    elimination, 2x2 nodal block PCG on BSR), its adjoint solve K lambda = e_tip
    (zeroed on constrained DOFs) and its element loop g_e = -lambda_e^T K_e u_e /
    E_e.  The reference has no adjoint: this is the repository's restatement on the
    reference's algorithm and threading.  ``sample_iters`` > 0 caps both PCG solves
    and extrapolates their loop time to ``iterations`` (forward, adjoint); 0 runs
    and measures the complete solves.  BASELINE INFRASTRUCTURE (the oracle)."""
    from oracle import lf_oracle as O
    m = model.copy()
    m.settings.reordering = "none"
    t0 = time.perf_counter()
    out = O.solve_model(m, stop_after="dirichlet", assembly="coloring")
    tm = out["timing"]
    setup_ms = tm["assembly_ms"] + tm["loads_ms"] + tm["boundary_ms"]
    parts = {"assembly_loads_dirichlet_ms": setup_ms}
    solves = {}
    u = None
    for name, rhs in (("forward", out["fc"]), ("adjoint", None)):
        if rhs is None:
            rhs = np.zeros(m.n_dofs)
            rhs[tip_dof] = 1.0
            rhs[out["constraint_dofs"]] = 0.0
        t = time.perf_counter()
        x, rep = O.pcg(out["rowptr"], out["col"], out["Kc"], rhs, 1e-8, 10 ** 6, "bsr", "block", "chunk", 1, m.xy,
                       iteration_cap=sample_iters)
        total = (time.perf_counter() - t) * 1e3
        its = max(1, rep["iterations"])
        if sample_iters > 0 and iterations is not None:
            full = iterations[0 if name == "forward" else 1]
            ms = total - rep["solve_ms"] + rep["solve_ms"] / its * full
        else:
            full, ms = rep["iterations"], total
        solves[name] = {"ms": round(ms, 1), "iterations": full, "measured": sample_iters == 0}
        parts[f"{name}_solve_ms"] = ms
        if name == "forward":
            u = x
        else:
            lam = x
    en = m.element_node_index()
    mi = m.material_index(m.element_material)
    t = time.perf_counter()
    O.adjoint_grad(m.xy, en, m.young[mi], m.poisson[mi], m.thickness[mi], m.settings.plane_mode, u, lam)
    parts["gradient_loop_ms"] = (time.perf_counter() - t) * 1e3
    return {"ms": round(sum(parts.values()), 1), "cores": O.num_threads(), "kind": "port",
            "parts_ms": {k: round(v, 1) for k, v in parts.items()}, "solves": solves,
            "wall_ms": round((time.perf_counter() - t0) * 1e3, 1)}


def adjoint_gpu_runs(model, tip_of, precisions, repeats: int, dist: Dist) -> tuple[dict, dict]:
    """Forward solve + adjoint solve + gradient on the GPU (device time, CUDA
    events), per precision: the mean over ``repeats`` runs after one warm run."""
    from lightfem_gb300.adjoint import ElasticProblem
    out, grads = {}, {}
    for precision in precisions:
        p = ElasticProblem(model, precision=precision, storage="bsr", preconditioner="block", tolerance=1e-8,
                           max_iterations=400000)
        y0 = p.young0.copy()
        dj = np.zeros(p.n_dofs)
        dj[tip_of(p)] = 1.0
        times, kernel = [], []
        for k in range(repeats + 1):
            p.ctx.event_record(4)
            p.solve(y0)
            g = p.gradient(dj)
            p.ctx.event_record(5)
            if k > 0:
                times.append(p.ctx.event_elapsed(4, 5))
                kernel.append(p.ctx.timings()["adjoint_kernel_ms"])
        grads[precision] = g
        out[precision] = {"ms": round(dist.max(statistics.mean(times)), 3),
                          "gradient_kernel_ms": round(statistics.mean(kernel), 4),
                          "forward_iterations": p.report.iterations, "forward_refinements": p.report.refinements,
                          "forward_fallback_fp64": int(p.report.fallback_fp64),
                          "adjoint_iterations": p.adjoint_report.iterations,
                          "adjoint_fallback_fp64": int(p.adjoint_report.fallback_fp64)}
        p.close()
    return out, grads


def adjoint_leg(args, dist: Dist) -> dict:
    """Adjoint at scale: the perturbed two-material beam geometry at 1000x1000 with
    log-normal element moduli (2,004,002 DOFs, 1,000,000 moduli).  Timed together:
    assembly, the forward mixed-precision PCG solve, the adjoint PCG solve for the
    tip-node y displacement and the gradient kernel (device time, CUDA events).  The
    gradient error is against an FP64 GPU forward + adjoint run on the same inputs.
    Also: the 400x400 log-normal cantilever (321,602 DOFs, 160,000 moduli) on the
    GPU in both precisions, and the CPU FP64 gradient of both workloads on all host
    cores (400x400 complete; 1000x1000 with both solves sampled and extrapolated to
    the GPU FP64 run's iteration counts)."""
    from lightfem_gb300 import mesh
    from lightfem_gb300.adjoint import ElasticProblem

    model = mesh.workload(5, scale=args.scale)
    model.sort_and_index()
    out = {"workload": "1000x1000 perturbed two-material Q4 beam (4.0 m x 2.0 m), log-normal E_e = 1 GPa exp(0.5 z), "
                       "2,004,002 DOFs, 1,000,000 element moduli",
           "objective": "tip-node y displacement (one adjoint PCG solve)", "tolerance": 1e-8,
           "storage": "bsr", "preconditioner": "block"}
    grads = {}
    for precision in ("mixed", "fp64"):
        p = ElasticProblem(model, precision=precision, storage="bsr", preconditioner="block", tolerance=1e-8,
                           max_iterations=400000)
        y0 = p.young0.copy()
        dj = np.zeros(p.n_dofs)
        dj[p.dof(mesh.tip_node_id(p.model), 1)] = 1.0
        times = []
        for k in range(3):
            p.ctx.event_record(4)
            p.solve(y0)
            g = p.gradient(dj)
            p.ctx.event_record(5)
            if k > 0:
                times.append(p.ctx.event_elapsed(4, 5))
        grads[precision] = g
        out[precision] = {"ms": round(dist.max(statistics.mean(times)), 3),
                          "forward_iterations": p.report.iterations, "forward_refinements": p.report.refinements,
                          "forward_fallback_fp64": int(p.report.fallback_fp64),
                          "adjoint_iterations": p.adjoint_report.iterations,
                          "adjoint_fallback_fp64": int(p.adjoint_report.fallback_fp64)}
        if precision == "mixed":
            # the gradient kernel alone: compliance sensitivity, no solve
            kt = []
            for k in range(4):
                p.ctx.event_record(6)
                p.gradient(None)
                p.ctx.event_record(7)
                if k > 0:
                    kt.append(p.ctx.event_elapsed(6, 7))
            e, n = p.n_elements, p.n_dofs
            alg = e * (16 + 8) + 2 * 8 * n + 8 * e
            ms = statistics.mean(kt)
            out["gradient_call"] = {"ms": round(ms, 4), "algorithmic_bytes": alg,
                                    "gbs_incl_download": round(alg / ms / 1e6, 1),
                                    "note": "lfgpu_adjoint(dj_du=NULL): kernel plus the 8 MB gradient download"}
        p.close()
    ref = grads["fp64"]
    out["grad_rel_err_vs_fp64"] = float(np.linalg.norm(grads["mixed"] - ref) / np.linalg.norm(ref))
    out["speedup_mixed_vs_fp64"] = round(out["fp64"]["ms"] / out["mixed"]["ms"], 3)

    # 400x400 log-normal cantilever: GPU both precisions, CPU complete.
    m4 = mesh.workload(4, scale=args.scale)
    m4.sort_and_index()
    tip4 = lambda p: p.dof(mesh.tip_node_id(p.model), 1)  # noqa: E731
    g4, gr4 = adjoint_gpu_runs(m4, tip4, ("mixed", "fp64"), 3, dist)
    out["cfg4"] = {"workload": "400x400 plane-stress cantilever, log-normal E_e = 1 GPa exp(0.5 z), 321,602 DOFs, "
                               "160,000 element moduli", **g4,
                   "grad_rel_err_vs_fp64": float(np.linalg.norm(gr4["mixed"] - gr4["fp64"]) /
                                                 np.linalg.norm(gr4["fp64"]))}
    if dist.rank == 0 and not args.no_cpu:
        p4 = ElasticProblem(m4, precision="fp64", storage="bsr", preconditioner="block", tolerance=1e-8)
        tip_dof4 = tip4(p4)
        p4.close()
        out["cfg4"]["cpu"] = cpu_adjoint(m4, tip_dof4)
        out["cfg4"]["speedup_gpu_mixed_vs_cpu"] = round(out["cfg4"]["cpu"]["ms"] / g4["mixed"]["ms"], 2)
        # 1000x1000: the two CPU solves sampled, extrapolated to the GPU FP64 iteration counts.
        p5 = ElasticProblem(model, precision="fp64", storage="bsr", preconditioner="block", tolerance=1e-8)
        tip_dof5 = p5.dof(mesh.tip_node_id(p5.model), 1)
        p5.close()
        its = (out["fp64"]["forward_iterations"], out["fp64"]["adjoint_iterations"])
        out["cpu"] = cpu_adjoint(model, tip_dof5, sample_iters=args.cpu_sample_iters, iterations=its)
        out["cpu"]["note"] = (f"both PCG solves capped at {args.cpu_sample_iters} iterations and extrapolated to "
                              f"the GPU FP64 run's {its[0]} + {its[1]} iterations; assembly, loads, elimination "
                              f"and the gradient loop measured")
        out["speedup_gpu_mixed_vs_cpu"] = round(out["cpu"]["ms"] / out["mixed"]["ms"], 2)
    return out


def beam_leg(args, dist: Dist) -> dict:
    """The 2000x1000 perturbed two-material beam (4,006,002 DOFs, 72,036,004
    nonzeros; gravity plus a 1 MPa top pressure): the same step (assembly, loads,
    Dirichlet, PCG to 1e-8, reactions) with mixed 2x2 nodal block-Jacobi PCG (FP32
    inner, FP64 refinement) and with FP64 PCG, BSR storage, device time."""
    from lightfem_gb300 import _native, mesh
    from lightfem_gb300.solver import upload_model

    model = mesh.workload(3, scale=args.scale)
    model.sort_and_index()
    ctx = _native.Context(dist_env()[2])
    upload_model(ctx, model)
    out = {"workload": "2000x1000 perturbed two-material Q4 beam (4.0 m x 2.0 m, E 200/70 GPa), gravity + 1 MPa "
                       "top pressure, 4,006,002 DOFs", "nnz": ctx.nnz, "storage": "bsr", "preconditioner": "block"}
    for precision in ("mixed", "fp64"):
        o = ctx.options(1e-8, 400000, "bsr", "block", precision, "reliable")
        times = []
        for k in range(2):
            ctx.event_record(0)
            ctx.assemble("coloring")
            ctx.apply_dirichlet()
            _, rep = ctx.solve(o, download=False)
            ctx.reactions(download=False)
            ctx.event_record(1)
            if k > 0 or precision == "fp64":
                times.append(ctx.event_elapsed(0, 1))
            if precision == "fp64":
                break
        out[precision] = {"step_ms": round(dist.max(statistics.mean(times)), 2), "solve_ms": round(rep.solve_ms, 2),
                          "iterations": rep.iterations, "refinements": rep.refinements,
                          "true_residual_rel": rep.true_residual / rep.initial_residual,
                          "final_residual_rel": rep.final_residual / rep.initial_residual,
                          "fallback_fp64": int(rep.fallback_fp64)}
    out["speedup_mixed_vs_fp64"] = round(out["fp64"]["step_ms"] / out["mixed"]["step_ms"], 3)
    ctx.close()
    return out


def run_ours(args) -> int:
    from lightfem_gb300 import _native
    from lightfem_gb300.solver import upload_model

    world, rank, local = dist_env()
    dist = Dist(world)
    model = build_model(args.scale)
    model.index_with_node_order(_native.host_rcm(model.node_ids, model.element_nodes))
    ctx = _native.Context(local)
    upload_model(ctx, model)
    n, nnz = ctx.n_dofs, ctx.nnz
    nblocks = nnz // 4
    tol = 1e-8

    def opts(precision, storage=args.storage, precond=args.precond, persistent=False):
        return ctx.options(tol, 200000, storage, precond, precision, "reliable", persistent=persistent)

    def step(o):
        ctx.event_record(0)
        ctx.assemble("coloring")
        ctx.apply_dirichlet()
        _, rep = ctx.solve(o, download=False)
        ctx.reactions(download=False)
        ctx.event_record(1)
        return ctx.event_elapsed(0, 1), rep

    main = opts("mixed")
    if args.profile_iters:
        # Profiling run (not a benchmark): one step with the PCG capped at
        # --profile-iters iterations, the same loop with its kernels launched on the
        # stream, then three standalone products of each kind.  IC(0) and the
        # subdomain blocks run in FP64.
        precision = args.profile_precision or ("fp64" if args.precond in ("ic0", "subdomain") else "mixed")
        if args.precond == "subdomain":
            ctx.set_subdomains(args.subdomain_nodes, args.subdomain_split)
        ctx.set_option(_native.OPTION_IC0_SWEEP, _native.IC0_SWEEP[args.ic0_sweep])
        capped = ctx.options(tol, args.profile_iters, args.storage, args.precond, precision, "reliable")
        ms, rep = step(capped)
        unrolled = ctx.options(tol, 10 ** 6, args.storage, args.precond, precision, "reliable",
                               unrolled=args.profile_iters)
        ms_u, rep_u = step(unrolled)
        x = np.random.default_rng(0).standard_normal(n)
        for st in ("csr", "bsr"):
            for prec in ("fp64", "mixed"):
                ctx.spmv(x, 1, st, prec, repeat=3)
        print(json.dumps({"profile_iters": args.profile_iters, "precision": precision,
                          "conditional_step_ms": ms, "conditional_solve_ms": rep.solve_ms,
                          "iterations": rep.iterations, "unrolled_step_ms": ms_u,
                          "unrolled_solve_ms": rep_u.solve_ms, "unrolled_iterations": rep_u.iterations,
                          "unrolled_kernel_ms": list(rep_u.phase_ms)}))
        ctx.close()
        return 0
    for _ in range(args.warmup):
        step(main)
    dist.barrier()
    launches0 = ctx.timings()["kernel_launches"]
    sampler = ClockSampler(gpu_index_for(local))
    times, reps = [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        ms, rep = step(main)
        times.append(ms)
        reps.append(rep)
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    launches = ctx.timings()["kernel_launches"] - launches0
    dist.barrier()
    ms_step = dist.max(statistics.mean(times))
    rep = reps[-1]
    u = ctx.download(_native.U)
    R = ctx.reactions()
    true_rel = rep.true_residual / rep.initial_residual
    # post-processing of this solution (element fields + nodal smoothing), warm
    ctx.postprocess()
    ctx.postprocess()
    postprocess_ms = ctx.timings()["postprocess_ms"]

    # FP64 PCG of the same storage and preconditioner
    fp64_times, fp64_rep = [], None
    for k in range(max(1, args.fp64_steps) + 1):
        ms, fp64_rep = step(opts("fp64"))
        if k > 0:
            fp64_times.append(ms)
    u64 = ctx.download(_native.U)
    fp64_ms = dist.max(statistics.mean(fp64_times))

    # other variants, one solve each (device time of the solve alone)
    variants = []
    ctx.set_subdomains(64, "rcb")  # the reference's default block setting, for the "subdomain" variant
    for prec, st, pc, pers in () if args.no_variants else (("mixed", "bsr", "block", False), ("mixed", "csr", "jacobi", False),
                               ("fp64", "csr", "jacobi", False), ("fp64", "bsr", "block", False),
                               ("mixed", "bsr", "subdomain", False),
                               ("mixed", "csr", "ic0", False), ("fp64", "csr", "ic0", False),
                               ("mixed", "bsr", "jacobi", True), ("fp64", "csr", "jacobi", True)):
        try:
            ms, r = step(opts(prec, st, pc, pers))
            variants.append({"precision": prec, "storage": st, "preconditioner": pc,
                             **({"subdomain_nodes": 64, "subdomain_split": "rcb"} if pc == "subdomain" else {}),
                             "loop": "persistent" if pers else "graph", "step_ms": round(ms, 2),
                             "solve_ms": round(r.solve_ms, 2), "iterations": r.iterations,
                             "refinements": r.refinements, "true_residual_rel": r.true_residual / r.initial_residual,
                             "final_residual_rel": r.final_residual / r.initial_residual,
                             **({"ic0_levels": r.ic0_levels, "setup_ms": round(r.preconditioner_setup_ms, 2)}
                                if pc == "ic0" else {})})
        except _native.GpuError as e:
            variants.append({"precision": prec, "storage": st, "preconditioner": pc, "error": str(e)})
    ctx.assemble("coloring")
    ctx.apply_dirichlet()

    # products: standalone launches, device-timed over 20 calls each
    x = np.random.default_rng(0).standard_normal(n)
    spmv = {}
    for st in ("csr", "bsr"):
        for prec, tag in (("fp64", "64"), ("mixed", "32")):
            _, ms = ctx.spmv(x, 1, st, prec, repeat=20)
            b = spmv_bytes(st + tag, n, nnz, nblocks)
            spmv[f"{st}{tag}"] = {"us": round(ms * 1e3, 2), "algorithmic_bytes": b, "gbs": round(b / ms / 1e6, 1)}

    # Roofline of the dominant kernel of the step: the inner solve's FP32 product
    # (mx_product, about half of the loop's device time).  The graph hides its
    # launches from events, so the same loop runs once more with every kernel
    # launched on the stream and an event after each launch; the product's average
    # launch time comes from those events.
    peaks = measured_peaks()
    ctx.assemble("coloring")
    ctx.apply_dirichlet()
    _, prof = ctx.solve(ctx.options(tol, 10 ** 6, args.storage, args.precond, "mixed", "reliable",
                                    unrolled=args.roofline_passes), download=False)
    product_us = prof.phase_ms[0] * 1e3 / args.roofline_passes
    kernel_name = f"mx_product<{args.storage.upper()}>"
    alg = product_bytes(n, prof.matrix_bytes_per_matvec, args.precond)
    achieved = alg / (product_us * 1e-6) / 1e9
    traffic = profiled_traffic(kernel_name)
    roofline = {"bound": "hbm", "kernel": kernel_name, "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 3), "traffic": traffic,
                "algorithmic_bytes": alg, "us_per_launch": round(product_us, 2), "launches_timed": args.roofline_passes,
                "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs, copy burst)",
                "loop_kernels_us": {"product": round(product_us, 2),
                                    "update": round(prof.phase_ms[1] * 1e3 / args.roofline_passes, 2),
                                    "replacement_check": round(prof.phase_ms[2] * 1e3 / args.roofline_passes, 2),
                                    "reprecondition_check": round(prof.phase_ms[3] * 1e3 / args.roofline_passes, 2)}}

    # End to end through the C ABI from pinned host buffers, as the reference's
    # host library would call it: the mesh, loads and constraints go up, the
    # pattern, map and colouring are built in the library (lfgpu_build_pattern),
    # and u and R come back.
    en = model.element_node_index().astype(np.int32)
    em = model.material_index(model.element_material).astype(np.int32)
    cd, cv = model.constraints()
    host = {"xy": pinned(np.ascontiguousarray(model.xy)), "en": pinned(en), "em": pinned(em),
            "young": pinned(model.young.copy()), "nu": pinned(model.poisson.copy()),
            "t": pinned(model.thickness.copy()), "f": pinned(model.nodal_load_vector()), "cd": pinned(cd),
            "cv": pinned(cv)}
    h2d = sum(int(a.nbytes) for a in host.values())
    e2e_times = []
    for k in range(args.e2e_steps + 1):
        ctx.event_record(2)
        ctx.set_mesh(host["xy"], host["en"], host["em"], host["young"], host["nu"], host["t"],
                     model.settings.plane_mode)
        ctx.build_pattern()
        ctx.set_loads(host["f"])
        ctx.set_constraints(host["cd"], host["cv"])
        ctx.assemble("coloring")
        ctx.apply_dirichlet()
        u_e2e, _ = ctx.solve(main, download=True)
        r_e2e = ctx.reactions(download=True)
        ctx.event_record(3)
        if k > 0:
            e2e_times.append(ctx.event_elapsed(2, 3))
    d2h = int(u_e2e.nbytes + r_e2e.nbytes)
    e2e_ms = dist.max(statistics.mean(e2e_times))

    adjoint = None if args.no_adjoint else adjoint_leg(args, dist)
    beam = None if args.no_beam else beam_leg(args, dist)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_solve_sample(model, args.storage, args.precond if args.precond != "block" else "block",
                               args.cpu_sample_iters)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(ms_step, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": DATA,
            "config": {"workload": WORKLOAD, "precision": "mixed (FP32 inner PCG, FP64 refinement)",
                       "storage": args.storage, "preconditioner": args.precond, "tolerance": tol,
                       "step": STEP_DESC, "loop": "device-driven CUDA graph (conditional WHILE)",
                       "l2": "inputs larger than L2 (K: 324 MB FP64 BSR, 162 MB FP32 BSR with 16-bit column offsets)"},
            "iterations": rep.iterations, "refinements": rep.refinements, "true_residual_rel": true_rel,
            "solve_ms": round(rep.solve_ms, 3),
            "fp64": {"step_ms": round(fp64_ms, 3), "iterations": fp64_rep.iterations,
                     "true_residual_rel": fp64_rep.true_residual / fp64_rep.initial_residual,
                     "final_residual_rel": fp64_rep.final_residual / fp64_rep.initial_residual,
                     "solve_ms": round(fp64_rep.solve_ms, 3)},
            "speedup_mixed_vs_fp64": round(fp64_ms / ms_step, 3),
            "true_residual_rel_mixed_fp64": [true_rel, fp64_rep.true_residual / fp64_rep.initial_residual],
            "mixed_vs_fp64_u_rel": float(np.linalg.norm(u - u64) / np.linalg.norm(u64)),
            "reaction_sum_y": float(R[1::2].sum()),
            "postprocess_ms": round(postprocess_ms, 3),
            "variants": variants, "spmv": spmv, "roofline": roofline, "clocks": clocks,
            "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "adjoint": adjoint,
            "beam_2000x1000": beam,
            "wall_s_timed": round(wall, 3),
        }
        if cpu is not None:
            line["cpu_baseline"] = {
                "value": round(cpu["value"], 1), "unit": "ms", "cores": cpu["threads"], "kind": "port",
                "sample": (f"{cpu['sample_iters']} FP64 PCG iterations ({args.storage}/{args.precond}) plus full "
                           f"assembly, elimination, setup and reactions, loop extrapolated to the reference's "
                           f"{cpu['full_iters']} iterations"),
                "per_iter_ms": round(cpu["per_iter_ms"], 4)}
        print(json.dumps(line), flush=True)
    ctx.close()
    dist.close()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--storage", choices=("csr", "bsr"), default="bsr")
    ap.add_argument("--precond", choices=("jacobi", "block", "ic0", "subdomain"), default="jacobi",
                    help="block: 2x2 nodal blocks; ic0 and subdomain only with --profile-iters (FP64 profiling run)")
    ap.add_argument("--subdomain-nodes", type=int, default=64, help="nodes per subdomain for --precond subdomain")
    ap.add_argument("--profile-precision", choices=("fp64", "mixed"), default=None,
                    help="precision of the --profile-iters run (default: fp64 for ic0 and subdomain, else mixed)")
    ap.add_argument("--subdomain-split", choices=("rcb", "chunk"), default="rcb")
    ap.add_argument("--ic0-sweep", choices=("auto", "levels", "polled"), default="auto",
                    help="IC(0) sweeps of the --profile-iters run (auto: levels where the average level is wide)")
    ap.add_argument("--scale", type=int, default=1, help="divide the mesh size (testing only)")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample-iters", type=int, default=300)
    ap.add_argument("--ref-sample-iters", type=int, default=300)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--roofline-passes", type=int, default=200,
                    help="loop passes launched on the stream to time the inner product per launch")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    ap.add_argument("--no-beam", action="store_true", help="skip the 2000x1000 beam measurement")
    ap.add_argument("--no-variants", action="store_true", help="skip the other storage/preconditioner variants")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="profiling run for ncu: one step capped at this many PCG iterations (not a benchmark)")
    args = ap.parse_args()
    if args.precond in ("ic0", "subdomain") and not args.profile_iters:
        ap.error(f"--precond {args.precond} is a profiling option (use it with --profile-iters)")
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    return run_reference(args) if args.impl == "reference" else run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
