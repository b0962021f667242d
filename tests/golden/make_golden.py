"""Regenerate the golden fixtures from the reference's own sources.

Run from the repository root on a machine with the reference's source tree:

    make -C oracle ref REF=<reference checkout>   # oracle/_ref/ref_dump from its sources
    python tests/golden/make_golden.py

Each case writes a small model through ``lightfem_gb300.mesh.to_fem``, runs
``oracle/_ref/ref_dump`` on it (the reference's parser, validator, assembly, Dirichlet,
preconditioners and PCG, see oracle/ref_dump.cpp) and stores the arrays in
``tests/golden/<case>.npz`` and the scalar reports in ``tests/golden/golden.json``.
The GPU machine has no reference tree; the tests only read these committed files.

Cases:
  single_q4  the one-element cantilever of tests/test_solver.cpp:41-62
  scrambled  the scrambled 2x2 mesh of tests/test_solver.cpp:143-174 (+ RCM)
  grid6      grid_model(6, 6) of tests/test_solver.cpp:371-396, every iterative variant
  beam       24x12 perturbed two-material beam: gravity + top pressure, colouring
  strain     16x8 plane-strain cantilever with RCM (the 1000x1000 workload's physics)
  adjoint    20x20 cantilever with log-normal per-element moduli + reference FD
  failures   degenerate inputs (NaN/inf/negative moduli, NaN/inf loads, a floating
             node): how the public solve() ends for each preconditioner and storage;
             a clockwise element and zero-length loaded edges: how the assembly ends
  cfg1       the 200x200 workload: iteration counts, residuals, full u and R of the
             Jacobi and IC(0) runs, every 101st DOF of the others
  cfg2       the 1000x1000 workload: known answers from the reference (reports,
             norms, max |u| and its DOF, every 2003rd u, u at 4000 seeded DOFs, R at
             every constrained DOF).  These runs take about half an hour on 8 cores; `--run-cfg2 DIR`
             makes them (ref_dump output per variant in DIR/cfg2_<variant>) and
             `--cfg2-dir DIR` reads them back.  Without either, the cfg2 entries
             already in golden.json and cfg2.npz are kept.

`--only cfg1,cfg2` remakes only the named sections and keeps the other fixtures.

Solve runs also carry the reference's post-processing (element centre and Gauss
point fields, smoothed nodal stress); the small cases keep them.
"""

from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from lightfem_gb300 import mesh  # noqa: E402
from lightfem_gb300.model import PLANE_STRAIN, Model, SolverSettings  # noqa: E402

REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
OUT = os.path.join(ROOT, "tests", "golden")


def run(model: Model, *args: str) -> tuple[dict, dict]:
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "m.fem")
        with open(path, "w") as fh:
            fh.write(mesh.to_fem(model, os.path.join(tmp, "out.vtk")))
        subprocess.run([REF_DUMP, path, tmp, *args], check=True)
        arrays = {f[:-4]: np.load(os.path.join(tmp, f)) for f in os.listdir(tmp) if f.endswith(".npy")}
        with open(os.path.join(tmp, "report.json")) as fh:
            report = json.load(fh)
    return arrays, report


def single_q4() -> Model:
    return Model(
        node_ids=np.array([1, 2, 3, 4]), xy=np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]),
        material_ids=np.array([1]), young=np.array([1.0e6]), poisson=np.array([0.25]), thickness=np.array([1.0]),
        element_ids=np.array([1]), element_nodes=np.array([[1, 2, 3, 4]]), element_material=np.array([1]),
        bc_node=np.array([1, 4]), bc_ux=np.zeros(2), bc_uy=np.zeros(2),
        load_node=np.array([2]), load_fx=np.zeros(1), load_fy=np.array([-1.0]),
        settings=SolverSettings(tolerance=1e-12, max_iterations=100))


def scrambled() -> Model:
    ids = np.array([1, 9, 3, 8, 2, 7, 4, 6, 5])
    xy = np.array([[0, 0], [1, 0], [2, 0], [0, 1], [1, 1], [2, 1], [0, 2], [1, 2], [2, 2]], dtype=float)
    return Model(
        node_ids=ids, xy=xy, material_ids=np.array([1]), young=np.array([1.0e6]), poisson=np.array([0.25]),
        thickness=np.array([1.0]), element_ids=np.array([1, 2, 3, 4]),
        element_nodes=np.array([[1, 9, 2, 8], [9, 3, 7, 2], [8, 2, 6, 4], [2, 7, 5, 6]]),
        element_material=np.ones(4, np.int64), bc_node=np.array([1, 4]), bc_ux=np.zeros(2), bc_uy=np.zeros(2),
        load_node=np.array([3, 5]), load_fx=np.zeros(2), load_fy=np.array([-1.0, -1.0]),
        settings=SolverSettings(tolerance=1e-12, max_iterations=200))


def grid6() -> Model:
    m = mesh.cantilever(6, 6, length=1.0, height=1.0, young=1.0e6, poisson=0.25, thickness=1.0,
                        total_load=-0.01 * 7, settings=SolverSettings(tolerance=1e-12, max_iterations=5000))
    m.load_fy[:] = -0.01
    return m


VARIANTS = {
    "csr_jacobi": ("storage=csr", "preconditioner=jacobi"),
    "bsr_jacobi": ("storage=bsr", "preconditioner=jacobi"),
    "csr_ic0": ("storage=csr", "preconditioner=ic0"),
    "bsr_ic0": ("storage=bsr", "preconditioner=ic0"),
    "bsr_block1": ("storage=bsr", "preconditioner=block", "subdomain_split=chunk", "subdomain_nodes=1"),
    "csr_block1": ("storage=csr", "preconditioner=block", "subdomain_split=chunk", "subdomain_nodes=1"),
    "bsr_block_rcb2": ("storage=bsr", "preconditioner=block", "subdomain_split=rcb", "subdomain_nodes=2"),
    "bsr_block_chunk4": ("storage=bsr", "preconditioner=block", "subdomain_split=chunk", "subdomain_nodes=4"),
    "bsr_block64": ("storage=bsr", "preconditioner=block", "subdomain_split=rcb", "subdomain_nodes=64"),
}


# The 1000x1000 runs: the reference's settings for each stored variant.
CFG2_VARIANTS = {
    "jacobi": ("storage=csr", "preconditioner=jacobi", "assembly=coloring"),
    "bsr_jacobi": ("storage=bsr", "preconditioner=jacobi", "assembly=coloring"),
    "block": ("storage=bsr", "preconditioner=block", "subdomain_split=chunk", "subdomain_nodes=1",
              "assembly=coloring"),
    "ic0": ("storage=csr", "preconditioner=ic0", "assembly=coloring"),
    "block64": ("storage=bsr", "preconditioner=block", "subdomain_split=rcb", "subdomain_nodes=64",
                "assembly=coloring"),
}


def failure_outcomes() -> tuple[dict, dict]:
    """How the reference's public solve() ends on each model of FAILURE_MODELS
    (tests/cases.py), for every preconditioner and storage, and on each model of
    ASSEMBLY_FAILURES.  Non-finite moduli and
    loads cannot pass the parser, so they go in as ref_dump overrides after
    parsing, with validation off (the solver needs only an indexed model)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cases import ASSEMBLY_FAILURES, FAILURE_MODELS
    outcomes, arrays = {}, {}
    for name, make in ASSEMBLY_FAILURES.items():  # the assembly stops before any solver choice
        outcomes[name] = {"csr_jacobi": terminating_outcome(make())}
    for name, make in FAILURE_MODELS.items():
        model = make()
        overrides = []
        for k in np.flatnonzero(~np.isfinite(model.young)):
            overrides.append(f"set_young={int(model.material_ids[k])}:{float(model.young[k])!r}")
            model.young[k] = 1.0e6
        for k in np.flatnonzero(~np.isfinite(model.load_fy)):
            overrides.append(f"set_fy={int(model.load_node[k])}:{float(model.load_fy[k])!r}")
            model.load_fy[k] = 0.0
        outcomes[name] = {}
        for precond in ("jacobi", "block", "ic0"):
            for storage in ("csr", "bsr"):
                va, vr = run(model, "outcome=1", "validate=0", f"storage={storage}", f"preconditioner={precond}",
                             "subdomain_split=chunk", "subdomain_nodes=1", *overrides)
                outcomes[name][f"{storage}_{precond}"] = vr
                if "u" in va:
                    arrays[f"{name}__{storage}_{precond}"] = va["u"]
    return outcomes, arrays


def terminating_outcome(model: Model) -> dict:
    """ref_dump's outcome stage on ``model``.  The reference computes element
    stiffness inside an OpenMP parallel region, and an exception cannot leave
    one: a non-positive Jacobian ends the process through std::terminate, which
    prints the exception's what().  That run is recorded as
    {"outcome": "terminate", "what": <message>}."""
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "m.fem")
        with open(path, "w") as fh:
            fh.write(mesh.to_fem(model, os.path.join(tmp, "out.vtk")))
        proc = subprocess.run([REF_DUMP, path, tmp, "outcome=1", "validate=0"], capture_output=True, text=True)
        if proc.returncode == 0:
            with open(os.path.join(tmp, "report.json")) as fh:
                return json.load(fh)
    what = [line.split("what():", 1)[1].strip() for line in proc.stderr.splitlines() if "what():" in line]
    if proc.returncode >= 0 or not what:
        raise RuntimeError(f"ref_dump failed: {proc.stderr}")
    return {"outcome": "terminate", "what": what[0]}


def save(name: str, arrays: dict) -> None:
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)


def main() -> None:
    import argparse
    ap = argparse.ArgumentParser(description="regenerate tests/golden from the reference's sources")
    ap.add_argument("--cfg2-dir", help="read the 1000x1000 reference runs from this directory")
    ap.add_argument("--run-cfg2", help="make the 1000x1000 reference runs in this directory (hours)")
    ap.add_argument("--failures-only", action="store_true",
                    help="remake only the failure-detection outcomes; keep every other fixture")
    ap.add_argument("--only", default="",
                    help="comma-separated sections to remake (single_q4, scrambled, grid6, beam, strain, adjoint, "
                         "failures, cfg1, cfg2); the others keep their fixtures")
    args = ap.parse_args()
    only = {x for x in args.only.split(",") if x}

    def want(section: str) -> bool:
        return not only or section in only

    if not os.path.exists(REF_DUMP):
        raise SystemExit("build the reference first: make -C oracle ref")
    if args.failures_only:
        with open(os.path.join(OUT, "golden.json")) as fh:
            golden = json.load(fh)
        golden["failures"], arrays = failure_outcomes()
        save("failures", arrays)
        with open(os.path.join(OUT, "golden.json"), "w") as fh:
            json.dump(golden, fh, indent=1, sort_keys=True)
        return
    golden: dict = {}
    if only and os.path.exists(os.path.join(OUT, "golden.json")):
        with open(os.path.join(OUT, "golden.json")) as fh:
            golden = json.load(fh)

    # --- single Q4 and scrambled mesh: every stage, serial and colouring assembly
    for name, model in (("single_q4", single_q4()), ("scrambled", scrambled())):
        if not want(name):
            continue
        arrays, report = run(model, "pattern=1", "ke=4", "precond=1", "subdomain_split=chunk",
                             "subdomain_nodes=1", "solve=1")
        col_arrays, col_report = run(model, "pattern=1", "assembly=coloring", "solve=1")
        arrays["K_coloring"] = col_arrays["K"]
        arrays["u_coloring"] = col_arrays["u"]
        for k in ("post_fields", "post_nodal"):
            arrays[k] = arrays[k].reshape(-1, 5, 7) if k == "post_fields" else arrays[k].reshape(-1, 4)
        report["coloring"] = col_report
        if name == "scrambled":
            rcm_arrays, rcm_report = run(model, "pattern=1", "reordering=rcm", "solve=1")
            for k in ("node_order", "rowptr", "col", "map", "K", "Kc", "fc", "u", "R", "colors"):
                arrays[f"rcm_{k}"] = rcm_arrays[k]
            report["rcm"] = rcm_report
        save(name, arrays)
        golden[name] = report

    if want("grid6"):
        grid6_fixtures(golden)
    if want("beam"):
        beam_fixtures(golden)
    if want("strain"):
        strain_fixtures(golden)
    if want("adjoint"):
        adjoint_fixtures(golden)
    if want("failures"):
        golden["failures"], arrays = failure_outcomes()
        save("failures", arrays)
    if want("cfg1"):
        cfg1_fixtures(golden)
    if want("cfg2"):
        cfg2_fixtures(golden, args)
    with open(os.path.join(OUT, "golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1, sort_keys=True)


def grid6_fixtures(golden: dict) -> None:
    """All iterative variants of tests/test_solver.cpp:398-448."""
    model = grid6()
    arrays, report = run(model, "pattern=1", "ke=2", "precond=1", "subdomain_split=rcb", "subdomain_nodes=2")
    golden["grid6"] = {"pattern": report}
    _, r_chunk = run(model, "precond=1", "subdomain_split=chunk", "subdomain_nodes=1")
    chunk_arrays, _ = run(model, "precond=1", "subdomain_split=chunk", "subdomain_nodes=1")
    arrays["z_block1"] = chunk_arrays["z_block"]
    golden["grid6"]["precond_chunk1"] = r_chunk
    for vname, opts in VARIANTS.items():
        va, vr = run(model, "solve=1", *opts)
        arrays[f"u_{vname}"] = va["u"]
        arrays[f"R_{vname}"] = va["R"]
        if vname == "csr_jacobi":
            arrays["post_fields"] = va["post_fields"].reshape(-1, 5, 7)
            arrays["post_nodal"] = va["post_nodal"].reshape(-1, 4)
        golden["grid6"][vname] = vr
    save("grid6", arrays)


def beam_fixtures(golden: dict) -> None:
    """Perturbed two-material beam with gravity and pressure."""
    model = mesh.perturbed_beam(24, 12, seed=7, settings=SolverSettings(
        tolerance=1e-10, max_iterations=20000, assembly="coloring"))
    arrays, report = run(model, "pattern=1", "ke=4", "precond=1", "subdomain_split=chunk", "subdomain_nodes=1")
    golden["beam"] = {"pattern": report}
    for vname in ("csr_jacobi", "bsr_jacobi", "csr_ic0", "bsr_block1", "bsr_block64"):
        va, vr = run(model, "solve=1", *VARIANTS[vname])
        arrays[f"u_{vname}"] = va["u"]
        arrays[f"R_{vname}"] = va["R"]
        if vname == "csr_jacobi":
            arrays["post_fields"] = va["post_fields"].reshape(-1, 5, 7)
            arrays["post_nodal"] = va["post_nodal"].reshape(-1, 4)
        golden["beam"][vname] = vr
    save("beam", arrays)


def strain_fixtures(golden: dict) -> None:
    """Plane strain + RCM."""
    model = mesh.cantilever(16, 8, young=70e9, poisson=0.33, plane_mode=PLANE_STRAIN,
                            settings=SolverSettings(tolerance=1e-10, max_iterations=20000, assembly="coloring",
                                                    reordering="rcm"))
    arrays, report = run(model, "pattern=1", "ke=2", "precond=1", "subdomain_split=chunk", "subdomain_nodes=1")
    golden["strain"] = {"pattern": report}
    for vname in ("csr_jacobi", "csr_ic0", "bsr_block1", "bsr_block64"):
        va, vr = run(model, "solve=1", *VARIANTS[vname])
        arrays[f"u_{vname}"] = va["u"]
        arrays[f"R_{vname}"] = va["R"]
        if vname == "csr_jacobi":
            arrays["post_fields"] = va["post_fields"].reshape(-1, 5, 7)
            arrays["post_nodal"] = va["post_nodal"].reshape(-1, 4)
        golden["strain"][vname] = vr
    save("strain", arrays)


def adjoint_fixtures(golden: dict) -> None:
    """Log-normal moduli, compliance and tip uy by central differences."""
    n = 20
    model = mesh.cantilever(n, n, poisson=0.3, per_element_young=mesh.lognormal_moduli(n * n, seed=11),
                            settings=SolverSettings(tolerance=1e-13, max_iterations=50000))
    tip = mesh.tip_node_id(model)
    rng = np.random.default_rng(5)
    elems = np.sort(rng.choice(n * n, size=16, replace=False))
    arrays, report = run(model, "solve=1", "fd=" + ",".join(str(int(e)) for e in elems), "fd_step=1e-6",
                         f"tip_node={tip}")
    report["tip_node"] = tip
    golden["adjoint"] = report
    save("adjoint", arrays)


# Full u and R of the 200x200 workload are kept for these variants (80,802 values
# each); the others keep every 101st DOF.
CFG1_FULL = ("csr_jacobi", "csr_ic0")
# DOFs of the 1000x1000 runs whose u and R are kept: seeded, sorted.
CFG2_SAMPLE = 4000


def cfg2_sample_dofs(n: int) -> np.ndarray:
    return np.sort(np.random.default_rng(20261204).choice(n, size=CFG2_SAMPLE, replace=False))


def cfg2_fixed_dofs() -> np.ndarray:
    """The constrained DOFs of the 1000x1000 workload, in node-ID order."""
    m = mesh.workload(2)
    m.sort_and_index()
    return np.sort(m.constraints()[0]).astype(np.int64)


def cfg1_fixtures(golden: dict) -> None:
    """The 200x200 workload: iteration counts and fields."""
    model = mesh.workload(1)
    arrays, report = run(model, "pattern=1")
    keep = {"rowptr_sum": np.array([arrays["rowptr"].sum()]), "col_sum": np.array([arrays["col"].sum()]),
            "map_sum": np.array([arrays["map"].sum()]), "K_sample": arrays["K"][::997],
            "Kc_sample": arrays["Kc"][::997], "fc": arrays["fc"], "colors": arrays["colors"]}
    golden["cfg1"] = {"pattern": report, "nnz": int(arrays["col"].shape[0])}
    for vname in ("csr_jacobi", "bsr_jacobi", "csr_ic0", "bsr_block1", "bsr_block64"):
        va, vr = run(model, "solve=1", *VARIANTS[vname])
        if vname in CFG1_FULL:
            keep[f"u_{vname}_full"] = va["u"]
            keep[f"R_{vname}_full"] = va["R"]
        keep[f"u_{vname}"] = va["u"][::101]
        keep[f"R_{vname}"] = va["R"][::101]
        vr["u_norm"] = float(np.linalg.norm(va["u"]))
        vr["R_norm"] = float(np.linalg.norm(va["R"]))
        golden["cfg1"][vname] = vr
    save("cfg1", keep)


def cfg2_fixtures(golden: dict, args) -> None:
    """The 1000x1000 workload (long runs, made separately): the reports, u at every
    2003rd DOF, and u and R at CFG2_SAMPLE seeded DOFs with max |u| and its DOF."""
    cfg2 = {}
    keep = {}
    big = args.cfg2_dir or args.run_cfg2
    if args.run_cfg2:
        model = mesh.workload(2)
        with open(os.path.join(big, "cfg2.fem"), "w") as fh:
            fh.write(mesh.to_fem(model, os.path.join(big, "out.vtk")))
        for vname, opts in CFG2_VARIANTS.items():
            d = os.path.join(big, f"cfg2_{vname}")
            os.makedirs(d, exist_ok=True)
            subprocess.run([REF_DUMP, os.path.join(big, "cfg2.fem"), d, "solve=1", *opts], check=True)
    for vname in (CFG2_VARIANTS if big else ()):
        d = os.path.join(big, f"cfg2_{vname}")
        if os.path.exists(os.path.join(d, "report.json")):
            with open(os.path.join(d, "report.json")) as fh:
                rep = json.load(fh)
            u = np.load(os.path.join(d, "u.npy"))
            r = np.load(os.path.join(d, "R.npy"))
            rep["u_norm"] = float(np.linalg.norm(u))
            rep["R_norm"] = float(np.linalg.norm(r))
            rep["R_y_sum"] = float(r[1::2].sum())
            rep["u_absmax"] = float(np.abs(u).max())
            rep["u_absmax_dof"] = int(np.abs(u).argmax())
            cfg2[vname] = rep
            keep[f"u_{vname}"] = u[::2003]
            dofs = cfg2_sample_dofs(u.shape[0])
            keep["sample_dofs"] = dofs
            keep[f"u_{vname}_sample"] = u[dofs]
            # The reactions that carry load: every constrained DOF (the clamped edge).
            fixed = cfg2_fixed_dofs()
            keep["fixed_dofs"] = fixed
            keep[f"R_{vname}_fixed"] = r[fixed]
    if cfg2:
        golden["cfg2"] = cfg2
        save("cfg2", keep)
    elif os.path.exists(os.path.join(OUT, "golden.json")):
        with open(os.path.join(OUT, "golden.json")) as fh:
            old = json.load(fh)
        if "cfg2" in old:
            golden["cfg2"] = old["cfg2"]


if __name__ == "__main__":
    main()
