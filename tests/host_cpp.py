"""Drive the C++ host layer (lightfem_gb300/host/lightfem_gpu_solve.hpp) from the tests:
compile tests/host/solve_model.cpp against liblfgpu, write a model in its line
format, run it and read back what it wrote."""

from __future__ import annotations

import os
import subprocess

import numpy as np

from lightfem_gb300.model import EDGE_PRESSURE, PLANE_STRAIN, Model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "lightfem_gb300", "_lib")


def compile_driver(out_dir: str) -> str:
    """g++ the driver; liblfgpu.so must already be built."""
    exe = os.path.join(out_dir, "solve_model")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "lightfem_gb300", "host"),
           os.path.join(ROOT, "tests", "host", "solve_model.cpp"), "-L", LIB_DIR, "-llfgpu",
           f"-Wl,-rpath,{LIB_DIR}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _num(x: float) -> str:
    return repr(float(x))


def write_model(model: Model, path: str) -> None:
    """The model's records in the default line format (IDs as given, unsorted)."""
    s = model.settings
    mixed = getattr(s, "precision", "fp64") == "mixed"
    atomic = s.assembly == "atomic" or getattr(s, "gpu_assembly", "coloring") == "atomic"
    lines = [
        f"setting plane_mode {'strain' if s.plane_mode == PLANE_STRAIN else 'stress'}",
        f"setting solver {'gpu_mixed' if mixed else 'gpu'}",
        f"setting tolerance {_num(s.tolerance)}",
        f"setting max_iterations {int(s.max_iterations)}",
        f"setting reordering {s.reordering}",
        f"setting assembly {'atomic' if atomic else 'gpu'}",
        f"setting storage {s.storage}",
        f"setting preconditioner {s.preconditioner}",
        f"setting subdomain_split {s.subdomain_split}",
        f"setting subdomain_nodes {int(s.subdomain_nodes)}",
    ]
    for i, (x, y) in zip(model.node_ids, model.xy):
        lines.append(f"node {int(i)} {_num(x)} {_num(y)}")
    for i, e, nu, t in zip(model.material_ids, model.young, model.poisson, model.thickness):
        lines.append(f"material {int(i)} {_num(e)} {_num(nu)} {_num(t)}")
    for i, nodes, mat in zip(model.element_ids, model.element_nodes, model.element_material):
        lines.append(f"q4 {int(i)} {' '.join(str(int(n)) for n in nodes)} {int(mat)}")
    for n, ux, uy in zip(model.bc_node, model.bc_ux, model.bc_uy):
        lines.append(f"fix {int(n)} {'-' if np.isnan(ux) else _num(ux)} {'-' if np.isnan(uy) else _num(uy)}")
    for n, fx, fy in zip(model.load_node, model.load_fx, model.load_fy):
        lines.append(f"load {int(n)} {_num(fx)} {_num(fy)}")
    for e, bx, by in zip(model.body_element, model.body_bx, model.body_by):
        lines.append(f"body {int(e)} {_num(bx)} {_num(by)}")
    for e, side, kind, a, b in zip(model.edge_element, model.edge_side, model.edge_kind, model.edge_first,
                                   model.edge_second):
        lines.append(f"edge {int(e)} {int(side)} {'pressure' if kind == EDGE_PRESSURE else 'traction'} "
                     f"{_num(a)} {_num(b)}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def run(exe: str, model: Model, work_dir: str, extra_lines: tuple[str, ...] = (), index: bool = True):
    """Solve ``model`` through the C++ layer.  Returns (kind, message, result):
    kind "converged" with a dict of the written arrays and report, or the
    exception kind with its message and None."""
    os.makedirs(work_dir, exist_ok=True)
    path = os.path.join(work_dir, "model.txt")
    write_model(model, path)
    if extra_lines:
        with open(path, "a") as fh:
            fh.write("\n".join(extra_lines) + "\n")
    cmd = [exe, path, work_dir] + ([] if index else ["--no-index"])
    subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=600)
    with open(os.path.join(work_dir, "outcome.txt")) as fh:
        outcome = fh.read()
    if outcome != "converged":
        kind, _, message = outcome.partition("\t")
        return kind, message, None
    out = {}
    for name, dtype in (("node_ids", np.int64), ("u", np.float64), ("R", np.float64), ("f", np.float64),
                        ("K", np.float64), ("row_offsets", np.uint64), ("columns", np.uint64),
                        ("element_fields", np.float64), ("node_stress", np.float64)):
        out[name] = np.fromfile(os.path.join(work_dir, f"{name}.bin"), dtype=dtype)
    report = {}
    with open(os.path.join(work_dir, "report.txt")) as fh:
        for line in fh:
            key, _, value = line.rstrip("\n").partition(" ")
            report[key] = value
    out["report"] = report
    return "converged", "", out


def id_order(node_ids: np.ndarray, v: np.ndarray) -> np.ndarray:
    """A DOF vector in the driver's node order, put in node-ID order."""
    order = np.argsort(node_ids, kind="stable")
    out = np.empty_like(v)
    out[0::2] = v[2 * order]
    out[1::2] = v[2 * order + 1]
    return out
