"""``LinearElasticSolver.solve(model) -> AnalysisResult`` on the GPU.

Mirrors the reference's top-level solve (``LinearElasticSolver::solve``,
src/solver.cpp:875-960) stage by stage, with every numeric stage running in
liblfgpu through the C ABI:

    reordering (RCM, src/solver.cpp:886-892)        lfgpu_rcm (device)
    pattern + map + colours (src/solver.cpp:228-235) lfgpu_build_pattern (device; colours on a host thread)
    element stiffness + assembly + loads             lfgpu_assemble
    retain K, f; Dirichlet; zero-pivot sweep         lfgpu_apply_dirichlet
    solve_iterative (src/solver.cpp:675-747)         lfgpu_solve
    reactions (src/solver.cpp:953-954)               lfgpu_reactions
    postprocess + smoothing (src/solver.cpp:756-871) lfgpu_postprocess

Errors keep the reference's wording and exception kinds: a failed solve raises
``RuntimeError`` with the message ``pcg_solve`` throws, non-convergence raises
``RuntimeError("PCG did not converge: ...")`` (src/solver.cpp:948-950).
VTK/CSV output stays with the reference host library.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .model import EDGE_PRESSURE, Model


@dataclass
class CsrMatrix:
    row_offsets: np.ndarray
    column_indices: np.ndarray
    values: np.ndarray

    def rows(self) -> int:
        return self.row_offsets.shape[0] - 1

    def nonzeros(self) -> int:
        return self.values.shape[0]


@dataclass
class LinearSolverReport:
    """``LinearSolverReport`` (include/lightfem/solver.hpp:12-34) plus GPU fields."""

    converged: bool = False
    iterations: int = 0
    initial_residual: float = 0.0
    final_residual: float = 0.0
    message: str = ""
    preconditioner: str = "jacobi"
    solve_ms: float = 0.0
    matvec_ms: float = 0.0
    matvec_calls: int = 0
    storage: str = "csr"
    matrix_bytes_per_matvec: int = 0
    storage_convert_ms: float = 0.0
    preconditioner_setup_ms: float = 0.0
    preconditioner_apply_ms: float = 0.0
    subdomains: int = 0
    capture_ratio: float = 0.0
    precision: str = "fp64"
    refinements: int = 0
    true_residual: float = 0.0
    fallback_fp64: bool = False
    ic0_breakdowns: int = 0


@dataclass
class CsrProfile:
    """``CsrProfile`` (include/lightfem/sparse.hpp:103-108)."""

    dimension: int = 0
    nonzeros: int = 0
    bandwidth: int = 0
    profile: int = 0


@dataclass
class PerformanceReport:
    reordering: str = "none"
    before: CsrProfile = field(default_factory=CsrProfile)
    after: CsrProfile = field(default_factory=CsrProfile)
    rcm_ms: float = 0.0
    assembly: str = "coloring"
    coloring_count: int = 0
    pattern_ms: float = 0.0
    element_stiffness_ms: float = 0.0
    assembly_ms: float = 0.0
    boundary_ms: float = 0.0
    retain_matrix_ms: float = 0.0
    postprocess_ms: float = 0.0
    total_ms: float = 0.0


@dataclass
class AnalysisResult:
    """``AnalysisResult`` (include/lightfem/solver.hpp:76-86).  ``element_results``
    is E x 5 x 7 in element order: the centre, then the Gauss points (-g,-g),
    (g,-g), (g,g), (-g,g), each strain xx, yy, xy, stress xx, yy, xy, von Mises
    (ElementResult); ``node_results`` is N x 4 in node order: smoothed stress xx,
    yy, xy and von Mises (NodeResult)."""

    stiffness: CsrMatrix | None
    load: np.ndarray
    displacement: np.ndarray
    reaction: np.ndarray
    solver: LinearSolverReport
    performance: PerformanceReport = field(default_factory=PerformanceReport)
    element_results: np.ndarray | None = None
    node_results: np.ndarray | None = None


_MESSAGES = {
    _native.ERR_NONFINITE_DIAG: "Jacobi preconditioner encountered a non-finite diagonal",
    _native.ERR_NOT_SPD: "PCG encountered non-positive curvature; system is not SPD",
    _native.ERR_RHO_INITIAL: "PCG failed to form a positive initial preconditioned residual",
    _native.ERR_RHO: "PCG preconditioned residual became non-positive or non-finite",
}


def c_fixed(x: float) -> str:
    """``std::to_string(double)``: printf's ``%f``, with C's spelling of NaN and
    infinity."""
    if math.isnan(x):
        return "-nan" if math.copysign(1.0, x) < 0 else "nan"
    if math.isinf(x):
        return "-inf" if x < 0 else "inf"
    return f"{x:f}"


def mechanism_message(ctx: _native.Context, model: Model) -> str:
    """The zero-pivot exception of src/solver.cpp:926-936, from the DOF, load and
    diagonal the library reports and the node's ID and coordinates."""
    _, dof, load, diag = ctx.failure_detail()
    node = dof // 2
    return ("the structure is a mechanism: a bar end has no transverse stiffness but carries a transverse load; "
            f"add a support there or load the bar along its axis [dof {dof} load {c_fixed(load)} diag "
            f"{c_fixed(diag)} node {int(model.node_ids[node])} xy {c_fixed(float(model.xy[node, 0]))},"
            f"{c_fixed(float(model.xy[node, 1]))}]")


def edge_message(model: Model) -> str | None:
    """q4_edge_traction / q4_edge_pressure's exception (src/element.cpp:189, :206)
    for the first loaded edge of zero length in record order, as the reference
    meets them; None if the host finds none."""
    if not model.edge_element.size:
        return None
    nodes = model.element_node_index()
    elems = model.element_index(model.edge_element)
    for k in range(elems.shape[0]):
        side = int(model.edge_side[k])
        if not 1 <= side <= 4:
            continue
        a, b = model.xy[nodes[elems[k], side - 1]], model.xy[nodes[elems[k], side % 4]]
        if not math.hypot(b[0] - a[0], b[1] - a[1]) > 1.0e-14:
            kind = "pressure" if int(model.edge_kind[k]) == EDGE_PRESSURE else "traction"
            return f"Q4 edge {kind} received a zero-length edge"
    return None


def gpu_preconditioner(settings) -> str:
    """The library preconditioner for a reference setting: ``block`` with
    ``subdomain_nodes 1`` is the 2x2 nodal form fused into the loop kernels; any
    other size is the general subdomain block-Jacobi (``set_subdomains``)."""
    if settings.preconditioner == "block" and int(settings.subdomain_nodes) != 1:
        return "subdomain"
    return settings.preconditioner


def solve_options(settings) -> _native.SolveOptions:
    return _native.Context.options(settings.tolerance, settings.max_iterations, settings.storage,
                                   gpu_preconditioner(settings), settings.precision, settings.refinement)


def set_mesh(ctx: _native.Context, model: Model) -> None:
    """Nodes, elements and materials of an indexed model into ``ctx``."""
    ctx.set_mesh(model.xy, model.element_node_index(), model.material_index(model.element_material), model.young,
                 model.poisson, model.thickness, model.settings.plane_mode)


def rcm_order(ctx: _native.Context, model: Model) -> np.ndarray:
    """reverse_cuthill_mckee (src/reordering.cpp:11-62) on the device: node IDs in
    the new order.  The model must be in ascending-ID node order (sort_and_index),
    which is how the reference ranks ties."""
    set_mesh(ctx, model)
    return model.node_ids[ctx.rcm()]


def upload_model(ctx: _native.Context, model: Model) -> None:
    """Mesh, pattern, loads and constraints of an indexed model into ``ctx``."""
    set_mesh(ctx, model)
    ctx.build_pattern()
    body_e = model.element_index(model.body_element) if model.body_element.size else None
    edge_e = model.element_index(model.edge_element) if model.edge_element.size else None
    ctx.set_loads(model.nodal_load_vector(), body_e, model.body_bx, model.body_by, edge_e, model.edge_side,
                  model.edge_kind, model.edge_first, model.edge_second)
    dofs, vals = model.constraints()
    ctx.set_constraints(dofs, vals)


class LinearElasticSolver:
    """GPU drop-in for ``lightfem::LinearElasticSolver`` (include/lightfem/solver.hpp:89-92)."""

    def __init__(self, device: int = 0, retain_matrix: bool = True, postprocess: bool = True):
        self.device = device
        self.retain_matrix = retain_matrix
        self.postprocess = postprocess
        self.context: _native.Context | None = None

    def solve(self, model: Model) -> AnalysisResult:
        if not model.indexed:
            raise RuntimeError("model must pass validation and sort_and_index before solving")
        t0 = time.perf_counter()
        s = model.settings
        perf = PerformanceReport(reordering=s.reordering)
        if self.context is None:
            self.context = _native.Context(self.device)
        ctx = self.context
        if s.reordering == "rcm":
            set_mesh(ctx, model)
            perf.before = CsrProfile(**ctx.mesh_profile())
            model.index_with_node_order(model.node_ids[ctx.rcm()])
            perf.rcm_ms = ctx.timings()["rcm_ms"]
        upload_model(ctx, model)
        perf.after = CsrProfile(**ctx.mesh_profile())
        if s.reordering != "rcm":  # as the reference: "before" mirrors "after" without reordering
            perf.before = perf.after
        strategy = "atomic" if s.assembly == "atomic" or s.gpu_assembly == "atomic" else "coloring"
        try:
            ctx.assemble(strategy)
        except _native.GpuError as err:
            if err.code == _native.ERR_JACOBIAN:
                raise RuntimeError("Q4 stiffness evaluation received a non-positive Jacobian") from err
            if err.code == _native.ERR_EDGE:
                raise RuntimeError(edge_message(model) or str(err)) from err
            raise
        try:
            ctx.apply_dirichlet()
        except _native.GpuError as err:
            if err.code == _native.ERR_MECHANISM:
                raise RuntimeError(mechanism_message(ctx, model)) from err
            raise
        if gpu_preconditioner(s) == "subdomain":
            ctx.set_subdomains(s.subdomain_nodes, s.subdomain_split)
        try:
            u, rep = ctx.solve(solve_options(s))
        except _native.GpuError as err:
            raise RuntimeError(_MESSAGES.get(err.code, str(err))) from err
        report = LinearSolverReport(
            converged=bool(rep.converged), iterations=rep.iterations, initial_residual=rep.initial_residual,
            final_residual=rep.final_residual, preconditioner=s.preconditioner, solve_ms=rep.solve_ms,
            matvec_ms=rep.matvec_ms, matvec_calls=rep.matvec_calls, storage=s.storage,
            matrix_bytes_per_matvec=rep.matrix_bytes_per_matvec, storage_convert_ms=rep.storage_convert_ms,
            preconditioner_setup_ms=rep.preconditioner_setup_ms,
            preconditioner_apply_ms=rep.preconditioner_apply_ms, subdomains=rep.subdomains,
            capture_ratio=rep.capture_ratio, precision=s.precision, refinements=rep.refinements,
            true_residual=rep.true_residual, fallback_fp64=bool(rep.fallback_fp64),
            ic0_breakdowns=rep.ic0_breakdowns,
            message="converged" if rep.converged else "maximum iterations reached without convergence")
        if rep.initial_residual <= rep.final_residual and rep.iterations == 0 and rep.converged:
            report.message = "initial residual satisfies tolerance"
        if not report.converged:
            raise RuntimeError("PCG did not converge: " + report.message)
        reaction = ctx.reactions()
        fields = nodal = None
        if self.postprocess:
            try:
                fields, nodal = ctx.postprocess()
            except _native.GpuError as err:
                raise RuntimeError(str(err)) from err
        tm = ctx.timings()
        perf.assembly = strategy
        perf.coloring_count = tm["coloring_count"]
        perf.pattern_ms = tm["pattern_ms"]
        perf.assembly_ms = tm["assembly_ms"]
        perf.boundary_ms = tm["boundary_ms"]
        perf.postprocess_ms = tm["reactions_ms"] + (tm["postprocess_ms"] if self.postprocess else 0.0)
        stiffness = None
        if self.retain_matrix:
            rp, col, _, _ = ctx.download_pattern()
            stiffness = CsrMatrix(rp, col, ctx.download(_native.K_FULL))
        load = ctx.download(_native.F_FULL)
        perf.total_ms = (time.perf_counter() - t0) * 1e3
        return AnalysisResult(stiffness=stiffness, load=load, displacement=u, reaction=reaction, solver=report,
                              performance=perf, element_results=fields, node_results=nodal)
