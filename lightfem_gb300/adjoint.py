"""Sensitivities of the solve path with respect to per-element Young's moduli,
behind ``torch.autograd.Function``.

The reference has no adjoint: this module adds one on top of the same GPU solve.
For K(E) u = f with every element stiffness linear in its modulus
(K_e = E_e * K_e(1), ``q4_stiffness`` src/element.cpp:130-161 scales D by E):

* a displacement objective J(u) has dJ/dE_e = -lambda_e^T K_e u_e / E_e with
  K lambda = dJ/du (dJ/du zeroed on the constrained DOFs, whose displacements are
  prescribed): one extra PCG solve, then the adjoint kernel (lfgpu_adjoint);
* compliance c = f^T u is self-adjoint (lambda = u): dc/dE_e = -u_e^T K_e u_e / E_e
  with no extra solve.

``displacements(young, problem)`` returns u as a differentiable tensor, so any torch
objective of u (a tip displacement, a weighted sum ...) gets its gradient with
respect to all moduli from one adjoint solve.  ``compliance(young, problem)``
returns c directly and differentiates without a solve.  Every call goes through
liblfgpu (ctypes binding of the C ABI); there is no CPU path.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native
from .model import Model
from .solver import gpu_preconditioner, upload_model


class ElasticProblem:
    """A mesh with fixed loads and supports whose element moduli vary.

    Every element gets its own material entry (modulus, Poisson ratio and
    thickness of its original material), so ``young`` has one value per element in
    element-ID order.  DOFs follow the model's node order after the optional RCM
    reordering: node ``k`` of ``node_ids`` owns DOFs ``2k`` and ``2k+1``.

    ``preconditioner`` overrides the model's setting with a library name:
    ``jacobi``, ``block`` (2x2 nodal blocks), ``subdomain`` (the model's
    subdomain_nodes and subdomain_split) or ``ic0``.  Without it the model's
    settings decide, as LinearElasticSolver does.
    """

    def __init__(self, model: Model, *, precision: str | None = None, storage: str | None = None,
                 preconditioner: str | None = None, tolerance: float | None = None,
                 max_iterations: int | None = None, adjoint_tolerance: float | None = None, device: int = 0):
        if not model.indexed:
            raise RuntimeError("model must pass validation and sort_and_index before solving")
        m = model.copy()
        s = m.settings
        if s.reordering == "rcm":
            m.index_with_node_order(_native.host_rcm(m.node_ids, m.element_nodes))
        mi = m.material_index(m.element_material)
        m.young, m.poisson, m.thickness = m.young[mi].copy(), m.poisson[mi].copy(), m.thickness[mi].copy()
        m.material_ids = m.element_ids.copy()
        m.element_material = m.element_ids.copy()
        self.model = m
        self.young0 = m.young.copy()
        self.n_elements = m.n_elements
        self.n_dofs = m.n_dofs
        self.node_ids = m.node_ids
        self.strategy = "atomic" if s.assembly == "atomic" or s.gpu_assembly == "atomic" else "coloring"
        tol = tolerance if tolerance is not None else s.tolerance
        maxit = max_iterations if max_iterations is not None else s.max_iterations
        precond = preconditioner or gpu_preconditioner(s)
        self.options = _native.Context.options(tol, maxit, storage or s.storage, precond,
                                               precision or s.precision, s.refinement)
        self.adjoint_options = _native.Context.options(
            adjoint_tolerance if adjoint_tolerance is not None else tol, maxit, storage or s.storage,
            precond, precision or s.precision, s.refinement)
        _, values = m.constraints()
        self.homogeneous_supports = bool(np.all(np.asarray(values) == 0.0))
        self.ctx = _native.Context(device)
        upload_model(self.ctx, m)
        if precond == "subdomain":
            self.ctx.set_subdomains(s.subdomain_nodes, s.subdomain_split)
        self._solved_for: np.ndarray | None = None
        self.report = None
        self.adjoint_report = None
        self._load: np.ndarray | None = None

    def dof(self, node_id: int, component: int) -> int:
        """DOF index of ``component`` (0 = x, 1 = y) of node ``node_id``."""
        return 2 * int(self.model.node_index([node_id])[0]) + int(component)

    def _check_young(self, young) -> np.ndarray:
        y = np.ascontiguousarray(young, dtype=np.float64).reshape(-1)
        if y.shape[0] != self.n_elements:
            raise ValueError(f"expected {self.n_elements} element moduli, got {y.shape[0]}")
        if not np.all(np.isfinite(y)) or np.any(y <= 0.0):
            raise ValueError("element moduli must be positive and finite")
        return y

    def solve(self, young) -> np.ndarray:
        """Assemble with these moduli, apply the supports and solve; returns u."""
        y = self._check_young(young)
        self.ctx.set_young(y)
        self.ctx.assemble(self.strategy)
        self.ctx.apply_dirichlet()
        u, rep = self.ctx.solve(self.options)
        if not rep.converged:
            raise RuntimeError("PCG did not converge: maximum iterations reached without convergence")
        self.report = rep
        self._solved_for = y.copy()
        return u

    def ensure_solution(self, young) -> None:
        """Re-solve if the device state holds another set of moduli."""
        y = self._check_young(young)
        if self._solved_for is None or not np.array_equal(self._solved_for, y):
            self.solve(y)

    def load(self) -> np.ndarray:
        """The assembled load vector f (moduli do not enter it)."""
        if self._load is None:
            self._load = self.ctx.download(_native.F_FULL)
        return self._load

    def gradient(self, dj_du: np.ndarray | None = None) -> np.ndarray:
        """dJ/dE for the last solve: compliance when ``dj_du`` is None, else the
        objective whose gradient with respect to u is ``dj_du`` (one adjoint solve)."""
        if self._solved_for is None:
            raise RuntimeError("solve before asking for a gradient")
        if dj_du is None and not self.homogeneous_supports:
            raise RuntimeError("the compliance gradient needs zero prescribed displacements")
        g, rep = self.ctx.adjoint(dj_du, None if dj_du is None else self.adjoint_options)
        self.adjoint_report = rep
        return g

    def close(self) -> None:
        self.ctx.close()


def _to_numpy(t: torch.Tensor) -> np.ndarray:
    return t.detach().to("cpu", torch.float64).contiguous().numpy()


class DisplacementFunction(torch.autograd.Function):
    """u(E): forward solves K(E) u = f; backward solves K lambda = grad_u and returns
    -lambda_e^T K_e u_e / E_e for every element."""

    @staticmethod
    def forward(ctx, young: torch.Tensor, problem: ElasticProblem) -> torch.Tensor:
        y = _to_numpy(young)
        u = problem.solve(y)
        ctx.problem = problem
        ctx.young = y
        return torch.from_numpy(u).to(device=young.device, dtype=young.dtype)

    @staticmethod
    def backward(ctx, grad_u: torch.Tensor):
        problem: ElasticProblem = ctx.problem
        problem.ensure_solution(ctx.young)
        g = problem.gradient(_to_numpy(grad_u))
        return torch.from_numpy(g).to(device=grad_u.device, dtype=grad_u.dtype), None


class ComplianceFunction(torch.autograd.Function):
    """c(E) = f^T u(E); backward needs no extra solve (lambda = u)."""

    @staticmethod
    def forward(ctx, young: torch.Tensor, problem: ElasticProblem) -> torch.Tensor:
        y = _to_numpy(young)
        u = problem.solve(y)
        ctx.problem = problem
        ctx.young = y
        c = float(np.dot(problem.load(), u))
        return torch.tensor(c, device=young.device, dtype=young.dtype)

    @staticmethod
    def backward(ctx, grad_c: torch.Tensor):
        problem: ElasticProblem = ctx.problem
        problem.ensure_solution(ctx.young)
        g = problem.gradient(None) * float(grad_c)
        return torch.from_numpy(g).to(device=grad_c.device, dtype=grad_c.dtype), None


def displacements(young: torch.Tensor, problem: ElasticProblem) -> torch.Tensor:
    return DisplacementFunction.apply(young, problem)


def compliance(young: torch.Tensor, problem: ElasticProblem) -> torch.Tensor:
    return ComplianceFunction.apply(young, problem)
