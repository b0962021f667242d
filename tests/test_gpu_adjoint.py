"""The adjoint behind torch.autograd.Function on the 400x400 log-normal-modulus
cantilever (321,602 DOFs, 160,000 element moduli), through the C ABI.

Bars:
* against the CPU FP64 reference gradient (the oracle's PCG solves of K u = f and
  K lambda = e_tip, then its own element loop): 1e-6 relative (2-norm over all
  elements), for compliance and for the tip-node y displacement;
* against central finite differences with a 1e-6 relative step on 64 seeded
  random elements.  Finite differences of FP64 solves carry the rounding of the
  assembled K(E +/- h), whose effect on J does not shrink with the solver
  tolerance; it dominates for elements with little strain energy.  So the bar is
  5e-3 of the largest sensitivity among the 64 per element and 1e-2 relative
  over the 64 together.
"""

import numpy as np
import pytest

from lightfem_gb300 import mesh

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-10


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def cfg4(native):
    from lightfem_gb300.adjoint import ElasticProblem
    model = mesh.workload(4)
    model.sort_and_index()
    problem = ElasticProblem(model, tolerance=TOL, max_iterations=200000)
    tip = problem.dof(mesh.tip_node_id(problem.model), 1)
    yield problem, tip
    problem.close()


@pytest.fixture(scope="module")
def cpu_reference(cfg4, oracle):
    problem, tip = cfg4
    m = problem.model.copy()
    m.settings.reordering = "none"  # already in the problem's node order
    out = oracle.solve_model(m, tolerance=TOL, max_iterations=200000)
    assert out["report"]["converged"]
    en = m.element_node_index()
    mi = m.material_index(m.element_material)
    args = (m.xy, en, m.young[mi], m.poisson[mi], m.thickness[mi], m.settings.plane_mode)
    u = out["u"]
    dj = np.zeros(problem.n_dofs)
    dj[tip] = 1.0
    dj[out["constraint_dofs"]] = 0.0
    lam, rep = oracle.pcg(out["rowptr"], out["col"], out["Kc"], dj, TOL, 200000)
    assert rep["converged"]
    return {"u": u, "f": out["f"], "dc": oracle.adjoint_grad(*args, u, u), "dtip": oracle.adjoint_grad(*args, u, lam)}


def test_compliance_gradient_matches_cpu_reference(cfg4, cpu_reference):
    from lightfem_gb300.adjoint import compliance
    problem, _ = cfg4
    young = torch.tensor(problem.young0, dtype=torch.float64, requires_grad=True)
    c = compliance(young, problem)
    c.backward()
    ref_c = float(cpu_reference["f"] @ cpu_reference["u"])
    assert abs(c.item() - ref_c) <= 1e-8 * abs(ref_c)
    assert rel(young.grad.numpy(), cpu_reference["dc"]) <= 1e-6
    assert problem.adjoint_report.iterations == 0  # self-adjoint: no second solve


def test_tip_gradient_matches_cpu_reference(cfg4, cpu_reference):
    from lightfem_gb300.adjoint import displacements
    problem, tip = cfg4
    young = torch.tensor(problem.young0, dtype=torch.float64, requires_grad=True)
    u = displacements(young, problem)
    assert rel(u.detach().numpy(), cpu_reference["u"]) <= 1e-8
    u[tip].backward()
    assert problem.adjoint_report.converged and problem.adjoint_report.iterations > 0
    assert rel(young.grad.numpy(), cpu_reference["dtip"]) <= 1e-6


def test_general_objective_chains_through_autograd(cfg4):
    """J = w.u + (u_tip)^2: torch forms dJ/du, one adjoint solve maps it to dJ/dE."""
    from lightfem_gb300.adjoint import displacements
    problem, tip = cfg4
    w = torch.from_numpy(np.random.default_rng(5).standard_normal(problem.n_dofs))
    young = torch.tensor(problem.young0, dtype=torch.float64, requires_grad=True)
    u = displacements(young, problem)
    j = (w * u).sum() + u[tip] ** 2
    j.backward()
    dj_du = w.numpy().copy()
    dj_du[tip] += 2.0 * u[tip].item()
    problem.ensure_solution(problem.young0)
    direct = problem.gradient(dj_du)
    assert rel(young.grad.numpy(), direct) <= 1e-12


def test_gradients_match_central_differences(cfg4):
    from lightfem_gb300.adjoint import ElasticProblem, compliance, displacements
    problem, tip = cfg4
    y0 = problem.young0.copy()
    young = torch.tensor(y0, dtype=torch.float64, requires_grad=True)
    compliance(young, problem).backward()
    dc = young.grad.numpy().copy()
    young = torch.tensor(y0, dtype=torch.float64, requires_grad=True)
    displacements(young, problem)[tip].backward()
    dtip = young.grad.numpy().copy()

    model = mesh.workload(4)
    model.sort_and_index()
    fd = ElasticProblem(model, tolerance=1e-11, max_iterations=200000)
    fd.solve(y0)
    f = fd.load()
    elements = np.random.default_rng(64).choice(problem.n_elements, 64, replace=False)
    fd_c, fd_t = [], []
    for e in elements:
        h = 1e-6 * y0[e]
        yp, ym = y0.copy(), y0.copy()
        yp[e] += h
        ym[e] -= h
        up = fd.solve(yp)
        um = fd.solve(ym)
        fd_c.append((f @ up - f @ um) / (2.0 * h))
        fd_t.append((up[tip] - um[tip]) / (2.0 * h))
    fd.close()
    for got, want in ((np.array(fd_c), dc[elements]), (np.array(fd_t), dtip[elements])):
        assert np.all(np.abs(got - want) <= 5e-3 * np.abs(want).max())
        assert rel(got, want) <= 1e-2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_subdomain_preconditioner_gradient(cfg4, cpu_reference, precision):
    """The forward and adjoint solves with the reference's default block
    preconditioner (64-node RCB subdomains) give the same tip-displacement
    gradient as the CPU FP64 reference."""
    from lightfem_gb300.adjoint import ElasticProblem, displacements
    problem, tip = cfg4
    model = problem.model.copy()
    model.settings.reordering = "none"  # the problem's model is already reordered
    model.settings.preconditioner, model.settings.subdomain_nodes, model.settings.subdomain_split = "block", 64, "rcb"
    sub = ElasticProblem(model, precision=precision, tolerance=TOL, max_iterations=200000)
    try:
        young = torch.tensor(sub.young0, dtype=torch.float64, requires_grad=True)
        u = displacements(young, sub)
        assert rel(u.detach().numpy(), cpu_reference["u"]) <= 1e-7
        u[tip].backward()
        assert sub.report.subdomains > 0 and sub.adjoint_report.converged
        assert rel(young.grad.numpy(), cpu_reference["dtip"]) <= 1e-6
    finally:
        sub.close()
