"""Failure detection of the CUDA path against the reference.

Each of FAILURE_MODELS (tests/cases.py) makes the reference's public solve()
stop, or finish, in one known way: the zero-pivot sweep (src/solver.cpp:920-940),
the Jacobi setup (inverse_diagonal_of, :656-669), the three checks of pcg_solve
(:579-581, :591-593, :616-618) or the "initial residual satisfies tolerance" exit
(:573-578, where sqrt(max(0, NaN)) is 0).  The "failures" entry of golden.json
and tests/golden/failures.npz hold how the reference ended on each; the GPU solve
must end the same way.  Every failure here is a status the kernels set and the
host reads after the launch: none of these cases faults, traps or hangs the GPU.
"""

import numpy as np
import pytest

from cases import ASSEMBLY_FAILURES, FAILURE_DETERMINISTIC, FAILURE_MODELS, assembly_failure_message, by_id_order, \
    failure_case, indexed, outcome_kind
from conftest import load_golden
from lightfem_gb300.solver import LinearElasticSolver

pytestmark = pytest.mark.gpu

_PCG_KINDS = ("rho_initial", "not_spd", "rho")


def gpu_outcome(model, precision="fp64", ref_message=None):
    """How LinearElasticSolver.solve ends: "converged" (with the result) or the
    kind of the reference exception its message carries.  An exception of the
    reference's kind must carry ``ref_message``, the reference's own, character
    for character (the zero-pivot one prints the DOF, its load and diagonal and
    the node)."""
    model.settings.precision = precision
    try:
        return "converged", LinearElasticSolver().solve(model)
    except RuntimeError as err:
        if str(err).startswith("PCG did not converge"):
            return "maxit", None
        kind = outcome_kind(str(err))
        if ref_message is not None and ref_message != "converged" and kind == outcome_kind(ref_message):
            assert str(err) == ref_message
        return kind, None


@pytest.mark.parametrize("storage", ["csr", "bsr"])
@pytest.mark.parametrize("precond", ["jacobi", "block", "ic0"])
@pytest.mark.parametrize("name", list(FAILURE_MODELS))
def test_fp64_failure_matches_reference(native, golden_json, name, precond, storage):
    ref = golden_json["failures"][name][f"{storage}_{precond}"]
    want = outcome_kind(ref["outcome"])
    model = failure_case(name, storage, precond)
    got, res = gpu_outcome(model, ref_message=ref["outcome"])
    assert got == want
    if want != "converged":
        return
    assert abs(res.solver.iterations - ref["iterations"]) <= 2
    u_ref = load_golden("failures")[f"{name}__{storage}_{precond}"]
    u = by_id_order(model, res.displacement)
    assert np.linalg.norm(u - u_ref) <= 1e-8 * np.linalg.norm(u_ref) or np.array_equal(u, u_ref)


@pytest.mark.parametrize("storage", ["csr", "bsr"])
@pytest.mark.parametrize("precond", ["jacobi", "block"])
@pytest.mark.parametrize("name", list(FAILURE_MODELS))
def test_mixed_failure_matches_reference(native, golden_json, name, precond, storage):
    """The FP32-inner solve ends as the FP64 reference does where the outcome is
    fixed at the start.  On an indefinite K (negative modulus) where breakdown comes
    later, it must either break down with one of pcg_solve's errors or reach the
    FP64 target on the true residual."""
    ref = golden_json["failures"][name][f"{storage}_{precond}"]
    want = outcome_kind(ref["outcome"])
    model = failure_case(name, storage, precond)
    got, res = gpu_outcome(model, precision="mixed", ref_message=ref["outcome"])
    if name in FAILURE_DETERMINISTIC or want == "converged":
        assert got == want
    else:
        assert got in ("converged", *_PCG_KINDS)
    if got == "converged" and np.all(np.isfinite(model.load_fy)):
        target = model.settings.tolerance * max(1.0, res.solver.initial_residual)
        assert res.solver.true_residual <= 1.2 * target


@pytest.mark.parametrize("name", list(ASSEMBLY_FAILURES))
def test_assembly_failure_message(native, golden_json, name):
    """A clockwise element and a zero-length loaded edge stop the assembly with
    the reference's exception text; for edges, the kind of the first failing
    record in record order names it.  (Where the reference's OpenMP region turns
    the Jacobian exception into std::terminate, the GPU path raises it.)"""
    with pytest.raises(RuntimeError) as err:
        LinearElasticSolver().solve(indexed(ASSEMBLY_FAILURES[name]()))
    assert str(err.value) == assembly_failure_message(golden_json, name)


@pytest.mark.parametrize("precond", ["jacobi", "block"])
def test_mixed_direct_form_indefinite(native, precond):
    """From 150,000 nodes on the mixed loop runs in its direct form, where every CTA
    of the update forms alpha from the product's per-CTA p.q pairs and the update
    makes pcg_solve's curvature check (src/solver.cpp:591-593).  On the 1000x1000
    cantilever with one element's modulus at -10x the others (an indefinite K)
    the solve must end with one of pcg_solve's errors, not run on or stall."""
    from lightfem_gb300 import mesh
    from lightfem_gb300.solver import upload_model

    m = mesh.workload(2)
    ne = m.element_ids.shape[0]
    young = np.full(ne, 70.0e9)
    young[ne // 2 + 500] = -7.0e11
    m.material_ids = np.arange(1, ne + 1)
    m.young, m.poisson, m.thickness = young, np.full(ne, 0.33), np.full(ne, 0.01)
    m.element_material = np.arange(1, ne + 1)
    m.sort_and_index()
    m.index_with_node_order(native.host_rcm(m.node_ids, m.element_nodes))
    ctx = native.Context(0)
    upload_model(ctx, m)
    ctx.assemble("coloring")
    ctx.apply_dirichlet()
    with pytest.raises(native.GpuError) as err:
        ctx.solve(ctx.options(1e-8, 200000, "bsr", precond, "mixed"), download=False)
    assert err.value.code in (native.ERR_NOT_SPD, native.ERR_RHO), str(err.value)
    ctx.close()
