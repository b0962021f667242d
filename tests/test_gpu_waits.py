"""Bounded device-side waits: a wait that runs out ends the call with
LFGPU_ERR_TIMEOUT instead of hanging, and the handle stays usable.

Every spin-wait of the kernels (the persistent solver's grid barrier, the mixed
update's wait for beta, the IC(0) sweeps' operand polls, the level sweeps'
mbarrier waits) gives up after the handle's wait limit, records
LFGPU_ERR_TIMEOUT, raises the abort flag that ends every other wait, and lets its
kernel run to the end.  The limit is a handle
option (LFGPU_OPTION_WAIT_LIMIT_NS, 4 s by default); here it is set to 1 ns, so
the first wait that has to spin at all runs out.  Nothing is faulted, trapped or
hung: the waits end on their own limit, on waits the kernels make in every solve.

The level sweeps' waits are not made to run out here.  A CTA of the sweep's
cluster that gave up no longer knows which of its peers' stores into its shared
memory are still in flight; it waits for its peers at a cluster barrier and then
a grace period before it exits, which bounds the path but does not prove it safe,
so it is not exercised on a shared GPU.

The reference has no device waits; a solve that ends this way maps to the
runtime_error path of src/main.cpp:162-164 like its other PCG failures
(src/solver.cpp:579-593).
"""

import numpy as np
import pytest

from cases import CASES, indexed
from conftest import load_golden
from lightfem_gb300 import mesh
from lightfem_gb300.solver import upload_model

pytestmark = pytest.mark.gpu

SHORT_NS = 1


def _system(native, model):
    model = indexed(model)
    if model.settings.reordering == "rcm":
        model.index_with_node_order(native.host_rcm(model.node_ids, model.element_nodes))
    ctx = native.Context(0)
    upload_model(ctx, model)
    ctx.assemble("coloring")
    ctx.apply_dirichlet()
    return model, ctx


def _expect_timeout(native, ctx, options):
    with pytest.raises(native.GpuError) as err:
        ctx.solve(options)
    assert err.value.code == native.ERR_TIMEOUT, str(err.value)
    status, index, aborted, _ = ctx.failure_detail()
    assert status == native.ERR_TIMEOUT
    assert aborted == 1.0  # the wait raised the abort flag that stops every other wait
    return index


def _solves_grid6_after(native, ctx, golden_json):
    """The same handle, back at the default limit, solves grid6 to the reference's
    answer: nothing of the expired waits is left behind."""
    ctx.set_option(native.OPTION_WAIT_LIMIT_NS, 4_000_000_000)
    model = indexed(CASES["grid6"]())
    upload_model(ctx, model)
    ctx.assemble("coloring")
    ctx.apply_dirichlet()
    u, rep = ctx.solve(ctx.options(model.settings.tolerance, model.settings.max_iterations, "csr", "jacobi"))
    ref = golden_json["grid6"]["csr_jacobi"]
    assert rep.converged and abs(rep.iterations - ref["iterations"]) <= 2
    g = load_golden("grid6")
    order = np.argsort(model.node_ids, kind="stable")
    u_by_id = u.reshape(-1, 2)[order].ravel()
    assert np.linalg.norm(u_by_id - g["u_csr_jacobi"]) <= 1e-8 * np.linalg.norm(g["u_csr_jacobi"])


def test_persistent_grid_barrier_expires(native, golden_json):
    """The persistent cooperative solver's grid barrier: with a 1 ns limit the
    first CTA to arrive gives up before the others arrive."""
    model, ctx = _system(native, mesh.workload(1, scale=4))
    ctx.set_option(native.OPTION_WAIT_LIMIT_NS, SHORT_NS)
    index = _expect_timeout(native, ctx, ctx.options(1e-8, 10000, "csr", "jacobi", persistent=1))
    assert index >= 0  # the CTA whose barrier wait ran out
    _solves_grid6_after(native, ctx, golden_json)
    ctx.close()


def test_mixed_update_direction_wait_expires(native, golden_json):
    """The mixed loop's update in its direct form (a pointwise preconditioner on a
    mesh of 150,000 nodes or more): its CTAs wait for the last one's beta before
    they form the next direction; with a 1 ns limit the first CTA to wait gives up
    and the solve ends."""
    model, ctx = _system(native, mesh.workload(2))  # 1000x1000, 1,002,001 nodes
    ctx.set_option(native.OPTION_WAIT_LIMIT_NS, SHORT_NS)
    index = _expect_timeout(native, ctx, ctx.options(1e-8, 10000, "bsr", "jacobi", "mixed"))
    assert index >= 0  # the CTA whose wait ran out
    _solves_grid6_after(native, ctx, golden_json)
    ctx.close()


def test_ic0_polled_sweep_wait_expires(native, golden_json):
    """The dependency-polled IC(0) sweep: a row whose operand lies in an earlier,
    unfinished row chunk polls for it; with a 1 ns limit that poll gives up."""
    model, ctx = _system(native, mesh.workload(2, scale=5))  # 200x200, 80,802 rows in 79 chunks
    ctx.set_option(native.OPTION_IC0_SWEEP, native.IC0_SWEEP["polled"])
    # Factor at the default limit (the factorisation waits on rows too), so that the
    # solve's waits are the sweeps'.
    ctx.apply_preconditioner(ctx.download(native.F_CONSTRAINED), "ic0")
    ctx.set_option(native.OPTION_WAIT_LIMIT_NS, SHORT_NS)
    _expect_timeout(native, ctx, ctx.options(1e-8, 10000, "csr", "ic0"))
    _solves_grid6_after(native, ctx, golden_json)
    ctx.close()


def test_wait_limit_must_be_positive(native):
    ctx = native.Context(0)
    with pytest.raises(native.GpuError) as err:
        ctx.set_option(native.OPTION_WAIT_LIMIT_NS, 0)
    assert err.value.code == native.ERR_ARGUMENT
    ctx.close()
