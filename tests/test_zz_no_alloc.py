"""lfgpu_residual_norm_noalloc: the allocation-free residual norm (static device
scratch) against the residual lfgpu_solve reports, through the C ABI.

The inputs live in device memory the caller owns (torch CUDA tensors here); the
entry point itself allocates nothing.  Bar: 1e-12 relative, the bar the assembly
parity tests use; the per-row arithmetic is the same as the solve's own true
residual and only the order of the final sum of squares differs.
"""

import numpy as np
import pytest

from lightfem_gb300 import mesh
from lightfem_gb300.solver import upload_model

RTOL = 1e-12


def test_rejects_systems_beyond_the_scratch(native):
    """Sizes above the static scratch are refused before any device work."""
    with pytest.raises(native.GpuError, match="static scratch limit"):
        native.residual_norm_noalloc(native.NOALLOC_MAX_ROWS + 1, None, None, None, None, None)


# 160x48 elements: 15,778 rows, 247 blocks of 64 rows, so the last block's final
# sum reads each partial in one pass.  400x100: 81,002 rows, 1,266 blocks, so
# every thread of the last block adds several partials.
@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny", [(160, 48), (400, 100)])
def test_matches_solve_true_residual_on_consecutive_calls(native, nx, ny):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    model = mesh.cantilever(nx, ny)
    model.sort_and_index()
    ctx = native.Context(0)
    upload_model(ctx, model)
    ctx.assemble("coloring")
    ctx.apply_dirichlet()
    u_host, rep = ctx.solve(ctx.options(tolerance=1e-10, max_iterations=100000))
    assert rep.converged

    rp, col, _, _ = ctx.download_pattern()
    dev = torch.device("cuda", 0)
    rowptr = torch.from_numpy(rp.astype(np.int32)).to(dev)
    cols = torch.from_numpy(col).to(dev)
    vals = torch.from_numpy(ctx.download(native.K_CONSTRAINED)).to(dev)
    f = torch.from_numpy(ctx.download(native.F_CONSTRAINED)).to(dev)
    u = torch.from_numpy(u_host).to(dev)
    zero = torch.zeros_like(u)
    n = ctx.n_dofs
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()

    def norm(x, s=None):
        return native.residual_norm_noalloc(n, rowptr.data_ptr(), cols.data_ptr(), vals.data_ptr(), x.data_ptr(),
                                            f.data_ptr(), None if s is None else s.cuda_stream)

    first = norm(u)
    second = norm(zero, stream)  # ||f - K 0|| = ||f||, the solve's initial residual
    third = norm(u, stream)
    assert rep.true_residual > 0.0
    assert abs(first - rep.true_residual) <= RTOL * rep.true_residual
    assert abs(second - rep.initial_residual) <= RTOL * rep.initial_residual
    assert third == first  # the scratch carries nothing from one call into the next


@pytest.mark.gpu
def test_empty_system(native):
    assert native.residual_norm_noalloc(0, None, None, None, None, None) == 0.0
