"""The C ABI library loads and exports every entry point include/lfgpu.h declares;
host-only entry points work without a GPU.  CPU only: no compute call needs CUDA."""

import ctypes
import os
import re

import numpy as np

from cases import CASES, indexed
from conftest import ROOT, load_golden


def declared_functions():
    text = open(os.path.join(ROOT, "include", "lfgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(lfgpu_\w+)\s*\(", text, re.M)))


def test_header_and_binding_agree(native):
    declared = declared_functions()
    assert len(declared) >= 20
    assert set(declared) == set(native.EXPORTED)


def test_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(native.LIB_PATH)
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert native.library().lfgpu_version().decode().startswith("lfgpu")


def test_host_rcm_matches_reference(native):
    for name in ("strain",):
        g = load_golden(name)
        model = indexed(CASES[name]())
        order = native.host_rcm(model.node_ids, model.element_nodes)
        np.testing.assert_array_equal(order, g["node_order"])
    g = load_golden("scrambled")
    model = indexed(CASES["scrambled"]())
    np.testing.assert_array_equal(native.host_rcm(model.node_ids, model.element_nodes), g["rcm_node_order"])


def test_host_rcm_rejects_unknown_node(native):
    import pytest
    with pytest.raises(native.GpuError):
        native.host_rcm(np.array([1, 2, 3, 4]), np.array([[1, 2, 3, 99]]))


def test_create_without_gpu_fails_cleanly(native):
    """Without a visible device the handle refuses to open (no silent fallback)."""
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    with pytest.raises(native.GpuError):
        native.Context(0)


def test_host_subdomains_match_oracle(native, oracle):
    """The library's node split (split_by_chunks / split_by_coordinates,
    src/precond.cpp:19-105) equals the oracle's, ties between equal coordinates
    included, on structured, perturbed and reordered meshes."""
    from lightfem_gb300 import mesh
    meshes = [indexed(CASES[name]()) for name in ("grid6", "beam", "strain")]
    meshes.append(indexed(mesh.workload(1)))
    for model in meshes:
        for per in (1, 2, 3, 7, 64, 100):
            for split in ("rcb", "chunk"):
                got, n_got = native.host_subdomains(model.xy, per, split)
                want, n_want = oracle.subdomain_split(model.xy, per, split)
                assert n_got == n_want
                np.testing.assert_array_equal(got, want)


def test_host_subdomains_rejects_bad_arguments(native):
    import ctypes
    import pytest
    lib = native.library()
    xy = np.zeros((4, 2))
    owner = np.empty(4, np.uint32)
    count = ctypes.c_int64()
    for per, split in ((0, 0), (-3, 1), (4, 2), (4, -1)):
        rc = lib.lfgpu_host_subdomains(4, xy.ctypes.data, per, split, owner.ctypes.data, ctypes.byref(count))
        assert rc == native.ERR_ARGUMENT, (per, split)
    with pytest.raises(KeyError):
        native.host_subdomains(xy, 4, "metis")


def test_block_setting_maps_to_library_preconditioner():
    """`preconditioner block` with subdomain_nodes 1 is the fused 2x2 nodal form;
    any other size (the reference's default is 64) is the general subdomain form."""
    from lightfem_gb300.model import SolverSettings
    from lightfem_gb300.solver import gpu_preconditioner
    assert gpu_preconditioner(SolverSettings(preconditioner="block", subdomain_nodes=1)) == "block"
    assert gpu_preconditioner(SolverSettings(preconditioner="block")) == "subdomain"
    assert gpu_preconditioner(SolverSettings(preconditioner="block", subdomain_nodes=7)) == "subdomain"
    assert gpu_preconditioner(SolverSettings(preconditioner="jacobi", subdomain_nodes=7)) == "jacobi"
    assert gpu_preconditioner(SolverSettings(preconditioner="ic0")) == "ic0"
