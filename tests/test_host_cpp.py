"""The C++ host layer (lightfem_gb300/host/) on the CPU: it compiles against
liblfgpu and against the reference's own types, keeps the reference's host-side
errors, and stops with a run-time error where the library finds no device (no
fallback)."""

import os
import subprocess

import pytest

from cases import grid6
from host_cpp import ROOT, compile_driver, run


@pytest.fixture(scope="module")
def driver(native, tmp_path_factory):
    return compile_driver(str(tmp_path_factory.mktemp("host")))


def test_binding_compiles_against_reference_types():
    """tests/host/reference_binding.cpp instantiates the solve template with
    lightfem::Model and lightfem::AnalysisResult (include/lightfem/model.hpp,
    include/lightfem/solver.hpp)."""
    from oracle.reference import make_args

    out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "tests", "host"), "binding-check", *make_args()],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    if "unavailable" in out.stdout:
        pytest.skip("the reference's headers are not mounted here")
    assert "binding compiled" in out.stdout


def test_duplicate_node_id(driver, tmp_path):
    """Model::sort_and_index (src/model.cpp:13-21, 24-39): std::logic_error."""
    m = grid6()
    m.node_ids[5] = m.node_ids[4]
    kind, message, _ = run(driver, m, str(tmp_path))
    assert (kind, message) == ("logic_error", f"duplicate node ID: {int(m.node_ids[4])}")


def test_unindexed_model(driver, tmp_path):
    """LinearElasticSolver::solve (src/solver.cpp:875-878)."""
    kind, message, _ = run(driver, grid6(), str(tmp_path), index=False)
    assert (kind, message) == ("logic_error", "model must pass validation and sort_and_index before solving")


def test_truss_model_keeps_the_cpu_path(driver, tmp_path):
    kind, message, _ = run(driver, grid6(), str(tmp_path), extra_lines=("truss 1 1 2 1 0.01",))
    assert kind == "invalid_argument" and "truss" in message


def test_unknown_node_in_element(driver, tmp_path):
    """A Q4 element naming a missing node (q4_dof_indices, src/element.cpp:120-123),
    found on the host before a device is opened."""
    m = grid6()
    m.element_nodes[3, 2] = 10_000
    kind, message, _ = run(driver, m, str(tmp_path))
    assert (kind, message) == ("logic_error", "validated Q4 element references an unknown node")


def test_unknown_node_in_boundary(driver, tmp_path):
    """collect_constraints (src/solver.cpp:343-345)."""
    m = grid6()
    m.bc_node[0] = 10_000
    kind, message, _ = run(driver, m, str(tmp_path))
    assert (kind, message) == ("logic_error", "validated boundary references an unknown node")


def test_without_a_device_the_solve_stops(driver, tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    kind, message, _ = run(driver, grid6(), str(tmp_path))
    assert kind == "runtime_error" and message.startswith("lfgpu_create failed")
