"""The C++ host layer on the GPU: LinearElasticSolver::solve through
lightfem_gpu::solve (lightfem_gb300/host/lightfem_gpu_solve.hpp) reaches the reference's
results, gives the Python host's arrays bit for bit (both drive the same C ABI in
the same stage order), and ends every failure model the reference's way, with
the reference's exception kind and message."""

import numpy as np
import pytest

from cases import ASSEMBLY_FAILURES, CASES, FAILURE_MODELS, VARIANTS, assembly_failure_message, indexed
from conftest import load_golden
from host_cpp import compile_driver, id_order, run
from lightfem_gb300.solver import LinearElasticSolver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(native, tmp_path_factory):
    return compile_driver(str(tmp_path_factory.mktemp("host")))


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def configured(name, variant, precision="fp64"):
    m = CASES[name]()
    storage, precond, split, nodes = VARIANTS[variant]
    m.settings.storage, m.settings.preconditioner = storage, precond
    m.settings.subdomain_split, m.settings.subdomain_nodes = split, nodes
    m.settings.precision = precision
    return m


@pytest.mark.parametrize("variant", ["csr_jacobi", "bsr_block1", "csr_ic0", "bsr_block64"])
@pytest.mark.parametrize("name", ["grid6", "beam", "strain"])
def test_solve_matches_reference_and_python_host(driver, golden_json, name, variant, tmp_path):
    if variant not in golden_json[name]:
        pytest.skip("variant not in the golden set")
    g = load_golden(name)
    ref = golden_json[name][variant]
    kind, message, out = run(driver, configured(name, variant), str(tmp_path))
    assert kind == "converged", message
    rep = out["report"]
    assert abs(int(rep["iterations"]) - ref["iterations"]) <= 2
    assert rel(id_order(out["node_ids"], out["u"]), g[f"u_{variant}"]) <= 1e-8
    assert rel(id_order(out["node_ids"], out["R"]), g[f"R_{variant}"]) <= 1e-8
    assert int(rep["before_bandwidth"]) == ref["bandwidth_before"]
    assert int(rep["after_bandwidth"]) == ref["bandwidth_after"]
    assert int(rep["before_profile"]) == ref["profile_before"]
    assert int(rep["after_profile"]) == ref["profile_after"]
    assert int(rep["after_nonzeros"]) == ref["nnz"]

    model = indexed(configured(name, variant))
    py = LinearElasticSolver().solve(model)
    np.testing.assert_array_equal(out["node_ids"], model.node_ids)
    np.testing.assert_array_equal(out["u"], py.displacement)
    np.testing.assert_array_equal(out["R"], py.reaction)
    np.testing.assert_array_equal(out["f"], py.load)
    np.testing.assert_array_equal(out["K"], py.stiffness.values)
    np.testing.assert_array_equal(out["row_offsets"], py.stiffness.row_offsets)
    np.testing.assert_array_equal(out["columns"], py.stiffness.column_indices)
    np.testing.assert_array_equal(out["element_fields"], py.element_results.reshape(-1))
    np.testing.assert_array_equal(out["node_stress"], py.node_results.reshape(-1))
    assert int(rep["iterations"]) == py.solver.iterations


def test_mixed_precision_reaches_the_fp64_answer(driver, golden_json, tmp_path):
    g = load_golden("beam")
    kind, message, out = run(driver, configured("beam", "bsr_jacobi", precision="mixed"), str(tmp_path))
    assert kind == "converged", message
    assert rel(id_order(out["node_ids"], out["u"]), g["u_bsr_jacobi"]) <= 1e-8


@pytest.mark.parametrize("name", list(FAILURE_MODELS))
def test_failure_ends_as_the_reference(driver, golden_json, name, tmp_path):
    ref = golden_json["failures"][name]["csr_jacobi"]
    m = FAILURE_MODELS[name]()
    m.settings.storage, m.settings.preconditioner = "csr", "jacobi"
    kind, message, out = run(driver, m, str(tmp_path))
    if ref["outcome"] == "converged":
        assert kind == "converged", message
        assert abs(int(out["report"]["iterations"]) - ref["iterations"]) <= 2
    else:
        assert (kind, message) == ("runtime_error", ref["outcome"])


@pytest.mark.parametrize("name", list(ASSEMBLY_FAILURES))
def test_assembly_failure_message(driver, golden_json, name, tmp_path):
    kind, message, _ = run(driver, ASSEMBLY_FAILURES[name](), str(tmp_path))
    assert (kind, message) == ("runtime_error", assembly_failure_message(golden_json, name))
