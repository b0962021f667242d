"""The small models behind the golden fixtures (the same ones
tests/golden/make_golden.py feeds to the reference), rebuilt without the reference."""

from __future__ import annotations

import numpy as np

from lightfem_gb300 import mesh
from lightfem_gb300.model import PLANE_STRAIN, Model, SolverSettings


def single_q4() -> Model:
    return Model(
        node_ids=np.array([1, 2, 3, 4]), xy=np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]]),
        material_ids=np.array([1]), young=np.array([1.0e6]), poisson=np.array([0.25]), thickness=np.array([1.0]),
        element_ids=np.array([1]), element_nodes=np.array([[1, 2, 3, 4]]), element_material=np.array([1]),
        bc_node=np.array([1, 4]), bc_ux=np.zeros(2), bc_uy=np.zeros(2),
        load_node=np.array([2]), load_fx=np.zeros(1), load_fy=np.array([-1.0]),
        settings=SolverSettings(tolerance=1e-12, max_iterations=100))


def scrambled() -> Model:
    ids = np.array([1, 9, 3, 8, 2, 7, 4, 6, 5])
    xy = np.array([[0, 0], [1, 0], [2, 0], [0, 1], [1, 1], [2, 1], [0, 2], [1, 2], [2, 2]], dtype=float)
    return Model(
        node_ids=ids, xy=xy, material_ids=np.array([1]), young=np.array([1.0e6]), poisson=np.array([0.25]),
        thickness=np.array([1.0]), element_ids=np.array([1, 2, 3, 4]),
        element_nodes=np.array([[1, 9, 2, 8], [9, 3, 7, 2], [8, 2, 6, 4], [2, 7, 5, 6]]),
        element_material=np.ones(4, np.int64), bc_node=np.array([1, 4]), bc_ux=np.zeros(2), bc_uy=np.zeros(2),
        load_node=np.array([3, 5]), load_fx=np.zeros(2), load_fy=np.array([-1.0, -1.0]),
        settings=SolverSettings(tolerance=1e-12, max_iterations=200))


def grid6() -> Model:
    m = mesh.cantilever(6, 6, length=1.0, height=1.0, young=1.0e6, poisson=0.25, thickness=1.0,
                        total_load=-0.01 * 7, settings=SolverSettings(tolerance=1e-12, max_iterations=5000))
    m.load_fy[:] = -0.01
    return m


def beam() -> Model:
    return mesh.perturbed_beam(24, 12, seed=7, settings=SolverSettings(
        tolerance=1e-10, max_iterations=20000, assembly="coloring"))


def strain() -> Model:
    return mesh.cantilever(16, 8, young=70e9, poisson=0.33, plane_mode=PLANE_STRAIN,
                           settings=SolverSettings(tolerance=1e-10, max_iterations=20000, assembly="coloring",
                                                   reordering="rcm"))


def adjoint_model() -> Model:
    n = 20
    return mesh.cantilever(n, n, poisson=0.3, per_element_young=mesh.lognormal_moduli(n * n, seed=11),
                           settings=SolverSettings(tolerance=1e-13, max_iterations=50000))


def fan(sectors: int = 20) -> Model:
    """Kite-shaped quads around one centre node, which belongs to every element (more
    elements at one node than the device pattern build takes), plus an isolated
    node that belongs to no element.  Node IDs are scrambled."""
    theta = 2.0 * np.pi * np.arange(sectors) / sectors
    mid = theta + np.pi / sectors
    xy = np.vstack([[0.0, 0.0], np.c_[np.cos(theta), np.sin(theta)], 2.0 * np.c_[np.cos(mid), np.sin(mid)],
                    [5.0, 5.0]])
    ids = np.random.default_rng(3).permutation(xy.shape[0]) + 100
    ring = lambda i: ids[1 + (i % sectors)]
    outer = lambda i: ids[1 + sectors + i]
    conn = np.array([[ids[0], ring(i), outer(i), ring(i + 1)] for i in range(sectors)])
    return Model(node_ids=ids, xy=xy, material_ids=np.array([1]), young=np.array([1.0e6]),
                 poisson=np.array([0.25]), thickness=np.array([1.0]), element_ids=np.arange(1, sectors + 1),
                 element_nodes=conn, element_material=np.ones(sectors, np.int64),
                 settings=SolverSettings(tolerance=1e-12, max_iterations=1000))


def element_moduli(model, element, value):
    """grid6 with one material per element and ``value`` as element ``element``'s modulus."""
    ne = model.element_ids.shape[0]
    young = np.full(ne, 1.0e6)
    young[element] = value
    model.material_ids = np.arange(1, ne + 1)
    model.young, model.poisson, model.thickness = young, np.full(ne, 0.25), np.ones(ne)
    model.element_material = np.arange(1, ne + 1)
    return model


def huge_thickness(model, element, value):
    """grid6 with element ``element`` ``value`` thick: its K_e overflows to +inf on
    the diagonal whichever order the products are taken in."""
    model = element_moduli(model, element, 1.0e6)
    model.thickness[element] = value
    return model


def floating_node(model, loaded):
    """grid6 plus a node that belongs to no element (zero rows of K)."""
    new_id = int(model.node_ids.max()) + 1
    model.node_ids = np.append(model.node_ids, new_id)
    model.xy = np.vstack([model.xy, [9.0, 9.0]])
    if loaded:
        model.load_node = np.append(model.load_node, new_id)
        model.load_fx = np.append(model.load_fx, 0.0)
        model.load_fy = np.append(model.load_fy, -1.0)
    return model


def flipped_element(model, element):
    """``model`` with one element's nodes in clockwise order: detJ < 0 at every
    Gauss point (q4_kinematics, src/element.cpp:52-54)."""
    model.element_nodes[element] = model.element_nodes[element][::-1].copy()
    return model


def collapsed_edge(kinds):
    """One Q4 whose nodes 3 and 4 coincide (a triangle: detJ = (1 - eta)/8 > 0 at
    the Gauss points, so the stiffness is fine) with one edge load per entry of
    ``kinds`` ((side, EDGE_*) pairs, in record order).  Edge 3 has zero length."""
    from lightfem_gb300.model import EDGE_PRESSURE
    sides = np.array([k[0] for k in kinds])
    kind = np.array([k[1] for k in kinds])
    return Model(
        node_ids=np.array([1, 2, 3, 4]), xy=np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [0.0, 1.0]]),
        material_ids=np.array([1]), young=np.array([1.0e6]), poisson=np.array([0.25]), thickness=np.array([1.0]),
        element_ids=np.array([1]), element_nodes=np.array([[1, 2, 3, 4]]), element_material=np.array([1]),
        bc_node=np.array([1, 2]), bc_ux=np.zeros(2), bc_uy=np.zeros(2),
        edge_element=np.ones(len(kinds), np.int64), edge_side=sides, edge_kind=kind,
        edge_first=np.where(kind == EDGE_PRESSURE, 1.0, 0.0), edge_second=np.where(kind == EDGE_PRESSURE, 0.0, -1.0),
        settings=SolverSettings(tolerance=1e-12, max_iterations=100))


# Models whose assembly stops with the reference's element exceptions
# (src/element.cpp:52-54, :189, :206).  The "failures" entry of golden.json holds
# how the reference ended on each.
ASSEMBLY_FAILURES = {
    "flipped_element": lambda: flipped_element(grid6(), 7),
    "collapsed_edge_pressure": lambda: collapsed_edge([(1, 0), (3, 1)]),
    "collapsed_edge_traction": lambda: collapsed_edge([(1, 1), (3, 0), (3, 1)]),
}


def assembly_failure_message(golden_json, name):
    """The message the reference ended with on ASSEMBLY_FAILURES[name].  Its
    element stiffness runs inside an OpenMP parallel region, which an exception
    cannot leave, so a non-positive Jacobian ends the reference's process through
    std::terminate; the golden then keeps the exception's what()."""
    ref = golden_json["failures"][name]["csr_jacobi"]
    return ref["what"] if ref["outcome"] == "terminate" else ref["outcome"]


def with_load(value):
    def make():
        m = grid6()
        m.load_fy[0] = value
        return m
    return make


def _zero_loads(m):
    m.load_fy[:] = 0.0
    return m


# Models on which the reference's solve stops, or finishes, in one known way (the
# zero-pivot sweep, the Jacobi setup, pcg_solve's three checks, or the "initial
# residual satisfies tolerance" exit).
FAILURE_MODELS = {
    "nan_load": with_load(np.nan),               # r0 = sqrt(max(0, NaN)) = 0: converged at once
    "inf_load": with_load(np.inf),               # r0 = inf <= tol * inf: converged at once
    "zero_load": lambda: _zero_loads(grid6()),
    "nan_modulus": lambda: element_moduli(grid6(), 14, np.nan),      # NaN pivots swept to 1
    "nan_modulus_loaded": lambda: element_moduli(grid6(), 35, np.nan),  # ... one of them loaded
    "huge_thickness": lambda: huge_thickness(grid6(), 14, 1.0e307),  # +inf diagonal survives
    "negative_modulus_half": lambda: element_moduli(grid6(), 14, -0.5e6),
    "negative_modulus_1": lambda: element_moduli(grid6(), 14, -1.0e6),
    "negative_modulus_5": lambda: element_moduli(grid6(), 14, -5.0e6),
    "negative_modulus_50": lambda: element_moduli(grid6(), 14, -5.0e7),
    "floating_node": lambda: floating_node(grid6(), loaded=False),
    "floating_node_loaded": lambda: floating_node(grid6(), loaded=True),
}

# Failure cases whose outcome is fixed before the first search direction is formed
# or at its first product, so an FP32 inner loop must end the same way.
FAILURE_DETERMINISTIC = {"nan_load", "inf_load", "zero_load", "nan_modulus", "nan_modulus_loaded",
                         "huge_thickness", "floating_node", "floating_node_loaded"}
_ORACLE_STATUS = {1: "rho_initial", 2: "not_spd", 3: "rho"}


def failure_case(name, storage, precond):
    """A failure model, indexed, with the storage and preconditioner set (block =
    2x2 nodal blocks)."""
    m = FAILURE_MODELS[name]()
    m.settings.storage, m.settings.preconditioner = storage, precond
    m.settings.subdomain_split, m.settings.subdomain_nodes = "chunk", 1
    return indexed(m)


# The reference's exception messages (src/solver.cpp:579-581, :591-593, :616-618,
# :656-669, :926-936) by the kind the failure tests compare.
_OUTCOME_TEXT = {
    "mechanism": "the structure is a mechanism",
    "nonfinite_diag": "Jacobi preconditioner encountered a non-finite diagonal",
    "rho_initial": "PCG failed to form a positive initial preconditioned residual",
    "not_spd": "PCG encountered non-positive curvature; system is not SPD",
    "rho": "PCG preconditioned residual became non-positive or non-finite",
}


def outcome_kind(message: str) -> str:
    """The kind of a reference solve() outcome ("converged" or an exception message)."""
    if message == "converged":
        return message
    for kind, text in _OUTCOME_TEXT.items():
        if message.startswith(text):
            return kind
    raise ValueError(f"unknown outcome: {message}")


def oracle_outcome(oracle, model):
    """How the oracle's solve of ``model`` ends: "mechanism", "nonfinite_diag",
    "rho_initial", "not_spd", "rho", "maxit" or "converged" (then with its output)."""
    try:
        out = oracle.solve_model(model.copy())
    except RuntimeError as err:
        if "mechanism" in str(err):
            return "mechanism", None
        if "PCG setup" in str(err):  # the oracle's Jacobi setup threw on a non-finite diagonal
            return "nonfinite_diag", None
        raise
    rep = out["report"]
    if rep["status"]:
        return _ORACLE_STATUS[int(rep["status"])], None
    return ("converged" if rep["converged"] else "maxit"), out


CASES = {"single_q4": single_q4, "scrambled": scrambled, "grid6": grid6, "beam": beam, "strain": strain}

# (storage, preconditioner, subdomain_split, subdomain_nodes) of each golden variant
VARIANTS = {
    "csr_jacobi": ("csr", "jacobi", "rcb", 1),
    "bsr_jacobi": ("bsr", "jacobi", "rcb", 1),
    "csr_ic0": ("csr", "ic0", "rcb", 1),
    "bsr_ic0": ("bsr", "ic0", "rcb", 1),
    "bsr_block1": ("bsr", "block", "chunk", 1),
    "csr_block1": ("csr", "block", "chunk", 1),
    "bsr_block_rcb2": ("bsr", "block", "rcb", 2),
    "bsr_block_chunk4": ("bsr", "block", "chunk", 4),
    "bsr_block64": ("bsr", "block", "rcb", 64),
}


def indexed(model: Model) -> Model:
    model.sort_and_index()
    return model


def by_id_order(model: Model, v: np.ndarray) -> np.ndarray:
    """Reorder a DOF vector of the model's current node order into node-ID order."""
    order = np.argsort(model.node_ids, kind="stable")
    out = np.empty_like(v)
    out[0::2] = v[2 * order]
    out[1::2] = v[2 * order + 1]
    return out
