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
