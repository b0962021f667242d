"""Array form of a LightFEM model and of the host-side indexing the solve path consumes.

Mirrors ``include/lightfem/model.hpp`` (``Model``, ``Node``, ``Material``, ``Q4Element``,
``DirichletBC``, ``NodalLoad``, ``BodyForce``, ``EdgeLoad``, ``SolverSettings``) with one
numpy array per field instead of one struct per entity.  Only what the solve path needs
is kept: trusses, VTK/CSV options and parsing stay with the reference host library.

Indexing follows ``Model::sort_and_index`` / ``Model::rebuild_indices``
(src/model.cpp:24-39, 74-92): entities are sorted by ID and node ``k`` in index order
owns DOFs ``2k`` and ``2k+1``.  ``index_with_node_order`` follows src/model.cpp:41-72.
"""

from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np

PLANE_STRESS = 0
PLANE_STRAIN = 1

EDGE_TRACTION = 0
EDGE_PRESSURE = 1


@dataclass
class SolverSettings:
    """``SolverSettings`` (include/lightfem/model.hpp:94-112) plus the GPU selectors.

    ``assembly`` and ``solver`` take the reference's values; ``"gpu"`` in either selects
    the CUDA path, exactly as the ``[settings]`` keys would in a ``.fem`` file.
    ``precision`` ("fp64" | "mixed") and ``refinement`` ("reliable" | "restart") only
    matter on the GPU path.
    """

    plane_mode: int = PLANE_STRESS
    solver: str = "pcg"
    tolerance: float = 1.0e-10
    max_iterations: int = 5000
    reordering: str = "none"
    assembly: str = "serial"
    threads: int = 0
    storage: str = "csr"
    preconditioner: str = "jacobi"
    subdomain_split: str = "rcb"
    subdomain_nodes: int = 64
    precision: str = "fp64"
    refinement: str = "reliable"
    gpu_assembly: str = "coloring"


@dataclass
class Model:
    node_ids: np.ndarray            # int64 [N]
    xy: np.ndarray                  # float64 [N, 2]
    material_ids: np.ndarray        # int64 [M]
    young: np.ndarray               # float64 [M]
    poisson: np.ndarray             # float64 [M]
    thickness: np.ndarray           # float64 [M]
    element_ids: np.ndarray         # int64 [E]
    element_nodes: np.ndarray       # int64 [E, 4] node IDs, counter-clockwise
    element_material: np.ndarray    # int64 [E] material IDs
    bc_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    bc_ux: np.ndarray = field(default_factory=lambda: np.zeros(0))   # NaN = free
    bc_uy: np.ndarray = field(default_factory=lambda: np.zeros(0))   # NaN = free
    load_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    load_fx: np.ndarray = field(default_factory=lambda: np.zeros(0))
    load_fy: np.ndarray = field(default_factory=lambda: np.zeros(0))
    body_element: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    body_bx: np.ndarray = field(default_factory=lambda: np.zeros(0))
    body_by: np.ndarray = field(default_factory=lambda: np.zeros(0))
    edge_element: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    edge_side: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))   # 1..4
    edge_kind: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))   # EDGE_*
    edge_first: np.ndarray = field(default_factory=lambda: np.zeros(0))   # tx or pressure
    edge_second: np.ndarray = field(default_factory=lambda: np.zeros(0))  # ty
    settings: SolverSettings = field(default_factory=SolverSettings)
    indexed: bool = False

    # ------------------------------------------------------------------ indexing
    @property
    def n_nodes(self) -> int:
        return int(self.node_ids.shape[0])

    @property
    def n_elements(self) -> int:
        return int(self.element_ids.shape[0])

    @property
    def n_dofs(self) -> int:
        return 2 * self.n_nodes

    def copy(self) -> "Model":
        return replace(self, settings=replace(self.settings))

    def sort_and_index(self) -> None:
        """Sort nodes, materials and elements by ID (src/model.cpp:24-39)."""
        for ids_name, fields in (
            ("node_ids", ("xy",)),
            ("material_ids", ("young", "poisson", "thickness")),
            ("element_ids", ("element_nodes", "element_material")),
        ):
            ids = getattr(self, ids_name)
            order = np.argsort(ids, kind="stable")
            sorted_ids = ids[order]
            if sorted_ids.size > 1 and np.any(sorted_ids[1:] == sorted_ids[:-1]):
                raise ValueError(f"duplicate {ids_name[:-4]} ID")
            setattr(self, ids_name, sorted_ids)
            for name in fields:
                setattr(self, name, getattr(self, name)[order])
        self.indexed = True

    def index_with_node_order(self, node_order: np.ndarray) -> None:
        """Place nodes in the given ID order; DOFs follow (src/model.cpp:41-72)."""
        node_order = np.asarray(node_order, dtype=np.int64)
        if node_order.shape[0] != self.n_nodes:
            raise ValueError("node reordering must contain every model node exactly once")
        pos = self.node_index(node_order)
        if np.unique(pos).shape[0] != pos.shape[0]:
            raise ValueError("node reordering references an unknown or duplicate node ID")
        self.node_ids = self.node_ids[pos]
        self.xy = self.xy[pos]
        self.indexed = True

    def node_index(self, ids: np.ndarray) -> np.ndarray:
        """Index of each node ID in the current node order (``Model::find_node``)."""
        ids = np.asarray(ids, dtype=np.int64)
        order = np.argsort(self.node_ids, kind="stable")
        sorted_ids = self.node_ids[order]
        where = np.searchsorted(sorted_ids, ids)
        where = np.clip(where, 0, max(sorted_ids.shape[0] - 1, 0))
        if ids.size and not np.all(sorted_ids[where] == ids):
            raise ValueError("model references an unknown node ID")
        return order[where]

    def material_index(self, ids: np.ndarray) -> np.ndarray:
        ids = np.asarray(ids, dtype=np.int64)
        where = np.searchsorted(self.material_ids, ids)
        where = np.clip(where, 0, max(self.material_ids.shape[0] - 1, 0))
        if ids.size and not np.all(self.material_ids[where] == ids):
            raise ValueError("element references an unknown material")
        return where

    def element_index(self, ids: np.ndarray) -> np.ndarray:
        ids = np.asarray(ids, dtype=np.int64)
        where = np.searchsorted(self.element_ids, ids)
        where = np.clip(where, 0, max(self.element_ids.shape[0] - 1, 0))
        if ids.size and not np.all(self.element_ids[where] == ids):
            raise ValueError("load references an unknown element")
        return where

    def element_node_index(self) -> np.ndarray:
        """[E, 4] node indices of every Q4 element (``q4_coordinates`` order)."""
        return self.node_index(self.element_nodes.reshape(-1)).reshape(-1, 4)

    def element_dofs(self) -> np.ndarray:
        """[E, 8] DOFs ``[ux1, uy1, ..., ux4, uy4]`` (src/element.cpp:114-128)."""
        nodes = self.element_node_index()
        dofs = np.empty((nodes.shape[0], 8), dtype=np.int64)
        dofs[:, 0::2] = 2 * nodes
        dofs[:, 1::2] = 2 * nodes + 1
        return dofs

    def constraints(self) -> tuple[np.ndarray, np.ndarray]:
        """Sorted (dof, value) pairs of the prescribed displacements (src/solver.cpp:340-351)."""
        idx = self.node_index(self.bc_node)
        dofs, vals = [], []
        for k in range(idx.shape[0]):
            if not np.isnan(self.bc_ux[k]):
                dofs.append(2 * idx[k])
                vals.append(self.bc_ux[k])
            if not np.isnan(self.bc_uy[k]):
                dofs.append(2 * idx[k] + 1)
                vals.append(self.bc_uy[k])
        dofs = np.asarray(dofs, dtype=np.int64)
        vals = np.asarray(vals, dtype=np.float64)
        order = np.argsort(dofs, kind="stable")
        return dofs[order], vals[order]

    def nodal_load_vector(self) -> np.ndarray:
        """Nodal loads summed into f in record order (src/solver.cpp:303-308)."""
        f = np.zeros(self.n_dofs)
        idx = self.node_index(self.load_node)
        for k in range(idx.shape[0]):
            f[2 * idx[k]] += self.load_fx[k]
            f[2 * idx[k] + 1] += self.load_fy[k]
        return f
