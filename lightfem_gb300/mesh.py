"""Seeded structured Q4 meshes for the solve-path workloads, and a ``.fem`` writer.

The generators play the role of the reference's ``tools/gen_mesh.py`` (row-major node
numbering ``j*(nx+1)+i+1``, counter-clockwise elements, left edge clamped), extended
with the perturbed two-material beam and the log-normal per-element moduli that the
larger workloads call for.  Every random draw comes from ``numpy.random.default_rng``
with an explicit seed, so a model is a pure function of its arguments.

``to_fem`` writes the model in the reference's input format
(docs/input_format.md, parsed by src/input_parser.cpp:162-341) with ``repr`` floats,
which ``std::stod`` reads back bit-for-bit, so the reference CLI and this package see
identical numbers.
"""

from __future__ import annotations

import io

import numpy as np

from .model import (EDGE_PRESSURE, EDGE_TRACTION, PLANE_STRAIN, PLANE_STRESS, Model,
                    SolverSettings)


def _grid(nx: int, ny: int, length: float, height: float):
    i = np.arange(nx + 1)
    j = np.arange(ny + 1)
    jj, ii = np.meshgrid(j, i, indexing="ij")
    node_ids = (jj * (nx + 1) + ii + 1).reshape(-1).astype(np.int64)
    xy = np.stack([ii.reshape(-1) * (length / nx), jj.reshape(-1) * (height / ny)], axis=1)
    ei = np.arange(nx)
    ej = np.arange(ny)
    ejj, eii = np.meshgrid(ej, ei, indexing="ij")
    eii = eii.reshape(-1)
    ejj = ejj.reshape(-1)

    def nid(a, b):
        return b * (nx + 1) + a + 1

    conn = np.stack([nid(eii, ejj), nid(eii + 1, ejj), nid(eii + 1, ejj + 1), nid(eii, ejj + 1)],
                    axis=1).astype(np.int64)
    element_ids = np.arange(1, nx * ny + 1, dtype=np.int64)
    return node_ids, xy, element_ids, conn, eii, ejj


def _clamp_left(nx: int, ny: int):
    nodes = (np.arange(ny + 1) * (nx + 1) + 1).astype(np.int64)
    zeros = np.zeros(ny + 1)
    return nodes, zeros, zeros.copy()


def cantilever(nx: int, ny: int, *, length: float = 2.0, height: float = 1.0,
               young: float = 200e9, poisson: float = 0.3, thickness: float = 0.01,
               total_load: float = -1000.0, plane_mode: int = PLANE_STRESS,
               per_element_young: np.ndarray | None = None,
               settings: SolverSettings | None = None) -> Model:
    """Clamped-left cantilever with ``total_load`` (N, in y) shared equally by the
    right-edge nodes.  ``per_element_young`` gives every element its own material."""
    node_ids, xy, element_ids, conn, _, _ = _grid(nx, ny, length, height)
    E = nx * ny
    if per_element_young is None:
        material_ids = np.array([1], np.int64)
        young_arr = np.array([young])
        element_material = np.ones(E, np.int64)
    else:
        per_element_young = np.asarray(per_element_young, dtype=np.float64)
        assert per_element_young.shape == (E,)
        material_ids = element_ids.copy()
        young_arr = per_element_young.copy()
        element_material = element_ids.copy()
    M = material_ids.shape[0]
    bc_node, bc_ux, bc_uy = _clamp_left(nx, ny)
    load_node = (np.arange(ny + 1) * (nx + 1) + nx + 1).astype(np.int64)
    model = Model(
        node_ids=node_ids, xy=xy, material_ids=material_ids, young=young_arr,
        poisson=np.full(M, poisson), thickness=np.full(M, thickness),
        element_ids=element_ids, element_nodes=conn, element_material=element_material,
        bc_node=bc_node, bc_ux=bc_ux, bc_uy=bc_uy,
        load_node=load_node, load_fx=np.zeros(ny + 1), load_fy=np.full(ny + 1, total_load / (ny + 1)),
        settings=settings or SolverSettings(plane_mode=plane_mode),
    )
    model.settings.plane_mode = plane_mode
    return model


def perturbed_beam(nx: int, ny: int, *, seed: int, length: float = 4.0, height: float = 2.0,
                   jitter: float = 0.2, materials=((200e9, 0.3), (70e9, 0.33)),
                   thickness: float = 0.01, density_g: float = 7850.0 * 9.81,
                   top_pressure: float = 1.0e6, plane_mode: int = PLANE_STRESS,
                   per_element_young: np.ndarray | None = None,
                   settings: SolverSettings | None = None) -> Model:
    """Clamped-left beam with interior nodes jittered uniformly within +/-``jitter`` of
    the element size, two materials split at mid-span (by element column), a body
    force ``-density_g`` in y on every element and ``top_pressure`` on the top edge
    (local edge 3 of the top-row elements)."""
    node_ids, xy, element_ids, conn, eii, ejj = _grid(nx, ny, length, height)
    hx, hy = length / nx, height / ny
    rng = np.random.default_rng(seed)
    shift = rng.uniform(-jitter, jitter, size=xy.shape) * np.array([hx, hy])
    ii = (node_ids - 1) % (nx + 1)
    jj = (node_ids - 1) // (nx + 1)
    interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
    xy = xy + shift * interior[:, None]
    E = nx * ny
    if per_element_young is None:
        material_ids = np.array([1, 2], np.int64)
        young = np.array([materials[0][0], materials[1][0]])
        poisson = np.array([materials[0][1], materials[1][1]])
        element_material = np.where(eii < nx // 2, 1, 2).astype(np.int64)
    else:
        per_element_young = np.asarray(per_element_young, dtype=np.float64)
        assert per_element_young.shape == (E,)
        material_ids = element_ids.copy()
        young = per_element_young.copy()
        poisson = np.where(eii < nx // 2, materials[0][1], materials[1][1])
        element_material = element_ids.copy()
    M = material_ids.shape[0]
    bc_node, bc_ux, bc_uy = _clamp_left(nx, ny)
    top = element_ids[ejj == ny - 1]
    model = Model(
        node_ids=node_ids, xy=xy, material_ids=material_ids, young=young, poisson=poisson,
        thickness=np.full(M, thickness), element_ids=element_ids, element_nodes=conn,
        element_material=element_material, bc_node=bc_node, bc_ux=bc_ux, bc_uy=bc_uy,
        body_element=element_ids.copy(), body_bx=np.zeros(E), body_by=np.full(E, -density_g),
        edge_element=top, edge_side=np.full(top.shape[0], 3, np.int64),
        edge_kind=np.full(top.shape[0], EDGE_PRESSURE, np.int64),
        edge_first=np.full(top.shape[0], top_pressure), edge_second=np.zeros(top.shape[0]),
        settings=settings or SolverSettings(plane_mode=plane_mode),
    )
    model.settings.plane_mode = plane_mode
    check_jacobians(model)
    return model


def lognormal_moduli(n: int, *, seed: int, scale: float = 1.0e9, sigma: float = 0.5) -> np.ndarray:
    """``E_e = scale * exp(sigma * z_e)`` with ``z_e ~ N(0, 1)`` i.i.d."""
    return scale * np.exp(sigma * np.random.default_rng(seed).standard_normal(n))


# ---------------------------------------------------------------------- workloads
CONFIG_SEEDS = {3: 20261203, 4: 20261204, 5: 20261205}


def workload(cfg: int, scale: int = 1, **overrides) -> Model:
    """The solve-path workloads, by number.  ``scale`` > 1 divides both grid
    dimensions (a small case with the same physics for tests).

    1: 200x200 plane-stress cantilever, 2 m x 1 m, E 200 GPa, nu 0.3, -1000 N on the
       right edge, colouring assembly, Jacobi PCG, tolerance 1e-8.
    2: 1000x1000 plane-strain cantilever, same geometry and loads, E 70 GPa, nu 0.33,
       RCM ordering, tolerance 1e-8.
    3: 2000x1000 perturbed two-material beam, 4 m x 2 m, gravity + 1 MPa top pressure.
    4: 400x400 plane-stress cantilever with log-normal per-element moduli (adjoint).
    5: workload-3 geometry at 1000x1000 with log-normal per-element moduli.
    """
    settings = SolverSettings(tolerance=1e-8, max_iterations=200000, assembly="coloring",
                              storage="csr", preconditioner="jacobi")
    if cfg == 1:
        n = max(1, 200 // scale)
        m = cantilever(n, n, young=200e9, poisson=0.3, settings=settings)
    elif cfg == 2:
        n = max(1, 1000 // scale)
        settings.reordering = "rcm"
        m = cantilever(n, n, young=70e9, poisson=0.33, plane_mode=PLANE_STRAIN, settings=settings)
    elif cfg == 3:
        m = perturbed_beam(max(2, 2000 // scale), max(1, 1000 // scale), seed=CONFIG_SEEDS[3],
                           settings=settings)
    elif cfg == 4:
        n = max(1, 400 // scale)
        m = cantilever(n, n, poisson=0.3, settings=settings,
                       per_element_young=lognormal_moduli(n * n, seed=CONFIG_SEEDS[4]))
    elif cfg == 5:
        n = max(2, 1000 // scale)
        m = perturbed_beam(n, n, seed=CONFIG_SEEDS[5], settings=settings,
                           per_element_young=lognormal_moduli(n * n, seed=CONFIG_SEEDS[5]))
    else:
        raise ValueError(f"unknown workload {cfg}")
    for key, value in overrides.items():
        setattr(m.settings, key, value)
    return m


def tip_node_id(model: Model) -> int:
    """Right-edge node closest to mid-height (the tip displacement objective)."""
    x = model.xy[:, 0]
    right = np.flatnonzero(np.isclose(x, x.max()))
    mid = 0.5 * (model.xy[:, 1].min() + model.xy[:, 1].max())
    return int(model.node_ids[right[np.argmin(np.abs(model.xy[right, 1] - mid))]])


def check_jacobians(model: Model) -> None:
    """Every element must have a positive Jacobian at its four Gauss points (the same
    test ``q4_kinematics`` applies, src/element.cpp:51-54)."""
    idx = model.node_index(model.element_nodes.reshape(-1)).reshape(-1, 4)
    x = model.xy[idx, 0]
    y = model.xy[idx, 1]
    g = 0.57735026918962576451
    for xi, eta in ((-g, -g), (g, -g), (g, g), (-g, g)):
        dxi = 0.25 * np.array([-(1 - eta), (1 - eta), (1 + eta), -(1 + eta)])
        deta = 0.25 * np.array([-(1 - xi), -(1 + xi), (1 + xi), (1 - xi)])
        det = (x @ dxi) * (y @ deta) - (x @ deta) * (y @ dxi)
        if not np.all(det > 1e-14):
            raise ValueError("generated mesh has a non-positive Jacobian")


# ---------------------------------------------------------------------- .fem output
def to_fem(model: Model, output: str = "result.vtk") -> str:
    """Render the model in the reference's ``.fem`` format."""
    s = model.settings
    out = io.StringIO()
    w = out.write
    w("[settings]\n")
    w(f"plane_mode {'plane_strain' if s.plane_mode == PLANE_STRAIN else 'plane_stress'}\n")
    w("solver pcg\n")
    w(f"tolerance {s.tolerance!r}\n")
    w(f"max_iterations {int(s.max_iterations)}\n")
    w(f"reordering {s.reordering}\n")
    w(f"assembly {s.assembly if s.assembly != 'gpu' else 'serial'}\n")
    w(f"threads {int(s.threads)}\n")
    w(f"storage {s.storage}\n")
    w(f"preconditioner {s.preconditioner}\n")
    w(f"subdomain_split {s.subdomain_split}\n")
    w(f"subdomain_nodes {int(s.subdomain_nodes)}\n")
    w(f"output {output}\n")
    w("[materials]\n")
    w("".join(f"{int(i)} {float(e)!r} {float(n)!r} {float(t)!r}\n" for i, e, n, t in
              zip(model.material_ids, model.young, model.poisson, model.thickness)))
    w("[nodes]\n")
    w("".join(f"{int(i)} {float(x)!r} {float(y)!r}\n" for i, (x, y) in zip(model.node_ids, model.xy)))
    w("[elements]\n")
    w("".join(f"{int(i)} {int(c[0])} {int(c[1])} {int(c[2])} {int(c[3])} {int(m)}\n"
              for i, c, m in zip(model.element_ids, model.element_nodes, model.element_material)))

    def cval(v):
        return "free" if np.isnan(v) else repr(float(v))

    w("[boundary]\n")
    w("".join(f"{int(n)} {cval(a)} {cval(b)}\n" for n, a, b in zip(model.bc_node, model.bc_ux, model.bc_uy)))
    if model.load_node.size:
        w("[loads]\n")
        w("".join(f"{int(n)} {float(a)!r} {float(b)!r}\n"
                  for n, a, b in zip(model.load_node, model.load_fx, model.load_fy)))
    if model.body_element.size:
        w("[body_forces]\n")
        w("".join(f"{int(e)} {float(a)!r} {float(b)!r}\n"
                  for e, a, b in zip(model.body_element, model.body_bx, model.body_by)))
    if model.edge_element.size:
        w("[edge_loads]\n")
        for e, side, kind, a, b in zip(model.edge_element, model.edge_side, model.edge_kind,
                                       model.edge_first, model.edge_second):
            if kind == EDGE_TRACTION:
                w(f"{int(e)} {int(side)} traction {float(a)!r} {float(b)!r}\n")
            else:
                w(f"{int(e)} {int(side)} pressure {float(a)!r}\n")
    return out.getvalue()
