"""ctypes binding of the CPU oracle (oracle/lf_oracle.cpp) — TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py use
this module; the lightfem_gb300 package never imports it.  ``solve_model`` runs the
reference's solve path on the CPU exactly as ``LinearElasticSolver::solve``
(src/solver.cpp:875-960) sequences it and returns every intermediate.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liblf_oracle.so")

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, d, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int
        sig = {
            "lfo_num_threads": (i32, []),
            "lfo_set_threads": (None, [i32]),
            "lfo_q4_stiffness": (i32, [vp, d, d, d, i32, vp]),
            "lfo_pattern_build": (vp, [i64, i64, i64, vp]),
            "lfo_pattern_nnz": (i64, [vp]),
            "lfo_pattern_copy": (None, [vp, vp, vp, vp]),
            "lfo_pattern_free": (None, [vp]),
            "lfo_element_colors": (i64, [i64, i64, vp, vp]),
            "lfo_assemble": (i64, [vp, i64, vp, vp, vp, vp, i32, vp, vp, vp, vp, i64]),
            "lfo_element_loads": (i32, [vp, vp, vp, i64, vp, vp, vp, i64, vp, vp, vp, vp, vp, vp]),
            "lfo_apply_dirichlet": (i64, [i64, vp, vp, vp, vp, i64, vp, vp]),
            "lfo_spmv_csr": (None, [i64, vp, vp, vp, vp, vp]),
            "lfo_bsr_count": (i64, [i64, vp, vp, vp]),
            "lfo_bsr_convert": (None, [i64, vp, vp, vp, vp, vp, vp]),
            "lfo_precond_apply": (i32, [i64, vp, vp, vp, i32, i32, i64, vp, vp, vp, vp]),
            "lfo_pcg": (i32, [i64, vp, vp, vp, vp, d, i64, i32, i32, i32, i64, vp, vp, vp, vp, i64]),
            "lfo_adjoint_grad": (i32, [vp, i64, vp, vp, vp, vp, i32, vp, vp, vp]),
            "lfo_postprocess": (i32, [vp, i64, i64, vp, vp, vp, i32, vp, vp, vp]),
            "lfo_rcm": (None, [i64, vp, i64, vp, vp]),
            "lfo_subdomain_split": (i64, [i64, vp, i64, i32, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return None if a is None else a.ctypes.data


def set_threads(n: int) -> None:
    lib().lfo_set_threads(int(n))


def num_threads() -> int:
    return lib().lfo_num_threads()


def q4_stiffness(xy, young, poisson, thickness, plane_strain=0) -> np.ndarray:
    xy = _c(xy).reshape(8)
    k = np.empty(64)
    if lib().lfo_q4_stiffness(_p(xy), young, poisson, thickness, int(plane_strain), _p(k)) != 0:
        raise RuntimeError("Q4 stiffness evaluation received a non-positive Jacobian")
    return k.reshape(8, 8)


def pattern(n: int, elem_dofs: np.ndarray):
    dofs = _c(elem_dofs, np.int64)
    per = dofs.shape[1]
    h = lib().lfo_pattern_build(n, dofs.shape[0], per, _p(dofs))
    nnz = lib().lfo_pattern_nnz(h)
    rp = np.empty(n + 1, np.int64)
    col = np.empty(nnz, np.int64)
    mp = np.empty(dofs.shape[0] * per * per, np.int64)
    lib().lfo_pattern_copy(h, _p(rp), _p(col), _p(mp))
    lib().lfo_pattern_free(h)
    return rp, col, mp.reshape(dofs.shape[0], per * per)


def colors(n_nodes: int, elem_nodes: np.ndarray) -> np.ndarray:
    en = _c(elem_nodes, np.int64)
    out = np.empty(en.shape[0], np.int64)
    lib().lfo_element_colors(n_nodes, en.shape[0], _p(en), _p(out))
    return out


def rcm(node_ids, elem_node_ids) -> np.ndarray:
    ids = _c(node_ids, np.int64)
    en = _c(elem_node_ids, np.int64)
    out = np.empty(ids.shape[0], np.int64)
    lib().lfo_rcm(ids.shape[0], _p(ids), en.shape[0], _p(en), _p(out))
    return out


def spmv(rp, col, val, x) -> np.ndarray:
    rp, col, val, x = _c(rp, np.int64), _c(col, np.int64), _c(val), _c(x)
    y = np.empty(rp.shape[0] - 1)
    lib().lfo_spmv_csr(rp.shape[0] - 1, _p(rp), _p(col), _p(val), _p(x), _p(y))
    return y


def bsr(rp, col, val):
    rp, col, val = _c(rp, np.int64), _c(col, np.int64), _c(val)
    n = rp.shape[0] - 1
    nb = lib().lfo_bsr_count(n, _p(rp), _p(col), _p(val))
    bp = np.empty(n // 2 + 1, np.int64)
    bc = np.empty(nb, np.int64)
    bv = np.empty(4 * nb)
    lib().lfo_bsr_convert(n, _p(rp), _p(col), _p(val), _p(bp), _p(bc), _p(bv))
    return bp, bc, bv.reshape(nb, 4)


PRECOND = {"jacobi": 0, "block": 1, "ic0": 2}
SPLIT = {"chunk": 0, "rcb": 1}
STORAGE = {"csr": 0, "bsr": 1}


def subdomain_split(xy, nodes_per, split="rcb"):
    """split_by_chunks / split_by_coordinates: (owner per node, subdomain count)."""
    xy = _c(xy)
    owner = np.empty(xy.shape[0], np.uint32)
    count = lib().lfo_subdomain_split(xy.shape[0], _p(xy), int(nodes_per), SPLIT[split], _p(owner))
    return owner, int(count)


def precond_apply(rp, col, val, r, precond="jacobi", split="chunk", nodes_per=1, xy=None):
    rp, col, val, r = _c(rp, np.int64), _c(col, np.int64), _c(val), _c(r)
    z = np.empty_like(r)
    stats = np.zeros(8)
    xy = None if xy is None else _c(xy)
    lib().lfo_precond_apply(rp.shape[0] - 1, _p(rp), _p(col), _p(val), PRECOND[precond], SPLIT[split], nodes_per,
                            _p(xy), _p(r), _p(z), _p(stats))
    return z, stats


def pcg(rp, col, val, b, tol, maxit, storage="csr", precond="jacobi", split="chunk", nodes_per=1, xy=None,
        iteration_cap=0):
    rp, col, val, b = _c(rp, np.int64), _c(col, np.int64), _c(val), _c(b)
    x = np.empty_like(b)
    rep = np.zeros(9)
    stats = np.zeros(8)
    xy = None if xy is None else _c(xy)
    rc = lib().lfo_pcg(rp.shape[0] - 1, _p(rp), _p(col), _p(val), _p(b), tol, maxit, STORAGE[storage],
                       PRECOND[precond], SPLIT[split], nodes_per, _p(xy), _p(x), _p(rep), _p(stats), iteration_cap)
    if rc != 0:
        raise RuntimeError("oracle PCG setup failed")
    keys = ["converged", "iterations", "initial_residual", "final_residual", "solve_ms", "matvec_ms",
            "matvec_calls", "precond_apply_ms", "status"]
    report = dict(zip(keys, rep.tolist()))
    report["iterations"] = int(report["iterations"])
    report["stats"] = stats
    return x, report


def adjoint_grad(xy, elem_nodes, young_e, nu_e, t_e, plane_strain, u, lam) -> np.ndarray:
    xy, en = _c(xy), _c(elem_nodes, np.int64)
    g = np.empty(en.shape[0])
    rc = lib().lfo_adjoint_grad(_p(xy), en.shape[0], _p(en), _p(_c(young_e)), _p(_c(nu_e)), _p(_c(t_e)),
                                int(plane_strain), _p(_c(u)), _p(_c(lam)), _p(g))
    if rc != 0:
        raise RuntimeError("non-positive Jacobian")
    return g


def postprocess(xy, elem_nodes, young_e, nu_e, plane_strain, u):
    """Element fields (E x 5 x 7: centre + 4 Gauss points, each strain[3], stress[3],
    von Mises) and smoothed nodal stress (N x 4) for displacements u."""
    xy, en = _c(xy), _c(elem_nodes, np.int64)
    fields = np.empty((en.shape[0], 5, 7))
    nodal = np.empty((xy.shape[0], 4))
    rc = lib().lfo_postprocess(_p(xy), xy.shape[0], en.shape[0], _p(en), _p(_c(young_e)), _p(_c(nu_e)),
                               int(plane_strain), _p(_c(u)), _p(fields), _p(nodal))
    if rc != 0:
        raise RuntimeError("Q4 stiffness evaluation received a non-positive Jacobian")
    return fields, nodal


def solve_model(model, *, storage=None, preconditioner=None, assembly=None, split=None, nodes_per=None,
                tolerance=None, max_iterations=None, iteration_cap=0, stop_after=None):
    """The reference solve path on the CPU; returns a dict of every stage.

    ``model`` is an indexed lightfem_gb300.model.Model (it is reordered in place when
    its settings ask for RCM, as the reference reorders its Model).
    ``stop_after="assembly"`` / ``"dirichlet"`` ends early (bounded baselines).
    """
    s = model.settings
    storage = storage or s.storage
    preconditioner = preconditioner or s.preconditioner
    assembly = assembly or s.assembly
    split = split or s.subdomain_split
    nodes_per = nodes_per or s.subdomain_nodes
    tolerance = tolerance or s.tolerance
    max_iterations = max_iterations or s.max_iterations
    out: dict = {"timing": {}}
    t = time.perf_counter()
    if s.reordering == "rcm":
        model.index_with_node_order(rcm(model.node_ids, model.element_nodes))
    out["node_order"] = model.node_ids.copy()
    n = model.n_dofs
    en = model.element_node_index()
    dofs = model.element_dofs()
    rp, col, mp = pattern(n, dofs)
    out.update(rowptr=rp, col=col, map=mp)
    out["timing"]["pattern_ms"] = (time.perf_counter() - t) * 1e3
    cl = colors(model.n_nodes, en)
    out["colors"] = cl
    mi = model.material_index(model.element_material)
    young_e, nu_e, t_e = model.young[mi], model.poisson[mi], model.thickness[mi]
    order = None
    color_ptr = None
    if assembly == "coloring":
        order = np.argsort(cl, kind="stable").astype(np.int64)
        color_ptr = np.concatenate([[0], np.cumsum(np.bincount(cl))]).astype(np.int64)
    K = np.zeros(col.shape[0])
    t = time.perf_counter()
    rc = lib().lfo_assemble(_p(_c(model.xy)), en.shape[0], _p(_c(en, np.int64)), _p(_c(young_e)), _p(_c(nu_e)),
                            _p(_c(t_e)), int(s.plane_mode), _p(_c(mp, np.int64)), _p(order), _p(K),
                            _p(color_ptr), 0 if color_ptr is None else color_ptr.shape[0] - 1)
    if rc != 0:
        raise RuntimeError("Q4 stiffness evaluation received a non-positive Jacobian")
    out["timing"]["assembly_ms"] = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    f = model.nodal_load_vector()
    be = model.element_index(model.body_element) if model.body_element.size else np.zeros(0, np.int64)
    ee = model.element_index(model.edge_element) if model.edge_element.size else np.zeros(0, np.int64)
    rc = lib().lfo_element_loads(_p(_c(model.xy)), _p(_c(en, np.int64)), _p(_c(t_e)), be.shape[0],
                                 _p(_c(be, np.int64)), _p(_c(model.body_bx)), _p(_c(model.body_by)), ee.shape[0],
                                 _p(_c(ee, np.int64)), _p(_c(model.edge_side, np.int64)),
                                 _p(_c(model.edge_kind, np.int64)), _p(_c(model.edge_first)),
                                 _p(_c(model.edge_second)), _p(f))
    if rc != 0:
        raise RuntimeError("element load evaluation failed")
    out["timing"]["loads_ms"] = (time.perf_counter() - t) * 1e3
    out.update(K=K.copy(), f=f.copy())
    if stop_after == "assembly":
        return out
    cd, cv = model.constraints()
    Kc, fc = K.copy(), f.copy()
    t = time.perf_counter()
    rc = lib().lfo_apply_dirichlet(n, _p(_c(rp, np.int64)), _p(_c(col, np.int64)), _p(Kc), _p(fc), cd.shape[0],
                                   _p(_c(cd, np.int64)), _p(_c(cv)))
    out["timing"]["boundary_ms"] = (time.perf_counter() - t) * 1e3
    if rc != 0:
        raise RuntimeError("the structure is a mechanism")
    out.update(Kc=Kc, fc=fc, constraint_dofs=cd, constraint_values=cv)
    if stop_after == "dirichlet":
        return out
    u, rep = pcg(rp, col, Kc, fc, tolerance, max_iterations, storage, preconditioner, split, nodes_per,
                 model.xy, iteration_cap)
    out["u"] = u
    out["report"] = rep
    out["R"] = spmv(rp, col, K, u) - f
    return out
