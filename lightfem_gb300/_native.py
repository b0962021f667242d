"""ctypes binding of liblfgpu.so (the C ABI declared in include/lfgpu.h).

Loading fails loudly: there is no CPU fallback anywhere in this package.  If the
library is missing, build it with ``lightfem_gb300.build.build()``.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p

import numpy as np

# The in-tree build; LFGPU_LIBRARY names another build of the same sources.
LIB_PATH = os.environ.get("LFGPU_LIBRARY") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib",
                                                           "liblfgpu.so")

# enums of include/lfgpu.h
OK = 0
ERR_ARGUMENT, ERR_CUDA, ERR_STATE, ERR_JACOBIAN, ERR_EDGE, ERR_MECHANISM = 1, 2, 3, 4, 5, 6
ERR_NOT_SPD, ERR_RHO_INITIAL, ERR_RHO, ERR_NONFINITE_DIAG, ERR_TIMEOUT, ERR_NOMEM, ERR_UNSUPPORTED = (
    7, 8, 9, 10, 11, 12, 13)
ERR_SCRATCH_LIMIT = 14
NOALLOC_MAX_ROWS = 4194304  # LFGPU_NOALLOC_MAX_ROWS
ASSEMBLY = {"coloring": 0, "atomic": 1}
STORAGE = {"csr": 0, "bsr": 1}
PRECOND = {"jacobi": 0, "block": 1, "ic0": 2, "subdomain": 3}  # block: 2x2 nodal; subdomain: any size
SPLIT = {"rcb": 0, "chunk": 1}
SUBDOMAIN_MAX_DOFS = 1024  # LFGPU_SUBDOMAIN_MAX_DOFS
PRECISION = {"fp64": 0, "mixed": 1}
REFINEMENT = {"reliable": 0, "restart": 1}
K_FULL, K_CONSTRAINED, F_FULL, F_CONSTRAINED, U, R = range(6)
OPTION_WAIT_LIMIT_NS, OPTION_IC0_SWEEP = 0, 1  # lfgpu_set_option
IC0_SWEEP = {"auto": 0, "levels": 1, "polled": 2}


class SolveOptions(ctypes.Structure):
    _fields_ = [("tolerance", c_double), ("max_iterations", c_int64), ("storage", c_int32),
                ("preconditioner", c_int32), ("precision", c_int32), ("refinement", c_int32),
                ("inner_reduction", c_double), ("max_refinements", c_int64), ("persistent", c_int32),
                ("unrolled", c_int32)]


class Report(ctypes.Structure):
    _fields_ = [("converged", c_int32), ("status", c_int32), ("iterations", c_int64), ("refinements", c_int64),
                ("initial_residual", c_double), ("final_residual", c_double), ("true_residual", c_double),
                ("solve_ms", c_double), ("matvec_ms", c_double), ("matvec_calls", c_int64),
                ("matrix_bytes_per_matvec", c_int64), ("storage_convert_ms", c_double),
                ("preconditioner_setup_ms", c_double), ("preconditioner_apply_ms", c_double),
                ("subdomains", c_int64), ("capture_ratio", c_double), ("degenerate_subdomains", c_int64),
                ("ic0_breakdowns", c_int64), ("ic0_levels", c_int64), ("fallback_fp64", c_int64),
                ("phase_ms", c_double * 6)]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["phase_ms"] = list(self.phase_ms)
        return d


class Timings(ctypes.Structure):
    _fields_ = [("pattern_ms", c_double), ("assembly_ms", c_double), ("boundary_ms", c_double),
                ("reactions_ms", c_double), ("coloring_count", c_int64), ("kernel_launches", c_int64),
                ("postprocess_ms", c_double), ("rcm_ms", c_double), ("adjoint_kernel_ms", c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GpuError(RuntimeError):
    """A non-zero status from liblfgpu; ``code`` is the lfgpu_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


_lib = None

_SIGNATURES = {
    "lfgpu_create": (c_int, [c_int, POINTER(c_void_p)]),
    "lfgpu_destroy": (c_int, [c_void_p]),
    "lfgpu_last_error": (c_char_p, [c_void_p]),
    "lfgpu_version": (c_char_p, []),
    "lfgpu_failure_detail": (c_int, [c_void_p, POINTER(c_int32), POINTER(c_int64), c_void_p]),
    "lfgpu_set_option": (c_int, [c_void_p, c_int32, c_int64]),
    "lfgpu_set_mesh": (c_int, [c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_void_p, c_int64, c_void_p,
                               c_void_p, c_void_p, c_int32]),
    "lfgpu_set_young": (c_int, [c_void_p, c_void_p]),
    "lfgpu_set_pattern": (c_int, [c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "lfgpu_build_pattern": (c_int, [c_void_p]),
    "lfgpu_pattern_info": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    "lfgpu_download_pattern": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "lfgpu_set_loads": (c_int, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                                c_void_p, c_void_p, c_void_p, c_void_p]),
    "lfgpu_set_constraints": (c_int, [c_void_p, c_int64, c_void_p, c_void_p]),
    "lfgpu_assemble": (c_int, [c_void_p, c_int32]),
    "lfgpu_apply_dirichlet": (c_int, [c_void_p]),
    "lfgpu_solve": (c_int, [c_void_p, POINTER(SolveOptions), c_void_p, POINTER(Report)]),
    "lfgpu_reactions": (c_int, [c_void_p, c_void_p]),
    "lfgpu_download": (c_int, [c_void_p, c_int32, c_void_p]),
    "lfgpu_timings_get": (c_int, [c_void_p, POINTER(Timings)]),
    "lfgpu_event_record": (c_int, [c_void_p, c_int32]),
    "lfgpu_event_elapsed": (c_int, [c_void_p, c_int32, c_int32, POINTER(c_double)]),
    "lfgpu_spmv": (c_int, [c_void_p, c_int32, c_int32, c_int32, c_void_p, c_void_p, c_int32, POINTER(c_double)]),
    "lfgpu_adjoint": (c_int, [c_void_p, c_void_p, POINTER(SolveOptions), c_void_p, POINTER(Report)]),
    "lfgpu_postprocess": (c_int, [c_void_p, c_void_p, c_void_p]),
    "lfgpu_rcm": (c_int, [c_void_p, c_void_p]),
    "lfgpu_mesh_profile": (c_int, [c_void_p, c_void_p]),
    "lfgpu_apply_preconditioner": (c_int, [c_void_p, c_int32, c_void_p, c_void_p, POINTER(c_double)]),
    "lfgpu_residual_norm_noalloc": (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                            POINTER(c_double)]),
    "lfgpu_set_subdomains": (c_int, [c_void_p, c_int64, c_int32]),
    "lfgpu_host_rcm": (c_int, [c_int64, c_void_p, c_int64, c_void_p, c_void_p]),
    "lfgpu_host_subdomains": (c_int, [c_int64, c_void_p, c_int64, c_int32, c_void_p, POINTER(c_int64)]),
}

EXPORTED = tuple(_SIGNATURES)


def library() -> ctypes.CDLL:
    """Load liblfgpu.so once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with lightfem_gb300.build.build() "
                              "(the CUDA path has no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _arr(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a), dtype=dtype)


def host_rcm(node_ids: np.ndarray, element_node_ids: np.ndarray) -> np.ndarray:
    """reverse_cuthill_mckee (src/reordering.cpp:11-62) on node IDs -> new ID order."""
    ids = _arr(node_ids, np.int64)
    en = _arr(element_node_ids, np.int64).reshape(-1)
    out = np.empty(ids.shape[0], np.int64)
    rc = library().lfgpu_host_rcm(ids.shape[0], _ptr(ids), en.shape[0] // 4, _ptr(en), _ptr(out))
    if rc != OK:
        raise GpuError(rc, "RCM ordering failed: element references an unknown node ID")
    return out


def host_subdomains(xy: np.ndarray, nodes_per_subdomain: int, split: str = "rcb") -> tuple[np.ndarray, int]:
    """split_by_coordinates / split_by_chunks (src/precond.cpp:19-105): the
    subdomain of every node (node index order) and the subdomain count."""
    pts = _arr(xy, np.float64).reshape(-1, 2)
    owner = np.empty(pts.shape[0], np.uint32)
    count = c_int64()
    rc = library().lfgpu_host_subdomains(pts.shape[0], _ptr(pts), int(nodes_per_subdomain), SPLIT[split],
                                         _ptr(owner), ctypes.byref(count))
    if rc != OK:
        raise GpuError(rc, f"subdomain split failed with status {rc}")
    return owner, int(count.value)


def residual_norm_noalloc(n_rows: int, row_offsets: int, columns: int, values: int, u: int, f: int,
                          stream: int | None = None) -> float:
    """||f - K u||_2 of a CSR system in the caller's device memory (raw device
    pointers: int32 offsets and columns, float64 values, u and f), computed with
    no device allocation; see lfgpu_residual_norm_noalloc in include/lfgpu.h."""
    out = c_double()
    rc = library().lfgpu_residual_norm_noalloc(int(n_rows), row_offsets, columns, values, u, f, stream,
                                               ctypes.byref(out))
    if rc == ERR_SCRATCH_LIMIT:
        raise GpuError(rc, f"residual_norm_noalloc: {n_rows} rows exceed the static scratch limit of "
                           f"{NOALLOC_MAX_ROWS} rows")
    if rc != OK:
        raise GpuError(rc, f"residual_norm_noalloc failed with status {rc}")
    return out.value


class Context:
    """One liblfgpu handle: a CUDA stream and the device copy of one model."""

    def __init__(self, device: int = 0):
        self._lib = library()
        h = c_void_p()
        rc = self._lib.lfgpu_create(device, ctypes.byref(h))
        if rc != OK:
            raise GpuError(rc, f"lfgpu_create failed with status {rc} (is a CUDA device visible?)")
        self._h = h
        self.n_dofs = 0
        self.nnz = 0
        self.n_elements = 0

    # -- plumbing
    def _check(self, rc: int) -> None:
        if rc != OK:
            msg = self._lib.lfgpu_last_error(self._h).decode()
            raise GpuError(rc, msg)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.lfgpu_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_option(self, option: int, value: int) -> None:
        """lfgpu_set_option: OPTION_WAIT_LIMIT_NS (ns) or OPTION_IC0_SWEEP (IC0_SWEEP values)."""
        self._check(self._lib.lfgpu_set_option(self._h, option, value))

    # -- model
    def set_mesh(self, xy, element_nodes, element_material, young, poisson, thickness, plane_mode: int) -> None:
        xy = _arr(xy, np.float64).reshape(-1, 2)
        en = _arr(element_nodes, np.int32).reshape(-1, 4)
        em = _arr(element_material, np.int32).reshape(-1)
        young = _arr(young, np.float64)
        poisson = _arr(poisson, np.float64)
        thickness = _arr(thickness, np.float64)
        self._keep_mesh = (xy, en, em, young, poisson, thickness)
        self._check(self._lib.lfgpu_set_mesh(self._h, xy.shape[0], _ptr(xy), en.shape[0], _ptr(en), _ptr(em),
                                             young.shape[0], _ptr(young), _ptr(poisson), _ptr(thickness),
                                             int(plane_mode)))
        self.n_dofs = 2 * xy.shape[0]
        self.n_elements = en.shape[0]

    def set_young(self, young) -> None:
        young = _arr(young, np.float64)
        self._check(self._lib.lfgpu_set_young(self._h, _ptr(young)))

    def set_pattern(self, row_offsets, columns, element_value_index, element_color=None) -> None:
        rp = _arr(row_offsets, np.int64)
        col = _arr(columns, np.int32)
        mp = _arr(element_value_index, np.int32).reshape(-1)
        colors = None if element_color is None else _arr(element_color, np.int32)
        self._check(self._lib.lfgpu_set_pattern(self._h, rp.shape[0] - 1, col.shape[0], _ptr(rp), _ptr(col),
                                                _ptr(mp), _ptr(colors)))
        self.nnz = col.shape[0]

    def build_pattern(self) -> None:
        self._check(self._lib.lfgpu_build_pattern(self._h))
        n, nnz, nc = c_int64(), c_int64(), c_int64()
        self._check(self._lib.lfgpu_pattern_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(nc)))
        self.nnz = nnz.value
        self.n_colors = nc.value

    def download_pattern(self):
        rp = np.empty(self.n_dofs + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        mp = np.empty(self.n_elements * 64, np.int32)
        colors = np.empty(self.n_elements, np.int32)
        self._check(self._lib.lfgpu_download_pattern(self._h, _ptr(rp), _ptr(col), _ptr(mp), _ptr(colors)))
        return rp, col, mp.reshape(-1, 64), colors

    def set_loads(self, nodal=None, body_element=None, body_bx=None, body_by=None, edge_element=None,
                  edge_side=None, edge_kind=None, edge_first=None, edge_second=None) -> None:
        nodal = None if nodal is None else _arr(nodal, np.float64)
        nb = 0 if body_element is None else len(body_element)
        ne = 0 if edge_element is None else len(edge_element)
        be = _arr(body_element if nb else np.zeros(0), np.int32)
        bx = _arr(body_bx if nb else np.zeros(0), np.float64)
        by = _arr(body_by if nb else np.zeros(0), np.float64)
        ee = _arr(edge_element if ne else np.zeros(0), np.int32)
        es = _arr(edge_side if ne else np.zeros(0), np.int32)
        ek = _arr(edge_kind if ne else np.zeros(0), np.int32)
        ea = _arr(edge_first if ne else np.zeros(0), np.float64)
        eb = _arr(edge_second if ne else np.zeros(0), np.float64)
        self._check(self._lib.lfgpu_set_loads(self._h, _ptr(nodal), nb, _ptr(be), _ptr(bx), _ptr(by), ne,
                                              _ptr(ee), _ptr(es), _ptr(ek), _ptr(ea), _ptr(eb)))

    def set_constraints(self, dofs, values) -> None:
        d = _arr(dofs, np.int64)
        v = _arr(values, np.float64)
        self._check(self._lib.lfgpu_set_constraints(self._h, d.shape[0], _ptr(d), _ptr(v)))

    # -- solve path
    def assemble(self, strategy: str = "coloring") -> None:
        self._check(self._lib.lfgpu_assemble(self._h, ASSEMBLY[strategy]))

    def apply_dirichlet(self) -> None:
        self._check(self._lib.lfgpu_apply_dirichlet(self._h))

    @staticmethod
    def options(tolerance: float, max_iterations: int, storage: str = "csr", preconditioner: str = "jacobi",
                precision: str = "fp64", refinement: str = "reliable", inner_reduction: float = 0.0,
                max_refinements: int = 0, persistent: int = 0, unrolled: int = 0) -> SolveOptions:
        return SolveOptions(float(tolerance), int(max_iterations), STORAGE[storage], PRECOND[preconditioner],
                            PRECISION[precision], REFINEMENT[refinement], float(inner_reduction),
                            int(max_refinements), int(persistent), int(unrolled))

    def solve(self, options: SolveOptions, download: bool = True):
        rep = Report()
        u = np.empty(self.n_dofs) if download else None
        rc = self._lib.lfgpu_solve(self._h, ctypes.byref(options), _ptr(u), ctypes.byref(rep))
        if rc != OK:
            msg = self._lib.lfgpu_last_error(self._h).decode()
            err = GpuError(rc, msg)
            err.report = rep
            raise err
        return u, rep

    def reactions(self, download: bool = True):
        r = np.empty(self.n_dofs) if download else None
        self._check(self._lib.lfgpu_reactions(self._h, _ptr(r)))
        return r

    def download(self, which: int) -> np.ndarray:
        size = self.nnz if which in (K_FULL, K_CONSTRAINED) else self.n_dofs
        out = np.empty(size)
        self._check(self._lib.lfgpu_download(self._h, which, _ptr(out)))
        return out

    def failure_detail(self) -> tuple[int, int, float, float]:
        """(status, index, load, diagonal) of the last failure a kernel reported
        (``lfgpu_failure_detail``); load and diagonal are set for a zero pivot
        carrying load."""
        status, index = c_int32(0), c_int64(0)
        values = np.zeros(2)
        self._check(self._lib.lfgpu_failure_detail(self._h, ctypes.byref(status), ctypes.byref(index),
                                                   values.ctypes.data))
        return int(status.value), int(index.value), float(values[0]), float(values[1])

    def timings(self) -> dict:
        t = Timings()
        self._check(self._lib.lfgpu_timings_get(self._h, ctypes.byref(t)))
        return t.as_dict()

    def event_record(self, slot: int) -> None:
        """Record event ``slot`` on this handle's stream (device timing across calls)."""
        self._check(self._lib.lfgpu_event_record(self._h, int(slot)))

    def event_elapsed(self, slot_a: int, slot_b: int) -> float:
        ms = c_double()
        self._check(self._lib.lfgpu_event_elapsed(self._h, int(slot_a), int(slot_b), ctypes.byref(ms)))
        return ms.value

    def spmv(self, x, which: int = 1, storage: str = "csr", precision: str = "fp64", repeat: int = 1):
        x = _arr(x, np.float64)
        y = np.empty(self.n_dofs)
        ms = c_double()
        self._check(self._lib.lfgpu_spmv(self._h, which, STORAGE[storage], PRECISION[precision], _ptr(x), _ptr(y),
                                         int(repeat), ctypes.byref(ms)))
        return y, ms.value

    def mesh_profile(self) -> dict:
        """csr_profile of the pattern this mesh produces (dimension, nonzeros,
        bandwidth, profile), computed on the device."""
        out = np.empty(4, np.int64)
        self._check(self._lib.lfgpu_mesh_profile(self._h, _ptr(out)))
        return dict(zip(("dimension", "nonzeros", "bandwidth", "profile"), (int(v) for v in out)))

    def rcm(self) -> np.ndarray:
        """Reverse Cuthill-McKee order of this mesh's node indices, on the device."""
        out = np.empty(self.n_dofs // 2, np.int64)
        self._check(self._lib.lfgpu_rcm(self._h, _ptr(out)))
        return out

    def postprocess(self):
        """Element fields (E x 5 x 7: centre + 4 Gauss points; strain xx, yy, xy,
        stress xx, yy, xy, von Mises) and smoothed nodal stress (N x 4)."""
        fields = np.empty((self.n_elements, 5, 7))
        nodal = np.empty((self.n_dofs // 2, 4))
        self._check(self._lib.lfgpu_postprocess(self._h, _ptr(fields), _ptr(nodal)))
        return fields, nodal

    def set_subdomains(self, nodes_per_subdomain: int = 64, split: str = "rcb") -> None:
        """The split of the "subdomain" preconditioner (subdomain_nodes, subdomain_split)."""
        self._check(self._lib.lfgpu_set_subdomains(self._h, int(nodes_per_subdomain), SPLIT[split]))

    def apply_preconditioner(self, r, preconditioner: str = "jacobi"):
        """z = M^-1 r for the constrained K; returns (z, device ms)."""
        r = _arr(r, np.float64)
        z = np.empty(self.n_dofs)
        ms = c_double()
        self._check(self._lib.lfgpu_apply_preconditioner(self._h, PRECOND[preconditioner], _ptr(r), _ptr(z),
                                                         ctypes.byref(ms)))
        return z, ms.value

    def adjoint(self, dj_du=None, options: SolveOptions | None = None):
        grad = np.empty(self.n_elements)
        rep = Report()
        d = None if dj_du is None else _arr(dj_du, np.float64)
        self._check(self._lib.lfgpu_adjoint(self._h, _ptr(d), None if options is None else ctypes.byref(options),
                                            _ptr(grad), ctypes.byref(rep)))
        return grad, rep
