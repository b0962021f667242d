"""The library's element colouring against the oracle's restatement of the
reference's (element_colors, src/solver.cpp:100-133), on the CPU.

lfgpu_build_pattern colours the mesh on a host thread with a first fit from
per-node colour masks, and falls back to the walk over node -> element lists when
a mesh needs more than 64 colours.  tests/host/colors_check.cpp runs both on a
mesh file; both must equal the oracle's colours element for element, on Q4 grids
in natural and RCM node order, random connectivity, and meshes with a node in
every element (one colour per element: the fallback).
"""

import os
import subprocess

import numpy as np
import pytest

from host_cpp import ROOT
from lightfem_gb300 import mesh


@pytest.fixture(scope="module")
def colors_check(tmp_path_factory):
    out = tmp_path_factory.mktemp("colors")
    exe = os.path.join(out, "colors_check")
    subprocess.run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fopenmp", "-I",
                    os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "lightfem_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "host", "colors_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)

    def run(n_nodes, en, name):
        en = np.ascontiguousarray(en, dtype=np.int32)
        path, res = os.path.join(out, name + ".bin"), os.path.join(out, name + ".out")
        with open(path, "wb") as fh:
            fh.write(np.array([n_nodes, en.shape[0]], np.int64).tobytes())
            fh.write(en.tobytes())
        subprocess.run([exe, path, res], check=True)
        got = np.fromfile(res, np.int32)
        return got[: en.shape[0]], got[en.shape[0]:]

    return run


def _grid(rcm):
    m = mesh.workload(1, scale=4)  # 50x50 cantilever
    m.sort_and_index()
    if rcm:
        from lightfem_gb300 import _native
        m.index_with_node_order(_native.host_rcm(m.node_ids, m.element_nodes))
    return m.n_nodes, m.element_node_index()


def _random(seed, hub):
    rng = np.random.default_rng(seed)
    n_nodes, n_elem = int(rng.integers(50, 2000)), int(rng.integers(1, 3000))
    en = rng.integers(0, n_nodes, size=(n_elem, 4))
    if hub:
        en[:, 0] = 0
    return n_nodes, en


CASES_ = {
    "grid_natural": lambda: _grid(False),
    "grid_rcm": lambda: _grid(True),
    **{f"random_{k}": (lambda k=k: _random(k, False)) for k in range(6)},
    **{f"hub_{k}": (lambda k=k: _random(100 + k, True)) for k in range(3)},
    "fan_64": lambda: (1 + 3 * 64, np.array([[0, 1 + 3 * e, 2 + 3 * e, 3 + 3 * e] for e in range(64)])),
    "fan_65": lambda: (1 + 3 * 65, np.array([[0, 1 + 3 * e, 2 + 3 * e, 3 + 3 * e] for e in range(65)])),
}


@pytest.mark.parametrize("name", list(CASES_))
def test_colours_equal_oracle(colors_check, oracle, name):
    n_nodes, en = CASES_[name]()
    by_masks, by_lists = colors_check(n_nodes, en, name)
    want = oracle.colors(n_nodes, en)
    np.testing.assert_array_equal(by_masks, want)
    np.testing.assert_array_equal(by_lists, want)
