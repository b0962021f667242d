"""The threaded .fem parser and VTK / CSV writers of the C++ host layer
(lightfem_gb300/host/lightfem_gpu_io.hpp) against the reference's own
(InputParser, src/input_parser.cpp:162-341; write_vtk and write_csv_results,
src/vtk_writer.cpp:110-337), on the CPU.

tests/host/io_check.cpp links the reference's objects (built from its sources by
`make -C oracle ref`) and, for every input, compares the parsed records field by
field, or the failure message when both fail, and the VTK and CSV files byte for
byte after a reference solve.  Skipped where no reference tree is available.
"""

import os
import subprocess

import pytest

from cases import CASES
from host_cpp import ROOT
from lightfem_gb300 import mesh

MESH = {
    "beam": lambda: CASES["beam"](),
    "strain": lambda: CASES["strain"](),
    "grid6": lambda: CASES["grid6"](),
    "cantilever_50x50": lambda: mesh.workload(1, scale=4),
    "cantilever_200x200": lambda: mesh.workload(1),
}

# Inputs that fail: the first failing line decides the message.
BAD = {
    "unknown_section": "[settings]\nsolver pcg\n[nodez]\n1 0 0\n",
    "open_header": "[nodes\n1 0 0\n",
    "data_first": "# header comes later\n1 0 0\n[nodes]\n",
    "bad_number": "[nodes]\n1 0.0 0.0\n2 1.0 abc\n",
    "infinite": "[nodes]\n1 inf 0\n",
    "big_integer": "[nodes]\n99999999999 0 0\n",
    "negative_size": "[settings]\nmax_iterations -5\n",
    "field_count": "[materials]\n1 2e11 0.3\n",
    "duplicate_setting": "[settings]\nsolver pcg\ntolerance 1e-8\nSolver cg\n",
    "unknown_setting": "[settings]\ncolour blue\n",
    "plane_mode": "[settings]\nplane_mode axisymmetric\n",
    "boundary_type": "[boundary]\n1 clamped\n",
    "edge_type": "[edge_loads]\n1 2 shear 5\n",
    "edge_short": "[edge_loads]\n1 2 pressure\n",
    "edge_traction_count": "[edge_loads]\n1 2 traction 5\n",
}

# Inputs that parse (and some that also validate): comments, blanks, CRLF, tabs,
# aliases, constraints and every record kind.
GOOD = {
    "aliases": ("# a tiny frame\r\n[SETTINGS]\r\n  plane_mode   PLANE_STRAIN  \r\nthreads 2\n"
                "deformation_scale 2.5\ncsv_prefix out/x\n\n[materials]\n1\t2e11\t0.3\t0.01 # steel\n"
                "[nodes]\n1 0 0\n2 1 0\n3 1 1\n4 0 1\n5 2 0\n[elements]\n1 1 2 3 4 1\n"
                "[bars]\n7 2 5 1 1e-4\n[dirichlet]\n1 fixed\n4 roller_x\n5 free 0\n"
                "[forces]\n3 0 -1\n[body_loads]\n1 0 -9.81\n[tractions]\n1 2 traction 1 2\n1 3 pressure 4\n"),
}


def _write(tmp_path, name, text):
    path = os.path.join(str(tmp_path), name + ".fem")
    with open(path, "w", newline="") as fh:
        fh.write(text)
    return path


@pytest.fixture(scope="module")
def io_check(tmp_path_factory):
    from oracle.reference import make_args
    args = make_args()
    if not args:
        pytest.skip("no reference tree here")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", *args], check=True)
    out = str(tmp_path_factory.mktemp("io"))
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "tests", "host"), "io-check", *args, f"OUT={out}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(out, "io_check")


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_parser_and_writers_match_reference(io_check, tmp_path, threads):
    files = [_write(tmp_path, name, mesh.to_fem(make(), os.path.join(str(tmp_path), name + ".vtk")))
             for name, make in MESH.items()]
    files += [_write(tmp_path, name, text) for name, text in {**GOOD, **BAD}.items()]
    r = subprocess.run([io_check, str(tmp_path), str(threads), *files], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == len(files), r.stdout
    for name in MESH:
        assert f"{name}.fem (" in r.stdout and "files identical" in r.stdout


def test_earliest_failure_wins_across_pieces(io_check, tmp_path):
    """A large input with two bad lines far apart (in different threads' pieces):
    the earlier line's message, as the serial parser reports it; and a settings
    failure that comes after a record failure does not mask it."""
    text = mesh.to_fem(mesh.workload(1, scale=2), "x.vtk")
    lines = text.split("\n")
    late, early = int(len(lines) * 0.9), int(len(lines) * 0.4)
    lines[late] = "bad line"
    lines[early] = lines[early] + " extra"
    files = [_write(tmp_path, "two_errors", "\n".join(lines))]
    settings_after = "[nodes]\n1 0 x\n[settings]\nsolver a\nsolver b\n"
    files.append(_write(tmp_path, "settings_after", settings_after))
    r = subprocess.run([io_check, str(tmp_path), "6", *files], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f":{early + 1}: expected" in r.stdout
    assert "settings_after.fem:2: invalid number for y: x" in r.stdout
