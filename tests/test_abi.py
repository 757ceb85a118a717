"""The C-ABI library: it loads, exports every entry point declared in
include/*.h, and its host-only parts (mesh generation, RCM) reproduce the
reference's output bit for bit.  No GPU needed."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from helpers import bits_equal

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(simall_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(sg):
    lib = sg._lib.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    assert len(declared_functions()) >= 39
    for n in ("CreatePlugin", "GetPluginAbi"):
        assert n in exported


def test_plugin_abi_version(sg):
    L = sg.load()
    assert L.GetPluginAbi() == 1  # kPluginAbiVersion, plugins/IPlugin.hpp:20


def test_status_strings(sg):
    L = sg.load()
    for code in range(16):
        assert L.simall_status_string(code) and L.simall_status_string(code) != b"unknown status"
    assert L.simall_version().startswith(b"simall_gb300")


def test_context_without_gpu_fails_loudly(sg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sg.SimallError) as e:
        sg.Context(0)
    assert e.value.status == 12


def test_null_arguments_rejected(sg):
    L = sg.load()
    assert L.simall_solver_create(None, None, None) == 1
    assert L.simall_solver_solve(None, None, None, 0, None) == 1
    assert L.simall_pressure_system_create(None, None, None, 0, None) == 1
    assert L.simall_gpu_axpy(1.0, None, None, 3, None) == 1


@pytest.mark.parametrize("case", ["box_6x5x4_distorted.npz", "box_8x8x8_rcm_walls.npz", "box_9x7x5_rcm_outlet.npz",
                                  "cavity_16x16x1_mesh.npz"])
def test_host_mesh_generator_matches_reference_fixture(sg, case):
    from simall_gb300 import workloads as W

    g = np.load(os.path.join(GOLD, case))
    nx, ny, nz = (int(v) for v in g["dims"])
    amp = float(g["amp"])
    shift = W.interior_node_shift(nx, ny, nz, amp=amp, seed=int(g["seed"])) if amp else None
    m = sg.cartesian(nx, ny, nz, node_shift=shift)
    if int(g["renumber"]):
        st = sg.rcm(m)
        assert st == tuple(int(v) for v in g["rcm_stats"])
    nb = np.where(m.neighbor == sg.mesh.BOUNDARY, -1, m.neighbor.astype(np.int64))
    assert np.array_equal(m.owner.astype(np.int64), g["owner"]) and np.array_equal(nb, g["neighbor"])
    assert np.array_equal(m.boundary_zone, g["zone"])
    assert np.array_equal(m.cell_face_offsets, g["cfOff"])
    assert np.array_equal(m.cell_face_indices.astype(np.int64), g["cfIdx"])
    for mine, ref in [("area_x", "ax"), ("area_y", "ay"), ("area_z", "az"), ("centroid_x", "fcx"),
                      ("centroid_y", "fcy"), ("centroid_z", "fcz"), ("volume", "vol"), ("cell_centroid_x", "ccx"),
                      ("cell_centroid_y", "ccy"), ("cell_centroid_z", "ccz")]:
        assert bits_equal(getattr(m, mine), g[ref]), mine


def test_host_mesh_larger_against_oracle(sg, oracle):
    from simall_gb300 import workloads as W

    dims = (14, 11, 9)
    sh = W.interior_node_shift(*dims, seed=21)
    m = sg.cartesian(*dims, node_shift=sh)
    o = oracle.cartesian_mesh(*dims, node_shift=sh)
    assert bits_equal(m.area_x, o.ax) and bits_equal(m.volume, o.vol) and bits_equal(m.cell_centroid_z, o.ccz)
    st = sg.rcm(m)
    _, ost = oracle.rcm(o)
    assert st == ost and np.array_equal(m.owner.astype(np.int64), o.owner)
