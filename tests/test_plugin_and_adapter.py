"""The drop-in boundary as a SimAll host sees it: the reference's own
PluginLoader loads libsimall_gpu.so (plugins/IPlugin.hpp ABI v1) and files it
under the Gpu category, and the header-only ILinearSolver adapter
(include/simall_gpu_solver.hpp) compiles against SimAll's headers and solves
through the library."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER_TEST = os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp")


def _reference_src():
    """src/ of the reference tree oracle/build_ref.sh compiled (recorded in
    oracle/_ref/REFERENCE_ROOT), or SIMALL_REFERENCE's; None where neither."""
    root = os.environ.get("SIMALL_REFERENCE")
    rec = os.path.join(ROOT, "oracle", "_ref", "REFERENCE_ROOT")
    if not root and os.path.exists(rec):
        with open(rec) as f:
            root = f.read().strip()
    return os.path.join(root, "src") if root and os.path.isdir(os.path.join(root, "src")) else None


def test_reference_plugin_loader_accepts_library(sg, ref):
    cookie, name, version, category = ref.plugin_load(sg._lib.lib_path())
    assert cookie > 0
    assert name == "simall_gb300_pressure" and version
    assert category == 23  # PluginCategory::Gpu, plugins/SimAllPluginSdk.hpp:96


def test_adapter_compiles_against_reference_headers():
    src = _reference_src()
    if src is None:
        pytest.skip("SimAll source tree not present")
    subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Werror", f"-I{src}",
                    f"-I{os.path.dirname(src)}", f"-I{ROOT}/include", ADAPTER_TEST], check=True)


@pytest.mark.gpu
def test_adapter_solves_through_the_library(sg, tmp_path):
    lib = sg._lib.lib_path()
    exe = str(tmp_path / "adapter_main")
    subprocess.run(["g++", "-std=c++20", "-O1", f"-I{ROOT}/tests/cpp/standin", f"-I{ROOT}/include", ADAPTER_TEST,
                    "-o", exe, lib, f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" ok") == 5
