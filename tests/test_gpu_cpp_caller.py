"""The C ABI from C++ callers: compiles tests/cpp/cartpole_receding_horizon.cpp (plain C ABI) and
tests/cpp/cartpole_mirror.cpp (the C++ host mirror include/mppi_gb.hpp, with the reference's class and method names)
against libmppi_gb.so and runs the reference example's receding-horizon loop (examples/cartpole_example.cu:62-85);
tests/cpp/cartpole_plant.cpp drives the GPU controller through the C++ BasePlant (include/mppi_gb_plant.hpp);
tests/cpp/controllers_mirror.cpp runs the mirror's Colored, Tube and Robust controllers."""
import shutil
import subprocess
from pathlib import Path

import pytest

from mppi_generic_vendor_gb300 import _abi as A

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_cpp_receding_horizon_swings_up(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    lib = Path(A.lib()._name)
    exe = tmp_path / "cartpole"
    subprocess.run([gxx, "-std=c++17", "-O2", str(ROOT / "tests" / "cpp" / "cartpole_receding_horizon.cpp"),
                    "-I", str(ROOT / "include"), str(lib), f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_mirror_receding_horizon(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    lib = Path(A.lib()._name)
    exe = tmp_path / "mirror"
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                    str(ROOT / "tests" / "cpp" / "cartpole_mirror.cpp"), "-I", str(ROOT / "include"), str(lib),
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_base_plant_drives_the_gpu_controller(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    lib = Path(A.lib()._name)
    exe = tmp_path / "plant"
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-pthread",
                    str(ROOT / "tests" / "cpp" / "cartpole_plant.cpp"), "-I", str(ROOT / "include"), str(lib),
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_mirror_colored_tube_robust_controllers(tmp_path):
    """tests/cpp/controllers_mirror.cpp: the C++ mirror's ColoredMPPIController, TubeMPPIController (with the DDP
    feedback) and RobustMPPIController each drive a double integrator to its goal."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    lib = Path(A.lib()._name)
    exe = tmp_path / "controllers"
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                    str(ROOT / "tests" / "cpp" / "controllers_mirror.cpp"), "-I", str(ROOT / "include"), str(lib),
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
