"""The test plugin library (tests/plugins/di_plugins.cu) and the ctypes mirrors of its structs."""
import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "plugins" / "di_plugins.cu"
# the oracle's model ids for the three pairs (oracle/mppi_oracle.cpp, TestDIPlugin)
ORACLE_MODEL = {"di_quadratic": 101, "di_symplectic_quadratic": 102, "di_constrained_quadratic": 103}


class DIPlugin(C.Structure):
    _fields_ = [("damping", C.c_float)]


class DIConstrainedPlugin(C.Structure):
    _fields_ = [("damping", C.c_float), ("a_max", C.c_float), ("speed_gain", C.c_float)]


class QuadraticWallCost(C.Structure):
    _fields_ = [("s_goal", C.c_float * 4), ("s_coeffs", C.c_float * 4), ("wall_x", C.c_float),
                ("crash_cost", C.c_float), ("terminal_coeff", C.c_float)]


def library_path():
    from mppi_generic_vendor_gb300.plugin import build_plugin

    return build_plugin(SOURCE)
