"""Callers' own Dynamics / Cost plugins (include/mppi_gb_plugin.cuh) from Python.

``build_plugin(source)`` compiles a .cu file that expands ``MPPI_GB_PLUGIN(name, Dyn, Cost)`` into a shared library
linked against libmppi_gb.so (the engine is instantiated over the plugin pair inside that library, with the engine's
own compile flags).  ``PluginLibrary(path, name)`` loads it; ``PluginDynamics`` / ``PluginCost`` hold the plugin
structs as ctypes structures whose fields mirror the C++ structs; ``PluginMPPIController`` is a
``BatchedMPPIController`` whose handle the plugin library's ``name_create`` made — every other method is the
same C entry point as for the built-in models; ``PluginTubeMPPIController`` and ``PluginRobustMPPIController`` are
the Tube-MPPI and R-MPPI controllers over a plugin pair (the reference's controllers take any Dynamics / Cost pair).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

from . import _abi as A
from . import build as B
from .controller import BatchedMPPIController, RobustMPPIController, TubeMPPIController, _Plugin

INCLUDE = B.INCLUDE


def build_plugin(source, out_dir=None, name=None, extra_flags=()) -> Path:
    """Compile `source` into lib<stem>.so (in out_dir, default a _build folder beside the source) for sm_103a with
    the engine's flags; rebuilt when the source, the engine headers or libmppi_gb.so are newer than the library."""
    src = Path(source).resolve()
    out_dir = Path(out_dir) if out_dir is not None else src.parent / "_build"
    out_dir.mkdir(parents=True, exist_ok=True)
    lib = out_dir / f"lib{name or src.stem}.so"
    engine_lib = B.build()
    deps = [src, engine_lib, *INCLUDE.glob("*"), *B.CSRC.glob("*.cuh")]
    if lib.exists() and lib.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return lib
    cmd = [B.nvcc_path(), *B.ARCH_FLAGS, *B.NVCC_FLAGS, "-diag-suppress", "128", *extra_flags, "-shared",
           "-o", str(lib), str(src), "-L" + str(engine_lib.parent), "-lmppi_gb",
           "-Xlinker", "-rpath," + str(engine_lib.parent), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return lib


class PluginLibrary:
    """A compiled plugin library and one plugin pair `name` it exports (name_create, name_model_dims,
    name_param_sizes)."""

    def __init__(self, path, name):
        A.lib()  # the engine library first: the plugin library resolves its engine symbols against it
        self.path = Path(path)
        self.name = name
        self._lib = C.CDLL(str(self.path))
        self._create = getattr(self._lib, f"{name}_create")
        self._create.restype = C.c_int
        self._create.argtypes = [C.c_int, A._IP, A._IP, C.POINTER(A.ControllerParams), C.POINTER(A.SamplingParams),
                                 C.POINTER(A.ControlConstraints), A._P, C.c_size_t, A._P, C.c_size_t, A._FP, A._P,
                                 C.POINTER(A._P)]
        dims = getattr(self._lib, f"{name}_model_dims")
        dims.restype = C.c_int
        s, c, o = C.c_int(), C.c_int(), C.c_int()
        A.check(dims(C.byref(s), C.byref(c), C.byref(o)), f"{name}_model_dims")
        self.STATE_DIM, self.CONTROL_DIM, self.OUTPUT_DIM = s.value, c.value, o.value
        sizes = getattr(self._lib, f"{name}_param_sizes")
        sizes.restype = C.c_int
        db, cb = C.c_size_t(), C.c_size_t()
        A.check(sizes(C.byref(db), C.byref(cb)), f"{name}_param_sizes")
        self.dyn_bytes, self.cost_bytes = db.value, cb.value

    def create(self, *args):
        A.check(self._create(*args), f"{self.name}_create")


class PluginDynamics(_Plugin):
    """The dynamics struct of a plugin pair (a ctypes structure laid out as the C++ struct)."""

    model_id = A.MODEL_PLUGIN

    def __init__(self, library: PluginLibrary, params):
        if C.sizeof(params) != library.dyn_bytes:
            raise ValueError(f"dynamics struct is {C.sizeof(params)} bytes; the plugin's is {library.dyn_bytes}")
        super().__init__(params)
        self.library = library
        self.STATE_DIM, self.CONTROL_DIM, self.OUTPUT_DIM = (library.STATE_DIM, library.CONTROL_DIM,
                                                             library.OUTPUT_DIM)
        flt_max = 3.4028234663852886e38
        self.control_rngs = [(-flt_max, flt_max)] * self.CONTROL_DIM

    def setControlRanges(self, ranges):
        self.control_rngs = [tuple(r) for r in ranges]


class PluginCost(_Plugin):
    """The cost struct of a plugin pair."""

    def __init__(self, library: PluginLibrary, params):
        if C.sizeof(params) != library.cost_bytes:
            raise ValueError(f"cost struct is {C.sizeof(params)} bytes; the plugin's is {library.cost_bytes}")
        super().__init__(params)
        self.library = library


class PluginMPPIController(BatchedMPPIController):
    """BatchedMPPIController over a plugin pair: one PluginDynamics / PluginCost (or one per instance)."""

    def _create_handle(self, cp, sp, cc, init, stream):
        lib = self.model_.library
        dyn_t, cost_t = type(self._dyn_arr[0]), type(self._cost_arr[0])
        h = C.c_void_p()
        lib.create(self.num_instances, self.K.ctypes.data_as(A._IP), self.T.ctypes.data_as(A._IP), C.byref(cp),
                   C.byref(sp), C.byref(cc), C.cast(self._dyn_arr, C.c_void_p),
                   C.sizeof(dyn_t) * self.num_instances, C.cast(self._cost_arr, C.c_void_p),
                   C.sizeof(cost_t) * self.num_instances, init, C.c_void_p(stream or None), C.byref(h))
        return h


class PluginTubeMPPIController(PluginMPPIController, TubeMPPIController):
    """TubeMPPIController over a plugin pair: TubeMPPIController's constructor and methods, the plugin library's
    handle."""


class PluginRobustMPPIController(PluginMPPIController, RobustMPPIController):
    """RobustMPPIController over a plugin pair: RobustMPPIController's constructor and methods, the plugin library's
    handle.  Both R-MPPI rollouts run the plugin's own step, its computeRunningCost with each system's crash flag and
    its own enforceConstraints when it defines one."""
