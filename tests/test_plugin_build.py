"""A caller's plugin pair compiles against include/mppi_gb_plugin.cuh outside the engine's sources and exports the C
entry points MPPI_GB_PLUGIN promises (no GPU: compilation, symbols, and the host-only size / dimension queries)."""
import ctypes as C

import pytest

import _plugins
from mppi_generic_vendor_gb300 import _abi as A
from mppi_generic_vendor_gb300.plugin import PluginCost, PluginDynamics, PluginLibrary


@pytest.fixture(scope="module")
def plugin_lib():
    return _plugins.library_path()


@pytest.mark.parametrize("name,dyn_struct", [("di_quadratic", _plugins.DIPlugin),
                                             ("di_symplectic_quadratic", _plugins.DIPlugin),
                                             ("di_constrained_quadratic", _plugins.DIConstrainedPlugin)])
def test_plugin_library_exports_and_sizes(plugin_lib, name, dyn_struct):
    lib = PluginLibrary(plugin_lib, name)
    assert (lib.STATE_DIM, lib.CONTROL_DIM, lib.OUTPUT_DIM) == (4, 2, 4)
    assert lib.dyn_bytes == C.sizeof(dyn_struct)
    assert lib.cost_bytes == C.sizeof(_plugins.QuadraticWallCost)
    d = PluginDynamics(lib, dyn_struct(0.1))
    assert d.model_id == A.MODEL_PLUGIN and d.STATE_DIM == 4
    PluginCost(lib, _plugins.QuadraticWallCost())
    with pytest.raises(ValueError):
        PluginDynamics(lib, _plugins.QuadraticWallCost())


def test_engine_exports_the_adoption_entry_points():
    for n in ("mppi_handle_adopt", "mppi_get_model_dims"):
        assert hasattr(A.lib(), n)
    h = C.c_void_p()
    # a plugin built against another header version is refused (no engine is touched)
    assert A.lib().mppi_handle_adopt(C.c_void_p(1), A.lib().mppi_abi_version() + 1, C.byref(h)) == A.MPPI_EINVAL
    assert b"ABI version" in A.lib().mppi_last_error_string()
