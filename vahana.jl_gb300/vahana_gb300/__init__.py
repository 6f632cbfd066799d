"""vahana_gb300: GB300-native transition step of Vahana.jl behind its API.

All compute runs in libvahana_gb300.so (hand-written sm_103a kernels); this
package is the host-side mirror of the reference's public functions.
"""
from ._lib import LIBPATH, VahanaError, exported_symbols, lib  # noqa: F401
from .api import *  # noqa: F401,F403
from .api import (Edge, ModelTypes, Simulation, TypeInfo, agent_id, agent_nr,  # noqa: F401
                  apply, apply_, process_nr, type_nr)


def build():
    """Compile the CUDA library in-tree (sm_103a)."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("_vg_build", os.path.join(here, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()
