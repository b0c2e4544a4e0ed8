"""lue_gb300 — GB300-native flow routing (accu, accu_threshold, accu_fraction, kinematic_wave and the
inflow-count / downstream-ordering machinery under them) behind LUE's operation interface.

- ``lue_gb300.framework``: the Python mirror of ``lue.framework``'s routing operations.
- ``include/lue_gb300.h``: the C ABI (liblue_gb300.so), for C, C++ and FFI callers.
- ``lue_gb300/csrc/lue_gb300.hpp``: the C++ mirror of ``lue::value_policies::`` over that ABI.
"""
__version__ = "0.1.0"


def build(force=False, verbose=False):
    """Compile liblue_gb300.so (nvcc, sm_103a) and liblue_synth.so in-tree."""
    from . import _build
    return _build.build_all(force=force, verbose=verbose)
