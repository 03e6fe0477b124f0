"""GB300-native (sm_103a) single-bunch turn loop with PyHEADTAIL's API.

The package keeps PyHEADTAIL's element classes and their ``track(beam)``
contract for the hot path -- transverse segment maps with chromaticity and
amplitude detuning, RF systems / linear longitudinal maps, uniform-bin
slicing and multi-turn resonator / resistive-wall wakes -- and runs the
per-particle work in hand-written CUDA kernels behind the C ABI of
``include/pyheadtail_gb300.h`` (``libphk.so``).

Module layout follows the reference: ``particles.particles.Particles``,
``particles.slicing.UniformBinSlicer``, ``trackers.transverse_tracking``,
``trackers.detuners``, ``trackers.longitudinal_tracking``,
``impedances.wakes`` and ``impedances.wake_kicks``; ``batched`` runs many
bunches in one launch and ``turngraph`` captures a whole turn in a CUDA
graph.
"""
__version__ = '0.1.0'


def load_library():
    """Build (if needed) and load libphk.so; raises if that fails."""
    from . import _native
    return _native.load()
