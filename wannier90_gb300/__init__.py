"""wannier90_gb300: GB300 (sm_103a) engine for Wannier90's MLWF spread minimisation.

The compute lives in the CUDA library ``lib/libw90gb300.so`` (sources in ``csrc/``),
reached through the reference-named C ABI of ``include/wannier90_gb300.h``.
:mod:`wannier90_gb300.library` mirrors Wannier90's Python/f90wrap library interface,
:mod:`wannier90_gb300.w90io` reads and writes the reference's file formats, and
:mod:`wannier90_gb300.synth` generates the seeded tight-binding workloads.
"""
__all__ = ["library", "w90io", "synth", "build"]
