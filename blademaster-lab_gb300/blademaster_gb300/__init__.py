"""GB300-native material substep of BladeMaster-Lab's topology-aware TLMPM cutting solver.

Drop-in for the reference's ``blademaster_warp`` step/state API on the path
the Franka run, the prescribed-path scenes and the free-fall experiment use:
``solver.Config`` / ``solver.Solver``, ``coupling.ExternalToolPort`` /
``ToolState`` / ``Reaction``, ``geometry``, ``topology`` and ``presets``.
All per-substep work runs in hand-written sm_103a CUDA behind the C-ABI of
include/blademaster_gb300.h; there is no CPU fallback.
"""

__version__ = "0.1.0"
