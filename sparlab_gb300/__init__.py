"""GB300-native SIMP inner loop (density filter, SIMP, assembly, SA-AMG
preconditioned CG, sensitivities, OC) behind SparLab's LinearSolver and
ComplianceObjective interfaces.  The compute path is the CUDA library
``libsimp_gb300.so`` (sm_103a) reached through the C ABI of
``include/simp_gpu.h``; nothing here computes on the CPU."""
from . import problems  # noqa: F401

__all__ = ["problems"]
