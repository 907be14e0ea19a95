"""GB300-native batched per-cell geochemistry (PFLOTRAN's RReact step).

The compute path is the C-ABI shared library built from csrc/ (hand-written
sm_103a CUDA); this package holds the host-side mirror of its interface:
ctypes structures (abi), reaction-network tables in PFLOTRAN's layout
(network), per-cell SoA batches (cells), seeded workloads (workloads) and the
library loader (lib).
"""
