"""pyhalma_gb300 — pyHALMA's halo-finding hot path on one GB300 (sm_103a).

Drop-in modules mirroring the reference's own (same function names and signatures):
  ``pyhalma_gb300.fof``              python_scripts/fof.py
  ``pyhalma_gb300.halo_gas``         python_scripts/halo_gas.py (potential, RPS, most bound)
  ``pyhalma_gb300.halo_properties``  python_scripts/halo_properties.py (reductions)
New capabilities:
  ``pyhalma_gb300.unbinding``        batched iterative unbinding, one-call snapshot pipeline
  ``pyhalma_gb300.autograd``         differentiable softened potential (torch)
  ``pyhalma_gb300.autotune``         tile-shape autotuner for the batched pair kernel
All compute runs in libhalma_gb300.so (hand-written CUDA, C ABI in include/halma.h).
"""
__version__ = "0.1.0"
