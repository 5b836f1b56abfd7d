"""GB300-native (sm_103a) prover hot path for pyZKP: BN254 G1 MSM and Fr NTT / iNTT / coset NTT.

* ``pyzkp_gb300._native``  -- ctypes binding of the C ABI (include/zkgpu.h)
* ``pyzkp_gb300.plugin``   -- KernelFns for the reference's KernelRegistry (drop-in for the Metal backend)
* ``pyzkp_gb300.synth``    -- seeded synthetic workloads
* ``pyzkp_gb300.build``    -- in-tree nvcc build of libzkgpu.so
"""

__all__ = ["_native", "synth", "build"]
