"""pplacer_gb300: GB300 (sm_103a) placement-likelihood engine behind pplacer's
Linear / Glv API.

* ``pplacer_gb300.linear`` -- drop-in for pplacer_src/linear_c.c (FP64 on the GPU)
* ``pplacer_gb300.engine`` -- batched placement (FP32 GLVs, exact int32 exponents)
* ``pplacer_gb300.model``  -- host-side model construction (Diagd, Gamma rates)
* ``pplacer_gb300.synth``  -- seeded synthetic workloads
* ``pplacer_gb300.build``  -- nvcc build of the CUDA library (sm_103a)
"""
