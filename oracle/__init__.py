"""CPU FP64 oracle for the 2D pair-HMM hot path -- TEST INFRASTRUCTURE ONLY.

A NumPy float64 restatement of the reference's (evoldoers/tkf-mixdom)
pair-HMM forward/backward, E-step and emission-count code, against which the
CUDA path is compared: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.
The product package never does, and the product fails loudly when its CUDA
library is missing instead of falling back to this code.

Parity pin: ``tests/golden/*.npz`` hold outputs of the reference's own
Python modules, run in this container under a NumPy implementation of the
subset of the JAX API they use (``tests/golden/jax_shim.py``,
``tests/golden/make_golden.py``).  ``tests/test_oracle_golden.py`` checks
this restatement against them.
"""
