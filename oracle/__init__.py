"""CPU oracle for the ADFWI propagator hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, on the CPU and in plain PyTorch tensor arithmetic, the
algorithm of the reference's time-stepping loops:

* ``acoustic.py``: ``ADFWI/propagator/acoustic_kernels.py`` (pad 16-37,
  step_forward 40-176, forward_kernel 179-301);
* ``elastic.py``: ``ADFWI/propagator/elastic_kernels.py`` (DiffCoef 20-58,
  D-operators 66-108, pad 175-216, PML steps 222-579, ABL steps 585-912,
  forward_kernel 917-1037).

It is differentiable through torch autograd (the reference's own gradient
mechanism), so it also serves as the gradient oracle. It is pinned against the
golden vectors in ``tests/golden/`` that the reference itself produced
(``tests/golden/make_golden.py``), see ``tests/test_oracle_golden.py``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package; the product (``adfwi_gb300``) never does.
Every function here refuses to run on a non-CPU device.
"""
from .acoustic import acoustic_forward, pad_edge  # noqa: F401
from .elastic import elastic_forward, diff_coef  # noqa: F401
