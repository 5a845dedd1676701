"""Test infrastructure only: CPU checkers for the diffren_gb300 CUDA path.

Nothing in the product imports this package. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline and
``--impl reference`` legs) use it, and only as the checker or the timed CPU
baseline.

* ``oracle.raster``: ctypes wrappers over ``raster_oracle.c`` (this repo's C
  restatement of the reference rasterizer) and, where it was built, over
  ``_ref/libref_raster.so`` (the reference's own CPU rasterizer compiled in
  place from the reference tree by ``oracle/Makefile``).
* ``oracle.splat``: numpy float32 restatement of interpolation, splatting,
  normalization and compositing with the reference's operation order.
* ``oracle.torch_ref``: the same continuous math in torch (any dtype) with
  autograd, standing in for ``jax.grad`` through the reference.

Parity pins: the C restatement is checked bit-exactly against the compiled
reference CPU rasterizer (golden fixtures in ``tests/golden``, generated by
``tests/golden/make_golden.py``), and against the reference's golden PNGs and
known-answer vectors where the reference tree is present.
"""
