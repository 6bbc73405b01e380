"""CPU oracle for the MandoCT reconstruction hot path -- TEST INFRASTRUCTURE.

This package restates, in float64 NumPy (and, for the timed CPU baseline, in
OpenMP C: ``cpu_ref.c``), the arithmetic of the reference's Taichi kernels:

  * ``fbp_ops``  -- run_mgfbp.py (filter taps, weighting, Toeplitz row filter,
                    pixel-driven FDK backprojection);
  * ``fpj_ops``  -- run_mgfpj_v3.py (ray-driven trilinear forward projection,
                    binning);
  * ``ir_ops``   -- run_mgfbp_iterative_recon_IRN_CGLS.py and ..._piccs.py
                    (effective ray map, masked projector, unmatched per-view
                    backprojector, TV reweighting, D^T W D, CGLS solves).

Every function cites the reference file:line it follows.  Parity of this
oracle is pinned against golden fixtures produced by running the reference's
own Python sources (``tests/golden/make_golden.py``, which executes them on the
CPU through a small Taichi-API stand-in).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import or execute anything in this package, and only as the checker or the
timed CPU baseline.  The product (``reconstruction_program_taichi_gb300``)
never calls it: its compute path is the CUDA library, and it fails loudly when
that library is missing.
"""

PI = 3.1415926536  # the reference's constant (run_mgfbp.py:16)
