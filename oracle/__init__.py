"""CPU oracle for the COV3D projection / covariance-SGD / mean-CG / Wiener hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this directory; only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it, and
only as the checker (or as the timed CPU port of the reference algorithm).

* ``nufft_oracle``  -- float64 numpy restatement of the reference's NUFFT plans, projection
  operators, cost functions, CG and latent-MAP solve, each function citing the reference
  file:line it follows; plus an exact direct-sum NUDFT and the exponential-of-semicircle
  (ES) kernel algorithm of the FINUFFT paper.
* ``es_oracle.c``   -- the same interpolation / spreading loops in plain C (float64 and
  float32 builds, OpenMP over points or slabs), for sizes numpy cannot reach in seconds
  and for the timed CPU baseline.
* ``cpu_step``      -- the covariance-SGD step, mean CG and Wiener solve assembled from the
  two above (the CPU port timed by ``bench.py --impl reference``).

Parity pinning: the discretized (trilinear / nearest, ``grid_sample`` semantics) functions
are pinned against fixtures produced by running the reference itself
(``tests/golden/make_golden.py``); the ES-kernel functions are pinned against the
direct-sum NUDFT, which in turn is pinned against the reference's own Fourier-slice
known-answer test (``tests/test_torch_wraps.py:266-278``).
"""
