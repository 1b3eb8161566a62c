"""Oracle for MST-CFD's density-based residual path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker or the timed CPU
baseline.  The product (``mst-cfd_gb300``) never imports it.

* ``mstoracle.c``  -- C restatement of the reference path (built to
  ``oracle/_build/libmstoracle.so``), wrapped by :mod:`oracle.pyoracle`.
* ``ref/``         -- recipe that compiles the reference's own sources into
  ``oracle/_ref`` (only where the reference checkout exists), wrapped by
  :mod:`oracle.refrun`.
"""
