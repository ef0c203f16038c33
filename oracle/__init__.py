"""CPU oracle for the ray-casting sampler path -- TEST INFRASTRUCTURE.

Everything under ``oracle/`` is the checker, never the product:

* ``ytoracle.c`` -- a C restatement of yt's sampler path (walk_volume, the
  four samplers, lens extents and ray vectors, the transfer-function lookup,
  ghost-zone vertex centring), compiled with ``-ffp-contract=off``.
* ``cpu.py`` -- ctypes binding of that library and its build step.
* ``glue.py`` -- numpy restatements of the Python glue around the sampler
  (camera orientation, lens parameters, transfer-function tables, the AMR
  kd-tree build and viewpoint order, brick slicing, the render loop).
* ``build_ref.py`` / ``ref_trace.pyx`` -- build the reference's own compiled
  sampler from its sources (only where the reference checkout exists) for
  pinning the restatement and generating golden fixtures.

Only ``tests/``, ``__graft_entry__.smoke`` and the CPU-baseline leg of
``bench.py`` may import this package.
"""
