"""ORACLE — TEST INFRASTRUCTURE ONLY.

CPU restatement of the LIGGGHTS-INL sphere timestep (``dem_oracle.c``) and
the recipe that compiles the reference itself (``ref/``).  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
this package; the GPU product never imports it.
"""
