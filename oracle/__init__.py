"""CPU oracle for the RCWA raster layer path — test infrastructure only.

Nothing in the product path imports this package. Only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only as the
checker (or as the timed CPU restatement of the reference), never as the computation that is
shipped or measured on the GPU.
"""
