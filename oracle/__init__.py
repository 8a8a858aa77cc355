"""CPU oracle for the NNAP energy/force/virial path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``, never by the product package ``jse_gb300``.

* ``oracle.model``   -- model-file loader and parameter packing (FP64), a restatement of
                        the reference's Java loader.
* ``oracle.native``  -- ctypes bindings to ``nnap_oracle.cpp`` (an FP64 C++ restatement
                        of the reference's per-atom arithmetic, neighbor search and
                        accumulators) and, when it has been built, to ``_ref/``
                        (the reference's own headers expanded by ``nnapgen.py``).
* ``oracle.nnapgen`` -- expander for the reference's NNAPGEN template markers.
"""
