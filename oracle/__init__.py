"""CPU oracle for the VoxelEncoding hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; the product library never does.
"""
