"""CPU oracle for the GPU partitioning path (test infrastructure only).

``hp_oracle`` restates the reference's FP64 algorithm in NumPy; ``refshim``
and ``refrun`` run the unmodified reference in this container to pin it.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
arm use this package.
"""
