"""CPU oracle for the inverse-iteration path -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package; the product library never does.
"""
