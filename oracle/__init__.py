"""CPU oracle for the split-operator propagation path (test infrastructure only).

Imported only by the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``; never by the product package.
"""
