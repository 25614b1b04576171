"""CPU oracle for the KISS FFT hot path -- test infrastructure only.

Loaded by the tests, by ``__graft_entry__.smoke()`` and by the CPU-baseline
leg of ``bench.py``.  The GPU library never imports or links anything here.
"""
