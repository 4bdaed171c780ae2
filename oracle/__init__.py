"""CPU oracle for the MULTIANS decode path (test infrastructure only).

Loaded by tests/, by ``__graft_entry__.smoke()`` to compare the CUDA
decoder's output against, and by ``bench.py`` for its CPU baseline.  The
product package never imports it.
"""
