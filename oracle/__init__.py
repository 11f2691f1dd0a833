"""Test oracle for the PADO GPU library (TEST INFRASTRUCTURE ONLY).

``oracle.orc`` wraps the CPU restatement (liboracle.so); ``oracle.ref`` wraps
the reference's own labelers when they were built into ``oracle/_ref``.  Only
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
package, and only as the checker or the timed CPU baseline.
"""
