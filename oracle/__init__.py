"""CPU oracle for the PT-MC hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py use
this package, and only as the checker or as the timed CPU baseline.
"""
