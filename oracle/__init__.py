"""CPU oracle for the path-tracing hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference
arm import this package; the product package never does.
"""
