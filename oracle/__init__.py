"""CPU oracle for the retrofire render path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package.  The product (retrofire_gb300) never does.
"""
