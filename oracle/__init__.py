"""The oracle: TEST INFRASTRUCTURE ONLY.

CPU restatements of the reference's droplet step used as parity checkers and
as the timed CPU baseline. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may import this package; the product path never does.
"""
