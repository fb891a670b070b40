"""CPU restatement of the reference's arithmetic for this path — the checker.

Test infrastructure only: loaded by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py; never by the product package.
"""
