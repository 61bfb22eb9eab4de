"""Test infrastructure: FP64 CPU restatement of the reference path (the checker).  Imported only
by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg."""
