"""CPU oracle for the GB300 PageRank path (test infrastructure only).

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
legs: as the checker, or as the timed CPU baseline.  Never the product path.
"""
