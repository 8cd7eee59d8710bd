"""CPU oracle of the PENTrack tracking hot path -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the checker of the GPU engine; the product (pentrack_gb300) never imports it.
"""
