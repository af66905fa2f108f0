"""CPU oracle for the RaccoonGPURender hot path — test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
as the checker; the product package never imports it.
"""
