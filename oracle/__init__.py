"""CPU oracle for voxelis' batched SVO-DAG edit path — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this package, as the checker
or the timed CPU baseline; the product library never does.
"""
