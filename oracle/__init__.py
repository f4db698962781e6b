"""Oracle: CPU restatement of the reference's interpolation hot path.

TEST INFRASTRUCTURE ONLY. Imported by tests/, by the smoke check in
__graft_entry__.py and by bench.py's CPU-baseline leg, as the checker and the
CPU baseline -- never by the spinterps_gb300 package.
"""
