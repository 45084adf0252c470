"""TEST INFRASTRUCTURE ONLY: the CPU oracle for the all-pairs normalised
cross-correlation.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg may import this package, and only as the checker or the timed
CPU baseline; the product (``seismic_gb300``) never imports it.
"""
