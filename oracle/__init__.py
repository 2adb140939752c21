"""CPU oracle of the raster path -- test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use
this package, as the checker and the timed CPU restatement.  The library
(skity_gb300) never imports it.
"""
