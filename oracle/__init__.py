"""CPU oracle of the loops SpMV/SpMM path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker or the timed CPU baseline; the product
(edge_loops_gb300/, include/) never imports it.

oracle.c restates the reference's CPU SpMV loop, its merge-path search and
split points, its work_oriented split and its group_mapped mapping (each
function cites the reference file:line it follows).  Parity of the
restatement is pinned against fixtures produced by the reference's own code
(tests/golden/, made by tests/golden/make_golden.py from oracle/_ref).
"""
from .oracle import *  # noqa: F401,F403
