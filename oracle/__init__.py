"""CPU checkers for the Malevich draw path (TEST INFRASTRUCTURE ONLY).

`oracle.c` restates the reference's pipeline core in scalar C; `ref_build.py` compiles the
reference's own core headless. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg may import this package; the malevich_gb300 product never does.
"""
