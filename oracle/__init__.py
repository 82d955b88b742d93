"""CPU oracle of the ADER-DG element update (TEST INFRASTRUCTURE ONLY).

Imported by tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py; never
by the product package.
"""
