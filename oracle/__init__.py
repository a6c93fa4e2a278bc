"""CPU oracle of the ReSTIR GI frame pipeline -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the checker; the product library never uses it.
"""
