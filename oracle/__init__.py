"""CPU oracle of the lattice-Boltzmann time step -- test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product (thesis_gb300) never imports it.
"""
