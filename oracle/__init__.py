"""CPU oracle of the lattice Boltzmann update: test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, as the checker; the product (boltzmannfluids_gb300) never does.
"""
