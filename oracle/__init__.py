"""CPU oracle of torch-fem's forward + adjoint path: test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg;
never by the product package.
"""
