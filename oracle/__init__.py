"""CPU oracle of the reference's GPU cloth step.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product (licenta_gb300/).
"""
