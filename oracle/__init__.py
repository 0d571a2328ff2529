"""CPU oracle for the photon-geodesic hot path -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU
baseline leg; never by the package.
"""
