"""Test infrastructure only: the CPU oracle of the BROADCAST DNC5 hot path.

A C++ restatement of the reference Fortran (broadcast_oracle.hpp) and its
ctypes front end (oracle.py).  Imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg; never by the broadcast_gb300 package.
"""
