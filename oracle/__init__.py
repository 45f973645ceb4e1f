"""CPU restatement of the turbulentBL time step (test infrastructure only).

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
See tbl_oracle.cpp for what is restated and the parity status (unpinned
against the reference binary: no Fortran/MPI toolchain is available).
"""
