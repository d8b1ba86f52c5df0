"""CPU oracle for the GeoPhyInv FDTD hot path -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package.  The product (geophyinv.jl_gb300/) never does.
"""
