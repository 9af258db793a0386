"""CPU FP64 oracle of the reference transient path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this package.  Parity status: unpinned (see topo_oracle.h).
"""
from .oracle import *  # noqa: F401,F403
