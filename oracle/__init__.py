"""CPU oracle for the CVO registration path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
use this package, as the checker.  The product library never imports it.
"""
from .oracle import *  # noqa: F401,F403
