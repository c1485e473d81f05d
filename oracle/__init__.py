"""TEST INFRASTRUCTURE ONLY: the CPU oracle for the Biot-Savart / BEM hot path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker.  The product library never imports it.
"""
from .oracle import *  # noqa: F401,F403
