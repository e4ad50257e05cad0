"""CPU oracle of the FlOF hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the CPU legs of bench.py import this
package; the product package ofblend_gb300 never does.
"""
from .binding import Oracle, build, dims_of, get, ncomp  # noqa: F401
