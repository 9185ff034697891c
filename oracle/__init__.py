"""CPU oracle for the falling-sand world tick (test infrastructure only).

Loaded by tests/, by ``__graft_entry__.smoke()`` and by bench.py's CPU baseline;
the product package never imports it.
"""
from .binding import Oracle, OracleWorld, build_oracle, PARTICLE_DTYPE, BODY_DTYPE  # noqa: F401
