"""CPU oracle of mosaic-art-rust's tile matching-and-placement path.

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
benchmark's CPU-baseline leg, as the checker.  The shipped library never uses
it.  See oracle.h for what it restates and how it is pinned.
"""
from .binding import OracleJob, build_oracle, lib  # noqa: F401
