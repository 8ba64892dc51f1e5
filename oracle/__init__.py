"""CPU checkers for the GB300 SIMPLE/SST path (test infrastructure only).

``simple_oracle.c`` restates the reference algorithm in plain C; ``refdriver``
runs the unmodified reference sources where they are available.  Only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
package, and only as the checker.
"""
