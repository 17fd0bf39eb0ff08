"""Oracles for the Moldy force path -- TEST INFRASTRUCTURE ONLY.

``oracle.port`` is a C restatement of the reference's force_calc/kernel/ewald
algorithm (oracle/port/moldy_port.c), used by the tests as the parity checker
and by bench.py as the timed CPU baseline.  ``oracle.ref`` runs the reference's
own sources, compiled in place by oracle/build_ref.sh, where those sources are
present.  Nothing on the product path imports this package.
"""
